"""CPU checks of integer identities the CUDA kernels rely on.

The register Schur kernel (csrc/schur.cuh, div19 / div19_magic) splits flat indices
t = i r + q (t < 2^12, divisors r, m <= 128) with floor(t / d) = (t * ceil(2^19 / d)) >> 19 in
32-bit unsigned arithmetic instead of a run-time integer division.  The identity (a case of
Granlund and Montgomery's division by invariant integers) is checked here over its whole
stated domain, together with the 32-bit range of the product.
"""


def test_multiply_shift_quotient_exact_on_its_domain():
    for d in range(1, 129):
        g = (2 ** 19 + d - 1) // d
        for t in range(2 ** 12):
            assert (t * g) >> 19 == t // d, (t, d)
            assert t * g < 2 ** 32
