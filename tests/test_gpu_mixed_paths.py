"""GPU parity of the mixed-precision machinery's less-travelled paths, against the CPU oracle.

* The per-system FP64 fallback: handles whose refinement budget or tolerance cannot be met
  send every system, or some of them, to the FP64 re-solve; all rows (re-solved or not) must
  still match the oracle, and the statistics must say how many fell back.
* Hyperviscosity (src/hyperviscosity_operator.jl:97-161) in mixed precision with PHS r^5 and
  K = 4 (the configuration of the time-stepping example, examples/adv_diff_test.jl:95-101).
* The shared-memory mixed kernel, which takes what the register kernels do not: stencils of
  more than 64 nodes, more than 32 monomials, or more than 8 operators.
* The closed-form right-hand sides of the register kernel (PHS r^3 with every operator in
  {E, Dx, Dy, Dxx, Dyy, Dxy, Lap}, and r^5 with the K = 4 pair Dxk/Dyk): operator subsets and
  orders, stencil sizes of each register instantiation, and evaluation points off the nodes
  (rows that share a nearest node's factorisation).  The full r^3 set is also covered by
  test_gpu_parity.py::test_weights_all_ops.

Bars as in test_gpu_parity.py: 1e-9 row-relative for mixed weights of well-conditioned
systems (PHS r^3, degree <= 3), 5e-9 for r^5 or degree >= 4 (where the oracle's explicit
inverse and any LU already differ by ~cond(A) * 1e-16 * growth).
"""
import numpy as np
import pytest

from conftest import rel_row_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-9
HARD_TOL = 5e-9


def tol_for(p, deg):
    return HARD_TOL if (p >= 5 or deg >= 4) else MIXED_TOL


def grid(pkg, nx, seed):
    return pkg.nodesets.jittered_grid(nx, seed=seed)[0]


def check_against_oracle(s, ref, ops, n, tol):
    for o in s.ops:
        _, col, val = s.csr_arrays(o)
        assert (col.reshape(-1, n) == ref["cols"]).all(), o
        err = rel_row_err(val, ref["W"][ops.index(o)])
        assert err < tol, (o, err)


def test_forced_fallback_every_system(pkg, orc, gpu):
    """max_refine = 1 allows one correction and no convergence test, so every system is queued
    for the FP64 re-solve: n_fallback equals the number of systems and the weights are the
    FP64 kernel's."""
    X = grid(pkg, 48, seed=13)
    p, n, deg = 3, 30, 3
    ops = ("Dx", "Dy", "Lap")
    ref = orc.generate(X, X, p, n, deg, ops)
    with pkg.Handle(max_refine=1) as h:
        with pkg.OperatorSet(X, None, p, n, deg, ops=ops, precision="mixed", handle=h) as s:
            st = s.stats.as_dict()
            assert st["n_systems"] == len(X)
            assert st["n_fallback"] == st["n_systems"], st
            assert sum(st["refine_hist"]) == 0
            check_against_oracle(s, ref, ops, n, FP64_TOL)


def test_forced_fallback_some_systems(pkg, orc, gpu):
    """refine_tol = 1e-17 sits below what a double-float solution can resolve for many
    systems: those stall and fall back while others still converge.  Both kinds of rows are
    checked against the oracle."""
    X = grid(pkg, 48, seed=14)
    p, n, deg = 3, 30, 3
    ops = ("Dx", "Dy", "Lap")
    ref = orc.generate(X, X, p, n, deg, ops)
    with pkg.Handle(refine_tol=1e-17, max_refine=4) as h:
        with pkg.OperatorSet(X, None, p, n, deg, ops=ops, precision="mixed", handle=h) as s:
            st = s.stats.as_dict()
            assert 0 < st["n_fallback"] <= st["n_systems"], st
            assert st["n_fallback"] + sum(st["refine_hist"]) == st["n_systems"], st
            check_against_oracle(s, ref, ops, n, MIXED_TOL)


def test_forced_fallback_uneven_sizes(pkg, orc, gpu):
    """The FP64 re-solve of systems of mixed (k, degree) classes and boundary classes (the
    queue holds systems of every shape class the binned mixed launches took)."""
    d = pkg.nodesets.rectangle_with_ghosts(total=6000, seed=15, main_fraction=0.4)
    X, cls, nn, dd = d["X"], d["node_class"], d["n"], d["deg"]
    ops = ("Dx", "Dy", "Lap")
    with pkg.Handle(max_refine=1) as h:
        with pkg.OperatorSet(X, None, 3, 0, 0, ops=ops, precision="mixed", node_class=cls, n_per_node=nn,
                             deg_per_node=dd, handle=h) as s:
            st = s.stats.as_dict()
            assert st["n_fallback"] == len(X), st
            for k, g in pkg.nodesets.SIZE_CLASSES:
                rows = np.nonzero((nn == k) & (dd == g))[0]
                ref = orc.generate(X, X[rows], 3, k, g, ops, cls=cls)
                for q, o in enumerate(ops):
                    rp, col, val = s.csr_arrays(o)
                    W = np.stack([val[rp[r]:rp[r + 1]] for r in rows])
                    C = np.stack([col[rp[r]:rp[r + 1]] for r in rows])
                    assert (C == ref["cols"]).all()
                    assert rel_row_err(W, ref["W"][q]) < max(FP64_TOL, tol_for(3, g)), (o, k)


@pytest.mark.parametrize("n,deg", [(30, 3), (42, 5), (20, 2)])
def test_mixed_hyperviscosity_r5_k4(pkg, orc, gpu, n, deg):
    """hyperviscosity_operator in mixed precision: PHS r^5, K = 4, Dxk and Dyk (and their sum)
    against the oracle; whatever needed the FP64 fallback is included."""
    X = grid(pkg, 48, seed=16)
    p, K = 5, 4
    ops = ("Dxk", "Dyk", "HV")
    ref = orc.generate(X, X, p, n, deg, ops, k_deriv=K)
    with pkg.OperatorSet(X, None, p, n, deg, ops=ops, k_deriv=K, precision="mixed") as s:
        check_against_oracle(s, ref, ops, n, tol_for(p, deg))
        st = s.stats.as_dict()
        assert st["n_fallback"] + sum(st["refine_hist"]) == st["n_systems"]


def test_mixed_hyperviscosity_drop_in(pkg, orc, gpu):
    """The drop-in hyperviscosity_operator(k, X, Y, p, n, polydeg) with precision="mixed"
    returns the oracle's CSC matrices (src/hyperviscosity_operator.jl:26-175)."""
    X = grid(pkg, 40, seed=17)
    p, n, deg, K = 5, 30, 3, 4
    Dxk, Dyk = pkg.hyperviscosity_operator(K, X, X, p, n, deg, precision="mixed")
    ref = orc.generate(X, X, p, n, deg, ("Dxk", "Dyk"), k_deriv=K)
    for q, A in enumerate((Dxk, Dyk)):
        cp, rv, nz = orc.to_csc(len(X), len(X), ref["cols"], ref["W"][q])
        assert np.array_equal(A.indptr, cp - 1)
        assert np.array_equal(A.indices, rv - 1)
        # row-relative error through the CSC values: compare per row after a CSR conversion
        W = A.tocsr()
        Wr = orc_csr(len(X), ref["cols"], ref["W"][q])
        num = abs(W - Wr).max(axis=1).toarray().ravel()
        den = abs(Wr).max(axis=1).toarray().ravel()
        assert (num / den).max() < HARD_TOL


def orc_csr(N, cols, W):
    import scipy.sparse as sp

    n = cols.shape[1]
    return sp.csr_matrix((W.ravel(), (np.repeat(np.arange(len(cols)), n), cols.ravel())), shape=(len(cols), N))


@pytest.mark.parametrize("p,n,deg", [(3, 80, 3), (3, 90, 2), (3, 70, 6)])
def test_generic_mixed_kernel_large_stencils(pkg, orc, gpu, p, n, deg):
    """Stencils of more than 64 nodes (and degree 6: 28 monomials, s = 98) take the
    shared-memory mixed kernel."""
    X = grid(pkg, 40, seed=18)
    ops = ("Dx", "Dy", "Lap")
    ref = orc.generate(X, X, p, n, deg, ops)
    with pkg.OperatorSet(X, None, p, n, deg, ops=ops, precision="mixed") as s:
        check_against_oracle(s, ref, ops, n, tol_for(p, deg))
        st = s.stats.as_dict()
        assert st["n_fallback"] + sum(st["refine_hist"]) == st["n_systems"]


def test_generic_mixed_kernel_many_operators(pkg, orc, gpu):
    """All ten operators at once (E, Dx, Dy, Dxx, Dyy, Dxy, Lap, Dxk, Dyk, HV; more than the
    register kernels' 8) take the shared-memory mixed kernel."""
    X = grid(pkg, 40, seed=19)
    p, n, deg, K = 5, 30, 3, 2
    ops = ("E", "Dx", "Dy", "Dxx", "Dyy", "Dxy", "Lap", "Dxk", "Dyk", "HV")
    ref = orc.generate(X, X, p, n, deg, ops, k_deriv=K)
    with pkg.OperatorSet(X, None, p, n, deg, ops=ops, k_deriv=K, precision="mixed") as s:
        assert len(s.ops) == 10
        check_against_oracle(s, ref, ops, n, HARD_TOL)


def test_generic_mixed_kernel_forced_fallback(pkg, orc, gpu):
    """The shared-memory mixed kernel's fallback queue (n = 80, every system re-solved in FP64).
    80-node systems are worse conditioned than the 1e-10 bar assumes (cond(A) <~ 1e5), so the
    FP64 LU and the oracle's explicit inverse are compared at the mixed bar."""
    X = grid(pkg, 32, seed=20)
    p, n, deg = 3, 80, 3
    ops = ("Dx", "Lap")
    ref = orc.generate(X, X, p, n, deg, ops)
    with pkg.Handle(max_refine=1) as h:
        with pkg.OperatorSet(X, None, p, n, deg, ops=ops, precision="mixed", handle=h) as s:
            assert s.stats.n_fallback == len(X)
            check_against_oracle(s, ref, ops, n, MIXED_TOL)


@pytest.mark.parametrize("wpb", [8, 16])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_fixed_cta_size_beyond_shared_memory(pkg, orc, gpu, wpb, precision):
    """A fixed CTA size (rbffd_options.warps_per_block) larger than a 60-node, degree-5
    system's shared memory allows: the launches lower it to what fits instead of failing, and
    the weights still match the oracle."""
    X = grid(pkg, 40, seed=21)
    p, n, deg = 3, 60, 5
    ops = ("Dx", "Dy", "Lap")
    ref = orc.generate(X, X, p, n, deg, ops)
    with pkg.Handle(warps_per_block=wpb) as h:
        with pkg.OperatorSet(X, None, p, n, deg, ops=ops, precision=precision, handle=h) as s:
            check_against_oracle(s, ref, ops, n, HARD_TOL)


@pytest.mark.parametrize("tol", [1e-11, 1e-10])
def test_loose_refine_tol_keeps_its_promise(pkg, orc, gpu, tol):
    """A looser refine_tol stops the refinement earlier, but only on a contraction measured
    from two corrections: the weights stay within ~10 x the tolerance of the oracle (stopping
    on the first correction's estimate erred by ~1e3 x the tolerance)."""
    X = grid(pkg, 64, seed=23)
    p, n, deg = 3, 30, 3
    ops = ("Dx", "Dy", "Lap")
    ref = orc.generate(X, X, p, n, deg, ops)
    with pkg.Handle(refine_tol=tol) as h:
        with pkg.OperatorSet(X, None, p, n, deg, ops=ops, precision="mixed", handle=h) as s:
            st = s.stats.as_dict()
            assert st["refine_hist"][1] == 0, st
            check_against_oracle(s, ref, ops, n, max(MIXED_TOL, 10 * tol))


@pytest.mark.parametrize("ops", [("Lap",), ("Dx",), ("Dy", "Lap"), ("Lap", "Dx"), ("Lap", "Dy", "Dx")])
@pytest.mark.parametrize("n,deg", [(30, 3), (45, 4), (60, 5)])
def test_closed_form_rhs_operator_subsets(pkg, orc, gpu, ops, n, deg):
    X = grid(pkg, 48, seed=8)
    ref = orc.generate(X, X, 3, n, deg, ops)
    with pkg.OperatorSet(X, None, 3, n, deg, ops=ops, precision="mixed") as s:
        check_against_oracle(s, ref, ops, n, tol_for(3, deg))


def test_closed_form_rhs_noncollocated(pkg, orc, gpu):
    X = grid(pkg, 40, seed=9)
    Y = np.random.default_rng(10).uniform(0.02, 0.98, (3000, 2))
    ops = ("Dx", "Dy", "Lap")
    ref = orc.generate(X, Y, 3, 20, 3, ops)
    with pkg.OperatorSet(X, Y, 3, 20, 3, ops=ops, precision="mixed") as s:
        check_against_oracle(s, ref, ops, 20, MIXED_TOL)


@pytest.mark.parametrize("ops", [("Dxk", "Dyk"), ("Dyk",), ("Dyk", "Dxk")])
@pytest.mark.parametrize("n,deg", [(20, 2), (30, 3), (45, 4), (60, 5)])
def test_closed_form_rhs_hyperviscosity_pair(pkg, orc, gpu, ops, n, deg):
    """PHS r^5 with K = 4 and only Dxk/Dyk (the time-stepping example's pair) takes the closed
    form d4/dx4 r^5 = 15 r (3 + 6 u - u^2), u = x^2 / r^2, and 4! at x^4 or y^4 in the
    polynomial rows; degrees 4 and 5 have those monomials."""
    X = grid(pkg, 48, seed=17)
    ref = orc.generate(X, X, 5, n, deg, ops, k_deriv=4)
    with pkg.OperatorSet(X, None, 5, n, deg, ops=ops, k_deriv=4, precision="mixed") as s:
        check_against_oracle(s, ref, ops, n, tol_for(5, deg))


def test_closed_form_rhs_hyperviscosity_noncollocated(pkg, orc, gpu):
    X = grid(pkg, 40, seed=18)
    Y = np.random.default_rng(19).uniform(0.02, 0.98, (3000, 2))
    ops = ("Dxk", "Dyk")
    ref = orc.generate(X, Y, 5, 30, 3, ops, k_deriv=4)
    with pkg.OperatorSet(X, Y, 5, 30, 3, ops=ops, k_deriv=4, precision="mixed") as s:
        check_against_oracle(s, ref, ops, 30, tol_for(5, 3))
