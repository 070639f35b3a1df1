// Host build of the device routine in csrc/phi_fixed.cuh, loaded by test_phi_fixed.py through
// ctypes: the fixed-point conversion and r^3 / r^2 of node pairs, to be checked against exact
// rational arithmetic.
#include "../radialbasisfinitedifferences.jl_gb300/csrc/phi_fixed.cuh"

extern "C" {

void fx_to_fixed61(const double *x, int64_t n, int64_t *out)
{
    for (int64_t i = 0; i < n; i++) out[i] = rbffd_fx::to_fixed61(x[i]);
}

// pts: n pairs as (xi, yi, xj, yj) doubles with |coordinate| < 2.
void fx_r3(const double *pts, int64_t n, double *r3, double *r2)
{
    using namespace rbffd_fx;
    for (int64_t k = 0; k < n; k++) {
        const double *q = pts + 4 * k;
        r3[k] = r3_fixed(to_fixed61(q[0]), to_fixed61(q[1]), to_fixed61(q[2]), to_fixed61(q[3]), r2 + k);
    }
}
}
