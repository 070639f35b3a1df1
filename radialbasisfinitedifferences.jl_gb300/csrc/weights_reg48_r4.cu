// Schur-complement mixed solve (schur.cuh) for stencils of 33..48 nodes with at most 16
// monomials and at most 4 operators (one instantiation per translation unit).
#include "schur.cuh"

cudaError_t launch_schur_48_16_4(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st)
{
    return launch_schur<48, 16, 4>(a, ops, wpb, num_sms, st);
}
