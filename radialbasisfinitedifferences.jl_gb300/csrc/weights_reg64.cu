// Schur-complement mixed solves (schur.cuh) for stencils of 33..64 nodes: two Phi rows per lane.
// Dispatcher only: each instantiation is compiled in its own translation unit
// (weights_reg64_m<SM>_r<RMAX>.cu) so that the build compiles the four kernels in parallel.
#include "schur.cuh"

cudaError_t launch_schur_sp64(const SolveArgs &a, const OpTable &ops, int SM, int RMAX, int wpb, int num_sms,
                              cudaStream_t st)
{
    if (SM == 16) return RMAX == 4 ? launch_schur_64_16_4(a, ops, wpb, num_sms, st)
                                   : launch_schur_64_16_8(a, ops, wpb, num_sms, st);
    return RMAX == 4 ? launch_schur_64_32_4(a, ops, wpb, num_sms, st)
                     : launch_schur_64_32_8(a, ops, wpb, num_sms, st);
}
