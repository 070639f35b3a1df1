// Schur-complement mixed solves (schur.cuh) for stencils of 33..64 nodes: two Phi rows per lane.
#include "schur.cuh"

cudaError_t launch_schur_sp64(const SolveArgs &a, const OpTable &ops, int SM, int RMAX, int wpb, int num_sms,
                              cudaStream_t st)
{
    if (SM == 16) return RMAX == 4 ? launch_schur<64, 16, 4>(a, ops, wpb, num_sms, st)
                                   : launch_schur<64, 16, 8>(a, ops, wpb, num_sms, st);
    return RMAX == 4 ? launch_schur<64, 32, 4>(a, ops, wpb, num_sms, st)
                     : launch_schur<64, 32, 8>(a, ops, wpb, num_sms, st);
}
