// Mixed-precision weight solves with the Schur-complement FP32 preconditioner (schur.cuh):
// instantiations for stencils of at most 32 nodes and the dispatcher used by the operator
// builder.  Stencils of 33..48 nodes (at most 16 monomials) are instantiated in
// weights_reg48_r<RMAX>.cu, the rest up to 64 nodes in weights_reg64*.cu.
#include "schur.cuh"

size_t schur_smem_per_warp(int SP, int SM, int max_n, int max_m, int nops)
{
    return make_schur_layout(SP, SM, max_n, max_m, nops).total;
}

size_t solve_mixed_reg_smem_per_warp(int S, int max_n, int max_m, int nops)
{
    return schur_smem_per_warp(S <= 32 ? 32 : 64, max_m <= 16 ? 16 : 32, max_n, max_m, nops);
}

cudaError_t launch_schur_sp32(const SolveArgs &a, const OpTable &ops, int SM, int RMAX, int wpb, int num_sms,
                              cudaStream_t st)
{
    if (SM == 16) return RMAX == 4 ? launch_schur<32, 16, 4>(a, ops, wpb, num_sms, st)
                                   : launch_schur<32, 16, 8>(a, ops, wpb, num_sms, st);
    return RMAX == 4 ? launch_schur<32, 32, 4>(a, ops, wpb, num_sms, st)
                     : launch_schur<32, 32, 8>(a, ops, wpb, num_sms, st);
}

// Schur-complement mixed solve for stencils of at most 64 nodes, at most 32 monomials and at
// most 8 operators in scaled coordinates; cudaErrorNotSupported for other shapes (the
// shared-memory mixed kernel of weights.cu takes those).
cudaError_t launch_solve_mixed_reg(const SolveArgs &a, const OpTable &ops, int max_m, int wpb, int num_sms,
                                   cudaStream_t st)
{
    (void)max_m;
    if (a.nsys <= 0) return cudaSuccess;
    const int r = ops.nops;
    if (r > 8 || a.max_n > 64 || a.max_m > 32 || a.unscaled_overload) return cudaErrorNotSupported;
    if (wpb > 16 || wpb < 1) wpb = 4;  // launch_schur lowers it to what the kernel and shared memory allow
    const int SM = a.max_m <= 16 ? 16 : 32;
    const int RMAX = r <= 4 ? 4 : 8;
    if (a.max_n <= 32) return launch_schur_sp32(a, ops, SM, RMAX, wpb, num_sms, st);
    if (a.max_n <= 48 && SM == 16)
        return RMAX == 4 ? launch_schur_48_16_4(a, ops, wpb, num_sms, st) : launch_schur_48_16_8(a, ops, wpb, num_sms, st);
    return launch_schur_sp64(a, ops, SM, RMAX, wpb, num_sms, st);
}
