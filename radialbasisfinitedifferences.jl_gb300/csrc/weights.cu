// Batched local RBF-FD weight solves: one warp per local system.
//
// For every interpolation node j with at least one evaluation row, the warp
//   1. gathers the stencil, centres it on x_j and scales each axis by 1/max|dx|
//      (src/scalestencil.jl:10-21),
//   2. assembles A = [Phi P; P' 0] (src/rbfblock.jl:14-20, src/polynomialblock.jl:26-28,
//      src/interpolationmatrix.jl:3-5) in shared memory,
//   3. LU-factors it with partial pivoting (the reference inverts it, :8; solving with the
//      factors gives the same weights to rounding),
//   4. for each evaluation row builds the right-hand side [L phi(y~ - x~_i); L P(y~)] with
//      exact zeros replaced by eps (src/generate_operator.jl:122-157), solves, unscales
//      (:161-166; src/hyperviscosity_operator.jl:159-160) and writes the weights straight
//      into the CSR rows of every requested operator.
//
// GB300 executes FP64 at 1/64 of the FP32 rate, and an FP64 warp instruction costs the
// same whatever its active mask.  Both kernels therefore keep every FP64 instruction
// lane-full (flat (row, column) work distribution) and move everything that need not be
// FP64 -- pivot comparisons, index arithmetic, norms -- to the integer and FP32 pipes.
//
// FP64 kernel: FP64 assembly, flat-mapped right-looking LU in shared memory, FP64 solves.
// Mixed kernel: FP32 assembly and LU (one row per lane, virtual pivoting, vectorised row
// updates), then iterative refinement with residuals b - A x computed in FP64 against the
// FP64 matrix, corrections solved with the FP32 factors, until the predicted relative
// weight error is below refine_tol; a system whose refinement stalls is queued for the
// FP64 kernel.
#include "solve_common.cuh"

namespace {

// ---------------------------------------------------------------------------
// FP64 kernel.  Systems: a.sys_node[sys] for sys in [0, nsys), or the subset list.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) solve_fp64_kernel(SolveArgs a, OpTable ops, const int32_t *subset,
                                                         const int *subset_count)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Layout L = make_layout(a.max_s, a.max_n, ops.nops, false);
    unsigned char *base = smem_raw + (size_t)wib * L.total;
    double *A = (double *)(base + L.A);
    double *xs = (double *)(base + L.xs);
    double *B = (double *)(base + L.B);
    double *dinv = (double *)(base + L.dinv);
    int *piv = (int *)(base + L.piv);
    int *pinv = (int *)(base + L.pinv);
    int *sid = (int *)(base + L.sid);

    int64_t nwork = subset ? (int64_t)*subset_count : a.nsys;
    int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // systems claimed from a counter when one is given (persistent CTAs even out the tail),
    // else a fixed grid stride
    const bool claim = a.next_sys && !subset;
    auto next = [&](int64_t cur) -> int64_t {
        if (!claim) return cur + nw;
        unsigned long long v = 0ull;
        if (lane == 0) v = atomicAdd(a.next_sys, 1ull);
        return (int64_t)__shfl_sync(RBFFD_FULL, v, 0);
    };
    for (int64_t w = claim ? next(0) : gw; w < nwork; w = next(w)) {
        int64_t sys = subset ? (int64_t)subset[w] : (a.sys_list ? (int64_t)a.sys_list[w] : a.sys_base + w);
        int j = a.sys_node[sys];
        int n = a.n_node ? a.n_node[j] : a.n;
        int deg = a.deg_node ? a.deg_node[j] : a.deg;
        int m = npoly(deg), s = n + m, lda = lda64_of(s);
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        assemble64(A, lda, xs, n, m, deg, ops.p, lane);
        bool ok = warp_lu64(A, lda, s, piv, dinv, lane);
        if (!ok) {
            if (lane == 0) atomicMin((unsigned long long *)a.first_bad, (unsigned long long)j);
            continue;
        }
        __syncwarp();
        make_pinv(piv, pinv, s, lane);
        int64_t r0, r1;
        system_rows(a, sys, j, r0, r1);
        for (int64_t t = r0; t < r1; t++) {
            int64_t row = row_id(a, t);
            double yx, yy;
            if (a.unscaled_overload) {
                yx = xs[0];
                yy = xs[1];
            } else {
                double2 yp = eval_point(a, row);
                yx = (yp.x - xc.x) * sx;  // src/generate_operator.jl:110,120
                yy = (yp.y - xc.y) * sy;
            }
            build_rhs(ops, xs, n, m, yx, yy, sx, sy, a.unscaled_overload, pinv, B, lane);
            warp_lu_solve64(A, lda, s, dinv, B, ops.nops, lane);
            write_row(a, ops, row, B, n, sid, sx, sy, lane);
            __syncwarp();
        }
        // a mixed-precision build whose class the autotuner gave to this kernel: the system
        // needed no refinement step
        if (a.hist && !subset && lane == 0) atomicAdd(&a.hist[0], 1ull);
    }
}

// ---------------------------------------------------------------------------
// Mixed-precision kernel.  NS = row slots per lane (s <= 32*NS), RMAX >= nops.
// ---------------------------------------------------------------------------
template <int NS, int RMAX>
__global__ void __launch_bounds__(256) solve_mixed_kernel(SolveArgs a, OpTable ops)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Layout L = make_layout(a.max_s, a.max_n, ops.nops, true);
    unsigned char *base = smem_raw + (size_t)wib * L.total;
    double *A = (double *)(base + L.A);
    float *A32 = (float *)(base + L.A32);
    double *xs = (double *)(base + L.xs);
    double *B = (double *)(base + L.B);
    double *X = (double *)(base + L.X);
    float *R32 = (float *)(base + L.R32);
    float *dinv32 = (float *)(base + L.dinv);
    int *perm = (int *)(base + L.piv);
    int *sid = (int *)(base + L.sid);
    float *prow = (float *)(base + L.prow);
    const int r = ops.nops;

    int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    auto next = [&](int64_t cur) -> int64_t {
        if (!a.next_sys) return cur + nw;
        unsigned long long v = 0ull;
        if (lane == 0) v = atomicAdd(a.next_sys, 1ull);
        return (int64_t)__shfl_sync(RBFFD_FULL, v, 0);
    };
    for (int64_t ts = a.next_sys ? next(0) : gw; ts < a.nsys; ts = next(ts)) {
        const int64_t sys = a.sys_list ? (int64_t)a.sys_list[ts] : a.sys_base + ts;
        int j = a.sys_node[sys];
        int n = a.n_node ? a.n_node[j] : a.n;
        int deg = a.deg_node ? a.deg_node[j] : a.deg;
        int m = npoly(deg), s = n + m, lda = lda64_of(s), lda32 = lda32_of(s);
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        // FP32 coordinates live in the X area until the refinement needs it
        float2 *x32 = reinterpret_cast<float2 *>(X);
        for (int l = lane; l < n; l += 32) x32[l] = make_float2((float)xs[2 * l], (float)xs[2 * l + 1]);
        __syncwarp();
        assemble32_rows(A32, lda32, x32, n, m, deg, ops.p, lane);
        int ps[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) ps[k] = NOTYET;
        bool ok = warp_lu32_rows<NS>(A32, lda32, s, ps, perm, dinv32, prow, lane);
        bool fallback = !ok;
        if (ok) assemble64(A, lda, xs, n, m, deg, ops.p, lane);
        int64_t r0, r1;
        system_rows(a, sys, j, r0, r1);
        int iters_max = 0;
        for (int64_t t = r0; t < r1 && !fallback; t++) {
            int64_t row = row_id(a, t);
            double2 yp = eval_point(a, row);
            double yx = (yp.x - xc.x) * sx, yy = (yp.y - xc.y) * sy;
            build_rhs(ops, xs, n, m, yx, yy, sx, sy, 0, nullptr, B, lane);
            float e_prev = 1.0f;
            bool conv = false;
            int it;
            for (it = 0; it < a.max_refine; it++) {
                // residual of the current x (x = 0 at it 0) -> FP32
                if (it == 0) {
                    for (int e = lane; e < s * r; e += 32) R32[e] = (float)B[e];
                } else {
                    for (int e = lane; e < s * r; e += 32) {
                        int i = e / r, q = e - i * r;
                        const double *Ai = A + i * lda;
                        const double *Xq = X + q;
                        double acc = B[e];
                        int jmax = i < n ? s : n;  // the m x m block is zero
                        for (int jj = 0; jj < jmax; jj++) acc = fma(-Ai[jj], Xq[jj * r], acc);
                        R32[e] = (float)acc;
                    }
                }
                __syncwarp();
                warp_lu32_rows_solve<NS, RMAX>(A32, lda32, s, ps, perm, dinv32, R32, r, lane);
                // x += d; relative size of the correction over the weight rows (FP32 norms)
                float dmax = 0.0f, xmax = 0.0f;
                for (int e = lane; e < s * r; e += 32) {
                    float d = R32[e];
                    double xv = (it == 0 ? 0.0 : X[e]) + (double)d;
                    X[e] = xv;
                    if (e < n * r) {
                        dmax = fmaxf(dmax, fabsf(d));
                        xmax = fmaxf(xmax, fabsf((float)xv));
                    }
                }
                dmax = warp_max_f(dmax);
                xmax = warp_max_f(xmax);
                __syncwarp();
                float e_cur = xmax > 0.0f ? dmax / xmax : 0.0f;
                if (!(e_cur == e_cur) || isinf(e_cur)) break;  // NaN / inf
                if (it >= 1) {  // the contraction rho from two corrections, as in schur.cuh
                    float rho = e_prev > 0.0f ? e_cur / e_prev : 0.0f;
                    if (e_cur == 0.0f || (it >= 2 && (double)rho * (double)e_cur <= a.refine_tol)) {
                        conv = true;
                        break;
                    }
                    if (rho > 0.5f) break;  // stalled
                }
                e_prev = e_cur;
            }
            if (!conv) {
                fallback = true;
                break;
            }
            if (it > iters_max) iters_max = it;
            write_row(a, ops, row, X, n, sid, sx, sy, lane);
            __syncwarp();
        }
        if (lane == 0) {
            if (fallback) {
                int pos = atomicAdd(a.fallback_count, 1);
                a.fallback_list[pos] = (int32_t)sys;
            } else {
                atomicAdd(&a.hist[iters_max < 7 ? iters_max : 7], 1ull);
            }
        }
        __syncwarp();
    }
}

// Grid of a persistent launch: as many CTAs of wpb warps as fit on the GPU at once (fewer when
// there is less work).  wpb is lowered until wpb warps' shared memory fits a CTA.
template <typename K>
cudaError_t launch_persistent(K kernel, int &wpb, int num_sms, size_t per_warp, int64_t nwork, cudaStream_t st,
                              int *blocks_out, size_t *smem_out)
{
    int dev = 0, smem_cap = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (wpb < 1) wpb = 1;
    while (wpb > 1 && per_warp * wpb > (size_t)smem_cap) wpb--;
    if (per_warp * wpb > (size_t)smem_cap) return cudaErrorNotSupported;
    const size_t smem = per_warp * wpb;
    *smem_out = smem;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, wpb * 32, smem);
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int64_t want = (nwork + wpb - 1) / wpb;
    int64_t cap = (int64_t)num_sms * occ;
    *blocks_out = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    return cudaSuccess;
}

}  // namespace

size_t solve_fp64_smem_per_warp(int max_s, int max_n, int nops)
{
    return make_layout(max_s, max_n, nops, false).total;
}

size_t solve_mixed_smem_per_warp(int max_s, int max_n, int nops)
{
    return make_layout(max_s, max_n, nops, true).total;
}

static cudaError_t launch_fp64_impl(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms,
                                    cudaStream_t st, const int32_t *subset, const int *subset_count,
                                    int64_t nwork_hint)
{
    size_t smem = 0;
    int blocks = 0;
    cudaError_t e = launch_persistent(solve_fp64_kernel, wpb, num_sms, solve_fp64_smem_per_warp(a.max_s, a.max_n, ops.nops),
                                      nwork_hint, st, &blocks, &smem);
    if (e != cudaSuccess) return e;
    solve_fp64_kernel<<<blocks, wpb * 32, smem, st>>>(a, ops, subset, subset_count);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp64(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st)
{
    if (a.nsys <= 0) return cudaSuccess;
    return launch_fp64_impl(a, ops, wpb, num_sms, st, nullptr, nullptr, a.nsys);
}

cudaError_t launch_solve_fp64_subset(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms,
                                     cudaStream_t st, int64_t count)
{
    if (count <= 0) return cudaSuccess;
    return launch_fp64_impl(a, ops, wpb, num_sms, st, a.fallback_list, a.fallback_count, count);
}

template <int NS, int RMAX>
static cudaError_t launch_mixed_t(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st)
{
    size_t smem = 0;
    int blocks = 0;
    cudaError_t e = launch_persistent(solve_mixed_kernel<NS, RMAX>, wpb, num_sms,
                                      solve_mixed_smem_per_warp(a.max_s, a.max_n, ops.nops), a.nsys, st, &blocks, &smem);
    if (e != cudaSuccess) return e;
    solve_mixed_kernel<NS, RMAX><<<blocks, wpb * 32, smem, st>>>(a, ops);
    return cudaGetLastError();
}

cudaError_t launch_solve_mixed(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st)
{
    if (a.nsys <= 0) return cudaSuccess;
    int ns = (a.max_s + 31) / 32;
    int r = ops.nops;
    if (r <= 3) {
        switch (ns) {
        case 1: return launch_mixed_t<1, 3>(a, ops, wpb, num_sms, st);
        case 2: return launch_mixed_t<2, 3>(a, ops, wpb, num_sms, st);
        case 3: return launch_mixed_t<3, 3>(a, ops, wpb, num_sms, st);
        default: return launch_mixed_t<4, 3>(a, ops, wpb, num_sms, st);
        }
    }
    switch (ns) {
    case 1: return launch_mixed_t<1, RBFFD_MAX_OPS>(a, ops, wpb, num_sms, st);
    case 2: return launch_mixed_t<2, RBFFD_MAX_OPS>(a, ops, wpb, num_sms, st);
    case 3: return launch_mixed_t<3, RBFFD_MAX_OPS>(a, ops, wpb, num_sms, st);
    default: return launch_mixed_t<4, RBFFD_MAX_OPS>(a, ops, wpb, num_sms, st);
    }
}
