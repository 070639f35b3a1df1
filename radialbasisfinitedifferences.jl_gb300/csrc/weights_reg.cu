// Mixed-precision weight solves with the FP32 factorisation held in registers.
//
// One warp per local system of size s <= S (S a compile-time bound: 32, 40 or 64).  Lane l
// holds rows l and l + 32 of A32 = [Phi P; P' 0] in registers, so every column index of the
// LU and of the triangular solves is a compile-time register index: the elimination is a
// straight run of independent FMAs, and only the pivot row travels through shared memory
// (one broadcast LDS.128 per four columns).  Pivoting is virtual -- rows never move, ps[]
// records the step at which a row became the pivot -- which keeps every lane's rows in its
// own registers.
//
// The FP64 side keeps Phi and P (not the full saddle matrix) in shared memory for the
// residuals b - A x of the iterative refinement; the refinement, convergence test and
// FP64 fallback queue are those of the shared-memory mixed kernel in weights.cu.
#include <type_traits>

#include "solve_common.cuh"

namespace {

constexpr int PADROW = -1;

// Compile-time loop: f(std::integral_constant<int, I>) for I in [B, E).  Used where every
// iteration index must be a compile-time register index (a plain unrolled loop is not
// guaranteed to be unrolled when its body is large).
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F &&f)
{
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}  // pivot step of padding rows (i >= s): never a pivot, never updated

struct RegLayout {
    size_t phi, P, xs, x32, Pb, B, X, R32, dinv, perm, sid, prow, total;
};

__host__ __device__ inline int ldphi_of(int n) { return n | 1; }

__host__ __device__ inline RegLayout make_reg_layout(int S, int max_n, int max_m, int nops)
{
    RegLayout L;
    size_t o = 0;
    L.phi = o;  // also the stage of fill_rows (used before Phi64 is assembled)
    size_t phi_bytes = sizeof(double) * max_n * ldphi_of(max_n);
    size_t stage_bytes = sizeof(float) * 32 * 4 * (((S + 3) >> 2) | 1);
    o += al16(phi_bytes > stage_bytes ? phi_bytes : stage_bytes);
    L.P = o;
    o += al16(sizeof(double) * max_n * max_m);
    L.xs = o;
    o += al16(sizeof(double) * 2 * max_n);
    L.x32 = o;
    o += al16(sizeof(float2) * max_n);
    L.Pb = o;
    o += al16(sizeof(float) * max_n * max_m);
    L.B = o;
    o += al16(sizeof(double) * S * nops);
    L.X = o;
    o += al16(sizeof(double) * S * nops);
    L.R32 = o;
    o += al16(sizeof(float) * S * nops);
    L.dinv = o;
    o += al16(sizeof(float) * S);
    L.perm = o;
    o += al16(sizeof(int) * S);
    L.sid = o;
    o += al16(sizeof(int) * max_n);
    L.prow = o;
    o += al16(sizeof(float) * (S + 4));
    L.total = o;
    return L;
}

// Select a (c true) or b in one PTX instruction.  Written as inline PTX so the compiler
// cannot fold a chain of slot selects back into a dynamically indexed register array,
// which would move the whole register matrix to local memory.
__device__ __forceinline__ float sel_f32(bool c, float a, float b)
{
    float r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.s32 p, %3, 0;\n\tselp.f32 %0, %1, %2, p;\n\t}"
        : "=f"(r)
        : "f"(a), "f"(b), "r"((int)c));
    return r;
}

template <int S>
struct RegRows {
    static constexpr int NS = (S + 31) / 32;
    float a[NS][S];
    int ps[NS];
};

// Fill the register rows of A32 from FP32 coordinates (x32) and monomials (Pb, n x m).
// Each lane computes its row in a runtime loop into a private shared-memory stage (odd
// 16-byte stride), then loads it into registers with compile-time indices.
template <int S>
__device__ __forceinline__ void fill_rows(RegRows<S> &R, const float2 *x32, const float *Pb, float *stage, int n,
                                          int m, int p, int lane)
{
    constexpr int LD = 4 * (((S + 3) >> 2) | 1);
    int s = n + m;
    float *mine = stage + lane * LD;
    static_for<0, RegRows<S>::NS>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        int i = lane + 32 * k;
        R.ps[k] = i < s ? NOTYET : PADROW;
        if (i < n) {
            float2 xi = x32[i];
            for (int j = 0; j < n; j++) {
                float2 xj = x32[j];
                float dx = xi.x - xj.x, dy = xi.y - xj.y;
                mine[j] = phi32(fmaf(dx, dx, dy * dy), p);
            }
            for (int j = n; j < s; j++) mine[j] = Pb[i * m + (j - n)];
        } else if (i < s) {
            for (int j = 0; j < n; j++) mine[j] = Pb[j * m + (i - n)];
            for (int j = n; j < s; j++) mine[j] = 0.0f;
        } else {
            for (int j = 0; j < s; j++) mine[j] = 0.0f;
        }
        for (int j = s; j < LD; j++) mine[j] = 0.0f;
#pragma unroll
        for (int j4 = 0; j4 < (S + 3) / 4; j4++) {
            float4 v = reinterpret_cast<const float4 *>(mine)[j4];
            if (4 * j4 + 0 < S) R.a[k][4 * j4 + 0] = v.x;
            if (4 * j4 + 1 < S) R.a[k][4 * j4 + 1] = v.y;
            if (4 * j4 + 2 < S) R.a[k][4 * j4 + 2] = v.z;
            if (4 * j4 + 3 < S) R.a[k][4 * j4 + 3] = v.w;
        }
    });
}

// In-register LU with virtual partial pivoting.  perm[c] = pivot row of step c, dinv[c] =
// 1 / U[c][c] (shared memory).  Returns false (warp-uniform) on a zero / non-finite pivot.
template <int S>
__device__ __forceinline__ bool reg_lu(RegRows<S> &R, int s, int *perm, float *dinv, float *prow, int lane)
{
    constexpr int NS = RegRows<S>::NS;
    bool ok = true;
    static_for<0, S>([&](auto CC) {
        constexpr int c = decltype(CC)::value;
        if (c >= s || !ok) return;
        float best = -1.0f;
        int bi = INT_MAX;
#pragma unroll
        for (int k = 0; k < NS; k++) {
            if (R.ps[k] == NOTYET) {
                float v = fabsf(R.a[k][c]);
                if (v > best) {
                    best = v;
                    bi = lane + 32 * k;
                }
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            float ob = __shfl_xor_sync(RBFFD_FULL, best, o);
            int oi = __shfl_xor_sync(RBFFD_FULL, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (!(best > 0.0f) || isinf(best)) {
            ok = false;
            return;
        }
        // the owner lane publishes the pivot row, columns [c & ~3, S)
        if (lane == (bi & 31)) {
            int oslot = bi >> 5;
#pragma unroll
            for (int j4 = c >> 2; j4 < (S + 3) / 4; j4++) {
                float e[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    int j = 4 * j4 + u;
                    float v = 0.0f;
                    if (j < S) {
                        v = R.a[0][j];
#pragma unroll
                        for (int k = 1; k < NS; k++) v = sel_f32(oslot == k, R.a[k][j], v);
                    }
                    e[u] = v;
                }
                reinterpret_cast<float4 *>(prow)[j4] = make_float4(e[0], e[1], e[2], e[3]);
            }
        }
        if (lane == 0) perm[c] = bi;
#pragma unroll
        for (int k = 0; k < NS; k++)
            if (lane + 32 * k == bi) R.ps[k] = c;
        __syncwarp();
        float rinv = 1.0f / prow[c];
        if (lane == 0) dinv[c] = rinv;
        float l[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) {
            l[k] = R.ps[k] == NOTYET ? R.a[k][c] * rinv : 0.0f;
            if (R.ps[k] == NOTYET) R.a[k][c] = l[k];
        }
#pragma unroll
        for (int j4 = (c + 1) >> 2; j4 < (S + 3) / 4; j4++) {
            float4 pv = reinterpret_cast<const float4 *>(prow)[j4];
            float pj[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
            for (int u = 0; u < 4; u++) {
                int j = 4 * j4 + u;
                if (j > c && j < S) {
#pragma unroll
                    for (int k = 0; k < NS; k++) R.a[k][j] = fmaf(-l[k], pj[u], R.a[k][j]);
                }
            }
        }
        __syncwarp();
    });
    return ok;
}

// Solve with the register factors.  R32 (s x r floats, original row order) holds the
// right-hand sides on entry and the solution (by variable) on exit.
template <int S, int RMAX>
__device__ __forceinline__ void reg_solve(const RegRows<S> &R, int s, const int *perm, const float *dinv, float *R32,
                                          int r, int lane)
{
    constexpr int NS = RegRows<S>::NS;
    float b[NS][RMAX];
#pragma unroll
    for (int k = 0; k < NS; k++) {
        int i = lane + 32 * k;
#pragma unroll
        for (int q = 0; q < RMAX; q++) b[k][q] = (i < s && q < r) ? R32[i * r + q] : 0.0f;
    }
    __syncwarp();
    static_for<0, S>([&](auto CC) {
        constexpr int c = decltype(CC)::value;
        if (c >= s) return;
        int p = perm[c];
        int pl = p & 31, pk = p >> 5;
        float mult[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) mult[k] = R.ps[k] > c ? R.a[k][c] : 0.0f;
#pragma unroll
        for (int q = 0; q < RMAX; q++) {
            float v = b[0][q];
#pragma unroll
            for (int k = 1; k < NS; k++) v = sel_f32(pk == k, b[k][q], v);
            float y = __shfl_sync(RBFFD_FULL, v, pl);
#pragma unroll
            for (int k = 0; k < NS; k++) b[k][q] = fmaf(-mult[k], y, b[k][q]);
        }
    });
    static_for<0, S>([&](auto CC) {
        constexpr int c = S - 1 - decltype(CC)::value;
        if (c < s) {
            int p = perm[c];
            int pl = p & 31, pk = p >> 5;
            float dv = dinv[c];
            float mult[NS];
#pragma unroll
            for (int k = 0; k < NS; k++) mult[k] = (R.ps[k] < c && R.ps[k] >= 0) ? R.a[k][c] : 0.0f;
#pragma unroll
            for (int q = 0; q < RMAX; q++) {
                float v = b[0][q];
#pragma unroll
                for (int k = 1; k < NS; k++) v = sel_f32(pk == k, b[k][q], v);
                float x = __shfl_sync(RBFFD_FULL, v, pl) * dv;
                if (lane == 0 && q < r) R32[c * r + q] = x;
#pragma unroll
                for (int k = 0; k < NS; k++) b[k][q] = fmaf(-mult[k], x, b[k][q]);
            }
        }
    });
    __syncwarp();
}

template <int S, int RMAX>
__global__ void __launch_bounds__(128, 1) solve_mixed_reg_kernel(SolveArgs a, OpTable ops, int max_m)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    RegLayout L = make_reg_layout(S, a.max_n, max_m, ops.nops);
    unsigned char *base = smem_raw + (size_t)wib * L.total;
    double *phi = (double *)(base + L.phi);
    double *P = (double *)(base + L.P);
    double *xs = (double *)(base + L.xs);
    float2 *x32 = (float2 *)(base + L.x32);
    float *Pb = (float *)(base + L.Pb);
    double *B = (double *)(base + L.B);
    double *X = (double *)(base + L.X);
    float *R32 = (float *)(base + L.R32);
    float *dinv = (float *)(base + L.dinv);
    int *perm = (int *)(base + L.perm);
    int *sid = (int *)(base + L.sid);
    float *prow = (float *)(base + L.prow);
    const int r = ops.nops;

    int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sys = gw; sys < a.nsys; sys += nw) {
        int j = a.sys_node[sys];
        int n = a.n_node ? a.n_node[j] : a.n;
        int deg = a.deg_node ? a.deg_node[j] : a.deg;
        int m = npoly(deg), s = n + m, ldp = ldphi_of(n);
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        for (int l = lane; l < n; l += 32) {
            float2 v = make_float2((float)xs[2 * l], (float)xs[2 * l + 1]);
            x32[l] = v;
            monomial_row<float>(v.x, v.y, deg, Pb + l * m, 1);
        }
        __syncwarp();
        RegRows<S> R;
        fill_rows<S>(R, x32, Pb, (float *)phi, n, m, ops.p, lane);
        __syncwarp();
        bool ok = reg_lu<S>(R, s, perm, dinv, prow, lane);
        bool fallback = !ok;
        if (ok) {
            // FP64 Phi (upper triangle mirrored) and P for the residuals
            int npairs = n * (n - 1) / 2;
            for (int t = lane; t < npairs; t += 32) {
                int i, jj;
                tri_pair(t, n, i, jj);
                double dx = xs[2 * i] - xs[2 * jj], dy = xs[2 * i + 1] - xs[2 * jj + 1];
                double v = phi64(fma(dx, dx, dy * dy), ops.p);
                phi[i * ldp + jj] = v;
                phi[jj * ldp + i] = v;
            }
            for (int i = lane; i < n; i += 32) {
                phi[i * ldp + i] = 0.0;
                monomial_row<double>(xs[2 * i], xs[2 * i + 1], deg, P + i * m, 1);
            }
            __syncwarp();
        }
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
                if (it == 0) {
                    for (int e = lane; e < s * r; e += 32) R32[e] = (float)B[e];
                } else {
                    // r = b - A x in FP64, A = [Phi P; P' 0]
                    for (int e = lane; e < s * r; e += 32) {
                        int i = e / r, q = e - i * r;
                        double acc = B[e];
                        if (i < n) {
                            const double *Pi = phi + i * ldp;
                            for (int jj = 0; jj < n; jj++) acc = fma(-Pi[jj], X[jj * r + q], acc);
                            const double *Qi = P + i * m;
                            for (int l = 0; l < m; l++) acc = fma(-Qi[l], X[(n + l) * r + q], acc);
                        } else {
                            int l = i - n;
                            for (int jj = 0; jj < n; jj++) acc = fma(-P[jj * m + l], X[jj * r + q], acc);
                        }
                        R32[e] = (float)acc;
                    }
                }
                __syncwarp();
                reg_solve<S, RMAX>(R, s, perm, dinv, R32, r, lane);
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
                if (!(e_cur == e_cur) || isinf(e_cur)) break;
                if (it >= 1) {
                    float rho = e_prev > 0.0f ? e_cur / e_prev : 0.0f;
                    if ((double)rho * (double)e_cur <= a.refine_tol || e_cur == 0.0f) {
                        conv = true;
                        break;
                    }
                    if (rho > 0.5f) break;
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

template <int S, int RMAX>
cudaError_t launch_reg(const SolveArgs &a, const OpTable &ops, int max_m, int wpb, int num_sms, cudaStream_t st)
{
    size_t smem = make_reg_layout(S, a.max_n, max_m, ops.nops).total * wpb;
    auto kern = solve_mixed_reg_kernel<S, RMAX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, wpb * 32, smem);
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int64_t want = (a.nsys + wpb - 1) / wpb;
    int64_t cap = (int64_t)num_sms * occ;
    int blocks = (int)(want < cap ? want : cap);
    kern<<<blocks, wpb * 32, smem, st>>>(a, ops, max_m);
    return cudaGetLastError();
}

}  // namespace

size_t solve_mixed_reg_smem_per_warp(int S, int max_n, int max_m, int nops)
{
    return make_reg_layout(S, max_n, max_m, nops).total;
}

// Register-resident mixed solve for max_s <= 64 and nops <= 6; returns
// cudaErrorNotSupported for shapes it does not cover.
cudaError_t launch_solve_mixed_reg(const SolveArgs &a, const OpTable &ops, int max_m, int wpb, int num_sms,
                                   cudaStream_t st)
{
    if (a.nsys <= 0) return cudaSuccess;
    int r = ops.nops;
    if (r > 6 || a.max_s > 64 || a.unscaled_overload) return cudaErrorNotSupported;
    if (wpb > 4) wpb = 4;
    if (a.max_s <= 32) return r <= 3 ? launch_reg<32, 3>(a, ops, max_m, wpb, num_sms, st)
                                     : launch_reg<32, 6>(a, ops, max_m, wpb, num_sms, st);
    if (a.max_s <= 40) return r <= 3 ? launch_reg<40, 3>(a, ops, max_m, wpb, num_sms, st)
                                     : launch_reg<40, 6>(a, ops, max_m, wpb, num_sms, st);
    return r <= 3 ? launch_reg<64, 3>(a, ops, max_m, wpb, num_sms, st)
                  : launch_reg<64, 6>(a, ops, max_m, wpb, num_sms, st);
}
