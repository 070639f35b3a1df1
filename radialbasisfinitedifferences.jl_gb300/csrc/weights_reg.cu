// Mixed-precision weight solves: FP32 preconditioner from the Schur complement of the
// saddle system, FP64 residuals, iterative refinement.
//
// The local system is A = [Phi P; P' 0] (n stencil nodes, m monomials).  Its FP32
// preconditioner is built without ever factoring the (n+m)-row matrix:
//   1. Phi^-1 by in-place Gauss-Jordan in registers -- lane l holds Phi rows l (and l+32),
//      so every column index is a compile-time register index and an elimination step is a
//      straight run of independent FMAs (only the pivot row goes through shared memory);
//   2. G = Phi^-1 P (n x m) and the Schur complement S = -P' G (m x m), inverted the same way;
//   3. a correction A^-1 r = [w; lambda] is applied as five small dependency-free matvecs:
//      t = Phi^-1 r1, lambda = S^-1 (r2 - P' t), w = Phi^-1 (r1 - P lambda).
// Compared with factoring the whole system this needs one register row per lane for
// n <= 32 (a third of the FMAs and registers), which raises occupancy.  The FP64 side keeps
// Phi and P in shared memory for the residuals b - A x; refinement, convergence test and the
// FP64 fallback queue are those of the shared-memory mixed kernel in weights.cu.
//
// Pivoting is virtual: rows never move; ps[i] records the step at which row i was the pivot
// and perm[c] the pivot row of step c.  The Gauss-Jordan result B then satisfies
// B[perm[c]][j] = inv(M)[c][perm[j]], so x = inv(M) b is x[ps[i]] = B[i] . b' with
// b'_j = b[perm[j]].
#include <type_traits>

#include "solve_common.cuh"

namespace {

constexpr int PADROW = -1;  // pivot step of padding rows: never a pivot, never updated
constexpr int SMAX = 32;    // Schur complement rows (monomials) handled in registers

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

template <int S>
__host__ __device__ constexpr int stage_ld()
{
    return 4 * (((S + 3) >> 2) | 1);  // odd number of 16-byte groups: conflict-free LDS.128
}

// Per-warp shared-memory carve-up.
struct RegLayout {
    size_t phi, P, xs, x32, P32, Pp, G, Sm, B, X, R32, T, U, Lam, V, bp, dinvP, permP, dinvS, permS, sid, prow,
        total;
};

__host__ __device__ inline int ldphi_of(int n) { return n | 1; }

__host__ __device__ inline RegLayout make_reg_layout(int SP, int max_n, int max_m, int nops)
{
    RegLayout L;
    size_t o = 0;
    int n4 = (max_n + 3) & ~3, s = max_n + max_m, rq = (nops + 3) / 4;
    L.phi = o;  // also the staging area of the register fills (used before Phi64 exists)
    size_t phi_bytes = sizeof(double) * max_n * ldphi_of(max_n);
    size_t stage_bytes = sizeof(float) * 32 * 4 * (((SP + 3) >> 2) | 1);
    size_t stage2 = sizeof(float) * 32 * 4 * (((SMAX + 3) >> 2) | 1);
    if (stage2 > stage_bytes) stage_bytes = stage2;
    o += al16(phi_bytes > stage_bytes ? phi_bytes : stage_bytes);
    L.P = o;
    o += al16(sizeof(double) * max_n * max_m);
    L.xs = o;
    o += al16(sizeof(double) * 2 * max_n);
    L.x32 = o;
    o += al16(sizeof(float2) * max_n);
    L.P32 = o;
    o += al16(sizeof(float) * max_n * max_m);
    L.Pp = o;
    o += al16(sizeof(float) * max_m * n4);
    L.G = o;
    o += al16(sizeof(float) * max_n * max_m);
    L.Sm = o;
    o += al16(sizeof(float) * max_m * max_m);
    L.B = o;
    o += al16(sizeof(double) * s * nops);
    L.X = o;
    o += al16(sizeof(double) * s * nops);
    L.R32 = o;
    o += al16(sizeof(float) * s * nops);
    L.T = o;
    o += al16(sizeof(float) * max_n * nops);
    L.U = o;
    o += al16(sizeof(float) * max_m * nops);
    L.Lam = o;
    o += al16(sizeof(float) * max_m * nops);
    L.V = o;
    o += al16(sizeof(float) * max_n * nops);
    L.bp = o;
    o += al16(sizeof(float4) * (SP > SMAX ? SP : SMAX) * rq);
    L.dinvP = o;
    o += al16(sizeof(float) * SP);
    L.permP = o;
    o += al16(sizeof(int) * SP);
    L.dinvS = o;
    o += al16(sizeof(float) * SMAX);
    L.permS = o;
    o += al16(sizeof(int) * SMAX);
    L.sid = o;
    o += al16(sizeof(int) * max_n);
    L.prow = o;
    o += al16(sizeof(float) * ((SP > SMAX ? SP : SMAX) + 4));
    L.total = o;
    return L;
}

// Load register rows (rows < nrows real) from a per-lane stage written by `row_fn`, which
// fills columns [0, ncols) of row i and must zero nothing (padding is handled here).
template <int S, typename Fn>
__device__ __forceinline__ void load_rows(RegRows<S> &R, float *stage, int nrows, int ncols, int lane, Fn &&row_fn)
{
    constexpr int LD = stage_ld<S>();
    float *mine = stage + lane * LD;
    static_for<0, RegRows<S>::NS>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        int i = lane + 32 * k;
        R.ps[k] = i < nrows ? NOTYET : PADROW;
        if (i < nrows) row_fn(i, mine);
        for (int j = (i < nrows ? ncols : 0); j < LD; j++) mine[j] = 0.0f;
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

// In-place Gauss-Jordan inversion of the s x s leading block in registers, virtual partial
// pivoting.  Step c picks the pivot among rows not yet used (largest |a[c]|, lowest row on
// ties: one redux.sync max over the |a| bit patterns, one redux.sync min over row ids),
// publishes it through shared memory and eliminates column c from every other row.  A pivot
// row is kept multiplied by its pivot (the elimination is linear, so later updates apply
// unchanged) and divided by it once at the end, so each step is a uniform FMA sweep.
template <int S>
__device__ __forceinline__ bool reg_gj(RegRows<S> &R, int s, int *perm, float *dinv, float *prow, int lane)
{
    constexpr int NS = RegRows<S>::NS;
    bool ok = true;
    static_for<0, S>([&](auto CC) {
        constexpr int c = decltype(CC)::value;
        if (c >= s || !ok) return;
        unsigned key = 0u;
        int brow = INT_MAX;
#pragma unroll
        for (int k = 0; k < NS; k++) {
            unsigned kk = (unsigned)__float_as_int(fabsf(R.a[k][c]));
            if (R.ps[k] == NOTYET && kk > key) {
                key = kk;
                brow = lane + 32 * k;
            }
        }
        unsigned m = __reduce_max_sync(RBFFD_FULL, key);
        if (m == 0u || m >= 0x7f800000u) {  // zero, inf or NaN pivot
            ok = false;
            return;
        }
        int bi = (int)__reduce_min_sync(RBFFD_FULL, (unsigned)(key == m ? brow : INT_MAX));
        if (lane == (bi & 31)) {
            int oslot = bi >> 5;
#pragma unroll
            for (int j4 = 0; j4 < (S + 3) / 4; j4++) {
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
        __syncwarp();
        float inv = 1.0f / prow[c];
        if (lane == 0) dinv[c] = inv;
        float fs[NS];
        bool piv[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) {
            piv[k] = (lane + 32 * k == bi);
            bool elim = R.ps[k] != PADROW && !piv[k];
            fs[k] = elim ? R.a[k][c] * inv : 0.0f;
            if (piv[k]) R.ps[k] = c;
        }
#pragma unroll
        for (int j4 = 0; j4 < (S + 3) / 4; j4++) {
            float4 pv = reinterpret_cast<const float4 *>(prow)[j4];
            float pj[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
            for (int u = 0; u < 4; u++) {
                int j = 4 * j4 + u;
                if (j < S && j != c) {
#pragma unroll
                    for (int k = 0; k < NS; k++) R.a[k][j] = fmaf(-fs[k], pj[u], R.a[k][j]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NS; k++) {
            float nc = piv[k] ? 1.0f : -fs[k];
            if (R.ps[k] != PADROW) R.a[k][c] = nc;
        }
        __syncwarp();
    });
    if (ok) {
#pragma unroll
        for (int k = 0; k < NS; k++) {
            float d = (R.ps[k] >= 0 && R.ps[k] < s) ? dinv[R.ps[k]] : 0.0f;
#pragma unroll
            for (int j = 0; j < S; j++) R.a[k][j] *= d;
        }
    }
    return ok;
}

// out[ps[i]][q] = B[i] . in[perm[.]][q] for q < r: x = inv(M) b with the Gauss-Jordan
// result B (s x s).  in/out are s x r floats (row-major); bp is scratch (s x RQ float4).
template <int S, int RMAX>
__device__ __forceinline__ void reg_apply(const RegRows<S> &R, int s, const int *perm, const float *in, float *out,
                                          float4 *bp, int r, int lane)
{
    constexpr int NS = RegRows<S>::NS;
    constexpr int RQ = (RMAX + 3) / 4;
    for (int t = lane; t < s * RQ; t += 32) {
        int j = t / RQ, g = t - j * RQ;
        const float *src = in + perm[j] * r;
        float e[4];
#pragma unroll
        for (int u = 0; u < 4; u++) e[u] = (4 * g + u < r) ? src[4 * g + u] : 0.0f;
        bp[t] = make_float4(e[0], e[1], e[2], e[3]);
    }
    __syncwarp();
    float acc[NS][4 * RQ];
#pragma unroll
    for (int k = 0; k < NS; k++)
#pragma unroll
        for (int q = 0; q < 4 * RQ; q++) acc[k][q] = 0.0f;
#pragma unroll
    for (int j = 0; j < S; j++) {
        if (j < s) {
#pragma unroll
            for (int g = 0; g < RQ; g++) {
                float4 v = bp[j * RQ + g];
#pragma unroll
                for (int k = 0; k < NS; k++) {
                    acc[k][4 * g + 0] = fmaf(R.a[k][j], v.x, acc[k][4 * g + 0]);
                    acc[k][4 * g + 1] = fmaf(R.a[k][j], v.y, acc[k][4 * g + 1]);
                    acc[k][4 * g + 2] = fmaf(R.a[k][j], v.z, acc[k][4 * g + 2]);
                    acc[k][4 * g + 3] = fmaf(R.a[k][j], v.w, acc[k][4 * g + 3]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NS; k++) {
        int v = R.ps[k];
        if (v >= 0 && v < s) {
#pragma unroll
            for (int q = 0; q < RMAX; q++)
                if (q < r) out[v * r + q] = acc[k][q];
        }
    }
    __syncwarp();
}

// Correction x = inv(A) rr for A = [Phi P; P' 0] via the Schur complement; rr (s x r)
// in, x (s x r, by variable) out -- may alias.
template <int SP, int RMAX>
__device__ __forceinline__ void schur_apply(const RegRows<SP> &RP, const RegRows<SMAX> &RS, int n, int m, int r,
                                            const int *permP, const int *permS, const float *P32, const float *rr,
                                            float *x, float *T, float *U, float *Lam, float *V, float4 *bp, int lane)
{
    reg_apply<SP, RMAX>(RP, n, permP, rr, T, bp, r, lane);  // t = Phi^-1 r1
    for (int e = lane; e < m * r; e += 32) {                  // u = r2 - P' t
        int l = e / r, q = e - l * r;
        float acc = rr[(n + l) * r + q];
        for (int i = 0; i < n; i++) acc = fmaf(-P32[i * m + l], T[i * r + q], acc);
        U[e] = acc;
    }
    __syncwarp();
    reg_apply<SMAX, RMAX>(RS, m, permS, U, Lam, bp, r, lane);  // lambda = S^-1 u
    for (int e = lane; e < n * r; e += 32) {                     // v = r1 - P lambda
        int i = e / r, q = e - i * r;
        float acc = rr[e];
        for (int l = 0; l < m; l++) acc = fmaf(-P32[i * m + l], Lam[l * r + q], acc);
        V[e] = acc;
    }
    __syncwarp();
    reg_apply<SP, RMAX>(RP, n, permP, V, x, bp, r, lane);  // w = Phi^-1 v
    for (int e = lane; e < m * r; e += 32) x[n * r + e] = Lam[e];
    __syncwarp();
}

// One element (i, q) of r = b - A x, A = [Phi P; P' 0], as four partial sums.
__device__ __forceinline__ double residual_elem(const double *phi, int ldp, const double *P, int n, int m, int r,
                                                const double *B, const double *X, int e)
{
    int i = e / r, q = e - i * r;
    double a0 = B[e], a1 = 0.0, a2 = 0.0, a3 = 0.0;
    const double *Xq = X + q;
    if (i < n) {
        const double *Pi = phi + i * ldp;
        int jj = 0;
        for (; jj + 4 <= n; jj += 4) {
            a0 = fma(-Pi[jj], Xq[jj * r], a0);
            a1 = fma(-Pi[jj + 1], Xq[(jj + 1) * r], a1);
            a2 = fma(-Pi[jj + 2], Xq[(jj + 2) * r], a2);
            a3 = fma(-Pi[jj + 3], Xq[(jj + 3) * r], a3);
        }
        for (; jj < n; jj++) a0 = fma(-Pi[jj], Xq[jj * r], a0);
        const double *Qi = P + i * m;
        const double *Xl = Xq + n * r;
        int l = 0;
        for (; l + 2 <= m; l += 2) {
            a1 = fma(-Qi[l], Xl[l * r], a1);
            a2 = fma(-Qi[l + 1], Xl[(l + 1) * r], a2);
        }
        for (; l < m; l++) a3 = fma(-Qi[l], Xl[l * r], a3);
    } else {
        int l = i - n;
        int jj = 0;
        for (; jj + 4 <= n; jj += 4) {
            a0 = fma(-P[jj * m + l], Xq[jj * r], a0);
            a1 = fma(-P[(jj + 1) * m + l], Xq[(jj + 1) * r], a1);
            a2 = fma(-P[(jj + 2) * m + l], Xq[(jj + 2) * r], a2);
            a3 = fma(-P[(jj + 3) * m + l], Xq[(jj + 3) * r], a3);
        }
        for (; jj < n; jj++) a0 = fma(-P[jj * m + l], Xq[jj * r], a0);
    }
    return (a0 + a1) + (a2 + a3);
}

// FP64 residual r = b - A x -> FP32; two elements per lane for eight independent chains.
__device__ __forceinline__ void residual64(const double *phi, int ldp, const double *P, int n, int m, int r,
                                           const double *B, const double *X, float *R32, int lane)
{
    int tot = (n + m) * r;
    for (int e = lane; e < tot; e += 64) {
        int e2 = e + 32;
        double v1 = residual_elem(phi, ldp, P, n, m, r, B, X, e);
        double v2 = e2 < tot ? residual_elem(phi, ldp, P, n, m, r, B, X, e2) : 0.0;
        R32[e] = (float)v1;
        if (e2 < tot) R32[e2] = (float)v2;
    }
    __syncwarp();
}

template <int SP, int RMAX>
__global__ void __launch_bounds__(128, 1) solve_mixed_schur_kernel(SolveArgs a, OpTable ops)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int max_m = a.max_m;
    RegLayout L = make_reg_layout(SP, a.max_n, max_m, ops.nops);
    unsigned char *base = smem_raw + (size_t)wib * L.total;
    double *phi = (double *)(base + L.phi);
    double *P = (double *)(base + L.P);
    double *xs = (double *)(base + L.xs);
    float2 *x32 = (float2 *)(base + L.x32);
    float *P32 = (float *)(base + L.P32);
    float *Pp = (float *)(base + L.Pp);
    float *G = (float *)(base + L.G);
    float *Sm = (float *)(base + L.Sm);
    double *B = (double *)(base + L.B);
    double *X = (double *)(base + L.X);
    float *R32 = (float *)(base + L.R32);
    float *T = (float *)(base + L.T);
    float *U = (float *)(base + L.U);
    float *Lam = (float *)(base + L.Lam);
    float *V = (float *)(base + L.V);
    float4 *bp = (float4 *)(base + L.bp);
    float *dinvP = (float *)(base + L.dinvP);
    int *permP = (int *)(base + L.permP);
    float *dinvS = (float *)(base + L.dinvS);
    int *permS = (int *)(base + L.permS);
    int *sid = (int *)(base + L.sid);
    float *prow = (float *)(base + L.prow);
    float *stage = (float *)phi;
    const int r = ops.nops;

    int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sys = gw; sys < a.nsys; sys += nw) {
        int j = a.sys_node[sys];
        int n = a.n_node ? a.n_node[j] : a.n;
        int deg = a.deg_node ? a.deg_node[j] : a.deg;
        int m = npoly(deg), s = n + m, ldp = ldphi_of(n), n4 = (n + 3) & ~3;
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        for (int l = lane; l < n; l += 32) {
            float2 v = make_float2((float)xs[2 * l], (float)xs[2 * l + 1]);
            x32[l] = v;
            monomial_row<float>(v.x, v.y, deg, P32 + l * m, 1);
        }
        __syncwarp();
        // (1) Phi^-1 in registers
        RegRows<SP> RP;
        const int p = ops.p;
        load_rows<SP>(RP, stage, n, n, lane, [&](int i, float *row) {
            float2 xi = x32[i];
            for (int jj = 0; jj < n; jj++) {
                float2 xj = x32[jj];
                float dx = xi.x - xj.x, dy = xi.y - xj.y;
                row[jj] = phi32(fmaf(dx, dx, dy * dy), p);
            }
        });
        __syncwarp();
        bool ok = reg_gj<SP>(RP, n, permP, dinvP, prow, lane);
        RegRows<SMAX> RS;
        if (ok) {
            // (2) G = Phi^-1 P, S = -P' G
            for (int t = lane; t < m * n4; t += 32) {
                int l = t / n4, jj = t - l * n4;
                Pp[t] = jj < n ? P32[permP[jj] * m + l] : 0.0f;
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < RegRows<SP>::NS; k++) {
                int v = RP.ps[k];
                for (int l = 0; l < m; l++) {
                    const float4 *pl = reinterpret_cast<const float4 *>(Pp + l * n4);
                    float acc = 0.0f;
#pragma unroll
                    for (int j4 = 0; j4 < SP / 4; j4++) {
                        if (4 * j4 < n) {
                            float4 w = pl[j4];
                            acc = fmaf(RP.a[k][4 * j4 + 0], w.x, acc);
                            acc = fmaf(RP.a[k][4 * j4 + 1], w.y, acc);
                            acc = fmaf(RP.a[k][4 * j4 + 2], w.z, acc);
                            acc = fmaf(RP.a[k][4 * j4 + 3], w.w, acc);
                        }
                    }
                    if (v >= 0 && v < n) G[v * m + l] = acc;
                }
            }
            __syncwarp();
            for (int t = lane; t < m * m; t += 32) {
                int aa = t / m, bb = t - aa * m;
                float acc = 0.0f;
                for (int i = 0; i < n; i++) acc = fmaf(P32[i * m + aa], G[i * m + bb], acc);
                Sm[t] = -acc;
            }
            __syncwarp();
            load_rows<SMAX>(RS, stage, m, m, lane, [&](int i, float *row) {
                for (int jj = 0; jj < m; jj++) row[jj] = Sm[i * m + jj];
            });
            __syncwarp();
            ok = reg_gj<SMAX>(RS, m, permS, dinvS, prow, lane);
        }
        bool fallback = !ok;
        if (ok) {
            // FP64 Phi (upper triangle mirrored) and P for the residuals
            int npairs = n * (n - 1) / 2;
            for (int t = lane; t < npairs; t += 64) {
                int i, jj, i2 = 0, j2 = 1;
                tri_pair(t, n, i, jj);
                bool two = t + 32 < npairs;
                if (two) tri_pair(t + 32, n, i2, j2);
                double dx = xs[2 * i] - xs[2 * jj], dy = xs[2 * i + 1] - xs[2 * jj + 1];
                double dx2 = xs[2 * i2] - xs[2 * j2], dy2 = xs[2 * i2 + 1] - xs[2 * j2 + 1];
                double v = phi64(fma(dx, dx, dy * dy), p);
                double v2 = phi64(fma(dx2, dx2, dy2 * dy2), p);
                phi[i * ldp + jj] = v;
                phi[jj * ldp + i] = v;
                if (two) {
                    phi[i2 * ldp + j2] = v2;
                    phi[j2 * ldp + i2] = v2;
                }
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
                    __syncwarp();
                } else {
                    residual64(phi, ldp, P, n, m, r, B, X, R32, lane);
                }
                schur_apply<SP, RMAX>(RP, RS, n, m, r, permP, permS, P32, R32, R32, T, U, Lam, V, bp, lane);
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

template <int SP, int RMAX>
cudaError_t launch_schur(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st)
{
    size_t per_warp = make_reg_layout(SP, a.max_n, a.max_m, ops.nops).total;
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    while (wpb > 1 && per_warp * wpb > (size_t)smem_max) wpb--;
    if (per_warp * wpb > (size_t)smem_max) return cudaErrorNotSupported;
    size_t smem = per_warp * wpb;
    auto kern = solve_mixed_schur_kernel<SP, RMAX>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, wpb * 32, smem);
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int64_t want = (a.nsys + wpb - 1) / wpb;
    int64_t cap = (int64_t)num_sms * occ;
    int blocks = (int)(want < cap ? want : cap);
    kern<<<blocks, wpb * 32, smem, st>>>(a, ops);
    return cudaGetLastError();
}

}  // namespace

size_t solve_mixed_reg_smem_per_warp(int S, int max_n, int max_m, int nops)
{
    return make_reg_layout(S, max_n, max_m, nops).total;
}

// Schur-complement mixed solve for stencils of at most 64 nodes, at most 32 monomials and at
// most 6 operators; returns cudaErrorNotSupported for other shapes.
cudaError_t launch_solve_mixed_reg(const SolveArgs &a, const OpTable &ops, int max_m, int wpb, int num_sms,
                                   cudaStream_t st)
{
    (void)max_m;
    if (a.nsys <= 0) return cudaSuccess;
    int r = ops.nops;
    if (r > 6 || a.max_n > 64 || a.max_m > SMAX || a.unscaled_overload) return cudaErrorNotSupported;
    if (wpb > 4) wpb = 4;
    if (a.max_n <= 32) return r <= 4 ? launch_schur<32, 4>(a, ops, wpb, num_sms, st)
                                     : launch_schur<32, 8>(a, ops, wpb, num_sms, st);
    return r <= 4 ? launch_schur<64, 4>(a, ops, wpb, num_sms, st) : launch_schur<64, 8>(a, ops, wpb, num_sms, st);
}
