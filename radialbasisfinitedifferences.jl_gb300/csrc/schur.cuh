// Mixed-precision weight solves: FP32 preconditioner built from the Schur complement of the
// saddle system, an FP64 first residual, iterative refinement.  One warp per local system.
//
// The local system of src/generate_operator.jl (rbfblock/polynomialblock) is
//   A = [Phi P; P' 0],  Phi_ij = phi(|x_i - x_j|) (n x n),  P_il = monomial l at x_i (n x m).
// Its FP32 inverse is never formed.  The kernel keeps
//   * Phi^-1 in registers: lane l holds the Gauss-Jordan result for row l (and l + 32), so an
//     elimination step is a run of independent FMAs on compile-time register indices and only
//     the pivot row travels through shared memory;
//   * G = Phi^-1 P (n x m) and Sinv = S^-1, S = -P' G (m x m), in shared memory.
// A correction A^-1 [r1; r2] = [w; lambda] is then
//   lambda = Sinv (r2 - G' r1),   w = Phi^-1 r1 - G lambda,
// i.e. one register matvec plus three short shared-memory matvecs.  Refinement x += A^-1 (b - A x)
// keeps Phi (packed as its lower triangle) and P in FP64; the pairwise Phi = r^p comes from exact
// fixed-point integer arithmetic (phi_fixed.cuh).  The first residual b - A x0 is formed with
// FP64 products; from then on x and the residual are double-float pairs and each new residual
// r - A d is a double-float FP32 dot product.  Refinement stops when the estimated relative
// error of the weights rho * |dx| / |x| is below refine_tol; a system that stalls (rho > 1/2),
// meets a zero pivot or produces a non-finite value goes to the FP64 fallback queue, as in the
// shared-memory mixed kernel of weights.cu.  Warps claim systems from a counter.
//
// FP64 instructions are the scarce resource (1/64 of the FP32 rate), so every FP64 instruction
// works on lane-parallel data, conversions between float and double use the integer pipe, and
// maxima and comparisons use integer keys.
//
// Pivoting is virtual: rows never move.  ps[i] is the step at which row i was the pivot and
// perm[c] the pivot row of step c; the Gauss-Jordan result B then satisfies
// inv(M)[ps[i]][perm[j]] = B[i][j].
#pragma once

#include <type_traits>

#include "solve_common.cuh"
#include "phi_fixed.cuh"

namespace {

constexpr int PADROW = -1;  // pivot step of padding rows: never a pivot, never updated

// Register budget: 16 resident warps per SM for stencils of <= 32 nodes (<= 128 registers per
// thread) and 8 for larger ones (the 2 x 48 or 2 x 64 register-resident Phi^-1 entries of a
// lane need up to 255).  A CTA may hold all of an SM's warps (512 or 256 threads).
#define RBFFD_SCHUR_MAX_THREADS(SP) ((SP) <= 32 ? 512 : 256)

// Compile-time loop: f(std::integral_constant<int, I>) for I in [B, E).
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F &&f)
{
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// Select a (c true) or b in one PTX instruction, so that a chain of slot selects is not folded
// back into a dynamically indexed register array (which would live in local memory).
__device__ __forceinline__ float sel_f32(bool c, float a, float b)
{
    float r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.s32 p, %3, 0;\n\tselp.f32 %0, %1, %2, p;\n\t}"
        : "=f"(r)
        : "f"(a), "f"(b), "r"((int)c));
    return r;
}

// floor(t / d) for 0 <= t < 2^12 and 1 <= d <= 128 by a multiply and a shift, g = div19_magic(d)
// = ceil(2^19 / d) (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994: 19 = 12 + ceil(log2 d) bits make the quotient exact), instead of
// the instruction sequence of a run-time integer division.
__host__ __device__ inline uint32_t div19_magic(int d) { return (524288u + (uint32_t)d - 1u) / (uint32_t)d; }
__device__ __forceinline__ int div19(int t, uint32_t g) { return (int)(((uint32_t)t * g) >> 19); }

template <int S>
struct RegRows {
    static constexpr int NS = (S + 31) / 32;
    float a[NS][S];
    int ps[NS];
};

// Per-warp shared-memory carve-up.  The setup-only arrays (x32, P32, Pp, Sm) share storage
// with the refinement arrays (B, X, R32, U, Lam, bp).
struct SchurLayout {
    size_t phi, P, xs, sid, G, Sinv, permP, dinvP, permS, dinvS, prow, sc;
    size_t x32, P32, Pp, Sm;
    size_t B, X, R32, U, Lam, bp;
    size_t total;
    int ldg, lds;
};

__host__ __device__ inline SchurLayout make_schur_layout(int SP, int SM, int max_n, int max_m, int nops)
{
    SchurLayout L;
    const int n4 = (max_n + 3) & ~3, s = max_n + max_m, rq = (nops + 3) / 4;
    const int wmax = SP > SM ? SP : SM;
    L.ldg = max_m | 1;
    L.lds = max_m | 1;
    size_t o = 0;
    L.phi = o;
    o += al16(sizeof(double) * (size_t)max_n * (max_n + 1) / 2);
    L.P = o;
    o += al16(sizeof(double) * max_n * max_m);
    L.xs = o;
    o += al16(sizeof(double) * 2 * max_n);
    L.sid = o;
    o += al16(sizeof(int) * max_n);
    L.G = o;
    o += al16(sizeof(float) * max_n * L.ldg);
    L.Sinv = o;
    o += al16(sizeof(float) * max_m * L.lds);
    L.permP = o;
    o += al16(sizeof(int) * SP);
    L.dinvP = o;
    o += al16(sizeof(float) * SP);
    L.permS = o;
    o += al16(sizeof(int) * SM);
    L.dinvS = o;
    o += al16(sizeof(float) * SM);
    L.prow = o;
    o += al16(sizeof(float) * (wmax + 4));
    L.sc = o;
    o += al16(sizeof(double) * (2 * nops + 2));
    // union: setup arrays
    size_t u = o;
    L.x32 = u;
    u += al16(sizeof(float2) * max_n);
    L.P32 = u;
    u += al16(sizeof(float) * max_n * max_m);
    L.Pp = u;
    u += al16(sizeof(float) * max_m * n4);
    L.Sm = u;
    u += al16(sizeof(float) * max_m * max_m);
    // the fixed-point coordinates of the Phi assembly (after the setup arrays are dead)
    if (u < L.x32 + al16(sizeof(longlong2) * max_n)) u = L.x32 + al16(sizeof(longlong2) * max_n);
    // union: refinement arrays
    size_t v = o;
    L.B = v;
    v += al16(sizeof(double) * s * nops);
    L.X = v;
    v += al16(sizeof(double) * s * nops);
    L.R32 = v;
    v += al16(sizeof(float) * s * nops);
    L.U = v;
    v += al16(sizeof(float) * max_m * nops);
    L.Lam = v;
    v += al16(sizeof(float4) * max_m * rq);
    L.bp = v;
    v += al16(sizeof(float4) * max_n * rq);
    L.total = u > v ? u : v;
    return L;
}

// Phi rows in FP32 straight into registers: row i = lane + 32 k, column j compile-time.
template <int SP>
__device__ __forceinline__ void fill_phi_rows(RegRows<SP> &R, const float2 *x32, int n, int p, int lane)
{
    static_for<0, RegRows<SP>::NS>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        const int i = lane + 32 * k;
        const bool act = i < n;
        R.ps[k] = act ? NOTYET : PADROW;
        float2 xi = x32[act ? i : 0];
        static_for<0, SP>([&](auto JJ) {
            constexpr int j = decltype(JJ)::value;
            float v = 0.0f;
            if (j < n) {
                float2 xj = x32[j];
                float dx = xi.x - xj.x, dy = xi.y - xj.y;
                v = act ? phi32(fmaf(dx, dx, dy * dy), p) : 0.0f;
            }
            R.a[k][j] = v;
        });
    });
}

// In-place Gauss-Jordan inversion of the s x s leading block in registers with virtual partial
// pivoting.  Step c picks the pivot among rows not yet used (largest |a[c]|, lowest row on
// ties: a redux.sync max over the |a| bit patterns, then a redux.sync min over row ids),
// publishes it through shared memory and eliminates column c from every other row.  A pivot
// row stays multiplied by its pivot (elimination is linear, so later updates apply unchanged)
// and is divided by it once at the end, so each step is a uniform FMA sweep.  Fails on a
// zero, subnormal, infinite or NaN pivot.
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
            unsigned kk = __float_as_uint(R.a[k][c]) & 0x7fffffffu;
            if (R.ps[k] == NOTYET && kk > key) {
                key = kk;
                brow = lane + 32 * k;
            }
        }
        unsigned mk = __reduce_max_sync(RBFFD_FULL, key);
        if (mk < 0x00800000u || mk >= 0x7f800000u) {
            ok = false;
            return;
        }
        int bi = (int)__reduce_min_sync(RBFFD_FULL, (unsigned)(key == mk ? brow : INT_MAX));
        if (lane == (bi & 31)) {
            const int oslot = bi >> 5;
#pragma unroll
            for (int j4 = 0; j4 < (S + 3) / 4; j4++) {
                float e[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int j = 4 * j4 + u;
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
        const float inv = __fdividef(1.0f, prow[c]);
        if (lane == 0) dinv[c] = inv;
        float fs[NS];
        bool piv[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) {
            piv[k] = (lane + 32 * k == bi);
            const bool elim = R.ps[k] != PADROW && !piv[k];
            fs[k] = elim ? R.a[k][c] * inv : 0.0f;
            if (piv[k]) R.ps[k] = c;
        }
#pragma unroll
        for (int j4 = 0; j4 < (S + 3) / 4; j4++) {
            const float4 pv = reinterpret_cast<const float4 *>(prow)[j4];
            const float pj[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int j = 4 * j4 + u;
                if (j < S && j != c) {
#pragma unroll
                    for (int k = 0; k < NS; k++) R.a[k][j] = fmaf(-fs[k], pj[u], R.a[k][j]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NS; k++) {
            if (R.ps[k] != PADROW) R.a[k][c] = piv[k] ? 1.0f : -fs[k];
        }
        __syncwarp();
    });
    if (ok) {
#pragma unroll
        for (int k = 0; k < NS; k++) {
            const float d = (R.ps[k] >= 0 && R.ps[k] < s) ? dinv[R.ps[k]] : 0.0f;
#pragma unroll
            for (int j = 0; j < S; j++) R.a[k][j] *= d;
        }
    }
    return ok;
}

// G = Phi^-1 P, S = -P' G, Sinv = S^-1 (natural order).  Returns false on a singular S.
template <int SP, int SM>
__device__ __forceinline__ bool build_schur(const RegRows<SP> &RP, int n, int m, uint32_t gm, const int *permP,
                                            const float *P32, float *Pp, float *G, int ldg, float *Sm, float *Sinv,
                                            int lds, int *permS, float *dinvS, float *prow, int lane)
{
    constexpr int NS = RegRows<SP>::NS;
    const int n4 = (n + 3) & ~3;
    for (int l = 0; l < m; l++)
        for (int jj = lane; jj < n4; jj += 32) Pp[l * n4 + jj] = jj < n ? P32[permP[jj] * m + l] : 0.0f;
    __syncwarp();
#pragma unroll
    for (int k = 0; k < NS; k++) {
        if (32 * k >= n) break;
        const int v = RP.ps[k];
        const bool own = v >= 0 && v < n;
        for (int l = 0; l < m; l += 2) {
            const int l1 = l + 1 < m ? l + 1 : l;
            const float4 *p0 = reinterpret_cast<const float4 *>(Pp + l * n4);
            const float4 *p1 = reinterpret_cast<const float4 *>(Pp + l1 * n4);
            float a0 = 0.0f, a1 = 0.0f, b0 = 0.0f, b1 = 0.0f;
#pragma unroll
            for (int j4 = 0; j4 < SP / 4; j4 += 2) {
                if (4 * j4 < n) {
                    const float4 w = p0[j4], z = p1[j4];
                    a0 = fmaf(RP.a[k][4 * j4 + 0], w.x, a0);
                    b0 = fmaf(RP.a[k][4 * j4 + 0], z.x, b0);
                    a0 = fmaf(RP.a[k][4 * j4 + 1], w.y, a0);
                    b0 = fmaf(RP.a[k][4 * j4 + 1], z.y, b0);
                    a0 = fmaf(RP.a[k][4 * j4 + 2], w.z, a0);
                    b0 = fmaf(RP.a[k][4 * j4 + 2], z.z, b0);
                    a0 = fmaf(RP.a[k][4 * j4 + 3], w.w, a0);
                    b0 = fmaf(RP.a[k][4 * j4 + 3], z.w, b0);
                }
                if (4 * j4 + 4 < n) {
                    const float4 w = p0[j4 + 1], z = p1[j4 + 1];
                    a1 = fmaf(RP.a[k][4 * j4 + 4], w.x, a1);
                    b1 = fmaf(RP.a[k][4 * j4 + 4], z.x, b1);
                    a1 = fmaf(RP.a[k][4 * j4 + 5], w.y, a1);
                    b1 = fmaf(RP.a[k][4 * j4 + 5], z.y, b1);
                    a1 = fmaf(RP.a[k][4 * j4 + 6], w.z, a1);
                    b1 = fmaf(RP.a[k][4 * j4 + 6], z.z, b1);
                    a1 = fmaf(RP.a[k][4 * j4 + 7], w.w, a1);
                    b1 = fmaf(RP.a[k][4 * j4 + 7], z.w, b1);
                }
            }
            if (own) {
                G[v * ldg + l] = a0 + a1;
                if (l + 1 < m) G[v * ldg + l + 1] = b0 + b1;
            }
        }
    }
    __syncwarp();
    for (int t = lane; t < m * m; t += 32) {
        const int aa = div19(t, gm), bb = t - aa * m;
        float s0 = 0.0f, s1 = 0.0f;
        int i = 0;
        for (; i + 2 <= n; i += 2) {
            s0 = fmaf(P32[i * m + aa], G[i * ldg + bb], s0);
            s1 = fmaf(P32[(i + 1) * m + aa], G[(i + 1) * ldg + bb], s1);
        }
        if (i < n) s0 = fmaf(P32[i * m + aa], G[i * ldg + bb], s0);
        Sm[t] = -(s0 + s1);
    }
    __syncwarp();
    RegRows<SM> RS;
    {
        const bool act = lane < m;
        RS.ps[0] = act ? NOTYET : PADROW;
        static_for<0, SM>([&](auto BB) {
            constexpr int b = decltype(BB)::value;
            float v = 0.0f;
            if (act && b < m) v = Sm[lane * m + b];
            RS.a[0][b] = v;
        });
    }
    __syncwarp();
    const bool ok = reg_gj<SM>(RS, m, permS, dinvS, prow, lane);
    if (ok) {
        const int v = RS.ps[0];
        if (v >= 0 && v < m) {
            static_for<0, SM>([&](auto BB) {
                constexpr int b = decltype(BB)::value;
                if (b < m) Sinv[v * lds + permS[b]] = RS.a[0][b];
            });
        }
    }
    __syncwarp();
    return ok;
}

// R32 <- A^-1 R32 (s x r, row-major) through Phi^-1 (registers), G and Sinv.
template <int SP, int RMAX>
__device__ __forceinline__ void schur_correct(const RegRows<SP> &RP, int n, int m, int r, uint32_t gr,
                                              const int *permP, const float *G, int ldg, const float *Sinv, int lds,
                                              float *R32, float *U, float *Lam, float4 *bp, int lane)
{
    constexpr int NS = RegRows<SP>::NS;
    constexpr int RQ = (RMAX + 3) / 4;
    // (1) permuted r1 rows as float4 groups; u = r2 - G' r1
    for (int t = lane; t < n * RQ; t += 32) {
        const int jj = t / RQ, g = t - jj * RQ;
        const float *src = R32 + permP[jj] * r;
        float e[4];
#pragma unroll
        for (int u = 0; u < 4; u++) e[u] = (4 * g + u < r) ? src[4 * g + u] : 0.0f;
        bp[t] = make_float4(e[0], e[1], e[2], e[3]);
    }
    for (int e = lane; e < m * r; e += 32) {
        const int l = div19(e, gr), q = e - l * r;
        float u0 = R32[(n + l) * r + q], u1 = 0.0f;
        int i = 0;
        for (; i + 2 <= n; i += 2) {
            u0 = fmaf(-G[i * ldg + l], R32[i * r + q], u0);
            u1 = fmaf(-G[(i + 1) * ldg + l], R32[(i + 1) * r + q], u1);
        }
        if (i < n) u0 = fmaf(-G[i * ldg + l], R32[i * r + q], u0);
        U[e] = u0 + u1;
    }
    __syncwarp();
    // (2) lambda = Sinv u (shared memory); t = Phi^-1 r1 (registers)
    for (int e = lane; e < m * r; e += 32) {
        const int l = div19(e, gr), q = e - l * r;
        float v0 = 0.0f, v1 = 0.0f;
        int aa = 0;
        for (; aa + 2 <= m; aa += 2) {
            v0 = fmaf(Sinv[l * lds + aa], U[aa * r + q], v0);
            v1 = fmaf(Sinv[l * lds + aa + 1], U[(aa + 1) * r + q], v1);
        }
        if (aa < m) v0 = fmaf(Sinv[l * lds + aa], U[aa * r + q], v0);
        Lam[l * 4 * RQ + q] = v0 + v1;
    }
    float acc[NS][4 * RQ];
#pragma unroll
    for (int k = 0; k < NS; k++)
#pragma unroll
        for (int q = 0; q < 4 * RQ; q++) acc[k][q] = 0.0f;
#pragma unroll
    for (int jj = 0; jj < SP; jj++) {
        if (jj < n) {
#pragma unroll
            for (int g = 0; g < RQ; g++) {
                const float4 v = bp[jj * RQ + g];
#pragma unroll
                for (int k = 0; k < NS; k++) {
                    acc[k][4 * g + 0] = fmaf(RP.a[k][jj], v.x, acc[k][4 * g + 0]);
                    acc[k][4 * g + 1] = fmaf(RP.a[k][jj], v.y, acc[k][4 * g + 1]);
                    acc[k][4 * g + 2] = fmaf(RP.a[k][jj], v.z, acc[k][4 * g + 2]);
                    acc[k][4 * g + 3] = fmaf(RP.a[k][jj], v.w, acc[k][4 * g + 3]);
                }
            }
        }
    }
    __syncwarp();
    // (3) w = t - G lambda
    const float4 *Lam4 = reinterpret_cast<const float4 *>(Lam);
#pragma unroll
    for (int k = 0; k < NS; k++) {
        const int v = RP.ps[k];
        const bool own = v >= 0 && v < n;
        const int vv = own ? v : 0;
        for (int l = 0; l < m; l++) {
            const float gv = G[vv * ldg + l];
#pragma unroll
            for (int g = 0; g < RQ; g++) {
                const float4 lm = Lam4[l * RQ + g];
                acc[k][4 * g + 0] = fmaf(-gv, lm.x, acc[k][4 * g + 0]);
                acc[k][4 * g + 1] = fmaf(-gv, lm.y, acc[k][4 * g + 1]);
                acc[k][4 * g + 2] = fmaf(-gv, lm.z, acc[k][4 * g + 2]);
                acc[k][4 * g + 3] = fmaf(-gv, lm.w, acc[k][4 * g + 3]);
            }
        }
        if (own) {
#pragma unroll
            for (int q = 0; q < RMAX; q++)
                if (q < r) R32[v * r + q] = acc[k][q];
        }
    }
    for (int e = lane; e < m * r; e += 32) {
        const int l = div19(e, gr), q = e - l * r;
        R32[(n + l) * r + q] = Lam[l * 4 * RQ + q];
    }
    __syncwarp();
}

// a = hi + lo with hi the float truncation of a and lo the float truncation of the remaining
// 29 mantissa bits (|a - hi - lo| <= 2^-47 |a|), from the bit fields (integer pipe).
__device__ __forceinline__ void split_f64(double a, float &hi, float &lo)
{
    hi = f64_to_f32(a);
    const unsigned h = (unsigned)__double2hiint(a), l = (unsigned)__double2loint(a);
    const int e = (int)((h >> 20) & 0x7ffu);
    const unsigned rem = l & 0x1fffffffu;  // mantissa bits below the float's 23
    // rem * 2^(e - 1075), exact in the integer-to-float conversion up to rounding of 29 -> 24 bits
    const int ex = e - 1075 + 127;
    const float scale = ex > 0 && ex < 255 ? __uint_as_float((unsigned)ex << 23) : 0.0f;
    const float v = __uint2float_rz(rem) * scale;
    lo = (h & 0x80000000u) ? -v : v;
}

// Exact sum s + e = a + b of two floats (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Double-float (hi, lo) + d, renormalised: the refinement's solution and residual vectors are
// kept in this form (48 significant bits) so that their updates need no FP64 instruction.
__device__ __forceinline__ float2 df_add(float2 x, float d)
{
    float s, e;
    two_sum(x.x, d, s, e);
    float hi, lo;
    two_sum(s, e + x.y, hi, lo);
    return make_float2(hi, lo);
}

// A double as a double-float pair (split_f64: |v - hi - lo| <= 2^-47 |v|).
__device__ __forceinline__ float2 df_from_f64(double v)
{
    float hi, lo;
    split_f64(v, hi, lo);
    return make_float2(hi, lo);
}

// Phi lower triangle (with its zero diagonal) packed by rows: element (i, j <= i) at
// i (i + 1) / 2 + j.
__device__ __forceinline__ int tri_off(int i) { return (i * (i + 1)) >> 1; }

// NE (1 or 2) elements (i, q) of r = b - A x for the Phi rows, elements e0 + lane + 32 u.
template <int NE>
__device__ __forceinline__ void residual_phi_rows(const double *phiP, const double *P, int n, int m, int r,
                                                  uint32_t gr, double *B, const double *X, float *R32, int e0,
                                                  bool store_r, int lane)
{
    const int tot = n * r;
    int ee[NE], ii[NE], qq[NE], off[NE];
    double a0[NE], a1[NE];
#pragma unroll
    for (int u = 0; u < NE; u++) {
        ee[u] = e0 + lane + 32 * u;
        const int ec = ee[u] < tot ? ee[u] : tot - 1;
        ii[u] = div19(ec, gr);
        qq[u] = ec - ii[u] * r;
        off[u] = tri_off(ii[u]);
        a0[u] = B[ec];
        a1[u] = 0.0;
    }
    int offj = 0;  // tri_off(jj)
    int jj = 0;
    for (; jj + 2 <= n; jj += 2) {
        const int offj1 = offj + jj + 1;
#pragma unroll
        for (int u = 0; u < NE; u++) {
            const int ad0 = jj <= ii[u] ? off[u] + jj : offj + ii[u];
            const int ad1 = jj + 1 <= ii[u] ? off[u] + jj + 1 : offj1 + ii[u];
            a0[u] = fma(-phiP[ad0], X[jj * r + qq[u]], a0[u]);
            a1[u] = fma(-phiP[ad1], X[(jj + 1) * r + qq[u]], a1[u]);
        }
        offj = offj1 + jj + 2;
    }
    if (jj < n) {
#pragma unroll
        for (int u = 0; u < NE; u++) {
            const int ad0 = jj <= ii[u] ? off[u] + jj : offj + ii[u];
            a0[u] = fma(-phiP[ad0], X[jj * r + qq[u]], a0[u]);
        }
    }
    const double *Xl = X + n * r;
    int l = 0;
    for (; l + 2 <= m; l += 2) {
#pragma unroll
        for (int u = 0; u < NE; u++) {
            a0[u] = fma(-P[ii[u] * m + l], Xl[l * r + qq[u]], a0[u]);
            a1[u] = fma(-P[ii[u] * m + l + 1], Xl[(l + 1) * r + qq[u]], a1[u]);
        }
    }
    if (l < m) {
#pragma unroll
        for (int u = 0; u < NE; u++) a0[u] = fma(-P[ii[u] * m + l], Xl[l * r + qq[u]], a0[u]);
    }
#pragma unroll
    for (int u = 0; u < NE; u++)
        if (ee[u] < tot) {
            const double v = a0[u] + a1[u];
            if (store_r) reinterpret_cast<float2 *>(B)[ee[u]] = df_from_f64(v);
            R32[ee[u]] = f64_to_f32(v);
        }
}

// R32 <- float(B - A X) (and B <- B - A X as double-float pairs when store_r) with FP64
// products, lane-per-element: ceil(n r / 32) lane-full passes
// of n + m FMAs for the Phi rows (two passes interleaved per lane), one pass of n FMAs per 32
// elements for the P' rows.  Phi is read from its packed lower triangle.
__device__ __forceinline__ void residual_schur(const double *phiP, const double *P, int n, int m, int r, uint32_t gr,
                                              double *B, const double *X, float *R32, bool store_r, int lane)
{
    const int tot = n * r;
    for (int e0 = 0; e0 < tot; e0 += 64) {
        if (e0 + 32 < tot)
            residual_phi_rows<2>(phiP, P, n, m, r, gr, B, X, R32, e0, store_r, lane);
        else
            residual_phi_rows<1>(phiP, P, n, m, r, gr, B, X, R32, e0, store_r, lane);
    }
    for (int e = lane; e < m * r; e += 32) {
        const int l = div19(e, gr), q = e - l * r;
        double a0 = B[(n + l) * r + q], a1 = 0.0;
        int jj = 0;
        for (; jj + 2 <= n; jj += 2) {
            a0 = fma(-P[jj * m + l], X[jj * r + q], a0);
            a1 = fma(-P[(jj + 1) * m + l], X[(jj + 1) * r + q], a1);
        }
        if (jj < n) a0 = fma(-P[jj * m + l], X[jj * r + q], a0);
        const double v = a0 + a1;
        if (store_r) reinterpret_cast<float2 *>(B)[(n + l) * r + q] = df_from_f64(v);
        R32[(n + l) * r + q] = f64_to_f32(v);
    }
    __syncwarp();
}

// s_hi + s_lo += a * d for floats a, d: the product exactly (TwoProduct by FMA), the sum by
// TwoSum into s_hi with every rounding error collected in s_lo (the double-float dot product
// of Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 2005).
__device__ __forceinline__ void df_mac(float a, float d, float &s_hi, float &s_lo)
{
    const float p = a * d;
    const float e = fmaf(a, d, -p);
    const float s = s_hi + p;
    const float bb = s - s_hi;
    const float err = (s_hi - (s - bb)) + (p - bb);
    s_hi = s;
    s_lo += err + e;
}

// df_mac on two sums at once (packed FP32, fma.rn.f32x2 and relatives): (sh, sl) += a (d.x, d.y)
// + al (d.x, d.y), with a2 = (a, a), na2 = (-a, -a), al2 = (al, al).  Differences x - y are
// fma(y, -1, x), exact like the subtraction.  The same operations as df_mac followed by
// sl = fmaf(al, d, sl) on each half, except that the product's error enters sl after the
// TwoSum error instead of with it.
__device__ __forceinline__ void df_mac2(float2 a2, float2 na2, float2 al2, float2 d, float2 &sh, float2 &sl)
{
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 p = __fmul2_rn(a2, d);
    const float2 ne = __ffma2_rn(na2, d, p);  // -(a d - p), exact
    const float2 s = __fadd2_rn(sh, p);
    const float2 bb = __ffma2_rn(sh, m1, s);                                            // s - sh
    const float2 err = __fadd2_rn(__ffma2_rn(__ffma2_rn(bb, m1, s), m1, sh), __ffma2_rn(bb, m1, p));  // TwoSum error
    sh = s;
    sl = __ffma2_rn(al2, d, __ffma2_rn(ne, m1, __fadd2_rn(sl, err)));
}

// The packed Phi and P of a system rewritten in place as their double-float splits (float2
// (hi, lo) in the same 8 bytes per element), for the later residuals of a system with a single
// evaluation row: its FP64 first residual, the only user of the exact FP64 values, is done.
__device__ __forceinline__ void presplit_phi_p(double *phiP, double *P, int n, int m, int lane)
{
    const int nphi = tri_off(n);
    for (int e = lane; e < nphi; e += 32) reinterpret_cast<float2 *>(phiP)[e] = df_from_f64(phiP[e]);
    for (int e = lane; e < n * m; e += 32) reinterpret_cast<float2 *>(P)[e] = df_from_f64(P[e]);
    __syncwarp();
}

// Element `ad` of an FP64 array as (hi, lo): split on the fly, or read when PRE (the array was
// rewritten by presplit_phi_p).
template <bool PRE>
__device__ __forceinline__ void split_at(const double *a, int ad, float &hi, float &lo)
{
    if constexpr (PRE) {
        const float2 v = reinterpret_cast<const float2 *>(a)[ad];
        hi = v.x;
        lo = v.y;
    } else {
        split_f64(a[ad], hi, lo);
    }
}

// Residual after a correction, r_new = r_old - A d, without FP64 instructions: d (the last
// correction, R32) is a float vector, A = hi + lo splits exactly enough, A d is accumulated as
// a double-float sum and subtracted from r_old, itself a double-float pair.  The error of
// A d is ~2^-44 |A||d| with |d| ~ 1e-5 |x|, and the pair holds r_old to 2^-47 of its size
// (~1e-5 |A||x|), both far below FP64 rounding of |A||x|, so the refinement converges as with
// an FP64 residual.  B holds r_old as (hi, lo) pairs and receives r_new; R32 receives hi.
// Phi rows lane-per-row (the split of Phi_ij shared by the row's operators, two operators per
// packed instruction), P' rows lane-per-element.  PRE: Phi and P hold their splits already.
template <int SP, int SM, int RMAX, bool PRE>
__device__ __forceinline__ void residual_df(const double *phiP, const double *P, int n, int m, int r, uint32_t gr,
                                            double *B, float *R32, int lane)
{
    constexpr int NS = RegRows<SP>::NS;
    float sh[NS][RMAX], sl[NS][RMAX];
    // Phi and P rows: the operators' sums in pairs (q, q + 1), packed FP32; a pair past r
    // computes on zeros
    constexpr int QP = (RMAX + 1) / 2;
#pragma unroll
    for (int k = 0; k < NS; k++) {
        float2 SH[QP], SL[QP];
#pragma unroll
        for (int u = 0; u < QP; u++) SH[u] = SL[u] = make_float2(0.0f, 0.0f);
        if (32 * k < n) {
            const int i = lane + 32 * k;
            const int ii = i < n ? i : n - 1;
            const int offi = tri_off(ii);
            auto column = [&](float ah, float al, const float *dj) {
                const float2 a2 = make_float2(ah, ah), na2 = make_float2(-ah, -ah), al2 = make_float2(al, al);
#pragma unroll
                for (int u = 0; u < QP; u++) {
                    if (2 * u < r) {
                        const float2 d = make_float2(dj[2 * u], 2 * u + 1 < r ? dj[2 * u + 1] : 0.0f);
                        df_mac2(a2, na2, al2, d, SH[u], SL[u]);
                    }
                }
            };
            int offj = 0;
            for (int jj = 0; jj < n; jj++) {
                const int ad = jj <= ii ? offi + jj : offj + ii;
                offj += jj + 1;
                float ah, al;
                split_at<PRE>(phiP, ad, ah, al);
                column(ah, al, R32 + jj * r);
            }
            for (int l = 0; l < m; l++) {
                float ah, al;
                split_at<PRE>(P, ii * m + l, ah, al);
                column(ah, al, R32 + (n + l) * r);
            }
        }
#pragma unroll
        for (int u = 0; u < QP; u++) {
            sh[k][2 * u] = SH[u].x;
            sl[k][2 * u] = SL[u].x;
            if (2 * u + 1 < RMAX) {
                sh[k][2 * u + 1] = SH[u].y;
                sl[k][2 * u + 1] = SL[u].y;
            }
        }
    }
    constexpr int PE = (SM * RMAX + 31) / 32;  // P' elements per lane (m r <= SM RMAX)
    float th[PE], tl[PE];
#pragma unroll
    for (int u = 0; u < PE; u++) {
        th[u] = tl[u] = 0.0f;
        const int e = lane + 32 * u;
        if (e < m * r) {
            const int l = div19(e, gr), q = e - l * r;
            for (int jj = 0; jj < n; jj++) {
                float ah, al;
                split_at<PRE>(P, jj * m + l, ah, al);
                const float d = R32[jj * r + q];
                df_mac(ah, d, th[u], tl[u]);
                tl[u] = fmaf(al, d, tl[u]);
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < NS; k++) {
        const int i = lane + 32 * k;
        if (i < n) {
#pragma unroll
            for (int q = 0; q < RMAX; q++) {
                if (q < r) {
                    float2 *b2 = reinterpret_cast<float2 *>(B) + i * r + q;
                    const float2 v = df_add(df_add(*b2, -sh[k][q]), -sl[k][q]);
                    *b2 = v;
                    R32[i * r + q] = v.x;
                }
            }
        }
    }
#pragma unroll
    for (int u = 0; u < PE; u++) {
        const int e = lane + 32 * u;
        if (e < m * r) {
            const int idx = n * r + e;
            float2 *b2 = reinterpret_cast<float2 *>(B) + idx;
            const float2 v = df_add(df_add(*b2, -th[u]), -tl[u]);
            *b2 = v;
            R32[idx] = v.x;
        }
    }
    __syncwarp();
}

// (i, j) of the t-th strictly lower pair (row-major: t = i (i - 1) / 2 + j) for stencils of
// up to 64 nodes, as (i << 8) | j: one cached load instead of a square root and fix-ups.
struct PairTable {
    uint16_t ij[64 * 63 / 2];
};
constexpr PairTable make_pair_table()
{
    PairTable T{};
    int t = 0;
    for (int i = 1; i < 64; i++)
        for (int j = 0; j < i; j++) T.ij[t++] = (uint16_t)((i << 8) | j);
    return T;
}
__device__ const PairTable g_pair_table = make_pair_table();

// Pairs per lane per pass of the FP64 Phi assembly (independent Heron chains in flight); 3 and
// 4 measured slower than 2 (register pressure at the 128-register budget).
#ifndef RBFFD_PHI_NP
#define RBFFD_PHI_NP 2
#endif

// One pass of the packed FP64 Phi: strictly lower pairs t0 + lane + 32 u, u < NP, stored at
// tri_off(i) + j = t + i.
template <int NP>
__device__ __forceinline__ void phi_pair_pass(const double *xs, int n, int p, double *phiP, int t0, int lane)
{
    const int npairs = n * (n - 1) / 2;
    double v[NP];
    int ti[NP];
#pragma unroll
    for (int u = 0; u < NP; u++) {
        const int t = t0 + lane + 32 * u;
        const int ij = g_pair_table.ij[t < npairs ? t : 0];
        const int i = ij >> 8, j = ij & 0xff;
        const double dx = xs[2 * i] - xs[2 * j], dy = xs[2 * i + 1] - xs[2 * j + 1];
        v[u] = phi64_nr(fma(dx, dx, dy * dy), p);
        ti[u] = t < npairs ? t + i : -1;
    }
#pragma unroll
    for (int u = 0; u < NP; u++)
        if (ti[u] >= 0) phiP[ti[u]] = v[u];
}

// One pass of the packed Phi for odd p >= 3 from 61-bit fixed-point coordinates xf (no FP64
// instruction for p = 3; r^(p-3) as FP64 products of r^2 otherwise).
template <int NP>
__device__ __forceinline__ void phi_pair_pass_fx(const longlong2 *xf, int n, int p, double *phiP, int t0, int lane)
{
    const int npairs = n * (n - 1) / 2;
    double v[NP];
    int ti[NP];
#pragma unroll
    for (int u = 0; u < NP; u++) {
        const int t = t0 + lane + 32 * u;
        const int ij = g_pair_table.ij[t < npairs ? t : 0];
        const int i = ij >> 8, j = ij & 0xff;
        const longlong2 a = xf[i], b = xf[j];
        double r2 = 0.0;
        double f = rbffd_fx::r3_fixed(a.x, a.y, b.x, b.y, p > 3 ? &r2 : nullptr);
        for (int e = 3; e < p; e += 2) f *= r2;
        v[u] = f;
        ti[u] = t < npairs ? t + i : -1;
    }
#pragma unroll
    for (int u = 0; u < NP; u++)
        if (ti[u] >= 0) phiP[ti[u]] = v[u];
}

// The packed FP64 Phi, its zero diagonal and the FP64 P rows.  Odd p >= 3 with all scaled
// coordinates below 2 in magnitude (every scaled stencil) takes the fixed-point pair routine;
// xf (16 bytes per node) is free scratch at this point.
__device__ __forceinline__ void assemble_phi_packed(const double *xs, int n, int m, int deg, int p, double *phiP,
                                                    double *P, longlong2 *xf, int lane)
{
    constexpr int NP = RBFFD_PHI_NP;
    const int npass = (n * (n - 1) / 2 + 32 * NP - 1) / (32 * NP);
    bool fx = (p & 1) && p >= 3;
    if (fx) {
        bool in_range = true;
        for (int i = lane; i < n; i += 32)
            in_range = in_range && rbffd_fx::fixed61_ok(xs[2 * i]) && rbffd_fx::fixed61_ok(xs[2 * i + 1]);
        fx = __all_sync(RBFFD_FULL, in_range);
    }
    if (fx) {
        for (int i = lane; i < n; i += 32)
            xf[i] = make_longlong2(rbffd_fx::to_fixed61(xs[2 * i]), rbffd_fx::to_fixed61(xs[2 * i + 1]));
        __syncwarp();
        for (int q = 0; q < npass; q++) phi_pair_pass_fx<NP>(xf, n, p, phiP, 32 * NP * q, lane);
    } else {
        for (int q = 0; q < npass; q++) phi_pair_pass<NP>(xs, n, p, phiP, 32 * NP * q, lane);
    }
    for (int i = lane; i < n; i += 32) {
        phiP[tri_off(i) + i] = 0.0;
        monomial_row<double>(xs[2 * i], xs[2 * i + 1], deg, P + i * m, 1);
    }
    __syncwarp();
}

__device__ __forceinline__ int ifact(int e)
{
    int c = 1;
    for (int t = 2; t <= e; t++) c *= t;
    return c;
}

// Right-hand sides of one evaluation point y~ (scaled coordinates) into B (s x r).  Same
// formulas as build_rhs, with r and 1/r from sqrt_nr / recip_nr, per-system scale factors
// sc[2 q + c] = sx^a sy^b precomputed, and the polynomial rows of a point at the stencil
// centre (y~ = 0: the common collocated case) from integers.
__device__ __forceinline__ void build_rhs_schur(const OpTable &ops, const double *xs, int n, int m, double yx,
                                                double yy, const double *sc, bool need_rinv, double *B, int lane)
{
    const int r = ops.nops;
    const bool at0 = is_zero64(yx) && is_zero64(yy);
    const int closed = ops.r3_closed;
    for (int i = lane; i < n; i += 32) {
        // y~ - x~_i; at the centre (the collocated case) the negation is a sign flip on the
        // integer pipe instead of an FP64 subtraction from zero
        double cx = at0 ? neg64(xs[2 * i]) : yx - xs[2 * i], cy = at0 ? neg64(xs[2 * i + 1]) : yy - xs[2 * i + 1];
        if (is_zero64(cx)) cx = EPS64;
        if (is_zero64(cy)) cy = EPS64;
        const double r2 = fma(cx, cx, cy * cy);
        double y0;
        const double rr = sqrt_nr(r2, y0);
        const double rinv = need_rinv ? recip_nr(rr, y0) : 0.0;
        if (closed) {
            // r^3 = r^2 r; d/dx r^3 = 3 x r; d2/dx2 r^3 = 3 r + 3 x^2 / r; d2/dxdy r^3 = 3 x y / r
            // (y alike); sx^2 d2/dx2 r^3 + sy^2 d2/dy2 r^3 = (3 (2 sx^2 + sy^2) x^2
            // + 3 (sx^2 + 2 sy^2) y^2) / r (with r^2 = x^2 + y^2).  For Dx, Dy and Lap: 8 FP64
            // operations per node after r and 1/r instead of 17.
            const double t3 = (closed & 2) ? 3.0 * rr : 0.0;
            const double q3 = (closed & 8) ? 3.0 * rinv : 0.0;
            const double lap = (closed & 4) ? fma(sc[2 * r] * cx, cx, (sc[2 * r + 1] * cy) * cy) * rinv : 0.0;
            for (int q = 0; q < r; q++) {
                const OpDesc &od = ops.op[q];
                const int oa = od.c[0].a, ob = od.c[0].b;
                double v;
                if (od.ncomp == 2)
                    v = lap;  // Lap
                else if (oa + ob == 0)
                    v = r2 * rr;  // E
                else if (oa + ob == 1)
                    v = t3 * (oa ? cx : cy);  // Dx, Dy
                else if (oa == 1)
                    v = (q3 * cx) * cy;  // Dxy
                else {
                    const double c = oa ? cx : cy;  // Dxx, Dyy
                    v = fma(q3 * c, c, t3);
                }
                B[i * r + q] = v;
            }
            continue;
        }
        if (ops.r5_hv4) {
            // d4/dx4 r^5 = -15 x^4 / r^3 + 90 x^2 / r + 45 r = 15 r (3 + u (6 - u)), u = x^2 / r^2
            // (u in [0, 1]: no cancellation): 5 FP64 operations per operator instead of 13
            const double rinv2 = rinv * rinv, r15 = 15.0 * rr;
            for (int q = 0; q < r; q++) {
                const double c = ops.op[q].c[0].a ? cx : cy;
                const double u = (c * c) * rinv2;
                B[i * r + q] = r15 * fma(u, 6.0 - u, 3.0);
            }
            continue;
        }
        for (int q = 0; q < r; q++) {
            const OpDesc &od = ops.op[q];
            double v = 0.0;
            for (int cidx = 0; cidx < od.ncomp; cidx++) {
                const OpComp &oc = od.c[cidx];
                double cv = 0.0;
                for (int t = 0; t < oc.nterm; t++) {
                    const RbfTerm &tm = oc.t[t];
                    double tv = tm.coef;
                    for (int e = 0; e < tm.ex; e++) tv *= cx;
                    for (int e = 0; e < tm.ey; e++) tv *= cy;
                    if (tm.er >= 0)
                        for (int e = 0; e < tm.er; e++) tv *= rr;
                    else
                        for (int e = 0; e < -tm.er; e++) tv *= rinv;
                    cv = t == 0 ? tv : cv + tv;  // no FP64 addition to an initial zero
                }
                if (od.ncomp > 1) cv *= sc[2 * q + cidx];
                v = cidx == 0 ? cv : v + cv;
            }
            B[i * r + q] = v;
        }
    }
    if (ops.r5_hv4 && at0) {
        // the polynomial rows at the centre: 4! at x^4 (Dxk) or y^4 (Dyk), zero elsewhere
        for (int l = lane; l < m; l += 32)
            for (int q = 0; q < r; q++) B[(n + l) * r + q] = l == (ops.op[q].c[0].a ? 10 : 14) ? 24.0 : 0.0;
        __syncwarp();
        return;
    }
    if (closed && at0) {
        // the polynomial rows at the centre: a! b! at the monomial x^a y^b of the operator
        // d^(a+b)/dx^a dy^b (index (a + b)(a + b + 1)/2 + b), zero elsewhere; 2 sx^2 at x^2 and
        // 2 sy^2 at y^2 for Lap
        for (int l = lane; l < m; l += 32)
            for (int q = 0; q < r; q++) {
                const OpDesc &od = ops.op[q];
                const int oa = od.c[0].a, ob = od.c[0].b, t = oa + ob;
                double v = 0.0;
                if (od.ncomp == 2)
                    v = l == 3 ? twice64(sc[2 * q]) : l == 5 ? twice64(sc[2 * q + 1]) : 0.0;
                else if (l == t * (t + 1) / 2 + ob)
                    v = (oa == 2 || ob == 2) ? 2.0 : 1.0;
                B[(n + l) * r + q] = v;
            }
        __syncwarp();
        return;
    }
    for (int l = lane; l < m; l += 32) {
        int t = 0, rem = l;
        while (rem > t) {
            rem -= t + 1;
            t++;
        }
        const int ea = t - rem, eb = rem;
        for (int q = 0; q < r; q++) {
            const OpDesc &od = ops.op[q];
            double v = 0.0;
            for (int cidx = 0; cidx < od.ncomp; cidx++) {
                const OpComp &oc = od.c[cidx];
                if (oc.a > ea || oc.b > eb) continue;
                double cv;
                if (at0) {
                    if (oc.a != ea || oc.b != eb) continue;
                    cv = f32_to_f64((float)(ifact(ea) * ifact(eb)));
                } else {
                    cv = falling(ea, oc.a) * falling(eb, oc.b) * ipow(yx, ea - oc.a) * ipow(yy, eb - oc.b);
                }
                if (od.ncomp > 1) cv *= sc[2 * q + cidx];
                v += cv;
            }
            B[(n + l) * r + q] = v;
        }
    }
    __syncwarp();
}

// One output row from the double-float solution: hi + lo (exact in FP64), times the
// operator's scale factor sx^a sy^b (sc, the same product write_row forms) when it is applied
// after the solve.
__device__ __forceinline__ void write_row_df(const SolveArgs &a, const OpTable &ops, int64_t row, const float2 *X2,
                                             int n, const int *sid, const double *sc, int lane)
{
    const int64_t off = a.row_ptr[row - a.row_begin];
    const int r = ops.nops;
    for (int l = lane; l < n; l += 32) a.col[off + l] = sid[l];
    for (int l = lane; l < n; l += 32) {
        const int64_t d = a.csc_pos ? (int64_t)a.csc_pos[off + l] : off + l;
        for (int q = 0; q < r; q++) {
            const float2 x = X2[l * r + q];
            const double v = f32_to_f64(x.x) + f32_to_f64(x.y);
            a.val[(int64_t)q * a.nnz + d] = ops.op[q].post_scale ? sc[2 * q] * v : v;
        }
    }
}

// Systems are claimed from a counter, a CTA's warps together: at a CTA barrier one thread
// takes the next wpb systems for the CTA's wpb warps, so that the warps of a CTA start every
// system at the same time.  The kernel is large (the elimination, the Schur complement and the
// residuals are unrolled over compile-time register indices), and warps that drift apart -- as
// they do when systems need different numbers of refinement steps -- run different parts of it
// at once, which an SM's instruction cache cannot hold: on 45-node stencils with degree 4 (a
// quarter of the systems needing one more step than the rest) the free-running kernel spent
// 18 warp-cycles per issued instruction waiting for instructions and ran at 510 ns per system
// against 180-240 ns while its warps were still in step.  Without a counter (a.next_sys null)
// warps take systems by a fixed grid stride.
template <int SP, int SM, int RMAX>
__global__ void __launch_bounds__(RBFFD_SCHUR_MAX_THREADS(SP), 1) solve_mixed_schur_kernel(SolveArgs a, OpTable ops)
{
    __shared__ unsigned long long cta_claim;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const SchurLayout L = make_schur_layout(SP, SM, a.max_n, a.max_m, ops.nops);
    unsigned char *base = smem_raw + (size_t)wib * L.total;
    double *phiP = (double *)(base + L.phi);
    double *P = (double *)(base + L.P);
    double *xs = (double *)(base + L.xs);
    int *sid = (int *)(base + L.sid);
    float *G = (float *)(base + L.G);
    float *Sinv = (float *)(base + L.Sinv);
    int *permP = (int *)(base + L.permP);
    float *dinvP = (float *)(base + L.dinvP);
    int *permS = (int *)(base + L.permS);
    float *dinvS = (float *)(base + L.dinvS);
    float *prow = (float *)(base + L.prow);
    double *sc = (double *)(base + L.sc);
    float2 *x32 = (float2 *)(base + L.x32);
    longlong2 *xf = (longlong2 *)(base + L.x32);
    float *P32 = (float *)(base + L.P32);
    float *Pp = (float *)(base + L.Pp);
    float *Sm = (float *)(base + L.Sm);
    double *B = (double *)(base + L.B);
    double *X = (double *)(base + L.X);
    float *R32 = (float *)(base + L.R32);
    float *U = (float *)(base + L.U);
    float *Lam = (float *)(base + L.Lam);
    float4 *bp = (float4 *)(base + L.bp);
    const int r = ops.nops, p = ops.p, ldg = L.ldg, lds = L.lds;
    const uint32_t gr = div19_magic(r);

    const float tol32 = f64_to_f32(a.refine_tol);
    bool need_rinv = false;
    for (int q = 0; q < r; q++)
        for (int c = 0; c < ops.op[q].ncomp; c++)
            for (int t = 0; t < ops.op[q].c[c].nterm; t++) need_rinv |= ops.op[q].c[c].t[t].er < 0;

    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool claim = a.next_sys != nullptr;
    const int wpb = blockDim.x >> 5;
    int64_t ts = gw - nw;
    for (;;) {
        if (claim) {
            __syncthreads();  // every warp of the CTA is done with its previous system
            if (threadIdx.x == 0) cta_claim = atomicAdd(a.next_sys, (unsigned long long)wpb);
            __syncthreads();
            const int64_t first = (int64_t)cta_claim;
            if (first >= a.nsys) break;  // uniform over the CTA
            ts = first + wib;
            if (ts >= a.nsys) continue;  // no system for this warp in the last round
        } else {
            ts += nw;
            if (ts >= a.nsys) break;
        }
        const int64_t sys = a.sys_list ? (int64_t)a.sys_list[ts] : a.sys_base + ts;
        const int j = a.sys_node[sys];
        const int n = a.n_node ? a.n_node[j] : a.n;
        const int deg = a.deg_node ? a.deg_node[j] : a.deg;
        const int m = npoly(deg), s = n + m;
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        for (int l = lane; l < n; l += 32) {
            const float2 v = make_float2(f64_to_f32(xs[2 * l]), f64_to_f32(xs[2 * l + 1]));
            x32[l] = v;
            monomial_row<float>(v.x, v.y, deg, P32 + l * m, 1);
        }
        if (lane < 2 * r) {
            const int q = lane >> 1, c = lane & 1;
            if (c < ops.op[q].ncomp) sc[lane] = ipow(sx, ops.op[q].c[c].a) * ipow(sy, ops.op[q].c[c].b);
        } else if ((ops.r3_closed & 4) && lane < 2 * r + 2) {
            // the closed-form Lap of r^3: 3 (2 sx^2 + sy^2) and 3 (sx^2 + 2 sy^2)
            const double sx2 = sx * sx, sy2 = sy * sy;
            sc[lane] = 3.0 * (lane == 2 * r ? twice64(sx2) + sy2 : sx2 + twice64(sy2));
        }
        __syncwarp();
        RegRows<SP> RP;
        fill_phi_rows<SP>(RP, x32, n, p, lane);
        bool ok = reg_gj<SP>(RP, n, permP, dinvP, prow, lane);
        if (ok)
            ok = build_schur<SP, SM>(RP, n, m, div19_magic(m), permP, P32, Pp, G, ldg, Sm, Sinv, lds, permS, dinvS,
                                     prow, lane);
        bool fallback = !ok;
        if (ok) assemble_phi_packed(xs, n, m, deg, p, phiP, P, xf, lane);
        int64_t r0, r1;
        system_rows(a, sys, j, r0, r1);
        // a system with one evaluation row (the collocated case) needs its exact FP64 Phi and P
        // only for that row's first residual; the later residuals then read them pre-split
        const bool one_row = r1 - r0 == 1;
        bool presplit = false;
        int iters_max = 0;
        for (int64_t t = r0; t < r1 && !fallback; t++) {
            const int64_t row = row_id(a, t);
            const double2 yp = eval_point(a, row);
            const double yx = (yp.x - xc.x) * sx, yy = (yp.y - xc.y) * sy;
            build_rhs_schur(ops, xs, n, m, yx, yy, sc, need_rinv, B, lane);
            float e_prev = 1.0f;
            bool conv = false;
            int it;
            for (it = 0; it < a.max_refine; it++) {
                if (it == 0) {
                    for (int e = lane; e < s * r; e += 32) R32[e] = f64_to_f32(B[e]);
                    __syncwarp();
                } else if (it == 1) {
                    residual_schur(phiP, P, n, m, r, gr, B, X, R32, true, lane);
                } else if (one_row) {
                    if (!presplit) {
                        presplit_phi_p(phiP, P, n, m, lane);
                        presplit = true;
                    }
                    residual_df<SP, SM, RMAX, true>(phiP, P, n, m, r, gr, B, R32, lane);
                } else {
                    residual_df<SP, SM, RMAX, false>(phiP, P, n, m, r, gr, B, R32, lane);
                }
                schur_correct<SP, RMAX>(RP, n, m, r, gr, permP, G, ldg, Sinv, lds, R32, U, Lam, bp, lane);
                // x0 is kept as FP64 for the FP64 first residual; from the first update on, x is
                // a double-float pair in the same 8 bytes of each element.
                unsigned dkey = 0u, xkey = 0u;
                for (int e = lane; e < s * r; e += 32) {
                    const float d = R32[e];
                    float xh;
                    if (it == 0) {
                        X[e] = f32_to_f64(d);
                        xh = d;
                    } else {
                        float2 *x2 = reinterpret_cast<float2 *>(X) + e;
                        const float2 v = df_add(it == 1 ? make_float2(f64_to_f32(X[e]), 0.0f) : *x2, d);
                        *x2 = v;
                        xh = v.x;
                    }
                    if (e < n * r) {
                        dkey = max(dkey, __float_as_uint(d) & 0x7fffffffu);
                        xkey = max(xkey, __float_as_uint(xh) & 0x7fffffffu);
                    }
                }
                dkey = __reduce_max_sync(RBFFD_FULL, dkey);
                xkey = __reduce_max_sync(RBFFD_FULL, xkey);
                __syncwarp();
                const float dmax = __uint_as_float(dkey);
                const float xmax = __uint_as_float(xkey);
                const float e_cur = xmax > 0.0f ? __fdividef(dmax, xmax) : 0.0f;
                if (!(e_cur == e_cur) || isinf(e_cur)) break;
                // Predicted error after this correction: rho * e_cur, rho the observed contraction.
                // rho is taken from two corrections (it >= 2): at it = 1 the ratio to the first
                // solve measures the error of x0 in the direction of the solution only and can
                // fall far below the contraction (systems stopped there erred ~1e3x the
                // tolerance at refine_tol 1e-11).
                if (it >= 1) {
                    const float rho = e_prev > 0.0f ? __fdividef(e_cur, e_prev) : 0.0f;
                    if (e_cur == 0.0f || (it >= 2 && rho * e_cur <= tol32)) {
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
            write_row_df(a, ops, row, reinterpret_cast<const float2 *>(X), n, sid, sc, lane);
            __syncwarp();
        }
        if (lane == 0) {
            if (fallback) {
                const int pos = atomicAdd(a.fallback_count, 1);
                a.fallback_list[pos] = (int32_t)sys;
            } else {
                atomicAdd(&a.hist[iters_max < 7 ? iters_max : 7], 1ull);
            }
        }
        __syncwarp();
    }
}

template <int SP, int SM, int RMAX>
cudaError_t launch_schur(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st)
{
    const size_t per_warp = make_schur_layout(SP, SM, a.max_n, a.max_m, ops.nops).total;
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    while (wpb > 1 && per_warp * wpb > (size_t)smem_max) wpb--;
    if (per_warp * wpb > (size_t)smem_max) return cudaErrorNotSupported;
    auto kern = solve_mixed_schur_kernel<SP, SM, RMAX>;
    cudaFuncAttributes fa;
    cudaError_t ea = cudaFuncGetAttributes(&fa, kern);
    if (ea != cudaSuccess) return ea;
    while (wpb > 1 && wpb * 32 > fa.maxThreadsPerBlock) wpb--;
    const size_t smem = per_warp * wpb;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, wpb * 32, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int64_t want = (a.nsys + wpb - 1) / wpb;
    const int64_t cap = (int64_t)num_sms * occ;
    const int blocks = (int)(want < cap ? want : cap);
    kern<<<blocks, wpb * 32, smem, st>>>(a, ops);
    return cudaGetLastError();
}

}  // namespace

// Launchers of the Schur-complement kernel for stencils of at most 32 (weights_reg.cu) and at
// most 64 nodes (weights_reg64.cu).  SM (16 or 32) bounds the number of monomials and RMAX
// (4 or 8) the number of operators.
cudaError_t launch_schur_sp32(const SolveArgs &a, const OpTable &ops, int SM, int RMAX, int wpb, int num_sms,
                              cudaStream_t st);
cudaError_t launch_schur_sp64(const SolveArgs &a, const OpTable &ops, int SM, int RMAX, int wpb, int num_sms,
                              cudaStream_t st);
// Stencils of 33..48 nodes with at most 16 monomials (weights_reg48_r<RMAX>.cu).
cudaError_t launch_schur_48_16_4(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st);
cudaError_t launch_schur_48_16_8(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st);
size_t schur_smem_per_warp(int SP, int SM, int max_n, int max_m, int nops);
// The four 64-node instantiations, one per translation unit (weights_reg64_m<SM>_r<RMAX>.cu).
cudaError_t launch_schur_64_16_4(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st);
cudaError_t launch_schur_64_16_8(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st);
cudaError_t launch_schur_64_32_4(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st);
cudaError_t launch_schur_64_32_8(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms, cudaStream_t st);
