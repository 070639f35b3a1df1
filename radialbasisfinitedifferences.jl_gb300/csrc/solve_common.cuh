// Device helpers shared by the weight-solve translation units (weights.cu, weights_reg.cu):
// shared-memory layouts, basis functions, stencil gather and scaling, FP64 assembly, the
// right-hand sides of the operators, the FP64 and lane-per-row FP32 factorisations and the
// CSR row writer.  See weights.cu for the algorithm.
#pragma once

#include <float.h>
#include <limits.h>
#include <math_constants.h>

#include "rbffd_internal.cuh"

namespace {

constexpr double EPS64 = 2.220446049250313e-16;  // Julia eps(Float64)
constexpr int NOTYET = 0x7fffffff;                // pivot step of a row not yet eliminated

__host__ __device__ __forceinline__ int npoly(int d) { return (d + 1) * (d + 2) / 2; }
__host__ __device__ __forceinline__ size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }
// FP64 leading dimension: odd, so that a column walk is bank-conflict free.
__host__ __device__ __forceinline__ int lda64_of(int s) { return s | 1; }
// FP32 lane-per-row leading dimension: a multiple of 4 floats (16-byte rows for LDS.128)
// with an odd number of 16-byte groups.
__host__ __device__ __forceinline__ int lda32_of(int s) { return 4 * (((s + 3) >> 2) | 1); }

// Per-warp shared-memory carve-up (same computation on host and device).
struct Layout {
    size_t A, A32, xs, B, X, R32, dinv, piv, pinv, sid, prow, total;
};

__host__ __device__ inline Layout make_layout(int max_s, int max_n, int nops, bool mixed)
{
    Layout L;
    size_t o = 0;
    L.A = o;
    o += al16(sizeof(double) * max_s * lda64_of(max_s));
    L.A32 = o;
    if (mixed) o += al16(sizeof(float) * max_s * lda32_of(max_s));
    L.xs = o;
    o += al16(sizeof(double) * 2 * max_n);
    L.B = o;
    o += al16(sizeof(double) * max_s * nops);
    L.X = o;
    if (mixed) o += al16(sizeof(double) * max_s * nops);
    L.R32 = o;
    if (mixed) o += al16(sizeof(float) * max_s * nops);
    L.dinv = o;
    o += al16(sizeof(double) * max_s);
    L.piv = o;
    o += al16(sizeof(int) * max_s);
    L.pinv = o;
    o += al16(sizeof(int) * max_s);
    L.sid = o;
    o += al16(sizeof(int) * max_n);
    L.prow = o;
    if (mixed) o += al16(sizeof(float) * (lda32_of(max_s) + 4));
    L.total = o;
    return L;
}

__device__ __forceinline__ double ipow(double x, int e)
{
    double r = 1.0;
    for (int i = 0; i < e; i++) r *= x;
    return r;
}

// |x| as an ordered unsigned key (integer pipe; no FP64 comparison instruction).
__device__ __forceinline__ unsigned long long abs_key(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

__device__ __forceinline__ double warp_max_abs(double v)
{
    unsigned long long k = abs_key(v);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(RBFFD_FULL, k, o);
        k = t > k ? t : k;
    }
    return __longlong_as_double((long long)k);
}

__device__ __forceinline__ float warp_max_f(float v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(RBFFD_FULL, v, o));
    return v;
}

__device__ __forceinline__ bool is_zero64(double x) { return abs_key(x) == 0ull; }
// 2 x for a normal double (exponent field + 1, integer pipe); zero, subnormal and
// non-finite x take the FP64 addition.
__device__ __forceinline__ double twice64(double x)
{
    const int hi = __double2hiint(x);
    const unsigned ex = ((unsigned)hi >> 20) & 0x7ffu;
    if (ex == 0u || ex >= 0x7feu) return x + x;
    return __hiloint2double(hi + (1 << 20), __double2loint(x));
}

// -x by flipping the sign bit (integer pipe; exact, like the FP64 negation)
__device__ __forceinline__ double neg64(double x)
{
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}

// sqrt(a) for a positive normal double, without a library call: an FP32 reciprocal square
// root of the mantissa (exponent split off on the integer pipe, a = a' 4^k with a' in [1, 4))
// seeds Heron's iteration s <- s + (a - s^2) / (2 s), with 1 / (2 s) taken from the seed;
// the error goes 2^-22 -> 2^-44 -> below FP64 rounding.  y0 returns the seed (~1/sqrt(a)).
__device__ __forceinline__ double sqrt_nr(double a, double &y0)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const int ex = (int)((hi >> 20) & 0x7ffu) - 1023;
    const int k = ex >> 1;  // floor(ex / 2)
    const unsigned fb = ((unsigned)(ex - 2 * k + 127) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const float yf = rsqrtf(__uint_as_float(fb));
    const double yd = f32_to_f64(yf);
    y0 = __hiloint2double(__double2hiint(yd) - k * (1 << 20), __double2loint(yd));  // yf 2^-k
    const double h = __hiloint2double(__double2hiint(y0) - (1 << 20), __double2loint(y0));  // y0 / 2
    double s = a * y0;
    s = fma(fma(-s, s, a), h, s);
    return fma(fma(-s, s, a), h, s);
}

// 1/s from a seed y0 ~ 1/s (relative error ~2^-22) by two Newton-Raphson steps
// y <- y + y (1 - s y).
__device__ __forceinline__ double recip_nr(double s, double y0)
{
    double y = fma(y0, fma(-s, y0, 1.0), y0);
    return fma(y, fma(-s, y, 1.0), y);
}

// 1/a for a finite nonzero double: FP32 reciprocal of the mantissa (the exponent split off on
// the integer pipe) refined by two Newton-Raphson steps y <- y + y (1 - a y), error
// 2^-22 -> 2^-44 -> rounding level; subnormal a takes the division.
__device__ __forceinline__ double recip64(double a)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const int ex = (int)((hi >> 20) & 0x7ffu) - 1023;
    if (ex == -1023) return 1.0 / a;
    const unsigned fb = (hi & 0x80000000u) | (127u << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const float yf = __fdividef(1.0f, __uint_as_float(fb));  // mantissa in [1, 2): |yf| in (0.5, 1]
    const double yd = f32_to_f64(yf);
    double y = __hiloint2double(__double2hiint(yd) - ex * (1 << 20), __double2loint(yd));
    y = fma(y, fma(-a, y, 1.0), y);
    return fma(y, fma(-a, y, 1.0), y);
}

// phi = r^p from r^2 without library calls.
__device__ __forceinline__ double phi64_nr(double r2, int p)
{
    double v = r2;
    for (int i = 1; i < (p >> 1); i++) v *= r2;
    if (p < 2) v = 1.0;
    if (p & 1) {
        double y0;
        const double rt = sqrt_nr(r2, y0);
        v *= rt;
    }
    // r^p of a subnormal r^2 underflows to 0 in FP64.  r2 >= +0, so r2 >= DBL_MIN exactly when
    // its high word (sign 0) reaches the smallest normal exponent: an integer compare instead
    // of an FP64 one.
    return __double2hiint(r2) >= 0x00100000 ? v : 0.0;
}

// phi = r^p from r^2 (odd p: r^(p-1) * r; even p: (r^2)^(p/2)).
__device__ __forceinline__ double phi64(double r2, int p)
{
    double v = r2;
    for (int i = 1; i < (p >> 1); i++) v *= r2;
    if (p < 2) v = 1.0;
    return (p & 1) ? v * sqrt(r2) : v;
}

__device__ __forceinline__ float phi32(float r2, int p)
{
    float r = r2 > 0.0f ? r2 * rsqrtf(r2) : 0.0f;
    float v = (p & 1) ? r : 1.0f;
    for (int i = 0; i < (p >> 1); i++) v *= r2;
    return v;
}

// (i, j), 0 <= i < j < n, of the t-th upper-triangle pair in row-major order.
__device__ __forceinline__ void tri_pair(int t, int n, int &i, int &j)
{
    float nn = 2.0f * n - 1.0f;
    int ii = (int)((nn - sqrtf(nn * nn - 8.0f * t)) * 0.5f);
    if (ii < 0) ii = 0;
    if (ii > n - 2) ii = n - 2;
    while (ii > 0 && ii * n - ii * (ii + 1) / 2 > t) ii--;
    while (ii < n - 2 && (ii + 1) * n - (ii + 1) * (ii + 2) / 2 <= t) ii++;
    i = ii;
    j = t - (ii * n - ii * (ii + 1) / 2) + ii + 1;
}

// Monomials of total degree <= deg at (x, y), order t = 0..deg, a = t..0: x^a y^(t-a).
// One multiply per monomial: within a degree, x^a y^(t-a) = x^(a+1) y^(t-a-1) * (y / x) is
// avoided (x may be 0); instead each degree starts from x^t and swaps one x for one y.
template <typename T>
__device__ __forceinline__ void monomial_row(T x, T y, int deg, T *row, int stride)
{
    T xp[RBFFD_MAX_DEG + 1], yp[RBFFD_MAX_DEG + 1];
    xp[0] = (T)1;
    yp[0] = (T)1;
#pragma unroll
    for (int e = 1; e <= RBFFD_MAX_DEG; e++) {
        if (e <= deg) {
            xp[e] = xp[e - 1] * x;
            yp[e] = yp[e - 1] * y;
        }
    }
    int l = 0;
#pragma unroll
    for (int t = 0; t <= RBFFD_MAX_DEG; t++) {
        if (t > deg) break;
#pragma unroll
        for (int a = t; a >= 0; a--) {
            T v = (a == 0) ? yp[t] : ((t - a == 0) ? xp[a] : xp[a] * yp[t - a]);
            row[(size_t)l * stride] = v;
            l++;
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 warp LU with partial pivoting on an s x s row-major matrix in shared memory.
// Full-row interchanges as in LAPACK getf2, multipliers scaled by the reciprocal pivot;
// the trailing update is distributed over (row, column) pairs so that every DFMA
// instruction is lane-full.  Returns false (warp-uniform) on a zero / non-finite pivot.
// ---------------------------------------------------------------------------
__device__ bool warp_lu64(double *A, int lda, int s, int *piv, double *dinv, int lane)
{
    for (int c = 0; c < s; c++) {
        unsigned long long best = 0;
        int bi = c;
        for (int i = c + lane; i < s; i += 32) {
            unsigned long long v = abs_key(A[i * lda + c]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            unsigned long long ob = __shfl_xor_sync(RBFFD_FULL, best, o);
            int oi = __shfl_xor_sync(RBFFD_FULL, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        // zero, inf or NaN pivot: singular (NaN keys exceed the inf key)
        if (best == 0ull || best >= 0x7ff0000000000000ull) return false;
        if (lane == 0) piv[c] = bi;
        if (bi != c)
            for (int j = lane; j < s; j += 32) {
                double t = A[c * lda + j];
                A[c * lda + j] = A[bi * lda + j];
                A[bi * lda + j] = t;
            }
        __syncwarp();
        double rinv = recip64(A[c * lda + c]);
        if (lane == 0) dinv[c] = rinv;
        for (int i = c + 1 + lane; i < s; i += 32) A[i * lda + c] *= rinv;
        __syncwarp();
        int nr = s - c - 1;
        if (nr > 0) {
            int tot = nr * nr;
            int q = lane / nr, r = lane - q * nr;
            int dq = 32 / nr, dr = 32 - dq * nr;
            const double *rowc = A + c * lda + c + 1;
            for (int t = lane; t < tot; t += 32) {
                double *rowi = A + (c + 1 + q) * lda;
                rowi[c + 1 + r] = fma(-rowi[c], rowc[r], rowi[c + 1 + r]);
                r += dr;
                q += dq;
                if (r >= nr) {
                    r -= nr;
                    q++;
                }
            }
        }
        __syncwarp();
    }
    return true;
}

// Row permutation of the FP64 factorisation: pinv[i] = position of original row i.
__device__ __forceinline__ void make_pinv(const int *piv, int *pinv, int s, int lane)
{
    if (lane == 0) {
        for (int i = 0; i < s; i++) pinv[i] = i;
        for (int c = 0; c < s; c++) {
            int p = piv[c];
            if (p != c) {
                int t = pinv[c];
                pinv[c] = pinv[p];
                pinv[p] = t;
            }
        }
    }
    __syncwarp();
    int pv[RBFFD_MAX_S / 32];
#pragma unroll
    for (int k = 0; k < RBFFD_MAX_S / 32; k++) {
        int c = lane + 32 * k;
        pv[k] = c < s ? pinv[c] : 0;
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < RBFFD_MAX_S / 32; k++) {
        int c = lane + 32 * k;
        if (c < s) pinv[pv[k]] = c;
    }
    __syncwarp();
}

// Forward/backward substitution with the FP64 LU factors on B (s x r, row-major, rows
// already in pivot order), lane-full over (row, column) pairs.
__device__ void warp_lu_solve64(const double *A, int lda, int s, const double *dinv, double *B, int r,
                                int lane)
{
    for (int c = 0; c < s - 1; c++) {
        int tot = (s - c - 1) * r;
        for (int t = lane; t < tot; t += 32) {
            int i = c + 1 + t / r, q = t - (t / r) * r;
            B[i * r + q] = fma(-A[i * lda + c], B[c * r + q], B[i * r + q]);
        }
        __syncwarp();
    }
    for (int c = s - 1; c >= 0; c--) {
        for (int q = lane; q < r; q += 32) B[c * r + q] *= dinv[c];
        __syncwarp();
        int tot = c * r;
        for (int t = lane; t < tot; t += 32) {
            int i = t / r, q = t - i * r;
            B[i * r + q] = fma(-A[i * lda + c], B[c * r + q], B[i * r + q]);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// FP32 LU, one row per lane (rows lane, lane+32, ... ; NS slots), matrix in shared memory
// with 16-byte rows.  Virtual pivoting: rows never move; ps[k] records the step at which the
// row in slot k became the pivot (NOTYET before).  perm[c] = pivot row of step c and
// dinv[c] = 1 / U[c][c].  The pivot row is copied to prow (entries <= c zeroed) so that
// every other row updates itself with broadcast LDS.128 reads and FMAs.
// ---------------------------------------------------------------------------
template <int NS>
__device__ __forceinline__ bool warp_lu32_rows(float *A, int lda, int s, int *ps, int *perm, float *dinv, float *prow,
                               int lane)
{
    for (int c = 0; c < s; c++) {
        float best = -1.0f;
        int bi = INT_MAX;
#pragma unroll
        for (int k = 0; k < NS; k++) {
            int i = lane + 32 * k;
            if (i < s && ps[k] == NOTYET) {
                float v = fabsf(A[i * lda + c]);
                if (v > best) {  // rows ascend with k: first maximum kept
                    best = v;
                    bi = i;
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
        if (!(best > 0.0f) || isinf(best)) return false;
        // copy the pivot row (columns >= c; zeros below c so the vector update skips them)
        const float *src = A + bi * lda;
        int c4 = c & ~3;
        for (int j = c4 + lane; j < lda; j += 32) prow[j] = j > c ? src[j] : 0.0f;
        if (lane == 0) {
            perm[c] = bi;
            dinv[c] = 1.0f / src[c];
        }
#pragma unroll
        for (int k = 0; k < NS; k++)
            if (lane + 32 * k == bi) ps[k] = c;
        __syncwarp();
        float rinv = 1.0f / src[c];
#pragma unroll
        for (int k = 0; k < NS; k++) {
            int i = lane + 32 * k;
            if (i < s && ps[k] == NOTYET) {
                float *row = A + i * lda;
                float l = row[c] * rinv;
                const float4 *p4 = reinterpret_cast<const float4 *>(prow);
                float4 *r4 = reinterpret_cast<float4 *>(row);
                for (int j4 = c4 >> 2; j4 < (lda >> 2); j4++) {
                    float4 a = r4[j4], b = p4[j4];
                    a.x = fmaf(-l, b.x, a.x);
                    a.y = fmaf(-l, b.y, a.y);
                    a.z = fmaf(-l, b.z, a.z);
                    a.w = fmaf(-l, b.w, a.w);
                    r4[j4] = a;
                }
                row[c] = l;
            }
        }
        __syncwarp();
    }
    return true;
}

// Solve with the lane-per-row FP32 factors.  R (s x r floats, row-major, original row
// order) holds the right-hand sides on entry and the solution (by variable) on exit.
template <int NS, int RMAX>
__device__ __forceinline__ void warp_lu32_rows_solve(const float *A, int lda, int s, const int *ps, const int *perm,
                                     const float *dinv, float *R, int r, int lane)
{
    float b[NS][RMAX];
#pragma unroll
    for (int k = 0; k < NS; k++) {
        int i = lane + 32 * k;
#pragma unroll
        for (int q = 0; q < RMAX; q++) b[k][q] = (i < s && q < r) ? R[i * r + q] : 0.0f;
    }
    __syncwarp();
    // forward: rows still active at step c subtract L[i][c] * y_c
    for (int c = 0; c < s; c++) {
        int p = perm[c];
        int pl = p & 31, pk = p >> 5;
#pragma unroll
        for (int q = 0; q < RMAX; q++) {
            if (q >= r) break;
            float v = b[0][q];
#pragma unroll
            for (int k = 1; k < NS; k++)
                if (pk == k) v = b[k][q];
            float y = __shfl_sync(RBFFD_FULL, v, pl);
#pragma unroll
            for (int k = 0; k < NS; k++) {
                int i = lane + 32 * k;
                if (i < s && ps[k] > c) b[k][q] = fmaf(-A[i * lda + c], y, b[k][q]);
            }
        }
    }
    // backward: x_c = b[perm[c]] / U[c][c]; earlier pivot rows subtract U[i][c] * x_c
    for (int c = s - 1; c >= 0; c--) {
        int p = perm[c];
        int pl = p & 31, pk = p >> 5;
        float dv = dinv[c];
#pragma unroll
        for (int q = 0; q < RMAX; q++) {
            if (q >= r) break;
            float v = b[0][q];
#pragma unroll
            for (int k = 1; k < NS; k++)
                if (pk == k) v = b[k][q];
            float x = __shfl_sync(RBFFD_FULL, v, pl) * dv;
            if (lane == 0) R[c * r + q] = x;
#pragma unroll
            for (int k = 0; k < NS; k++) {
                int i = lane + 32 * k;
                if (i < s && ps[k] < c) b[k][q] = fmaf(-A[i * lda + c], x, b[k][q]);
            }
        }
    }
    __syncwarp();
}

// Stencil gather and scalestencil.  Writes xs (2n, scaled coordinates) and sid (n).
__device__ __forceinline__ void load_stencil(const SolveArgs &a, int j, int n, double *xs, int *sid,
                                             double2 &xc, double &sx, double &sy, int lane)
{
    const int32_t *nb = a.nbr + (a.nbr_ptr ? a.nbr_ptr[j] : (int64_t)j * a.n);
    xc = a.unscaled_overload ? a.X[nb[0]] : a.X[j];
    double mx = 0.0, my = 0.0;
    for (int l = lane; l < n; l += 32) {
        int id = nb[l];
        sid[l] = id;
        double2 p = a.X[id];
        double dx = p.x - xc.x, dy = p.y - xc.y;
        xs[2 * l] = dx;
        xs[2 * l + 1] = dy;
        if (abs_key(dx) > abs_key(mx)) mx = dx;
        if (abs_key(dy) > abs_key(my)) my = dy;
    }
    if (a.unscaled_overload) {
        sx = sy = 1.0;
        __syncwarp();
        if (lane == 0) {
            xs[0] = EPS64;  // src/generate_operator.jl:410
            xs[1] = EPS64;
        }
    } else {
        mx = warp_max_abs(mx);
        my = warp_max_abs(my);
        sx = recip64(mx);  // 1.0 / max|x_j - x_c| (src/scalestencil.jl:17-18)
        sy = recip64(my);
        for (int l = lane; l < n; l += 32) {
            xs[2 * l] *= sx;
            xs[2 * l + 1] *= sy;
        }
    }
    __syncwarp();
}

// A = [Phi P; P' 0] in FP64 (Phi over the upper triangle, mirrored).
__device__ __forceinline__ void assemble64(double *A, int lda, const double *xs, int n, int m, int deg,
                                           int p, int lane)
{
    int npairs = n * (n - 1) / 2;
    for (int t = lane; t < npairs; t += 32) {
        int i, j;
        tri_pair(t, n, i, j);
        double dx = xs[2 * i] - xs[2 * j], dy = xs[2 * i + 1] - xs[2 * j + 1];
        double v = phi64_nr(fma(dx, dx, dy * dy), p);
        A[i * lda + j] = v;
        A[j * lda + i] = v;
    }
    for (int i = lane; i < n; i += 32) {
        A[i * lda + i] = 0.0;
        monomial_row<double>(xs[2 * i], xs[2 * i + 1], deg, A + i * lda + n, 1);
    }
    __syncwarp();
    // P' rows (copy, no arithmetic) and the zero block
    for (int t = lane; t < m * n; t += 32) {
        int l = t / n, i = t - l * n;
        A[(n + l) * lda + i] = A[i * lda + n + l];
    }
    for (int t = lane; t < m * m; t += 32) {
        int i = t / m, j = t - i * m;
        A[(n + i) * lda + n + j] = 0.0;
    }
    __syncwarp();
}

// A32 = [Phi P; P' 0] in FP32 (lane-per-row layout), from FP32 coordinates in xs32.
__device__ __forceinline__ void assemble32_rows(float *A, int lda, const float2 *xs32, int n, int m,
                                                int deg, int p, int lane)
{
    int s = n + m;
    // Phi and P rows: row i = lane + 32k handles its own row
    for (int i = lane; i < n; i += 32) {
        float2 xi = xs32[i];
        float *row = A + i * lda;
        for (int j = 0; j < n; j++) {
            float2 xj = xs32[j];
            float dx = xi.x - xj.x, dy = xi.y - xj.y;
            row[j] = phi32(fmaf(dx, dx, dy * dy), p);
        }
        monomial_row<float>(xi.x, xi.y, deg, row + n, 1);
        for (int j = s; j < lda; j++) row[j] = 0.0f;
    }
    __syncwarp();
    for (int t = lane; t < m * lda; t += 32) {
        int l = t / lda, j = t - l * lda;
        A[(n + l) * lda + j] = j < n ? A[j * lda + n + l] : 0.0f;
    }
    __syncwarp();
}

__device__ __forceinline__ double falling(int e, int k)
{
    double c = 1.0;
    for (int t = 0; t < k; t++) c *= (double)(e - t);
    return c;
}

// Right-hand sides of one evaluation point y~ (FP64), written to B at row dst(i) for the
// original row i (dst = pinv when B is in pivot order, identity otherwise).
__device__ __forceinline__ void build_rhs(const OpTable &ops, const double *xs, int n, int m,
                                          double yx, double yy, double sx, double sy, int unscaled,
                                          const int *pinv, double *B, int lane)
{
    int r = ops.nops;
    for (int i = lane; i < n; i += 32) {
        double cx, cy;
        if (unscaled) {
            cx = xs[2 * i];
            cy = xs[2 * i + 1];
        } else {
            const bool at0 = is_zero64(yx) && is_zero64(yy);  // the collocated case: a sign flip
            cx = at0 ? neg64(xs[2 * i]) : yx - xs[2 * i];
            cy = at0 ? neg64(xs[2 * i + 1]) : yy - xs[2 * i + 1];
            if (is_zero64(cx)) cx = EPS64;
            if (is_zero64(cy)) cy = EPS64;
        }
        const double r2 = fma(cx, cx, cy * cy);
        double rr, rinv;
        if (r2 >= DBL_MIN && r2 <= 1e300) {
            double y0;
            rr = sqrt_nr(r2, y0);
            rinv = recip_nr(rr, y0);
        } else {
            rr = sqrt(r2);
            rinv = 1.0 / rr;
        }
        int row = pinv ? pinv[i] : i;
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
                if (od.ncomp > 1) cv *= ipow(sx, oc.a) * ipow(sy, oc.b);
                v = cidx == 0 ? cv : v + cv;
            }
            B[row * r + q] = v;
        }
    }
    for (int l = lane; l < m; l += 32) {
        int t = 0, rem = l;
        while (rem > t) {
            rem -= t + 1;
            t++;
        }
        int ea = t - rem, eb = rem;
        int row = pinv ? pinv[n + l] : n + l;
        for (int q = 0; q < r; q++) {
            const OpDesc &od = ops.op[q];
            double v = 0.0;
            for (int cidx = 0; cidx < od.ncomp; cidx++) {
                const OpComp &oc = od.c[cidx];
                if (oc.a > ea || oc.b > eb) continue;
                double cv = falling(ea, oc.a) * falling(eb, oc.b) * ipow(yx, ea - oc.a) * ipow(yy, eb - oc.b);
                if (od.ncomp > 1) cv *= ipow(sx, oc.a) * ipow(sy, oc.b);
                v += cv;
            }
            B[row * r + q] = v;
        }
    }
    __syncwarp();
}

// Write the first n solution rows of every operator, unscaled, into the CSR row.
__device__ __forceinline__ void write_row(const SolveArgs &a, const OpTable &ops, int64_t row,
                                          const double *Xs, int n, const int *sid, double sx, double sy,
                                          int lane)
{
    int64_t off = a.row_ptr[row - a.row_begin];
    int r = ops.nops;
    for (int l = lane; l < n; l += 32) a.col[off + l] = sid[l];
    for (int q = 0; q < r; q++) {
        const OpDesc &od = ops.op[q];
        double *dst = a.val + (int64_t)q * a.nnz;
        const double f = od.post_scale ? ipow(sx, od.c[0].a) * ipow(sy, od.c[0].b) : 1.0;
        for (int l = lane; l < n; l += 32) {
            const int64_t d = a.csc_pos ? (int64_t)a.csc_pos[off + l] : off + l;
            dst[d] = od.post_scale ? f * Xs[l * r + q] : Xs[l * r + q];
        }
    }
}

__device__ __forceinline__ void system_rows(const SolveArgs &a, int64_t sys, int j, int64_t &r0, int64_t &r1)
{
    if (a.sys_rows) {
        r0 = a.sys_rows[sys];
        r1 = a.sys_rows[sys + 1];
    } else {
        r0 = j;
        r1 = (int64_t)j + 1;
    }
}

__device__ __forceinline__ int64_t row_id(const SolveArgs &a, int64_t t)
{
    return a.sys_rows ? (int64_t)a.rows_list[t] : t;
}

__device__ __forceinline__ double2 eval_point(const SolveArgs &a, int64_t row)
{
    return a.Y ? a.Y[row] : a.X[row];
}

}  // namespace
