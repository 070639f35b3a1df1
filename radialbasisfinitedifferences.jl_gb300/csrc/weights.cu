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
// The FP64 kernel does all of it in FP64.  The mixed kernel assembles and factors in FP32,
// then refines in FP64: residual b - A x with A assembled in FP64, correction solved with
// the FP32 factors, until the predicted relative weight error is below refine_tol; a
// system whose refinement stalls is queued for the FP64 kernel.
#include <float.h>
#include <limits.h>
#include <math_constants.h>

#include "rbffd_internal.cuh"

namespace {

constexpr double EPS64 = 2.220446049250313e-16;  // Julia eps(Float64)

__host__ __device__ __forceinline__ int npoly(int d) { return (d + 1) * (d + 2) / 2; }
__host__ __device__ __forceinline__ size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }
__host__ __device__ __forceinline__ int lda_of(int s) { return s | 1; }

// Per-warp shared-memory carve-up (same computation on host and device).
struct Layout {
    size_t A, A32, xs, B, X, R32, dinv, piv, pinv, sid, total;
};

__host__ __device__ inline Layout make_layout(int max_s, int max_n, int nops, bool mixed)
{
    Layout L;
    size_t o = 0;
    int ld = lda_of(max_s);
    L.A = o;
    o += al16(sizeof(double) * max_s * ld);
    L.A32 = o;
    if (mixed) o += al16(sizeof(float) * max_s * ld);
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
    L.total = o;
    return L;
}

__device__ __forceinline__ double ipow(double x, int e)
{
    double r = 1.0;
    for (int i = 0; i < e; i++) r *= x;
    return r;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(RBFFD_FULL, v, o));
    return v;
}

// phi = r^p from r^2 (odd p: r^(p-1) * r; even p: r^2^(p/2)).
__device__ __forceinline__ double phi64(double r2, int p)
{
    double v = ipow(r2, p >> 1);
    return (p & 1) ? v * sqrt(r2) : v;
}

__device__ __forceinline__ float phi32(float r2, int p)
{
    float v = 1.0f;
    for (int i = 0; i < (p >> 1); i++) v *= r2;
    return (p & 1) ? v * sqrtf(r2) : v;
}

// (i, j), 0 <= i < j < n, of the t-th upper-triangle pair in row-major order.
__device__ __forceinline__ void tri_pair(int t, int n, int &i, int &j)
{
    // row start of row i: i*n - i*(i+1)/2
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
template <typename T>
__device__ __forceinline__ void monomial_row(T x, T y, int deg, T *row, int stride)
{
    T xp[RBFFD_MAX_DEG + 1], yp[RBFFD_MAX_DEG + 1];
    xp[0] = 1;
    yp[0] = 1;
#pragma unroll
    for (int e = 1; e <= RBFFD_MAX_DEG; e++) {
        xp[e] = xp[e - 1] * x;
        yp[e] = yp[e - 1] * y;
    }
    int l = 0;
    for (int t = 0; t <= deg; t++)
        for (int a = t; a >= 0; a--) {
            T v = 1;
#pragma unroll
            for (int e = 0; e <= RBFFD_MAX_DEG; e++)
                if (e == a) v = xp[e];
#pragma unroll
            for (int e = 0; e <= RBFFD_MAX_DEG; e++)
                if (e == t - a) v *= yp[e];
            row[(size_t)l * stride] = v;
            l++;
        }
}

// ---------------------------------------------------------------------------
// Warp LU with partial pivoting on an s x s row-major matrix in shared memory.
// Full-row interchanges as in LAPACK getf2; multipliers scaled by the reciprocal pivot.
// Returns false (warp-uniform) on a zero / non-finite pivot.
// ---------------------------------------------------------------------------
template <typename T>
__device__ bool warp_lu(T *A, int lda, int s, int *piv, T *dinv, int lane)
{
    for (int c = 0; c < s; c++) {
        T best = (T)-1;
        int bi = c;
        for (int i = c + lane; i < s; i += 32) {
            T v = fabs(A[i * lda + c]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            T ob = __shfl_xor_sync(RBFFD_FULL, best, o);
            int oi = __shfl_xor_sync(RBFFD_FULL, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (!(best > (T)0) || isinf(best)) return false;
        if (lane == 0) piv[c] = bi;
        if (bi != c)
            for (int j = lane; j < s; j += 32) {
                T t = A[c * lda + j];
                A[c * lda + j] = A[bi * lda + j];
                A[bi * lda + j] = t;
            }
        __syncwarp();
        T rinv = (T)1 / A[c * lda + c];
        if (lane == 0) dinv[c] = rinv;
        for (int i = c + 1 + lane; i < s; i += 32) A[i * lda + c] *= rinv;
        __syncwarp();
        int nr = s - c - 1;
        if (nr > 0) {
            int tot = nr * nr;
            int q = lane / nr, r = lane - q * nr;
            int dq = 32 / nr, dr = 32 - dq * nr;
            const T *rowc = A + c * lda + c + 1;
            for (int t = lane; t < tot; t += 32) {
                T *rowi = A + (c + 1 + q) * lda;
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

// Row permutation of the factorisation: pinv[i] = position of original row i.
__device__ __forceinline__ void make_pinv(const int *piv, int *pinv, int s, int lane)
{
    if (lane == 0) {
        for (int i = 0; i < s; i++) pinv[i] = i;
        // perm[c] = original row at position c; built by applying the interchanges
        for (int c = 0; c < s; c++) {
            int p = piv[c];
            if (p != c) {
                int t = pinv[c];
                pinv[c] = pinv[p];
                pinv[p] = t;
            }
        }
        // pinv currently holds perm; invert in place via a scratch pass
    }
    __syncwarp();
    // invert: perm -> pinv.  Each lane reads perm entries first, then writes.
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

// Forward/backward substitution with the LU factors on B (s x r, row-major, rows already
// in pivot order).  TB is the type of the right-hand sides.
template <typename T, typename TB>
__device__ void warp_lu_solve(const T *A, int lda, int s, const T *dinv, TB *B, int r, int lane)
{
    for (int c = 0; c < s - 1; c++) {
        int tot = (s - c - 1) * r;
        for (int t = lane; t < tot; t += 32) {
            int i = c + 1 + t / r, q = t - (t / r) * r;
            B[i * r + q] = fma(-(TB)A[i * lda + c], B[c * r + q], B[i * r + q]);
        }
        __syncwarp();
    }
    for (int c = s - 1; c >= 0; c--) {
        for (int q = lane; q < r; q += 32) B[c * r + q] *= (TB)dinv[c];
        __syncwarp();
        int tot = c * r;
        for (int t = lane; t < tot; t += 32) {
            int i = t / r, q = t - i * r;
            B[i * r + q] = fma(-(TB)A[i * lda + c], B[c * r + q], B[i * r + q]);
        }
        __syncwarp();
    }
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
        mx = fmax(mx, fabs(dx));
        my = fmax(my, fabs(dy));
    }
    if (a.unscaled_overload) {
        sx = sy = 1.0;
        __syncwarp();
        if (lane == 0) {
            xs[0] = EPS64;  // src/generate_operator.jl:410
            xs[1] = EPS64;
        }
    } else {
        mx = warp_max(mx);
        my = warp_max(my);
        sx = 1.0 / mx;
        sy = 1.0 / my;
        for (int l = lane; l < n; l += 32) {
            xs[2 * l] *= sx;
            xs[2 * l + 1] *= sy;
        }
    }
    __syncwarp();
}

// A = [Phi P; P' 0] in FP64.
__device__ __forceinline__ void assemble64(double *A, int lda, const double *xs, int n, int m,
                                           int deg, int p, int lane)
{
    int s = n + m;
    int npairs = n * (n - 1) / 2;
    for (int t = lane; t < npairs; t += 32) {
        int i, j;
        tri_pair(t, n, i, j);
        double dx = xs[2 * i] - xs[2 * j], dy = xs[2 * i + 1] - xs[2 * j + 1];
        double v = phi64(dx * dx + dy * dy, p);
        A[i * lda + j] = v;
        A[j * lda + i] = v;
    }
    for (int i = lane; i < n; i += 32) {
        A[i * lda + i] = 0.0;
        monomial_row<double>(xs[2 * i], xs[2 * i + 1], deg, A + i * lda + n, 1);
        monomial_row<double>(xs[2 * i], xs[2 * i + 1], deg, A + n * lda + i, lda);
    }
    for (int t = lane; t < m * m; t += 32) {
        int i = t / m, j = t - i * m;
        A[(n + i) * lda + n + j] = 0.0;
    }
    (void)s;
    __syncwarp();
}

// A32 = [Phi P; P' 0] in FP32 from FP32 coordinates.
__device__ __forceinline__ void assemble32(float *A, int lda, const double *xs, int n, int m,
                                           int deg, int p, int lane)
{
    int npairs = n * (n - 1) / 2;
    for (int t = lane; t < npairs; t += 32) {
        int i, j;
        tri_pair(t, n, i, j);
        float dx = (float)xs[2 * i] - (float)xs[2 * j], dy = (float)xs[2 * i + 1] - (float)xs[2 * j + 1];
        float v = phi32(dx * dx + dy * dy, p);
        A[i * lda + j] = v;
        A[j * lda + i] = v;
    }
    for (int i = lane; i < n; i += 32) {
        A[i * lda + i] = 0.0f;
        float x = (float)xs[2 * i], y = (float)xs[2 * i + 1];
        monomial_row<float>(x, y, deg, A + i * lda + n, 1);
        monomial_row<float>(x, y, deg, A + n * lda + i, lda);
    }
    for (int t = lane; t < m * m; t += 32) {
        int i = t / m, j = t - i * m;
        A[(n + i) * lda + n + j] = 0.0f;
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
__device__ __forceinline__ void build_rhs(const OpTable &ops, const double *xs, int n, int m, int deg,
                                          double yx, double yy, double sx, double sy,
                                          int unscaled, const int *pinv, double *B, int lane)
{
    int r = ops.nops;
    for (int i = lane; i < n; i += 32) {
        double cx, cy;
        if (unscaled) {
            cx = xs[2 * i];
            cy = xs[2 * i + 1];
        } else {
            cx = yx - xs[2 * i];
            cy = yy - xs[2 * i + 1];
            if (cx == 0.0) cx = EPS64;
            if (cy == 0.0) cy = EPS64;
        }
        double rr = sqrt(cx * cx + cy * cy);
        double rinv = 1.0 / rr;
        int row = pinv ? pinv[i] : i;
        for (int q = 0; q < r; q++) {
            const OpDesc &od = ops.op[q];
            double v = 0.0;
            for (int cidx = 0; cidx < od.ncomp; cidx++) {
                const OpComp &oc = od.c[cidx];
                double cv = 0.0;
                for (int t = 0; t < oc.nterm; t++) {
                    const RbfTerm &tm = oc.t[t];
                    double tv = tm.coef * ipow(cx, tm.ex) * ipow(cy, tm.ey);
                    tv *= tm.er >= 0 ? ipow(rr, tm.er) : ipow(rinv, -tm.er);
                    cv += tv;
                }
                if (od.ncomp > 1) cv *= ipow(sx, oc.a) * ipow(sy, oc.b);
                v += cv;
            }
            B[row * r + q] = v;
        }
    }
    for (int l = lane; l < m; l += 32) {
        // monomial l: t = degree, a = x exponent
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
    (void)deg;
    __syncwarp();
}

// Write the first n solution rows of every operator, unscaled, into the CSR row.
__device__ __forceinline__ void write_row(const SolveArgs &a, const OpTable &ops, int64_t row,
                                          const double *Xs, int n, const int *sid, double sx,
                                          double sy, int lane)
{
    int64_t off = a.row_ptr[row - a.row_begin];
    int r = ops.nops;
    for (int l = lane; l < n; l += 32) a.col[off + l] = sid[l];
    for (int q = 0; q < r; q++) {
        const OpDesc &od = ops.op[q];
        double f = 1.0;
        if (od.post_scale) f = ipow(sx, od.c[0].a) * ipow(sy, od.c[0].b);
        double *dst = a.val + (int64_t)q * a.nnz + off;
        for (int l = lane; l < n; l += 32) dst[l] = f * Xs[l * r + q];
    }
}

__device__ __forceinline__ void system_rows(const SolveArgs &a, int64_t sys, int j, int64_t &r0,
                                            int64_t &r1)
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

// ---------------------------------------------------------------------------
// FP64 kernel.  Systems: a.sys_node[sys] for sys in [0, nsys), or the subset list.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) solve_fp64_kernel(SolveArgs a, OpTable ops,
                                                         const int32_t *subset,
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
    for (int64_t w = gw; w < nwork; w += nw) {
        int64_t sys = subset ? (int64_t)subset[w] : w;
        int j = a.sys_node[sys];
        int n = a.n_node ? a.n_node[j] : a.n;
        int deg = a.deg_node ? a.deg_node[j] : a.deg;
        int m = npoly(deg), s = n + m, lda = lda_of(s);
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        assemble64(A, lda, xs, n, m, deg, ops.p, lane);
        bool ok = warp_lu<double>(A, lda, s, piv, dinv, lane);
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
            build_rhs(ops, xs, n, m, deg, yx, yy, sx, sy, a.unscaled_overload, pinv, B, lane);
            warp_lu_solve<double, double>(A, lda, s, dinv, B, ops.nops, lane);
            write_row(a, ops, row, B, n, sid, sx, sy, lane);
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed-precision kernel.
// ---------------------------------------------------------------------------
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
    int *piv = (int *)(base + L.piv);
    int *pinv = (int *)(base + L.pinv);
    int *sid = (int *)(base + L.sid);
    const int r = ops.nops;

    int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sys = gw; sys < a.nsys; sys += nw) {
        int j = a.sys_node[sys];
        int n = a.n_node ? a.n_node[j] : a.n;
        int deg = a.deg_node ? a.deg_node[j] : a.deg;
        int m = npoly(deg), s = n + m, lda = lda_of(s);
        double2 xc;
        double sx, sy;
        load_stencil(a, j, n, xs, sid, xc, sx, sy, lane);
        assemble32(A32, lda, xs, n, m, deg, ops.p, lane);
        bool ok = warp_lu<float>(A32, lda, s, piv, dinv32, lane);
        bool fallback = !ok;
        if (ok) {
            assemble64(A, lda, xs, n, m, deg, ops.p, lane);
            __syncwarp();
            make_pinv(piv, pinv, s, lane);
        }
        int64_t r0, r1;
        system_rows(a, sys, j, r0, r1);
        int iters_max = 0;
        for (int64_t t = r0; t < r1 && !fallback; t++) {
            int64_t row = row_id(a, t);
            double yx, yy;
            {
                double2 yp = eval_point(a, row);
                yx = (yp.x - xc.x) * sx;
                yy = (yp.y - xc.y) * sy;
            }
            // b in original row order
            build_rhs(ops, xs, n, m, deg, yx, yy, sx, sy, 0, nullptr, B, lane);
            for (int e = lane; e < s * r; e += 32) X[e] = 0.0;
            __syncwarp();
            double e_prev = 1.0;
            bool conv = false;
            int it;
            for (it = 0; it < a.max_refine; it++) {
                // residual (x = 0 at it 0) -> FP32 in pivot order
                if (it == 0) {
                    for (int e = lane; e < s * r; e += 32) {
                        int i = e / r, q = e - i * r;
                        R32[pinv[i] * r + q] = (float)B[e];
                    }
                } else {
                    for (int e = lane; e < s * r; e += 32) {
                        int i = e / r, q = e - i * r;
                        double acc = B[e];
                        const double *Ai = A + i * lda;
                        int jmax = i < n ? s : n;  // the m x m block is zero
                        for (int jj = 0; jj < jmax; jj++) acc = fma(-Ai[jj], X[jj * r + q], acc);
                        R32[pinv[i] * r + q] = (float)acc;
                    }
                }
                __syncwarp();
                warp_lu_solve<float, float>(A32, lda, s, dinv32, R32, r, lane);
                // x += d; relative size of the correction over the weight rows
                double dmax = 0.0, xmax = 0.0;
                for (int e = lane; e < s * r; e += 32) {
                    double d = (double)R32[e];
                    double xv = X[e] + d;
                    X[e] = xv;
                    if (e < n * r) {
                        dmax = fmax(dmax, fabs(d));
                        xmax = fmax(xmax, fabs(xv));
                    }
                }
                dmax = warp_max(dmax);
                xmax = warp_max(xmax);
                __syncwarp();
                double e_cur = xmax > 0.0 ? dmax / xmax : 0.0;
                if (!(e_cur == e_cur)) break;  // NaN
                if (it >= 1) {
                    double rho = e_prev > 0.0 ? e_cur / e_prev : 0.0;
                    if (rho * e_cur <= a.refine_tol || e_cur == 0.0) {
                        conv = true;
                        break;
                    }
                    if (rho > 0.5) break;  // stalled
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
    size_t per = solve_fp64_smem_per_warp(a.max_s, a.max_n, ops.nops);
    size_t smem = per * wpb;
    cudaError_t e = cudaFuncSetAttribute(solve_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, solve_fp64_kernel, wpb * 32, smem);
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int64_t want = (nwork_hint + wpb - 1) / wpb;
    int64_t cap = (int64_t)num_sms * occ;
    int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    solve_fp64_kernel<<<blocks, wpb * 32, smem, st>>>(a, ops, subset, subset_count);
    return cudaGetLastError();
}

cudaError_t launch_solve_fp64(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms,
                              cudaStream_t st)
{
    if (a.nsys <= 0) return cudaSuccess;
    return launch_fp64_impl(a, ops, wpb, num_sms, st, nullptr, nullptr, a.nsys);
}

// FP64 re-solve of the systems the mixed kernel queued (count read on the device).
cudaError_t launch_solve_fp64_subset(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms,
                                     cudaStream_t st, int64_t count)
{
    if (count <= 0) return cudaSuccess;
    return launch_fp64_impl(a, ops, wpb, num_sms, st, a.fallback_list, a.fallback_count, count);
}

cudaError_t launch_solve_mixed(const SolveArgs &a, const OpTable &ops, int wpb, int num_sms,
                               cudaStream_t st)
{
    if (a.nsys <= 0) return cudaSuccess;
    size_t per = solve_mixed_smem_per_warp(a.max_s, a.max_n, ops.nops);
    size_t smem = per * wpb;
    cudaError_t e = cudaFuncSetAttribute(solve_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, solve_mixed_kernel, wpb * 32, smem);
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int64_t want = (a.nsys + wpb - 1) / wpb;
    int64_t cap = (int64_t)num_sms * occ;
    int blocks = (int)(want < cap ? want : cap);
    solve_mixed_kernel<<<blocks, wpb * 32, smem, st>>>(a, ops);
    return cudaGetLastError();
}
