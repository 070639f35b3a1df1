/*
 * rbffd_oracle.c -- CPU ORACLE for the RBF-FD hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, never the product: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arm load it.  The product path (the CUDA
 * library) never links or calls it.
 *
 * It restates, in plain FP64 C, the algorithm of RadialBasisFiniteDifferences.jl
 * (v0.1.0).  Each function cites the reference file:line it follows.  Compile with
 * -ffp-contract=off so that squared distances are rounded exactly as the CUDA kNN
 * computes them (dx*dx + dy*dy, two roundings, no FMA): kNN index sets are then
 * bit-identical between this file and the GPU.
 *
 * Parity pinning.  The reference is pure Julia; Julia is not installed here, so the
 * reference cannot be run and it ships no golden weights, kNN indices or matrices.
 * This oracle is pinned to the reference's own end-to-end tests, reproduced on the
 * reference's own fixtures (the CSV files in test/data, converted by tests/golden/make_golden.py):
 *   - test/poisson_test.jl:132   Poisson on Tominec's fitted nodes, rel. L2 err < 0.0027
 *   - test/hyperviscosity_test.jl:32-33   Dxk ~ Dxx, Dyk ~ Dyy (isapprox, rtol sqrt(eps))
 * plus mathematical known-answer tests (polynomial reproduction, E = I when collocated,
 * Lap = Dxx + Dyy, brute-force kNN).  Weight-level parity with the Julia package itself
 * is therefore pinned only through those end-to-end tests ("weight-level parity unpinned").
 *
 * Third-party arithmetic the reference calls and that is restated here:
 *   NearestNeighbors.jl 0.4.13 KDTree + knn(..., sortres=true): exact k nearest
 *       neighbours sorted by distance; restated as an exact uniform-grid search with
 *       the total order (d^2, index).
 *   Symbolics.jl 5.5.1 derivatives of sqrt(x^2+y^2)^p: restated in closed form
 *       (chain rule for f(s) = s^(p/2), s = x^2 + y^2).
 *   DynamicPolynomials 0.5.2 / StaticPolynomials 1.3.7 monomials of total degree <= d:
 *       restated as x^a y^b, a+b <= d, in the order t = 0..d, a = t..0.  The weights do
 *       not depend on the order of the polynomial basis (same span).
 *   LinearAlgebra inv (OpenBLAS 0.3.21 getrf+getri): restated as partial-pivoting LU
 *       followed by an explicit inverse, then M_inv * RHS as the reference does.
 *   SparseArrays sparse(I,J,V): restated as a counting sort into 1-based CSC that keeps
 *       explicit zeros.
 *   HNSW.jl 0.1 HierarchicalNSW + knn_search (processmesh's nearest interior node): an
 *       approximate nearest-neighbour graph search; restated as the exact nearest node
 *       (the two agree whenever the graph search finds the true neighbour).
 *   Statistics mean of a Vector{Float64}: a sum in index order divided by the length
 *       (Julia's own summation order is blocked and SIMD-reassociated, so the last bit of
 *       the mean may differ).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ESINGULAR 3
#define ORC_ENOMEM 5

/* Operator codes (shared with the CUDA library's op list). */
enum { OP_E = 0, OP_DX, OP_DY, OP_DXX, OP_DYY, OP_DXY, OP_LAP, OP_DXK, OP_DYK, OP_HV, OP_COUNT };

static const double ORC_EPS = 2.220446049250313e-16; /* Julia eps(Float64) */

static int set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int orc_max_threads(void) { return set_threads(0); }

/* ------------------------------------------------------------------------- */
/* Exact kNN on a uniform grid.                                              */
/* Follows src/generate_operator.jl:43-47 (KDTree + knn(tree, X, n, true) and */
/* knn(tree, Y, 1)) and the boundary masking of src/calculateneighbors.jl:16-42 */
/* (class c = 0 interior, +b boundary b, -b ghost of boundary b).            */
/* ------------------------------------------------------------------------- */

typedef struct {
    double x0, y0, cs;
    int nx, ny;
    int32_t *start; /* nx*ny + 1 */
    int32_t *pts;   /* N, point ids ordered by cell */
} orc_grid;

static void grid_free(orc_grid *g)
{
    free(g->start);
    free(g->pts);
}

static int grid_build(orc_grid *g, const double *X, int64_t N)
{
    double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
    for (int64_t i = 0; i < N; i++) {
        double x = X[2 * i], y = X[2 * i + 1];
        if (!isfinite(x) || !isfinite(y)) return ORC_EINVAL;
        if (x < xmin) xmin = x;
        if (x > xmax) xmax = x;
        if (y < ymin) ymin = y;
        if (y > ymax) ymax = y;
    }
    double w = xmax - xmin, h = ymax - ymin;
    double area = (w > 0 ? w : 1.0) * (h > 0 ? h : 1.0);
    double cs = sqrt(2.0 * area / (double)N); /* ~2 points per cell */
    if (!(cs > 0)) cs = 1.0;
    int nx = (int)(w / cs) + 1, ny = (int)(h / cs) + 1;
    while ((int64_t)nx * ny > 4 * N + 16) {
        cs *= 1.5;
        nx = (int)(w / cs) + 1;
        ny = (int)(h / cs) + 1;
    }
    g->x0 = xmin;
    g->y0 = ymin;
    g->cs = cs;
    g->nx = nx;
    g->ny = ny;
    int64_t nc = (int64_t)nx * ny;
    g->start = (int32_t *)calloc((size_t)nc + 1, sizeof(int32_t));
    g->pts = (int32_t *)malloc((size_t)N * sizeof(int32_t));
    int32_t *cell = (int32_t *)malloc((size_t)N * sizeof(int32_t));
    if (!g->start || !g->pts || !cell) {
        free(cell);
        grid_free(g);
        return ORC_ENOMEM;
    }
    for (int64_t i = 0; i < N; i++) {
        int cx = (int)((X[2 * i] - xmin) / cs), cy = (int)((X[2 * i + 1] - ymin) / cs);
        if (cx >= nx) cx = nx - 1;
        if (cy >= ny) cy = ny - 1;
        cell[i] = cy * nx + cx;
        g->start[cell[i] + 1]++;
    }
    for (int64_t c = 0; c < nc; c++) g->start[c + 1] += g->start[c];
    int32_t *fill = (int32_t *)malloc((size_t)nc * sizeof(int32_t));
    memcpy(fill, g->start, (size_t)nc * sizeof(int32_t));
    for (int64_t i = 0; i < N; i++) g->pts[fill[cell[i]]++] = (int32_t)i;
    free(fill);
    free(cell);
    return ORC_OK;
}

/* (d2, idx) total order */
static inline int key_less(double da, int32_t ia, double db, int32_t ib)
{
    return da < db || (da == db && ia < ib);
}

static inline int class_allowed(int32_t cq, int32_t cc)
{
    /* calculateneighbors.jl:23-30: a boundary/ghost query of boundary b sees interior,
       every boundary, and only the ghosts of b; calculateneighbors.jl:83-87: interior
       queries see the whole set (ghosts included). */
    if (cq == 0) return 1;
    int32_t b = cq > 0 ? cq : -cq;
    return cc >= 0 || cc == -b;
}

/* Exact k nearest neighbours of (qx,qy), sorted by (d2, idx).  Returns number found. */
static int knn_query(const orc_grid *g, const double *X, const int32_t *cls, int32_t cq,
                     double qx, double qy, int k, int32_t *oi, double *od)
{
    int found = 0;
    int cx = (int)floor((qx - g->x0) / g->cs), cy = (int)floor((qy - g->y0) / g->cs);
    if (cx < 0) cx = 0;
    if (cx >= g->nx) cx = g->nx - 1;
    if (cy < 0) cy = 0;
    if (cy >= g->ny) cy = g->ny - 1;
    for (int R = 0;; R++) {
        int x_lo = cx - R, x_hi = cx + R, y_lo = cy - R, y_hi = cy + R;
        for (int yy = y_lo; yy <= y_hi; yy++) {
            if (yy < 0 || yy >= g->ny) continue;
            int ring_row = (yy == y_lo || yy == y_hi);
            for (int xx = x_lo; xx <= x_hi; xx++) {
                if (xx < 0 || xx >= g->nx) continue;
                if (!ring_row && xx != x_lo && xx != x_hi) continue;
                int c = yy * g->nx + xx;
                for (int32_t t = g->start[c]; t < g->start[c + 1]; t++) {
                    int32_t j = g->pts[t];
                    if (cls && !class_allowed(cq, cls[j])) continue;
                    double dx = qx - X[2 * j], dy = qy - X[2 * j + 1];
                    double d2 = dx * dx + dy * dy;
                    if (found == k && !key_less(d2, j, od[k - 1], oi[k - 1])) continue;
                    int pos = found < k ? found : k - 1;
                    while (pos > 0 && key_less(d2, j, od[pos - 1], oi[pos - 1])) {
                        od[pos] = od[pos - 1];
                        oi[pos] = oi[pos - 1];
                        pos--;
                    }
                    od[pos] = d2;
                    oi[pos] = j;
                    if (found < k) found++;
                }
            }
        }
        /* distance from q to the outside of the searched square of cells */
        double bound = INFINITY;
        if (x_lo > 0) bound = fmin(bound, qx - (g->x0 + x_lo * g->cs));
        if (x_hi < g->nx - 1) bound = fmin(bound, (g->x0 + (x_hi + 1) * g->cs) - qx);
        if (y_lo > 0) bound = fmin(bound, qy - (g->y0 + y_lo * g->cs));
        if (y_hi < g->ny - 1) bound = fmin(bound, (g->y0 + (y_hi + 1) * g->cs) - qy);
        if (bound == INFINITY) break; /* whole grid searched */
        if (found == k && bound > 0 && od[k - 1] < bound * bound * (1.0 - 1e-12)) break;
    }
    return found;
}

/* Brute force kNN (small N only; used to pin the grid search). */
int orc_knn_brute(const double *X, int64_t N, const double *Q, int64_t M, int k,
                  const int32_t *cls_x, const int32_t *cls_q, int32_t *idx, double *d2)
{
    if (k <= 0 || N <= 0) return ORC_EINVAL;
    for (int64_t q = 0; q < M; q++) {
        int found = 0;
        int32_t *oi = idx + q * k;
        double *od = d2 + q * k;
        int32_t cq = cls_q ? cls_q[q] : 0;
        for (int64_t j = 0; j < N; j++) {
            if (cls_x && !class_allowed(cq, cls_x[j])) continue;
            double dx = Q[2 * q] - X[2 * j], dy = Q[2 * q + 1] - X[2 * j + 1];
            double dd = dx * dx + dy * dy;
            if (found == k && !key_less(dd, (int32_t)j, od[k - 1], oi[k - 1])) continue;
            int pos = found < k ? found : k - 1;
            while (pos > 0 && key_less(dd, (int32_t)j, od[pos - 1], oi[pos - 1])) {
                od[pos] = od[pos - 1];
                oi[pos] = oi[pos - 1];
                pos--;
            }
            od[pos] = dd;
            oi[pos] = (int32_t)j;
            if (found < k) found++;
        }
        if (found < k) return ORC_EINVAL;
    }
    return ORC_OK;
}

/* kNN of M query points Q among N nodes X.  cls_x (nullable) gives node classes and
   cls_q (nullable) the query classes (a query with class 0 sees every node).
   idx: M*k 0-based node ids, d2 (nullable): M*k squared distances. */
int orc_knn(const double *X, int64_t N, const double *Q, int64_t M, int k, const int32_t *cls_x,
            const int32_t *cls_q, int32_t *idx, double *d2, int nthreads)
{
    if (k <= 0 || N <= 0 || M < 0) return ORC_EINVAL;
    orc_grid g;
    int rc = grid_build(&g, X, N);
    if (rc) return rc;
    set_threads(nthreads);
    int bad = 0;
#pragma omp parallel
    {
        double *tmp = d2 ? NULL : (double *)malloc((size_t)k * sizeof(double));
#pragma omp for schedule(dynamic, 256)
        for (int64_t q = 0; q < M; q++) {
            double *od = d2 ? d2 + q * k : tmp;
            int32_t cq = cls_q ? cls_q[q] : 0;
            int f = knn_query(&g, X, cls_x, cq, Q[2 * q], Q[2 * q + 1], k, idx + q * k, od);
            if (f < k) {
#pragma omp atomic write
                bad = 1;
            }
        }
        free(tmp);
    }
    grid_free(&g);
    return bad ? ORC_EINVAL : ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* Basis functions.                                                          */
/* ------------------------------------------------------------------------- */

static double fact(int n)
{
    double f = 1;
    for (int i = 2; i <= n; i++) f *= i;
    return f;
}

static double ipow(double x, int e)
{
    double r = 1;
    for (int i = 0; i < e; i++) r *= x;
    return r;
}

static double rpow(double r, int e) { return e >= 0 ? ipow(r, e) : 1.0 / ipow(r, -e); }

/* d^a/dx^a d^b/dy^b of phi = r^p, r = sqrt(x^2+y^2): src/rbfbasis.jl:9-30 and
   src/rbfbasis_k.jl:9-20 build these symbolically; closed form used here:
   sum_{i<=a/2, j<=b/2} a!/(i!(a-2i)!) b!/(j!(b-2j)!) (2x)^(a-2i) (2y)^(b-2j) f^(q)(s),
   q = a+b-i-j, f(s) = s^(p/2), f^(q)(s) = (p/2)(p/2-1)...(p/2-q+1) r^(p-2q). */
double orc_phi(int p, int a, int b, double x, double y)
{
    double r = sqrt(x * x + y * y);
    double sum = 0.0;
    for (int i = 0; 2 * i <= a; i++) {
        for (int j = 0; 2 * j <= b; j++) {
            int q = a + b - i - j;
            double c = fact(a) / (fact(i) * fact(a - 2 * i)) * fact(b) / (fact(j) * fact(b - 2 * j));
            double ff = 1.0;
            for (int t = 0; t < q; t++) ff *= (0.5 * p - t);
            if (ff == 0.0) continue;
            sum += c * ff * ipow(2.0 * x, a - 2 * i) * ipow(2.0 * y, b - 2 * j) * rpow(r, p - 2 * q);
        }
    }
    return sum;
}

static int npoly(int d) { return d < 0 ? 0 : (d + 1) * (d + 2) / 2; }

/* monomial j of the basis: t = 0..d, a = t..0, x^a y^(t-a) (src/polynomialbasis.jl:8-9) */
static void mono_exp(int j, int *ea, int *eb)
{
    int t = 0;
    while (j > t) {
        j -= t + 1;
        t++;
    }
    *ea = t - j;
    *eb = j;
}

/* d^a/dx^a d^b/dy^b of x^ea y^eb at (x,y) (src/polynomialbasis.jl:14-30,
   src/polynomialbasis_k.jl:14-19) */
static double mono_d(int ea, int eb, int a, int b, double x, double y)
{
    if (a > ea || b > eb) return 0.0;
    double c = 1.0;
    for (int t = 0; t < a; t++) c *= (ea - t);
    for (int t = 0; t < b; t++) c *= (eb - t);
    return c * ipow(x, ea - a) * ipow(y, eb - b);
}

/* operator -> (derivative orders, post-solve scale exponents) */
static void op_orders(int op, int K, int *a1, int *b1, int *a2, int *b2, int *two)
{
    *two = 0;
    *a2 = *b2 = 0;
    switch (op) {
    case OP_E: *a1 = 0; *b1 = 0; break;
    case OP_DX: *a1 = 1; *b1 = 0; break;
    case OP_DY: *a1 = 0; *b1 = 1; break;
    case OP_DXX: *a1 = 2; *b1 = 0; break;
    case OP_DYY: *a1 = 0; *b1 = 2; break;
    case OP_DXY: *a1 = 1; *b1 = 1; break;
    case OP_LAP: *a1 = 2; *b1 = 0; *a2 = 0; *b2 = 2; *two = 1; break;
    case OP_DXK: *a1 = K; *b1 = 0; break;
    case OP_DYK: *a1 = 0; *b1 = K; break;
    default: /* OP_HV */ *a1 = K; *b1 = 0; *a2 = 0; *b2 = K; *two = 1; break;
    }
}

/* ------------------------------------------------------------------------- */
/* Dense helpers: LU with partial pivoting and explicit inverse               */
/* (src/interpolationmatrix.jl:8 `inv(A)`).                                    */
/* ------------------------------------------------------------------------- */

static int lu_factor(int s, double *A, int *piv)
{
    for (int c = 0; c < s; c++) {
        int p = c;
        double best = fabs(A[c * s + c]);
        for (int i = c + 1; i < s; i++) {
            double v = fabs(A[i * s + c]);
            if (v > best) {
                best = v;
                p = i;
            }
        }
        piv[c] = p;
        if (best == 0.0 || !isfinite(best)) return ORC_ESINGULAR;
        if (p != c)
            for (int j = 0; j < s; j++) {
                double t = A[c * s + j];
                A[c * s + j] = A[p * s + j];
                A[p * s + j] = t;
            }
        double rinv = 1.0 / A[c * s + c];
        for (int i = c + 1; i < s; i++) A[i * s + c] *= rinv;
        for (int i = c + 1; i < s; i++) {
            double l = A[i * s + c];
            if (l == 0.0) continue;
            for (int j = c + 1; j < s; j++) A[i * s + j] -= l * A[c * s + j];
        }
    }
    return ORC_OK;
}

/* Solve LU x = P b for nrhs columns of B (s x nrhs, row-major), in place. */
static void lu_solve(int s, const double *LU, const int *piv, double *B, int nrhs)
{
    for (int c = 0; c < s; c++)
        if (piv[c] != c)
            for (int q = 0; q < nrhs; q++) {
                double t = B[c * nrhs + q];
                B[c * nrhs + q] = B[piv[c] * nrhs + q];
                B[piv[c] * nrhs + q] = t;
            }
    for (int i = 1; i < s; i++)
        for (int c = 0; c < i; c++) {
            double l = LU[i * s + c];
            for (int q = 0; q < nrhs; q++) B[i * nrhs + q] -= l * B[c * nrhs + q];
        }
    for (int i = s - 1; i >= 0; i--) {
        for (int c = i + 1; c < s; c++) {
            double u = LU[i * s + c];
            for (int q = 0; q < nrhs; q++) B[i * nrhs + q] -= u * B[c * nrhs + q];
        }
        for (int q = 0; q < nrhs; q++) B[i * nrhs + q] /= LU[i * s + i];
    }
}

/* ------------------------------------------------------------------------- */
/* Local system of one X node: scalestencil + interpolationmatrix.           */
/* src/scalestencil.jl:10-21, src/rbfblock.jl:14-20, src/polynomialblock.jl:26-28, */
/* src/interpolationmatrix.jl:3-8.                                            */
/* ------------------------------------------------------------------------- */

typedef struct {
    int s, n, m;
    double *A;    /* s*s, LU factors after factor */
    double *Ainv; /* s*s explicit inverse (use_inverse) */
    double *xs;   /* 2n scaled stencil coordinates */
    double *rhs;  /* s*nops */
    double *sol;  /* s*nops */
    int *piv;
} orc_ws;

static int ws_alloc(orc_ws *w, int n, int m, int nops)
{
    w->n = n;
    w->m = m;
    w->s = n + m;
    int s = w->s;
    w->A = (double *)malloc(sizeof(double) * s * s);
    w->Ainv = (double *)malloc(sizeof(double) * s * s);
    w->xs = (double *)malloc(sizeof(double) * 2 * n);
    w->rhs = (double *)malloc(sizeof(double) * s * (nops > 0 ? nops : 1));
    w->sol = (double *)malloc(sizeof(double) * s * (nops > 0 ? nops : 1));
    w->piv = (int *)malloc(sizeof(int) * s);
    return (w->A && w->Ainv && w->xs && w->rhs && w->sol && w->piv) ? ORC_OK : ORC_ENOMEM;
}

static void ws_free(orc_ws *w)
{
    free(w->A);
    free(w->Ainv);
    free(w->xs);
    free(w->rhs);
    free(w->sol);
    free(w->piv);
}

/* Fill A = [Phi P; P' 0] for scaled coordinates xs (n points), factor it. */
static int build_and_factor(orc_ws *w, int p, int deg, int use_inverse)
{
    int n = w->n, m = w->m, s = w->s;
    double *A = w->A;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) {
            /* rbfblock.jl:16: D[i,j] = X[i] - X[j]; Phi = rbf.(D) */
            double dx = w->xs[2 * i] - w->xs[2 * j], dy = w->xs[2 * i + 1] - w->xs[2 * j + 1];
            A[i * s + j] = orc_phi(p, 0, 0, dx, dy);
        }
        for (int l = 0; l < m; l++) {
            int ea, eb;
            mono_exp(l, &ea, &eb);
            double v = mono_d(ea, eb, 0, 0, w->xs[2 * i], w->xs[2 * i + 1]);
            A[i * s + n + l] = v;
            A[(n + l) * s + i] = v;
        }
    }
    for (int a = n; a < s; a++)
        for (int b = n; b < s; b++) A[a * s + b] = 0.0;
    (void)deg;
    int rc = lu_factor(s, A, w->piv);
    if (rc) return rc;
    if (use_inverse) {
        /* inv(A): solve A X = I column by column */
        double *I = w->Ainv;
        memset(I, 0, sizeof(double) * s * s);
        for (int i = 0; i < s; i++) I[i * s + i] = 1.0;
        lu_solve(s, A, w->piv, I, s);
    }
    return ORC_OK;
}

/* Right-hand side of one evaluation point.  src/generate_operator.jl:122-157:
   stencil_coord_i = y~ - x~_i with exact zeros replaced by eps(); RBF part
   L phi(stencil_coord_i); polynomial part L P(y~) (polylinearoperator.jl:36-44).
   Combined operators (Lap, Dxk+Dyk) scale each term by the chain rule up front.
   When `negate` is set the RBF argument is x~_i (the 4-argument overload, :433). */
static void build_rhs(orc_ws *w, int p, int nops, const int *ops, int K, double yx, double yy,
                      double sx, double sy, int unscaled_overload)
{
    int n = w->n, m = w->m;
    for (int q = 0; q < nops; q++) {
        int a1, b1, a2, b2, two;
        op_orders(ops[q], K, &a1, &b1, &a2, &b2, &two);
        double c1 = 1.0, c2 = 0.0;
        if (two) {
            c1 = ipow(sx, a1) * ipow(sy, b1);
            c2 = ipow(sx, a2) * ipow(sy, b2);
        }
        for (int i = 0; i < n; i++) {
            double dx, dy;
            if (unscaled_overload) {
                dx = w->xs[2 * i];
                dy = w->xs[2 * i + 1];
            } else {
                dx = yx - w->xs[2 * i];
                dy = yy - w->xs[2 * i + 1];
                if (dx == 0) dx = ORC_EPS;
                if (dy == 0) dy = ORC_EPS;
            }
            double v = c1 * orc_phi(p, a1, b1, dx, dy);
            if (two) v += c2 * orc_phi(p, a2, b2, dx, dy);
            w->rhs[i * nops + q] = v;
        }
        for (int l = 0; l < m; l++) {
            int ea, eb;
            mono_exp(l, &ea, &eb);
            double v = c1 * mono_d(ea, eb, a1, b1, yx, yy);
            if (two) v += c2 * mono_d(ea, eb, a2, b2, yx, yy);
            w->rhs[(n + l) * nops + q] = v;
        }
    }
}

/* Post-solve chain-rule scale of generate_operator.jl:161-166 and
   hyperviscosity_operator.jl:159-160. */
static double op_post_scale(int op, int K, double sx, double sy)
{
    switch (op) {
    case OP_E: return 1.0;
    case OP_DX: return sx;
    case OP_DY: return sy;
    case OP_DXX: return sx * sx;
    case OP_DYY: return sy * sy;
    case OP_DXY: return sx * sy;
    case OP_DXK: return ipow(sx, K);
    case OP_DYK: return ipow(sy, K);
    default: return 1.0; /* combined operators were scaled in the RHS */
    }
}

static void solve_point(orc_ws *w, int nops, int use_inverse)
{
    int s = w->s, n = w->n;
    if (use_inverse) {
        /* stenc = M_inv * RHS, rows 1..n kept (generate_operator.jl:158-166) */
        for (int i = 0; i < n; i++)
            for (int q = 0; q < nops; q++) {
                double acc = 0.0;
                for (int j = 0; j < s; j++) acc += w->Ainv[i * s + j] * w->rhs[j * nops + q];
                w->sol[i * nops + q] = acc;
            }
    } else {
        memcpy(w->sol, w->rhs, sizeof(double) * s * nops);
        lu_solve(s, w->A, w->piv, w->sol, nops);
    }
}

/*
 * generate_operator(X, Y, p, n, polydeg) (src/generate_operator.jl:29-190) and the
 * boundary-aware overload (:192-352, neighbours from calculateneighbors) when cls != NULL;
 * hyperviscosity_operator (src/hyperviscosity_operator.jl:26-175, :177-312) when the ops
 * list holds OP_DXK/OP_DYK with K = k_deriv.
 *
 * Outputs (caller-allocated):
 *   nbr  (nullable) N*n stencil node ids (0-based, self first), only rows of nodes that
 *        are the nearest node of some Y point are written;
 *   nn   (nullable) M nearest-X ids of the Y points;
 *   cols M*n column ids (0-based) of each operator row;
 *   W    nops*M*n weights, op-major.
 * use_inverse = 1 follows the reference (explicit inverse, then multiply);
 * 0 solves with the LU factors instead.
 * Returns 0, ORC_EINVAL, ORC_ESINGULAR (bad_node receives the failing X node).
 */
int orc_generate(const double *X, int64_t N, const double *Y, int64_t M, int p, int n, int deg,
                 const int32_t *cls, int nops, const int32_t *ops_in, int k_deriv, int use_inverse,
                 int32_t *nbr, int32_t *nn, int32_t *cols, double *W, int64_t *bad_node,
                 int nthreads)
{
    if (N <= 0 || M < 0 || n <= 0 || n > N || deg < 0 || p <= 0 || nops <= 0 || nops > 16)
        return ORC_EINVAL;
    int ops[16];
    for (int q = 0; q < nops; q++) {
        if (ops_in[q] < 0 || ops_in[q] >= OP_COUNT) return ORC_EINVAL;
        ops[q] = ops_in[q];
    }
    int m = npoly(deg);
    set_threads(nthreads);
    /* knn(tree, Y, 1): nearest X node of each Y point, no mask (calculateneighbors.jl:90-94) */
    int32_t *nny = (int32_t *)malloc(sizeof(int32_t) * (size_t)(M > 0 ? M : 1));
    if (!nny) return ORC_ENOMEM;
    int rc = orc_knn(X, N, Y, M, 1, NULL, NULL, nny, NULL, nthreads);
    if (rc) {
        free(nny);
        return rc;
    }
    if (nn) memcpy(nn, nny, sizeof(int32_t) * (size_t)M);
    /* group Y points by their nearest X node (counting sort) */
    int64_t *ystart = (int64_t *)calloc((size_t)N + 1, sizeof(int64_t));
    int64_t *yord = (int64_t *)malloc(sizeof(int64_t) * (size_t)(M > 0 ? M : 1));
    for (int64_t i = 0; i < M; i++) ystart[nny[i] + 1]++;
    for (int64_t j = 0; j < N; j++) ystart[j + 1] += ystart[j];
    {
        int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)N);
        memcpy(fill, ystart, sizeof(int64_t) * (size_t)N);
        for (int64_t i = 0; i < M; i++) yord[fill[nny[i]]++] = i;
        free(fill);
    }
    /* needed X nodes and their stencils (knn(tree, X, n, true), generate_operator.jl:45) */
    int64_t nneed = 0;
    for (int64_t j = 0; j < N; j++)
        if (ystart[j + 1] > ystart[j]) nneed++;
    int64_t *need = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nneed > 0 ? nneed : 1));
    double *Q = (double *)malloc(sizeof(double) * 2 * (size_t)(nneed > 0 ? nneed : 1));
    int32_t *cq = cls ? (int32_t *)malloc(sizeof(int32_t) * (size_t)(nneed > 0 ? nneed : 1)) : NULL;
    int32_t *st = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * (size_t)(nneed > 0 ? nneed : 1));
    nneed = 0;
    for (int64_t j = 0; j < N; j++)
        if (ystart[j + 1] > ystart[j]) {
            need[nneed] = j;
            Q[2 * nneed] = X[2 * j];
            Q[2 * nneed + 1] = X[2 * j + 1];
            if (cq) cq[nneed] = cls[j];
            nneed++;
        }
    rc = orc_knn(X, N, Q, nneed, n, cls, cq, st, NULL, nthreads);
    int64_t first_bad = -1;
    if (rc == ORC_OK) {
#pragma omp parallel
        {
            orc_ws w;
            int arc = ws_alloc(&w, n, m, nops);
#pragma omp for schedule(dynamic, 64)
            for (int64_t t = 0; t < nneed; t++) {
                if (arc) continue;
                int64_t j = need[t];
                const int32_t *sj = st + t * n;
                if (nbr) memcpy(nbr + j * n, sj, sizeof(int32_t) * n);
                /* scalestencil.jl:10-21 (centre = X[j] = first stencil node) */
                double xc = X[2 * j], yc = X[2 * j + 1];
                double mx = 0.0, my = 0.0;
                for (int i = 0; i < n; i++) {
                    double dx = X[2 * sj[i]] - xc, dy = X[2 * sj[i] + 1] - yc;
                    if (fabs(dx) > mx) mx = fabs(dx);
                    if (fabs(dy) > my) my = fabs(dy);
                }
                double sx = 1.0 / mx, sy = 1.0 / my;
                for (int i = 0; i < n; i++) {
                    w.xs[2 * i] = (X[2 * sj[i]] - xc) * sx;
                    w.xs[2 * i + 1] = (X[2 * sj[i] + 1] - yc) * sy;
                }
                int frc = build_and_factor(&w, p, deg, use_inverse);
                if (frc) {
#pragma omp critical
                    {
                        if (first_bad < 0 || j < first_bad) first_bad = j;
                    }
                    continue;
                }
                for (int64_t u = ystart[j]; u < ystart[j + 1]; u++) {
                    int64_t i = yord[u];
                    /* generate_operator.jl:110,120: Yscaled = (Y - X[j]) .* scale */
                    double yx = (Y[2 * i] - xc) * sx, yy = (Y[2 * i + 1] - yc) * sy;
                    build_rhs(&w, p, nops, ops, k_deriv, yx, yy, sx, sy, 0);
                    solve_point(&w, nops, use_inverse);
                    for (int l = 0; l < n; l++) cols[i * n + l] = sj[l];
                    for (int q = 0; q < nops; q++) {
                        double f = op_post_scale(ops[q], k_deriv, sx, sy);
                        for (int l = 0; l < n; l++) W[(int64_t)q * M * n + i * n + l] = f * w.sol[l * nops + q];
                    }
                }
            }
            ws_free(&w);
        }
        if (first_bad >= 0) rc = ORC_ESINGULAR;
    }
    if (bad_node) *bad_node = first_bad;
    free(nny);
    free(ystart);
    free(yord);
    free(need);
    free(Q);
    free(cq);
    free(st);
    return rc;
}

/*
 * The collocated, unscaled overloads generate_operator(X, p, n, polydeg)
 * (src/generate_operator.jl:354-491) and hyperviscosity_operator(k, X, p, n, polydeg)
 * (src/hyperviscosity_operator.jl:314-440): no scalestencil; X_shift = x_j - x_c with the
 * centre replaced by (eps, eps) (:410); the RHS is evaluated at stencil_coord = X_shift
 * (:433) and the polynomial RHS at X_shift[1] (:429); no post-solve scaling.
 */
int orc_generate_unscaled(const double *X, int64_t N, int p, int n, int deg, int nops,
                          const int32_t *ops_in, int k_deriv, int use_inverse, int32_t *cols,
                          double *W, int64_t *bad_node, int nthreads)
{
    if (N <= 0 || n <= 0 || n > N || deg < 0 || p <= 0 || nops <= 0 || nops > 16) return ORC_EINVAL;
    int ops[16];
    for (int q = 0; q < nops; q++) {
        if (ops_in[q] < 0 || ops_in[q] >= OP_COUNT) return ORC_EINVAL;
        ops[q] = ops_in[q];
    }
    int m = npoly(deg);
    set_threads(nthreads);
    int32_t *st = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * (size_t)N);
    if (!st) return ORC_ENOMEM;
    int rc = orc_knn(X, N, X, N, n, NULL, NULL, st, NULL, nthreads);
    int64_t first_bad = -1;
    if (rc == ORC_OK) {
#pragma omp parallel
        {
            orc_ws w;
            int arc = ws_alloc(&w, n, m, nops);
#pragma omp for schedule(dynamic, 64)
            for (int64_t j = 0; j < N; j++) {
                if (arc) continue;
                const int32_t *sj = st + j * n;
                double xc = X[2 * sj[0]], yc = X[2 * sj[0] + 1];
                for (int i = 0; i < n; i++) {
                    w.xs[2 * i] = X[2 * sj[i]] - xc;
                    w.xs[2 * i + 1] = X[2 * sj[i] + 1] - yc;
                }
                w.xs[0] = ORC_EPS;
                w.xs[1] = ORC_EPS;
                int frc = build_and_factor(&w, p, deg, use_inverse);
                if (frc) {
#pragma omp critical
                    {
                        if (first_bad < 0 || j < first_bad) first_bad = j;
                    }
                    continue;
                }
                build_rhs(&w, p, nops, ops, k_deriv, w.xs[0], w.xs[1], 1.0, 1.0, 1);
                solve_point(&w, nops, use_inverse);
                for (int l = 0; l < n; l++) cols[j * n + l] = sj[l];
                for (int q = 0; q < nops; q++)
                    for (int l = 0; l < n; l++) W[(int64_t)q * N * n + j * n + l] = w.sol[l * nops + q];
            }
            ws_free(&w);
        }
        if (first_bad >= 0) rc = ORC_ESINGULAR;
    }
    if (bad_node) *bad_node = first_bad;
    free(st);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Sparse assembly and application.                                          */
/* ------------------------------------------------------------------------- */

/* sparse(I, J, V) of generate_operator.jl:171-182: row i holds n entries (cols[i*n+l],
   W[i*n+l]).  Produces 1-based CSC (colptr N+1, rowval nnz, nzval nnz) with rows
   ascending inside each column and explicit zeros kept. */
int orc_to_csc(int64_t M, int64_t N, int n, const int32_t *cols, const double *W, int64_t *colptr,
               int64_t *rowval, double *nzval)
{
    int64_t nnz = M * n;
    memset(colptr, 0, sizeof(int64_t) * (size_t)(N + 1));
    for (int64_t e = 0; e < nnz; e++) {
        if (cols[e] < 0 || cols[e] >= N) return ORC_EINVAL;
        colptr[cols[e] + 1]++;
    }
    for (int64_t j = 0; j < N; j++) colptr[j + 1] += colptr[j];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N > 0 ? N : 1));
    if (!fill) return ORC_ENOMEM;
    memcpy(fill, colptr, sizeof(int64_t) * (size_t)N);
    for (int64_t i = 0; i < M; i++)
        for (int l = 0; l < n; l++) {
            int64_t e = i * n + l, t = fill[cols[e]]++;
            rowval[t] = i + 1;
            nzval[t] = W[e];
        }
    free(fill);
    for (int64_t j = 0; j <= N; j++) colptr[j] += 1;
    return ORC_OK;
}

/* y = A x for the row-stencil form (CSR with n entries per row), OpenMP over rows. */
void orc_spmv_rows(int64_t M, int n, const int32_t *cols, const double *W, const double *x, double *y,
                   int nthreads)
{
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; i++) {
        double acc = 0.0;
        for (int l = 0; l < n; l++) acc += W[i * n + l] * x[cols[i * n + l]];
        y[i] = acc;
    }
}

/* y = A x for 1-based CSC, single thread, as SparseArrays' CSC * Vector does
   (the apply site examples/adv_diff_test.jl:151-152). */
void orc_spmv_csc(int64_t M, int64_t N, const int64_t *colptr, const int64_t *rowval,
                  const double *nzval, const double *x, double *y)
{
    memset(y, 0, sizeof(double) * (size_t)M);
    for (int64_t j = 0; j < N; j++) {
        double xj = x[j];
        for (int64_t t = colptr[j] - 1; t < colptr[j + 1] - 1; t++) y[rowval[t] - 1] += nzval[t] * xj;
    }
}

/* ------------------------------------------------------------------------- */
/* Mesh ingest: processmesh after its file reads.                            */
/* ------------------------------------------------------------------------- */

/* processmesh (src/processmesh.jl:1-192) on arrays already read from the CGNS file:
     V    nv vertices (x, y)                       extractcoordinates.jl:1-14
     tri  3 ntri 1-based vertex ids of the triangles (TriElements/ElementConnectivity)
     bc   2 nbc 1-based vertex ids of the boundary line elements of every marker,
          concatenated in element-range order (each marker's ElementConnectivity)
   Outputs:
     Y    (ntri + 2 nbc) points: the triangles' centroids (extractelements.jl:16-17,
          processmesh.jl:23-27), the lines' midpoints (processmesh.jl:89, 116), then the
          ghost nodes (processmesh.jl:167-181, genghostnodes.jl:1-6)
     nrm, tng  nbc unit normals [-dy, dx] / |.| and tangents [dx, dy] / |.| of the lines
          (calculatenormal.jl:1-17), all multiplied by the sign of
          dot(line 1 midpoint - its nearest centroid, normal 1) (processmesh.jl:120-133)
     offset  the mean distance of the midpoints to their nearest centroid
          (processmesh.jl:135-165); ghost = midpoint + normal * offset.
   Returns ORC_EINVAL on an empty mesh or a vertex id out of range. */
int orc_process_mesh(const double *V, int64_t nv, const int64_t *tri, int64_t ntri, const int64_t *bc,
                     int64_t nbc, double *Y, double *nrm, double *tng, double *offset)
{
    if (nv <= 0 || ntri <= 0 || nbc <= 0) return ORC_EINVAL;
    for (int64_t t = 0; t < 3 * ntri; t++)
        if (tri[t] < 1 || tri[t] > nv) return ORC_EINVAL;
    for (int64_t t = 0; t < 2 * nbc; t++)
        if (bc[t] < 1 || bc[t] > nv) return ORC_EINVAL;
    for (int64_t e = 0; e < ntri; e++) {
        const double *a = V + 2 * (tri[3 * e] - 1), *b = V + 2 * (tri[3 * e + 1] - 1), *c = V + 2 * (tri[3 * e + 2] - 1);
        Y[2 * e] = (a[0] + b[0] + c[0]) / 3.0; /* mean of three SVectors: ((a + b) + c) / 3 */
        Y[2 * e + 1] = (a[1] + b[1] + c[1]) / 3.0;
    }
    double *M = Y + 2 * ntri, *G = Y + 2 * (ntri + nbc);
    for (int64_t e = 0; e < nbc; e++) {
        const double *a = V + 2 * (bc[2 * e] - 1), *b = V + 2 * (bc[2 * e + 1] - 1);
        M[2 * e] = (a[0] + b[0]) / 2.0;
        M[2 * e + 1] = (a[1] + b[1]) / 2.0;
        const double dx = b[0] - a[0], dy = b[1] - a[1];
        const double len = sqrt(dy * dy + dx * dx); /* norm([-dy, dx]) */
        nrm[2 * e] = -dy / len;
        nrm[2 * e + 1] = dx / len;
        tng[2 * e] = dx / len;
        tng[2 * e + 1] = dy / len;
    }
    int32_t *nn = (int32_t *)malloc(sizeof(int32_t) * (size_t)nbc);
    double *d2 = (double *)malloc(sizeof(double) * (size_t)nbc);
    if (!nn || !d2) {
        free(nn);
        free(d2);
        return ORC_ENOMEM;
    }
    int rc = orc_knn(Y, ntri, M, nbc, 1, NULL, NULL, nn, d2, 1);
    if (rc) {
        free(nn);
        free(d2);
        return rc;
    }
    const double *c0 = Y + 2 * (int64_t)nn[0];
    const double dt = (M[0] - c0[0]) * nrm[0] + (M[1] - c0[1]) * nrm[1];
    const double sg = dt > 0.0 ? 1.0 : (dt < 0.0 ? -1.0 : dt); /* Julia sign */
    double sum = 0.0;
    for (int64_t e = 0; e < nbc; e++) sum += sqrt(d2[e]);
    const double off = fabs(sum / (double)nbc);
    for (int64_t e = 0; e < 2 * nbc; e++) {
        nrm[e] = sg * nrm[e];
        tng[e] = sg * tng[e];
        G[e] = M[e] + nrm[e] * off;
    }
    *offset = off;
    free(nn);
    free(d2);
    return ORC_OK;
}
