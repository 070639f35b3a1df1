/*
 * rbffd.h -- C ABI of the GB300-native RBF-FD hot path.
 *
 * Drop-in boundary for RadialBasisFiniteDifferences.jl (v0.1.0).  The Julia host keeps
 * its public API (generate_operator, hyperviscosity_operator, calculateneighbors) and
 * ccalls the entry points below, which run kNN stencil selection, the per-node local
 * RBF-FD weight solves and the sparse operator build on one sm_103a GPU and hand back
 * the same SparseMatrixCSC{Float64,Int64} data (1-based colptr/rowval, nzval, explicit
 * zeros kept).  Device-resident operator sets (rbffd_opset_*) serve time stepping:
 * SpMV / multi-field SpMM and RK4 stages captured in a CUDA graph.
 *
 * Conventions
 *   - Points are AoS doubles (x0,y0,x1,y1,...): the memory layout of Julia's
 *     Vector{SVector{2,Float64}}.
 *   - node_class (nullable, N entries) encodes the index ranges of the boundary-aware
 *     overloads: 0 interior (X_idx_in), +b boundary b (X_idx_bc[b]), -b ghost of
 *     boundary b (X_idx_bc_g[b]), b = 1, 2, ...
 *   - Output buffers are caller-allocated; every call returns an rbffd_status.
 *   - One handle per host thread.  Calls on one handle are serialised on the handle's
 *     CUDA stream; a handle is not re-entrant.
 *   - No entry point falls back to the CPU.  Without a usable sm_103a GPU every call
 *     returns RBFFD_ECUDA.
 */
#ifndef RBFFD_H
#define RBFFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RBFFD_VERSION_MAJOR 0
#define RBFFD_VERSION_MINOR 1

typedef enum {
    RBFFD_OK = 0,
    RBFFD_EINVAL = 1,    /* bad argument: sizes, k > #candidates, NaN coordinates, ... */
    RBFFD_ECUDA = 2,     /* CUDA runtime failure or no usable GPU */
    RBFFD_ESINGULAR = 3, /* a local system is singular (stats.first_bad_node) */
    RBFFD_ETIMEOUT = 4,  /* a bounded device wait gave up */
    RBFFD_ENOMEM = 5     /* device or host allocation failed */
} rbffd_status;

/* Operators (bit i of an op mask <-> operator code i).  The reference's generate_operator
   returns (E, Dx, Dy, Dxx, Dyy, Dxy) (src/generate_operator.jl:189); hyperviscosity_operator
   returns (Dxk, Dyk) (src/hyperviscosity_operator.jl:174).  LAP = Dxx + Dyy and
   HV = Dxk + Dyk are solved from one combined right-hand side. */
enum {
    RBFFD_OP_E = 0,
    RBFFD_OP_DX = 1,
    RBFFD_OP_DY = 2,
    RBFFD_OP_DXX = 3,
    RBFFD_OP_DYY = 4,
    RBFFD_OP_DXY = 5,
    RBFFD_OP_LAP = 6,
    RBFFD_OP_DXK = 7,
    RBFFD_OP_DYK = 8,
    RBFFD_OP_HV = 9,
    RBFFD_OP_COUNT = 10
};
#define RBFFD_MASK(op) (1u << (op))
#define RBFFD_MASK_GENERATE                                                                   \
    (RBFFD_MASK(RBFFD_OP_E) | RBFFD_MASK(RBFFD_OP_DX) | RBFFD_MASK(RBFFD_OP_DY) |             \
     RBFFD_MASK(RBFFD_OP_DXX) | RBFFD_MASK(RBFFD_OP_DYY) | RBFFD_MASK(RBFFD_OP_DXY))
#define RBFFD_MASK_HYPERVISCOSITY (RBFFD_MASK(RBFFD_OP_DXK) | RBFFD_MASK(RBFFD_OP_DYK))

/* Precision of the local solves. */
enum {
    RBFFD_PREC_FP64 = 0,  /* assemble, LU-factor and solve in FP64 */
    RBFFD_PREC_MIXED = 1  /* FP32 assembly + LU on the scaled stencil, FP64 residuals and
                             iterative refinement, per-stencil FP64 fallback when it stalls */
};

/* Where pointers passed to rbffd_opset_create live. */
enum { RBFFD_MEM_HOST = 0, RBFFD_MEM_DEVICE = 1 };

typedef struct rbffd_handle rbffd_handle;
typedef struct rbffd_opset rbffd_opset;
typedef struct rbffd_rk4 rbffd_rk4;

typedef struct {
    int device;          /* CUDA device ordinal */
    int warps_per_block; /* weight-solve CTA size in warps; 0 = autotune */
    int max_refine;      /* mixed precision: refinement iterations before fallback (0 = 6) */
    double refine_tol;   /* mixed precision: stop when the predicted relative weight error
                            is below this (0 = 1e-12) */
} rbffd_options;

typedef struct {
    double ms_upload, ms_grid, ms_knn, ms_solve, ms_fallback, ms_csr, ms_total;
    int64_t n_systems;      /* local systems factored */
    int64_t n_rows;         /* operator rows (evaluation points) */
    int64_t n_fallback;     /* mixed: systems re-solved in FP64 */
    int64_t first_bad_node; /* 0-based X node of the first singular system, -1 if none */
    int64_t refine_hist[8]; /* mixed: systems that converged after i refinement steps (i = 0:
                               solved directly in FP64, a class the autotuner timed faster so) */
    int64_t nnz;            /* nonzeros per operator */
    int64_t kernel_launches;/* CUDA kernels this call launched */
} rbffd_stats;

/* Caller-owned CSC arrays of one operator (Julia SparseMatrixCSC{Float64,Int64}). */
typedef struct {
    int64_t *colptr; /* ncols + 1, 1-based */
    int64_t *rowval; /* nnz, 1-based, ascending within each column */
    double *nzval;   /* nnz */
} rbffd_csc;

/* Problem description of rbffd_opset_create. */
typedef struct {
    const double *X; /* N interpolation nodes (AoS) */
    int64_t N;
    const double *Y; /* M evaluation points (AoS); NULL = collocated (Y = X) */
    int64_t M;
    int p;                      /* PHS exponent (odd, r^p) */
    int n;                      /* stencil size (uniform; ignored if n_per_node) */
    int polydeg;                /* polynomial degree (uniform; ignored if deg_per_node) */
    const int32_t *node_class;  /* nullable, see Conventions */
    const int32_t *n_per_node;  /* nullable: per-node stencil size */
    const int32_t *deg_per_node;/* nullable: per-node polynomial degree */
    uint32_t op_mask;           /* operators to build */
    int k_deriv;                /* derivative order of DXK/DYK/HV */
    int precision;              /* RBFFD_PREC_* */
    int memspace;               /* RBFFD_MEM_* of X, Y, node_class, n/deg arrays */
    int64_t row_begin, row_end; /* evaluation rows [row_begin,row_end) to build (sharding);
                                   row_end <= 0 means all rows */
} rbffd_problem;

int rbffd_version(void);
const char *rbffd_status_string(int status);

int rbffd_create(const rbffd_options *opt, rbffd_handle **out);
void rbffd_destroy(rbffd_handle *h);
/* Text of the last error on this handle (never NULL). */
const char *rbffd_last_error(const rbffd_handle *h);
/* The weight-solve autotuner's choices on this handle, one line per shape class of local
   systems seen so far ("mixed n<=30 m<=10 ops=3 p=3: schur x4 warps (timed on ... systems:
   candidate times)"); classes too small to time get a heuristic choice and no line.  The text
   stays valid until the next call on the handle.  No reference counterpart (the reference
   runs the solves in a Threads.@threads loop, src/generate_operator.jl:55,89). */
const char *rbffd_autotune_report(const rbffd_handle *h);
/* The handle's cudaStream_t, as void*. */
void *rbffd_stream(rbffd_handle *h);
int rbffd_synchronize(rbffd_handle *h);

/* ---------------------------------------------------------------------------------
 * Drop-in entry points (host buffers in, caller-allocated host CSC out).
 * ------------------------------------------------------------------------------ */

/* generate_operator(X, Y, p, n, polydeg) -- src/generate_operator.jl:29-190 -- and, with
   node_class != NULL, the boundary-aware overload generate_operator(X, Y, p, n, polydeg,
   X_idx_in, X_idx_bc, X_idx_bc_g, Y_idx_in, Y_idx_bc, Y_idx_bc_g) -- :192-352.
   out[] has one rbffd_csc per set bit of op_mask, in increasing bit order; each is an
   M x N matrix with nnz = M * n.  Y == X (same pointer, M == N) is the collocated case.
   Collocated calls with one stencil size download the CSC pattern while the weights are
   solved and, from 8192 nodes on, the values of each completed range of columns while the
   remaining rows solve; the outputs are complete when the call returns. */
int rbffd_generate_operator(rbffd_handle *h, const double *X, int64_t N, const double *Y,
                            int64_t M, int p, int n, int polydeg, const int32_t *node_class,
                            uint32_t op_mask, int precision, rbffd_csc *out,
                            rbffd_stats *stats);

/* hyperviscosity_operator(k_deriv, X, Y, p, n, polydeg[, index ranges]) --
   src/hyperviscosity_operator.jl:26-175 and :177-312.  out[0] = Dxk, out[1] = Dyk. */
int rbffd_hyperviscosity_operator(rbffd_handle *h, int k_deriv, const double *X, int64_t N,
                                  const double *Y, int64_t M, int p, int n, int polydeg,
                                  const int32_t *node_class, int precision, rbffd_csc *out,
                                  rbffd_stats *stats);

/* The collocated, unscaled overloads generate_operator(X, p, n, polydeg)
   (src/generate_operator.jl:354-491) and hyperviscosity_operator(k, X, p, n, polydeg)
   (src/hyperviscosity_operator.jl:314-440), reproduced as the reference computes them:
   no stencil scaling, centre shifted to (eps, eps), RBF right-hand side evaluated at
   x_j - x_c.  k_deriv is used when op_mask holds DXK/DYK/HV. */
int rbffd_generate_operator_unscaled(rbffd_handle *h, const double *X, int64_t N, int p, int n,
                                     int polydeg, uint32_t op_mask, int k_deriv,
                                     rbffd_csc *out, rbffd_stats *stats);

/* calculateneighbors(X, Y, n, X_idx_in, X_idx_bc, X_idx_bc_g, ...) --
   src/calculateneighbors.jl:1-97 (node_class == NULL: the plain knn of
   src/generate_operator.jl:43-47).  idxs_x: N x n 1-based ids sorted by distance (self
   first); dists_x: N x n Euclidean distances (nullable); idxs_y_x / dists_y_x: nearest
   node of each Y point (nullable when M == 0). */
int rbffd_calculateneighbors(rbffd_handle *h, const double *X, int64_t N, const double *Y,
                             int64_t M, int n, const int32_t *node_class, int64_t *idxs_x,
                             double *dists_x, int64_t *idxs_y_x, double *dists_y_x);

/* processmesh(meshname, markernames) -- src/processmesh.jl:1-192 -- after its HDF5/CGNS
   reads (extractcoordinates.jl, extractelements.jl), which stay with the caller.
   vertices: nv points (x, y) (Base/dom-1/GridCoordinates); tri: 3 ntri 1-based vertex ids
   (TriElements/ElementConnectivity); bc: 2 nbc 1-based vertex ids, the line elements of
   every marker concatenated in element-range order.  Y receives ntri + 2 nbc points: the
   triangle centroids, the line midpoints, then the ghost nodes; normals / tangents (nbc x 2)
   the lines' unit normals [-dy, dx]/|.| and tangents, oriented by the sign of
   dot(first midpoint - its nearest centroid, first normal); *offset the mean distance of
   the midpoints to their nearest centroid (ghost = midpoint + normal * offset).  The nearest
   centroid is exact (the reference's HNSW search is approximate).  Host pointers. */
int rbffd_process_mesh(rbffd_handle *h, const double *vertices, int64_t nv, const int64_t *tri,
                       int64_t ntri, const int64_t *bc, int64_t nbc, double *Y, double *normals,
                       double *tangents, double *offset);

/* ---------------------------------------------------------------------------------
 * Device-resident operator sets (time stepping, benchmarks).
 * ------------------------------------------------------------------------------ */

int rbffd_opset_create(rbffd_handle *h, const rbffd_problem *prob, rbffd_opset **out,
                       rbffd_stats *stats);
void rbffd_opset_destroy(rbffd_handle *h, rbffd_opset *s);
/* Shape: rows (evaluation points built), cols (N), nnz per operator, op count. */
int rbffd_opset_shape(const rbffd_opset *s, int64_t *rows, int64_t *cols, int64_t *nnz,
                      int *nops);
/* Device CSR of operator `op` (its index among the set's ops): row_ptr (rows+1, int64),
   col (nnz, int32 0-based), val (nnz, double).  Pointers stay owned by the set. */
int rbffd_opset_device_csr(const rbffd_opset *s, int op, const int64_t **row_ptr,
                           const int32_t **col, const double **val);
/* Copy one operator to caller-allocated host CSC (1-based, Julia layout). */
int rbffd_opset_export_csc(rbffd_handle *h, rbffd_opset *s, int op, rbffd_csc *out);
/* Copy one operator to caller-allocated host CSR (0-based int64 row_ptr / int32 col). */
int rbffd_opset_export_csr(rbffd_handle *h, rbffd_opset *s, int op, int64_t *row_ptr,
                           int32_t *col, double *val);
/* Copy the stencils (N x n 0-based, uniform n only) and nearest-node ids of the rows. */
int rbffd_opset_export_stencils(rbffd_handle *h, rbffd_opset *s, int32_t *nbr, int32_t *nn);

/* y = A_op x on the handle's stream; x, y device pointers (FP64, cols / rows long). */
int rbffd_spmv(rbffd_handle *h, rbffd_opset *s, int op, const double *x, double *y);
/* Y = A_op X for nfields fields, X row-major [cols][nfields], Y [rows][nfields];
   dtype 0 = FP64 weights and fields, 1 = FP32 weights and fields. */
int rbffd_spmm(rbffd_handle *h, rbffd_opset *s, int op, const void *x, void *y, int nfields,
               int dtype);

/* ---------------------------------------------------------------------------------
 * Time stepping: explicit RK4 for du/dt = L u on nfields fields, the semi-discrete system
 * the reference integrates in examples/adv_diff_test.jl:144-199 (cons_sys, SSPRK43).
 * ------------------------------------------------------------------------------ */

/* L = sum over the sets' operators of coef[i] * A_i, in set order then operator order
   (sets: collocated, full, built from one node set with one stencil size, so they share a
   sparsity pattern; e.g. {Dx, Dy, Lap} with r^3 and {HV} with r^5).  fixed_rows (host,
   nullable, rows bytes): rows held at their initial values (du = 0), the Dirichlet
   overwrite of examples/adv_diff_test.jl:166-167.  dtype 0: FP64 weights and fields,
   1: FP32.  Fields are row-major [rows][nfields] device arrays.  FP32 with nfields in
   {4, 8, 16, 32, 64, 128} applies L tile by tile from shared memory (tiles of 64 rows of a
   Z-curve order of the nodes, each tile's stencil-column union staged by asynchronous
   copies, groups of 8 rows applied together with dense weights over the group's columns)
   and in difference form, sum_t w_t (v_t - v_ref) + (sum_t w_t) v_ref with v_ref a node of
   the tile, whose FP32 error scales with the field's differences rather than its size. */
int rbffd_rk4_create(rbffd_handle *h, rbffd_opset *const *sets, int nsets, const double *coef,
                     const uint8_t *fixed_rows, int nfields, int dtype, rbffd_rk4 **out);
/* Advance u (device, in place) by nsteps steps of size dt.  Pairs of steps run as one
   captured CUDA graph (4 fused stage kernels per step), re-captured when u or dt change.
   Without ghost closures L is constant and a classic RK4 step equals the degree-4 Taylor
   polynomial of exp(dt L); it is evaluated in Horner form (u + dt/4 L u, then u + dt/3 L w,
   u + dt/2 L w, u + dt L w), which needs no stage accumulator.  With closures the stage form
   is used. */
int rbffd_rk4_run(rbffd_handle *h, rbffd_rk4 *rk, void *u, double dt, int64_t nsteps);
/* y = L x for the stepper's fields (x, y device [rows][nfields]). */
int rbffd_rk4_apply(rbffd_handle *h, rbffd_rk4 *rk, const void *x, void *y);
void rbffd_rk4_destroy(rbffd_handle *h, rbffd_rk4 *rk);

/* ---------------------------------------------------------------------------------
 * Ghost-node closure (examples/adv_diff_test.jl:108-141, 160-176).  For a boundary with
 * boundary nodes B and ghost nodes G (|B| = |G|: one ghost per boundary node,
 * src/genghostnodes.jl) and an operator A of a collocated set (Dx for the left/right, Dy for
 * the top/bottom boundary in the example), the ghost values for which A u = 0 on B are
 *     u[G] = -inv(A[B, G]) * (A[B, not G] * u[not G]).
 * ------------------------------------------------------------------------------ */
typedef struct rbffd_ghost rbffd_ghost;

/* bnodes, gnodes: host, nb 0-based node ids each.  inv(A[B, G]) is formed once, on the GPU
   (dense Gauss-Jordan with partial pivoting: the reference's inv(Array(w_bc_g))); a
   singular block returns RBFFD_ESINGULAR.  The closure reads the set's operator, so the set
   must outlive it. */
int rbffd_ghost_create(rbffd_handle *h, rbffd_opset *s, int op, const int32_t *bnodes,
                       const int32_t *gnodes, int64_t nb, rbffd_ghost **out);
/* Overwrite u[G] (device fields [rows][nfields], dtype 0: FP64, 1: FP32) in place. */
int rbffd_ghost_apply(rbffd_handle *h, rbffd_ghost *g, void *u, int nfields, int dtype);
void rbffd_ghost_destroy(rbffd_handle *h, rbffd_ghost *g);
/* Apply the closures (in order) to the input of every RK4 stage before L is applied; the
   first stage's input is the state itself, which is overwritten as the reference's cons_sys
   overwrites u.  ng = 0 removes them.  The closures must outlive the stepper's use. */
int rbffd_rk4_set_closure(rbffd_handle *h, rbffd_rk4 *rk, rbffd_ghost *const *g, int ng);

/* ---------------------------------------------------------------------------------
 * Least squares on an operator set: the assembly and solve of test/poisson_test.jl:75-121
 * (`D[rows_b, :] .= c_b .* A_b[rows_b, :]`, row scaling, `D \ f`) on the GPU.  Row i of D is
 * sum_q coef[q * rows + i] * A_q[i, :] over the set's operators (set order: E, Dx, Dy, Dxx, Dyy,
 * Dxy, Lap, ...), and u minimises ||D u - f||_2, computed by CGLS (conjugate gradients on
 * the normal equations, Hestenes-Stiefel form) with the set's CSR and CSC patterns; 50
 * iterations run as one CUDA graph between convergence checks.  The reference solves with
 * a sparse QR factorisation; CGLS reaches the same least-squares solution iteratively.
 * ------------------------------------------------------------------------------ */
typedef struct {
    int64_t iterations; /* CGLS iterations done */
    double relres;      /* ||D^T (f - D u)|| / ||D^T (f - D u0)|| at exit */
    double ms;          /* device time of the iterations */
} rbffd_lsq_info;

/* coef: host, nops x rows (row-major by operator); f: host, rows; u: host, N (initial guess
   in, solution out).  Stops when relres <= tol or after maxit iterations (relres is checked
   every 50 iterations). */
int rbffd_lsq_cgls(rbffd_handle *h, rbffd_opset *s, const double *coef, const double *f, double *u,
                   int64_t maxit, double tol, rbffd_lsq_info *info);

/* ---------------------------------------------------------------------------------
 * Allocation-free kNN (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory: hosts whose device memory belongs to
 * another allocator that must not be bypassed (a CUDA.jl or PyTorch caching pool),
 * programs with a device-memory budget fixed at start-up, and code that must not
 * synchronise the device as cudaMalloc/cudaFree may.  The stencils of all N nodes
 * (k nearest, self first, ties by lower id -- the same sets as rbffd_calculateneighbors)
 * are written to caller-owned device buffers: idx_dev (N x k, 0-based int32) and d2_dev
 * (N x k squared distances, nullable).  X_dev: N device points (AoS, 16-byte aligned).
 * stream: a cudaStream_t (NULL = default stream); the call synchronises it.
 *
 * Scratch lives in one static device array of RBFFD_NOALLOC_SCRATCH_BYTES per GPU, held
 * until the process exits; N above RBFFD_NOALLOC_MAX_NODES is rejected with RBFFD_EINVAL
 * (message in rbffd_last_error(NULL)).  The first call on each device looks the array's
 * address up (make it before any stream capture).  With CUDA's default lazy module loading
 * that first call is also when the array is placed in device memory, so it needs 5 MiB of
 * free device memory (RBFFD_ECUDA if there is none; CUDA_MODULE_LOADING=EAGER places it at
 * library load instead): make it before the caller's allocator reserves the device's
 * memory.  Calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller.
 * ------------------------------------------------------------------------------ */
#define RBFFD_NOALLOC_MAX_NODES 65536
#define RBFFD_NOALLOC_SCRATCH_BYTES (5u << 20)
int rbffd_knn_noalloc(const double *X_dev, int64_t N, int k, int32_t *idx_dev, double *d2_dev,
                      void *stream);

/* ---------------------------------------------------------------------------------
 * Diagnostics.
 * ------------------------------------------------------------------------------ */

/* Measured FP64 and FP32 CUDA-core FMA throughput of `device` in TFLOP/s (the peaks that
   bound the weight solves; no reference counterpart). */
int rbffd_measure_fma_peaks(int device, double *fp64_tflops, double *fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif /* RBFFD_H */
