// Internal declarations shared by the CUDA translation units of librbffd.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "rbffd.h"

#define RBFFD_FULL 0xffffffffu
#define RBFFD_MAX_OPS 10
#define RBFFD_MAX_TERMS 6
#define RBFFD_MAX_S 128   // largest local system (n + m) the solve kernels accept
#define RBFFD_MAX_K 128   // largest stencil size the kNN kernel accepts
#define RBFFD_MAX_DEG 8   // largest polynomial degree

// ---------------------------------------------------------------------------
// Operator descriptors (host-built, passed by value to the solve kernels).
//   Each operator is one or two derivative components (a, b) = d^a/dx^a d^b/dy^b.
//   The RBF part of component c is sum_t coef * x^ex * y^ey * r^er (closed form of
//   d^a/dx^a d^b/dy^b r^p).  Single-component operators are unscaled after the solve
//   by sx^a sy^b (src/generate_operator.jl:161-166); two-component operators (LAP, HV)
//   scale each component by sx^a sy^b inside the right-hand side.
// ---------------------------------------------------------------------------
struct RbfTerm {
    double coef;
    int ex, ey, er;
};

struct OpComp {
    int a, b;  // derivative orders
    int nterm;
    RbfTerm t[RBFFD_MAX_TERMS];
};

struct OpDesc {
    int ncomp;       // 1 or 2
    int post_scale;  // 1: multiply weights by sx^a sy^b after the solve
    OpComp c[2];
};

struct OpTable {
    int nops;
    int p;
    // Nonzero when p = 3 and every operator is E, Dx, Dy, Dxx, Dyy, Dxy or Lap (the
    // reference's generate_operator set and the Laplacian): the register Schur kernel then
    // forms their right-hand sides from closed forms instead of the term table.  Bit 0 set,
    // bit 1: 3r needed (Dx, Dy, Dxx, Dyy), bit 2: some Lap, bit 3: 3/r needed (Dxx, Dyy, Dxy).
    int r3_closed;
    // 1 when p = 5, K = 4 and every operator is Dxk or Dyk (the hyperviscosity pair of the
    // time-stepping example): closed forms likewise.
    int r5_hv4;
    OpDesc op[RBFFD_MAX_OPS];
};

// Text returned by rbffd_last_error(NULL) on this thread (errors of calls without a handle).
void set_handleless_error(const std::string &msg);

// Build the descriptor table for the ops in `ops` (RBFFD_OP_* codes).
bool build_op_table(const int *ops, int nops, int p, int k_deriv, OpTable *t, std::string *err);

// ---------------------------------------------------------------------------
// Device scratch helpers.
// ---------------------------------------------------------------------------
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// ---------------------------------------------------------------------------
// Uniform grid of cells over the node set (kNN candidate lookup).
// ---------------------------------------------------------------------------
struct GridDev {
    double x0, y0, cs;
    int nx, ny;
    const int32_t *start;  // nx*ny + 1 offsets into pts/ids/cls
    const double2 *pts;    // node coordinates in cell order
    const int32_t *ids;    // node ids in cell order
    const int32_t *cls;    // node classes in cell order (nullable)
};

// Conversions between float and double on the integer pipe (bit-field arithmetic; GB300
// runs FP64 conversions on its 1/64-rate FP64 pipe).
namespace {
// float -> double from the IEEE-754 bit fields (exact for normal numbers; subnormals flush to
// a signed zero; inf and NaN are kept).
__device__ __forceinline__ double f32_to_f64(float f)
{
    unsigned u = __float_as_uint(f);
    unsigned e = (u >> 23) & 0xffu;
    unsigned sign = u & 0x80000000u;
    unsigned mant = u & 0x7fffffu;
    unsigned e64 = e == 255u ? 2047u : e + (1023u - 127u);
    unsigned hi = e == 0u ? sign : (sign | (e64 << 20) | (mant >> 3));
    unsigned lo = e == 0u ? 0u : (mant << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// double -> float by truncation of the mantissa (|error| < 1 ulp of float), from the bit
// fields.  Magnitudes above the float range give inf, below the normal range a signed zero;
// NaN stays NaN.
__device__ __forceinline__ float f64_to_f32(double d)
{
    unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    unsigned sign = hi & 0x80000000u;
    int e = (int)((hi >> 20) & 0x7ffu);
    int e32 = e - 1023 + 127;
    unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
    unsigned out;
    if (e == 2047)
        out = sign | 0x7f800000u | ((((hi & 0xfffffu) | lo) != 0u) ? 0x400000u : 0u);
    else if (e32 >= 255)
        out = sign | 0x7f800000u;
    else if (e32 <= 0)
        out = sign;
    else
        out = sign | ((unsigned)e32 << 23) | mant;
    return __uint_as_float(out);
}

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers implemented in the .cu files.  All run on `st` and return a
// cudaError_t of the launch; device-side failures are reported through flag words.
// ---------------------------------------------------------------------------

// exclusive scan of n int64 values (in place allowed), out has n+1 entries (out[n] = total).
cudaError_t scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, void *tmp,
                               size_t tmp_bytes, cudaStream_t st);
size_t scan_tmp_bytes(int64_t n);

// bounding box of N points: out[0..3] = xmin, xmax, ymin, ymax; out_bad[0] = #non-finite.
cudaError_t launch_bbox(const double2 *X, int64_t N, double *partial, int nblocks, double *out,
                        int *out_bad, cudaStream_t st);

cudaError_t launch_grid_fill(const double2 *X, const int32_t *cls, int64_t N, double x0,
                             double y0, double cs, int nx, int ny, int64_t *cell_count,
                             int32_t *cell_of, cudaStream_t st);
cudaError_t launch_grid_scatter(const double2 *X, const int32_t *cls, int64_t N,
                                const int32_t *cell_of, const int64_t *cell_start64,
                                int32_t *cell_start32, int64_t ncell, int32_t *fill,
                                double2 *pts, int32_t *ids, int32_t *gcls, cudaStream_t st);

// kNN: for each query its k nearest grid nodes allowed by the class mask, sorted by
// (d^2, id).  Node queries (node_query): query q is node q_node[q] (or q) with coordinates
// Q[node], class qcls[node], size kq[node] (or kuni), output at out_ptr[node] (or node*k).
// Point queries: coordinates Q[q], class 0 (sees every node), size kuni, output at q*kuni.
cudaError_t launch_knn(const GridDev &g, const double2 *Q, const int32_t *qcls,
                       const int32_t *q_node, bool node_query, int64_t nq,
                       const int32_t *kq, int kuni, int kmax, const int64_t *out_ptr,
                       int32_t *out_idx, double *out_d2, int r0, int *err_flag,
                       int num_sms, cudaStream_t st);

// Weight solves.
struct SolveArgs {
    const double2 *X;
    const double2 *Y;          // nullable: collocated (row y <-> node y)
    const int32_t *nbr;        // stencils
    const int64_t *nbr_ptr;    // nullable: uniform stencils of length n
    const int32_t *n_node;     // nullable per-node stencil size
    const int32_t *deg_node;   // nullable per-node degree
    int n, deg;                // uniform values
    const int32_t *sys_node;   // X node of every system
    const int32_t *sys_list;   // nullable: this launch solves systems sys_list[0..nsys), else
                               // sys_base + 0..nsys
    int64_t sys_base;
    const int64_t *sys_rows;   // nullable: rows of system i are rows_list[sys_rows[i]..sys_rows[i+1])
    const int32_t *rows_list;  // row ids (global evaluation-point ids)
    int64_t nsys;
    int64_t row_begin;         // rows are stored at (row - row_begin)
    const int64_t *row_ptr;    // local row -> offset in col/val
    int32_t *col;              // nnz
    double *val;               // nops * nnz (op-major)
    int64_t nnz;
    int max_s, max_n, max_m;   // largest s / n / m over the systems (smem sizing)
    int64_t *first_bad;        // atomicMin of failing node (init INT64_MAX)
    int32_t *fallback_list;    // mixed: systems needing FP64 (nullable for plain)
    int *fallback_count;
    unsigned long long *hist;  // mixed: refinement histogram [8]
    int max_refine;
    double refine_tol;
    int unscaled_overload;     // generate_operator(X,p,n,polydeg) quirk
    unsigned long long *next_sys;  // nullable, zeroed: the solve kernels claim systems from this
                                   // counter instead of a fixed grid stride
    const int32_t *csc_pos;        // nullable: entry e of the CSR layout is stored at val position
                                   // csc_pos[e] (the CSC order of an export), col stays CSR
};

cudaError_t launch_solve_fp64(const SolveArgs &a, const OpTable &ops, int warps_per_block,
                              int num_sms, cudaStream_t st);
cudaError_t launch_solve_mixed(const SolveArgs &a, const OpTable &ops, int warps_per_block,
                               int num_sms, cudaStream_t st);
// Register-resident FP32 factorisation (max_s <= 64, nops <= 6); cudaErrorNotSupported
// for other shapes.
cudaError_t launch_solve_mixed_reg(const SolveArgs &a, const OpTable &ops, int max_m, int warps_per_block,
                                   int num_sms, cudaStream_t st);
size_t solve_mixed_reg_smem_per_warp(int S, int max_n, int max_m, int nops);
// FP64 re-solve of the systems the mixed kernel queued in a.fallback_list.
cudaError_t launch_solve_fp64_subset(const SolveArgs &a, const OpTable &ops, int warps_per_block,
                                     int num_sms, cudaStream_t st, int64_t count);
size_t solve_fp64_smem_per_warp(int max_s, int max_n, int nops);
size_t solve_mixed_smem_per_warp(int max_s, int max_n, int nops);

// Sparse kernels.
// FP64 SpMV of a general CSR operator (thread per row); uniform stencils use the SELL-32 kernel.
cudaError_t launch_spmv_f64(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                            const double *val, const double *x, double *y, int num_sms, cudaStream_t st);
cudaError_t launch_spmm(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                        const void *val, const void *x, void *y, int nfields, int dtype,
                        cudaStream_t st);
// RK4 stage (mode 0: first stage, 1: middle stages, 2: last stage), see sparse.cu.
// Ghost-node closure building blocks (sparse.cu).
cudaError_t ghost_build(int64_t N, int64_t nb, const int32_t *bnodes, const int32_t *gnodes, const int64_t *row_ptr,
                        const int32_t *col, const double *val, int32_t *gidx, double *M, double *fcol, int *flag,
                        cudaStream_t st);
cudaError_t ghost_apply(int64_t nb, const int32_t *bnodes, const int32_t *gnodes, const int64_t *row_ptr,
                        const int32_t *col, const double *val, const int32_t *gidx, const double *M, void *u, int F,
                        int dtype, double *y, cudaStream_t st);
// CGLS building blocks (sparse.cu).
int lsq_partials();
cudaError_t launch_combine_rows(int64_t rows, const int64_t *row_ptr, const double *val, int64_t nnz, int nops,
                                const double *coef, double *out, cudaStream_t st);
cudaError_t launch_lsq_spmv(int64_t rows, const int64_t *row_ptr, const int32_t *col, const double *val,
                            const double *x, const double *b, double *y, double *part, cudaStream_t st);
cudaError_t launch_lsq_spmv_t(int64_t cols, const int64_t *colptr1, const int64_t *rowval1, int64_t row_begin,
                              const double *vcsc, const double *x, double *y, double *part, cudaStream_t st);
cudaError_t launch_lsq_final(const double *part, double *sc, int slot, int shift, cudaStream_t st);
cudaError_t launch_lsq_update_ur(int64_t cols, int64_t rows, double *u, const double *p, double *r, const double *q,
                                 const double *sc, cudaStream_t st);
cudaError_t launch_lsq_update_p(int64_t cols, double *p, const double *s, const double *sc, int first, cudaStream_t st);
// SELL-32 copy of a uniform-stencil operator set (all operators) and the SpMV on it.
int64_t sell_padded(int64_t rows, int K);
cudaError_t launch_csr_to_sell(int64_t rows, int K, const int32_t *col, const double *val, int nops, int64_t nnz,
                               int32_t *scol, double *sval, cudaStream_t st);
cudaError_t launch_spmv_sell(int64_t rows, int K, const int32_t *scol, const double *sval, const double *x, double *y,
                             int num_sms, cudaStream_t st);
cudaError_t launch_rk4_stage(int64_t rows, const int32_t *order, const int64_t *row_ptr, const int32_t *col,
                             const void *val, const void *w, const void *u, void *acc, void *out,
                             const uint8_t *fixed, int F, double c, int mode, int dtype, int num_sms, cudaStream_t st);
cudaError_t launch_combine_ops(int64_t nnz, const double *const *vals, const double *coef, int nq,
                               double *out64, float *out32, cudaStream_t st);
cudaError_t launch_count_diff(int64_t n, const int32_t *a, const int32_t *b, unsigned long long *cnt,
                              cudaStream_t st);
cudaError_t launch_csc_count(int64_t nnz, const int32_t *col, int64_t *colcount,
                             cudaStream_t st);
cudaError_t launch_csc_scatter(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                               int64_t row_begin, const int64_t *colstart, int64_t *fill,
                               int64_t *rowval, int64_t *perm, cudaStream_t st);
// Sorts each column segment of (rowval, perm) by row; row_limit bounds the row ids.  With inv
// non-null it also writes the inverse permutation inv[perm[p]] = p (int32 positions).
cudaError_t launch_csc_sort_segments(int64_t ncols, const int64_t *colstart, int64_t *rowval,
                                     int64_t *perm, int64_t row_limit, cudaStream_t st, int32_t *inv = nullptr);
cudaError_t launch_gather_f64(int64_t nnz, const int64_t *perm, const double *src, double *dst,
                              cudaStream_t st);
cudaError_t launch_add_i64(int64_t n, int64_t *a, int64_t v, cudaStream_t st);
// Collocated uniform stencils (row r = node r, nbr N x n) solved in C chunks of consecutive
// rows: cp[i] = the number of leading CSC entries (columns referenced only by rows of chunks
// <= i) that are final once chunks 0..i are solved; colstart1 = the 1-based CSC column starts;
// cm: C ints of scratch.
constexpr int RBFFD_MAX_CHUNKS = 8;
cudaError_t launch_chunk_bounds(int64_t N, int n, const int32_t *nbr, int C, const int64_t *colstart1, int *cm,
                                int64_t *cp, cudaStream_t st);
cudaError_t launch_f64_to_f32(int64_t n, const double *a, float *b, cudaStream_t st);
