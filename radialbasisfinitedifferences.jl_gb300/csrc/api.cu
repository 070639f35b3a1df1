// C ABI of librbffd (include/rbffd.h): handles, device-resident operator sets and the
// drop-in entry points that mirror RadialBasisFiniteDifferences.jl's public functions.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "rbffd_internal.cuh"
#include "rk4_tiled.cuh"
#include "tune.cuh"

#define RBFFD_EXPORT extern "C" __attribute__((visibility("default")))

struct rbffd_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    rbffd_options opt{};
    std::string err;
    int num_sms = 0;
    cudaEvent_t ev[8] = {};
    cudaStream_t side = nullptr;  // overlaps the CSC export pattern with the weight solves
    cudaEvent_t side_ev[2] = {};
    static constexpr int kClassStreams = 8;
    cudaStream_t cls_st[kClassStreams] = {};  // one persistent solve launch per shape class
    cudaEvent_t cls_ev[kClassStreams + 1] = {};
    SolveTuner tuner;                         // per-class kernel and CTA size
    std::string tune_report;
};

struct rbffd_opset {
    int64_t N = 0, M = 0, rows = 0, row_begin = 0, nnz = 0;
    int nops = 0;
    int ops[RBFFD_OP_COUNT] = {};
    bool collocated = true, uniform = true;
    int n = 0;
    double2 *X = nullptr;
    int32_t *nbr = nullptr;
    int64_t *nbr_ptr = nullptr;
    int32_t *nn = nullptr;  // X node of each row
    int64_t *row_ptr = nullptr;
    int32_t *col = nullptr;
    double *val = nullptr;
    float *val32 = nullptr;
    int32_t *sell_col = nullptr;  // SELL-32 copy for the SpMV (uniform stencils), built on first use
    double *sell_val = nullptr;
    int64_t *csc_colptr = nullptr, *csc_rowval = nullptr, *csc_perm = nullptr;
    double *csc_tmp = nullptr;
    std::vector<void *> owned;
};

namespace {

thread_local std::string g_create_error;

int fail(rbffd_handle *h, int code, const std::string &msg)
{
    if (h) h->err = msg;
    return code;
}

#define CK(expr)                                                                               \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess)                                                                 \
            return fail(h, _e == cudaErrorMemoryAllocation ? RBFFD_ENOMEM : RBFFD_ECUDA,       \
                        std::string(#expr) + ": " + cudaGetErrorString(_e));                   \
    } while (0)

// Stream-ordered device allocations that are released together.
struct Arena {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit Arena(cudaStream_t s) : st(s) {}
    template <typename T>
    cudaError_t get(T **p, size_t count)
    {
        void *q = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes < 16) bytes = 16;
        cudaError_t e = cudaMallocAsync(&q, bytes, st);
        if (e != cudaSuccess) return e;
        ptrs.push_back(q);
        *p = (T *)q;
        return cudaSuccess;
    }
    template <typename T>
    cudaError_t zeros(T **p, size_t count)
    {
        cudaError_t e = get(p, count);
        if (e != cudaSuccess) return e;
        return cudaMemsetAsync(*p, 0, std::max<size_t>(count * sizeof(T), 16), st);
    }
    void release_to(std::vector<void *> &dst)
    {
        dst.insert(dst.end(), ptrs.begin(), ptrs.end());
        ptrs.clear();
    }
    ~Arena()
    {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
};

__global__ void set_i64(int64_t *a, int64_t v) { *a = v; }

__global__ void iota_i32(int32_t *a, int64_t n, int64_t base)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = (int32_t)(base + i);
}

__global__ void uniform_ptr(int64_t *a, int64_t n, int64_t step)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = i * step;
}

// Shape classes of the mixed solve kernels: bin = 2 * (n > 32) + (m > 16) for n <= 64 and
// m <= 32 (the register kernels' instantiations), NBIN - 1 for anything larger.
constexpr int NBIN = 5;
static_assert(NBIN <= rbffd_handle::kClassStreams, "one class stream per shape class");

// Shape classes of one build run on forked streams (1) or one after another on the handle's
// stream (0).
// Mean nodes per cell of the kNN grid.  Measured at 1M nodes, k = 30 (kNN ms): 0.5 nodes per
// cell 2.95, 0.75 2.73, 1 2.50, 1.25 3.59, 1.5 2.58, 2 2.99, 3 2.67, 4 2.62; the uneven batch
// (k 20..60, boundary classes) 4.50 at 1 against 5.05 at 2.  The first search square (knn_r0)
// follows from it.
#ifndef RBFFD_GRID_NODES_PER_CELL
#define RBFFD_GRID_NODES_PER_CELL 1.0
#endif
// Chunks of rows of the drop-in calls' weight solves, whose CSC values are downloaded while
// the later chunks solve (0: gather and download all values after the solves).
#ifndef RBFFD_EXPORT_CHUNKS
#define RBFFD_EXPORT_CHUNKS 8
#endif
#ifndef RBFFD_CLASS_CONCURRENT
#define RBFFD_CLASS_CONCURRENT 1
#endif
__host__ __device__ inline int solve_bin(int n, int m)
{
    if (n > 64 || m > 32) return NBIN - 1;
    return 2 * (n > 32 ? 1 : 0) + (m > 16 ? 1 : 0);
}

// Per-bin system counts and largest n, m (cnt[0..NBIN), maxn[NBIN..2NBIN), maxm[2NBIN..3NBIN)).
// Per class b: cnt[b] systems, cnt[NBIN + b] their largest n, cnt[2 NBIN + b] their largest m.
// Warp-aggregated into shared memory (a ballot per class), then one global atomic per class
// and block: three global atomics per system on 15 addresses took ~0.9 ms per 524,288 systems.
__global__ void bin_count(const int32_t *sys_node, int64_t nsys, const int32_t *n_node, const int32_t *deg_node,
                          int n0, int deg0, unsigned long long *cnt)
{
    __shared__ unsigned long long sc[3 * NBIN];
    for (int i = threadIdx.x; i < 3 * NBIN; i += blockDim.x) sc[i] = 0ull;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nsys; base += stride) {
        const int64_t t = base + threadIdx.x;
        const bool act = t < nsys;
        int b = -1, n = 0, m = 0;
        if (act) {
            const int j = sys_node[t];
            n = n_node ? n_node[j] : n0;
            const int d = deg_node ? deg_node[j] : deg0;
            m = (d + 1) * (d + 2) / 2;
            b = solve_bin(n, m);
        }
#pragma unroll
        for (int c = 0; c < NBIN; c++) {
            const unsigned mask = __ballot_sync(RBFFD_FULL, b == c);
            if (!mask) continue;
            const unsigned mn = __reduce_max_sync(RBFFD_FULL, b == c ? (unsigned)n : 0u);
            const unsigned mm = __reduce_max_sync(RBFFD_FULL, b == c ? (unsigned)m : 0u);
            if (lane == 0) {
                atomicAdd(&sc[c], (unsigned long long)__popc(mask));
                atomicMax(&sc[NBIN + c], (unsigned long long)mn);
                atomicMax(&sc[2 * NBIN + c], (unsigned long long)mm);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * NBIN; i += blockDim.x) {
        if (i < NBIN) {
            if (sc[i]) atomicAdd(cnt + i, sc[i]);
        } else if (sc[i]) {
            atomicMax(cnt + i, sc[i]);
        }
    }
}

struct BinOffsets {
    int64_t off[NBIN];
};

// The systems of class b listed from list[off[b]] on (in no particular order); one atomic per
// class and warp.
__global__ void bin_scatter(const int32_t *sys_node, int64_t nsys, const int32_t *n_node, const int32_t *deg_node,
                            int n0, int deg0, BinOffsets bo, unsigned long long *fill, int32_t *list)
{
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < nsys; base += stride) {
        const int64_t t = base + threadIdx.x;
        int b = -1;
        if (t < nsys) {
            const int j = sys_node[t];
            const int n = n_node ? n_node[j] : n0;
            const int d = deg_node ? deg_node[j] : deg0;
            b = solve_bin(n, (d + 1) * (d + 2) / 2);
        }
#pragma unroll
        for (int c = 0; c < NBIN; c++) {
            const unsigned mask = __ballot_sync(RBFFD_FULL, b == c);
            if (!mask) continue;
            unsigned long long p0 = 0ull;
            if (lane == __ffs(mask) - 1) p0 = atomicAdd(fill + c, (unsigned long long)__popc(mask));
            p0 = __shfl_sync(RBFFD_FULL, p0, __ffs(mask) - 1);
            if (b == c) list[bo.off[c] + (int64_t)p0 + __popc(mask & below)] = (int32_t)t;
        }
    }
}

__global__ void mark_nodes(const int32_t *nn, int64_t rows, int64_t *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x)
        flag[nn[i]] = 1;
}

__global__ void compact_nodes(const int64_t *flag, const int64_t *pos, int64_t N, int32_t *sys_node)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) sys_node[pos[i]] = (int32_t)i;
}

__global__ void count_rows(const int32_t *nn, int64_t rows, const int64_t *pos, unsigned long long *cnt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[pos[nn[i]]], 1ull);
}

__global__ void scatter_rows(const int32_t *nn, int64_t rows, int64_t row_begin, const int64_t *pos,
                             const int64_t *start, unsigned long long *fill, int32_t *rows_list)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = pos[nn[i]];
        int64_t at = start[s] + (int64_t)atomicAdd(&fill[s], 1ull);
        rows_list[at] = (int32_t)(row_begin + i);
    }
}

// Rows of one system are written in any order; make the order deterministic (ascending).
__global__ void sort_row_lists(const int64_t *start, int64_t nsys, int32_t *rows_list)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nsys; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = start[s], b = start[s + 1];
        for (int64_t i = a + 1; i < b; i++) {
            int32_t v = rows_list[i];
            int64_t j = i - 1;
            while (j >= a && rows_list[j] > v) {
                rows_list[j + 1] = rows_list[j];
                j--;
            }
            rows_list[j + 1] = v;
        }
    }
}

__global__ void row_len_kernel(const int32_t *nn, int64_t rows, const int32_t *n_node, int n_uni,
                               int64_t *len)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x)
        len[i] = n_node ? n_node[nn[i]] : n_uni;
}

__global__ void i32_to_i64(const int32_t *a, int64_t *b, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

__global__ void knn_export(const int32_t *idx, const double *d2, int64_t n, int64_t *oidx, double *odist)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        oidx[i] = (int64_t)idx[i] + 1;
        if (odist) odist[i] = sqrt(d2[i]);
    }
}

// processmesh after its file reads (src/processmesh.jl): triangle centroids, mean of three
// vertices summed in order then divided (extractelements.jl:16-17).  Vertex ids are 1-based;
// an id out of range sets *bad.
__global__ void mesh_centroids(const double2 *V, int64_t nv, const int64_t *tri, int64_t ntri, double2 *C, int *bad)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ntri; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = tri[3 * e] - 1, b = tri[3 * e + 1] - 1, c = tri[3 * e + 2] - 1;
        if (a < 0 || a >= nv || b < 0 || b >= nv || c < 0 || c >= nv) {
            atomicExch(bad, 1);
            C[e] = make_double2(0.0, 0.0);
            continue;
        }
        const double2 pa = V[a], pb = V[b], pc = V[c];
        C[e] = make_double2(__ddiv_rn(__dadd_rn(__dadd_rn(pa.x, pb.x), pc.x), 3.0),
                            __ddiv_rn(__dadd_rn(__dadd_rn(pa.y, pb.y), pc.y), 3.0));
    }
}

// Boundary line elements: midpoints, and the unit normal [-dy, dx] / |.| and tangent
// [dx, dy] / |.| of calculatenormal (src/calculatenormal.jl:1-17), with |.| =
// sqrt(dy^2 + dx^2) in that order, every operation rounded once.
__global__ void mesh_lines(const double2 *V, int64_t nv, const int64_t *bc, int64_t nbc, double2 *M, double2 *Nrm,
                           double2 *Tng, int *bad)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nbc; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = bc[2 * e] - 1, b = bc[2 * e + 1] - 1;
        if (a < 0 || a >= nv || b < 0 || b >= nv) {
            atomicExch(bad, 1);
            M[e] = Nrm[e] = Tng[e] = make_double2(0.0, 0.0);
            continue;
        }
        const double2 pa = V[a], pb = V[b];
        M[e] = make_double2(__ddiv_rn(__dadd_rn(pa.x, pb.x), 2.0), __ddiv_rn(__dadd_rn(pa.y, pb.y), 2.0));
        const double dx = __dsub_rn(pb.x, pa.x), dy = __dsub_rn(pb.y, pa.y);
        const double len = __dsqrt_rn(__dadd_rn(__dmul_rn(dy, dy), __dmul_rn(dx, dx)));
        Nrm[e] = make_double2(__ddiv_rn(-dy, len), __ddiv_rn(dx, len));
        Tng[e] = make_double2(__ddiv_rn(dx, len), __ddiv_rn(dy, len));
    }
}

// One CTA: the ghost offset (the mean distance of the midpoints to their nearest centroid,
// per-thread sums over contiguous ranges then a fixed tree: a deterministic order), the
// orientation sign from the first line (processmesh.jl:120-133), and the ghost nodes
// midpoint + normal * offset (genghostnodes.jl:1-6).  Needs blockDim.x == 256.
__global__ void mesh_ghosts(const double2 *C, const double2 *M, const int32_t *nn, const double *d2, int64_t nbc,
                            double2 *Nrm, double2 *Tng, double2 *G, double *offset)
{
    __shared__ double part[256];
    const int t = threadIdx.x;
    const int64_t chunk = (nbc + 255) / 256, e0 = t * chunk, e1 = e0 + chunk < nbc ? e0 + chunk : nbc;
    double s = 0.0;
    for (int64_t e = e0; e < e1; e++) s = __dadd_rn(s, __dsqrt_rn(d2[e]));
    part[t] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) part[t] = __dadd_rn(part[t], part[t + w]);
        __syncthreads();
    }
    const double off = fabs(__ddiv_rn(part[0], (double)nbc));
    const double2 m0 = M[0], c0 = C[nn[0]], n0 = Nrm[0];
    const double dt = __dadd_rn(__dmul_rn(__dsub_rn(m0.x, c0.x), n0.x), __dmul_rn(__dsub_rn(m0.y, c0.y), n0.y));
    const double sg = dt > 0.0 ? 1.0 : (dt < 0.0 ? -1.0 : dt);  // Julia's sign
    __syncthreads();  // every thread has read the first normal
    for (int64_t e = t; e < nbc; e += blockDim.x) {
        const double2 nv = make_double2(__dmul_rn(sg, Nrm[e].x), __dmul_rn(sg, Nrm[e].y));
        Nrm[e] = nv;
        Tng[e] = make_double2(__dmul_rn(sg, Tng[e].x), __dmul_rn(sg, Tng[e].y));
        G[e] = make_double2(__dadd_rn(M[e].x, __dmul_rn(nv.x, off)), __dadd_rn(M[e].y, __dmul_rn(nv.y, off)));
    }
    if (t == 0) *offset = off;
}

int nblk(int64_t n, int t = 256)
{
    int64_t b = (n + t - 1) / t;
    if (b < 1) b = 1;
    if (b > 65535 * 8) b = 65535 * 8;
    return (int)b;
}

int npoly_h(int d) { return (d + 1) * (d + 2) / 2; }

double ff_h(double x, int q)
{
    double c = 1.0;
    for (int t = 0; t < q; t++) c *= (x - t);
    return c;
}

double fact_h(int n)
{
    double f = 1;
    for (int i = 2; i <= n; i++) f *= i;
    return f;
}

bool comp_terms(int p, int a, int b, OpComp *c)
{
    c->a = a;
    c->b = b;
    c->nterm = 0;
    for (int i = 0; 2 * i <= a; i++)
        for (int j = 0; 2 * j <= b; j++) {
            int q = a + b - i - j;
            double coef = fact_h(a) / (fact_h(i) * fact_h(a - 2 * i)) * fact_h(b) /
                          (fact_h(j) * fact_h(b - 2 * j)) * ldexp(1.0, a - 2 * i + b - 2 * j) *
                          ff_h(0.5 * p, q);
            if (coef == 0.0) continue;
            if (c->nterm >= RBFFD_MAX_TERMS) return false;
            c->t[c->nterm++] = RbfTerm{coef, a - 2 * i, b - 2 * j, p - 2 * q};
        }
    return true;
}

// Host copies of small per-node arrays (for sizing / validation).
bool fetch_i32(rbffd_handle *h, const int32_t *src, int64_t n, int memspace, std::vector<int32_t> &dst)
{
    dst.resize(n);
    if (memspace == RBFFD_MEM_DEVICE) {
        if (cudaMemcpyAsync(dst.data(), src, n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
            return false;
        return cudaStreamSynchronize(h->stream) == cudaSuccess;
    }
    memcpy(dst.data(), src, n * sizeof(int32_t));
    return true;
}

// Upload (or borrow) an array of `bytes`; device pointers are used in place when aligned.
template <typename T>
cudaError_t stage(rbffd_handle *h, Arena &ar, const void *src, size_t count, int memspace, T **dst)
{
    if (memspace == RBFFD_MEM_DEVICE && ((uintptr_t)src % alignof(T)) == 0) {
        *dst = (T *)src;
        return cudaSuccess;
    }
    cudaError_t e = ar.get(dst, count);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(*dst, src, count * sizeof(T),
                           memspace == RBFFD_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                           h->stream);
}

struct GridBuild {
    GridDev g{};
    int64_t ncell = 0;
    double rho = 1;
};

int build_grid(rbffd_handle *h, Arena &ar, const double2 *dX, const int32_t *dcls, int64_t N, GridBuild &gb)
{
    const int nb = 256;
    double *partial, *box;
    int *bad;
    CK(ar.get(&partial, 4 * nb));
    CK(ar.get(&box, 4));
    CK(ar.get(&bad, 1));
    CK(launch_bbox(dX, N, partial, nb, box, bad, h->stream));
    double hb[4];
    int hbad = 0;
    CK(cudaMemcpyAsync(hb, box, sizeof(hb), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (hbad) return fail(h, RBFFD_EINVAL, "non-finite node coordinates");
    double w = hb[1] - hb[0], hh = hb[3] - hb[2];
    double area = (w > 0 ? w : 1.0) * (hh > 0 ? hh : 1.0);
    double cs = sqrt(RBFFD_GRID_NODES_PER_CELL * area / (double)N);
    if (!(cs > 0)) cs = 1.0;
    int64_t nx = (int64_t)(w / cs) + 1, ny = (int64_t)(hh / cs) + 1;
    while (nx * ny > 4 * N + 16) {
        cs *= 1.5;
        nx = (int64_t)(w / cs) + 1;
        ny = (int64_t)(hh / cs) + 1;
    }
    int64_t ncell = nx * ny;
    int64_t *count, *start64;
    int32_t *cell_of, *start32, *fill, *ids, *gcls = nullptr;
    double2 *pts;
    void *tmp;
    size_t tb = scan_tmp_bytes(ncell);
    CK(ar.zeros(&count, ncell + 1));
    CK(ar.get(&start64, ncell + 1));
    CK(ar.get(&cell_of, N));
    CK(ar.get(&start32, ncell + 1));
    CK(ar.get(&fill, ncell));
    CK(ar.get(&ids, N));
    CK(ar.get(&pts, N));
    if (dcls) CK(ar.get(&gcls, N));
    CK(ar.get((char **)&tmp, tb));
    CK(launch_grid_fill(dX, dcls, N, hb[0], hb[2], cs, (int)nx, (int)ny, count, cell_of, h->stream));
    CK(scan_exclusive_i64(count, start64, ncell, tmp, tb, h->stream));
    CK(launch_grid_scatter(dX, dcls, N, cell_of, start64, start32, ncell, fill, pts, ids, gcls, h->stream));
    gb.g = GridDev{hb[0], hb[2], cs, (int)nx, (int)ny, start32, pts, ids, gcls};
    gb.ncell = ncell;
    gb.rho = (double)N / (double)ncell;
    return RBFFD_OK;
}

// The kNN's first search square: the smallest radius whose square is expected to hold k nodes
// (plus RBFFD_KNN_R0_ADJ).  At 1 node per cell, k = 30: 3.00 / 2.50 / 2.75 ms for -1 / 0 / +1.
#ifndef RBFFD_KNN_R0_ADJ
#define RBFFD_KNN_R0_ADJ 0
#endif
int knn_r0(double rho, int k)
{
    double r = (sqrt((double)k / (rho > 0 ? rho : 1.0)) - 1.0) * 0.5;
    int r0 = (int)ceil(r) + RBFFD_KNN_R0_ADJ;
    return r0 < 0 ? 0 : r0;
}

float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

struct Flags {
    int knn_err;
    int fallback_count;
    int64_t first_bad;
    unsigned long long hist[8];
};

int ops_from_mask(uint32_t mask, int *ops)
{
    int n = 0;
    for (int b = 0; b < RBFFD_OP_COUNT; b++)
        if (mask & (1u << b)) ops[n++] = b;
    return n;
}

// CTA size of the FP64 re-solve of the fallback queue (a small, irregular launch that the
// autotuner does not time): the largest CTA (<= 8 warps) whose shared memory still lets >= 2
// CTAs share an SM.
int fallback_wpb(rbffd_handle *h, size_t per_warp)
{
    if (h->opt.warps_per_block > 0) return h->opt.warps_per_block;
    const size_t budget = 110 * 1024;
    int w = 8;
    while (w > 1 && per_warp * w > budget) w >>= 1;
    return w;
}

}  // namespace

void set_handleless_error(const std::string &msg) { g_create_error = msg; }

// Closed-form right-hand sides for r^3 with Dx/Dy/Lap in the register Schur kernel (0: the
// term table for every operator).
#ifndef RBFFD_RHS_CLOSED
#define RBFFD_RHS_CLOSED 1
#endif
bool build_op_table(const int *ops, int nops, int p, int k_deriv, OpTable *t, std::string *err)
{
    memset(t, 0, sizeof(*t));
    t->nops = nops;
    t->p = p;
    int closed = 1;
    for (int q = 0; q < nops; q++) {
        switch (ops[q]) {
        case RBFFD_OP_E: break;
        case RBFFD_OP_DX:
        case RBFFD_OP_DY: closed |= 2; break;
        case RBFFD_OP_DXX:
        case RBFFD_OP_DYY: closed |= 2 | 8; break;
        case RBFFD_OP_DXY: closed |= 8; break;
        case RBFFD_OP_LAP: closed |= 4; break;
        default: closed = 0;  // any other operator: the term table
        }
        if (!closed) break;
    }
    t->r3_closed = (RBFFD_RHS_CLOSED && p == 3) ? closed : 0;
    bool hv4 = nops > 0;
    for (int q = 0; q < nops; q++) hv4 = hv4 && (ops[q] == RBFFD_OP_DXK || ops[q] == RBFFD_OP_DYK);
    t->r5_hv4 = RBFFD_RHS_CLOSED && p == 5 && k_deriv == 4 && hv4;
    for (int q = 0; q < nops; q++) {
        OpDesc &d = t->op[q];
        int code = ops[q];
        int comps[2][2] = {{0, 0}, {0, 0}};
        d.ncomp = 1;
        switch (code) {
        case RBFFD_OP_E: break;
        case RBFFD_OP_DX: comps[0][0] = 1; break;
        case RBFFD_OP_DY: comps[0][1] = 1; break;
        case RBFFD_OP_DXX: comps[0][0] = 2; break;
        case RBFFD_OP_DYY: comps[0][1] = 2; break;
        case RBFFD_OP_DXY: comps[0][0] = 1; comps[0][1] = 1; break;
        case RBFFD_OP_LAP: comps[0][0] = 2; comps[1][1] = 2; d.ncomp = 2; break;
        case RBFFD_OP_DXK: comps[0][0] = k_deriv; break;
        case RBFFD_OP_DYK: comps[0][1] = k_deriv; break;
        case RBFFD_OP_HV: comps[0][0] = k_deriv; comps[1][1] = k_deriv; d.ncomp = 2; break;
        default: *err = "unknown operator code"; return false;
        }
        d.post_scale = d.ncomp == 1;
        for (int c = 0; c < d.ncomp; c++)
            if (!comp_terms(p, comps[c][0], comps[c][1], &d.c[c])) {
                *err = "derivative order too high";
                return false;
            }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Handle.
// ---------------------------------------------------------------------------
RBFFD_EXPORT int rbffd_version(void) { return RBFFD_VERSION_MAJOR * 100 + RBFFD_VERSION_MINOR; }

RBFFD_EXPORT const char *rbffd_status_string(int s)
{
    switch (s) {
    case RBFFD_OK: return "ok";
    case RBFFD_EINVAL: return "invalid argument";
    case RBFFD_ECUDA: return "CUDA error";
    case RBFFD_ESINGULAR: return "singular local system";
    case RBFFD_ETIMEOUT: return "device wait timed out";
    case RBFFD_ENOMEM: return "out of memory";
    default: return "unknown status";
    }
}

RBFFD_EXPORT int rbffd_create(const rbffd_options *opt, rbffd_handle **out)
{
    if (!out) return RBFFD_EINVAL;
    *out = nullptr;
    rbffd_handle *h = new rbffd_handle();
    if (opt) h->opt = *opt;
    if (h->opt.max_refine <= 0) h->opt.max_refine = 6;
    if (!(h->opt.refine_tol > 0)) h->opt.refine_tol = 1e-12;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        delete h;
        return RBFFD_ECUDA;
    }
    h->device = h->opt.device;
    if (h->device < 0 || h->device >= ndev) {
        g_create_error = "device ordinal out of range";
        delete h;
        return RBFFD_EINVAL;
    }
    cudaDeviceProp prop;
    if ((e = cudaSetDevice(h->device)) != cudaSuccess ||
        (e = cudaGetDeviceProperties(&prop, h->device)) != cudaSuccess) {
        g_create_error = std::string("cuda: ") + cudaGetErrorString(e);
        delete h;
        return RBFFD_ECUDA;
    }
    if (prop.major * 10 + prop.minor < 100) {
        g_create_error = "librbffd is built for sm_103a (Blackwell); device is sm_" +
                         std::to_string(prop.major) + std::to_string(prop.minor);
        delete h;
        return RBFFD_ECUDA;
    }
    h->num_sms = prop.multiProcessorCount;
    // Keep freed stream-ordered memory in the device pool instead of returning it to the
    // driver at every synchronisation: operator sets of ~1 GB are built and dropped per call.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, h->device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        g_create_error = std::string("cuda: ") + cudaGetErrorString(e);
        delete h;
        return RBFFD_ECUDA;
    }
    for (auto &ev : h->ev) cudaEventCreate(&ev);
    if ((e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking)) != cudaSuccess) {
        g_create_error = std::string("cuda: ") + cudaGetErrorString(e);
        cudaStreamDestroy(h->stream);
        delete h;
        return RBFFD_ECUDA;
    }
    for (auto &ev : h->side_ev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (auto &cs : h->cls_st) cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    for (auto &ev : h->cls_ev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    *out = h;
    return RBFFD_OK;
}

RBFFD_EXPORT void rbffd_destroy(rbffd_handle *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->side);
    for (auto &ev : h->ev) cudaEventDestroy(ev);
    for (auto &ev : h->side_ev) cudaEventDestroy(ev);
    for (auto &ev : h->cls_ev) cudaEventDestroy(ev);
    for (auto &cs : h->cls_st) cudaStreamDestroy(cs);
    cudaStreamDestroy(h->stream);
    cudaStreamDestroy(h->side);
    delete h;
}

RBFFD_EXPORT const char *rbffd_last_error(const rbffd_handle *h)
{
    if (!h) return g_create_error.c_str();
    return h->err.c_str();
}

RBFFD_EXPORT const char *rbffd_autotune_report(const rbffd_handle *h)
{
    if (!h) return "";
    return h->tune_report.c_str();
}

RBFFD_EXPORT void *rbffd_stream(rbffd_handle *h) { return h ? (void *)h->stream : nullptr; }

RBFFD_EXPORT int rbffd_synchronize(rbffd_handle *h)
{
    if (!h) return RBFFD_EINVAL;
    CK(cudaStreamSynchronize(h->stream));
    return RBFFD_OK;
}

// ---------------------------------------------------------------------------
// Operator sets.
// ---------------------------------------------------------------------------
// Used by opset_build for a collocated uniform set, whose CSR pattern is known before the
// weights (col = nbr, row r at r * n): build() runs on the main stream before the weight
// solves are launched, download() after they are enqueued (copies on the side stream overlap
// the solves).  The drop-in calls use it for the CSC pattern of their outputs.
struct PatternHook {
    virtual int build(rbffd_handle *h, int64_t N, int n, const int64_t *row_ptr, const int32_t *nbr) = 0;
    virtual int download(rbffd_handle *h) = 0;
    // > 0: the values are written straight into CSC order (csc_pos) and the systems are solved
    // in that many chunks of consecutive rows; chunk_done(i) runs once chunk i's launch is on
    // stream st (it may download the columns that chunks 0..i complete).
    virtual int chunks() const { return 0; }
    virtual const int32_t *csc_pos() const { return nullptr; }
    virtual int chunk_done(rbffd_handle *, int, cudaStream_t, const double *, int64_t) { return RBFFD_OK; }
    // After the FP64 re-solve of stalled systems (n_fallback of them).
    virtual void solved(int64_t) {}
    virtual ~PatternHook() {}
};

static int opset_build(rbffd_handle *h, const rbffd_problem *pb, int unscaled, rbffd_opset **out,
                       rbffd_stats *stats, PatternHook *hook = nullptr)
{
    if (!h) return RBFFD_EINVAL;
    if (!pb || !out) return fail(h, RBFFD_EINVAL, "null argument");
    *out = nullptr;
    cudaSetDevice(h->device);
    const int64_t N = pb->N;
    if (N <= 0 || !pb->X) return fail(h, RBFFD_EINVAL, "empty node set");
    if (N > INT32_MAX / 2) return fail(h, RBFFD_EINVAL, "too many nodes");
    if (pb->p <= 0) return fail(h, RBFFD_EINVAL, "PHS exponent must be positive");
    if (pb->precision != RBFFD_PREC_FP64 && pb->precision != RBFFD_PREC_MIXED)
        return fail(h, RBFFD_EINVAL, "unknown precision mode");
    if (pb->memspace != RBFFD_MEM_HOST && pb->memspace != RBFFD_MEM_DEVICE)
        return fail(h, RBFFD_EINVAL, "unknown memspace");
    bool collocated = pb->Y == nullptr || (pb->Y == pb->X && pb->M == N);
    if (unscaled) collocated = true;
    int64_t M = collocated ? N : pb->M;
    if (M <= 0) return fail(h, RBFFD_EINVAL, "empty evaluation set");
    int64_t rb = pb->row_begin, re = pb->row_end > 0 ? pb->row_end : M;
    if (rb < 0 || rb >= re || re > M) return fail(h, RBFFD_EINVAL, "bad row range");
    int64_t rows = re - rb;
    int ops[RBFFD_OP_COUNT];
    if (pb->op_mask == 0 || (pb->op_mask >> RBFFD_OP_COUNT)) return fail(h, RBFFD_EINVAL, "bad op mask");
    int nops = ops_from_mask(pb->op_mask, ops);
    bool needk = (pb->op_mask & (RBFFD_MASK(RBFFD_OP_DXK) | RBFFD_MASK(RBFFD_OP_DYK) | RBFFD_MASK(RBFFD_OP_HV))) != 0;
    if (needk && (pb->k_deriv < 0 || pb->k_deriv > 10)) return fail(h, RBFFD_EINVAL, "k_deriv out of range");
    OpTable table;
    std::string terr;
    if (!build_op_table(ops, nops, pb->p, pb->k_deriv, &table, &terr)) return fail(h, RBFFD_EINVAL, terr);

    // stencil sizes and degrees
    std::vector<int32_t> hn, hdeg;
    bool uniform = !pb->n_per_node && !pb->deg_per_node;
    int max_n = pb->n, max_deg = pb->polydeg, max_s = 0;
    if (pb->n_per_node) {
        if (!fetch_i32(h, pb->n_per_node, N, pb->memspace, hn)) return fail(h, RBFFD_ECUDA, "copy n_per_node");
        max_n = *std::max_element(hn.begin(), hn.end());
    }
    if (pb->deg_per_node) {
        if (!fetch_i32(h, pb->deg_per_node, N, pb->memspace, hdeg)) return fail(h, RBFFD_ECUDA, "copy deg_per_node");
        max_deg = *std::max_element(hdeg.begin(), hdeg.end());
    }
    for (int64_t i = 0; i < N; i++) {
        int n = hn.empty() ? pb->n : hn[i];
        int d = hdeg.empty() ? pb->polydeg : hdeg[i];
        if (n < 1 || n > N || n > RBFFD_MAX_K) return fail(h, RBFFD_EINVAL, "stencil size out of range");
        if (d < 0 || d > RBFFD_MAX_DEG) return fail(h, RBFFD_EINVAL, "polynomial degree out of range");
        max_s = std::max(max_s, n + npoly_h(d));
        if (hn.empty() && hdeg.empty()) break;
    }
    if (max_s > RBFFD_MAX_S) return fail(h, RBFFD_EINVAL, "local system larger than 128");
    if (pb->precision == RBFFD_PREC_MIXED && unscaled)
        return fail(h, RBFFD_EINVAL, "the unscaled overload is FP64 only");

    cudaStream_t st = h->stream;
    Arena keep(st), tmp(st);
    rbffd_opset *os = new rbffd_opset();
    auto bail = [&](int code) {
        delete os;
        return code;
    };
    int rc;
    CK(cudaEventRecord(h->ev[0], st));
    // ---- upload
    double2 *dX, *dY = nullptr;
    int32_t *dcls = nullptr, *dn = nullptr, *ddeg = nullptr;
    {
        cudaError_t e = stage(h, keep, pb->X, (size_t)N, pb->memspace, &dX);
        if (e == cudaSuccess && !collocated) e = stage(h, tmp, pb->Y, (size_t)M, pb->memspace, &dY);
        if (e == cudaSuccess && pb->node_class) e = stage(h, tmp, pb->node_class, (size_t)N, pb->memspace, &dcls);
        if (e == cudaSuccess && pb->n_per_node) e = stage(h, keep, pb->n_per_node, (size_t)N, pb->memspace, &dn);
        if (e == cudaSuccess && pb->deg_per_node) e = stage(h, tmp, pb->deg_per_node, (size_t)N, pb->memspace, &ddeg);
        if (e != cudaSuccess) return bail(fail(h, RBFFD_ECUDA, std::string("upload: ") + cudaGetErrorString(e)));
    }
    CK(cudaEventRecord(h->ev[1], st));
    // ---- grid
    GridBuild gb;
    if ((rc = build_grid(h, tmp, dX, dcls, N, gb)) != RBFFD_OK) return bail(rc);
    CK(cudaEventRecord(h->ev[2], st));
    Flags *dflags;
    CK(tmp.zeros(&dflags, 1));
    set_i64<<<1, 1, 0, st>>>(&dflags->first_bad, INT64_MAX);  // stream-ordered: no host round trip
    // ---- nearest node of every row and the systems to factor
    int32_t *nn;  // rows
    int32_t *sys_node;
    int64_t *sys_rows = nullptr;
    int32_t *rows_list = nullptr;
    int64_t nsys;
    CK(keep.get(&nn, rows));
    if (collocated) {
        iota_i32<<<nblk(rows), 256, 0, st>>>(nn, rows, rb);
        sys_node = nn;
        nsys = rows;
    } else {
        // knn(tree, Y, 1): point queries, every node visible (calculateneighbors.jl:90-94)
        CK(launch_knn(gb.g, dY + rb, nullptr, nullptr, false, rows, nullptr, 1, 1, nullptr, nn, nullptr,
                      knn_r0(gb.rho, 1), &dflags->knn_err, h->num_sms, st));
        int64_t *flag, *pos;
        size_t tb = scan_tmp_bytes(N);
        void *scratch;
        CK(tmp.zeros(&flag, N));
        CK(tmp.get(&pos, N + 1));
        CK(tmp.get((char **)&scratch, tb));
        mark_nodes<<<nblk(rows), 256, 0, st>>>(nn, rows, flag);
        CK(scan_exclusive_i64(flag, pos, N, scratch, tb, st));
        CK(cudaMemcpyAsync(&nsys, pos + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CK(tmp.get(&sys_node, nsys));
        compact_nodes<<<nblk(N), 256, 0, st>>>(flag, pos, N, sys_node);
        int64_t *cnt, *fill;
        size_t tb2 = scan_tmp_bytes(nsys);
        void *scratch2;
        CK(tmp.zeros(&cnt, nsys + 1));
        CK(tmp.zeros(&fill, nsys));
        CK(tmp.get(&sys_rows, nsys + 1));
        CK(tmp.get(&rows_list, rows));
        CK(tmp.get((char **)&scratch2, tb2));
        count_rows<<<nblk(rows), 256, 0, st>>>(nn, rows, pos, (unsigned long long *)cnt);
        CK(scan_exclusive_i64(cnt, sys_rows, nsys, scratch2, tb2, st));
        scatter_rows<<<nblk(rows), 256, 0, st>>>(nn, rows, rb, pos, sys_rows, (unsigned long long *)fill, rows_list);
        sort_row_lists<<<nblk(nsys), 256, 0, st>>>(sys_rows, nsys, rows_list);
    }
    // ---- stencils: knn(tree, X, n, true) / calculateneighbors masks
    int32_t *nbr;
    int64_t *nbr_ptr = nullptr;
    if (uniform) {
        CK(keep.get(&nbr, (size_t)N * max_n));
    } else {
        int64_t *len;
        size_t tb = scan_tmp_bytes(N);
        void *scratch;
        CK(tmp.get(&len, N));
        CK(keep.get(&nbr_ptr, N + 1));
        CK(tmp.get((char **)&scratch, tb));
        if (dn) {
            i32_to_i64<<<nblk(N), 256, 0, st>>>(dn, len, N);
        } else {
            // uniform n with per-node degrees
            std::vector<int64_t> hl(N, pb->n);
            CK(cudaMemcpyAsync(len, hl.data(), N * sizeof(int64_t), cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));
        }
        CK(scan_exclusive_i64(len, nbr_ptr, N, scratch, tb, st));
        int64_t tot;
        CK(cudaMemcpyAsync(&tot, nbr_ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CK(keep.get(&nbr, tot));
    }
    CK(launch_knn(gb.g, dX, dcls, sys_node, true, nsys, dn, pb->n, max_n, nbr_ptr, nbr, nullptr,
                  knn_r0(gb.rho, max_n), &dflags->knn_err, h->num_sms, st));
    CK(cudaEventRecord(h->ev[3], st));
    // ---- CSR row pointers
    int64_t *row_ptr;
    int64_t nnz;
    CK(keep.get(&row_ptr, rows + 1));
    if (uniform) {
        uniform_ptr<<<nblk(rows + 1), 256, 0, st>>>(row_ptr, rows, pb->n);
        nnz = rows * (int64_t)pb->n;
    } else {
        int64_t *len;
        size_t tb = scan_tmp_bytes(rows);
        void *scratch;
        CK(tmp.get(&len, rows));
        CK(tmp.get((char **)&scratch, tb));
        row_len_kernel<<<nblk(rows), 256, 0, st>>>(nn, rows, dn, pb->n, len);
        CK(scan_exclusive_i64(len, row_ptr, rows, scratch, tb, st));
        CK(cudaMemcpyAsync(&nnz, row_ptr + rows, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    const bool hook_on = hook && collocated && uniform && rb == 0 && rows == N;
    if (hook_on) {
        int rc2 = hook->build(h, N, pb->n, row_ptr, nbr);
        if (rc2) return bail(rc2);
    }
    const int nchunk = hook_on ? hook->chunks() : 0;
    if (nchunk > 0) {  // the pattern's download first on the side stream, the values' behind it
        int rc2 = hook->download(h);
        if (rc2) return bail(rc2);
    }
    int32_t *col;
    double *val;
    CK(keep.get(&col, nnz));
    CK(keep.get(&val, (size_t)nnz * nops));
    // ---- weight solves
    SolveArgs a{};
    int64_t n_bin_launches = 0, n_solve_launches = 1;
    a.X = dX;
    a.Y = collocated ? nullptr : dY;
    a.nbr = nbr;
    a.nbr_ptr = nbr_ptr;
    a.n_node = dn;
    a.deg_node = ddeg;
    a.n = pb->n;
    a.deg = pb->polydeg;
    a.sys_node = sys_node;
    a.sys_rows = sys_rows;
    a.rows_list = rows_list;
    a.nsys = nsys;
    a.row_begin = rb;
    a.row_ptr = row_ptr;
    a.col = col;
    a.val = val;
    a.nnz = nnz;
    a.max_s = max_s;
    a.max_n = max_n;
    a.max_m = npoly_h(max_deg);
    a.first_bad = &dflags->first_bad;
    a.max_refine = h->opt.max_refine;
    a.refine_tol = h->opt.refine_tol;
    a.unscaled_overload = unscaled;
    if (nchunk > 0) a.csc_pos = hook->csc_pos();
    int32_t *fb_list = nullptr;
    if (pb->precision == RBFFD_PREC_MIXED) {
        CK(tmp.get(&fb_list, nsys));
        a.fallback_list = fb_list;
        a.fallback_count = &dflags->fallback_count;
        a.hist = dflags->hist;
    }
    // Systems binned by shape class (per-node n / degree arrays), so that small stencils do
    // not run with the shared-memory and register budget of the largest; each class is one
    // persistent launch (warps claim systems from a counter) with the kernel and CTA size the
    // autotuner chose for that class, and the classes' launches run on forked streams so that
    // one class's tail overlaps the next class's start.
    std::vector<SolveArgs> launches;
    if ((dn || ddeg) && nsys > 0) {
        unsigned long long *cnt, hc[3 * NBIN];
        int32_t *list;
        CK(tmp.zeros(&cnt, 4 * NBIN));
        CK(tmp.get(&list, nsys));
        const int bblk = std::min(nblk(nsys), h->num_sms * 8);
        bin_count<<<bblk, 256, 0, st>>>(sys_node, nsys, dn, ddeg, pb->n, pb->polydeg, cnt);
        CK(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        BinOffsets bo;
        int64_t o = 0;
        for (int b = 0; b < NBIN; b++) {
            bo.off[b] = o;
            o += (int64_t)hc[b];
        }
        bin_scatter<<<bblk, 256, 0, st>>>(sys_node, nsys, dn, ddeg, pb->n, pb->polydeg, bo,
                                                cnt + 3 * NBIN, list);
        n_bin_launches = 2;
        for (int b = 0; b < NBIN; b++) {
            if (hc[b] == 0) continue;
            SolveArgs ab = a;
            ab.sys_list = list + bo.off[b];
            ab.nsys = (int64_t)hc[b];
            ab.max_n = (int)hc[NBIN + b];
            ab.max_m = (int)hc[2 * NBIN + b];
            ab.max_s = ab.max_n + ab.max_m;
            launches.push_back(ab);
        }
    } else if (nchunk > 1 && nsys >= (int64_t)nchunk * 1024) {
        // chunks of consecutive systems (rows), each its own persistent launch
        for (int c = 0; c < nchunk; c++) {
            SolveArgs ac = a;
            ac.sys_base = (int64_t)c * nsys / nchunk;
            ac.nsys = (int64_t)(c + 1) * nsys / nchunk - ac.sys_base;
            launches.push_back(ac);
        }
    } else {
        launches.push_back(a);
    }
    const bool chunked = nchunk > 0 && (int)launches.size() == nchunk;
    {
        unsigned long long *claim;
        int32_t *sample_list;
        CK(tmp.zeros(&claim, launches.size()));
        CK(tmp.get(&sample_list, tune_sample_systems(h->num_sms)));
        for (size_t i = 0; i < launches.size(); i++) launches[i].next_sys = claim + i;
        std::vector<SolveConfig> cfg(launches.size());
        for (size_t i = 0; i < launches.size(); i++)
            CK(h->tuner.choose(launches[i], table, pb->precision, h->opt.warps_per_block, h->num_sms, sample_list, st,
                               &cfg[i]));
        if (chunked) {
            // chunks alternate between two forked streams, so that a chunk's persistent CTAs
            // start as the previous chunk's drain; the columns each chunk completes are
            // downloaded on the side stream meanwhile (in chunk order there, so a download
            // also follows every earlier chunk)
            CK(cudaEventRecord(h->cls_ev[rbffd_handle::kClassStreams], st));
            for (int k = 0; k < 2; k++) CK(cudaStreamWaitEvent(h->cls_st[k], h->cls_ev[rbffd_handle::kClassStreams], 0));
            for (size_t i = 0; i < launches.size(); i++) {
                cudaStream_t cs = h->cls_st[i & 1];
                CK(launch_solve_config(launches[i], table, cfg[i], h->num_sms, cs));
                int rc2 = hook->chunk_done(h, (int)i, cs, val, nnz);
                if (rc2) return bail(rc2);
            }
            for (int k = 0; k < 2; k++) {
                CK(cudaEventRecord(h->cls_ev[k], h->cls_st[k]));
                CK(cudaStreamWaitEvent(st, h->cls_ev[k], 0));
            }
        } else if (launches.size() == 1 || !RBFFD_CLASS_CONCURRENT) {
            for (size_t i = 0; i < launches.size(); i++)
                CK(launch_solve_config(launches[i], table, cfg[i], h->num_sms, st));
            for (int c = 0; c < nchunk; c++) {  // values in CSC order but solved in one launch
                int rc2 = hook->chunk_done(h, c, st, val, nnz);
                if (rc2) return bail(rc2);
            }
        } else {
            CK(cudaEventRecord(h->cls_ev[rbffd_handle::kClassStreams], st));
            for (size_t i = 0; i < launches.size(); i++) {
                cudaStream_t cs = h->cls_st[i];
                CK(cudaStreamWaitEvent(cs, h->cls_ev[rbffd_handle::kClassStreams], 0));
                CK(launch_solve_config(launches[i], table, cfg[i], h->num_sms, cs));
                CK(cudaEventRecord(h->cls_ev[i], cs));
            }
            for (size_t i = 0; i < launches.size(); i++) CK(cudaStreamWaitEvent(st, h->cls_ev[i], 0));
        }
        n_solve_launches = (int64_t)launches.size();
        h->tune_report = h->tuner.report();
    }
    if (hook_on && nchunk == 0) {
        int rc2 = hook->download(h);
        if (rc2) return bail(rc2);
    }
    CK(cudaEventRecord(h->ev[4], st));
    Flags hf;
    CK(cudaMemcpyAsync(&hf, dflags, sizeof(Flags), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (pb->precision == RBFFD_PREC_MIXED && hf.fallback_count > 0 && !hf.knn_err) {
        int wpb = fallback_wpb(h, solve_fp64_smem_per_warp(max_s, max_n, nops));
        CK(launch_solve_fp64_subset(a, table, wpb, h->num_sms, st, hf.fallback_count));
        CK(cudaMemcpyAsync(&hf.first_bad, &dflags->first_bad, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    }
    if (hook_on) hook->solved(pb->precision == RBFFD_PREC_MIXED ? hf.fallback_count : 0);
    CK(cudaEventRecord(h->ev[5], st));
    CK(cudaStreamSynchronize(st));
    if (hf.knn_err) return bail(fail(h, RBFFD_EINVAL, "fewer candidate nodes than the stencil size"));
    if (hf.first_bad != INT64_MAX) {
        if (stats) stats->first_bad_node = hf.first_bad;
        return bail(fail(h, RBFFD_ESINGULAR, "singular local system at node " + std::to_string(hf.first_bad)));
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->ms_upload = elapsed(h->ev[0], h->ev[1]);
        stats->ms_grid = elapsed(h->ev[1], h->ev[2]);
        stats->ms_knn = elapsed(h->ev[2], h->ev[3]);
        stats->ms_solve = elapsed(h->ev[3], h->ev[4]);
        stats->ms_fallback = elapsed(h->ev[4], h->ev[5]);
        stats->ms_total = elapsed(h->ev[0], h->ev[5]);
        stats->n_systems = nsys;
        stats->n_rows = rows;
        stats->n_fallback = pb->precision == RBFFD_PREC_MIXED ? hf.fallback_count : 0;
        stats->first_bad_node = -1;
        for (int i = 0; i < 8; i++) stats->refine_hist[i] = (int64_t)hf.hist[i];
        stats->nnz = nnz;
        // kernels launched: grid (bbox 2, fill 1, scan 3, scatter/narrow/cell sort 3), row
        // grouping, stencil offsets, kNN, row pointers, solve (+ FP64 fallback)
        int64_t nk = 9;
        nk += collocated ? 1 : 12;
        if (!uniform) nk += (dn ? 1 : 0) + 3;
        nk += 1;
        nk += uniform ? 1 : 4;
        nk += n_bin_launches + n_solve_launches;
        if (pb->precision == RBFFD_PREC_MIXED && hf.fallback_count > 0) nk += 1;
        stats->kernel_launches = nk;
    }
    os->N = N;
    os->M = M;
    os->rows = rows;
    os->row_begin = rb;
    os->nnz = nnz;
    os->nops = nops;
    memcpy(os->ops, ops, sizeof(int) * nops);
    os->collocated = collocated;
    os->uniform = uniform;
    os->n = pb->n;
    os->X = dX;
    os->nbr = nbr;
    os->nbr_ptr = nbr_ptr;
    os->nn = nn;
    os->row_ptr = row_ptr;
    os->col = col;
    os->val = val;
    keep.release_to(os->owned);
    *out = os;
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_opset_create(rbffd_handle *h, const rbffd_problem *pb, rbffd_opset **out,
                                    rbffd_stats *stats)
{
    return opset_build(h, pb, 0, out, stats);
}

RBFFD_EXPORT void rbffd_opset_destroy(rbffd_handle *h, rbffd_opset *s)
{
    if (!s) return;
    if (h) {
        cudaSetDevice(h->device);
        for (void *p : s->owned) cudaFreeAsync(p, h->stream);
        cudaStreamSynchronize(h->stream);
    } else {
        for (void *p : s->owned) cudaFree(p);
    }
    delete s;
}

RBFFD_EXPORT int rbffd_opset_shape(const rbffd_opset *s, int64_t *rows, int64_t *cols, int64_t *nnz, int *nops)
{
    if (!s) return RBFFD_EINVAL;
    if (rows) *rows = s->rows;
    if (cols) *cols = s->N;
    if (nnz) *nnz = s->nnz;
    if (nops) *nops = s->nops;
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_opset_device_csr(const rbffd_opset *s, int op, const int64_t **row_ptr,
                                        const int32_t **col, const double **val)
{
    if (!s || op < 0 || op >= s->nops) return RBFFD_EINVAL;
    if (row_ptr) *row_ptr = s->row_ptr;
    if (col) *col = s->col;
    if (val) *val = s->val + (size_t)op * s->nnz;
    return RBFFD_OK;
}

static int ensure_csc(rbffd_handle *h, rbffd_opset *s)
{
    if (s->csc_perm) return RBFFD_OK;
    cudaStream_t st = h->stream;
    Arena keep(st), tmp(st);
    int64_t N = s->N;
    int64_t *count, *colstart, *fill, *rowval, *perm;
    double *buf;
    size_t tb = scan_tmp_bytes(N);
    void *scratch;
    CK(tmp.zeros(&count, N + 1));
    CK(keep.get(&colstart, N + 1));
    CK(tmp.zeros(&fill, N));
    CK(keep.get(&rowval, s->nnz));
    CK(keep.get(&perm, s->nnz));
    CK(keep.get(&buf, s->nnz));
    CK(tmp.get((char **)&scratch, tb));
    CK(launch_csc_count(s->nnz, s->col, count, st));
    CK(scan_exclusive_i64(count, colstart, N, scratch, tb, st));
    CK(launch_csc_scatter(s->rows, s->row_ptr, s->col, s->row_begin, colstart, fill, rowval, perm, st));
    CK(launch_csc_sort_segments(N, colstart, rowval, perm, s->row_begin + s->rows, st));
    // Julia is 1-based
    CK(launch_add_i64(N + 1, colstart, 1, st));
    CK(launch_add_i64(s->nnz, rowval, 1, st));
    CK(cudaStreamSynchronize(st));
    s->csc_colptr = colstart;
    s->csc_rowval = rowval;
    s->csc_perm = perm;
    s->csc_tmp = buf;
    keep.release_to(s->owned);
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_opset_export_csc(rbffd_handle *h, rbffd_opset *s, int op, rbffd_csc *out)
{
    if (!h) return RBFFD_EINVAL;
    if (!s || !out || op < 0 || op >= s->nops) return fail(h, RBFFD_EINVAL, "bad export arguments");
    cudaSetDevice(h->device);
    int rc = ensure_csc(h, s);
    if (rc) return rc;
    cudaStream_t st = h->stream;
    CK(launch_gather_f64(s->nnz, s->csc_perm, s->val + (size_t)op * s->nnz, s->csc_tmp, st));
    if (out->colptr)
        CK(cudaMemcpyAsync(out->colptr, s->csc_colptr, (s->N + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    if (out->rowval)
        CK(cudaMemcpyAsync(out->rowval, s->csc_rowval, s->nnz * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    if (out->nzval)
        CK(cudaMemcpyAsync(out->nzval, s->csc_tmp, s->nnz * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_opset_export_csr(rbffd_handle *h, rbffd_opset *s, int op, int64_t *row_ptr,
                                        int32_t *col, double *val)
{
    if (!h) return RBFFD_EINVAL;
    if (!s || op < 0 || op >= s->nops) return fail(h, RBFFD_EINVAL, "bad export arguments");
    cudaSetDevice(h->device);
    cudaStream_t st = h->stream;
    if (row_ptr) CK(cudaMemcpyAsync(row_ptr, s->row_ptr, (s->rows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    if (col) CK(cudaMemcpyAsync(col, s->col, s->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (val)
        CK(cudaMemcpyAsync(val, s->val + (size_t)op * s->nnz, s->nnz * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_opset_export_stencils(rbffd_handle *h, rbffd_opset *s, int32_t *nbr, int32_t *nn)
{
    if (!h) return RBFFD_EINVAL;
    if (!s) return fail(h, RBFFD_EINVAL, "null set");
    cudaSetDevice(h->device);
    cudaStream_t st = h->stream;
    if (nbr) {
        if (!s->uniform) return fail(h, RBFFD_EINVAL, "stencil export needs a uniform stencil size");
        CK(cudaMemcpyAsync(nbr, s->nbr, (size_t)s->N * s->n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    }
    if (nn) CK(cudaMemcpyAsync(nn, s->nn, s->rows * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_spmv(rbffd_handle *h, rbffd_opset *s, int op, const double *x, double *y)
{
    if (!h) return RBFFD_EINVAL;
    if (!s || op < 0 || op >= s->nops || !x || !y) return fail(h, RBFFD_EINVAL, "bad spmv arguments");
    if (s->uniform) {
        const int64_t padded = sell_padded(s->rows, s->n);
        if (!s->sell_val) {
            int32_t *sc;
            double *sv;
            CK(cudaMallocAsync((void **)&sc, (size_t)padded * sizeof(int32_t), h->stream));
            s->owned.push_back(sc);
            CK(cudaMallocAsync((void **)&sv, (size_t)padded * s->nops * sizeof(double), h->stream));
            s->owned.push_back(sv);
            CK(launch_csr_to_sell(s->rows, s->n, s->col, s->val, s->nops, s->nnz, sc, sv, h->stream));
            s->sell_col = sc;
            s->sell_val = sv;
        }
        CK(launch_spmv_sell(s->rows, s->n, s->sell_col, s->sell_val + (size_t)op * padded, x, y, h->num_sms,
                            h->stream));
        return RBFFD_OK;
    }
    CK(launch_spmv_f64(s->rows, s->row_ptr, s->col, s->val + (size_t)op * s->nnz, x, y, h->num_sms, h->stream));
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_spmm(rbffd_handle *h, rbffd_opset *s, int op, const void *x, void *y, int nfields,
                            int dtype)
{
    if (!h) return RBFFD_EINVAL;
    if (!s || op < 0 || op >= s->nops || !x || !y || nfields <= 0 || (dtype != 0 && dtype != 1))
        return fail(h, RBFFD_EINVAL, "bad spmm arguments");
    const void *v = s->val + (size_t)op * s->nnz;
    if (dtype == 1) {
        if (!s->val32) {
            float *v32;
            CK(cudaMallocAsync((void **)&v32, (size_t)s->nnz * s->nops * sizeof(float), h->stream));
            s->owned.push_back(v32);
            CK(launch_f64_to_f32((int64_t)s->nnz * s->nops, s->val, v32, h->stream));
            s->val32 = v32;
        }
        v = s->val32 + (size_t)op * s->nnz;
    }
    CK(launch_spmm(s->rows, s->row_ptr, s->col, v, x, y, nfields, dtype, h->stream));
    return RBFFD_OK;
}

// ---------------------------------------------------------------------------
// RK4 time stepping on device-resident operators.
// ---------------------------------------------------------------------------
struct rbffd_ghost {
    int64_t N = 0, nb = 0;
    const int64_t *row_ptr = nullptr;  // the operator's CSR (owned by its set)
    const int32_t *col = nullptr;
    const double *val = nullptr;
    int32_t *bnodes = nullptr, *gnodes = nullptr, *gidx = nullptr;
    double *M = nullptr;  // [I | inv(A[B, G])] after the reduction, nb x 2nb
    double *y = nullptr;  // nb x ycap scratch
    int ycap = 0;
    std::vector<void *> owned;
};

struct rbffd_rk4 {
    int64_t rows = 0, nnz = 0;
    int F = 0, dtype = 0;
    int64_t *row_ptr = nullptr;
    int32_t *col = nullptr;
    double *val64 = nullptr;
    float *val32 = nullptr;
    uint8_t *fixed = nullptr;
    int32_t *order = nullptr;  // rows in Morton (Z-curve) order of their nodes
    std::vector<rbffd_ghost *> closures;  // applied to every stage input, in order
    void *unext = nullptr, *wA = nullptr, *wB = nullptr, *acc = nullptr;
    TileOp tiles;  // FP32 tiled stage layout (rk4_tiled.cu), when `tiled`
    bool tiled = false;
    cudaGraphExec_t graph2 = nullptr;  // two steps u -> unext -> u
    const void *graph_u = nullptr;
    double graph_dt = 0.0;
    std::vector<void *> owned;
};

namespace {
// Enqueue one RK4 step u -> out on stream st.
cudaError_t rk4_closures(rbffd_rk4 *rk, void *w, cudaStream_t st)
{
    for (rbffd_ghost *g : rk->closures) {
        cudaError_t e = ghost_apply(g->nb, g->bnodes, g->gnodes, g->row_ptr, g->col, g->val, g->gidx, g->M, w, rk->F,
                                    rk->dtype, g->y, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// One Horner stage out = u + c L v (held rows: out = u), on the tiled FP32 kernel when the
// stepper has the tile layout and the buffers are 16-byte aligned.
cudaError_t rk4_horner_stage(rbffd_handle *h, rbffd_rk4 *rk, const void *v, const void *u, void *out, double c,
                             cudaStream_t st)
{
    const bool aligned = ((((uintptr_t)v) | ((uintptr_t)u) | ((uintptr_t)out)) & 15u) == 0;
    if (rk->tiled && aligned)
        return launch_tile_stage(rk->tiles, (const float *)v, (const float *)u, (float *)out, rk->F, c, h->num_sms,
                                 st);
    const void *val = rk->dtype == 0 ? (const void *)rk->val64 : (const void *)rk->val32;
    return launch_rk4_stage(rk->rows, rk->order, rk->row_ptr, rk->col, val, v, u, rk->acc, out, rk->fixed, rk->F, c,
                            3, rk->dtype, h->num_sms, st);
}

// Enqueue one RK4 step u -> out on stream st.
//
// Without ghost closures the system du/dt = L u (rows held fixed have zero rows in L) is linear
// with a constant operator, and classic RK4's step is then exactly the degree-4 Taylor
// polynomial of exp(dt L):  u + dt L u + dt^2/2 L^2 u + dt^3/6 L^3 u + dt^4/24 L^4 u.  It is
// evaluated in Horner form,
//     w1 = u + dt/4 L u,  w2 = u + dt/3 L w1,  w3 = u + dt/2 L w2,  out = u + dt L w3,
// four operator applications as in the stage form, without the stage-sum accumulator (each
// stage reads v and u and writes one array).  With closures, the closures are applied to every
// stage input first (u itself for the first stage, as the reference's cons_sys overwrites u),
// which is not a constant linear map between stages, so the classic stage form is used.
cudaError_t rk4_enqueue_step(rbffd_handle *h, rbffd_rk4 *rk, void *u, void *out, double dt, cudaStream_t st)
{
    if (rk->closures.empty()) {
        const void *in[4] = {u, rk->wA, rk->wB, rk->wA};
        void *o[4] = {rk->wA, rk->wB, rk->wA, out};
        const double c[4] = {0.25 * dt, dt / 3.0, 0.5 * dt, dt};
        for (int i = 0; i < 4; i++) {
            cudaError_t e = rk4_horner_stage(h, rk, in[i], u, o[i], c[i], st);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    const void *val = rk->dtype == 0 ? (const void *)rk->val64 : (const void *)rk->val32;
    struct Stage {
        void *w, *o;
        double c;
        int mode;
    } stages[4] = {{u, rk->wA, 0.5 * dt, 0}, {rk->wA, rk->wB, 0.5 * dt, 1}, {rk->wB, rk->wA, dt, 1},
                   {rk->wA, out, dt / 6.0, 2}};
    for (const Stage &sg : stages) {
        cudaError_t e = rk4_closures(rk, sg.w, st);
        if (e != cudaSuccess) return e;
        e = launch_rk4_stage(rk->rows, rk->order, rk->row_ptr, rk->col, val, sg.w, u, rk->acc, sg.o, rk->fixed, rk->F,
                             sg.c, sg.mode, rk->dtype, h->num_sms, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}
}  // namespace

RBFFD_EXPORT int rbffd_rk4_create(rbffd_handle *h, rbffd_opset *const *sets, int nsets, const double *coef,
                                  const uint8_t *fixed_rows, int nfields, int dtype, rbffd_rk4 **out)
{
    if (!h) return RBFFD_EINVAL;
    if (!sets || nsets <= 0 || !coef || !out || nfields <= 0 || (dtype != 0 && dtype != 1))
        return fail(h, RBFFD_EINVAL, "bad rk4 arguments");
    *out = nullptr;
    cudaSetDevice(h->device);
    const rbffd_opset *s0 = sets[0];
    for (int i = 0; i < nsets; i++) {
        const rbffd_opset *s = sets[i];
        if (!s || !s->collocated || s->row_begin != 0 || s->rows != s->N || s->N != s0->N || s->nnz != s0->nnz)
            return fail(h, RBFFD_EINVAL, "rk4 needs collocated full operator sets of one node set");
    }
    cudaStream_t st = h->stream;
    Arena keep(st), tmp(st);
    int nq = 0;
    for (int i = 0; i < nsets; i++) nq += sets[i]->nops;
    std::vector<const double *> hv;
    for (int i = 0; i < nsets; i++)
        for (int q = 0; q < sets[i]->nops; q++) hv.push_back(sets[i]->val + (size_t)q * sets[i]->nnz);
    // every set must share the first set's stencils
    unsigned long long *diff;
    CK(tmp.zeros(&diff, 1));
    for (int i = 1; i < nsets; i++) CK(launch_count_diff(s0->nnz, s0->col, sets[i]->col, diff, st));
    unsigned long long hdiff = 0;
    CK(cudaMemcpyAsync(&hdiff, diff, sizeof(hdiff), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hdiff) return fail(h, RBFFD_EINVAL, "operator sets do not share one stencil pattern");
    rbffd_rk4 *rk = new rbffd_rk4();
    rk->rows = s0->rows;
    rk->nnz = s0->nnz;
    rk->F = nfields;
    rk->dtype = dtype;
    auto bail = [&](int code) {
        delete rk;
        return code;
    };
    const double **dvals;
    double *dcoef;
    cudaError_t e = cudaSuccess;
#define CKB(expr)                                                                                            \
    do {                                                                                                     \
        e = (expr);                                                                                          \
        if (e != cudaSuccess) return bail(fail(h, RBFFD_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e))); \
    } while (0)
    CKB(tmp.get(&dvals, nq));
    CKB(tmp.get(&dcoef, nq));
    CKB(cudaMemcpyAsync(dvals, hv.data(), sizeof(double *) * nq, cudaMemcpyHostToDevice, st));
    CKB(cudaMemcpyAsync(dcoef, coef, sizeof(double) * nq, cudaMemcpyHostToDevice, st));
    CKB(keep.get(&rk->row_ptr, rk->rows + 1));
    CKB(keep.get(&rk->col, rk->nnz));
    CKB(keep.get(&rk->val64, rk->nnz));
    CKB(keep.get(&rk->val32, rk->nnz));
    CKB(cudaMemcpyAsync(rk->row_ptr, s0->row_ptr, sizeof(int64_t) * (rk->rows + 1), cudaMemcpyDeviceToDevice, st));
    CKB(cudaMemcpyAsync(rk->col, s0->col, sizeof(int32_t) * rk->nnz, cudaMemcpyDeviceToDevice, st));
    CKB(launch_combine_ops(rk->nnz, dvals, dcoef, nq, rk->val64, rk->val32, st));
    {
        // Z-curve order of the nodes (16 bits per axis over the bounding box): consecutive
        // rows of the order are spatial neighbours, so the stage kernel's gathers hit L1
        std::vector<double2> hx(rk->rows);
        CKB(cudaMemcpyAsync(hx.data(), s0->X, sizeof(double2) * rk->rows, cudaMemcpyDeviceToHost, st));
        CKB(cudaStreamSynchronize(st));
        double x0 = hx[0].x, x1 = hx[0].x, y0 = hx[0].y, y1 = hx[0].y;
        for (const double2 &q : hx) {
            x0 = std::min(x0, q.x);
            x1 = std::max(x1, q.x);
            y0 = std::min(y0, q.y);
            y1 = std::max(y1, q.y);
        }
        const double sxq = x1 > x0 ? 65535.0 / (x1 - x0) : 0.0, syq = y1 > y0 ? 65535.0 / (y1 - y0) : 0.0;
        auto spread = [](uint32_t v) {
            uint64_t z = v & 0xffffu;
            z = (z | (z << 8)) & 0x00ff00ffu;
            z = (z | (z << 4)) & 0x0f0f0f0fu;
            z = (z | (z << 2)) & 0x33333333u;
            z = (z | (z << 1)) & 0x55555555u;
            return z;
        };
        std::vector<std::pair<uint64_t, int32_t>> kv(rk->rows);
        for (int64_t i = 0; i < rk->rows; i++) {
            const uint32_t qx = (uint32_t)((hx[i].x - x0) * sxq), qy = (uint32_t)((hx[i].y - y0) * syq);
            kv[i] = {spread(qx) | (spread(qy) << 1), (int32_t)i};
        }
        std::sort(kv.begin(), kv.end());
        std::vector<int32_t> ho(rk->rows);
        for (int64_t i = 0; i < rk->rows; i++) ho[i] = kv[i].second;
        CKB(keep.get(&rk->order, rk->rows));
        CKB(cudaMemcpyAsync(rk->order, ho.data(), sizeof(int32_t) * rk->rows, cudaMemcpyHostToDevice, st));
        CKB(cudaStreamSynchronize(st));
    }
    if (fixed_rows) {
        CKB(keep.get(&rk->fixed, rk->rows));
        CKB(cudaMemcpyAsync(rk->fixed, fixed_rows, rk->rows, cudaMemcpyHostToDevice, st));
    }
    if (dtype == 1 && tile_stage_supported(nfields)) {
        // FP32 tile layout: tiles of 64 consecutive rows of the Z-curve order, each tile's
        // stencil-column union, groups of 8 rows with dense weights over their columns
        // (rk4_tiled.cu)
        int kmax = s0->uniform ? s0->n : 0;
        if (!s0->uniform) {
            std::vector<int64_t> hp(rk->rows + 1);
            CKB(cudaMemcpyAsync(hp.data(), rk->row_ptr, sizeof(int64_t) * (rk->rows + 1), cudaMemcpyDeviceToHost, st));
            CKB(cudaStreamSynchronize(st));
            for (int64_t i = 0; i < rk->rows; i++) kmax = std::max<int>(kmax, (int)(hp[i + 1] - hp[i]));
        }
        TileOp t;
        t.KP = kmax;
        t.F = nfields;
        t.ntile = (rk->rows + TileOp::T - 1) / TileOp::T;
        const int64_t ngroup = t.ntile * (TileOp::T / TileOp::G);
        int32_t *cnt, *gcnt;
        CKB(tmp.get(&cnt, t.ntile));
        CKB(tmp.get(&gcnt, ngroup));
        CKB(launch_tile_build(t, rk->rows, rk->order, rk->row_ptr, rk->col, rk->val32, rk->val64, rk->fixed, 0, cnt,
                              gcnt, h->num_sms, st));
        std::vector<int32_t> hc(t.ntile), hg(ngroup);
        CKB(cudaMemcpyAsync(hc.data(), cnt, sizeof(int32_t) * t.ntile, cudaMemcpyDeviceToHost, st));
        CKB(cudaMemcpyAsync(hg.data(), gcnt, sizeof(int32_t) * ngroup, cudaMemcpyDeviceToHost, st));
        CKB(cudaStreamSynchronize(st));
        std::vector<int32_t> hu(t.ntile + 1), hgp(ngroup + 1);
        int64_t tot = 0, gtot = 0;
        for (int64_t i = 0; i < t.ntile; i++) {
            hu[i] = (int32_t)tot;
            tot += hc[i];
            t.ucap = std::max(t.ucap, hc[i]);
            int64_t tile_cols = 0;
            for (int g = 0; g < TileOp::T / TileOp::G; g++) {
                const int64_t gi = i * (TileOp::T / TileOp::G) + g;
                hgp[gi] = (int32_t)gtot;
                gtot += hg[gi];
                tile_cols += hg[gi];
            }
            t.gcap = (int)std::max<int64_t>(t.gcap, tile_cols);
        }
        hu[t.ntile] = (int32_t)tot;
        hgp[ngroup] = (int32_t)gtot;
        int smem_max = 0;
        cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
        if (tot < INT32_MAX && 8 * gtot < INT32_MAX && tile_stage_smem(t, nfields) <= (size_t)smem_max) {
            int32_t *uptr, *gptr;
            CKB(keep.get(&uptr, t.ntile + 1));
            CKB(keep.get(&gptr, ngroup + 1));
            CKB(keep.get(&t.uni, tot));
            CKB(keep.get(&t.gslot, gtot));
            CKB(keep.get(&t.gw, 8 * gtot));
            CKB(keep.get(&t.rowinfo, (size_t)t.ntile * TileOp::T));
            CKB(cudaMemcpyAsync(uptr, hu.data(), sizeof(int32_t) * (t.ntile + 1), cudaMemcpyHostToDevice, st));
            CKB(cudaMemcpyAsync(gptr, hgp.data(), sizeof(int32_t) * (ngroup + 1), cudaMemcpyHostToDevice, st));
            t.uptr = uptr;
            t.gptr = gptr;
            CKB(launch_tile_build(t, rk->rows, rk->order, rk->row_ptr, rk->col, rk->val32, rk->val64, rk->fixed, 1,
                                  cnt, gcnt, h->num_sms, st));
            CKB(cudaStreamSynchronize(st));
            if (tile_stage_prepare(t, nfields) == cudaSuccess) {
                rk->tiles = t;
                rk->tiled = true;
            }
            cudaGetLastError();
        }
    }
    size_t fb = (size_t)rk->rows * nfields * (dtype == 0 ? 8 : 4);
    char *bufs;
    CKB(keep.get(&bufs, 4 * fb));
    rk->unext = bufs;
    rk->wA = bufs + fb;
    rk->wB = bufs + 2 * fb;
    rk->acc = bufs + 3 * fb;
    CKB(cudaStreamSynchronize(st));
#undef CKB
    keep.release_to(rk->owned);
    *out = rk;
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_rk4_apply(rbffd_handle *h, rbffd_rk4 *rk, const void *x, void *y)
{
    if (!h) return RBFFD_EINVAL;
    if (!rk || !x || !y) return fail(h, RBFFD_EINVAL, "bad rk4_apply arguments");
    const void *val = rk->dtype == 0 ? (const void *)rk->val64 : (const void *)rk->val32;
    CK(launch_spmm(rk->rows, rk->row_ptr, rk->col, val, x, y, rk->F, rk->dtype, h->stream));
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_rk4_run(rbffd_handle *h, rbffd_rk4 *rk, void *u, double dt, int64_t nsteps)
{
    if (!h) return RBFFD_EINVAL;
    if (!rk || !u || nsteps < 0) return fail(h, RBFFD_EINVAL, "bad rk4_run arguments");
    cudaSetDevice(h->device);
    cudaStream_t st = h->stream;
    if (nsteps >= 2 && (!rk->graph2 || rk->graph_u != u || rk->graph_dt != dt)) {
        if (rk->graph2) {
            cudaGraphExecDestroy(rk->graph2);
            rk->graph2 = nullptr;
        }
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaError_t e1 = rk4_enqueue_step(h, rk, u, rk->unext, dt, st);
        cudaError_t e2 = e1 == cudaSuccess ? rk4_enqueue_step(h, rk, rk->unext, u, dt, st) : e1;
        cudaError_t e3 = cudaStreamEndCapture(st, &g);
        CK(e2);
        CK(e3);
        cudaError_t e4 = cudaGraphInstantiate(&rk->graph2, g, 0);
        cudaGraphDestroy(g);
        CK(e4);
        rk->graph_u = u;
        rk->graph_dt = dt;
    }
    for (int64_t i = 0; i + 2 <= nsteps; i += 2) CK(cudaGraphLaunch(rk->graph2, st));
    if (nsteps % 2) {
        CK(rk4_enqueue_step(h, rk, u, rk->unext, dt, st));
        size_t fb = (size_t)rk->rows * rk->F * (rk->dtype == 0 ? 8 : 4);
        CK(cudaMemcpyAsync(u, rk->unext, fb, cudaMemcpyDeviceToDevice, st));
    }
    return RBFFD_OK;
}

RBFFD_EXPORT void rbffd_rk4_destroy(rbffd_handle *h, rbffd_rk4 *rk)
{
    if (!rk) return;
    if (rk->graph2) cudaGraphExecDestroy(rk->graph2);
    if (h) {
        cudaSetDevice(h->device);
        for (void *p : rk->owned) cudaFreeAsync(p, h->stream);
        cudaStreamSynchronize(h->stream);
    }
    delete rk;
}

// ---------------------------------------------------------------------------
// Ghost-node closure (examples/adv_diff_test.jl:108-141, 160-176).
// ---------------------------------------------------------------------------
RBFFD_EXPORT int rbffd_ghost_create(rbffd_handle *h, rbffd_opset *s, int op, const int32_t *bnodes,
                                    const int32_t *gnodes, int64_t nb, rbffd_ghost **out)
{
    if (!h) return RBFFD_EINVAL;
    if (!s || !bnodes || !gnodes || !out || nb <= 0 || op < 0 || op >= s->nops)
        return fail(h, RBFFD_EINVAL, "bad ghost arguments");
    *out = nullptr;
    if (!s->collocated || s->row_begin != 0 || s->rows != s->N)
        return fail(h, RBFFD_EINVAL, "the ghost closure needs a collocated full operator set");
    if (nb > 46340) return fail(h, RBFFD_EINVAL, "more than 46340 ghost nodes in one boundary");
    std::vector<char> seen(s->N, 0);
    for (int64_t i = 0; i < nb; i++) {
        if (bnodes[i] < 0 || bnodes[i] >= s->N || gnodes[i] < 0 || gnodes[i] >= s->N)
            return fail(h, RBFFD_EINVAL, "ghost or boundary node out of range");
        if (seen[gnodes[i]]++) return fail(h, RBFFD_EINVAL, "repeated ghost node");
    }
    cudaSetDevice(h->device);
    cudaStream_t st = h->stream;
    Arena keep(st), tmp(st);
    rbffd_ghost *g = new rbffd_ghost();
    auto bail = [&](int code) {
        delete g;
        return code;
    };
    g->N = s->N;
    g->nb = nb;
    g->row_ptr = s->row_ptr;
    g->col = s->col;
    g->val = s->val + (size_t)op * s->nnz;
    cudaError_t e = cudaSuccess;
#define CKG(expr)                                                                                            \
    do {                                                                                                     \
        e = (expr);                                                                                          \
        if (e != cudaSuccess) return bail(fail(h, RBFFD_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e))); \
    } while (0)
    double *fcol;
    int *flag;
    CKG(keep.get(&g->bnodes, nb));
    CKG(keep.get(&g->gnodes, nb));
    CKG(keep.get(&g->gidx, s->N));
    CKG(keep.get(&g->M, (size_t)nb * 2 * nb));
    CKG(tmp.get(&fcol, nb));
    CKG(tmp.zeros(&flag, 1));
    CKG(cudaMemcpyAsync(g->bnodes, bnodes, sizeof(int32_t) * nb, cudaMemcpyHostToDevice, st));
    CKG(cudaMemcpyAsync(g->gnodes, gnodes, sizeof(int32_t) * nb, cudaMemcpyHostToDevice, st));
    CKG(ghost_build(s->N, nb, g->bnodes, g->gnodes, g->row_ptr, g->col, g->val, g->gidx, g->M, fcol, flag, st));
    int hflag = 0;
    CKG(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKG(cudaStreamSynchronize(st));
#undef CKG
    if (hflag) return bail(fail(h, RBFFD_ESINGULAR, "singular ghost block A[B, G]"));
    keep.release_to(g->owned);
    *out = g;
    return RBFFD_OK;
}

static cudaError_t ghost_scratch(rbffd_handle *h, rbffd_ghost *g, int F)
{
    if (g->ycap >= F) return cudaSuccess;
    double *y;
    cudaError_t e = cudaMallocAsync((void **)&y, sizeof(double) * g->nb * F, h->stream);
    if (e != cudaSuccess) return e;
    g->owned.push_back(y);
    g->y = y;
    g->ycap = F;
    return cudaSuccess;
}

RBFFD_EXPORT int rbffd_ghost_apply(rbffd_handle *h, rbffd_ghost *g, void *u, int nfields, int dtype)
{
    if (!h) return RBFFD_EINVAL;
    if (!g || !u || nfields <= 0 || (dtype != 0 && dtype != 1)) return fail(h, RBFFD_EINVAL, "bad ghost_apply arguments");
    cudaSetDevice(h->device);
    CK(ghost_scratch(h, g, nfields));
    CK(ghost_apply(g->nb, g->bnodes, g->gnodes, g->row_ptr, g->col, g->val, g->gidx, g->M, u, nfields, dtype, g->y,
                   h->stream));
    return RBFFD_OK;
}

RBFFD_EXPORT void rbffd_ghost_destroy(rbffd_handle *h, rbffd_ghost *g)
{
    if (!g) return;
    if (h) {
        cudaSetDevice(h->device);
        for (void *p : g->owned) cudaFreeAsync(p, h->stream);
        cudaStreamSynchronize(h->stream);
    }
    delete g;
}

RBFFD_EXPORT int rbffd_rk4_set_closure(rbffd_handle *h, rbffd_rk4 *rk, rbffd_ghost *const *g, int ng)
{
    if (!h) return RBFFD_EINVAL;
    if (!rk || ng < 0 || (ng > 0 && !g)) return fail(h, RBFFD_EINVAL, "bad closure arguments");
    cudaSetDevice(h->device);
    std::vector<rbffd_ghost *> list;
    for (int i = 0; i < ng; i++) {
        if (!g[i] || g[i]->N != rk->rows) return fail(h, RBFFD_EINVAL, "closure of another node set");
        CK(ghost_scratch(h, g[i], rk->F));
        list.push_back(g[i]);
    }
    CK(cudaStreamSynchronize(h->stream));
    rk->closures = list;
    if (rk->graph2) {  // the captured steps no longer match
        cudaGraphExecDestroy(rk->graph2);
        rk->graph2 = nullptr;
    }
    return RBFFD_OK;
}

// ---------------------------------------------------------------------------
// Least squares by CGLS on an operator set (test/poisson_test.jl:75-121).
// ---------------------------------------------------------------------------
namespace {
cudaError_t cgls_iteration(rbffd_opset *s, const double *dD, const double *dDc, double *du, double *r, double *q,
                           double *p, double *sv, double *part, double *sc, cudaStream_t st)
{
    cudaError_t e;
    if ((e = launch_lsq_spmv(s->rows, s->row_ptr, s->col, dD, p, nullptr, q, part, st)) != cudaSuccess) return e;
    if ((e = launch_lsq_final(part, sc, 1, 1, st)) != cudaSuccess) return e;
    if ((e = launch_lsq_update_ur(s->N, s->rows, du, p, r, q, sc, st)) != cudaSuccess) return e;
    if ((e = launch_lsq_spmv_t(s->N, s->csc_colptr, s->csc_rowval, s->row_begin, dDc, r, sv, part, st)) !=
        cudaSuccess)
        return e;
    if ((e = launch_lsq_final(part, sc, 2, 0, st)) != cudaSuccess) return e;
    return launch_lsq_update_p(s->N, p, sv, sc, 0, st);
}
}  // namespace

RBFFD_EXPORT int rbffd_lsq_cgls(rbffd_handle *h, rbffd_opset *s, const double *coef, const double *f, double *u,
                                int64_t maxit, double tol, rbffd_lsq_info *info)
{
    if (!h) return RBFFD_EINVAL;
    if (!s || !coef || !f || !u || maxit < 0 || !(tol >= 0.0)) return fail(h, RBFFD_EINVAL, "bad lsq arguments");
    cudaSetDevice(h->device);
    int rc = ensure_csc(h, s);
    if (rc) return rc;
    cudaStream_t st = h->stream;
    Arena tmp(st);
    const int64_t rows = s->rows, cols = s->N, nnz = s->nnz;
    double *dcoef, *dD, *dDc, *df, *du, *r, *q, *p, *sv, *part, *sc;
    CK(tmp.get(&dcoef, (size_t)s->nops * rows));
    CK(tmp.get(&dD, nnz));
    CK(tmp.get(&dDc, nnz));
    CK(tmp.get(&df, rows));
    CK(tmp.get(&du, cols));
    CK(tmp.get(&r, rows));
    CK(tmp.get(&q, rows));
    CK(tmp.get(&p, cols));
    CK(tmp.get(&sv, cols));
    CK(tmp.get(&part, lsq_partials()));
    CK(tmp.zeros(&sc, 4));
    CK(cudaMemcpyAsync(dcoef, coef, sizeof(double) * s->nops * rows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(df, f, sizeof(double) * rows, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(du, u, sizeof(double) * cols, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(h->ev[0], st));
    CK(launch_combine_rows(rows, s->row_ptr, s->val, nnz, s->nops, dcoef, dD, st));
    CK(launch_gather_f64(nnz, s->csc_perm, dD, dDc, st));
    // r = f - D u, s = D^T r, p = s, gamma0 = ||s||^2
    CK(launch_lsq_spmv(rows, s->row_ptr, s->col, dD, du, df, r, part, st));
    CK(launch_lsq_spmv_t(cols, s->csc_colptr, s->csc_rowval, s->row_begin, dDc, r, sv, part, st));
    CK(launch_lsq_final(part, sc, 2, 0, st));
    CK(launch_lsq_update_p(cols, p, sv, sc, 1, st));
    CK(cudaMemcpyAsync(sc, sc + 2, sizeof(double), cudaMemcpyDeviceToDevice, st));
    double hsc[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(hsc, sc, sizeof(hsc), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const double g0 = hsc[2];
    double relres = g0 > 0.0 ? 1.0 : 0.0;
    int64_t it = 0;
    constexpr int CHUNK = 50;
    cudaGraphExec_t gx = nullptr;
    while (g0 > 0.0 && it < maxit && relres > tol) {
        const int64_t n = maxit - it < CHUNK ? maxit - it : CHUNK;
        if (n == CHUNK) {
            if (!gx) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                cudaError_t e1 = cudaSuccess;
                for (int k = 0; k < CHUNK && e1 == cudaSuccess; k++)
                    e1 = cgls_iteration(s, dD, dDc, du, r, q, p, sv, part, sc, st);
                cudaError_t e2 = cudaStreamEndCapture(st, &g);
                CK(e1);
                CK(e2);
                cudaError_t e3 = cudaGraphInstantiate(&gx, g, 0);
                cudaGraphDestroy(g);
                CK(e3);
            }
            CK(cudaGraphLaunch(gx, st));
        } else {
            for (int64_t k = 0; k < n; k++) CK(cgls_iteration(s, dD, dDc, du, r, q, p, sv, part, sc, st));
        }
        it += n;
        CK(cudaMemcpyAsync(hsc, sc, sizeof(hsc), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        relres = hsc[2] > 0.0 ? sqrt(hsc[2] / g0) : 0.0;
    }
    if (gx) cudaGraphExecDestroy(gx);
    CK(cudaEventRecord(h->ev[1], st));
    CK(cudaMemcpyAsync(u, du, sizeof(double) * cols, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (info) {
        info->iterations = it;
        info->relres = relres;
        info->ms = elapsed(h->ev[0], h->ev[1]);
    }
    return RBFFD_OK;
}

// ---------------------------------------------------------------------------
// Drop-in entry points.
// ---------------------------------------------------------------------------
static int export_all(rbffd_handle *h, rbffd_opset *s, rbffd_csc *out)
{
    for (int q = 0; q < s->nops; q++) {
        int rc = rbffd_opset_export_csc(h, s, q, &out[q]);
        if (rc) return rc;
    }
    return RBFFD_OK;
}

// The CSC pattern of a collocated uniform set depends on the stencils only, so the drop-in
// calls build it before the weight solves and download colptr/rowval into every output on the
// side stream while the solves run; the values follow once the solves finish.
//
// With nchunk > 0 the weight solves write their values straight into CSC order (csc_pos, the
// inverse of the CSC gather permutation) and run in nchunk launches of consecutive rows; as
// each completes, the CSC columns that no later row references are final and are downloaded
// on the side stream while the next chunks solve, instead of gathering and downloading all
// values after the solves.  Systems that the FP64 fallback re-solves afterwards make the
// export download every value again.
struct EarlyCsc : PatternHook {
    rbffd_csc *out = nullptr;
    int nops = 0;
    int64_t N = 0, nnz = 0;
    int64_t *colstart = nullptr, *rowval = nullptr, *perm = nullptr;
    bool active = false;
    int nchunk = 0;                 // requested; 0 after build() when chunking does not apply
    int32_t *inv = nullptr;         // CSR position -> CSC position
    int64_t hcp[RBFFD_MAX_CHUNKS] = {};  // CSC entries final after chunks 0..i
    cudaEvent_t chunk_ev[RBFFD_MAX_CHUNKS] = {};
    int64_t n_fallback = 0;

    int chunks() const override { return active ? nchunk : 0; }
    const int32_t *csc_pos() const override { return inv; }

    int build(rbffd_handle *h, int64_t N_, int n, const int64_t *row_ptr, const int32_t *nbr) override
    {
        // on the main stream, ahead of the weight solves (their persistent grid would hold
        // every SM until its end); only the download runs beside the solves
        cudaStream_t st = h->stream;
        N = N_;
        nnz = N_ * n;
        int64_t *count, *fill;
        void *scratch;
        const size_t tb = scan_tmp_bytes(N);
        CK(cudaMallocAsync((void **)&count, sizeof(int64_t) * (N + 1), st));
        CK(cudaMallocAsync((void **)&fill, sizeof(int64_t) * N, st));
        CK(cudaMallocAsync(&scratch, tb, st));
        CK(cudaMallocAsync((void **)&colstart, sizeof(int64_t) * (N + 1), st));
        CK(cudaMallocAsync((void **)&rowval, sizeof(int64_t) * nnz, st));
        CK(cudaMallocAsync((void **)&perm, sizeof(int64_t) * nnz, st));
        active = true;
        CK(cudaMemsetAsync(count, 0, sizeof(int64_t) * (N + 1), st));
        CK(cudaMemsetAsync(fill, 0, sizeof(int64_t) * N, st));
        if (nchunk > 0 && (nchunk > RBFFD_MAX_CHUNKS || nnz > INT32_MAX || N < (int64_t)nchunk * 1024)) nchunk = 0;
        if (nchunk > 0) CK(cudaMallocAsync((void **)&inv, sizeof(int32_t) * nnz, st));
        CK(launch_csc_count(nnz, nbr, count, st));
        CK(scan_exclusive_i64(count, colstart, N, scratch, tb, st));
        // rows 1-based as scattered (Julia's rowval); the sort writes the inverse permutation
        CK(launch_csc_scatter(N, row_ptr, nbr, 1, colstart, fill, rowval, perm, st));
        CK(launch_csc_sort_segments(N, colstart, rowval, perm, N + 1, st, inv));
        CK(launch_add_i64(N + 1, colstart, 1, st));  // Julia is 1-based
        CK(cudaFreeAsync(count, st));
        CK(cudaFreeAsync(fill, st));
        CK(cudaFreeAsync(scratch, st));
        CK(cudaEventRecord(h->side_ev[0], st));
        if (nchunk > 0) {
            int *cm;
            int64_t *cp;
            CK(cudaMallocAsync((void **)&cm, sizeof(int) * nchunk, st));
            CK(cudaMallocAsync((void **)&cp, sizeof(int64_t) * nchunk, st));
            CK(launch_chunk_bounds(N, n, nbr, nchunk, colstart, cm, cp, st));
            CK(cudaMemcpyAsync(hcp, cp, sizeof(int64_t) * nchunk, cudaMemcpyDeviceToHost, st));
            CK(cudaFreeAsync(cm, st));
            CK(cudaFreeAsync(cp, st));
            CK(cudaStreamSynchronize(st));
            for (int i = 0; i < nchunk; i++)
                if (!chunk_ev[i]) CK(cudaEventCreateWithFlags(&chunk_ev[i], cudaEventDisableTiming));
        }
        return RBFFD_OK;
    }

    // Columns final after chunk i: CSC entries [hcp[i-1], hcp[i]) of every operator.
    int chunk_done(rbffd_handle *h, int i, cudaStream_t cs, const double *val, int64_t nnz_) override
    {
        cudaStream_t ss = h->side;
        CK(cudaEventRecord(chunk_ev[i], cs));
        CK(cudaStreamWaitEvent(ss, chunk_ev[i], 0));
        const int64_t a = i ? hcp[i - 1] : 0, b = hcp[i];
        if (b <= a) return RBFFD_OK;
        for (int q = 0; q < nops; q++)
            if (out[q].nzval)
                CK(cudaMemcpyAsync(out[q].nzval + a, val + (size_t)q * nnz_ + a, sizeof(double) * (b - a),
                                   cudaMemcpyDeviceToHost, ss));
        return RBFFD_OK;
    }

    void solved(int64_t nfb) override { n_fallback = nfb; }

    int download(rbffd_handle *h) override
    {
        cudaStream_t ss = h->side;
        CK(cudaStreamWaitEvent(ss, h->side_ev[0], 0));
        for (int q = 0; q < nops; q++) {
            if (out[q].colptr)
                CK(cudaMemcpyAsync(out[q].colptr, colstart, sizeof(int64_t) * (N + 1), cudaMemcpyDeviceToHost, ss));
            if (out[q].rowval)
                CK(cudaMemcpyAsync(out[q].rowval, rowval, sizeof(int64_t) * nnz, cudaMemcpyDeviceToHost, ss));
        }
        CK(cudaEventRecord(h->side_ev[1], ss));
        return RBFFD_OK;
    }

    void release(rbffd_handle *h)
    {
        cudaStreamSynchronize(h->side);
        if (colstart) cudaFreeAsync(colstart, h->side);
        if (rowval) cudaFreeAsync(rowval, h->side);
        if (perm) cudaFreeAsync(perm, h->side);
        if (inv) cudaFreeAsync(inv, h->side);
        cudaStreamSynchronize(h->side);
        colstart = rowval = perm = nullptr;
        inv = nullptr;
        for (cudaEvent_t &e : chunk_ev)
            if (e) {
                cudaEventDestroy(e);
                e = nullptr;
            }
    }
};

// Build the operator set of a drop-in call and write its CSC matrices into `out`.
static int build_and_export(rbffd_handle *h, const rbffd_problem *pb, int unscaled, rbffd_csc *out,
                            rbffd_stats *stats)
{
    rbffd_opset *s = nullptr;
    EarlyCsc ec;
    ec.out = out;
    ec.nops = __builtin_popcount(pb->op_mask);
    ec.nchunk = RBFFD_EXPORT_CHUNKS;
    int rc = opset_build(h, pb, unscaled, &s, stats, &ec);
    if (rc) {
        ec.release(h);
        return rc;
    }
    if (ec.active && ec.nchunk > 0) {
        // the values were written in CSC order and downloaded chunk by chunk; systems re-solved
        // by the FP64 fallback after their chunk's download need the values again
        cudaError_t e = cudaSuccess;
        if (ec.n_fallback > 0) {
            e = cudaStreamWaitEvent(h->side, h->ev[5], 0);
            for (int q = 0; q < s->nops && e == cudaSuccess; q++)
                if (out[q].nzval)
                    e = cudaMemcpyAsync(out[q].nzval, s->val + (size_t)q * s->nnz, sizeof(double) * s->nnz,
                                        cudaMemcpyDeviceToHost, h->side);
        }
        cudaError_t e2 = cudaStreamSynchronize(h->side);
        if (e == cudaSuccess) e = e2;
        rc = e == cudaSuccess ? RBFFD_OK : fail(h, RBFFD_ECUDA, std::string("csc export: ") + cudaGetErrorString(e));
    } else if (ec.active) {
        // values in CSC order: each operator gathered into its own buffer on the main stream and
        // downloaded on the side stream as soon as its gather is done, so that the copies of
        // one operator overlap the gathers of the next
        cudaStream_t st = h->stream, ss = h->side;
        double *buf = nullptr;
        cudaError_t e = cudaStreamWaitEvent(st, h->side_ev[1], 0);
        if (e == cudaSuccess) e = cudaMallocAsync((void **)&buf, sizeof(double) * s->nnz * s->nops, st);
        for (int q = 0; q < s->nops && e == cudaSuccess; q++) {
            if (!out[q].nzval) continue;
            double *bq = buf + (size_t)q * s->nnz;
            e = launch_gather_f64(s->nnz, ec.perm, s->val + (size_t)q * s->nnz, bq, st);
            if (e == cudaSuccess) e = cudaEventRecord(h->side_ev[0], st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ss, h->side_ev[0], 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(out[q].nzval, bq, sizeof(double) * s->nnz, cudaMemcpyDeviceToHost, ss);
        }
        cudaError_t e2 = cudaStreamSynchronize(ss);
        if (e == cudaSuccess) e = e2;
        if (buf) cudaFreeAsync(buf, st);
        e2 = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = e2;
        rc = e == cudaSuccess ? RBFFD_OK : fail(h, RBFFD_ECUDA, std::string("csc export: ") + cudaGetErrorString(e));
    } else {
        rc = export_all(h, s, out);
    }
    ec.release(h);
    rbffd_opset_destroy(h, s);
    return rc;
}

RBFFD_EXPORT int rbffd_generate_operator(rbffd_handle *h, const double *X, int64_t N, const double *Y,
                                         int64_t M, int p, int n, int polydeg, const int32_t *node_class,
                                         uint32_t op_mask, int precision, rbffd_csc *out,
                                         rbffd_stats *stats)
{
    if (!h) return RBFFD_EINVAL;
    if (!out) return fail(h, RBFFD_EINVAL, "null output");
    rbffd_problem pb{};
    pb.X = X;
    pb.N = N;
    pb.Y = Y;
    pb.M = M;
    pb.p = p;
    pb.n = n;
    pb.polydeg = polydeg;
    pb.node_class = node_class;
    pb.op_mask = op_mask;
    pb.precision = precision;
    pb.memspace = RBFFD_MEM_HOST;
    return build_and_export(h, &pb, 0, out, stats);
}

RBFFD_EXPORT int rbffd_hyperviscosity_operator(rbffd_handle *h, int k_deriv, const double *X, int64_t N,
                                               const double *Y, int64_t M, int p, int n, int polydeg,
                                               const int32_t *node_class, int precision, rbffd_csc *out,
                                               rbffd_stats *stats)
{
    if (!h) return RBFFD_EINVAL;
    if (!out) return fail(h, RBFFD_EINVAL, "null output");
    rbffd_problem pb{};
    pb.X = X;
    pb.N = N;
    pb.Y = Y;
    pb.M = M;
    pb.p = p;
    pb.n = n;
    pb.polydeg = polydeg;
    pb.node_class = node_class;
    pb.op_mask = RBFFD_MASK_HYPERVISCOSITY;
    pb.k_deriv = k_deriv;
    pb.precision = precision;
    pb.memspace = RBFFD_MEM_HOST;
    return build_and_export(h, &pb, 0, out, stats);
}

RBFFD_EXPORT int rbffd_generate_operator_unscaled(rbffd_handle *h, const double *X, int64_t N, int p, int n,
                                                  int polydeg, uint32_t op_mask, int k_deriv, rbffd_csc *out,
                                                  rbffd_stats *stats)
{
    if (!h) return RBFFD_EINVAL;
    if (!out) return fail(h, RBFFD_EINVAL, "null output");
    rbffd_problem pb{};
    pb.X = X;
    pb.N = N;
    pb.p = p;
    pb.n = n;
    pb.polydeg = polydeg;
    pb.op_mask = op_mask;
    pb.k_deriv = k_deriv;
    pb.precision = RBFFD_PREC_FP64;
    pb.memspace = RBFFD_MEM_HOST;
    rbffd_opset *s = nullptr;
    int rc = opset_build(h, &pb, 1, &s, stats);
    if (rc) return rc;
    rc = export_all(h, s, out);
    rbffd_opset_destroy(h, s);
    return rc;
}

RBFFD_EXPORT int rbffd_process_mesh(rbffd_handle *h, const double *vertices, int64_t nv, const int64_t *tri,
                                    int64_t ntri, const int64_t *bc, int64_t nbc, double *Y, double *normals,
                                    double *tangents, double *offset)
{
    if (!h) return RBFFD_EINVAL;
    if (!vertices || nv <= 0 || !tri || ntri <= 0 || ntri > INT32_MAX || !bc || nbc <= 0 || !Y || !normals ||
        !tangents || !offset)
        return fail(h, RBFFD_EINVAL, "bad process_mesh arguments");
    cudaSetDevice(h->device);
    cudaStream_t st = h->stream;
    Arena tmp(st);
    double2 *dV, *dY, *dN, *dT;
    int64_t *dtri, *dbc;
    int *bad;
    CK(stage(h, tmp, vertices, (size_t)nv, RBFFD_MEM_HOST, &dV));
    CK(stage(h, tmp, tri, (size_t)(3 * ntri), RBFFD_MEM_HOST, &dtri));
    CK(stage(h, tmp, bc, (size_t)(2 * nbc), RBFFD_MEM_HOST, &dbc));
    CK(tmp.get(&dY, ntri + 2 * nbc));
    CK(tmp.get(&dN, nbc));
    CK(tmp.get(&dT, nbc));
    CK(tmp.zeros(&bad, 1));
    double2 *C = dY, *M = dY + ntri, *G = dY + ntri + nbc;
    mesh_centroids<<<nblk(ntri), 256, 0, st>>>(dV, nv, dtri, ntri, C, bad);
    mesh_lines<<<nblk(nbc), 256, 0, st>>>(dV, nv, dbc, nbc, M, dN, dT, bad);
    CK(cudaGetLastError());
    int hbad = 0;
    CK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hbad) return fail(h, RBFFD_EINVAL, "process_mesh: vertex id out of range");
    // the nearest centroid of every midpoint (processmesh.jl:120-127, 135-160), exact
    GridBuild gb;
    int rc = build_grid(h, tmp, C, nullptr, ntri, gb);
    if (rc) return rc;
    int32_t *nn;
    double *d2, *doff;
    int *err;
    CK(tmp.get(&nn, nbc));
    CK(tmp.get(&d2, nbc));
    CK(tmp.get(&doff, 1));
    CK(tmp.zeros(&err, 1));
    CK(launch_knn(gb.g, M, nullptr, nullptr, false, nbc, nullptr, 1, 1, nullptr, nn, d2, knn_r0(gb.rho, 1), err,
                  h->num_sms, st));
    mesh_ghosts<<<1, 256, 0, st>>>(C, M, nn, d2, nbc, dN, dT, G, doff);
    CK(cudaGetLastError());
    int herr = 0;
    CK(cudaMemcpyAsync(Y, dY, sizeof(double2) * (size_t)(ntri + 2 * nbc), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(normals, dN, sizeof(double2) * (size_t)nbc, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(tangents, dT, sizeof(double2) * (size_t)nbc, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(offset, doff, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (herr) return fail(h, RBFFD_EINVAL, "process_mesh: nearest-centroid search failed");
    return RBFFD_OK;
}

RBFFD_EXPORT int rbffd_calculateneighbors(rbffd_handle *h, const double *X, int64_t N, const double *Y,
                                          int64_t M, int n, const int32_t *node_class, int64_t *idxs_x,
                                          double *dists_x, int64_t *idxs_y_x, double *dists_y_x)
{
    if (!h) return RBFFD_EINVAL;
    if (!X || N <= 0 || n < 1 || n > N || n > RBFFD_MAX_K || !idxs_x || M < 0 || (M > 0 && (!Y || !idxs_y_x)))
        return fail(h, RBFFD_EINVAL, "bad calculateneighbors arguments");
    cudaSetDevice(h->device);
    cudaStream_t st = h->stream;
    Arena tmp(st);
    double2 *dX, *dY = nullptr;
    int32_t *dcls = nullptr;
    CK(stage(h, tmp, X, (size_t)N, RBFFD_MEM_HOST, &dX));
    if (M > 0) CK(stage(h, tmp, Y, (size_t)M, RBFFD_MEM_HOST, &dY));
    if (node_class) CK(stage(h, tmp, node_class, (size_t)N, RBFFD_MEM_HOST, &dcls));
    GridBuild gb;
    int rc = build_grid(h, tmp, dX, dcls, N, gb);
    if (rc) return rc;
    int *err;
    int32_t *idx;
    double *d2;
    int64_t *oidx;
    double *od;
    int64_t tot = N * (int64_t)n, big = std::max<int64_t>(tot, M);
    CK(tmp.zeros(&err, 1));
    CK(tmp.get(&idx, big));
    CK(tmp.get(&d2, big));
    CK(tmp.get(&oidx, big));
    CK(tmp.get(&od, big));
    CK(launch_knn(gb.g, dX, dcls, nullptr, true, N, nullptr, n, n, nullptr, idx, d2, knn_r0(gb.rho, n), err,
                  h->num_sms, st));
    knn_export<<<nblk(tot), 256, 0, st>>>(idx, d2, tot, oidx, od);
    CK(cudaMemcpyAsync(idxs_x, oidx, tot * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    if (dists_x) CK(cudaMemcpyAsync(dists_x, od, tot * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (M > 0) {
        CK(launch_knn(gb.g, dY, nullptr, nullptr, false, M, nullptr, 1, 1, nullptr, idx, d2, knn_r0(gb.rho, 1), err,
                      h->num_sms, st));
        knn_export<<<nblk(M), 256, 0, st>>>(idx, d2, M, oidx, od);
        CK(cudaMemcpyAsync(idxs_y_x, oidx, M * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        if (dists_y_x) CK(cudaMemcpyAsync(dists_y_x, od, M * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (herr) return fail(h, RBFFD_EINVAL, "fewer candidate nodes than the stencil size");
    return RBFFD_OK;
}
