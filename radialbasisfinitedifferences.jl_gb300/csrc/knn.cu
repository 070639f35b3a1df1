// Grid-bucket build and exact kNN stencil selection on the GPU.
//
// Replaces KDTree(X) + knn(tree, X, n, true) / knn(tree, Y, 1)
// (src/generate_operator.jl:43-47) and the boundary-masked searches of calculateneighbors
// (src/calculateneighbors.jl:16-42, :83-94).  Squared distances are rounded exactly as
// dx*dx + dy*dy with two roundings and no FMA, and candidates are ordered by (d^2, id), so
// the selected index sets are bit-identical to the CPU oracle's.  Only candidates that pass an
// FP32 screen against the current k-th distance get that exact FP64 distance, and the ring
// search stops on an FP32 lower bound of the distance to the unsearched cells; both are
// conservative, so the exact keys alone decide the result.
#include <float.h>
#include <limits.h>
#include <math_constants.h>

#include "rbffd_internal.cuh"

// ---------------------------------------------------------------------------
// Exclusive scan (int64), three phases: block sums, scan of block sums, add.
// ---------------------------------------------------------------------------
namespace {
constexpr int SCAN_BLOCK = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int64_t SCAN_TILE = (int64_t)SCAN_BLOCK * SCAN_ITEMS;

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v)
{
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(RBFFD_FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns exclusive prefix, total in *tot.
__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t *sh, int64_t *tot)
{
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int64_t inc = warp_incl_scan(v);
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < nw ? sh[lane] : 0;
        int64_t si = warp_incl_scan(s);
        if (lane < nw) sh[lane] = si - s;
        if (lane == nw - 1) sh[32] = si;
    }
    __syncthreads();
    int64_t r = inc - v + sh[w];
    *tot = sh[32];
    __syncthreads();
    return r;
}

__global__ void scan_block_sums(const int64_t *in, int64_t n, int64_t *bsum)
{
    __shared__ int64_t sh[33];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int64_t v = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t t = base + (int64_t)i * SCAN_BLOCK + threadIdx.x;
        if (t < n) v += in[t];
    }
    int64_t tot;
    block_excl_scan(v, sh, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void scan_block_offsets(int64_t *bsum, int64_t nb)
{
    __shared__ int64_t sh[33];
    int64_t carry = 0;
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        int64_t t = base + threadIdx.x;
        int64_t v = t < nb ? bsum[t] : 0;
        int64_t tot;
        int64_t ex = block_excl_scan(v, sh, &tot);
        if (t < nb) bsum[t] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void scan_apply(const int64_t *in, int64_t n, const int64_t *bsum, int64_t *out)
{
    __shared__ int64_t sh[33];
    __shared__ int64_t vals[SCAN_TILE];
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t t = base + (int64_t)i * SCAN_BLOCK + threadIdx.x;
        vals[i * SCAN_BLOCK + threadIdx.x] = t < n ? in[t] : 0;
    }
    __syncthreads();
    // each thread owns SCAN_ITEMS consecutive values
    int64_t loc[SCAN_ITEMS];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        loc[i] = vals[threadIdx.x * SCAN_ITEMS + i];
        s += loc[i];
    }
    int64_t tot;
    int64_t ex = block_excl_scan(s, sh, &tot) + bsum[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; i++) {
        vals[threadIdx.x * SCAN_ITEMS + i] = ex;
        ex += loc[i];
    }
    __syncthreads();
    for (int i = 0; i < SCAN_ITEMS; i++) {
        int64_t t = base + (int64_t)i * SCAN_BLOCK + threadIdx.x;
        if (t < n) out[t] = vals[i * SCAN_BLOCK + threadIdx.x];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = bsum[gridDim.x];
}
}  // namespace

size_t scan_tmp_bytes(int64_t n)
{
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb < 1) nb = 1;
    return (size_t)(nb + 1) * sizeof(int64_t);
}

cudaError_t scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, void *tmp,
                               size_t tmp_bytes, cudaStream_t st)
{
    if (tmp_bytes < scan_tmp_bytes(n)) return cudaErrorInvalidValue;
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb < 1) nb = 1;
    int64_t *bsum = (int64_t *)tmp;
    scan_block_sums<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(in, n, bsum);
    scan_block_offsets<<<1, 1024, 0, st>>>(bsum, nb);
    scan_apply<<<(unsigned)nb, SCAN_BLOCK, 0, st>>>(in, n, bsum, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Bounding box.
// ---------------------------------------------------------------------------
__global__ void bbox_partial(const double2 *X, int64_t N, double *partial, int *bad)
{
    double xmin = DBL_MAX, xmax = -DBL_MAX, ymin = DBL_MAX, ymax = -DBL_MAX;
    int nb = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        double2 p = X[i];
        if (!isfinite(p.x) || !isfinite(p.y)) {
            nb++;
            continue;
        }
        xmin = fmin(xmin, p.x);
        xmax = fmax(xmax, p.x);
        ymin = fmin(ymin, p.y);
        ymax = fmax(ymax, p.y);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        xmin = fmin(xmin, __shfl_xor_sync(RBFFD_FULL, xmin, o));
        xmax = fmax(xmax, __shfl_xor_sync(RBFFD_FULL, xmax, o));
        ymin = fmin(ymin, __shfl_xor_sync(RBFFD_FULL, ymin, o));
        ymax = fmax(ymax, __shfl_xor_sync(RBFFD_FULL, ymax, o));
        nb += __shfl_xor_sync(RBFFD_FULL, nb, o);
    }
    __shared__ double sh[4][32];
    __shared__ int shb[32];
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) {
        sh[0][w] = xmin;
        sh[1][w] = xmax;
        sh[2][w] = ymin;
        sh[3][w] = ymax;
        shb[w] = nb;
    }
    __syncthreads();
    if (w == 0) {
        xmin = lane < nw ? sh[0][lane] : DBL_MAX;
        xmax = lane < nw ? sh[1][lane] : -DBL_MAX;
        ymin = lane < nw ? sh[2][lane] : DBL_MAX;
        ymax = lane < nw ? sh[3][lane] : -DBL_MAX;
        nb = lane < nw ? shb[lane] : 0;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            xmin = fmin(xmin, __shfl_xor_sync(RBFFD_FULL, xmin, o));
            xmax = fmax(xmax, __shfl_xor_sync(RBFFD_FULL, xmax, o));
            ymin = fmin(ymin, __shfl_xor_sync(RBFFD_FULL, ymin, o));
            ymax = fmax(ymax, __shfl_xor_sync(RBFFD_FULL, ymax, o));
            nb += __shfl_xor_sync(RBFFD_FULL, nb, o);
        }
        if (lane == 0) {
            partial[4 * blockIdx.x + 0] = xmin;
            partial[4 * blockIdx.x + 1] = xmax;
            partial[4 * blockIdx.x + 2] = ymin;
            partial[4 * blockIdx.x + 3] = ymax;
            if (nb) atomicAdd(bad, nb);
        }
    }
}

__global__ void bbox_final(const double *partial, int nb, double *out)
{
    double xmin = DBL_MAX, xmax = -DBL_MAX, ymin = DBL_MAX, ymax = -DBL_MAX;
    for (int i = threadIdx.x; i < nb; i += 32) {
        xmin = fmin(xmin, partial[4 * i]);
        xmax = fmax(xmax, partial[4 * i + 1]);
        ymin = fmin(ymin, partial[4 * i + 2]);
        ymax = fmax(ymax, partial[4 * i + 3]);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        xmin = fmin(xmin, __shfl_xor_sync(RBFFD_FULL, xmin, o));
        xmax = fmax(xmax, __shfl_xor_sync(RBFFD_FULL, xmax, o));
        ymin = fmin(ymin, __shfl_xor_sync(RBFFD_FULL, ymin, o));
        ymax = fmax(ymax, __shfl_xor_sync(RBFFD_FULL, ymax, o));
    }
    if (threadIdx.x == 0) {
        out[0] = xmin;
        out[1] = xmax;
        out[2] = ymin;
        out[3] = ymax;
    }
}

cudaError_t launch_bbox(const double2 *X, int64_t N, double *partial, int nblocks, double *out,
                        int *out_bad, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(out_bad, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    bbox_partial<<<nblocks, 256, 0, st>>>(X, N, partial, out_bad);
    bbox_final<<<1, 32, 0, st>>>(partial, nblocks, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Grid fill (cell histogram) and scatter into cell order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cell_coord(double v, double v0, double cs, int nmax)
{
    int c = (int)floor((v - v0) / cs);
    return c < 0 ? 0 : (c >= nmax ? nmax - 1 : c);
}

__global__ void grid_fill_kernel(const double2 *X, int64_t N, double x0, double y0, double cs,
                                 int nx, int ny, unsigned long long *count, int32_t *cell_of)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        double2 p = X[i];
        int c = cell_coord(p.y, y0, cs, ny) * nx + cell_coord(p.x, x0, cs, nx);
        cell_of[i] = c;
        atomicAdd(&count[c], 1ull);
    }
}

cudaError_t launch_grid_fill(const double2 *X, const int32_t *cls, int64_t N, double x0,
                             double y0, double cs, int nx, int ny, int64_t *cell_count,
                             int32_t *cell_of, cudaStream_t st)
{
    (void)cls;
    int nb = (int)((N + 255) / 256);
    if (nb > 65535) nb = 65535;
    grid_fill_kernel<<<nb, 256, 0, st>>>(X, N, x0, y0, cs, nx, ny,
                                         (unsigned long long *)cell_count, cell_of);
    return cudaGetLastError();
}

__global__ void grid_scatter_kernel(const double2 *X, const int32_t *cls, int64_t N,
                                    const int32_t *cell_of, const int64_t *start, int32_t *fill,
                                    double2 *pts, int32_t *ids, int32_t *gcls)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        int c = cell_of[i];
        int64_t pos = start[c] + atomicAdd(&fill[c], 1);
        pts[pos] = X[i];
        ids[pos] = (int32_t)i;
        if (gcls) gcls[pos] = cls[i];
    }
}

// Order the points of each cell by id so that the grid (and thus every candidate sweep)
// is deterministic.  Cells hold a handful of points: insertion sort per cell.
__global__ void grid_sort_cells(const int32_t *start, int64_t ncell, double2 *pts, int32_t *ids,
                                int32_t *gcls)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
         c += (int64_t)gridDim.x * blockDim.x) {
        int a = start[c], b = start[c + 1];
        for (int i = a + 1; i < b; i++) {
            int32_t id = ids[i];
            double2 p = pts[i];
            int32_t cl = gcls ? gcls[i] : 0;
            int j = i - 1;
            while (j >= a && ids[j] > id) {
                ids[j + 1] = ids[j];
                pts[j + 1] = pts[j];
                if (gcls) gcls[j + 1] = gcls[j];
                j--;
            }
            ids[j + 1] = id;
            pts[j + 1] = p;
            if (gcls) gcls[j + 1] = cl;
        }
    }
}

__global__ void narrow_i64_to_i32(const int64_t *a, int32_t *b, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (int32_t)a[i];
}

cudaError_t launch_grid_scatter(const double2 *X, const int32_t *cls, int64_t N,
                                const int32_t *cell_of, const int64_t *cell_start64,
                                int32_t *cell_start32, int64_t ncell, int32_t *fill,
                                double2 *pts, int32_t *ids, int32_t *gcls, cudaStream_t st)
{
    int nb = (int)((N + 255) / 256);
    if (nb > 65535) nb = 65535;
    cudaError_t e = cudaMemsetAsync(fill, 0, sizeof(int32_t) * ncell, st);
    if (e != cudaSuccess) return e;
    grid_scatter_kernel<<<nb, 256, 0, st>>>(X, cls, N, cell_of, cell_start64, fill, pts, ids,
                                            gcls);
    int nc = (int)((ncell + 1 + 255) / 256);
    if (nc > 65535) nc = 65535;
    narrow_i64_to_i32<<<nc, 256, 0, st>>>(cell_start64, cell_start32, ncell + 1);
    grid_sort_cells<<<nc, 256, 0, st>>>(cell_start32, ncell, pts, ids, gcls);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// kNN: one warp per query.  The current k best candidates are kept sorted across
// the warp, striped (element t = s*32 + lane lives in slot s of lane `lane`).
// Candidates are swept ring by ring around the query's cell in chunks of 32; a
// candidate that beats the current k-th element is inserted with one ballot (its
// rank) and one shuffle-up of the list.  The sweep stops once the k-th squared
// distance is below the squared distance to the unsearched part of the grid.
// ---------------------------------------------------------------------------
namespace {

// Candidate keys: the IEEE bit pattern of a non-negative squared distance orders exactly
// like the value, so (d2, id) is compared with integer instructions only (FP64 compares
// run on the 1/64-rate FP64 pipe of GB300).
__device__ __forceinline__ bool key_less(unsigned long long da, int ia, unsigned long long db, int ib)
{
    return da < db || (da == db && ia < ib);
}

__device__ __forceinline__ bool class_allowed(int cq, int cc)
{
    if (cq == 0) return true;
    int b = cq > 0 ? cq : -cq;
    return cc >= 0 || cc == -b;
}

constexpr unsigned long long KEY_INF = 0x7ff0000000000000ull;  // bits of +inf

template <int KS>
struct TopK {
    unsigned long long d[KS];
    int id[KS];
    unsigned long long kd;  // current k-th key (warp uniform)
    int ki;
    int k;

    __device__ __forceinline__ void init(int kk)
    {
#pragma unroll
        for (int s = 0; s < KS; s++) {
            d[s] = KEY_INF;
            id[s] = INT_MAX;
        }
        kd = KEY_INF;
        ki = INT_MAX;
        k = kk;
    }

    __device__ __forceinline__ void refresh_kth()
    {
        int t = k - 1, ss = t >> 5, sl = t & 31;
        unsigned long long v = d[0];
        int vi = id[0];
#pragma unroll
        for (int s = 1; s < KS; s++)
            if (s == ss) {
                v = d[s];
                vi = id[s];
            }
        kd = __shfl_sync(RBFFD_FULL, v, sl);
        ki = __shfl_sync(RBFFD_FULL, vi, sl);
    }

    __device__ __forceinline__ void insert(unsigned long long cd, int ci, int lane)
    {
        int pos = 0;
#pragma unroll
        for (int s = 0; s < KS; s++) pos += __popc(__ballot_sync(RBFFD_FULL, key_less(d[s], id[s], cd, ci)));
#pragma unroll
        for (int s = KS - 1; s >= 0; s--) {
            unsigned long long ud = __shfl_up_sync(RBFFD_FULL, d[s], 1);
            int ui = __shfl_up_sync(RBFFD_FULL, id[s], 1);
            if (s > 0) {
                unsigned long long wd = __shfl_sync(RBFFD_FULL, d[s - 1], 31);
                int wi = __shfl_sync(RBFFD_FULL, id[s - 1], 31);
                if (lane == 0) {
                    ud = wd;
                    ui = wi;
                }
            }
            int t = s * 32 + lane;
            if (t > pos) {
                d[s] = ud;
                id[s] = ui;
            } else if (t == pos) {
                d[s] = cd;
                id[s] = ci;
            }
        }
        refresh_kth();
    }

    // Element p of the list (slot p / 32 of lane p % 32), read by every lane for its own p.
    __device__ __forceinline__ void fetch(int p, unsigned long long &od, int &oi) const
    {
        const int src = p & 31, ss = p >> 5;
        od = KEY_INF;
        oi = INT_MAX;
#pragma unroll
        for (int s = 0; s < KS; s++) {
            const unsigned long long v = __shfl_sync(RBFFD_FULL, d[s], src);
            const int vi = __shfl_sync(RBFFD_FULL, id[s], src);
            if (s == ss) {
                od = v;
                oi = vi;
            }
        }
    }

    // Merge 32 candidates sorted ascending across the lanes (lane j holds the j-th; unused
    // lanes hold (KEY_INF, INT_MAX)) into the list, keeping its first 32 KS entries.  New
    // element j goes to rank j + #{old < it}, old element p to p + #{new <= it}: a permutation
    // (ties between equal padding keys aside, which are interchangeable).  The ranks are found
    // by binary lifting with shuffles and the merged list is assembled in the warp's shared
    // buffer (md, mi: 32 KS entries).
    __device__ __forceinline__ void merge(unsigned long long cd, int ci, int lane, unsigned long long *md, int *mi)
    {
        constexpr int NL = 32 * KS;
        int po = 0;
#pragma unroll
        for (int step = NL / 2; step >= 1; step >>= 1) {
            unsigned long long od;
            int oi;
            fetch(po + step - 1, od, oi);
            if (key_less(od, oi, cd, ci)) po += step;
        }
        {
            unsigned long long od;
            int oi;
            fetch(po, od, oi);
            if (key_less(od, oi, cd, ci)) po++;
        }
        const int rn = lane + po;
        int ro[KS];
#pragma unroll
        for (int s = 0; s < KS; s++) {
            int pn = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const unsigned long long nd = __shfl_sync(RBFFD_FULL, cd, pn + step - 1);
                const int ni = __shfl_sync(RBFFD_FULL, ci, pn + step - 1);
                if (!key_less(d[s], id[s], nd, ni)) pn += step;
            }
            const unsigned long long nd = __shfl_sync(RBFFD_FULL, cd, pn);
            const int ni = __shfl_sync(RBFFD_FULL, ci, pn);
            if (!key_less(d[s], id[s], nd, ni)) pn++;
            ro[s] = s * 32 + lane + pn;
        }
        if (rn < NL) {
            md[rn] = cd;
            mi[rn] = ci;
        }
#pragma unroll
        for (int s = 0; s < KS; s++)
            if (ro[s] < NL) {
                md[ro[s]] = d[s];
                mi[ro[s]] = id[s];
            }
        __syncwarp();
#pragma unroll
        for (int s = 0; s < KS; s++) {
            d[s] = md[s * 32 + lane];
            id[s] = mi[s * 32 + lane];
        }
        __syncwarp();
        refresh_kth();
    }
};

// Ascending bitonic sort of one (key, id) per lane across the warp.
__device__ __forceinline__ void warp_sort32(unsigned long long &cd, int &ci, int lane)
{
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const unsigned long long od = __shfl_xor_sync(RBFFD_FULL, cd, j);
            const int oi = __shfl_xor_sync(RBFFD_FULL, ci, j);
            const bool want_min = ((lane & j) == 0) == ((lane & k) == 0);
            const bool take = want_min ? key_less(od, oi, cd, ci) : key_less(cd, ci, od, oi);
            if (take) {
                cd = od;
                ci = oi;
            }
        }
    }
}

// Candidates of one batch that enter the list; at least this many are merged in bulk (sort +
// merge, ~250 instructions) rather than inserted one at a time (~25 each).
// Survivor batches of at least this many keys are merged in bulk (sort + ranks), smaller ones
// inserted one by one.  1M nodes, k = 30: 2.50 / 2.50 / 2.47 ms at 6 / 10 / 14.
#ifndef RBFFD_KNN_MERGE_MIN
#define RBFFD_KNN_MERGE_MIN 10
#endif
constexpr int MERGE_MIN = RBFFD_KNN_MERGE_MIN;

// Exact FP64 keys of the queued candidates queue[0..cnt) (one per lane) and their insertion.
template <int KS>
__device__ __forceinline__ void take_queued(const GridDev &g, TopK<KS> &tk, const int64_t *queue, int cnt, double qx,
                                            double qy, int lane, unsigned long long *md, int *mi)
{
    unsigned long long cd = KEY_INF;
    int ci = INT_MAX;
    if (lane < cnt) {
        const int64_t t = queue[lane];
        const double2 p = g.pts[t];
        const double dx = __dsub_rn(qx, p.x), dy = __dsub_rn(qy, p.y);
        cd = (unsigned long long)__double_as_longlong(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        ci = g.ids[t];
    }
    const bool enters = key_less(cd, ci, tk.kd, tk.ki);
    unsigned m = __ballot_sync(RBFFD_FULL, enters);
    if (__popc(m) >= MERGE_MIN) {
        if (!enters) {
            cd = KEY_INF;
            ci = INT_MAX;
        }
        warp_sort32(cd, ci, lane);
        tk.merge(cd, ci, lane, md, mi);
        return;
    }
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const unsigned long long sd = __shfl_sync(RBFFD_FULL, cd, src);
        const int si = __shfl_sync(RBFFD_FULL, ci, src);
        if (key_less(sd, si, tk.kd, tk.ki)) tk.insert(sd, si, lane);
    }
}

// Sweep the candidate segments [sa, sa+sl) held by lanes 0..nseg-1.  Candidates are screened
// in FP32 against the current k-th distance (a bound that covers the conversions and FP32
// rounding, so no candidate that can enter is dropped); the survivors are queued and their
// exact FP64 distances computed 32 at a time, so the FP64 work (GB300: 1/64 rate) scales with
// the survivors instead of all candidates.  The exact keys, and so the result, are unchanged.
template <int KS>
__device__ __forceinline__ void sweep_segments(const GridDev &g, TopK<KS> &tk, int nseg, int64_t sa, int sl,
                                               double qx, double qy, int cq, int64_t *queue, int lane,
                                               unsigned long long *md, int *mi)
{
    // exclusive offsets of the segments
    int inc = sl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(RBFFD_FULL, inc, o);
        if (lane >= o) inc += t;
    }
    int off = inc - sl;
    int total = __shfl_sync(RBFFD_FULL, inc, 31);
    const float qx32 = f64_to_f32(qx), qy32 = f64_to_f32(qy);
    int qn = 0;  // queued survivors (warp uniform), < 32 between batches
    for (int base = 0; base < total; base += 32) {
        int pos = base + lane;
        // find my segment: the last segment whose offset <= pos
        int seg = 0;
        for (int s = 1; s < nseg; s++) {
            int os = __shfl_sync(RBFFD_FULL, off, s);
            if (os <= pos) seg = s;
        }
        int64_t a = __shfl_sync(RBFFD_FULL, sa, seg);
        int os = __shfl_sync(RBFFD_FULL, off, seg);
        // float upper bound of the current k-th squared distance (inf while the list fills)
        const float kd32 = f64_to_f32(__longlong_as_double((long long)tk.kd)) * (1.0f + 0x1p-20f);
        bool pass = false;
        int64_t t = 0;
        if (pos < total) {
            t = a + (pos - os);
            int cc = g.cls ? g.cls[t] : 0;
            if (class_allowed(cq, cc)) {
                const double2 p = g.pts[t];
                // the truncating conversions err by < 2^-23 relative, the FP32 difference and
                // square sum by < 2^-24 each: err bounds |d32 - d2|
                const float px = f64_to_f32(p.x), py = f64_to_f32(p.y);
                const float dx = qx32 - px, dy = qy32 - py;
                const float ex = 0x1p-22f * (fabsf(qx32) + fabsf(px)), ey = 0x1p-22f * (fabsf(qy32) + fabsf(py));
                const float d32 = fmaf(dx, dx, dy * dy);
                const float err = ex * (2.0f * fabsf(dx) + ex) + ey * (2.0f * fabsf(dy) + ey) + 0x1p-21f * d32;
                pass = !(d32 - err > kd32);  // NaN (coordinates beyond the float range) keeps it
            }
        }
        const unsigned m = __ballot_sync(RBFFD_FULL, pass);
        if (pass) queue[qn + __popc(m & ((1u << lane) - 1u))] = t;
        qn += __popc(m);
        __syncwarp();
        if (qn >= 32) {
            take_queued<KS>(g, tk, queue, 32, qx, qy, lane, md, mi);
            const int rest = qn - 32;
            const int64_t mv = lane < rest ? queue[32 + lane] : 0;
            __syncwarp();
            if (lane < rest) queue[lane] = mv;
            qn = rest;
            __syncwarp();
        }
    }
    if (qn > 0) take_queued<KS>(g, tk, queue, qn, qx, qy, lane, md, mi);
    __syncwarp();
}

// Resident 256-thread CTAs per SM requested for k <= 32 (64 registers); 5 (51 registers):
// 2.62 against 2.50 ms.
#ifndef RBFFD_KNN_MINB
#define RBFFD_KNN_MINB 4
#endif
template <int KS>
__global__ void __launch_bounds__(256, (KS == 1 ? RBFFD_KNN_MINB : 2)) knn_kernel(GridDev g, const double2 *__restrict__ Q,
                                                  const int32_t *__restrict__ qcls,
                                                  const int32_t *__restrict__ q_node,
                                                  bool node_query, int64_t nq,
                                                  const int32_t *__restrict__ kq, int kuni,
                                                  const int64_t *__restrict__ out_ptr,
                                                  int32_t *__restrict__ out_idx,
                                                  double *__restrict__ out_d2, int r0,
                                                  int *err_flag)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    __shared__ int64_t queue_all[8][64];  // survivors of the FP32 screen, per warp
    __shared__ unsigned long long merge_d[8][32 * KS];  // bulk-merge buffers, per warp
    __shared__ int merge_i[8][32 * KS];
    int64_t *queue = queue_all[threadIdx.x >> 5];
    unsigned long long *md = merge_d[threadIdx.x >> 5];
    int *mi = merge_i[threadIdx.x >> 5];
    for (int64_t q = warp; q < nq; q += nwarps) {
        // node queries: query q is node q_node[q] (or q) of the set; its coordinates, class,
        // stencil size and output row are taken by node id.  Point queries: Q[q], class 0.
        int64_t node = node_query ? (q_node ? (int64_t)q_node[q] : q) : q;
        double2 qp = Q[node];
        int cq = (node_query && qcls) ? qcls[node] : 0;
        int k = (node_query && kq) ? kq[node] : kuni;
        TopK<KS> tk;
        tk.init(k);
        // The query's cell only seeds the search, so it is taken in FP32; the stopping test
        // below uses the offset of q from the same cell's corner, fx = (qx - x0) - cx cs, formed
        // once per query in FP64 (four FP64 instructions instead of a division per axis).
        const double dqx = qp.x - g.x0, dqy = qp.y - g.y0;
        const float cs32 = f64_to_f32(g.cs), ics32 = __frcp_rn(cs32);
        int cx = __float2int_rd(f64_to_f32(dqx) * ics32), cy = __float2int_rd(f64_to_f32(dqy) * ics32);
        cx = cx < 0 ? 0 : (cx >= g.nx ? g.nx - 1 : cx);
        cy = cy < 0 ? 0 : (cy >= g.ny ? g.ny - 1 : cy);
        const float fx = f64_to_f32(fma(-f32_to_f64((float)cx), g.cs, dqx));
        const float fy = f64_to_f32(fma(-f32_to_f64((float)cy), g.cs, dqy));
        bool done = false;
        for (int R = r0; !done; R++) {
            // segments of this sweep: the full square at R = r0, then the ring at radius R
            if (R == r0) {
                int ylo = max(cy - R, 0), yhi = min(cy + R, g.ny - 1);
                int xlo = max(cx - R, 0), xhi = min(cx + R, g.nx - 1);
                for (int y0r = ylo; y0r <= yhi; y0r += 32) {
                    int nseg = min(32, yhi - y0r + 1);
                    int64_t sa = 0;
                    int sl = 0;
                    if (lane < nseg) {
                        int row = y0r + lane;
                        int c0 = row * g.nx + xlo, c1 = row * g.nx + xhi + 1;
                        sa = g.start[c0];
                        sl = g.start[c1] - g.start[c0];
                    }
                    sweep_segments<KS>(g, tk, nseg, sa, sl, qp.x, qp.y, cq, queue, lane, md, mi);
                }
            } else {
                // ring: bottom row, top row (full width), then left/right cells of the middle rows.
                // A segment whose FP32 lower bound of the distance to q is beyond the current
                // k-th distance (an FP32 upper bound of it) is skipped: none of its nodes can
                // enter.  The bound carries the same margins as the stopping test below.
                int nmid = 2 * R - 1;
                int nseg_all = 2 + 2 * nmid;
                const float kd32 = f64_to_f32(__longlong_as_double((long long)tk.kd)) * (1.0f + 0x1p-20f);
                const float mg = 0x1p-20f * (float)(R + 1) * cs32;
                for (int s0 = 0; s0 < nseg_all; s0 += 32) {
                    int nseg = min(32, nseg_all - s0);
                    int64_t sa = 0;
                    int sl = 0;
                    int s = s0 + lane;
                    if (lane < nseg) {
                        int row, xa, xb;
                        if (s < 2) {
                            row = s == 0 ? cy - R : cy + R;
                            xa = max(cx - R, 0);
                            xb = min(cx + R, g.nx - 1);
                        } else {
                            int r = (s - 2) >> 1;
                            row = cy - R + 1 + r;
                            xa = xb = ((s - 2) & 1) ? cx + R : cx - R;
                        }
                        bool far = false;
                        if (kd32 < CUDART_INF_F) {
                            float gx = 0.0f, gy;
                            if (s < 2) {
                                gy = s == 0 ? fmaf((float)(R - 1), cs32, fy) : fmaf((float)R, cs32, -fy);
                            } else {
                                gx = ((s - 2) & 1) ? fmaf((float)R, cs32, -fx) : fmaf((float)(R - 1), cs32, fx);
                                const int dyc = row - cy;
                                gy = dyc < 0 ? fmaf((float)(-dyc - 1), cs32, fy)
                                             : (dyc > 0 ? fmaf((float)dyc, cs32, -fy) : 0.0f);
                            }
                            gx = fmaxf(gx - mg, 0.0f);
                            gy = fmaxf(gy - mg, 0.0f);
                            far = fmaf(gx, gx, gy * gy) * (1.0f - 0x1p-18f) > kd32;
                        }
                        if (!far && row >= 0 && row < g.ny && xa <= xb && xa >= 0 && xb < g.nx) {
                            int c0 = row * g.nx + xa, c1 = row * g.nx + xb + 1;
                            sa = g.start[c0];
                            sl = g.start[c1] - g.start[c0];
                        }
                    }
                    sweep_segments<KS>(g, tk, nseg, sa, sl, qp.x, qp.y, cq, queue, lane, md, mi);
                }
            }
            // distance from q to the unsearched cells: to the sides of the searched square
            // [cx - R, cx + R] x [cy - R, cy + R] that are not the grid's edge, in FP32.  The
            // error is absolute, not relative to the bound: cs32 and fx are truncations of
            // FP64 values (each off by up to 2^-23 of its size), and a side term is small only
            // when |fx| is close to R cs or (R + 1) cs, so the term can exceed the true
            // distance by up to ~2^-22 (R + 1) cs however small it is.  2^-20 (R + 1) cs32 is
            // taken off every bound before the test (it covers that error with room for the
            // cell assignment of the grid build, relative 2^-50), and the square of what is
            // left is shrunk by 2^-18 for the FP32 roundings of the last FMA and the square:
            // a lower bound, so the exact keys decide.
            float bound = CUDART_INF_F;
            if (cx - R > 0) bound = fminf(bound, fmaf((float)R, cs32, fx));
            if (cx + R < g.nx - 1) bound = fminf(bound, fmaf((float)(R + 1), cs32, -fx));
            if (cy - R > 0) bound = fminf(bound, fmaf((float)R, cs32, fy));
            if (cy + R < g.ny - 1) bound = fminf(bound, fmaf((float)(R + 1), cs32, -fy));
            if (bound == CUDART_INF_F) done = true;
            else {
                const float safe = fmaf(-0x1p-20f * (float)(R + 1), cs32, bound);
                if (safe > 0.0f) {
                    const float b2 = safe * safe * (1.0f - 0x1p-18f);
                    done = tk.kd < (unsigned long long)__double_as_longlong(f32_to_f64(b2));
                }
            }
        }
        int64_t ob = out_ptr ? out_ptr[node] : node * (int64_t)k;
        bool short_list = !(tk.kd < KEY_INF);
        if (short_list && lane == 0) atomicOr(err_flag, 1);
#pragma unroll
        for (int s = 0; s < KS; s++) {
            int t = s * 32 + lane;
            if (t < k) {
                out_idx[ob + t] = short_list ? -1 : tk.id[s];
                if (out_d2) out_d2[ob + t] = __longlong_as_double((long long)tk.d[s]);
            }
        }
    }
}
}  // namespace

cudaError_t launch_knn(const GridDev &g, const double2 *Q, const int32_t *qcls,
                       const int32_t *q_node, bool node_query, int64_t nq, const int32_t *kq, int kuni, int kmax,
                       const int64_t *out_ptr, int32_t *out_idx, double *out_d2, int r0,
                       int *err_flag, int num_sms, cudaStream_t st)
{
    if (nq <= 0) return cudaSuccess;
    int threads = 256;
    int64_t want = (nq * 32 + threads - 1) / threads;
    int64_t cap = (int64_t)num_sms * 16;
    int blocks = (int)(want < cap ? want : cap);
    if (blocks < 1) blocks = 1;
    if (kmax <= 32)
        knn_kernel<1><<<blocks, threads, 0, st>>>(g, Q, qcls, q_node, node_query, nq, kq, kuni, out_ptr,
                                                  out_idx, out_d2, r0, err_flag);
    else if (kmax <= 64)
        knn_kernel<2><<<blocks, threads, 0, st>>>(g, Q, qcls, q_node, node_query, nq, kq, kuni, out_ptr,
                                                  out_idx, out_d2, r0, err_flag);
    else if (kmax <= 128)
        knn_kernel<4><<<blocks, threads, 0, st>>>(g, Q, qcls, q_node, node_query, nq, kq, kuni, out_ptr,
                                                  out_idx, out_d2, r0, err_flag);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}
