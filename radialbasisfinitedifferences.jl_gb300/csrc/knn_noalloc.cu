// rbffd_knn_noalloc: the kNN stencil search for callers that cannot allocate device memory.
//
// Who needs it: hosts whose device memory is owned by another allocator that must not be
// bypassed (a Julia CUDA.jl or PyTorch caching pool running the time-stepping loop),
// programs that fix their device-memory budget at start-up and must not grow it, and code
// paths that must not synchronise the device (cudaMalloc/cudaFree may).  rbffd_calculateneighbors
// allocates its grid and output staging per call; this entry point allocates nothing.
//
// Its grid scratch (bounding-box partials, cell histogram and offsets, nodes in cell order)
// lives in one file-scope __device__ array of RBFFD_NOALLOC_SCRATCH_BYTES that every GPU
// loading the library holds until the process exits.  The node count is limited to
// RBFFD_NOALLOC_MAX_NODES.  Inputs and outputs are caller-owned device buffers.
//
// Host code may not use the array's name as a device address (it is a host-side stand-in),
// so the first call on each device, with that device current, looks the address up with
// cudaGetSymbolAddress and caches it; make that first call before any stream capture.
// Under CUDA's default lazy module loading the array is only placed in device memory when
// this translation unit's module is first loaded on a device -- by that first call's
// cudaGetSymbolAddress (at library load instead with CUDA_MODULE_LOADING=EAGER).  That first
// call can therefore itself need the array's 5 MiB of free device memory, and returns
// RBFFD_ECUDA if the device has none left: make it before the caller's allocator reserves
// the device's memory.  Later calls need no device memory at all.
// Every call reuses the same array and leaves its contents behind; everything that must
// start at zero is cleared by the call itself.  Calls that overlap on the GPU (two streams,
// two host threads) race on the array and must be serialised by the caller.
#include <math.h>
#include <string.h>

#include <mutex>
#include <string>

#include "rbffd_internal.cuh"

#define RBFFD_EXPORT extern "C" __attribute__((visibility("default")))

static __device__ __align__(256) unsigned char g_knn_scratch[RBFFD_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};
// Messages go where rbffd_last_error(NULL) reads them (this entry point has no handle).
int noalloc_fail(int code, const std::string &msg)
{
    set_handleless_error(msg);
    return code;
}

// Device address of g_knn_scratch on the current device (looked up once per device).
cudaError_t scratch_address(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_knn_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = (unsigned char *)g_scratch_addr[dev];
    return cudaSuccess;
}

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

// Carve the scratch for N nodes and ncell cells; returns false if it does not fit.
struct Carve {
    double *partial, *box;
    int *bad, *err;
    int64_t *count, *start64;
    int32_t *start32, *fill, *cell_of, *ids;
    double2 *pts;
    void *scan_tmp;
    size_t scan_bytes;
};

bool carve(unsigned char *base, int64_t N, int64_t ncell, int nblk, Carve &c)
{
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + o;
        o += up256(bytes);
        return p;
    };
    c.partial = (double *)take(sizeof(double) * 4 * nblk);
    c.box = (double *)take(sizeof(double) * 4);
    c.bad = (int *)take(sizeof(int));
    c.err = (int *)take(sizeof(int));
    c.count = (int64_t *)take(sizeof(int64_t) * (ncell + 1));
    c.start64 = (int64_t *)take(sizeof(int64_t) * (ncell + 1));
    c.start32 = (int32_t *)take(sizeof(int32_t) * (ncell + 1));
    c.fill = (int32_t *)take(sizeof(int32_t) * ncell);
    c.cell_of = (int32_t *)take(sizeof(int32_t) * N);
    c.ids = (int32_t *)take(sizeof(int32_t) * N);
    c.pts = (double2 *)take(sizeof(double2) * N);
    c.scan_bytes = scan_tmp_bytes(ncell);
    c.scan_tmp = take(c.scan_bytes);
    return o <= RBFFD_NOALLOC_SCRATCH_BYTES;
}

#define CKN(expr)                                                                                    \
    do {                                                                                             \
        cudaError_t _e = (expr);                                                                     \
        if (_e != cudaSuccess) return noalloc_fail(RBFFD_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

}  // namespace

RBFFD_EXPORT int rbffd_knn_noalloc(const double *X_dev, int64_t N, int k, int32_t *idx_dev, double *d2_dev,
                                   void *stream)
{
    if (!X_dev || !idx_dev) return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: null buffer");
    if (N < 1 || N > RBFFD_NOALLOC_MAX_NODES)
        return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: N = " + std::to_string(N) + " outside [1, " +
                                              std::to_string(RBFFD_NOALLOC_MAX_NODES) + "]");
    if (k < 1 || k > N || k > RBFFD_MAX_K)
        return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: k out of range");
    if (((uintptr_t)X_dev) % 16 != 0) return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: X must be 16-byte aligned");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    CKN(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(RBFFD_ECUDA, "rbffd_knn_noalloc: device ordinal too large");
    unsigned char *base = nullptr;
    CKN(scratch_address(dev, &base));
    const double2 *X = (const double2 *)X_dev;
    const int nblk = 256;
    // bounding box
    Carve c;
    carve(base, N, 1, nblk, c);
    CKN(launch_bbox(X, N, c.partial, nblk, c.box, c.bad, st));
    double hb[4];
    int hbad = 0;
    CKN(cudaMemcpyAsync(hb, c.box, sizeof(hb), cudaMemcpyDeviceToHost, st));
    CKN(cudaMemcpyAsync(&hbad, c.bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    if (hbad) return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: non-finite node coordinates");
    // grid of ~2 nodes per cell, at most 2N + 16 cells (the cell count only affects speed)
    double w = hb[1] - hb[0], hh = hb[3] - hb[2];
    double area = (w > 0 ? w : 1.0) * (hh > 0 ? hh : 1.0);
    double cs = sqrt(2.0 * area / (double)N);
    if (!(cs > 0)) cs = 1.0;
    int64_t nx = (int64_t)(w / cs) + 1, ny = (int64_t)(hh / cs) + 1;
    while (nx * ny > 2 * N + 16) {
        cs *= 1.5;
        nx = (int64_t)(w / cs) + 1;
        ny = (int64_t)(hh / cs) + 1;
    }
    int64_t ncell = nx * ny;
    if (!carve(base, N, ncell, nblk, c)) return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: grid does not fit the scratch");
    CKN(cudaMemsetAsync(c.count, 0, sizeof(int64_t) * (ncell + 1), st));
    CKN(cudaMemsetAsync(c.err, 0, sizeof(int), st));
    CKN(launch_grid_fill(X, nullptr, N, hb[0], hb[2], cs, (int)nx, (int)ny, c.count, c.cell_of, st));
    CKN(scan_exclusive_i64(c.count, c.start64, ncell, c.scan_tmp, c.scan_bytes, st));
    CKN(launch_grid_scatter(X, nullptr, N, c.cell_of, c.start64, c.start32, ncell, c.fill, c.pts, c.ids, nullptr, st));
    GridDev g{hb[0], hb[2], cs, (int)nx, (int)ny, c.start32, c.pts, c.ids, nullptr};
    double rho = (double)N / (double)ncell;
    int r0 = (int)ceil((sqrt((double)k / rho) - 1.0) * 0.5);
    if (r0 < 0) r0 = 0;
    int ndev_sms = 0;
    CKN(cudaDeviceGetAttribute(&ndev_sms, cudaDevAttrMultiProcessorCount, dev));
    CKN(launch_knn(g, X, nullptr, nullptr, true, N, nullptr, k, k, nullptr, idx_dev, d2_dev, r0, c.err, ndev_sms, st));
    int herr = 0;
    CKN(cudaMemcpyAsync(&herr, c.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    if (herr) return noalloc_fail(RBFFD_EINVAL, "rbffd_knn_noalloc: fewer candidate nodes than k");
    return RBFFD_OK;
}
