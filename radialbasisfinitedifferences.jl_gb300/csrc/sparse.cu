// Sparse operator kernels: CSR SpMV / multi-field SpMM (the stencil application of the
// time-stepping right-hand side, examples/adv_diff_test.jl:151-152) and the CSR -> CSC
// transpose that hands the operators back as Julia SparseMatrixCSC data
// (sparse(I, J, V), src/generate_operator.jl:171-182: rows ascending in each column,
// explicit zeros kept).
#include "rbffd_internal.cuh"

namespace {

// SpMV, one thread per row.  GB300 runs FP64 at 1/64 of the FP32 rate and an FP64 warp
// instruction costs the same whatever its active mask, so a cross-lane reduction of partial
// sums (5 FP64 adds per row) would cost more than the row's own FMAs; here every FP64
// instruction is one lane's FMA of its own row.  All of a row's weight and index loads are
// independent and issued before the x gathers (streaming hints keep x in L2).
__global__ void __launch_bounds__(256) spmv_f64_rows(int64_t rows, const int64_t *__restrict__ row_ptr,
                                                     const int32_t *__restrict__ col,
                                                     const double *__restrict__ val,
                                                     const double *__restrict__ x, double *__restrict__ y)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows;
         r += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = row_ptr[r], b = row_ptr[r + 1];
        double acc = 0.0;
        int64_t t = a;
        for (; t + 4 <= b; t += 4) {
            double w0 = __ldcs(val + t), w1 = __ldcs(val + t + 1), w2 = __ldcs(val + t + 2), w3 = __ldcs(val + t + 3);
            int c0 = __ldcs(col + t), c1 = __ldcs(col + t + 1), c2 = __ldcs(col + t + 2), c3 = __ldcs(col + t + 3);
            acc = fma(w0, __ldg(x + c0), acc);
            acc = fma(w1, __ldg(x + c1), acc);
            acc = fma(w2, __ldg(x + c2), acc);
            acc = fma(w3, __ldg(x + c3), acc);
        }
        for (; t < b; t++) acc = fma(__ldcs(val + t), __ldg(x + __ldcs(col + t)), acc);
        __stcs(y + r, acc);
    }
}

// Uniform stencil size K (even): row r occupies [r*K, r*K + K); 16-byte weight loads and
// 8-byte index loads, fully unrolled.
template <int K>
__global__ void __launch_bounds__(256) spmv_f64_uniform(int64_t rows, const int32_t *__restrict__ col,
                                                        const double *__restrict__ val,
                                                        const double *__restrict__ x, double *__restrict__ y)
{
    static_assert(K % 2 == 0, "even K");
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const double2 *v2 = reinterpret_cast<const double2 *>(val + r * K);
        const int2 *c2 = reinterpret_cast<const int2 *>(col + r * K);
        double2 w[K / 2];
        int2 c[K / 2];
#pragma unroll
        for (int i = 0; i < K / 2; i++) {
            w[i] = __ldcs(v2 + i);
            c[i] = __ldcs(c2 + i);
        }
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < K / 2; i++) {
            acc = fma(w[i].x, __ldg(x + c[i].x), acc);
            acc = fma(w[i].y, __ldg(x + c[i].y), acc);
        }
        __stcs(y + r, acc);
    }
}

// Multi-field SpMM: one warp per row, lanes over fields.  X is [cols][F] row-major.
template <typename T>
__global__ void __launch_bounds__(256) spmm_kernel(int64_t rows, const int64_t *__restrict__ row_ptr,
                                                   const int32_t *__restrict__ col,
                                                   const T *__restrict__ val,
                                                   const T *__restrict__ x, T *__restrict__ y, int F)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < rows; r += nw) {
        int64_t a = row_ptr[r], b = row_ptr[r + 1];
        for (int f0 = 0; f0 < F; f0 += 64) {
            T acc0 = 0, acc1 = 0;
            int f = f0 + lane;
            for (int64_t t = a; t < b; t++) {
                T w = val[t];
                int64_t c = col[t];
                const T *xr = x + c * F;
                if (f < F) acc0 = fma(w, xr[f], acc0);
                if (f + 32 < F) acc1 = fma(w, xr[f + 32], acc1);
            }
            if (f < F) y[r * F + f] = acc0;
            if (f + 32 < F) y[r * F + f + 32] = acc1;
        }
    }
}

__global__ void csc_count_kernel(int64_t nnz, const int32_t *col, unsigned long long *cnt)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz;
         t += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[col[t]], 1ull);
}

// Scatter every CSR entry to its column; rowval gets the 0-based row id, perm the CSR position.
__global__ void csc_scatter_kernel(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                                   int64_t row_begin, const int64_t *colstart,
                                   unsigned long long *fill, int64_t *rowval, int64_t *perm)
{
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < rows; r += nw) {
        for (int64_t t = row_ptr[r] + lane; t < row_ptr[r + 1]; t += 32) {
            int c = col[t];
            int64_t pos = colstart[c] + (int64_t)atomicAdd(&fill[c], 1ull);
            rowval[pos] = r + row_begin;
            perm[pos] = t;
        }
    }
}

// Sort each column segment by row.  Warp per column: rank of each entry = number of entries
// with a smaller row (rows inside a column are distinct); segments longer than 256 fall back
// to one lane's insertion sort.
__global__ void csc_sort_kernel(int64_t ncols, const int64_t *colstart, int64_t *rowval,
                                int64_t *perm)
{
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < ncols; c += nw) {
        int64_t a = colstart[c], b = colstart[c + 1];
        int len = (int)(b - a);
        if (len <= 1) continue;
        if (len <= 256) {
            int64_t rv[8], pv[8];
            int rk[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                int t = lane + 32 * k;
                rv[k] = t < len ? rowval[a + t] : INT64_MAX;
                pv[k] = t < len ? perm[a + t] : 0;
                rk[k] = 0;
            }
            int nchunk = (len + 31) / 32;
            for (int kk = 0; kk < nchunk; kk++) {
#pragma unroll 4
                for (int src = 0; src < 32; src++) {
                    int64_t other = 0;
#pragma unroll
                    for (int k = 0; k < 8; k++)
                        if (k == kk) other = __shfl_sync(RBFFD_FULL, rv[k], src);
#pragma unroll
                    for (int k = 0; k < 8; k++) rk[k] += (other < rv[k]) ? 1 : 0;
                }
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < 8; k++) {
                int t = lane + 32 * k;
                if (t < len) {
                    rowval[a + rk[k]] = rv[k];
                    perm[a + rk[k]] = pv[k];
                }
            }
        } else if (lane == 0) {
            for (int64_t i = a + 1; i < b; i++) {
                int64_t rvi = rowval[i], pvi = perm[i];
                int64_t j = i - 1;
                while (j >= a && rowval[j] > rvi) {
                    rowval[j + 1] = rowval[j];
                    perm[j + 1] = perm[j];
                    j--;
                }
                rowval[j + 1] = rvi;
                perm[j + 1] = pvi;
            }
        }
        __syncwarp();
    }
}

__global__ void gather_f64_kernel(int64_t n, const int64_t *perm, const double *src, double *dst)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        dst[t] = src[perm[t]];
}

__global__ void add_i64_kernel(int64_t n, int64_t *a, int64_t v)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        a[t] += v;
}

__global__ void f64_to_f32_kernel(int64_t n, const double *a, float *b)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        b[t] = (float)a[t];
}

int blocks_for(int64_t n, int threads, int64_t cap = 65535 * 4)
{
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

}  // namespace

cudaError_t launch_spmv_f64(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                            const double *val, const double *x, double *y, int group, int num_sms,
                            cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    int threads = 256;
    int blocks = blocks_for(rows, threads, (int64_t)num_sms * 64);
    // `group` carries the uniform stencil size (0 = general CSR)
    switch (group) {
    case 20: spmv_f64_uniform<20><<<blocks, threads, 0, st>>>(rows, col, val, x, y); break;
    case 30: spmv_f64_uniform<30><<<blocks, threads, 0, st>>>(rows, col, val, x, y); break;
    case 42: spmv_f64_uniform<42><<<blocks, threads, 0, st>>>(rows, col, val, x, y); break;
    default: spmv_f64_rows<<<blocks, threads, 0, st>>>(rows, row_ptr, col, val, x, y); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_spmm(int64_t rows, const int64_t *row_ptr, const int32_t *col, const void *val,
                        const void *x, void *y, int nfields, int dtype, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    int threads = 256;
    int blocks = blocks_for(rows * 32, threads, 152 * 64);
    if (dtype == 0)
        spmm_kernel<double><<<blocks, threads, 0, st>>>(rows, row_ptr, col, (const double *)val,
                                                        (const double *)x, (double *)y, nfields);
    else
        spmm_kernel<float><<<blocks, threads, 0, st>>>(rows, row_ptr, col, (const float *)val,
                                                       (const float *)x, (float *)y, nfields);
    return cudaGetLastError();
}

cudaError_t launch_csc_count(int64_t nnz, const int32_t *col, int64_t *colcount, cudaStream_t st)
{
    csc_count_kernel<<<blocks_for(nnz, 256), 256, 0, st>>>(nnz, col, (unsigned long long *)colcount);
    return cudaGetLastError();
}

cudaError_t launch_csc_scatter(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                               int64_t row_begin, const int64_t *colstart, int64_t *fill,
                               int64_t *rowval, int64_t *perm, cudaStream_t st)
{
    csc_scatter_kernel<<<blocks_for(rows * 32, 256), 256, 0, st>>>(
        rows, row_ptr, col, row_begin, colstart, (unsigned long long *)fill, rowval, perm);
    return cudaGetLastError();
}

cudaError_t launch_csc_sort_segments(int64_t ncols, const int64_t *colstart, int64_t *rowval,
                                     int64_t *perm, cudaStream_t st)
{
    csc_sort_kernel<<<blocks_for(ncols * 32, 256), 256, 0, st>>>(ncols, colstart, rowval, perm);
    return cudaGetLastError();
}

cudaError_t launch_gather_f64(int64_t nnz, const int64_t *perm, const double *src, double *dst,
                              cudaStream_t st)
{
    gather_f64_kernel<<<blocks_for(nnz, 256), 256, 0, st>>>(nnz, perm, src, dst);
    return cudaGetLastError();
}

cudaError_t launch_add_i64(int64_t n, int64_t *a, int64_t v, cudaStream_t st)
{
    add_i64_kernel<<<blocks_for(n, 256), 256, 0, st>>>(n, a, v);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(int64_t n, const double *a, float *b, cudaStream_t st)
{
    f64_to_f32_kernel<<<blocks_for(n, 256), 256, 0, st>>>(n, a, b);
    return cudaGetLastError();
}
