// FMA-throughput microbenchmark: the FP64 and FP32 (CUDA-core, non-tensor) peaks that bound
// the weight solves.  Each thread runs 8 independent FMA chains on operands taken from kernel
// arguments (no constant folding) and stores the sums (no dead-code elimination).
#include "rbffd_internal.cuh"

#define RBFFD_EXPORT extern "C" __attribute__((visibility("default")))

namespace {
template <typename T>
__global__ void __launch_bounds__(256) fma_chain(T a, T b, int iters, T *out)
{
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
      x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++) {
            x0 = fma(x0, a, b);
            x1 = fma(x1, a, b);
            x2 = fma(x2, a, b);
            x3 = fma(x3, a, b);
            x4 = fma(x4, a, b);
            x5 = fma(x5, a, b);
            x6 = fma(x6, a, b);
            x7 = fma(x7, a, b);
        }
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-1.2345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // practically never
}

template <typename T>
double run(int blocks, int iters, cudaStream_t st)
{
    T *out = nullptr;
    cudaMallocAsync((void **)&out, sizeof(T) * blocks * 256, st);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chain<T><<<blocks, 256, 0, st>>>((T)0.999999, (T)1e-7, iters / 8, out);  // warm-up
    cudaEventRecord(e0, st);
    fma_chain<T><<<blocks, 256, 0, st>>>((T)0.999999, (T)1e-7, iters, out);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaFreeAsync(out, st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double flops = 2.0 * 8 * 16 * (double)iters * blocks * 256;
    return ms > 0 ? flops / (ms * 1e-3) / 1e12 : 0.0;
}
}  // namespace

// Measured FP64 and FP32 FMA throughput of `device` in TFLOP/s (2 flops per FMA).
RBFFD_EXPORT int rbffd_measure_fma_peaks(int device, double *fp64_tflops, double *fp32_tflops)
{
    if (cudaSetDevice(device) != cudaSuccess) return RBFFD_ECUDA;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return RBFFD_ECUDA;
    cudaStream_t st;
    if (cudaStreamCreate(&st) != cudaSuccess) return RBFFD_ECUDA;
    int blocks = prop.multiProcessorCount * 8;
    if (fp64_tflops) *fp64_tflops = run<double>(blocks, 512, st);
    if (fp32_tflops) *fp32_tflops = run<float>(blocks, 8192, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return e == cudaSuccess ? RBFFD_OK : RBFFD_ECUDA;
}
