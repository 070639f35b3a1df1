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

// SELL-32 layout of a uniform-stencil operator (sliced ELLPACK with slice height 32, one warp):
// slice (tile) i holds rows 32i..32i+31 column-major, entry t of row 32i + l at
// (i*K + t)*32 + l, so the t-th weights and column ids of a warp's 32 rows are one contiguous
// 256-byte / 128-byte line.  Rows past the end are padded with weight 0 and column 0.
__global__ void __launch_bounds__(256) csr_to_sell_kernel(int64_t rows, int K, const int32_t *__restrict__ col,
                                                          const double *__restrict__ val, int nops, int64_t nnz,
                                                          int64_t padded, int32_t *__restrict__ scol,
                                                          double *__restrict__ sval)
{
    const int lane = threadIdx.x & 31;
    const int64_t ntile = (rows + 31) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t tile = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; tile < ntile; tile += nw) {
        const int64_t r = tile * 32 + lane;
        const bool ok = r < rows;
        const int64_t src = (ok ? r : 0) * K, dst = tile * 32 * K + lane;
        for (int t = 0; t < K; t++) scol[dst + 32 * t] = ok ? col[src + t] : 0;
        for (int q = 0; q < nops; q++)
            for (int t = 0; t < K; t++) sval[q * padded + dst + 32 * t] = ok ? val[q * nnz + src + t] : 0.0;
    }
}

// FP64 SpMV on the SELL-32 layout: warp per 32-row slice, lane per row.  Every weight and
// column-id load is a fully coalesced line, so no shared-memory staging is needed and the
// kernel runs at full occupancy (the latency of the x gathers is hidden by warps, not
// stages); each row accumulates in four independent FP64 chains.
// Streamed read-only loads with an L2 evict-first hint, written as non-volatile asm so that
// the compiler may schedule them freely (all of a batch's weight and column-id loads in flight
// together).
__device__ __forceinline__ double ld_stream(const double *p, unsigned long long pol)
{
    double v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int ld_stream(const int32_t *p, unsigned long long pol)
{
    int v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}

// Entries per batch of loads in the SELL SpMV, and its CTAs per SM (the grid: beyond the
// 8 resident ones, later waves even out the slices per warp).  1M rows, k = 30, fraction of
// measured HBM: batch 10 / 8 CTAs 75.0 %, batch 15 74.9 -> 75.9 %, 16 CTAs 77.4-78.1 %,
// batch 15 and 16 CTAs 78.6 %, 32 CTAs 76.8 %, 64 CTAs 76.6 %.
#ifndef RBFFD_SPMV_BATCH
#define RBFFD_SPMV_BATCH 15
#endif
#ifndef RBFFD_SPMV_CTAS_PER_SM
#define RBFFD_SPMV_CTAS_PER_SM 16
#endif
template <int K>
__global__ void __launch_bounds__(256) spmv_f64_sell(int64_t rows, int kr, const int32_t *__restrict__ scol,
                                                     const double *__restrict__ sval, const double *__restrict__ x,
                                                     double *__restrict__ y)
{
    const int k = K > 0 ? K : kr;
    const int lane = threadIdx.x & 31;
    const int64_t ntile = (rows + 31) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    for (int64_t tile = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; tile < ntile; tile += nw) {
        const int32_t *c = scol + tile * 32 * k + lane;
        const double *v = sval + tile * 32 * k + lane;
        double a[4] = {0.0, 0.0, 0.0, 0.0};
        if constexpr (K > 0) {
            // batches of entries: the batch's column/weight loads, then its x gathers, then the
            // FMAs (65 % -> 75 % of HBM against one entry at a time)
            constexpr int BT = RBFFD_SPMV_BATCH;
#pragma unroll
            for (int t0 = 0; t0 < K; t0 += BT) {
                int cc[BT];
                double vv[BT], xx[BT];
#pragma unroll
                for (int u = 0; u < BT; u++)
                    if (t0 + u < K) {
                        cc[u] = ld_stream(c + 32 * (t0 + u), pol);
                        vv[u] = ld_stream(v + 32 * (t0 + u), pol);
                    }
#pragma unroll
                for (int u = 0; u < BT; u++)
                    if (t0 + u < K) xx[u] = __ldg(x + cc[u]);
#pragma unroll
                for (int u = 0; u < BT; u++)
                    if (t0 + u < K) a[(t0 + u) & 3] = fma(vv[u], xx[u], a[(t0 + u) & 3]);
            }
        } else {
            int t = 0;
            for (; t + 4 <= k; t += 4) {
#pragma unroll
                for (int u = 0; u < 4; u++)
                    a[u] = fma(ld_stream(v + 32 * (t + u), pol), __ldg(x + ld_stream(c + 32 * (t + u), pol)), a[u]);
            }
            for (; t < k; t++) a[0] = fma(ld_stream(v + 32 * t, pol), __ldg(x + ld_stream(c + 32 * t, pol)), a[0]);
        }
        const int64_t r = tile * 32 + lane;
        if (r < rows) __stcs(y + r, (a[0] + a[1]) + (a[2] + a[3]));
    }
}


// v[f] = sum_t val[t] x[col[t]][f] for one row, lanes over fields f = f0 + lane and f0 + lane + 32:
// the row's column ids and weights are loaded once, coalesced (lane t holds entry t), and
// broadcast by shuffles, so the x gathers do not wait on dependent index loads.
template <typename T>
__device__ __forceinline__ void row_fields(int64_t a, int len, const int32_t *__restrict__ col,
                                           const T *__restrict__ val, const T *__restrict__ x, int F, int f0,
                                           int lane, T &v0, T &v1)
{
    const int f = f0 + lane, g = f + 32;
    for (int t0 = 0; t0 < len; t0 += 32) {
        const int tl = t0 + lane;
        int cl = 0;
        T wl = 0;
        if (tl < len) {
            cl = __ldg(col + a + tl);
            wl = __ldg(val + a + tl);
        }
        const int cnt = len - t0 < 32 ? len - t0 : 32;
#pragma unroll 6
        for (int t = 0; t < cnt; t++) {
            const int cc = __shfl_sync(0xffffffffu, cl, t);
            const T wt = __shfl_sync(0xffffffffu, wl, t);
            const T *xr = x + (int64_t)cc * F;
            if (f < F) v0 = fma(wt, __ldg(xr + f), v0);
            if (g < F) v1 = fma(wt, __ldg(xr + g), v1);
        }
    }
}

// Multi-field SpMM: one warp per row, lanes over fields.  X is [cols][F] row-major.
template <typename T>
__global__ void __launch_bounds__(256) spmm_kernel(int64_t rows, const int64_t *__restrict__ row_ptr,
                                                   const int32_t *__restrict__ col,
                                                   const T *__restrict__ val,
                                                   const T *__restrict__ x, T *__restrict__ y, int F)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < rows; r += nw) {
        const int64_t a = row_ptr[r];
        const int len = (int)(row_ptr[r + 1] - a);
        for (int f0 = 0; f0 < F; f0 += 64) {
            T v0 = 0, v1 = 0;
            row_fields<T>(a, len, col, val, x, F, f0, lane, v0, v1);
            const int f = f0 + lane, g = f + 32;
            if (f < F) y[r * F + f] = v0;
            if (g < F) y[r * F + g] = v1;
        }
    }
}

// One RK4 stage of du/dt = L u on F fields (classic RK4; examples/adv_diff_test.jl solves the
// same semi-discrete system with SSPRK43).  v = L w for every row, v = 0 on fixed rows (held
// at their initial values, the Dirichlet overwrite of examples/adv_diff_test.jl:166-167),
// then the epilogue folds the RK bookkeeping in, so no stage derivative is stored:
//   mode 0 (stage 1): acc  = v;          wnext = u + c v
//   mode 1 (stage 2, 3): acc += 2 v;     wnext = u + c v
//   mode 2 (stage 4): unext = u + c (acc + v)        (c = dt / 6)
//   mode 3 (any stage of the Horner form, see api.cu): out = u + c v  (no accumulator)
// Rows are visited in `order` (a spatial locality order of the nodes): a CTA takes chunks of
// 64 consecutive rows of that order and its 8 warps work on neighbouring rows together, so the
// gathered rows of w (F values each) are shared through L1 instead of being re-read from L2.
template <typename T>
__global__ void __launch_bounds__(256) rk4_stage_kernel(int64_t rows, const int32_t *__restrict__ order,
                                                        const int64_t *__restrict__ row_ptr,
                                                        const int32_t *__restrict__ col, const T *__restrict__ val,
                                                        const T *__restrict__ w, const T *__restrict__ u,
                                                        T *__restrict__ acc, T *__restrict__ out,
                                                        const uint8_t *__restrict__ fixed, int F, T c, int mode)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t nchunk = (rows + 63) >> 6;
    for (int64_t ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
        for (int k = 0; k < 8; k++) {
            const int64_t idx = ch * 64 + k * 8 + wib;
            if (idx >= rows) break;
            const int64_t r = order ? (int64_t)order[idx] : idx;
            const int64_t a = row_ptr[r];
            const int len = (int)(row_ptr[r + 1] - a);
            const bool fx = fixed && fixed[r];
            for (int f0 = 0; f0 < F; f0 += 64) {
                const int f = f0 + lane, g = f + 32;
                T v0 = 0, v1 = 0;
                if (!fx) row_fields<T>(a, len, col, val, w, F, f0, lane, v0, v1);
                const int64_t o = r * F;
                if (f < F) {
                    if (mode == 0) {
                        acc[o + f] = v0;
                        out[o + f] = fma(c, v0, u[o + f]);
                    } else if (mode == 1) {
                        acc[o + f] = fma((T)2, v0, acc[o + f]);
                        out[o + f] = fma(c, v0, u[o + f]);
                    } else if (mode == 2) {
                        out[o + f] = fma(c, acc[o + f] + v0, u[o + f]);
                    } else {
                        out[o + f] = fma(c, v0, u[o + f]);
                    }
                }
                if (g < F) {
                    if (mode == 0) {
                        acc[o + g] = v1;
                        out[o + g] = fma(c, v1, u[o + g]);
                    } else if (mode == 1) {
                        acc[o + g] = fma((T)2, v1, acc[o + g]);
                        out[o + g] = fma(c, v1, u[o + g]);
                    } else if (mode == 2) {
                        out[o + g] = fma(c, acc[o + g] + v1, u[o + g]);
                    } else {
                        out[o + g] = fma(c, v1, u[o + g]);
                    }
                }
            }
        }
    }
}

// 16-byte vectors of fields: 4 floats or 2 doubles per lane.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using V = float4;
    static constexpr int N = 4;
    __device__ static V zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
    __device__ static V fma1(float a, V x, V y)
    {
        return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
    }
    __device__ static V add(V a, V b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
};
template <>
struct Vec16<double> {
    using V = double2;
    static constexpr int N = 2;
    __device__ static V zero() { return make_double2(0.0, 0.0); }
    __device__ static V fma1(double a, V x, V y) { return make_double2(fma(a, x.x, y.x), fma(a, x.y, y.y)); }
    __device__ static V add(V a, V b) { return make_double2(a.x + b.x, a.y + b.y); }
};

// Sum over the row's entries of val[t] * x[col[t]][...] for this lane's 16-byte group of
// fields: LPR = F / Vec16::N lanes share a row (a warp holds 32 / LPR rows), entries are
// loaded once per LPR-wide round and broadcast inside the row's lane group by shuffles;
// rows past their length (or past the end) contribute weight 0 from column 0.
template <typename T>
__device__ __forceinline__ typename Vec16<T>::V row_vec(int64_t a, int len, int lenmax, const int32_t *__restrict__ col,
                                                       const T *__restrict__ val, const T *__restrict__ x, int F,
                                                       int LPR, int sl)
{
    using VT = Vec16<T>;
    typename VT::V s0 = VT::zero(), s1 = VT::zero();
    const typename VT::V *xv = reinterpret_cast<const typename VT::V *>(x) + sl;
    const int FV = F / VT::N;
    for (int t0 = 0; t0 < lenmax; t0 += LPR) {
        const int tl = t0 + sl;
        int cl = 0;
        T wl = 0;
        if (tl < len) {
            cl = __ldg(col + a + tl);
            wl = __ldg(val + a + tl);
        }
        const int cnt = lenmax - t0 < LPR ? lenmax - t0 : LPR;
        int t = 0;
        for (; t + 4 <= cnt; t += 4) {  // four independent gathers in flight
            int c[4];
            T wv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                c[u] = __shfl_sync(0xffffffffu, cl, t + u, LPR);
                wv[u] = __shfl_sync(0xffffffffu, wl, t + u, LPR);
            }
            typename VT::V xg[4];
#pragma unroll
            for (int u = 0; u < 4; u++) xg[u] = __ldg(xv + (int64_t)c[u] * FV);
            s0 = VT::fma1(wv[0], xg[0], s0);
            s1 = VT::fma1(wv[1], xg[1], s1);
            s0 = VT::fma1(wv[2], xg[2], s0);
            s1 = VT::fma1(wv[3], xg[3], s1);
        }
        for (; t + 2 <= cnt; t += 2) {
            const int c0 = __shfl_sync(0xffffffffu, cl, t, LPR), c1 = __shfl_sync(0xffffffffu, cl, t + 1, LPR);
            const T w0 = __shfl_sync(0xffffffffu, wl, t, LPR), w1 = __shfl_sync(0xffffffffu, wl, t + 1, LPR);
            s0 = VT::fma1(w0, __ldg(xv + (int64_t)c0 * FV), s0);
            s1 = VT::fma1(w1, __ldg(xv + (int64_t)c1 * FV), s1);
        }
        if (t < cnt) {
            const int c0 = __shfl_sync(0xffffffffu, cl, t, LPR);
            const T w0 = __shfl_sync(0xffffffffu, wl, t, LPR);
            s0 = VT::fma1(w0, __ldg(xv + (int64_t)c0 * FV), s0);
        }
    }
    return VT::add(s0, s1);
}

// RK4 stage (same modes as rk4_stage_kernel) with 16-byte field vectors: F / Vec16::N lanes
// per row, 32 / that rows per warp, rows in Z-order chunks of (at least) 64 per CTA.  Needs F a multiple
// of Vec16::N with F / Vec16::N dividing 32.
template <typename T>
__global__ void __launch_bounds__(256) rk4_stage_vec_kernel(int64_t rows, const int32_t *__restrict__ order,
                                                            const int64_t *__restrict__ row_ptr,
                                                            const int32_t *__restrict__ col, const T *__restrict__ val,
                                                            const T *__restrict__ w, const T *__restrict__ u,
                                                            T *__restrict__ acc, T *__restrict__ out,
                                                            const uint8_t *__restrict__ fixed, int F, T c, int mode)
{
    using VT = Vec16<T>;
    using V = typename VT::V;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int LPR = F / VT::N, RPW = 32 / LPR, sub = lane / LPR, sl = lane - sub * LPR;
    // chunks of CH consecutive rows of the order: 64, or one row group of the whole CTA when
    // that is larger (8 warps x RPW rows)
    const int CH = 8 * RPW > 64 ? 8 * RPW : 64;
    const int64_t nchunk = (rows + CH - 1) / CH;
    for (int64_t ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
        for (int k = 0; k < CH; k += 8 * RPW) {
            const int64_t idx = ch * CH + k + wib * RPW + sub;
            const bool valid = idx < rows;
            const int64_t r = valid ? (order ? (int64_t)order[idx] : idx) : 0;
            const int64_t a = valid ? row_ptr[r] : 0;
            const bool fx = !valid || (fixed && fixed[r]);
            const int len = fx ? 0 : (int)(row_ptr[r + 1] - a);
            const int lenmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)len);
            if (lenmax == 0 && !__any_sync(0xffffffffu, valid)) break;
            V v = VT::zero();
            if (lenmax > 0) v = row_vec<T>(a, len, lenmax, col, val, w, F, LPR, sl);
            if (!valid) continue;
            const int64_t o = r * (F / VT::N) + sl;
            const V uu = reinterpret_cast<const V *>(u)[o];
            V *po = reinterpret_cast<V *>(out) + o;
            V *pa = reinterpret_cast<V *>(acc) + o;
            if (mode == 0) {
                *pa = v;
                *po = VT::fma1(c, v, uu);
            } else if (mode == 1) {
                *pa = VT::fma1((T)2, v, *pa);
                *po = VT::fma1(c, v, uu);
            } else if (mode == 2) {
                *po = VT::fma1(c, VT::add(*pa, v), uu);
            } else {
                *po = VT::fma1(c, v, uu);
            }
        }
    }
}

// y = A x on F fields with 16-byte field vectors (rows in natural order).
template <typename T>
__global__ void __launch_bounds__(256) spmm_vec_kernel(int64_t rows, const int64_t *__restrict__ row_ptr,
                                                       const int32_t *__restrict__ col, const T *__restrict__ val,
                                                       const T *__restrict__ x, T *__restrict__ y, int F)
{
    using VT = Vec16<T>;
    using V = typename VT::V;
    const int lane = threadIdx.x & 31;
    const int LPR = F / VT::N, RPW = 32 / LPR, sub = lane / LPR, sl = lane - sub * LPR;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r0 = warp * RPW; r0 < rows; r0 += nw * RPW) {
        const int64_t r = r0 + sub;
        const bool valid = r < rows;
        const int64_t a = valid ? row_ptr[r] : 0;
        const int len = valid ? (int)(row_ptr[r + 1] - a) : 0;
        const int lenmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)len);
        const V v = row_vec<T>(a, len, lenmax, col, val, x, F, LPR, sl);
        if (valid) reinterpret_cast<V *>(y)[r * (F / VT::N) + sl] = v;
    }
}

// ---------------------------------------------------------------------------------------
// CGLS for min ||D u - f|| (the least-squares solve of test/poisson_test.jl:115-119).
// D is an operator set's sparsity pattern with row-wise combined values; D^T products use
// the set's CSC permutation.  Scalars stay on the device: sc[0] = gamma (= ||D^T r||^2 of the
// last iteration), sc[1] = ||D p||^2, sc[2] = the new gamma.  Reductions are deterministic
// (fixed grid, per-block partials summed by one block in a fixed order).
constexpr int LSQ_BLOCKS = 256;

// D[t] = sum_q coef[q * rows + row(t)] * val[q * nnz + t] (thread per row)
__global__ void combine_rows_kernel(int64_t rows, const int64_t *__restrict__ row_ptr, const double *__restrict__ val,
                                    int64_t nnz, int nops, const double *__restrict__ coef, double *__restrict__ out)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t t = row_ptr[r]; t < row_ptr[r + 1]; t++) {
            double v = 0.0;
            for (int q = 0; q < nops; q++) v = fma(coef[(int64_t)q * rows + r], val[(int64_t)q * nnz + t], v);
            out[t] = v;
        }
    }
}

__device__ __forceinline__ void block_sum_to(double v, double *part)
{
    __shared__ double red[32];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) part[blockIdx.x] = v;
    }
}

// y = D x (thread per row) and per-block partial sums of y^2; with b != null, y = b - D x.
__global__ void __launch_bounds__(256) lsq_spmv_kernel(int64_t rows, const int64_t *__restrict__ row_ptr,
                                                       const int32_t *__restrict__ col, const double *__restrict__ val,
                                                       const double *__restrict__ x, const double *__restrict__ b,
                                                       double *__restrict__ y, double *__restrict__ part)
{
    double acc2 = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int64_t t = row_ptr[r]; t < row_ptr[r + 1]; t++) v = fma(val[t], x[col[t]], v);
        if (b) v = b[r] - v;
        y[r] = v;
        acc2 = fma(v, v, acc2);
    }
    block_sum_to(acc2, part);
}

// y = D^T x through the CSC (1-based colptr/rowval as exported to Julia, values vcsc in CSC
// order), thread per column, and per-block partial sums of y^2.
__global__ void __launch_bounds__(256) lsq_spmv_t_kernel(int64_t cols, const int64_t *__restrict__ colptr1,
                                                         const int64_t *__restrict__ rowval1, int64_t row_begin,
                                                         const double *__restrict__ vcsc, const double *__restrict__ x,
                                                         double *__restrict__ y, double *__restrict__ part)
{
    double acc2 = 0.0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cols; j += (int64_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int64_t k = colptr1[j] - 1; k < colptr1[j + 1] - 1; k++) v = fma(vcsc[k], x[rowval1[k] - 1 - row_begin], v);
        y[j] = v;
        acc2 = fma(v, v, acc2);
    }
    block_sum_to(acc2, part);
}

// sc[slot] = sum of the partials (one block, fixed order); with shift, first sc[0] = sc[2].
__global__ void lsq_final_kernel(const double *__restrict__ part, double *__restrict__ sc, int slot, int shift)
{
    double v = 0.0;
    for (int i = threadIdx.x; i < LSQ_BLOCKS; i += blockDim.x) v += part[i];
    __shared__ double red[32];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        if (shift) sc[0] = sc[2];
        sc[slot] = t;
    }
}

// u += alpha p (cols), r -= alpha q (rows), alpha = gamma / ||q||^2
__global__ void lsq_update_ur(int64_t cols, int64_t rows, double *__restrict__ u, const double *__restrict__ p,
                              double *__restrict__ r, const double *__restrict__ q, const double *__restrict__ sc)
{
    const double alpha = sc[1] > 0.0 ? sc[0] / sc[1] : 0.0;
    const int64_t n = cols > rows ? cols : rows;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < cols) u[i] = fma(alpha, p[i], u[i]);
        if (i < rows) r[i] = fma(-alpha, q[i], r[i]);
    }
}

// p = s + beta p, beta = gamma_new / gamma (p = s on the first call: first != 0)
__global__ void lsq_update_p(int64_t cols, double *__restrict__ p, const double *__restrict__ s,
                             const double *__restrict__ sc, int first)
{
    const double beta = (!first && sc[0] > 0.0) ? sc[2] / sc[0] : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cols; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], s[i]);
}

// ---------------------------------------------------------------------------------------
// Ghost-node closure (examples/adv_diff_test.jl:108-141, 160-176): u[G] = -inv(A[B,G]) A[B,~G] u.
// gidx[node] = position of the node in G, -1 otherwise.

// Left half of [W | I] (nb x 2nb, row-major): W[i][j] = A[B[i], G[j]], thread per boundary row.
__global__ void ghost_extract_kernel(int64_t nb, const int32_t *__restrict__ bnodes, const int64_t *__restrict__ row_ptr,
                                     const int32_t *__restrict__ col, const double *__restrict__ val,
                                     const int32_t *__restrict__ gidx, double *__restrict__ W)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = bnodes[i];
        for (int64_t t = row_ptr[r]; t < row_ptr[r + 1]; t++) {
            const int j = gidx[col[t]];
            if (j >= 0) W[i * 2 * nb + j] += val[t];
        }
    }
}

// Gauss-Jordan on [W | I] (nb x 2nb), step c: pivot row search by one block (largest |W[i][c]|
// over rows i >= c, lowest row on ties), swap into row c.
__global__ void gj_pivot_kernel(int64_t nb, double *__restrict__ M, int c, int *__restrict__ flag)
{
    __shared__ unsigned long long bk[256];
    __shared__ int bi[256];
    unsigned long long best = 0;
    int brow = INT_MAX;
    for (int64_t i = c + threadIdx.x; i < nb; i += blockDim.x) {
        const unsigned long long k = (unsigned long long)__double_as_longlong(M[i * 2 * nb + c]) & 0x7fffffffffffffffull;
        if (k > best || (k == best && (int)i < brow)) {
            best = k;
            brow = (int)i;
        }
    }
    bk[threadIdx.x] = best;
    bi[threadIdx.x] = brow;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
        if ((int)threadIdx.x < o) {
            const unsigned long long k = bk[threadIdx.x + o];
            const int r = bi[threadIdx.x + o];
            if (k > bk[threadIdx.x] || (k == bk[threadIdx.x] && r < bi[threadIdx.x])) {
                bk[threadIdx.x] = k;
                bi[threadIdx.x] = r;
            }
        }
        __syncthreads();
    }
    const int p = bi[0];
    if (bk[0] == 0ull || bk[0] >= 0x7ff0000000000000ull) {
        if (threadIdx.x == 0) *flag = 1;  // singular (zero, inf or NaN pivot)
        return;
    }
    if (p != c)
        for (int64_t j = threadIdx.x; j < 2 * nb; j += blockDim.x) {
            const double t = M[(int64_t)c * 2 * nb + j];
            M[(int64_t)c * 2 * nb + j] = M[(int64_t)p * 2 * nb + j];
            M[(int64_t)p * 2 * nb + j] = t;
        }
}

// Step c: multipliers fcol[i] = M[i][c] / M[c][c] of every other row.
__global__ void gj_factors_kernel(int64_t nb, const double *__restrict__ M, int c, const int *__restrict__ flag,
                                  double *__restrict__ fcol)
{
    if (*flag) return;
    const int64_t w = 2 * nb;
    const double rp = 1.0 / M[(int64_t)c * w + c];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x)
        fcol[i] = i == c ? 0.0 : M[i * w + c] * rp;
}

// Step c: eliminate column c from every other row with the (unscaled) pivot row, thread per
// element of the augmented matrix (column c itself is cleared by gj_finish_kernel).
__global__ void gj_eliminate_kernel(int64_t nb, double *__restrict__ M, int c, const int *__restrict__ flag,
                                    const double *__restrict__ fcol)
{
    if (*flag) return;
    const int64_t w = 2 * nb;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nb * w; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / w, j = e - i * w;
        if (i == c || j == c) continue;
        M[i * w + j] = fma(-fcol[i], M[(int64_t)c * w + j], M[i * w + j]);
    }
}

// Step c: clear column c of the other rows and divide the pivot row by its pivot (the pivot
// element itself is left: column c is not read again).
__global__ void gj_finish_kernel(int64_t nb, double *__restrict__ M, int c, const int *__restrict__ flag)
{
    if (*flag) return;
    const int64_t w = 2 * nb;
    const double rp = 1.0 / M[(int64_t)c * w + c];
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < w; j += (int64_t)gridDim.x * blockDim.x) {
        if (j != c) M[(int64_t)c * w + j] *= rp;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x)
        if (i != c) M[i * w + c] = 0.0;
}

// y[i][f] = sum over row B[i] of A, columns outside G, of val * u[col][f] (warp per row).
template <typename T>
__global__ void __launch_bounds__(256) ghost_rows_kernel(int64_t nb, const int32_t *__restrict__ bnodes,
                                                         const int64_t *__restrict__ row_ptr,
                                                         const int32_t *__restrict__ col, const double *__restrict__ val,
                                                         const int32_t *__restrict__ gidx, const T *__restrict__ u,
                                                         int F, double *__restrict__ y)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < nb; i += nw) {
        const int64_t r = bnodes[i];
        for (int f = lane; f < F; f += 32) {
            double acc = 0.0;
            for (int64_t t = row_ptr[r]; t < row_ptr[r + 1]; t++) {
                const int c = col[t];
                if (gidx[c] < 0) acc = fma(val[t], (double)u[(int64_t)c * F + f], acc);
            }
            y[i * F + f] = acc;
        }
    }
}

// u[G[j]][f] = -sum_i Winv[j][i] y[i][f] (Winv = the right half of the reduced [W | I]).
template <typename T>
__global__ void ghost_write_kernel(int64_t nb, const int32_t *__restrict__ gnodes, const double *__restrict__ M,
                                   const double *__restrict__ y, int F, T *__restrict__ u)
{
    const int64_t w = 2 * nb;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nb * F; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / F;
        const int f = (int)(e - j * F);
        double acc = 0.0;
        for (int64_t i = 0; i < nb; i++) acc = fma(M[j * w + nb + i], y[i * F + f], acc);
        u[(int64_t)gnodes[j] * F + f] = (T)(-acc);
    }
}

__global__ void ghost_index_kernel(int64_t nb, const int32_t *__restrict__ gnodes, int32_t *__restrict__ gidx)
{
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nb; j += (int64_t)gridDim.x * blockDim.x)
        gidx[gnodes[j]] = (int32_t)j;
}

__global__ void fill_i32_kernel(int64_t n, int32_t *a, int32_t v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void eye_right_kernel(int64_t nb, double *M)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x)
        M[i * 2 * nb + nb + i] = 1.0;
}

// val_out = sum_q coef[q] * val_q (operators with one sparsity pattern), in FP64 and FP32.
__global__ void combine_ops_kernel(int64_t nnz, const double *const *vals, const double *coef, int nq,
                                   double *out64, float *out32)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz; t += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int q = 0; q < nq; q++) acc = fma(coef[q], vals[q][t], acc);
        out64[t] = acc;
        out32[t] = (float)acc;
    }
}

// Count entries where two column arrays differ (operator sets must share a stencil pattern).
__global__ void count_diff_kernel(int64_t n, const int32_t *a, const int32_t *b, unsigned long long *cnt)
{
    unsigned long long local = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        local += a[t] != b[t];
    if (local) atomicAdd(cnt, local);
}

__global__ void csc_count_kernel(int64_t nnz, const int32_t *col, unsigned long long *cnt)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz;
         t += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[col[t]], 1ull);
}

// Scatter every CSR entry to its column; rowval gets the row id plus row_begin (a row offset,
// or 1 for 1-based rows), perm the CSR position.
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
// With inv non-null, also inv[perm[p]] = p for every final position p (the inverse of the
// gather permutation: CSR position -> CSC position).
__global__ void csc_sort_kernel(int64_t ncols, const int64_t *colstart, int64_t *rowval,
                                int64_t *perm, bool keys32, int32_t *inv)
{
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = warp; c < ncols; c += nw) {
        int64_t a = colstart[c], b = colstart[c + 1];
        int len = (int)(b - a);
        if (len <= 1) {
            if (inv && len == 1 && lane == 0) inv[perm[a]] = (int32_t)a;
            continue;
        }
        if (keys32 && len <= 64) {
            // The common case (a column of a kNN operator holds ~k rows): rank sort of two
            // register slots with 32-bit keys.  Row ids within a column are distinct, and the
            // padding key 0xffffffff exceeds every row id, so ranks are a permutation of [0, len).
            const int t1 = lane + 32;
            const int64_t r0 = lane < len ? rowval[a + lane] : 0, p0 = lane < len ? perm[a + lane] : 0;
            const int64_t r1 = t1 < len ? rowval[a + t1] : 0, p1 = t1 < len ? perm[a + t1] : 0;
            const unsigned k0 = lane < len ? (unsigned)r0 : 0xffffffffu, k1 = t1 < len ? (unsigned)r1 : 0xffffffffu;
            int rk0 = 0, rk1 = 0;
#pragma unroll 8
            for (int src = 0; src < 32; src++) {
                const unsigned o = __shfl_sync(RBFFD_FULL, k0, src);
                rk0 += o < k0;
                rk1 += o < k1;
            }
            if (len > 32) {
#pragma unroll 8
                for (int src = 0; src < 32; src++) {
                    const unsigned o = __shfl_sync(RBFFD_FULL, k1, src);
                    rk0 += o < k0;
                    rk1 += o < k1;
                }
            }
            __syncwarp();
            if (lane < len) {
                rowval[a + rk0] = r0;
                perm[a + rk0] = p0;
                if (inv) inv[p0] = (int32_t)(a + rk0);
            }
            if (t1 < len) {
                rowval[a + rk1] = r1;
                perm[a + rk1] = p1;
                if (inv) inv[p1] = (int32_t)(a + rk1);
            }
        } else if (len <= 256) {
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
                    if (inv) inv[pv[k]] = (int32_t)(a + rk[k]);
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
            if (inv)
                for (int64_t i = a; i < b; i++) inv[perm[i]] = (int32_t)i;
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

// cm[k] = min over the rows of chunk k (rows [k N / C, (k + 1) N / C)) of the smallest column
// the row's stencil references; per-block minima first, one atomic per block and chunk.
__global__ void chunk_min_col_kernel(int64_t N, int n, const int32_t *nbr, int C, int *cm)
{
    __shared__ int bm[RBFFD_MAX_CHUNKS];
    for (int k = threadIdx.x; k < C; k += blockDim.x) bm[k] = INT_MAX;
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
        int mc = INT_MAX;
        for (int t = 0; t < n; t++) mc = min(mc, nbr[r * n + t]);
        int k = 0;
        while (k + 1 < C && r >= (int64_t)(k + 1) * N / C) k++;
        atomicMin(&bm[k], mc);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < C; k += blockDim.x)
        if (bm[k] != INT_MAX) atomicMin(&cm[k], bm[k]);
}

// Columns [0, cb[i]) are referenced only by rows of chunks <= i: cb[i] = min over k > i of
// cm[k] (all columns after the last chunk); cp[i] = their CSC entry count (colstart 1-based).
__global__ void chunk_bounds_kernel(int64_t N, int C, const int *cm, const int64_t *colstart1, int64_t *cp)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t b = N;
    for (int i = C - 1; i >= 0; i--) {
        cp[i] = colstart1[b] - 1;
        if (i > 0 && (int64_t)cm[i] < b) b = cm[i];
    }
    for (int i = 1; i < C; i++)  // monotone (each bound covers the one before)
        if (cp[i] < cp[i - 1]) cp[i] = cp[i - 1];
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

// The 16-byte field-vector kernels apply when F is a multiple of the vector width, the lanes
// of a row (F / width) divide a warp, and every field array is 16-byte aligned.
bool vec_fields_ok(int F, int dtype, const void *a, const void *b, const void *c, const void *d)
{
    const int vw = dtype == 0 ? 2 : 4;
    if (F % vw) return false;
    const int lpr = F / vw;
    if (lpr > 32 || (32 % lpr)) return false;
    return ((((uintptr_t)a) | ((uintptr_t)b) | ((uintptr_t)c) | ((uintptr_t)d)) & 15u) == 0;
}


}  // namespace

cudaError_t launch_spmv_f64(int64_t rows, const int64_t *row_ptr, const int32_t *col,
                            const double *val, const double *x, double *y, int num_sms, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    const int threads = 256;
    const int blocks = blocks_for(rows, threads, (int64_t)num_sms * 64);
    spmv_f64_rows<<<blocks, threads, 0, st>>>(rows, row_ptr, col, val, x, y);
    return cudaGetLastError();
}

int64_t sell_padded(int64_t rows, int K) { return ((rows + 31) / 32) * 32 * (int64_t)K; }

cudaError_t launch_csr_to_sell(int64_t rows, int K, const int32_t *col, const double *val, int nops, int64_t nnz,
                               int32_t *scol, double *sval, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    const int64_t ntile = (rows + 31) / 32;
    csr_to_sell_kernel<<<blocks_for(ntile * 32, 256), 256, 0, st>>>(rows, K, col, val, nops, nnz,
                                                                     sell_padded(rows, K), scol, sval);
    return cudaGetLastError();
}

cudaError_t launch_spmv_sell(int64_t rows, int K, const int32_t *scol, const double *sval, const double *x, double *y,
                             int num_sms, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    const int64_t ntile = (rows + 31) / 32;
    const int blocks = blocks_for(ntile * 32, 256, (int64_t)num_sms * RBFFD_SPMV_CTAS_PER_SM);
    if (K == 30)
        spmv_f64_sell<30><<<blocks, 256, 0, st>>>(rows, K, scol, sval, x, y);
    else
        spmv_f64_sell<0><<<blocks, 256, 0, st>>>(rows, K, scol, sval, x, y);
    return cudaGetLastError();
}

cudaError_t launch_combine_rows(int64_t rows, const int64_t *row_ptr, const double *val, int64_t nnz, int nops,
                                const double *coef, double *out, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    combine_rows_kernel<<<blocks_for(rows, 256), 256, 0, st>>>(rows, row_ptr, val, nnz, nops, coef, out);
    return cudaGetLastError();
}

cudaError_t launch_lsq_spmv(int64_t rows, const int64_t *row_ptr, const int32_t *col, const double *val,
                            const double *x, const double *b, double *y, double *part, cudaStream_t st)
{
    lsq_spmv_kernel<<<LSQ_BLOCKS, 256, 0, st>>>(rows, row_ptr, col, val, x, b, y, part);
    return cudaGetLastError();
}

cudaError_t launch_lsq_spmv_t(int64_t cols, const int64_t *colptr1, const int64_t *rowval1, int64_t row_begin,
                              const double *vcsc, const double *x, double *y, double *part, cudaStream_t st)
{
    lsq_spmv_t_kernel<<<LSQ_BLOCKS, 256, 0, st>>>(cols, colptr1, rowval1, row_begin, vcsc, x, y, part);
    return cudaGetLastError();
}

cudaError_t launch_lsq_final(const double *part, double *sc, int slot, int shift, cudaStream_t st)
{
    lsq_final_kernel<<<1, 256, 0, st>>>(part, sc, slot, shift);
    return cudaGetLastError();
}

cudaError_t launch_lsq_update_ur(int64_t cols, int64_t rows, double *u, const double *p, double *r, const double *q,
                                 const double *sc, cudaStream_t st)
{
    const int64_t n = cols > rows ? cols : rows;
    lsq_update_ur<<<blocks_for(n, 256), 256, 0, st>>>(cols, rows, u, p, r, q, sc);
    return cudaGetLastError();
}

cudaError_t launch_lsq_update_p(int64_t cols, double *p, const double *s, const double *sc, int first, cudaStream_t st)
{
    lsq_update_p<<<blocks_for(cols, 256), 256, 0, st>>>(cols, p, s, sc, first);
    return cudaGetLastError();
}

int lsq_partials() { return LSQ_BLOCKS; }

// Dense inverse of the ghost block: [W | I] in M (nb x 2nb, row-major) reduced to [I | W^-1].
cudaError_t ghost_build(int64_t N, int64_t nb, const int32_t *bnodes, const int32_t *gnodes, const int64_t *row_ptr,
                        const int32_t *col, const double *val, int32_t *gidx, double *M, double *fcol, int *flag,
                        cudaStream_t st)
{
    fill_i32_kernel<<<blocks_for(N, 256), 256, 0, st>>>(N, gidx, -1);
    ghost_index_kernel<<<blocks_for(nb, 256), 256, 0, st>>>(nb, gnodes, gidx);
    cudaError_t e = cudaMemsetAsync(M, 0, sizeof(double) * nb * 2 * nb, st);
    if (e != cudaSuccess) return e;
    ghost_extract_kernel<<<blocks_for(nb, 256), 256, 0, st>>>(nb, bnodes, row_ptr, col, val, gidx, M);
    eye_right_kernel<<<blocks_for(nb, 256), 256, 0, st>>>(nb, M);
    for (int c = 0; c < (int)nb; c++) {
        gj_pivot_kernel<<<1, 256, 0, st>>>(nb, M, c, flag);
        gj_factors_kernel<<<blocks_for(nb, 256), 256, 0, st>>>(nb, M, c, flag, fcol);
        gj_eliminate_kernel<<<blocks_for(nb * 2 * nb, 256), 256, 0, st>>>(nb, M, c, flag, fcol);
        gj_finish_kernel<<<blocks_for(2 * nb, 256), 256, 0, st>>>(nb, M, c, flag);
    }
    return cudaGetLastError();
}

cudaError_t ghost_apply(int64_t nb, const int32_t *bnodes, const int32_t *gnodes, const int64_t *row_ptr,
                        const int32_t *col, const double *val, const int32_t *gidx, const double *M, void *u, int F,
                        int dtype, double *y, cudaStream_t st)
{
    if (nb <= 0) return cudaSuccess;
    const int blocks = blocks_for(nb * 32, 256);
    if (dtype == 0) {
        ghost_rows_kernel<double><<<blocks, 256, 0, st>>>(nb, bnodes, row_ptr, col, val, gidx, (const double *)u, F, y);
        ghost_write_kernel<double><<<blocks_for(nb * F, 256), 256, 0, st>>>(nb, gnodes, M, y, F, (double *)u);
    } else {
        ghost_rows_kernel<float><<<blocks, 256, 0, st>>>(nb, bnodes, row_ptr, col, val, gidx, (const float *)u, F, y);
        ghost_write_kernel<float><<<blocks_for(nb * F, 256), 256, 0, st>>>(nb, gnodes, M, y, F, (float *)u);
    }
    return cudaGetLastError();
}

cudaError_t launch_spmm(int64_t rows, const int64_t *row_ptr, const int32_t *col, const void *val,
                        const void *x, void *y, int nfields, int dtype, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    int threads = 256;
    if (vec_fields_ok(nfields, dtype, x, y, y, y)) {
        const int rpw = 32 / (nfields / (dtype == 0 ? 2 : 4));
        const int blocks = blocks_for((rows + rpw - 1) / rpw * 32, threads, 152 * 64);
        if (dtype == 0)
            spmm_vec_kernel<double><<<blocks, threads, 0, st>>>(rows, row_ptr, col, (const double *)val,
                                                                (const double *)x, (double *)y, nfields);
        else
            spmm_vec_kernel<float><<<blocks, threads, 0, st>>>(rows, row_ptr, col, (const float *)val,
                                                               (const float *)x, (float *)y, nfields);
        return cudaGetLastError();
    }
    int blocks = blocks_for(rows * 32, threads, 152 * 64);
    if (dtype == 0)
        spmm_kernel<double><<<blocks, threads, 0, st>>>(rows, row_ptr, col, (const double *)val,
                                                        (const double *)x, (double *)y, nfields);
    else
        spmm_kernel<float><<<blocks, threads, 0, st>>>(rows, row_ptr, col, (const float *)val,
                                                       (const float *)x, (float *)y, nfields);
    return cudaGetLastError();
}

cudaError_t launch_rk4_stage(int64_t rows, const int32_t *order, const int64_t *row_ptr, const int32_t *col,
                             const void *val, const void *w, const void *u, void *acc, void *out,
                             const uint8_t *fixed, int F, double c, int mode, int dtype, int num_sms, cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    int blocks = blocks_for((rows + 63) / 64, 1, (int64_t)num_sms * 8);
    if (vec_fields_ok(F, dtype, w, u, acc, out)) {
        if (dtype == 0)
            rk4_stage_vec_kernel<double><<<blocks, 256, 0, st>>>(rows, order, row_ptr, col, (const double *)val,
                                                                 (const double *)w, (const double *)u, (double *)acc,
                                                                 (double *)out, fixed, F, c, mode);
        else
            rk4_stage_vec_kernel<float><<<blocks, 256, 0, st>>>(rows, order, row_ptr, col, (const float *)val,
                                                                (const float *)w, (const float *)u, (float *)acc,
                                                                (float *)out, fixed, F, (float)c, mode);
        return cudaGetLastError();
    }
    if (dtype == 0)
        rk4_stage_kernel<double><<<blocks, 256, 0, st>>>(rows, order, row_ptr, col, (const double *)val, (const double *)w,
                                                         (const double *)u, (double *)acc, (double *)out, fixed, F, c,
                                                         mode);
    else
        rk4_stage_kernel<float><<<blocks, 256, 0, st>>>(rows, order, row_ptr, col, (const float *)val, (const float *)w,
                                                        (const float *)u, (float *)acc, (float *)out, fixed, F,
                                                        (float)c, mode);
    return cudaGetLastError();
}

cudaError_t launch_combine_ops(int64_t nnz, const double *const *vals, const double *coef, int nq, double *out64,
                               float *out32, cudaStream_t st)
{
    combine_ops_kernel<<<blocks_for(nnz, 256), 256, 0, st>>>(nnz, vals, coef, nq, out64, out32);
    return cudaGetLastError();
}

cudaError_t launch_count_diff(int64_t n, const int32_t *a, const int32_t *b, unsigned long long *cnt,
                              cudaStream_t st)
{
    count_diff_kernel<<<blocks_for(n, 256), 256, 0, st>>>(n, a, b, cnt);
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
                                     int64_t *perm, int64_t row_limit, cudaStream_t st, int32_t *inv)
{
    const bool keys32 = row_limit < 0xffffffffll;  // row ids fit 32-bit keys below the padding key
    csc_sort_kernel<<<blocks_for(ncols * 32, 256), 256, 0, st>>>(ncols, colstart, rowval, perm, keys32, inv);
    return cudaGetLastError();
}

cudaError_t launch_gather_f64(int64_t nnz, const int64_t *perm, const double *src, double *dst,
                              cudaStream_t st)
{
    gather_f64_kernel<<<blocks_for(nnz, 256), 256, 0, st>>>(nnz, perm, src, dst);
    return cudaGetLastError();
}

cudaError_t launch_chunk_bounds(int64_t N, int n, const int32_t *nbr, int C, const int64_t *colstart1, int *cm,
                                int64_t *cp, cudaStream_t st)
{
    if (C < 1 || C > RBFFD_MAX_CHUNKS) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(cm, 0x7f, sizeof(int) * C, st);  // 0x7f7f7f7f: above any column
    if (e != cudaSuccess) return e;
    chunk_min_col_kernel<<<blocks_for(N, 256, 4096), 256, 0, st>>>(N, n, nbr, C, cm);
    chunk_bounds_kernel<<<1, 32, 0, st>>>(N, C, cm, colstart1, cp);
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
