// Tiled FP32 stencil application for the RK4 stages of du/dt = L u on F fields (the
// right-hand side of examples/adv_diff_test.jl:151-152 applied to many fields at once).
//
// The per-row stage kernels of sparse.cu gather, for every row, its k neighbours' field rows
// (F values each) through L1/L2: 30 gathers of a 256-byte row per output row at F = 64, which
// makes them L1-throughput bound at ~20 % of HBM.  Here rows are grouped into tiles of 64
// consecutive rows of the Z-curve order (spatially compact blocks of nodes).  The union of a
// tile's stencil columns (~2.6 x 64 columns at k = 30) is copied into shared memory once per
// stage by asynchronous 16-byte copies (cp.async.cg, L2 only) spread over the CTA's threads,
// together with the tile's weights and row records.  (One TMA bulk copy per 256-byte field
// row was measured first: ~170 small bulk copies per tile held a tile to ~7 us, about three
// times its compute time.)
//
// Each warp computes one group of 8 rows.  The group's weights are stored dense over the
// group's own columns (~70 at k = 30, ~45 % of them nonzero): for every such column a lane
// reads the column's field row once from shared memory (its F / 32 fields) and the column's
// 8 weights as two broadcast float4s, and updates all 8 rows.  Against one row at a time this
// cuts the shared-memory gathers per output row from ~30 to ~9 and needs no per-entry index
// arithmetic; the zero weights cost FMAs, of which the FP32 pipe has plenty here.  A CTA is one
// tile (8 warps, single-buffered); up to three CTAs share an SM, so one tile's copies overlap
// the others' arithmetic.
//
// The sum is evaluated in difference form against a reference node of the tile,
//     (L v)_i = sum_t w_t (v_{c_t} - v_ref) + s_i v_ref,   s_i = sum_t w_t (FP64 row sum),
// which equals the plain sum in exact arithmetic.  The operator's rows nearly sum to zero (it
// is made of derivatives) while its weights are large (nu/h^2, gamma/h^4), so the plain FP32
// sum loses digits to cancellation; the differences of a smooth field across a tile are
// small, and their FP32 products carry an error proportional to them instead of to |v|.  The
// subtraction is done in registers as each column row is read.
//
// Stage (Horner form of classic RK4 for a constant operator, see api.cu):
//     out_i = u_i + c (L v)_i  on free rows,   out_i = u_i on held rows.
#include "rbffd_internal.cuh"
#include "rk4_tiled.cuh"

namespace {

constexpr int TT = TileOp::T, TG = TileOp::G, NGRP = TileOp::T / TileOp::G;

// ---------------------------------------------------------------------------------------
// Tile build.  One CTA of 8 warps per tile: sort the tile's stencil column ids and keep the
// distinct ones (the union), map every entry to its slot in the union; then warp g sorts the
// slots of group g's rows, keeps the distinct ones (the group's columns) and writes, per
// column, the 8 rows' weights.  P (a power of two >= T * KP) keys for the tile, PG (a power
// of two >= G * KP) per group, in shared memory.
// ---------------------------------------------------------------------------------------
__device__ void block_bitonic_sort(int32_t *key, int P)
{
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int32_t a = key[i], b = key[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        key[i] = b;
                        key[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__device__ void warp_bitonic_sort(int32_t *key, int P, int lane)
{
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int32_t a = key[i], b = key[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        key[i] = b;
                        key[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Exclusive block scan of one int per thread; returns the prefix, *total gets the sum.
__device__ int block_scan_excl(int v, int *sh, int *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(RBFFD_FULL, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int s = lane < nw ? sh[lane] : 0;
        int si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(RBFFD_FULL, si, o);
            if (lane >= o) si += t;
        }
        if (lane < nw) sh[lane] = si - s;
        if (lane == nw - 1) sh[32] = si;
    }
    __syncthreads();
    const int r = inc - v + sh[w];
    *total = sh[32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ int lower_bound_i32(const int32_t *a, int n, int32_t v)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// mode 0: cnt[tile] = union size, gcnt[tile * 8 + g] = group g's column count rounded up to a
// multiple of 4.  mode 1: union ids, group columns and weights, row records.
__global__ void __launch_bounds__(32 * NGRP) tile_build_kernel(TileOp t, int64_t rows, const int32_t *__restrict__ order,
                                                         const int64_t *__restrict__ row_ptr,
                                                         const int32_t *__restrict__ col,
                                                         const float *__restrict__ val32,
                                                         const double *__restrict__ val64,
                                                         const uint8_t *__restrict__ fixed, int P, int PG, int mode,
                                                         int32_t *__restrict__ cnt, int32_t *__restrict__ gcnt)
{
    extern __shared__ __align__(16) int32_t tb_smem[];
    const int KP = t.KP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;  // blockDim = 32 * NGRP
    int32_t *key = tb_smem;                                       // P
    int32_t *uq = key + P;                                        // P
    float *rw = reinterpret_cast<float *>(uq + P);                // T x KP entry weights
    int32_t *rslot = reinterpret_cast<int32_t *>(rw + TT * KP);   // T x KP entry slots (-1: none)
    int32_t *gk = rslot + TT * KP;                                // NGRP x PG group slots
    int32_t *gu = gk + NGRP * PG;                                 // NGRP x PG distinct group slots
    __shared__ int sh[33];
    __shared__ int rlen[TT];
    for (int64_t tile = blockIdx.x; tile < t.ntile; tile += gridDim.x) {
        for (int e = threadIdx.x; e < P; e += blockDim.x) {
            int32_t id = INT_MAX;
            if (e < TT * KP) {
                const int i = e / KP, k = e - i * KP;
                const int64_t gi = tile * TT + i;
                if (gi < rows) {
                    const int32_t r = order[gi];
                    const int64_t a = row_ptr[r];
                    if (k < (int)(row_ptr[r + 1] - a)) id = col[a + k];
                }
            }
            key[e] = id;
        }
        __syncthreads();
        block_bitonic_sort(key, P);
        // distinct keys: a contiguous chunk of P / blockDim per thread
        const int per = P / blockDim.x, b0 = threadIdx.x * per;
        int c = 0;
        for (int e = b0; e < b0 + per; e++) c += key[e] != INT_MAX && (e == 0 || key[e] != key[e - 1]);
        int total;
        int pos = block_scan_excl(c, sh, &total);
        const int32_t ubase = mode ? t.uptr[tile] : 0;
        for (int e = b0; e < b0 + per; e++) {
            if (key[e] != INT_MAX && (e == 0 || key[e] != key[e - 1])) {
                uq[pos] = key[e];
                if (mode) t.uni[ubase + pos] = key[e];
                pos++;
            }
        }
        __syncthreads();
        // each row's entries as union slots
        for (int e = threadIdx.x; e < TT * KP; e += blockDim.x) {
            const int i = e / KP, k = e - i * KP;
            const int64_t gi = tile * TT + i;
            int len = 0, s = -1;
            float w = 0.0f;
            if (gi < rows) {
                const int32_t r = order[gi];
                const int64_t a = row_ptr[r];
                len = (int)(row_ptr[r + 1] - a);
                if (k < len) {
                    s = lower_bound_i32(uq, total, col[a + k]);
                    w = val32[a + k];
                }
            }
            rslot[e] = s;
            rw[e] = w;
            if (k == 0) rlen[i] = len;
        }
        __syncthreads();
        // group `warp`: its rows' slots, sorted, the distinct ones in gu
        {
            int32_t *gb = gk + warp * PG, *go = gu + warp * PG;
            for (int e = lane; e < PG; e += 32) {
                int32_t v = INT_MAX;
                if (e < TG * KP) {
                    const int s = rslot[(warp * TG + e / KP) * KP + e % KP];
                    if (s >= 0) v = s;
                }
                gb[e] = v;
            }
            __syncwarp();
            warp_bitonic_sort(gb, PG, lane);
            const int gper = PG / 32, e0 = lane * gper;
            int gc = 0;
            for (int e = e0; e < e0 + gper; e++) gc += gb[e] != INT_MAX && (e == 0 || gb[e] != gb[e - 1]);
            int inc = gc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int tv = __shfl_up_sync(RBFFD_FULL, inc, o);
                if (lane >= o) inc += tv;
            }
            const int Cg = __shfl_sync(RBFFD_FULL, inc, 31);
            int gp = inc - gc;
            for (int e = e0; e < e0 + gper; e++)
                if (gb[e] != INT_MAX && (e == 0 || gb[e] != gb[e - 1])) go[gp++] = gb[e];
            __syncwarp();
            const int Cg4 = (Cg + 3) & ~3;
            if (mode == 0) {
                if (lane == 0) gcnt[tile * NGRP + warp] = Cg4;
            } else {
                const int64_t base = t.gptr[tile * NGRP + warp];
                for (int j = lane; j < Cg4; j += 32) {
                    const int s = j < Cg ? go[j] : 0;  // padding: slot 0 with zero weights
                    float w8[TG];
#pragma unroll
                    for (int r = 0; r < TG; r++) {
                        w8[r] = 0.0f;
                        const int i = warp * TG + r;
                        if (j < Cg)
                            for (int k = 0; k < rlen[i]; k++)
                                if (rslot[i * KP + k] == s) w8[r] = rw[i * KP + k];
                    }
                    t.gslot[base + j] = (uint32_t)s * (uint32_t)t.F;
                    float4 *dst = reinterpret_cast<float4 *>(t.gw + (base + j) * TG);
                    dst[0] = make_float4(w8[0], w8[1], w8[2], w8[3]);
                    dst[1] = make_float4(w8[4], w8[5], w8[6], w8[7]);
                }
            }
        }
        // row records: the row, its FP64 row sum (as FP32), whether it is held
        if (mode == 1 && (int)threadIdx.x < TT) {
            const int i = threadIdx.x;
            const int64_t gi = tile * TT + i;
            int4 ri = make_int4(-1, 0, 0, 0);
            if (gi < rows) {
                const int32_t r = order[gi];
                double acc = 0.0;
                for (int64_t a = row_ptr[r]; a < row_ptr[r + 1]; a++) acc += val64[a];
                ri = make_int4(r, __float_as_int((float)acc), 0, (fixed && fixed[r]) ? 1 : 0);
            }
            t.rowinfo[gi] = ri;
        }
        if (mode == 0 && threadIdx.x == 0) cnt[tile] = total;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Stage kernel.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 16-byte asynchronous global -> shared copy through L2 (LDGSTS), completion tracked per thread
// by commit groups.
__device__ __forceinline__ void cp16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Shared-memory layout of a stage CTA (byte offsets): union field rows (ucap x F floats) at 0,
// the union's column ids, the tile's row records, group columns and weights, the reference row,
// the groups' first columns.
struct StageArgs {
    TileOp t;
    const float *v;  // stage input, gathered (rows x F)
    const float *u;  // RK4 state (rows x F); may equal v
    float *out;      // rows x F
    float c;
    uint32_t idofs, rofs, sofs, wofs, vrofs, gofs, bytes;
};

// F / 32 fields per lane (F >= 32); one field on each of the first F lanes otherwise.
template <int N>
struct Fv {
    float a[N];
};
template <int N>
__device__ __forceinline__ Fv<N> ld_fields(const float *p)
{
    Fv<N> r;
    if constexpr (N == 4) {
        const float4 q = *reinterpret_cast<const float4 *>(p);
        r.a[0] = q.x;
        r.a[1] = q.y;
        r.a[2] = q.z;
        r.a[3] = q.w;
    } else if constexpr (N == 2) {
        const float2 q = *reinterpret_cast<const float2 *>(p);
        r.a[0] = q.x;
        r.a[1] = q.y;
    } else {
        r.a[0] = *p;
    }
    return r;
}
template <int N>
__device__ __forceinline__ void st_fields(float *p, const Fv<N> &v)
{
    if constexpr (N == 4)
        *reinterpret_cast<float4 *>(p) = make_float4(v.a[0], v.a[1], v.a[2], v.a[3]);
    else if constexpr (N == 2)
        *reinterpret_cast<float2 *>(p) = make_float2(v.a[0], v.a[1]);
    else
        *p = v.a[0];
}

// A tile's ids and offsets, loaded into registers one tile ahead (their global loads are in
// flight while the current tile is copied and computed) and stored to shared memory when the
// current tile's copies have been issued.  Up to three union ids per thread.
struct TileMeta {
    int32_t a = 0, U = 0, g0 = 0, gn = 0, gofs = 0, ref = 0, row = -1;
    int32_t id[3] = {0, 0, 0};
    __device__ void load(const TileOp &t, int64_t tile)
    {
        if ((int)threadIdx.x < TT) row = t.rowinfo[tile * TT + threadIdx.x].x;
        a = t.uptr[tile];
        U = t.uptr[tile + 1] - a;
        g0 = t.gptr[tile * NGRP];
        gn = t.gptr[tile * NGRP + NGRP] - g0;
        if ((int)threadIdx.x <= NGRP) gofs = t.gptr[tile * NGRP + threadIdx.x] - g0;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int i = threadIdx.x + q * blockDim.x;
            if (i < U) id[q] = t.uni[a + i];
        }
        ref = t.rowinfo[tile * TT + TT / 2].x;   // the tile's reference node: its middle row,
        if (ref < 0) ref = t.rowinfo[tile * TT].x;  // or its first, when the tile is short
    }
    // Also starts moving the tile's rows of u (read by its epilogue) from DRAM into L2.
    __device__ void store(const TileOp &t, int32_t *ids, int *goff, int *refrow, const float *u) const
    {
        if (row >= 0)
            for (int o = 0; o < t.F; o += 32)  // one 128-byte line per prefetch
                asm volatile("prefetch.global.L2 [%0];" ::"l"(u + (size_t)row * t.F + o));
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int i = threadIdx.x + q * blockDim.x;
            if (i < U) ids[i] = id[q];
        }
        for (int i = threadIdx.x + 3 * blockDim.x; i < U; i += blockDim.x) ids[i] = t.uni[a + i];
        if ((int)threadIdx.x <= NGRP) goff[threadIdx.x] = gofs;
        if (threadIdx.x == 0) *refrow = ref;
    }
};

// One stage over all tiles: persistent CTAs (one tile at a time, 8 warps) walk the tiles with
// a stride of gridDim.x.  Per tile: issue the copies of the group columns, weights, row
// records and reference row (contiguous per tile) and of the union's field rows (by the ids
// stored one tile earlier); load the next tile's ids and offsets into registers; wait,
// barrier; store the next tile's ids and offsets (nothing reads them before the next
// barrier); warp g computes group g from shared memory and writes its 8 rows; barrier.
// Resident CTAs per SM requested (registers) and the unroll of the column loop.  Measured at
// 2048^2 nodes, 64 fields (ms per step): 3 CTAs unrolled 1x 5.12, 2x 5.02, 4x 5.25; 2 CTAs
// unrolled 2x 5.46.
#ifndef RBFFD_TILE_MINB
#define RBFFD_TILE_MINB 3
#endif
#ifndef RBFFD_TILE_UNROLL
#define RBFFD_TILE_UNROLL 2
#endif
// 32 and 64 fields: each half-warp takes every other column (0: the whole warp per column).
#ifndef RBFFD_TILE_CW2
#define RBFFD_TILE_CW2 1
#endif
#ifndef RBFFD_TILE_UNROLL_CW2
#define RBFFD_TILE_UNROLL_CW2 1
#endif
constexpr int kTileUnroll = RBFFD_TILE_UNROLL, kTileUnrollCW2 = RBFFD_TILE_UNROLL_CW2;
template <int F>
__global__ void __launch_bounds__(32 * NGRP, (F >= 128 ? 2 : RBFFD_TILE_MINB)) rk4_tile_stage_kernel(StageArgs s)
{
    extern __shared__ __align__(128) unsigned char ts_smem[];
    // CW columns in flight per warp (one per half-warp when 2), LPC lanes per column, FPL
    // fields per lane
    constexpr int CW = (RBFFD_TILE_CW2 && (F == 32 || F == 64)) ? 2 : 1, LPC = 32 / CW;
    constexpr int FPL = F >= LPC ? F / LPC : 1, Q4 = F / 4;
    constexpr int kUnroll = CW == 2 ? kTileUnrollCW2 : kTileUnroll;
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    const TileOp &t = s.t;
    float *fb = reinterpret_cast<float *>(ts_smem);
    int32_t *ids = reinterpret_cast<int32_t *>(ts_smem + s.idofs);
    int4 *rinfo = reinterpret_cast<int4 *>(ts_smem + s.rofs);
    uint32_t *gsl = reinterpret_cast<uint32_t *>(ts_smem + s.sofs);
    float *gwt = reinterpret_cast<float *>(ts_smem + s.wofs);
    float *vref = reinterpret_cast<float *>(ts_smem + s.vrofs);
    int *goff = reinterpret_cast<int *>(ts_smem + s.gofs);
    int *refrow = goff + NGRP + 1;
    const int cl = lane & (LPC - 1);
    const bool lact = cl * FPL < F;  // F < 32: only the first F lanes hold fields
    const int lofs = lact ? cl * FPL : 0;
    int64_t tile = blockIdx.x;
    if (tile >= t.ntile) return;
    TileMeta cur;
    cur.load(t, tile);
    cur.store(t, ids, goff, refrow, s.u);
    __syncthreads();
    for (; tile < t.ntile; tile += gridDim.x) {
        const int U = cur.U, g0 = cur.g0, gn = cur.gn;
        const int c0 = goff[g], cn = goff[g + 1] - c0;
        for (int c = threadIdx.x; c < gn / 4; c += blockDim.x) cp16(gsl + 4 * c, t.gslot + g0 + 4 * c);
        for (int c = threadIdx.x; c < 2 * gn; c += blockDim.x) cp16(gwt + 4 * c, t.gw + (size_t)g0 * TG + 4 * c);
        for (int c = threadIdx.x; c < TT; c += blockDim.x) cp16(rinfo + c, t.rowinfo + tile * TT + c);
        if ((int)threadIdx.x < Q4) cp16(vref + 4 * threadIdx.x, s.v + (size_t)(*refrow) * F + 4 * threadIdx.x);
        for (int c = threadIdx.x; c < U * Q4; c += blockDim.x) {
            const int row = c / Q4, part = c - row * Q4;
            cp16(fb + 4 * c, s.v + (size_t)ids[row] * F + 4 * part);
        }
        cp_commit();
        const int64_t nxt = tile + gridDim.x;
        if (nxt < t.ntile) cur.load(t, nxt);
        cp_wait_all();
        __syncthreads();  // the tile is in shared memory; its ids and offsets are consumed
        if (nxt < t.ntile) cur.store(t, ids, goff, refrow, s.u);  // read after the next barrier
        {
            // With CW = 2 the two half-warps take alternate columns of the group (j + half,
            // j + half + 2 of each block of four), so that a column's field row and weights
            // are read by 16 lanes; their partial sums are added at the end, half 0 finishing
            // rows 0-3 and half 1 rows 4-7.  The s_i v_ref term enters through half 0 only.
            const int half = CW == 2 ? lane >> 4 : 0;
            const Fv<FPL> vr = ld_fields<FPL>(vref + lofs);
            float rs[TG];
#pragma unroll
            for (int r = 0; r < TG; r++) rs[r] = half == 0 ? __int_as_float(rinfo[g * TG + r].y) : 0.0f;
            const uint4 *sl4 = reinterpret_cast<const uint4 *>(gsl + c0);
            const float4 *w4 = reinterpret_cast<const float4 *>(gwt + (size_t)c0 * TG);
            const float *fbl = fb + lofs;
            // Packed FP32: one fma.rn.f32x2 updates two rows.  The weights of rows (2i, 2i+1)
            // are adjacent in the group's weight record, so they form a register pair as
            // loaded.  With two or more fields per lane, A holds (row 2i field 2e, row 2i+1
            // field 2e+1) and B (row 2i field 2e+1, row 2i+1 field 2e), so that the column's
            // differences (d_2e, d_2e+1) and their swap serve all row pairs; with one field per
            // lane the difference is duplicated.
            constexpr int RP = TG / 2, NP = FPL >= 2 ? FPL / 2 : 1;
            float2 A[RP][NP], B[RP][NP];
            float2 nv[NP];
#pragma unroll
            for (int e = 0; e < NP; e++) {
                if constexpr (FPL >= 2) {
                    nv[e] = make_float2(-vr.a[2 * e], -vr.a[2 * e + 1]);
#pragma unroll
                    for (int i = 0; i < RP; i++) {
                        A[i][e] = make_float2(rs[2 * i] * vr.a[2 * e], rs[2 * i + 1] * vr.a[2 * e + 1]);
                        B[i][e] = make_float2(rs[2 * i] * vr.a[2 * e + 1], rs[2 * i + 1] * vr.a[2 * e]);
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < RP; i++) A[i][e] = make_float2(rs[2 * i] * vr.a[0], rs[2 * i + 1] * vr.a[0]);
                }
            }
            auto column = [&](const Fv<FPL> &xq, const float4 wa, const float4 wb) {
                const float2 wp[RP] = {make_float2(wa.x, wa.y), make_float2(wa.z, wa.w), make_float2(wb.x, wb.y),
                                       make_float2(wb.z, wb.w)};
#pragma unroll
                for (int e = 0; e < NP; e++) {
                    if constexpr (FPL >= 2) {
                        const float2 d = __fadd2_rn(make_float2(xq.a[2 * e], xq.a[2 * e + 1]), nv[e]);
                        const float2 ds = make_float2(d.y, d.x);
#pragma unroll
                        for (int i = 0; i < RP; i++) {
                            A[i][e] = __ffma2_rn(wp[i], d, A[i][e]);
                            B[i][e] = __ffma2_rn(wp[i], ds, B[i][e]);
                        }
                    } else {
                        const float d = xq.a[0] - vr.a[0];
                        const float2 dd = make_float2(d, d);
#pragma unroll
                        for (int i = 0; i < RP; i++) A[i][e] = __ffma2_rn(wp[i], dd, A[i][e]);
                    }
                }
            };
#pragma unroll kUnroll
            for (int j = 0; j < cn; j += 4) {
                const uint4 s4 = sl4[j >> 2];
                if constexpr (CW == 2) {
                    const uint32_t sc[2] = {half ? s4.y : s4.x, half ? s4.w : s4.z};
                    Fv<FPL> x[2];
#pragma unroll
                    for (int q = 0; q < 2; q++) x[q] = ld_fields<FPL>(fbl + sc[q]);
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const int col = j + half + 2 * q;
                        column(x[q], w4[2 * col], w4[2 * col + 1]);
                    }
                } else {
                    const uint32_t sc[4] = {s4.x, s4.y, s4.z, s4.w};
                    Fv<FPL> x[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) x[q] = ld_fields<FPL>(fbl + sc[q]);
#pragma unroll
                    for (int q = 0; q < 4; q++) column(x[q], w4[2 * (j + q)], w4[2 * (j + q) + 1]);
                }
            }
            float acc[TG][FPL];
#pragma unroll
            for (int i = 0; i < RP; i++) {
#pragma unroll
                for (int e = 0; e < NP; e++) {
                    if constexpr (FPL >= 2) {
                        acc[2 * i][2 * e] = A[i][e].x;
                        acc[2 * i + 1][2 * e + 1] = A[i][e].y;
                        acc[2 * i][2 * e + 1] = B[i][e].x;
                        acc[2 * i + 1][2 * e] = B[i][e].y;
                    } else {
                        acc[2 * i][0] = A[i][e].x;
                        acc[2 * i + 1][0] = A[i][e].y;
                    }
                }
            }
            // rows this lane finishes: all 8 (CW = 1) or 4 of them (CW = 2)
            constexpr int NR = TG / CW;
            float fin[NR][FPL];
#pragma unroll
            for (int r = 0; r < NR; r++) {
#pragma unroll
                for (int f = 0; f < FPL; f++) {
                    if constexpr (CW == 2) {
                        const float send = half ? acc[r][f] : acc[r + NR][f];
                        const float keep = half ? acc[r + NR][f] : acc[r][f];
                        fin[r][f] = keep + __shfl_xor_sync(RBFFD_FULL, send, 16);
                    } else {
                        fin[r][f] = acc[r][f];
                    }
                }
            }
            if (lact) {
                // all rows' u loads issued before the first store
                const int rb = g * TG + half * NR;
                int4 ri[NR];
                Fv<FPL> uu[NR];
#pragma unroll
                for (int r = 0; r < NR; r++) {
                    ri[r] = rinfo[rb + r];
                    uu[r] = ld_fields<FPL>(s.u + (size_t)(ri[r].x < 0 ? 0 : ri[r].x) * F + lofs);
                }
#pragma unroll
                for (int r = 0; r < NR; r++) {
                    if (ri[r].x < 0) continue;
                    Fv<FPL> res;
#pragma unroll
                    for (int f = 0; f < FPL; f++) res.a[f] = ri[r].w ? uu[r].a[f] : fmaf(s.c, fin[r][f], uu[r].a[f]);
                    st_fields<FPL>(s.out + (size_t)ri[r].x * F + lofs, res);
                }
            }
        }
        __syncthreads();  // the buffer is free; the next tile's ids and offsets are visible
    }
}

// Shared memory of one CTA (offsets in StageArgs).
void stage_layout(const TileOp &t, int F, StageArgs &s)
{
    auto up128 = [](uint32_t b) { return (b + 127u) & ~127u; };
    s.idofs = up128((uint32_t)t.ucap * (uint32_t)F * 4u);
    s.rofs = s.idofs + up128((uint32_t)t.ucap * 4u);
    s.sofs = s.rofs + up128((uint32_t)TT * 16u);
    s.wofs = s.sofs + up128((uint32_t)t.gcap * 4u);
    s.vrofs = s.wofs + up128((uint32_t)t.gcap * TG * 4u);
    s.gofs = s.vrofs + up128((uint32_t)F * 4u);
    s.bytes = s.gofs + up128((uint32_t)(NGRP + 2) * 4u);  // goff[NGRP + 1], the reference row
}

int pow2_at_least(int v, int lo)
{
    int P = lo;
    while (P < v) P <<= 1;
    return P;
}

size_t build_smem(const TileOp &t, int P, int PG)
{
    return (size_t)2 * P * sizeof(int32_t) + (size_t)TT * t.KP * (sizeof(float) + sizeof(int32_t)) +
           (size_t)2 * NGRP * PG * sizeof(int32_t);
}

template <int F>
cudaError_t prepare_t(TileOp &t, size_t smem)
{
    cudaError_t e =
        cudaFuncSetAttribute(rk4_tile_stage_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rk4_tile_stage_kernel<F>, 32 * NGRP, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    t.ctas_per_sm = occ;
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_tile_build(TileOp &t, int64_t rows, const int32_t *order, const int64_t *row_ptr,
                              const int32_t *col, const float *val32, const double *val64, const uint8_t *fixed,
                              int mode, int32_t *cnt, int32_t *gcnt, int num_sms, cudaStream_t st)
{
    if (t.KP < 1 || !tile_stage_supported(t.F)) return cudaErrorInvalidValue;
    const int P = pow2_at_least(TT * t.KP, 256), PG = pow2_at_least(TG * t.KP, 32);
    const size_t smem = build_smem(t, P, PG);
    cudaError_t e = cudaFuncSetAttribute(tile_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int64_t blocks = t.ntile < (int64_t)num_sms * 8 ? t.ntile : (int64_t)num_sms * 8;
    if (blocks < 1) blocks = 1;
    tile_build_kernel<<<(int)blocks, 32 * NGRP, smem, st>>>(t, rows, order, row_ptr, col, val32, val64, fixed, P, PG,
                                                           mode, cnt, gcnt);
    return cudaGetLastError();
}

size_t tile_stage_smem(const TileOp &t, int F)
{
    StageArgs s{};
    stage_layout(t, F, s);
    return s.bytes;
}

bool tile_stage_supported(int F) { return F == 4 || F == 8 || F == 16 || F == 32 || F == 64 || F == 128; }

cudaError_t tile_stage_prepare(TileOp &t, int F)
{
    const size_t smem = tile_stage_smem(t, F);
    switch (F) {
    case 4: return prepare_t<4>(t, smem);
    case 8: return prepare_t<8>(t, smem);
    case 16: return prepare_t<16>(t, smem);
    case 32: return prepare_t<32>(t, smem);
    case 64: return prepare_t<64>(t, smem);
    case 128: return prepare_t<128>(t, smem);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_tile_stage(const TileOp &t, const float *v, const float *u, float *out, int F, double c,
                              int num_sms, cudaStream_t st)
{
    if (t.ntile <= 0) return cudaSuccess;
    if (F != t.F) return cudaErrorInvalidValue;  // the layout's offsets are for t.F fields
    if (t.ctas_per_sm < 1) return cudaErrorInvalidConfiguration;  // tile_stage_prepare not run
    StageArgs s{};
    s.t = t;
    s.v = v;
    s.u = u;
    s.out = out;
    s.c = (float)c;
    stage_layout(t, F, s);
    const size_t smem = s.bytes;
    const int64_t cap = (int64_t)num_sms * t.ctas_per_sm;
    const int blocks = (int)(t.ntile < cap ? t.ntile : cap);
    const int nt = 32 * NGRP;
    switch (F) {
    case 4: rk4_tile_stage_kernel<4><<<blocks, nt, smem, st>>>(s); break;
    case 8: rk4_tile_stage_kernel<8><<<blocks, nt, smem, st>>>(s); break;
    case 16: rk4_tile_stage_kernel<16><<<blocks, nt, smem, st>>>(s); break;
    case 32: rk4_tile_stage_kernel<32><<<blocks, nt, smem, st>>>(s); break;
    case 64: rk4_tile_stage_kernel<64><<<blocks, nt, smem, st>>>(s); break;
    case 128: rk4_tile_stage_kernel<128><<<blocks, nt, smem, st>>>(s); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
