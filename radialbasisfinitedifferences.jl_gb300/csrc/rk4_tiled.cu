// Tiled FP32 stencil application for the RK4 stages of du/dt = L u on F fields (the
// right-hand side of examples/adv_diff_test.jl:151-152 applied to many fields at once).
//
// The per-row stage kernels of sparse.cu gather, for every row, its k neighbours' field rows
// (F values each) through L1/L2: 30 gathers of a 256-byte row per output row at F = 64, which
// makes them L1-throughput bound at ~20 % of HBM.  Here rows are grouped into tiles of T
// consecutive rows of the Z-curve order (spatially compact blocks of nodes).  The union of a
// tile's stencil columns (~2.6 T columns for T = 64, k = 30) is copied into shared memory once
// per stage by asynchronous 16-byte copies (cp.async.cg, L2 only) spread over all threads of
// the CTA, double-buffered so that the next tile's copies run while the current tile is
// computed.  (One TMA bulk copy per 256-byte field row was measured first: 172 small bulk
// copies per tile held a tile to ~7 us, about three times its compute time.)  Column ids are
// stored per tile as 16-bit slots into that union, so an entry costs 4 + 2 bytes of HBM
// instead of 4 + 4.
//
// The sum is evaluated in difference form against a reference node of the tile,
//     (L v)_i = sum_t w_t (v_{c_t} - v_ref) + s_i v_ref,   s_i = sum_t w_t (FP64 row sum),
// which equals the plain sum in exact arithmetic.  The operator's rows nearly sum to zero (it
// is made of derivatives) while its weights are large (nu/h^2, gamma/h^4), so the plain FP32
// sum loses digits to cancellation; the differences of a smooth field across a tile are
// small, and their FP32 products carry an error proportional to them instead of to |v|.
//
// Stage (Horner form of classic RK4 for a constant operator, see api.cu):
//     out_i = u_i + c (L v)_i  on free rows,   out_i = u_i on held rows.
#include "rbffd_internal.cuh"
#include "rk4_tiled.cuh"

namespace {

// ---------------------------------------------------------------------------------------
// Tile build: sort each tile's stencil column ids, keep the distinct ones (the union), map
// every entry to its slot in the union.  One CTA per tile; P (a power of two >= T * KP) keys
// in shared memory.
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

// mode 0: cnt[tile] = union size, cnt2[tile] = the largest merged entry count of its row
// pairs.  mode 1: union ids, row records and the merged pair entries.  Rows 2j and 2j + 1 of a
// tile form pair j: their stencils are merged into one list of (slot, w_2j, w_2j+1) with a
// zero weight where a row does not use the column, so that the stage reads each neighbour row
// once for both rows.  bad |= 2 when a union exceeds 65535 slots.
__global__ void __launch_bounds__(256) tile_build_kernel(TileOp t, int64_t rows, const int32_t *__restrict__ order,
                                                         const int64_t *__restrict__ row_ptr,
                                                         const int32_t *__restrict__ col,
                                                         const float *__restrict__ val32,
                                                         const double *__restrict__ val64,
                                                         const uint8_t *__restrict__ fixed, int P, int mode,
                                                         int32_t *__restrict__ cnt, int32_t *__restrict__ cnt2,
                                                         int *bad)
{
    extern __shared__ __align__(16) int32_t tb_smem[];
    const int T = t.T, KP = t.KP;
    int32_t *key = tb_smem;                                          // P
    int32_t *uq = key + P;                                           // P
    float *rw = reinterpret_cast<float *>(uq + P);                   // T x KP row weights
    uint16_t *rslot = reinterpret_cast<uint16_t *>(rw + T * KP);     // T x KP row slots
    __shared__ int sh[33];
    __shared__ int rlen[256];  // T <= 256
    __shared__ int maxm;
    for (int64_t tile = blockIdx.x; tile < t.ntile; tile += gridDim.x) {
        for (int e = threadIdx.x; e < P; e += blockDim.x) {
            int32_t id = INT_MAX;
            if (e < T * KP) {
                const int i = e / KP, k = e - i * KP;
                const int64_t gi = tile * T + i;
                if (gi < rows) {
                    const int32_t r = order[gi];
                    const int64_t a = row_ptr[r];
                    if (k < (int)(row_ptr[r + 1] - a)) id = col[a + k];
                }
            }
            key[e] = id;
        }
        if (threadIdx.x == 0) maxm = 0;
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
        for (int e = threadIdx.x; e < T * KP; e += blockDim.x) {
            const int i = e / KP, k = e - i * KP;
            const int64_t gi = tile * T + i;
            int len = 0;
            if (gi < rows) {
                const int32_t r = order[gi];
                const int64_t a = row_ptr[r];
                len = (int)(row_ptr[r + 1] - a);
                if (k < len) {
                    rslot[e] = (uint16_t)lower_bound_i32(uq, total, col[a + k]);
                    rw[e] = val32[a + k];
                }
            }
            if (k == 0) rlen[i] = len;
        }
        __syncthreads();
        // merge the rows of each pair: row a's entries (with row b's weight where b has the same
        // column), then row b's entries that row a does not have
        for (int j = threadIdx.x; j < T / 2; j += blockDim.x) {
            const int ia = 2 * j, ib = ia + 1;
            const int la = rlen[ia], lb = rlen[ib];
            const int64_t base = (tile * (T / 2) + j) * (int64_t)t.KPP;
            int m = 0;
            for (int ta = 0; ta < la; ta++) {
                const uint16_t sa = rslot[ia * KP + ta];
                float wb = 0.0f;
                for (int tb = 0; tb < lb; tb++)
                    if (rslot[ib * KP + tb] == sa) wb = rw[ib * KP + tb];
                if (mode) {
                    t.pslot[base + m] = sa;
                    t.pw[base + m] = make_float2(rw[ia * KP + ta], wb);
                }
                m++;
            }
            for (int tb = 0; tb < lb; tb++) {
                const uint16_t sb = rslot[ib * KP + tb];
                bool in_a = false;
                for (int ta = 0; ta < la; ta++) in_a |= rslot[ia * KP + ta] == sb;
                if (in_a) continue;
                if (mode) {
                    t.pslot[base + m] = sb;
                    t.pw[base + m] = make_float2(0.0f, rw[ib * KP + tb]);
                }
                m++;
            }
            if (mode == 0) {
                atomicMax(&maxm, m);
                continue;
            }
            for (int q = m; q < t.KPP; q++) {  // padding: slot 0, zero weights
                t.pslot[base + q] = 0;
                t.pw[base + q] = make_float2(0.0f, 0.0f);
            }
            // row records: the row, its FP64 row sum (as FP32), the pair's entry quads (first
            // row), whether it is held
            for (int h = 0; h < 2; h++) {
                const int i = ia + h;
                const int64_t gi = tile * T + i;
                int4 ri = make_int4(-1, 0, 0, 0);
                if (gi < rows) {
                    const int32_t r = order[gi];
                    double acc = 0.0;
                    for (int64_t a = row_ptr[r]; a < row_ptr[r + 1]; a++) acc += val64[a];
                    ri = make_int4(r, __float_as_int((float)acc), h == 0 ? (m + 3) >> 2 : 0,
                                   (fixed && fixed[r]) ? 1 : 0);
                }
                t.rowinfo[gi] = ri;
            }
        }
        __syncthreads();
        if (mode == 0 && threadIdx.x == 0) {
            cnt[tile] = total;
            cnt2[tile] = maxm;
            if (total > 65535) atomicOr(bad, 2);
        }
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
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

struct StageArgs {
    TileOp t;
    const float *v;      // stage input, gathered (rows x F)
    const float *u;      // RK4 state (rows x F); may equal v
    float *out;          // rows x F
    float c;
    // shared-memory layout of one buffer: union field rows, weights, slots, row records, the
    // tile's own rows of u, the reference row, column ids (the union's, then the tile's rows)
    uint32_t wofs, sofs, rofs, uofs, refofs, idofs, bufbytes;
};

// The copies of one tile into `buf`, spread over all threads in 16-byte pieces: the union's
// field rows of v, the tile's own rows of u, the tile's reference row of v (its middle row, or
// its first when the tile is short), the merged pair entries and the row records, from the ids
// in `ids` (a shared-memory list filled one tile ahead: U union columns, then the T rows); one
// commit group per thread and tile.  After these land the tile is computed from shared memory.
template <int F>
__device__ __forceinline__ void issue_tile(const StageArgs &s, int64_t tile, int U, const int32_t *ids,
                                           unsigned char *buf)
{
    constexpr int Q4 = F / 4;  // 16-byte pieces per field row
    const TileOp &t = s.t;
    for (int c = threadIdx.x; c < U * Q4; c += blockDim.x) {
        const int row = c / Q4, part = c % Q4;
        cp16(buf + (size_t)c * 16, s.v + (size_t)ids[row] * F + 4 * part);
    }
    for (int c = threadIdx.x; c < t.T * Q4; c += blockDim.x) {
        const int row = c / Q4, part = c % Q4;
        const int32_t r = ids[U + row];
        if (r >= 0) cp16(buf + s.uofs + (size_t)c * 16, s.u + (size_t)r * F + 4 * part);
    }
    if ((int)threadIdx.x < Q4) {
        int32_t r = ids[U + t.T / 2];
        if (r < 0) r = ids[U];
        cp16(buf + s.refofs + (size_t)threadIdx.x * 16, s.v + (size_t)r * F + 4 * threadIdx.x);
    }
    const int eb = (t.T / 2) * t.KPP;  // merged pair entries of the tile
    const unsigned char *wsrc = reinterpret_cast<const unsigned char *>(t.pw + (size_t)tile * eb);
    for (int c = threadIdx.x; c < eb / 2; c += blockDim.x) cp16(buf + s.wofs + (size_t)c * 16, wsrc + (size_t)c * 16);
    const unsigned char *ssrc = reinterpret_cast<const unsigned char *>(t.pslot + (size_t)tile * eb);
    for (int c = threadIdx.x; c < eb / 8; c += blockDim.x) cp16(buf + s.sofs + (size_t)c * 16, ssrc + (size_t)c * 16);
    const int4 *rsrc = t.rowinfo + (size_t)tile * t.T;
    for (int c = threadIdx.x; c < t.T; c += blockDim.x) cp16(buf + s.rofs + (size_t)c * 16, rsrc + c);
    cp_commit();
}

// The ids list of a tile: its union's columns, then its rows (-1 past the end of the order).
// Loads up to two union ids and one row per thread into registers (issued early, stored late).
struct TileIds {
    int32_t a = 0, U = 0, id0 = 0, id1 = 0, row = -1;
    __device__ void load(const TileOp &t, int64_t tile)
    {
        a = t.uptr[tile];
        U = t.uptr[tile + 1] - a;
        if ((int)threadIdx.x < U) id0 = t.uni[a + threadIdx.x];
        if ((int)threadIdx.x + (int)blockDim.x < U) id1 = t.uni[a + threadIdx.x + blockDim.x];
        if ((int)threadIdx.x < t.T) row = t.rowinfo[tile * t.T + threadIdx.x].x;
    }
    __device__ void store(const TileOp &t, int32_t *ids) const
    {
        if ((int)threadIdx.x < U) ids[threadIdx.x] = id0;
        if ((int)threadIdx.x + (int)blockDim.x < U) ids[threadIdx.x + blockDim.x] = id1;
        for (int i = threadIdx.x + 2 * blockDim.x; i < U; i += blockDim.x) ids[i] = t.uni[a + i];
        if ((int)threadIdx.x < t.T) ids[U + threadIdx.x] = row;
    }
};

__device__ __forceinline__ float4 f4_fma(float a, float4 x, float4 y)
{
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ float4 f4_sub(float4 a, float4 b)
{
    return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 f4_add(float4 a, float4 b)
{
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float4 f4_shfl_xor(float4 a, int off)
{
    return make_float4(__shfl_xor_sync(RBFFD_FULL, a.x, off), __shfl_xor_sync(RBFFD_FULL, a.y, off),
                       __shfl_xor_sync(RBFFD_FULL, a.z, off), __shfl_xor_sync(RBFFD_FULL, a.w, off));
}

// How the lanes of a warp share a tile's row pairs at F fields: each half-warp (16 lanes) takes
// one pair; in it, LPR lanes cover a row's F fields with V float4s each (lane sl holds float4s
// sl, sl + LPR, ..., so that LPR lanes read one 128-byte piece of a field row per load), and
// SPLIT = 16 / LPR lane groups take every SPLIT-th entry quad of the pair, their partial sums
// combined by shuffles at the end.  Two float4s per lane at F >= 64 halve the weight and slot
// loads and the slot arithmetic per FMA and double the gathers in flight per lane.
template <int F>
struct StageShape {
    static constexpr int V = F >= 64 ? 2 : 1;
    static constexpr int LPR = F / (4 * V);
    static constexpr int SPLIT = 16 / LPR;
    static_assert(LPR >= 1 && LPR <= 16 && 16 % LPR == 0, "F / (4 V) lanes must divide a half-warp");
};

// One stage over all tiles.  Persistent CTAs walk the tiles with a stride of gridDim.x.
// Software pipeline per tile k: issue the copies of tile k + 1 (into the other buffer, with the
// ids stored one tile earlier), load the ids of tile k + 2 into registers, wait for this
// thread's copies of tile k, barrier, subtract the reference row from the union rows, barrier,
// compute tile k from shared memory, store the ids of tile k + 2, barrier.
//
// Difference form against a tile-wide reference row v_ref (a node of the tile):
//     (L v)_i = sum_t w_t (v_{c_t} - v_ref) + s_i v_ref,   s_i = sum_t w_t (FP64 row sum),
// equal to the plain sum in exact arithmetic; the differences of a smooth field across a tile
// are small, so the FP32 products carry an error proportional to them instead of to |v|, and
// the subtraction is paid once per union row and tile instead of once per entry.
template <int F>
__global__ void __launch_bounds__(512, 1) rk4_tile_stage_kernel(StageArgs s)
{
    extern __shared__ __align__(128) unsigned char ts_smem[];
    constexpr int Q4 = F / 4, V = StageShape<F>::V, LPR = StageShape<F>::LPR, SPLIT = StageShape<F>::SPLIT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int pr = lane >> 4, g = (lane & 15) / LPR, sl = lane % LPR;
    const TileOp &t = s.t;
    const int T = t.T, KQ = t.KPP >> 2;
    const int64_t G = gridDim.x;
    int64_t tile = blockIdx.x;
    if (tile >= t.ntile) return;
    auto bufp = [&](int b) { return ts_smem + (size_t)b * s.bufbytes; };
    auto idsp = [&](int b) { return reinterpret_cast<int32_t *>(bufp(b) + s.idofs); };
    int U0 = 0, U1 = 0;  // union sizes of the tiles whose ids sit in buffers 0 and 1
    {
        TileIds cur;
        cur.load(t, tile);
        cur.store(t, idsp(0));
        U0 = cur.U;
        if (tile + G < t.ntile) {
            TileIds nx;
            nx.load(t, tile + G);
            nx.store(t, idsp(1));
            U1 = nx.U;
        }
    }
    __syncthreads();
    issue_tile<F>(s, tile, U0, idsp(0), bufp(0));
    for (int k = 0; tile < t.ntile; k++, tile += G) {
        const int b = k & 1;
        unsigned char *buf = bufp(b);
        const int U = b ? U1 : U0;
        const int64_t nxt = tile + G, n2 = nxt + G;
        if (nxt < t.ntile) issue_tile<F>(s, nxt, b ? U0 : U1, idsp(b ^ 1), bufp(b ^ 1));
        TileIds pre;
        if (n2 < t.ntile) pre.load(t, n2);
        if (nxt < t.ntile)
            cp_wait<1>();
        else
            cp_wait<0>();
        __syncthreads();
        float4 *fb = reinterpret_cast<float4 *>(buf);
        const float4 *ref = reinterpret_cast<const float4 *>(buf + s.refofs);
        {
            const float4 rv = ref[threadIdx.x % Q4];  // blockDim is a multiple of Q4
            for (int c = threadIdx.x; c < U * Q4; c += blockDim.x) fb[c] = f4_sub(fb[c], rv);
        }
        __syncthreads();
        float4 vref[V];
#pragma unroll
        for (int v = 0; v < V; v++) vref[v] = ref[v * LPR + sl];
        const float4 *fbl = fb + sl;
        const float4 *ub = reinterpret_cast<const float4 *>(buf + s.uofs);
        const float4 *wbase = reinterpret_cast<const float4 *>(buf + s.wofs);  // 2 entries per float4
        const uint2 *sbase = reinterpret_cast<const uint2 *>(buf + s.sofs);    // 4 slots per uint2
        const int4 *rinfo = reinterpret_cast<const int4 *>(buf + s.rofs);
        for (int pj0 = 0; pj0 < T / 2; pj0 += 2 * nw) {
            // every lane of the warp reaches the shuffles below: no early exit per pair
            const int pj = pj0 + 2 * warp + pr;
            const bool live = pj < T / 2;
            const int4 ra = live ? rinfo[2 * pj] : make_int4(-1, 0, 0, 0);
            const int4 rb = live ? rinfo[2 * pj + 1] : make_int4(-1, 0, 0, 0);
            const int nq = ra.x >= 0 ? ra.z : 0;
            const float rsa = g == 0 ? __int_as_float(ra.y) : 0.0f, rsb = g == 0 ? __int_as_float(rb.y) : 0.0f;
            float4 acca[V], accb[V];
#pragma unroll
            for (int v = 0; v < V; v++) {
                acca[v] = make_float4(rsa * vref[v].x, rsa * vref[v].y, rsa * vref[v].z, rsa * vref[v].w);
                accb[v] = make_float4(rsb * vref[v].x, rsb * vref[v].y, rsb * vref[v].z, rsb * vref[v].w);
            }
            const float4 *wr = wbase + (live ? pj : 0) * (2 * KQ);
            const uint2 *sr = sbase + (live ? pj : 0) * KQ;
#pragma unroll 2
            for (int q = g; q < nq; q += SPLIT) {
                const float4 w01 = wr[2 * q], w23 = wr[2 * q + 1];  // (wa0, wb0, wa1, wb1), (wa2, wb2, wa3, wb3)
                const uint2 sv = sr[q];
                const float4 *p0 = fbl + (sv.x & 0xffffu) * Q4, *p1 = fbl + (sv.x >> 16) * Q4;
                const float4 *p2 = fbl + (sv.y & 0xffffu) * Q4, *p3 = fbl + (sv.y >> 16) * Q4;
                float4 x0[V], x1[V], x2[V], x3[V];
#pragma unroll
                for (int v = 0; v < V; v++) {
                    x0[v] = p0[v * LPR];
                    x1[v] = p1[v * LPR];
                    x2[v] = p2[v * LPR];
                    x3[v] = p3[v * LPR];
                }
#pragma unroll
                for (int v = 0; v < V; v++) {
                    acca[v] = f4_fma(w01.x, x0[v], acca[v]);
                    accb[v] = f4_fma(w01.y, x0[v], accb[v]);
                    acca[v] = f4_fma(w01.z, x1[v], acca[v]);
                    accb[v] = f4_fma(w01.w, x1[v], accb[v]);
                    acca[v] = f4_fma(w23.x, x2[v], acca[v]);
                    accb[v] = f4_fma(w23.y, x2[v], accb[v]);
                    acca[v] = f4_fma(w23.z, x3[v], acca[v]);
                    accb[v] = f4_fma(w23.w, x3[v], accb[v]);
                }
            }
            float4 *outp = reinterpret_cast<float4 *>(s.out);
            if constexpr (SPLIT == 1) {
                if (ra.x >= 0) {
                    const float4 *ur = ub + (2 * pj) * Q4 + sl;
                    float4 *o = outp + (int64_t)ra.x * Q4 + sl;
#pragma unroll
                    for (int v = 0; v < V; v++) {
                        const float4 uu = ur[v * LPR];
                        o[v * LPR] = ra.w ? uu : f4_fma(s.c, acca[v], uu);
                    }
                }
                if (rb.x >= 0) {
                    const float4 *ur = ub + (2 * pj + 1) * Q4 + sl;
                    float4 *o = outp + (int64_t)rb.x * Q4 + sl;
#pragma unroll
                    for (int v = 0; v < V; v++) {
                        const float4 uu = ur[v * LPR];
                        o[v * LPR] = rb.w ? uu : f4_fma(s.c, accb[v], uu);
                    }
                }
            } else {
                // sum the SPLIT groups' partials: butterfly over all but the lowest group bit,
                // then one exchange in which even groups keep row a and odd groups row b
#pragma unroll
                for (int off = 8; off >= 2 * LPR; off >>= 1)
#pragma unroll
                    for (int v = 0; v < V; v++) {
                        acca[v] = f4_add(acca[v], f4_shfl_xor(acca[v], off));
                        accb[v] = f4_add(accb[v], f4_shfl_xor(accb[v], off));
                    }
                const bool odd = g & 1;
                float4 mine[V];
#pragma unroll
                for (int v = 0; v < V; v++) {
                    const float4 other = f4_shfl_xor(odd ? acca[v] : accb[v], LPR);
                    mine[v] = f4_add(odd ? accb[v] : acca[v], other);
                }
                const int4 r = odd ? rb : ra;
                if (g < 2 && r.x >= 0) {
                    const float4 *ur = ub + (2 * pj + g) * Q4 + sl;
                    float4 *o = outp + (int64_t)r.x * Q4 + sl;
#pragma unroll
                    for (int v = 0; v < V; v++) {
                        const float4 uu = ur[v * LPR];
                        o[v * LPR] = r.w ? uu : f4_fma(s.c, mine[v], uu);
                    }
                }
            }
        }
        if (n2 < t.ntile) {
            pre.store(t, idsp(b));
            if (b)
                U1 = pre.U;
            else
                U0 = pre.U;
        }
        __syncthreads();
    }
}

// Shared memory of one buffer (offsets in StageArgs).
void stage_layout(const TileOp &t, int F, StageArgs &s)
{
    auto up128 = [](uint32_t b) { return (b + 127u) & ~127u; };
    s.wofs = up128((uint32_t)t.ucap * (uint32_t)F * 4u);
    s.sofs = s.wofs + up128((uint32_t)(t.T / 2) * t.KPP * 8u);
    s.rofs = s.sofs + up128((uint32_t)(t.T / 2) * t.KPP * 2u);
    s.uofs = s.rofs + up128((uint32_t)t.T * 16u);
    s.refofs = s.uofs + up128((uint32_t)t.T * (uint32_t)F * 4u);
    s.idofs = s.refofs + up128((uint32_t)F * 4u);
    s.bufbytes = up128(s.idofs + (uint32_t)(t.ucap + t.T) * 4u);
}

int build_keys(const TileOp &t)
{
    int P = 256;
    while (P < t.T * t.KP) P <<= 1;
    return P;
}

size_t build_smem(const TileOp &t)
{
    return (size_t)2 * build_keys(t) * sizeof(int32_t) + (size_t)t.T * t.KP * (sizeof(float) + sizeof(uint16_t)) + 16;
}

}  // namespace

cudaError_t launch_tile_build(TileOp &t, int64_t rows, const int32_t *order, const int64_t *row_ptr,
                              const int32_t *col, const float *val32, const double *val64, const uint8_t *fixed,
                              int mode, int32_t *cnt, int32_t *cnt2, int *bad, int num_sms, cudaStream_t st)
{
    if (t.T > 256 || (t.T & 1)) return cudaErrorInvalidValue;
    const int P = build_keys(t);
    const size_t smem = build_smem(t);
    cudaError_t e = cudaFuncSetAttribute(tile_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int64_t blocks = t.ntile < (int64_t)num_sms * 8 ? t.ntile : (int64_t)num_sms * 8;
    if (blocks < 1) blocks = 1;
    tile_build_kernel<<<(int)blocks, 256, smem, st>>>(t, rows, order, row_ptr, col, val32, val64, fixed, P, mode, cnt,
                                                     cnt2, bad);
    return cudaGetLastError();
}

size_t tile_stage_smem(const TileOp &t, int F)
{
    StageArgs s{};
    stage_layout(t, F, s);
    return (size_t)2 * s.bufbytes;
}

bool tile_stage_supported(int F) { return F == 4 || F == 8 || F == 16 || F == 32 || F == 64 || F == 128; }

cudaError_t tile_stage_prepare(const TileOp &t, int F)
{
    const int smem = (int)tile_stage_smem(t, F);
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    switch (F) {
    case 4: return cudaFuncSetAttribute(rk4_tile_stage_kernel<4>, a, smem);
    case 8: return cudaFuncSetAttribute(rk4_tile_stage_kernel<8>, a, smem);
    case 16: return cudaFuncSetAttribute(rk4_tile_stage_kernel<16>, a, smem);
    case 32: return cudaFuncSetAttribute(rk4_tile_stage_kernel<32>, a, smem);
    case 64: return cudaFuncSetAttribute(rk4_tile_stage_kernel<64>, a, smem);
    case 128: return cudaFuncSetAttribute(rk4_tile_stage_kernel<128>, a, smem);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_tile_stage(const TileOp &t, const float *v, const float *u, float *out, int F, double c,
                              int num_sms, cudaStream_t st)
{
    if (t.ntile <= 0) return cudaSuccess;
    StageArgs s{};
    s.t = t;
    s.v = v;
    s.u = u;
    s.out = out;
    s.c = (float)c;
    stage_layout(t, F, s);
    const size_t smem = (size_t)2 * s.bufbytes;
    const int blocks = (int)(t.ntile < (int64_t)num_sms ? t.ntile : (int64_t)num_sms);
    switch (F) {
    case 4: rk4_tile_stage_kernel<4><<<blocks, 512, smem, st>>>(s); break;
    case 8: rk4_tile_stage_kernel<8><<<blocks, 512, smem, st>>>(s); break;
    case 16: rk4_tile_stage_kernel<16><<<blocks, 512, smem, st>>>(s); break;
    case 32: rk4_tile_stage_kernel<32><<<blocks, 512, smem, st>>>(s); break;
    case 64: rk4_tile_stage_kernel<64><<<blocks, 512, smem, st>>>(s); break;
    case 128: rk4_tile_stage_kernel<128><<<blocks, 512, smem, st>>>(s); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}
