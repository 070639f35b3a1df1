// Tiled FP32 stencil application of the RK4 stages (rk4_tiled.cu): tile layout and launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// Rows grouped into tiles of T = 64 consecutive rows of the RK4 row order (a Z-curve order of
// the nodes), each tile into 8 groups of G = 8 consecutive rows.  Per tile: the sorted distinct
// stencil columns (the union, uptr/uni).  Per group: its distinct columns as positions of their
// field rows in the tile's staged union (gslot = slot * F, sorted, padded with slot 0 to a
// multiple of 4) and, for each of them,
// the FP32 weights of the group's 8 rows (gw, 8 floats per column, 0 where a row does not use
// the column).  gptr[ntile * 8 + 1]: the groups' first columns, consecutive groups adjacent.
// rowinfo, one 16-byte record per position of the row order (padded to ntile * T): x = the row
// (-1 for padding), y = the bits of the FP32 row sum of the FP64 weights, z = 0, w = 1 for a
// held row.  KP: the longest row; ucap: the largest union; gcap: the most group columns of a
// tile.
struct TileOp {
// Rows per tile (8 per group, one group per warp).  2048^2 nodes, 64 fields: 5.35 / 5.02 /
// 5.91 ms per step at 32 / 64 / 128.
#ifndef RBFFD_TILE_ROWS
#define RBFFD_TILE_ROWS 64
#endif
    static constexpr int T = RBFFD_TILE_ROWS, G = 8;
    int F = 0;  // fields per row (the staged union rows' stride)
    int KP = 0;
    int64_t ntile = 0;
    int ucap = 0, gcap = 0;
    const int32_t *uptr = nullptr;   // ntile + 1
    int32_t *uni = nullptr;          // uptr[ntile]
    const int32_t *gptr = nullptr;   // ntile * T / G + 1
    uint32_t *gslot = nullptr;       // gptr[last]
    float *gw = nullptr;             // 8 * gptr[last]
    int4 *rowinfo = nullptr;         // ntile * T
    int ctas_per_sm = 0;             // stage CTAs resident per SM (set by tile_stage_prepare)
};

// Dynamic shared memory of the stage kernel's CTA.
size_t tile_stage_smem(const TileOp &t, int F);
// Field counts the stage kernel takes.
bool tile_stage_supported(int F);

// mode 0: cnt[tile] = size of the tile's union, gcnt[tile * 8 + g] = group g's column count
// (a multiple of 4); the layout's arrays are not touched.  mode 1: fill the layout (uptr and
// gptr must hold the exclusive scans of the counts).
cudaError_t launch_tile_build(TileOp &t, int64_t rows, const int32_t *order, const int64_t *row_ptr,
                              const int32_t *col, const float *val32, const double *val64, const uint8_t *fixed,
                              int mode, int32_t *cnt, int32_t *gcnt, int num_sms, cudaStream_t st);

// Raise the stage kernel's dynamic shared-memory limit for this layout and field count and
// record its CTAs per SM in t (once, before the first launch; launches may then be captured
// into a CUDA graph).
cudaError_t tile_stage_prepare(TileOp &t, int F);

// out = u + c (L v) on free rows, out = u on held rows (as built into rowinfo), FP32, F fields
// per row; v, u, out 16-byte aligned, v and u may alias.
cudaError_t launch_tile_stage(const TileOp &t, const float *v, const float *u, float *out, int F, double c,
                              int num_sms, cudaStream_t st);
