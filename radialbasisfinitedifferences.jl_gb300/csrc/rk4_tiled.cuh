// Tiled FP32 stencil application of the RK4 stages (rk4_tiled.cu): tile layout and launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// Rows grouped into tiles of T consecutive rows of the RK4 row order (a Z-curve order of the
// nodes).  Per tile: the sorted distinct stencil columns (the union, uptr/uni), and per row KP
// entries (KP = the longest row rounded up to a multiple of 4) as 16-bit slots into the union and FP32
// weights, tile-major and row-major inside the tile; rows shorter than KP are padded with
// their own slot and weight 0.  rowinfo, one 16-byte record per position of the row order
// (padded to ntile * T): x = the row (-1 for padding), y = the bits of the FP32 row sum of the
// FP64 weights, z = the slot of the row's own node in the union, w = 1 for a held row.
struct TileOp {
    int T = 0, KP = 0;
    int64_t ntile = 0;
    int ucap = 0;                    // largest union of a tile
    const int32_t *uptr = nullptr;   // ntile + 1
    int32_t *uni = nullptr;          // uptr[ntile]
    float *w = nullptr;              // ntile * T * KP
    uint16_t *slot = nullptr;        // ntile * T * KP
    int4 *rowinfo = nullptr;         // ntile * T
};

// Dynamic shared memory of the stage kernel (two buffers).
size_t tile_stage_smem(const TileOp &t, int F);
// Field counts the stage kernel takes (F / 4 lanes per row must divide a warp).
bool tile_stage_supported(int F);

// mode 0: cnt[tile] = size of the tile's union (uptr, uni, w, ... unused).  mode 1: fill the
// layout (uptr must hold the exclusive scan of the counts).  bad |= 1 if a row's own node is
// not among its columns, |= 2 if a union exceeds 65535 columns.
cudaError_t launch_tile_build(TileOp &t, int64_t rows, const int32_t *order, const int64_t *row_ptr,
                              const int32_t *col, const float *val32, const double *val64, const uint8_t *fixed,
                              int mode, int32_t *cnt, int *bad, int num_sms, cudaStream_t st);

// Raise the stage kernel's dynamic shared-memory limit for this layout and field count (once,
// before the first launch; launches may then be captured into a CUDA graph).
cudaError_t tile_stage_prepare(const TileOp &t, int F);

// out = u + c (L v) on free rows, out = u on held rows (as built into rowinfo), FP32, F fields
// per row; v, u, out 16-byte aligned, v and u may alias.
cudaError_t launch_tile_stage(const TileOp &t, const float *v, const float *u, float *out, int F, double c,
                              int num_sms, cudaStream_t st);
