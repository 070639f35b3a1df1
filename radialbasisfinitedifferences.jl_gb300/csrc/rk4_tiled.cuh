// Tiled FP32 stencil application of the RK4 stages (rk4_tiled.cu): tile layout and launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// Rows grouped into tiles of T consecutive rows of the RK4 row order (a Z-curve order of the
// nodes), and rows 2j, 2j + 1 of a tile into pair j.  Per tile: the sorted distinct stencil
// columns (the union, uptr/uni); per pair KPP merged entries (KPP = the largest merged count,
// rounded up to a multiple of 4): a 16-bit slot into the union and the two rows' FP32 weights
// for that column (0 where a row does not use it), tile-major, padded with slot 0 and zero
// weights.  rowinfo, one 16-byte record per position of the row order (padded to ntile * T):
// x = the row (-1 for padding), y = the bits of the FP32 row sum of the FP64 weights, z = the
// pair's entry quads (first row of the pair), w = 1 for a held row.  KP: the longest row.
struct TileOp {
    int T = 0, KP = 0, KPP = 0;
    int64_t ntile = 0;
    int ucap = 0;                    // largest union of a tile
    const int32_t *uptr = nullptr;   // ntile + 1
    int32_t *uni = nullptr;          // uptr[ntile]
    float2 *pw = nullptr;            // ntile * T/2 * KPP
    uint16_t *pslot = nullptr;       // ntile * T/2 * KPP
    int4 *rowinfo = nullptr;         // ntile * T
};

// Dynamic shared memory of the stage kernel (two buffers).
size_t tile_stage_smem(const TileOp &t, int F);
// Field counts the stage kernel takes (F / 4 lanes per row must divide a warp).
bool tile_stage_supported(int F);

// mode 0: cnt[tile] = size of the tile's union, cnt2[tile] = its largest merged pair (uptr,
// uni, pw, ... unused).  mode 1: fill the layout (uptr must hold the exclusive scan of the
// counts, KPP the rounded maximum of cnt2).  bad |= 2 if a union exceeds 65535 columns.
cudaError_t launch_tile_build(TileOp &t, int64_t rows, const int32_t *order, const int64_t *row_ptr,
                              const int32_t *col, const float *val32, const double *val64, const uint8_t *fixed,
                              int mode, int32_t *cnt, int32_t *cnt2, int *bad, int num_sms, cudaStream_t st);

// Raise the stage kernel's dynamic shared-memory limit for this layout and field count (once,
// before the first launch; launches may then be captured into a CUDA graph).
cudaError_t tile_stage_prepare(const TileOp &t, int F);

// out = u + c (L v) on free rows, out = u on held rows (as built into rowinfo), FP32, F fields
// per row; v, u, out 16-byte aligned, v and u may alias.
cudaError_t launch_tile_stage(const TileOp &t, const float *v, const float *u, float *out, int F, double c,
                              int num_sms, cudaStream_t st);
