// Brick-tiled voxelizer shared by the single-volume path (tissue.cu) and the
// batched path (batch.cu).  Kernels in voxel_bricks.cu (-fmad=false).
//
// The volume (or every tile of a batch) is cut into bricks of
// kBrickX x kBrickY x kBrickZ voxels.  Each segment is binned to the bricks
// its clipped box overlaps (count, scan, fill on the device); one CTA then
// owns one brick: it keeps the brick's 64-bit winner keys
// (float_bits(dist^2) << 32 | (0xFFFFFFFF - segment), see below) and, for
// multi-bundle volumes, the per-voxel bundle minimum in shared memory, runs
// both key passes over the brick's segments, and finally decodes every
// voxel's winner into label and orientation, written once to HBM.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fpgb_common.cuh"
#include "tissue.cuh"

namespace fpgb {

constexpr int kBrickX = 8, kBrickY = 8, kBrickZ = 32;
constexpr int kBrickVoxels = kBrickX * kBrickY * kBrickZ;

// One volume of the voxelizer: a tile of a batch, or the single volume.
struct TileDev {
   int64_t vox_base;   // first voxel of the tile in a batch-wide voxel numbering
   int64_t n_vox;
   int64_t brick_base; // first brick of the tile
   int32_t X, Y, Z;
   int32_t max_layer;
   int32_t layer_base; // first LayerDev of the tile
   int32_t nb[3];      // bricks along x, y, z
};

// Bricks of an X x Y x Z volume along each axis and in total.
void tile_bricks(int64_t X, int64_t Y, int64_t Z, int32_t nb[3], int64_t *n_bricks);

// Number of (segment, brick) pairs of one segment (its clipped box).
int64_t segment_brick_pairs(const SegDev &S);

// Device scratch of the voxelizer for n_bricks bricks and n_pairs pairs.
size_t brick_workspace_bytes(int64_t n_bricks, int64_t n_pairs);

// Brick ranges to voxelize as separate launches, in order: launch c covers
// bricks [bound[c], bound[c + 1]), and after(ctx, c, s) runs on the host once
// it is enqueued on stream s (to queue work that waits for those bricks, e.g.
// the copy of their part of the output).  With `alt` set, odd chunks run on
// alt: launches on one stream each wait for the previous launch's slowest
// brick, and two streams let a chunk's last bricks share the GPU with the
// next chunk's first (the chunks write disjoint outputs).  The stream passed
// to launch_voxel_bricks waits for alt before it returns.
struct BrickChunks {
   int n;
   const int64_t *bound; // n + 1 brick indices, bound[0] = 0, bound[n] = n_bricks
   int (*after)(void *ctx, int chunk, cudaStream_t s);
   void *ctx;
   cudaStream_t alt;
};

// Bins the segments to bricks and voxelizes every tile.  labels[t] / vecs[t]
// are the tile's output arrays (vecs[t] may be null: labels only).
// seg_tile may be null when there is one tile.  `ws` holds
// brick_workspace_bytes(n_bricks, n_pairs) bytes, 256-byte aligned.
// `chunks` may be null: one launch over every brick.
int launch_voxel_bricks(const SegDev *segs, const int32_t *seg_tile, int64_t n_segs,
                        const TileDev *tiles, int64_t n_tiles, int64_t n_bricks, int64_t n_pairs,
                        const LayerDev *layers, bool multi_bundle, int32_t *const *labels,
                        float *const *vecs, void *ws, unsigned long long *counters,
                        cudaStream_t st, const BrickChunks *chunks = nullptr);

} // namespace fpgb
