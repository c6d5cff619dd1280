// Shared declarations of the batched path (batch.cu, batch_tissue.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fpgb_common.cuh"
#include "tissue.cuh"

namespace fpgb {

struct TileDev {
   int64_t vox_base; // first voxel of the tile in the key / label arenas
   int64_t n_vox;
   int32_t X, Y, Z;
   int32_t max_layer;
   int32_t layer_base; // first LayerDev of the tile
   int32_t pad_;
};

// Voxelizer over all tiles of a batch: key pass then write pass (compiled
// with -fmad=false in batch_tissue.cu, like tissue.cu).
int launch_batch_tissue(const SegDev *segs, const int32_t *seg_tile, int64_t n_segs,
                        const TileDev *tiles, int64_t n_tiles, int64_t max_tile_voxels,
                        const LayerDev *layers, unsigned long long *keys, unsigned *min_bundle,
                        int32_t *const *labels, float *const *vecs,
                        unsigned long long *counters, int sms, cudaStream_t st);

} // namespace fpgb
