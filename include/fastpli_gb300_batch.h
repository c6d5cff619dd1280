/*
 * fastpli_gb300 — batched forward model: many tissue tiles of uneven size,
 * each with its own fiber bundles, layers and tilt set, voxelized and marched
 * by one fixed launch sequence (voxelizer key pass, write pass, one
 * persistent march kernel pulling (tile-tilt, ray block) items from a queue).
 * No counterpart in the reference, which runs one volume and one tilt per
 * call (src/simulation/simulator.cpp:182); every tile's labels, vectors and
 * images are bit-identical to the single-volume entry points of
 * fastpli_gb300.h.
 *
 * Life cycle: create (host planning) -> info/layout (sizes and offsets) ->
 * caller allocates one output arena and one workspace (256-byte aligned) ->
 * upload (tables to the device, binds the buffers) -> run (device work only:
 * no allocation and no host synchronisation, so a stream capture of
 * fpgb_batch_run is a complete CUDA graph of the batch and can be replayed)
 * -> warnings -> destroy.
 */
#ifndef FASTPLI_GB300_BATCH_H_
#define FASTPLI_GB300_BATCH_H_

#include <stddef.h>
#include <stdint.h>

#include "fastpli_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fpgb_batch fpgb_batch;

typedef struct fpgb_batch_sizes {
   int64_t n_tiles;
   int64_t n_pairs;  /* (tile, tilt) pairs */
   int64_t n_items;  /* work items of the persistent march */
   int64_t n_segments;
   int64_t total_voxels;
   int64_t steps;    /* ray-voxel steps of all pairs */
   size_t arena_bytes;     /* outputs: labels, vectors, images (+ epa) */
   size_t workspace_bytes; /* keys, tables, queue */
   size_t upload_bytes;    /* host-to-device bytes of fpgb_batch_upload */
} fpgb_batch_sizes;

/* Tile t: vols[t], fibers[t], background absorption background_mu[t] (props
 * row 0 mu; NULL = 0), tilts[2k], tilts[2k+1] = (theta, phi) for k in
 * [tilt_off[t], tilt_off[t+1]).  One PLI setup for all tiles.  want_epa adds
 * transmittance/direction/retardation per pair.  rays_per_item is reserved
 * (pass 0): work items are 128 rays. */
int fpgb_batch_create(int64_t n_tiles, const fpgb_volume *vols,
                      const fpgb_fibers *fibers, const double *background_mu,
                      const fpgb_setup *setup, const int64_t *tilt_off,
                      const double *tilts, int want_epa, int rays_per_item,
                      fpgb_batch **out);
int fpgb_batch_info(const fpgb_batch *b, fpgb_batch_sizes *info);
/* Byte offsets into the arena: label_off/vector_off [n_tiles],
 * image_off/epa_off [n_pairs] (epa: t, d, r arrays of X*Y doubles each, -1
 * when not requested); n_props [n_tiles].  Any pointer may be NULL. */
int fpgb_batch_layout(const fpgb_batch *b, int64_t *label_off,
                      int64_t *vector_off, int64_t *image_off, int64_t *epa_off,
                      int64_t *n_props);
int fpgb_batch_props(const fpgb_batch *b, int64_t tile, double *props,
                     int64_t props_cap);
int fpgb_batch_upload(fpgb_batch *b, void *d_arena, void *d_workspace,
                      void *stream);
/* Launch configuration: march_ctas_per_sm (<= 0: as many as fit) resident
 * CTAs per SM for the persistent march; items_per_grab (<= 0: 4) work items
 * of 128 rays taken per queue access; march_coop (Lerp/Slerp) 1 = steps that
 * need interpolation are compacted across each warp, 0 = one thread per ray.
 * All three are tuning knobs only (results are bit-identical across them);
 * fastpli_gb300.autotune picks them. */
int fpgb_batch_run(fpgb_batch *b, int march_ctas_per_sm, int items_per_grab,
                   int march_coop, void *stream);
/* Ray-block shape of the march's work items (a tuning knob: results are
 * bit-identical across shapes): 0 = blocks of 128 consecutive rays (x * Y + y
 * order, the default), 1, 2, 3, 4 = rectangles of 2 x 64, 4 x 32, 8 x 16,
 * 16 x 8 rays (x by y).  Replaces the item list on the device when the batch is bound
 * (synchronises the stream).  A CUDA graph captured before must be captured
 * again. */
int fpgb_batch_set_shape(fpgb_batch *b, int shape, void *stream);
/* One stage of fpgb_batch_run: stages = 1 the voxelizer only, 2 the march
 * only (of the volumes the last voxelizer run left in the arena), 3 both
 * (= fpgb_batch_run).  Lets a caller time or overlap the two stages
 * separately; the results are those of fpgb_batch_run. */
int fpgb_batch_run_stages(fpgb_batch *b, int stages, int march_ctas_per_sm,
                          int items_per_grab, int march_coop, void *stream);
/* Synchronises; fails with FPGB_EINVAL when a label was out of range.
 * fp64_replays (may be NULL) counts voxelizer candidates decided in FP64. */
int fpgb_batch_warnings(const fpgb_batch *b, fpgb_warnings *w,
                        int64_t *fp64_replays, void *stream);
int fpgb_batch_destroy(fpgb_batch *b);

#ifdef __cplusplus
}
#endif

#endif /* FASTPLI_GB300_BATCH_H_ */
