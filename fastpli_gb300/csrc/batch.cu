// Batched forward model: many tissue tiles of uneven size, each with its own
// fibers, layers and tilt set, voxelized and marched by one fixed sequence of
// launches that can be captured once in a CUDA graph and replayed.
//
//   voxelizer     the brick voxelizer (voxel_bricks.cu) over the bricks of
//                 ALL tiles, numbered consecutively; each brick writes its
//                 tile's labels and vectors;
//   batch_march   a persistent kernel: CTAs pull work items (tile-tilt pair,
//                 block of rays) from an atomic counter in cost order until
//                 the queue is empty, and march them with the same per-ray
//                 code as the plain kernel (march_core.cuh).
//
// Every tile is computed with exactly the arithmetic of the single-volume
// path, so a tile's results are bit-identical alone, in any batch, and
// through fpgb_generate_tissue / fpgb_run_simulation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ff.cuh"
#include "fpgb_common.cuh"
#include "march_core.cuh"
#include "raymarch.cuh"
#include "tissue.cuh"
#include "voxel_bricks.cuh"

namespace fpgb {


// A work item: one block of 128 rays of one (tile, tilt) pair.  Its shape is
// a launch parameter the autotuner picks: shape 0 is 128 consecutive rays in
// the ray order x * Y + y (lines along y that wrap to the next x: no idle
// lanes but on the last block of a pair); shape s = 1, 2, 3 is a rectangle
// of 2^s x (128 >> s) rays, x by y, s = 1 .. 4 (neighbouring rays in x share more of the
// 8-corner neighbourhoods of a tilted march; idle lanes where the rectangle
// overhangs the tile; 16 x 8, shape 4, marched the 64-tile mixture 0.7%
// faster than 8 x 16).  ray_begin is the first ray (shape 0) or the
// rectangle's corner ray x0 * Y + y0.
constexpr int kItemShapes = 5;

struct BatchItem {
   int32_t pair;
   int32_t tilted;
   int64_t ray_begin;
   int32_t ray_count; // shape 0: rays of the block
   int32_t x0, y0;    // shape > 0: the rectangle's corner
   int32_t pad_;
};

struct fpgb_batch_impl {
   fpgb_setup setup{};
   std::vector<double> rotations;
   std::vector<TissuePlan> tiles;
   std::vector<TileDev> tile_dev;
   std::vector<size_t> seg_base; // first segment of each tile, n_tiles + 1 entries
   int64_t n_segs = 0;
   RawArray<int32_t> seg_tile;
   std::vector<LayerDev> layers;
   std::vector<MarchPlan> pairs;
   std::vector<int32_t> pair_tile;
   std::vector<BatchItem> items;
   // arena layout (bytes)
   std::vector<size_t> label_off, vector_off, image_off, epa_off;
   size_t arena_bytes = 0;
   // workspace layout (bytes)
   size_t ws_bricks = 0, ws_segs = 0, ws_segtile = 0, ws_layers = 0, ws_tiles = 0, ws_prm = 0,
          ws_items = 0, ws_tables = 0, ws_counters = 0, ws_bytes = 0;
   std::vector<size_t> table_off; // per pair: lut then ztab, relative to ws_tables
   int64_t total_vox = 0, steps = 0;
   int64_t n_bricks = 0, brick_pairs = 0;
   bool any_multi_bundle = false;
   int want_epa = 0;
   // bound buffers
   char *arena = nullptr, *ws = nullptr;
   int rays_per_item = 0;
   int shape = 0;          // ray-block shape of the items (BatchItem)
   size_t max_items = 0;   // items of the shape with the most (sizes ws_items)
   int64_t n_untilted = 0; // items [0, n_untilted) untilted, the rest tilted
   int sms = 1;
   int fit[2][2] = {{1, 1}, {1, 1}}; // resident CTAs per SM: [untilted / tilted][per-thread / coop]
   int fit_columns = 1;               // ... of the columns-only kernel
   bool untilted_columns = true;      // every untilted pair is a vertical column
   bool narrow = true; // every (tile, tilt) pair allows 32-bit index arithmetic
};

// ----------------------------------------------------------------------------
// kernels
// ----------------------------------------------------------------------------
// Persistent march: every CTA loops taking the next item from the queue.
// The loop ends when the counter passes n_items; there is no wait on any
// other CTA or kernel.
static_assert(sizeof(MarchParams) % 16 == 0, "MarchParams is copied as int4");
constexpr int kBatchThreads = 128; // one work item = one CTA-width block of rays

// COLUMNS: every pair of the launch is a vertical column (MarchParams::column,
// the untilted pairs of a batch with step 1): the kernel carries only the
// column path and its few registers (more resident warps for its streaming
// loads; held to 6 CTAs per SM, 80 registers: 0.3% faster than 5 at 92);
// MODE, TILT, COOP and WIDE are then unused.  (A min-blocks bound of 0 leaves
// the other instantiations as compiled without one.)
template <int MODE, bool TILT, bool COOP, bool WIDE, bool COLUMNS = false>
__global__ void __launch_bounds__(128, COLUMNS ? 6 : 0)
batch_march(const MarchParams *__restrict__ prm, const BatchItem *__restrict__ items,
            int64_t n_items, int chunk, unsigned long long *__restrict__ next,
            unsigned long long *__restrict__ counters, int shape) {
   __shared__ unsigned long long s_item;
   // the item's parameter block, staged in shared memory (read like the
   // plain kernel reads its by-value parameters)
   __shared__ __align__(16) MarchParams sP;
   __shared__ CoopScratch scratch[(COOP && !COLUMNS) ? kBatchThreads / 32 : 1];
   int cur = -1;
   for (;;) {
      if (threadIdx.x == 0)
         s_item = atomicAdd(next, (unsigned long long)chunk);
      __syncthreads();
      const unsigned long long it0 = s_item;
      if (it0 >= (unsigned long long)n_items)
         return;
      const unsigned long long it1 = min(it0 + (unsigned long long)chunk,
                                         (unsigned long long)n_items);
      for (unsigned long long it = it0; it < it1; it++) {
         const BatchItem w = items[it];
         if (w.pair != cur) {
            __syncthreads(); // everyone is done with the previous block
            const int4 *src = reinterpret_cast<const int4 *>(prm + w.pair);
            int4 *dst = reinterpret_cast<int4 *>(&sP);
            for (int i = threadIdx.x; i < (int)(sizeof(MarchParams) / 16); i += blockDim.x)
               dst[i] = src[i];
            cur = w.pair;
            __syncthreads();
         }
         int64_t ray;
         bool valid;
         if (shape == 0) {
            ray = w.ray_begin + threadIdx.x;
            valid = (int)threadIdx.x < w.ray_count;
         } else { // 2^shape x (128 >> shape) rectangle, y fastest
            const int dx = (int)threadIdx.x >> (7 - shape);
            const int dy = (int)threadIdx.x & ((kBatchThreads >> shape) - 1);
            const int64_t x = (int64_t)w.x0 + dx, y = (int64_t)w.y0 + dy;
            valid = x < sP.X && y < sP.Y;
            ray = valid ? x * sP.Y + y : w.ray_begin;
         }
         if constexpr (COLUMNS) {
            if (valid)
               march_one_ray_column(sP, ray, sP.label, sP.vec, sP.image, sP.epa_t, sP.epa_d,
                                    sP.epa_r, counters);
         } else if (!TILT && sP.column) {
            if (valid)
               march_one_ray_column(sP, ray, sP.label, sP.vec, sP.image, sP.epa_t, sP.epa_d,
                                    sP.epa_r, counters);
         } else if (MODE == 0 || !COOP) {
            if (valid)
               march_one_ray<MODE, TILT, WIDE>(sP, ray, sP.label, sP.vec, sP.image, sP.epa_t,
                                         sP.epa_d, sP.epa_r, counters);
         } else {
            march_ray_coop<MODE, TILT, WIDE>(sP, ray, valid, sP.label, sP.vec, sP.image, sP.epa_t,
                                       sP.epa_d, sP.epa_r, counters, scratch[threadIdx.x >> 5]);
         }
      }
      __syncthreads(); // s_item is rewritten for the next chunk
   }
}

template <int MODE, bool TILT, bool WIDE>
int batch_march_fit_w(int fit[2]) {
   FPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
       &fit[0], batch_march<MODE, TILT, false, WIDE>, kBatchThreads, 0));
   FPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
       &fit[1], batch_march<MODE, TILT, true, WIDE>, kBatchThreads, 0));
   return FPGB_OK;
}

// resident CTAs per SM of the columns-only kernel
int batch_columns_fit(int *fit) {
   FPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
       fit, batch_march<0, false, false, false, true>, kBatchThreads, 0));
   return FPGB_OK;
}

// The untilted pairs when all of them are columns: the columns-only kernel
// with as many CTAs as are resident.
int launch_batch_columns(const MarchParams *prm, const BatchItem *items, int64_t n_items,
                         unsigned long long *next, unsigned long long *counters, int sms,
                         int fit, int chunk, int shape, cudaStream_t st) {
   if (n_items <= 0)
      return FPGB_OK;
   const int64_t grid = std::min<int64_t>((int64_t)sms * std::max(fit, 1),
                                          (n_items + chunk - 1) / chunk);
   batch_march<0, false, false, false, true><<<(unsigned)grid, kBatchThreads, 0, st>>>(
       prm, items, n_items, chunk, next, counters, shape);
   FPGB_CUDA_TRY(cudaGetLastError());
   return FPGB_OK;
}

template <int MODE, bool TILT>
int batch_march_fit(int fit[2], bool narrow) {
   return narrow ? batch_march_fit_w<MODE, TILT, false>(fit)
                 : batch_march_fit_w<MODE, TILT, true>(fit);
}

template <int MODE, bool TILT>
int launch_batch_march(const MarchParams *prm, const BatchItem *items, int64_t n_items,
                       unsigned long long *next, unsigned long long *counters, int sms,
                       const int fits[2], int ctas_per_sm, int chunk, int coop, bool narrow,
                       int shape, cudaStream_t st) {
   if (n_items <= 0)
      return FPGB_OK;
   const bool cp = MODE != 0 && coop != 0;
   const int fit = fits[cp ? 1 : 0];
   const int per_sm = std::max(1, std::min(ctas_per_sm > 0 ? ctas_per_sm : fit, fit));
   const int64_t grid = std::min<int64_t>((int64_t)sms * per_sm, (n_items + chunk - 1) / chunk);
#define FPGB_BM(C, W)                                                                         \
   batch_march<MODE, TILT, C, W><<<(unsigned)grid, kBatchThreads, 0, st>>>(                    \
       prm, items, n_items, chunk, next, counters, shape)
   if (cp) {
      if (narrow)
         FPGB_BM(true, false);
      else
         FPGB_BM(true, true);
   } else {
      if (narrow)
         FPGB_BM(false, false);
      else
         FPGB_BM(false, true);
   }
#undef FPGB_BM
   FPGB_CUDA_TRY(cudaGetLastError());
   return FPGB_OK;
}

// ----------------------------------------------------------------------------
// host
// ----------------------------------------------------------------------------
namespace {

int sm_count_now() {
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   return sms > 0 ? sms : 1;
}

size_t take(size_t &cursor, size_t bytes) {
   const size_t at = cursor;
   cursor += align_up(std::max<size_t>(bytes, 1), 256);
   return at;
}

// Work items of ray-block shape `shape` (BatchItem), most expensive first
// (rays x steps per ray) in two queues (untilted, then tilted: separate
// kernels), so that the dynamic queue balances well.  A pair's full blocks
// all cost 128 n_z: the pairs are ordered by n_z and their full blocks
// emitted in that order, and the blocks that overhang the tile are merged in
// by cost (no sort over the ~10^6 items of a large batch).
void make_items(fpgb_batch_impl *B, int shape) {
   const int64_t R = B->rays_per_item;
   const int64_t tx = int64_t(1) << shape, ty = R >> shape;
   std::vector<int32_t> order(B->pairs.size());
   for (size_t p = 0; p < order.size(); p++)
      order[p] = (int32_t)p;
   auto tilted = [&](int32_t p) { return B->pairs[p].prm.tilted; };
   auto nz = [&](int32_t p) { return (int64_t)B->pairs[p].prm.n_z; };
   std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
      if (tilted(a) != tilted(b))
         return tilted(a) < tilted(b);
      return nz(a) > nz(b);
   });
   struct Keyed {
      int64_t cost;
      BatchItem it;
   };
   std::vector<Keyed> full[2], part[2];
   for (int32_t p : order) {
      const MarchParams &M = B->pairs[p].prm;
      const int tl = M.tilted ? 1 : 0;
      if (shape == 0) {
         const int64_t rays = M.X * M.Y;
         for (int64_t r0 = 0; r0 < rays; r0 += R) {
            BatchItem it{};
            it.pair = p;
            it.tilted = M.tilted;
            it.ray_begin = r0;
            it.ray_count = (int32_t)std::min<int64_t>(R, rays - r0);
            (it.ray_count == R ? full : part)[tl].push_back({it.ray_count * nz(p), it});
         }
      } else {
         for (int64_t x0 = 0; x0 < M.X; x0 += tx)
            for (int64_t y0 = 0; y0 < M.Y; y0 += ty) {
               BatchItem it{};
               it.pair = p;
               it.tilted = M.tilted;
               it.x0 = (int32_t)x0;
               it.y0 = (int32_t)y0;
               it.ray_begin = x0 * M.Y + y0;
               const int64_t n = std::min(tx, M.X - x0) * std::min(ty, M.Y - y0);
               it.ray_count = (int32_t)n;
               (n == R ? full : part)[tl].push_back({n * nz(p), it});
            }
      }
   }
   auto by_cost = [](const Keyed &a, const Keyed &b) { return a.cost > b.cost; };
   B->items.clear();
   B->items.reserve(full[0].size() + full[1].size() + part[0].size() + part[1].size());
   for (int tl = 0; tl < 2; tl++) {
      std::stable_sort(part[tl].begin(), part[tl].end(), by_cost);
      std::vector<Keyed> merged(full[tl].size() + part[tl].size());
      std::merge(full[tl].begin(), full[tl].end(), part[tl].begin(), part[tl].end(),
                 merged.begin(), by_cost);
      for (const Keyed &k : merged)
         B->items.push_back(k.it);
   }
   B->n_untilted = 0;
   while (B->n_untilted < (int64_t)B->items.size() && !B->items[B->n_untilted].tilted)
      B->n_untilted++;
   B->shape = shape;
}

int plan_batch(int64_t n_tiles, const fpgb_volume *vols, const fpgb_fibers *fibers,
               const double *background_mu, const fpgb_setup *setup, const int64_t *tilt_off,
               const double *tilts, int want_epa, int rays_per_item, fpgb_batch_impl *B) {
   if (n_tiles <= 0 || !vols || !fibers || !tilt_off || !tilts) {
      set_error("batch: empty or null input");
      return FPGB_EINVAL;
   }
   if (n_tiles > 65535) { // the write pass puts tiles on grid.y
      set_error("batch: at most 65535 tiles per batch, got %lld", (long long)n_tiles);
      return FPGB_EINVAL;
   }
   FPGB_TRY(check_setup(setup));
   B->setup = *setup;
   B->rotations.assign(setup->filter_rotations, setup->filter_rotations + setup->n_rho);
   B->setup.filter_rotations = B->rotations.data();
   B->want_epa = want_epa;
   (void)rays_per_item; // items are one CTA wide; fpgb_batch_run groups them
   B->rays_per_item = kBatchThreads;
   B->tiles.resize(n_tiles);
   // tiles are planned in parallel (each plan runs serially inside: nested
   // OpenMP regions get one thread); the first error in tile order wins
   std::vector<int> rc(n_tiles, FPGB_OK);
   std::vector<std::string> err(n_tiles);
#pragma omp parallel for schedule(dynamic, 1)
   for (int64_t t = 0; t < n_tiles; t++) {
      rc[t] = plan_tissue(&vols[t], &fibers[t], &B->tiles[t]);
      if (rc[t] != FPGB_OK)
         err[t] = fpgb_last_error();
   }
   for (int64_t t = 0; t < n_tiles; t++)
      if (rc[t] != FPGB_OK) {
         set_error("%s", err[t].c_str());
         return rc[t];
      }
   int64_t vox = 0;
   std::vector<size_t> seg_base(n_tiles + 1, 0);
   for (int64_t t = 0; t < n_tiles; t++) {
      TissuePlan &P = B->tiles[t];
      if (P.X * P.Y * P.Z >= (int64_t(1) << 32)) {
         set_error("batch: tile %lld has 2^32 voxels or more", (long long)t);
         return FPGB_EINVAL;
      }
      if (background_mu)
         P.props[1] = background_mu[t];
      TileDev T{};
      T.vox_base = vox;
      T.n_vox = P.X * P.Y * P.Z;
      T.brick_base = B->n_bricks;
      int64_t nbr = 0;
      tile_bricks(P.X, P.Y, P.Z, T.nb, &nbr);
      B->n_bricks += nbr;
      B->brick_pairs += P.brick_pairs;
      T.X = (int32_t)P.X;
      T.Y = (int32_t)P.Y;
      T.Z = (int32_t)P.Z;
      T.max_layer = P.max_layer;
      T.layer_base = (int32_t)B->layers.size();
      B->tile_dev.push_back(T);
      seg_base[t + 1] = seg_base[t] + P.segs.size();
      for (int64_t b = 0; b < P.n_bundles; b++)
         B->layers.push_back(P.layers[b]);
      if (P.n_bundles == 0)
         B->layers.push_back(LayerDev{});
      B->any_multi_bundle |= P.n_bundles > 1;
      vox += T.n_vox;
   }
   if (seg_base[n_tiles] > 0xFFFFFFF0ull) {
      set_error("batch: too many segments");
      return FPGB_EINVAL;
   }
   // the tiles keep their own segment tables; the upload places them one
   // after the other (segment s of the batch belongs to the tile whose range
   // [seg_base[t], seg_base[t+1]) holds it)
   B->seg_base = seg_base;
   B->n_segs = (int64_t)seg_base[n_tiles];
   B->seg_tile.reset(seg_base[n_tiles]);
#pragma omp parallel for schedule(dynamic, 1)
   for (int64_t t = 0; t < n_tiles; t++)
      std::fill(B->seg_tile.data() + seg_base[t], B->seg_tile.data() + seg_base[t + 1],
                (int32_t)t);
   B->total_vox = vox;

   // (tile, tilt) pairs and their march plans
   for (int64_t t = 0; t < n_tiles; t++) {
      const TissuePlan &P = B->tiles[t];
      const int64_t dim[3] = {P.X, P.Y, P.Z};
      if (tilt_off[t + 1] < tilt_off[t]) {
         set_error("batch: tilt offsets must not decrease");
         return FPGB_EINVAL;
      }
      for (int64_t k = tilt_off[t]; k < tilt_off[t + 1]; k++) {
         MarchPlan mp;
         FPGB_TRY(plan_march(&B->setup, dim, P.props.data(), (int64_t)P.props.size() / 2,
                             tilts[2 * k], tilts[2 * k + 1], &mp));
         mp.prm.tilted = (mp.prm.rotate || mp.prm.dx_fx != 0 || mp.prm.dy_fx != 0) ? 1 : 0;
         if (!mp.prm.tilted && !mp.prm.column)
            B->untilted_columns = false;
         B->steps += mp.steps;
         B->narrow = B->narrow && march_narrow(mp.prm);
         B->pairs.push_back(std::move(mp));
         B->pair_tile.push_back((int32_t)t);
      }
   }

   // the workspace holds the longest item list of any shape
   for (int sh = 0; sh < kItemShapes; sh++) {
      const int64_t tx = int64_t(1) << sh, ty = (int64_t)B->rays_per_item >> sh;
      size_t n = 0;
      for (const MarchPlan &mp : B->pairs)
         n += sh == 0 ? (size_t)((mp.prm.X * mp.prm.Y + ty - 1) / ty)
                      : (size_t)(((mp.prm.X + tx - 1) / tx) * ((mp.prm.Y + ty - 1) / ty));
      B->max_items = std::max(B->max_items, n);
   }
   make_items(B, 0);

   // output arena: per tile label + vector, per pair image (+ epa)
   size_t a = 0;
   for (int64_t t = 0; t < n_tiles; t++) {
      const int64_t n = B->tile_dev[t].n_vox;
      B->label_off.push_back(take(a, sizeof(int32_t) * n));
      B->vector_off.push_back(take(a, sizeof(float) * 3 * n));
   }
   for (size_t p = 0; p < B->pairs.size(); p++) {
      const MarchParams &M = B->pairs[p].prm;
      B->image_off.push_back(take(a, sizeof(double) * M.X * M.Y * M.n_rho));
      B->epa_off.push_back(want_epa ? take(a, sizeof(double) * 3 * M.X * M.Y) : 0);
   }
   B->arena_bytes = a;

   // workspace
   size_t w = 0;
   B->ws_bricks = take(w, brick_workspace_bytes(B->n_bricks, B->brick_pairs));
   B->ws_segs = take(w, sizeof(SegDev) * B->n_segs);
   B->ws_segtile = take(w, sizeof(int32_t) * B->seg_tile.size());
   B->ws_layers = take(w, sizeof(LayerDev) * B->layers.size());
   B->ws_tiles = take(w, sizeof(TileDev) * B->tile_dev.size() + 2 * sizeof(void *) * n_tiles);
   B->ws_prm = take(w, sizeof(MarchParams) * B->pairs.size());
   B->ws_items = take(w, sizeof(BatchItem) * B->max_items);
   size_t tab = 0;
   for (const MarchPlan &mp : B->pairs) {
      B->table_off.push_back(tab);
      tab += march_table_bytes(mp);
   }
   B->ws_tables = take(w, tab);
   B->ws_counters = take(w, sizeof(unsigned long long) * (kCounterWords + 2));
   B->ws_bytes = w;
   return FPGB_OK;
}

int upload_batch(fpgb_batch_impl *B, void *arena, void *ws, cudaStream_t st) {
   if (!arena || !ws || reinterpret_cast<uintptr_t>(arena) % 256 ||
       reinterpret_cast<uintptr_t>(ws) % 256) {
      set_error("batch: arena and workspace must be non-null and 256-byte aligned");
      return FPGB_EINVAL;
   }
   B->arena = static_cast<char *>(arena);
   B->ws = static_cast<char *>(ws);
   char *W = B->ws;
   for (size_t t = 0; t < B->tiles.size(); t++)
      if (!B->tiles[t].segs.empty())
         FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_segs + sizeof(SegDev) * B->seg_base[t],
                                       B->tiles[t].segs.data(),
                                       sizeof(SegDev) * B->tiles[t].segs.size(),
                                       cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_segtile, B->seg_tile.data(),
                                 sizeof(int32_t) * B->seg_tile.size(), cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_layers, B->layers.data(),
                                 sizeof(LayerDev) * B->layers.size(), cudaMemcpyHostToDevice, st));
   // tile table followed by the per-tile label / vector pointer arrays
   const size_t nt = B->tile_dev.size();
   std::vector<char> tiles(sizeof(TileDev) * nt + 2 * sizeof(void *) * nt);
   std::memcpy(tiles.data(), B->tile_dev.data(), sizeof(TileDev) * nt);
   void **lp = reinterpret_cast<void **>(tiles.data() + sizeof(TileDev) * nt);
   for (size_t t = 0; t < nt; t++) {
      lp[t] = B->arena + B->label_off[t];
      lp[nt + t] = B->arena + B->vector_off[t];
   }
   FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_tiles, tiles.data(), tiles.size(),
                                 cudaMemcpyHostToDevice, st));
   // per-pair parameter blocks with their tables and buffers bound; the
   // pairs' tables are staged on the host and go up in one copy
   std::vector<MarchParams> prm(B->pairs.size());
   size_t tab_bytes = 0;
   for (size_t p = 0; p < B->pairs.size(); p++)
      tab_bytes = std::max(tab_bytes, B->table_off[p] + march_table_bytes(B->pairs[p]));
   std::vector<char> tab(tab_bytes);
   for (size_t p = 0; p < B->pairs.size(); p++) {
      const MarchPlan &mp = B->pairs[p];
      MarchParams M = mp.prm;
      char *tb = W + B->ws_tables + B->table_off[p];
      char *zt = tb + align_up(sizeof(LabelOptics) * mp.lut.size(), 256);
      std::memcpy(tab.data() + B->table_off[p], mp.lut.data(),
                  sizeof(LabelOptics) * mp.lut.size());
      std::memcpy(tab.data() + (zt - (W + B->ws_tables)), mp.ztab.data(),
                  sizeof(ZStep) * mp.ztab.size());
      M.lut = reinterpret_cast<const LabelOptics *>(tb);
      M.ztab = reinterpret_cast<const ZStep *>(zt);
      const int t = B->pair_tile[p];
      M.label = reinterpret_cast<const int32_t *>(B->arena + B->label_off[t]);
      M.vec = reinterpret_cast<const float *>(B->arena + B->vector_off[t]);
      M.image = reinterpret_cast<double *>(B->arena + B->image_off[p]);
      if (B->want_epa) {
         double *e = reinterpret_cast<double *>(B->arena + B->epa_off[p]);
         const int64_t n = M.X * M.Y;
         M.epa_t = e;
         M.epa_d = e + n;
         M.epa_r = e + 2 * n;
      } else {
         M.epa_t = M.epa_d = M.epa_r = nullptr;
      }
      prm[p] = M;
   }
   if (tab_bytes)
      FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_tables, tab.data(), tab_bytes,
                                    cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_prm, prm.data(), sizeof(MarchParams) * prm.size(),
                                 cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(W + B->ws_items, B->items.data(),
                                 sizeof(BatchItem) * B->items.size(), cudaMemcpyHostToDevice, st));
   // host staging vectors must outlive the asynchronous copies
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   // device queries happen here, so that fpgb_batch_run issues stream work only
   B->sms = sm_count_now();
   switch (B->setup.interpolate) {
   case 0:
      FPGB_TRY((batch_march_fit<0, false>(B->fit[0], B->narrow)));
      FPGB_TRY((batch_march_fit<0, true>(B->fit[1], B->narrow)));
      break;
   case 1:
      FPGB_TRY((batch_march_fit<1, false>(B->fit[0], B->narrow)));
      FPGB_TRY((batch_march_fit<1, true>(B->fit[1], B->narrow)));
      break;
   default:
      FPGB_TRY((batch_march_fit<2, false>(B->fit[0], B->narrow)));
      FPGB_TRY((batch_march_fit<2, true>(B->fit[1], B->narrow)));
      break;
   }
   FPGB_TRY(batch_columns_fit(&B->fit_columns));
   return FPGB_OK;
}


// All device work of one batch: no allocation, no host synchronisation, so
// a stream capture of this call is a complete graph of the batch.  stages:
// bit 0 the voxelizer, bit 1 the march (which reads the voxelizer's output).
int run_batch(fpgb_batch_impl *B, int march_ctas_per_sm, int chunk, int coop, cudaStream_t st,
              int stages = 3) {
   if (!B->arena || !B->ws) {
      set_error("batch: buffers not bound (call fpgb_batch_upload first)");
      return FPGB_EINVAL;
   }
   char *W = B->ws;
   auto *segs = reinterpret_cast<const SegDev *>(W + B->ws_segs);
   auto *seg_tile = reinterpret_cast<const int32_t *>(W + B->ws_segtile);
   auto *layers = reinterpret_cast<const LayerDev *>(W + B->ws_layers);
   auto *tiles = reinterpret_cast<const TileDev *>(W + B->ws_tiles);
   const size_t nt = B->tile_dev.size();
   auto *lptr = reinterpret_cast<int32_t *const *>(W + B->ws_tiles + sizeof(TileDev) * nt);
   auto *vptr = reinterpret_cast<float *const *>(W + B->ws_tiles + sizeof(TileDev) * nt +
                                                 sizeof(void *) * nt);
   auto *prm = reinterpret_cast<const MarchParams *>(W + B->ws_prm);
   auto *items = reinterpret_cast<const BatchItem *>(W + B->ws_items);
   auto *counters = reinterpret_cast<unsigned long long *>(W + B->ws_counters);
   unsigned long long *next = counters + kCounterWords;

   if (stages & 1) {
      FPGB_CUDA_TRY(cudaMemsetAsync(counters, 0,
                                    sizeof(unsigned long long) * (kCounterWords + 2), st));
      FPGB_TRY(launch_voxel_bricks(segs, seg_tile, B->n_segs, tiles, (int64_t)nt,
                                   B->n_bricks, B->brick_pairs, layers, B->any_multi_bundle,
                                   lptr, vptr, W + B->ws_bricks, counters, st));
   } else {
      // the march's queue counters only: the voxelizer's warnings stay
      FPGB_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(unsigned long long) * 2, st));
   }
   if (!(stages & 2))
      return FPGB_OK;
   const int64_t n0 = B->n_untilted, n1 = (int64_t)B->items.size() - B->n_untilted;
   const int ch = chunk > 0 ? chunk : 4;
#define FPGB_BATCH_MARCH(M)                                                                    \
   if (B->untilted_columns)                                                                    \
      FPGB_TRY(launch_batch_columns(prm, items, n0, next, counters, B->sms, B->fit_columns,    \
                                    ch, B->shape, st));                                        \
   else                                                                                        \
      FPGB_TRY((launch_batch_march<M, false>(prm, items, n0, next, counters, B->sms,           \
                                             B->fit[0], march_ctas_per_sm, ch, coop,           \
                                             B->narrow, B->shape, st)));                       \
   FPGB_TRY((launch_batch_march<M, true>(prm, items + n0, n1, next + 1, counters, B->sms,      \
                                         B->fit[1], march_ctas_per_sm, ch, coop, B->narrow,    \
                                         B->shape, st)))
   switch (B->setup.interpolate) {
   case 0: FPGB_BATCH_MARCH(0); break;
   case 1: FPGB_BATCH_MARCH(1); break;
   default: FPGB_BATCH_MARCH(2); break;
   }
#undef FPGB_BATCH_MARCH
   return FPGB_OK;
}

} // namespace
} // namespace fpgb

using namespace fpgb;

struct fpgb_batch : fpgb_batch_impl {};

extern "C" {

int fpgb_batch_create(int64_t n_tiles, const fpgb_volume *vols, const fpgb_fibers *fibers,
                      const double *background_mu, const fpgb_setup *setup,
                      const int64_t *tilt_off, const double *tilts, int want_epa,
                      int rays_per_item, fpgb_batch **out) {
   if (!out) {
      set_error("batch: null output handle");
      return FPGB_EINVAL;
   }
   *out = nullptr;
   std::unique_ptr<fpgb_batch> B(new fpgb_batch());
   FPGB_TRY(plan_batch(n_tiles, vols, fibers, background_mu, setup, tilt_off, tilts, want_epa,
                       rays_per_item, B.get()));
   *out = B.release();
   return FPGB_OK;
}

int fpgb_batch_info(const fpgb_batch *b, fpgb_batch_sizes *info) {
   if (!b || !info) {
      set_error("batch: null argument");
      return FPGB_EINVAL;
   }
   info->n_tiles = (int64_t)b->tiles.size();
   info->n_pairs = (int64_t)b->pairs.size();
   info->n_items = (int64_t)b->items.size();
   info->n_segments = b->n_segs;
   info->total_voxels = b->total_vox;
   info->steps = b->steps;
   info->arena_bytes = b->arena_bytes;
   info->workspace_bytes = b->ws_bytes;
   size_t up = sizeof(SegDev) * b->n_segs + sizeof(int32_t) * b->seg_tile.size() +
               sizeof(LayerDev) * b->layers.size() +
               (sizeof(TileDev) + 2 * sizeof(void *)) * b->tile_dev.size() +
               sizeof(MarchParams) * b->pairs.size() + sizeof(BatchItem) * b->items.size();
   for (const MarchPlan &mp : b->pairs)
      up += sizeof(LabelOptics) * mp.lut.size() + sizeof(ZStep) * mp.ztab.size();
   info->upload_bytes = up;
   return FPGB_OK;
}

int fpgb_batch_layout(const fpgb_batch *b, int64_t *label_off, int64_t *vector_off,
                      int64_t *image_off, int64_t *epa_off, int64_t *n_props) {
   if (!b) {
      set_error("batch: null handle");
      return FPGB_EINVAL;
   }
   for (size_t t = 0; t < b->tiles.size(); t++) {
      if (label_off)
         label_off[t] = (int64_t)b->label_off[t];
      if (vector_off)
         vector_off[t] = (int64_t)b->vector_off[t];
      if (n_props)
         n_props[t] = (int64_t)b->tiles[t].props.size() / 2;
   }
   for (size_t p = 0; p < b->pairs.size(); p++) {
      if (image_off)
         image_off[p] = (int64_t)b->image_off[p];
      if (epa_off)
         epa_off[p] = b->want_epa ? (int64_t)b->epa_off[p] : -1;
   }
   return FPGB_OK;
}

int fpgb_batch_props(const fpgb_batch *b, int64_t tile, double *props, int64_t props_cap) {
   if (!b || tile < 0 || tile >= (int64_t)b->tiles.size() || !props) {
      set_error("batch: bad tile or buffer");
      return FPGB_EINVAL;
   }
   const std::vector<double> &p = b->tiles[tile].props;
   if (props_cap < (int64_t)p.size() / 2) {
      set_error("batch: props_cap too small");
      return FPGB_EINVAL;
   }
   std::memcpy(props, p.data(), sizeof(double) * p.size());
   return FPGB_OK;
}

int fpgb_batch_upload(fpgb_batch *b, void *d_arena, void *d_workspace, void *stream) {
   if (!b) {
      set_error("batch: null handle");
      return FPGB_EINVAL;
   }
   return upload_batch(b, d_arena, d_workspace, as_stream(stream));
}

int fpgb_batch_run(fpgb_batch *b, int march_ctas_per_sm, int items_per_grab, int march_coop,
                   void *stream) {
   if (!b) {
      set_error("batch: null handle");
      return FPGB_EINVAL;
   }
   return run_batch(b, march_ctas_per_sm, items_per_grab, march_coop, as_stream(stream));
}

int fpgb_batch_set_shape(fpgb_batch *b, int shape, void *stream) {
   if (!b || shape < 0 || shape >= kItemShapes) {
      set_error("batch: null handle or ray-block shape not in 0..%d", kItemShapes - 1);
      return FPGB_EINVAL;
   }
   if (shape == b->shape)
      return FPGB_OK;
   make_items(b, shape);
   if (b->ws) { // bound: replace the device's item list
      cudaStream_t st = as_stream(stream);
      FPGB_CUDA_TRY(cudaMemcpyAsync(b->ws + b->ws_items, b->items.data(),
                                    sizeof(BatchItem) * b->items.size(), cudaMemcpyHostToDevice,
                                    st));
      FPGB_CUDA_TRY(cudaStreamSynchronize(st)); // the host list may change again
   }
   return FPGB_OK;
}

int fpgb_batch_run_stages(fpgb_batch *b, int stages, int march_ctas_per_sm, int items_per_grab,
                          int march_coop, void *stream) {
   if (!b || stages < 1 || stages > 3) {
      set_error("batch: null handle or stages not in 1..3");
      return FPGB_EINVAL;
   }
   return run_batch(b, march_ctas_per_sm, items_per_grab, march_coop, as_stream(stream), stages);
}

int fpgb_batch_warnings(const fpgb_batch *b, fpgb_warnings *w, int64_t *fp64_replays,
                        void *stream) {
   if (!b || !b->ws) {
      set_error("batch: buffers not bound");
      return FPGB_EINVAL;
   }
   cudaStream_t st = as_stream(stream);
   unsigned long long h[kCounterWords];
   FPGB_CUDA_TRY(cudaMemcpyAsync(h, b->ws + b->ws_counters, sizeof h, cudaMemcpyDeviceToHost, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   if (h[6] & kStatusLabelRange) {
      set_error("batch: label out of range");
      return FPGB_EINVAL;
   }
   if (h[6] & kStatusOverflow) { // the device binning disagreed with the host plan
      set_error("batch: internal error, segment-brick lists overflowed");
      return FPGB_ECUDA;
   }
   if (w) {
      warnings_from_counters(reinterpret_cast<const long long *>(h), w);
      w->overlap = w->overlap > 0 ? 1 : 0;
      int64_t sp = 0;
      for (const TissuePlan &t : b->tiles)
         sp += t.single_point;
      w->single_point = sp;
   }
   if (fp64_replays)
      *fp64_replays = (int64_t)h[9];
   return FPGB_OK;
}

int fpgb_batch_destroy(fpgb_batch *b) {
   delete b;
   return FPGB_OK;
}

} // extern "C"
