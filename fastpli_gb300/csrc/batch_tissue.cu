// Voxelizer kernels of the batched path.  Compiled with -fmad=false: the
// FP64 replay of the reference arithmetic (tissue_eval.cuh) must round every
// product and sum separately.  See batch.cu for the batch as a whole.
#include <cuda_runtime.h>

#include <algorithm>

#include "batch.cuh"
#include "ff.cuh"
#include "fpgb_common.cuh"
#include "tissue.cuh"
#include "tissue_eval.cuh"

namespace fpgb {

__global__ void __launch_bounds__(128)
batch_keys(const SegDev *__restrict__ segs, const int32_t *__restrict__ seg_tile,
           int64_t n_segs, const TileDev *__restrict__ tiles,
           const LayerDev *__restrict__ layers, unsigned long long *__restrict__ keys,
           unsigned *__restrict__ min_bundle, unsigned long long *__restrict__ counters) {
   unsigned long long n_slow = 0;
   for (int64_t s = blockIdx.x; s < n_segs; s += gridDim.x) {
      const SegDev &S = segs[s];
      const TileDev T = tiles[seg_tile[s]];
      const float f_ly = layers[T.layer_base + S.bundle].f_ly_squ;
      const int ex = S.ext[0], ey = S.ext[1], ez = S.ext[2];
      const int plane = ey * ez;
      const unsigned long long inv_idx = (unsigned long long)(0xFFFFFFFFu - (unsigned)s);
      const float vfx = S.vf[0], vfy = S.vf[1], vfz = S.vf[2];
      const float c2f = S.c2f;
      const bool fast_ok = S.pscale < 0x1p22f;
      for (int pl = threadIdx.x; pl < plane; pl += blockDim.x) {
         const int iy = pl / ez, iz = pl - (pl / ez) * ez;
         const int y = S.lo[1] + iy, z = S.lo[2] + iz;
         const float ly = (float)(y - S.base[1]) + 0.5f;
         const float lz = (float)(z - S.base[2]) + 0.5f;
         const float wy = ly - S.pf[1];
         const float wz = lz - S.pf[2];
         FastRow row;
         if (fast_ok)
            fast_row(S, ly, lz, row);
         for (int ix = 0; ix < ex; ix++) {
            const int x = S.lo[0] + ix;
            const float lx = (float)(x - S.base[0]) + 0.5f;
            const float wx = lx - S.pf[0];
            const float c1f = wx * vfx + wy * vfy + wz * vfz;
            const float w2 = wx * wx + wy * wy + wz * wz;
            float d2f;
            if (c1f <= 0.f) {
               d2f = w2;
            } else if (c1f >= c2f) {
               const float ux = wx - vfx, uy = wy - vfy, uz = wz - vfz;
               d2f = ux * ux + uy * uy + uz * uz;
            } else {
               d2f = w2 - c1f * (c1f / c2f);
            }
            if (d2f - (1e-4f + 3.8e-6f * (w2 + c2f)) > S.thr_f)
               continue;
            float dist_squ, r_sqr;
            FastCand fc;
            if (fast_ok && fast_candidate_row(S, lx, row, fc)) {
               dist_squ = fc.dist_squ;
               r_sqr = fc.r_sqr;
            } else {
               const double pt[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
               double cl[3];
               exact_dist(S, pt, cl, dist_squ, r_sqr);
               n_slow++;
            }
            if (dist_squ > f_ly * r_sqr)
               continue;
            const int64_t ind = T.vox_base + ((int64_t)x * T.Y + y) * T.Z + z;
            atomicMin(&keys[ind], ((unsigned long long)__float_as_uint(dist_squ) << 32) | inv_idx);
            if (min_bundle)
               atomicMin(&min_bundle[ind], (unsigned)S.bundle);
         }
      }
   }
   if (n_slow)
      atomicAdd(&counters[9], n_slow);
}

__global__ void __launch_bounds__(256, 3)
batch_write(const unsigned long long *__restrict__ keys, const SegDev *__restrict__ segs,
            const TileDev *__restrict__ tiles, const LayerDev *__restrict__ layers,
            int32_t *const *__restrict__ labels, float *const *__restrict__ vecs,
            const unsigned *__restrict__ min_bundle,
            unsigned long long *__restrict__ counters) {
   const TileDev T = tiles[blockIdx.y];
   int32_t *label = labels[blockIdx.y];
   float *vec = vecs[blockIdx.y];
   const unsigned *minb = min_bundle ? min_bundle + T.vox_base : nullptr;
   const unsigned long long *key = keys + T.vox_base;
   unsigned long long n_overflow = 0, n_overlap = 0, n_slow = 0;
   // one warp per (x, y) row of the tile, lanes along z
   const int lane = threadIdx.x & 31;
   const int64_t n_rows = (int64_t)T.X * T.Y;
   const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
   for (int64_t row = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); row < n_rows;
        row += warps) {
   const int x = (int)(row / T.Y), y = (int)(row - (row / T.Y) * T.Y);
   for (int z = lane; z < T.Z; z += 32) {
      const int64_t i = row * T.Z + z;
      const unsigned long long k = key[i];
      if (k == ~0ull) {
         label[i] = 0;
         vec[3 * i + 0] = 0.f;
         vec[3 * i + 1] = 0.f;
         vec[3 * i + 2] = 0.f;
         continue;
      }
      const unsigned seg = 0xFFFFFFFFu - (unsigned)(k & 0xFFFFFFFFull);
      const float dist_squ = __uint_as_float((unsigned)(k >> 32));
      const SegDev &S = segs[seg];
      const LayerDev &L = layers[T.layer_base + S.bundle];
      const float lpt[3] = {(float)(x - S.base[0]) + 0.5f, (float)(y - S.base[1]) + 0.5f,
                            (float)(z - S.base[2]) + 0.5f};
      FastCand fc;
      const bool fast = S.pscale < 0x1p22f && fast_candidate(S, lpt, fc);
      float r_sqr = fc.r_sqr;
      double cl[3];
      if (!fast) {
         const double pt[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
         float d_chk;
         exact_dist(S, pt, cl, d_chk, r_sqr);
      }
      const float qv = dist_squ / r_sqr;
      int ly = 0;
      while (ly < L.n && qv > L.sq_fdown[ly])
         ly++;
      label[i] = ly + 1 + S.bundle * T.max_layer;
      if (minb && minb[i] < (unsigned)S.bundle)
         n_overlap++;
      char m = 'b';
      if (ly < L.n)
         m = L.model[ly];
      else
         n_overflow++;
      float o[3] = {0.f, 0.f, 0.f};
      if (m == 'p') {
         o[0] = S.vp[0];
         o[1] = S.vp[1];
         o[2] = S.vp[2];
      } else if (m == 'r') {
         if (!(fast && fast_radial(S, fc, o))) {
            const double pt[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
            if (fast) {
               float d_chk, r_chk;
               exact_dist(S, pt, cl, d_chk, r_chk);
            }
            n_slow++;
            double nv[3] = {pt[0] - cl[0], pt[1] - cl[1], pt[2] - cl[2]};
            double n2 = 0.0;
            n2 = n2 + nv[0] * nv[0];
            n2 = n2 + nv[1] * nv[1];
            n2 = n2 + nv[2] * nv[2];
            if (n2 > 0) {
               const double inv = 1.0 / sqrt(n2);
               nv[0] = nv[0] * inv;
               nv[1] = nv[1] * inv;
               nv[2] = nv[2] * inv;
            }
            o[0] = (float)nv[0];
            o[1] = (float)nv[1];
            o[2] = (float)nv[2];
         }
      }
      vec[3 * i + 0] = o[0];
      vec[3 * i + 1] = o[1];
      vec[3 * i + 2] = o[2];
   }
   }
   if (n_overlap)
      atomicAdd(&counters[0], n_overlap);
   if (n_overflow)
      atomicAdd(&counters[5], n_overflow);
   if (n_slow)
      atomicAdd(&counters[9], n_slow);
}

int launch_batch_tissue(const SegDev *segs, const int32_t *seg_tile, int64_t n_segs,
                        const TileDev *tiles, int64_t n_tiles, int64_t max_tile_voxels,
                        const LayerDev *layers, unsigned long long *keys, unsigned *min_bundle,
                        int32_t *const *labels, float *const *vecs,
                        unsigned long long *counters, int sms, cudaStream_t st) {
   if (n_segs > 0) {
      batch_keys<<<(unsigned)std::min<int64_t>(n_segs, 1 << 30), 128, 0, st>>>(
          segs, seg_tile, n_segs, tiles, layers, keys, min_bundle, counters);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   if (n_tiles > 0) {
      (void)max_tile_voxels;
      const unsigned gx = (unsigned)std::max<int64_t>(1, (int64_t)sms * 12 / n_tiles + 1);
      dim3 grid(gx, (unsigned)n_tiles);
      batch_write<<<grid, 256, 0, st>>>(keys, segs, tiles, layers, labels, vecs, min_bundle,
                                        counters);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   return FPGB_OK;
}

} // namespace fpgb
