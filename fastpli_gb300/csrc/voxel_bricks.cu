// Brick-tiled voxelizer (declarations and overview in voxel_bricks.cuh).
//
// Compiled with -fmad=false: the FP64 replay of the reference arithmetic
// (tissue_eval.cuh) must round every product and sum separately, and the
// FP32 estimate of the key passes must be the same in both passes.
//
// Winner keys.  A voxel's key is float_bits(dist^2) << 32 |
// (0xFFFFFFFF - segment): the minimum over every accepted (segment, voxel)
// candidate is the smallest distance, ties going to the LAST segment, which
// is the reference's `>=` overwrite rule (generator.cpp:329-340).  Keys live
// in shared memory for the lifetime of the brick's CTA and are minimised
// with shared-memory atomics.
//
// Two key passes over the brick's segments:
//
//   BOUND  every candidate that is certainly accepted (FP32 estimate plus its
//          bound at or below f_ly_squ * min(r0, r1)^2) stores an upper bound
//          ub of its exact dist^2 as the key ub << 32 | 0xFFFFFFFF, and its
//          bundle in the bundle minimum;
//   EXACT  a candidate whose lower bound exceeds the voxel's current key
//          cannot be the minimum and is skipped; the rest are evaluated with
//          the reference's arithmetic (two-float fast path, FP64 replay) and
//          stored as exact keys.
//
// The true winner w (smallest exact dist^2 among accepted candidates, last
// segment on ties) is never skipped: every stored value is >= its distance
// (an upper bound belongs to an accepted candidate, whose exact distance is
// >= w's), and w's lower bound is <= its own distance.  Candidates tied with
// w are not skipped either, so the tie rule holds.  An upper-bound key is
// >= w's exact key (equal only when w is segment 0: the same value), so the
// final key is w's, bit for bit.  A candidate that the bound filter skips
// but that was not certainly accepted is still decided exactly when the
// bundle minimum is kept (multi-bundle volumes), so that stays exact too.
#include <cuda_runtime.h>

#include <algorithm>

#include "ff.cuh"
#include "fpgb_common.cuh"
#include "tissue.cuh"
#include "tissue_eval.cuh"
#include "voxel_bricks.cuh"

namespace fpgb {

constexpr int kBrickThreads = 256;
constexpr int kBrickWarps = kBrickThreads / 32;
static_assert(kBrickZ == 32, "the write phase maps one lane to one z of a brick row");

void tile_bricks(int64_t X, int64_t Y, int64_t Z, int32_t nb[3], int64_t *n_bricks) {
   nb[0] = (int32_t)((X + kBrickX - 1) / kBrickX);
   nb[1] = (int32_t)((Y + kBrickY - 1) / kBrickY);
   nb[2] = (int32_t)((Z + kBrickZ - 1) / kBrickZ);
   *n_bricks = (int64_t)nb[0] * nb[1] * nb[2];
}

FPGB_HD int64_t brick_range(int lo, int ext, int b, int &b0) {
   b0 = lo / b;
   return ext > 0 ? (lo + ext - 1) / b - b0 + 1 : 0;
}

int64_t segment_brick_pairs(const SegDev &S) {
   int b0;
   return brick_range(S.lo[0], S.ext[0], kBrickX, b0) * brick_range(S.lo[1], S.ext[1], kBrickY, b0) *
          brick_range(S.lo[2], S.ext[2], kBrickZ, b0);
}

size_t brick_workspace_bytes(int64_t n_bricks, int64_t n_pairs) {
   size_t w = 0;
   w += align_up(sizeof(unsigned) * (n_bricks + 1), 256); // offsets
   w += align_up(sizeof(unsigned) * std::max<int64_t>(n_bricks, 1), 256); // counts, then cursors
   w += align_up(sizeof(unsigned) * std::max<int64_t>(n_pairs, 1), 256);  // segment lists
   return w;
}

// ---------------------------------------------------------------- binning ---
template <bool FILL>
__global__ void brick_bin(const SegDev *__restrict__ segs, const int32_t *__restrict__ seg_tile,
                          int64_t n_segs, const TileDev *__restrict__ tiles,
                          unsigned *__restrict__ counts, const unsigned *__restrict__ offsets,
                          unsigned *__restrict__ list, int64_t n_pairs,
                          unsigned long long *__restrict__ counters) {
   for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_segs;
        s += (int64_t)gridDim.x * blockDim.x) {
      const SegDev &S = segs[s];
      const TileDev &T = tiles[seg_tile ? seg_tile[s] : 0];
      int bx0, by0, bz0;
      const int64_t nx = brick_range(S.lo[0], S.ext[0], kBrickX, bx0);
      const int64_t ny = brick_range(S.lo[1], S.ext[1], kBrickY, by0);
      const int64_t nz = brick_range(S.lo[2], S.ext[2], kBrickZ, bz0);
      for (int64_t i = 0; i < nx; i++)
         for (int64_t j = 0; j < ny; j++)
            for (int64_t k = 0; k < nz; k++) {
               const int64_t b =
                   T.brick_base + ((bx0 + i) * T.nb[1] + (by0 + j)) * T.nb[2] + (bz0 + k);
               const unsigned slot = atomicAdd(&counts[b], 1u);
               if (FILL) {
                  const int64_t at = (int64_t)offsets[b] + slot;
                  if (at < offsets[b + 1] && at < n_pairs)
                     list[at] = (unsigned)s;
                  else
                     atomicOr(&counters[6], (unsigned long long)kStatusOverflow);
               }
            }
   }
}

// Exclusive scan of the per-brick counts, one CTA walking the counts in tiles
// of 1024 x 8: each thread loads 8 consecutive counts (two 16-byte loads when
// the tile is whole: the arrays start 256-byte aligned and a thread's first
// index is a multiple of 8), the thread sums are scanned across the block
// (warp shuffles, then the 32 warp sums) and the running total carries from
// tile to tile.  offsets[n] receives the total; a total of 2^32 - 1 or more
// is reported as an overflow of the 32-bit offsets.
constexpr int kScanPer = 8;

__global__ void __launch_bounds__(1024)
brick_scan(const unsigned *__restrict__ counts, int64_t n, unsigned *__restrict__ offsets,
           unsigned long long *__restrict__ counters) {
   __shared__ unsigned long long wsum[32];
   const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
   // the callers' workspaces are 256-byte aligned; checked anyway before any
   // 16-byte access
   const bool vec = (((uintptr_t)counts | (uintptr_t)offsets) & 15) == 0;
   unsigned long long carry = 0; // total of the tiles before this one (the same in every thread)
   for (int64_t base = 0; base < n; base += (int64_t)blockDim.x * kScanPer) {
      const int64_t i0 = base + (int64_t)t * kScanPer;
      unsigned v[kScanPer];
      if (vec && i0 + kScanPer <= n) {
         const uint4 a = *reinterpret_cast<const uint4 *>(counts + i0);
         const uint4 b = *reinterpret_cast<const uint4 *>(counts + i0 + 4);
         v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w;
         v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
      } else {
#pragma unroll
         for (int k = 0; k < kScanPer; k++)
            v[k] = i0 + k < n ? counts[i0 + k] : 0u;
      }
      unsigned long long s = 0;
#pragma unroll
      for (int k = 0; k < kScanPer; k++)
         s += v[k];
      unsigned long long x = s; // inclusive scan over the warp
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
         const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
         if (lane >= o)
            x += y;
      }
      if (lane == 31)
         wsum[wid] = x;
      __syncthreads();
      if (wid == 0) { // inclusive scan of the warp sums
         unsigned long long w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0ull;
#pragma unroll
         for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
               w += y;
         }
         wsum[lane] = w;
      }
      __syncthreads();
      unsigned long long run = carry + (wid ? wsum[wid - 1] : 0ull) + (x - s);
      unsigned o8[kScanPer];
#pragma unroll
      for (int k = 0; k < kScanPer; k++) {
         o8[k] = (unsigned)run;
         run += v[k];
      }
      if (vec && i0 + kScanPer <= n) {
         *reinterpret_cast<uint4 *>(offsets + i0) = make_uint4(o8[0], o8[1], o8[2], o8[3]);
         *reinterpret_cast<uint4 *>(offsets + i0 + 4) = make_uint4(o8[4], o8[5], o8[6], o8[7]);
      } else {
#pragma unroll
         for (int k = 0; k < kScanPer; k++)
            if (i0 + k < n)
               offsets[i0 + k] = o8[k];
      }
      carry += wsum[31];
      __syncthreads(); // wsum is rewritten by the next tile
   }
   if (t == 0) {
      offsets[n] = (unsigned)carry;
      if (carry >= 0xFFFFFFFFull)
         atomicOr(&counters[6], (unsigned long long)kStatusOverflow);
   }
}

// ------------------------------------------------------------ key passes ---
// The inputs of the sweeps of one segment (SegDev offsets 96..175: pf, vf,
// c2f, c2_rcp, thr_f, acc_f, base, lo, ext, bundle) in five 16-byte loads.
struct SegSweep {
   float4 a; // pf[0..2], vf[0]
   float4 b; // vf[1..2], c2f, c2_rcp
   float4 c; // thr_f, acc_f, base[0..1] (int bits)
   int4 d;   // base[2], lo[0..2]
   int4 e;   // ext[0..2], bundle
};

__device__ __forceinline__ SegSweep load_sweep(const SegDev &S) {
   const float4 *f = reinterpret_cast<const float4 *>(&S.pf[0]);
   const int4 *i = reinterpret_cast<const int4 *>(&S.pf[0]);
   return SegSweep{__ldg(f), __ldg(f + 1), __ldg(f + 2), __ldg(i + 3), __ldg(i + 4)};
}

// The part of segment S's clipped box inside the brick (origin o, extent n),
// swept as columns along x: its ey x ez (y, z) cells are numbered z fastest,
// lane l of chunk c owns cell 32 c + l and visits the ex voxels of that
// cell's x column.  The y and z parts of the estimate are computed once per
// cell; each voxel then costs six fused operations (approx_dist2_x).
struct SubBox {
   int x0, y0, z0, ex, ey, ez, ncell;
   float inv_ez; // 1/ez for the division-free cell split
};

__device__ __forceinline__ bool sub_box(const SegSweep &w, int ox, int oy, int oz, int nx,
                                        int ny, int nz, SubBox &b) {
   b.x0 = max(w.d.y, ox);
   b.y0 = max(w.d.z, oy);
   b.z0 = max(w.d.w, oz);
   b.ex = min(w.d.y + w.e.x, ox + nx) - b.x0;
   b.ey = min(w.d.z + w.e.y, oy + ny) - b.y0;
   b.ez = min(w.d.w + w.e.z, oz + nz) - b.z0;
   if (b.ex <= 0 || b.ey <= 0 || b.ez <= 0)
      return false;
   b.ncell = b.ey * b.ez;
   b.inv_ez = __frcp_rn((float)b.ez);
   return true;
}

__device__ __forceinline__ int brick_index(int x, int y, int z, int ox, int oy, int oz) {
   return ((x - ox) * kBrickY + (y - oy)) * kBrickZ + (z - oz);
}

// Per-segment inputs of the FP32 estimate, held in registers over a sweep.
struct SegFP32 {
   float pfx, pfy, pfz, vx, vy, vz, c2f, rc2, thr, acc;
   int bx, by, bz;
};

__device__ __forceinline__ SegFP32 seg_fp32(const SegSweep &w) {
   return SegFP32{w.a.x, w.a.y, w.a.z, w.a.w, w.b.x, w.b.y, w.b.z, w.b.w, w.c.x, w.c.y,
                  __float_as_int(w.c.z), __float_as_int(w.c.w), w.d.x};
}

// A lane's (y, z) cell of a chunk: its brick index at x = x0, and the y / z
// parts of the estimate.  (c + 1/2) / ez lies at least 1/(2 ez) >= 2^-6 from
// an integer for c < 256 and ez <= 32, far beyond the float error of the
// product, so the truncation is the exact quotient.
struct Cell {
   int li;
   float a, b;
};

__device__ __forceinline__ Cell cell_of(const SubBox &b, const SegFP32 &g, int c, int ox, int oy,
                                        int oz) {
   const int iy = (int)(((float)c + 0.5f) * b.inv_ez);
   const int y = b.y0 + iy, z = b.z0 + (c - iy * b.ez);
   // voxel centre - float(p - base): (y - base) + 1/2 is exact in float
   const float wy = ((float)(y - g.by) + 0.5f) - g.pfy;
   const float wz = ((float)(z - g.bz) + 0.5f) - g.pfz;
   return Cell{brick_index(b.x0, y, z, ox, oy, oz), dist2_yz_dot(wy, wz, g.vy, g.vz),
               dist2_yz_len(wy, wz)};
}

// FP32 estimate of the candidate at x offset gx = (x - base) + 1/2 of a
// cell: its dist^2 lies in [lo, hi] (directed rounding of estimate -/+
// bound).
__device__ __forceinline__ void candidate_bounds(const SegFP32 &g, const Cell &c, float gx,
                                                 float &lo, float &hi) {
   float mg;
   const float d2f = approx_dist2_x(gx - g.pfx, c.a, c.b, g.vx, g.c2f, g.rc2, mg);
   lo = __fsub_rd(d2f, mg);
   hi = __fadd_ru(d2f, mg);
}

// BOUND pass of one segment over its sub-box: the upper bound of every
// certainly accepted candidate goes to the voxel's 32-bit bound (a float
// >= 0, so its bits order like the value).  Lanes take cells independently.
template <bool MULTI>
__device__ __forceinline__ void brick_bound(const SegSweep &sw, const SubBox &b, int ox, int oy,
                                            int oz, unsigned *sub, unsigned *sminb, int lane) {
   const SegFP32 g = seg_fp32(sw);
   const unsigned bundle = (unsigned)sw.e.w;
   const float gx0 = (float)(b.x0 - g.bx) + 0.5f;
   for (int c0 = lane; c0 < b.ncell; c0 += 32) {
      const Cell c = cell_of(b, g, c0, ox, oy, oz);
      float gx = gx0;
      int li = c.li;
      for (int i = 0; i < b.ex; i++, gx += 1.f, li += kBrickY * kBrickZ) {
         float lo, hi;
         candidate_bounds(g, c, gx, lo, hi);
         if (hi <= g.acc) {
            atomicMin(&sub[li], __float_as_uint(hi));
            if (MULTI)
               atomicMin(&sminb[li], bundle);
         }
      }
   }
}

// Exact evaluation of one candidate: the two-float path, with the FP64
// replay of the reference arithmetic for the few it leaves undecided.  Out of
// line: one shared copy of these large bodies keeps the sweep loops that call
// them small in the instruction cache.
//
// float(|closest - point|^2) and float(r(t)^2) (generator.cpp:327-328) of
// (S, voxel x y z); returns true when the FP64 replay ran.
__device__ __noinline__ bool cand_dist(const SegDev &S, int x, int y, int z, float &dist_squ,
                                       float &r_sqr) {
   const float lpt[3] = {(float)(x - S.base[0]) + 0.5f, (float)(y - S.base[1]) + 0.5f,
                         (float)(z - S.base[2]) + 0.5f};
   FastCand fc;
   if (S.pscale < 0x1p22f && fast_candidate(S, lpt, fc)) {
      dist_squ = fc.dist_squ;
      r_sqr = fc.r_sqr;
      return false;
   }
   const double pt[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
   double cl[3];
   exact_dist(S, pt, cl, dist_squ, r_sqr);
   return true;
}

// float(vm::unit(point - closest)) of the 'r' layer (generator.cpp:365-371);
// returns true when the FP64 replay ran.
__device__ __noinline__ bool cand_radial(const SegDev &S, int x, int y, int z, float o[3]) {
   const float lpt[3] = {(float)(x - S.base[0]) + 0.5f, (float)(y - S.base[1]) + 0.5f,
                         (float)(z - S.base[2]) + 0.5f};
   FastCand fc;
   if (S.pscale < 0x1p22f && fast_candidate(S, lpt, fc) && fast_radial(S, fc, o))
      return false;
   const double pt[3] = {(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
   double cl[3];
   float d_chk, r_chk;
   exact_dist(S, pt, cl, d_chk, r_chk);
   // unit vector in the reference's double order
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
   return true;
}

// Queue entry flags (bits 0-10: voxel of the brick)
constexpr unsigned short kQueueCertain = 1u << 14;    // certainly accepted
constexpr unsigned short kQueueBundleOnly = 1u << 15; // cannot win; bundle minimum only
constexpr int kQueueCap = 64;

struct WarpQueue {
   unsigned slot[kQueueCap];       // position in the brick's segment list
   unsigned short entry[kQueueCap];
};

// Exact evaluation of one queued candidate (reference arithmetic: two-float
// fast path, FP64 replay) and its atomics.
template <bool MULTI>
__device__ __forceinline__ void brick_eval(const SegDev *__restrict__ segs,
                                           const unsigned *__restrict__ list,
                                           const LayerDev *__restrict__ layers, int layer_base,
                                           unsigned slot, unsigned short e, int ox, int oy, int oz,
                                           unsigned long long *skey, unsigned *sminb,
                                           unsigned long long &n_slow) {
   const unsigned s = list[slot];
   const SegDev &S = segs[s];
   const int li = e & (kBrickVoxels - 1);
   const int x = ox + (li >> 8), y = oy + ((li >> 5) & 7), z = oz + (li & 31);
   float dist_squ, r_sqr;
   if (cand_dist(S, x, y, z, dist_squ, r_sqr))
      n_slow++;
   if (dist_squ > layers[layer_base + S.bundle].f_ly_squ * r_sqr) // generator.cpp:329-331
      return;
   if (!(e & kQueueBundleOnly))
      atomicMin(&skey[li], ((unsigned long long)__float_as_uint(dist_squ) << 32) |
                               (unsigned long long)(0xFFFFFFFFu - s));
   if (MULTI && !(e & kQueueCertain))
      atomicMin(&sminb[li], (unsigned)S.bundle);
}

// EXACT pass, filter side: one segment over its sub-box; candidates that can
// still win (or, for the bundle minimum, might be accepted) go to the warp's
// queue, which is drained 32 entries at a time by all lanes together.
template <bool MULTI>
__device__ __forceinline__ void brick_filter(const SegSweep &sw, unsigned slot, const SubBox &b,
                                             int ox, int oy, int oz, unsigned long long *skey,
                                             WarpQueue &q, int &qn, int lane,
                                             const SegDev *__restrict__ segs,
                                             const unsigned *__restrict__ list,
                                             const LayerDev *__restrict__ layers, int layer_base,
                                             unsigned *sminb, unsigned long long &n_slow) {
   const SegFP32 g = seg_fp32(sw);
   const float gx0 = (float)(b.x0 - g.bx) + 0.5f;
   for (int c0 = 0; c0 < b.ncell; c0 += 32) { // whole warps: the queue is filled by ballot
      const bool in = c0 + lane < b.ncell;
      const Cell c = cell_of(b, g, in ? c0 + lane : 0, ox, oy, oz);
      float gx = gx0;
      int li = c.li;
      for (int i = 0; i < b.ex; i++, gx += 1.f, li += kBrickY * kBrickZ) {
         bool need = false;
         unsigned short e = 0;
         if (in) {
            float lo, hi;
            candidate_bounds(g, c, gx, lo, hi);
            if (!(lo > g.thr)) { // inside the outermost layer at the thickest end
               const bool certain = hi <= g.acc;
               // keys only decrease, so any value read bounds the final one
               // from above; the initial ~0 reads as NaN and skips nothing
               const unsigned long long cur =
                   *reinterpret_cast<volatile unsigned long long *>(&skey[li]);
               const bool loser = lo > __uint_as_float((unsigned)(cur >> 32));
               need = !(loser && (certain || !MULTI));
               e = (unsigned short)(li | (certain ? kQueueCertain : 0) |
                                    (loser ? kQueueBundleOnly : 0));
            }
         }
         const unsigned m = __ballot_sync(0xFFFFFFFFu, need);
         if (need) {
            const int at = qn + __popc(m & ((1u << lane) - 1u));
            q.slot[at] = slot;
            q.entry[at] = e;
         }
         qn += __popc(m);
         if (qn >= 32) { // drain 32 entries with every lane
            __syncwarp();
            const int at = qn - 32 + lane;
            brick_eval<MULTI>(segs, list, layers, layer_base, q.slot[at], q.entry[at], ox, oy,
                              oz, skey, sminb, n_slow);
            qn -= 32;
            __syncwarp();
         }
      }
   }
}

// --------------------------------------------------------- winner decode ---
// Label and orientation of voxel (x, y, z) of a tile from its winner key
// (generator.cpp:343-372): the layer by lower_bound on the squared layer
// scales, the vector by the layer's model ('p' segment direction, 'r'
// radial, 'b' none).
__device__ __forceinline__ void decode_voxel(unsigned long long key, int x, int y, int z,
                                             const SegDev *__restrict__ segs,
                                             const LayerDev *__restrict__ layers,
                                             int layer_base, int max_layer, unsigned minb,
                                             int32_t &label_out, float o[3], bool &defer,
                                             unsigned long long &n_overlap,
                                             unsigned long long &n_overflow,
                                             unsigned long long &n_slow) {
   o[0] = o[1] = o[2] = 0.f;
   defer = false;
   if (key == ~0ull) {
      label_out = 0;
      return;
   }
   const unsigned seg = 0xFFFFFFFFu - (unsigned)(key & 0xFFFFFFFFull);
   const float dist_squ = __uint_as_float((unsigned)(key >> 32));
   const SegDev &S = segs[seg];
   const LayerDev &L = layers[layer_base + S.bundle];
   // With a constant radius whose square rounds the same at every t
   // (rsq_const) and at both ends, r^2 at the winner is known without
   // evaluating the candidate again.
   const bool r_known = S.rsq_const == S.rsq0 && S.rsq_const == S.rsq1; // false for NaN
   float r_sqr = S.rsq_const;
   if (!r_known) {
      float d_chk;
      if (cand_dist(S, x, y, z, d_chk, r_sqr))
         n_slow++;
   }
   // std::lower_bound(scale^2, double(dist_squ / r_sqr)) (generator.cpp:345-349)
   const float qv = dist_squ / r_sqr;
   int ly = 0;
   while (ly < L.n && qv > L.sq_fdown[ly])
      ly++;
   label_out = ly + 1 + S.bundle * max_layer;
   if (minb < (unsigned)S.bundle)
      n_overlap++;
   char m = 'b';
   if (ly < L.n)
      m = L.model[ly];
   else
      n_overflow++;
   if (m == 'p') {
      o[0] = S.vp[0];
      o[1] = S.vp[1];
      o[2] = S.vp[2];
   } else if (m == 'r') { // the caller evaluates it with radial_vector, 32 at a time
      defer = true;
   }
}

// The 'r' orientation of voxel (x, y, z) for winner S: unit(point - closest)
// (generator.cpp:365-371) by the two-float path, FP64 replay when undecided.
__device__ __forceinline__ void radial_vector(const SegDev &S, int x, int y, int z, float o[3],
                                              unsigned long long &n_slow) {
   if (cand_radial(S, x, y, z, o))
      n_slow++;
}

// ------------------------------------------------------------- the brick ---
// 4 resident bricks per SM (64 registers, ~130 bytes of spill): 6% faster
// than 3 on config 2 — the passes are latency-bound and the extra warps hide
// more of it than the spills cost.
template <bool MULTI>
__global__ void __launch_bounds__(kBrickThreads, 4)
voxel_bricks(const SegDev *__restrict__ segs, const TileDev *__restrict__ tiles, int64_t n_tiles,
             int64_t brick_begin, int64_t brick_end, const unsigned *__restrict__ offsets,
             const unsigned *__restrict__ list, unsigned n_pairs,
             const LayerDev *__restrict__ layers,
             int32_t *const *__restrict__ labels, float *const *__restrict__ vecs,
             unsigned long long *__restrict__ counters) {
   __shared__ unsigned long long skey[kBrickVoxels];
   __shared__ unsigned sub[kBrickVoxels]; // BOUND pass: upper bound of the winner's dist^2
   __shared__ unsigned sminb[MULTI ? kBrickVoxels : 1];
   __shared__ WarpQueue queues[kBrickWarps];
   __shared__ unsigned s_next[2]; // next segment of the brick's list, per pass
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   unsigned long long n_slow = 0, n_overlap = 0, n_overflow = 0;

   for (int64_t brick = brick_begin + blockIdx.x; brick < brick_end; brick += gridDim.x) {
      // tile of the brick: last tile whose brick_base <= brick
      int64_t lo = 0, hi = n_tiles - 1;
      while (lo < hi) {
         const int64_t mid = (lo + hi + 1) >> 1;
         if (tiles[mid].brick_base <= brick)
            lo = mid;
         else
            hi = mid - 1;
      }
      const TileDev &T = tiles[lo];
      const int X = T.X, Y = T.Y, Z = T.Z;
      const int64_t lb = brick - T.brick_base;
      const int bz = (int)(lb % T.nb[2]);
      const int64_t rxy = lb / T.nb[2];
      const int by = (int)(rxy % T.nb[1]), bx = (int)(rxy / T.nb[1]);
      const int ox = bx * kBrickX, oy = by * kBrickY, oz = bz * kBrickZ;
      const int nx = min(kBrickX, X - ox), ny = min(kBrickY, Y - oy), nz = min(kBrickZ, Z - oz);
      const int layer_base = T.layer_base, max_layer = T.max_layer;

      for (int i = threadIdx.x; i < kBrickVoxels; i += kBrickThreads) {
         sub[i] = ~0u;
         if (MULTI)
            sminb[i] = ~0u;
      }
      // (clamped to the planned list size: every slot below it is written)
      const unsigned j1 = min(offsets[brick + 1], n_pairs), j0 = min(offsets[brick], j1);
      if (threadIdx.x < 2)
         s_next[threadIdx.x] = 0;
      __syncthreads();
      // BOUND pass: warps take segments from a shared counter
      for (;;) {
         unsigned j = 0;
         if (lane == 0)
            j = atomicAdd(&s_next[0], 1u);
         j = __shfl_sync(0xFFFFFFFFu, j, 0) + j0;
         if (j >= j1)
            break;
         const SegSweep sw = load_sweep(segs[list[j]]);
         SubBox b;
         if (sub_box(sw, ox, oy, oz, nx, ny, nz, b))
            brick_bound<MULTI>(sw, b, ox, oy, oz, sub, sminb, lane);
      }
      __syncthreads();
      // the bounds become the keys ub << 32 | 0xFFFFFFFF the EXACT pass
      // filters against and lowers (no bound: ~0, which reads as NaN)
      for (int i = threadIdx.x; i < kBrickVoxels; i += kBrickThreads)
         skey[i] = sub[i] == ~0u ? ~0ull : ((unsigned long long)sub[i] << 32) | 0xFFFFFFFFull;
      __syncthreads();
      // EXACT pass: warps take segments from a shared counter again
      {
         WarpQueue &q = queues[warp];
         int qn = 0;
         for (;;) {
            unsigned j = 0;
            if (lane == 0)
               j = atomicAdd(&s_next[1], 1u);
            j = __shfl_sync(0xFFFFFFFFu, j, 0) + j0;
            if (j >= j1)
               break;
            const SegSweep sw = load_sweep(segs[list[j]]);
            SubBox b;
            if (sub_box(sw, ox, oy, oz, nx, ny, nz, b))
               brick_filter<MULTI>(sw, j, b, ox, oy, oz, skey, q, qn, lane, segs, list, layers,
                                   layer_base, sminb, n_slow);
         }
         __syncwarp();
         if (lane < qn)
            brick_eval<MULTI>(segs, list, layers, layer_base, q.slot[lane], q.entry[lane], ox, oy,
                              oz, skey, sminb, n_slow);
      }
      __syncthreads();
      // one warp per (x, y) row of the brick, lane = z: coalesced stores.
      // Radial ('r') orientations of winners whose candidate the decode did
      // not evaluate go to the warp's queue and are computed 32 at a time
      // (a warp's row mixes 'b' and 'r' voxels: in place, half the lanes
      // would idle through the two-float unit vector).
      int32_t *label = labels[lo];
      float *vec = vecs[lo];
      WarpQueue &rq = queues[warp];
      int qn = 0;
      auto radial = [&](unsigned short li) {
         const int rx = ox + (li >> 8), ry = oy + ((li >> 5) & 7), rz = oz + (li & 31);
         const unsigned seg = 0xFFFFFFFFu - (unsigned)(skey[li] & 0xFFFFFFFFull);
         float o[3];
         radial_vector(segs[seg], rx, ry, rz, o, n_slow);
         const int64_t i = ((int64_t)rx * Y + ry) * Z + rz;
         vec[3 * i + 0] = o[0];
         vec[3 * i + 1] = o[1];
         vec[3 * i + 2] = o[2];
      };
      for (int r = warp; r < nx * ny; r += kBrickWarps) {
         const int lx = r / ny, ly = r - (r / ny) * ny;
         const int li = (lx * kBrickY + ly) * kBrickZ + lane;
         bool defer = false;
         if (lane < nz) {
            const int x = ox + lx, y = oy + ly, z = oz + lane;
            int32_t lab;
            float o[3];
            decode_voxel(skey[li], x, y, z, segs, layers, layer_base, max_layer,
                         MULTI ? sminb[li] : ~0u, lab, o, defer, n_overlap, n_overflow, n_slow);
            const int64_t i = ((int64_t)x * Y + y) * Z + z;
            label[i] = lab;
            defer = defer && vec;
            if (vec && !defer) {
               vec[3 * i + 0] = o[0];
               vec[3 * i + 1] = o[1];
               vec[3 * i + 2] = o[2];
            }
         }
         const unsigned m = __ballot_sync(0xFFFFFFFFu, defer);
         if (defer)
            rq.entry[qn + __popc(m & ((1u << lane) - 1u))] = (unsigned short)li;
         qn += __popc(m);
         if (qn >= 32) {
            __syncwarp();
            radial(rq.entry[qn - 32 + lane]);
            qn -= 32;
            __syncwarp();
         }
      }
      __syncwarp();
      if (lane < qn)
         radial(rq.entry[lane]);
      __syncthreads(); // shared keys are re-initialised for the next brick
   }
   if (n_overlap)
      atomicAdd(&counters[0], n_overlap);
   if (n_overflow)
      atomicAdd(&counters[5], n_overflow);
   if (n_slow)
      atomicAdd(&counters[9], n_slow);
}

int launch_voxel_bricks(const SegDev *segs, const int32_t *seg_tile, int64_t n_segs,
                        const TileDev *tiles, int64_t n_tiles, int64_t n_bricks, int64_t n_pairs,
                        const LayerDev *layers, bool multi_bundle, int32_t *const *labels,
                        float *const *vecs, void *ws, unsigned long long *counters,
                        cudaStream_t st, const BrickChunks *chunks) {
   if (n_tiles <= 0 || n_bricks <= 0)
      return FPGB_OK;
   if (chunks && (chunks->n < 1 || chunks->bound[0] != 0 || chunks->bound[chunks->n] != n_bricks)) {
      set_error("voxelizer: brick chunks do not cover the bricks");
      return FPGB_EINVAL;
   }
   if (n_pairs >= 0xFFFFFFFFll || n_segs >= 0xFFFFFFFFll) {
      set_error("voxelizer: %lld segment-brick pairs exceed the 32-bit lists",
                (long long)n_pairs);
      return FPGB_EINVAL;
   }
   char *w = static_cast<char *>(ws);
   auto *offsets = reinterpret_cast<unsigned *>(w);
   w += align_up(sizeof(unsigned) * (n_bricks + 1), 256);
   auto *counts = reinterpret_cast<unsigned *>(w);
   w += align_up(sizeof(unsigned) * std::max<int64_t>(n_bricks, 1), 256);
   auto *list = reinterpret_cast<unsigned *>(w);

   FPGB_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(unsigned) * n_bricks, st));
   if (n_segs > 0) {
      const unsigned g = (unsigned)std::min<int64_t>((n_segs + 255) / 256, 1 << 20);
      brick_bin<false><<<g, 256, 0, st>>>(segs, seg_tile, n_segs, tiles, counts, nullptr,
                                          nullptr, n_pairs, counters);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   brick_scan<<<1, 1024, 0, st>>>(counts, n_bricks, offsets, counters);
   FPGB_CUDA_TRY(cudaGetLastError());
   if (n_segs > 0) {
      FPGB_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(unsigned) * n_bricks, st));
      const unsigned g = (unsigned)std::min<int64_t>((n_segs + 255) / 256, 1 << 20);
      brick_bin<true><<<g, 256, 0, st>>>(segs, seg_tile, n_segs, tiles, counts, offsets, list,
                                         n_pairs, counters);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   const int n_launch = chunks ? chunks->n : 1;
   cudaStream_t alt = chunks && chunks->n > 1 ? chunks->alt : nullptr;
   cudaEvent_t joined[2] = {};
   auto launch_all = [&]() -> int {
      if (alt) { // alt starts after the binning
         FPGB_CUDA_TRY(cudaEventCreateWithFlags(&joined[0], cudaEventDisableTiming));
         FPGB_CUDA_TRY(cudaEventRecord(joined[0], st));
         FPGB_CUDA_TRY(cudaStreamWaitEvent(alt, joined[0], 0));
      }
      for (int c = 0; c < n_launch; c++) {
         const int64_t b0 = chunks ? chunks->bound[c] : 0;
         const int64_t b1 = chunks ? chunks->bound[c + 1] : n_bricks;
         cudaStream_t s = (alt && (c & 1)) ? alt : st;
         if (b1 > b0) {
            const unsigned grid = (unsigned)std::min<int64_t>(b1 - b0, 0x7FFFFFFF);
            if (multi_bundle)
               voxel_bricks<true><<<grid, kBrickThreads, 0, s>>>(segs, tiles, n_tiles, b0, b1,
                                                                offsets, list, (unsigned)n_pairs,
                                                                layers, labels, vecs, counters);
            else
               voxel_bricks<false><<<grid, kBrickThreads, 0, s>>>(segs, tiles, n_tiles, b0, b1,
                                                                 offsets, list, (unsigned)n_pairs,
                                                                 layers, labels, vecs, counters);
            FPGB_CUDA_TRY(cudaGetLastError());
         }
         if (chunks && chunks->after)
            FPGB_TRY(chunks->after(chunks->ctx, c, s));
      }
      if (alt) { // st's later work sees every chunk
         FPGB_CUDA_TRY(cudaEventCreateWithFlags(&joined[1], cudaEventDisableTiming));
         FPGB_CUDA_TRY(cudaEventRecord(joined[1], alt));
         FPGB_CUDA_TRY(cudaStreamWaitEvent(st, joined[1], 0));
      }
      return FPGB_OK;
   };
   const int rc = launch_all();
   for (cudaEvent_t e : joined)
      if (e)
         cudaEventDestroy(e);
   return rc;
}

} // namespace fpgb
