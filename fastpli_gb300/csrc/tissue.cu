// Voxelizer: fiber polylines -> int32 label field + float32 orientation field.
//
// Replaces PliGenerator::RunTissueGeneration / FillVoxelsAroundFiberSegment
// (src/simulation/generator.cpp:163-383, 475-526).  The reference walks every
// segment in order and overwrites a voxel when `dist[ind] >= dist_squ`
// (generator.cpp:343), so the final owner of a voxel is the segment with the
// smallest float distance and, among equal distances, the LAST one in
// processing order.  Here every (segment, voxel) candidate is independent:
//
//   binning       every segment's clipped bounding box is binned to the
//                 8 x 8 x 32 voxel bricks it overlaps;
//   voxel_bricks  one CTA per brick keeps the brick's 64-bit keys
//                 (float bits of dist_squ) << 32 | (0xFFFFFFFF - seg), i.e.
//                 smallest distance, then largest segment index, in shared
//                 memory: a first sweep stores FP32 upper bounds of the
//                 candidates certainly inside, a second the exact
//                 double->float distance of the reference for every
//                 candidate that can still win; then it decodes each
//                 voxel's winner and writes its label and orientation
//                 (voxel_bricks.cu).
//
// This translation unit is compiled with -fmad=false: the label and vector
// decisions depend on separately rounded double products and sums
// (generator.cpp:324-349, vemath.hpp:342-344,390-402), which a fused
// multiply-add would change.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "ff.cuh"
#include "fpgb_common.cuh"
#include "tissue.cuh"
#include "tissue_eval.cuh"
#include "voxel_bricks.cuh"

namespace fpgb {

// ======================================================================
// host planning (double precision, reference operation order)
// ======================================================================
namespace {

struct Box {
   double mn[3], mx[3];
   void empty() {
      for (int i = 0; i < 3; i++) {
         mn[i] = INFINITY;
         mx[i] = -INFINITY;
      }
   }
   // aabb::AABB(p, q) unsorted constructor (aabb.hpp:54-71)
   void from_pq(const double *p, const double *q) {
      for (int i = 0; i < 3; i++) {
         if (p[i] < q[i]) {
            mn[i] = p[i];
            mx[i] = q[i];
         } else {
            mn[i] = q[i];
            mx[i] = p[i];
         }
      }
   }
   void unite(const Box &a) { // aabb.hpp:90-97
      for (int i = 0; i < 3; i++) {
         if (a.mn[i] < mn[i])
            mn[i] = a.mn[i];
         if (a.mx[i] > mx[i])
            mx[i] = a.mx[i];
      }
   }
};

bool overlap(const Box &a, const Box &b) { // aabb.hpp:128-137
   for (int i = 0; i < 3; i++)
      if (a.mn[i] >= b.mx[i] || a.mx[i] <= b.mn[i])
         return false;
   return true;
}

// Fiber::CalculateVoi (fiber.cpp:83-99) of already transformed points.
Box fiber_box(const double *xyz, const double *r, int64_t n) {
   Box b;
   b.empty();
   if (n == 0)
      return b;
   const double lo[3] = {xyz[0] - r[0], xyz[1] - r[0], xyz[2] - r[0]};
   const double hi[3] = {xyz[0] + r[0], xyz[1] + r[0], xyz[2] + r[0]};
   b.from_pq(lo, hi);
   for (int64_t s = 0; s + 1 < n; s++) {
      const double rm = r[s] < r[s + 1] ? r[s + 1] : r[s];
      Box t;
      t.from_pq(xyz + 3 * s, xyz + 3 * (s + 1));
      for (int i = 0; i < 3; i++) {
         t.mn[i] -= rm;
         t.mx[i] += rm;
      }
      b.unite(t);
   }
   return b;
}

// double -> (hi, lo) float pair; |d - hi - lo| <= 2^-48 |d|
void split2(double d, float &hi, float &lo) {
   hi = (float)d;
   lo = (float)(d - (double)hi);
}

// Host-side constants of the two-float path, all derived in double exactly
// as the reference derives the corresponding values.
void fill_fast_fields(SegDev &S, const fpgb_volume *vol) {
   double ps = 0;
   for (int i = 0; i < 3; i++) {
      split2(S.p[i] - (double)S.base[i], S.pl_hi[i], S.pl_lo[i]);
      split2(S.v[i], S.v_hi[i], S.v_lo[i]);
      ps = std::max(ps, std::max(std::fabs(S.p[i]), std::fabs(S.q[i])));
      ps = std::max(ps, (double)vol->dim[i]);
   }
   S.pscale = (float)(ps + 2.0);
   split2(S.c2, S.c2_hi, S.c2_lo);
   S.c2_rcp = S.c2 > 0 ? (float)(1.0 / S.c2) : 0.f;
   split2(S.r0, S.r0_hi, S.r0_lo);
   split2(S.r1 - S.r0, S.dr_hi, S.dr_lo);
   // Fiber::CalcRadius at t = 0 and t = 1 is exactly r0 and r1
   // (fiber.cpp:115-120): r0*(1-0) + r1*0 = r0, r0*0 + r1*1 = r1
   S.rsq0 = (float)(S.r0 * S.r0);
   S.rsq1 = (float)(S.r1 * S.r1);
   // r0 == r1: every interior r(t) is r0 within a few ulp, so float(r^2) is
   // fixed unless r0^2 sits next to a float rounding boundary
   S.rsq_const = NAN;
   if (S.r0 == S.r1) {
      const double r2 = S.r0 * S.r0;
      const double eps = 64.0 * 0x1p-53;
      const float a = (float)(r2 * (1.0 - eps)), b = (float)(r2 * (1.0 + eps));
      if (a == b)
         S.rsq_const = a;
   }
   // 'p' layer vector: vm::unit(q - p) (generator.cpp:372-373, vemath.hpp:390-402)
   double n2 = 0.0;
   n2 = n2 + S.v[0] * S.v[0];
   n2 = n2 + S.v[1] * S.v[1];
   n2 = n2 + S.v[2] * S.v[2];
   double u[3] = {S.v[0], S.v[1], S.v[2]};
   if (n2 > 0) {
      const double inv = 1.0 / std::sqrt(n2);
      for (int i = 0; i < 3; i++)
         u[i] = u[i] * inv;
   }
   for (int i = 0; i < 3; i++)
      S.vp[i] = (float)u[i];
}

} // namespace

int plan_tissue(const fpgb_volume *vol, const fpgb_fibers *fb, TissuePlan *plan) {
   if (!vol || !fb) {
      set_error("generate_tissue: null volume or fibers");
      return FPGB_EINVAL;
   }
   // SetVolume (generator.cpp:49-53,115-117)
   if (vol->dim[0] <= 0 || vol->dim[1] <= 0 || vol->dim[2] <= 0) {
      set_error("dim.global[any] <= 0: [%lld,%lld,%lld]",
                (long long)vol->dim[0], (long long)vol->dim[1],
                (long long)vol->dim[2]);
      return FPGB_EINVAL;
   }
   if (!(vol->voxel_size > 0)) {
      set_error("voxel_size <= 0: %g", vol->voxel_size);
      return FPGB_EINVAL;
   }
   for (int i = 0; i < 3; i++)
      if (vol->dim[i] > (int64_t(1) << 30)) {
         set_error("dim[%d] = %lld exceeds 2^30", i, (long long)vol->dim[i]);
         return FPGB_EINVAL;
      }
   const int64_t nb = fb->n_bundles;
   if (nb < 0 || (nb > 0 && (!fb->bundle_fiber_off || !fb->fiber_point_off ||
                             !fb->bundle_layer_off))) {
      set_error("generate_tissue: malformed fiber bundle offsets");
      return FPGB_EINVAL;
   }
   plan->X = vol->dim[0];
   plan->Y = vol->dim[1];
   plan->Z = vol->dim[2];
   plan->n_bundles = nb;
   plan->segs.clear();
   plan->layers.assign(nb > 0 ? nb : 1, LayerDev{});
   plan->single_point = 0;

   // layers, sorted by scale (fiber_bundle.cpp:19-30,66,83-86)
   int max_layer = 0;
   for (int64_t b = 0; b < nb; b++) {
      const int64_t l0 = fb->bundle_layer_off[b], l1 = fb->bundle_layer_off[b + 1];
      const int n = int(l1 - l0);
      if (n < 0 || n > kMaxLayers) {
         set_error("bundle %lld has %d layers (1..%d supported)",
                   (long long)b, n, kMaxLayers);
         return FPGB_EINVAL;
      }
      std::vector<int> order(n);
      for (int i = 0; i < n; i++)
         order[i] = i;
      std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
         return fb->layer_scale[l0 + a] < fb->layer_scale[l0 + c];
      });
      LayerDev &L = plan->layers[b];
      L.n = n;
      for (int i = 0; i < n; i++) {
         const int64_t l = l0 + order[i];
         const char m = fb->layer_model[l];
         if (m != 'b' && m != 'p' && m != 'r') {
            set_error("Orientation must be \"b\", \"p\", or \"r\"");
            return FPGB_EINVAL;
         }
         L.scale_sq[i] = fb->layer_scale[l] * fb->layer_scale[l];
         L.model[i] = m;
         L.dn[i] = fb->layer_dn[l];
         L.mu[i] = fb->layer_mu[l];
      }
      for (int i = 0; i < n; i++) {
         float f = (float)L.scale_sq[i];
         if ((double)f > L.scale_sq[i])
            f = std::nextafter(f, -INFINITY);
         L.sq_fdown[i] = f;
      }
      if (n > 0) {
         L.f_ly_squ = (float)L.scale_sq[n - 1];
         L.sqrt_last = std::sqrt(L.scale_sq[n - 1]);
      }
      max_layer = std::max(max_layer, n);
   }
   plan->max_layer = max_layer;

   // property table (generator.cpp:496-526)
   plan->props.assign(2 * (nb * max_layer + 1), 0.0);
   for (int64_t b = 0; b < nb; b++)
      for (int l = 0; l < plan->layers[b].n; l++) {
         const int64_t id = 1 + l + b * max_layer;
         plan->props[2 * id + 1] = plan->layers[b].mu[l];
         plan->props[2 * id] =
             plan->layers[b].model[l] == 'b' ? 0.0 : plan->layers[b].dn[l];
      }

   // translate then resize (generator.cpp:185-197, fiber.cpp:128-150)
   const int64_t nf = nb > 0 ? fb->bundle_fiber_off[nb] : 0;
   const int64_t np = nf > 0 ? fb->fiber_point_off[nf] : 0;
   if (np > 0 && !fb->points) {
      set_error("generate_tissue: points == NULL");
      return FPGB_EINVAL;
   }
   RawArray<double> xyz, rad;
   xyz.reset((size_t)(3 * np));
   rad.reset((size_t)np);
   const bool translate =
       vol->origin[0] != 0 || vol->origin[1] != 0 || vol->origin[2] != 0;
   const double f = 1.0 / vol->voxel_size;
   // first non-finite coordinate (points are checked, translated and scaled
   // in parallel; the error names the lowest bad point as a serial scan would)
   int64_t bad = INT64_MAX;
#pragma omp parallel for schedule(static) reduction(min : bad)
   for (int64_t i = 0; i < np; i++) {
      const double *q = fb->points + 4 * i;
      if (!(std::isfinite(q[0]) && std::isfinite(q[1]) && std::isfinite(q[2]) &&
            std::isfinite(q[3]))) {
         bad = std::min(bad, i);
         continue;
      }
      for (int c = 0; c < 3; c++) {
         double v = q[c];
         if (translate)
            v = v + (-vol->origin[c]);
         xyz[3 * i + c] = v * f;
      }
      rad[i] = q[3] * f;
   }
   if (bad != INT64_MAX) {
      set_error("fiber point %lld is not finite", (long long)bad);
      return FPGB_EINVAL;
   }
   for (int64_t fi = 0; fi < nf; fi++) {
      const int64_t p0 = fb->fiber_point_off[fi], p1 = fb->fiber_point_off[fi + 1];
      if (p1 < p0 || p1 > np) {
         set_error("generate_tissue: malformed fiber_point_off");
         return FPGB_EINVAL;
      }
   }
   std::vector<Box> fbox(nf);
#pragma omp parallel for schedule(dynamic, 32)
   for (int64_t fi = 0; fi < nf; fi++) {
      const int64_t p0 = fb->fiber_point_off[fi], p1 = fb->fiber_point_off[fi + 1];
      fbox[fi] = fiber_box(xyz.data() + 3 * p0, rad.data() + p0, p1 - p0);
   }
   Box volbox;
   for (int i = 0; i < 3; i++) {
      volbox.mn[i] = 0.0;
      volbox.mx[i] = (double)vol->dim[i];
   }

   // segment table in the reference's processing order (generator.cpp:205-231):
   // which bundles overlap the volume is decided first, then the fibers are
   // planned in parallel into per-fiber lists that are concatenated in order
   std::vector<char> bundle_on(nb > 0 ? nb : 1, 0);
   std::vector<int32_t> fiber_bundle(nf);
   for (int64_t b = 0; b < nb; b++) {
      const int64_t f0 = fb->bundle_fiber_off[b], f1 = fb->bundle_fiber_off[b + 1];
      Box bb;
      bb.empty(); // fiber_bundle.cpp:147-154
      if (f1 > f0)
         bb = fbox[f0];
      for (int64_t fi = f0; fi < f1; fi++) {
         bb.unite(fbox[fi]);
         fiber_bundle[fi] = (int32_t)b;
      }
      bundle_on[b] = overlap(volbox, bb) ? 1 : 0;
   }
   // pass 1: segments each fiber keeps (its boxes only); pass 2 fills the
   // table in place at the fibers' prefix offsets
   std::vector<int64_t> fiber_segs(nf + 1, 0);
   std::vector<char> single(nf, 0);
   auto seg_box = [&](int64_t s, double rsl, SegDev &S) -> int64_t {
      const double *P = &xyz[3 * s], *Q = &xyz[3 * (s + 1)];
      const double r0 = rad[s], r1 = rad[s + 1];
      const double rmax = (r0 < r1 ? r1 : r0) * rsl;
      Box sb;
      sb.from_pq(P, Q);
      int64_t count = 1;
      for (int i = 0; i < 3; i++) {
         sb.mn[i] -= rmax;
         sb.mx[i] += rmax;
         if (volbox.mn[i] > sb.mn[i])
            sb.mn[i] = volbox.mn[i];
         if (volbox.mx[i] < sb.mx[i])
            sb.mx[i] = volbox.mx[i];
         if (!(sb.mn[i] <= sb.mx[i])) { // empty or non-finite box
            S.lo[i] = 0;
            S.ext[i] = 0;
            count = 0;
            continue;
         }
         // (int64) truncation as generator.cpp:304-305; the clamp only
         // restates that the box already lies in [0, dim]
         const int64_t lo = std::max<int64_t>(0, (int64_t)sb.mn[i]);
         const int64_t hi = std::min<int64_t>(vol->dim[i], (int64_t)(sb.mx[i] + 0.5));
         S.lo[i] = (int32_t)lo;
         S.ext[i] = (int32_t)(hi > lo ? hi - lo : 0);
         count *= S.ext[i];
      }
      return count;
   };
   auto fiber_used = [&](int64_t fi) -> bool {
      const int64_t b = fiber_bundle[fi];
      const int64_t p0 = fb->fiber_point_off[fi], p1 = fb->fiber_point_off[fi + 1];
      return bundle_on[b] && p1 - p0 > 1 && overlap(volbox, fbox[fi]) && plan->layers[b].n > 0;
   };
#pragma omp parallel for schedule(dynamic, 32)
   for (int64_t fi = 0; fi < nf; fi++) {
      const int64_t b = fiber_bundle[fi];
      const int64_t p0 = fb->fiber_point_off[fi], p1 = fb->fiber_point_off[fi + 1];
      if (bundle_on[b] && p1 - p0 <= 1)
         single[fi] = 1;
      if (!fiber_used(fi))
         continue;
      int64_t n = 0;
      SegDev S;
      for (int64_t s = p0; s + 1 < p1; s++)
         n += seg_box(s, plan->layers[b].sqrt_last, S) > 0;
      fiber_segs[fi + 1] = n;
   }
   for (int64_t fi = 0; fi < nf; fi++) {
      fiber_segs[fi + 1] += fiber_segs[fi];
      plan->single_point += single[fi];
   }
   plan->segs.reset((size_t)fiber_segs[nf]);
   SegDev *table = plan->segs.data();
   int64_t cand = 0, pairs = 0;
#pragma omp parallel for schedule(dynamic, 32) reduction(+ : cand, pairs)
   for (int64_t fi = 0; fi < nf; fi++) {
      if (!fiber_used(fi))
         continue;
      const int64_t b = fiber_bundle[fi];
      const LayerDev &L = plan->layers[b];
      const int64_t p0 = fb->fiber_point_off[fi], p1 = fb->fiber_point_off[fi + 1];
      int64_t at = fiber_segs[fi];
      for (int64_t s = p0; s + 1 < p1; s++) {
         SegDev S;
         std::memset(&S, 0, sizeof S);
         const int64_t count = seg_box(s, L.sqrt_last, S);
         if (count == 0)
            continue;
         const double *P = &xyz[3 * s], *Q = &xyz[3 * (s + 1)];
         const double r0 = rad[s], r1 = rad[s + 1];
         for (int i = 0; i < 3; i++) {
            S.p[i] = P[i];
            S.q[i] = Q[i];
            S.v[i] = Q[i] - P[i];
            const double base = std::floor(P[i]);
            S.base[i] = (int32_t)std::max(-2147483647.0, std::min(2147483647.0, base));
            S.pf[i] = (float)(P[i] - (double)S.base[i]);
            S.vf[i] = (float)S.v[i];
         }
         {
            double c = 0.0;
            c = c + S.v[0] * S.v[0];
            c = c + S.v[1] * S.v[1];
            c = c + S.v[2] * S.v[2];
            S.c2 = c;
         }
         S.c2f = (float)S.c2;
         S.r0 = r0;
         S.r1 = r1;
         fill_fast_fields(S, vol);
         const double rm = r0 < r1 ? r1 : r0;
         S.thr_f = (float)((double)L.f_ly_squ * rm * rm * (1.0 + 1e-3) + 1e-3);
         {
            const double rn = r0 < r1 ? r0 : r1;
            const double a = (double)L.f_ly_squ * rn * rn * (1.0 - 1e-5);
            float af = (float)a;
            if ((double)af > a)
               af = std::nextafter(af, 0.f);
            S.acc_f = af > 0.f ? af : -1.f;
         }
         S.bundle = (int32_t)b;
         table[at++] = S;
         cand += count;
         pairs += segment_brick_pairs(S);
      }
   }
   if (plan->segs.size() > 0xFFFFFFF0ull) {
      set_error("too many fiber segments: %zu", plan->segs.size());
      return FPGB_EINVAL;
   }
   plan->candidates = cand;
   plan->brick_pairs = pairs;
   return FPGB_OK;
}

// ======================================================================
// device code
// ======================================================================

// ======================================================================
// launch
// ======================================================================
// Device workspace of one voxelization: the tile header (one TileDev and the
// label / vector pointers), segment table, layers, counters, and the brick
// lists of the voxelizer.
static int64_t plan_bricks(const TissuePlan &p, int32_t nb[3]) {
   int64_t n = 0;
   tile_bricks(p.X, p.Y, p.Z, nb, &n);
   return n;
}

size_t tissue_workspace_bytes(const TissuePlan &p) {
   int32_t nb[3];
   const int64_t n_bricks = plan_bricks(p, nb);
   size_t b = align_up(sizeof(TileDev) + 2 * sizeof(void *), 256);
   b += align_up(sizeof(SegDev) * std::max<size_t>(p.segs.size(), 1), 256);
   b += align_up(sizeof(LayerDev) * p.layers.size(), 256);
   b += align_up(sizeof(unsigned long long) * kCounterWords, 256);
   b += brick_workspace_bytes(n_bricks, p.brick_pairs);
   return b;
}

int run_tissue(const TissuePlan &p, int only_label, int32_t *d_label,
               float *d_vector, void *d_ws, size_t ws_bytes,
               unsigned long long **d_counters_out, cudaStream_t st, int n_slabs,
               int (*after_slab)(void *ctx, int64_t x0, int64_t x1, cudaStream_t s), void *ctx,
               cudaStream_t alt) {
   const size_t need = tissue_workspace_bytes(p);
   if (ws_bytes < need) {
      set_error("generate_tissue: workspace %zu bytes < %zu needed", ws_bytes, need);
      return FPGB_ENOMEM;
   }
   if (reinterpret_cast<uintptr_t>(d_ws) % 256 != 0) {
      set_error("generate_tissue: workspace must be 256-byte aligned");
      return FPGB_EINVAL;
   }
   int32_t nb[3];
   const int64_t n_bricks = plan_bricks(p, nb);
   char *w = static_cast<char *>(d_ws);
   char *head = w;
   w += align_up(sizeof(TileDev) + 2 * sizeof(void *), 256);
   auto *segs = reinterpret_cast<SegDev *>(w);
   w += align_up(sizeof(SegDev) * std::max<size_t>(p.segs.size(), 1), 256);
   auto *layers = reinterpret_cast<LayerDev *>(w);
   w += align_up(sizeof(LayerDev) * p.layers.size(), 256);
   auto *counters = reinterpret_cast<unsigned long long *>(w);
   w += align_up(sizeof(unsigned long long) * kCounterWords, 256);

   // the single volume as tile 0 of the brick voxelizer
   struct {
      TileDev t;
      void *label, *vector;
   } h{};
   h.t.vox_base = 0;
   h.t.n_vox = p.X * p.Y * p.Z;
   h.t.brick_base = 0;
   h.t.X = (int32_t)p.X;
   h.t.Y = (int32_t)p.Y;
   h.t.Z = (int32_t)p.Z;
   h.t.max_layer = p.max_layer;
   h.t.layer_base = 0;
   for (int i = 0; i < 3; i++)
      h.t.nb[i] = nb[i];
   h.label = d_label;
   h.vector = only_label ? nullptr : d_vector;
   static_assert(sizeof(h) == sizeof(TileDev) + 2 * sizeof(void *), "tile header layout");

   FPGB_CUDA_TRY(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * kCounterWords, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(head, &h, sizeof(h), cudaMemcpyHostToDevice, st));
   if (!p.segs.empty())
      FPGB_CUDA_TRY(cudaMemcpyAsync(segs, p.segs.data(), sizeof(SegDev) * p.segs.size(),
                                    cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(layers, p.layers.data(), sizeof(LayerDev) * p.layers.size(),
                                 cudaMemcpyHostToDevice, st));
   auto *tile = reinterpret_cast<const TileDev *>(head);
   auto *lp = reinterpret_cast<int32_t *const *>(head + sizeof(TileDev));
   auto *vp = reinterpret_cast<float *const *>(head + sizeof(TileDev) + sizeof(void *));
   // x-slabs of whole brick columns: bricks are numbered x-major, so a range
   // of brick x indices is a contiguous brick range and a contiguous x range
   // of voxels
   struct Slabs {
      int64_t bx[65];
      int64_t X;
      int (*after)(void *, int64_t, int64_t, cudaStream_t);
      void *ctx;
      static int thunk(void *self, int c, cudaStream_t s) {
         const Slabs &S = *static_cast<const Slabs *>(self);
         const int64_t x0 = S.bx[c] * kBrickX, x1 = std::min(S.bx[c + 1] * kBrickX, S.X);
         return S.after ? S.after(S.ctx, x0, x1, s) : FPGB_OK;
      }
   } slabs;
   int64_t bound[65];
   BrickChunks chunks{};
   const int n = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)n_slabs, 64, nb[0]}));
   if (n > 1) {
      slabs.X = p.X;
      slabs.after = after_slab;
      slabs.ctx = ctx;
      for (int c = 0; c <= n; c++) {
         slabs.bx[c] = nb[0] * c / n;
         bound[c] = slabs.bx[c] * nb[1] * nb[2];
      }
      chunks = BrickChunks{n, bound, &Slabs::thunk, &slabs, alt};
   }
   FPGB_TRY(launch_voxel_bricks(segs, nullptr, (int64_t)p.segs.size(), tile, 1, n_bricks,
                                p.brick_pairs, layers, p.n_bundles > 1, lp, vp, w, counters, st,
                                n > 1 ? &chunks : nullptr));
   if (n == 1 && after_slab)
      FPGB_TRY(after_slab(ctx, 0, p.X, st));
   l2_end_state().store(1, std::memory_order_relaxed); // bricks run x-major: high x last
   if (d_counters_out)
      *d_counters_out = counters;
   return FPGB_OK;
}

// Copies of finished x-slabs of a host-buffer generation (page-locked
// outputs), queued on their own stream behind an event of the slab's launch.
// The slab launches alternate between two streams so that one slab's last
// bricks overlap the next slab's first; then thinner slabs pay: on the
// 512 x 512 x 120 bench volume a call took 4.24 ms with 8 slabs on one
// stream, 4.39 / 4.09 / 4.03 ms with 8 / 16 / 24 slabs on two (the copy
// alone is 2.62 ms).
constexpr int kCopySlabs = 24;

struct SlabCopy {
   int32_t *label;
   float *vector;
   const int32_t *d_label;
   const float *d_vector;
   int64_t row; // voxels per x
   cudaStream_t copy;
   std::vector<cudaEvent_t> events;

   static int after(void *self, int64_t x0, int64_t x1, cudaStream_t s) {
      SlabCopy &S = *static_cast<SlabCopy *>(self);
      cudaEvent_t ev;
      FPGB_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      S.events.push_back(ev);
      FPGB_CUDA_TRY(cudaEventRecord(ev, s));
      FPGB_CUDA_TRY(cudaStreamWaitEvent(S.copy, ev, 0));
      const int64_t v0 = x0 * S.row, nv = (x1 - x0) * S.row;
      FPGB_CUDA_TRY(cudaMemcpyAsync(S.label + v0, S.d_label + v0, sizeof(int32_t) * nv,
                                    cudaMemcpyDeviceToHost, S.copy));
      if (S.vector)
         FPGB_CUDA_TRY(cudaMemcpyAsync(S.vector + 3 * v0, S.d_vector + 3 * v0,
                                       sizeof(float) * 3 * nv, cudaMemcpyDeviceToHost, S.copy));
      return FPGB_OK;
   }
};

int finish_props(const TissuePlan &p, double *props, int64_t props_cap, int64_t *n_props) {
   const int64_t n = (int64_t)p.props.size() / 2;
   if (n_props)
      *n_props = n;
   if (props) {
      if (props_cap < n) {
         set_error("props_cap %lld < %lld rows", (long long)props_cap, (long long)n);
         return FPGB_EINVAL;
      }
      std::memcpy(props, p.props.data(), sizeof(double) * 2 * n);
   }
   return FPGB_OK;
}

int tissue_status_from_counters(const TissuePlan &p, const long long *h, fpgb_warnings *w) {
   if (h[6] & kStatusOverflow) { // the device binning disagreed with the host plan
      set_error("generate_tissue: internal error, segment-brick lists overflowed");
      return FPGB_ECUDA;
   }
   if (!w)
      return FPGB_OK;
   warnings_from_counters(h, w);
   w->overlap = w->overlap > 0 ? 1 : 0; // the reference warns once (generator.cpp:353-359)
   w->single_point = p.single_point;
   return FPGB_OK;
}

int read_tissue_warnings(const TissuePlan &p, unsigned long long *d_counters, fpgb_warnings *w,
                         cudaStream_t st) {
   if (!w)
      return FPGB_OK;
   long long h[kCounterWords];
   FPGB_CUDA_TRY(cudaMemcpyAsync(h, d_counters, sizeof h, cudaMemcpyDeviceToHost, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   return tissue_status_from_counters(p, h, w);
}

} // namespace fpgb

using namespace fpgb;

extern "C" {

size_t fpgb_generate_workspace_size(const fpgb_volume *vol, const fpgb_fibers *fibers) {
   TissuePlan p;
   if (plan_tissue(vol, fibers, &p) != FPGB_OK)
      return 0;
   return tissue_workspace_bytes(p);
}

int fpgb_generate_tissue_device(const fpgb_volume *vol, const fpgb_fibers *fibers,
                                int only_label, int32_t *d_label, float *d_vector,
                                double *props, int64_t props_cap, int64_t *n_props,
                                void *d_workspace, size_t workspace_bytes,
                                fpgb_warnings *warnings, void *stream) {
   TissuePlan p;
   FPGB_TRY(plan_tissue(vol, fibers, &p));
   if (!d_label || (!only_label && !d_vector)) {
      set_error("generate_tissue_device: null output buffer");
      return FPGB_EINVAL;
   }
   const size_t need = tissue_workspace_bytes(p);
   if (!d_workspace) {
      FPGB_TRY(pool_get(kSlotKeys, need, &d_workspace, as_stream(stream)));
      workspace_bytes = need;
   }
   unsigned long long *d_counters = nullptr;
   cudaStream_t st = as_stream(stream);
   FPGB_TRY(run_tissue(p, only_label, d_label, d_vector, d_workspace, workspace_bytes,
                       &d_counters, st));
   FPGB_TRY(finish_props(p, props, props_cap, n_props));
   return read_tissue_warnings(p, d_counters, warnings, st);
}

int fpgb_generate_tissue(const fpgb_volume *vol, const fpgb_fibers *fibers, int only_label,
                         int32_t *label, float *vector, double *props, int64_t props_cap,
                         int64_t *n_props, fpgb_warnings *warnings) {
   TissuePlan p;
   FPGB_TRY(plan_tissue(vol, fibers, &p));
   if (!label || (!only_label && !vector)) {
      set_error("generate_tissue: null output buffer");
      return FPGB_EINVAL;
   }
   const int64_t nvox = p.X * p.Y * p.Z;
   void *d_label = nullptr, *d_vec = nullptr, *d_ws = nullptr;
   FPGB_TRY(pool_get(kSlotLabel, sizeof(int32_t) * nvox, &d_label));
   if (!only_label)
      FPGB_TRY(pool_get(kSlotVector, sizeof(float) * 3 * nvox, &d_vec));
   const size_t need = tissue_workspace_bytes(p);
   FPGB_TRY(pool_get(kSlotKeys, need, &d_ws));
   cudaStream_t st = nullptr;
   unsigned long long *d_counters = nullptr;
   if (host_pinned(label) && (only_label || host_pinned(vector))) {
      // page-locked outputs: each x-slab's rows are copied on a second stream
      // while the next slabs are voxelized
      SlabCopy sc;
      sc.label = label;
      sc.vector = only_label ? nullptr : vector;
      sc.d_label = static_cast<const int32_t *>(d_label);
      sc.d_vector = static_cast<const float *>(d_vec);
      sc.row = p.Y * p.Z;
      cudaStream_t alt = nullptr;
      FPGB_CUDA_TRY(cudaStreamCreateWithFlags(&sc.copy, cudaStreamNonBlocking));
      cudaError_t e = cudaStreamCreateWithFlags(&alt, cudaStreamNonBlocking);
      int rc = e == cudaSuccess ? run_tissue(p, only_label, (int32_t *)d_label, (float *)d_vec,
                                             d_ws, need, &d_counters, st, kCopySlabs,
                                             &SlabCopy::after, &sc, alt)
                                : FPGB_ECUDA;
      if (e != cudaSuccess)
         set_error("generate_tissue: %s", cudaGetErrorString(e));
      e = cudaStreamSynchronize(sc.copy);
      for (cudaEvent_t ev : sc.events)
         cudaEventDestroy(ev);
      cudaStreamDestroy(sc.copy);
      if (alt) {
         cudaStreamSynchronize(alt);
         cudaStreamDestroy(alt);
      }
      FPGB_TRY(rc);
      if (e != cudaSuccess) {
         set_error("generate_tissue: %s", cudaGetErrorString(e));
         return FPGB_ECUDA;
      }
   } else {
      FPGB_TRY(run_tissue(p, only_label, (int32_t *)d_label, (float *)d_vec, d_ws, need,
                          &d_counters, st));
      // while the voxelizer runs
      prefault_host(label, sizeof(int32_t) * nvox);
      if (!only_label)
         prefault_host(vector, sizeof(float) * 3 * nvox);
      FPGB_CUDA_TRY(cudaMemcpyAsync(label, d_label, sizeof(int32_t) * nvox,
                                    cudaMemcpyDeviceToHost, st));
      if (!only_label)
         FPGB_CUDA_TRY(cudaMemcpyAsync(vector, d_vec, sizeof(float) * 3 * nvox,
                                       cudaMemcpyDeviceToHost, st));
   }
   FPGB_TRY(finish_props(p, props, props_cap, n_props));
   fpgb_warnings tmp;
   FPGB_TRY(read_tissue_warnings(p, d_counters, warnings ? warnings : &tmp, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   return FPGB_OK;
}

} // extern "C"
