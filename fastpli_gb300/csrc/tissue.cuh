// Voxelizer data layout shared by the plain, batched and no-allocation paths.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "fpgb_common.cuh"

namespace fpgb {

constexpr int kMaxLayers = 16;

// One fiber segment after translate + resize (voxel units), in the
// reference's processing order; its table index is the tie-break index.
struct __align__(16) SegDev {
   double p[3];   // segment start s0
   double q[3];   // segment end s1
   double v[3];   // s1 - s0 (generator.cpp:479)
   double r0, r1; // radii at s0, s1
   double c2;     // dot(v, v) (generator.cpp:486)
   // inputs of the voxelizer's sweeps: five 16-byte words at offset 96,
   // read with vector loads (SegSweep)
   float pf[3];   // p - base, for the FP32 prefilter
   float vf[3];   // float(v)
   float c2f;     // float(c2)
   float c2_rcp;  // float(1 / c2)
   float thr_f;   // prefilter bound on dist^2 (>= f_ly_squ * max(r0,r1)^2)
   float acc_f;   // dist^2 at or below which a candidate is certainly inside
                  // (<= f_ly_squ * min(r0,r1)^2, rounded down)
   int32_t base[3]; // floor(p)
   int32_t lo[3];   // clipped box start (generator.cpp:304)
   int32_t ext[3];  // clipped box extent
   int32_t bundle;
   // two-float copies (hi, lo) of the double inputs, for the fast path
   float pl_hi[3], pl_lo[3]; // p - base
   float v_hi[3], v_lo[3];   // v
   float c2_hi, c2_lo;       // c2
   float r0_hi, r0_lo;       // r0
   float dr_hi, dr_lo;       // r1 - r0
   float rsq0, rsq1;         // float(r^2) at t = 0 and t = 1 (exact)
   float rsq_const;          // float(r^2) for every interior t when r0 == r1
                             // and that rounding is certain; NaN otherwise
   float pscale;             // max |coordinate| met by this segment's arithmetic
   float vp[3];              // float(unit(q - p)): the 'p' layer vector (exact)
};
static_assert(offsetof(SegDev, pf) == 96 && offsetof(SegDev, bundle) == 172,
              "the sweep inputs of SegDev are five aligned 16-byte words");

// Layers of one bundle, sorted by scale (fiber_bundle.cpp:83-86).
struct LayerDev {
   int32_t n = 0;
   float f_ly_squ = 0.f; // float(scale^2 of the outermost layer)
   double sqrt_last = 0.0;
   double scale_sq[kMaxLayers] = {};
   // largest float <= scale_sq[l]: for a float q, (double)q > scale_sq[l]
   // exactly when q > sq_fdown[l], so the layer search needs no FP64
   float sq_fdown[kMaxLayers] = {};
   double dn[kMaxLayers] = {};
   double mu[kMaxLayers] = {};
   char model[kMaxLayers] = {};
};

// Growable array without value-initialisation (the segment table is written
// in full by the planner; zeroing 200+ bytes per segment first is waste).
template <class T> class RawArray {
 public:
   void reset(size_t n) {
      p_.reset(n ? new T[n] : nullptr);
      n_ = n;
   }
   void clear() { reset(0); }
   T *data() { return p_.get(); }
   const T *data() const { return p_.get(); }
   size_t size() const { return n_; }
   bool empty() const { return n_ == 0; }
   T &operator[](size_t i) { return p_[i]; }
   const T &operator[](size_t i) const { return p_[i]; }
   const T *begin() const { return p_.get(); }
   const T *end() const { return p_.get() + n_; }

 private:
   std::unique_ptr<T[]> p_;
   size_t n_ = 0;
};

struct TissuePlan {
   int64_t X = 0, Y = 0, Z = 0;
   int64_t n_bundles = 0;
   int max_layer = 0;
   int64_t single_point = 0; // fibers skipped with a warning
   int64_t candidates = 0;   // sum of clipped box volumes
   int64_t brick_pairs = 0;  // (segment, brick) pairs of the brick voxelizer
   RawArray<SegDev> segs;
   std::vector<LayerDev> layers;
   std::vector<double> props; // (dn, mu) rows
};

int plan_tissue(const fpgb_volume *vol, const fpgb_fibers *fb, TissuePlan *plan);
size_t tissue_workspace_bytes(const TissuePlan &p);
// Voxelizes the planned volume into d_label / d_vector on stream st.  With
// n_slabs > 1 the bricks are voxelized in that many x-slabs, one launch each
// (alternating between st and `alt` when alt is given), and
// after_slab(ctx, x0, x1, s) runs on the host as soon as the launch for
// voxels x0 <= x < x1 is enqueued on stream s (their label and vector rows
// are contiguous in the output, so their copy can start while later slabs
// run).  Work queued on st afterwards sees every slab.
int run_tissue(const TissuePlan &p, int only_label, int32_t *d_label, float *d_vector,
               void *d_ws, size_t ws_bytes, unsigned long long **d_counters_out,
               cudaStream_t st, int n_slabs = 1,
               int (*after_slab)(void *ctx, int64_t x0, int64_t x1, cudaStream_t s) = nullptr,
               void *ctx = nullptr, cudaStream_t alt = nullptr);

// Copies the planned (dn, mu) rows to props (host, props_cap rows) and their
// count to n_props; either may be null.
int finish_props(const TissuePlan &p, double *props, int64_t props_cap, int64_t *n_props);

// Decodes a voxelizer counter block copied to the host (kCounterWords
// words): FPGB_ECUDA, with the error set, when the device binning overflowed
// the host plan's segment-brick lists; otherwise the reference's warnings
// into w (when not null).
int tissue_status_from_counters(const TissuePlan &p, const long long *h, fpgb_warnings *w);

// Reads the voxelizer's counter block (synchronising st) into w: the
// reference's warnings, or FPGB_ECUDA when the device binning overflowed the
// host plan's segment-brick lists.  Does nothing when w is null.
int read_tissue_warnings(const TissuePlan &p, unsigned long long *d_counters, fpgb_warnings *w,
                         cudaStream_t st);

} // namespace fpgb
