// Ray-march parameter block shared by the plain and batched kernels.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <vector>

#include "fpgb_common.cuh"

namespace fpgb {

constexpr int kMaxRho = 64;

// Per-label optical constants (simulator.cpp:276-288, 309-316).
struct LabelOptics {
   float alog; // mu[1/mm] * 1e3 * thickness : per-step -log(attenuation)
   float kret; // pi/2 * dn * 4 * thickness / lambda : ret = kret*|v|*cos^2(alpha)
   int32_t kind; // 0: no effect, 1: attenuation only, 2: birefringent
   int32_t pad;
};

// One step of the z march.  Every ray of a call shares the same z sequence
// (the start height and the z step do not depend on the pixel), so the
// reference's double accumulation of z (simulator.cpp:259-261) is replayed on
// the host once and tabulated.
struct ZStep {
   int32_t iz;  // floor(z), already mirrored when flip_z (simulator.cpp:427-428)
   int32_t z0;  // floor(z - 0.5), not clamped, not mirrored
   float zf;    // (z - 0.5) - z0 in [0, 1)
   int32_t pad;
};

struct MarchParams {
   int64_t X, Y, Z;
   int32_t n_rho, mode, flip_z, untilt;
   int32_t n_props, n_z, frac_bits, rotate;
   int64_t dx_fx, dy_fx;  // x/y step in fixed point (frac_bits)
   double hstep[3];       // light_step * 0.5
   double hshift[2];      // 0.5 * shift (untilted view)
   double shift[2];       // shift (tilted view)
   double pc[3], pt[3], p1[3], p2[3];
   double A, B, C, Dd, D; // tilted-view 2x2 system (simulator.cpp:653-668)
   double rti[9];         // inverse tissue rotation (simulator.cpp:636-638)
   float rot[9];          // RotZYZ(phi, theta, -phi) for the optic axis
   float i4;              // light_intensity / 4
   float c2r[kMaxRho], s2r[kMaxRho]; // cos 2rho, sin 2rho of the filter angles
   float epa_sin[kMaxRho], epa_cos[kMaxRho]; // sin/cos(2*pi*i/n) of epa.py:29
   const LabelOptics *lut;
   const ZStep *ztab;
   // buffers of one (tile, tilt) pair of the batched path (unused by the
   // plain kernel, which takes them as launch arguments)
   const int32_t *label;
   const float *vec;
   double *image, *epa_t, *epa_d, *epa_r;
   int32_t tilted; // x/y advance or the axis rotates
   int32_t column; // vertical ray reading z = 0..Z-1 (or mirrored) in order:
                   // the column path applies (16-byte loads when Z % 4 == 0)
   // Lerp/Slerp rays that are not vertical columns: 1 = warp-cooperative
   // march (steps needing interpolation compacted across the warp), 0 = one
   // thread per ray.  Both give the same bits; the choice is speed only.
   int32_t coop;
   // kinds of labels 0..15, two bits each (kind_packed = 1 when every label
   // fits): the march reads a step's kind without a table load
   uint32_t kind_mask;
   int32_t kind_packed;
   // blocks run from the last unit down (the volume's high-x end first):
   // the order only decides which rays go first, never a result
   int32_t reverse;
};
static_assert(sizeof(MarchParams) % 16 == 0, "MarchParams is staged in 16-byte words");

struct MarchPlan {
   MarchParams prm;
   std::vector<LabelOptics> lut;
   std::vector<ZStep> ztab;
   int64_t steps; // X*Y*n_z
};

// Whether the march may use 32-bit index arithmetic (MarchIdx<false>):
// 3 X Y Z < 2^32 and ray positions below 2^30 voxels (frac_bits >= 32).
// FPGB_WIDE_INDEX=1 in the environment forces the 64-bit kernels (which
// every volume too large for the 32-bit ones uses) on any volume, so that
// tests can check on small volumes that both give the same bits.
inline bool march_narrow(const MarchParams &P) {
   const char *w = std::getenv("FPGB_WIDE_INDEX");
   if (w && w[0] == '1')
      return false;
   return P.frac_bits >= 32 && P.X > 0 && P.Y > 0 && P.Z > 0 &&
          (double)P.X * (double)P.Y * (double)P.Z * 3.0 < 4294967296.0;
}

int plan_march(const fpgb_setup *setup, const int64_t *dim, const double *props,
               int64_t n_props, double theta, double phi, MarchPlan *plan);

} // namespace fpgb

namespace fpgb {
int check_setup(const fpgb_setup *s);
size_t march_table_bytes(const MarchPlan &mp);
int init_counters(unsigned long long *d_counters, cudaStream_t st);
int finish_counters(const unsigned long long *d_counters, int64_t n_props, bool checked_all,
                    fpgb_warnings *w, cudaStream_t st);
} // namespace fpgb
