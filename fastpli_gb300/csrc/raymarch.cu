// Ray march: label + optic-axis volume -> polarizer-angle image stack.
//
// Replaces PliSimulator::RunSimulation (src/simulation/simulator.cpp:182-411)
// with one thread per CCD pixel ray.
//
// The polarizer-angle loop collapses.  The initial Stokes vector is circular,
// (I/2, 0, 0, -I/2) (simulator.cpp:207-214), which rotations about the
// s3 axis leave unchanged, and every step for filter angle rho is
// R(2rho - 2phi) . Ret(ret) . R(2phi - 2rho) on (s1, s2, s3)
// (simulator.cpp:322-336).  In the frame t = R(-2rho) s the step is
// R(-2phi) . Ret . R(2phi) for every rho, so one state vector per ray is
// marched and all rho come out in the epilogue:
//     I(rho) = I/4 * A * (1 - u1 cos 2rho + u2 sin 2rho),
// with u the unit state (u0 = (0, 0, -1)) and A the product of the per-step
// attenuations exp(-mu*thickness) (simulator.cpp:278,336), accumulated as a
// sum of exponents.  cos 2phi, sin 2phi and cos^2(alpha) come from the axis
// components directly (phi = atan2(vy, vx), alpha = asin(vz/|v|),
// simulator.cpp:315-320):
//     cos 2phi = (vx^2 - vy^2)/q, sin 2phi = 2 vx vy / q, cos^2 alpha = q/|v|^2,
// q = vx^2 + vy^2.
//
// Ray positions: the reference advances a double position by the light step
// (simulator.cpp:259-261).  Every ray shares the same z sequence, so the host
// replays that double loop once (ZStep table); x and y advance in 64-bit
// fixed point from a double start computed per ray in the reference's
// operation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "fpgb_common.cuh"
#include "march_core.cuh"
#include "raymarch.cuh"

namespace fpgb {

// ======================================================================
// host: setup checks and per-call constants
// ======================================================================
namespace {

// vm::rot_pi_cases::sin / cos (vemath.hpp:498-520)
double pc_sin(double v) {
   v = std::fmod(v, 2 * M_PI);
   if (v == 0 || v == M_PI || v == -M_PI)
      return 0;
   else if (v == M_PI_2 || v == -(M_PI + M_PI_2))
      return 1;
   else if (v == M_PI + M_PI_2 || v == -M_PI_2)
      return -1;
   return std::sin(v);
}
double pc_cos(double v) {
   v = std::fmod(v, 2 * M_PI);
   if (v == 0)
      return 1;
   else if (v == M_PI_2 || v == M_PI + M_PI_2 || v == -M_PI_2 || v == -(M_PI + M_PI_2))
      return 0;
   else if (v == M_PI || v == -M_PI)
      return -1;
   return std::cos(v);
}
void mat3_mul(const double *A, const double *B, double *R) {
   for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) {
         double s = 0;
         for (int k = 0; k < 3; k++)
            s += A[3 * m + k] * B[3 * k + n];
         R[3 * m + n] = s;
      }
}
void mat3_vec(const double *A, const double *v, double *r) {
   double t[3];
   for (int i = 0; i < 3; i++) {
      double s = 0.0;
      s = s + v[0] * A[3 * i + 0];
      s = s + v[1] * A[3 * i + 1];
      s = s + v[2] * A[3 * i + 2];
      t[i] = s;
   }
   std::memcpy(r, t, sizeof t);
}
// vm::rot_pi_cases::Mat3RotZYZ (vemath.hpp:536-544)
void rot_zyz(double g, double b, double a, double *R) {
   const double cg = pc_cos(g), sg = pc_sin(g), cb = pc_cos(b), sb = pc_sin(b);
   const double ca = pc_cos(a), sa = pc_sin(a);
   const double Zg[9] = {cg, -sg, 0, sg, cg, 0, 0, 0, 1};
   const double Yb[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb};
   const double Za[9] = {ca, -sa, 0, sa, ca, 0, 0, 0, 1};
   double T[9];
   mat3_mul(Yb, Za, T);
   mat3_mul(Zg, T, R);
}

} // namespace

int check_setup(const fpgb_setup *s) {
   if (!s) {
      set_error("pli_setup not set yet");
      return FPGB_EINVAL;
   }
   // Setup::Check (setup.hpp:48-71)
   if (!(s->step_size > 0)) {
      set_error("step_size <= 0: %g", s->step_size);
      return FPGB_EINVAL;
   }
   if (s->light_intensity < 0) {
      set_error("light intensity < 0: %g", s->light_intensity);
      return FPGB_EINVAL;
   }
   if (!(s->voxel_size > 0)) {
      set_error("voxel_size <= 0: %g", s->voxel_size);
      return FPGB_EINVAL;
   }
   if (!(s->wavelength > 0)) {
      set_error("wavelength <= 0: %g", s->wavelength);
      return FPGB_EINVAL;
   }
   if (s->tissue_refrection < 1) {
      set_error("tissue_refrection < 1: %g", s->tissue_refrection);
      return FPGB_EINVAL;
   }
   if (s->n_rho <= 0 || !s->filter_rotations) {
      set_error("filter_rotations is empty: []");
      return FPGB_EINVAL;
   }
   if (s->n_rho > kMaxRho) {
      set_error("at most %d filter rotations are supported, got %d", kMaxRho, s->n_rho);
      return FPGB_EINVAL;
   }
   if (s->interpolate < 0 || s->interpolate > 2) {
      set_error("Only NN, Lerp or Slerp are supported");
      return FPGB_EINVAL;
   }
   return FPGB_OK;
}

int plan_march(const fpgb_setup *s, const int64_t *dim, const double *props, int64_t n_props,
               double theta, double phi, MarchPlan *plan) {
   FPGB_TRY(check_setup(s));
   if (!dim || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) {
      set_error("global_dim[any] <= 0");
      return FPGB_EINVAL;
   }
   for (int i = 0; i < 3; i++)
      if (dim[i] > (int64_t(1) << 30)) {
         set_error("dim[%d] too large", i);
         return FPGB_EINVAL;
      }
   if (!props || n_props <= 0) {
      set_error("properties are empty");
      return FPGB_EINVAL;
   }
   // CheckInput (simulator.cpp:169-175)
   if (props[0] != 0) {
      set_error("background birefringence has to be 0");
      return FPGB_EINVAL;
   }
   for (int64_t i = 0; i < n_props; i++)
      if (props[2 * i + 1] < 0) { // PhyProps::Check (setup.hpp:38-41)
         set_error("mu < 0: %g", props[2 * i + 1]);
         return FPGB_EINVAL;
      }
   if (!std::isfinite(theta) || !std::isfinite(phi)) {
      set_error("theta/phi must be finite");
      return FPGB_EINVAL;
   }

   MarchParams &P = plan->prm;
   std::memset(&P, 0, sizeof P);
   P.X = dim[0];
   P.Y = dim[1];
   P.Z = dim[2];
   P.n_rho = s->n_rho;
   P.mode = s->interpolate;
   P.flip_z = s->flip_z ? 1 : 0;
   P.untilt = s->untilt_sensor_view ? 1 : 0;
   P.n_props = (int32_t)std::min<int64_t>(n_props, INT32_MAX);

   const double lambda = s->wavelength * 1e-9;               // simulator.cpp:200
   const double thickness = s->voxel_size * 1e-6 * s->step_size; // :201
   plan->lut.resize(n_props);
   for (int64_t l = 0; l < n_props; l++) {
      const double dn = props[2 * l], mu = props[2 * l + 1] * 1e3;
      LabelOptics &o = plan->lut[l];
      o.alog = (float)(mu * thickness);
      o.kret = (float)(M_PI_2 * (dn * 4.0 * thickness / lambda));
      if (dn == 0 || l == 0)
         o.kind = (mu == 0) ? 0 : 1; // simulator.cpp:280-288
      else
         o.kind = 2;
      o.pad = 0;
   }
   P.kind_packed = n_props <= 16 ? 1 : 0;
   P.kind_mask = 0;
   for (int64_t l = 0; l < n_props && l < 16; l++)
      P.kind_mask |= (uint32_t)plan->lut[l].kind << (2 * l);

   // tilt (simulator.cpp:216-231, 585-590)
   double rot[9];
   rot_zyz(phi, theta, -phi, rot);
   for (int i = 0; i < 9; i++)
      P.rot[i] = (float)rot[i];
   P.rotate = theta != 0 ? 1 : 0;
   const double dir[3] = {pc_cos(phi) * pc_sin(theta), pc_sin(phi) * pc_sin(theta),
                          pc_cos(theta)};
   const double step[3] = {dir[0] * s->step_size, dir[1] * s->step_size,
                           dir[2] * s->step_size};
   const double shift[3] = {dir[0] / std::cos(theta) * (double)P.Z,
                            dir[1] / std::cos(theta) * (double)P.Z,
                            dir[2] / std::cos(theta) * (double)P.Z};
   for (int i = 0; i < 3; i++)
      P.hstep[i] = step[i] * 0.5;
   P.hshift[0] = 0.5 * shift[0];
   P.hshift[1] = 0.5 * shift[1];
   P.shift[0] = shift[0];
   P.shift[1] = shift[1];
   if (!P.untilt) { // CalcStartingLightPositionsTilted (simulator.cpp:628-668)
      const double ang = std::asin(std::sin(-theta) * s->tissue_refrection);
      double rt[9];
      rot_zyz(phi, ang, -phi, rt);
      rot_zyz(phi, -ang, -phi, P.rti);
      P.pc[0] = (double)P.X * 0.5;
      P.pc[1] = (double)P.Y * 0.5;
      P.pc[2] = (double)P.Z * 0.5;
      const double t0[3] = {-P.pc[0], -P.pc[1], P.pc[2]};
      const double e1[3] = {1, 0, 0}, e2[3] = {0, 1, 0};
      mat3_vec(rt, t0, P.pt);
      mat3_vec(rt, e1, P.p1);
      mat3_vec(rt, e2, P.p2);
      P.A = P.p1[0];
      P.B = P.p2[0];
      P.C = P.p1[1];
      P.Dd = P.p2[1];
      P.D = P.A * P.Dd - P.C * P.B;
   }

   // replay the z loop (simulator.cpp:230-231, 259-261)
   if (!(step[2] > 0)) {
      set_error("light direction has no positive z component (theta=%g)", theta);
      return FPGB_EINVAL;
   }
   plan->ztab.clear();
   const int64_t cap = std::max<int64_t>(16 * P.Z, 1 << 16);
   for (double z = 0.0 + step[2] * 0.5; std::floor(z) >= 0 && std::floor(z) < (double)P.Z;
        z = z + step[2]) {
      if ((int64_t)plan->ztab.size() >= std::min<int64_t>(cap, 1 << 22)) {
         set_error("step_size too small: more than %lld steps per ray",
                   (long long)plan->ztab.size());
         return FPGB_EINVAL;
      }
      ZStep zs;
      int64_t iz = (int64_t)std::floor(z);
      zs.iz = (int32_t)(P.flip_z ? P.Z - 1 - iz : iz);
      const double zh = z - 0.5;
      const double z0 = std::floor(zh);
      zs.z0 = (int32_t)z0;
      zs.zf = (float)(zh - z0);
      zs.pad = 0;
      plan->ztab.push_back(zs);
   }
   P.n_z = (int32_t)plan->ztab.size();
   // vertical rays that visit every z of their column in order: theta = 0
   // with step 1 (simulator.cpp:259-261 then gives z = k + 1/2); at those
   // exact voxel centres Lerp and Slerp reduce to the voxel's own axis
   // (simulator.cpp:518-519)
   // Lerp / Slerp: the warp-cooperative march (the faster variant on every
   // volume measured; the batched path's autotuner may pick either)
   P.coop = P.mode != 0 ? 1 : 0;
   P.column = 0;
   if (theta == 0 && P.n_z == P.Z && step[0] == 0 && step[1] == 0) {
      bool seq = true;
      for (int32_t k = 0; k < P.n_z && seq; k++) {
         const ZStep &zs = plan->ztab[k];
         seq = zs.iz == (P.flip_z ? P.Z - 1 - k : k) && zs.zf == 0.f && zs.z0 == k;
      }
      P.column = seq ? 1 : 0;
   }
   plan->steps = P.X * P.Y * (int64_t)P.n_z;

   // fixed-point format for x/y: enough integer bits for every position a
   // ray can reach, the rest fraction (at most 52)
   const double reach = std::fabs(shift[0]) + std::fabs(shift[1]) +
                        (double)P.n_z * (std::fabs(step[0]) + std::fabs(step[1])) +
                        (double)std::max(P.X, P.Y) + 4.0;
   int ibits = 1;
   while (std::ldexp(1.0, ibits) < reach && ibits < 62)
      ibits++;
   P.frac_bits = std::min(52, 62 - ibits);
   if (P.frac_bits < 24) {
      set_error("volume too large for the fixed-point ray positions");
      return FPGB_EINVAL;
   }
   P.dx_fx = std::llrint(std::ldexp(step[0], P.frac_bits));
   P.dy_fx = std::llrint(std::ldexp(step[1], P.frac_bits));

   P.i4 = (float)(s->light_intensity / 4.0);
   const int n = s->n_rho;
   for (int r = 0; r < n; r++) {
      P.c2r[r] = (float)std::cos(2.0 * s->filter_rotations[r]);
      P.s2r[r] = (float)std::sin(2.0 * s->filter_rotations[r]);
      // rho_2 = 2 * linspace(0, pi, n, endpoint=False) (epa.py:29)
      const double rho2 = 2.0 * (M_PI / n * r);
      P.epa_sin[r] = (float)std::sin(rho2);
      P.epa_cos[r] = (float)std::cos(rho2);
   }
   return FPGB_OK;
}

// ======================================================================
// device
// ======================================================================
// 7 resident blocks per SM for the per-thread and column kernels (72
// registers: 3% faster than the 80-register default on config 2; 8 blocks
// spill too much); the cooperative kernel keeps the 5 its registers give it
// (6 measured the same).
template <int MODE, bool TILT, bool COOP, bool WIDE>
__global__ void __launch_bounds__(128, COOP ? 6 : 7)
march_rays(const MarchParams P, int64_t unit0, const int32_t *__restrict__ label,
           const float *__restrict__ vec, double *__restrict__ image,
           double *__restrict__ epa_t, double *__restrict__ epa_d, double *__restrict__ epa_r,
           unsigned long long *__restrict__ counters) {
   // launches may cover a range of units, in either order
   const int64_t unit = P.reverse ? unit0 + (int64_t)gridDim.x - 1 - blockIdx.x
                                  : unit0 + (int64_t)blockIdx.x;
   if (!TILT && P.column) { // 128 consecutive vertical rays per block
      const int64_t ray = unit * (int64_t)blockDim.x + threadIdx.x;
      if (ray < P.X * P.Y)
         march_one_ray_column(P, ray, label, vec, image, epa_t, epa_d, epa_r, counters);
      return;
   }
   int64_t ray; // one 4 x 32 tile of rays per block (tile_ray)
   const bool valid = tile_ray<MODE != 0 && COOP>(P, unit, threadIdx.x, ray);
   if (MODE == 0 || !COOP) {
      if (valid)
         march_one_ray<MODE, TILT, WIDE>(P, ray, label, vec, image, epa_t, epa_d, epa_r,
                                         counters);
   } else { // whole warps take part in the cooperative march
      __shared__ CoopScratch scratch[4];
      march_ray_coop<MODE, TILT, WIDE>(P, valid ? ray : 0, valid, label, vec, image, epa_t, epa_d,
                                 epa_r, counters, scratch[threadIdx.x >> 5]);
   }
}

// Full-volume label range check (simulator.cpp:149-167).
__global__ void label_minmax(const int32_t *__restrict__ label, int64_t n,
                             unsigned long long *__restrict__ counters) {
   int mn = INT32_MAX, mx = INT32_MIN;
   const int64_t n4 = (reinterpret_cast<uintptr_t>(label) % 16 == 0) ? n / 4 : 0;
   const int4 *l4 = reinterpret_cast<const int4 *>(label);
   for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
        i += (int64_t)gridDim.x * blockDim.x) {
      const int4 v = __ldg(l4 + i);
      mn = min(mn, min(min(v.x, v.y), min(v.z, v.w)));
      mx = max(mx, max(max(v.x, v.y), max(v.z, v.w)));
   }
   for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
        i += (int64_t)gridDim.x * blockDim.x) {
      const int v = __ldg(label + i);
      mn = min(mn, v);
      mx = max(mx, v);
   }
   for (int o = 16; o > 0; o >>= 1) {
      mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
   }
   if ((threadIdx.x & 31) == 0) {
      // counters[7] holds min + 2^31 and counters[8] max + 2^31 (unsigned order)
      atomicMin(&counters[7], (unsigned long long)((long long)mn + 2147483648LL));
      atomicMax(&counters[8], (unsigned long long)((long long)mx + 2147483648LL));
   }
}

// ======================================================================
// launch
// ======================================================================
namespace {
int sm_count() {
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   return sms > 0 ? sms : 1;
}
} // namespace

// The launch form of the plan: tables copied into caller-provided device
// memory (lut then ztab, 256-byte aligned) and pointed to from P.
static int prepare_march(const MarchPlan &mp, const int32_t *d_label, const float *d_vec,
                         void *d_tables, cudaStream_t st, MarchParams &P) {
   P = mp.prm;
   char *w = static_cast<char *>(d_tables);
   LabelOptics *lut = reinterpret_cast<LabelOptics *>(w);
   w += align_up(sizeof(LabelOptics) * mp.lut.size(), 256);
   ZStep *zt = reinterpret_cast<ZStep *>(w);
   FPGB_CUDA_TRY(cudaMemcpyAsync(lut, mp.lut.data(), sizeof(LabelOptics) * mp.lut.size(),
                                 cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(zt, mp.ztab.data(), sizeof(ZStep) * mp.ztab.size(),
                                 cudaMemcpyHostToDevice, st));
   P.lut = lut;
   P.ztab = zt;
   // 16-byte column loads (Z % 4 == 0) need 16-byte aligned fields
   if (P.Z % 4 == 0 &&
       (reinterpret_cast<uintptr_t>(d_label) % 16 || reinterpret_cast<uintptr_t>(d_vec) % 16))
      P.column = 0;
   return FPGB_OK;
}

static bool march_tilted(const MarchParams &P) {
   return P.rotate || P.dx_fx != 0 || P.dy_fx != 0;
}

// Blocks of one march: 128 consecutive rays each on the column path, else
// one 4 x 32 ray tile each (x-major: tile t holds pixel columns
// 4 (t / ceil(Y / 32)) ..+3).
static int64_t march_units(const MarchParams &P) {
   if (!march_tilted(P) && P.column)
      return (P.X * P.Y + 127) / 128;
   return ((P.X + kRayTileX - 1) / kRayTileX) * ((P.Y + kRayTileY - 1) / kRayTileY);
}

// Launches blocks [u0, u1) of the march.
static int launch_march_units(const MarchParams &P, const int32_t *d_label, const float *d_vec,
                              double *d_image, double *d_t, double *d_d, double *d_r,
                              unsigned long long *d_counters, int64_t u0, int64_t u1,
                              cudaStream_t st) {
   if (u1 <= u0)
      return FPGB_OK;
   const bool tilt = march_tilted(P);
   const unsigned grid = (unsigned)(u1 - u0);
   // separate kernels per march variant: the cooperative one holds shared
   // scratch and more registers, which must not cap the occupancy of the
   // per-thread one
#define FPGB_LAUNCH(M, T, C)                                                               \
   if (narrow)                                                                              \
      march_rays<M, T, C, false><<<grid, 128, 0, st>>>(P, u0, d_label, d_vec, d_image, d_t, \
                                                       d_d, d_r, d_counters);                \
   else                                                                                     \
      march_rays<M, T, C, true><<<grid, 128, 0, st>>>(P, u0, d_label, d_vec, d_image, d_t,  \
                                                      d_d, d_r, d_counters)
   const bool coop = P.coop != 0;
   const bool narrow = march_narrow(P);
   switch (P.mode * 4 + (tilt ? 2 : 0) + (coop ? 1 : 0)) {
   case 0: case 1: FPGB_LAUNCH(0, false, false); break;
   case 2: case 3: FPGB_LAUNCH(0, true, false); break;
   case 4: FPGB_LAUNCH(1, false, false); break;
   case 5: FPGB_LAUNCH(1, false, true); break;
   case 6: FPGB_LAUNCH(1, true, false); break;
   case 7: FPGB_LAUNCH(1, true, true); break;
   case 8: FPGB_LAUNCH(2, false, false); break;
   case 9: FPGB_LAUNCH(2, false, true); break;
   case 10: FPGB_LAUNCH(2, true, false); break;
   default: FPGB_LAUNCH(2, true, true); break;
   }
#undef FPGB_LAUNCH
   FPGB_CUDA_TRY(cudaGetLastError());
   return FPGB_OK;
}

int launch_march(const MarchPlan &mp, const int32_t *d_label, const float *d_vec,
                 double *d_image, double *d_t, double *d_d, double *d_r,
                 void *d_tables, unsigned long long *d_counters, cudaStream_t st) {
   MarchParams P;
   FPGB_TRY(prepare_march(mp, d_label, d_vec, d_tables, st, P));
   // start at the end of the volume the previous device-resident pass
   // (voxelizer or march) finished at: that part is still in L2
   std::atomic<int> &end = l2_end_state();
   P.reverse = end.load(std::memory_order_relaxed);
   end.store(P.reverse ? 0 : 1, std::memory_order_relaxed);
   return launch_march_units(P, d_label, d_vec, d_image, d_t, d_d, d_r, d_counters, 0,
                             march_units(P), st);
}

// Voxel x range [lo, hi] that the rays of march blocks [u0, u1) can read:
// exact on the column path; otherwise the start positions (affine in the
// pixel) at the corners of the blocks' pixel rectangle and their ends after
// n_z steps, widened by 2 voxels (interpolation neighbours, the fixed-point
// step's rounding).
static void march_units_x_range(const MarchParams &P, int64_t u0, int64_t u1, int64_t &lo,
                                int64_t &hi) {
   int64_t cx0, cx1;
   if (!march_tilted(P) && P.column) {
      cx0 = u0 * 128 / P.Y;
      cx1 = (std::min(u1 * 128, P.X * P.Y) - 1) / P.Y;
      lo = cx0;
      hi = cx1;
      return;
   }
   const int64_t nby = (P.Y + kRayTileY - 1) / kRayTileY;
   cx0 = (u0 / nby) * kRayTileX;
   cx1 = std::min(P.X - 1, ((u1 - 1) / nby) * kRayTileX + kRayTileX - 1);
   const double dxd = std::ldexp((double)P.dx_fx, -P.frac_bits) * (double)(P.n_z > 0 ? P.n_z - 1 : 0);
   double mn = INFINITY, mx = -INFINITY;
   for (int64_t cx : {cx0, cx1})
      for (int64_t cy : {(int64_t)0, P.Y - 1}) {
         double sx, sy;
         ray_start(P, cx, cy, sx, sy);
         mn = std::min({mn, sx, sx + dxd});
         mx = std::max({mx, sx, sx + dxd});
      }
   if (!(mn > -1e15 && mx < 1e15)) { // not finite: every slab
      lo = 0;
      hi = P.X - 1;
      return;
   }
   lo = std::max<int64_t>(0, (int64_t)std::floor(mn) - 2);
   hi = std::min<int64_t>(P.X - 1, (int64_t)std::floor(mx) + 2);
}

size_t march_table_bytes(const MarchPlan &mp) {
   return align_up(sizeof(LabelOptics) * mp.lut.size(), 256) +
          align_up(sizeof(ZStep) * mp.ztab.size(), 256);
}

int launch_label_check(const int32_t *d_label, int64_t n, unsigned long long *d_counters,
                       cudaStream_t st) {
   const int64_t blocks = std::min<int64_t>((n / 4 + 255) / 256 + 1, (int64_t)sm_count() * 8);
   label_minmax<<<(unsigned)blocks, 256, 0, st>>>(d_label, n, d_counters);
   FPGB_CUDA_TRY(cudaGetLastError());
   return FPGB_OK;
}

// counters: [0..5] warnings, [6] status, [7] min label + 2^31, [8] max + 2^31
int init_counters(unsigned long long *d_counters, cudaStream_t st) {
   unsigned long long h[kCounterWords] = {0};
   h[7] = ~0ull;
   h[8] = 0;
   FPGB_CUDA_TRY(cudaMemcpyAsync(d_counters, h, sizeof h, cudaMemcpyHostToDevice, st));
   return FPGB_OK;
}

// Reads the counters back (synchronising) and turns status bits and label
// range violations into errors.
int finish_counters(const unsigned long long *d_counters, int64_t n_props, bool checked_all,
                    fpgb_warnings *w, cudaStream_t st) {
   unsigned long long h[kCounterWords];
   FPGB_CUDA_TRY(cudaMemcpyAsync(h, d_counters, sizeof h, cudaMemcpyDeviceToHost, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   if (checked_all) {
      const long long mn = (long long)h[7] - 2147483648LL;
      const long long mx = (long long)h[8] - 2147483648LL;
      if (mn < 0 || mx < 0) {
         set_error("label < 0 detected");
         return FPGB_EINVAL;
      }
      if (mx >= n_props) {
         set_error("label exceed properties.size()");
         return FPGB_EINVAL;
      }
   }
   if (h[6] & kStatusLabelRange) {
      set_error("label < 0 or label exceed properties.size()");
      return FPGB_EINVAL;
   }
   if (w)
      warnings_from_counters(reinterpret_cast<const long long *>(h), w);
   return FPGB_OK;
}

static int run_sim_planned(const MarchPlan &mp, const int32_t *d_label, const float *d_vector,
                           int64_t n_props, double *d_image, double *d_t, double *d_d,
                           double *d_r, fpgb_warnings *warnings, bool check_all,
                           cudaStream_t st) {
   if (!d_label || !d_vector) {
      set_error("run_simulation: null label/vector buffer");
      return FPGB_EINVAL;
   }
   void *tables = nullptr, *counters = nullptr;
   FPGB_TRY(pool_get(kSlotProps, march_table_bytes(mp), &tables, st));
   FPGB_TRY(pool_get(kSlotCounters, sizeof(unsigned long long) * kCounterWords, &counters, st));
   auto *cnt = static_cast<unsigned long long *>(counters);
   FPGB_TRY(init_counters(cnt, st));
   if (check_all)
      FPGB_TRY(launch_label_check(d_label, mp.prm.X * mp.prm.Y * mp.prm.Z, cnt, st));
   FPGB_TRY(launch_march(mp, d_label, d_vector, d_image, d_t, d_d, d_r, tables, cnt, st));
   if (warnings || check_all)
      return finish_counters(cnt, n_props, check_all, warnings, st);
   return FPGB_OK;
}

// Host-buffer march over page-locked label / vector fields: the volume goes
// up in x-slabs on a second stream, and the rays are launched in chunks,
// each as soon as every slab its rays can read (march_units_x_range) is on
// the device, so most of the march runs under the copy.  Same kernels and
// bits as the one-launch march.
// Consecutive chunks that wait for the same slab go out as one launch: a
// chunk alone fills a third of the GPU, and the chunks that need the last
// slab would otherwise run one after another after the copy (measured on
// config 2: 4 slabs / 8 single-chunk launches left 0.47 ms of march after
// the 2.41 ms copy).
// With a page-locked host image, the image rows each launch completes go
// down on a third stream while the later launches run, so only the last
// launch's rows are copied after the march.
constexpr int kUpSlabs = 8, kRayChunks = 32;

// Image rows (pixel columns x) every ray of which lies in blocks [0, u).
static int64_t march_units_rows_done(const MarchParams &P, int64_t u) {
   if (!march_tilted(P) && P.column)
      return std::min(P.X, u * 128 / P.Y);
   return std::min(P.X, (u / ((P.Y + kRayTileY - 1) / kRayTileY)) * kRayTileX);
}

static int run_sim_pipelined(const MarchPlan &mp, const int32_t *label, const float *vector,
                             int32_t *d_label, float *d_vec, int64_t n_props, double *d_img,
                             double *h_image, fpgb_warnings *warnings, cudaStream_t st) {
   const int64_t X = mp.prm.X, row = mp.prm.Y * mp.prm.Z;
   const int64_t img_row = mp.prm.Y * mp.prm.n_rho; // doubles per image row
   void *tables = nullptr, *counters = nullptr;
   FPGB_TRY(pool_get(kSlotProps, march_table_bytes(mp), &tables, st));
   FPGB_TRY(pool_get(kSlotCounters, sizeof(unsigned long long) * kCounterWords, &counters, st));
   auto *cnt = static_cast<unsigned long long *>(counters);
   FPGB_TRY(init_counters(cnt, st));
   MarchParams P;
   FPGB_TRY(prepare_march(mp, d_label, d_vec, tables, st, P));
   cudaStream_t up = nullptr, down = nullptr;
   cudaEvent_t ev[kUpSlabs] = {};
   cudaEvent_t done[kRayChunks + 1] = {};
   int n_done = 0;
   int64_t rows_copied = 0;
   int64_t slab_end[kUpSlabs];
   int rc = FPGB_OK;
   // after a launch: copy the image rows [rows_copied, r1) it completed
   auto copy_rows = [&](int64_t r1) -> int {
      if (!h_image || r1 <= rows_copied)
         return FPGB_OK;
      FPGB_CUDA_TRY(cudaEventCreateWithFlags(&done[n_done], cudaEventDisableTiming));
      FPGB_CUDA_TRY(cudaEventRecord(done[n_done], st));
      FPGB_CUDA_TRY(cudaStreamWaitEvent(down, done[n_done++], 0));
      FPGB_CUDA_TRY(cudaMemcpyAsync(h_image + rows_copied * img_row, d_img + rows_copied * img_row,
                                    sizeof(double) * (r1 - rows_copied) * img_row,
                                    cudaMemcpyDeviceToHost, down));
      rows_copied = r1;
      return FPGB_OK;
   };
   auto run = [&]() -> int {
      FPGB_CUDA_TRY(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking));
      if (h_image)
         FPGB_CUDA_TRY(cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking));
      // the slab copies must not start before the stream's earlier work
      // (the previous call's march may still read these buffers)
      FPGB_CUDA_TRY(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
      FPGB_CUDA_TRY(cudaEventRecord(ev[0], st));
      FPGB_CUDA_TRY(cudaStreamWaitEvent(up, ev[0], 0));
      for (int s = 0; s < kUpSlabs; s++) {
         const int64_t x0 = X * s / kUpSlabs, x1 = X * (s + 1) / kUpSlabs;
         slab_end[s] = x1;
         if (x1 > x0) {
            FPGB_CUDA_TRY(cudaMemcpyAsync(d_label + x0 * row, label + x0 * row,
                                          sizeof(int32_t) * (x1 - x0) * row,
                                          cudaMemcpyHostToDevice, up));
            FPGB_CUDA_TRY(cudaMemcpyAsync(d_vec + 3 * x0 * row, vector + 3 * x0 * row,
                                          sizeof(float) * 3 * (x1 - x0) * row,
                                          cudaMemcpyHostToDevice, up));
         }
         if (s > 0)
            FPGB_CUDA_TRY(cudaEventCreateWithFlags(&ev[s], cudaEventDisableTiming));
         FPGB_CUDA_TRY(cudaEventRecord(ev[s], up));
      }
      const int64_t nu = march_units(P);
      int waited = -1;
      int64_t g0 = 0; // first unit of the pending launch
      for (int c = 0; c < kRayChunks; c++) {
         const int64_t u0 = nu * c / kRayChunks, u1 = nu * (c + 1) / kRayChunks;
         if (u1 <= u0)
            continue;
         int64_t lo, hi;
         march_units_x_range(P, u0, u1, lo, hi);
         int s = 0;
         while (s < kUpSlabs - 1 && slab_end[s] <= hi)
            s++;
         s = std::max(s, waited);
         if (s > waited && u0 > g0) { // launch the chunks that the slabs so far cover
            FPGB_TRY(launch_march_units(P, d_label, d_vec, d_img, nullptr, nullptr, nullptr,
                                        cnt, g0, u0, st));
            FPGB_TRY(copy_rows(march_units_rows_done(P, u0)));
            g0 = u0;
         }
         if (s > waited) {
            FPGB_CUDA_TRY(cudaStreamWaitEvent(st, ev[s], 0));
            waited = s;
         }
      }
      FPGB_TRY(launch_march_units(P, d_label, d_vec, d_img, nullptr, nullptr, nullptr, cnt, g0,
                                  nu, st));
      FPGB_TRY(copy_rows(X)); // every launch is done: all remaining rows
      if (waited < kUpSlabs - 1)
         FPGB_CUDA_TRY(cudaStreamWaitEvent(st, ev[kUpSlabs - 1], 0));
      return launch_label_check(d_label, X * row, cnt, st);
   };
   rc = run();
   for (cudaStream_t s : {up, down})
      if (s) {
         cudaStreamSynchronize(s);
         cudaStreamDestroy(s);
      }
   for (cudaEvent_t e : ev)
      if (e)
         cudaEventDestroy(e);
   for (cudaEvent_t e : done)
      if (e)
         cudaEventDestroy(e);
   FPGB_TRY(rc);
   return finish_counters(cnt, n_props, true, warnings, st);
}

static int run_sim_device(const fpgb_setup *setup, const int64_t *dim, const int32_t *d_label,
                          const float *d_vector, const double *props, int64_t n_props,
                          double theta, double phi, double *d_image, double *d_t, double *d_d,
                          double *d_r, fpgb_warnings *warnings, bool check_all,
                          cudaStream_t st) {
   MarchPlan mp;
   FPGB_TRY(plan_march(setup, dim, props, n_props, theta, phi, &mp));
   return run_sim_planned(mp, d_label, d_vector, n_props, d_image, d_t, d_d, d_r, warnings,
                          check_all, st);
}

// The streams a multi-tilt call spreads its tilts over (per device, created
// on first use and kept for the process), and the lock that keeps two
// calls' work on them in one order: a tilt's tables live in the stream's
// pool slot, so one call's uploads must not land between another call's
// upload and march on the same stream.
constexpr int kTiltStreams = 4;

static std::mutex &tilt_issue_mutex() {
   static std::mutex mu;
   return mu;
}

static int tilt_streams(cudaStream_t *out) { // caller holds tilt_issue_mutex
   static cudaStream_t streams[64][kTiltStreams] = {};
   int dev = 0;
   FPGB_CUDA_TRY(cudaGetDevice(&dev));
   if (dev < 0 || dev >= 64) {
      set_error("run_simulations: device %d out of range", dev);
      return FPGB_EINVAL;
   }
   for (int i = 0; i < kTiltStreams; i++) {
      if (!streams[dev][i])
         FPGB_CUDA_TRY(cudaStreamCreateWithFlags(&streams[dev][i], cudaStreamNonBlocking));
      out[i] = streams[dev][i];
   }
   return FPGB_OK;
}

} // namespace fpgb

using namespace fpgb;

extern "C" {

int64_t fpgb_count_steps(const fpgb_setup *setup, const int64_t *dim, double theta,
                         double phi) {
   MarchPlan mp;
   const double props[2] = {0.0, 0.0};
   if (plan_march(setup, dim, props, 1, theta, phi, &mp) != FPGB_OK)
      return -1;
   return mp.steps;
}

int fpgb_run_simulation_device(const fpgb_setup *setup, const int64_t *dim,
                               const int32_t *d_label, const float *d_vector,
                               const double *props, int64_t n_props, double theta, double phi,
                               double *d_image, fpgb_warnings *warnings, void *stream) {
   if (!d_image) {
      set_error("run_simulation: null image buffer");
      return FPGB_EINVAL;
   }
   return run_sim_device(setup, dim, d_label, d_vector, props, n_props, theta, phi, d_image,
                         nullptr, nullptr, nullptr, warnings, false, as_stream(stream));
}

int fpgb_run_simulation_epa_device(const fpgb_setup *setup, const int64_t *dim,
                                   const int32_t *d_label, const float *d_vector,
                                   const double *props, int64_t n_props, double theta,
                                   double phi, double *d_image, double *d_trans, double *d_dir,
                                   double *d_ret, fpgb_warnings *warnings, void *stream) {
   return run_sim_device(setup, dim, d_label, d_vector, props, n_props, theta, phi, d_image,
                         d_trans, d_dir, d_ret, warnings, false, as_stream(stream));
}

int fpgb_run_simulations_device(const fpgb_setup *setup, const int64_t *dim,
                                const int32_t *d_label, const float *d_vector,
                                const double *props, int64_t n_props, int64_t n_tilts,
                                const double *theta, const double *phi, double *const *d_images,
                                double *const *d_trans, double *const *d_dir,
                                double *const *d_ret, fpgb_warnings *warnings, void *stream) {
   if (n_tilts < 0 || (n_tilts > 0 && (!theta || !phi || !d_images))) {
      set_error("run_simulations: null tilt or image arrays");
      return FPGB_EINVAL;
   }
   if (!d_label || !d_vector) {
      set_error("run_simulation: null label/vector buffer");
      return FPGB_EINVAL;
   }
   // every tilt is planned (and its setup errors raised) before device work
   std::vector<MarchPlan> plans((size_t)n_tilts);
   for (int64_t k = 0; k < n_tilts; k++) {
      FPGB_TRY(plan_march(setup, dim, props, n_props, theta[k], phi[k], &plans[k]));
      if (!d_images[k]) {
         set_error("run_simulation: null image buffer");
         return FPGB_EINVAL;
      }
   }
   if (n_tilts == 0)
      return FPGB_OK;
   cudaStream_t st = as_stream(stream);
   void *counters = nullptr;
   FPGB_TRY(pool_get(kSlotCounters, sizeof(unsigned long long) * kCounterWords * n_tilts,
                     &counters, st));
   auto *cnt = static_cast<unsigned long long *>(counters);
   {
      std::lock_guard<std::mutex> lk(tilt_issue_mutex());
      cudaStream_t side[kTiltStreams];
      FPGB_TRY(tilt_streams(side));
      const int n_side = (int)std::min<int64_t>(n_tilts, kTiltStreams);
      std::vector<cudaEvent_t> evs;
      auto event_on = [&](cudaStream_t from, cudaStream_t to) -> int {
         cudaEvent_t e;
         FPGB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
         evs.push_back(e);
         FPGB_CUDA_TRY(cudaEventRecord(e, from));
         FPGB_CUDA_TRY(cudaStreamWaitEvent(to, e, 0));
         return FPGB_OK;
      };
      int joined = 0; // side streams that started after the caller's work
      auto issue = [&]() -> int {
         for (; joined < n_side; joined++)
            FPGB_TRY(event_on(st, side[joined]));
         for (int64_t k = 0; k < n_tilts; k++) {
            cudaStream_t s = side[k % kTiltStreams];
            void *tables = nullptr;
            FPGB_TRY(pool_get(kSlotProps, march_table_bytes(plans[k]), &tables, s));
            FPGB_TRY(init_counters(cnt + k * kCounterWords, s));
            FPGB_TRY(launch_march(plans[k], d_label, d_vector, d_images[k],
                                  d_trans ? d_trans[k] : nullptr, d_dir ? d_dir[k] : nullptr,
                                  d_ret ? d_ret[k] : nullptr, tables, cnt + k * kCounterWords,
                                  s));
         }
         return FPGB_OK;
      };
      int rc = issue();
      // the caller's stream waits for whatever was queued, also after an error
      for (int i = 0; i < joined; i++) {
         const int j = event_on(side[i], st);
         rc = rc == FPGB_OK ? j : rc;
      }
      for (cudaEvent_t e : evs)
         cudaEventDestroy(e);
      FPGB_TRY(rc);
   }
   if (warnings)
      for (int64_t k = 0; k < n_tilts; k++)
         FPGB_TRY(finish_counters(cnt + k * kCounterWords, n_props, false, &warnings[k], st));
   return FPGB_OK;
}

int fpgb_run_simulation(const fpgb_setup *setup, const int64_t *dim, const int32_t *label,
                        const float *vector, const double *props, int64_t n_props,
                        double theta, double phi, double *image, fpgb_warnings *warnings) {
   MarchPlan mp; // all host-side validation happens before any device work
   FPGB_TRY(plan_march(setup, dim, props, n_props, theta, phi, &mp));
   if (!label || !vector || !image) {
      set_error("run_simulation: null buffer");
      return FPGB_EINVAL;
   }
   const int64_t nvox = dim[0] * dim[1] * dim[2];
   const int64_t npix = dim[0] * dim[1];
   void *d_label = nullptr, *d_vec = nullptr, *d_img = nullptr;
   FPGB_TRY(pool_get(kSlotLabel, sizeof(int32_t) * nvox, &d_label));
   FPGB_TRY(pool_get(kSlotVector, sizeof(float) * 3 * nvox, &d_vec));
   FPGB_TRY(pool_get(kSlotImage, sizeof(double) * npix * setup->n_rho, &d_img));
   cudaStream_t st = nullptr;
   prefault_host(image, sizeof(double) * npix * setup->n_rho);
   fpgb_warnings tmp;
   if (host_pinned(label) && host_pinned(vector)) {
      // a page-locked image takes its rows as the launches complete them
      double *rows = host_pinned(image) ? image : nullptr;
      FPGB_TRY(run_sim_pipelined(mp, label, vector, (int32_t *)d_label, (float *)d_vec, n_props,
                                 (double *)d_img, rows, warnings ? warnings : &tmp, st));
      if (rows)
         return FPGB_OK;
   } else {
      FPGB_CUDA_TRY(cudaMemcpyAsync(d_label, label, sizeof(int32_t) * nvox,
                                    cudaMemcpyHostToDevice, st));
      FPGB_CUDA_TRY(cudaMemcpyAsync(d_vec, vector, sizeof(float) * 3 * nvox,
                                    cudaMemcpyHostToDevice, st));
      FPGB_TRY(run_sim_planned(mp, (const int32_t *)d_label, (const float *)d_vec, n_props,
                               (double *)d_img, nullptr, nullptr, nullptr,
                               warnings ? warnings : &tmp, true, st));
   }
   FPGB_CUDA_TRY(cudaMemcpyAsync(image, d_img, sizeof(double) * npix * setup->n_rho,
                                 cudaMemcpyDeviceToHost, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   return FPGB_OK;
}

} // extern "C"
