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
#include <vector>

#include "fpgb_common.cuh"
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
struct F3 {
   float x, y, z;
};
__device__ __forceinline__ bool is_zero(F3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ F3 load_vec(const float *__restrict__ vec, int64_t idx) {
   const float *p = vec + 3 * idx;
   return F3{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}

// LinearOrientationInterpolation / VectorOrientationAddition
// (simulator.cpp:449-471)
__device__ __forceinline__ F3 lerp_axis(F3 v, F3 u, float t) {
   if (is_zero(v))
      return u;
   if (is_zero(u))
      return v;
   const F3 a{v.x * (1.f - t), v.y * (1.f - t), v.z * (1.f - t)};
   const F3 b{u.x * t, u.y * t, u.z * t};
   if (dot3(a, b) >= 0.f)
      return F3{a.x + b.x, a.y + b.y, a.z + b.z};
   return F3{a.x - b.x, a.y - b.y, a.z - b.z};
}

// sin(sqrt(y)) / sqrt(y) by its Taylor series in y = x^2, truncated after
// y^5 (remainder < y^6 / 13! <= 4e-13 for y <= 0.36)
__device__ __forceinline__ float sinc_sq(float y) {
   float p = -1.f / 39916800.f;
   p = fmaf(p, y, 1.f / 362880.f);
   p = fmaf(p, y, -1.f / 5040.f);
   p = fmaf(p, y, 1.f / 120.f);
   p = fmaf(p, y, -1.f / 6.f);
   return fmaf(p, y, 1.f);
}

// SphericalInterpolation (simulator.cpp:473-494) in FP32.  The weights
// sin((1-t)th)/sin(th) and sin(t th)/sin(th) are evaluated as
// (1-t) S((1-t)^2 th^2) / S(th^2) and t S(t^2 th^2) / S(th^2), S(y) =
// sin(sqrt y)/sqrt y, for th < 0.6 (smooth fibre fields), which needs no
// sine calls and stays accurate as th -> 0; larger angles use sinf.
__device__ __forceinline__ F3 slerp_axis(F3 v, F3 u, float t) {
   if (is_zero(v))
      return u;
   if (is_zero(u))
      return v;
   float d = dot3(v, u);
   if (d < 0.f) {
      u = F3{-u.x, -u.y, -u.z};
      d = -d;
   }
   const F3 df{v.x - u.x, v.y - u.y, v.z - u.z};
   if (dot3(df, df) < 1e-12f)
      return v;
   const float c = fminf(d * rsqrtf(dot3(v, v) * dot3(u, u)), 1.f);
   const float th = acosf(c);
   float w0, w1;
   if (th < 0.6f) {
      const float y = th * th, s = 1.f - t;
      const float inv = __fdividef(1.f, sinc_sq(y));
      w0 = s * sinc_sq(s * s * y) * inv;
      w1 = t * sinc_sq(t * t * y) * inv;
   } else {
      const float inv = __fdividef(1.f, sinf(th));
      w0 = sinf((1.f - t) * th) * inv;
      w1 = sinf(t * th) * inv;
   }
   return F3{v.x * w0 + u.x * w1, v.y * w0 + u.y * w1, v.z * w0 + u.z * w1};
}

template <int MODE>
__device__ __forceinline__ F3 interp_axis(F3 v, F3 u, float t) {
   if (MODE == 1)
      return lerp_axis(v, u, t);
   return slerp_axis(v, u, t);
}

__device__ __forceinline__ int64_t clampi(int64_t v, int64_t hi) {
   return v < 0 ? 0 : (v > hi ? hi : v);
}

// Trilinear axis interpolation over same-label neighbours
// (simulator.cpp:496-555).  fx, fy: fixed-point positions of the ray.
template <int MODE>
__device__ F3 axis_interp(const MarchParams &P, const int32_t *__restrict__ label,
                          const float *__restrict__ vec, int64_t px, int64_t py,
                          const ZStep &zs, int lab) {
   const int F = P.frac_bits;
   const int64_t half = int64_t(1) << (F - 1);
   const int64_t hx = px - half, hy = py - half;
   const int64_t fx0 = hx >> F, fy0 = hy >> F;
   const uint64_t mask = (uint64_t(1) << F) - 1;
   const float scale = __int_as_float((127 - F) << 23); // 2^-F
   const float xf = (float)(int64_t)((uint64_t)hx & mask) * scale;
   const float yf = (float)(int64_t)((uint64_t)hy & mask) * scale;
   const int64_t x0 = clampi(fx0, P.X - 1), x1 = clampi(fx0 + (xf != 0.f), P.X - 1);
   const int64_t y0 = clampi(fy0, P.Y - 1), y1 = clampi(fy0 + (yf != 0.f), P.Y - 1);
   int64_t z0 = clampi(zs.z0, P.Z - 1), z1 = clampi((int64_t)zs.z0 + (zs.zf != 0.f), P.Z - 1);
   const float xd = (x0 != x1) ? xf : 0.f;
   const float yd = (y0 != y1) ? yf : 0.f;
   const float zd = (z0 != z1) ? zs.zf : 0.f;
   if (P.flip_z) {
      z0 = P.Z - 1 - z0;
      z1 = P.Z - 1 - z1;
   }
   const int64_t YZ = P.Y * P.Z;
   const bool ax = x0 != x1, ay = y0 != y1, az = z0 != z1;
   if (!ax && !ay && !az)
      return load_vec(vec, x0 * YZ + y0 * P.Z + z0);
   // Corners along a collapsed axis coincide, and interpolating a vector
   // with itself returns it unchanged (both the reference's Lerp and Slerp),
   // so collapsed levels are skipped without changing the result.
   F3 c[8];
#pragma unroll
   for (int k = 0; k < 8; k++) {
      if (((k & 1) && !ax) || ((k & 2) && !ay) || ((k & 4) && !az))
         continue;
      const int64_t xi = (k & 1) ? x1 : x0, yi = (k & 2) ? y1 : y0, zi = (k & 4) ? z1 : z0;
      const int64_t idx = xi * YZ + yi * P.Z + zi;
      if (__ldg(label + idx) == lab)
         c[k] = load_vec(vec, idx);
      else
         c[k] = F3{0.f, 0.f, 0.f};
   }
   F3 c00 = c[0], c10 = c[2], c01 = c[4], c11 = c[6];
   if (ax) {
      c00 = interp_axis<MODE>(c[0], c[1], xd);
      if (az)
         c01 = interp_axis<MODE>(c[4], c[5], xd);
      if (ay) {
         c10 = interp_axis<MODE>(c[2], c[3], xd);
         if (az)
            c11 = interp_axis<MODE>(c[6], c[7], xd);
      }
   }
   F3 c0 = c00, c1 = c01;
   if (ay) {
      c0 = interp_axis<MODE>(c00, c10, yd);
      if (az)
         c1 = interp_axis<MODE>(c01, c11, yd);
   }
   if (az)
      return interp_axis<MODE>(c0, c1, zd);
   return c0;
}

// Ray start in the reference's double operation order
// (simulator.cpp:663-681, 735-736, 230-231); explicit _rn intrinsics keep
// every product and sum separately rounded.
__device__ __forceinline__ void ray_start(const MarchParams &P, int64_t cx, int64_t cy,
                                          double &sx, double &sy) {
   const double ex = __dadd_rn((double)cx, 0.5), ey = __dadd_rn((double)cy, 0.5);
   if (P.untilt) {
      sx = __dadd_rn(__dadd_rn(ex, -P.hshift[0]), P.hstep[0]);
      sy = __dadd_rn(__dadd_rn(ey, -P.hshift[1]), P.hstep[1]);
      return;
   }
   const double e = __dadd_rn(__dadd_rn(ex, -P.pc[0]), -P.pt[0]);
   const double f = __dadd_rn(__dadd_rn(ey, -P.pc[1]), -P.pt[1]);
   const double Ds = __dadd_rn(__dmul_rn(e, P.Dd), -__dmul_rn(f, P.B));
   const double Dt = __dadd_rn(__dmul_rn(P.A, f), -__dmul_rn(P.C, e));
   const double s = __ddiv_rn(Ds, P.D), t = __ddiv_rn(Dt, P.D);
   double rel[3];
#pragma unroll
   for (int i = 0; i < 3; i++) {
      const double p = __dadd_rn(__dadd_rn(__dadd_rn(P.pc[i], P.pt[i]), __dmul_rn(P.p1[i], s)),
                                 __dmul_rn(P.p2[i], t));
      rel[i] = __dadd_rn(p, -P.pc[i]);
   }
   double tis[2];
#pragma unroll
   for (int i = 0; i < 2; i++) {
      double a = __dmul_rn(rel[0], P.rti[3 * i + 0]);
      a = __dadd_rn(a, __dmul_rn(rel[1], P.rti[3 * i + 1]));
      a = __dadd_rn(a, __dmul_rn(rel[2], P.rti[3 * i + 2]));
      tis[i] = __dadd_rn(a, P.pc[i]);
   }
   sx = __dadd_rn(__dadd_rn(tis[0], -P.shift[0]), P.hstep[0]);
   sy = __dadd_rn(__dadd_rn(tis[1], -P.shift[1]), P.hstep[1]);
}

// Fixed point with an exact integer part: floor(v) is kept as is and only
// the fraction is truncated to frac_bits, so the first voxel index of the
// ray is exactly the reference's floor() of its double start.
__device__ __forceinline__ int64_t to_fixed(double v, int frac_bits) {
   const double fl = floor(v);
   const int64_t i = (int64_t)fl;
   const int64_t f = (int64_t)floor(ldexp(v - fl, frac_bits));
   return i * (int64_t(1) << frac_bits) + f;
}

// sin and cos of a small angle by their Taylor series (|x| <= 0.25:
// remainders below x^9/9! and x^10/10!, under 1e-11); larger angles use
// sincosf.
__device__ __forceinline__ void sincos_small(float x, float &s, float &c) {
   if (fabsf(x) <= 0.25f) {
      const float y = x * x;
      float ps = -1.f / 5040.f;
      ps = fmaf(ps, y, 1.f / 120.f);
      ps = fmaf(ps, y, -1.f / 6.f);
      s = fmaf(ps * y, x, x);
      float pc = 1.f / 40320.f;
      pc = fmaf(pc, y, -1.f / 720.f);
      pc = fmaf(pc, y, 1.f / 24.f);
      pc = fmaf(pc, y, -0.5f);
      c = fmaf(pc, y, 1.f);
   } else {
      sincosf(x, &s, &c);
   }
}

// One birefringent step on the unit state (u1, u2, u3).
__device__ __forceinline__ void retard(float &u1, float &u2, float &u3, F3 v, float n2,
                                       float kret) {
   const float xx = v.x * v.x, yy = v.y * v.y;
   const float q = xx + yy;
   if (q > 0.f) {
      const float ret = kret * q * rsqrtf(n2);
      float sr, cr;
      sincos_small(ret, sr, cr);
      const float iq = __fdividef(1.f, q);
      const float c = (xx - yy) * iq, s = 2.f * v.x * v.y * iq;
      const float a1 = u1 * c - u2 * s;
      const float c1 = u1 * s + u2 * c;
      const float b1 = c1 * cr + u3 * sr;
      u3 = -c1 * sr + u3 * cr;
      u1 = a1 * c + b1 * s;
      u2 = -a1 * s + b1 * c;
   }
}

template <int MODE, bool TILT>
__global__ void __launch_bounds__(128)
march_rays(const MarchParams P, const int32_t *__restrict__ label,
           const float *__restrict__ vec, double *__restrict__ image,
           double *__restrict__ epa_t, double *__restrict__ epa_d, double *__restrict__ epa_r,
           unsigned long long *__restrict__ counters) {
   const int64_t n_rays = P.X * P.Y;
   const int64_t ray = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
   if (ray >= n_rays)
      return;
   const int64_t cx = ray / P.Y, cy = ray - (ray / P.Y) * P.Y;
   const int F = P.frac_bits;
   int64_t px, py;
   {
      double sx, sy;
      ray_start(P, cx, cy, sx, sy);
      px = to_fixed(sx, F);
      py = to_fixed(sy, F);
   }
   const int64_t YZ = P.Y * P.Z;
   float u1 = 0.f, u2 = 0.f, u3 = -1.f, L = 0.f;
   bool w_zero = false, w_norm = false, bad_label = false;
   int64_t ix = px >> F, iy = py >> F;
   bool inside = ix >= 0 && ix < P.X && iy >= 0 && iy < P.Y;
   for (int k = 0; k < P.n_z; k++) {
      if (TILT && k > 0) {
         px += P.dx_fx;
         py += P.dy_fx;
         ix = px >> F;
         iy = py >> F;
         inside = ix >= 0 && ix < P.X && iy >= 0 && iy < P.Y;
      }
      const ZStep zs = P.ztab[k];
      int lab = 0;
      int64_t idx = 0;
      if (inside) {
         idx = ix * YZ + iy * P.Z + zs.iz;
         lab = __ldg(label + idx);
         if (lab < 0 || lab >= P.n_props) {
            bad_label = true;
            lab = 0;
         }
      }
      const LabelOptics o = P.lut[lab];
      if (o.kind == 0)
         continue;
      if (o.kind == 1) {
         L += o.alog;
         continue;
      }
      F3 v;
      if (MODE == 0)
         v = load_vec(vec, idx);
      else
         v = axis_interp<MODE>(P, label, vec, px, py, zs, lab);
      if (is_zero(v)) { // simulator.cpp:292-297: no attenuation either
         w_zero = true;
         continue;
      }
      const float n2 = dot3(v, v);
      if (n2 - 1.f > 1e-5f)
         w_norm = true;
      if (TILT && P.rotate) {
         v = F3{P.rot[0] * v.x + P.rot[1] * v.y + P.rot[2] * v.z,
                P.rot[3] * v.x + P.rot[4] * v.y + P.rot[5] * v.z,
                P.rot[6] * v.x + P.rot[7] * v.y + P.rot[8] * v.z};
      }
      retard(u1, u2, u3, v, n2, o.kret);
      L += o.alog;
   }
   // analyser and the rho epilogue (simulator.cpp:346-362)
   const float amp = P.i4 * expf(-L);
   float a0 = 0.f, a1 = 0.f, b1 = 0.f;
   double *out = image + ray * P.n_rho;
   for (int r = 0; r < P.n_rho; r++) {
      const float I = amp * (1.f - u1 * P.c2r[r] + u2 * P.s2r[r]);
      if (image)
         out[r] = (double)I;
      a0 += I;
      a1 += I * P.epa_sin[r];
      b1 += I * P.epa_cos[r];
   }
   if (epa_t || epa_d || epa_r) { // epa.py:31-43
      const float n = (float)P.n_rho;
      a0 = a0 / n;
      a1 = 2.f * a1 / n;
      b1 = 2.f * b1 / n;
      if (epa_t)
         epa_t[ray] = 2.0 * (double)a0;
      if (epa_d) {
         float d = 0.5f * atan2f(-b1, a1) + 3.14159265358979f;
         if (d >= 3.14159265358979f)
            d -= 3.14159265358979f;
         epa_d[ray] = (double)d;
      }
      if (epa_r) {
         if ((double)a0 < 2.220446049250313e-16 * 100)
            a0 = 1.f;
         epa_r[ray] = (double)(sqrtf(a1 * a1 + b1 * b1) / a0);
      }
   }
   if (w_zero)
      atomicAdd(&counters[2], 1ull);
   if (w_norm)
      atomicAdd(&counters[3], 1ull);
   if (bad_label)
      atomicOr(&counters[6], (unsigned long long)kStatusLabelRange);
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

int launch_march(const MarchPlan &mp, const int32_t *d_label, const float *d_vec,
                 double *d_image, double *d_t, double *d_d, double *d_r,
                 void *d_tables, unsigned long long *d_counters, cudaStream_t st) {
   MarchParams P = mp.prm;
   // tables: lut then ztab, 256-byte aligned, in caller-provided device memory
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
   const int64_t n_rays = P.X * P.Y;
   const unsigned grid = (unsigned)((n_rays + 127) / 128);
   const bool tilt = P.rotate || P.dx_fx != 0 || P.dy_fx != 0;
#define FPGB_LAUNCH(M, T)                                                                  \
   march_rays<M, T><<<grid, 128, 0, st>>>(P, d_label, d_vec, d_image, d_t, d_d, d_r, d_counters)
   switch (P.mode * 2 + (tilt ? 1 : 0)) {
   case 0: FPGB_LAUNCH(0, false); break;
   case 1: FPGB_LAUNCH(0, true); break;
   case 2: FPGB_LAUNCH(1, false); break;
   case 3: FPGB_LAUNCH(1, true); break;
   case 4: FPGB_LAUNCH(2, false); break;
   default: FPGB_LAUNCH(2, true); break;
   }
#undef FPGB_LAUNCH
   FPGB_CUDA_TRY(cudaGetLastError());
   return FPGB_OK;
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
   FPGB_CUDA_TRY(cudaMemcpyAsync(d_label, label, sizeof(int32_t) * nvox,
                                 cudaMemcpyHostToDevice, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(d_vec, vector, sizeof(float) * 3 * nvox,
                                 cudaMemcpyHostToDevice, st));
   fpgb_warnings tmp;
   FPGB_TRY(run_sim_planned(mp, (const int32_t *)d_label, (const float *)d_vec, n_props,
                            (double *)d_img, nullptr, nullptr, nullptr,
                            warnings ? warnings : &tmp, true, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(image, d_img, sizeof(double) * npix * setup->n_rho,
                                 cudaMemcpyDeviceToHost, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   return FPGB_OK;
}

} // extern "C"
