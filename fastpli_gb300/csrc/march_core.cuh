// Device side of the ray march shared by the plain kernel (raymarch.cu)
// and the persistent batched kernel (batch.cu).
//
// Both translation units are compiled with -fmad=false and the fused
// multiply-adds of the hot arithmetic are written out (fmaf): the compiler
// then contracts nothing on its own, and the same source gives the same bits
// in every kernel that inlines it — plain or batched, per-thread or
// cooperative march, column path — whatever the surrounding code.  (With
// contraction left to the compiler, the same column code inlined into two
// kernels differed in the last bit of a few pixels.)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fpgb_common.cuh"
#include "raymarch.cuh"

namespace fpgb {

struct F3 {
   float x, y, z;
};
__device__ __forceinline__ bool is_zero(F3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
__device__ __forceinline__ float dot3(F3 a, F3 b) {
   return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x));
}

template <typename U>
__device__ __forceinline__ F3 load_vec(const float *__restrict__ vec, U idx) {
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
// y^4 (remainder < y^5 / 11! <= 1.6e-10 for y <= 0.36)
__device__ __forceinline__ float sinc_sq(float y) {
   float p = 1.f / 362880.f;
   p = fmaf(p, y, -1.f / 5040.f);
   p = fmaf(p, y, 1.f / 120.f);
   p = fmaf(p, y, -1.f / 6.f);
   return fmaf(p, y, 1.f);
}

// acos(1 - x)^2 for x = 1 - cos(th) in [0, 1 - cos 0.6]: 2x g(x) with g a
// cubic least-squares fit (on Chebyshev nodes of that interval) of
// g(x) = (2 asin(sqrt(x / 2)))^2 / (2x), relative error < 2e-7.  The
// interpolation weights below depend on th^2 only weakly (their derivative
// in th^2 is below 0.1), so neither this error nor the rounding of
// 1 - cos(th) near th = 0 moves them by more than ~1e-8.
__device__ __forceinline__ float acos_sq(float x) {
   float g = 0.01572742f;
   g = fmaf(g, x, 0.0443475f);
   g = fmaf(g, x, 0.16666762f);
   g = fmaf(g, x, 1.f);
   return (x + x) * g;
}

// SphericalInterpolation (simulator.cpp:473-494) in FP32.  The weights
// sin((1-t)th)/sin(th) and sin(t th)/sin(th) are evaluated as
// (1-t) S((1-t)^2 th^2) / S(th^2) and t S(t^2 th^2) / S(th^2), S(y) =
// sin(sqrt y)/sqrt y, for th < 0.6 (smooth fibre fields), with th^2 taken
// from cos(th) directly (acos_sq): no inverse cosine and no sine calls, and
// accurate as th -> 0.  Larger angles use acosf and the hardware sine.  The
// reference's flip of u (when v.u < 0) is carried as the sign of u's weight.
__device__ __forceinline__ F3 slerp_axis(F3 v, F3 u, float t) {
   if (is_zero(v))
      return u;
   if (is_zero(u))
      return v;
   const float d0 = dot3(v, u);
   const float sg = d0 < 0.f ? -1.f : 1.f;
   const F3 df{fmaf(-sg, u.x, v.x), fmaf(-sg, u.y, v.y), fmaf(-sg, u.z, v.z)};
   if (dot3(df, df) < 1e-12f)
      return v;
   const float c = fminf(fabsf(d0) * rsqrtf(dot3(v, v) * dot3(u, u)), 1.f);
   float w0, w1;
   if (c > 0.825335615f) { // th < 0.6
      const float y = acos_sq(1.f - c), s = 1.f - t;
      const float inv = __fdividef(1.f, sinc_sq(y));
      w0 = s * sinc_sq(s * s * y) * inv;
      w1 = t * sinc_sq(t * t * y) * inv;
   } else { // th in [0.6, pi/2]: the hardware sine is accurate to ~5e-7 here
      const float th = acosf(c);
      const float inv = __fdividef(1.f, __sinf(th));
      w0 = __sinf((1.f - t) * th) * inv;
      w1 = __sinf(t * th) * inv;
   }
   w1 *= sg;
   return F3{fmaf(v.x, w0, u.x * w1), fmaf(v.y, w0, u.y * w1), fmaf(v.z, w0, u.z * w1)};
}

template <int MODE>
__device__ __forceinline__ F3 interp_axis(F3 v, F3 u, float t) {
   if (MODE == 1)
      return lerp_axis(v, u, t);
   return slerp_axis(v, u, t);
}

// Index arithmetic of the march.  Narrow (WIDE = false): coordinates in
// 32-bit integers and the linear voxel index in unsigned 32 bits, for volumes
// with 3 X Y Z < 2^32 whose fixed-point format has frac_bits >= 32 (ray
// positions below 2^30 voxels; march_narrow picks it).  Wide: 64 bits
// throughout.  Both give the same bits.
template <bool WIDE> struct MarchIdx {
   using C = int64_t; // coordinate
   using U = int64_t; // linear voxel index
};
template <> struct MarchIdx<false> {
   using C = int32_t;
   using U = uint32_t;
};

// floor(p / 2^F) of a fixed-point position
template <bool WIDE>
__device__ __forceinline__ typename MarchIdx<WIDE>::C fx_floor(int64_t p, int F) {
   if constexpr (WIDE)
      return p >> F;
   else
      return (int32_t)(p >> 32) >> (F - 32); // F >= 32: one shift of the high word
}

// The fraction of a fixed-point position, truncated to 23 bits and built
// from its bits: exact, no conversion instruction (absolute error < 2^-23,
// far below the image tolerance).  Needs F >= 24.
__device__ __forceinline__ float fx_frac(int64_t p, int F) {
   const uint32_t m = (uint32_t)((uint64_t)p >> (F - 23)) & 0x7FFFFFu;
   return __uint_as_float(0x3F800000u | m) - 1.f;
}

// Whether the position has a nonzero fraction (llceil != llfloor).
__device__ __forceinline__ bool fx_has_frac(int64_t p, int F) {
   return ((uint64_t)p << (64 - F)) != 0;
}

template <typename C> __device__ __forceinline__ C clampc(C v, C hi) {
   return v < 0 ? C(0) : (v > hi ? hi : v);
}

// Linear index (x * Y + y) * Z + z of voxel (x, y, z).
template <bool WIDE>
__device__ __forceinline__ typename MarchIdx<WIDE>::U
voxel_index(const MarchParams &P, typename MarchIdx<WIDE>::C x, typename MarchIdx<WIDE>::C y,
            typename MarchIdx<WIDE>::C z) {
   using U = typename MarchIdx<WIDE>::U;
   return ((U)x * (U)P.Y + (U)y) * (U)P.Z + (U)z;
}

// Trilinear axis interpolation over same-label neighbours
// (simulator.cpp:496-555).  px, py: fixed-point positions of the ray.
template <int MODE, bool WIDE>
__device__ F3 axis_interp(const MarchParams &P, const int32_t *__restrict__ label,
                          const float *__restrict__ vec, int64_t px, int64_t py,
                          const ZStep &zs, int lab) {
   using C = typename MarchIdx<WIDE>::C;
   using U = typename MarchIdx<WIDE>::U;
   const int F = P.frac_bits;
   const int64_t half = int64_t(1) << (F - 1);
   const int64_t hx = px - half, hy = py - half;
   const C fx0 = fx_floor<WIDE>(hx, F), fy0 = fx_floor<WIDE>(hy, F);
   const C xm = (C)P.X - 1, ym = (C)P.Y - 1, zm = (C)P.Z - 1;
   const C x0 = clampc<C>(fx0, xm), x1 = clampc<C>(fx0 + (C)fx_has_frac(hx, F), xm);
   const C y0 = clampc<C>(fy0, ym), y1 = clampc<C>(fy0 + (C)fx_has_frac(hy, F), ym);
   C z0 = clampc<C>((C)zs.z0, zm), z1 = clampc<C>((C)zs.z0 + (C)(zs.zf != 0.f), zm);
   const bool ax = x0 != x1, ay = y0 != y1, az = z0 != z1;
   const float xd = ax ? fx_frac(hx, F) : 0.f;
   const float yd = ay ? fx_frac(hy, F) : 0.f;
   const float zd = az ? zs.zf : 0.f;
   if (P.flip_z) {
      z0 = zm - z0;
      z1 = zm - z1;
   }
   const U base = voxel_index<WIDE>(P, x0, y0, z0);
   if (!ax && !ay && !az)
      return load_vec(vec, base);
   // corner offsets along each axis (the z one is negative when mirrored;
   // unsigned wrap-around then still lands on the right index)
   const U ox = (U)(x1 - x0) * (U)P.Y * (U)P.Z, oy = (U)(y1 - y0) * (U)P.Z, oz = (U)(z1 - z0);
   // Corners along a collapsed axis coincide, and interpolating a vector
   // with itself returns it unchanged (both the reference's Lerp and Slerp),
   // so collapsed levels are skipped without changing the result.
   F3 c[8];
#pragma unroll
   for (int k = 0; k < 8; k++) {
      if (((k & 1) && !ax) || ((k & 2) && !ay) || ((k & 4) && !az))
         continue;
      const U idx = base + ((k & 1) ? ox : U(0)) + ((k & 2) ? oy : U(0)) + ((k & 4) ? oz : U(0));
      // GetVec(...) * (GetLabel(...) == label) (simulator.cpp:533-540)
      const float m = (__ldg(label + idx) == lab) ? 1.f : 0.f;
      const F3 u = load_vec(vec, idx);
      c[k] = F3{u.x * m, u.y * m, u.z * m};
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

// IEEE double add / multiply / divide, each rounded once: the device's _rn
// intrinsics, the host's plain operators (its code is built without
// contraction).
__host__ __device__ __forceinline__ double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
   return __dadd_rn(a, b);
#else
   return a + b;
#endif
}
__host__ __device__ __forceinline__ double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
   return __dmul_rn(a, b);
#else
   return a * b;
#endif
}
__host__ __device__ __forceinline__ double ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
   return __ddiv_rn(a, b);
#else
   return a / b;
#endif
}

// Ray start in the reference's double operation order
// (simulator.cpp:663-681, 735-736, 230-231), every product and sum
// separately rounded.  Host and device: the host bounds which voxels a range
// of rays can reach.
__host__ __device__ __forceinline__ void ray_start(const MarchParams &P, int64_t cx, int64_t cy,
                                          double &sx, double &sy) {
   const double ex = dadd((double)cx, 0.5), ey = dadd((double)cy, 0.5);
   if (P.untilt) {
      sx = dadd(dadd(ex, -P.hshift[0]), P.hstep[0]);
      sy = dadd(dadd(ey, -P.hshift[1]), P.hstep[1]);
      return;
   }
   const double e = dadd(dadd(ex, -P.pc[0]), -P.pt[0]);
   const double f = dadd(dadd(ey, -P.pc[1]), -P.pt[1]);
   const double Ds = dadd(dmul(e, P.Dd), -dmul(f, P.B));
   const double Dt = dadd(dmul(P.A, f), -dmul(P.C, e));
   const double s = ddiv(Ds, P.D), t = ddiv(Dt, P.D);
   double rel[3];
#pragma unroll
   for (int i = 0; i < 3; i++) {
      const double p = dadd(dadd(dadd(P.pc[i], P.pt[i]), dmul(P.p1[i], s)),
                                 dmul(P.p2[i], t));
      rel[i] = dadd(p, -P.pc[i]);
   }
   double tis[2];
#pragma unroll
   for (int i = 0; i < 2; i++) {
      double a = dmul(rel[0], P.rti[3 * i + 0]);
      a = dadd(a, dmul(rel[1], P.rti[3 * i + 1]));
      a = dadd(a, dmul(rel[2], P.rti[3 * i + 2]));
      tis[i] = dadd(a, P.pc[i]);
   }
   sx = dadd(dadd(tis[0], -P.shift[0]), P.hstep[0]);
   sy = dadd(dadd(tis[1], -P.shift[1]), P.hstep[1]);
}

// floor(v * 2^frac_bits) computed exactly with integer operations on the
// bits of v (no FP64 instructions: GB300's FP64 pipe is narrow).  The host
// picks frac_bits so that |v| * 2^frac_bits < 2^62.
__device__ __forceinline__ int64_t to_fixed(double v, int frac_bits) {
   const unsigned long long b = (unsigned long long)__double_as_longlong(v);
   const bool neg = (b >> 63) != 0;
   const int e = (int)((b >> 52) & 0x7FF);
   unsigned long long m = b & ((1ull << 52) - 1);
   if (e == 0) // zero or subnormal: floor is 0 or -1
      return (neg && m) ? -1 : 0;
   m |= 1ull << 52;
   const int sh = e - 1075 + frac_bits; // v * 2^F = m * 2^sh
   unsigned long long q;
   bool rem = false;
   if (sh >= 0) {
      q = m << sh;
   } else if (sh > -64) {
      q = m >> (-sh);
      rem = (m & ((1ull << (-sh)) - 1)) != 0;
   } else {
      q = 0;
      rem = true;
   }
   const long long r = (long long)q;
   return neg ? -(r + (rem ? 1 : 0)) : r;
}

// float -> double by rebuilding the bit pattern with integer operations
// (exact: every float is a double); zero and non-finite values keep their
// meaning, subnormal floats go through the conversion instruction.
__device__ __forceinline__ double widen(float f) {
   const unsigned u = __float_as_uint(f);
   const unsigned ex = (u >> 23) & 0xFFu;
   const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
   const unsigned long long man = (unsigned long long)(u & 0x7FFFFFu) << 29;
   if (ex == 0u) {
      if ((u & 0x7FFFFFu) == 0u)
         return __longlong_as_double((long long)sign);
      return (double)f;
   }
   const unsigned long long e64 = ex == 0xFFu ? 0x7FFull : (unsigned long long)(ex - 127u + 1023u);
   return __longlong_as_double((long long)(sign | (e64 << 52) | man));
}

// sin and cos of the per-step retardance.  Small angles (|x| <= 0.25, the
// common case: about 0.01 rad per 0.2 µm voxel) by their Taylor series
// (remainders below x^9/9! and x^10/10!, under 1e-11); |x| <= pi by the
// hardware sine/cosine (absolute error ~5e-7); beyond that sincosf.
__device__ __forceinline__ void sincos_small(float x, float &s, float &c) {
   if (fabsf(x) > 0.25f) {
      if (fabsf(x) <= 3.14159265f) {
         __sincosf(x, &s, &c);
      } else {
         sincosf(x, &s, &c);
      }
   } else {
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
   }
}

// Analyser and the rho / epa epilogue of one ray (simulator.cpp:346-362,
// epa.py:31-43), plus its warning / status counters.
__device__ __forceinline__ void ray_epilogue(const MarchParams &P, int64_t ray, float u1, float u2,
                                             float L, double *__restrict__ image,
                                             double *__restrict__ epa_t,
                                             double *__restrict__ epa_d,
                                             double *__restrict__ epa_r, bool w_zero,
                                             bool w_norm, bool bad_label,
                                             unsigned long long *__restrict__ counters) {
   const float amp = P.i4 * expf(-L);
   float a0 = 0.f, a1 = 0.f, b1 = 0.f;
   double *out = image + ray * P.n_rho;
   for (int r = 0; r < P.n_rho; r++) {
      const float I = amp * fmaf(u2, P.s2r[r], fmaf(-u1, P.c2r[r], 1.f));
      if (image)
         out[r] = widen(I);
      a0 += I;
      a1 = fmaf(I, P.epa_sin[r], a1);
      b1 = fmaf(I, P.epa_cos[r], b1);
   }
   if (epa_t || epa_d || epa_r) {
      const float n = (float)P.n_rho;
      a0 = a0 / n;
      a1 = 2.f * a1 / n;
      b1 = 2.f * b1 / n;
      if (epa_t)
         epa_t[ray] = widen(2.f * a0);
      if (epa_d) {
         float d = 0.5f * atan2f(-b1, a1) + 3.14159265358979f;
         if (d >= 3.14159265358979f)
            d -= 3.14159265358979f;
         epa_d[ray] = widen(d);
      }
      if (epa_r) {
         if (a0 < 2.220446e-14f)
            a0 = 1.f;
         epa_r[ray] = widen(sqrtf(a1 * a1 + b1 * b1) / a0);
      }
   }
   if (w_zero)
      atomicAdd(&counters[2], 1ull);
   if (w_norm)
      atomicAdd(&counters[3], 1ull);
   if (bad_label)
      atomicOr(&counters[6], (unsigned long long)kStatusLabelRange);
}

// Fixed-point start of ray `ray` (CCD pixel x = ray / Y, y = ray % Y).
__device__ __forceinline__ void ray_setup(const MarchParams &P, int64_t ray, int64_t &px,
                                          int64_t &py) {
   const int64_t cx = ray / P.Y, cy = ray - (ray / P.Y) * P.Y;
   double sx, sy;
   ray_start(P, cx, cy, sx, sy);
   px = to_fixed(sx, P.frac_bits);
   py = to_fixed(sy, P.frac_bits);
}

// The rotation of one birefringent step, from the (tilted) optic axis v and
// |v_untilted|^2 = n2: cos 2phi, sin 2phi, cos ret, sin ret
// (simulator.cpp:309-320).  Returns false when vx = vy = 0 (no rotation).
__device__ __forceinline__ bool retard_params(F3 v, float n2, float kret, float &c, float &s,
                                              float &cr, float &sr) {
   const float xx = v.x * v.x, yy = v.y * v.y;
   const float q = fmaf(v.x, v.x, yy);
   if (!(q > 0.f))
      return false;
   const float ret = kret * q * rsqrtf(n2);
   sincos_small(ret, sr, cr);
   const float iq = __fdividef(1.f, q);
   c = (xx - yy) * iq;
   s = 2.f * v.x * v.y * iq;
   return true;
}

// Apply R(-2phi) Ret R(2phi) to the unit state (simulator.cpp:322-336 in the
// rho-free frame).
__device__ __forceinline__ void apply_retard(float &u1, float &u2, float &u3, float c, float s,
                                             float cr, float sr) {
   const float a1 = fmaf(u1, c, -u2 * s);
   const float c1 = fmaf(u1, s, u2 * c);
   const float b1 = fmaf(c1, cr, u3 * sr);
   u3 = fmaf(-c1, sr, u3 * cr);
   u1 = fmaf(a1, c, b1 * s);
   u2 = fmaf(-a1, s, b1 * c);
}

// One CCD-pixel ray, one thread, every step in order.  The label of step
// k + 1 is loaded while step k is worked on, and a step's kind comes from a
// register mask (labels below 16), so the cheap steps wait on one load
// instead of a chain of two.
template <int MODE, bool TILT, bool WIDE>
__device__ __forceinline__ void march_one_ray(const MarchParams &P, int64_t ray,
                                              const int32_t *__restrict__ label,
                                              const float *__restrict__ vec,
                                              double *__restrict__ image,
                                              double *__restrict__ epa_t,
                                              double *__restrict__ epa_d,
                                              double *__restrict__ epa_r,
                                              unsigned long long *__restrict__ counters) {
   using C = typename MarchIdx<WIDE>::C;
   using U = typename MarchIdx<WIDE>::U;
   const int F = P.frac_bits;
   const int n_z = P.n_z;
   int64_t px, py;
   ray_setup(P, ray, px, py);
   float u1 = 0.f, u2 = 0.f, u3 = -1.f, L = 0.f;
   bool w_zero = false, w_norm = false, bad_label = false;
   const C X = (C)P.X, Y = (C)P.Y;
   C ix = fx_floor<WIDE>(px, F), iy = fx_floor<WIDE>(py, F);
   bool inside = ix >= 0 && ix < X && iy >= 0 && iy < Y;
   U idx = 0;
   int lab = 0;
   if (inside && n_z > 0) {
      idx = voxel_index<WIDE>(P, ix, iy, (C)P.ztab[0].iz);
      lab = __ldg(label + idx);
   }
   for (int k = 0; k < n_z; k++) {
      // next step's position and label
      if (TILT) {
         ix = fx_floor<WIDE>(px + P.dx_fx, F);
         iy = fx_floor<WIDE>(py + P.dy_fx, F);
         inside = ix >= 0 && ix < X && iy >= 0 && iy < Y;
      }
      U idx_n = 0;
      int lab_n = 0;
      if (inside && k + 1 < n_z) {
         idx_n = voxel_index<WIDE>(P, ix, iy, (C)P.ztab[k + 1].iz);
         lab_n = __ldg(label + idx_n);
      }
      // step k
      [&] {
         if (lab < 0 || lab >= P.n_props) { // (0 outside the volume)
            bad_label = true;
            lab = 0;
         }
         const int kind = P.kind_packed ? (int)((P.kind_mask >> (2 * lab)) & 3u)
                                        : P.lut[lab].kind;
         if (kind == 0)
            return;
         const LabelOptics o = P.lut[lab];
         if (kind == 1) {
            L += o.alog;
            return;
         }
         F3 v;
         if (MODE == 0)
            v = load_vec(vec, idx);
         else
            v = axis_interp<MODE, WIDE>(P, label, vec, px, py, P.ztab[k], lab);
         if (is_zero(v)) { // simulator.cpp:292-297: no attenuation either
            w_zero = true;
            return;
         }
         const float n2 = dot3(v, v);
         if (n2 - 1.f > 1e-5f)
            w_norm = true;
         if (TILT && P.rotate) {
            v = F3{dot3(F3{P.rot[0], P.rot[1], P.rot[2]}, v),
                   dot3(F3{P.rot[3], P.rot[4], P.rot[5]}, v),
                   dot3(F3{P.rot[6], P.rot[7], P.rot[8]}, v)};
         }
         float c, s, cr, sr;
         if (retard_params(v, n2, o.kret, c, s, cr, sr))
            apply_retard(u1, u2, u3, c, s, cr, sr);
         L += o.alog;
      }();
      if (TILT) {
         px += P.dx_fx;
         py += P.dy_fx;
      }
      idx = idx_n;
      lab = lab_n;
   }
   ray_epilogue(P, ray, u1, u2, L, image, epa_t, epa_d, epa_r, w_zero, w_norm, bad_label,
                counters);
}

// Rays of a 128-thread block: a 4 (x) x 32 (y) tile of CCD pixels.  The
// per-thread march gives each warp a 4 x 8 patch of it: the 8-corner
// neighbourhoods of the warp's rays then cover 5 x 9 voxel columns instead of
// the 2 x 33 of 32 rays in a line, so more of each step's gathers hit the
// same L1 lines (5% faster on config 2).  The cooperative march keeps a line
// of 32 rays per warp (x fixed), which suits its compaction better.  Returns
// false for tile positions outside the image.
constexpr int kRayTileX = 4, kRayTileY = 32;

template <bool COOP>
__device__ __forceinline__ bool tile_ray(const MarchParams &P, int64_t tile, int tid,
                                         int64_t &ray) {
   const int64_t nby = (P.Y + kRayTileY - 1) / kRayTileY;
   const int w = tid >> 5, l = tid & 31;
   const int64_t x = (tile / nby) * kRayTileX + (COOP ? w : (l >> 3));
   const int64_t y = (tile % nby) * kRayTileY + (COOP ? l : w * 8 + (l & 7));
   ray = x * P.Y + y;
   return x < P.X && y < P.Y;
}

// Vertical ray through its whole column in order (MarchParams::column):
// labels and axes stream in as 16-byte loads, four voxels at a time, when
// Z % 4 == 0 (the column then starts 16-byte aligned), else one voxel at a
// time.  Same arithmetic per step as the warp march, in the same order.  Interpolation modes need nothing else here: at the
// exact voxel centres of such a ray every interpolation axis collapses.
__device__ __forceinline__ void march_one_ray_column(const MarchParams &P, int64_t ray,
                                                     const int32_t *__restrict__ label,
                                                     const float *__restrict__ vec,
                                                     double *__restrict__ image,
                                                     double *__restrict__ epa_t,
                                                     double *__restrict__ epa_d,
                                                     double *__restrict__ epa_r,
                                                     unsigned long long *__restrict__ counters) {
   const int64_t base = ray * P.Z; // ray = cx * Y + cy: its column (cx, cy, 0..Z-1)
   float u1 = 0.f, u2 = 0.f, u3 = -1.f, L = 0.f;
   bool w_zero = false, w_norm = false, bad_label = false;
   // one voxel of the column, in z order (mirrored for flip_z)
   auto step = [&](int lab, const F3 &v) {
      if (lab < 0 || lab >= P.n_props) {
         bad_label = true;
         lab = 0;
      }
      const LabelOptics o = P.lut[lab];
      if (o.kind == 0)
         return;
      if (o.kind == 1) {
         L += o.alog;
         return;
      }
      if (is_zero(v)) {
         w_zero = true;
         return;
      }
      const float n2 = dot3(v, v);
      if (n2 - 1.f > 1e-5f)
         w_norm = true;
      float cc, ss, cr, sr;
      if (retard_params(v, n2, o.kret, cc, ss, cr, sr))
         apply_retard(u1, u2, u3, cc, ss, cr, sr);
      L += o.alog;
   };
   if ((P.Z & 3) == 0) {
      // 16-byte columns: labels and axes stream in four voxels at a time;
      // the next quad's loads are issued before the current quad is processed
      const int4 *lab4 = reinterpret_cast<const int4 *>(label + base);
      const float4 *vec4 = reinterpret_cast<const float4 *>(vec + 3 * base);
      const int nq = (int)(P.Z >> 2);
      int q = P.flip_z ? nq - 1 : 0; // mirrored columns are read backwards
      int4 nl = __ldg(lab4 + q);
      float4 na = __ldg(vec4 + 3 * q), nb = __ldg(vec4 + 3 * q + 1), nc = __ldg(vec4 + 3 * q + 2);
      for (int qi = 0; qi < nq; qi++) {
         const int4 l4 = nl;
         const float4 a = na, b = nb, c = nc;
         if (qi + 1 < nq) {
            q = P.flip_z ? nq - 2 - qi : qi + 1;
            nl = __ldg(lab4 + q);
            na = __ldg(vec4 + 3 * q);
            nb = __ldg(vec4 + 3 * q + 1);
            nc = __ldg(vec4 + 3 * q + 2);
         }
         const int labs[4] = {l4.x, l4.y, l4.z, l4.w};
         const F3 vs[4] = {F3{a.x, a.y, a.z}, F3{a.w, b.x, b.y}, F3{b.z, b.w, c.x},
                           F3{c.y, c.z, c.w}};
#pragma unroll
         for (int jj = 0; jj < 4; jj++) {
            const int j = P.flip_z ? 3 - jj : jj;
            step(labs[j], vs[j]);
         }
      }
   } else {
      // columns of any length (not 16-byte aligned): four voxels at a time
      // with scalar loads, the next four's 16 loads issued before the
      // current four are processed; the last Z % 4 voxels one by one
      const int Z = (int)P.Z, dz = P.flip_z ? -1 : 1;
      const int n4 = Z >> 2;
      int64_t i = base + (P.flip_z ? Z - 1 : 0); // next voxel to load, in step order
      int nl[4];
      float nx[4], ny[4], nz[4];
      auto load4 = [&](int64_t i0) {
#pragma unroll
         for (int j = 0; j < 4; j++) {
            const int64_t ij = i0 + j * dz;
            nl[j] = __ldg(label + ij);
            nx[j] = __ldg(vec + 3 * ij);
            ny[j] = __ldg(vec + 3 * ij + 1);
            nz[j] = __ldg(vec + 3 * ij + 2);
         }
      };
      if (n4 > 0)
         load4(i);
      for (int c = 0; c < n4; c++) {
         int l4[4];
         F3 v4[4];
#pragma unroll
         for (int j = 0; j < 4; j++) {
            l4[j] = nl[j];
            v4[j] = F3{nx[j], ny[j], nz[j]};
         }
         i += 4 * dz;
         if (c + 1 < n4)
            load4(i);
#pragma unroll
         for (int j = 0; j < 4; j++)
            step(l4[j], v4[j]);
      }
      for (int k = 4 * n4; k < Z; k++, i += dz)
         step(__ldg(label + i), F3{__ldg(vec + 3 * i), __ldg(vec + 3 * i + 1),
                                   __ldg(vec + 3 * i + 2)});
   }
   ray_epilogue(P, ray, u1, u2, L, image, epa_t, epa_d, epa_r, w_zero, w_norm, bad_label,
                counters);
}

// ----------------------------------------------------------------------------
// Warp-cooperative march for Lerp/Slerp.  Interpolating the optic axis of a
// birefringent step costs ~20x a plain step, and within a warp different rays
// need it at different steps, so a one-ray-per-thread loop pays it on almost
// every step.  Here each warp takes its 32 rays through kCoopSteps steps at a
// time in three phases:
//   1. every lane classifies its steps (label, optics) and writes one job
//      descriptor per birefringent step into shared memory;
//   2. the warp's jobs are compacted and shared out to all 32 lanes, each job
//      producing that step's rotation (cos 2phi, sin 2phi, cos/sin ret) from
//      the interpolated axis — the interpolated axis of a step depends only on
//      its position, not on the state;
//   3. every lane applies its steps' rotations and attenuations in order.
// The arithmetic per step is the same as march_one_ray's.  Windows of 4 steps
// keep the scratch at 17 KB per 128-thread block: the march lives on L1 hits
// of its 8-corner gathers, and shared memory comes out of the same 256 KB
// (8-step windows: 2.30 ms for config 2's five tilts, 4 steps: 2.12 ms,
// 2 steps: 2.43 ms, the compaction then having too few jobs to fill warps).
// ----------------------------------------------------------------------------
constexpr int kCoopSteps = 4;
constexpr int kCoopSlots = kCoopSteps * 32; // per warp
constexpr int kCoopFields = 8;

struct CoopScratch {
   float f[kCoopFields][kCoopSlots]; // slot = step * 32 + lane
   unsigned short list[kCoopSlots];
};

// job status codes written to field 4
constexpr int kJobRotate = 0, kJobIdentity = 1, kJobZero = 2, kJobNorm = 4;

template <int MODE, bool TILT, bool WIDE>
__device__ __forceinline__ void coop_job(const MarchParams &P, const int32_t *__restrict__ label,
                                         const float *__restrict__ vec, CoopScratch &S,
                                         int slot) {
   const int x0 = __float_as_int(S.f[0][slot]);
   const int y0 = __float_as_int(S.f[1][slot]);
   const int z0 = __float_as_int(S.f[2][slot]);
   const int fl = __float_as_int(S.f[3][slot]);
   const float xd = S.f[4][slot], yd = S.f[5][slot], zd = S.f[6][slot];
   const int lab = __float_as_int(S.f[7][slot]);
   const bool ax = fl & 1, ay = fl & 2, az = fl & 4;
   using C = typename MarchIdx<WIDE>::C;
   using U = typename MarchIdx<WIDE>::U;
   const int dz = ((fl >> 3) & 3) - 1; // z1 - z0
   const U base = voxel_index<WIDE>(P, (C)x0, (C)y0, (C)z0);
   F3 v;
   if (!ax && !ay && !az) {
      v = load_vec(vec, base);
   } else {
      const U ox = (U)P.Y * (U)P.Z, oy = (U)P.Z, oz = (U)(C)dz;
      F3 c[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
         if (((k & 1) && !ax) || ((k & 2) && !ay) || ((k & 4) && !az))
            continue;
         const U idx =
             base + ((k & 1) ? ox : U(0)) + ((k & 2) ? oy : U(0)) + ((k & 4) ? oz : U(0));
         // GetVec(...) * (GetLabel(...) == label) (simulator.cpp:533-540);
         // label and axis loads are issued together
         const float m = (__ldg(label + idx) == lab) ? 1.f : 0.f;
         const F3 u = load_vec(vec, idx);
         c[k] = F3{u.x * m, u.y * m, u.z * m};
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
      v = az ? interp_axis<MODE>(c0, c1, zd) : c0;
   }
   int status;
   float c = 1.f, s = 0.f, cr = 1.f, sr = 0.f;
   if (is_zero(v)) {
      status = kJobZero;
   } else {
      const float n2 = dot3(v, v);
      status = (n2 - 1.f > 1e-5f) ? kJobNorm : 0;
      if (TILT && P.rotate) {
         v = F3{dot3(F3{P.rot[0], P.rot[1], P.rot[2]}, v),
                dot3(F3{P.rot[3], P.rot[4], P.rot[5]}, v),
                dot3(F3{P.rot[6], P.rot[7], P.rot[8]}, v)};
      }
      if (!retard_params(v, n2, P.lut[lab].kret, c, s, cr, sr))
         status |= kJobIdentity;
   }
   S.f[0][slot] = c;
   S.f[1][slot] = s;
   S.f[2][slot] = cr;
   S.f[3][slot] = sr;
   S.f[4][slot] = __int_as_float(status);
}

template <int MODE, bool TILT, bool WIDE>
__device__ __forceinline__ void march_ray_coop(const MarchParams &P, int64_t ray, bool active,
                                               const int32_t *__restrict__ label,
                                               const float *__restrict__ vec,
                                               double *__restrict__ image,
                                               double *__restrict__ epa_t,
                                               double *__restrict__ epa_d,
                                               double *__restrict__ epa_r,
                                               unsigned long long *__restrict__ counters,
                                               CoopScratch &S) {
   using C = typename MarchIdx<WIDE>::C;
   const int lane = threadIdx.x & 31;
   const int F = P.frac_bits;
   int64_t px = 0, py = 0;
   if (active)
      ray_setup(P, ray, px, py);
   const int64_t half = int64_t(1) << (F - 1);
   const C xm = (C)P.X - 1, ym = (C)P.Y - 1, zm = (C)P.Z - 1;
   float u1 = 0.f, u2 = 0.f, u3 = -1.f, L = 0.f;
   bool w_zero = false, w_norm = false, bad_label = false;
   for (int k0 = 0; k0 < P.n_z; k0 += kCoopSteps) {
      // phase 1: classify this lane's steps, write job descriptors
      unsigned kinds = 0; // 2 bits per step
      float alog[kCoopSteps];
#pragma unroll
      for (int j = 0; j < kCoopSteps; j++) {
         const int k = k0 + j;
         alog[j] = 0.f;
         if (!active || k >= P.n_z)
            continue;
         if (TILT && k > 0) {
            px += P.dx_fx;
            py += P.dy_fx;
         }
         const C ix = fx_floor<WIDE>(px, F), iy = fx_floor<WIDE>(py, F);
         const ZStep zs = P.ztab[k];
         int lab = 0;
         if (ix >= 0 && ix <= xm && iy >= 0 && iy <= ym) {
            lab = __ldg(label + voxel_index<WIDE>(P, ix, iy, (C)zs.iz));
            if (lab < 0 || lab >= P.n_props) {
               bad_label = true;
               lab = 0;
            }
         }
         const LabelOptics o = P.lut[lab];
         alog[j] = o.alog;
         kinds |= (unsigned)o.kind << (2 * j);
         if (o.kind != 2)
            continue;
         // trilinear corners as in axis_interp (simulator.cpp:510-530)
         const int64_t hx = px - half, hy = py - half;
         const C fx0 = fx_floor<WIDE>(hx, F), fy0 = fx_floor<WIDE>(hy, F);
         const C x0 = clampc<C>(fx0, xm), x1 = clampc<C>(fx0 + (C)fx_has_frac(hx, F), xm);
         const C y0 = clampc<C>(fy0, ym), y1 = clampc<C>(fy0 + (C)fx_has_frac(hy, F), ym);
         C z0 = clampc<C>((C)zs.z0, zm), z1 = clampc<C>((C)zs.z0 + (C)(zs.zf != 0.f), zm);
         const int ax = x0 != x1, ay = y0 != y1, az = z0 != z1;
         const float xf = ax ? fx_frac(hx, F) : 0.f;
         const float yf = ay ? fx_frac(hy, F) : 0.f;
         const float zd = az ? zs.zf : 0.f;
         if (P.flip_z) {
            z0 = zm - z0;
            z1 = zm - z1;
         }
         const int slot = j * 32 + lane;
         S.f[0][slot] = __int_as_float((int)x0);
         S.f[1][slot] = __int_as_float((int)y0);
         S.f[2][slot] = __int_as_float((int)z0);
         S.f[3][slot] = __int_as_float(ax | (ay << 1) | (az << 2) | ((int)(z1 - z0 + 1) << 3));
         S.f[4][slot] = xf;
         S.f[5][slot] = yf;
         S.f[6][slot] = zd;
         S.f[7][slot] = __int_as_float(lab);
      }
      // phase 2: compact the warp's jobs and share them out
      unsigned jobs = 0;
#pragma unroll
      for (int j = 0; j < kCoopSteps; j++)
         jobs |= (((kinds >> (2 * j)) & 3u) == 2u) ? (1u << j) : 0u;
      const int cnt = __popc(jobs);
      int pre = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
         const int v = __shfl_up_sync(0xffffffffu, pre, o);
         if (lane >= o)
            pre += v;
      }
      const int total = __shfl_sync(0xffffffffu, pre, 31);
      pre -= cnt;
      for (unsigned m = jobs; m; m &= m - 1) {
         const int j = __ffs(m) - 1;
         S.list[pre++] = (unsigned short)(j * 32 + lane);
      }
      __syncwarp();
      for (int t = lane; t < total; t += 32)
         coop_job<MODE, TILT, WIDE>(P, label, vec, S, S.list[t]);
      __syncwarp();
      // phase 3: apply this lane's steps in order
#pragma unroll
      for (int j = 0; j < kCoopSteps; j++) {
         const unsigned kind = (kinds >> (2 * j)) & 3u;
         if (kind == 1u) {
            L += alog[j];
         } else if (kind == 2u) {
            const int slot = j * 32 + lane;
            const int st = __float_as_int(S.f[4][slot]);
            if (st & kJobZero) { // simulator.cpp:292-297: no attenuation either
               w_zero = true;
               continue;
            }
            if (st & kJobNorm)
               w_norm = true;
            if (!(st & kJobIdentity))
               apply_retard(u1, u2, u3, S.f[0][slot], S.f[1][slot], S.f[2][slot],
                            S.f[3][slot]);
            L += alog[j];
         }
      }
      __syncwarp(); // the scratch is rewritten by the next block of steps
   }
   if (active)
      ray_epilogue(P, ray, u1, u2, L, image, epa_t, epa_d, epa_r, w_zero, w_norm, bad_label,
                   counters);
}

} // namespace fpgb
