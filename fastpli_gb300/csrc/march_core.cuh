// Device side of the ray march shared by the plain kernel (raymarch.cu)
// and the persistent batched kernel (batch.cu).
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
   } else { // th in [0.6, pi/2]: the hardware sine is accurate to ~5e-7 here
      const float inv = __fdividef(1.f, __sinf(th));
      w0 = __sinf((1.f - t) * th) * inv;
      w1 = __sinf(t * th) * inv;
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

// One CCD-pixel ray: start, march, analyser and the rho/epa epilogue.  Used
// by the plain per-call kernel and by the persistent batched kernel, so both
// produce bit-identical images.
template <int MODE, bool TILT>
__device__ __forceinline__ void march_one_ray(const MarchParams &P, int64_t ray,
                                              const int32_t *__restrict__ label,
                                              const float *__restrict__ vec,
                                              double *__restrict__ image,
                                              double *__restrict__ epa_t,
                                              double *__restrict__ epa_d,
                                              double *__restrict__ epa_r,
                                              unsigned long long *__restrict__ counters) {
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
         out[r] = widen(I);
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

} // namespace fpgb
