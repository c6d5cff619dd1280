// Two-float ("double-float") arithmetic: a value is hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits from FP32 instructions.
// Built on Knuth's error-free TwoSum and the FMA-based TwoProduct; these
// are the textbook error-free transformations, written out here.  GB300 runs
// FP64 at a small fraction of its FP32 rate, so the voxelizer evaluates its
// double-precision geometry this way and only drops to FP64 when a result
// lies too close to a float rounding boundary to be decided.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#ifndef FPGB_HD
#define FPGB_HD __host__ __device__ __forceinline__
#endif

namespace fpgb {

struct ff {
   float hi, lo;
};

// exact: a + b = s + e (Knuth TwoSum)
FPGB_HD ff two_sum(float a, float b) {
   const float s = a + b;
   const float bb = s - a;
   const float e = (a - (s - bb)) + (b - bb);
   return ff{s, e};
}

// exact when |a| >= |b| (Dekker FastTwoSum)
FPGB_HD ff quick_two_sum(float a, float b) {
   const float s = a + b;
   const float e = b - (s - a);
   return ff{s, e};
}

// exact: a * b = p + e, using one fused multiply-add
FPGB_HD ff two_prod(float a, float b) {
   const float p = a * b;
   const float e = fmaf(a, b, -p);
   return ff{p, e};
}

FPGB_HD ff ff_from(float a) { return ff{a, 0.f}; }

FPGB_HD ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

FPGB_HD ff ff_add(ff a, ff b) {
   ff s = two_sum(a.hi, b.hi);
   const ff t = two_sum(a.lo, b.lo);
   s.lo += t.hi;
   s = quick_two_sum(s.hi, s.lo);
   s.lo += t.lo;
   return quick_two_sum(s.hi, s.lo);
}

FPGB_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

// Cheaper addition: the two low parts are added in one rounding.  Its error
// is a few units of 2^-48 of |a| + |b| (not of the result), which is the
// form every bound of the voxelizer's fast path is stated in.
FPGB_HD ff ff_add_sloppy(ff a, ff b) {
   ff s = two_sum(a.hi, b.hi);
   s.lo += a.lo + b.lo;
   return quick_two_sum(s.hi, s.lo);
}

FPGB_HD ff ff_sub_sloppy(ff a, ff b) { return ff_add_sloppy(a, ff_neg(b)); }

FPGB_HD ff ff_add_f(ff a, float b) {
   ff s = two_sum(a.hi, b);
   s.lo += a.lo;
   return quick_two_sum(s.hi, s.lo);
}

FPGB_HD ff ff_mul(ff a, ff b) {
   ff p = two_prod(a.hi, b.hi);
   p.lo += a.hi * b.lo + a.lo * b.hi;
   return quick_two_sum(p.hi, p.lo);
}

FPGB_HD ff ff_mul_f(ff a, float b) {
   ff p = two_prod(a.hi, b);
   p.lo += a.lo * b;
   return quick_two_sum(p.hi, p.lo);
}

FPGB_HD ff ff_sqr(ff a) {
   ff p = two_prod(a.hi, a.hi);
   p.lo += 2.f * a.hi * a.lo;
   return quick_two_sum(p.hi, p.lo);
}

// a / b by one correction step of the FP32 quotient
FPGB_HD ff ff_div(ff a, ff b) {
   const float q1 = a.hi / b.hi;
   const ff r = ff_sub(a, ff_mul_f(b, q1));
   const float q2 = r.hi / b.hi;
   const ff r2 = ff_sub(r, ff_mul_f(b, q2));
   const float q3 = r2.hi / b.hi;
   ff q = quick_two_sum(q1, q2);
   return ff_add_f(q, q3);
}

// sqrt(a) for a > 0 by one Newton correction of the FP32 root
FPGB_HD ff ff_sqrt(ff a) {
   const float s = sqrtf(a.hi);
   const ff r = ff_sub(a, two_prod(s, s));
   return quick_two_sum(s, r.hi / (2.f * s));
}

// a / b given r ~ 1/b (any float within a few ulp): two residual
// corrections of the FP32 quotient, no division instruction.
FPGB_HD ff ff_div_rcp(ff a, ff b, float r) {
   const float q1 = a.hi * r;
   const ff e1 = ff_sub_sloppy(a, ff_mul_f(b, q1));
   const float q2 = e1.hi * r;
   const ff e2 = ff_sub_sloppy(e1, ff_mul_f(b, q2));
   const float q3 = e2.hi * r;
   return ff_add_f(quick_two_sum(q1, q2), q3);
}

FPGB_HD ff ff_norm2_sloppy(const ff a[3]) {
   ff s = ff_sqr(a[0]);
   s = ff_add_sloppy(s, ff_sqr(a[1]));
   return ff_add_sloppy(s, ff_sqr(a[2]));
}

FPGB_HD ff ff_dot3(const ff a[3], const ff b[3]) {
   ff s = ff_mul(a[0], b[0]);
   s = ff_add(s, ff_mul(a[1], b[1]));
   return ff_add(s, ff_mul(a[2], b[2]));
}

FPGB_HD ff ff_norm2(const ff a[3]) {
   ff s = ff_sqr(a[0]);
   s = ff_add(s, ff_sqr(a[1]));
   return ff_add(s, ff_sqr(a[2]));
}

// The float nearest to every real in [x - e, x + e], or false when the
// interval straddles a rounding boundary (round-to-nearest-even is
// monotone, so equal roundings of both ends decide every point between).
FPGB_HD bool ff_round_unique(ff x, float e, float &out) {
   const ff lo = ff_add_f(x, -e);
   const ff hi = ff_add_f(x, e);
   if (lo.hi != hi.hi)
      return false;
   out = lo.hi;
   return true;
}

} // namespace fpgb
