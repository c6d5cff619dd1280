// Exact (FP64) and two-float evaluation of one (segment, voxel) candidate of
// the voxelizer.  Host+device: the kernels use it, and a host build checks
// the two-float decisions against the FP64 replay.
#pragma once

#include <cmath>

#include "ff.cuh"
#include "tissue.cuh"

namespace fpgb {

// Closest point of `pt` on segment S and its parameter t, in the reference's
// double operation order (generator.cpp:475-494).  -fmad=false keeps every
// product and sum separately rounded.
FPGB_HD void closest_point(const SegDev &S, const double pt[3],
                                              double cl[3], double &t) {
   const double w0 = pt[0] - S.p[0], w1 = pt[1] - S.p[1], w2 = pt[2] - S.p[2];
   double c1 = 0.0;
   c1 = c1 + w0 * S.v[0];
   c1 = c1 + w1 * S.v[1];
   c1 = c1 + w2 * S.v[2];
   if (c1 < 0) {
      cl[0] = S.p[0];
      cl[1] = S.p[1];
      cl[2] = S.p[2];
      t = 0.0;
   } else if (S.c2 <= c1) {
      cl[0] = S.q[0];
      cl[1] = S.q[1];
      cl[2] = S.q[2];
      t = 1.0;
   } else {
      const double b = c1 / S.c2;
      cl[0] = S.p[0] + S.v[0] * b;
      cl[1] = S.p[1] + S.v[1] * b;
      cl[2] = S.p[2] + S.v[2] * b;
      t = b;
   }
}

// FP32 estimate of a candidate's dist^2 from segment-local inputs (w = voxel
// centre - float(p - base), float(v), float(c2), float(1 / c2)), and a bound:
// the float that the reference's double arithmetic produces (exact_dist)
// lies in [d2f - margin, d2f + margin].
//
// The estimate is |w - t v|^2 = w.w - 2 t (w.v) + t^2 (v.v) at t = clamp(w.v /
// v.v, 0, 1) — the closest-point parameter, so no branch: for t = 0 it is
// |w|^2, for t = 1 |w - v|^2, in between |w|^2 - (w.v)^2 / v.v.  An error in
// t only raises the value by v.v (dt)^2 (the expression is the squared
// distance to a point of the segment, minimal at the exact t).  The y and z
// parts of w.w and w.v are passed in (a = wy vy + wz vz, b = wy^2 + wz^2):
// the voxelizer's sweep computes them once per (y, z) cell and visits the x
// of the cell's column, so the per-candidate work is six fused operations.
// The bound covers the rounding of the float inputs, of every FP32 operation
// (fused multiply-adds: one rounding each, the same on the host and the
// device) and of the reference's own final rounding; a host build checks it
// over every voxel of random segment boxes (tests/test_voxel_fastpath.py).
FPGB_HD float dist2_yz_dot(float wy, float wz, float vy, float vz) {
   return fmaf(wz, vz, wy * vy);
}
FPGB_HD float dist2_yz_len(float wy, float wz) { return fmaf(wz, wz, wy * wy); }

FPGB_HD float approx_dist2_x(float wx, float a, float b, float vx, float c2f, float rc2,
                             float &margin) {
   const float c1 = fmaf(wx, vx, a);
   const float w2 = fmaf(wx, wx, b);
   const float t = fminf(fmaxf(c1 * rc2, 0.f), 1.f);
   const float m = fmaf(t, c2f, -2.f * c1);
   margin = fmaf(3.8e-6f, w2 + c2f, 1e-4f);
   return fmaf(t, m, w2);
}

FPGB_HD float approx_dist2(float wx, float wy, float wz, float vx, float vy, float vz,
                           float c2f, float rc2, float &margin) {
   return approx_dist2_x(wx, dist2_yz_dot(wy, wz, vy, vz), dist2_yz_len(wy, wz), vx, c2f, rc2,
                         margin);
}

// float(|cl - pt|^2) and float(r(t)^2) exactly as generator.cpp:327-328.
FPGB_HD void exact_dist(const SegDev &S, const double pt[3],
                                           double cl[3], float &dist_squ,
                                           float &r_sqr) {
   double t;
   closest_point(S, pt, cl, t);
   const double d0 = cl[0] - pt[0], d1 = cl[1] - pt[1], d2 = cl[2] - pt[2];
   double l2 = 0.0;
   l2 = l2 + d0 * d0;
   l2 = l2 + d1 * d1;
   l2 = l2 + d2 * d2;
   dist_squ = (float)l2;
   const double r = S.r0 * (1.0 - t) + S.r1 * t; // fiber.cpp:115-120
   r_sqr = (float)(r * r);
}

// ----------------------------------------------------------------------
// Two-float fast path.  For one (segment, voxel) pair it evaluates the
// reference's double arithmetic in two-float precision (~2^-46 relative)
// with an explicit bound E on |two-float value - value the reference's
// double arithmetic produces| (rounding of the reference itself included,
// generously).  A float result is accepted only when every real in
// [value - E, value + E] rounds to the same float; branch decisions only
// when the compared quantities differ by more than their bound.  Anything
// else returns false and the caller replays the reference in FP64, so the
// outcome is always the reference's, bit for bit.
// ----------------------------------------------------------------------
struct FastCand {
   float dist_squ, r_sqr;
   ff d[3];  // closest - point
   float dn; // |d|
   float m;  // magnitude scale of the terms that make up d
};

// Per-(y, z) row terms of the candidate evaluation (hoisted out of the x loop).
struct FastRow {
   ff wy, wz, c1yz; // point - p along y and z, and their part of dot(w, v)
   float wyz2;      // float estimate of wy^2 + wz^2
};

FPGB_HD void fast_row(const SegDev &S, float ly, float lz, FastRow &r) {
   r.wy = ff_add_f(ff{-S.pl_hi[1], -S.pl_lo[1]}, ly);
   r.wz = ff_add_f(ff{-S.pl_hi[2], -S.pl_lo[2]}, lz);
   r.c1yz = ff_add_sloppy(ff_mul(r.wy, ff{S.v_hi[1], S.v_lo[1]}),
                          ff_mul(r.wz, ff{S.v_hi[2], S.v_lo[2]}));
   r.wyz2 = r.wy.hi * r.wy.hi + r.wz.hi * r.wz.hi;
}

FPGB_HD bool fast_candidate_row(const SegDev &S, float lx, const FastRow &row, FastCand &c) {
   ff w[3], v[3];
   w[0] = ff_add_f(ff{-S.pl_hi[0], -S.pl_lo[0]}, lx); // point - p
   w[1] = row.wy;
   w[2] = row.wz;
#pragma unroll
   for (int i = 0; i < 3; i++)
      v[i] = ff{S.v_hi[i], S.v_lo[i]};
   const ff c1 = ff_add_sloppy(ff_mul(w[0], v[0]), row.c1yz);
   const float wn = sqrtf(w[0].hi * w[0].hi + row.wyz2);
   const ff c2{S.c2_hi, S.c2_lo};
   const float vn = sqrtf(S.c2_hi);
   const float ec = 0x1p-42f * (wn * vn + 1.f);
   int branch;
   if (c1.hi < -ec) {
      branch = 0; // c1 < 0: closest = s0, t = 0 (generator.cpp:483-484)
   } else {
      const ff dq = ff_sub_sloppy(c1, c2);
      if (dq.hi > ec)
         branch = 1; // c2 <= c1: closest = s1, t = 1 (:487-488)
      else if (c1.hi > ec && dq.hi < -ec)
         branch = 2; // interior: b = c1 / c2 (:490-493)
      else
         return false;
   }
   float bmag;
   if (branch == 0) {
      bmag = 0.f;
#pragma unroll
      for (int i = 0; i < 3; i++)
         c.d[i] = ff_neg(w[i]);
      c.r_sqr = S.rsq0;
   } else if (branch == 1) {
      bmag = 1.f;
#pragma unroll
      for (int i = 0; i < 3; i++)
         c.d[i] = ff_sub_sloppy(v[i], w[i]);
      c.r_sqr = S.rsq1;
   } else {
      const ff b = ff_div_rcp(c1, c2, S.c2_rcp);
      bmag = b.hi;
#pragma unroll
      for (int i = 0; i < 3; i++)
         c.d[i] = ff_sub_sloppy(ff_mul(v[i], b), w[i]);
      if (!std::isnan(S.rsq_const)) {
         c.r_sqr = S.rsq_const;
      } else { // r = r0 (1 - t) + r1 t  (fiber.cpp:115-120)
         const ff R = ff_add(ff{S.r0_hi, S.r0_lo}, ff_mul(ff{S.dr_hi, S.dr_lo}, b));
         const ff R2 = ff_sqr(R);
         const float er =
             0x1p-40f * (R2.hi + fabsf(R.hi) * fabsf(S.dr_hi) * (bmag + wn / vn + 1.f));
         if (!ff_round_unique(R2, er, c.r_sqr))
            return false;
      }
   }
   const ff D = ff_norm2_sloppy(c.d);
   c.dn = sqrtf(fmaxf(D.hi, 0.f));
   c.m = wn + vn * bmag + 1.f;
   const float ed = 0x1p-41f * c.m * (c.dn + 0x1p-20f * c.m) +
                    0x1p-47f * S.pscale * (2.f * c.dn + 1.f);
   return ff_round_unique(D, ed, c.dist_squ);
}

FPGB_HD bool fast_candidate(const SegDev &S, const float pt[3], FastCand &c) {
   FastRow row;
   fast_row(S, pt[1], pt[2], row);
   return fast_candidate_row(S, pt[0], row, c);
}

// float(unit(point - closest)) of the 'r' layer (generator.cpp:370-371)
FPGB_HD bool fast_radial(const SegDev &S, const FastCand &c, float out[3]) {
   if (!(c.dn > 0x1p-10f))
      return false;
   const ff n2 = ff_norm2(c.d);
   const ff inv = ff_div(ff_from(-1.f), ff_sqrt(n2)); // nv = -d
   const float ex = (0x1p-41f * c.m + 0x1p-47f * S.pscale) / c.dn + 0x1p-43f;
#pragma unroll
   for (int i = 0; i < 3; i++)
      if (!ff_round_unique(ff_mul(c.d[i], inv), ex, out[i]))
         return false;
   return true;
}


} // namespace fpgb
