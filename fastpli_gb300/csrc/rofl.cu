// ROFL tilt analysis (src/fastpli/analysis/rofl.py:16-63,
// _ROFL_with_jacobi.py:47-522; Schmitz et al., Front. Neuroanat. 2018,
// doi:10.3389/fnana.2018.00075) of every pixel of a 5-tilt image series,
// one warp per pixel, FP64.
//
// Per pixel, as the reference: the untilted direction (epa.direction) starts
// the fit; the measurements are centered (I / mean - 1) and weighted by
// 1 / sigma of the gain noise model; a 6 x 6 grid over inclination and t_rel
// picks the start point (first minimum); a Levenberg-Marquardt fit of
// (direction, inclination, t_rel) minimises the weighted residuals of the
// model sin(pi/2 t cos^2 alpha) sin(2 (rho - phi)) over all tilts; the result
// is folded into the PLI range and its standard deviations come from the
// reference's covariance formula.
//
// The reference fits with MINPACK (scipy.optimize.leastsq with a
// forward-difference Jacobian, or with its own approximate Jacobian in
// grad_mode); this kernel runs its own Marquardt iteration on the same
// objective with the exact Jacobian (or, in grad_mode, the reference's
// approximate one), converged more tightly, so results agree to the
// reference's stopping tolerance and the evaluation count (n_fev: model
// evaluations) is this kernel's own.
//
// Lanes hold the measurements i = lane + 32 q (tilt i / R, rotation i % R);
// every lane carries the three parameters and the iteration state, so the
// control flow is warp-uniform and sums are warp reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "fpgb_common.cuh"

namespace fpgb {

constexpr int kRoflMaxRot = 32;
constexpr int kRoflPerLane = (5 * kRoflMaxRot + 31) / 32;
constexpr int kRoflMaxEval = 400;

struct RoflParams {
   int n_rot;
   int grad_mode;
   double tau, gain, dir_offset, cos_tau;
   double rho[kRoflMaxRot];    // linspace(0, pi, R + 1)[:-1] + dir_offset
   double rho2s[kRoflMaxRot];  // sin / cos of 2 linspace(0, pi, R, False)
   double rho2c[kRoflMaxRot];  //   (epa.direction of the untilted series)
   double mat[4][9];           // tilt rotations, psi = 0, pi/2, pi, 3 pi/2
   double incl[6], trel[6];    // start grid
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      v += __shfl_xor_sync(0xffffffffu, v, o);
   return v;
}

// numpy.remainder for b > 0: result in [0, b)
__device__ __forceinline__ double pymod(double a, double b) {
   double m = fmod(a, b);
   if (m != 0.0 && m < 0.0)
      m += b;
   return m == 0.0 ? 0.0 : m;
}

// _symmetrize_angles (_ROFL_with_jacobi.py:64-74)
__device__ __forceinline__ void symmetrize(double &dir, double &incl) {
   const double s = -pymod(floor(dir / M_PI), 2.0) + 0.5; // +-0.5
   incl = (pymod(incl + M_PI / 2.0, M_PI) - M_PI / 2.0) * (s > 0.0 ? 1.0 : -1.0);
   dir = pymod(dir, M_PI);
}

// (direction, inclination, t_rel) seen in tilt j (:150-183), folded and
// |t_rel| as the model uses them (:186-212)
struct Tilted {
   double phi[5], alpha[5], trel[5];
};

__device__ __forceinline__ void tilted(const RoflParams &P, double phi, double alpha,
                                       double trel, Tilted &T) {
   double sp, cp, sa, ca;
   sincos(phi, &sp, &cp);
   sincos(alpha, &sa, &ca);
   const double v0 = ca * cp, v1 = ca * sp, v2 = sa;
   T.phi[0] = phi;
   T.alpha[0] = alpha;
   T.trel[0] = trel;
#pragma unroll
   for (int t = 0; t < 4; t++) {
      const double *M = P.mat[t];
      const double w0 = M[0] * v0 + M[1] * v1 + M[2] * v2;
      const double w1 = M[3] * v0 + M[4] * v1 + M[5] * v2;
      const double w2 = M[6] * v0 + M[7] * v1 + M[8] * v2;
      T.phi[t + 1] = atan(w1 / w0);
      T.alpha[t + 1] = asin(w2);
      T.trel[t + 1] = trel / P.cos_tau;
   }
#pragma unroll
   for (int j = 0; j < 5; j++) {
      symmetrize(T.phi[j], T.alpha[j]);
      T.trel[j] = fabs(T.trel[j]);
   }
}

struct Meas {
   double c[kRoflPerLane], w[kRoflPerLane];
   int j[kRoflPerLane], k[kRoflPerLane];
   int n; // measurements of this lane
};

// weighted residuals of this lane for parameters p; returns the warp's chi^2
__device__ __forceinline__ double residuals(const RoflParams &P, const Meas &m, double phi,
                                            double alpha, double trel,
                                            double r[kRoflPerLane]) {
   Tilted T;
   tilted(P, phi, alpha, trel, T);
   double amp[5];
#pragma unroll
   for (int j = 0; j < 5; j++) {
      const double ca = cos(T.alpha[j]);
      amp[j] = sin(M_PI / 2.0 * T.trel[j] * ca * ca);
   }
   double s = 0.0;
#pragma unroll
   for (int q = 0; q < kRoflPerLane; q++) {
      r[q] = 0.0;
      if (q < m.n) {
         const int j = m.j[q];
         const double model = amp[j] * sin(2.0 * (P.rho[m.k[q]] - T.phi[j]));
         r[q] = m.w[q] * (model - m.c[q]);
         s += r[q] * r[q];
      }
   }
   return warp_sum(s);
}

// the reference's Jacobian of the model with respect to each tilt's own
// angles (_calc_Jacobi, :215-258), weighted; used by grad_mode and by the
// covariance
__device__ __forceinline__ void model_jacobi(const RoflParams &P, const Meas &m, double phi,
                                             double alpha, double trel,
                                             double J[3][kRoflPerLane]) {
   Tilted T;
   tilted(P, phi, alpha, trel, T);
#pragma unroll
   for (int q = 0; q < kRoflPerLane; q++) {
      J[0][q] = J[1][q] = J[2][q] = 0.0;
      if (q < m.n) {
         const int j = m.j[q];
         double sa, ca;
         sincos(T.alpha[j], &sa, &ca);
         const double arg = M_PI / 2.0 * T.trel[j] * ca * ca;
         double sarg, carg;
         sincos(arg, &sarg, &carg);
         double s2, c2;
         sincos(2.0 * (P.rho[m.k[q]] - T.phi[j]), &s2, &c2);
         J[0][q] = m.w[q] * (-2.0 * c2 * sarg);
         J[1][q] = m.w[q] * (-M_PI * T.trel[j] * ca * sa * carg * s2);
         J[2][q] = m.w[q] * (M_PI / 2.0 * ca * ca * s2 * carg);
      }
   }
}

// Exact derivatives of the weighted residuals with respect to the fit
// parameters (phi, alpha, t_rel): the model's derivatives in each tilt's own
// angles (as _calc_Jacobi) chained through the tilt rotation (atan of the
// rotated axis for the direction, asin for the inclination), the folding of
// _symmetrize_angles (slope 1 for the direction, +-1 for the inclination) and
// |t_rel|.  Used in place of MINPACK's forward differences of the same
// objective: the same minimum, reached without the O(sqrt(eps)) gradient
// error that stalls a finite-difference iteration near it.
__device__ __forceinline__ void exact_jacobi(const RoflParams &P, const Meas &m, double phi,
                                             double alpha, double trel,
                                             double J[3][kRoflPerLane]) {
   double sp, cp, sa, ca;
   sincos(phi, &sp, &cp);
   sincos(alpha, &sa, &ca);
   const double v[3] = {ca * cp, ca * sp, sa};
   const double vp[3] = {-ca * sp, ca * cp, 0.0};  // dv / dphi
   const double va[3] = {-sa * cp, -sa * sp, ca};  // dv / dalpha
   double tp[5], ta[5], tt[5], dpp[5], dpa[5], dap[5], daa[5], dtt[5];
#pragma unroll
   for (int j = 0; j < 5; j++) {
      double pj, aj, tj;
      if (j == 0) {
         pj = phi, aj = alpha, tj = trel;
         dpp[0] = 1.0, dpa[0] = 0.0, dap[0] = 0.0, daa[0] = 1.0, dtt[0] = 1.0;
      } else {
         const double *M = P.mat[j - 1];
         double w[3], wp[3], wa[3];
#pragma unroll
         for (int r = 0; r < 3; r++) {
            w[r] = M[3 * r] * v[0] + M[3 * r + 1] * v[1] + M[3 * r + 2] * v[2];
            wp[r] = M[3 * r] * vp[0] + M[3 * r + 1] * vp[1] + M[3 * r + 2] * vp[2];
            wa[r] = M[3 * r] * va[0] + M[3 * r + 1] * va[1] + M[3 * r + 2] * va[2];
         }
         pj = atan(w[1] / w[0]);
         aj = asin(w[2]);
         tj = trel / P.cos_tau;
         const double den = w[0] * w[0] + w[1] * w[1];
         const double sq = sqrt(fmax(1.0 - w[2] * w[2], 0.0));
         dpp[j] = (w[0] * wp[1] - w[1] * wp[0]) / den;
         dpa[j] = (w[0] * wa[1] - w[1] * wa[0]) / den;
         dap[j] = wp[2] / sq;
         daa[j] = wa[2] / sq;
         dtt[j] = 1.0 / P.cos_tau;
      }
      const double s = (-pymod(floor(pj / M_PI), 2.0) + 0.5) > 0.0 ? 1.0 : -1.0;
      symmetrize(pj, aj);
      dap[j] *= s;
      daa[j] *= s;
      dtt[j] *= tj >= 0.0 ? 1.0 : -1.0;
      tp[j] = pj;
      ta[j] = aj;
      tt[j] = fabs(tj);
   }
#pragma unroll
   for (int q = 0; q < kRoflPerLane; q++) {
      J[0][q] = J[1][q] = J[2][q] = 0.0;
      if (q < m.n) {
         const int j = m.j[q];
         double sa2, ca2;
         sincos(ta[j], &sa2, &ca2);
         const double arg = M_PI / 2.0 * tt[j] * ca2 * ca2;
         double sarg, carg;
         sincos(arg, &sarg, &carg);
         double s2, c2;
         sincos(2.0 * (P.rho[m.k[q]] - tp[j]), &s2, &c2);
         const double dm_p = -2.0 * c2 * sarg;
         const double dm_a = -M_PI * tt[j] * ca2 * sa2 * carg * s2;
         const double dm_t = M_PI / 2.0 * ca2 * ca2 * s2 * carg;
         J[0][q] = m.w[q] * (dm_p * dpp[j] + dm_a * dap[j]);
         J[1][q] = m.w[q] * (dm_p * dpa[j] + dm_a * daa[j]);
         J[2][q] = m.w[q] * (dm_t * dtt[j]);
      }
   }
}

// numpy's pairwise sum of n < 128 contiguous doubles (8 partial sums)
__device__ __forceinline__ double np_sum(const double *a, int n, int stride) {
   if (n < 8) {
      double s = 0.0; // numpy adds from -0.0; same value for these data
      for (int i = 0; i < n; i++)
         s += a[i * stride];
      return s;
   }
   double r[8];
#pragma unroll
   for (int i = 0; i < 8; i++)
      r[i] = a[i * stride];
   int i = 8;
   for (; i + 8 <= n; i += 8)
#pragma unroll
      for (int t = 0; t < 8; t++)
         r[t] += a[(i + t) * stride];
   double s = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
   for (; i < n; i++)
      s += a[i * stride];
   return s;
}

// 3x3 solve by Cramer's rule (the damped normal equations are symmetric
// positive definite)
__device__ __forceinline__ bool solve3(const double A[6], const double b[3], double x[3]) {
   // A = [a0 a1 a2; a1 a3 a4; a2 a4 a5]
   const double c00 = A[3] * A[5] - A[4] * A[4];
   const double c01 = A[2] * A[4] - A[1] * A[5];
   const double c02 = A[1] * A[4] - A[2] * A[3];
   const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
   if (!(fabs(det) > 0.0) || !isfinite(det))
      return false;
   const double c11 = A[0] * A[5] - A[2] * A[2];
   const double c12 = A[1] * A[2] - A[0] * A[4];
   const double c22 = A[0] * A[3] - A[1] * A[1];
   x[0] = (c00 * b[0] + c01 * b[1] + c02 * b[2]) / det;
   x[1] = (c01 * b[0] + c11 * b[1] + c12 * b[2]) / det;
   x[2] = (c02 * b[0] + c12 * b[1] + c22 * b[2]) / det;
   return true;
}

__global__ void __launch_bounds__(128)
rofl_fit(const double *__restrict__ data, int64_t n_pix, const unsigned char *__restrict__ mask,
         const RoflParams P, double *__restrict__ out, unsigned long long *__restrict__ status) {
   const int lane = threadIdx.x & 31;
   const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
   const int R = P.n_rot, M = 5 * R;
   for (int64_t p = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); p < n_pix;
        p += warps) {
      double *o = out + 8 * p;
      if (mask && !mask[p]) {
         if (lane < 8)
            o[lane] = nan("");
         continue;
      }
      // tilt t, rotation k of pixel p: data[(t * n_pix + p) * R + k]
      double trans[5];
#pragma unroll
      for (int t = 0; t < 5; t++)
         trans[t] = np_sum(data + (t * n_pix + p) * R, R, 1) / R; // np.mean
      // epa.direction of the untilted series (epa.py:48-77) + dir_offset
      double phi0;
      {
         const double *d0 = data + p * R;
         double ps[kRoflMaxRot], pc[kRoflMaxRot];
         for (int k = 0; k < R; k++) {
            ps[k] = d0[k] * P.rho2s[k];
            pc[k] = d0[k] * P.rho2c[k];
         }
         const double a1 = 2.0 * np_sum(ps, R, 1) / R, b1 = 2.0 * np_sum(pc, R, 1) / R;
         phi0 = pymod(0.5 * atan2(-b1, a1) + M_PI, M_PI) + P.dir_offset;
      }
      Meas m;
      m.n = 0;
#pragma unroll
      for (int q = 0; q < kRoflPerLane; q++) {
         const int i = lane + 32 * q;
         m.c[q] = m.w[q] = 0.0;
         m.j[q] = m.k[q] = 0;
         if (i < M) {
            const int t = i / R, k = i - (i / R) * R;
            const double v = data[(t * n_pix + p) * R + k], tr = trans[t];
            m.c[q] = v / tr - 1.0; // _calc_centered_vals (:47-61)
            const double sig = sqrt(P.gain * (v / (tr * tr) + v * v / (tr * tr * tr * R)));
            m.w[q] = 1.0 / sig;
            m.j[q] = t;
            m.k[q] = k;
            m.n = q + 1;
         }
      }
      double r[kRoflPerLane];
      // start grid (:261-328): inclination outer, t_rel inner, first minimum
      double x[3] = {phi0, P.incl[0], P.trel[0]};
      {
         double best = INFINITY;
         for (int a = 0; a < 6; a++)
            for (int t = 0; t < 6; t++) {
               const double c = residuals(P, m, phi0, P.incl[a], P.trel[t], r);
               if (c < best) {
                  best = c;
                  x[1] = P.incl[a];
                  x[2] = P.trel[t];
               }
            }
      }
      // Levenberg-Marquardt with Marquardt's diagonal scaling
      int n_fev = 0;
      double cost = residuals(P, m, x[0], x[1], x[2], r);
      n_fev++;
      double lam = 1e-3;
      bool done = false;
      while (!done && n_fev < kRoflMaxEval) {
         double J[3][kRoflPerLane];
         if (P.grad_mode)
            model_jacobi(P, m, x[0], x[1], x[2], J);
         else
            exact_jacobi(P, m, x[0], x[1], x[2], J);
         double A[6], g[3];
         {
            double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int q = 0; q < kRoflPerLane; q++) {
               a[0] += J[0][q] * J[0][q];
               a[1] += J[0][q] * J[1][q];
               a[2] += J[0][q] * J[2][q];
               a[3] += J[1][q] * J[1][q];
               a[4] += J[1][q] * J[2][q];
               a[5] += J[2][q] * J[2][q];
               a[6] += J[0][q] * r[q];
               a[7] += J[1][q] * r[q];
               a[8] += J[2][q] * r[q];
            }
#pragma unroll
            for (int e = 0; e < 6; e++)
               A[e] = warp_sum(a[e]);
#pragma unroll
            for (int e = 0; e < 3; e++)
               g[e] = -warp_sum(a[6 + e]);
         }
         const double dA[3] = {fmax(A[0], 1e-300), fmax(A[3], 1e-300), fmax(A[5], 1e-300)};
         bool improved = false;
         while (n_fev < kRoflMaxEval) {
            const double D[6] = {A[0] + lam * dA[0], A[1], A[2], A[3] + lam * dA[1], A[4],
                                 A[5] + lam * dA[2]};
            double dx[3];
            if (!solve3(D, g, dx)) {
               lam *= 10.0;
               if (lam > 1e16)
                  break;
               continue;
            }
            const double xn[3] = {x[0] + dx[0], x[1] + dx[1], x[2] + dx[2]};
            double rn[kRoflPerLane];
            const double cn = residuals(P, m, xn[0], xn[1], xn[2], rn);
            n_fev++;
            if (cn < cost) {
               const double red = (cost - cn) / fmax(cost, 1e-300);
               const double step = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
               const double xn2 = sqrt(xn[0] * xn[0] + xn[1] * xn[1] + xn[2] * xn[2]);
               x[0] = xn[0];
               x[1] = xn[1];
               x[2] = xn[2];
#pragma unroll
               for (int q = 0; q < kRoflPerLane; q++)
                  r[q] = rn[q];
               cost = cn;
               lam = fmax(lam * 0.1, 1e-15);
               improved = true;
               if (red <= 1e-15 || step <= 1e-13 * (xn2 + 1e-13) || cost == 0.0)
                  done = true;
               break;
            }
            lam *= 10.0;
            if (lam > 1e16)
               break;
         }
         if (!improved)
            done = true; // no descent left at machine precision
      }
      if (!done)
         atomicAdd(&status[0], 1ull); // evaluation budget reached
      // result (:481-520): fold, |t_rel|, covariance from the reference's
      // Jacobian at the folded point and its own 3x3 inverse
      double d = x[0], a = x[1];
      symmetrize(d, a);
      const double t = fabs(x[2]);
      const double sigma_sq = cost / (double)(M - 3);
      double J[3][kRoflPerLane];
      model_jacobi(P, m, d, a, t, J);
      double mm[9];
      {
         double s[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
         for (int q = 0; q < kRoflPerLane; q++) {
            s[0] += J[0][q] * J[0][q];
            s[1] += J[0][q] * J[1][q];
            s[2] += J[0][q] * J[2][q];
            s[3] += J[1][q] * J[1][q];
            s[4] += J[1][q] * J[2][q];
            s[5] += J[2][q] * J[2][q];
         }
#pragma unroll
         for (int e = 0; e < 6; e++)
            s[e] = warp_sum(s[e]);
         mm[0] = s[0], mm[1] = s[1], mm[2] = s[2];
         mm[3] = s[1], mm[4] = s[3], mm[5] = s[4];
         mm[6] = s[2], mm[7] = s[4], mm[8] = s[5];
      }
      // _invertmatrix (:14-44) with the reference's determinant expression
      // (its fourth term is m20 * m12, without a third factor)
      const double det = mm[0] * mm[4] * mm[8] + mm[3] * mm[7] * mm[2] + mm[6] * mm[5] -
                         mm[0] * mm[7] * mm[5] - mm[6] * mm[4] * mm[2] - mm[3] * mm[1] * mm[8];
      const double i00 = (mm[4] * mm[8] - mm[5] * mm[7]) / det;
      const double i11 = (mm[0] * mm[8] - mm[2] * mm[6]) / det;
      const double i22 = (mm[0] * mm[4] - mm[1] * mm[3]) / det;
      if (lane == 0) {
         o[0] = d;
         o[1] = a;
         o[2] = t;
         o[3] = sqrt(fabs(i00 * sigma_sq));
         o[4] = sqrt(fabs(i11 * sigma_sq));
         o[5] = sqrt(fabs(i22 * sigma_sq));
         o[6] = cost;
         o[7] = (double)n_fev;
      }
   }
}

} // namespace fpgb

using namespace fpgb;

extern "C" {

int fpgb_rofl_device(const double *d_data, int64_t n_pix, int64_t n_rot, double tilt_angle,
                     double gain, double dir_offset, int grad_mode, const unsigned char *d_mask,
                     double *d_out, int64_t *n_unconverged, void *stream) {
   if (!d_data || !d_out || n_pix < 0 || n_rot <= 3 || n_rot > kRoflMaxRot) {
      set_error("rofl: null buffer, n_pix < 0, or n_rot outside 4..%d", kRoflMaxRot);
      return FPGB_EINVAL;
   }
   if (!(gain > 1.0)) {
      set_error("rofl gain <= 1");
      return FPGB_EINVAL;
   }
   RoflParams P;
   std::memset(&P, 0, sizeof P);
   P.n_rot = (int)n_rot;
   P.grad_mode = grad_mode ? 1 : 0;
   P.tau = tilt_angle;
   P.gain = gain;
   P.dir_offset = dir_offset;
   P.cos_tau = std::cos(tilt_angle);
   // numpy.linspace(start, stop, num): start + k * ((stop - start) / div)
   for (int k = 0; k < P.n_rot; k++) {
      P.rho[k] = (double)k * (M_PI / (double)n_rot) + dir_offset;
      const double r2 = 2.0 * ((double)k * (M_PI / (double)n_rot));
      P.rho2s[k] = std::sin(r2);
      P.rho2c[k] = std::cos(r2);
   }
   for (int t = 0; t < 4; t++) { // _create_rotation_matrix (:77-96)
      const double psi = (double)t * (2.0 * M_PI / 4.0);
      const double c = std::cos(psi), s = std::sin(psi), ct = std::cos(tilt_angle),
                   st = std::sin(tilt_angle);
      double *M = P.mat[t];
      M[0] = ct * c * c + s * s;
      M[1] = (ct - 1) * s * c;
      M[2] = c * st;
      M[3] = (ct - 1) * s * c;
      M[4] = ct * s * s + c * c;
      M[5] = s * st;
      M[6] = -c * st;
      M[7] = -s * st;
      M[8] = ct;
   }
   for (int k = 0; k < 6; k++) { // linspace(-pi/2, pi/2, 8)[1:-1], linspace(0, .9, 8)[1:-1]
      P.incl[k] = (double)(k + 1) * (M_PI / 7.0) + (-M_PI / 2.0);
      P.trel[k] = (double)(k + 1) * (0.9 / 7.0);
   }
   cudaStream_t st = as_stream(stream);
   void *w = nullptr;
   FPGB_TRY(pool_get(kSlotCounters, sizeof(unsigned long long) * kCounterWords, &w, st));
   auto *status = static_cast<unsigned long long *>(w);
   FPGB_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned long long), st));
   if (n_pix > 0) {
      const int64_t blocks = std::min<int64_t>((n_pix + 3) / 4, 152 * 64);
      rofl_fit<<<(unsigned)blocks, 128, 0, st>>>(d_data, n_pix, d_mask, P, d_out, status);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   if (n_unconverged) {
      unsigned long long h = 0;
      FPGB_CUDA_TRY(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, st));
      FPGB_CUDA_TRY(cudaStreamSynchronize(st));
      *n_unconverged = (int64_t)h;
   }
   return FPGB_OK;
}

} // extern "C"
