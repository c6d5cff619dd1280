// ROFL tilt analysis (src/fastpli/analysis/rofl.py:16-63,
// _ROFL_with_jacobi.py:47-522; Schmitz et al., Front. Neuroanat. 2018,
// doi:10.3389/fnana.2018.00075) of every pixel of a 5-tilt image series,
// one thread per pixel, FP64.
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
// The fit is MINPACK's Levenberg-Marquardt as the reference calls it
// (scipy.optimize.leastsq: forward differences, or in grad_mode the
// reference's own Jacobian; the same tolerances, scaling and budget of 150
// evaluations), restated below; n_fev is MINPACK's evaluation count.
//
// One thread per pixel, not one warp: GB300 runs FP64 at a small fraction
// of its FP32 rate, so the kernel is bound by FP64 instructions issued, and
// a warp per pixel would repeat every per-pixel step (the tilt rotations,
// the 3 x 3 trust-region algebra) in all 32 lanes.  A thread walks the
// 5 R measurements of its pixel in the reference's order, so every sum is
// taken in the order MINPACK (sequential) or numpy (pairwise) takes it.
// Compiled with -fmad=false: products and sums round separately, as in the
// reference, except where a fused multiply-add is written out.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "fpgb_common.cuh"

namespace fpgb {

constexpr int kRoflMaxRot = 32;
constexpr int kRoflSmallRot = 10; // the usual 6 - 9 rotations: 50 measurements

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

// numpy.remainder for b > 0: result in [0, b)
__device__ __forceinline__ double pymod(double a, double b) {
   double m = fmod(a, b);
   if (m != 0.0 && m < 0.0)
      m += b;
   return m == 0.0 ? 0.0 : m;
}

// CUDA's FP64 sin, cos, sincos, atan and asin called out of line: one copy
// of each in the kernel's code instead of one per call site (the fit is
// bound by instruction fetch while the threads of a warp are in different
// phases of their fits)
__device__ __noinline__ double ol_sin(double x) { return sin(x); }
__device__ __noinline__ double ol_cos(double x) { return cos(x); }
__device__ __noinline__ void ol_sincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __noinline__ double ol_atan(double x) { return atan(x); }
__device__ __noinline__ double ol_asin(double x) { return asin(x); }

// _symmetrize_angles (_ROFL_with_jacobi.py:64-74)
__device__ __forceinline__ void symmetrize(double &dir, double &incl) {
   const double s = -pymod(floor(dir / M_PI), 2.0) + 0.5; // +-0.5
   incl = (pymod(incl + M_PI / 2.0, M_PI) - M_PI / 2.0) * (s > 0.0 ? 1.0 : -1.0);
   dir = pymod(dir, M_PI);
}

// np.dot of a 3 x 3 matrix row and a 3-vector (_calculate_rotated_fiber_params,
// :179) as numpy 2.5 on x86-64 rounds it where the reference's results were
// recorded: fma(a2, v2, fma(a0, v0, a1 v1)), found by comparing np.dot with
// exact rational arithmetic (all of 6,000 random rows agreed with this form,
// at most 76% with any other order, fused or not)
__device__ __forceinline__ double np_dot3(const double *a, double v0, double v1, double v2) {
   return fma(a[2], v2, fma(a[0], v0, a[1] * v1));
}

// (direction, inclination, t_rel) seen in tilt j (:150-183), folded and
// |t_rel| as the model uses them (:186-212)
struct Tilted {
   double phi[5], alpha[5], trel[5];
};

__device__ __forceinline__ void tilted(const RoflParams &P, double phi, double alpha,
                                       double trel, Tilted &T) {
   double sp, cp, sa, ca;
   ol_sincos(phi, &sp, &cp);
   ol_sincos(alpha, &sa, &ca);
   const double v0 = ca * cp, v1 = ca * sp, v2 = sa;
   T.phi[0] = phi;
   T.alpha[0] = alpha;
   T.trel[0] = trel;
#pragma unroll
   for (int t = 0; t < 4; t++) {
      const double *M = P.mat[t];
      const double w0 = np_dot3(M, v0, v1, v2);
      const double w1 = np_dot3(M + 3, v0, v1, v2);
      const double w2 = np_dot3(M + 6, v0, v1, v2);
      T.phi[t + 1] = ol_atan(w1 / w0);
      T.alpha[t + 1] = ol_asin(w2);
      T.trel[t + 1] = trel / P.cos_tau;
   }
#pragma unroll
   for (int j = 0; j < 5; j++) {
      symmetrize(T.phi[j], T.alpha[j]);
      T.trel[j] = fabs(T.trel[j]);
   }
}

// weighted residuals r[i] = w[i] (model_i - c[i]) (_residuum, :407-410) of
// the 5 R measurements, i = tilt * R + rotation (the order of the
// reference's flattened intensity curves, :186-212).  Out of line, like the
// Jacobian and the trust-region step below: one copy of each large body
// keeps the kernel's code in the instruction cache while the threads of a
// warp are in different phases of their fits.
__device__ __noinline__ void px_residuals(const RoflParams &P, const double *c,
                                             const double *w, double phi, double alpha,
                                             double trel, double *r) {
   Tilted T;
   tilted(P, phi, alpha, trel, T);
   const int R = P.n_rot;
#pragma unroll
   for (int j = 0; j < 5; j++) {
      const double ca = ol_cos(T.alpha[j]);
      const double amp = ol_sin(M_PI / 2.0 * T.trel[j] * (ca * ca));
      const int i0 = j * R;
      for (int k = 0; k < R; k++)
         r[i0 + k] = w[i0 + k] * (amp * ol_sin(2.0 * (P.rho[k] - T.phi[j])) - c[i0 + k]);
   }
}

// the reference's Jacobian of the model with respect to each tilt's own
// angles (_calc_Jacobi, :215-258), weighted (_weighted_jacobi, :393-403):
// columns J[0..2][i] at J + col[0..2]; used by grad_mode and by the
// covariance
__device__ __noinline__ void px_jacobi(const RoflParams &P, const double *w, double phi,
                                          double alpha, double trel, double *J,
                                          const int col[3]) {
   Tilted T;
   tilted(P, phi, alpha, trel, T);
   const int R = P.n_rot;
#pragma unroll
   for (int j = 0; j < 5; j++) {
      const double ca = ol_cos(T.alpha[j]), sa = ol_sin(T.alpha[j]);
      const double arg = M_PI / 2.0 * T.trel[j] * (ca * ca);
      const double sarg = ol_sin(arg), carg = ol_cos(arg);
      const double dal = -M_PI * T.trel[j] * ca * sa * carg; // times s2
      const double dtr = M_PI / 2.0 * (ca * ca);             // times s2, cos(arg)
      const int i0 = j * R;
      for (int k = 0; k < R; k++) {
         const double d2 = 2.0 * (P.rho[k] - T.phi[j]);
         const double s2 = ol_sin(d2), c2 = ol_cos(d2);
         const double wi = w[i0 + k];
         J[col[0] + i0 + k] = -2.0 * c2 * sarg * wi;
         J[col[1] + i0 + k] = dal * s2 * wi;
         J[col[2] + i0 + k] = dtr * s2 * carg * wi;
      }
   }
}

// numpy's pairwise sum (np.sum of a contiguous float64 array, n <= 256):
// blocks of at most 128 values with 8 partial sums, longer arrays split once
// at a multiple of 8; get(i) gives the i-th value
template <class Get> __device__ __forceinline__ double np_sum_block(Get get, int b, int n) {
   if (n < 8) {
      double s = 0.0; // numpy adds from -0.0; same value for these data
      for (int i = 0; i < n; i++)
         s += get(b + i);
      return s;
   }
   double r[8];
#pragma unroll
   for (int i = 0; i < 8; i++)
      r[i] = get(b + i);
   int i = 8;
   for (; i + 8 <= n; i += 8)
#pragma unroll
      for (int t = 0; t < 8; t++)
         r[t] += get(b + i + t);
   double s = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
   for (; i < n; i++)
      s += get(b + i);
   return s;
}

template <class Get> __device__ __forceinline__ double np_sum(Get get, int n) {
   if (n <= 128)
      return np_sum_block(get, 0, n);
   int n2 = n / 2;
   n2 -= n2 % 8;
   return np_sum_block(get, 0, n2) + np_sum_block(get, n2, n - n2);
}

// sum of squares in MINPACK's enorm order (sequential; every value of these
// fits lies in enorm's unscaled range or is zero)
__device__ __noinline__ double seq_sumsq(const double *r, int n) {
   double s = 0.0;
   for (int i = 0; i < n; i++)
      s = s + r[i] * r[i];
   return s;
}

// sum over i of a[i] b[i], sequential (qrfac's and qtf's column products)
__device__ __noinline__ double seq_dot(const double *a, const double *b, int n) {
   double s = 0.0;
   for (int i = 0; i < n; i++)
      s = s + a[i] * b[i];
   return s;
}

// b[i] = b[i] - t a[i] (qrfac's Householder update)
__device__ __noinline__ void seq_axmy(const double *a, double *b, double t, int n) {
   for (int i = 0; i < n; i++)
      b[i] = b[i] - t * a[i];
}

// x^3 rounded once, as numpy's x**3 (pow) gives it: the exact cube as a
// double-double (Dekker's product through fma) rounded to the nearest double
__device__ __forceinline__ double cube_rn(double x) {
   const double p = x * x;
   const double pe = fma(x, x, -p); // x^2 = p + pe exactly
   const double h = p * x;
   const double he = fma(p, x, -h); // p x = h + he exactly
   return h + (he + pe * x);
}

// ----------------------------------------------------------------------------
// MINPACK's Levenberg-Marquardt (lmdif with a forward-difference Jacobian,
// lmder with the reference's own Jacobian in grad_mode), restated from the
// published algorithm (More, "The Levenberg-Marquardt algorithm:
// implementation and theory", 1978; MINPACK-1, 1980) as
// scipy.optimize.leastsq runs it for the reference (_ROFL_with_jacobi.py:
// 472-486): ftol = xtol = 1.49012e-8, gtol = 0, maxfev = 150, factor 100,
// automatic scaling, epsfcn = machine epsilon.  The m x 3 Jacobian and the
// residual vectors are the thread's own; the loops over the measurements
// run in MINPACK's order, so the iterates differ from the reference's only
// where CUDA's FP64 trigonometry rounds differently from the reference's
// numpy (a last-bit difference in some evaluations, which MINPACK's
// stopping tests can turn into a different last step).
// ----------------------------------------------------------------------------
constexpr double kMpEps = 2.220446049250313e-16;     // machine epsilon (dpmpar(1))
constexpr double kMpDwarf = 2.2250738585072014e-308; // smallest normal (dpmpar(2))
constexpr double kMpTol = 1.49012e-08;               // leastsq's ftol and xtol
constexpr int kMpMaxFev = 150;

__device__ __forceinline__ double mp_norm3(const double v[3]) {
   double s = 0.0;
   s = s + v[0] * v[0];
   s = s + v[1] * v[1];
   s = s + v[2] * v[2];
   return sqrt(s);
}

// qrsolv: solves (R; D) x = (qtb; 0) in the least-squares sense for the
// 3 x 3 upper triangular R of a pivoted QR (ipvt) and diagonal D; r's
// strict lower triangle receives S's, sdiag its diagonal
__device__ __noinline__ void mp_qrsolv(double r[3][3], const int ipvt[3], const double dg[3],
                          const double qtb[3], double x[3], double sdiag[3]) {
   double wa[3];
   for (int j = 0; j < 3; j++) {
      for (int i = j; i < 3; i++)
         r[i][j] = r[j][i];
      x[j] = r[j][j];
      wa[j] = qtb[j];
   }
   for (int j = 0; j < 3; j++) {
      const int l = ipvt[j];
      if (dg[l] != 0.0) {
         for (int k = j; k < 3; k++)
            sdiag[k] = 0.0;
         sdiag[j] = dg[l];
         double qtbpj = 0.0;
         for (int k = j; k < 3; k++) {
            if (sdiag[k] == 0.0)
               continue;
            double sn, cs;
            if (fabs(r[k][k]) < fabs(sdiag[k])) {
               const double cotan = r[k][k] / sdiag[k];
               sn = 0.5 / sqrt(0.25 + 0.25 * (cotan * cotan));
               cs = sn * cotan;
            } else {
               const double tn = sdiag[k] / r[k][k];
               cs = 0.5 / sqrt(0.25 + 0.25 * (tn * tn));
               sn = cs * tn;
            }
            r[k][k] = cs * r[k][k] + sn * sdiag[k];
            const double temp = cs * wa[k] + sn * qtbpj;
            qtbpj = -sn * wa[k] + cs * qtbpj;
            wa[k] = temp;
            for (int i = k + 1; i < 3; i++) {
               const double t2 = cs * r[i][k] + sn * sdiag[i];
               sdiag[i] = -sn * r[i][k] + cs * sdiag[i];
               r[i][k] = t2;
            }
         }
      }
      sdiag[j] = r[j][j];
      r[j][j] = x[j];
   }
   int nsing = 3;
   for (int j = 0; j < 3; j++) {
      if (sdiag[j] == 0.0 && nsing == 3)
         nsing = j;
      if (nsing < 3)
         wa[j] = 0.0;
   }
   for (int j = nsing - 1; j >= 0; j--) {
      double sum = 0.0;
      for (int i = j + 1; i < nsing; i++)
         sum = sum + r[i][j] * wa[i];
      wa[j] = (wa[j] - sum) / sdiag[j];
   }
   for (int j = 0; j < 3; j++)
      x[ipvt[j]] = wa[j];
}

// lmpar: the Levenberg-Marquardt parameter par and step x for trust radius
// delta (r: R in its upper triangle; its lower triangle is scratch)
__device__ __noinline__ void mp_lmpar(double r[3][3], const int ipvt[3], const double dg[3],
                         const double qtb[3], double delta, double &par, double x[3]) {
   double wa1[3], wa2[3], sdiag[3];
   int nsing = 3;
   for (int j = 0; j < 3; j++) {
      wa1[j] = qtb[j];
      if (r[j][j] == 0.0 && nsing == 3)
         nsing = j;
      if (nsing < 3)
         wa1[j] = 0.0;
   }
   for (int j = nsing - 1; j >= 0; j--) {
      wa1[j] = wa1[j] / r[j][j];
      const double temp = wa1[j];
      for (int i = 0; i < j; i++)
         wa1[i] = wa1[i] - r[i][j] * temp;
   }
   for (int j = 0; j < 3; j++)
      x[ipvt[j]] = wa1[j];
   int iter = 0;
   for (int j = 0; j < 3; j++)
      wa2[j] = dg[j] * x[j];
   double dxnorm = mp_norm3(wa2);
   double fp = dxnorm - delta;
   if (fp <= 0.1 * delta) {
      par = 0.0;
      return;
   }
   double parl = 0.0;
   if (nsing >= 3) {
      for (int j = 0; j < 3; j++) {
         const int l = ipvt[j];
         wa1[j] = dg[l] * (wa2[l] / dxnorm);
      }
      for (int j = 0; j < 3; j++) {
         double sum = 0.0;
         for (int i = 0; i < j; i++)
            sum = sum + r[i][j] * wa1[i];
         wa1[j] = (wa1[j] - sum) / r[j][j];
      }
      const double temp = mp_norm3(wa1);
      parl = ((fp / delta) / temp) / temp;
   }
   for (int j = 0; j < 3; j++) {
      double sum = 0.0;
      for (int i = 0; i <= j; i++)
         sum = sum + r[i][j] * qtb[i];
      wa1[j] = sum / dg[ipvt[j]];
   }
   const double gnorm = mp_norm3(wa1);
   double paru = gnorm / delta;
   if (paru == 0.0)
      paru = kMpDwarf / fmin(delta, 0.1);
   par = fmax(par, parl);
   par = fmin(par, paru);
   if (par == 0.0)
      par = gnorm / dxnorm;
   for (;;) {
      iter++;
      if (par == 0.0)
         par = fmax(kMpDwarf, 0.001 * paru);
      const double temp = sqrt(par);
      for (int j = 0; j < 3; j++)
         wa1[j] = temp * dg[j];
      mp_qrsolv(r, ipvt, wa1, qtb, x, sdiag);
      for (int j = 0; j < 3; j++)
         wa2[j] = dg[j] * x[j];
      dxnorm = mp_norm3(wa2);
      const double fp_old = fp;
      fp = dxnorm - delta;
      if (fabs(fp) <= 0.1 * delta || (parl == 0.0 && fp <= fp_old && fp_old < 0.0) ||
          iter == 10)
         break;
      for (int j = 0; j < 3; j++) {
         const int l = ipvt[j];
         wa1[j] = dg[l] * (wa2[l] / dxnorm);
      }
      for (int j = 0; j < 3; j++) {
         wa1[j] = wa1[j] / sdiag[j];
         const double t2 = wa1[j];
         for (int i = j + 1; i < 3; i++)
            wa1[i] = wa1[i] - r[i][j] * t2;
      }
      const double t3 = mp_norm3(wa1);
      const double parc = ((fp / delta) / t3) / t3;
      if (fp > 0.0)
         parl = fmax(parl, par);
      if (fp < 0.0)
         paru = fmin(paru, par);
      par = fmax(parl, par + parc);
   }
}

// The fit for one pixel (one thread): x in: the start point, out: the last
// accepted point; F (2 x MAXM) holds the residuals, *cur the half that
// holds them at x on return; J (3 x MAXM) is the Jacobian's workspace.
// Returns MINPACK's info (5: evaluation budget spent); nfev counts as
// MINPACK counts (lmdif: 1 + 3 per Jacobian + 1 per trial step; lmder:
// 1 + 1 per trial step).
template <int MAXM>
__device__ int mp_fit(const RoflParams &P, const double *c, const double *w, int M, double x[3],
                      double *F, int &cur, double *J, int &nfev) {
   const double epsfd = sqrt(kMpEps); // sqrt(max(epsfcn, epsmch)), epsfcn = eps
   cur = 0;
   px_residuals(P, c, w, x[0], x[1], x[2], F);
   nfev = 1;
   double fnorm = sqrt(seq_sumsq(F, M));
   double par = 0.0, delta = 0.0, xnorm = 0.0;
   double dg[3] = {1.0, 1.0, 1.0};
   int iter = 1;
   for (;;) {
      double *fv = F + cur * MAXM, *wa4 = F + (1 - cur) * MAXM;
      // the Jacobian's columns, J + col[j] after the pivoting swaps
      int col[3] = {0, MAXM, 2 * MAXM};
      if (P.grad_mode) {
         px_jacobi(P, w, x[0], x[1], x[2], J, col);
      } else { // fdjac2
#pragma unroll 1
         for (int j = 0; j < 3; j++) {
            const double temp = x[j];
            double h = epsfd * fabs(temp);
            if (h == 0.0)
               h = epsfd;
            double xp[3] = {x[0], x[1], x[2]};
            xp[j] = temp + h;
            double *Jj = J + col[j];
            px_residuals(P, c, w, xp[0], xp[1], xp[2], Jj);
            for (int i = 0; i < M; i++)
               Jj[i] = (Jj[i] - fv[i]) / h;
         }
         nfev += 3;
      }
      // qrfac with column pivoting
      double acnorm[3], rdiag[3], wa[3];
      int ipvt[3] = {0, 1, 2};
#pragma unroll
      for (int j = 0; j < 3; j++) {
         acnorm[j] = sqrt(seq_sumsq(J + col[j], M));
         rdiag[j] = wa[j] = acnorm[j];
      }
#pragma unroll
      for (int j = 0; j < 3; j++) {
         int kmax = j;
#pragma unroll
         for (int k = j; k < 3; k++)
            if (rdiag[k] > rdiag[kmax])
               kmax = k;
#pragma unroll
         for (int k = j + 1; k < 3; k++)
            if (k == kmax) {
               const int tc = col[j];
               col[j] = col[k];
               col[k] = tc;
               rdiag[k] = rdiag[j];
               wa[k] = wa[j];
               const int t = ipvt[j];
               ipvt[j] = ipvt[k];
               ipvt[k] = t;
            }
         double *aj = J + col[j];
         double ajnorm = sqrt(seq_sumsq(aj + j, M - j));
         if (ajnorm != 0.0) {
            if (aj[j] < 0.0)
               ajnorm = -ajnorm;
            for (int i = j; i < M; i++)
               aj[i] = aj[i] / ajnorm;
            aj[j] = aj[j] + 1.0;
#pragma unroll
            for (int k = j + 1; k < 3; k++) {
               double *ak = J + col[k];
               const double sum = seq_dot(aj + j, ak + j, M - j);
               const double temp = sum / aj[j];
               seq_axmy(aj + j, ak + j, temp, M - j);
               if (rdiag[k] != 0.0) {
                  const double t2 = ak[j] / rdiag[k];
                  rdiag[k] = rdiag[k] * sqrt(fmax(0.0, 1.0 - t2 * t2));
                  const double q2 = rdiag[k] / wa[k];
                  if (0.05 * (q2 * q2) <= kMpEps) {
                     rdiag[k] = sqrt(seq_sumsq(ak + j + 1, M - j - 1));
                     wa[k] = rdiag[k];
                  }
               }
            }
         }
         rdiag[j] = -ajnorm;
      }
      if (iter == 1) {
#pragma unroll
         for (int j = 0; j < 3; j++)
            dg[j] = acnorm[j] == 0.0 ? 1.0 : acnorm[j];
         const double w3[3] = {dg[0] * x[0], dg[1] * x[1], dg[2] * x[2]};
         xnorm = mp_norm3(w3);
         delta = 100.0 * xnorm;
         if (delta == 0.0)
            delta = 100.0;
      }
      // (Q^T fvec) in its first 3 rows (wa4 is the residual buffer's free
      // half), and R's diagonal restored
      double qtf[3];
      for (int i = 0; i < M; i++)
         wa4[i] = fv[i];
#pragma unroll
      for (int j = 0; j < 3; j++) {
         double *aj = J + col[j];
         if (aj[j] != 0.0) {
            const double sum = seq_dot(aj + j, wa4 + j, M - j);
            const double temp = -sum / aj[j];
            for (int i = j; i < M; i++)
               wa4[i] = wa4[i] + aj[i] * temp;
         }
         aj[j] = rdiag[j];
         qtf[j] = wa4[j];
      }
      double R[3][3];
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
         for (int i = 0; i < 3; i++)
            R[i][j] = i <= j ? J[col[j] + i] : 0.0;
      double gnorm = 0.0;
      if (fnorm != 0.0) {
#pragma unroll
         for (int j = 0; j < 3; j++) {
            const int l = ipvt[j];
            const double an = l == 0 ? acnorm[0] : (l == 1 ? acnorm[1] : acnorm[2]);
            if (an != 0.0) {
               double sum = 0.0;
#pragma unroll
               for (int i = 0; i <= j; i++)
                  sum = sum + R[i][j] * (qtf[i] / fnorm);
               gnorm = fmax(gnorm, fabs(sum / an));
            }
         }
      }
      if (gnorm <= 0.0) // gtol = 0
         return 4;
#pragma unroll
      for (int j = 0; j < 3; j++)
         dg[j] = fmax(dg[j], acnorm[j]);
      // inner loop: trial steps until one is accepted
      for (;;) {
         double rr[3][3];
#pragma unroll
         for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++)
               rr[i][j] = R[i][j];
         double p[3];
         mp_lmpar(rr, ipvt, dg, qtf, delta, par, p);
         double w1[3], w2[3], w3[3];
#pragma unroll
         for (int j = 0; j < 3; j++) {
            w1[j] = -p[j];
            w2[j] = x[j] + w1[j];
            w3[j] = dg[j] * w1[j];
         }
         const double pnorm = mp_norm3(w3);
         if (iter == 1)
            delta = fmin(delta, pnorm);
         px_residuals(P, c, w, w2[0], w2[1], w2[2], wa4);
         nfev++;
         const double fnorm1 = sqrt(seq_sumsq(wa4, M));
         double actred = -1.0;
         if (0.1 * fnorm1 < fnorm) {
            const double t = fnorm1 / fnorm;
            actred = 1.0 - t * t;
         }
#pragma unroll
         for (int j = 0; j < 3; j++) {
            w3[j] = 0.0;
            const int l = ipvt[j];
            const double temp = l == 0 ? w1[0] : (l == 1 ? w1[1] : w1[2]);
#pragma unroll
            for (int i = 0; i <= j; i++)
               w3[i] = w3[i] + R[i][j] * temp;
         }
         const double temp1 = mp_norm3(w3) / fnorm;
         const double temp2 = (sqrt(par) * pnorm) / fnorm;
         const double prered = temp1 * temp1 + (temp2 * temp2) / 0.5;
         const double dirder = -(temp1 * temp1 + temp2 * temp2);
         const double ratio = prered != 0.0 ? actred / prered : 0.0;
         if (ratio <= 0.25) {
            double temp = actred >= 0.0 ? 0.5 : 0.5 * dirder / (dirder + 0.5 * actred);
            if (0.1 * fnorm1 >= fnorm || temp < 0.1)
               temp = 0.1;
            delta = temp * fmin(delta, pnorm / 0.1);
            par = par / temp;
         } else if (par == 0.0 || ratio >= 0.75) {
            delta = pnorm / 0.5;
            par = 0.5 * par;
         }
         if (ratio >= 1e-4) { // accepted: the trial residuals become fvec
#pragma unroll
            for (int j = 0; j < 3; j++)
               x[j] = w2[j];
            const double w5[3] = {dg[0] * x[0], dg[1] * x[1], dg[2] * x[2]};
            xnorm = mp_norm3(w5);
            cur = 1 - cur;
            fnorm = fnorm1;
            iter++;
         }
         int info = 0;
         const bool fsmall = fabs(actred) <= kMpTol && prered <= kMpTol && 0.5 * ratio <= 1.0;
         if (fsmall)
            info = 1;
         if (delta <= kMpTol * xnorm)
            info = fsmall ? 3 : 2;
         if (info != 0)
            return info;
         if (nfev >= kMpMaxFev)
            info = 5;
         if (fabs(actred) <= kMpEps && prered <= kMpEps && 0.5 * ratio <= 1.0)
            info = 6; // tolerances too small (6, 7, 8)
         if (delta <= kMpEps * xnorm)
            info = 7;
         if (gnorm <= kMpEps)
            info = 8;
         if (info != 0)
            return info;
         if (ratio >= 1e-4)
            break; // a new Jacobian at the accepted point
         // rejected: wa4 (the free half) is scratch again
      }
   }
}

// One thread per pixel.  MAXR bounds n_rot: the measurement arrays of the
// pixel (7 x 5 MAXR doubles) live in the thread's local memory, which is
// interleaved across the threads of a warp and cached in L1.  Held to 80
// registers (6 CTAs per SM, some values spilled to L1): on 512 x 512 pixels
// of 5 x 9 measurements 319 ms, against 334 ms at 96 registers (5 CTAs),
// 361 ms at 128 (4 CTAs) and 462 ms at 168 (3 CTAs).
template <int MAXR>
__global__ void __launch_bounds__(128, 6)
rofl_fit(const double *__restrict__ data, int64_t n_pix, const unsigned char *__restrict__ mask,
         const RoflParams P, double *__restrict__ out, unsigned long long *__restrict__ status) {
   constexpr int MAXM = 5 * MAXR;
   const int R = P.n_rot, M = 5 * R;
   double c[MAXM], w[MAXM], F[2 * MAXM], J[3 * MAXM];
   // pixels are taken one at a time from a counter (status[1]): a thread
   // whose fit ended early starts the next pixel instead of idling until
   // the slowest pixel of a fixed share is done
   for (;;) {
      const int64_t p = (int64_t)atomicAdd(&status[1], 1ull);
      if (p >= n_pix)
         break;
      double *o = out + 8 * p;
      if (mask && !mask[p]) {
#pragma unroll
         for (int e = 0; e < 8; e++)
            o[e] = nan("");
         continue;
      }
      // tilt t, rotation k of pixel p: data[(t * n_pix + p) * R + k]
      double trans[5];
#pragma unroll
      for (int t = 0; t < 5; t++) {
         const double *d = data + (t * n_pix + p) * R;
         trans[t] = np_sum([&](int k) { return d[k]; }, R) / R; // np.mean
      }
      // epa.direction of the untilted series (epa.py:48-77) + dir_offset
      double phi0;
      {
         const double *d0 = data + p * R;
         const double a1 = 2.0 * np_sum([&](int k) { return d0[k] * P.rho2s[k]; }, R) / R;
         const double b1 = 2.0 * np_sum([&](int k) { return d0[k] * P.rho2c[k]; }, R) / R;
         phi0 = pymod(0.5 * atan2(-b1, a1) + M_PI, M_PI) + P.dir_offset;
      }
      // _calc_centered_vals (:47-61)
#pragma unroll
      for (int t = 0; t < 5; t++) {
         const double *d = data + (t * n_pix + p) * R;
         const double tr = trans[t], tr2 = tr * tr, tr3r = cube_rn(tr) * R;
         for (int k = 0; k < R; k++) {
            const double v = d[k];
            c[t * R + k] = v / tr - 1.0;
            w[t * R + k] = 1.0 / sqrt(P.gain * (v / tr2 + v * v / tr3r));
         }
      }
      // start grid (:261-328): inclination outer, t_rel inner, the first
      // minimum of the pairwise row sums (np.argmin: a NaN wins)
      double x[3] = {phi0, P.incl[0], P.trel[0]};
      {
         double best = INFINITY;
         for (int a = 0; a < 6; a++)
            for (int t = 0; t < 6; t++) {
               px_residuals(P, c, w, phi0, P.incl[a], P.trel[t], F);
               const double cost = np_sum([&](int i) { return F[i] * F[i]; }, M);
               if (cost < best || (isnan(cost) && !isnan(best))) {
                  best = cost;
                  x[1] = P.incl[a];
                  x[2] = P.trel[t];
               }
            }
      }
      // MINPACK's fit, as scipy.optimize.leastsq runs it for the reference
      int n_fev = 0, cur = 0;
      const int info = mp_fit<MAXM>(P, c, w, M, x, F, cur, J, n_fev);
      if (info == 5)
         atomicAdd(&status[0], 1ull); // evaluation budget reached
      const double *fv = F + cur * MAXM;
      const double cost = np_sum([&](int i) { return fv[i] * fv[i]; }, M); // np.sum(np.square)
      // result (:488-520): fold, |t_rel|, covariance from the reference's
      // Jacobian at the folded point and its own 3x3 inverse
      double d = x[0], a = x[1];
      symmetrize(d, a);
      const double t = fabs(x[2]);
      const double sigma_sq = cost / (double)(M - 3);
      const int col[3] = {0, MAXM, 2 * MAXM};
      px_jacobi(P, w, d, a, t, J, col);
      double s[6] = {0, 0, 0, 0, 0, 0};
      for (int i = 0; i < M; i++) {
         const double j0 = J[i], j1 = J[MAXM + i], j2 = J[2 * MAXM + i];
         s[0] += j0 * j0;
         s[1] += j0 * j1;
         s[2] += j0 * j2;
         s[3] += j1 * j1;
         s[4] += j1 * j2;
         s[5] += j2 * j2;
      }
      const double mm[9] = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
      // _invertmatrix (:14-44) with the reference's determinant expression
      // (its fourth term is m20 * m12, without a third factor)
      const double det = mm[0] * mm[4] * mm[8] + mm[3] * mm[7] * mm[2] + mm[6] * mm[5] -
                         mm[0] * mm[7] * mm[5] - mm[6] * mm[4] * mm[2] - mm[3] * mm[1] * mm[8];
      const double i00 = (mm[4] * mm[8] - mm[5] * mm[7]) / det;
      const double i11 = (mm[0] * mm[8] - mm[2] * mm[6]) / det;
      const double i22 = (mm[0] * mm[4] - mm[1] * mm[3]) / det;
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
   // status[0]: pixels at the evaluation limit, status[1]: next pixel
   FPGB_CUDA_TRY(cudaMemsetAsync(status, 0, 2 * sizeof(unsigned long long), st));
   if (n_pix > 0) {
      // as many CTAs as are resident at once (the pixels are taken from the
      // counter), fewer for small maps
      const bool small = P.n_rot <= kRoflSmallRot;
      int dev = 0, sms = 0, per_sm = 0;
      FPGB_CUDA_TRY(cudaGetDevice(&dev));
      FPGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      FPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, small ? rofl_fit<kRoflSmallRot> : rofl_fit<kRoflMaxRot>, 128, 0));
      const int64_t blocks =
          std::max<int64_t>(1, std::min<int64_t>((n_pix + 127) / 128,
                                                 (int64_t)sms * std::max(per_sm, 1)));
      if (small)
         rofl_fit<kRoflSmallRot><<<(unsigned)blocks, 128, 0, st>>>(d_data, n_pix, d_mask, P,
                                                                   d_out, status);
      else
         rofl_fit<kRoflMaxRot><<<(unsigned)blocks, 128, 0, st>>>(d_data, n_pix, d_mask, P,
                                                                 d_out, status);
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
