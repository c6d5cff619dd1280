// Host-side check of the voxelizer's two-float fast path: for every
// candidate of random fiber segments, fast_candidate()/fast_radial() must
// either decline (FP64 replay) or return exactly the floats that the FP64
// replay of the reference arithmetic returns.  Runs on the CPU only (the
// evaluation functions are __host__ __device__); no GPU is touched.
//
//   nvcc -O2 -std=c++17 -fmad=false -Xcompiler -ffp-contract=off \
//        -I include tests/native/voxel_fastpath_check.cu -o check && ./check SEED N
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "../../fastpli_gb300/csrc/capi.cu"
#include "../../fastpli_gb300/csrc/tissue.cu"
#include "../../fastpli_gb300/csrc/voxel_bricks.cu"

using namespace fpgb;

int main(int argc, char **argv) {
   const unsigned seed = argc > 1 ? (unsigned)atoi(argv[1]) : 1u;
   const int n_fibers = argc > 2 ? atoi(argv[2]) : 200;
   // mode 1: lattice-aligned fibers (axis-parallel, quarter-voxel
   // coordinates, radii with exact squares) that produce exact ties
   const int mode = argc > 3 ? atoi(argv[3]) : 0;
   std::mt19937_64 rng(seed);
   std::uniform_real_distribution<double> U(0.0, 1.0);
   fpgb_volume vol{{96, 80, 64}, {0.37, -1.25, 0.5}, 0.2};
   std::vector<double> pts;
   std::vector<int64_t> foff{0};
   for (int f = 0; f < n_fibers; f++) {
      const int n = 2 + (int)(U(rng) * 6);
      double c[3] = {U(rng) * 19.2, U(rng) * 16.0, U(rng) * 12.8};
      double d[3] = {U(rng) - 0.5, U(rng) - 0.5, U(rng) - 0.5};
      double r0 = 0.3 + U(rng) * 1.5;
      bool taper = f % 3 == 0;
      if (mode == 1) {
         for (int i = 0; i < 3; i++) {
            c[i] = std::floor(c[i] * 4.0) / 4.0;
            d[i] = 0;
         }
         d[f % 3] = (f % 2) ? 1.0 : -1.0;
         r0 = 0.2 * (1 + f % 5) ;
         taper = false;
      }
      for (int k = 0; k < n; k++) {
         for (int i = 0; i < 3; i++)
            pts.push_back(c[i] + d[i] * 4.0 * k + (mode == 1 ? 0.0 : (U(rng) - 0.5) * 0.5));
         pts.push_back(taper ? r0 * (0.6 + 0.8 * U(rng)) : r0);
      }
      foff.push_back(foff.back() + n);
   }
   const int64_t boff[2] = {0, n_fibers};
   const int64_t loff[2] = {0, 3};
   const double sc[3] = {0.5, 0.8, 1.0}, dn[3] = {0, -0.002, 0.004}, mu[3] = {1, 2, 3};
   const char md[3] = {'b', 'p', 'r'};
   fpgb_fibers fb{1, boff, foff.data(), pts.data(), loff, sc, dn, mu, md};
   TissuePlan plan;
   if (plan_tissue(&vol, &fb, &plan) != FPGB_OK) {
      printf("plan failed: %s\n", fpgb_last_error());
      return 2;
   }
   long long n = 0, fast = 0, bad = 0, vec_fast = 0, vec_bad = 0;
   long long bound_bad = 0, certain = 0, certain_bad = 0;
   double worst = 0.0; // largest |reference - estimate| / bound
   for (const SegDev &S : plan.segs) {
      for (int ix = 0; ix < S.ext[0]; ix++)
         for (int iy = 0; iy < S.ext[1]; iy++)
            for (int iz = 0; iz < S.ext[2]; iz++) {
               const int64_t x = S.lo[0] + ix, y = S.lo[1] + iy, z = S.lo[2] + iz;
               const double pt[3] = {x + 0.5, y + 0.5, z + 0.5};
               double cl[3];
               float d_ex, r_ex;
               exact_dist(S, pt, cl, d_ex, r_ex);
               const float lpt[3] = {(float)(x - S.base[0]) + 0.5f,
                                     (float)(y - S.base[1]) + 0.5f,
                                     (float)(z - S.base[2]) + 0.5f};
               // FP32 estimate and its two-sided bound, and the certain-accept
               // threshold of the two-pass key sweep
               float mg;
               const float d2f = approx_dist2(lpt[0] - S.pf[0], lpt[1] - S.pf[1],
                                              lpt[2] - S.pf[2], S.vf[0], S.vf[1], S.vf[2],
                                              S.c2f, S.c2_rcp, mg);
               worst = std::max(worst, std::fabs((double)d_ex - (double)d2f) / (double)mg);
               if (!((double)d_ex <= (double)d2f + mg && (double)d_ex >= (double)d2f - mg)) {
                  if (bound_bad < 5)
                     printf("BOUND dist %.9g estimate %.9g margin %.3g\n", d_ex, d2f, mg);
                  bound_bad++;
               }
               if ((double)d2f + mg <= (double)S.acc_f) {
                  certain++;
                  if (d_ex > sc[2] * sc[2] * r_ex) // generator.cpp:329-331, outermost layer
                     certain_bad++;
               }
               FastCand fc;
               n++;
               if (!fast_candidate(S, lpt, fc))
                  continue;
               fast++;
               if (fc.dist_squ != d_ex || fc.r_sqr != r_ex) {
                  if (bad < 5)
                     printf("MISMATCH seg dist %.9g vs %.9g r2 %.9g vs %.9g\n", fc.dist_squ,
                            d_ex, fc.r_sqr, r_ex);
                  bad++;
               }
               float o[3];
               if (fast_radial(S, fc, o)) {
                  vec_fast++;
                  double nv[3] = {pt[0] - cl[0], pt[1] - cl[1], pt[2] - cl[2]};
                  double n2 = 0.0;
                  n2 = n2 + nv[0] * nv[0];
                  n2 = n2 + nv[1] * nv[1];
                  n2 = n2 + nv[2] * nv[2];
                  const double inv = 1.0 / std::sqrt(n2);
                  for (int i = 0; i < 3; i++)
                     if ((float)(nv[i] * inv) != o[i])
                        vec_bad++;
               }
            }
   }
   printf("candidates %lld fast %lld (%.6f) mismatches %lld vectors_fast %lld vector_mismatches %lld"
          " bound_violations %lld (largest error %.3f of the bound) certain %lld"
          " certain_rejected %lld\n",
          n, fast, n ? (double)fast / n : 0.0, bad, vec_fast, vec_bad, bound_bad, worst, certain,
          certain_bad);
   return (bad || vec_bad || bound_bad || certain_bad) ? 1 : 0;
}
