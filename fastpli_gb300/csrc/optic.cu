// Optic stage after the ray march (src/fastpli/simulation/optic.py) and epa
// on arbitrary image stacks (src/fastpli/analysis/epa.py:9-45).
//
//   filter_resample  optic.py:169-187: for every polarizer angle, a 2-D
//                    Gaussian blur of width sigma / scale (scipy.ndimage
//                    gaussian_filter semantics: separable, axis 0 then
//                    axis 1, mode 'reflect', truncate 4.0, FP64), then the
//                    block-average resample of optic.py:85-120 (every input
//                    pixel i goes to floor((i + 0.5) * scale), summed in
//                    input order and divided by the count).  Images stay in
//                    the march's [X, Y, n_rho] layout throughout.
//   noise            the negative-binomial CCD model the reference's
//                    pipelines use (noise_model = lambda x:
//                    np.random.negative_binomial(x / (g - 1), 1 / g),
//                    e.g. tests/simulation/simpli_test.py:276-277): a Gamma
//                    mixture of Poissons, sampled per pixel from a
//                    counter-based generator, so a pixel's draw depends only
//                    on (seed, offset + pixel index).
//   epa              t, d, r of an image stack, FP64.
//
// Compiled with -fmad=false: the filter sums are formed in scipy's order
// (centre tap first, then symmetric pairs from the outermost inward) with
// every product and sum rounded separately.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "fpgb_common.cuh"

namespace fpgb {

constexpr int kMaxRadius = 255;

struct GaussTaps {
   int radius;
   double w[kMaxRadius + 1]; // w[j] = weight at offset +-j
};

// scipy.ndimage._gaussian_kernel1d(sigma, 0, radius) with
// radius = int(truncate * sigma + 0.5): exp(-0.5 / sigma^2 * x^2) normalised.
static int gauss_taps(double sd, GaussTaps &g) {
   const double r = 4.0 * sd + 0.5;
   if (!(r < kMaxRadius + 1)) {
      set_error("optic: filter width %g needs more than %d taps per side", sd, kMaxRadius);
      return FPGB_EINVAL;
   }
   g.radius = (int)r;
   const double k = -0.5 / (sd * sd);
   std::vector<double> full(2 * g.radius + 1);
   double sum = 0.0;
   for (int x = -g.radius; x <= g.radius; x++) {
      full[x + g.radius] = std::exp(k * (double)((int64_t)x * x));
      sum += full[x + g.radius];
   }
   for (int j = 0; j <= g.radius; j++)
      g.w[j] = full[g.radius + j] / sum;
   return FPGB_OK;
}

// mode 'reflect' (d c b a | a b c d | d c b a), repeated for short lines
__device__ __forceinline__ int64_t reflect_index(int64_t i, int64_t n) {
   const int64_t p = 2 * n;
   int64_t m = i % p;
   if (m < 0)
      m += p;
   return m < n ? m : p - 1 - m;
}

// One axis of the separable filter over [X, Y, R]: `stride` is the element
// distance between neighbours along the axis, `n` its length.
__global__ void gauss_axis(const double *__restrict__ in, double *__restrict__ out, int64_t total,
                           int64_t n, int64_t stride, const GaussTaps g) {
   for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
        e += (int64_t)gridDim.x * blockDim.x) {
      const int64_t c = (e / stride) % n; // position along the axis
      const double *base = in + (e - c * stride);
      // correlate1d with a symmetric kernel (scipy ni_filters.c order):
      // centre tap first, then (x[c-j] + x[c+j]) * w[j] from j = radius down
      double acc = base[c * stride] * g.w[0];
      for (int j = g.radius; j >= 1; j--) {
         const double a = base[reflect_index(c - j, n) * stride];
         const double b = base[reflect_index(c + j, n) * stride];
         acc = acc + (a + b) * g.w[j];
      }
      out[e] = acc;
   }
}

// Block-average resample: output pixel (u, v, r) sums input rows
// [xo[u], xo[u+1]) and columns [yo[v], yo[v+1]) in input order (optic.py:
// 103-117) and divides by the count (0 / 0 = NaN as numpy's divide).
__global__ void resample_blocks(const double *__restrict__ in, double *__restrict__ out,
                                int64_t Y, int64_t R, int64_t SX, int64_t SY,
                                const int64_t *__restrict__ xo, const int64_t *__restrict__ yo) {
   const int64_t total = SX * SY * R;
   for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
        e += (int64_t)gridDim.x * blockDim.x) {
      const int64_t r = e % R, uv = e / R;
      const int64_t u = uv / SY, v = uv - (uv / SY) * SY;
      double acc = 0.0;
      for (int64_t i = xo[u]; i < xo[u + 1]; i++)
         for (int64_t j = yo[v]; j < yo[v + 1]; j++)
            acc = acc + in[(i * Y + j) * R + r];
      const int64_t cnt = (xo[u + 1] - xo[u]) * (yo[v + 1] - yo[v]);
      out[e] = acc / (double)cnt;
   }
}

// ------------------------------------------------------------------ noise ---
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): 10 rounds of the 4x32 bijection keyed by a
// 64-bit key, on a 128-bit counter.
struct U4 {
   unsigned x, y, z, w;
};

__device__ __forceinline__ U4 philox(U4 c, unsigned k0, unsigned k1) {
#pragma unroll
   for (int i = 0; i < 10; i++) {
      const unsigned lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
      const unsigned lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
      c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
   }
   return c;
}

// Stream of uniforms in (0, 1) for one pixel: blocks of four 32-bit words,
// 53-bit doubles from two words.
struct PixelRng {
   U4 ctr;
   unsigned k0, k1;
   U4 buf;
   int left;
   __device__ PixelRng(uint64_t seed, uint64_t pixel) {
      ctr = U4{(unsigned)pixel, (unsigned)(pixel >> 32), 0u, 0u};
      k0 = (unsigned)seed;
      k1 = (unsigned)(seed >> 32);
      left = 0;
   }
   __device__ unsigned next32() {
      if (left == 0) {
         buf = philox(ctr, k0, k1);
         ctr.z++;
         if (ctr.z == 0)
            ctr.w++;
         left = 4;
      }
      const unsigned v = left == 4 ? buf.x : left == 3 ? buf.y : left == 2 ? buf.z : buf.w;
      left--;
      return v;
   }
   __device__ double uniform() { // (0, 1): never 0, never 1
      const uint64_t a = next32() >> 5, b = next32() >> 6;
      return ((double)(a * 67108864ull + b) + 0.5) * 0x1p-53;
   }
   __device__ double normal() { // Box-Muller
      const double u = uniform(), v = uniform();
      return sqrt(-2.0 * log(u)) * cospi(2.0 * v);
   }
};

constexpr int kMaxRejections = 1000;

// Gamma(shape k, scale 1): Marsaglia & Tsang, "A simple method for
// generating gamma variables", ACM TOMS 26 (2000); k < 1 via
// Gamma(k + 1) * U^(1/k).
__device__ double gamma_sample(PixelRng &g, double k, bool &ok) {
   double boost = 1.0;
   if (k < 1.0) {
      boost = pow(g.uniform(), 1.0 / k);
      k += 1.0;
   }
   const double d = k - 1.0 / 3.0, c = 1.0 / sqrt(9.0 * d);
   for (int it = 0; it < kMaxRejections; it++) {
      const double x = g.normal();
      double v = 1.0 + c * x;
      if (v <= 0.0)
         continue;
      v = v * v * v;
      const double u = g.uniform();
      if (log(u) < 0.5 * x * x + d - d * v + d * log(v))
         return d * v * boost;
   }
   ok = false;
   return k * boost;
}

// Poisson(lam): multiplication method below 10, otherwise PTRS (Hoermann,
// "The transformed rejection method for generating Poisson random
// variables", Insurance: Mathematics and Economics 12, 1993).
__device__ double poisson_sample(PixelRng &g, double lam, bool &ok) {
   if (lam <= 0.0)
      return 0.0;
   if (lam < 10.0) {
      const double L = exp(-lam);
      double p = 1.0;
      for (int k = 0; k < 4 * kMaxRejections; k++) {
         p *= g.uniform();
         if (p <= L)
            return (double)k;
      }
      ok = false;
      return lam;
   }
   const double slam = sqrt(lam), loglam = log(lam);
   const double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
   const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
   for (int it = 0; it < kMaxRejections; it++) {
      const double U = g.uniform() - 0.5, V = g.uniform();
      const double us = 0.5 - fabs(U);
      const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
      if (us >= 0.07 && V <= vr)
         return k;
      if (k < 0.0 || (us < 0.013 && V > us))
         continue;
      if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0))
         return k;
   }
   ok = false;
   return lam;
}

// out = NegBinomial(n = x / (gain - 1), p = 1 / gain) per pixel: Poisson of
// a Gamma(n, scale gain - 1) rate (mean x, variance gain * x).  Pixels with
// x <= 0 or non-finite x are flagged (numpy refuses n <= 0) and copied.
__global__ void nb_noise(const double *__restrict__ in, double *__restrict__ out, int64_t n,
                         double gain, uint64_t seed, uint64_t offset,
                         unsigned long long *__restrict__ status) {
   unsigned long long bad = 0, stuck = 0;
   for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
        e += (int64_t)gridDim.x * blockDim.x) {
      const double x = in[e];
      if (!(x > 0.0) || !isfinite(x)) {
         out[e] = x;
         bad++;
         continue;
      }
      PixelRng g(seed, offset + (uint64_t)e);
      bool ok = true;
      const double lam = gamma_sample(g, x / (gain - 1.0), ok) * (gain - 1.0);
      out[e] = poisson_sample(g, lam, ok);
      stuck += ok ? 0 : 1;
   }
   if (bad)
      atomicAdd(&status[0], bad);
   if (stuck)
      atomicAdd(&status[1], stuck);
}

// -------------------------------------------------------------------- epa ---
// epa.py:9-45 in FP64: a0 = mean, a1 = 2 mean(I sin 2rho), b1 = 2 mean(I cos 2rho)
// with rho = linspace(0, pi, n, endpoint=False); t = 2 a0,
// d = (atan2(-b1, a1) / 2 + pi) mod pi, r = |(a1, b1)| / a0 (a0 < 100 eps -> 1).
struct EpaTable {
   int n;
   double s[64], c[64];
};

__global__ void epa_stack(const double *__restrict__ img, int64_t n_pix, const EpaTable T,
                          double *__restrict__ t, double *__restrict__ d,
                          double *__restrict__ r) {
   for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_pix;
        p += (int64_t)gridDim.x * blockDim.x) {
      const double *I = img + p * T.n;
      double s0 = 0.0, s1 = 0.0, s2 = 0.0;
      for (int k = 0; k < T.n; k++) {
         const double v = I[k];
         s0 = s0 + v;
         s1 = s1 + v * T.s[k];
         s2 = s2 + v * T.c[k];
      }
      double a0 = s0 / T.n;
      const double a1 = 2.0 * s1 / T.n, b1 = 2.0 * s2 / T.n;
      t[p] = 2.0 * a0;
      double dd = 0.5 * atan2(-b1, a1) + M_PI;
      dd = fmod(dd, M_PI); // operands positive: Python's % and fmod agree
      d[p] = dd;
      if (a0 < 100.0 * 2.220446049250313e-16)
         a0 = 1.0;
      r[p] = sqrt(a1 * a1 + b1 * b1) / a0;
   }
}

static unsigned grid_for(int64_t n, int threads) {
   return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 64));
}

} // namespace fpgb

using namespace fpgb;

extern "C" {

int fpgb_optic_resample_size(int64_t X, int64_t Y, double scale, int64_t *out_dim) {
   if (X <= 0 || Y <= 0 || !(scale > 0.0) || !std::isfinite(scale) || !out_dim) {
      set_error("optic: need X, Y > 0 and a finite scale > 0");
      return FPGB_EINVAL;
   }
   // int(round(n * scale)): Python rounds halves to even, as rint does
   out_dim[0] = (int64_t)std::nearbyint((double)X * scale);
   out_dim[1] = (int64_t)std::nearbyint((double)Y * scale);
   return FPGB_OK;
}

int fpgb_optic_filter_resample_device(const double *d_image, int64_t X, int64_t Y, int64_t n_rho,
                                      double sigma, double scale, double *d_out, void *stream) {
   int64_t od[2];
   FPGB_TRY(fpgb_optic_resample_size(X, Y, scale, od));
   if (!d_image || !d_out || n_rho <= 0 || !(sigma >= 0.0) || !std::isfinite(sigma)) {
      set_error("optic: null buffer, n_rho <= 0 or sigma not finite and >= 0");
      return FPGB_EINVAL;
   }
   const int64_t SX = od[0], SY = od[1];
   if (SX <= 0 || SY <= 0) {
      set_error("optic: scale %g turns %lldx%lld into an empty image", scale, (long long)X,
                (long long)Y);
      return FPGB_EINVAL;
   }
   cudaStream_t st = as_stream(stream);
   // block boundaries: input pixel i goes to floor((i + 0.5) * scale)
   // (optic.py:103-110), a non-decreasing map; pixels past the last output
   // row are dropped
   std::vector<int64_t> bounds(SX + 1 + SY + 1);
   auto fill = [&](int64_t n, int64_t S, int64_t *b) {
      int64_t i = 0;
      for (int64_t u = 0; u <= S; u++) {
         while (i < n && (int64_t)std::floor(((double)i + 0.5) * scale) < u)
            i++;
         b[u] = i;
      }
   };
   fill(X, SX, bounds.data());
   fill(Y, SY, bounds.data() + SX + 1);
   const int64_t total = X * Y * n_rho;
   void *ws = nullptr;
   const size_t tmp_bytes = align_up(sizeof(double) * total, 256);
   FPGB_TRY(pool_get(kSlotOptic, 2 * tmp_bytes + sizeof(int64_t) * bounds.size(), &ws, st));
   double *t0 = static_cast<double *>(ws);
   double *t1 = reinterpret_cast<double *>(static_cast<char *>(ws) + tmp_bytes);
   auto *d_bounds = reinterpret_cast<int64_t *>(static_cast<char *>(ws) + 2 * tmp_bytes);
   FPGB_CUDA_TRY(cudaMemcpyAsync(d_bounds, bounds.data(), sizeof(int64_t) * bounds.size(),
                                 cudaMemcpyHostToDevice, st));
   const double *src = d_image;
   if (sigma > 0.0) { // optic.py:52-53: sigma == 0 leaves the image as is
      GaussTaps g;
      std::memset(&g, 0, sizeof g);
      FPGB_TRY(gauss_taps(sigma / scale, g));
      gauss_axis<<<grid_for(total, 256), 256, 0, st>>>(d_image, t0, total, X, Y * n_rho, g);
      FPGB_CUDA_TRY(cudaGetLastError());
      gauss_axis<<<grid_for(total, 256), 256, 0, st>>>(t0, t1, total, Y, n_rho, g);
      FPGB_CUDA_TRY(cudaGetLastError());
      src = t1;
   }
   resample_blocks<<<grid_for(SX * SY * n_rho, 256), 256, 0, st>>>(
       src, d_out, Y, n_rho, SX, SY, d_bounds, d_bounds + SX + 1);
   FPGB_CUDA_TRY(cudaGetLastError());
   return FPGB_OK;
}

int fpgb_optic_filter_resample(const double *image, int64_t X, int64_t Y, int64_t n_rho,
                               double sigma, double scale, double *out) {
   int64_t od[2];
   FPGB_TRY(fpgb_optic_resample_size(X, Y, scale, od));
   if (!image || !out) {
      set_error("optic: null buffer");
      return FPGB_EINVAL;
   }
   const int64_t n_in = X * Y * n_rho, n_out = od[0] * od[1] * n_rho;
   void *d_in = nullptr, *d_out = nullptr;
   FPGB_TRY(pool_get(kSlotImage, sizeof(double) * n_in, &d_in));
   FPGB_TRY(pool_get(kSlotEpa, sizeof(double) * n_out, &d_out));
   cudaStream_t st = nullptr;
   prefault_host(out, sizeof(double) * n_out);
   FPGB_CUDA_TRY(cudaMemcpyAsync(d_in, image, sizeof(double) * n_in, cudaMemcpyHostToDevice, st));
   FPGB_TRY(fpgb_optic_filter_resample_device((const double *)d_in, X, Y, n_rho, sigma, scale,
                                              (double *)d_out, st));
   FPGB_CUDA_TRY(cudaMemcpyAsync(out, d_out, sizeof(double) * n_out, cudaMemcpyDeviceToHost, st));
   FPGB_CUDA_TRY(cudaStreamSynchronize(st));
   return FPGB_OK;
}

int fpgb_optic_noise_device(const double *d_in, int64_t n, double gain, uint64_t seed,
                            uint64_t offset, double *d_out, int64_t *n_invalid, void *stream) {
   if (!d_in || !d_out || n < 0 || !(gain > 1.0) || !std::isfinite(gain)) {
      set_error("optic noise: null buffer, n < 0 or gain not finite and > 1");
      return FPGB_EINVAL;
   }
   cudaStream_t st = as_stream(stream);
   void *w = nullptr;
   FPGB_TRY(pool_get(kSlotCounters, sizeof(unsigned long long) * kCounterWords, &w, st));
   auto *status = static_cast<unsigned long long *>(w);
   FPGB_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned long long) * 2, st));
   if (n > 0) {
      nb_noise<<<grid_for(n, 128), 128, 0, st>>>(d_in, d_out, n, gain, seed, offset, status);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   if (n_invalid) {
      unsigned long long h[2];
      FPGB_CUDA_TRY(cudaMemcpyAsync(h, status, sizeof h, cudaMemcpyDeviceToHost, st));
      FPGB_CUDA_TRY(cudaStreamSynchronize(st));
      if (h[1]) {
         set_error("optic noise: %llu samplers hit their iteration limit", h[1]);
         return FPGB_ETIMEOUT;
      }
      *n_invalid = (int64_t)h[0];
   }
   return FPGB_OK;
}

int fpgb_epa_device(const double *d_image, int64_t n_pix, int64_t n_rho, double *d_t,
                    double *d_d, double *d_r, void *stream) {
   if (!d_image || !d_t || !d_d || !d_r || n_pix < 0 || n_rho <= 0 || n_rho > 64) {
      set_error("epa: null buffer, n_pix < 0 or n_rho outside 1..64");
      return FPGB_EINVAL;
   }
   EpaTable T;
   std::memset(&T, 0, sizeof T);
   T.n = (int)n_rho;
   for (int k = 0; k < T.n; k++) { // 2 * linspace(0, pi, n, endpoint=False)
      const double rho2 = 2.0 * ((M_PI / (double)n_rho) * (double)k);
      T.s[k] = std::sin(rho2);
      T.c[k] = std::cos(rho2);
   }
   if (n_pix > 0) {
      epa_stack<<<grid_for(n_pix, 128), 128, 0, as_stream(stream)>>>(d_image, n_pix, T, d_t, d_d,
                                                                     d_r);
      FPGB_CUDA_TRY(cudaGetLastError());
   }
   return FPGB_OK;
}

} // extern "C"
