// Throughput microbenchmarks for the roofline of the forward model (not part
// of the path's C ABI; built into a separate library, libfpgb_peaks.so).
//
// The march's roofline is the slowest of HBM, FP32 and SFU throughput at the
// per-step operation counts of the reference formulas; the voxelizer's is
// FP64 or L2-atomic throughput per candidate test.  MEASURED_PEAKS.json holds
// HBM and bf16 only, so these kernels measure the rest on the device they run
// on: independent dependency chains in every thread, a grid of 8 resident
// blocks per SM, timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void fp32_fma(float *out, int iters, float a, float b) {
   float x[kChains];
#pragma unroll
   for (int c = 0; c < kChains; c++)
      x[c] = threadIdx.x + c;
   for (int i = 0; i < iters; i++)
#pragma unroll
      for (int c = 0; c < kChains; c++)
         x[c] = fmaf(x[c], a, b);
   float s = 0.f;
#pragma unroll
   for (int c = 0; c < kChains; c++)
      s += x[c];
   out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void fp64_fma(double *out, int iters, double a, double b) {
   double x[kChains];
#pragma unroll
   for (int c = 0; c < kChains; c++)
      x[c] = threadIdx.x + c;
   for (int i = 0; i < iters; i++)
#pragma unroll
      for (int c = 0; c < kChains; c++)
         x[c] = fma(x[c], a, b);
   double s = 0.0;
#pragma unroll
   for (int c = 0; c < kChains; c++)
      s += x[c];
   out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// one special-function-unit operation (the approximate reciprocal square
// root, a single instruction) per chain step
__device__ __forceinline__ float rsqrt_approx(float x) {
   float y;
   asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
   return y;
}

__global__ void sfu_rsqrt(float *out, int iters) {
   float x[kChains];
#pragma unroll
   for (int c = 0; c < kChains; c++)
      x[c] = 1.f + threadIdx.x + c;
   for (int i = 0; i < iters; i++)
#pragma unroll
      for (int c = 0; c < kChains; c++)
         x[c] = rsqrt_approx(x[c]);
   float s = 0.f;
#pragma unroll
   for (int c = 0; c < kChains; c++)
      s += x[c];
   out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// atomicMin on 64-bit words spread over a buffer that stays in L2
__global__ void l2_atomics(unsigned long long *buf, unsigned mask, int iters) {
   unsigned h = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u;
   for (int i = 0; i < iters; i++) {
      h = h * 1664525u + 1013904223u;
      atomicMin(&buf[h & mask], (unsigned long long)h);
   }
}

int sms_now() {
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   return sms > 0 ? sms : 1;
}

template <class F> double timed(F launch, cudaStream_t st) {
   launch(); // warm-up
   cudaEvent_t e0, e1;
   cudaEventCreate(&e0);
   cudaEventCreate(&e1);
   cudaEventRecord(e0, st);
   launch();
   cudaEventRecord(e1, st);
   cudaEventSynchronize(e1);
   float ms = 0.f;
   cudaEventElapsedTime(&ms, e0, e1);
   cudaEventDestroy(e0);
   cudaEventDestroy(e1);
   return ms * 1e-3;
}

} // namespace

extern "C" {

// out[0] FP32 flop/s (2 per FMA), out[1] SFU op/s, out[2] FP64 flop/s,
// out[3] L2 64-bit atomicMin/s.  Returns 0, or a CUDA error code.
int fpgb_measure_peaks(double *out, void *stream) {
   cudaStream_t st = static_cast<cudaStream_t>(stream);
   const int blocks = sms_now() * 8;
   const int64_t threads = (int64_t)blocks * kThreads;
   void *buf = nullptr;
   const size_t atom_words = size_t(1) << 20; // 8 MB: L2-resident
   if (cudaMalloc(&buf, sizeof(double) * threads + sizeof(unsigned long long) * atom_words))
      return (int)cudaGetLastError();
   float *f = static_cast<float *>(buf);
   double *d = static_cast<double *>(buf);
   auto *a = reinterpret_cast<unsigned long long *>(static_cast<char *>(buf) +
                                                    sizeof(double) * threads);
   cudaMemsetAsync(a, 0xFF, sizeof(unsigned long long) * atom_words, st);
   const int it32 = 4096, itsfu = 1024, it64 = 64, itat = 64;
   const double t32 = timed([&] { fp32_fma<<<blocks, kThreads, 0, st>>>(f, it32, 0.999f, 1e-3f); }, st);
   const double tsf = timed([&] { sfu_rsqrt<<<blocks, kThreads, 0, st>>>(f, itsfu); }, st);
   const double t64 = timed([&] { fp64_fma<<<blocks, kThreads, 0, st>>>(d, it64, 0.999, 1e-3); }, st);
   const double tat = timed(
       [&] { l2_atomics<<<blocks, kThreads, 0, st>>>(a, (unsigned)(atom_words - 1), itat); }, st);
   const cudaError_t err = cudaGetLastError();
   cudaFree(buf);
   if (err != cudaSuccess)
      return (int)err;
   out[0] = 2.0 * kChains * (double)it32 * threads / t32;
   out[1] = (double)kChains * itsfu * threads / tsf;
   out[2] = 2.0 * kChains * (double)it64 * threads / t64;
   out[3] = (double)itat * threads / tat;
   return 0;
}

} // extern "C"
