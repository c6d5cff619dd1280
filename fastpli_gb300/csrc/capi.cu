// Library-wide C-ABI helpers: error string, version, cached device pool,
// host page pre-faulting.
#include <cuda_runtime.h>
#include <omp.h>
#include <unistd.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <utility>

#include "fpgb_common.cuh"

namespace fpgb {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
   char buf[1024];
   va_list ap;
   va_start(ap, fmt);
   vsnprintf(buf, sizeof buf, fmt, ap);
   va_end(ap);
   g_last_error = buf;
}

namespace {
struct PoolEntry {
   void *ptr = nullptr;
   size_t bytes = 0;
};
std::mutex g_pool_mu;
// A buffer is keyed by the calling host thread as well as by (device,
// stream, slot): a call takes its buffers, then enqueues work into them after
// the pool lock is dropped, so a buffer may only ever be replaced by the
// thread that uses it.  Two threads on one stream (e.g. the legacy default
// stream) therefore never free each other's buffers mid-call.
struct PoolKey {
   int dev;
   uintptr_t stream;
   int slot;
   std::thread::id thread;
   bool operator<(const PoolKey &o) const {
      if (dev != o.dev)
         return dev < o.dev;
      if (stream != o.stream)
         return stream < o.stream;
      if (slot != o.slot)
         return slot < o.slot;
      return thread < o.thread;
   }
};
std::map<PoolKey, PoolEntry> g_pool;
} // namespace

int pool_get(int slot, size_t bytes, void **ptr, cudaStream_t stream) {
   int dev = 0;
   FPGB_CUDA_TRY(cudaGetDevice(&dev));
   std::lock_guard<std::mutex> lk(g_pool_mu);
   PoolEntry &e =
       g_pool[PoolKey{dev, reinterpret_cast<uintptr_t>(stream), slot, std::this_thread::get_id()}];
   if (e.bytes < bytes) {
      if (e.ptr) {
         // This thread's earlier calls may still have work queued on any
         // stream that uses the buffer: wait for the device before giving
         // the memory back.
         FPGB_CUDA_TRY(cudaDeviceSynchronize());
         FPGB_CUDA_TRY(cudaFree(e.ptr));
         e.ptr = nullptr;
         e.bytes = 0;
      }
      size_t want = align_up(bytes < 256 ? 256 : bytes, 1 << 20);
      cudaError_t err = cudaMalloc(&e.ptr, want);
      if (err != cudaSuccess) {
         e.ptr = nullptr;
         set_error("device pool: cudaMalloc(%zu) failed: %s", want,
                   cudaGetErrorString(err));
         return FPGB_ENOMEM;
      }
      e.bytes = want;
   }
   *ptr = e.ptr;
   return FPGB_OK;
}

std::atomic<int> &l2_end_state() {
   static std::atomic<int> state[64] = {};
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
      dev = 0;
   return state[dev];
}

bool host_pinned(const void *p) {
   cudaPointerAttributes a;
   const bool pinned =
       p && cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost;
   cudaGetLastError();
   return pinned;
}

void prefault_host(void *p, size_t bytes) {
   if (!p || bytes < (size_t(8) << 20))
      return;
   if (host_pinned(p))
      return; // page-locked: resident already
   const int64_t pg = (int64_t)sysconf(_SC_PAGESIZE);
   if (pg <= 0)
      return;
   volatile char *c = static_cast<volatile char *>(p);
   const int64_t n = ((int64_t)bytes + pg - 1) / pg;
#pragma omp parallel for schedule(static) num_threads(std::min(16, omp_get_max_threads()))
   for (int64_t i = 0; i < n; i++)
      c[i * pg] = 0;
}

int pool_release_all() {
   int dev = 0;
   FPGB_CUDA_TRY(cudaGetDevice(&dev));
   std::lock_guard<std::mutex> lk(g_pool_mu);
   FPGB_CUDA_TRY(cudaDeviceSynchronize());
   for (auto it = g_pool.begin(); it != g_pool.end();) {
      if (it->first.dev == dev) {
         if (it->second.ptr)
            FPGB_CUDA_TRY(cudaFree(it->second.ptr));
         it = g_pool.erase(it);
      } else {
         ++it;
      }
   }
   return FPGB_OK;
}

int pool_release_thread() {
   int dev = 0;
   FPGB_CUDA_TRY(cudaGetDevice(&dev));
   const std::thread::id me = std::this_thread::get_id();
   std::lock_guard<std::mutex> lk(g_pool_mu);
   bool any = false;
   for (const auto &kv : g_pool)
      any = any || (kv.first.dev == dev && kv.first.thread == me && kv.second.ptr);
   if (!any)
      return FPGB_OK;
   FPGB_CUDA_TRY(cudaDeviceSynchronize()); // this thread's queued work may still use them
   for (auto it = g_pool.begin(); it != g_pool.end();) {
      if (it->first.dev == dev && it->first.thread == me) {
         if (it->second.ptr)
            FPGB_CUDA_TRY(cudaFree(it->second.ptr));
         it = g_pool.erase(it);
      } else {
         ++it;
      }
   }
   return FPGB_OK;
}

int warnings_from_counters(const long long *h, fpgb_warnings *w) {
   if (!w)
      return FPGB_OK;
   w->overlap = h[0];
   w->single_point = h[1];
   w->zero_axis = h[2];
   w->not_normalized = h[3];
   w->empty_light = h[4];
   w->layer_overflow = h[5];
   return FPGB_OK;
}

} // namespace fpgb

extern "C" {

const char *fpgb_last_error(void) { return fpgb::g_last_error.c_str(); }

const char *fpgb_version(void) { return "fastpli_gb300 0.1.0 (sm_103a)"; }

int fpgb_release_pool(void) { return fpgb::pool_release_all(); }

int fpgb_release_thread_pool(void) { return fpgb::pool_release_thread(); }

} // extern "C"
