// Shared host/device plumbing of libfastpli_gb300: error reporting, the
// cached device pool, launch helpers.  No simulation logic lives here.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/fastpli_gb300.h"
#include "../../include/fastpli_gb300_batch.h"

namespace fpgb {

// ---------------------------------------------------------------- errors ---
void set_error(const char *fmt, ...);

#define FPGB_CUDA_TRY(expr)                                                    \
   do {                                                                        \
      cudaError_t e_ = (expr);                                                 \
      if (e_ != cudaSuccess) {                                                 \
         ::fpgb::set_error("%s failed: %s (%s:%d)", #expr,                     \
                           cudaGetErrorString(e_), __FILE__, __LINE__);        \
         return FPGB_ECUDA;                                                    \
      }                                                                        \
   } while (0)

#define FPGB_TRY(expr)                                                         \
   do {                                                                        \
      int rc_ = (expr);                                                        \
      if (rc_ != FPGB_OK)                                                      \
         return rc_;                                                           \
   } while (0)

// Device status word bits written by kernels (never __trap: a kernel that
// detects bad input records it and carries on with a safe value).
enum StatusBits : unsigned {
   kStatusLabelRange = 1u << 0, // a label < 0 or >= n_props was met
   kStatusTimeout = 1u << 1,    // a bounded wait gave up
   kStatusOverflow = 1u << 2,   // a capacity was exceeded
};

// Per-call device counters: [0..5] fpgb_warnings order, [6] status bits,
// [7] label min, [8] label max.
constexpr int kCounterWords = 10;

// ------------------------------------------------------------ device pool ---
// Grow-only cache of device buffers per (device, slot), reused across calls
// of the host-buffer entry points so repeated calls do not cudaMalloc.
enum PoolSlot : int {
   kSlotLabel = 0,
   kSlotVector,
   kSlotImage,
   kSlotKeys,
   kSlotSegments,
   kSlotCounters,
   kSlotProps,
   kSlotEpa,
   kSlotStaging,
   kSlotOptic,
   kNumSlots
};
// Buffers are cached per (device, stream, slot, host thread): concurrent
// calls never share a buffer, and a buffer is only grown (freed and
// re-allocated) by the thread that owns it.  pool_release_all frees every
// buffer of the device and must not overlap other calls of the library.
int pool_get(int slot, size_t bytes, void **ptr, cudaStream_t stream = nullptr);
int pool_release_all();
// Frees the calling thread's buffers on the current device (after
// synchronising it): for threads that end, e.g. a server's worker.
int pool_release_thread();

// Touch one byte of every page of a host output buffer from several threads,
// so that the device-to-host copy that follows finds its pages mapped.  A
// copy into never-touched pageable memory is paced by page faults (one
// thread, ~25 GB/s on a Grace host with 64 KiB pages); faulting the pages in
// parallel first, while the GPU still computes, lets the copy itself run at
// ~145 GB/s.  The bytes written are overwritten by the copy.  Buffers under
// 8 MiB are left alone.
void prefault_host(void *p, size_t bytes);
// Whether host pointer p is page-locked (its copies run asynchronously at
// the link's rate).
bool host_pinned(const void *p);

// Which x end of a volume the last device-resident pass on the current device
// finished at (1 = high x, 0 = low x or unknown); the march starts there so
// its first rays hit the part of the volume still in L2.  Performance only.
std::atomic<int> &l2_end_state();

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

inline cudaStream_t as_stream(void *s) {
   return reinterpret_cast<cudaStream_t>(s);
}

int warnings_from_counters(const long long *h, fpgb_warnings *w);

} // namespace fpgb
