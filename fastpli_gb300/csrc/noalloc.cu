// Voxelizer entry point that allocates no device memory.
//
// The regular device entry point (fpgb_generate_tissue_device) needs a
// scratch workspace: the segment and layer tables and the segment lists of
// the voxel bricks (the per-voxel keys live in shared memory).  It takes that workspace from the caller or from the library's own
// cudaMalloc'ed pool.  Some callers can do neither: applications whose
// device memory is already owned by another allocator (a framework that has
// reserved the GPU for its caching allocator, a host that budgets HBM per
// tenant), or code paths that must not issue allocation calls at all
// (cudaMalloc and cudaFree synchronize the device and can fail under memory
// pressure mid-run).  fpgb_generate_tissue_noalloc serves them: its scratch
// is a fixed, file-scope __device__ array of kNoAllocScratchBytes that every
// GPU loading this library holds until the process exits.
//
// Rules of use (also in include/fastpli_gb300.h):
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture;
//   * every call on a device shares the same array and the array keeps the
//     previous call's contents; each call re-initialises the parts it reads
//     (tables, brick counts and lists, counters) before use;
//   * calls whose device work overlaps (different streams, or host threads
//     without ordering) race on the array: serialise them;
//   * problems whose scratch exceeds the array are rejected with
//     FPGB_EINVAL before any device work.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "fpgb_common.cuh"
#include "tissue.cuh"

namespace fpgb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20; // 64 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// the symbol g_noalloc_scratch names a host-side shadow, not device memory,
// so the address must come from the runtime.
int noalloc_scratch(void **out) {
   int dev = 0;
   FPGB_CUDA_TRY(cudaGetDevice(&dev));
   if (dev < 0 || dev >= kMaxDevices) {
      set_error("generate_tissue_noalloc: device ordinal %d out of range", dev);
      return FPGB_EINVAL;
   }
   std::lock_guard<std::mutex> lk(g_noalloc_mu);
   if (!g_noalloc_ptr[dev]) {
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
         set_error("generate_tissue_noalloc: cudaGetSymbolAddress failed: %s",
                   cudaGetErrorString(e));
         return FPGB_ECUDA;
      }
      g_noalloc_ptr[dev] = p;
   }
   *out = g_noalloc_ptr[dev];
   return FPGB_OK;
}

} // namespace
} // namespace fpgb

using namespace fpgb;

extern "C" int fpgb_generate_tissue_noalloc(const fpgb_volume *vol, const fpgb_fibers *fibers,
                                            int only_label, int32_t *d_label,
                                            float *d_vector, double *props,
                                            int64_t props_cap, int64_t *n_props,
                                            fpgb_warnings *warnings, void *stream) {
   TissuePlan p;
   FPGB_TRY(plan_tissue(vol, fibers, &p));
   if (!d_label || (!only_label && !d_vector)) {
      set_error("generate_tissue_noalloc: null output buffer");
      return FPGB_EINVAL;
   }
   const size_t need = tissue_workspace_bytes(p);
   if (need > kNoAllocScratchBytes) {
      set_error("generate_tissue_noalloc: this volume (%lld voxels) and its %zu fiber "
                "segments need %zu bytes of scratch, more than the fixed %zu bytes; "
                "use fpgb_generate_tissue_device with a workspace instead",
                (long long)(p.X * p.Y * p.Z), p.segs.size(), need, kNoAllocScratchBytes);
      return FPGB_EINVAL;
   }
   const int64_t rows = (int64_t)p.props.size() / 2;
   if (props && props_cap < rows) { // refused before any device work
      set_error("props_cap %lld < %lld rows", (long long)props_cap, (long long)rows);
      return FPGB_EINVAL;
   }
   void *scratch = nullptr;
   FPGB_TRY(noalloc_scratch(&scratch));
   cudaStream_t st = as_stream(stream);
   unsigned long long *d_counters = nullptr;
   FPGB_TRY(run_tissue(p, only_label, d_label, d_vector, scratch, kNoAllocScratchBytes,
                       &d_counters, st));
   // the same completion as fpgb_generate_tissue_device: props, then the
   // warnings and the binning-overflow status from the counter block
   FPGB_TRY(finish_props(p, props, props_cap, n_props));
   return read_tissue_warnings(p, d_counters, warnings, st);
}
