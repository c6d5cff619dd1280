// Host-side check of the voxelizer's counter-block decode shared by
// fpgb_generate_tissue_device, fpgb_generate_tissue and
// fpgb_generate_tissue_noalloc (tissue_status_from_counters): a block whose
// status word carries the binning-overflow bit must turn into FPGB_ECUDA
// with an error message, with or without a warnings struct; a clean block
// must decode into the reference's warning counts.  No GPU is touched.
//
//   nvcc -O2 -std=c++17 -I include tests/native/tissue_status_check.cu -o check && ./check
#include <cstdio>
#include <cstring>

#include "../../fastpli_gb300/csrc/capi.cu"
#include "../../fastpli_gb300/csrc/tissue.cu"
#include "../../fastpli_gb300/csrc/voxel_bricks.cu"

using namespace fpgb;

static int fails = 0;
#define CHECK(c)                                                                   \
   do {                                                                            \
      if (!(c)) {                                                                  \
         std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);                   \
         fails++;                                                                  \
      }                                                                            \
   } while (0)

int main() {
   TissuePlan p;
   p.single_point = 3;
   long long h[kCounterWords] = {};
   h[0] = 17; // overlapping voxels
   h[2] = 4;  // zero axis
   h[5] = 2;  // layer overflow
   fpgb_warnings w;
   std::memset(&w, 0x55, sizeof w);
   CHECK(tissue_status_from_counters(p, h, &w) == FPGB_OK);
   CHECK(w.overlap == 1 && w.single_point == 3 && w.zero_axis == 4 && w.layer_overflow == 2);
   CHECK(tissue_status_from_counters(p, h, nullptr) == FPGB_OK);

   h[6] = kStatusOverflow;
   CHECK(tissue_status_from_counters(p, h, &w) == FPGB_ECUDA);
   CHECK(std::strstr(fpgb_last_error(), "overflowed") != nullptr);
   fpgb::set_error("%s", "");
   CHECK(tissue_status_from_counters(p, h, nullptr) == FPGB_ECUDA);
   CHECK(std::strstr(fpgb_last_error(), "overflowed") != nullptr);

   h[6] = kStatusLabelRange; // other status bits are not the voxelizer's
   CHECK(tissue_status_from_counters(p, h, &w) == FPGB_OK);
   std::printf("%s\n", fails ? "FAILED" : "ok");
   return fails ? 1 : 0;
}
