// Instantiations of the fused stage kernel with the viscous terms, FP64
// arithmetic (bit-faithful to the CPU reference): 1-D and 2-D, WENO5.
#include "mfc_launch.h"

namespace mfc {

void register_stage_visc_fp64(std::vector<StageEntry>& r) {
  r.push_back(stage_entry<1, 1, 5, double, 128, 1, 128, false, 1, true>());
  r.push_back(stage_entry<1, 2, 5, double, 128, 1, 128, false, 1, true>());
  r.push_back(stage_entry<2, 1, 5, double, 16, 16, 256, false, 1, true>());
  r.push_back(stage_entry<2, 2, 5, double, 16, 16, 256, false, 1, true>());
  r.push_back(stage_entry<2, 2, 5, double, 32, 16, 512, false, 1, true>());
  r.push_back(stage_entry<2, 2, 5, double, 32, 16, 640, false, 1, true>());
}

}  // namespace mfc
