// Instantiations of the fused stage kernel with the viscous terms, split
// precision (FP32 reconstruction, Riemann and viscous fluxes; FP64 state):
// 1-D and 2-D, WENO5.
#include "mfc_launch.h"

namespace mfc {

void register_stage_visc_fp32(std::vector<StageEntry>& r) {
  r.push_back(stage_entry<1, 1, 5, float, 128, 1, 128, false, 1, true>());
  r.push_back(stage_entry<1, 2, 5, float, 128, 1, 128, false, 1, true>());
  r.push_back(stage_entry<2, 1, 5, float, 16, 16, 256, false, 1, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, false, 1, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, false, 4, true>());
  // with the learned WENO gate (the gate chooses the weights; the viscous
  // fluxes are those of the split path)
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, true, 1, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, true, 4, true>());
  r.push_back(stage_entry<2, 1, 5, float, 16, 16, 256, true, 1, true>());
}

}  // namespace mfc
