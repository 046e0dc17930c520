// Instantiations of the fused stage kernel for 2-D cases, split precision:
// FP32 WENO and HLLC, FP64 state, pressure recovery and RK update.
#include "mfc_launch.h"

namespace mfc {

void register_stage_2d_fp32(std::vector<StageEntry>& r) {
  // the first entry is the default: the autotuner's usual choice on GB300,
  // interior tiles staged by one TMA bulk tensor copy
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, false, 5, false, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, false, 5>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 16, 256>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 32, 512>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 8, 256>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256>());
  r.push_back(stage_entry<2, 2, 5, float, 64, 8, 512>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, false, 6>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 8, 128>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 128>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 16, 256, false, 1, false, true>());
  r.push_back(stage_entry<2, 1, 5, float, 32, 16, 256>());
  r.push_back(stage_entry<2, 2, 3, float, 32, 16, 256>());
  r.push_back(stage_entry<2, 2, 1, float, 32, 16, 256>());
  r.push_back(stage_entry<2, 1, 3, float, 32, 16, 256>());
  r.push_back(stage_entry<2, 1, 1, float, 32, 16, 256>());
  // split precision with the learned WENO gate
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, true, 5, false, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, true, 5>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 16, 256, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, true>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 32, 512, true>());
  r.push_back(stage_entry<2, 2, 5, float, 32, 8, 256, true>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 16, 256, true, 4>());
  r.push_back(stage_entry<2, 2, 5, float, 16, 8, 128, true, 8>());
  r.push_back(stage_entry<2, 1, 5, float, 32, 16, 256, true>());
}

}  // namespace mfc
