// Instantiations of the fused stage kernel for 2-D cases, FP64 arithmetic.
// Tile variants (TX x TY cells, NT threads) are chosen by the autotuner; the
// first entry per configuration is the default until it runs (on GB300 the
// autotuner takes the 640-thread TMA entry for two fluids and WENO5).
#include "mfc_launch.h"

namespace mfc {

void register_stage_2d_fp64(std::vector<StageEntry>& r) {
// 32x16 tiles with 544 threads (17 warps): the 528 x faces and 544 y faces
// of a tile take one pass each, as do its 3808 x reconstructions (7 per
// thread), so fewer threads wait at the barriers between the phases.
#define MFC_2D(NF, WO)                                           \
  r.push_back(stage_entry<2, NF, WO, double, 32, 16, 512>());   \
  r.push_back(stage_entry<2, NF, WO, double, 16, 16, 256>());   \
  r.push_back(stage_entry<2, NF, WO, double, 32, 16, 544>());
  MFC_2D(2, 5)
  MFC_2D(1, 5)
#undef MFC_2D
  // interior tiles staged by one TMA bulk tensor copy
  r.push_back(stage_entry<2, 2, 5, double, 32, 16, 544, false, 1, false, true>());
  r.push_back(stage_entry<2, 2, 5, double, 32, 16, 512, false, 1, false, true>());
  r.push_back(stage_entry<2, 2, 5, double, 16, 16, 256, false, 1, false, true>());
  // 640 threads (20 warps, 96 registers: five warps on each sub-partition):
  // the fastest on GB300 (1.12e8 cell-updates/s at 1024x512 against 1.10e8
  // for 544 threads; 576/608 in between, 672-768 capped at 80 registers and
  // slower)
  r.push_back(stage_entry<2, 2, 5, double, 32, 16, 640, false, 1, false, true>());
  r.push_back(stage_entry<2, 2, 3, double, 16, 16, 256>());
  r.push_back(stage_entry<2, 2, 1, double, 16, 16, 256>());
  r.push_back(stage_entry<2, 1, 3, double, 16, 16, 256>());
  r.push_back(stage_entry<2, 1, 1, double, 16, 16, 256>());
}

}  // namespace mfc
