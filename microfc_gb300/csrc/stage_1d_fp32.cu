// Instantiations of the fused stage kernel for 1-D cases, split precision.
#include "mfc_launch.h"

namespace mfc {

void register_stage_1d_fp32(std::vector<StageEntry>& r) {
#define MFC_1D(NF, WO) r.push_back(stage_entry<1, NF, WO, float, 128, 1, 128>());
  MFC_1D(1, 1) MFC_1D(1, 3) MFC_1D(1, 5)
  MFC_1D(2, 1) MFC_1D(2, 3) MFC_1D(2, 5)
#undef MFC_1D
}

}  // namespace mfc
