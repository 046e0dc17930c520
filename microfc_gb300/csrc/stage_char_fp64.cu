// Instantiations of the fused stage kernel that reconstructs the
// characteristic fields instead of the primitive variables (FP64, inviscid,
// WENO3/5; the fused kernel in 1-D and 2-D, the directional sweeps in 3-D;
// mfc_gpu_set_reconstruction).  The first entry per
// configuration is the default.
#include "mfc_launch.h"

namespace mfc {

void register_stage_char_fp64(std::vector<StageEntry>& r) {
#define MFC_CHAR(ND, NF, WO, TX, TY, NT) \
  r.push_back(stage_entry<ND, NF, WO, double, TX, TY, NT, false, 1, false, false, false, true>());
  MFC_CHAR(2, 2, 5, 32, 16, 512)
  MFC_CHAR(2, 2, 5, 16, 16, 256)
  MFC_CHAR(2, 1, 5, 32, 16, 512)
  MFC_CHAR(2, 2, 3, 16, 16, 256)
  MFC_CHAR(2, 1, 3, 16, 16, 256)
  MFC_CHAR(1, 2, 5, 128, 1, 128)
  MFC_CHAR(1, 1, 5, 128, 1, 128)
  MFC_CHAR(1, 2, 3, 128, 1, 128)
  MFC_CHAR(1, 1, 3, 128, 1, 128)
#undef MFC_CHAR
  // 3-D: the directional sweeps
  r.push_back(Sweep3D<2, 5, double, 32, 4, 2, 16, 16, 256, false, 0, true>::entry());
  r.push_back(Sweep3D<1, 5, double, 32, 4, 2, 16, 16, 256, false, 0, true>::entry());
  r.push_back(Sweep3D<2, 3, double, 32, 4, 2, 16, 16, 256, false, 0, true>::entry());
}

}  // namespace mfc
