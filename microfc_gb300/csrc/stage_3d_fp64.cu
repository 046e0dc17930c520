// Instantiations of the 3-D directional sweeps, FP64 arithmetic.
#include "mfc_launch.h"

namespace mfc {

void register_stage_3d_fp64(std::vector<StageEntry>& r) {
  r.push_back(Sweep3D<2, 5, double, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 5, double, 32, 4, 2, 16, 16, 256, true>::entry());  // TMA-staged tiles
  // 320 threads at 96 registers, two blocks per SM (20 warps): 7.09e7
  // cell-updates/s at 256^3 against 7.02e7 for 256 threads
  r.push_back(Sweep3D<2, 5, double, 32, 4, 2, 16, 16, 320, true, 2, false, 2>::entry());
  r.push_back(Sweep3D<1, 5, double, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 3, double, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 1, double, 32, 4, 2, 16, 16, 256>::entry());
}

}  // namespace mfc
