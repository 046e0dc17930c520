// Instantiations of the 3-D directional sweeps, FP64 arithmetic.
#include "mfc_launch.h"

namespace mfc {

void register_stage_3d_fp64(std::vector<StageEntry>& r) {
  r.push_back(Sweep3D<2, 5, double, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 5, double, 32, 4, 2, 16, 16, 256, true>::entry());  // TMA-staged tiles
  r.push_back(Sweep3D<1, 5, double, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 3, double, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 1, double, 32, 4, 2, 16, 16, 256>::entry());
}

}  // namespace mfc
