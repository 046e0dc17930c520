// Instantiations of the 3-D directional sweeps, split precision.
#include "mfc_launch.h"

namespace mfc {

void register_stage_3d_fp32(std::vector<StageEntry>& r) {
  // default: fastest at 256^3, tiles staged by one TMA bulk tensor copy, the
  // z sweep (with the RK combination) register-capped to 5 blocks per SM
  r.push_back(Sweep3D<2, 5, float, 32, 4, 2, 16, 16, 256, true, 5>::entry());
  r.push_back(Sweep3D<2, 5, float, 32, 4, 2, 16, 16, 256, true>::entry());
  r.push_back(Sweep3D<2, 5, float, 32, 4, 2, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 5, float, 32, 8, 1, 16, 16, 256, true>::entry());
  r.push_back(Sweep3D<2, 5, float, 32, 4, 2, 16, 32, 256>::entry());
  r.push_back(Sweep3D<2, 5, float, 32, 8, 1, 16, 16, 256>::entry());
  r.push_back(Sweep3D<2, 5, float, 32, 4, 2, 32, 8, 256>::entry());
  r.push_back(Sweep3D<1, 5, float, 32, 4, 2, 16, 32, 256>::entry());
  r.push_back(Sweep3D<2, 3, float, 32, 4, 2, 16, 32, 256>::entry());
  r.push_back(Sweep3D<2, 1, float, 32, 4, 2, 16, 32, 256>::entry());
}

}  // namespace mfc
