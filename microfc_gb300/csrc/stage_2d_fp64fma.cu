// Instantiations of the fused stage kernel for 2-D WENO5 cases in FP64 with
// the compiler's multiply-add contraction (MFC_PREC_FP64_FMA).  This unit is
// compiled with -fmad=true (microfc_gb300/build.py): the same source as the
// bit-faithful FP64 kernels, but adds and multiplies may fuse into FMAs, as
// a CPU build of the reference with default flags fuses them.  The results
// are no longer bit-identical to the contraction-off oracle; their distance
// from it is measured by tests/test_fp64_fma.py and reported by bench.py.
#include "mfc_launch.h"

namespace mfc {

void register_stage_2d_fp64fma(std::vector<StageEntry>& r) {
#define MFC_2D_FMA(NF)                                                           \
  r.push_back(stage_entry<2, NF, 5, double, 32, 16, 544, false, 1, false, false, true>()); \
  r.push_back(stage_entry<2, NF, 5, double, 32, 16, 512, false, 1, false, false, true>()); \
  r.push_back(stage_entry<2, NF, 5, double, 16, 16, 256, false, 1, false, false, true>());
  MFC_2D_FMA(2)
  MFC_2D_FMA(1)
#undef MFC_2D_FMA
  r.push_back(stage_entry<2, 2, 5, double, 32, 16, 640, false, 1, false, false, true>());
}

}  // namespace mfc
