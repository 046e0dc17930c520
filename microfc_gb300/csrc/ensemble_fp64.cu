// Instantiations of the ensemble stage kernel, FP64 (bit-faithful) arithmetic.
#include "mfc_ensemble.cuh"

namespace mfc {

void register_ensemble_fp64(std::vector<EnsembleEntry>& r) {
  r.push_back(ensemble_entry<2, 5, double, 16, 16, 256>());
  r.push_back(ensemble_entry<2, 5, double, 32, 16, 512>());
  r.push_back(ensemble_entry<2, 5, double, 32, 8, 256>());
  // with the viscous terms (mfc_gpu_ensemble_set_viscosity)
  r.push_back(ensemble_entry<2, 5, double, 16, 16, 256, false, 1, false, true>());
  r.push_back(ensemble_entry<2, 5, double, 32, 16, 512, false, 1, false, true>());
}

}  // namespace mfc
