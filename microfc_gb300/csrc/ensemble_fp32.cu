// Instantiations of the ensemble stage kernel, split precision.
#include "mfc_ensemble.cuh"

namespace mfc {

void register_ensemble_fp32(std::vector<EnsembleEntry>& r) {
  r.push_back(ensemble_entry<2, 5, float, 32, 16, 256>());
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256>());
  r.push_back(ensemble_entry<2, 5, float, 32, 8, 256>());
  r.push_back(ensemble_entry<2, 5, float, 32, 32, 512>());
  r.push_back(ensemble_entry<2, 5, float, 64, 8, 256>());
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, false, 4>());
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, false, 5>());
  // interior tiles staged by one TMA bulk tensor copy
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, false, 5, true>());
  // with the viscous terms (mfc_gpu_ensemble_set_viscosity)
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, false, 1, false, true>());
  r.push_back(ensemble_entry<2, 5, float, 32, 16, 256, false, 1, false, true>());
}

}  // namespace mfc

namespace mfc {

void register_ensemble_gated(std::vector<EnsembleEntry>& r) {
  r.push_back(ensemble_entry<2, 5, float, 32, 16, 256, true>());
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, true>());
  r.push_back(ensemble_entry<2, 5, float, 32, 32, 512, true>());
  // register-capped 16x16 tiles: four or five blocks per SM
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, true, 4>());
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, true, 5>());
  // interior tiles staged by one TMA bulk tensor copy (four blocks per SM:
  // the five-block cap spills the TMA kernel's registers)
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, true, 4, true>());
  // with the viscous terms (mfc_gpu_ensemble_set_viscosity)
  r.push_back(ensemble_entry<2, 5, float, 16, 16, 256, true, 1, false, true>());
}

}  // namespace mfc
