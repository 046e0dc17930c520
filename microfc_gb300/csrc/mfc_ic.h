// Device initial condition (pre_process on the GPU): the target state block
// and the launcher shared by the single-case and ensemble entry points.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/mfc_gpu.h"

namespace mfc {

struct IcTarget {
  int nd, nf;
  int n[3];               // interior cells per used direction
  int64_t sy, sz, sv;     // element strides of the SoA block
  const double* gammas;   // num_fluids values
  const double* pi_infs;
  double* q;              // register 0 of the case
  const double* cb[3];    // host cell boundaries x_cb(-1:m) ... of the case, or null
};

// Launches the generator on `stream`; returns "" or the reason it refused.
// domain == null: the grid is t.cb (any rectilinear grid, e.g. stretched).
std::string generate_ic(const IcTarget& t, const mfc_patch* patches, int num_patches, const double* domain,
                        cudaStream_t stream, int64_t* launches);

}  // namespace mfc
