// Internal launcher registry: every compiled instantiation of the stage
// kernel registers one entry; the C ABI picks the entry matching the case's
// dimensionality, fluid count, WENO order, precision and tile variant.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "mfc_device.cuh"
#include "mfc_stage.cuh"

namespace mfc {

struct StageEntry {
  int nd, nf, wo, prec;  // prec: 0 = FP64, 1 = split (FP32 WENO/HLLC)
  int tx, ty, nt;
  size_t smem;
  cudaError_t (*prepare)();
  cudaError_t (*launch)(const DevParams& P, const double* qin, const double* qbase, double* qout, double dt,
                        int kind, cudaStream_t st);
};

template <int ND, int NF, int WO, class RT, int TX, int TY, int NT>
cudaError_t stage_prepare() {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY>;
  return cudaFuncSetAttribute(stage_kernel<ND, NF, WO, RT, TX, TY, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)Sh::kSmemBytes);
}

template <int ND, int NF, int WO, class RT, int TX, int TY, int NT>
cudaError_t stage_launch(const DevParams& P, const double* qin, const double* qbase, double* qout, double dt,
                         int kind, cudaStream_t st) {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY>;
  const dim3 grid((unsigned)((P.n[0] + TX - 1) / TX), ND > 1 ? (unsigned)((P.n[1] + TY - 1) / TY) : 1u, 1u);
  stage_kernel<ND, NF, WO, RT, TX, TY, NT><<<grid, NT, Sh::kSmemBytes, st>>>(P, qin, qbase, qout, dt, kind);
  return cudaGetLastError();
}

template <int ND, int NF, int WO, class RT, int TX, int TY, int NT>
StageEntry stage_entry() {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY>;
  return StageEntry{ND, NF, WO, sizeof(RT) == 8 ? 0 : 1, TX, TY, NT, Sh::kSmemBytes,
                    &stage_prepare<ND, NF, WO, RT, TX, TY, NT>, &stage_launch<ND, NF, WO, RT, TX, TY, NT>};
}

// The default (first registered) launcher of a configuration, or nullptr.
const StageEntry* find_stage(int nd, int nf, int wo, int prec);

// Records msg as the calling thread's mfc_gpu_last_error() and returns code.
int report_error(int code, const std::string& msg);

// Defined in the instantiation translation units.
void register_stage_1d_fp64(std::vector<StageEntry>& r);
void register_stage_1d_fp32(std::vector<StageEntry>& r);
void register_stage_2d_fp64(std::vector<StageEntry>& r);
void register_stage_2d_fp32(std::vector<StageEntry>& r);

}  // namespace mfc
