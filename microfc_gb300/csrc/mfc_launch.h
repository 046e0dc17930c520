// Internal launcher registry: every compiled instantiation of the stage
// kernel registers one entry; the C ABI picks the entry matching the case's
// dimensionality, fluid count, WENO order, precision and tile variant.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include <type_traits>
#include <utility>

#include "../../include/mfc_gpu.h"
#include "mfc_device.cuh"
#include "mfc_stage.cuh"
#include "mfc_sweep.cuh"

namespace mfc {

struct StageEntry {
  int nd, nf, wo, prec;  // prec: an MFC_PREC_* value
  int tx, ty, nt;
  size_t smem;
  int kernels;  // kernel launches per RK stage (1 in 1-D/2-D, 3 sweeps in 3-D)
  cudaError_t (*prepare)();
  cudaError_t (*launch)(const DevParams& P, const UniformCoef& U, const double* qin, const double* qbase,
                        double* qout, double dt, int kind, cudaStream_t st);
  bool visc = false;  // compiled with the viscous terms
  bool tma = false;   // interior tiles staged by a TMA bulk tensor copy
  bool chr = false;   // WENO of the characteristic fields (MFC_RECON_CHARACTERISTIC)
};

// Launches a stage kernel with programmatic stream serialization, so that
// it may become resident while the previous kernel on the stream drains
// (the kernel waits for that kernel's results with griddep_wait).
template <class... KArgs, class... Args>
cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                             Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// MINB > 1 selects the register-capped kernel (stage_kernel_mb); TMA the
// kernel that stages interior tiles with a bulk tensor copy; FMA the
// instantiations compiled with multiply-add contraction (MFC_PREC_FP64_FMA).
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, int MINB, bool VISC, bool TMA = false,
          bool FMA = false, bool CHAR = false>
constexpr auto stage_func() {
  static_assert(MINB == 1 || !VISC || !TMA, "register-capped viscous variants load their tiles without TMA");
  static_assert(!TMA || (ND == 2 && !VISC), "TMA staging is compiled for the inviscid 2-D kernel");
  static_assert(!CHAR || (!TMA && MINB == 1), "characteristic-field WENO uses the plain stage kernel");
  if constexpr (TMA && MINB > 1) return &stage_kernel_tma_mb<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, FMA>;
  else if constexpr (TMA) return &stage_kernel_tma<ND, NF, WO, RT, TX, TY, NT, GATE, FMA>;
  else if constexpr (MINB > 1) return &stage_kernel_mb<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, FMA, VISC>;
  else return &stage_kernel<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, FMA, CHAR>;
}

// Dynamic shared memory of a launch: without the coefficient records on a
// uniform grid; a TMA kernel's records sit past its staging area.
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool VISC, bool TMA>
constexpr size_t stage_launch_smem(bool shared_coef) {
  return stage_smem_total<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>(shared_coef);
}

template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE = false, int MINB = 1, bool VISC = false,
          bool TMA = false, bool FMA = false, bool CHAR = false>
cudaError_t stage_prepare() {
  return cudaFuncSetAttribute(stage_func<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, VISC, TMA, FMA, CHAR>(),
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)stage_launch_smem<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>(false));
}

template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE = false, int MINB = 1, bool VISC = false,
          bool TMA = false, bool FMA = false, bool CHAR = false>
cudaError_t stage_launch(const DevParams& P, const UniformCoef& U, const double* qin, const double* qbase,
                         double* qout, double dt, int kind, cudaStream_t st) {
  const dim3 grid((unsigned)((P.n[0] + TX - 1) / TX), ND > 1 ? (unsigned)((P.n[1] + TY - 1) / TY) : 1u, 1u);
  // a uniform grid stages no coefficient records: launch without their share
  const bool shared_coef = U.on[0] && (ND < 2 || U.on[1]);
  const size_t smem = stage_launch_smem<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>(shared_coef);
  if constexpr (TMA) {
    // the map of this launch's input register; without one (a layout the
    // copy engine does not take) every tile takes the plain loads
    using Sh = StageShape<ND, NF, WO, RT, TX, TY>;
    TileMap T{};
    encode_tile_map(T, qin, P.n[0], P.n[1], Sh::S, P.sy, P.sv, TmaBox<TX, Sh::H>::kWidth, Sh::LY);
    return launch_dependent(stage_func<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, VISC, TMA, FMA, CHAR>(), grid, dim3(NT), smem,
                            st, P, U, T, qin, qbase, qout, dt, kind);
  } else {
    return launch_dependent(stage_func<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, VISC, TMA, FMA, CHAR>(), grid, dim3(NT), smem,
                            st, P, U, qin, qbase, qout, dt, kind);
  }
}

// prec of a registry entry: 0 FP64, 1 split, 2 split with the learned gate,
// 3 FP64 with multiply-add contraction
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE = false, int MINB = 1, bool VISC = false,
          bool TMA = false, bool FMA = false, bool CHAR = false>
StageEntry stage_entry() {
  static_assert(!FMA || sizeof(RT) == 8, "the contracted variant is FP64");
  return StageEntry{ND,
                    NF,
                    WO,
                    FMA ? 3 : sizeof(RT) == 8 ? 0 : (GATE ? 2 : 1),
                    TX,
                    TY,
                    NT,
                    stage_launch_smem<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>(false),
                    1,
                    &stage_prepare<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, VISC, TMA, FMA, CHAR>,
                    &stage_launch<ND, NF, WO, RT, TX, TY, NT, GATE, MINB, VISC, TMA, FMA, CHAR>,
                    VISC,
                    TMA,
                    CHAR};
}

// 3-D: three directional sweeps per stage (mfc_sweep.cuh).  The x sweep uses
// TA0 x TB0 x TC0 tiles (x along the sweep); the y and z sweeps use
// TA1 x TB1 x 1 tiles with x across the pencils.  TMA: tiles whose sweep
// halo lies inside the domain arrive by one bulk tensor copy.
// MINB2 > 0 caps the registers of the z sweep (which also does the RK
// combination) so that MINB2 of its blocks fit on an SM; MINB01 does the same
// for the x and y sweeps.
template <int NF, int WO, class RT, int TA0, int TB0, int TC0, int TA1, int TB1, int NT, bool TMA = false,
          int MINB2 = 0, bool CHAR = false, int MINB01 = 0>
struct Sweep3D {
  template <int DIR>
  using K = std::conditional_t<DIR == 0, SweepShape<NF, WO, RT, 0, TA0, TB0, TC0>,
                               SweepShape<NF, WO, RT, DIR, TA1, TB1, 1>>;
  template <int DIR>
  static constexpr auto func() {
    if constexpr (DIR == 0) return &sweep_kernel<NF, WO, RT, 0, TA0, TB0, TC0, NT, TMA, MINB01, CHAR>;
    else if constexpr (DIR == 2) return &sweep_kernel<NF, WO, RT, 2, TA1, TB1, 1, NT, TMA, MINB2, CHAR>;
    else return &sweep_kernel<NF, WO, RT, DIR, TA1, TB1, 1, NT, TMA, MINB01, CHAR>;
  }

  template <int DIR>
  static cudaError_t prep() {
    return cudaFuncSetAttribute(func<DIR>(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K<DIR>::kSmemBytes);
  }
  static cudaError_t prepare() {
    cudaError_t e = prep<0>();
    if (e == cudaSuccess) e = prep<1>();
    if (e == cudaSuccess) e = prep<2>();
    return e;
  }
  // the map of the sweep's box (none: plain loads): the stage input for the
  // x sweep, the primitives the x sweep stores (the work buffer's second
  // segment, reconstruction type) for the y and z sweeps
  template <int DIR>
  static TileMap tile_map(const DevParams& P, const double* qin) {
    TileMap T{};
    if constexpr (TMA && K<DIR>::kTmaFits) {
      constexpr int S = K<DIR>::S;
      const void* base = DIR == 0 ? static_cast<const void*>(qin)
                                  : static_cast<const void*>(static_cast<const RT*>(P.work) + int64_t(S) * P.sv);
      encode_tile_map_3d(T, base, K<DIR>::kStageElem, P.n[0], P.n[1], P.n[2], S, P.sy, P.sz, P.sv, K<DIR>::BX,
                         K<DIR>::BY, K<DIR>::BZ);
    }
    return T;
  }
  static cudaError_t launch(const DevParams& P, const UniformCoef& U, const double* qin, const double* qbase,
                            double* qout, double dt, int kind, cudaStream_t st) {
    const unsigned nx = P.n[0], ny = P.n[1], nz = P.n[2];
    const dim3 g0((nx + TA0 - 1) / TA0, (ny + TB0 - 1) / TB0, (nz + TC0 - 1) / TC0);
    const dim3 g1((nx + TB1 - 1) / TB1, (ny + TA1 - 1) / TA1, nz);
    const dim3 g2((nx + TB1 - 1) / TB1, (nz + TA1 - 1) / TA1, ny);
    const TileMap T0 = tile_map<0>(P, qin), T1 = tile_map<1>(P, qin), T2 = tile_map<2>(P, qin);
    cudaError_t e =
        launch_dependent(func<0>(), g0, dim3(NT), K<0>::kSmemBytes, st, P, U, T0, qin, qbase, qout, dt, kind);
    if (e == cudaSuccess)
      e = launch_dependent(func<1>(), g1, dim3(NT), K<1>::kSmemBytes, st, P, U, T1, qin, qbase, qout, dt, kind);
    if (e == cudaSuccess)
      e = launch_dependent(func<2>(), g2, dim3(NT), K<2>::kSmemBytes, st, P, U, T2, qin, qbase, qout, dt, kind);
    return e;
  }
  static StageEntry entry() {
    static_assert(!TMA || (K<0>::kTmaFits && K<1>::kTmaFits && K<2>::kTmaFits),
                  "the TMA box of every sweep must fit its WENO and flux arrays");
    return StageEntry{3, NF, WO, sizeof(RT) == 8 ? 0 : 1, TA0, TB1, NT, K<1>::kSmemBytes, 3, &prepare, &launch,
                      false, TMA, CHAR};
  }
};

// What the standalone entry points of other translation units need from a
// context (mfc_gpu_ctx is private to mfc_capi.cu).
struct CtxView {
  const DevParams* dev = nullptr;  // the context's kernel parameters
  const double* q0 = nullptr;      // register 0 (q_cons_ts(1))
  cudaStream_t stream = nullptr;
  int nd = 0, nf = 0, wo = 0, S = 0, prec = 0;
  int n[3] = {1, 1, 1};
  bool visc = false, has_proc = false;
  int64_t* launches = nullptr;     // the context's launch counter
};
bool ctx_view(mfc_gpu_ctx* c, CtxView& v);

// The context's device scratch, at least `bytes` long (grown on demand, freed
// with the context); for entry points that synchronise before returning.
cudaError_t ctx_scratch(mfc_gpu_ctx* c, size_t bytes, void** out);

// weno_Re_flux = T (mfc_visc_grad.cu): device buffers of the gradient
// preparation -- the velocities ([ND][ny+10][nx+10] from x = y = -5; one row
// in 1-D), the cell gradients ([ND*ND][ny+6][nx+6] from x = y = -3; one row
// in 1-D), the face gradients (ViscParams::fg), the cell widths of each
// direction for cells -kCoefPad .. n-1+kCoefPad and, for the split and gated
// precisions, an FP32 table per direction: the WENO coefficients of those
// cells ([kNumCoef][n + 2 kCoefPad]) followed by their inverse widths.
struct ViscGradBuffers {
  double* vel = nullptr;
  double* g = nullptr;
  double* fg[2] = {nullptr, nullptr};
  double* w[2] = {nullptr, nullptr};
  float* cf[2] = {nullptr, nullptr};
};
// Prepares the face gradients of the stage input q on stream st (3 launches
// in 1-D, 4 in 2-D), reconstructing in FP32 when fp32 is set (split and
// gated contexts), else in FP64.
cudaError_t visc_gradients_launch(int nd, int nf, bool fp32, const DevParams& P, const ViscGradBuffers& B,
                                  const double* q, cudaStream_t st);

// The default (first registered) launcher of a configuration, or nullptr.
const StageEntry* find_stage(int nd, int nf, int wo, int prec, bool visc = false, bool chr = false);

// Records msg as the calling thread's mfc_gpu_last_error() and returns code.
int report_error(int code, const std::string& msg);

// Gate training samples of a 2-D state (mfc_gate.cu).
int gate_samples(const DevParams& P, int nf, const double* q, int dir, float* xout, float* dev_out, cudaStream_t st);

// FP32 gate parameters (host) -> FP16 device copy (mfc_gate.cu).
int gate_upload(const float* host_params, void* dev_half, cudaStream_t st);

// Defined in the instantiation translation units.
void register_stage_1d_fp64(std::vector<StageEntry>& r);
void register_stage_1d_fp32(std::vector<StageEntry>& r);
void register_stage_2d_fp64(std::vector<StageEntry>& r);
void register_stage_2d_fp64fma(std::vector<StageEntry>& r);
void register_stage_2d_fp32(std::vector<StageEntry>& r);
void register_stage_3d_fp64(std::vector<StageEntry>& r);
void register_stage_3d_fp32(std::vector<StageEntry>& r);
void register_stage_visc_fp64(std::vector<StageEntry>& r);
void register_stage_visc_fp32(std::vector<StageEntry>& r);
void register_stage_char_fp64(std::vector<StageEntry>& r);

}  // namespace mfc
