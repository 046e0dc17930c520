// Ensemble of independent 2-D cases advanced together: one persistent launch
// per RK stage walks a work list of (case, tile) pairs, so 64 small cases of
// uneven size fill the GPU like one large one.  Each tile runs exactly the
// single-case stage_tile, so every case gets the same bits it would get
// alone.  The per-case parameter blocks travel in the kernel's parameter
// space (__grid_constant__), which keeps their fields in the constant bank.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "mfc_device.cuh"
#include "mfc_stage.cuh"

namespace mfc {

constexpr int kMaxEnsemble = 96;

struct EnsCase {
  DevParams P;
  double* reg[3];         // RK registers; reg[0] holds q_cons_ts(1)
  double dt, dt_last;     // the case's dt and its (possibly trimmed) last-step dt
  int tiles_x, tile_base; // tiles per row, first tile in the work list
};

struct EnsParams {
  int num_cases, total_tiles, stage, time_stepper, last_step;
  // TMA maps of every case's registers, [register][case] (device memory),
  // for the tile variant launched; null: plain loads
  const TileMap* maps;
  // split WENO5: the coefficient record every cell of every case shares when
  // all cases have uniform grids (the FP32 records of a uniform grid do not
  // depend on its spacing); all off otherwise
  UniformCoefT<2> U;
  EnsCase c[kMaxEnsemble];
};
static_assert(sizeof(EnsParams) <= 32764, "ensemble parameters must fit the kernel parameter space");

// One persistent block's walk over the work list (the body of both kernels).
// TMA: interior tiles arrive by one bulk tensor copy; the block initialises
// its mbarrier once and alternates its phase per copied tile.
// VISC: every case carries its viscosity parameters (DevParams::visc).
template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool TMA, bool VISC = false>
__device__ __forceinline__ void ensemble_walk(const EnsParams& E) {
  static_assert(!VISC || !TMA, "the viscous ensemble kernels load their tiles plainly");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t parity = 0;
  if constexpr (TMA) {
    if (E.maps != nullptr && threadIdx.x == 0)
      mbar_init(smem_addr(tma_staging<2, NF, WO, RT, TX, TY>(smem_raw) + tma_stage_bytes<2, NF, WO, RT, TX, TY>()),
                1);
    __syncthreads();
  }
  for (int t = blockIdx.x; t < E.total_tiles; t += gridDim.x) {
    int lo = 0, hi = E.num_cases - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (E.c[mid].tile_base <= t) lo = mid;
      else hi = mid - 1;
    }
    const EnsCase& C = E.c[lo];
    const int lt = t - C.tile_base;
    const int x0 = (lt % C.tiles_x) * TX, y0 = (lt / C.tiles_x) * TY;
    const double* in;
    double* out;
    int kind, reg;
    if (E.stage == 0) {
      in = C.reg[0], out = C.reg[1], kind = kRkEuler, reg = 0;
    } else if (E.time_stepper == 2) {
      in = C.reg[1], out = C.reg[0], kind = kRk2Final, reg = 1;
    } else if (E.stage == 1) {
      in = C.reg[1], out = C.reg[2], kind = kRk3Mid, reg = 1;
    } else {
      in = C.reg[2], out = C.reg[0], kind = kRk3Final, reg = 2;
    }
    const TileMap* T = (TMA && E.maps != nullptr) ? E.maps + reg * E.num_cases + lo : nullptr;
    stage_tile<2, NF, WO, RT, TX, TY, NT, GATE, VISC, UniformCoefT<2>, TMA>(
        C.P, in, C.reg[0], out, E.last_step ? C.dt_last : C.dt, kind, x0, y0, smem_raw, &E.U, T, &parity);
    __syncthreads();  // the next tile reuses the shared memory
  }
}

template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool TMA, bool VISC = false>
__global__ void __launch_bounds__(NT) ensemble_stage_kernel(const __grid_constant__ EnsParams E) {
  ensemble_walk<NF, WO, RT, TX, TY, NT, GATE, TMA, VISC>(E);
}

// The same with the registers capped so that MINB blocks fit on an SM.
template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, int MINB, bool TMA>
__global__ void __launch_bounds__(NT, MINB) ensemble_stage_kernel_mb(const __grid_constant__ EnsParams E) {
  ensemble_walk<NF, WO, RT, TX, TY, NT, GATE, TMA>(E);
}

template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, int MINB, bool TMA, bool VISC = false>
constexpr auto ensemble_func() {
  static_assert(!VISC || MINB == 1, "register-capped ensemble variants are inviscid");
  if constexpr (MINB > 1) return &ensemble_stage_kernel_mb<NF, WO, RT, TX, TY, NT, GATE, MINB, TMA>;
  else return &ensemble_stage_kernel<NF, WO, RT, TX, TY, NT, GATE, TMA, VISC>;
}

struct EnsembleEntry {
  int nf, wo, prec, tx, ty, nt;
  size_t smem, smem_shared_coef;  // dynamic shared memory: per-cell records / shared record
  const void* func;
  cudaError_t (*launch)(const EnsParams& E, int grid, size_t smem, cudaStream_t st);
  bool tma;    // interior tiles staged by TMA (needs EnsParams::maps)
  int box_w;   // x extent of the TMA box (cells), box_h rows
  int box_h;
  bool visc;   // compiled with the viscous terms
};

template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, int MINB = 1, bool TMA = false,
          bool VISC = false>
cudaError_t ensemble_launch(const EnsParams& E, int grid, size_t smem, cudaStream_t st) {
  ensemble_func<NF, WO, RT, TX, TY, NT, GATE, MINB, TMA, VISC>()<<<grid, NT, smem, st>>>(E);
  return cudaGetLastError();
}

template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool TMA, bool VISC = false>
constexpr size_t ensemble_smem(bool shared_coef) {
  return stage_smem_total<2, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>(shared_coef);
}

// prec: 0 FP64, 1 split, 2 split with the learned gate
template <int NF, int WO, class RT, int TX, int TY, int NT, bool GATE = false, int MINB = 1, bool TMA = false,
          bool VISC = false>
EnsembleEntry ensemble_entry() {
  using Sh = StageShape<2, NF, WO, RT, TX, TY>;
  return EnsembleEntry{NF,
                       WO,
                       sizeof(RT) == 8 ? 0 : (GATE ? 2 : 1),
                       TX,
                       TY,
                       NT,
                       ensemble_smem<NF, WO, RT, TX, TY, NT, GATE, TMA, VISC>(false),
                       ensemble_smem<NF, WO, RT, TX, TY, NT, GATE, TMA, VISC>(true),
                       reinterpret_cast<const void*>(ensemble_func<NF, WO, RT, TX, TY, NT, GATE, MINB, TMA, VISC>()),
                       &ensemble_launch<NF, WO, RT, TX, TY, NT, GATE, MINB, TMA, VISC>,
                       TMA,
                       TmaBox<TX, Sh::H>::kWidth,
                       Sh::LY,
                       VISC};
}

void register_ensemble_fp64(std::vector<EnsembleEntry>& r);
void register_ensemble_fp32(std::vector<EnsembleEntry>& r);
void register_ensemble_gated(std::vector<EnsembleEntry>& r);

}  // namespace mfc
