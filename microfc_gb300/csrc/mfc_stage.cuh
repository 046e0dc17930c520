// The fused RK-stage kernel: one launch computes, for a TX x TY tile of
// cells, everything MicroFC's s_compute_rhs does (m_rhs.fpp:405-679) and the
// RK stage update that follows it (m_time_steppers.fpp:298-348):
//
//   phase 1  load the tile plus an H-cell halo of the conservative state from
//            HBM (coalesced along x), apply the ghost-cell boundary conditions
//            by index mapping and convert to primitive variables in FP64
//   phase 2  x-direction WENO of every variable of every cell that borders a
//            face of the tile
//   phase 3  x-direction HLLC on the TX+1 faces of each row
//   phase 4  x flux divergence + alpha*div(u) into registers, and y WENO
//   phase 5  y-direction HLLC
//   phase 6  y flux divergence, RK combination, store (coalesced)
//
// Interface states and fluxes live only in shared memory; per stage HBM sees
// one read of the stage input (plus halo re-reads, which hit L2) and of the
// RK base register, and one write of the stage output.
#pragma once

#include "mfc_device.cuh"
#include "mfc_gate.cuh"
#include "mfc_tma.cuh"

namespace mfc {

// One cell's FP32 WENO coefficients from shared memory: kCoefRec floats,
// 16-byte aligned, as float4 loads.
template <class RT>
__device__ __forceinline__ void load_coef_record(const RT* __restrict__ rec, RT (&c)[kCoefRec]) {
  if constexpr (sizeof(RT) == 4) {
#pragma unroll
    for (int k = 0; k < kCoefRec / 4; ++k) {
      const float4 v = reinterpret_cast<const float4*>(rec)[k];
      c[4 * k] = v.x;
      c[4 * k + 1] = v.y;
      c[4 * k + 2] = v.z;
      c[4 * k + 3] = v.w;
    }
  }
}

// Precision changes of the accumulation type: identity for FP64, the
// integer bit-field conversions for the split path's FP32.
template <class T>
__device__ __forceinline__ T narrow(double x) {
  if constexpr (sizeof(T) == 4) return d2f_bits(x);
  else return x;
}
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f2d_bits(x); }

// Work distribution of a split WENO5 phase: NPOS positions (cells of the
// tile's rows or columns) times S items (the variable pairs).  Each full
// pass gives a thread one position with all S items, so that the position's
// index arithmetic, gate flag and coefficient record serve S
// reconstructions; the NPOS % NT positions left over are dealt out per
// (position, item), so that no thread does more than ceil(S * NPOS / NT).
// f(p, v, all): position p, all items when all, else item v.
template <int NPOS, int S, int NT, class F>
__device__ __forceinline__ void deal_positions(const int tid, F&& f) {
  constexpr int FULL = (NPOS / NT) * NT, REM = NPOS - FULL;
  for (int p = tid; p < FULL; p += NT) f(p, 0, true);
  if constexpr (REM > 0) {
    for (int it = tid; it < REM * S; it += NT) {
      const int v = it / REM;
      f(FULL + (it - v * REM), v, false);
    }
  }
}

template <int ND, int NF, int WO, class RT, int TX, int TY, bool VISC = false>
struct StageShape {
  using Q = Eqs<ND, NF>;
  static constexpr int S = Q::S;
  static constexpr int H = (WO + 1) / 2;  // halo depth
  static constexpr int TYE = (ND > 1) ? TY : 1;
  static constexpr int LX = TX + 2 * H;
  static constexpr int LY = (ND > 1) ? TY + 2 * H : 1;
  // split WENO5 keeps the primitive variables and the WENO values in
  // interleaved pairs (2p, 2p+1), reconstructed two at a time with packed
  // FP32 instructions; SP counts the variables with the padding one
  static constexpr bool PAIR = sizeof(RT) == 4 && WO == 5;
  static constexpr int SP = PAIR ? (S + 1) / 2 * 2 : S;
  static constexpr int NQ = SP * LY * LX;  // primitive tile
  // WENO outputs (left and right face values), x and y layouts share space
  static constexpr int NWX = SP * TYE * (TX + 2);
  static constexpr int NWY = (ND > 1) ? SP * (TY + 2) * TX : 0;
  static constexpr int NW = NWX > NWY ? NWX : NWY;
  // fluxes + interface velocity (+ the viscous x-momentum, y-momentum and
  // energy source fluxes)
  static constexpr int NR = S + 1 + (VISC ? 3 : 0);
  static constexpr int NFX = NR * TYE * (TX + 1);
  static constexpr int NFY = (ND > 1) ? NR * (TY + 1) * TX : 0;
  static constexpr int NFL = NFX > NFY ? NFX : NFY;
  // split precision: the tile's WENO coefficients, converted to FP32 once and
  // stored as one 16-byte aligned record of kCoefRec floats per cell, so that
  // a WENO evaluation loads them with 7 vector loads
  static constexpr int NCX = TX + 2, NCY = (ND > 1) ? TY + 2 : 0;
  static constexpr int NCOEF = (sizeof(RT) == 4 && WO == 5) ? kCoefRec * (NCX + NCY) : 0;
  // FP64 WENO5: the tile's coefficients as doubles in [k][cell] order (x
  // cells, then y cells), staged once per tile so that the reconstructions
  // read them from shared memory instead of issuing kNumCoef global loads
  // each
  static constexpr int NCOEF64 = (sizeof(RT) == 8 && WO == 5) ? kNumCoef * (NCX + NCY) : 0;
  // offsets (in RT elements) of the arrays, each rounded up to 16 bytes
  static constexpr int align16(int n) { return (n * int(sizeof(RT)) + 15) / 16 * 16 / int(sizeof(RT)); }
  static constexpr int OW = align16(NQ), OF = OW + 2 * align16(NW), OC = OF + align16(NFL);
  // layout: [primitive tile, WENO values, fluxes][learned gate][coefficient
  // records]; the records come last so that a uniform grid, which never
  // stages them, can launch without their share
  static constexpr size_t kMainBytes = sizeof(RT) * size_t(OC);
  static constexpr size_t kCoefBytes = sizeof(RT) * size_t(NCOEF + NCOEF64);
  static constexpr size_t kSmemBytes = kMainBytes + kCoefBytes;
};

// Shared memory of the learned gate.  Its own region holds one flag per
// (cell, direction) reconstructed by the tile.  The gate phase's scratch --
// one 16x16 FP16 input block per warp, then the MLP's lane fragments
// (kGateFragWords words per lane, word-major) -- lives in the WENO value
// arrays, which are not written before the gate phase ends.
template <int ND, int TX, int TY, int NT>
struct GateShape {
  static constexpr int NGX = (TX + 2) * ((ND > 1) ? TY : 1);
  static constexpr int NGY = (ND > 1) ? TX * (TY + 2) : 0;
  static constexpr size_t kFragOff = size_t(NT / 32) * 512;
  static constexpr size_t kScratchBytes = kFragOff + size_t(kGateFragWords) * 32 * 4;
  static constexpr size_t kBytes = ((NGX + NGY + 15) / 16) * 16;
};

// The TMA staging area of a stage tile (2-D): after the primitive tile,
// 128-byte aligned, the box of all variables, then its mbarrier and a flag.
template <int ND, int NF, int WO, class RT, int TX, int TY>
__device__ __forceinline__ unsigned char* tma_staging(unsigned char* smem_raw) {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY>;
  const uintptr_t a = reinterpret_cast<uintptr_t>(smem_raw + Sh::OW * sizeof(RT));
  return reinterpret_cast<unsigned char*>((a + 127) & ~uintptr_t(127));
}
template <int ND, int NF, int WO, class RT, int TX, int TY>
constexpr uint32_t tma_stage_bytes() {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY>;
  return uint32_t(TmaBox<TX, Sh::H>::kWidth) * Sh::LY * Sh::S * 8;
}

// Offset of the split path's coefficient records in a block's shared
// memory: after the main arrays and the gate's flags, and after the TMA
// staging area (worst-case alignment) of a TMA kernel, so that records
// staged before the copy lands are not overwritten.
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool VISC, bool TMA>
constexpr size_t stage_coef_offset() {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY, VISC>;
  size_t o = Sh::kMainBytes + (GATE ? GateShape<ND, TX, TY, NT>::kBytes : 0);
  if constexpr (TMA) {
    const size_t t =
        (sizeof(RT) * size_t(Sh::OW) + 128 + tma_stage_bytes<ND, NF, WO, RT, TX, TY>() + 16 + 15) / 16 * 16;
    o = o > t ? o : t;
  }
  return o;
}

// Dynamic shared memory of one block: without the split path's coefficient
// records when the grid is uniform (every direction reads the shared
// record); the FP64 coefficients are always staged.
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool VISC, bool TMA>
constexpr size_t stage_smem_total(bool shared_coef) {
  using Sh = StageShape<ND, NF, WO, RT, TX, TY, VISC>;
  return stage_coef_offset<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>() +
         (shared_coef && Sh::NCOEF64 == 0 ? 0 : Sh::kCoefBytes);
}

// WENO of the characteristic fields at one position (FP64): the stencil of
// the position's cell, at(v, o) = primitive variable v at offset o along DIR,
// is projected on the characteristic fields of the quasi-linear primitive
// system frozen at the cell's own state; each field is reconstructed with
// the cell's coefficients; the face values are mapped back to primitive
// variables into L(v) / R(v).  The fields (no counterpart in the
// reference, which reconstructs the primitive variables) in the slots of
// the primitive variables:
//   partial density i: alpha_i rho_i - kappa_i p,  kappa_i = alpha_i rho_i / (rho c^2)
//   normal momentum:   p - rho c u_n   (the u_n - c wave)
//   energy:            p + rho c u_n   (the u_n + c wave)
//   tangential velocities and volume fractions unchanged,
// with rho = max(sum alpha_i rho_i, 1e-16), Gamma = sum alpha_i Gamma_i,
// Pi = sum alpha_i Pi_i and c^2 = max(((Gamma + 1) p + Pi) / (Gamma rho),
// 1e-16), the mixture sound speed of the HLLC solver.  Back:
// p = (w+ + w-) 0.5, u_n = (w+ - w-) / (2 rho c), alpha_i rho_i = w_i + kappa_i p.
// The oracle (Solver::weno with char_decomp) evaluates the same expressions
// in the same order.
template <int ND, int NF, int WO, int DIR, class At, class OutL, class OutR>
__device__ __forceinline__ void char_weno_position(const double (&c)[kCoefRec], const At& at, const double eps,
                                                   const DevParams& P, const OutL& L, const OutR& R) {
  using Q = Eqs<ND, NF>;
  constexpr int S = Q::S, UN = Q::MOM + DIR;
  double rho = 0.0, gam = 0.0, pinf = 0.0;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    rho = rho + at(f, 0);
    gam = gam + at(Q::ADV + f, 0) * P.gammas[f];
    pinf = pinf + at(Q::ADV + f, 0) * P.pi_infs[f];
  }
  rho = fmax(rho, 1e-16);
  const double c2 = fmax(div_rn((gam + 1.0) * at(Q::E, 0) + pinf, divisor(gam * rho)), 1e-16);
  const double rc = rho * sqrt(c2);
  const DivisorF64 Dk = divisor(rho * c2);
  double kap[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) kap[f] = div_rn(at(f, 0), Dk);
#pragma unroll 1
  for (int v = 0; v < S; ++v) {
    double st[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int o = k - 2;
      if (o < -(WO / 2) || o > WO / 2) {
        st[k] = 0.0;
      } else if (v < NF) {
        double kv = kap[0];
#pragma unroll
        for (int f = 1; f < NF; ++f) kv = v == f ? kap[f] : kv;
        st[k] = at(v, o) - kv * at(Q::E, o);
      } else if (v == UN) {
        st[k] = at(Q::E, o) - rc * at(UN, o);
      } else if (v == Q::E) {
        st[k] = at(Q::E, o) + rc * at(UN, o);
      } else {
        st[k] = at(v, o);
      }
    }
    double vl, vr;
    weno_cell<WO, double>(c, st, eps, vl, vr);
    L(v) = vl;
    R(v) = vr;
  }
  const DivisorF64 D2 = divisor(2.0 * rc);
  auto back = [&](const auto& O) {
    const double wm = O(UN), wp = O(Q::E);
    const double pr = (wp + wm) * 0.5;
    O(Q::E) = pr;
    O(UN) = div_rn(wp - wm, D2);
#pragma unroll
    for (int f = 0; f < NF; ++f) O(f) = O(f) + kap[f] * pr;
  };
  back(L);
  back(R);
}

// One tile of one RK stage; the tile's first cell is (x0, y0).  Used by the
// single-case kernel (one tile per block) and by the ensemble kernel (many
// tiles of many cases per persistent block).  smem_raw must hold
// stage_smem_total() (of shared_coef = true when U covers every
// direction).
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE = false, bool VISC = false,
          class UC = UniformCoef, bool TMA = false, bool CHAR = false>
__device__ __forceinline__ void stage_tile(const DevParams& P, const double* __restrict__ qin,
                                           const double* __restrict__ qbase, double* __restrict__ qout,
                                           const double dt, const int kind, const int x0, const int y0,
                                           unsigned char* smem_raw, const UC* U = nullptr,
                                           const TileMap* T = nullptr, uint32_t* tma_parity = nullptr) {
  static_assert(!GATE || (sizeof(RT) == 4 && WO == 5), "the learned gate runs on the split-precision WENO5 path");
  static_assert(!CHAR || (sizeof(RT) == 8 && WO > 1 && !VISC && !GATE && ND < 3),
                "characteristic-field WENO is compiled for the inviscid FP64 1-D/2-D WENO3/5 kernel");
  using Sh = StageShape<ND, NF, WO, RT, TX, TY, VISC>;
  using Q = Eqs<ND, NF>;
  constexpr int S = Sh::S, H = Sh::H, LX = Sh::LX, LY = Sh::LY, TYE = Sh::TYE;
  constexpr int CPT = (TX * TYE + NT - 1) / NT;  // interior cells per thread
  // split precision: FP32 reconstruction, Riemann solve and flux divergence;
  // the plain path keeps everything in FP64 in the reference's order
  constexpr bool kSplit = sizeof(RT) == 4;
  using AT = RT;  // type of the flux-divergence accumulation

  RT* sq = reinterpret_cast<RT*>(smem_raw);  // [S][LY][LX] primitive ([S/2][LY][LX][2] in pairs)
  RT* wl = sq + Sh::OW;                       // left-face values
  RT* wr = wl + Sh::align16(Sh::NW);          // right-face values
  RT* fl = sq + Sh::OF;                       // fluxes [S+1][...]
  // split: FP32 x coefficients [TX+2][kCoefRec], after the gate's share
  RT* scx = reinterpret_cast<RT*>(smem_raw + stage_coef_offset<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, TMA>());
  // split: FP32 y coefficients [TY+2][kCoefRec]; FP64: [kNumCoef][TY+2]
  RT* scy = scx + (Sh::NCOEF64 > 0 ? kNumCoef : kCoefRec) * Sh::NCX;
  // element of variable v in the primitive tile and in the x / y WENO values
  constexpr bool kPair = Sh::PAIR;
  constexpr int NCX_ = TX + 2, NCY_ = TY + 2;
  auto qi = [](int v, int ly, int lx) {
    return kPair ? (((v >> 1) * LY + ly) * LX + lx) * 2 + (v & 1) : (v * LY + ly) * LX + lx;
  };
  auto wxi = [](int v, int ty, int cx) {
    return kPair ? (((v >> 1) * TYE + ty) * NCX_ + cx) * 2 + (v & 1) : (v * TYE + ty) * NCX_ + cx;
  };
  auto wyi = [](int v, int cy, int tx) {
    return kPair ? (((v >> 1) * NCY_ + cy) * TX + tx) * 2 + (v & 1) : (v * NCY_ + cy) * TX + tx;
  };
  (void)wyi;

  const int tid = threadIdx.x;
  const int nx = P.n[0], ny = P.n[1];

  RT gam_i[NF], pi_i[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    if constexpr (kSplit) {
      gam_i[f] = P.gammas_f[f];
      pi_i[f] = P.pi_infs_f[f];
    } else {
      gam_i[f] = P.gammas[f];
      pi_i[f] = P.pi_infs[f];
    }
  }
  RT eps;
  if constexpr (kSplit) eps = P.weno_eps_f;
  else eps = P.weno_eps;
  // split WENO5 on a uniform grid: every cell of a direction shares one
  // coefficient record, read from the kernel parameters
  const bool ux = Sh::NCOEF > 0 && U != nullptr && U->on[0];
  const bool uy = Sh::NCOEF > 0 && ND > 1 && U != nullptr && U->on[1];
  (void)ux;
  (void)uy;

  // ---- phase 1: load + BCs + cons -> prim --------------------------------
  if constexpr (Sh::NCOEF > 0) {
    // the tile's coefficient records (constant tables: staged before the
    // wait for the previous stage); global reads coalesced along the cells,
    // records written per cell
    for (int it = ux ? kCoefRec * Sh::NCX : tid; it < kCoefRec * Sh::NCX; it += NT) {
      const int cx = it % Sh::NCX, k = it / Sh::NCX;
      scx[cx * kCoefRec + k] =
          k < kNumCoef ? d2f_bits(__ldg(P.coef[0] + k * P.cstride[0] + clamp_coef_index(x0 - 1 + cx, nx) + P.coff))
                       : 0.f;
    }
    if constexpr (ND > 1) {
      for (int it = uy ? kCoefRec * Sh::NCY : tid; it < kCoefRec * Sh::NCY; it += NT) {
        const int cy = it % Sh::NCY, k = it / Sh::NCY;
        scy[cy * kCoefRec + k] =
            k < kNumCoef
                ? d2f_bits(__ldg(P.coef[1] + k * P.cstride[1] + clamp_coef_index(y0 - 1 + cy, ny) + P.coff))
                : 0.f;
      }
    }
  }
  if constexpr (Sh::NCOEF64 > 0 && !CHAR) {
    // FP64 WENO5: the tile's coefficients, [k][cell], before the wait
    for (int it = tid; it < kNumCoef * Sh::NCX; it += NT) {
      const int cx = it % Sh::NCX, k = it / Sh::NCX;
      scx[k * Sh::NCX + cx] = __ldg(P.coef[0] + k * P.cstride[0] + clamp_coef_index(x0 - 1 + cx, nx) + P.coff);
    }
    if constexpr (ND > 1) {
      for (int it = tid; it < kNumCoef * Sh::NCY; it += NT) {
        const int cy = it % Sh::NCY, k = it / Sh::NCY;
        scy[k * Sh::NCY + cy] = __ldg(P.coef[1] + k * P.cstride[1] + clamp_coef_index(y0 - 1 + cy, ny) + P.coff);
      }
    }
  }
  // one cell of the tile: BCs already applied, cons -> prim into the tile
  auto store_prim = [&](double (&q)[S], const int ly, const int lx) {
    if constexpr (kSplit) {
      float pr[S];
      cons_to_prim_split<ND, NF>(q, P, pr);
#pragma unroll
      for (int v = 0; v < S; ++v) sq[qi(v, ly, lx)] = pr[v];
      if constexpr (Sh::SP > S) sq[qi(S, ly, lx)] = 0.f;  // the padding lane
    } else {
      cons_to_prim<ND, NF>(q, P);
#pragma unroll
      for (int v = 0; v < S; ++v) sq[qi(v, ly, lx)] = RT(q[v]);
    }
  };
  // corners are never read, except the four diagonal neighbours of the tile
  // that the viscous cross derivatives use
  auto unused_corner = [](const int lx, const int ly) {
    const bool hx = lx < H || lx >= H + TX;
    const bool hy = (ND > 1) && (ly < H || ly >= H + TY);
    return hx && hy && !(VISC && (lx == H - 1 || lx == H + TX) && (ly == H - 1 || ly == H + TY));
  };

  // TMA staging: a tile whose halo lies inside the domain (no boundary
  // condition, no processor halo) arrives in one bulk tensor copy of all
  // variables into the WENO and flux arrays, which are free until phase 2
  // (the coefficient records sit past the staging area).
  bool use_tma = false;
  unsigned char* stg = nullptr;
  uint32_t bar = 0;
  using Box = TmaBox<TX, H>;
  constexpr uint32_t kStageBytes = tma_stage_bytes<ND, NF, WO, RT, TX, TY>();
  if constexpr (TMA && ND == 2 && !VISC) {
    use_tma = T != nullptr && T->on && x0 >= H && x0 + TX + H <= nx && y0 >= H && y0 + TY + H <= ny;
    if (use_tma) {
      stg = tma_staging<ND, NF, WO, RT, TX, TY>(smem_raw);
      bar = smem_addr(stg + kStageBytes);
      // one tile per block: a fresh barrier; a block walking many tiles
      // (tma_parity given) initialised it once and alternates its phase
      if (tid == 0 && tma_parity == nullptr) mbar_init(bar, 1);
    }
  }
  griddep_wait();  // the state below is the previous stage's output
  if (kind != kRkEuler && kind != kRhsOnly) {
    // the RK base register's rows of the tile, read only by the last phase:
    // every 128-byte line prefetched into L2 while the tile is worked on
    constexpr int kLines = (TX * 8 + 127) / 128;
    for (int it = tid; it < S * TYE * kLines; it += NT) {
      const int line = it % kLines, r = it / kLines, ty = r % TYE, v = r / TYE;
      const int gx = x0 + line * 16, gy = (ND > 1) ? y0 + ty : 0;
      if (gx >= nx || gy >= ny) continue;
      asm volatile("prefetch.global.L2 [%0];" ::"l"(qbase + gy * P.sy + gx + v * P.sv));
    }
  }
  if (use_tma) {
    const uint32_t par = tma_parity ? *tma_parity : 0u;
    volatile int* landed = reinterpret_cast<volatile int*>(stg + kStageBytes + 8);
    if (tid == 0) {
      // a walking block: its reads of this memory for the previous tile come
      // first, and its maps live in global memory
      if (tma_parity) {
        fence_proxy_async_smem();
        tensormap_acquire(&T->map);
      }
      mbar_arrive_expect_tx(bar, kStageBytes);
      tma_load_3d(smem_addr(stg), &T->map, x0 - Box::kLead, y0 - H, 0, bar);
      const bool ok = mbar_wait_bounded(bar, par, 1000000000ull);  // 1 s
      if (!ok) (void)mbar_wait_bounded(bar, par, 1000000000ull);    // the copy may still be in flight
      *landed = ok ? 1 : 0;
    }
    __syncthreads();
    if (*landed == 0) {
      if (tid == 0 && P.status) atomicOr(P.status, MFC_FLAG_TIMEOUT);
      return;
    }
    (void)mbar_try_wait(bar, par);  // completed: each thread acquires the copy's writes
    if (tma_parity) *tma_parity ^= 1u;
    const double* sd = reinterpret_cast<const double*>(stg);
    for (int c = tid; c < LX * LY; c += NT) {
      const int lx = c % LX, ly = c / LX;
      if (unused_corner(lx, ly)) continue;
      double q[S];
#pragma unroll
      for (int v = 0; v < S; ++v) q[v] = sd[(v * LY + ly) * Box::kWidth + lx + (Box::kLead - H)];
      store_prim(q, ly, lx);
    }
  } else {  // plain loads, with the boundary conditions and processor halos
    for (int c = tid; c < LX * LY; c += NT) {
      const int lx = c % LX, ly = c / LX;
      if (unused_corner(lx, ly)) continue;
      bool fx = false, fy = false;
      const int rx = x0 - H + lx, ry = (ND > 1) ? y0 - H + ly : 0;
      // processor boundaries: ghost cells come from the neighbour's halo buffer
      const int px = rx < 0 ? (P.bc_beg[0] >= 0 ? 0 : -1) : (rx >= nx && P.bc_end[0] >= 0 ? 1 : -1);
      const int py = (ND > 1) ? (ry < 0 ? (P.bc_beg[1] >= 0 ? 0 : -1) : (ry >= ny && P.bc_end[1] >= 0 ? 1 : -1)) : -1;
      const double* src;
      int64_t vs = P.sv;
      // cells of partial edge tiles beyond the first H ghosts are never stored:
      // their depth is clamped.  y strips are nx + 2 wide (the x ghost cells
      // -1 and nx of the neighbour's rows come first and last).
      if (px >= 0 && py >= 0) {
        // between two processor boundaries (the viscous corner cells): the
        // diagonal neighbour's cell, forwarded by the y neighbour
        const int d = min(py == 0 ? -1 - ry : ry - ny, H - 1);
        src = P.halo[2 + py] + (int64_t)d * (nx + 2) + (px == 0 ? 0 : nx + 1);
        vs = (int64_t)H * (nx + 2);
      } else if (px >= 0) {
        const int d = min(px == 0 ? -1 - rx : rx - nx, H - 1);
        const int yy = (ND > 1) ? map_cell(ry, ny, P.bc_beg[1], P.bc_end[1], &fy) : 0;
        src = P.halo[px] + (int64_t)yy * H + d;
        vs = (int64_t)ny * H;
      } else if (py >= 0) {
        const int d = min(py == 0 ? -1 - ry : ry - ny, H - 1);
        const int xx = map_cell(rx, nx, P.bc_beg[0], P.bc_end[0], &fx);
        src = P.halo[2 + py] + (int64_t)d * (nx + 2) + xx + 1;
        vs = (int64_t)H * (nx + 2);
      } else {
        const int gx = map_cell(rx, nx, P.bc_beg[0], P.bc_end[0], &fx);
        const int gy = (ND > 1) ? map_cell(ry, ny, P.bc_beg[1], P.bc_end[1], &fy) : 0;
        src = qin + gy * P.sy + gx;
      }
      double q[S];
#pragma unroll
      for (int v = 0; v < S; ++v) q[v] = __ldg(src + v * vs);
      if (fx) q[Q::MOM] = -q[Q::MOM];
      if (ND > 1 && fy) q[Q::MOM + 1] = -q[Q::MOM + 1];
      store_prim(q, ly, lx);
    }
  }
  __syncthreads();

  // ---- learned gate: one flag per (cell, direction), tensor-core MLP -------
  // The first stage of a time step (and an RHS evaluation) runs the network
  // on every reconstructed position of the tile; with P.gate_flags it also
  // stores the decisions, and the step's later stages read them back instead
  // of running the network again: the gate judges each cell once per time
  // step, on the state at t^n.  Every stored position (including the ghost
  // positions x = -1, nx and y = -1, ny next to the domain) is written by
  // exactly one tile.
  const uint8_t* gflag = nullptr;
  if constexpr (GATE) {
    using G = GateShape<ND, TX, TY, NT>;
    constexpr int NG = G::NGX + G::NGY;
    uint8_t* flags = smem_raw + Sh::kMainBytes;
    // position p of the tile: its slot in the stored planes (false: beyond
    // the planes, a cell of a partial edge tile whose results are not kept)
    // and whether this tile is the one that stores it
    auto flag_slot = [&](const int p, int64_t& slot, bool& owner) {
      if (p < G::NGX) {
        const int cx = p % (TX + 2), ty = p / (TX + 2);
        const int gx = x0 - 1 + cx, gy = y0 + ty;
        slot = (int64_t)gy * (nx + 2) + (gx + 1);
        owner = (cx >= 1 && cx <= TX) || gx == -1 || gx == nx;
        return gx >= -1 && gx <= nx && gy < ny;
      }
      const int p2 = p - G::NGX, tx = p2 % TX, cy = p2 / TX;
      const int gx = x0 + tx, gy = y0 - 1 + cy;
      slot = (int64_t)ny * (nx + 2) + (int64_t)(gy + 1) * nx + gx;
      owner = (cy >= 1 && cy <= TY) || gy == -1 || gy == ny;
      return gx < nx && gy >= -1 && gy <= ny;
    };
    if (P.gate_flags != nullptr && kind != kRkEuler && kind != kRhsOnly) {
      // a later stage of the step: the first stage's decisions
      for (int p = tid; p < NG; p += NT) {
        int64_t slot;
        bool owner;
        flags[p] = flag_slot(p, slot, owner) ? __ldg(P.gate_flags + slot) : uint8_t(1);
      }
    } else {
      static_assert(G::kScratchBytes <= 2 * sizeof(RT) * size_t(Sh::align16(Sh::NW)),
                    "the gate's scratch must fit the WENO value arrays");
      unsigned char* scratch = reinterpret_cast<unsigned char*>(wl);
      __half* gin = reinterpret_cast<__half*>(scratch);
      uint32_t* frag = reinterpret_cast<uint32_t*>(scratch + G::kFragOff);
      const int warp = tid >> 5, lane = tid & 31;
      const uint32_t* gsrc =
          reinterpret_cast<const uint32_t*>(static_cast<const unsigned char*>(P.gate_w) + kGateFragOffset);
      for (int i = tid; i < kGateFragWords * 8; i += NT)
        reinterpret_cast<uint4*>(frag)[i] = __ldg(reinterpret_cast<const uint4*>(gsrc) + i);
      __syncthreads();
      const GateFragsSmem F{frag + 4 * lane};
      __half* my = gin + warp * 256;
      constexpr int NCH = (NG + 15) / 16;
      for (int ch = warp; ch < NCH; ch += NT / 32) {
        const int cell = ch * 16 + (lane & 15);
        const int var = lane < 16 ? Q::ADV : Q::E;  // alpha_1 | pressure
        float s[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        if (cell < G::NGX) {
          const int cx = cell % (TX + 2), ty = cell / (TX + 2);
#pragma unroll
          for (int k = 0; k < 5; ++k) s[k] = sq[qi(var, (ND > 1) ? ty + H : 0, cx + H - 1 + k - 2)];
        } else if (cell < NG) {
          const int c2 = cell - G::NGX, tx = c2 % TX, cy = c2 / TX;
#pragma unroll
          for (int k = 0; k < 5; ++k) s[k] = sq[qi(var, cy + H - 1 + k - 2, tx + H)];
        }
        float xf[5];
        gate_norm5_var(s, xf, lane < 16 ? 0 : 1);
        // columns 0..7 (alpha_1) or 8..15 (pressure) of the cell's row: five
        // features and three zeros, one 16-byte store
        const uint4 half8 = make_uint4(pack_h2(xf[0], xf[1]), pack_h2(xf[2], xf[3]), pack_h2(xf[4], 0.f), 0u);
        reinterpret_cast<uint4*>(my + (lane & 15) * 16)[lane >> 4] = half8;
        __syncwarp();
        float lo, hi;
        gate_mlp16(my, F, lo, hi);
        if ((lane & 3) == 0) {
          const int c_lo = ch * 16 + (lane >> 2), c_hi = c_lo + 8;
          if (c_lo < NG) flags[c_lo] = lo > 0.f;
          if (c_hi < NG) flags[c_hi] = hi > 0.f;
        }
        __syncwarp();
      }
      __syncthreads();
      if (P.gate_flags != nullptr && kind == kRkEuler) {
        // the first stage stores the decisions of the positions it owns
        for (int p = tid; p < NG; p += NT) {
          int64_t slot;
          bool owner;
          if (flag_slot(p, slot, owner) && owner) P.gate_flags[slot] = flags[p];
        }
      }
    }
    gflag = flags;
    __syncthreads();
  }

  // ---- phase 2: x WENO over cells x0-1 .. x0+TX of the interior rows -------
  {
    constexpr int NCX = TX + 2;
    // variable v of the cell at (cx, ty); c: the cell's coefficient record
    auto x_recon = [&](const RT* __restrict__ c, const int cx, const int ty, const int v) {
      RT st[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const int o = k - 2;
        st[k] = (o >= -(WO / 2) && o <= WO / 2) ? sq[qi(v, (ND > 1) ? ty + H : 0, cx + H - 1 + o)] : RT(0);
      }
      RT vl, vr;
      weno_cell<WO, RT>(c, st, eps, vl, vr);
      wl[wxi(v, ty, cx)] = vl;
      wr[wxi(v, ty, cx)] = vr;
    };
    if constexpr (kPair) {
      constexpr int NPR = Sh::SP / 2;  // variable pairs
      const f32x2 eps2 = f2_pack(eps, eps);
      // variable pair pr of the cell at (cx, ty); C(k): coefficient k as a (c, c) pair
      auto x_pair = [&](const auto& C, const int cx, const int ty, const int pr, const bool nonlin) {
        const f32x2* row = reinterpret_cast<const f32x2*>(sq) + (pr * LY + ((ND > 1) ? ty + H : 0)) * LX + cx + H - 1;
        f32x2 st[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) st[k] = row[k - 2];
        f32x2 vl, vr;
        if constexpr (GATE) {
          if (nonlin) weno5_pair_fast(C, st, eps2, vl, vr);
          else weno5_pair_linear(C, st, vl, vr);
        } else {
          weno5_pair_fast(C, st, eps2, vl, vr);
        }
        reinterpret_cast<f32x2*>(wl)[(pr * TYE + ty) * NCX + cx] = vl;
        reinterpret_cast<f32x2*>(wr)[(pr * TYE + ty) * NCX + cx] = vr;
      };
      // UNI: the shared record of a uniform grid, else the cell's staged
      // record (reloaded per pair: keeping it live across them costs
      // registers); chosen once per block
      auto x_positions = [&](auto uni) {
        constexpr bool UNI = decltype(uni)::value;
        deal_positions<TYE * NCX, NPR, NT>(tid, [&](const int p, const int v, const bool all) {
          const int cx = p % NCX, ty = p / NCX;
          bool nonlin = true;
          if constexpr (GATE) nonlin = gflag[p] != 0;
          auto one = [&](const int w) {
            if constexpr (UNI) {
              const f32x2* rec = U->rec[0];
              x_pair([&](int k) { return rec[k]; }, cx, ty, w, nonlin);
            } else {
              RT c[kCoefRec];
              load_coef_record(scx + cx * kCoefRec, c);
              x_pair([&](int k) { return f2_pack(c[k], c[k]); }, cx, ty, w, nonlin);
            }
          };
          if (all) {
#pragma unroll 1
            for (int w = 0; w < NPR; ++w) one(w);
          } else {
            one(v);
          }
        });
      };
      if (ux) x_positions(FlagC<true>{});
      else x_positions(FlagC<false>{});
    } else if constexpr (CHAR) {
      // characteristic fields: one thread per position, all variables
      const double* cf = P.coef[0];
      const int cs = P.cstride[0];
      for (int it = tid; it < TYE * NCX; it += NT) {
        const int cx = it % NCX, ty = it / NCX;
        RT c[kCoefRec];
        const int gi = clamp_coef_index(x0 - 1 + cx, nx) + P.coff;
#pragma unroll
        for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(cf + k * cs + gi));
        const int ly = (ND > 1) ? ty + H : 0, lx = cx + H - 1;
        char_weno_position<ND, NF, WO, 0>(
            c, [&](int v, int o) { return sq[qi(v, ly, lx + o)]; }, eps, P,
            [&](int v) -> RT& { return wl[wxi(v, ty, cx)]; }, [&](int v) -> RT& { return wr[wxi(v, ty, cx)]; });
      }
    } else if constexpr (sizeof(RT) == 8 && WO > 1) {
      // FP64: positions cx = 1 .. TX feed two faces each; the tile-edge
      // positions feed one -- cell x0 - 1 only its right-face value (the left
      // state of face x0 - 1/2), cell x0 + TX only its left-face value -- so
      // only that value is formed there (weno_cell_side, the same bits).  The
      // edge items go to the threads that have one interior item fewer.
      // the tile's staged coefficients (WENO3: from global memory)
      const double* cf = P.coef[0];
      const int cs = P.cstride[0];
      auto coef = [&](const int cx, RT (&c)[kCoefRec]) {
        if constexpr (Sh::NCOEF64 > 0) {
#pragma unroll
          for (int k = 0; k < kNumCoef; ++k) c[k] = scx[k * Sh::NCX + cx];
        } else {
          const int gi = clamp_coef_index(x0 - 1 + cx, nx) + P.coff;
#pragma unroll
          for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(cf + k * cs + gi));
        }
      };
      constexpr int NI = S * TYE * TX, NE = S * TYE * 2;
      for (int it = tid; it < NI; it += NT) {
        const int cx = 1 + it % TX, r = it / TX;
        const int ty = r % TYE, v = r / TYE;
        RT c[kCoefRec];
        coef(cx, c);
        x_recon(c, cx, ty, v);
      }
      for (int it = (tid + NT - NI % NT) % NT; it < NE; it += NT) {
        const int side = it / (S * TYE), r = it % (S * TYE);
        const int ty = r % TYE, v = r / TYE, cx = side ? NCX - 1 : 0;
        RT c[kCoefRec];
        coef(cx, c);
        RT st[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const int o = k - 2;
          st[k] = (o >= -(WO / 2) && o <= WO / 2) ? sq[qi(v, (ND > 1) ? ty + H : 0, cx + H - 1 + o)] : RT(0);
        }
        if (side) wl[wxi(v, ty, cx)] = weno_cell_side<WO, 0, RT>(c, st, eps);
        else wr[wxi(v, ty, cx)] = weno_cell_side<WO, 1, RT>(c, st, eps);
      }
    } else {
      // split WENO1/3 (and FP64 WENO1): coefficients per reconstruction from global memory
      const double* cf = P.coef[0];
      const int cs = P.cstride[0];
      for (int it = tid; it < S * TYE * NCX; it += NT) {
        const int cx = it % NCX;
        const int r = it / NCX;
        const int ty = r % TYE, v = r / TYE;
        RT c[kCoefRec];
        if constexpr (WO > 1) {
          const int gi = clamp_coef_index(x0 - 1 + cx, nx) + P.coff;
#pragma unroll
          for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(cf + k * cs + gi));
        }
        x_recon(c, cx, ty, v);
      }
    }
  }
  __syncthreads();

  // ---- phase 3: x HLLC on faces x0-1/2 .. x0+TX-1/2 ------------------------
  {
    constexpr int NFXr = TX + 1;
    for (int it = tid; it < TYE * NFXr; it += NT) {
      const int f = it % NFXr, ty = it / NFXr;
      const int gface = x0 - 1 + f;  // face gface+1/2
      RT qL[S], qR[S], F[S], us;
      const bool lfr = (gface == -1 && P.bc_beg[0] == -4);      // qL(-1) = qR(0)
      const bool rfl = (gface == nx - 1 && P.bc_end[0] == -4);  // qR(m+1) = qL(m)
#pragma unroll
      for (int v = 0; v < S; ++v) {
        const RT a = wr[wxi(v, ty, f)];
        const RT b = wl[wxi(v, ty, f + 1)];
        qL[v] = lfr ? b : a;
        qR[v] = rfl ? a : b;
      }
      if constexpr (VISC) {
        RT vs[ND], dxv[2] = {RT(0), RT(0)}, dyv[2] = {RT(0), RT(0)}, vf[3];
        hllc_face<ND, NF, 0, RT, true>(qL, qR, gam_i, pi_i, F, us, vs);
        const ViscParams& V = *P.visc;
        if (V.fg[0] != nullptr) {
          // weno_Re_flux = T: the prepared face gradients (clamped indices
          // for the rows and faces of partial tiles, whose results are dropped)
          const int gy = (ND > 1) ? min(y0 + ty, ny - 1) : 0;
          const int64_t plane = (int64_t)(ND > 1 ? ny : 1) * (nx + 1);
          const double* g = V.fg[0] + (int64_t)gy * (nx + 1) + (min(max(gface, -1), nx - 1) + 1);
#pragma unroll
          for (int c = 0; c < ND; ++c) {
            dxv[c] = narrow<RT>(__ldg(g + (c * ND) * plane));
            if constexpr (ND > 1) dyv[c] = narrow<RT>(__ldg(g + (c * ND + 1) * plane));
          }
        } else {
          const int ly = (ND > 1) ? ty + H : 0, lx = f + H - 1;  // the face's left cell
          auto U = [&](int c, int x, int y) { return sq[qi(Q::MOM + c, y, x)]; };
          const auto Dx = divisor(narrow<RT>(__ldg(V.dcc[0] + min(x0 + f, nx))));  // x_cc(j+1) - x_cc(j)
#pragma unroll
          for (int c = 0; c < ND; ++c) {
            const RT g = div_rn(U(c, lx + 1, ly) - U(c, lx, ly), Dx);
            dxv[c] = RT(0.5) * (g + g);
          }
          if constexpr (ND > 1) {
            const int gy = min(y0 + ty, ny - 1);
            const auto D0 = divisor(narrow<RT>(__ldg(V.dcc[1] + gy))),
                       D1 = divisor(narrow<RT>(__ldg(V.dcc[1] + gy + 1)));
#pragma unroll
            for (int c = 0; c < ND; ++c) {
              auto Ly = [&](int x) { return div_rn(U(c, x, ly) - U(c, x, ly - 1), D0); };
              auto Ry = [&](int x) { return div_rn(U(c, x, ly + 1) - U(c, x, ly), D1); };
              const RT A = RT(0.25) * (Ly(lx + 1) + Ry(lx + 1) + Ly(lx) + Ry(lx));
              dyv[c] = RT(0.5) * (A + A);
            }
          }
        }
        viscous_face_flux<ND, NF, 0, RT>(qL, qR, V, vs, dxv, dyv, vf);
#pragma unroll
        for (int t = 0; t < 3; ++t) fl[((S + 1 + t) * TYE + ty) * NFXr + f] = vf[t];
      } else if constexpr (kSplit) {
        hllc_face_fast<ND, NF, 0>(qL, qR, gam_i, pi_i, F, us);
      } else {
        hllc_face<ND, NF, 0, RT>(qL, qR, gam_i, pi_i, F, us);
      }
#pragma unroll
      for (int v = 0; v < S; ++v) fl[(v * TYE + ty) * NFXr + f] = F[v];
      fl[(S * TYE + ty) * NFXr + f] = us;
    }
  }
  __syncthreads();

  // ---- phase 4: x flux divergence (registers) + y WENO ----------------------
  AT rhs[CPT][S];
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    const int e = tid + k * NT;
    if (e >= TX * TYE) break;
    const int tx = e % TX, ty = e / TX;
    const int gx = x0 + tx;
    constexpr int NFXr = TX + 1;
    const AT inv = narrow<AT>(__ldg(P.inv_d[0] + (gx < nx ? gx : nx - 1)));
#pragma unroll
    for (int v = 0; v < S; ++v)
      rhs[k][v] = inv * (AT(fl[(v * TYE + ty) * NFXr + tx]) - AT(fl[(v * TYE + ty) * NFXr + tx + 1]));
    const AT du = AT(fl[(S * TYE + ty) * NFXr + tx + 1]) - AT(fl[(S * TYE + ty) * NFXr + tx]);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const AT a = AT(sq[qi(Q::ADV + f, ND > 1 ? ty + H : 0, tx + H)]);
      rhs[k][Q::ADV + f] = mul_add(inv * a, du, rhs[k][Q::ADV + f]);
    }
    if constexpr (VISC) {  // m_rhs.fpp:591-603: momentum .. energy
#pragma unroll
      for (int t = 0; t <= ND; ++t) {
        const int v = t < ND ? Q::MOM + t : Q::E, r = S + 1 + (t < ND ? t : 2);
        rhs[k][v] = mul_add(inv, AT(fl[(r * TYE + ty) * NFXr + tx]) - AT(fl[(r * TYE + ty) * NFXr + tx + 1]), rhs[k][v]);
      }
    }
  }
  if constexpr (ND > 1) {
    constexpr int NCY = TY + 2;
    // variable v of the cell at (tx, cy)
    auto y_recon = [&](const RT* __restrict__ c, const int tx, const int cy, const int v) {
      RT st[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const int o = k - 2;
        st[k] = (o >= -(WO / 2) && o <= WO / 2) ? sq[qi(v, cy + H - 1 + o, tx + H)] : RT(0);
      }
      RT vl, vr;
      weno_cell<WO, RT>(c, st, eps, vl, vr);
      wl[wyi(v, cy, tx)] = vl;
      wr[wyi(v, cy, tx)] = vr;
    };
    if constexpr (kPair) {
      constexpr int NPR = Sh::SP / 2;
      const f32x2 eps2 = f2_pack(eps, eps);
      auto y_pair = [&](const auto& C, const int tx, const int cy, const int pr, const bool nonlin) {
        const f32x2* col = reinterpret_cast<const f32x2*>(sq) + (pr * LY + cy + H - 1) * LX + tx + H;
        f32x2 st[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) st[k] = col[(k - 2) * LX];
        f32x2 vl, vr;
        if constexpr (GATE) {
          if (nonlin) weno5_pair_fast(C, st, eps2, vl, vr);
          else weno5_pair_linear(C, st, vl, vr);
        } else {
          weno5_pair_fast(C, st, eps2, vl, vr);
        }
        reinterpret_cast<f32x2*>(wl)[(pr * NCY + cy) * TX + tx] = vl;
        reinterpret_cast<f32x2*>(wr)[(pr * NCY + cy) * TX + tx] = vr;
      };
      auto y_positions = [&](auto uni) {
        constexpr bool UNI = decltype(uni)::value;
        deal_positions<NCY * TX, NPR, NT>(tid, [&](const int p, const int v, const bool all) {
          const int tx = p % TX, cy = p / TX;
          bool nonlin = true;
          if constexpr (GATE) nonlin = gflag[GateShape<ND, TX, TY, NT>::NGX + p] != 0;
          auto one = [&](const int w) {
            if constexpr (UNI) {
              const f32x2* rec = U->rec[1];
              y_pair([&](int k) { return rec[k]; }, tx, cy, w, nonlin);
            } else {
              RT c[kCoefRec];
              load_coef_record(scy + cy * kCoefRec, c);
              y_pair([&](int k) { return f2_pack(c[k], c[k]); }, tx, cy, w, nonlin);
            }
          };
          if (all) {
#pragma unroll 1
            for (int w = 0; w < NPR; ++w) one(w);
          } else {
            one(v);
          }
        });
      };
      if (uy) y_positions(FlagC<true>{});
      else y_positions(FlagC<false>{});
    } else if constexpr (CHAR) {
      const double* cf = P.coef[1];
      const int cs = P.cstride[1];
      for (int it = tid; it < NCY * TX; it += NT) {
        const int tx = it % TX, cy = it / TX;
        RT c[kCoefRec];
        const int gi = clamp_coef_index(y0 - 1 + cy, ny) + P.coff;
#pragma unroll
        for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(cf + k * cs + gi));
        const int ly = cy + H - 1, lx = tx + H;
        char_weno_position<ND, NF, WO, 1>(
            c, [&](int v, int o) { return sq[qi(v, ly + o, lx)]; }, eps, P,
            [&](int v) -> RT& { return wl[wyi(v, cy, tx)]; }, [&](int v) -> RT& { return wr[wyi(v, cy, tx)]; });
      }
    } else if constexpr (sizeof(RT) == 8 && WO > 1) {
      // FP64: rows cy = 1 .. TY feed two faces each; row y0 - 1 only its
      // upper-face value, row y0 + TY only its lower-face value (as in x)
      const double* cf = P.coef[1];
      const int cs = P.cstride[1];
      auto coef = [&](const int cy, RT (&c)[kCoefRec]) {
        if constexpr (Sh::NCOEF64 > 0) {
#pragma unroll
          for (int k = 0; k < kNumCoef; ++k) c[k] = scy[k * Sh::NCY + cy];
        } else {
          const int gi = clamp_coef_index(y0 - 1 + cy, ny) + P.coff;
#pragma unroll
          for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(cf + k * cs + gi));
        }
      };
      constexpr int NI = S * TY * TX, NE = S * 2 * TX;
      for (int it = tid; it < NI; it += NT) {
        const int tx = it % TX, r = it / TX;
        const int cy = 1 + r % TY, v = r / TY;
        RT c[kCoefRec];
        coef(cy, c);
        y_recon(c, tx, cy, v);
      }
      for (int it = (tid + NT - NI % NT) % NT; it < NE; it += NT) {
        const int side = it / (S * TX), r = it % (S * TX);
        const int tx = r % TX, v = r / TX, cy = side ? NCY - 1 : 0;
        RT c[kCoefRec];
        coef(cy, c);
        RT st[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const int o = k - 2;
          st[k] = (o >= -(WO / 2) && o <= WO / 2) ? sq[qi(v, cy + H - 1 + o, tx + H)] : RT(0);
        }
        if (side) wl[wyi(v, cy, tx)] = weno_cell_side<WO, 0, RT>(c, st, eps);
        else wr[wyi(v, cy, tx)] = weno_cell_side<WO, 1, RT>(c, st, eps);
      }
    } else {
      const double* cf = P.coef[1];
      const int cs = P.cstride[1];
      for (int it = tid; it < S * NCY * TX; it += NT) {
        const int tx = it % TX;
        const int r = it / TX;
        const int cy = r % NCY, v = r / NCY;
        RT c[kCoefRec];
        if constexpr (WO > 1) {
          const int gi = clamp_coef_index(y0 - 1 + cy, ny) + P.coff;
#pragma unroll
          for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(cf + k * cs + gi));
        }
        y_recon(c, tx, cy, v);
      }
    }
    __syncthreads();

    // ---- phase 5: y HLLC on faces y0-1/2 .. y0+TY-1/2 ----------------------
    constexpr int NFYr = TY + 1;
    for (int it = tid; it < NFYr * TX; it += NT) {
      const int tx = it % TX, f = it / TX;
      const int gface = y0 - 1 + f;
      RT qL[S], qR[S], F[S], us;
      const bool lfr = (gface == -1 && P.bc_beg[1] == -4);
      const bool rfl = (gface == ny - 1 && P.bc_end[1] == -4);
#pragma unroll
      for (int v = 0; v < S; ++v) {
        const RT a = wr[wyi(v, f, tx)];
        const RT b = wl[wyi(v, f + 1, tx)];
        qL[v] = lfr ? b : a;
        qR[v] = rfl ? a : b;
      }
      if constexpr (VISC) {
        RT vs[ND], dxv[2], dyv[2], vf[3];
        hllc_face<ND, NF, 1, RT, true>(qL, qR, gam_i, pi_i, F, us, vs);
        const ViscParams& V = *P.visc;
        const int gx = min(x0 + tx, nx - 1);
        if (V.fg[1] != nullptr) {
          // weno_Re_flux = T: the prepared face gradients
          const int64_t plane = (int64_t)(ny + 1) * nx;
          const double* g = V.fg[1] + (int64_t)(min(max(gface, -1), ny - 1) + 1) * nx + gx;
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            dxv[c] = narrow<RT>(__ldg(g + (c * 2) * plane));
            dyv[c] = narrow<RT>(__ldg(g + (c * 2 + 1) * plane));
          }
        } else {
          const int ly = f + H - 1, lx = tx + H;  // the face's lower cell
          auto U = [&](int c, int x, int y) { return sq[qi(Q::MOM + c, y, x)]; };
          const auto Dy = divisor(narrow<RT>(__ldg(V.dcc[1] + min(y0 + f, ny))));  // y_cc(k+1) - y_cc(k)
          const auto D0 = divisor(narrow<RT>(__ldg(V.dcc[0] + gx))),
                     D1 = divisor(narrow<RT>(__ldg(V.dcc[0] + gx + 1)));
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            auto Lx = [&](int y) { return div_rn(U(c, lx, y) - U(c, lx - 1, y), D0); };
            auto Rx = [&](int y) { return div_rn(U(c, lx + 1, y) - U(c, lx, y), D1); };
            const RT A = RT(0.25) * (Lx(ly + 1) + Rx(ly + 1) + Lx(ly) + Rx(ly));
            dxv[c] = RT(0.5) * (A + A);
            const RT g = div_rn(U(c, lx, ly + 1) - U(c, lx, ly), Dy);
            dyv[c] = RT(0.5) * (g + g);
          }
        }
        viscous_face_flux<ND, NF, 1, RT>(qL, qR, V, vs, dxv, dyv, vf);
#pragma unroll
        for (int t = 0; t < 3; ++t) fl[((S + 1 + t) * NFYr + f) * TX + tx] = vf[t];
      } else if constexpr (kSplit) {
        hllc_face_fast<ND, NF, 1>(qL, qR, gam_i, pi_i, F, us);
      } else {
        hllc_face<ND, NF, 1, RT>(qL, qR, gam_i, pi_i, F, us);
      }
#pragma unroll
      for (int v = 0; v < S; ++v) fl[(v * NFYr + f) * TX + tx] = F[v];
      fl[(S * NFYr + f) * TX + tx] = us;
    }
    __syncthreads();

    // ---- phase 6a: y flux divergence ------------------------------------------
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int e = tid + k * NT;
      if (e >= TX * TY) break;
      const int tx = e % TX, ty = e / TX;
      const int gy = y0 + ty;
      const AT inv = narrow<AT>(__ldg(P.inv_d[1] + (gy < ny ? gy : ny - 1)));
#pragma unroll
      for (int v = 0; v < S; ++v)
        rhs[k][v] = mul_add(inv, AT(fl[(v * NFYr + ty) * TX + tx]) - AT(fl[(v * NFYr + ty + 1) * TX + tx]), rhs[k][v]);
      const AT du = AT(fl[(S * NFYr + ty + 1) * TX + tx]) - AT(fl[(S * NFYr + ty) * TX + tx]);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const AT a = AT(sq[qi(Q::ADV + f, ty + H, tx + H)]);
        rhs[k][Q::ADV + f] = mul_add(inv * a, du, rhs[k][Q::ADV + f]);
      }
      if constexpr (VISC) {  // m_rhs.fpp:639-651
#pragma unroll
        for (int t = 0; t <= ND; ++t) {
          const int v = t < ND ? Q::MOM + t : Q::E, r = S + 1 + (t < ND ? t : 2);
          rhs[k][v] = mul_add(inv, AT(fl[(r * NFYr + ty) * TX + tx]) - AT(fl[(r * NFYr + ty + 1) * TX + tx]), rhs[k][v]);
        }
      }
    }
  }

  // ---- phase 6b: RK combination and store ------------------------------------
  griddep_launch_dependents();
  bool bad = false;
  const float dtf = kSplit ? __double2float_rn(dt) : 0.f;  // the split path's increments are FP32
  (void)dtf;
  double icfl = 0.0;
  // KIND: the stage's combination as a compile-time constant, chosen once
  // per block rather than once per cell and variable
  auto finish = [&](auto kind_c) {
    constexpr int KIND = decltype(kind_c)::value;
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      const int e = tid + k * NT;
      if (e >= TX * TYE) break;
      const int tx = e % TX, ty = e / TX;
      const int gx = x0 + tx, gy = y0 + ty;
      if (gx >= nx || (ND > 1 && gy >= ny)) continue;
      const int64_t o = gy * P.sy + gx;
#pragma unroll
      for (int v = 0; v < S; ++v) {
        double out;
        if constexpr (KIND == kRhsOnly) {
          out = widen(rhs[k][v]);
        } else {
          const double b = __ldg(qbase + o + v * P.sv);
          double in = b;
          if constexpr (KIND != kRkEuler) in = __ldg(qin + o + v * P.sv);
          if constexpr (kSplit) out = rk_combine_split(KIND, b, in, dtf, rhs[k][v]);
          else out = rk_combine(KIND, b, in, dt, rhs[k][v]);
        }
        bad |= not_finite(out);
        qout[o + v * P.sv] = out;
      }
    }
  };
  switch (kind) {
    case kRkEuler: finish(KindC<kRkEuler>{}); break;
    case kRk2Final: finish(KindC<kRk2Final>{}); break;
    case kRk3Mid: finish(KindC<kRk3Mid>{}); break;
    case kRk3Final: finish(KindC<kRk3Final>{}); break;
    default: finish(KindC<kRhsOnly>{}); break;
  }
  // the stability monitor (the last stage of a monitored step) reads the new
  // state back: this thread's own stores
  bool nonphys = false;
  if (P.monitor) {
    for (int k = 0; k < CPT; ++k) {
      const int e = tid + k * NT;
      if (e >= TX * TYE) break;
      const int tx = e % TX, ty = e / TX;
      const int gx = x0 + tx, gy = y0 + ty;
      if (gx >= nx || (ND > 1 && gy >= ny)) continue;
      const int64_t o = gy * P.sy + gx;
      double qn[S];
#pragma unroll
      for (int v = 0; v < S; ++v) qn[v] = qout[o + v * P.sv];
      double inv[ND];
      inv[0] = __ldg(P.inv_d[0] + gx);
      if constexpr (ND > 1) inv[1] = __ldg(P.inv_d[1] + gy);
      bool np;
      const double c = cell_icfl<ND, NF>(qn, P, dt, inv, np);
      nonphys |= np;
      if (!(c <= icfl)) icfl = c;  // keeps NaN
    }
  }
  if (bad && P.status) atomicOr(P.status, MFC_FLAG_NAN);
  if (nonphys && P.status) atomicOr(P.status, MFC_FLAG_NEG_PRESSURE);
  if (P.monitor) monitor_max(P.monitor, icfl);
}

// FMA tags the instantiations of the translation unit compiled with
// multiply-add contraction (-fmad=true), so that their host-side symbols
// differ from the bit-faithful ones; the kernel body does not use it.
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE = false, bool VISC = false,
          bool FMA = false, bool CHAR = false>
__global__ void __launch_bounds__(NT) stage_kernel(const DevParams P, const __grid_constant__ UniformCoef U,
                                                   const double* __restrict__ qin, const double* __restrict__ qbase,
                                                   double* __restrict__ qout, const double dt, const int kind) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_tile<ND, NF, WO, RT, TX, TY, NT, GATE, VISC, UniformCoef, false, CHAR>(P, qin, qbase, qout, dt, kind,
                                                                               blockIdx.x * TX,
                                                     (ND > 1) ? blockIdx.y * TY : 0, smem_raw, &U);
}

// The same kernel with its registers capped so that MINB blocks fit on an SM.
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, int MINB, bool FMA = false,
          bool VISC = false>
__global__ void __launch_bounds__(NT, MINB) stage_kernel_mb(const DevParams P, const __grid_constant__ UniformCoef U,
                                                            const double* __restrict__ qin,
                                                            const double* __restrict__ qbase,
                                                            double* __restrict__ qout, const double dt,
                                                            const int kind) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_tile<ND, NF, WO, RT, TX, TY, NT, GATE, VISC>(P, qin, qbase, qout, dt, kind, blockIdx.x * TX,
                                                     (ND > 1) ? blockIdx.y * TY : 0, smem_raw, &U);
}

// The kernel with TMA staging of interior tiles (2-D, inviscid); T maps the
// stage input qin.  MINB > 1 caps the registers as stage_kernel_mb does.
template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, bool FMA = false>
__global__ void __launch_bounds__(NT) stage_kernel_tma(const DevParams P, const __grid_constant__ UniformCoef U,
                                                       const __grid_constant__ TileMap T,
                                                       const double* __restrict__ qin,
                                                       const double* __restrict__ qbase, double* __restrict__ qout,
                                                       const double dt, const int kind) {
  extern __shared__ __align__(128) unsigned char smem_tma[];
  stage_tile<ND, NF, WO, RT, TX, TY, NT, GATE, false, UniformCoef, true>(
      P, qin, qbase, qout, dt, kind, blockIdx.x * TX, (ND > 1) ? blockIdx.y * TY : 0, smem_tma, &U, &T);
}

template <int ND, int NF, int WO, class RT, int TX, int TY, int NT, bool GATE, int MINB, bool FMA = false>
__global__ void __launch_bounds__(NT, MINB) stage_kernel_tma_mb(const DevParams P, const __grid_constant__ UniformCoef U,
                                                                const __grid_constant__ TileMap T,
                                                                const double* __restrict__ qin,
                                                                const double* __restrict__ qbase,
                                                                double* __restrict__ qout, const double dt,
                                                                const int kind) {
  extern __shared__ __align__(128) unsigned char smem_tma[];
  stage_tile<ND, NF, WO, RT, TX, TY, NT, GATE, false, UniformCoef, true>(
      P, qin, qbase, qout, dt, kind, blockIdx.x * TX, (ND > 1) ? blockIdx.y * TY : 0, smem_tma, &U, &T);
}

}  // namespace mfc
