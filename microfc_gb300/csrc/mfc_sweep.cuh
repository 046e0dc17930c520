// Directional sweep kernel for 3-D cases (the reference is 2-D; this is its
// z-extension).  A 3-D RK stage is three launches, one per direction, each
// computing that direction's part of s_compute_rhs (m_rhs.fpp:469-656):
//
//   x sweep: rhs  = 1/dx (F_{i-1/2} - F_{i+1/2});  rhs_a += 1/dx alpha (u*_{i+1/2} - u*_{i-1/2})
//   y sweep: rhs += ... (same in y)
//   z sweep: rhs += ... (same in z), then the RK combination (m_time_steppers.fpp)
//
// which is the reference's accumulation order, so the FP64 variant
// reproduces the oracle bit for bit.  A block owns TA cells along the sweep
// direction for TB x TC pencils; it loads them plus an H-cell halo along the
// sweep (coalesced: x is always one of the fastest-varying thread indices),
// converts to primitive variables, reconstructs every variable of the TA+2
// cells that border the block's faces, solves TA+1 Riemann problems per
// pencil and forms the flux divergence.  The partial RHS lives in a global
// buffer (FP64, or FP32 on the split path) between the sweeps.
//
// The x sweep also stores the primitive variables of the cells it owns (the
// work buffer's second segment, [S][z][y][x] in the reconstruction type),
// and the y and z sweeps read them instead of converting the state again:
// the conversion's FP64 operations (E - Pi, and the divisions of the plain
// path) run once per cell and stage instead of three times, and the split
// path's y and z sweeps load 4-byte instead of 8-byte values.  The stored
// values are the bits the conversion gives, and a reflected ghost cell's
// normal velocity is the stored one negated, which is what converting the
// reflected momentum gives (the conversion is odd in the momentum), so the
// result is unchanged bit for bit.  Ghost cells of processor boundaries come
// from the halo buffers as conservative values and are converted as before.
#pragma once

#include "mfc_device.cuh"
#include "mfc_stage.cuh"

namespace mfc {

template <int NF, int WO, class RT, int DIR, int TA, int TB, int TC>
struct SweepShape {
  using Q = Eqs<3, NF>;
  static constexpr int S = Q::S;
  static constexpr int H = (WO + 1) / 2;
  static constexpr int LA = TA + 2 * H;
  static constexpr int NP = TB * TC;          // pencils per block
  static constexpr int NQ = S * NP * LA;      // primitive tile [S][pencil][LA]
  static constexpr int NW = S * NP * (TA + 2);
  static constexpr int NFL = (S + 1) * NP * (TA + 1);
  // split precision: FP32 coefficient records of kCoefRec floats per cell (float4 loads)
  static constexpr int NCOEF = (sizeof(RT) == 4 && WO == 5) ? kCoefRec * (TA + 2) : 0;
  static constexpr int align16(int n) { return (n * int(sizeof(RT)) + 15) / 16 * 16 / int(sizeof(RT)); }
  static constexpr int OC = align16(NQ + 2 * NW + NFL);
  static constexpr size_t kSmemBytes = sizeof(RT) * (size_t(OC) + size_t(NCOEF));
  // TMA staging box of the tile (x, y, z extents; all S variables), in the
  // WENO and flux arrays: DIR 0 starts x on an even cell
  static constexpr int BX = DIR == 0 ? TmaBox<TA, H>::kWidth : TB;
  static constexpr int BY = DIR == 0 ? TB : (DIR == 1 ? LA : TC);
  static constexpr int BZ = DIR == 0 ? TC : (DIR == 1 ? TC : LA);
  // the x sweep stages the FP64 state, the y and z sweeps the stored primitives
  static constexpr int kStageElem = DIR == 0 ? 8 : int(sizeof(RT));
  static constexpr uint32_t kStageBytes = uint32_t(BX) * BY * BZ * S * kStageElem;
  static constexpr bool kTmaFits = (BX * kStageElem) % 16 == 0 && BX <= 256 && BY <= 256 && BZ <= 256 &&
                                   size_t(kStageBytes) + 128 + 16 <= sizeof(RT) * size_t(OC - NQ);
};

// Pencil p of a block and position a along the sweep -> global (x, y, z).
// DIR 0: a = x, pencils over (y = b, z = c); DIR 1: a = y, pencils over
// (x = b, z = c); DIR 2: a = z, pencils over (x = b, y = c).
template <int DIR>
__device__ __forceinline__ void sweep_coords(int a, int b, int c, int& x, int& y, int& z) {
  if (DIR == 0) { x = a; y = b; z = c; }
  else if (DIR == 1) { x = b; y = a; z = c; }
  else { x = b; y = c; z = a; }
}

// TMA: a tile whose sweep halo lies inside the domain arrives by one bulk
// tensor copy (T maps the stage input qin on the x sweep and the stored
// primitives on the y and z sweeps; T.on = 0: plain loads only).
// MINB > 0 caps the registers so that MINB blocks fit on an SM; MINB = 0
// leaves the minimum unspecified (ptxas allocates as without the bound).
// CHAR: WENO of the characteristic fields (char_weno_position, FP64).
template <int NF, int WO, class RT, int DIR, int TA, int TB, int TC, int NT, bool TMA = false, int MINB = 0,
          bool CHAR = false>
__global__ void __launch_bounds__(NT, MINB) sweep_kernel(const DevParams P, const __grid_constant__ UniformCoef U,
                                                   const __grid_constant__ TileMap T, const double* __restrict__ qin,
                                                   const double* __restrict__ qbase, double* __restrict__ qout,
                                                   const double dt, const int kind) {
  using Sh = SweepShape<NF, WO, RT, DIR, TA, TB, TC>;
  using Q = Eqs<3, NF>;
  constexpr int S = Sh::S, H = Sh::H, LA = Sh::LA, NP = Sh::NP;
  constexpr bool kSplit = sizeof(RT) == 4;
  using AT = RT;
  constexpr int OA = DIR, OB = DIR == 0 ? 1 : 0, OC = DIR == 2 ? 1 : 2;  // axis index of a, b, c

  extern __shared__ __align__(16) unsigned char smem_raw[];
  RT* sq = reinterpret_cast<RT*>(smem_raw);
  RT* wl = sq + Sh::NQ;
  RT* wr = wl + Sh::NW;
  RT* fl = wr + Sh::NW;
  RT* sc = sq + Sh::OC;  // 16-byte aligned coefficient records
  // split WENO5 keeps the variables in interleaved pairs (2p, 2p+1) of the
  // primitive tile and the WENO values, reconstructed two at a time with
  // packed FP32 instructions (sys_size is even in 3-D)
  constexpr bool kPair = Sh::NCOEF > 0;
  static_assert(!kPair || S % 2 == 0, "3-D pairs need an even number of variables");
  auto qi = [](int v, int p, int la) {
    return kPair ? (((v >> 1) * NP + p) * LA + la) * 2 + (v & 1) : (v * NP + p) * LA + la;
  };
  auto wi = [](int v, int p, int ca) {
    return kPair ? (((v >> 1) * NP + p) * (TA + 2) + ca) * 2 + (v & 1) : (v * NP + p) * (TA + 2) + ca;
  };

  const int tid = threadIdx.x;
  // block origin: blockIdx.x tiles the fastest non-sweep axis for DIR != 0
  int a0, b0, c0;
  if (DIR == 0) { a0 = blockIdx.x * TA; b0 = blockIdx.y * TB; c0 = blockIdx.z * TC; }
  else { b0 = blockIdx.x * TB; a0 = blockIdx.y * TA; c0 = blockIdx.z * TC; }
  const int na = P.n[OA], nb = P.n[OB], nc = P.n[OC];

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
  // split WENO5 on a uniform grid: one coefficient record for the whole sweep
  const bool ua = Sh::NCOEF > 0 && U.on[DIR];
  (void)ua;
  const int64_t st[3] = {1, P.sy, P.sz};

  // ---- load + BCs + cons -> prim ------------------------------------------------
  // the tile's coefficient records come from constant tables: staged before
  // the wait for the previous kernel
  if constexpr (Sh::NCOEF > 0) {
    for (int it = ua ? kCoefRec * (TA + 2) : tid; it < kCoefRec * (TA + 2); it += NT) {
      const int ca = it % (TA + 2), k = it / (TA + 2);
      sc[ca * kCoefRec + k] =
          k < kNumCoef
              ? d2f_bits(__ldg(P.coef[DIR] + k * P.cstride[DIR] + clamp_coef_index(a0 - 1 + ca, na) + P.coff))
              : 0.f;
    }
  }
  // the primitives of the stage input: written by the x sweep for the cells
  // it owns, read by the y and z sweeps
  RT* const gprim = reinterpret_cast<RT*>(P.work) + int64_t(S) * P.sv;
  // one cell: BCs applied, cons -> prim into the tile; the x sweep also
  // stores the cells of its own tile (la = H .. H+TA-1 inside the domain;
  // own: the cell's offset, or -1)
  auto store_prim = [&](double (&q)[S], const int p, const int la, const int64_t own) {
    RT pr[S];
    if constexpr (kSplit) {
      cons_to_prim_split<3, NF>(q, P, pr);
    } else {
      cons_to_prim<3, NF>(q, P);
#pragma unroll
      for (int v = 0; v < S; ++v) pr[v] = q[v];
    }
#pragma unroll
    for (int v = 0; v < S; ++v) sq[qi(v, p, la)] = pr[v];
    if (DIR == 0 && own >= 0) {
#pragma unroll
      for (int v = 0; v < S; ++v) gprim[own + v * P.sv] = pr[v];
    }
  };
  // x sweep: the offset of tile cell (la, pb, pc) when the block owns it
  auto owned = [&](const int la, const int pb, const int pc) -> int64_t {
    const int ga = a0 - H + la, gb = b0 + pb, gc = c0 + pc;
    if (la < H || la >= H + TA || ga >= na || gb >= nb || gc >= nc) return -1;
    return int64_t(gc) * P.sz + int64_t(gb) * P.sy + ga;
  };
  bool use_tma = false;
  unsigned char* stg = nullptr;
  uint32_t bar = 0;
  if constexpr (TMA && Sh::kTmaFits) {
    use_tma = T.on && a0 >= H && a0 + TA + H <= na && b0 + TB <= nb && c0 + TC <= nc;
    if (use_tma) {
      const uintptr_t a = reinterpret_cast<uintptr_t>(wl);
      stg = reinterpret_cast<unsigned char*>((a + 127) & ~uintptr_t(127));
      bar = smem_addr(stg + Sh::kStageBytes);
      if (tid == 0) mbar_init(bar, 1);
    }
  }
  griddep_wait();  // the state (and the partial RHS) below are earlier kernels' output
  if constexpr (DIR > 0) {
    // The operands of the block's last phase that the tile load does not
    // bring in: the partial RHS (y and z sweeps) and, on the z sweep, the RK
    // registers.  Every 128-byte line of the block's rows (TB cells along x
    // per variable and row; rows start 128-byte aligned) is prefetched into
    // L2 while the tile is reconstructed: at 256^3 a register is 1 GB and
    // none of them stays in L2 between the sweeps.
    const int arrays = DIR == 1 || kind == kRhsOnly ? 1 : (kind == kRkEuler ? 2 : 3);
    constexpr int kLinesD = (TB * 8 + 127) / 128, kLinesA = (TB * int(sizeof(AT)) + 127) / 128;
    constexpr int kLines = kLinesD > kLinesA ? kLinesD : kLinesA;
    const int nrow = S * TA * TC;
    const AT* rb = reinterpret_cast<const AT*>(P.work);
    for (int it = tid; it < arrays * nrow * kLines; it += NT) {
      const int line = it % kLines, r = it / kLines;
      const int arr = r / nrow, l = r - arr * nrow;
      const int v = l % S, ta = (l / S) % TA, pc = l / (S * TA);
      const int per_line = arr == 0 ? 128 / int(sizeof(AT)) : 16;  // elements of a 128-byte line
      const int gb = b0 + line * per_line;
      const int ga = a0 + ta, gc = c0 + pc;
      if (ga >= na || gc >= nc || gb >= nb || line >= (arr == 0 ? kLinesA : kLinesD)) continue;
      int x, y, z;
      sweep_coords<DIR>(ga, gb, gc, x, y, z);
      const int64_t o = z * P.sz + y * P.sy + x + v * P.sv;
      const void* ptr = arr == 0 ? static_cast<const void*>(rb + o)
                                 : arr == 1 ? static_cast<const void*>(qbase + o) : static_cast<const void*>(qin + o);
      asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
    }
  }
  if (use_tma) {
    volatile int* landed = reinterpret_cast<volatile int*>(stg + Sh::kStageBytes + 8);
    if (tid == 0) {
      mbar_arrive_expect_tx(bar, Sh::kStageBytes);
      if (DIR == 0) tma_load_4d(smem_addr(stg), &T.map, a0 - TmaBox<TA, H>::kLead, b0, c0, 0, bar);
      else if (DIR == 1) tma_load_4d(smem_addr(stg), &T.map, b0, a0 - H, c0, 0, bar);
      else tma_load_4d(smem_addr(stg), &T.map, b0, c0, a0 - H, 0, bar);
      const bool ok = mbar_wait_bounded(bar, 0, 1000000000ull);  // 1 s
      if (!ok) (void)mbar_wait_bounded(bar, 0, 1000000000ull);    // the copy may still be in flight
      *landed = ok ? 1 : 0;
    }
    __syncthreads();
    if (*landed == 0) {
      if (tid == 0 && P.status) atomicOr(P.status, MFC_FLAG_TIMEOUT);
      return;
    }
    (void)mbar_try_wait(bar, 0);  // completed: each thread acquires the copy's writes
    for (int it = tid; it < NP * LA; it += NT) {
      int la, pb, pc;
      if (DIR == 0) { la = it % LA; pb = (it / LA) % TB; pc = it / (LA * TB); }
      else { pb = it % TB; la = (it / TB) % LA; pc = it / (TB * LA); }
      // box element (x, y, z) of variable v: ((v * BZ + z) * BY + y) * BX + x
      int bx, by, bz;
      if (DIR == 0) { bx = la + TmaBox<TA, H>::kLead - H; by = pb; bz = pc; }
      else if (DIR == 1) { bx = pb; by = la; bz = pc; }
      else { bx = pb; by = pc; bz = la; }
      if constexpr (DIR == 0) {
        const double* sd = reinterpret_cast<const double*>(stg);
        double q[S];
#pragma unroll
        for (int v = 0; v < S; ++v) q[v] = sd[((v * Sh::BZ + bz) * Sh::BY + by) * Sh::BX + bx];
        store_prim(q, pc * TB + pb, la, owned(la, pb, pc));
      } else {
        const RT* sd = reinterpret_cast<const RT*>(stg);
#pragma unroll
        for (int v = 0; v < S; ++v) sq[qi(v, pc * TB + pb, la)] = sd[((v * Sh::BZ + bz) * Sh::BY + by) * Sh::BX + bx];
      }
    }
  } else {  // plain loads, with the boundary conditions and processor halos
    // thread order: the a index fastest for the x sweep, the pencil b index
    // fastest otherwise, so that global loads are coalesced along x
    for (int it = tid; it < NP * LA; it += NT) {
      int la, pb, pc;
      if (DIR == 0) { la = it % LA; pb = (it / LA) % TB; pc = it / (LA * TB); }
      else { pb = it % TB; la = (it / TB) % LA; pc = it / (TB * LA); }
      bool fa = false, dummy = false;
      const int ra = a0 - H + la;
      // processor boundary along the sweep: the ghost cell comes from the
      // neighbour's halo buffer (x: [S][nz][ny][H], y: [S][nz][H][nx],
      // z: [S][H][ny][nx]; depth 0 next to the boundary)
      const int side = ra < 0 ? (P.bc_beg[OA] >= 0 ? 0 : -1) : (ra >= na && P.bc_end[OA] >= 0 ? 1 : -1);
      const int gb = map_cell(b0 + pb, nb, P.bc_beg[OB], P.bc_end[OB], &dummy);
      const int gc = map_cell(c0 + pc, nc, P.bc_beg[OC], P.bc_end[OC], &dummy);
      const double* src;
      int64_t vs = P.sv;
      if (side >= 0) {
        const int d = min(side == 0 ? -1 - ra : ra - na, H - 1);  // deeper cells of partial tiles are never stored
        int x, y, z;
        sweep_coords<DIR>(d, gb, gc, x, y, z);
        const int nx = P.n[0], ny = P.n[1], nz = P.n[2];
        const double* h = P.halo[2 * DIR + side];
        if (DIR == 0) { src = h + ((int64_t)z * ny + y) * H + d; vs = (int64_t)nz * ny * H; }
        else if (DIR == 1) { src = h + ((int64_t)z * H + d) * nx + x; vs = (int64_t)nz * H * nx; }
        else { src = h + ((int64_t)d * ny + y) * nx + x; vs = (int64_t)H * ny * nx; }
      } else {
        const int ga = map_cell(ra, na, P.bc_beg[OA], P.bc_end[OA], &fa);
        const int64_t o = ga * st[OA] + gb * st[OB] + gc * st[OC];
        if constexpr (DIR > 0) {
          // the stored primitives; a reflected cell's normal velocity negated
          const int p = pc * TB + pb;
#pragma unroll
          for (int v = 0; v < S; ++v) sq[qi(v, p, la)] = __ldg(gprim + o + v * P.sv);
          if (fa) sq[qi(Q::MOM + DIR, p, la)] = -sq[qi(Q::MOM + DIR, p, la)];
          continue;
        }
        src = qin + o;
      }
      double q[S];
#pragma unroll
      for (int v = 0; v < S; ++v) q[v] = __ldg(src + v * vs);
      if (fa) q[Q::MOM + DIR] = -q[Q::MOM + DIR];
      store_prim(q, pc * TB + pb, la, DIR == 0 ? owned(la, pb, pc) : -1);
    }
  }
  __syncthreads();

  // ---- WENO along the sweep for cells a0-1 .. a0+TA --------------------------------
  constexpr int NCA = TA + 2;
  // variable v of cell ca of pencil p; c: the cell's coefficient record
  auto recon = [&](const RT* __restrict__ c, const int ca, const int p, const int v) {
    RT stc[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int o = k - 2;
      stc[k] = (o >= -(WO / 2) && o <= WO / 2) ? sq[qi(v, p, ca + H - 1 + o)] : RT(0);
    }
    RT vl, vr;
    weno_cell<WO, RT>(c, stc, eps, vl, vr);
    wl[wi(v, p, ca)] = vl;
    wr[wi(v, p, ca)] = vr;
  };
  if constexpr (kPair) {
    constexpr int NPR = S / 2;
    const f32x2 eps2 = f2_pack(eps, eps);
    // variable pair pr of cell ca of pencil p; C(k): coefficient k as a (c, c) pair
    auto pair = [&](const auto& C, const int ca, const int p, const int pr) {
      const f32x2* line = reinterpret_cast<const f32x2*>(sq) + (pr * NP + p) * LA + ca + H - 1;
      f32x2 stc[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) stc[k] = line[k - 2];
      f32x2 vl, vr;
      weno5_pair_fast(C, stc, eps2, vl, vr);
      reinterpret_cast<f32x2*>(wl)[(pr * NP + p) * NCA + ca] = vl;
      reinterpret_cast<f32x2*>(wr)[(pr * NP + p) * NCA + ca] = vr;
    };
    // UNI: the shared record of a uniform grid, else the cell's staged
    // record; chosen once per block
    auto positions = [&](auto uni) {
      constexpr bool UNI = decltype(uni)::value;
      deal_positions<NP * NCA, NPR, NT>(tid, [&](const int q, const int v, const bool all) {
        const int ca = q % NCA, p = q / NCA;
        auto one = [&](const int w) {
          if constexpr (UNI) {
            const f32x2* rec = U.rec[DIR];
            pair([&](int k) { return rec[k]; }, ca, p, w);
          } else {
            RT c[kCoefRec];
            load_coef_record(sc + ca * kCoefRec, c);
            pair([&](int k) { return f2_pack(c[k], c[k]); }, ca, p, w);
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
    if (ua) positions(FlagC<true>{});
    else positions(FlagC<false>{});
  } else if constexpr (CHAR) {
    static_assert(sizeof(RT) == 8 && WO > 1, "characteristic-field WENO is compiled for FP64 WENO3/5");
    // one thread per position, all variables
    for (int it = tid; it < NP * NCA; it += NT) {
      const int ca = it % NCA, p = it / NCA;
      double c[kCoefRec];
      const int gi = clamp_coef_index(a0 - 1 + ca, na) + P.coff;
#pragma unroll
      for (int k = 0; k < kNumCoef; ++k) c[k] = __ldg(P.coef[DIR] + k * P.cstride[DIR] + gi);
      char_weno_position<3, NF, WO, DIR>(
          c, [&](int v, int o) { return sq[qi(v, p, ca + H - 1 + o)]; }, eps, P,
          [&](int v) -> RT& { return wl[wi(v, p, ca)]; }, [&](int v) -> RT& { return wr[wi(v, p, ca)]; });
    }
  } else {
    for (int it = tid; it < S * NP * NCA; it += NT) {
      const int ca = it % NCA;
      const int r = it / NCA;
      const int p = r % NP, v = r / NP;
      RT c[kCoefRec];
      if constexpr (WO > 1) {
        const int gi = clamp_coef_index(a0 - 1 + ca, na) + P.coff;
#pragma unroll
        for (int k = 0; k < kNumCoef; ++k) c[k] = RT(__ldg(P.coef[DIR] + k * P.cstride[DIR] + gi));
      }
      recon(c, ca, p, v);
    }
  }
  __syncthreads();

  // ---- HLLC on faces a0-1/2 .. a0+TA-1/2 ---------------------------------------------
  constexpr int NFA = TA + 1;
  for (int it = tid; it < NP * NFA; it += NT) {
    const int f = it % NFA, p = it / NFA;
    const int gface = a0 - 1 + f;
    RT qL[S], qR[S], F[S], us;
    const bool lfr = (gface == -1 && P.bc_beg[OA] == -4);
    const bool rfl = (gface == na - 1 && P.bc_end[OA] == -4);
#pragma unroll
    for (int v = 0; v < S; ++v) {
      const RT a = wr[wi(v, p, f)];
      const RT b = wl[wi(v, p, f + 1)];
      qL[v] = lfr ? b : a;
      qR[v] = rfl ? a : b;
    }
    if constexpr (kSplit) hllc_face_fast<3, NF, DIR>(qL, qR, gam_i, pi_i, F, us);
    else hllc_face<3, NF, DIR, RT>(qL, qR, gam_i, pi_i, F, us);
#pragma unroll
    for (int v = 0; v < S; ++v) fl[(v * NP + p) * NFA + f] = F[v];
    fl[(S * NP + p) * NFA + f] = us;
  }
  __syncthreads();

  // ---- flux divergence, accumulation, RK on the last sweep ---------------------------
  griddep_launch_dependents();
  AT* rhs_buf = reinterpret_cast<AT*>(P.work);
  bool bad = false, nonphys = false;
  double icfl = 0.0;
  const float dtf = kSplit ? __double2float_rn(dt) : 0.f;  // the split path's increments are FP32
  (void)dtf;
  // KIND: the stage's combination as a compile-time constant, so that the z
  // sweep chooses it once per block rather than once per cell and variable
  auto finish = [&](auto kind_c) {
    constexpr int KIND = decltype(kind_c)::value;
    for (int it = tid; it < NP * TA; it += NT) {
      int ta, pb, pc;
      if (DIR == 0) { ta = it % TA; pb = (it / TA) % TB; pc = it / (TA * TB); }
      else { pb = it % TB; ta = (it / TB) % TA; pc = it / (TB * TA); }
      const int ga = a0 + ta, gb = b0 + pb, gc = c0 + pc;
      if (ga >= na || gb >= nb || gc >= nc) continue;
      const int p = pc * TB + pb;
      int x, y, z;
      sweep_coords<DIR>(ga, gb, gc, x, y, z);
      const int64_t o = z * P.sz + y * P.sy + x;
      const AT inv = narrow<AT>(__ldg(P.inv_d[DIR] + ga));
      AT r[S];
#pragma unroll
      for (int v = 0; v < S; ++v) {
        const AT diff = AT(fl[(v * NP + p) * NFA + ta]) - AT(fl[(v * NP + p) * NFA + ta + 1]);
        r[v] = (DIR == 0) ? inv * diff : mul_add(inv, diff, rhs_buf[o + v * P.sv]);
      }
      const AT du = AT(fl[(S * NP + p) * NFA + ta + 1]) - AT(fl[(S * NP + p) * NFA + ta]);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const AT a = AT(sq[qi(Q::ADV + f, p, ta + H)]);
        r[Q::ADV + f] = mul_add(inv * a, du, r[Q::ADV + f]);
      }
      if constexpr (DIR < 2) {
#pragma unroll
        for (int v = 0; v < S; ++v) rhs_buf[o + v * P.sv] = r[v];
        continue;
      }
#pragma unroll
      for (int v = 0; v < S; ++v) {
        double out;
        if constexpr (KIND == kRhsOnly) {
          out = widen(r[v]);
        } else {
          const double b = __ldg(qbase + o + v * P.sv);
          double in = b;
          if constexpr (KIND != kRkEuler) in = __ldg(qin + o + v * P.sv);
          if constexpr (kSplit) out = rk_combine_split(KIND, b, in, dtf, r[v]);
          else out = rk_combine(KIND, b, in, dt, r[v]);
        }
        bad |= not_finite(out);
        qout[o + v * P.sv] = out;
      }
    }
    // the stability monitor (the last stage of a monitored step) reads the
    // new state back: this thread's own stores, from L1
    if (DIR == 2 && P.monitor) {
      for (int it = tid; it < NP * TA; it += NT) {
        const int pb = it % TB, ta = (it / TB) % TA, pc = it / (TB * TA);
        const int ga = a0 + ta, gb = b0 + pb, gc = c0 + pc;
        if (ga >= na || gb >= nb || gc >= nc) continue;
        int x, y, z;
        sweep_coords<DIR>(ga, gb, gc, x, y, z);
        const int64_t o = z * P.sz + y * P.sy + x;
        double qn[S];
#pragma unroll
        for (int v = 0; v < S; ++v) qn[v] = qout[o + v * P.sv];
        const double inv[3] = {__ldg(P.inv_d[0] + x), __ldg(P.inv_d[1] + y), __ldg(P.inv_d[2] + z)};
        bool np;
        const double c = cell_icfl<3, NF>(qn, P, dt, inv, np);
        nonphys |= np;
        if (!(c <= icfl)) icfl = c;  // keeps NaN
      }
    }
  };
  if constexpr (DIR < 2) {
    finish(KindC<kRhsOnly>{});  // the x and y sweeps store the partial RHS whatever the kind
  } else {
    switch (kind) {
      case kRkEuler: finish(KindC<kRkEuler>{}); break;
      case kRk2Final: finish(KindC<kRk2Final>{}); break;
      case kRk3Mid: finish(KindC<kRk3Mid>{}); break;
      case kRk3Final: finish(KindC<kRk3Final>{}); break;
      default: finish(KindC<kRhsOnly>{}); break;
    }
  }
  if (bad && P.status) atomicOr(P.status, MFC_FLAG_NAN);
  if (nonphys && P.status) atomicOr(P.status, MFC_FLAG_NEG_PRESSURE);
  if (DIR == 2 && P.monitor) monitor_max(P.monitor, icfl);
}

}  // namespace mfc
