// Host-side grid tables of the hot path: ghost layers of the cell widths
// (s_populate_grid_variables_buffers, src/simulation/m_start_up.fpp:517-655)
// and the grid-dependent WENO coefficients (s_compute_weno_coefficients,
// src/simulation/m_weno.fpp:168-363), computed in FP64 in the reference's
// operation order, plus the checks of s_check_input_file that apply to the
// path (m_start_up.fpp:117-290).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mfc_gpu.h"
#include "mfc_device.cuh"

namespace mfc {

struct AxisHost {
  int s = 0, b = 0;           // s = last interior index (m), b = buff_size
  std::vector<double> cb, d;  // cb(-1-b : s+b), d(-b : s+b)
  double& CB(int i) { return cb[(size_t)(i + 1 + b)]; }
  double& D(int i) { return d[(size_t)(i + b)]; }
};

// Widths and boundaries of the ghost cells (cell centres are not used by the
// hot path).
// Processor boundaries (bc >= 0) take the neighbour's widths when given
// (wb/we[i] = width of the ghost cell at depth i, as the reference exchanges
// them in s_mpi_sendrecv_grid_variables_buffers), else the edge width.
inline void grid_ghosts(AxisHost& a, int bcb, int bce, const double* wb = nullptr, const double* we = nullptr) {
  const int s = a.s, b = a.b;
  for (int i = 0; i <= s; ++i) a.D(i) = a.CB(i) - a.CB(i - 1);
  for (int i = 1; i <= b; ++i)
    a.D(-i) = (bcb >= 0 && wb) ? wb[i - 1] : (bcb <= -3 || bcb >= 0) ? a.D(0) : bcb == -2 ? a.D(i - 1) : a.D(s - (i - 1));
  for (int i = 1; i <= b; ++i) a.CB(-1 - i) = a.CB(-i) - a.D(-i);
  for (int i = 1; i <= b; ++i)
    a.D(s + i) = (bce >= 0 && we) ? we[i - 1] : (bce <= -3 || bce >= 0) ? a.D(s) : bce == -2 ? a.D(s - (i - 1)) : a.D(i - 1);
  for (int i = 1; i <= b; ++i) a.CB(s + i) = a.CB(s + (i - 1)) + a.D(s + i);
}

// One cell's record: polyL[3][2], polyR[3][2], dL[3], dR[3], beta[3][3]
// (layout kPL .. kBeta), for cell i+1 from the boundaries s_cb(i-2 .. i+3),
// m_weno.fpp:193-346.
inline void weno_record(AxisHost& a, int i, int wo, double* r) {
  auto S = [&](int k) { return a.CB(k); };
  auto sq = [](double x) { return x * x; };
  double* pL = r + kPL;
  double* pR = r + kPR;
  double* dL = r + kDL;
  double* dR = r + kDR;
  double* be = r + kBeta;
  std::fill(r, r + kNumCoef, 0.0);
  if (wo == 3) {
    pR[0] = (S(i) - S(i + 1)) / (S(i) - S(i + 2));
    pR[2] = (S(i) - S(i + 1)) / (S(i - 1) - S(i + 1));
    pL[0] = -pR[0];
    pL[2] = -pR[2];
    dR[0] = (S(i - 1) - S(i + 1)) / (S(i - 1) - S(i + 2));
    dL[0] = (S(i - 1) - S(i)) / (S(i - 1) - S(i + 2));
    dR[1] = 1.0 - dR[0];
    dL[1] = 1.0 - dL[0];
    be[0] = 4.0 * sq(S(i) - S(i + 1)) / sq(S(i) - S(i + 2));
    be[3] = 4.0 * sq(S(i) - S(i + 1)) / sq(S(i - 1) - S(i + 1));
    return;
  }
  // polynomial coefficients [k][j] -> index 2k+j
  pR[0] = ((S(i) - S(i + 1)) * (S(i + 1) - S(i + 2))) / ((S(i) - S(i + 3)) * (S(i + 3) - S(i + 1)));
  pR[2] = ((S(i - 1) - S(i + 1)) * (S(i + 1) - S(i))) / ((S(i - 1) - S(i + 2)) * (S(i + 2) - S(i)));
  pR[3] = ((S(i) - S(i + 1)) * (S(i + 1) - S(i + 2))) / ((S(i - 1) - S(i + 1)) * (S(i - 1) - S(i + 2)));
  pR[5] = ((S(i) - S(i + 1)) * (S(i + 1) - S(i - 1))) / ((S(i - 2) - S(i)) * (S(i - 2) - S(i + 1)));
  pL[0] = ((S(i + 1) - S(i)) * (S(i) - S(i + 2))) / ((S(i) - S(i + 3)) * (S(i + 3) - S(i + 1)));
  pL[2] = ((S(i) - S(i - 1)) * (S(i) - S(i + 1))) / ((S(i - 1) - S(i + 2)) * (S(i) - S(i + 2)));
  pL[3] = ((S(i + 1) - S(i)) * (S(i) - S(i + 2))) / ((S(i - 1) - S(i + 1)) * (S(i - 1) - S(i + 2)));
  pL[5] = ((S(i - 1) - S(i)) * (S(i) - S(i + 1))) / ((S(i - 2) - S(i)) * (S(i - 2) - S(i + 1)));
  pR[1] = ((S(i) - S(i + 2)) + (S(i + 1) - S(i + 3))) / ((S(i) - S(i + 2)) * (S(i) - S(i + 3))) * ((S(i) - S(i + 1)));
  pR[4] = ((S(i - 2) - S(i + 1)) + (S(i - 1) - S(i + 1))) / ((S(i - 1) - S(i + 1)) * (S(i + 1) - S(i - 2))) *
          ((S(i + 1) - S(i)));
  pL[1] = ((S(i) - S(i + 2)) + (S(i) - S(i + 3))) / ((S(i) - S(i + 2)) * (S(i) - S(i + 3))) * ((S(i + 1) - S(i)));
  pL[4] = ((S(i - 2) - S(i)) + (S(i - 1) - S(i + 1))) / ((S(i - 2) - S(i + 1)) * (S(i + 1) - S(i - 1))) *
          ((S(i) - S(i + 1)));
  dR[0] = ((S(i - 2) - S(i + 1)) * (S(i + 1) - S(i - 1))) / ((S(i - 2) - S(i + 3)) * (S(i + 3) - S(i - 1)));
  dR[2] = ((S(i + 1) - S(i + 2)) * (S(i + 1) - S(i + 3))) / ((S(i - 2) - S(i + 2)) * (S(i - 2) - S(i + 3)));
  dL[0] = ((S(i - 2) - S(i)) * (S(i) - S(i - 1))) / ((S(i - 2) - S(i + 3)) * (S(i + 3) - S(i - 1)));
  dL[2] = ((S(i) - S(i + 2)) * (S(i) - S(i + 3))) / ((S(i - 2) - S(i + 2)) * (S(i - 2) - S(i + 3)));
  dR[1] = 1.0 - dR[0] - dR[2];
  dL[1] = 1.0 - dL[0] - dL[2];
  const double h = S(i) - S(i + 1);
  be[0] = 4.0 * sq(h) *
          (10.0 * sq(S(i + 1) - S(i)) + (S(i + 1) - S(i)) * (S(i + 2) - S(i + 1)) + sq(S(i + 2) - S(i + 1))) /
          (sq(S(i) - S(i + 3)) * sq(S(i + 1) - S(i + 3)));
  be[1] = 4.0 * sq(h) *
          (19.0 * sq(S(i + 1) - S(i)) - (S(i + 1) - S(i)) * (S(i + 3) - S(i + 1)) +
           2.0 * (S(i + 2) - S(i)) * ((S(i + 2) - S(i)) + (S(i + 3) - S(i + 1)))) /
          ((S(i) - S(i + 2)) * sq(S(i) - S(i + 3)) * (S(i + 3) - S(i + 1)));
  be[2] = 4.0 * sq(h) *
          (10.0 * sq(S(i + 1) - S(i)) + (S(i + 1) - S(i)) * ((S(i + 2) - S(i)) + (S(i + 3) - S(i + 1))) +
           sq((S(i + 2) - S(i)) + (S(i + 3) - S(i + 1)))) /
          (sq(S(i) - S(i + 2)) * sq(S(i) - S(i + 3)));
  be[3] = 4.0 * sq(h) *
          (10.0 * sq(S(i + 1) - S(i)) + sq(S(i) - S(i - 1)) + (S(i) - S(i - 1)) * (S(i + 1) - S(i))) /
          (sq(S(i - 1) - S(i + 2)) * sq(S(i) - S(i + 2)));
  be[4] = 4.0 * sq(h) *
          ((S(i) - S(i + 1)) * ((S(i) - S(i - 1)) + 20.0 * (S(i + 1) - S(i))) +
           (2.0 * (S(i) - S(i - 1)) + (S(i + 1) - S(i))) * (S(i + 2) - S(i))) /
          ((S(i + 1) - S(i - 1)) * sq(S(i - 1) - S(i + 2)) * (S(i + 2) - S(i)));
  be[5] = 4.0 * sq(h) *
          (10.0 * sq(S(i + 1) - S(i)) + (S(i + 1) - S(i)) * (S(i + 2) - S(i + 1)) + sq(S(i + 2) - S(i + 1))) /
          (sq(S(i - 1) - S(i + 1)) * sq(S(i - 1) - S(i + 2)));
  be[6] = 4.0 * sq(h) *
          (12.0 * sq(S(i + 1) - S(i)) + sq((S(i) - S(i - 2)) + (S(i) - S(i - 1))) +
           3.0 * ((S(i) - S(i - 2)) + (S(i) - S(i - 1))) * (S(i + 1) - S(i))) /
          (sq(S(i - 2) - S(i + 1)) * sq(S(i - 1) - S(i + 1)));
  be[7] = 4.0 * sq(h) *
          (19.0 * sq(S(i + 1) - S(i)) + ((S(i) - S(i - 2)) * (S(i) - S(i + 1))) +
           2.0 * (S(i + 1) - S(i - 1)) * ((S(i) - S(i - 2)) + (S(i + 1) - S(i - 1)))) /
          ((S(i - 2) - S(i)) * sq(S(i - 2) - S(i + 1)) * (S(i + 1) - S(i - 1)));
  be[8] = 4.0 * sq(h) *
          (10.0 * sq(S(i + 1) - S(i)) + sq(S(i) - S(i - 1)) + (S(i) - S(i - 1)) * (S(i + 1) - S(i))) /
          (sq(S(i - 2) - S(i)) * sq(S(i - 2) - S(i + 1)));
}

// Grid tables of all directions in one host array: per direction 1/dx(i)
// (the reference's 1d0/dx(k)) for the n interior cells, then kNumCoef
// coefficient rows over cells -kCoefPad .. n-1+kCoefPad (SoA).  Returns an
// empty string on success, else the reason.
struct GridTables {
  std::vector<double> host;
  size_t off_inv[3] = {0, 0, 0}, off_coef[3] = {0, 0, 0}, off_dcc[3] = {0, 0, 0};
  int cstride[3] = {0, 0, 0};
};

// ghost[d][side]: neighbour widths for processor boundaries (b values), or NULL
inline std::string build_grid_tables(const mfc_params* p, int nd, const int* n, int b, GridTables& t,
                                     const double* const (*ghost)[2] = nullptr) {
  const double* cbs[3] = {p->x_cb, p->y_cb, p->z_cb};
  const int bcb[3] = {p->bc_x_beg, p->bc_y_beg, p->bc_z_beg};
  const int bce[3] = {p->bc_x_end, p->bc_y_end, p->bc_z_end};
  const int polyn = (p->weno_order - 1) / 2;
  t.host.clear();
  for (int d = 0; d < nd; ++d) {
    AxisHost a;
    a.s = n[d] - 1;
    a.b = b;
    a.cb.assign((size_t)(a.s + 2 * a.b + 2), 0.0);
    a.d.assign((size_t)(a.s + 2 * a.b + 1), 0.0);
    for (int i = -1; i <= a.s; ++i) a.CB(i) = cbs[d][i + 1];
    grid_ghosts(a, bcb[d], bce[d], ghost ? ghost[d][0] : nullptr, ghost ? ghost[d][1] : nullptr);
    for (int i = 0; i <= a.s; ++i)
      if (!(a.D(i) > 0.0)) return "cell boundaries must increase";
    t.off_inv[d] = t.host.size();
    for (int i = 0; i <= a.s; ++i) t.host.push_back(1.0 / a.D(i));
    // cell centres x_cc(-1 .. s+1) (m_start_up.fpp:342-343 and the ghost
    // centres of s_populate_grid_variables_buffers), then their spacings
    // dcc(i) = x_cc(i) - x_cc(i-1), i = 0 .. s+1, for the viscous gradients
    {
      std::vector<double> cc((size_t)a.s + 3);  // cc[i + 1] = x_cc(i)
      for (int i = 0; i <= a.s; ++i) cc[(size_t)i + 1] = a.CB(i - 1) + a.D(i) / 2.0;
      cc[0] = cc[1] - (a.D(0) + a.D(-1)) / 2.0;
      cc[(size_t)a.s + 2] = cc[(size_t)a.s + 1] + (a.D(a.s) + a.D(a.s + 1)) / 2.0;
      t.off_dcc[d] = t.host.size();
      for (int i = 0; i <= a.s + 1; ++i) t.host.push_back(cc[(size_t)i + 1] - cc[(size_t)i]);
    }
    const int pad = kCoefPad;
    t.cstride[d] = n[d] + 2 * pad;
    t.off_coef[d] = t.host.size();
    t.host.resize(t.host.size() + (size_t)kNumCoef * t.cstride[d], 0.0);
    if (p->weno_order > 1) {
      // the reference defines coefficients for cells -b+polyn .. s+b-polyn
      const int lo = -b + polyn, hi = a.s + b - polyn;
      double rec[kNumCoef];
      for (int cell = -pad; cell <= a.s + pad; ++cell) {
        const int src = std::min(std::max(cell, lo), hi);
        weno_record(a, src - 1, p->weno_order, rec);
        for (int k = 0; k < kNumCoef; ++k) t.host[t.off_coef[d] + (size_t)k * t.cstride[d] + (cell + pad)] = rec[k];
      }
    }
  }
  return "";
}

// The device's truncating double -> float conversion (d2f_bits in
// mfc_device.cuh) on the host, through the same bit-level function.
inline float d2f_trunc(double x) {
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  const uint32_t r = d2f_trunc_word((uint32_t)(b >> 32), (uint32_t)b);
  float f;
  std::memcpy(&f, &r, sizeof f);
  return f;
}

// Split-precision WENO5 on a uniform grid: fills U.rec[d] (each coefficient
// as a (c, c) pair) and sets U.on[d] for every direction whose cells
// -kCoefPad .. n-1+kCoefPad all have the same FP32 coefficient record (the
// one the kernels would stage per cell), so that the kernels may use that
// one record everywhere with identical results.
inline void uniform_records(const GridTables& t, int nd, const int* n, int weno_order, int precision,
                            UniformCoef& U) {
  U = UniformCoef{};
  if (precision == MFC_PREC_FP64 || precision == MFC_PREC_FP64_FMA || weno_order != 5) return;
  for (int d = 0; d < nd; ++d) {
    const int cells = n[d] + 2 * kCoefPad;
    auto bits = [](float f) {
      uint32_t u;
      std::memcpy(&u, &f, sizeof u);
      return u;
    };
    bool same = true;
    float rec[kCoefRec] = {};
    for (int k = 0; k < kNumCoef && same; ++k) {
      const double* row = t.host.data() + t.off_coef[d] + (size_t)k * t.cstride[d];
      rec[k] = d2f_trunc(row[0]);
      for (int i = 1; i < cells && same; ++i) same = bits(d2f_trunc(row[i])) == bits(rec[k]);
    }
    if (!same) continue;
    U.on[d] = 1;
    for (int k = 0; k < kCoefRec; ++k) U.rec[d][k] = (unsigned long long)bits(rec[k]) << 32 | bits(rec[k]);
  }
}

// The checks of s_check_input_file that apply to the hot path.
// allow_processor: boundary values >= 0 (a neighbouring subdomain, exchanged
// through halo buffers) are accepted.
inline std::string validate_params(const mfc_params* p, bool allow_processor = false) {
  if (!p) return "params is NULL";
  if (p->m <= 0) return "Unsupported value of m";
  if (p->n < 0 || p->p < 0) return "Unsupported value of n or p";
  if (p->p > 0 && p->n == 0) return "p > 0 requires n > 0";
  if (p->num_fluids < 1 || p->num_fluids > 2) return "Unsupported value of num_fluids (1 or 2)";
  if (p->weno_order != 1 && p->weno_order != 3 && p->weno_order != 5) return "Unsupported value of weno_order";
  const int stcls = 5 * p->weno_order;  // num_stcls_min*weno_order, m_start_up.fpp:182-189
  if (p->m + 1 < stcls) return "Unsupported combination of values of m and weno_order";
  if (p->n > 0 && p->n + 1 < stcls) return "Unsupported combination of values of n and weno_order";
  if (!(p->weno_eps > 0.0) || p->weno_eps > 1e-6) return "Unsupported value of weno_eps";
  if (p->time_stepper < 1 || p->time_stepper > 3) return "Unsupported value of time_stepper";
  const int bcs[6] = {p->bc_x_beg, p->bc_x_end, p->bc_y_beg, p->bc_y_end, p->bc_z_beg, p->bc_z_end};
  const int ndim = 1 + (p->n > 0) + (p->p > 0);
  for (int d = 0; d < ndim; ++d) {
    for (int e = 0; e < 2; ++e) {
      const int bc = bcs[2 * d + e];
      if (bc >= 0 && !allow_processor)
        return "Unsupported boundary condition (processor boundaries need a context with halo buffers)";
      if (bc < -12 || (bc > -1 && !allow_processor)) return "Unsupported boundary condition";
    }
    if ((bcs[2 * d] == -1) != (bcs[2 * d + 1] == -1)) return "Periodic boundaries must be set at both ends";
  }
  for (int f = 0; f < p->num_fluids; ++f) {
    if (!(p->gammas[f] > 0.0)) return "Unsupported value of fluid_pp%gamma";
    if (p->pi_infs[f] < 0.0) return "Unsupported value of fluid_pp%pi_inf";
  }
  if (!p->x_cb) return "x_cb is NULL";
  if (p->n > 0 && !p->y_cb) return "y_cb is NULL";
  if (p->p > 0 && !p->z_cb) return "z_cb is NULL";
  if (p->p > 0 && p->p + 1 < stcls) return "Unsupported combination of values of p and weno_order";
  if (p->precision != MFC_PREC_FP64 && p->precision != MFC_PREC_SPLIT && p->precision != MFC_PREC_GATED &&
      p->precision != MFC_PREC_FP64_FMA)
    return "Unsupported precision";
  if (p->precision == MFC_PREC_FP64_FMA && (p->n == 0 || p->p > 0 || p->weno_order != 5))
    return "The contracted FP64 variant is compiled for 2-D WENO5 cases";
  if (p->precision == MFC_PREC_GATED && (p->n == 0 || p->p > 0 || p->weno_order != 5))
    return "The learned gate runs on 2-D WENO5 cases";
  return "";
}

}  // namespace mfc
