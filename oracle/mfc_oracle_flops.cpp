// Operation counting for the oracle (test infrastructure only).
//
// Instantiates the oracle with a scalar type that counts every floating-point
// add/subtract, multiply, divide, square root and comparison, runs one full
// time step and reports the counts per interior cell.  These are the
// algorithmic operation counts per cell-update used for the compute roofline.
// Built without OpenMP so the counters need no atomics.
#include <cmath>

#include "mfc_oracle.hpp"

namespace {

struct Counts {
  double add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0;
};
Counts g_counts;

struct CR {
  double v;
  CR() : v(0) {}
  CR(double x) : v(x) {}  // NOLINT: implicit on purpose, like a double
};
inline CR operator+(CR a, CR b) { g_counts.add += 1; return CR(a.v + b.v); }
inline CR operator-(CR a, CR b) { g_counts.add += 1; return CR(a.v - b.v); }
inline CR operator*(CR a, CR b) { g_counts.mul += 1; return CR(a.v * b.v); }
inline CR operator/(CR a, CR b) { g_counts.div += 1; return CR(a.v / b.v); }
inline CR operator-(CR a) { return CR(-a.v); }
inline bool operator<(CR a, CR b) { g_counts.cmp += 1; return a.v < b.v; }
inline bool operator>(CR a, CR b) { g_counts.cmp += 1; return a.v > b.v; }
inline bool operator<=(CR a, CR b) { g_counts.cmp += 1; return a.v <= b.v; }
inline bool operator>=(CR a, CR b) { g_counts.cmp += 1; return a.v >= b.v; }
inline CR sqrt(CR a) { g_counts.sqrt += 1; return CR(std::sqrt(a.v)); }
inline CR copysign(CR a, CR b) { return CR(std::copysign(a.v, b.v)); }
// std::min / std::max fall back on operator<, so they are counted as compares.

}  // namespace


extern "C" {
struct mfo_params;
}

// Same layout as mfo_params in mfc_oracle_capi.cpp.
struct mfo_params_layout {
  int m, n, p;
  int num_fluids;
  int weno_order;
  double weno_eps;
  int time_stepper;
  int bc_x_beg, bc_x_end, bc_y_beg, bc_y_end, bc_z_beg, bc_z_end;
  double gammas[mfc_oracle::kMaxFluids];
  double pi_infs[mfc_oracle::kMaxFluids];
};

extern "C" int mfo_count_ops(const mfo_params* qq, const double* x_cb, const double* y_cb, const double* z_cb,
                             const double* state, double dt, double* counts_out) {
  const auto* q = reinterpret_cast<const mfo_params_layout*>(qq);
  mfc_oracle::Params P;
  P.m = q->m; P.n = q->n; P.p = q->p;
  P.num_fluids = q->num_fluids;
  P.weno_order = q->weno_order;
  P.weno_eps = q->weno_eps;
  P.time_stepper = q->time_stepper;
  P.bc_x_beg = q->bc_x_beg; P.bc_x_end = q->bc_x_end;
  P.bc_y_beg = q->bc_y_beg; P.bc_y_end = q->bc_y_end;
  P.bc_z_beg = q->bc_z_beg; P.bc_z_end = q->bc_z_end;
  for (int i = 0; i < mfc_oracle::kMaxFluids; ++i) { P.gammas[i] = q->gammas[i]; P.pi_infs[i] = q->pi_infs[i]; }
  mfc_oracle::Solver<CR> s;
  s.init(P, x_cb, y_cb, z_cb);
  long c = 0;
  for (int v = 0; v < s.S; ++v)
    for (int k = 0; k <= P.p; ++k)
      for (int j = 0; j <= P.n; ++j)
        for (int i = 0; i <= P.m; ++i) s.q_cons_ts[0][v](i, j, k) = CR(state[c++]);
  s.dt = dt;
  g_counts = Counts{};
  s.tvd_rk(false);
  const double cells = double(P.m + 1) * (P.n + 1) * (P.p + 1);
  counts_out[0] = g_counts.add / cells;
  counts_out[1] = g_counts.mul / cells;
  counts_out[2] = g_counts.div / cells;
  counts_out[3] = g_counts.sqrt / cells;
  counts_out[4] = g_counts.cmp / cells;
  return 0;
}
