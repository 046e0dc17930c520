// MicroFC hot-path ORACLE -- test infrastructure only.
//
// A CPU restatement of MicroFC's right-hand side and TVD Runge-Kutta step for
// the 5-equation diffuse-interface model, written to follow the reference's
// Fortran loops in the same operation order, so that its FP64 results are the
// yardstick the CUDA kernels are checked against.  Nothing in the product
// package links or calls this file; only the tests, the smoke check and the
// CPU-baseline leg of the benchmark do.
//
// Parity status: parity unpinned against the reference build.  The reference
// is Fortran+Fypp and ships no tests, golden vectors or fixtures; no Fortran
// compiler exists where this oracle is built.  It is pinned instead by
// analytic known-answer tests (exact Sod solution, WENO5 order of accuracy,
// conservation, free-stream preservation, mirror symmetry) in tests/.
//
// Reference files followed (paths inside the MicroFC project):
//   grid ghosts          src/simulation/m_start_up.fpp:342-343, 517-655
//   WENO coefficients    src/simulation/m_weno.fpp:168-363
//   WENO1/3/5            src/simulation/m_weno.fpp:391-536
//   cons -> prim         src/common/m_variables_conversion.fpp:98-106, 187-227, 313-375
//   prim -> cons         src/common/m_variables_conversion.fpp:385-443
//   ghost-cell BCs       src/simulation/m_rhs.fpp:686-908
//   Riemann-state BCs    src/simulation/m_riemann_solvers.fpp:444-619
//   HLLC                 src/simulation/m_riemann_solvers.fpp:132-327
//   RHS assembly         src/simulation/m_rhs.fpp:405-679
//   TVD RK1/2/3          src/simulation/m_time_steppers.fpp:129-362
//   time loop, dt trim   src/simulation/p_main.fpp:196-318
//   grid, patches, IC    src/pre_process/m_grid.f90:54-137,
//                        src/pre_process/m_create_patches.fpp:47-313,
//                        src/pre_process/m_assign_patches.fpp:54-165,
//                        src/pre_process/m_initial_condition.fpp:42-112
//
// The reference is 1-D/2-D only.  The z direction (p > 0) extends the same
// formulas with the direction index cycle (3,1,2), exactly as the x and y
// sweeps use (1,2) and (2,1); it has no reference counterpart.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace mfc_oracle {

constexpr int kMaxFluids = 4;
constexpr double kSgmEps = 1e-16;  // m_global_parameters.fpp:39

struct Params {
  int m = 0, n = 0, p = 0;
  int num_fluids = 1;
  int weno_order = 5;
  double weno_eps = 1e-16;
  int time_stepper = 3;
  int bc_x_beg = -3, bc_x_end = -3;
  int bc_y_beg = -3, bc_y_end = -3;
  int bc_z_beg = -3, bc_z_end = -3;
  double gammas[kMaxFluids] = {0};   // fluid_pp(i)%gamma  = 1/(gamma_i - 1)
  double pi_infs[kMaxFluids] = {0};  // fluid_pp(i)%pi_inf = gamma_i pi_inf_i/(gamma_i - 1)
  double re[2][kMaxFluids] = {};     // fluid_pp(i)%Re(1:2), shear and bulk; <= 0: none
  bool char_decomp = false;          // characteristic-field WENO (see weno(); not in the reference)
  bool weno_re_flux = false;         // weno_Re_flux: viscous stresses from WENO-reconstructed gradients

  int num_dims() const { return 1 + (n > 0) + (p > 0); }
  int weno_polyn() const { return (weno_order - 1) / 2; }
  // Re_size / Re_idx of m_global_parameters.fpp:300-336: the fluids with a
  // positive Reynolds number, in index order
  int re_size(int i) const {
    int c = 0;
    for (int f = 0; f < num_fluids; ++f) c += re[i][f] > 0.0;
    return c;
  }
  int re_idx(int i, int q) const {
    for (int f = 0; f < num_fluids; ++f)
      if (re[i][f] > 0.0 && q-- == 0) return f;
    return -1;
  }
  bool viscous() const { return re_size(0) > 0 || re_size(1) > 0; }
  // m_global_parameters.fpp:354-359
  int buff_size() const { return viscous() ? 2 * weno_polyn() + 2 : weno_polyn() + 2; }
  int cont_end() const { return num_fluids; }          // contxe
  int mom_beg() const { return num_fluids + 1; }       // momxb (1-based)
  int E_idx() const { return num_fluids + num_dims() + 1; }
  int adv_beg() const { return E_idx() + 1; }
  int sys_size() const { return E_idx() + num_fluids; }
};

// ---------------------------------------------------------------------------
// Scalar fields with Fortran-style index ranges; x fastest.
template <class R>
struct Field {
  int xb = 0, xe = 0, yb = 0, ye = 0, zb = 0, ze = 0;
  long sx = 1, sy = 1, sz = 1;
  std::vector<R> d;
  void alloc(int xb_, int xe_, int yb_, int ye_, int zb_, int ze_) {
    xb = xb_; xe = xe_; yb = yb_; ye = ye_; zb = zb_; ze = ze_;
    sy = (long)(xe - xb + 1);
    sz = sy * (long)(ye - yb + 1);
    d.assign((size_t)(sz * (long)(ze - zb + 1)), R(0));
  }
  R& operator()(int i, int j, int k) { return d[(size_t)((i - xb) + (j - yb) * sy + (k - zb) * sz)]; }
  const R& operator()(int i, int j, int k) const {
    return d[(size_t)((i - xb) + (j - yb) * sy + (k - zb) * sz)];
  }
};

// One coordinate direction: cell boundaries s_cb(-1-b : s+b), widths ds(-b : s+b)
// and the WENO coefficients of that direction.
template <class R>
struct Axis {
  int s = 0, b = 0;
  std::vector<R> cb, d, cc;
  R& CB(int i) { return cb[(size_t)(i + 1 + b)]; }
  R& D(int i) { return d[(size_t)(i + b)]; }
  R& CC(int i) { return cc[(size_t)(i + b)]; }
  // WENO coefficients for cells i in [-b+polyn, s+b-polyn]
  int wb = 0;
  struct Coef { R polyL[3][2], polyR[3][2], dL[3], dR[3], beta[3][3]; };
  std::vector<Coef> coef;
  Coef& C(int i) { return coef[(size_t)(i - wb)]; }
};

// Ghost cells of the grid, m_start_up.fpp:517-655.  cb(-1:s) must be set.
template <class R>
void populate_grid_buffers(Axis<R>& a, int bc_beg, int bc_end) {
  const int s = a.s, b = a.b;
  for (int i = 0; i <= s; ++i) a.D(i) = a.CB(i) - a.CB(i - 1);
  for (int i = 0; i <= s; ++i) a.CC(i) = a.CB(i - 1) + a.D(i) / R(2);
  if (bc_beg <= -3) { for (int i = 1; i <= b; ++i) a.D(-i) = a.D(0); }
  else if (bc_beg == -2) { for (int i = 1; i <= b; ++i) a.D(-i) = a.D(i - 1); }
  else if (bc_beg == -1) { for (int i = 1; i <= b; ++i) a.D(-i) = a.D(s - (i - 1)); }
  for (int i = 1; i <= b; ++i) a.CB(-1 - i) = a.CB(-i) - a.D(-i);
  for (int i = 1; i <= b; ++i) a.CC(-i) = a.CC(1 - i) - (a.D(1 - i) + a.D(-i)) / R(2);
  if (bc_end <= -3) { for (int i = 1; i <= b; ++i) a.D(s + i) = a.D(s); }
  else if (bc_end == -2) { for (int i = 1; i <= b; ++i) a.D(s + i) = a.D(s - (i - 1)); }
  else if (bc_end == -1) { for (int i = 1; i <= b; ++i) a.D(s + i) = a.D(i - 1); }
  for (int i = 1; i <= b; ++i) a.CB(s + i) = a.CB(s + (i - 1)) + a.D(s + i);
  for (int i = 1; i <= b; ++i) a.CC(s + i) = a.CC(s + (i - 1)) + (a.D(s + (i - 1)) + a.D(s + i)) / R(2);
}

// WENO coefficients, m_weno.fpp:168-363 (the coefficient of cell i+1 is
// computed from cell boundaries s_cb(i-2..i+3)).
template <class R>
void compute_weno_coefficients(Axis<R>& a, int weno_order) {
  const int polyn = (weno_order - 1) / 2;
  const int b = a.b, s = a.s;
  a.wb = -b + polyn;
  const int we = s + b - polyn;
  a.coef.assign((size_t)std::max(0, we - a.wb + 1), typename Axis<R>::Coef{});
  if (weno_order == 1) return;
  auto sq = [](R x) { return x * x; };
  for (int i = a.wb - 1; i <= we - 1; ++i) {
    auto& c = a.C(i + 1);
    auto S = [&](int k) { return a.CB(k); };
    if (weno_order == 3) {
      c.polyR[0][0] = (S(i) - S(i + 1)) / (S(i) - S(i + 2));
      c.polyR[1][0] = (S(i) - S(i + 1)) / (S(i - 1) - S(i + 1));
      c.polyL[0][0] = -c.polyR[0][0];
      c.polyL[1][0] = -c.polyR[1][0];
      c.dR[0] = (S(i - 1) - S(i + 1)) / (S(i - 1) - S(i + 2));
      c.dL[0] = (S(i - 1) - S(i)) / (S(i - 1) - S(i + 2));
      c.dR[1] = R(1) - c.dR[0];
      c.dL[1] = R(1) - c.dL[0];
      c.beta[0][0] = R(4) * sq(S(i) - S(i + 1)) / sq(S(i) - S(i + 2));
      c.beta[1][0] = R(4) * sq(S(i) - S(i + 1)) / sq(S(i - 1) - S(i + 1));
      continue;
    }
    c.polyR[0][0] = ((S(i) - S(i + 1)) * (S(i + 1) - S(i + 2))) / ((S(i) - S(i + 3)) * (S(i + 3) - S(i + 1)));
    c.polyR[1][0] = ((S(i - 1) - S(i + 1)) * (S(i + 1) - S(i))) / ((S(i - 1) - S(i + 2)) * (S(i + 2) - S(i)));
    c.polyR[1][1] = ((S(i) - S(i + 1)) * (S(i + 1) - S(i + 2))) / ((S(i - 1) - S(i + 1)) * (S(i - 1) - S(i + 2)));
    c.polyR[2][1] = ((S(i) - S(i + 1)) * (S(i + 1) - S(i - 1))) / ((S(i - 2) - S(i)) * (S(i - 2) - S(i + 1)));
    c.polyL[0][0] = ((S(i + 1) - S(i)) * (S(i) - S(i + 2))) / ((S(i) - S(i + 3)) * (S(i + 3) - S(i + 1)));
    c.polyL[1][0] = ((S(i) - S(i - 1)) * (S(i) - S(i + 1))) / ((S(i - 1) - S(i + 2)) * (S(i) - S(i + 2)));
    c.polyL[1][1] = ((S(i + 1) - S(i)) * (S(i) - S(i + 2))) / ((S(i - 1) - S(i + 1)) * (S(i - 1) - S(i + 2)));
    c.polyL[2][1] = ((S(i - 1) - S(i)) * (S(i) - S(i + 1))) / ((S(i - 2) - S(i)) * (S(i - 2) - S(i + 1)));
    c.polyR[0][1] = ((S(i) - S(i + 2)) + (S(i + 1) - S(i + 3))) / ((S(i) - S(i + 2)) * (S(i) - S(i + 3))) *
                    ((S(i) - S(i + 1)));
    c.polyR[2][0] = ((S(i - 2) - S(i + 1)) + (S(i - 1) - S(i + 1))) /
                    ((S(i - 1) - S(i + 1)) * (S(i + 1) - S(i - 2))) * ((S(i + 1) - S(i)));
    c.polyL[0][1] = ((S(i) - S(i + 2)) + (S(i) - S(i + 3))) / ((S(i) - S(i + 2)) * (S(i) - S(i + 3))) *
                    ((S(i + 1) - S(i)));
    c.polyL[2][0] = ((S(i - 2) - S(i)) + (S(i - 1) - S(i + 1))) /
                    ((S(i - 2) - S(i + 1)) * (S(i + 1) - S(i - 1))) * ((S(i) - S(i + 1)));
    c.dR[0] = ((S(i - 2) - S(i + 1)) * (S(i + 1) - S(i - 1))) / ((S(i - 2) - S(i + 3)) * (S(i + 3) - S(i - 1)));
    c.dR[2] = ((S(i + 1) - S(i + 2)) * (S(i + 1) - S(i + 3))) / ((S(i - 2) - S(i + 2)) * (S(i - 2) - S(i + 3)));
    c.dL[0] = ((S(i - 2) - S(i)) * (S(i) - S(i - 1))) / ((S(i - 2) - S(i + 3)) * (S(i + 3) - S(i - 1)));
    c.dL[2] = ((S(i) - S(i + 2)) * (S(i) - S(i + 3))) / ((S(i - 2) - S(i + 2)) * (S(i - 2) - S(i + 3)));
    c.dR[1] = R(1) - c.dR[0] - c.dR[2];
    c.dL[1] = R(1) - c.dL[0] - c.dL[2];
    c.beta[0][0] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(10) * sq(S(i + 1) - S(i)) + (S(i + 1) - S(i)) * (S(i + 2) - S(i + 1)) + sq(S(i + 2) - S(i + 1))) /
                   (sq(S(i) - S(i + 3)) * sq(S(i + 1) - S(i + 3)));
    c.beta[0][1] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(19) * sq(S(i + 1) - S(i)) - (S(i + 1) - S(i)) * (S(i + 3) - S(i + 1)) +
                    R(2) * (S(i + 2) - S(i)) * ((S(i + 2) - S(i)) + (S(i + 3) - S(i + 1)))) /
                   ((S(i) - S(i + 2)) * sq(S(i) - S(i + 3)) * (S(i + 3) - S(i + 1)));
    c.beta[0][2] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(10) * sq(S(i + 1) - S(i)) + (S(i + 1) - S(i)) * ((S(i + 2) - S(i)) + (S(i + 3) - S(i + 1))) +
                    sq((S(i + 2) - S(i)) + (S(i + 3) - S(i + 1)))) /
                   (sq(S(i) - S(i + 2)) * sq(S(i) - S(i + 3)));
    c.beta[1][0] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(10) * sq(S(i + 1) - S(i)) + sq(S(i) - S(i - 1)) + (S(i) - S(i - 1)) * (S(i + 1) - S(i))) /
                   (sq(S(i - 1) - S(i + 2)) * sq(S(i) - S(i + 2)));
    c.beta[1][1] = R(4) * sq(S(i) - S(i + 1)) *
                   ((S(i) - S(i + 1)) * ((S(i) - S(i - 1)) + R(20) * (S(i + 1) - S(i))) +
                    (R(2) * (S(i) - S(i - 1)) + (S(i + 1) - S(i))) * (S(i + 2) - S(i))) /
                   ((S(i + 1) - S(i - 1)) * sq(S(i - 1) - S(i + 2)) * (S(i + 2) - S(i)));
    c.beta[1][2] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(10) * sq(S(i + 1) - S(i)) + (S(i + 1) - S(i)) * (S(i + 2) - S(i + 1)) + sq(S(i + 2) - S(i + 1))) /
                   (sq(S(i - 1) - S(i + 1)) * sq(S(i - 1) - S(i + 2)));
    c.beta[2][0] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(12) * sq(S(i + 1) - S(i)) + sq((S(i) - S(i - 2)) + (S(i) - S(i - 1))) +
                    R(3) * ((S(i) - S(i - 2)) + (S(i) - S(i - 1))) * (S(i + 1) - S(i))) /
                   (sq(S(i - 2) - S(i + 1)) * sq(S(i - 1) - S(i + 1)));
    c.beta[2][1] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(19) * sq(S(i + 1) - S(i)) + ((S(i) - S(i - 2)) * (S(i) - S(i + 1))) +
                    R(2) * (S(i + 1) - S(i - 1)) * ((S(i) - S(i - 2)) + (S(i + 1) - S(i - 1)))) /
                   ((S(i - 2) - S(i)) * sq(S(i - 2) - S(i + 1)) * (S(i + 1) - S(i - 1)));
    c.beta[2][2] = R(4) * sq(S(i) - S(i + 1)) *
                   (R(10) * sq(S(i + 1) - S(i)) + sq(S(i) - S(i - 1)) + (S(i) - S(i - 1)) * (S(i + 1) - S(i))) /
                   (sq(S(i - 2) - S(i)) * sq(S(i - 2) - S(i + 1)));
  }
}

// ---------------------------------------------------------------------------
template <class R>
struct Solver {
  Params P;
  int b = 0, S = 0, nd = 1;
  int xb, xe, yb, ye, zb, ze;     // full index ranges incl. ghosts
  Axis<R> ax[3];
  std::vector<Field<R>> q_cons_ts[2];  // RK registers (q_cons_ts(1:2))
  std::vector<Field<R>> qp;            // q_cons_qp / q_prim_qp (prim overwrites in place)
  std::vector<Field<R>> rhs;           // rhs_vf(0:m,0:n,0:p)
  std::vector<Field<R>> vL, vR;        // WENO face values, one direction at a time
  std::vector<Field<R>> flux;          // flux at face j+1/2 stored at j
  Field<R> fsrc;                       // interface velocity at face j+1/2
  Field<R> vflux[3];                   // viscous source flux at face j+1/2: x-momentum, y-momentum, energy
  // weno_Re_flux: grad[c][d] = cell-average d u_c / d x_d by the divergence
  // theorem from WENO face values of u_c along d; gL/gR[c][d] = its left-
  // and right-face WENO values along the current sweep direction
  Field<R> grad[2][2], gL[2][2], gR[2][2];
  double dt = 0;

  void init(const Params& p, const double* x_cb, const double* y_cb, const double* z_cb) {
    P = p;
    b = P.buff_size();
    S = P.sys_size();
    nd = P.num_dims();
    xb = -b; xe = P.m + b;
    yb = P.n > 0 ? -b : 0; ye = P.n > 0 ? P.n + b : 0;
    zb = P.p > 0 ? -b : 0; ze = P.p > 0 ? P.p + b : 0;
    const double* cbs[3] = {x_cb, y_cb, z_cb};
    const int ss[3] = {P.m, P.n, P.p};
    const int bcb[3] = {P.bc_x_beg, P.bc_y_beg, P.bc_z_beg};
    const int bce[3] = {P.bc_x_end, P.bc_y_end, P.bc_z_end};
    for (int d = 0; d < nd; ++d) {
      Axis<R>& a = ax[d];
      a.s = ss[d]; a.b = b;
      a.cb.assign((size_t)(a.s + 2 * b + 2), R(0));
      a.d.assign((size_t)(a.s + 2 * b + 1), R(0));
      a.cc.assign((size_t)(a.s + 2 * b + 1), R(0));
      for (int i = -1; i <= a.s; ++i) a.CB(i) = R(cbs[d][i + 1]);
      populate_grid_buffers(a, bcb[d], bce[d]);
      compute_weno_coefficients(a, P.weno_order);
    }
    for (int r = 0; r < 2; ++r) {
      q_cons_ts[r].resize((size_t)S);
      for (auto& f : q_cons_ts[r]) f.alloc(xb, xe, yb, ye, zb, ze);
    }
    qp.resize((size_t)S);
    vL.resize((size_t)S); vR.resize((size_t)S); flux.resize((size_t)S);
    rhs.resize((size_t)S);
    for (int v = 0; v < S; ++v) {
      qp[v].alloc(xb, xe, yb, ye, zb, ze);
      vL[v].alloc(xb, xe, yb, ye, zb, ze);
      vR[v].alloc(xb, xe, yb, ye, zb, ze);
      flux[v].alloc(xb, xe, yb, ye, zb, ze);
      rhs[v].alloc(0, P.m, 0, P.n, 0, P.p);
    }
    fsrc.alloc(xb, xe, yb, ye, zb, ze);
    if (P.viscous())
      for (auto& f : vflux) f.alloc(xb, xe, yb, ye, zb, ze);
    if (P.viscous() && P.weno_re_flux)
      for (int c = 0; c < nd; ++c)
        for (int d = 0; d < nd; ++d) {
          grad[c][d].alloc(xb, xe, yb, ye, zb, ze);
          gL[c][d].alloc(xb, xe, yb, ye, zb, ze);
          gR[c][d].alloc(xb, xe, yb, ye, zb, ze);
        }
  }

  // Velocity component c of a cell (primitive, after cons_to_prim).
  R U(int c, int i, int j) const { return qp[P.mom_beg() - 1 + c](i, j, 0); }
  // The one-sided velocity gradients of s_get_viscous (m_viscous.fpp:212-264,
  // weno_Re_flux = F): dqL_prim_dx_n(1) = L, dqR_prim_dx_n(1) = R.
  R Lx(int c, int i, int j) { return (U(c, i, j) - U(c, i - 1, j)) / (ax[0].CC(i) - ax[0].CC(i - 1)); }
  R Rx(int c, int i, int j) { return (U(c, i + 1, j) - U(c, i, j)) / (ax[0].CC(i + 1) - ax[0].CC(i)); }
  R Ly(int c, int i, int j) { return (U(c, i, j) - U(c, i, j - 1)) / (ax[1].CC(j) - ax[1].CC(j - 1)); }
  R Ry(int c, int i, int j) { return (U(c, i, j + 1) - U(c, i, j)) / (ax[1].CC(j + 1) - ax[1].CC(j)); }

  // weno_Re_flux = T, m_viscous.fpp:176-216 (s_reconstruct_cell_boundary_
  // values_visc, s_apply_scalar_divergence_theorem :381-455): the velocity
  // components WENO-reconstructed along each direction d over the WENO
  // window of d (the whole extended range across it), then the cell-average
  // gradient (1/ds) (vR - vL) on the extended range less one cell each side
  // (cells whose face values lie outside the window keep the zeros of the
  // allocation; no face flux reads them).
  void visc_gradients() {
    const int polyn = P.weno_polyn();
    const R eps = R(P.weno_eps);
    for (int d = 0; d < nd; ++d) {
      Axis<R>& a = ax[d];
      const int di = d == 0, dj = d == 1;
      int ib_ = xb, ie_ = xe, jb_ = yb, je_ = ye;
      if (d == 0) { ib_ = -b + polyn; ie_ = a.s + b - polyn; }
      else { jb_ = -b + polyn; je_ = a.s + b - polyn; }
      for (int c = 0; c < nd; ++c) {
        const Field<R>& u = qp[P.mom_beg() - 1 + c];
        Field<R>& uL = gL[c][d];  // scratch: the velocity's face values
        Field<R>& uR = gR[c][d];
        for (int j = jb_; j <= je_; ++j)
          for (int i = ib_; i <= ie_; ++i) {
            auto at = [&](int o) { return u(i + o * di, j + o * dj, 0); };
            weno_stencil(at, a.C(d == 0 ? i : j), eps, uL(i, j, 0), uR(i, j, 0));
          }
        int gib = xb, gie = xe, gjb = yb, gje = ye;
        if (d == 0) { gib = xb + 1; gie = xe - 1; }
        else { gjb = yb + 1; gje = ye - 1; }
        for (int j = gjb; j <= gje; ++j)
          for (int i = gib; i <= gie; ++i)
            grad[c][d](i, j, 0) = R(1) / a.D(d == 0 ? i : j) * (uR(i, j, 0) - uL(i, j, 0));
      }
    }
  }

  // weno_Re_flux = T, m_rhs.fpp:512-528 (s_reconstruct_cell_boundary_values_
  // visc_deriv, m_viscous.fpp:525-591): every gradient WENO-reconstructed
  // along the sweep direction over its WENO window.
  void visc_gradient_weno(int dir) {
    const int polyn = P.weno_polyn();
    const R eps = R(P.weno_eps);
    Axis<R>& a = ax[dir];
    const int di = dir == 0, dj = dir == 1;
    int ib_ = xb, ie_ = xe, jb_ = yb, je_ = ye;
    if (dir == 0) { ib_ = -b + polyn; ie_ = a.s + b - polyn; }
    else { jb_ = -b + polyn; je_ = a.s + b - polyn; }
    for (int c = 0; c < nd; ++c)
      for (int d = 0; d < nd; ++d) {
        const Field<R>& g = grad[c][d];
        for (int j = jb_; j <= je_; ++j)
          for (int i = ib_; i <= ie_; ++i) {
            auto at = [&](int o) { return g(i + o * di, j + o * dj, 0); };
            weno_stencil(at, a.C(dir == 0 ? i : j), eps, gL[c][d](i, j, 0), gR[c][d](i, j, 0));
          }
      }
  }

  // Viscous source flux of the face between (i,j) and its neighbour along dir,
  // s_compute_viscous_source_flux (m_riemann_solvers.fpp:683-902), with the
  // face gradients of s_get_viscous (m_viscous.fpp:159-370): the arithmetic
  // means of the left and right face values, which are the same numbers, and
  // the cross derivatives averaged over four one-sided gradients
  // (m_viscous.fpp:266-332).  re_avg: Re_avg(1:2); vs: vel_src(1:2).
  void viscous_flux(int dir, int i, int j, const R (&re_avg)[2], const R (&vs)[3], R (&out)[3]) {
    R dx[2] = {R(0), R(0)}, dy[2] = {R(0), R(0)};
    const int ndv = nd;
    if (P.weno_re_flux) {
      // the arithmetic mean of the right-face value of this cell and the
      // left-face value of the next (m_riemann_solvers.fpp:714-900)
      const int ni = i + (dir == 0), nj = j + (dir == 1);
      for (int c = 0; c < ndv; ++c) {
        dx[c] = R(0.5) * (gR[c][0](i, j, 0) + gL[c][0](ni, nj, 0));
        if (nd > 1) dy[c] = R(0.5) * (gR[c][1](i, j, 0) + gL[c][1](ni, nj, 0));
      }
    } else if (dir == 0) {
      for (int c = 0; c < ndv; ++c) dx[c] = R(0.5) * (Rx(c, i, j) + Lx(c, i + 1, j));
      if (nd > 1)
        for (int c = 0; c < ndv; ++c) {
          const R A = R(0.25) * (Ly(c, i + 1, j) + Ry(c, i + 1, j) + Ly(c, i, j) + Ry(c, i, j));
          dy[c] = R(0.5) * (A + A);
        }
    } else {
      for (int c = 0; c < ndv; ++c) {
        const R A = R(0.25) * (Lx(c, i, j + 1) + Rx(c, i, j + 1) + Lx(c, i, j) + Rx(c, i, j));
        dx[c] = R(0.5) * (A + A);
        dy[c] = R(0.5) * (Ry(c, i, j) + Ly(c, i, j + 1));
      }
    }
    R fm[2] = {R(0), R(0)}, fe = R(0);
    const bool shear = P.re_size(0) > 0, bulk = P.re_size(1) > 0;
    if (dir == 0) {
      if (shear) {
        const R tau = R(4.0 / 3.0) * dx[0] / re_avg[0];
        fm[0] = fm[0] - tau;
        fe = fe - vs[0] * tau;
      }
      if (bulk) {
        const R tau = dx[0] / re_avg[1];
        fm[0] = fm[0] - tau;
        fe = fe - vs[0] * tau;
      }
      if (nd > 1) {
        if (shear) {
          const R t[2] = {-(R(2.0 / 3.0) * dy[1] / re_avg[0]), (dy[0] + dx[1]) / re_avg[0]};
          for (int c = 0; c < 2; ++c) {
            fm[c] = fm[c] - t[c];
            fe = fe - vs[c] * t[c];
          }
        }
        if (bulk) {
          const R tau = dy[1] / re_avg[1];
          fm[0] = fm[0] - tau;
          fe = fe - vs[0] * tau;
        }
      }
    } else {
      if (shear) {
        const R t[2] = {(dy[0] + dx[1]) / re_avg[0], (R(4) * dy[1] - R(2) * dx[0]) / (R(3) * re_avg[0])};
        for (int c = 0; c < 2; ++c) {
          fm[c] = fm[c] - t[c];
          fe = fe - vs[c] * t[c];
        }
      }
      if (bulk) {
        const R tau = (dx[0] + dy[1]) / re_avg[1];
        fm[1] = fm[1] - tau;
        fe = fe - vs[1] * tau;
      }
    }
    out[0] = fm[0];
    out[1] = fm[1];
    out[2] = fe;
  }

  // Ghost-cell fill of q_cons_qp, m_rhs.fpp:686-908, extended to z.
  // dir: 0,1,2; interior ranges of the other directions follow the
  // reference: x ghosts over interior y, y ghosts over the full x range.
  void populate_buffers() {
    const int m = P.m, n = P.n, pp = P.p;
    const int momx = P.mom_beg() - 1;  // 0-based index of x-momentum
    auto fill = [&](int dir, int bc, bool at_end) {
      const int s = dir == 0 ? m : dir == 1 ? n : pp;
      const int mom = momx + dir;
      // loop ranges of the two other directions
      int r0b, r0e, r1b, r1e;
      if (dir == 0) { r0b = 0; r0e = n; r1b = 0; r1e = pp; }
      else if (dir == 1) { r0b = -b; r0e = m + b; r1b = 0; r1e = pp; }
      else { r0b = -b; r0e = m + b; r1b = yb; r1e = ye; }
      for (int v = 0; v < S; ++v)
        for (int t1 = r1b; t1 <= r1e; ++t1)
          for (int t0 = r0b; t0 <= r0e; ++t0)
            for (int j = 1; j <= b; ++j) {
              int dst = at_end ? s + j : -j, src;
              R sign = R(1);
              if (bc <= -3) src = at_end ? s : 0;
              else if (bc == -2) { src = at_end ? s - (j - 1) : j - 1; if (v == mom) sign = R(-1); }
              else src = at_end ? j - 1 : s - (j - 1);  // periodic
              R val;
              if (dir == 0) val = qp[v](src, t0, t1);
              else if (dir == 1) val = qp[v](t0, src, t1);
              else val = qp[v](t0, t1, src);
              if (sign < R(0)) val = -val;
              if (dir == 0) qp[v](dst, t0, t1) = val;
              else if (dir == 1) qp[v](t0, dst, t1) = val;
              else qp[v](t0, t1, dst) = val;
            }
    };
    fill(0, P.bc_x_beg, false); fill(0, P.bc_x_end, true);
    if (n == 0) return;
    fill(1, P.bc_y_beg, false); fill(1, P.bc_y_end, true);
    if (pp == 0) return;
    fill(2, P.bc_z_beg, false); fill(2, P.bc_z_end, true);
  }

  // m_variables_conversion.fpp:313-375 (simulation branch), over all cells
  // incl. ghosts.  Partial densities and volume fractions are aliased, so
  // only momentum -> velocity and energy -> pressure change.
  void cons_to_prim() {
    const int nf = P.num_fluids, mb = P.mom_beg() - 1, E = P.E_idx() - 1, ab = P.adv_beg() - 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = zb; k <= ze; ++k)
      for (int j = yb; j <= ye; ++j)
        for (int i = xb; i <= xe; ++i) {
          R rho = R(0), gam = R(0), pinf = R(0), dyn = R(0);
          for (int f = 0; f < nf; ++f) {
            rho = rho + qp[f](i, j, k);
            gam = gam + qp[ab + f](i, j, k) * R(P.gammas[f]);
            pinf = pinf + qp[ab + f](i, j, k) * R(P.pi_infs[f]);
          }
          rho = std::max(rho, R(kSgmEps));
          for (int d = 0; d < nd; ++d) {
            R mom = qp[mb + d](i, j, k);
            R vel = mom / rho;
            qp[mb + d](i, j, k) = vel;
            dyn = dyn + R(0.5) * mom * vel;
          }
          qp[E](i, j, k) = (qp[E](i, j, k) - dyn - pinf) / gam;
        }
  }

  // WENO1/3/5 of one stencil, m_weno.fpp:391-536: at(o) is the value at
  // offset o from the cell, cf the cell's coefficients; the left-face
  // (x_{j-1/2}) and right-face (x_{j+1/2}) values.
  template <class At, class Coef>
  void weno_stencil(const At& at, const Coef& cf, R eps, R& outL, R& outR) const {
    if (P.weno_order == 1) {
      outL = at(0);
      outR = at(0);
      return;
    }
    if (P.weno_order == 3) {
      R dvd0 = at(1) - at(0);
      R dvdm1 = at(0) - at(-1);
      R poly0 = at(0) + cf.polyL[0][0] * dvd0;
      R poly1 = at(0) + cf.polyL[1][0] * dvdm1;
      R beta0 = cf.beta[0][0] * dvd0 * dvd0 + eps;
      R beta1 = cf.beta[1][0] * dvdm1 * dvdm1 + eps;
      R a0 = cf.dL[0] / (beta0 * beta0), a1 = cf.dL[1] / (beta1 * beta1);
      R sa = a0 + a1;
      R w0 = a0 / sa, w1 = a1 / sa;
      outL = w0 * poly0 + w1 * poly1;
      poly0 = at(0) + cf.polyR[0][0] * dvd0;
      poly1 = at(0) + cf.polyR[1][0] * dvdm1;
      a0 = cf.dR[0] / (beta0 * beta0); a1 = cf.dR[1] / (beta1 * beta1);
      sa = a0 + a1;
      w0 = a0 / sa; w1 = a1 / sa;
      outR = w0 * poly0 + w1 * poly1;
      return;
    }
    R dvd1 = at(2) - at(1);
    R dvd0 = at(1) - at(0);
    R dvdm1 = at(0) - at(-1);
    R dvdm2 = at(-1) - at(-2);
    R poly[3], beta[3], alpha[3], omega[3];
    poly[0] = at(0) + cf.polyL[0][0] * dvd1 + cf.polyL[0][1] * dvd0;
    poly[1] = at(0) + cf.polyL[1][0] * dvd0 + cf.polyL[1][1] * dvdm1;
    poly[2] = at(0) + cf.polyL[2][0] * dvdm1 + cf.polyL[2][1] * dvdm2;
    beta[0] = cf.beta[0][0] * dvd1 * dvd1 + cf.beta[0][1] * dvd1 * dvd0 + cf.beta[0][2] * dvd0 * dvd0 + eps;
    beta[1] = cf.beta[1][0] * dvd0 * dvd0 + cf.beta[1][1] * dvd0 * dvdm1 + cf.beta[1][2] * dvdm1 * dvdm1 + eps;
    beta[2] = cf.beta[2][0] * dvdm1 * dvdm1 + cf.beta[2][1] * dvdm1 * dvdm2 + cf.beta[2][2] * dvdm2 * dvdm2 + eps;
    for (int l = 0; l < 3; ++l) alpha[l] = cf.dL[l] / (beta[l] * beta[l]);
    R sa = alpha[0] + alpha[1] + alpha[2];
    for (int l = 0; l < 3; ++l) omega[l] = alpha[l] / sa;
    outL = omega[0] * poly[0] + omega[1] * poly[1] + omega[2] * poly[2];
    poly[0] = at(0) + cf.polyR[0][0] * dvd1 + cf.polyR[0][1] * dvd0;
    poly[1] = at(0) + cf.polyR[1][0] * dvd0 + cf.polyR[1][1] * dvdm1;
    poly[2] = at(0) + cf.polyR[2][0] * dvdm1 + cf.polyR[2][1] * dvdm2;
    for (int l = 0; l < 3; ++l) alpha[l] = cf.dR[l] / (beta[l] * beta[l]);
    sa = alpha[0] + alpha[1] + alpha[2];
    for (int l = 0; l < 3; ++l) omega[l] = alpha[l] / sa;
    outR = omega[0] * poly[0] + omega[1] * poly[1] + omega[2] * poly[2];
  }

  // WENO reconstruction along direction dir, m_weno.fpp:391-536.
  // is1 = [-b+polyn, s+b-polyn] along dir; all other directions over their
  // full range (incl. ghosts), as in s_reconstruct_cell_boundary_values.
  //
  // P.char_decomp (no counterpart in the reference, which reconstructs the
  // primitive variables only): the stencil of cell j is first projected on
  // the characteristic fields of the quasi-linear primitive system along dir,
  // frozen at cell j's own state,
  //   slot f (partial density i):   alpha_i rho_i - kappa_i p,  kappa_i = alpha_i rho_i / (rho c^2)
  //   slot momx + dir:              p - rho c u_n   (the u_n - c wave)
  //   slot E:                       p + rho c u_n   (the u_n + c wave)
  //   tangential velocities, volume fractions: unchanged,
  // with rho = max(sum alpha_i rho_i, sgm_eps), Gamma = sum alpha_i Gamma_i,
  // Pi = sum alpha_i Pi_i and c^2 = max(((Gamma + 1) p + Pi) / (Gamma rho),
  // sgm_eps) (the mixture sound speed of m_riemann_solvers.fpp:220-223);
  // each field is reconstructed with the same weights, then both face values
  // are mapped back: p = (w_+ + w_-) 0.5, u_n = (w_+ - w_-) / (2 rho c),
  // alpha_i rho_i = w_i + kappa_i p.  WENO1 reconstructs nothing, so it
  // keeps the primitive path.
  void weno(int dir) {
    const int polyn = P.weno_polyn();
    Axis<R>& a = ax[dir];
    const int jb = -b + polyn, je = a.s + b - polyn;
    const R eps = R(P.weno_eps);
    const int di = dir == 0, dj = dir == 1, dk = dir == 2;
    // iteration box
    int ib_ = xb, ie_ = xe, jb_ = yb, je_ = ye, kb_ = zb, ke_ = ze;
    if (dir == 0) { ib_ = jb; ie_ = je; }
    if (dir == 1) { jb_ = jb; je_ = je; }
    if (dir == 2) { kb_ = jb; ke_ = je; }
    const bool chr = P.char_decomp && P.weno_order > 1;
    const int nf = P.num_fluids, un = P.mom_beg() - 1 + dir, E = P.E_idx() - 1, ab = P.adv_beg() - 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = kb_; k <= ke_; ++k)
      for (int j = jb_; j <= je_; ++j)
        for (int i = ib_; i <= ie_; ++i) {
          const int c = dir == 0 ? i : dir == 1 ? j : k;
          const auto& cf = a.C(c);
          if (!chr) {
            for (int v = 0; v < S; ++v) {
              const Field<R>& q = qp[v];
              auto at = [&](int o) { return q(i + o * di, j + o * dj, k + o * dk); };
              weno_stencil(at, cf, eps, vL[v](i, j, k), vR[v](i, j, k));
            }
            continue;
          }
          R rho = R(0), gam = R(0), pinf = R(0), kap[kMaxFluids];
          for (int f = 0; f < nf; ++f) {
            rho = rho + qp[f](i, j, k);
            gam = gam + qp[ab + f](i, j, k) * R(P.gammas[f]);
            pinf = pinf + qp[ab + f](i, j, k) * R(P.pi_infs[f]);
          }
          rho = std::max(rho, R(kSgmEps));
          const R c2 = std::max(((gam + R(1)) * qp[E](i, j, k) + pinf) / (gam * rho), R(kSgmEps));
          const R rc = rho * sqrt(c2);
          for (int f = 0; f < nf; ++f) kap[f] = qp[f](i, j, k) / (rho * c2);
          for (int v = 0; v < S; ++v) {
            auto at = [&](int o) {
              const int ii = i + o * di, jj = j + o * dj, kk = k + o * dk;
              if (v < nf) return qp[v](ii, jj, kk) - kap[v] * qp[E](ii, jj, kk);
              if (v == un) return qp[E](ii, jj, kk) - rc * qp[un](ii, jj, kk);
              if (v == E) return qp[E](ii, jj, kk) + rc * qp[un](ii, jj, kk);
              return qp[v](ii, jj, kk);
            };
            weno_stencil(at, cf, eps, vL[v](i, j, k), vR[v](i, j, k));
          }
          for (auto* w : {&vL, &vR}) {
            std::vector<Field<R>>& o = *w;
            const R wm = o[un](i, j, k), wp = o[E](i, j, k);
            const R pr = (wp + wm) * R(0.5);
            o[E](i, j, k) = pr;
            o[un](i, j, k) = (wp - wm) / (R(2) * rc);
            for (int f = 0; f < nf; ++f) o[f](i, j, k) = o[f](i, j, k) + kap[f] * pr;
          }
        }
  }

  // HLLC across faces j+1/2 of direction dir, m_riemann_solvers.fpp:132-327.
  // The caller's argument swap (m_rhs.fpp:545-556) is resolved here: the left
  // state of face j+1/2 is vR(j), the right state is vL(j+1).  Riemann-state
  // extrapolation (bc -4, m_riemann_solvers.fpp:480-615) is applied on the fly.
  void hllc(int dir) {
    const int nf = P.num_fluids, cxe = P.cont_end(), E = P.E_idx() - 1, ab = P.adv_beg() - 1;
    const int di = dir == 0, dj = dir == 1, dk = dir == 2;
    // dir_idx(1) is the sweep direction; dir_flg selects the normal
    // momentum component.  The loop order over the other components does not
    // change any value, so all components are visited in index order.
    const int idx1 = dir;
    const int s = ax[dir].s;
    const int bcb = dir == 0 ? P.bc_x_beg : dir == 1 ? P.bc_y_beg : P.bc_z_beg;
    const int bce = dir == 0 ? P.bc_x_end : dir == 1 ? P.bc_y_end : P.bc_z_end;
    int ib_ = 0, ie_ = P.m, jb_ = 0, je_ = P.n, kb_ = 0, ke_ = P.p;
    if (dir == 0) ib_ = -1;
    if (dir == 1) jb_ = -1;
    if (dir == 2) kb_ = -1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = kb_; k <= ke_; ++k)
      for (int j = jb_; j <= je_; ++j)
        for (int i = ib_; i <= ie_; ++i) {
          const int c = dir == 0 ? i : dir == 1 ? j : k;
          // L = vR at (i,j,k), R = vL at the next cell
          int li = i, lj = j, lk = k;
          int ri = i + di, rj = j + dj, rk = k + dk;
          bool useL_fromR = (c == -1 && bcb == -4);   // qL(-1) = qR(0)
          bool useR_fromL = (c == s && bce == -4);    // qR(s+1) = qL(s)
          auto QL = [&](int v) { return useL_fromR ? vL[v](ri, rj, rk) : vR[v](li, lj, lk); };
          auto QR = [&](int v) { return useR_fromL ? vR[v](li, lj, lk) : vL[v](ri, rj, rk); };
          R velL[3], velR[3];
          R vel_L_rms = R(0), vel_R_rms = R(0);
          for (int d = 0; d < nd; ++d) {
            velL[d] = QL(cxe + d);
            velR[d] = QR(cxe + d);
            vel_L_rms = vel_L_rms + velL[d] * velL[d];
            vel_R_rms = vel_R_rms + velR[d] * velR[d];
          }
          R pL = QL(E), pR = QR(E);
          R rhoL = R(0), gamL = R(0), piL = R(0), rhoR = R(0), gamR = R(0), piR = R(0);
          for (int f = 0; f < nf; ++f) {
            rhoL = rhoL + QL(f);
            gamL = gamL + QL(ab + f) * R(P.gammas[f]);
            piL = piL + QL(ab + f) * R(P.pi_infs[f]);
            rhoR = rhoR + QR(f);
            gamR = gamR + QR(ab + f) * R(P.gammas[f]);
            piR = piR + QR(ab + f) * R(P.pi_infs[f]);
          }
          R EL = gamL * pL + piL + R(0.5) * rhoL * vel_L_rms;
          R ER = gamR * pR + piR + R(0.5) * rhoR * vel_R_rms;
          R HL = (EL + pL) / rhoL;
          R HR = (ER + pR) / rhoR;
          R cL = (HL - R(0.5) * vel_L_rms) / gamL;
          R cR = (HR - R(0.5) * vel_R_rms) / gamR;
          cL = sqrt(cL);
          cR = sqrt(cR);
          R uL = velL[idx1], uR = velR[idx1];
          R sL = std::min(uL - cL, uR - cR);
          R sR = std::max(uR + cR, uL + cL);
          R sS = (pR - pL + rhoL * uL * (sL - uL) - rhoR * uR * (sR - uR)) / (rhoL * (sL - uL) - rhoR * (sR - uR));
          R sM = std::min(R(0), sL), sP = std::max(R(0), sR);
          R xiL = (sL - uL) / (sL - sS);
          R xiR = (sR - uR) / (sR - sS);
          R xiM = R(0.5) + copysign(R(0.5), sS);
          R xiP = R(0.5) - copysign(R(0.5), sS);
          for (int f = 0; f < cxe; ++f)
            flux[f](i, j, k) = xiM * QL(f) * (uL + sM * (xiL - R(1))) + xiP * QR(f) * (uR + sP * (xiR - R(1)));
          for (int id = 0; id < nd; ++id) {
            const R flg = id == dir ? R(1) : R(0);
            flux[cxe + id](i, j, k) =
                xiM * (rhoL * (uL * velL[id] + sM * (xiL * (flg * sS + (R(1) - flg) * velL[id]) - velL[id])) + flg * pL) +
                xiP * (rhoR * (uR * velR[id] + sP * (xiR * (flg * sS + (R(1) - flg) * velR[id]) - velR[id])) + flg * pR);
          }
          flux[E](i, j, k) = xiM * (uL * (EL + pL) + sM * (xiL * (EL + (sS - uL) * (rhoL * sS + pL / (sL - uL))) - EL)) +
                             xiP * (uR * (ER + pR) + sP * (xiR * (ER + (sS - uR) * (rhoR * sS + pR / (sR - uR))) - ER));
          for (int f = 0; f < nf; ++f)
            flux[ab + f](i, j, k) = xiM * QL(ab + f) * (uL + sM * (xiL - R(1))) + xiP * QR(ab + f) * (uR + sP * (xiR - R(1)));
          // vel_src(idx1) -> flux_src(advxb)
          fsrc(i, j, k) = xiM * (uL + R(1) * sM * (xiL - R(1))) + xiP * (uR + R(1) * sP * (xiR - R(1)));
          if (P.viscous()) {
            // Re_L/Re_R (m_riemann_solvers.fpp:169-199), Re_avg (:225-230),
            // vel_src of every component (:314-324)
            R re_avg[2], vs[3] = {R(0), R(0), R(0)}, vf[3];
            for (int r = 0; r < 2; ++r) {
              R reL = R(-1e6), reR = R(-1e6);
              if (P.re_size(r) > 0) reL = reR = R(0);
              for (int q = 0; q < P.re_size(r); ++q) {
                const int f = P.re_idx(r, q);
                reL = QL(ab + f) / R(P.re[r][f]) + reL;
                reR = QR(ab + f) / R(P.re[r][f]) + reR;
              }
              reL = R(1) / std::max(reL, R(kSgmEps));
              reR = R(1) / std::max(reR, R(kSgmEps));
              re_avg[r] = R(2) / (R(1) / reL + R(1) / reR);
            }
            for (int d = 0; d < nd; ++d) {
              const R flg = d == dir ? R(1) : R(0);
              vs[d] = xiM * (velL[d] + flg * sM * (xiL - R(1))) + xiP * (velR[d] + flg * sP * (xiR - R(1)));
            }
            viscous_flux(dir, i, j, re_avg, vs, vf);
            for (int t = 0; t < 3; ++t) vflux[t](i, j, k) = vf[t];
          }
        }
  }

  // Flux divergence and alpha*div(u), m_rhs.fpp:564-654.  The source term
  // reads the conservative volume fraction q_cons_qp, which is the same
  // memory as the primitive one (m_rhs.fpp:160-164) and never changed.
  void flux_add(int dir) {
    const int ab = P.adv_beg() - 1, nf = P.num_fluids;
    const int di = dir == 0, dj = dir == 1, dk = dir == 2;
    Axis<R>& a = ax[dir];
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k <= P.p; ++k)
      for (int j = 0; j <= P.n; ++j)
        for (int i = 0; i <= P.m; ++i) {
          const int c = dir == 0 ? i : dir == 1 ? j : k;
          const R inv = R(1) / a.D(c);
          for (int v = 0; v < S; ++v) {
            R df = flux[v](i - di, j - dj, k - dk) - flux[v](i, j, k);
            if (dir == 0) rhs[v](i, j, k) = inv * df;
            else rhs[v](i, j, k) = rhs[v](i, j, k) + inv * df;
          }
          for (int f = 0; f < nf; ++f)
            rhs[ab + f](i, j, k) =
                rhs[ab + f](i, j, k) + inv * qp[ab + f](i, j, k) * (fsrc(i, j, k) - fsrc(i - di, j - dj, k - dk));
          if (P.viscous()) {  // m_rhs.fpp:591-603, 639-651: momentum .. energy
            const int mb = P.mom_beg() - 1;
            for (int t = 0; t <= nd; ++t) {
              const int v = t < nd ? mb + t : P.E_idx() - 1;
              const Field<R>& F = vflux[t < nd ? t : 2];
              rhs[v](i, j, k) = rhs[v](i, j, k) + inv * (F(i - di, j - dj, k - dk) - F(i, j, k));
            }
          }
        }
  }

  // s_compute_rhs(q_cons_ts(reg)), m_rhs.fpp:405-679.  Returns false when the
  // early return at t_step == t_step_stop is taken (prim only).
  bool compute_rhs(int reg, bool last_step) {
    for (int v = 0; v < S; ++v) qp[v].d = q_cons_ts[reg][v].d;
    populate_buffers();
    cons_to_prim();
    if (last_step) return false;
    const bool wrf = P.viscous() && P.weno_re_flux;
    if (wrf) visc_gradients();
    for (int dir = 0; dir < nd; ++dir) {
      weno(dir);
      if (wrf) visc_gradient_weno(dir);
      hllc(dir);
      flux_add(dir);
    }
    return true;
  }

  // s_{1,2,3}_order_tvd_rk, m_time_steppers.fpp:129-362.
  void tvd_rk(bool last_step) {
    const R dtr = R(dt);
    auto upd = [&](auto fn) {
      for (int v = 0; v < S; ++v) {
        auto& q1 = q_cons_ts[0][v];
        auto& q2 = q_cons_ts[1][v];
        auto& r = rhs[v];
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 0; k <= P.p; ++k)
          for (int j = 0; j <= P.n; ++j)
            for (int i = 0; i <= P.m; ++i) fn(q1(i, j, k), q2(i, j, k), r(i, j, k));
      }
    };
    if (!compute_rhs(0, last_step)) return;
    if (P.time_stepper == 1) {
      upd([&](R& q1, R&, R& r) { q1 = q1 + dtr * r; });
      return;
    }
    upd([&](R& q1, R& q2, R& r) { q2 = q1 + dtr * r; });
    compute_rhs(1, false);
    if (P.time_stepper == 2) {
      upd([&](R& q1, R& q2, R& r) { q1 = (q1 + q2 + dtr * r) / R(2); });
      return;
    }
    upd([&](R& q1, R& q2, R& r) { q2 = (R(3) * q1 + q2 + dtr * r) / R(4); });
    compute_rhs(1, false);
    upd([&](R& q1, R& q2, R& r) { q1 = (q1 + R(2) * q2 + R(2) * dtr * r) / R(3); });
  }

  // The time loop of p_main.fpp:196-318 without I/O: runs t_step_start ..
  // t_step_stop, trimming dt on the way as the CPU build does.  Returns the
  // final dt.
  double run(int t_step_start, int t_step_stop, double dt0) {
    dt = dt0;
    int t_step = t_step_start;
    double mytime = t_step == 0 ? 0.0 : t_step * dt;
    double finaltime = t_step_stop * dt;
    for (;;) {
      mytime = mytime + dt;
      tvd_rk(t_step == t_step_stop);
      if (t_step == t_step_stop) break;
      if ((mytime + dt) >= finaltime) dt = finaltime - mytime;
      t_step = t_step + 1;
    }
    return dt;
  }
};

}  // namespace mfc_oracle
