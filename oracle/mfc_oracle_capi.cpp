// C ABI of the MicroFC oracle (test infrastructure only; see mfc_oracle.hpp).
//
// Loaded with ctypes by tests/, by __graft_entry__.smoke() and by the CPU
// baseline leg of bench.py.  All arrays are x-fastest over the interior
// cells (m+1)*(n+1)*(p+1) unless stated otherwise.
#include <cstdio>
#include <cstring>
#include <new>

#include "mfc_oracle.hpp"
#include "mfc_oracle_ic.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace mfc_oracle;

extern "C" {

// Mirrors the solver-relevant part of the reference's &user_inputs namelist
// (src/simulation/m_start_up.fpp:73-83), plus the z extent p.
struct mfo_params {
  int m, n, p;
  int num_fluids;
  int weno_order;
  double weno_eps;
  int time_stepper;
  int bc_x_beg, bc_x_end, bc_y_beg, bc_y_end, bc_z_beg, bc_z_end;
  double gammas[kMaxFluids];
  double pi_infs[kMaxFluids];
  double re_shear[kMaxFluids];  // fluid_pp(i)%Re(1); <= 0: inviscid
  double re_bulk[kMaxFluids];   // fluid_pp(i)%Re(2)
  int char_decomp;              // 1: WENO of the characteristic fields (Solver::weno)
  int weno_re_flux;             // 1: weno_Re_flux = T (viscous stresses from WENO-reconstructed gradients)
};

static Params to_params(const mfo_params* q) {
  Params P;
  P.m = q->m; P.n = q->n; P.p = q->p;
  P.num_fluids = q->num_fluids;
  P.weno_order = q->weno_order;
  P.weno_eps = q->weno_eps;
  P.time_stepper = q->time_stepper;
  P.bc_x_beg = q->bc_x_beg; P.bc_x_end = q->bc_x_end;
  P.bc_y_beg = q->bc_y_beg; P.bc_y_end = q->bc_y_end;
  P.bc_z_beg = q->bc_z_beg; P.bc_z_end = q->bc_z_end;
  for (int i = 0; i < kMaxFluids; ++i) { P.gammas[i] = q->gammas[i]; P.pi_infs[i] = q->pi_infs[i]; }
  for (int i = 0; i < kMaxFluids; ++i) { P.re[0][i] = q->re_shear[i]; P.re[1][i] = q->re_bulk[i]; }
  P.char_decomp = q->char_decomp != 0;
  P.weno_re_flux = q->weno_re_flux != 0;
  return P;
}

void* mfo_create(const mfo_params* q, const double* x_cb, const double* y_cb, const double* z_cb) {
  // every used direction needs its cell boundaries
  if (!q || !x_cb || (q->n > 0 && !y_cb) || (q->p > 0 && !z_cb)) return nullptr;
  // the viscous terms, and with them weno_Re_flux, are 1-D and 2-D
  if (q->weno_re_flux && q->p > 0) return nullptr;
  auto* s = new (std::nothrow) Solver<double>();
  if (!s) return nullptr;
  s->init(to_params(q), x_cb, y_cb, z_cb);
  return s;
}

void mfo_destroy(void* h) { delete static_cast<Solver<double>*>(h); }

int mfo_sys_size(void* h) { return static_cast<Solver<double>*>(h)->S; }

// reg: 0 = q_cons_ts(1), 1 = q_cons_ts(2)
void mfo_set_state(void* h, int reg, const double* interior) {
  auto* s = static_cast<Solver<double>*>(h);
  const Params& P = s->P;
  long c = 0;
  for (int v = 0; v < s->S; ++v)
    for (int k = 0; k <= P.p; ++k)
      for (int j = 0; j <= P.n; ++j)
        for (int i = 0; i <= P.m; ++i) s->q_cons_ts[reg][v](i, j, k) = interior[c++];
}

void mfo_get_state(void* h, int reg, double* interior) {
  auto* s = static_cast<Solver<double>*>(h);
  const Params& P = s->P;
  long c = 0;
  for (int v = 0; v < s->S; ++v)
    for (int k = 0; k <= P.p; ++k)
      for (int j = 0; j <= P.n; ++j)
        for (int i = 0; i <= P.m; ++i) interior[c++] = s->q_cons_ts[reg][v](i, j, k);
}

// s_compute_rhs on register reg; writes rhs (S x cells) and the primitive
// variables of the interior cells (S x cells).
void mfo_compute_rhs(void* h, int reg, double* rhs_out, double* prim_out) {
  auto* s = static_cast<Solver<double>*>(h);
  const Params& P = s->P;
  s->compute_rhs(reg, false);
  long c = 0;
  for (int v = 0; v < s->S; ++v)
    for (int k = 0; k <= P.p; ++k)
      for (int j = 0; j <= P.n; ++j)
        for (int i = 0; i <= P.m; ++i, ++c) {
          if (rhs_out) rhs_out[c] = s->rhs[v](i, j, k);
          if (prim_out) prim_out[c] = s->qp[v](i, j, k);
        }
}

// One call of s_{1,2,3}_order_tvd_rk with the given dt.
void mfo_tvd_rk(void* h, double dt, int last_step) {
  auto* s = static_cast<Solver<double>*>(h);
  s->dt = dt;
  s->tvd_rk(last_step != 0);
}

// The p_main.fpp time loop; returns the trimmed dt of the last step.
double mfo_run(void* h, int t_step_start, int t_step_stop, double dt) {
  return static_cast<Solver<double>*>(h)->run(t_step_start, t_step_stop, dt);
}

// The face window of direction dir that the Riemann solver reads: cells
// j = -1 .. s+1 along dir (s = m, n or p), interior cells across it.  Arrays
// are [S][e2][e1][e0] with e_dir = s_dir + 3 (cell j at index j + 1) and
// e_other = s_other + 1.
static void face_window(const Params& P, int dir, int (&lo)[3], int (&hi)[3]) {
  const int ss[3] = {P.m, P.n, P.p};
  for (int d = 0; d < 3; ++d) {
    lo[d] = 0;
    hi[d] = ss[d];
  }
  lo[dir] = -1;
  hi[dir] = ss[dir] + 1;
}

// s_weno along direction dir (m_weno.fpp:365-542, as
// s_reconstruct_cell_boundary_values calls it, m_rhs.fpp:920-952) of the
// primitive variables of register reg after s_populate_conservative_
// variables_buffers and cons -> prim (m_rhs.fpp:434-447).  vL/vR: left-face
// (x_{j-1/2}) and right-face (x_{j+1/2}) values over the face window.
void mfo_weno(void* h, int reg, int dir, double* vL_out, double* vR_out) {
  auto* s = static_cast<Solver<double>*>(h);
  for (int v = 0; v < s->S; ++v) s->qp[v].d = s->q_cons_ts[reg][v].d;
  s->populate_buffers();
  s->cons_to_prim();
  s->weno(dir);
  int lo[3], hi[3];
  face_window(s->P, dir, lo, hi);
  long c = 0;
  for (int v = 0; v < s->S; ++v)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i, ++c) {
          vL_out[c] = s->vL[v](i, j, k);
          vR_out[c] = s->vR[v](i, j, k);
        }
}

// s_hllc_riemann_solver along direction dir (m_riemann_solvers.fpp:71-351)
// with the Riemann-state buffers of bc -4 (:444-619).  qL_rs / qR_rs are the
// reference's qL_prim_rs / qR_prim_rs over the face window: the state left
// of face j+1/2 is qL_rs(j), the state right of it qR_rs(j+1).  (s_compute_rhs
// passes the right-face WENO values as qL_prim_rs and the left-face values
// as qR_prim_rs, m_rhs.fpp:545-556.)  Outputs for faces j = -1 .. s_dir
// (face j+1/2 at index j + 1): flux [S][...] with extent s_dir + 2 along dir,
// and flux_src(advxb) = vel_src(dir) (m_riemann_solvers.fpp:314-325).
void mfo_riemann(void* h, int dir, const double* qL_rs, const double* qR_rs, double* flux_out, double* src_out) {
  auto* s = static_cast<Solver<double>*>(h);
  int lo[3], hi[3];
  face_window(s->P, dir, lo, hi);
  long c = 0;
  for (int v = 0; v < s->S; ++v)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i, ++c) {
          s->vR[v](i, j, k) = qL_rs[c];  // the solver reads its left state from vR
          s->vL[v](i, j, k) = qR_rs[c];
        }
  s->hllc(dir);
  hi[dir] -= 1;  // faces -1/2 .. s+1/2
  c = 0;
  for (int v = 0; v <= s->S; ++v)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          if (v < s->S) flux_out[c++] = s->flux[v](i, j, k);
          else *src_out++ = s->fsrc(i, j, k);
        }
}

void mfo_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int mfo_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// ---------------------------------------------------------------------------
// pre_process restatement: uniform grid and patches -> conservative state.
// stretch: null, or {a_x, x_a, x_b, loops_x, a_y, y_a, y_b, loops_y} with
// loops 0 for a uniform direction.
int mfo_generate_ic(const mfo_params* q, const mfo_patch* patches, int num_patches, double x_beg, double x_end,
                    double y_beg, double y_end, double z_beg, double z_end, const double* stretch, double* x_cb,
                    double* y_cb, double* z_cb, double* cons_out) {
  return generate_ic(to_params(q), patches, num_patches, x_beg, x_end, y_beg, y_end, z_beg, z_end, stretch, x_cb,
                     y_cb, z_cb, cons_out);
}

// Operation counts of one full time step of the oracle, per interior cell.
// Defined in mfc_oracle_flops.cpp (built without OpenMP).
int mfo_count_ops(const mfo_params* q, const double* x_cb, const double* y_cb, const double* z_cb,
                  const double* state, double dt, double* counts_out);
}
