/*
 * mfc_gpu.h -- C ABI of the GB300-native MicroFC hot path.
 *
 * Drop-in boundary for MicroFC's right-hand side and TVD Runge-Kutta step of
 * the 5-equation diffuse-interface model (cons -> prim with the stiffened-gas
 * mixture EOS, WENO reconstruction, HLLC with the alpha*div(u) source, flux
 * divergence, RK update).  Every entry point is plain C: POD structs, raw
 * pointers and sizes, an int status (0 = success), and no C++ exception ever
 * crosses it.  A Fortran host binds it with ISO_C_BINDING; the Python host in
 * microfc_gb300/ binds it with ctypes.
 *
 * Reference interfaces replaced (paths inside the MicroFC project):
 *   mfc_gpu_init            s_initialize_{rhs,weno,riemann_solvers,time_steppers}_module
 *                           (src/simulation/m_rhs.fpp:123, m_weno.fpp:103,
 *                            m_riemann_solvers.fpp:357, m_time_steppers.fpp:53)
 *                           and the input namelist (m_start_up.fpp:73-83)
 *   mfc_gpu_upload/download the "!$acc update device/host(q_cons_ts(1))" transfers
 *                           (src/simulation/p_main.fpp:191-193, 295-296)
 *   mfc_gpu_compute_rhs     s_compute_rhs (src/simulation/m_rhs.fpp:405-679)
 *   mfc_gpu_weno            s_weno (src/simulation/m_weno.fpp:365-542)
 *   mfc_gpu_riemann         s_hllc_riemann_solver (src/simulation/m_riemann_solvers.fpp:71-351)
 *   mfc_gpu_tvd_rk          s_1st/2nd/3rd_order_tvd_rk (m_time_steppers.fpp:129, 197, 271)
 *   mfc_gpu_run             the time-stepping loop of p_main (p_main.fpp:196-318)
 *   mfc_gpu_status          the NaN scan of p_main.fpp:295-305 (as a device flag)
 *   mfc_gpu_finalize        s_finalize_*_module
 *
 * State layout handed across the ABI: one scalar field per equation, exactly
 * the reference's q_cons_vf(i)%sf, x fastest.  The device keeps all RK
 * registers resident in HBM as one SoA block [register][equation][z][y][x]
 * (rows padded to 256 bytes); ghost cells are never stored -- boundary
 * conditions are applied by index mapping inside the kernels.
 */
#ifndef MFC_GPU_H
#define MFC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFC_GPU_ABI_VERSION 1
#define MFC_MAX_FLUIDS 4

/* Status codes (non-zero means the host should abort, as s_mpi_abort does). */
#define MFC_OK 0
#define MFC_ERR_INVALID 1   /* bad argument / unsupported configuration   */
#define MFC_ERR_CUDA 2      /* CUDA runtime error                          */
#define MFC_ERR_NOMEM 3     /* device allocation failed                    */
#define MFC_ERR_STATE 4     /* NaN / non-physical state flagged by a kernel */

/* Bits of the device status word returned by mfc_gpu_status. */
#define MFC_FLAG_NAN 0x1u          /* NaN or Inf written to a conserved field */
#define MFC_FLAG_NEG_PRESSURE 0x2u /* non-positive squared sound speed         */
                                   /* ((gamma_mix+1) p + pi_inf_mix <= 0), set */
                                   /* by the stability monitor on the steps it */
                                   /* watches (mfc_gpu_set_monitor)            */
#define MFC_FLAG_TIMEOUT 0x4u      /* a bounded device wait gave up           */

/* Precision of the reconstruction/Riemann arithmetic. */
#define MFC_PREC_FP64 0  /* plain FP64 everywhere (parity path)                       */
#define MFC_PREC_SPLIT 1 /* FP32 WENO/HLLC; FP64 state, RK update, pressure recovery   */
#define MFC_PREC_GATED 2 /* MFC_PREC_SPLIT + the learned WENO gate (2-D, WENO5)         */
#define MFC_PREC_FP64_FMA 3 /* opt-in: FP64 with multiply-add contraction (2-D, WENO5);  */
                            /* faster, no longer bit-identical to the parity oracle      */

/*
 * Case parameters: the solver-relevant subset of the reference's &user_inputs
 * namelist (src/simulation/m_start_up.fpp:73-83) plus the z extent p (the
 * reference is 2-D only) and the GPU-specific precision/device choices.
 *
 * Cell boundaries are the reference's x_cb(-1:m), y_cb(-1:n), z_cb(-1:p)
 * (m+2, n+2, p+2 values) as read from x_cb.dat / y_cb.dat
 * (m_start_up.fpp:326-367); ghost widths and the grid-dependent WENO
 * coefficients are derived from them on the host exactly as
 * s_populate_grid_variables_buffers and s_compute_weno_coefficients do.
 */
typedef struct mfc_params {
  int32_t m, n, p;          /* interior cells minus one per direction (n = p = 0 in 1-D) */
  int32_t num_fluids;       /* 1 .. MFC_MAX_FLUIDS                                        */
  int32_t weno_order;       /* 1, 3 or 5                                                  */
  double weno_eps;          /* (0, 1e-6]                                                  */
  int32_t time_stepper;     /* 1, 2 or 3 (TVD RK order)                                   */
  int32_t bc_x_beg, bc_x_end, bc_y_beg, bc_y_end, bc_z_beg, bc_z_end; /* -1 .. -12         */
  double gammas[MFC_MAX_FLUIDS];  /* fluid_pp(i)%gamma  = 1/(gamma_i - 1)                 */
  double pi_infs[MFC_MAX_FLUIDS]; /* fluid_pp(i)%pi_inf = gamma_i*pi_inf_i/(gamma_i - 1)  */
  const double* x_cb;       /* host, m+2 values                                           */
  const double* y_cb;       /* host, n+2 values, or NULL when n == 0                      */
  const double* z_cb;       /* host, p+2 values, or NULL when p == 0                      */
  int32_t precision;        /* MFC_PREC_FP64, _SPLIT, _GATED or _FP64_FMA                  */
  int32_t device;           /* CUDA device ordinal (the reference binds local_rank % ndev) */
} mfc_params;

typedef struct mfc_gpu_ctx mfc_gpu_ctx;

/* Library ABI version; lets a host check it loaded a matching build. */
int mfc_gpu_abi_version(void);

/* Last error message of the calling thread (never NULL). */
const char* mfc_gpu_last_error(void);

/* Allocates the device state (3 RK registers + rhs + grid tables; 3-D cases
 * also a work area of 2 registers for the directional sweeps) and uploads
 * the grid.  Replaces s_initialize_*_module. */
int mfc_gpu_init(const mfc_params* params, mfc_gpu_ctx** ctx_out);

/* Number of equations (sys_size = 2*num_fluids + num_dims + 1). */
int mfc_gpu_sys_size(const mfc_gpu_ctx* ctx);

/* Copy equation `var` (0-based) of register 0 (q_cons_ts(1)) from/to a host
 * array.  host_sf points at element (0,0,0) of the interior; ld_y is the
 * distance in elements between consecutive y rows and ld_z between z planes.
 * A Fortran host passes c_loc(sf(0,0)) with ld_y = m + 2*buff_size + 1.
 * Synchronous with respect to the context's stream. */
int mfc_gpu_upload(mfc_gpu_ctx* ctx, int var, const double* host_sf, int64_t ld_y, int64_t ld_z);
int mfc_gpu_download(mfc_gpu_ctx* ctx, int var, double* host_sf, int64_t ld_y, int64_t ld_z);

/* Whole-state copies of register 0, [S][p+1][n+1][m+1] contiguous. */
int mfc_gpu_upload_state(mfc_gpu_ctx* ctx, const double* host_q);
int mfc_gpu_download_state(mfc_gpu_ctx* ctx, double* host_q);

/* Drop-in for s_compute_rhs(q_cons_ts(1), q_prim_vf, rhs_vf, t_step): computes
 * the RHS of register 0 into host arrays rhs_out and prim_out (either may be
 * NULL), both [S][p+1][n+1][m+1].  Uses the unfused sweep kernels; intended
 * for verification and for hosts that run their own time integrator. */
int mfc_gpu_compute_rhs(mfc_gpu_ctx* ctx, double* rhs_out, double* prim_out);

/* The two halves of a directional sweep, one call each, for hosts that call
 * s_weno or s_hllc_riemann_solver on their own (a host with its own flux
 * assembly, a verification harness that wants the face states).  Plain FP64
 * (MFC_PREC_FP64 contexts without processor boundaries), the arithmetic of
 * the fused kernels.  Face window of direction dir (0 = x, 1 = y, 2 = z; s =
 * m, n or p along dir): the cells j = -1 .. s+1 along dir and the interior
 * cells across it, host arrays [S][e2][e1][e0] (x fastest) with e_dir = s+3
 * (cell j at index j+1) and the other extents m+1, n+1, p+1.
 *
 * Drop-in for s_weno(v_vf, vL_x, vL_y, vR_x, vR_y, weno_dir, is1, is2)
 * (src/simulation/m_weno.fpp:365-542) as s_reconstruct_cell_boundary_values
 * calls it (m_rhs.fpp:920-952), on the primitive variables of register 0
 * with the case's boundary conditions in the ghost cells (m_rhs.fpp:434-447):
 * vL / vR receive the left-face (x_{j-1/2}) and right-face (x_{j+1/2}) values
 * over the face window, the part of the reference's is1 x is2 window that the
 * Riemann solver reads.  Synchronous (host arrays in and out); both entry
 * points work in a device scratch area that the context keeps between calls
 * and grows to the largest request (freed by mfc_gpu_finalize). */
int mfc_gpu_weno(mfc_gpu_ctx* ctx, int dir, double* vL, double* vR);

/* Drop-in for s_hllc_riemann_solver (src/simulation/m_riemann_solvers.fpp:
 * 71-351, inviscid contexts) with its Riemann-state buffers of bc -4
 * (:444-619).  qL_rs / qR_rs are its qL_prim_rs / qR_prim_rs over the face
 * window: the state left of face j+1/2 is qL_rs(j), the state right of it
 * qR_rs(j+1).  s_compute_rhs passes the right-face WENO values as qL_prim_rs
 * and the left-face values as qR_prim_rs (m_rhs.fpp:545-556): qL_rs = vR and
 * qR_rs = vL of mfc_gpu_weno.  Outputs for the faces j+1/2, j = -1 .. s
 * (index j+1, extent s+2 along dir): flux [S][...] (flux_vf) and flux_src
 * [...] = flux_src_vf(advxb), the interface velocity vel_src(dir) of the
 * alpha*div(u) source (:314-325). */
int mfc_gpu_riemann(mfc_gpu_ctx* ctx, int dir, const double* qL_rs, const double* qR_rs, double* flux,
                    double* flux_src);

/* Drop-in for s_{1,2,3}_order_tvd_rk(t_step, time_avg): one full time step of
 * register 0 with time step dt, as fused stage kernels (one launch per RK
 * stage).  When last_step != 0 the call does nothing, mirroring the early
 * return at t_step == t_step_stop (m_rhs.fpp:452).  Asynchronous. */
int mfc_gpu_tvd_rk(mfc_gpu_ctx* ctx, double dt, int last_step);

/* ---- Processor boundaries (domain decomposition, m_mpi_proxy.fpp:468-979).
 * A boundary value >= 0 in mfc_params (the neighbouring subdomain, as the
 * reference's bc_x%beg = rank) makes that side read its ghost cells from a
 * halo receive buffer instead of a physical boundary condition (the
 * neighbour's ghost cell widths come from mfc_gpu_set_halo_widths, as the
 * reference exchanges them).  Such a context is stepped stage
 * by stage: before stage s, every subdomain packs the strip next to each of
 * its processor boundaries from that stage's input (mfc_gpu_halo_pack) into
 * the neighbour's receive buffer (mfc_gpu_halo_buffer) -- directly when both
 * live on one GPU, or through a send/receive pair across GPUs -- and then
 * runs mfc_gpu_rk_stage.  mfc_gpu_tvd_rk and mfc_gpu_run refuse such a
 * context.  Layouts (depth d = 0 next to the boundary, H = (weno_order+1)/2):
 * x sides [S][p+1][n+1][H], y sides [S][p+1][H][m+1] in 3-D and [S][H][m+3]
 * in 2-D, z sides [S][H][n+1][m+1].  A 2-D y strip carries the sender's x
 * ghost cells -1 and m+1 of each row in its first and last column (from its
 * own x receive buffers at processor boundaries): the diagonal neighbours'
 * cells that the viscous corner gradients read.  So in 2-D the x strips of a
 * stage are exchanged first and the y strips packed after they arrived, as
 * the reference exchanges x before y (m_mpi_proxy.fpp). */
int mfc_gpu_rk_stage(mfc_gpu_ctx* ctx, int stage, double dt);
int mfc_gpu_halo_buffer(mfc_gpu_ctx* ctx, int dir, int side, double** dev_ptr, int64_t* count);
/* The neighbour's cell widths beyond a processor boundary (widths[i] = ghost
 * cell at depth i, count >= buff_size = (weno_order-1)/2 + 2), as the
 * reference exchanges its grid buffers (m_mpi_proxy.fpp); without them the
 * ghost cells repeat the edge cell's width.  Rebuilds the WENO tables. */
int mfc_gpu_set_halo_widths(mfc_gpu_ctx* ctx, int dir, int side, const double* widths, int count);
/* Packs, on the context's stream, the strip that the neighbour across
 * (dir, side) needs for stage `stage` into dst (device memory, layout of the
 * neighbour's receive buffer for its opposite side). */
int mfc_gpu_halo_pack(mfc_gpu_ctx* ctx, int stage, int dir, int side, double* dst);

/* The time loop of p_main (p_main.fpp:196-318) from t_step_start to
 * t_step_stop, including the trim of dt at the last step of the CPU build.
 * *dt_inout carries dt in and the final (possibly trimmed) dt out.
 * Synchronous; returns MFC_ERR_STATE if a kernel flagged a NaN. */
int mfc_gpu_run(mfc_gpu_ctx* ctx, int t_step_start, int t_step_stop, double* dt_inout);

/* Waits for the context's stream and returns the accumulated device status
 * bits (MFC_FLAG_*) in *flags; clears them when clear != 0. */
int mfc_gpu_status(mfc_gpu_ctx* ctx, uint32_t* flags, int clear);

/* Viscous terms (m_viscous.fpp, the viscous source flux of
 * m_riemann_solvers.fpp:683-902 and its divergence in m_rhs.fpp:591-651):
 * re_shear[i] / re_bulk[i] are fluid_pp(i+1)%Re(1) / %Re(2) for the
 * context's fluids (NULL or values <= 0: none).  The velocity gradients are
 * the reference's one-sided face differences (weno_Re_flux = F; see
 * mfc_gpu_set_viscous_gradients for weno_Re_flux = T).  1-D and
 * 2-D contexts, with or without processor boundaries; all-zero Reynolds
 * numbers switch back to the inviscid kernels.  Call before stepping. */
int mfc_gpu_set_viscosity(mfc_gpu_ctx* ctx, const double* re_shear, const double* re_bulk);

/* weno_Re_flux (m_viscous.fpp:176-216, 381-591; m_rhs.fpp:512-528): with
 * weno_re_flux != 0 the viscous stresses take their velocity gradients from
 * WENO reconstructions -- the velocities reconstructed to the faces along
 * each direction, cell gradients from them by the divergence theorem, those
 * gradients reconstructed along the sweep direction and averaged at each
 * face -- instead of the finite differences of weno_Re_flux = F.  Three
 * (1-D) or four (2-D) preparation kernels run before every RK stage; they
 * reconstruct in FP64 in FP64 contexts (bit-identical to the CPU build's
 * operation order) and in FP32 in split and gated ones.  Viscous (call
 * mfc_gpu_set_viscosity first) WENO5 contexts of the FP64, split or gated
 * precision without processor boundaries; 0 switches back to the finite
 * differences. */
int mfc_gpu_set_viscous_gradients(mfc_gpu_ctx* ctx, int weno_re_flux);

/* Variables the WENO reconstruction works on (no reference counterpart: the
 * reference reconstructs the primitive variables, m_weno.fpp:470-536).
 * MFC_RECON_CHARACTERISTIC projects each cell's stencil on the
 * characteristic fields of the quasi-linear primitive system along the sweep
 * direction, frozen at the cell's own state -- alpha_i rho_i - kappa_i p
 * (kappa_i = alpha_i rho_i / (rho c^2)), p -/+ rho c u_n, the tangential
 * velocities and the volume fractions, with the mixture sound speed
 * c^2 = ((Gamma + 1) p + Pi) / (Gamma rho) of the HLLC solver -- reconstructs
 * them with the same WENO weights and maps both face values back.  Plain
 * FP64 contexts, 1-D, 2-D (fused kernel) and 3-D (directional sweeps),
 * WENO3 or WENO5, inviscid, without processor boundaries (WENO1
 * reconstructs nothing and keeps the primitive kernel).
 * Call before stepping; MFC_RECON_PRIMITIVE switches back. */
#define MFC_RECON_PRIMITIVE 0
#define MFC_RECON_CHARACTERISTIC 1
int mfc_gpu_set_reconstruction(mfc_gpu_ctx* ctx, int variables);

/* Split and gated WENO5 on a uniform grid (no reference counterpart): when
 * every cell of a direction has the same FP32 coefficient record, the
 * kernels read that one record from their parameters instead of staging
 * per-cell records in shared memory, with identical results.  On by default;
 * enable = 0 forces the per-cell records.  *in_use (may be NULL) receives a
 * bit per direction (x = 1, y = 2, z = 4) that now uses the shared record. */
int mfc_gpu_set_uniform_coefficients(mfc_gpu_ctx* ctx, int enable, int* in_use);

/* Run-time stability monitor, the reference's ICFL of s_write_run_time_information
 * (src/simulation/m_data_output.fpp:178-310), fused into the last stage kernel
 * of every step: ICFL = dt / min_d(dx_d / (|u_d| + c)), maximised over the cells
 * of the step's new state.  mfc_gpu_set_monitor turns it on/off (and clears
 * the maximum); with it on, mfc_gpu_run fails like the reference when the
 * maximum is NaN or above 1.  mfc_gpu_icfl returns the maximum since the last
 * reset.  The monitor reads the state only; it changes no result. */
int mfc_gpu_set_monitor(mfc_gpu_ctx* ctx, int on);
int mfc_gpu_icfl(mfc_gpu_ctx* ctx, double* icfl_max, int reset);

/* No counterpart in the reference (whose dt is fixed by the case file).
 * num_steps time steps with dt chosen from the monitored ICFL so that every
 * step after the first runs at the given CFL number: dt_{n+1} = dt_n * cfl /
 * ICFL_n.  *dt_inout: first dt in, next dt out; *time_inout is advanced. */
int mfc_gpu_run_cfl(mfc_gpu_ctx* ctx, int num_steps, double cfl, double* dt_inout, double* time_inout);

/* Output without stalling the time loop (no counterpart in the reference,
 * whose "!$acc update host" at every t_step_save blocks, p_main.fpp:291-296).
 * mfc_gpu_snapshot copies register 0 at the current point of the context's
 * stream to a device staging buffer, then to pinned host slot `slot` (0 or
 * 1) on a second stream, so time steps launched afterwards run while the
 * copy is in flight.  mfc_gpu_snapshot_wait blocks until that copy has
 * landed and returns the slot's [S][p+1][n+1][m+1] array, valid until the
 * slot's next snapshot or mfc_gpu_finalize. */
int mfc_gpu_snapshot(mfc_gpu_ctx* ctx, int slot);
int mfc_gpu_snapshot_wait(mfc_gpu_ctx* ctx, int slot, const double** host_q);

/* The CUDA stream (cudaStream_t) the context launches on, for event timing. */
void* mfc_gpu_stream(mfc_gpu_ctx* ctx);

/* Number of kernel launches the context has issued since init. */
int64_t mfc_gpu_launch_count(const mfc_gpu_ctx* ctx);

/* Frees all device memory of the context. */
int mfc_gpu_finalize(mfc_gpu_ctx* ctx);

/* No counterpart in the reference (which tunes nothing).  Autotuner: times a
 * few first-stage launches of every compiled tile variant of the context's
 * configuration (the state is not advanced), keeps the fastest and returns
 * its index and per-launch time in milliseconds.  A variant that stages its
 * tiles by TMA (MFC_VARIANT_TMA) wins a tie within 1 %. */
int mfc_gpu_tune(mfc_gpu_ctx* ctx, int reps, int* variant_out, double* ms_out);
/* Pins tile variant `variant` (the numbering mfc_gpu_tune reports) and
 * returns its tile shape and threads per block; MFC_ERR_INVALID past the
 * last variant of the context's configuration. */
int mfc_gpu_select_variant(mfc_gpu_ctx* ctx, int variant, int* tx, int* ty, int* threads);
/* Features of tile variant `variant` of the context's configuration, as
 * MFC_VARIANT_* bits in *features; MFC_ERR_INVALID past the last variant. */
#define MFC_VARIANT_TMA 0x1u /* interior tiles arrive by one TMA bulk tensor copy (2-D and
                                3-D inviscid kernels)                                       */
int mfc_gpu_variant_features(mfc_gpu_ctx* ctx, int variant, uint32_t* features);

/* ---- Learned WENO gate (no reference counterpart).  A 10-32-32-1 MLP on a
 * cell's alpha_1 and p stencils picks nonlinear WENO5 or the optimal linear
 * weights per cell and direction (MFC_PREC_GATED).  Parameters are FP32
 * vectors of mfc_gate_param_count() values (W1[10][32], b1[32], W2[32][32],
 * b2[32], W3[32], b3); inference uses them rounded to FP16. */
int mfc_gate_param_count(void);
/* Floats of training workspace a batch needs. */
int mfc_gate_workspace_floats(int batch);
/* Sets the gate parameters (host FP32) of a MFC_PREC_GATED context; its
 * time steps fail until this has been called. */
int mfc_gpu_set_gate(mfc_gpu_ctx* ctx, const float* host_params);
/* Training samples of the context's current state (register 0) along
 * direction dir (0 = x, 1 = y) for all interior cells: features
 * x_dev[cells][10] and the label statistic dev_dev[cells] = max_k
 * |omega_k - d_k| over alpha_1, p and both faces.  Device pointers. */
int mfc_gpu_gate_samples(mfc_gpu_ctx* ctx, int dir, float* x_dev, float* dev_dev);
/* Forward + backward of a batch (device pointers): grad <- gradient of the
 * mean weighted binary cross-entropy, *loss <- summed loss.  Synchronous. */
int mfc_gate_gradients(const float* X, const float* T, int batch, const float* w, float pos_weight, float* grad,
                       float* work, float* loss, void* stream);
/* One Adam step on a batch (device pointers; asynchronous on stream). */
int mfc_gate_train_step(const float* X, const float* T, int batch, float* w, float* grad, float* m, float* v,
                        float* work, int step, float lr, float pos_weight, float* loss, void* stream);
/* Tensor-core inference (FP16 weights, FP32 accumulation) of n inputs;
 * wh_scratch holds mfc_gate_param_count() halves.  Synchronous. */
int mfc_gate_infer(const float* X, int n, const float* w, void* wh_scratch, float* logits, void* stream);

/* ---- Ensemble mode (no reference counterpart; the reference runs one case
 * per process).  Up to 96 independent 2-D cases that share num_fluids,
 * weno_order, precision, time_stepper (2 or 3) and device, each with its own
 * grid, boundary conditions, fluids and dt, advanced by one persistent
 * launch per RK stage over a work list of (case, tile) pairs. */
typedef struct mfc_gpu_ensemble mfc_gpu_ensemble;

int mfc_gpu_ensemble_init(const mfc_params* cases, const double* dts, int num_cases, mfc_gpu_ensemble** out);
/* Case state copies, [S][n+1][m+1] contiguous (register 0). */
int mfc_gpu_ensemble_upload(mfc_gpu_ensemble* ens, int case_index, const double* host_q);
int mfc_gpu_ensemble_download(mfc_gpu_ensemble* ens, int case_index, double* host_q);
/* Autotuner over the compiled ensemble tile variants (see mfc_gpu_tune). */
int mfc_gpu_ensemble_tune(mfc_gpu_ensemble* ens, int reps, int* variant_out, double* ms_out);
/* Pins the ensemble's tile variant (the numbering of mfc_gpu_ensemble_tune);
 * every variant gives the same bits.  Returns its tile shape. */
int mfc_gpu_ensemble_select_variant(mfc_gpu_ensemble* ens, int variant, int* tx, int* ty, int* threads);
/* MFC_VARIANT_* bits of ensemble tile variant `variant` (see
 * mfc_gpu_variant_features). */
int mfc_gpu_ensemble_variant_features(mfc_gpu_ensemble* ens, int variant, uint32_t* features);
/* Steps t_step_start .. t_step_stop-1 of every case; each case's last step
 * uses its dt after the p_main trim.  use_graph != 0 replays the stage
 * launches of a step from a CUDA graph.  Synchronous; MFC_ERR_STATE on NaN. */
int mfc_gpu_ensemble_run(mfc_gpu_ensemble* ens, int t_step_start, int t_step_stop, int use_graph);
void* mfc_gpu_ensemble_stream(mfc_gpu_ensemble* ens);
int64_t mfc_gpu_ensemble_launch_count(const mfc_gpu_ensemble* ens);
int mfc_gpu_ensemble_finalize(mfc_gpu_ensemble* ens);
/* Viscous terms for every case of an ensemble (see mfc_gpu_set_viscosity):
 * re_shear[i * num_fluids + f] / re_bulk[...] are case i's fluid_pp(f+1)%Re(1)
 * / %Re(2) (NULL or values <= 0: none).  One kernel advances all cases, so
 * every case must be viscous or none (MFC_ERR_INVALID otherwise); all-zero
 * Reynolds numbers switch back to the inviscid kernels.  FP64, split and
 * gated precision.  Call before stepping and before mfc_gpu_ensemble_tune
 * (it selects the first compiled viscous variant). */
int mfc_gpu_ensemble_set_viscosity(mfc_gpu_ensemble* ens, const double* re_shear, const double* re_bulk);
/* Gate parameters for a MFC_PREC_GATED ensemble (see mfc_gpu_set_gate). */
int mfc_gpu_ensemble_set_gate(mfc_gpu_ensemble* ens, const float* host_params);

/* ---- Initial condition on the device: the reference's pre_process patches
 * (src/pre_process/m_create_patches.fpp:47-534): line segment 1, circle 2,
 * rectangle 3, sweep line 4, ellipse 5, isentropic vortex 6, 2-D analytical
 * 7, 1-D analytical 15 and varcircle 18 (geometries 2-7 and 18 are
 * z-independent in 3-D); sphere 8 and cuboid 9 are the 3-D analogues of 2
 * and 3.  Then the smoothed-patch blend (m_assign_patches.fpp:54-165) and
 * prim -> cons (src/common/m_variables_conversion.fpp:385-443), on the
 * uniform grid of m_grid.f90:54-70 over the given domain.  Fields mirror
 * patch_icpp(i)%... of the case file; alter_patch[j] != 0 lets the patch
 * overwrite cells owned by patch j (j = 0: no patch yet).  Writes register 0
 * (q_cons_ts(1)) directly: no host initial condition and no file round trip.
 * Same operation order as the CPU pre_process; only tanh (smoothed circles,
 * spheres, ellipses and sweep lines) and exp (the analytical patches'
 * pressure bump) may differ from the host's libm in the last bit.  Refused:
 * a geometry the grid's dimensionality does not take, a smooth_patch_id
 * outside 1..num_patches on a patch that blends, an ellipse with a
 * non-positive semi-axis, a sweep line with a zero normal. */
#define MFC_MAX_PATCHES 10
typedef struct mfc_patch {
  int32_t geometry;                 /* 1-9, 15 or 18 (see above)                        */
  double x_centroid, y_centroid, z_centroid;
  double length_x, length_y, length_z;
  double radius;
  int32_t smoothen;                 /* circles, spheres, ellipses, sweep lines: tanh    */
                                    /* smoothed volume fraction                         */
  int32_t smooth_patch_id;          /* 1-based patch the smoothing blends into          */
  double smooth_coeff;
  int32_t alter_patch[MFC_MAX_PATCHES + 1];
  double alpha_rho[MFC_MAX_FLUIDS];
  double alpha[MFC_MAX_FLUIDS];
  double vel[3];
  double pres;
  double normal[3];                 /* sweep line: (a, b) of a x + b y + c >= 0          */
  double radii[3];                  /* ellipse: semi-axes along x and y                 */
  double epsilon;                   /* varcircle: thickness of the annulus              */
} mfc_patch;

/* domain: x_beg, x_end, y_beg, y_end, z_beg, z_end (unused directions
 * ignored), the uniform grid of m_grid.f90:54-70.  domain == NULL (single
 * case only): the context's own cell boundaries, with cell centres
 * (x_cb(i-1) + x_cb(i))/2 and the smallest cell width as the smoothing
 * length, as pre_process sets them on a stretched grid (m_grid.f90:72-90). */
int mfc_gpu_generate_ic(mfc_gpu_ctx* ctx, const mfc_patch* patches, int num_patches, const double* domain);
int mfc_gpu_ensemble_generate_ic(mfc_gpu_ensemble* ens, int case_index, const mfc_patch* patches, int num_patches,
                                 const double* domain);

/* No counterpart in the reference.  One time step like mfc_gpu_tvd_rk, for
 * callers that cannot allocate device memory (their device memory belongs to
 * another allocator -- a framework's caching pool, or an OpenACC runtime that
 * owns the state arrays -- or they must avoid the device-wide synchronisation
 * of cudaMalloc/cudaFree).  It allocates nothing: the intermediate RK
 * register, grid tables and status word live in a fixed file-scope device
 * array of about 58 MiB that each GPU loading the library holds until exit.
 * q_in (state at t^n) and q_out (state at t^{n+1}) are distinct device
 * arrays [S][p+1][n+1][ld_y], x fastest.  Limits: S*(n+1)*(p+1)*ld_y <=
 * 7*2^20 doubles and at most 4096 cells per direction; larger cases return
 * MFC_ERR_INVALID, and so does MFC_PREC_GATED (the gate's parameters live
 * in a context; MFC_PREC_FP64, _SPLIT and _FP64_FMA are taken).  Synchronous with respect to `stream` (a cudaStream_t,
 * NULL = legacy default stream); returns MFC_ERR_STATE if a NaN was written
 * or a TMA staging wait timed out (q_out is then incomplete).
 * All calls share the array: calls that overlap on the GPU race.  The first
 * call on a device looks up the array's address with that device current;
 * make it before any stream capture. */
int mfc_gpu_tvd_rk_noalloc(const mfc_params* params, const double* q_in, double* q_out, int64_t ld_y, double dt,
                           void* stream);

/* Diagnostic with no reference counterpart: measures the device's FP64 and
 * FP32 fused-multiply-add throughput (TFLOP/s, 2 flops per FMA), the
 * denominators of the compute roofline reported by the benchmark. */
int mfc_gpu_measure_peaks(int device, double* fp64_tflops, double* fp32_tflops);

/* Self-test with no reference counterpart: for i < n, q_fast[i] = a[i]/b[i]
 * through the plain path's correctly rounded shared-divisor division and
 * q_ieee[i] = a[i]/b[i] through the IEEE division; the two must agree bit
 * for bit.  All pointers are device memory; asynchronous on `stream`. */
int mfc_gpu_selftest_div(const double* a, const double* b, double* q_fast, double* q_ieee, long long n,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MFC_GPU_H */
