/*
 * p_main_host.c -- a C host that drives libmfc_gpu.so through
 * include/mfc_gpu.h with the call sequence of MicroFC's simulation program
 * (src/simulation/p_main.fpp), standing in for the Fortran bridge
 * (microfc_gb300/fortran/m_gpu_bridge.f90) where no Fortran compiler exists:
 *
 *   p_main.fpp:188-193  mfc_gpu_init (viscous cases: mfc_gpu_set_viscosity
 *                       with every fluid's Re(1:2), and with weno_Re_flux
 *                       mfc_gpu_set_viscous_gradients), then mfc_gpu_upload
 *                       of every q_cons_ts(1)%vf(i)%sf(-b:m+b, -b:n+b),
 *                       passed from sf(0,0) with the leading dimension m + 2b + 1
 *   p_main.fpp:196-203  t_step = t_step_start; mytime; finaltime
 *   p_main.fpp:229-235  one mfc_gpu_tvd_rk per time step (last_step at t_step_stop)
 *   p_main.fpp:284-288  dt trim: if (mytime + dt >= finaltime) dt = finaltime - mytime
 *   p_main.fpp:291-306  at save steps: mfc_gpu_status (the NaN scan), then
 *                       mfc_gpu_download of every variable into the padded arrays
 *   finalisation        mfc_gpu_finalize
 *
 * Input file (native byte order):
 *   int32 m, n, num_fluids, weno_order, time_stepper, bc_x_beg, bc_x_end,
 *         bc_y_beg, bc_y_end, t_step_start, t_step_stop, t_step_save,
 *         viscous, weno_re_flux
 *   double weno_eps, dt, gammas[num_fluids], pi_infs[num_fluids]
 *   double re_shear[num_fluids], re_bulk[num_fluids] (when viscous != 0)
 *   double x_cb[m+2], y_cb[n+2] (when n > 0)
 *   double sf[S][ny_pad][nx_pad]: every variable with its ghost layers,
 *         nx_pad = m + 2b + 1, ny_pad = n + 2b + 1 (1 when n == 0)
 * Output file: per save step int32 t_step then the S padded arrays; at the
 * end double dt (after the trim).  Exit status 0 on success; a library
 * error is printed with mfc_gpu_last_error() and exits 1, as the reference
 * aborts through s_mpi_abort.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mfc_gpu.h"

static void check(int rc, const char* what) {
  if (rc != MFC_OK) {
    fprintf(stderr, "%s: status %d: %s\n", what, rc, mfc_gpu_last_error());
    exit(1);
  }
}

static void read_exact(FILE* f, void* p, size_t bytes) {
  if (fread(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "short input file\n");
    exit(2);
  }
}

static void write_exact(FILE* f, const void* p, size_t bytes) {
  if (fwrite(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "short write\n");
    exit(2);
  }
}

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
    return 2;
  }
  FILE* in = fopen(argv[1], "rb");
  if (!in) return 2;
  int32_t hdr[14];
  read_exact(in, hdr, sizeof hdr);
  const int m = hdr[0], n = hdr[1], nf = hdr[2], wo = hdr[3], ts = hdr[4];
  const int t_step_start = hdr[9], t_step_stop = hdr[10], t_step_save = hdr[11];
  const int viscous = hdr[12], weno_re_flux = hdr[13];
  if (nf < 1 || nf > MFC_MAX_FLUIDS || m < 1 || n < 0 || t_step_save < 1) return 2;
  double weno_eps, dt;
  read_exact(in, &weno_eps, sizeof weno_eps);
  read_exact(in, &dt, sizeof dt);

  mfc_params prm;
  memset(&prm, 0, sizeof prm);
  prm.m = m;
  prm.n = n;
  prm.p = 0;
  prm.num_fluids = nf;
  prm.weno_order = wo;
  prm.weno_eps = weno_eps;
  prm.time_stepper = ts;
  prm.bc_x_beg = hdr[5];
  prm.bc_x_end = hdr[6];
  prm.bc_y_beg = hdr[7];
  prm.bc_y_end = hdr[8];
  prm.bc_z_beg = prm.bc_z_end = -3;
  read_exact(in, prm.gammas, sizeof(double) * (size_t)nf);
  read_exact(in, prm.pi_infs, sizeof(double) * (size_t)nf);
  double re_shear[MFC_MAX_FLUIDS] = {0}, re_bulk[MFC_MAX_FLUIDS] = {0};
  if (viscous) {
    read_exact(in, re_shear, sizeof(double) * (size_t)nf);
    read_exact(in, re_bulk, sizeof(double) * (size_t)nf);
  }
  double* x_cb = malloc(sizeof(double) * (size_t)(m + 2));
  double* y_cb = n > 0 ? malloc(sizeof(double) * (size_t)(n + 2)) : NULL;
  read_exact(in, x_cb, sizeof(double) * (size_t)(m + 2));
  if (y_cb) read_exact(in, y_cb, sizeof(double) * (size_t)(n + 2));
  prm.x_cb = x_cb;
  prm.y_cb = y_cb;
  prm.precision = MFC_PREC_FP64;
  prm.device = 0;

  const int nd = n > 0 ? 2 : 1;
  const int S = 2 * nf + nd + 1;
  const int b = (wo - 1) / 2 + 2;  /* buff_size */
  const int64_t nx_pad = m + 2 * b + 1, ny_pad = n > 0 ? n + 2 * b + 1 : 1;
  const int64_t per_var = nx_pad * ny_pad;
  double* sf = malloc(sizeof(double) * (size_t)(S * per_var));
  read_exact(in, sf, sizeof(double) * (size_t)(S * per_var));
  fclose(in);
  /* element (0, 0) of variable i: sf(0,0) behind b ghost rows and columns */
  const int64_t origin = (n > 0 ? b * nx_pad : 0) + b;

  mfc_gpu_ctx* ctx = NULL;
  check(mfc_gpu_init(&prm, &ctx), "mfc_gpu_init");
  if (viscous) {
    check(mfc_gpu_set_viscosity(ctx, re_shear, re_bulk), "mfc_gpu_set_viscosity");
    if (weno_re_flux) check(mfc_gpu_set_viscous_gradients(ctx, 1), "mfc_gpu_set_viscous_gradients");
  }
  for (int i = 0; i < S; ++i)
    check(mfc_gpu_upload(ctx, i, sf + i * per_var + origin, nx_pad, 0), "mfc_gpu_upload");

  FILE* out = fopen(argv[2], "wb");
  if (!out) return 2;
  int t_step = t_step_start;
  double mytime = t_step == 0 ? 0.0 : t_step * dt;
  const double finaltime = t_step_stop * dt;
  for (;;) {
    mytime = mytime + dt;
    check(mfc_gpu_tvd_rk(ctx, dt, t_step == t_step_stop), "mfc_gpu_tvd_rk");
    if (t_step == t_step_stop) break;
    if ((mytime + dt) >= finaltime) dt = finaltime - mytime;
    t_step = t_step + 1;
    if ((t_step - t_step_start) % t_step_save == 0 || t_step == t_step_stop) {
      uint32_t flags = 0;
      check(mfc_gpu_status(ctx, &flags, 0), "mfc_gpu_status");
      if (flags & MFC_FLAG_NAN) {
        fprintf(stderr, "NaN at t_step %d\n", t_step);
        return 1;
      }
      for (int i = 0; i < S; ++i)
        check(mfc_gpu_download(ctx, i, sf + i * per_var + origin, nx_pad, 0), "mfc_gpu_download");
      const int32_t ts32 = t_step;
      write_exact(out, &ts32, sizeof ts32);
      write_exact(out, sf, sizeof(double) * (size_t)(S * per_var));
    }
  }
  write_exact(out, &dt, sizeof dt);
  fclose(out);
  check(mfc_gpu_finalize(ctx), "mfc_gpu_finalize");
  free(sf);
  free(x_cb);
  free(y_cb);
  return 0;
}
