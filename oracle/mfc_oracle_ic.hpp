// pre_process restatement for the oracle (test infrastructure only).
//
// Uniform grid (src/pre_process/m_grid.f90:54-70), optionally stretched
// (m_grid.f90:72-90), the patch geometries of
// src/pre_process/m_create_patches.fpp:47-534 -- line segment (1), circle
// (2), rectangle (3), sweep line (4), ellipse (5), isentropic vortex (6), 2-D
// analytical (7), 1-D analytical (15), varcircle (18) -- plus sphere (8) and
// cuboid (9), the 3-D analogues that the reference does not have, the
// smoothed-patch blend of src/pre_process/m_assign_patches.fpp:54-165 and
// prim -> cons of src/common/m_variables_conversion.fpp:385-443.
#pragma once

#include <cmath>
#include <vector>

#include "mfc_oracle.hpp"

namespace mfc_oracle {

constexpr int kMaxPatches = 10;

extern "C" {
struct mfo_patch {
  int geometry;
  double x_centroid, y_centroid, z_centroid;
  double length_x, length_y, length_z;
  double radius;
  int smoothen;
  int smooth_patch_id;  // 1-based, as in the case file
  double smooth_coeff;
  int alter_patch[kMaxPatches + 1];  // alter_patch(0:num_patches)
  double alpha_rho[kMaxFluids];
  double alpha[kMaxFluids];
  double vel[3];
  double pres;
  double normal[3];  // sweep line
  double radii[3];   // ellipse
  double epsilon;    // varcircle
};
}

inline void uniform_grid(int m, double beg, double end, double* cb, double* cc, double* d) {
  const double dx = (end - beg) / double(m + 1);
  for (int i = 0; i <= m; ++i) {
    cc[i] = beg + 5e-1 * dx * double(2 * i + 1);
    cb[i] = beg + dx * double(i);  // x_cb(i-1), stored at offset +1
  }
  cb[m + 1] = end;
  *d = dx;
}

// The hyperbolic stretching of m_grid.f90:72-90 applied to the m+2 cell
// boundaries cb (x_cb(-1:m)); the centres become the boundaries' midpoints
// and the spacing the smallest width.
inline void stretch_grid(int m, double a, double xa, double xb, int loops, double* cb, double* cc, double* d) {
  const double length = std::fabs(cb[m + 1] - cb[0]);
  for (int i = 0; i <= m + 1; ++i) cb[i] = cb[i] / length;
  xa = xa / length;
  xb = xb / length;
  for (int l = 0; l < loops; ++l)
    for (int i = 0; i <= m + 1; ++i)
      cb[i] = cb[i] / a *
              (a + std::log(std::cosh(a * (cb[i] - xa))) + std::log(std::cosh(a * (cb[i] - xb))) -
               2.0 * std::log(std::cosh(a * (xb - xa) / 2.0)));
  for (int i = 0; i <= m + 1; ++i) cb[i] = cb[i] * length;
  double w = cb[1] - cb[0];
  for (int i = 0; i <= m; ++i) {
    cc[i] = (cb[i + 1] + cb[i]) / 2.0;
    if (cb[i + 1] - cb[i] < w) w = cb[i + 1] - cb[i];
  }
  *d = w;
}

inline int generate_ic(const Params& P, const mfo_patch* pt, int npatch, double x_beg, double x_end, double y_beg,
                       double y_end, double z_beg, double z_end, const double* stretch, double* x_cb, double* y_cb,
                       double* z_cb, double* cons_out) {
  if (npatch < 1 || npatch > kMaxPatches) return 1;
  const int m = P.m, n = P.n, p = P.p, S = P.sys_size(), nf = P.num_fluids, nd = P.num_dims();
  for (int ip = 0; ip < npatch; ++ip) {  // x-slabs in any dimension; 2-D patches need n > 0, 3-D ones p > 0
    const int g = pt[ip].geometry;
    const bool ok = g == 1 || g == 15 || ((g >= 2 && g <= 7) || g == 18 ? nd >= 2 : (g == 8 || g == 9) && nd == 3);
    if (!ok) return 2;
  }
  const int E = P.E_idx() - 1, ab = P.adv_beg() - 1, mb = P.mom_beg() - 1;
  std::vector<double> xcc(m + 1), ycc(n + 1), zcc(p + 1);
  double dx = 0, dy = 0, dz = 0;
  uniform_grid(m, x_beg, x_end, x_cb, xcc.data(), &dx);
  if (n > 0) uniform_grid(n, y_beg, y_end, y_cb, ycc.data(), &dy);
  if (stretch && stretch[3] >= 1)
    stretch_grid(m, stretch[0], stretch[1], stretch[2], (int)stretch[3], x_cb, xcc.data(), &dx);
  if (stretch && stretch[7] >= 1 && n > 0)
    stretch_grid(n, stretch[4], stretch[5], stretch[6], (int)stretch[7], y_cb, ycc.data(), &dy);
  if (p > 0) uniform_grid(p, z_beg, z_end, z_cb, zcc.data(), &dz);
  const long cells = long(m + 1) * (n + 1) * (p + 1);
  std::vector<double> prim((size_t)(S * cells), 0.0);
  std::vector<int> pid((size_t)cells, 0);
  auto Q = [&](int v, long c) -> double& { return prim[(size_t)(v * cells + c)]; };

  auto assign = [&](int ip, long c, double eta) {
    const mfo_patch& a = pt[ip];
    const mfo_patch& sm = pt[a.smooth_patch_id - 1];
    (void)sm;  // the smoothing patch's mixture is computed but unused in the reference
    double orig[32];
    for (int v = 0; v < S; ++v) orig[v] = Q(v, c);
    for (int f = 0; f < nf; ++f) Q(f, c) = eta * a.alpha_rho[f] + (1.0 - eta) * orig[f];
    for (int f = 0; f < nf; ++f) Q(ab + f, c) = eta * a.alpha[f] + (1.0 - eta) * orig[ab + f];
    for (int d = 0; d < nd; ++d) Q(mb + d, c) = (eta * a.vel[d] + (1.0 - eta) * orig[mb + d]);
    Q(E, c) = (eta * a.pres + (1.0 - eta) * orig[E]);
    if (1.0 - eta < 1e-16) pid[(size_t)c] = ip + 1;
  };

  for (int ip = 0; ip < npatch; ++ip) {
    const mfo_patch& a = pt[ip];
    for (int k = 0; k <= p; ++k)
      for (int j = 0; j <= n; ++j)
        for (int i = 0; i <= m; ++i) {
          const long c = i + long(m + 1) * (j + long(n + 1) * k);
          const int cur = pid[(size_t)c];
          const bool alter = cur >= 0 && cur <= kMaxPatches && a.alter_patch[cur];
          double eta = 1.0;
          bool hit = false;
          const double x = xcc[i], y = n > 0 ? ycc[j] : 0.0, z = p > 0 ? zcc[k] : 0.0;
          const double xc = a.x_centroid, yc = a.y_centroid;
          const int g = a.geometry;
          if (g == 1 || g == 15) {  // s_line_segment, s_1D_analytical
            hit = (xc - 0.5 * a.length_x) <= x && (xc + 0.5 * a.length_x) >= x && alter;
          } else if (g == 3 || g == 7 || g == 9) {  // s_rectangle, s_2D_analytical
            hit = (xc - 0.5 * a.length_x) <= x && (xc + 0.5 * a.length_x) >= x &&
                  (yc - 0.5 * a.length_y) <= y && (yc + 0.5 * a.length_y) >= y && alter;
            if (g == 9)
              hit = hit && (a.z_centroid - 0.5 * a.length_z) <= z && (a.z_centroid + 0.5 * a.length_z) >= z;
          } else if (g == 2 || g == 8) {  // s_circle
            double r2 = (x - xc) * (x - xc) + (y - yc) * (y - yc);
            double h = dx < dy ? dx : dy;
            if (g == 8) {
              r2 = r2 + (z - a.z_centroid) * (z - a.z_centroid);
              h = h < dz ? h : dz;
            }
            if (a.smoothen) eta = std::tanh(a.smooth_coeff / h * (std::sqrt(r2) - a.radius)) * (-0.5) + 0.5;
            hit = (r2 <= a.radius * a.radius && alter) || cur == a.smooth_patch_id;
          } else if (g == 4) {  // s_sweep_line (m_create_patches.fpp:323-371)
            const double A = a.normal[0], B = a.normal[1];
            const double C = -A * xc - B * yc;
            const double lin = A * x + B * y + C;
            if (a.smoothen)
              eta = 5e-1 + 5e-1 * std::tanh(a.smooth_coeff / (dx < dy ? dx : dy) * lin / std::sqrt(A * A + B * B));
            hit = (lin >= 0.0 && alter) || cur == a.smooth_patch_id;
          } else if (g == 5) {  // s_ellipse (m_create_patches.fpp:202-250)
            const double u = (x - xc) / a.radii[0], v = (y - yc) / a.radii[1];
            const double r2 = u * u + v * v;
            if (a.smoothen) eta = std::tanh(a.smooth_coeff / (dx < dy ? dx : dy) * (std::sqrt(r2) - 1.0)) * (-0.5) + 0.5;
            hit = (r2 <= 1.0 && alter) || cur == a.smooth_patch_id;
          } else if (g == 6) {  // s_isentropic_vortex (m_create_patches.fpp:379-419)
            hit = (x - xc) * (x - xc) + (y - yc) * (y - yc) <= a.radius * a.radius && alter;
          } else if (g == 18) {  // s_varcircle (m_create_patches.fpp:151-194)
            const double r = std::sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc));
            hit = r <= a.radius + a.epsilon / 2.0 && r >= a.radius - a.epsilon / 2.0 && alter;
          } else {
            return 2;
          }
          if (hit && (g == 7 || g == 15)) {
            // pressure bump at the cell's right boundaries x_cb(i), y_cb(j)
            // (m_create_patches.fpp:462-464, 523-525)
            assign(ip, c, eta);
            const double xb = x_cb[i + 1] - xc;
            double s2 = xb * xb;
            if (g == 7) {
              const double yb = y_cb[j + 1] - yc;
              s2 = s2 + yb * yb;
            }
            Q(E, c) = Q(E, c) * (1.0 + 0.2 * std::exp(-1.0 * s2 / (2.0 * 0.005)));
            continue;
          }
          if (hit) assign(ip, c, eta);
        }
  }
  // prim -> cons
  for (long c = 0; c < cells; ++c) {
    double rho = 0, gam = 0, pinf = 0;
    for (int f = 0; f < nf; ++f) {
      rho = rho + Q(f, c);
      gam = gam + Q(ab + f, c) * P.gammas[f];
      pinf = pinf + Q(ab + f, c) * P.pi_infs[f];
    }
    for (int f = 0; f < nf; ++f) cons_out[f * cells + c] = Q(f, c);
    double dyn = 0;
    for (int d = 0; d < nd; ++d) {
      double mom = rho * Q(mb + d, c);
      cons_out[(mb + d) * cells + c] = mom;
      dyn = dyn + mom * Q(mb + d, c) / 2.0;
    }
    cons_out[E * cells + c] = gam * Q(E, c) + dyn + pinf;
    for (int f = 0; f < nf; ++f) cons_out[(ab + f) * cells + c] = Q(ab + f, c);
  }
  return 0;
}

}  // namespace mfc_oracle
