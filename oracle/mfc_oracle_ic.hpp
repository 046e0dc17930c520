// pre_process restatement for the oracle (test infrastructure only).
//
// Uniform grid (src/pre_process/m_grid.f90:54-70), the patch geometries the
// benchmark cases use -- line segment (1), circle (2), rectangle (3) from
// src/pre_process/m_create_patches.fpp:47-313, plus sphere (8) and cuboid (9),
// the 3-D analogues that the reference does not have -- the smoothed-patch
// blend of src/pre_process/m_assign_patches.fpp:54-165 and prim -> cons of
// src/common/m_variables_conversion.fpp:385-443.
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

inline int generate_ic(const Params& P, const mfo_patch* pt, int npatch, double x_beg, double x_end, double y_beg,
                       double y_end, double z_beg, double z_end, double* x_cb, double* y_cb, double* z_cb,
                       double* cons_out) {
  if (npatch < 1 || npatch > kMaxPatches) return 1;
  const int m = P.m, n = P.n, p = P.p, S = P.sys_size(), nf = P.num_fluids, nd = P.num_dims();
  const int E = P.E_idx() - 1, ab = P.adv_beg() - 1, mb = P.mom_beg() - 1;
  std::vector<double> xcc(m + 1), ycc(n + 1), zcc(p + 1);
  double dx = 0, dy = 0, dz = 0;
  uniform_grid(m, x_beg, x_end, x_cb, xcc.data(), &dx);
  if (n > 0) uniform_grid(n, y_beg, y_end, y_cb, ycc.data(), &dy);
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
          if (a.geometry == 1) {
            hit = (a.x_centroid - 0.5 * a.length_x) <= x && (a.x_centroid + 0.5 * a.length_x) >= x && alter;
          } else if (a.geometry == 3 || a.geometry == 9) {
            hit = (a.x_centroid - 0.5 * a.length_x) <= x && (a.x_centroid + 0.5 * a.length_x) >= x &&
                  (a.y_centroid - 0.5 * a.length_y) <= y && (a.y_centroid + 0.5 * a.length_y) >= y && alter;
            if (a.geometry == 9)
              hit = hit && (a.z_centroid - 0.5 * a.length_z) <= z && (a.z_centroid + 0.5 * a.length_z) >= z;
          } else if (a.geometry == 2 || a.geometry == 8) {
            double r2 = (x - a.x_centroid) * (x - a.x_centroid) + (y - a.y_centroid) * (y - a.y_centroid);
            double h = dx < dy ? dx : dy;
            if (a.geometry == 8) {
              r2 = r2 + (z - a.z_centroid) * (z - a.z_centroid);
              h = h < dz ? h : dz;
            }
            if (a.smoothen) eta = std::tanh(a.smooth_coeff / h * (std::sqrt(r2) - a.radius)) * (-0.5) + 0.5;
            hit = (r2 <= a.radius * a.radius && alter) || cur == a.smooth_patch_id;
          } else {
            return 2;
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
