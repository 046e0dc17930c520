// Initial condition on the device: the reference's pre_process, one thread
// per cell.
//
//   grid     x_cc(i) = beg + 0.5 dx (2i + 1), dx = (end - beg)/(m + 1)
//            (src/pre_process/m_grid.f90:54-70) over a domain, or the
//            context's own cell boundaries with x_cc(i) = (x_cb(i) +
//            x_cb(i-1))/2 and dx the smallest width, as pre_process sets
//            them on a stretched grid (m_grid.f90:72-90)
//   patches  line segment (1), circle (2), rectangle (3), sweep line (4),
//            ellipse (5), isentropic vortex (6), 2-D analytical (7), 1-D
//            analytical (15), varcircle (18)
//            (src/pre_process/m_create_patches.fpp:47-534), sphere (8) and
//            cuboid (9) as the 3-D analogues of 2 and 3; a circle or sphere
//            with `smoothen` blends with eta = 1/2 - 1/2 tanh(c/h (r - R)),
//            h = min(dx, dy), with dz too for a sphere
//            (m_create_patches.fpp:124-128), an ellipse with the same form
//            in its scaled radius, a sweep line with 1/2 + 1/2 tanh of the
//            signed distance; the analytical patches multiply the pressure
//            by 1 + 0.2 exp(-s^2/0.01), s the distance of the cell's right
//            boundary corner from the centroid
//   blend    q = eta q_patch + (1 - eta) q_old on every primitive variable;
//            the cell joins the patch when 1 - eta < 1e-16
//            (m_assign_patches.fpp:54-165)
//   cons     alpha_rho, rho u, E = Gamma p + 1/2 rho |u|^2 + Pi, alpha
//            (src/common/m_variables_conversion.fpp:385-443)
//
// Patches are applied in order and only read the cell's own owner id, so
// cells are independent.  The unit is compiled without FMA contraction and
// follows the CPU pre_process's operation order; only tanh and exp may
// differ from the host's libm in the last bit.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mfc_gpu.h"
#include "mfc_ic.h"

namespace mfc {
namespace {

struct IcParams {
  int n[3], nd, nf, np;
  int64_t sy, sz, sv;
  double beg[3], end[3], d[3], h2, h3;  // smallest spacing of x-y (circles) and x-y-z (spheres)
  const double* cb[3];                  // device cell boundaries (m+2 values), or null: uniform
  double gammas[MFC_MAX_FLUIDS], pi_infs[MFC_MAX_FLUIDS];
  mfc_patch pt[MFC_MAX_PATCHES];
};

__global__ void ic_kernel(const __grid_constant__ IcParams I, double* __restrict__ q) {
  const int64_t cells = (int64_t)I.n[0] * I.n[1] * I.n[2];
  const int nf = I.nf, nd = I.nd;
  const int mb = nf, E = nf + nd, ab = nf + nd + 1, S = 2 * nf + nd + 1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % I.n[0]);
    const int j = (int)((c / I.n[0]) % I.n[1]);
    const int k = (int)(c / ((int64_t)I.n[0] * I.n[1]));
    // cell centre and right boundary x_cb(i) along direction d
    auto centre = [&](int d, int l) {
      return I.cb[d] ? (I.cb[d][l + 1] + I.cb[d][l]) / 2.0 : I.beg[d] + 5e-1 * I.d[d] * double(2 * l + 1);
    };
    auto right = [&](int d, int l) {
      return I.cb[d] ? I.cb[d][l + 1] : (l == I.n[d] - 1 ? I.end[d] : I.beg[d] + I.d[d] * double(l + 1));
    };
    const double x = centre(0, i);
    const double y = nd > 1 ? centre(1, j) : 0.0;
    const double z = nd > 2 ? centre(2, k) : 0.0;
    double pr[2 * MFC_MAX_FLUIDS + 4];
    for (int v = 0; v < S; ++v) pr[v] = 0.0;
    int pid = 0;
    for (int ip = 0; ip < I.np; ++ip) {
      const mfc_patch& a = I.pt[ip];
      const bool alter = pid >= 0 && pid <= MFC_MAX_PATCHES && a.alter_patch[pid];
      double eta = 1.0;
      bool hit;
      const double xc = a.x_centroid, yc = a.y_centroid;
      const int g = a.geometry;
      if (g == 1 || g == 15) {
        hit = (xc - 0.5 * a.length_x) <= x && (xc + 0.5 * a.length_x) >= x && alter;
      } else if (g == 3 || g == 7 || g == 9) {
        hit = (xc - 0.5 * a.length_x) <= x && (xc + 0.5 * a.length_x) >= x && (yc - 0.5 * a.length_y) <= y &&
              (yc + 0.5 * a.length_y) >= y && alter;
        if (g == 9) hit = hit && (a.z_centroid - 0.5 * a.length_z) <= z && (a.z_centroid + 0.5 * a.length_z) >= z;
      } else if (g == 2 || g == 8) {
        double r2 = (x - xc) * (x - xc) + (y - yc) * (y - yc);
        if (g == 8) r2 = r2 + (z - a.z_centroid) * (z - a.z_centroid);
        const double h = g == 8 ? I.h3 : I.h2;
        if (a.smoothen) eta = tanh(a.smooth_coeff / h * (sqrt(r2) - a.radius)) * (-0.5) + 0.5;
        hit = (r2 <= a.radius * a.radius && alter) || pid == a.smooth_patch_id;
      } else if (g == 4) {  // sweep line a x + b y + c >= 0 through the centroid
        const double A = a.normal[0], B = a.normal[1];
        const double C = -A * xc - B * yc;
        const double lin = A * x + B * y + C;
        if (a.smoothen) eta = 5e-1 + 5e-1 * tanh(a.smooth_coeff / I.h2 * lin / sqrt(A * A + B * B));
        hit = (lin >= 0.0 && alter) || pid == a.smooth_patch_id;
      } else if (g == 5) {  // ellipse
        const double u = (x - xc) / a.radii[0], v = (y - yc) / a.radii[1];
        const double r2 = u * u + v * v;
        if (a.smoothen) eta = tanh(a.smooth_coeff / I.h2 * (sqrt(r2) - 1.0)) * (-0.5) + 0.5;
        hit = (r2 <= 1.0 && alter) || pid == a.smooth_patch_id;
      } else if (g == 6) {  // isentropic vortex: an unsmoothed disc
        hit = (x - xc) * (x - xc) + (y - yc) * (y - yc) <= a.radius * a.radius && alter;
      } else {  // 18 (checked on the host): annulus of thickness epsilon
        const double r = sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc));
        hit = r <= a.radius + a.epsilon / 2.0 && r >= a.radius - a.epsilon / 2.0 && alter;
      }
      if (!hit) continue;
      for (int f = 0; f < nf; ++f) pr[f] = eta * a.alpha_rho[f] + (1.0 - eta) * pr[f];
      for (int f = 0; f < nf; ++f) pr[ab + f] = eta * a.alpha[f] + (1.0 - eta) * pr[ab + f];
      for (int d = 0; d < nd; ++d) pr[mb + d] = eta * a.vel[d] + (1.0 - eta) * pr[mb + d];
      pr[E] = eta * a.pres + (1.0 - eta) * pr[E];
      if (g == 7 || g == 15) {
        // distance of the cell's right boundaries x_cb(i), y_cb(j) from the centroid
        const double xb = right(0, i) - xc;
        double s2 = xb * xb;
        if (g == 7) {
          const double yb = right(1, j) - yc;
          s2 = s2 + yb * yb;
        }
        pr[E] = pr[E] * (1.0 + 0.2 * exp(-1.0 * s2 / (2.0 * 0.005)));
      }
      if (1.0 - eta < 1e-16) pid = ip + 1;
    }
    double rho = 0.0, gam = 0.0, pinf = 0.0;
    for (int f = 0; f < nf; ++f) {
      rho = rho + pr[f];
      gam = gam + pr[ab + f] * I.gammas[f];
      pinf = pinf + pr[ab + f] * I.pi_infs[f];
    }
    double* out = q + (int64_t)k * I.sz + (int64_t)j * I.sy + i;
    for (int f = 0; f < nf; ++f) out[f * I.sv] = pr[f];
    double dyn = 0.0;
    for (int d = 0; d < nd; ++d) {
      const double mom = rho * pr[mb + d];
      out[(mb + d) * I.sv] = mom;
      dyn = dyn + mom * pr[mb + d] / 2.0;
    }
    out[E * I.sv] = gam * pr[E] + dyn + pinf;
    for (int f = 0; f < nf; ++f) out[(ab + f) * I.sv] = pr[ab + f];
  }
}

}  // namespace

std::string generate_ic(const IcTarget& t, const mfc_patch* patches, int num_patches, const double* domain,
                        cudaStream_t stream, int64_t* launches) {
  if (!patches) return "generate_ic: null patches";
  if (num_patches < 1 || num_patches > MFC_MAX_PATCHES) return "generate_ic: num_patches must be 1..10";
  IcParams I{};
  I.nd = t.nd;
  I.nf = t.nf;
  I.np = num_patches;
  I.sy = t.sy;
  I.sz = t.sz;
  I.sv = t.sv;
  size_t cb_total = 0;
  for (int d = 0; d < 3; ++d) {
    I.n[d] = d < t.nd ? t.n[d] : 1;
    if (d >= t.nd) continue;
    if (domain) {
      if (!(domain[2 * d + 1] > domain[2 * d])) return "generate_ic: empty domain";
      I.beg[d] = domain[2 * d];
      I.end[d] = domain[2 * d + 1];
      I.d[d] = (domain[2 * d + 1] - domain[2 * d]) / double(I.n[d]);
    } else {
      if (!t.cb[d]) return "generate_ic: no domain and no cell boundaries";
      double w = t.cb[d][1] - t.cb[d][0];
      for (int l = 1; l < I.n[d]; ++l) w = t.cb[d][l + 1] - t.cb[d][l] < w ? t.cb[d][l + 1] - t.cb[d][l] : w;
      if (!(w > 0.0)) return "generate_ic: cell boundaries must increase";
      I.d[d] = w;
      cb_total += (size_t)I.n[d] + 1;
    }
  }
  I.h2 = t.nd > 1 ? (I.d[0] < I.d[1] ? I.d[0] : I.d[1]) : I.d[0];
  I.h3 = t.nd > 2 ? (I.h2 < I.d[2] ? I.h2 : I.d[2]) : I.h2;
  for (int f = 0; f < t.nf; ++f) {
    I.gammas[f] = t.gammas[f];
    I.pi_infs[f] = t.pi_infs[f];
  }
  for (int ip = 0; ip < num_patches; ++ip) {
    const mfc_patch& a = patches[ip];
    const int g = a.geometry;
    // x-slabs in any dimension; 2-D patches (z-independent in 3-D) need n > 0, spheres and cuboids p > 0
    const bool ok = g == 1 || g == 15 || (((g >= 2 && g <= 7) || g == 18) && t.nd >= 2) ||
                    ((g == 8 || g == 9) && t.nd == 3);
    if (!ok) return "generate_ic: patch " + std::to_string(ip + 1) + " has a geometry the grid does not support";
    // a patch that blends also takes the cells owned by smooth_patch_id (the patch's own id by default)
    if ((g == 2 || g == 4 || g == 5 || g == 8) && (a.smooth_patch_id < 1 || a.smooth_patch_id > num_patches))
      return "generate_ic: smooth_patch_id out of range";
    if (g == 5 && !(a.radii[0] > 0.0 && a.radii[1] > 0.0))
      return "generate_ic: patch " + std::to_string(ip + 1) + ": ellipse semi-axes must be positive";
    if (g == 4 && a.normal[0] == 0.0 && a.normal[1] == 0.0)
      return "generate_ic: patch " + std::to_string(ip + 1) + ": sweep line normal is zero";
    I.pt[ip] = a;
  }
  double* cb_dev = nullptr;  // the cell boundaries of a grid given by them, for this launch
  if (cb_total) {
    cudaError_t e = cudaMalloc(&cb_dev, cb_total * sizeof(double));
    if (e != cudaSuccess) return std::string("generate_ic: ") + cudaGetErrorString(e);
    size_t off = 0;
    for (int d = 0; d < t.nd && e == cudaSuccess; ++d) {
      e = cudaMemcpyAsync(cb_dev + off, t.cb[d], ((size_t)I.n[d] + 1) * sizeof(double), cudaMemcpyHostToDevice,
                          stream);
      I.cb[d] = cb_dev + off;
      off += (size_t)I.n[d] + 1;
    }
    if (e != cudaSuccess) {
      cudaFree(cb_dev);
      return std::string("generate_ic: ") + cudaGetErrorString(e);
    }
  }
  const int64_t cells = (int64_t)I.n[0] * I.n[1] * I.n[2];
  const int64_t blocks = (cells + 255) / 256 < 152 * 32 ? (cells + 255) / 256 : 152 * 32;
  ic_kernel<<<(unsigned)blocks, 256, 0, stream>>>(I, t.q);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && cb_dev) e = cudaStreamSynchronize(stream);  // the launch reads cb_dev
  if (cb_dev) cudaFree(cb_dev);
  if (e != cudaSuccess) return std::string("generate_ic launch: ") + cudaGetErrorString(e);
  if (launches) ++*launches;
  return "";
}

}  // namespace mfc
