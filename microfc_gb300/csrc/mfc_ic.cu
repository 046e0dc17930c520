// Initial condition on the device: the reference's pre_process for the
// patch geometries the benchmark cases use, one thread per cell.
//
//   grid     x_cc(i) = beg + 0.5 dx (2i + 1), dx = (end - beg)/(m + 1)
//            (src/pre_process/m_grid.f90:54-70)
//   patches  line segment (1), circle (2), rectangle (3)
//            (src/pre_process/m_create_patches.fpp:47-313), sphere (8) and
//            cuboid (9) as their 3-D analogues; a circle or sphere with
//            `smoothen` blends with eta = 1/2 - 1/2 tanh(c/h (r - R)),
//            h = min(dx, dy), with dz too for a sphere
//            (m_create_patches.fpp:124-128)
//   blend    q = eta q_patch + (1 - eta) q_old on every primitive variable;
//            the cell joins the patch when 1 - eta < 1e-16
//            (m_assign_patches.fpp:54-165)
//   cons     alpha_rho, rho u, E = Gamma p + 1/2 rho |u|^2 + Pi, alpha
//            (src/common/m_variables_conversion.fpp:385-443)
//
// Patches are applied in order and only read the cell's own owner id, so
// cells are independent.  The unit is compiled without FMA contraction and
// follows the CPU pre_process's operation order; only tanh may differ from
// the host's libm in the last bit.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mfc_gpu.h"
#include "mfc_ic.h"

namespace mfc {
namespace {

struct IcParams {
  int n[3], nd, nf, np;
  int64_t sy, sz, sv;
  double beg[3], d[3], h2, h3;  // smallest spacing of x-y (circles) and x-y-z (spheres)
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
    const double x = I.beg[0] + 5e-1 * I.d[0] * double(2 * i + 1);
    const double y = nd > 1 ? I.beg[1] + 5e-1 * I.d[1] * double(2 * j + 1) : 0.0;
    const double z = nd > 2 ? I.beg[2] + 5e-1 * I.d[2] * double(2 * k + 1) : 0.0;
    double pr[2 * MFC_MAX_FLUIDS + 4];
    for (int v = 0; v < S; ++v) pr[v] = 0.0;
    int pid = 0;
    for (int ip = 0; ip < I.np; ++ip) {
      const mfc_patch& a = I.pt[ip];
      const bool alter = pid >= 0 && pid <= MFC_MAX_PATCHES && a.alter_patch[pid];
      double eta = 1.0;
      bool hit;
      if (a.geometry == 1) {
        hit = (a.x_centroid - 0.5 * a.length_x) <= x && (a.x_centroid + 0.5 * a.length_x) >= x && alter;
      } else if (a.geometry == 3 || a.geometry == 9) {
        hit = (a.x_centroid - 0.5 * a.length_x) <= x && (a.x_centroid + 0.5 * a.length_x) >= x &&
              (a.y_centroid - 0.5 * a.length_y) <= y && (a.y_centroid + 0.5 * a.length_y) >= y && alter;
        if (a.geometry == 9)
          hit = hit && (a.z_centroid - 0.5 * a.length_z) <= z && (a.z_centroid + 0.5 * a.length_z) >= z;
      } else {  // 2, 8 (checked on the host)
        double r2 = (x - a.x_centroid) * (x - a.x_centroid) + (y - a.y_centroid) * (y - a.y_centroid);
        if (a.geometry == 8) r2 = r2 + (z - a.z_centroid) * (z - a.z_centroid);
        const double h = a.geometry == 8 ? I.h3 : I.h2;
        if (a.smoothen) eta = tanh(a.smooth_coeff / h * (sqrt(r2) - a.radius)) * (-0.5) + 0.5;
        hit = (r2 <= a.radius * a.radius && alter) || pid == a.smooth_patch_id;
      }
      if (!hit) continue;
      for (int f = 0; f < nf; ++f) pr[f] = eta * a.alpha_rho[f] + (1.0 - eta) * pr[f];
      for (int f = 0; f < nf; ++f) pr[ab + f] = eta * a.alpha[f] + (1.0 - eta) * pr[ab + f];
      for (int d = 0; d < nd; ++d) pr[mb + d] = eta * a.vel[d] + (1.0 - eta) * pr[mb + d];
      pr[E] = eta * a.pres + (1.0 - eta) * pr[E];
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
  if (!patches || !domain) return "generate_ic: null patches or domain";
  if (num_patches < 1 || num_patches > MFC_MAX_PATCHES) return "generate_ic: num_patches must be 1..10";
  IcParams I{};
  I.nd = t.nd;
  I.nf = t.nf;
  I.np = num_patches;
  I.sy = t.sy;
  I.sz = t.sz;
  I.sv = t.sv;
  for (int d = 0; d < 3; ++d) {
    I.n[d] = d < t.nd ? t.n[d] : 1;
    if (d < t.nd) {
      if (!(domain[2 * d + 1] > domain[2 * d])) return "generate_ic: empty domain";
      I.beg[d] = domain[2 * d];
      I.d[d] = (domain[2 * d + 1] - domain[2 * d]) / double(I.n[d]);
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
    const bool ok = (g == 1) || ((g == 2 || g == 3) && t.nd >= 2) || ((g == 8 || g == 9) && t.nd == 3);
    if (!ok) return "generate_ic: patch " + std::to_string(ip + 1) + " has a geometry the grid does not support";
    // a circle or sphere also takes the cells owned by smooth_patch_id (the patch's own id by default)
    if ((g == 2 || g == 8) && (a.smooth_patch_id < 1 || a.smooth_patch_id > num_patches))
      return "generate_ic: smooth_patch_id out of range";
    I.pt[ip] = a;
  }
  const int64_t cells = (int64_t)I.n[0] * I.n[1] * I.n[2];
  const int64_t blocks = (cells + 255) / 256 < 152 * 32 ? (cells + 255) / 256 : 152 * 32;
  ic_kernel<<<(unsigned)blocks, 256, 0, stream>>>(I, t.q);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return std::string("generate_ic launch: ") + cudaGetErrorString(e);
  if (launches) ++*launches;
  return "";
}

}  // namespace mfc
