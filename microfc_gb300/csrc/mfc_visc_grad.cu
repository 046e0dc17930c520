// weno_Re_flux = T: the velocity gradients of the viscous stresses from
// WENO reconstructions instead of finite differences.  The reference
// (m_viscous.fpp:176-216, 381-591; m_rhs.fpp:512-528; the averaging in
// s_compute_viscous_source_flux, m_riemann_solvers.fpp:683-902):
//
//   1. every velocity component u_c is WENO-reconstructed along each
//      direction d, and the cell-average gradient follows from the scalar
//      divergence theorem, G_cd = (1/ds) (u_c(right face) - u_c(left face));
//   2. every G_cd is WENO-reconstructed along the sweep direction, and the
//      face value is the mean of the right-face value of the cell before the
//      face and the left-face value of the cell after it.
//
// Kernels per RK stage prepare those face values from the stage input
// (plain FP64, the arithmetic and operation order of the oracle, so the
// result is bit-identical to it); the stage kernel's viscous flux reads them
// (ViscParams::fg).  Cells outside the domain take the boundary conditions
// by index mapping, as everywhere else.
//
// Regions (x0 = 0 .. nx-1, y0 = 0 .. ny-1 the interior):
//   x faces i+1/2, i = -1 .. nx-1, rows y0: need G on x = -3 .. nx+2, rows y0,
//     whose WENO along x reads u on x = -5 .. nx+4 and, for G_c1, along y on
//     rows -2 .. ny+1 (corner ghost cells);
//   y faces j+1/2, j = -1 .. ny-1, columns x0: need G on y = -3 .. ny+2,
//     columns x0.
// One launch computes G on the box x, y = -3 .. n+2 that holds both (each
// interior cell once; the 36 corner cells of the box are computed and not
// read), from the velocities of x, y = -5 .. n+4.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/mfc_gpu.h"
#include "mfc_launch.h"

namespace mfc {
namespace {

// Velocity component c of cell (i, j) of state q, with the boundary
// conditions (the reflected normal component negated), as cons_to_prim
// computes it.
template <int ND, int NF>
__device__ __forceinline__ double velocity(const DevParams& P, const double* __restrict__ q, int c, int i, int j) {
  bool fx = false, fy = false;
  const int gx = map_cell(i, P.n[0], P.bc_beg[0], P.bc_end[0], &fx);
  const int gy = ND > 1 ? map_cell(j, P.n[1], P.bc_beg[1], P.bc_end[1], &fy) : 0;
  const int64_t o = (int64_t)gy * P.sy + gx;
  double rho = 0.0;
#pragma unroll
  for (int f = 0; f < NF; ++f) rho = rho + __ldg(q + o + f * P.sv);
  rho = fmax(rho, 1e-16);
  double m = __ldg(q + o + (NF + c) * P.sv);
  if ((c == 0 && fx) || (c == 1 && fy)) m = -m;
  return div_rn(m, divisor(rho));
}

// The velocities of the cells x = -5 .. nx+4 (and y = -5 .. ny+4 in 2-D)
// once, into vel[c][row][col] (row = y + 5, col = x + 5), which every
// stencil of the cell gradients reads.
template <int ND, int NF>
__global__ void __launch_bounds__(256) visc_velocities(const DevParams P, const double* __restrict__ q,
                                                      const int ncol, const int nrow, double* __restrict__ vel) {
  const int64_t cells = (int64_t)ncol * nrow;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cells; t += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(t % ncol), row = (int)(t / ncol);
    const int i = col - 5, j = ND > 1 ? row - 5 : 0;
#pragma unroll
    for (int c = 0; c < ND; ++c) vel[(int64_t)c * cells + t] = velocity<ND, NF>(P, q, c, i, j);
  }
}

// The WENO coefficients of cell `cell` along direction d.
__device__ __forceinline__ void coef_of(const DevParams& P, int d, int cell, double (&c)[kCoefRec]) {
  const int gi = clamp_coef_index(cell, P.n[d]) + P.coff;
#pragma unroll
  for (int k = 0; k < kNumCoef; ++k) c[k] = __ldg(P.coef[d] + k * P.cstride[d] + gi);
}

// Step 1 on the ncol x nrow cells from (ib, jb): out[c*ND+d][row][col].
// w[d]: the cell widths ds of direction d for cells -kCoefPad .. n-1+kCoefPad.
template <int ND>
__global__ void __launch_bounds__(256) visc_cell_gradients(const DevParams P, const double* __restrict__ vel,
                                                          const int vcol, const int vrow,
                                                          const double* __restrict__ w0,
                                                          const double* __restrict__ w1, const int ib, const int jb,
                                                          const int ncol, const int nrow, double* __restrict__ out) {
  const int64_t cells = (int64_t)ncol * nrow;
  const int64_t vplane = (int64_t)vcol * vrow;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cells; t += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(t % ncol), row = (int)(t / ncol);
    const int i = ib + col, j = jb + row;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      const int cell = d == 0 ? i : j;
      double cf[kCoefRec];
      coef_of(P, d, cell, cf);
      const double* w = d == 0 ? w0 : w1;
      const double inv = div_rn(1.0, divisor(__ldg(w + clamp_coef_index(cell, P.n[d]) + kCoefPad)));
#pragma unroll
      for (int c = 0; c < ND; ++c) {
        double st[5];
#pragma unroll
        for (int o = 0; o < 5; ++o) {
          const int vi = i + (d == 0 ? o - 2 : 0) + 5, vj = ND > 1 ? j + (d == 1 ? o - 2 : 0) + 5 : 0;
          st[o] = __ldg(vel + c * vplane + (int64_t)vj * vcol + vi);
        }
        double vl, vr;
        weno_cell<5, double>(cf, st, P.weno_eps, vl, vr);
        out[((int64_t)(c * ND + d) * nrow + row) * ncol + col] = inv * (vr - vl);
      }
    }
  }
}

// Step 2 along dir: faces f+1/2 for f = -1 .. n_dir-1 of the interior lines
// across, from the cell gradients G of the region ([c*ND+d][grow][gcol],
// origin (gib, gjb)): out[c*ND+d][...] with the face index f+1 along dir.
template <int ND, int DIR>
__global__ void __launch_bounds__(256) visc_face_gradients(const DevParams P, const double* __restrict__ G,
                                                          const int gib, const int gjb, const int gncol,
                                                          const int gnrow, double* __restrict__ out) {
  const int nf = P.n[DIR] + 1;                 // faces along dir
  const int nl = DIR == 0 ? (ND > 1 ? P.n[1] : 1) : P.n[0];  // lines across
  const int64_t items = (int64_t)nf * nl;
  const int64_t plane_out = items;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < items; t += (int64_t)gridDim.x * blockDim.x) {
    int f, l;  // face index (0 = face -1/2) and line
    if (DIR == 0) { f = (int)(t % nf); l = (int)(t / nf); }
    else { l = (int)(t % nl); f = (int)(t / nl); }
    const int cl = f - 1, cr = f;  // the cells before and after the face, along dir
    double cfl[kCoefRec], cfr[kCoefRec];
    coef_of(P, DIR, cl, cfl);
    coef_of(P, DIR, cr, cfr);
    // element (a along dir, line l) of field k of the region
    auto at = [&](int k, int a) -> double {
      const int i = DIR == 0 ? a : l, j = DIR == 0 ? l : a;
      return __ldg(G + ((int64_t)k * gnrow + (j - gjb)) * gncol + (i - gib));
    };
#pragma unroll
    for (int k = 0; k < ND * ND; ++k) {
      double sl[5], sr[5];
#pragma unroll
      for (int o = 0; o < 5; ++o) {
        sl[o] = at(k, cl + o - 2);
        sr[o] = at(k, cr + o - 2);
      }
      const double right = weno_cell_side<5, 1, double>(cfl, sl, P.weno_eps);  // face value of the cell before
      const double left = weno_cell_side<5, 0, double>(cfr, sr, P.weno_eps);   // and of the cell after
      const int64_t o = DIR == 0 ? (int64_t)l * nf + f : (int64_t)f * nl + l;
      out[k * plane_out + o] = 0.5 * (right + left);
    }
  }
}

template <int ND, int NF>
cudaError_t launch_all(const DevParams& P, const ViscGradBuffers& B, const double* q, cudaStream_t st) {
  const int nx = P.n[0], ny = ND > 1 ? P.n[1] : 1;
  auto grid = [](int64_t items) { return (unsigned)std::min<int64_t>((items + 255) / 256, 152 * 16); };
  const int vcol = nx + 10, vrow = ND > 1 ? ny + 10 : 1;
  visc_velocities<ND, NF><<<grid((int64_t)vcol * vrow), 256, 0, st>>>(P, q, vcol, vrow, B.vel);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // G on x = -3 .. nx+2 (and y = -3 .. ny+2)
  const int gcol = nx + 6, grow = ND > 1 ? ny + 6 : 1, gjb = ND > 1 ? -3 : 0;
  visc_cell_gradients<ND><<<grid((int64_t)gcol * grow), 256, 0, st>>>(P, B.vel, vcol, vrow, B.w[0], B.w[1], -3, gjb,
                                                                       gcol, grow, B.g);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  visc_face_gradients<ND, 0><<<grid((int64_t)(nx + 1) * ny), 256, 0, st>>>(P, B.g, -3, gjb, gcol, grow, B.fg[0]);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if constexpr (ND > 1) {
    visc_face_gradients<ND, 1><<<grid((int64_t)nx * (ny + 1)), 256, 0, st>>>(P, B.g, -3, gjb, gcol, grow, B.fg[1]);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace

cudaError_t visc_gradients_launch(int nd, int nf, const DevParams& P, const ViscGradBuffers& B, const double* q,
                                  cudaStream_t st) {
  if (nd == 1 && nf == 1) return launch_all<1, 1>(P, B, q, st);
  if (nd == 1 && nf == 2) return launch_all<1, 2>(P, B, q, st);
  if (nd == 2 && nf == 1) return launch_all<2, 1>(P, B, q, st);
  if (nd == 2 && nf == 2) return launch_all<2, 2>(P, B, q, st);
  return cudaErrorInvalidValue;
}

}  // namespace mfc
