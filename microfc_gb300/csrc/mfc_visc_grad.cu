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
// Kernels per RK stage prepare those face values from the stage input; the
// stage kernel's viscous flux reads them (ViscParams::fg).  The velocities
// are FP64 in every precision; the two reconstructions run in RT: FP64 for
// the plain path (the arithmetic and operation order of the oracle, so the
// result is bit-identical to it), FP32 for the split and gated paths, whose
// stage kernels take the gradients in FP32 anyway.  The buffers stay FP64
// (an FP32 value widened, so the stage kernel narrows it back exactly).
// Cells outside the domain take the boundary conditions by index mapping,
// as everywhere else.
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

// The WENO coefficients of cell `cell` along direction d: FP64 from the
// context's grid tables, FP32 from the preparation's own table cft of that
// direction ([kNumCoef][n + 2 kCoefPad], then the inverse cell widths).
template <class RT>
__device__ __forceinline__ void coef_of(const DevParams& P, const float* __restrict__ cft, int d, int cell,
                                        RT (&c)[kCoefRec]) {
  const int gi = clamp_coef_index(cell, P.n[d]) + kCoefPad;
  if constexpr (sizeof(RT) == 4) {
    const int stride = P.n[d] + 2 * kCoefPad;
#pragma unroll
    for (int k = 0; k < kNumCoef; ++k) c[k] = __ldg(cft + k * stride + gi);
  } else {
#pragma unroll
    for (int k = 0; k < kNumCoef; ++k) c[k] = __ldg(P.coef[d] + k * P.cstride[d] + gi);
  }
}

// 1/ds of cell `cell` along direction d (w: the FP64 widths of the
// direction, cft: its FP32 table).
template <class RT>
__device__ __forceinline__ RT inverse_width(const DevParams& P, const double* __restrict__ w,
                                            const float* __restrict__ cft, int d, int cell) {
  const int gi = clamp_coef_index(cell, P.n[d]) + kCoefPad;
  if constexpr (sizeof(RT) == 4) return __ldg(cft + kNumCoef * (P.n[d] + 2 * kCoefPad) + gi);
  else return div_rn(1.0, divisor(__ldg(w + gi)));
}

// Step 1 on the ncol x nrow cells from (ib, jb): out[c*ND+d][row][col].
// B.w[d]: the cell widths ds of direction d for cells -kCoefPad ..
// n-1+kCoefPad; B.cf[d]: the FP32 table of the direction.
template <int ND, class RT>
__global__ void __launch_bounds__(256) visc_cell_gradients(const DevParams P, const ViscGradBuffers B,
                                                          const int vcol, const int vrow, const int ib, const int jb,
                                                          const int ncol, const int nrow, double* __restrict__ out) {
  const double* __restrict__ vel = B.vel;
  const int64_t cells = (int64_t)ncol * nrow;
  const int64_t vplane = (int64_t)vcol * vrow;
  const RT eps = narrow<RT>(P.weno_eps);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cells; t += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(t % ncol), row = (int)(t / ncol);
    const int i = ib + col, j = jb + row;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      const int cell = d == 0 ? i : j;
      RT cf[kCoefRec];
      coef_of(P, B.cf[d], d, cell, cf);
      const RT inv = inverse_width<RT>(P, B.w[d], B.cf[d], d, cell);
#pragma unroll
      for (int c = 0; c < ND; ++c) {
        RT st[5];
#pragma unroll
        for (int o = 0; o < 5; ++o) {
          const int vi = i + (d == 0 ? o - 2 : 0) + 5, vj = ND > 1 ? j + (d == 1 ? o - 2 : 0) + 5 : 0;
          st[o] = narrow<RT>(__ldg(vel + c * vplane + (int64_t)vj * vcol + vi));
        }
        RT vl, vr;
        weno_cell<5, RT>(cf, st, eps, vl, vr);
        out[((int64_t)(c * ND + d) * nrow + row) * ncol + col] = widen(inv * (vr - vl));
      }
    }
  }
}

// Step 2: the face values, from the cell gradients G of the region
// ([c*ND+d][grow][gcol], origin (gib, gjb)).  Each cell's gradients are
// WENO-reconstructed once, both face values together (weno_cell: the same
// operations as the one-sided form, so the same bits), and face F (between
// cells F-1 and F, F = 0 .. n_dir) takes 0.5 (right value of cell F-1 + left
// value of cell F).  out[c*ND+d][...], the face index F along dir.
//
// x faces: a warp covers 31 faces of one row.  Lane L reconstructs cell
// base + L - 1 (clamped to the last cell needed, nx); lanes 1..31 write face
// base + L - 1 with the right value of lane L-1 (shuffle) and their own left
// value.  Every lane of a warp runs the same iterations (the loop bound is
// per warp), so the full-mask shuffles are safe.
template <int ND, class RT>
__global__ void __launch_bounds__(256) visc_face_gradients_x(const DevParams P, const float* __restrict__ cft,
                                                            const double* __restrict__ G, const int gib,
                                                            const int gjb, const int gncol, const int gnrow,
                                                            double* __restrict__ out) {
  const int nx = P.n[0], nf = nx + 1;
  const int nl = ND > 1 ? P.n[1] : 1;  // rows
  const int chunks = (nf + 30) / 31;
  const int64_t warps = (int64_t)chunks * nl;
  const int64_t plane_out = (int64_t)nf * nl;
  const int lane = threadIdx.x & 31;
  const RT eps = narrow<RT>(P.weno_eps);
  const int64_t stride = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < warps; w += stride) {
    const int l = (int)(w / chunks), base = (int)(w % chunks) * 31;
    const int F = base + lane - 1;   // this lane's face (written by lanes 1..31 while F < nf)
    const int cell = min(F, nx);     // and its cell, -1 .. nx
    RT cf[kCoefRec];
    coef_of(P, cft, 0, cell, cf);
    const double* row = G + (int64_t)(l - gjb) * gncol + (cell - gib);
#pragma unroll
    for (int k = 0; k < ND * ND; ++k) {
      RT st[5];
#pragma unroll
      for (int o = 0; o < 5; ++o) st[o] = narrow<RT>(__ldg(row + (int64_t)k * gnrow * gncol + (o - 2)));
      RT vl, vr;
      weno_cell<5, RT>(cf, st, eps, vl, vr);
      const RT right = __shfl_up_sync(0xffffffffu, vr, 1);  // face value of the cell before
      if (lane >= 1 && F < nf) out[k * plane_out + (int64_t)l * nf + F] = widen(RT(0.5) * (right + vl));
    }
  }
}

// y faces: a thread walks one column through a run of R faces (cells
// f0-1 .. f0+R-1), carrying each cell's right values to the next face.
template <int ND, class RT, int R>
__global__ void __launch_bounds__(256) visc_face_gradients_y(const DevParams P, const float* __restrict__ cft,
                                                            const double* __restrict__ G, const int gib,
                                                            const int gjb, const int gncol, const int gnrow,
                                                            double* __restrict__ out) {
  const int nx = P.n[0], ny = P.n[1], nf = ny + 1;
  const int runs = (nf + R - 1) / R;
  const int64_t items = (int64_t)nx * runs;
  const int64_t plane_out = (int64_t)nf * nx;
  const RT eps = narrow<RT>(P.weno_eps);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < items; t += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(t % nx), f0 = (int)(t / nx) * R;
    RT prev[ND * ND];
#pragma unroll 1
    for (int j = -1; j < R; ++j) {
      const int cell = f0 + j;  // -1 .. ny
      if (cell > ny) break;
      RT cf[kCoefRec];
      coef_of(P, cft, 1, cell, cf);
      const double* col = G + (int64_t)(cell - gjb) * gncol + (l - gib);
#pragma unroll
      for (int k = 0; k < ND * ND; ++k) {
        RT st[5];
#pragma unroll
        for (int o = 0; o < 5; ++o) st[o] = narrow<RT>(__ldg(col + ((int64_t)k * gnrow + (o - 2)) * gncol));
        RT vl, vr;
        weno_cell<5, RT>(cf, st, eps, vl, vr);
        if (j >= 0) out[k * plane_out + (int64_t)cell * nx + l] = widen(RT(0.5) * (prev[k] + vl));
        prev[k] = vr;
      }
    }
  }
}

template <int ND, int NF, class RT>
cudaError_t launch_all(const DevParams& P, const ViscGradBuffers& B, const double* q, cudaStream_t st) {
  const int nx = P.n[0], ny = ND > 1 ? P.n[1] : 1;
  auto grid = [](int64_t items) { return (unsigned)std::min<int64_t>((items + 255) / 256, 152 * 16); };
  const int vcol = nx + 10, vrow = ND > 1 ? ny + 10 : 1;
  visc_velocities<ND, NF><<<grid((int64_t)vcol * vrow), 256, 0, st>>>(P, q, vcol, vrow, B.vel);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // G on x = -3 .. nx+2 (and y = -3 .. ny+2)
  const int gcol = nx + 6, grow = ND > 1 ? ny + 6 : 1, gjb = ND > 1 ? -3 : 0;
  visc_cell_gradients<ND, RT><<<grid((int64_t)gcol * grow), 256, 0, st>>>(P, B, vcol, vrow, -3, gjb, gcol, grow,
                                                                           B.g);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int64_t xwarps = (int64_t)((nx + 1 + 30) / 31) * ny;
  visc_face_gradients_x<ND, RT><<<grid(32 * xwarps), 256, 0, st>>>(P, B.cf[0], B.g, -3, gjb, gcol, grow, B.fg[0]);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if constexpr (ND > 1) {
    constexpr int R = sizeof(RT) == 8 ? 8 : 4;  // faces per thread (FP32 wants more threads)
    visc_face_gradients_y<ND, RT, R><<<grid((int64_t)nx * ((ny + 1 + R - 1) / R)), 256, 0, st>>>(
        P, B.cf[1], B.g, -3, gjb, gcol, grow, B.fg[1]);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace

cudaError_t visc_gradients_launch(int nd, int nf, bool fp32, const DevParams& P, const ViscGradBuffers& B,
                                  const double* q, cudaStream_t st) {
  if (fp32) {
    if (B.cf[0] == nullptr || (nd > 1 && B.cf[1] == nullptr)) return cudaErrorInvalidValue;
    if (nd == 1 && nf == 1) return launch_all<1, 1, float>(P, B, q, st);
    if (nd == 1 && nf == 2) return launch_all<1, 2, float>(P, B, q, st);
    if (nd == 2 && nf == 1) return launch_all<2, 1, float>(P, B, q, st);
    if (nd == 2 && nf == 2) return launch_all<2, 2, float>(P, B, q, st);
  } else {
    if (nd == 1 && nf == 1) return launch_all<1, 1, double>(P, B, q, st);
    if (nd == 1 && nf == 2) return launch_all<1, 2, double>(P, B, q, st);
    if (nd == 2 && nf == 1) return launch_all<2, 1, double>(P, B, q, st);
    if (nd == 2 && nf == 2) return launch_all<2, 2, double>(P, B, q, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace mfc
