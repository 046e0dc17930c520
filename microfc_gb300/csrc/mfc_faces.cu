// Standalone WENO reconstruction and HLLC Riemann solve (mfc_gpu_weno,
// mfc_gpu_riemann): the two halves of a directional sweep that the fused
// stage kernel keeps in shared memory, exposed one at a time for hosts that
// call s_weno (src/simulation/m_weno.fpp:365-542) or s_hllc_riemann_solver
// (src/simulation/m_riemann_solvers.fpp:71-351) on their own -- a host that
// keeps its own flux assembly, or a verification harness that wants the face
// states.  Plain FP64 arithmetic, the same device functions and operation
// order as the fused kernels (mfc::weno_cell, mfc::hllc_face), so the results
// are those of the fused path and of the CPU reference's loops.
//
// Face window of direction d (s = m, n or p along d): cells j = -1 .. s+1
// along d, the interior cells across it; arrays [S][e2][e1][e0], x fastest,
// with e_d = s_d + 3 (cell j at index j + 1) and e_other = s_other + 1.
// Faces j + 1/2 for j = -1 .. s are stored at index j + 1 (extent s_d + 2).
#include <cuda_runtime.h>

#include <initializer_list>
#include <string>

#include "../../include/mfc_gpu.h"
#include "mfc_launch.h"

namespace mfc {
namespace {

// extents of the face window (cells = 2 extra along dir, faces = 1 extra)
struct Window {
  int e[3];
  __host__ __device__ int64_t count() const { return (int64_t)e[0] * e[1] * e[2]; }
};
Window face_window(const int (&n)[3], int dir, int extra) {
  Window w{{n[0], n[1], n[2]}};
  w.e[dir] += extra;
  return w;
}

// One cell of the window: the WENO values of all variables from the
// stencil's five primitive states.  The stencil cells are the reference's
// ghost cells where they leave the domain (boundary conditions by index
// mapping, bc -2 flips the normal momentum); each is converted cons -> prim
// as s_convert_conservative_to_primitive_variables does.
template <int ND, int NF, int DIR>
__global__ void weno_window_kernel(const DevParams P, const double* __restrict__ q, const int wo, const Window w,
                                   double* __restrict__ vl, double* __restrict__ vr) {
  using Q = Eqs<ND, NF>;
  constexpr int S = Q::S;
  const int64_t cells = w.count();
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x) {
    int cell[3] = {(int)(c % w.e[0]), (int)((c / w.e[0]) % w.e[1]), (int)(c / ((int64_t)w.e[0] * w.e[1]))};
    cell[DIR] -= 1;  // window index -> cell j = -1 ..
    double st[S][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      int idx[3] = {cell[0], cell[1], cell[2]};
      idx[DIR] += k - 2;
      bool flip[3] = {false, false, false};
      int g[3] = {0, 0, 0};
#pragma unroll
      for (int d = 0; d < ND; ++d) g[d] = map_cell(idx[d], P.n[d], P.bc_beg[d], P.bc_end[d], &flip[d]);
      const int64_t o = g[2] * P.sz + g[1] * P.sy + g[0];
      double v[S];
#pragma unroll
      for (int s = 0; s < S; ++s) v[s] = __ldg(q + o + s * P.sv);
#pragma unroll
      for (int d = 0; d < ND; ++d)
        if (flip[d]) v[Q::MOM + d] = -v[Q::MOM + d];
      cons_to_prim<ND, NF>(v, P);
#pragma unroll
      for (int s = 0; s < S; ++s) st[s][k] = v[s];
    }
    double cf[kCoefRec];
    if (wo > 1) {
      const int gi = clamp_coef_index(cell[DIR], P.n[DIR]) + P.coff;
#pragma unroll
      for (int k = 0; k < kNumCoef; ++k) cf[k] = __ldg(P.coef[DIR] + k * P.cstride[DIR] + gi);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
      double a, b;
      if (wo == 5) weno_cell<5, double>(cf, st[s], P.weno_eps, a, b);
      else if (wo == 3) weno_cell<3, double>(cf, st[s], P.weno_eps, a, b);
      else weno_cell<1, double>(cf, st[s], P.weno_eps, a, b);
      vl[c + s * cells] = a;
      vr[c + s * cells] = b;
    }
  }
}

// One face j + 1/2 of the window: left state qL_rs(j), right state
// qR_rs(j + 1), with the Riemann-state extrapolation of bc -4 at the domain
// faces (m_riemann_solvers.fpp:480-615): qL_rs(-1) = qR_rs(0) and
// qR_rs(s+1) = qL_rs(s).
template <int ND, int NF, int DIR>
__global__ void riemann_window_kernel(const DevParams P, const double* __restrict__ ql, const double* __restrict__ qr,
                                      const Window cw, const Window fw, double* __restrict__ flux,
                                      double* __restrict__ src) {
  using Q = Eqs<ND, NF>;
  constexpr int S = Q::S;
  const int64_t faces = fw.count(), cells = cw.count();
  double gam[NF], pin[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    gam[f] = P.gammas[f];
    pin[f] = P.pi_infs[f];
  }
  int64_t step = 1;  // window stride along DIR
  if (DIR >= 1) step *= cw.e[0];
  if (DIR >= 2) step *= cw.e[1];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < faces; c += (int64_t)gridDim.x * blockDim.x) {
    const int f[3] = {(int)(c % fw.e[0]), (int)((c / fw.e[0]) % fw.e[1]), (int)(c / ((int64_t)fw.e[0] * fw.e[1]))};
    const int j = f[DIR] - 1;  // face j + 1/2
    // window index of cell j (index j + 1 along DIR)
    const int64_t lc = ((int64_t)f[2] * cw.e[1] + f[1]) * cw.e[0] + f[0];
    const int64_t rc = lc + step;
    const bool lfr = j == -1 && P.bc_beg[DIR] == -4;
    const bool rfl = j == P.n[DIR] - 1 && P.bc_end[DIR] == -4;
    double qL[S], qR[S], F[S], us;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const double a = __ldg(ql + lc + s * cells);  // qL_rs(j)
      const double b = __ldg(qr + rc + s * cells);  // qR_rs(j + 1)
      qL[s] = lfr ? __ldg(qr + rc + s * cells) : a;
      qR[s] = rfl ? __ldg(ql + lc + s * cells) : b;
    }
    hllc_face<ND, NF, DIR, double>(qL, qR, gam, pin, F, us);
#pragma unroll
    for (int s = 0; s < S; ++s) flux[c + s * faces] = F[s];
    src[c] = us;
  }
}

template <int ND, int NF>
cudaError_t launch_weno(const DevParams& P, const double* q, int wo, int dir, const Window& w, double* vl,
                        double* vr, cudaStream_t st) {
  const unsigned blocks = (unsigned)std::min<int64_t>((w.count() + 127) / 128, 152 * 16);
  if (dir == 0) weno_window_kernel<ND, NF, 0><<<blocks, 128, 0, st>>>(P, q, wo, w, vl, vr);
  else if constexpr (ND > 1) {
    if (dir == 1) weno_window_kernel<ND, NF, 1><<<blocks, 128, 0, st>>>(P, q, wo, w, vl, vr);
    else if constexpr (ND > 2) weno_window_kernel<ND, NF, 2><<<blocks, 128, 0, st>>>(P, q, wo, w, vl, vr);
  }
  return cudaGetLastError();
}

template <int ND, int NF>
cudaError_t launch_riemann(const DevParams& P, const double* ql, const double* qr, int dir, const Window& cw,
                           const Window& fw, double* flux, double* src, cudaStream_t st) {
  const unsigned blocks = (unsigned)std::min<int64_t>((fw.count() + 127) / 128, 152 * 16);
  if (dir == 0) riemann_window_kernel<ND, NF, 0><<<blocks, 128, 0, st>>>(P, ql, qr, cw, fw, flux, src);
  else if constexpr (ND > 1) {
    if (dir == 1) riemann_window_kernel<ND, NF, 1><<<blocks, 128, 0, st>>>(P, ql, qr, cw, fw, flux, src);
    else if constexpr (ND > 2) riemann_window_kernel<ND, NF, 2><<<blocks, 128, 0, st>>>(P, ql, qr, cw, fw, flux, src);
  }
  return cudaGetLastError();
}

template <class F>
cudaError_t dispatch(int nd, int nf, F&& f) {
  if (nd == 1) return nf == 1 ? f(std::integral_constant<int, 1>{}, std::integral_constant<int, 1>{})
                              : f(std::integral_constant<int, 1>{}, std::integral_constant<int, 2>{});
  if (nd == 2) return nf == 1 ? f(std::integral_constant<int, 2>{}, std::integral_constant<int, 1>{})
                              : f(std::integral_constant<int, 2>{}, std::integral_constant<int, 2>{});
  return nf == 1 ? f(std::integral_constant<int, 3>{}, std::integral_constant<int, 1>{})
                 : f(std::integral_constant<int, 3>{}, std::integral_constant<int, 2>{});
}

// Device buffers of one call, freed on every return path.
// Carves the context's scratch into consecutive arrays of the given byte
// sizes, each 256-byte aligned.
struct Buffers {
  double* p[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaError_t take(mfc_gpu_ctx* c, std::initializer_list<size_t> bytes) {
    size_t total = 0;
    for (size_t b : bytes) total += (b + 255) / 256 * 256;
    void* base = nullptr;
    const cudaError_t e = ctx_scratch(c, total, &base);
    if (e != cudaSuccess) return e;
    size_t off = 0;
    int i = 0;
    for (size_t b : bytes) {
      p[i++] = reinterpret_cast<double*>(static_cast<char*>(base) + off);
      off += (b + 255) / 256 * 256;
    }
    return cudaSuccess;
  }
};

std::string check_view(const CtxView& v, int dir, bool riemann) {
  if (dir < 0 || dir >= v.nd) return "dir must be 0 .. num_dims-1";
  if (v.prec != MFC_PREC_FP64) return "the standalone WENO and Riemann entry points evaluate plain FP64; create the "
                                      "context with MFC_PREC_FP64";
  if (v.has_proc) return "processor boundaries: the face window needs physical boundary conditions";
  if (riemann && v.visc) return "viscous contexts: the Riemann solver's viscous source flux needs the velocity "
                                "gradients of s_get_viscous; use mfc_gpu_compute_rhs";
  return "";
}

}  // namespace
}  // namespace mfc

extern "C" int mfc_gpu_weno(mfc_gpu_ctx* ctx, int dir, double* vL, double* vR) {
  mfc::CtxView v;
  if (!ctx || !vL || !vR || !mfc::ctx_view(ctx, v)) return mfc::report_error(MFC_ERR_INVALID, "NULL argument");
  const std::string why = mfc::check_view(v, dir, false);
  if (!why.empty()) return mfc::report_error(MFC_ERR_INVALID, why);
  const mfc::Window w = mfc::face_window(v.n, dir, 2);
  const size_t bytes = sizeof(double) * (size_t)(v.S * w.count());
  mfc::Buffers B;
  cudaError_t e;
  if ((e = B.take(ctx, {bytes, bytes})) != cudaSuccess) return mfc::report_error(MFC_ERR_NOMEM, cudaGetErrorString(e));
  e = mfc::dispatch(v.nd, v.nf, [&](auto ND, auto NF) {
    return mfc::launch_weno<decltype(ND)::value, decltype(NF)::value>(*v.dev, v.q0, v.wo, dir, w, B.p[0], B.p[1],
                                                                       v.stream);
  });
  if (e == cudaSuccess) e = cudaMemcpyAsync(vL, B.p[0], bytes, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(vR, B.p[1], bytes, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));
  *v.launches += 1;
  return MFC_OK;
}

extern "C" int mfc_gpu_riemann(mfc_gpu_ctx* ctx, int dir, const double* qL_rs, const double* qR_rs, double* flux,
                               double* flux_src) {
  mfc::CtxView v;
  if (!ctx || !qL_rs || !qR_rs || !flux || !flux_src || !mfc::ctx_view(ctx, v))
    return mfc::report_error(MFC_ERR_INVALID, "NULL argument");
  const std::string why = mfc::check_view(v, dir, true);
  if (!why.empty()) return mfc::report_error(MFC_ERR_INVALID, why);
  const mfc::Window cw = mfc::face_window(v.n, dir, 2), fw = mfc::face_window(v.n, dir, 1);
  const size_t in_bytes = sizeof(double) * (size_t)(v.S * cw.count());
  const size_t flux_bytes = sizeof(double) * (size_t)(v.S * fw.count());
  const size_t src_bytes = sizeof(double) * (size_t)fw.count();
  mfc::Buffers B;
  cudaError_t e;
  if ((e = B.take(ctx, {in_bytes, in_bytes, flux_bytes, src_bytes})) != cudaSuccess)
    return mfc::report_error(MFC_ERR_NOMEM, cudaGetErrorString(e));
  e = cudaMemcpyAsync(B.p[0], qL_rs, in_bytes, cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B.p[1], qR_rs, in_bytes, cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess)
    e = mfc::dispatch(v.nd, v.nf, [&](auto ND, auto NF) {
      return mfc::launch_riemann<decltype(ND)::value, decltype(NF)::value>(*v.dev, B.p[0], B.p[1], dir, cw, fw,
                                                                           B.p[2], B.p[3], v.stream);
    });
  if (e == cudaSuccess) e = cudaMemcpyAsync(flux, B.p[2], flux_bytes, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(flux_src, B.p[3], src_bytes, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  if (e != cudaSuccess) return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));
  *v.launches += 1;
  return MFC_OK;
}
