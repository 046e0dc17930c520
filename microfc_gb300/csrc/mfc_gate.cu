// Learned WENO gate: sample extraction from solver states, training kernels
// (forward, backward, weight gradients, Adam) and a tensor-core inference
// kernel for checking.  No reference counterpart.  See mfc_gate.cuh for the
// network and its inputs/label.
//
// Training layout: parameters in one FP32 vector (kGW1 .. kGB3); a batch is
// X [B][10] (row-major) and targets T [B] in {0, 1}.  The workspace holds
// per-sample activations and deltas: H1, dH1, H2, dH2 (4 x 32) and dz.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mfc_gpu.h"
#include "mfc_gate.cuh"
#include "mfc_launch.h"

namespace {

constexpr int kActs = 4 * mfc::kGateH + 1;  // per-sample workspace floats

// Features and weight deviation of every interior cell of a 2-D state along
// direction dir (0 = x, 1 = y), with the split path's cons -> prim.
template <int NF>
__global__ void gate_sample_kernel(const mfc::DevParams P, const double* __restrict__ q, int dir,
                                   float* __restrict__ xout, float* __restrict__ dev_out) {
  using Q = mfc::Eqs<2, NF>;
  const int nx = P.n[0], ny = P.n[1];
  const int64_t cells = (int64_t)nx * ny;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(c % nx), y = (int)(c / nx);
    // features from the split path's FP32 primitives (what the gated kernel
    // sees); label from the FP64 WENO5 weights of those normalised stencils
    float a[5], p[5];
    for (int k = 0; k < 5; ++k) {
      bool flip = false;
      int gx = x, gy = y;
      if (dir == 0) gx = mfc::map_cell(x + k - 2, nx, P.bc_beg[0], P.bc_end[0], &flip);
      else gy = mfc::map_cell(y + k - 2, ny, P.bc_beg[1], P.bc_end[1], &flip);
      double qq[Q::S];
      for (int v = 0; v < Q::S; ++v) qq[v] = q[gy * P.sy + gx + v * P.sv];
      if (flip) qq[Q::MOM + dir] = -qq[Q::MOM + dir];
      float pr[Q::S];
      mfc::cons_to_prim_split<2, NF>(qq, P, pr);
      a[k] = pr[Q::ADV];
      p[k] = pr[Q::E];
    }
    float feat[mfc::kGateIn];
    mfc::gate_features(a, p, feat);
    for (int k = 0; k < mfc::kGateIn; ++k) xout[c * mfc::kGateIn + k] = feat[k];
    double cf[mfc::kNumCoef];
    const int ci = (dir == 0 ? x : y) + P.coff;
    for (int k = 0; k < mfc::kNumCoef; ++k) cf[k] = P.coef[dir][k * P.cstride[dir] + ci];
    double na[5], np_[5];
    for (int k = 0; k < 5; ++k) {
      na[k] = feat[k];
      np_[k] = feat[5 + k];
    }
    dev_out[c] = (float)fmax(mfc::weno5_weight_deviation(cf, na, mfc::kGateLabelEps),
                             mfc::weno5_weight_deviation(cf, np_, mfc::kGateLabelEps));
  }
}

// Forward and backward of one sample per thread; loss summed into *loss.
__global__ void gate_fwd_bwd_kernel(const float* __restrict__ X, const float* __restrict__ T, int B,
                                    const float* __restrict__ w, float pos_weight, float* __restrict__ acts,
                                    float* __restrict__ loss) {
  using namespace mfc;
  __shared__ float sw[kGateParams];
  for (int i = threadIdx.x; i < kGateParams; i += blockDim.x) sw[i] = w[i];
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (b < B) {
    float x[kGateIn], h1[kGateH], h2[kGateH];
    for (int i = 0; i < kGateIn; ++i) x[i] = X[b * kGateIn + i];
    for (int j = 0; j < kGateH; ++j) {
      float s = sw[kGB1 + j];
      for (int i = 0; i < kGateIn; ++i) s = fmaf(x[i], sw[kGW1 + i * kGateH + j], s);
      h1[j] = fmaxf(s, 0.f);
    }
    for (int j = 0; j < kGateH; ++j) {
      float s = sw[kGB2 + j];
      for (int i = 0; i < kGateH; ++i) s = fmaf(h1[i], sw[kGW2 + i * kGateH + j], s);
      h2[j] = fmaxf(s, 0.f);
    }
    float z = sw[kGB3];
    for (int i = 0; i < kGateH; ++i) z = fmaf(h2[i], sw[kGW3 + i], z);
    const float t = T[b];
    const float sig = 1.f / (1.f + expf(-z));
    // weighted binary cross-entropy with logits, stable form
    const float sp_neg = fmaxf(-z, 0.f) + log1pf(expf(-fabsf(z)));  // -log sigmoid(z)
    const float sp_pos = sp_neg + z;                                   // -log(1 - sigmoid(z))
    l = pos_weight * t * sp_neg + (1.f - t) * sp_pos;
    const float dz = (sig * (pos_weight * t + 1.f - t) - pos_weight * t) / (float)B;
    float* a = acts + (size_t)b * kActs;
    float dh2[kGateH];
    for (int j = 0; j < kGateH; ++j) {
      dh2[j] = h2[j] > 0.f ? dz * sw[kGW3 + j] : 0.f;
      a[0 * kGateH + j] = h1[j];
      a[2 * kGateH + j] = h2[j];
      a[3 * kGateH + j] = dh2[j];
    }
    for (int i = 0; i < kGateH; ++i) {
      float s = 0.f;
      for (int j = 0; j < kGateH; ++j) s = fmaf(dh2[j], sw[kGW2 + i * kGateH + j], s);
      a[1 * kGateH + i] = h1[i] > 0.f ? s : 0.f;
    }
    a[4 * kGateH] = dz;
  }
  // block sum of the loss
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

// Weight gradients: 46 rows of 32 outputs (W1: 10 rows, b1, W2: 32 rows,
// b2, W3, b3); warp (row, chunk of samples) -> atomicAdd into g.
__global__ void gate_wgrad_kernel(const float* __restrict__ X, const float* __restrict__ acts, int B, int chunk,
                                  float* __restrict__ g) {
  using namespace mfc;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int rows = kGateIn + 1 + kGateH + 1 + 1 + 1;
  const int row = warp % rows, ck = warp / rows;
  const int b0 = ck * chunk, b1 = min(B, b0 + chunk);
  if (b0 >= B) return;
  float s = 0.f;
  int out = -1;
  if (row < kGateIn) {  // dW1[row][lane] = sum X[b][row] dH1[b][lane]
    for (int b = b0; b < b1; ++b) s = fmaf(X[b * kGateIn + row], acts[(size_t)b * kActs + kGateH + lane], s);
    out = kGW1 + row * kGateH + lane;
  } else if (row == kGateIn) {  // db1
    for (int b = b0; b < b1; ++b) s += acts[(size_t)b * kActs + kGateH + lane];
    out = kGB1 + lane;
  } else if (row < kGateIn + 1 + kGateH) {  // dW2[i][lane] = sum H1[b][i] dH2[b][lane]
    const int i = row - kGateIn - 1;
    for (int b = b0; b < b1; ++b)
      s = fmaf(acts[(size_t)b * kActs + i], acts[(size_t)b * kActs + 3 * kGateH + lane], s);
    out = kGW2 + i * kGateH + lane;
  } else if (row == kGateIn + 1 + kGateH) {  // db2
    for (int b = b0; b < b1; ++b) s += acts[(size_t)b * kActs + 3 * kGateH + lane];
    out = kGB2 + lane;
  } else if (row == kGateIn + 2 + kGateH) {  // dW3[lane] = sum H2[b][lane] dz[b]
    for (int b = b0; b < b1; ++b)
      s = fmaf(acts[(size_t)b * kActs + 2 * kGateH + lane], acts[(size_t)b * kActs + 4 * kGateH], s);
    out = kGW3 + lane;
  } else {  // db3
    if (lane == 0)
      for (int b = b0; b < b1; ++b) s += acts[(size_t)b * kActs + 4 * kGateH];
    out = lane == 0 ? kGB3 : -1;
  }
  if (out >= 0) atomicAdd(g + out, s);
}

// Adam (Kingma & Ba 2015) with bias correction.
__global__ void gate_adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                                 float* __restrict__ v, int step, float lr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mfc::kGateParams) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step));
  const float vh = vi / (1.f - powf(b2, (float)step));
  w[i] -= lr * mh / (sqrtf(vh) + eps);
}

// Lane fragments of the FP16 parameters in the GateFragsSmem layout.
__global__ void gate_frag_kernel(const __half* __restrict__ wh, uint32_t* __restrict__ frag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // (word, lane)
  if (i < mfc::kGateFragWords * 32) {
    const int word = i >> 5, lane = i & 31;
    frag[mfc::gate_frag_index(lane, word)] = mfc::gate_frag_word(wh, lane, word);
  }
}

__global__ void gate_to_half_kernel(const float* __restrict__ w, __half* __restrict__ h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < mfc::kGateParams) h[i] = __float2half_rn(w[i]);
}

// Tensor-core inference of n inputs (16 per warp); logits out.
__global__ void gate_infer_kernel(const float* __restrict__ X, int n, const __half* __restrict__ wh,
                                  float* __restrict__ logits) {
  __shared__ __align__(16) __half buf[8][16 * 16];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  mfc::GateFrags F;
  mfc::gate_load_frags(wh, F);
  const int base = (blockIdx.x * 8 + warp) * 16;
  __half* my = buf[warp];
  for (int k = lane; k < 256; k += 32) {
    const int r = k / 16, f = mfc::gate_feature_of_col(k % 16);
    const int b = base + r;
    my[k] = __float2half((b < n && f >= 0) ? X[b * mfc::kGateIn + f] : 0.f);
  }
  __syncwarp();
  float lo, hi;
  mfc::gate_mlp16(my, F, lo, hi);
  if ((lane & 3) == 0) {
    const int g = lane >> 2;
    if (base + g < n) logits[base + g] = lo;
    if (base + g + 8 < n) logits[base + g + 8] = hi;
  }
}

int cuda_fail(cudaError_t e) { return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e)); }

int run_fwd_bwd(const float* X, const float* T, int B, const float* w, float pos_weight, float* grad, float* work,
                float* loss, cudaStream_t st) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(loss, 0, sizeof(float), st)) != cudaSuccess) return cuda_fail(e);
  if ((e = cudaMemsetAsync(grad, 0, sizeof(float) * mfc::kGateParams, st)) != cudaSuccess) return cuda_fail(e);
  gate_fwd_bwd_kernel<<<(B + 255) / 256, 256, 0, st>>>(X, T, B, w, pos_weight, work, loss);
  const int chunk = 256, rows = mfc::kGateIn + 1 + mfc::kGateH + 3;
  const int warps = rows * ((B + chunk - 1) / chunk);
  gate_wgrad_kernel<<<(warps * 32 + 255) / 256, 256, 0, st>>>(X, work, B, chunk, grad);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
  return MFC_OK;
}

}  // namespace

extern "C" {

int mfc_gate_param_count(void) { return mfc::kGateParams; }

int mfc_gate_workspace_floats(int batch) { return batch * kActs; }

// Forward + backward on one batch: grad <- dL/dw (mean weighted BCE), *loss
// (device) <- summed loss.  All pointers are device pointers.
int mfc_gate_gradients(const float* X, const float* T, int batch, const float* w, float pos_weight, float* grad,
                       float* work, float* loss, void* stream) {
  if (!X || !T || !w || !grad || !work || !loss || batch < 1) return mfc::report_error(MFC_ERR_INVALID, "bad gate args");
  int rc = run_fwd_bwd(X, T, batch, w, pos_weight, grad, work, loss, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? MFC_OK : cuda_fail(e);
}

// One Adam step (step >= 1) on one batch; asynchronous on `stream`.
int mfc_gate_train_step(const float* X, const float* T, int batch, float* w, float* grad, float* m, float* v,
                        float* work, int step, float lr, float pos_weight, float* loss, void* stream) {
  if (!X || !T || !w || !grad || !m || !v || !work || !loss || batch < 1 || step < 1)
    return mfc::report_error(MFC_ERR_INVALID, "bad gate args");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = run_fwd_bwd(X, T, batch, w, pos_weight, grad, work, loss, st);
  if (rc) return rc;
  gate_adam_kernel<<<(mfc::kGateParams + 255) / 256, 256, 0, st>>>(w, grad, m, v, step, lr);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MFC_OK : cuda_fail(e);
}

// Tensor-core inference with FP16-rounded weights; w32: FP32 parameters,
// wh: scratch for kGateParams halves.  Synchronous.
int mfc_gate_infer(const float* X, int n, const float* w32, void* wh, float* logits, void* stream) {
  if (!X || !w32 || !wh || !logits || n < 1) return mfc::report_error(MFC_ERR_INVALID, "bad gate args");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  __half* h = static_cast<__half*>(wh);
  gate_to_half_kernel<<<(mfc::kGateParams + 255) / 256, 256, 0, st>>>(w32, h);
  gate_infer_kernel<<<(n + 127) / 128, 256, 0, st>>>(X, n, h, logits);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? MFC_OK : cuda_fail(e);
}

}  // extern "C"

// Samples of a context's current state (register 0); defined here, declared
// in mfc_gpu.h, needs the context internals exposed by mfc_capi.cu.
namespace mfc {
int gate_samples(const DevParams& P, int nf, const double* q, int dir, float* xout, float* dev_out,
                 cudaStream_t st) {
  const int64_t cells = (int64_t)P.n[0] * P.n[1];
  const unsigned blocks = (unsigned)std::min<int64_t>((cells + 255) / 256, 8192);
  if (nf == 1) gate_sample_kernel<1><<<blocks, 256, 0, st>>>(P, q, dir, xout, dev_out);
  else gate_sample_kernel<2><<<blocks, 256, 0, st>>>(P, q, dir, xout, dev_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? MFC_OK : cuda_fail(e);
}

int gate_upload(const float* host_params, void* dev_buf, cudaStream_t st) {
  std::vector<__half> h(kGateParams);
  for (int i = 0; i < kGateParams; ++i) {
    if (!std::isfinite(host_params[i])) return report_error(MFC_ERR_INVALID, "gate parameters must be finite");
    h[i] = __float2half_rn(host_params[i]);
  }
  cudaError_t e = cudaMemcpyAsync(dev_buf, h.data(), sizeof(__half) * kGateParams, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e);
  // the fused stage kernel's per-lane MMA fragments, computed once here
  gate_frag_kernel<<<(kGateFragWords * 32 + 255) / 256, 256, 0, st>>>(
      static_cast<const __half*>(dev_buf),
      reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(dev_buf) + kGateFragOffset));
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? MFC_OK : cuda_fail(e);
}
}  // namespace mfc
