// Learned WENO smoothness gate (no reference counterpart).
//
// A small MLP looks at one cell's 5-point stencils of alpha_1 and p in one
// direction and decides whether the cell needs the full nonlinear WENO5
// weights (m_weno.fpp:495-531) or can use the optimal linear weights d_k.
//
//   inputs  10: each stencil shifted by its minimum and divided by its range
//               max - min, floored at 1e-2 of the stencil's magnitude for p
//               and at 1e-2 for alpha_1 (a volume fraction is O(1)); below
//               the floor the inputs shrink with the stencil's amplitude, so
//               the network can tell a ripple from a jump
//   layers  10 -> 32 (ReLU) -> 32 (ReLU) -> 1 (logit; sigmoid > 1/2 <=> logit > 0)
//   label   max_k |omega_k - d_k| > 1e-3 for alpha_1 or p, left or right face,
//           with the WENO5 weights evaluated (in FP64) on those normalised
//           stencils and epsilon = 1e-2: a unit jump has beta ~ 1, and
//           variations under ~1e-3 of a variable's magnitude (beta below
//           epsilon) count as flat.  On the raw fields with the case's
//           epsilon = 1e-16 the weights react to any relative variation above
//           ~1e-13, so the round-off of the stiffened-gas pressure recovery
//           and the FP32 ripples of the split path would mark nearly every
//           cell.

// Inference runs on the tensor cores with FP16 weights and FP32
// accumulation (mma.sync m16n8k16, 16 cells per warp, the three layers
// chained in registers: the accumulator fragment of one layer is the A
// fragment of the next).  Training uses FP32 master weights.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mfc_device.cuh"

namespace mfc {

constexpr int kGateIn = 10, kGateH = 32;
constexpr int kGW1 = 0, kGB1 = kGW1 + kGateIn * kGateH, kGW2 = kGB1 + kGateH, kGB2 = kGW2 + kGateH * kGateH,
              kGW3 = kGB2 + kGateH, kGB3 = kGW3 + kGateH, kGateParams = kGB3 + 1;  // 1441
constexpr float kGateLabelTol = 1e-3f;
constexpr double kGateLabelEps = 1e-2;
constexpr float kGateRelFloor = 1e-2f, kGateAlphaFloor = 1e-2f;

// One stencil of 5 values -> 5 normalised inputs.
__device__ __forceinline__ void gate_norm5(const float (&s)[5], float* out, float abs_floor) {
  const float lo = fminf(fminf(fminf(s[0], s[1]), fminf(s[2], s[3])), s[4]);
  const float hi = fmaxf(fmaxf(fmaxf(s[0], s[1]), fmaxf(s[2], s[3])), s[4]);
  const float floor_ = fmaxf(fmaxf(fabsf(lo), fabsf(hi)) * kGateRelFloor, abs_floor);
  const float r = rcp_approx(fmaxf(hi - lo, floor_));
  const float off = -lo * r;
#pragma unroll
  for (int k = 0; k < 5; ++k) out[k] = fmaf(s[k], r, off);
}

// var 0: alpha_1 stencil, var 1: pressure stencil
__device__ __forceinline__ void gate_norm5_var(const float (&s)[5], float* out, int var) {
  gate_norm5(s, out, var == 0 ? kGateAlphaFloor : 1e-30f);
}

__device__ __forceinline__ void gate_features(const float (&a)[5], const float (&p)[5], float (&x)[kGateIn]) {
  gate_norm5_var(a, x, 0);
  gate_norm5_var(p, x + 5, 1);
}

// max_k |omega_k - d_k| over both faces of the FP64 WENO5 weights of one
// stencil (m_weno.fpp:495-528; the label of one variable).
__device__ __forceinline__ double weno5_weight_deviation(const double* __restrict__ c, const double (&v)[5],
                                                         double eps) {
  const double d1 = v[4] - v[3], d0 = v[3] - v[2], dm1 = v[2] - v[1], dm2 = v[1] - v[0];
  const double b0 = c[kBeta + 0] * d1 * d1 + c[kBeta + 1] * d1 * d0 + c[kBeta + 2] * d0 * d0 + eps;
  const double b1 = c[kBeta + 3] * d0 * d0 + c[kBeta + 4] * d0 * dm1 + c[kBeta + 5] * dm1 * dm1 + eps;
  const double b2 = c[kBeta + 6] * dm1 * dm1 + c[kBeta + 7] * dm1 * dm2 + c[kBeta + 8] * dm2 * dm2 + eps;
  double dev = 0.0;
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const double* d = c + (side ? kDR : kDL);
    const double a0 = d[0] / (b0 * b0), a1 = d[1] / (b1 * b1), a2 = d[2] / (b2 * b2);
    const double s = a0 + a1 + a2;
    dev = fmax(dev, fmax(fabs(a0 / s - d[0]), fmax(fabs(a1 / s - d[1]), fabs(a2 / s - d[2]))));
  }
  return dev;
}

// WENO5 with the optimal linear weights d_k (the gate's "smooth" branch),
// two variables at once (weno5_pair_fast's packed pairs).
template <class Coef>
__device__ __forceinline__ void weno5_pair_linear(const Coef& C, const f32x2 (&v)[5], f32x2& vL, f32x2& vR) {
  const f32x2 d1 = f2_sub(v[4], v[3]), d0 = f2_sub(v[3], v[2]), dm1 = f2_sub(v[2], v[1]), dm2 = f2_sub(v[1], v[0]);
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int kP = side ? kPR : kPL, kD = side ? kDR : kDL;
    const f32x2 p0 = f2_fma(C(kP + 1), d0, f2_fma(C(kP + 0), d1, v[2]));
    const f32x2 p1 = f2_fma(C(kP + 3), dm1, f2_fma(C(kP + 2), d0, v[2]));
    const f32x2 p2 = f2_fma(C(kP + 5), dm2, f2_fma(C(kP + 4), dm1, v[2]));
    const f32x2 val = f2_fma(C(kD + 2), p2, f2_fma(C(kD + 1), p1, f2_mul(C(kD + 0), p0)));
    if (side) vR = val;
    else vL = val;
  }
}

// ---------------------------------------------------------------------------
// Tensor-core inference.  Weight fragments of one lane (m16n8k16 layouts:
// lane = 4*g + t; A rows g, g+8 / cols 2t, 2t+1, 2t+8, 2t+9; B rows (k) 2t,
// 2t+1, 2t+8, 2t+9 / col (n) g; C rows g, g+8 / cols 2t, 2t+1).
//
// MMA input columns: the alpha_1 features sit in columns 0..4 and the
// pressure features in columns 8..12 (the rest are zero), so that each half
// of a cell's row is one 16-byte store.
__host__ __device__ constexpr int gate_feature_of_col(int k) { return k < 5 ? k : (k >= 8 && k < 13 ? k - 3 : -1); }

// A lane's fragments as 48 words (45 used): W1 0..7 (word 2j + r), W2 8..23
// (8 + 8s + 2j + r), W3 24..27 (24 + 2s + r), b1 28..35 (28 + 2j + c), b2
// 36..43, b3 44; gate_mlp16 reads them in groups of four words.
constexpr int kGateFragWords = 48;
struct GateFrags {
  uint32_t w1[4][2];     // layer 1: k 0..15 (inputs, 10 used), n-tiles 0..3
  uint32_t w2[2][4][2];  // layer 2: k-steps 0..1, n-tiles 0..3
  uint32_t w3[2][2];     // layer 3: k-steps 0..1, n-tile 0 (only column 0 used)
  float b1[4][2], b2[4][2], b3;
  __device__ uint32_t word(int w) const {
    if (w < 8) return w1[w >> 1][w & 1];
    if (w < 24) return w2[(w - 8) >> 3][((w - 8) >> 1) & 3][w & 1];
    if (w < 28) return w3[(w - 24) >> 1][w & 1];
    if (w < 36) return __float_as_uint(b1[(w - 28) >> 1][w & 1]);
    if (w < 44) return __float_as_uint(b2[(w - 36) >> 1][w & 1]);
    return w == 44 ? __float_as_uint(b3) : 0u;
  }
  __device__ uint4 group(int q) const { return make_uint4(word(4 * q), word(4 * q + 1), word(4 * q + 2), word(4 * q + 3)); }
};

// The same fragments in shared memory, [group][32 lanes][4 words], so that a
// warp reads one group of every lane with one conflict-free 16-byte load per
// lane; the fused stage kernel uses this form, which keeps its register
// count low.
// Device buffer of a gated context: the FP16 parameters, then (16-byte
// aligned) the precomputed lane fragments in this layout.
constexpr size_t kGateFragOffset = (2 * size_t(kGateParams) + 15) / 16 * 16;
constexpr size_t kGateBufferBytes = kGateFragOffset + size_t(kGateFragWords) * 32 * 4;
__host__ __device__ constexpr int gate_frag_index(int lane, int word) { return (word >> 2) * 128 + lane * 4 + (word & 3); }
struct GateFragsSmem {
  const uint32_t* p;  // group 0 of this lane
  __device__ uint4 group(int q) const { return *reinterpret_cast<const uint4*>(p + q * 128); }
};

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ uint32_t pack_h2_raw(__half lo, __half hi) {
  __half2 h;
  h.x = lo;
  h.y = hi;
  return *reinterpret_cast<const uint32_t*>(&h);
}

// ReLU of two accumulators as one packed FP16 pair: the rounding to FP16
// keeps the sign, so clamping after it equals clamping before it.
__device__ __forceinline__ uint32_t relu_h2(float lo, float hi) {
  const __half2 h = __hmax2(__floats2half2_rn(lo, hi), __float2half2_rn(0.f));
  return *reinterpret_cast<const uint32_t*>(&h);
}

// First-layer weight of MMA column k (the input layout above) and unit n.
__device__ __forceinline__ __half gate_w1(const __half* __restrict__ w, int k, int n) {
  const int f = gate_feature_of_col(k);
  return f >= 0 ? w[kGW1 + f * kGateH + n] : __float2half(0.f);
}

// One word of one lane's fragments (the numbering above), computed from the
// FP16 parameters.
__device__ __forceinline__ uint32_t gate_frag_word(const __half* __restrict__ w, int lane, int word) {
  const int g = lane >> 2, t = lane & 3;
  auto W2 = [&](int k, int n) { return w[kGW2 + k * kGateH + n]; };
  auto W3 = [&](int k, int n) { return n == 0 ? w[kGW3 + k] : __float2half(0.f); };
  if (word < 8) {
    const int j = word >> 1, r = word & 1, n = 8 * j + g;
    return r == 0 ? pack_h2_raw(gate_w1(w, 2 * t, n), gate_w1(w, 2 * t + 1, n))
                  : pack_h2_raw(gate_w1(w, 2 * t + 8, n), gate_w1(w, 2 * t + 9, n));
  }
  if (word < 24) {
    const int q = word - 8, r = q & 1, sj = q >> 1, s = sj >> 2, j = sj & 3, n = 8 * j + g;
    return r == 0 ? pack_h2_raw(W2(16 * s + 2 * t, n), W2(16 * s + 2 * t + 1, n))
                  : pack_h2_raw(W2(16 * s + 2 * t + 8, n), W2(16 * s + 2 * t + 9, n));
  }
  if (word < 28) {
    const int q = word - 24, s = q >> 1, r = q & 1;
    return r == 0 ? pack_h2_raw(W3(16 * s + 2 * t, g), W3(16 * s + 2 * t + 1, g))
                  : pack_h2_raw(W3(16 * s + 2 * t + 8, g), W3(16 * s + 2 * t + 9, g));
  }
  if (word < 36) {
    const int q = word - 28, j = q >> 1, c = q & 1;
    return __float_as_uint(__half2float(w[kGB1 + 8 * j + 2 * t + c]));
  }
  if (word < 44) {
    const int q = word - 36, j = q >> 1, c = q & 1;
    return __float_as_uint(__half2float(w[kGB2 + 8 * j + 2 * t + c]));
  }
  return word == 44 ? __float_as_uint(__half2float(w[kGB3])) : 0u;
}

// w: FP16 weights in the parameter layout (kGW1..kGB3), biases included.
__device__ __forceinline__ void gate_load_frags(const __half* __restrict__ w, GateFrags& F) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    F.w1[j][0] = gate_frag_word(w, lane, 2 * j);
    F.w1[j][1] = gate_frag_word(w, lane, 2 * j + 1);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      F.w2[s][j][0] = gate_frag_word(w, lane, 8 + 8 * s + 2 * j);
      F.w2[s][j][1] = gate_frag_word(w, lane, 8 + 8 * s + 2 * j + 1);
    }
    F.b1[j][0] = __uint_as_float(gate_frag_word(w, lane, 28 + 2 * j));
    F.b1[j][1] = __uint_as_float(gate_frag_word(w, lane, 28 + 2 * j + 1));
    F.b2[j][0] = __uint_as_float(gate_frag_word(w, lane, 36 + 2 * j));
    F.b2[j][1] = __uint_as_float(gate_frag_word(w, lane, 36 + 2 * j + 1));
  }
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    F.w3[s][0] = gate_frag_word(w, lane, 24 + 2 * s);
    F.w3[s][1] = gate_frag_word(w, lane, 24 + 2 * s + 1);
  }
  F.b3 = __uint_as_float(gate_frag_word(w, lane, 44));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t u4(const uint4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

// Logits of 16 cells.  xin: the cells' inputs, FP16, 16 halves per row in
// the column layout above, 16-byte aligned rows, in shared memory; the
// warp's lanes must all call this.  Returns, in lanes with t == 0, the
// logits of cells g (lo) and g + 8 (hi).
template <class Frags>
__device__ __forceinline__ void gate_mlp16(const __half* __restrict__ xin, const Frags& F, float& lo, float& hi) {
  const int lane = threadIdx.x & 31, t = lane & 3;
  // A fragment of the 16x16 input block: the four 8x8 quarters (rows 0-7 /
  // 8-15, columns 0-7 / 8-15) in one ldmatrix
  uint32_t a[4];
  {
    const __half* row = xin + ((lane & 7) + ((lane >> 3) & 1) * 8) * 16 + (lane >> 4) * 8;
    const uint32_t addr = (uint32_t)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
                 : "r"(addr));
  }
  float h[4][4];
  {
    const uint4 w0 = F.group(0), w1 = F.group(1), b0 = F.group(7), b1 = F.group(8);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint4& wg = j < 2 ? w0 : w1;
      const uint4& bg = j < 2 ? b0 : b1;
      const int o = 2 * (j & 1);
      h[j][0] = h[j][2] = __uint_as_float(u4(bg, o));
      h[j][1] = h[j][3] = __uint_as_float(u4(bg, o + 1));
      mma16816(h[j], a, u4(wg, o), u4(wg, o + 1));
    }
  }
  // layer-1 activations as the packed FP16 A fragments of layer 2's two k-steps
  uint32_t ah[2][4];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    ah[s][0] = relu_h2(h[2 * s][0], h[2 * s][1]);
    ah[s][1] = relu_h2(h[2 * s][2], h[2 * s][3]);
    ah[s][2] = relu_h2(h[2 * s + 1][0], h[2 * s + 1][1]);
    ah[s][3] = relu_h2(h[2 * s + 1][2], h[2 * s + 1][3]);
  }
  // layer 2 in two halves of 16 units, each followed by its k-step of
  // layer 3, so that only half of layer 2's accumulators are live at a time
  const uint4 w3 = F.group(6);
  const float b3 = __uint_as_float(F.group(11).x);
  float o[4] = {t == 0 ? b3 : 0.f, 0.f, t == 0 ? b3 : 0.f, 0.f};
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float g2[2][4];
    const uint4 bg = F.group(9 + half);  // b2 words 36 + 4 half .. 39 + 4 half
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
      g2[jj][0] = g2[jj][2] = __uint_as_float(u4(bg, 2 * jj));
      g2[jj][1] = g2[jj][3] = __uint_as_float(u4(bg, 2 * jj + 1));
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const uint4 wg = F.group(2 + 2 * s + half);  // W2 words 8 + 8 s + 4 half ..
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) mma16816(g2[jj], ah[s], u4(wg, 2 * jj), u4(wg, 2 * jj + 1));
    }
    uint32_t as[4];
    as[0] = relu_h2(g2[0][0], g2[0][1]);
    as[1] = relu_h2(g2[0][2], g2[0][3]);
    as[2] = relu_h2(g2[1][0], g2[1][1]);
    as[3] = relu_h2(g2[1][2], g2[1][3]);
    mma16816(o, as, u4(w3, 2 * half), u4(w3, 2 * half + 1));
  }
  lo = o[0];
  hi = o[2];
}

}  // namespace mfc
