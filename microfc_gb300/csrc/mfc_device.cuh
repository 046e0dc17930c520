// Device-side building blocks of the GB300 MicroFC hot path: the parameter
// block every kernel receives by value, boundary-condition index mapping,
// the stiffened-gas cons -> prim conversion, WENO1/3/5 and HLLC.
//
// The FP64 arithmetic follows the reference's operation order (file:line
// cited at each function); compiled without FMA contraction it reproduces
// the CPU reference bit for bit.  RT is the type of the reconstruction and
// Riemann arithmetic: double for the plain path, float for the
// split-precision path, which also uses the *_split / *_fast variants below.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mfc {

constexpr int kMaxFluids = 4;
constexpr int kNumCoef = 27;  // per cell: polyL[3][2], polyR[3][2], dL[3], dR[3], beta[3][3]
// offsets inside one coefficient record
constexpr int kPL = 0, kPR = 6, kDL = 12, kDR = 15, kBeta = 18;
// split precision: one cell's FP32 coefficients padded to a 16-byte record
constexpr int kCoefRec = 28;

struct DevParams {
  int n[3];             // interior cells per direction (m+1, n+1, p+1); 1 when unused
  int64_t sy, sz, sv;   // element strides: y row, z plane, equation
  int bc_beg[3], bc_end[3];
  double gammas[kMaxFluids], pi_infs[kMaxFluids];
  double weno_eps;
  // the same constants rounded to FP32 (split path), set by set_fp32_constants
  float gammas_f[kMaxFluids], pi_infs_f[kMaxFluids], weno_eps_f;
  const double* inv_d[3];  // 1/dx(i) for i = 0 .. n-1 (per direction)
  const double* coef[3];   // WENO coefficients, SoA: coef[k * cstride + (i + coff)],
                           // cells i = -kCoefPad .. n-1+kCoefPad, coff = kCoefPad
  int coff, cstride[3];
  uint32_t* status;
  // The two never coexist (the gate runs on 2-D cases only), so they share
  // one slot: the ensemble's 96 parameter blocks must fit the kernel
  // parameter space.
  union {
    // 3-D: partial RHS between the directional sweeps ([S][z][y][x], RT),
    // then the primitives of the stage input that the x sweep stores (same
    // layout, RT)
    void* work;
    // learned WENO gate: the decisions of a time step's first stage, one
    // byte per reconstructed cell and direction, reused by its later stages
    // (NULL: every stage runs the network).  x plane [ny][nx + 2] (cells x =
    // -1 .. nx), then y plane [ny + 2][nx] (cells y = -1 .. ny).
    uint8_t* gate_flags;
  };
  const void* gate_w;  // learned WENO gate: FP16 MLP parameters (mfc_gate.cuh layout)
  unsigned long long* monitor;  // set on a step's last stage: max ICFL of the new state (double bits)
  // processor boundaries (bc >= 0): device table of 6 halo buffers, [2*dir + side]
  // (NULL where the side is a physical boundary); the whole table is NULL
  // when the context has no processor boundary.  x sides: [S][nz][ny][H]
  // (depth fastest), y sides: [S][H][nx + 2] in 2-D (the x ghost cells -1
  // and nx of each row first and last), [S][nz][H][nx] in 3-D, z sides:
  // [S][H][ny][nx]; depth d = 0 is the ghost cell next to the boundary.
  const double* const* halo;
  const struct ViscParams* visc;  // viscous cases: Reynolds numbers and spacing tables (NULL: inviscid)
};

// Bytes of the stored gate decisions of an nx x ny case (DevParams::gate_flags).
inline size_t gate_flag_bytes(int nx, int ny) {
  return (size_t)ny * (size_t)(nx + 2) + (size_t)(ny + 2) * (size_t)nx;
}

// Rounds the EOS and WENO constants to FP32 once on the host (the split
// path's reconstruction and Riemann solve read them as floats).
inline void set_fp32_constants(DevParams& D) {
  for (int f = 0; f < kMaxFluids; ++f) {
    D.gammas_f[f] = (float)D.gammas[f];
    D.pi_infs_f[f] = (float)D.pi_infs[f];
  }
  D.weno_eps_f = (float)D.weno_eps;
}

// Split precision on a grid whose FP32 coefficient records are the same for
// every cell of a direction (uniform spacing): that one record per
// direction, each coefficient duplicated into both lanes of a packed FP32
// pair (the reconstruction works on pairs of variables).  The kernels
// receive it by value, so the reconstruction takes its coefficients from the
// constant bank instead of staging per-cell records in shared memory.
// on[d] = 0: per-cell records.
template <int NDIR>
struct UniformCoefT {
  int on[NDIR];
  unsigned long long rec[NDIR][kCoefRec];  // (c, c) pairs
};
using UniformCoef = UniformCoefT<3>;

// Viscous parameters: fluid_pp(i)%Re(1:2) as the reference's Re_size, Re_idx
// and Res (m_global_parameters.fpp:300-336, m_viscous.fpp:33-45), and the
// cell-centre spacings of the velocity gradients, dcc[d][i] = x_cc(i) -
// x_cc(i-1) for i = 0 .. n_d (m_start_up.fpp:342-343 and the ghost centres of
// s_populate_grid_variables_buffers).
struct ViscParams {
  double res[2][kMaxFluids];
  int re_size[2];
  int re_idx[2][kMaxFluids];
  const double* dcc[3];
  // weno_Re_flux = T: the face velocity gradients, prepared per stage by
  // visc_gradients_launch (mfc_visc_grad.cu), read instead of the finite
  // differences.  fg[0]: x faces [c*ND+d][ny][nx+1] (face i+1/2 at i+1),
  // fg[1]: y faces [c*ND+d][ny+1][nx] (face j+1/2 at j+1); d u_c / d x_d.
  // NULL: the finite differences of weno_Re_flux = F.
  const double* fg[2];
};


// Equation index layout, m_global_parameters.fpp:302-310 (0-based).
template <int ND, int NF>
struct Eqs {
  static constexpr int S = 2 * NF + ND + 1;
  static constexpr int MOM = NF;
  static constexpr int E = NF + ND;
  static constexpr int ADV = NF + ND + 1;
};

// Ghost-cell mapping of m_rhs.fpp:686-908: a cell index c outside [0, n) is
// replaced by the interior cell whose value the ghost holds; *flip is set
// when the normal momentum changes sign (symmetry, bc -2).  bc <= -3 is
// ghost-cell extrapolation, -2 symmetry, -1 periodic.  The final clamp only
// matters for cells of partial edge tiles that lie beyond the ghost layers;
// their values never reach a stored result.
__device__ __forceinline__ int map_cell(int c, int n, int bcb, int bce, bool* flip) {
  if (c < 0) {
    *flip = (bcb == -2);
    c = (bcb == -1) ? c + n : (bcb == -2) ? -c - 1 : 0;
  } else if (c >= n) {
    *flip = (bce == -2);
    c = (bce == -1) ? c - n : (bce == -2) ? 2 * n - 1 - c : n - 1;
  }
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

// Coefficient tables cover cells -kCoefPad .. n-1+kCoefPad; cells of partial
// edge tiles beyond that range reuse the last record (their results are
// never stored).
constexpr int kCoefPad = 4;
__device__ __forceinline__ int clamp_coef_index(int c, int n) {
  return c < -kCoefPad ? -kCoefPad : (c > n - 1 + kCoefPad ? n - 1 + kCoefPad : c);
}

// FP64 <-> FP32 conversions for the split path done with integer operations
// on the IEEE-754 bit fields, so that they do not occupy GB300's narrow FP64
// pipe (which executes the hardware conversion instructions).  double ->
// float truncates the significand (error < 1 ulp of float), flushes results
// below the smallest normal float to signed zero and maps everything above
// the float range (and NaN) to infinity; float -> double is exact for
// normal numbers, zero, infinities and NaNs (denormal floats are flushed to
// zero, as the split units run with -ftz=true).
//
// Bit-level forms, shared by host and device.  double -> float from the high
// and low words: |x| >= 2^-126 and below 2^128 gives (E - 896) << 23 | the top
// 23 significand bits; the subtraction is done before the shift so that the
// exponent and significand move together (4 integer operations plus the two
// range selects).
__host__ __device__ __forceinline__ uint32_t d2f_trunc_word(uint32_t hi, uint32_t lo) {
  const uint32_t a = hi & 0x7fffffffu;
  const uint32_t t = ((a - 0x38000000u) << 3) | (lo >> 29);
  const uint32_t r = a < 0x38100000u ? 0u : (a >= 0x47f00000u ? 0x7f800000u : t);
  return r | (hi & 0x80000000u);
}

// float -> double high word (the low word is the float's bits << 29 for
// normal floats, 0 otherwise): the exponent is rebiased by +896, or moved
// from all ones to all ones, so that infinities and NaNs stay what they are.
__host__ __device__ __forceinline__ uint32_t f2d_high_word(uint32_t b) {
  const uint32_t a = b & 0x7fffffffu;
  const uint32_t t = (a >> 3) + (a >= 0x7f800000u ? 0x70000000u : 0x38000000u);
  return (a < 0x00800000u ? 0u : t) | (b & 0x80000000u);
}

__device__ __forceinline__ float d2f_bits(double x) {
  return __uint_as_float(d2f_trunc_word((uint32_t)__double2hiint(x), (uint32_t)__double2loint(x)));
}

__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t lo = (b & 0x7fffffffu) < 0x00800000u ? 0u : (b << 29);
  return __hiloint2double((int)f2d_high_word(b), (int)lo);
}

// Programmatic dependent launch.  The single-case stage kernels are launched
// with cudaLaunchAttributeProgrammaticStreamSerialization, so the next RK
// stage's kernel may become resident while this one drains its last tiles:
// griddep_wait() holds a kernel until the previous one has completed and its
// stores are visible (everything before it may read only constant tables),
// griddep_launch_dependents() lets the next kernel start.  Both are no-ops
// in a kernel launched without the attribute.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Approximate FP32 reciprocal (PTX rcp.approx.ftz.f32); the split path
// refines it where more accuracy is needed.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// ---------------------------------------------------------------------------
// Correctly rounded FP64 division with a shared divisor.
//
// GB300 issues two FP64 operations per SM and clock, and an IEEE division
// costs several of them, so the WENO weights (alpha_k = d_k / b_k^2 for both
// faces, omega_k = alpha_k / sum alpha) would spend about half of the plain
// path's FP64 issue on divisions.  The quotient must still be the correctly
// rounded one (the plain path reproduces the CPU reference bit for bit).
// Here the reciprocal and every quotient are formed in 64-bit integer (and
// FP32) arithmetic, on pipes that sit idle while the FP64 pipe is the
// bottleneck (J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, 2nd ed., ch. 4-5 and 9: Newton-Raphson
// reciprocals, exact remainders, and the fact that a quotient of two
// doubles never lies exactly halfway between two doubles).
//
//   divisor(b): significand B (53 bits with the implicit one) of |b|;
//     r = FP32 reciprocal of B 2^-52 (rcp.approx, one FP32 Newton step);
//     R = 2^64 / (B 2^-52) (1 + e), |e| < 2^-46, by one Newton step from r
//     in 64-bit fixed point (all ones for B = 2^52).
//   div_rn(a):  significand A of |a|; As = A, or 2A when A < B, so that
//     As / B lies in [1, 2);  Q = floor(As R / 2^64) approximates
//     As 2^52 / B within 2^8;  D = As 2^52 - B Q is exact in 64 bits
//     (|D| < 2^61);  dl = floor(D / B) from D's top bits and R's top 24
//     bits, off by at most one;  Q += dl, D -= dl B leaves D / B in
//     (-2^-12, 1 + 2^-12), so the rounded quotient is Q + (2 D > B) (a tie
//     is impossible); a carry to 2^53 moves to the next binade.  Sign and
//     exponent come from a's and b's fields.
//
// Neither a divisor nor a quotient issues an FP64 operation.  The argument holds
// while |a| and |b| lie in [2^-250, 2^251): the quotient is then a normal
// double.  Anything else (zero, subnormal, huge, inf or NaN operands) takes
// the ordinary IEEE division, except a zero numerator over an in-window
// divisor, whose signed-zero quotient is written directly.
constexpr uint32_t kDivExpLo = 1023u - 250u, kDivExpSpan = 501u;
constexpr uint64_t kSigMask = 0xfffffffffffffULL, kSigOne = 1ULL << 52;

static __device__ __noinline__ double div_ieee(double a, double b) { return a / b; }

struct DivisorF64 {
  double b;
  uint64_t B, R;  // significand with the implicit one; 2^64 / (B 2^-52) in 64-bit fixed point
  uint32_t se;    // b's sign (bit 11) and biased exponent
  bool ok;        // b inside the window
};

__device__ __forceinline__ DivisorF64 divisor(double b) {
  const uint32_t hi = (uint32_t)__double2hiint(b), lo = (uint32_t)__double2loint(b);
  const uint32_t eb = (hi >> 20) & 0x7ffu;
  // FP32 reciprocal of b's significand rounded to 24 bits (a carry to 2.0 is
  // harmless), refined by one FP32 Newton step: r in [1/2, 1], |r f - 1| < 2^-23
  const float f = __uint_as_float(((0x3f800000u | ((hi & 0xfffffu) << 3) | (lo >> 29)) + ((lo >> 28) & 1u)));
  const float r0 = rcp_approx(f);
  const uint32_t rb = __float_as_uint(fmaf(r0, fmaf(-f, r0, 1.0f), r0));
  // R0 = r 2^64 = m 2^(40+k) (2^64 wraps to 0, which the step below undoes);
  // one Newton step in fixed point, R = R0 + R0 (2^116 - B R0) 2^-116, with
  // 2^116 - B R0 = e 2^(40+k) and e = 2^(76-k) - B m, which is small and so
  // equals minus the low 64 bits of B m
  const uint32_t k = (rb >> 23) - 126u;
  const uint64_t m = (rb & 0x7fffffu) | 0x800000u;
  const uint64_t B = (((uint64_t)hi << 32 | lo) & kSigMask) | kSigOne;
  const int64_t e = -(int64_t)(B * m);
  const int64_t corr = ((int64_t)m * (e >> 14)) >> (22 - 2 * k);
  const uint64_t R = B == kSigOne ? ~0ULL : (m << (40 + k)) + (uint64_t)corr;
  return {b, B, R, (hi >> 20) & 0xfffu, eb - kDivExpLo < kDivExpSpan};
}

__device__ __forceinline__ double div_rn(double a, const DivisorF64& d) {
  const int64_t ab = __double_as_longlong(a);
  const uint32_t ea = (uint32_t)(ab >> 52) & 0x7ffu;
  if (!d.ok || ea - kDivExpLo >= kDivExpSpan) {
    if (d.ok && (ab & 0x7fffffffffffffffLL) == 0)
      return __longlong_as_double((ab ^ __double_as_longlong(d.b)) & (int64_t)0x8000000000000000ULL);
    return div_ieee(a, d.b);
  }
  const uint64_t A = ((uint64_t)ab & kSigMask) | kSigOne;
  const uint32_t lt = A < d.B ? 1u : 0u;
  const uint64_t As = A << lt;
  uint64_t Q = __umul64hi(As, d.R);
  const int64_t D = (int64_t)((As << 52) - d.B * Q);
  const int64_t dl = ((D >> 32) * (int64_t)(d.R >> 40)) >> 44;
  Q += (uint64_t)dl;
  const int64_t D1 = D - dl * (int64_t)d.B;
  Q += (2 * D1 > (int64_t)d.B) ? 1u : 0u;
  const uint32_t carry = (uint32_t)(Q >> 53);  // rounded up to 2^53: the next binade
  Q >>= carry;
  const uint64_t eq = (uint64_t)(ea - (d.se & 0x7ffu) + 1023u - lt + carry);
  const uint64_t sign = (uint64_t)(((uint32_t)((uint64_t)ab >> 63)) ^ (d.se >> 11)) << 63;
  return __longlong_as_double((int64_t)(sign | (eq << 52) | (Q & kSigMask)));
}

// FP32 counterparts (split path): the division itself, under the unit's
// -prec-div setting.
struct DivisorF32 {
  float b;
};
__device__ __forceinline__ DivisorF32 divisor(float b) { return {b}; }
__device__ __forceinline__ float div_rn(float a, const DivisorF32& d) { return a / d.b; }

// True for an infinity or NaN: the exponent field of the high word is all
// ones.  The mask is applied in inline PTX so that the test stays an integer
// operation (an equivalent floating-point comparison would occupy GB300's
// narrow FP64 pipe).
__device__ __forceinline__ bool not_finite(double x) {
  uint32_t e;
  asm("and.b32 %0, %1, 0x7ff00000;" : "=r"(e) : "r"(__double2hiint(x)));
  return e == 0x7ff00000u;
}

// cons -> prim of one cell, m_variables_conversion.fpp:326-373 and
// s_compute_pressure :98-106.  q holds the S conservative values on entry and
// the primitive ones on exit (partial densities and volume fractions are the
// same in both sets).  Always FP64: the pressure recovery from total energy
// cancels digits in the stiffened-gas EOS.
template <int ND, int NF>
__device__ __forceinline__ void cons_to_prim(double (&q)[Eqs<ND, NF>::S], const DevParams& P) {
  using Q = Eqs<ND, NF>;
  double rho = 0.0, gam = 0.0, pinf = 0.0, dyn = 0.0;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    rho = rho + q[f];
    gam = gam + q[Q::ADV + f] * P.gammas[f];
    pinf = pinf + q[Q::ADV + f] * P.pi_infs[f];
  }
  rho = fmax(rho, 1e-16);
  const DivisorF64 R = divisor(rho);
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const double mom = q[Q::MOM + d];
    const double vel = div_rn(mom, R);
    q[Q::MOM + d] = vel;
    dyn = dyn + 0.5 * mom * vel;
  }
  q[Q::E] = div_rn(q[Q::E] - dyn - pinf, divisor(gam));
}

// The reference's run-time stability criterion of one cell
// (m_data_output.fpp:197-242): ICFL = dt / min_d(dx_d / (|u_d| + c)) with the
// mixture sound speed c = sqrt(((gamma + 1) p + pi_inf) / (gamma rho)),
// from the cell's conservative state.  Non-negative, so the bit patterns of
// the doubles order like their values (atomicMax on the bits).  nonphys is
// set when the squared sound speed is not positive ((gamma + 1) p + pi_inf
// <= 0 or NaN: a pressure below the stiffened gas's limit).
template <int ND, int NF>
__device__ __forceinline__ double cell_icfl(const double (&q)[Eqs<ND, NF>::S], const DevParams& P, double dt,
                                            const double (&inv_d)[ND], bool& nonphys) {
  using Q = Eqs<ND, NF>;
  double p[Q::S];
#pragma unroll
  for (int v = 0; v < Q::S; ++v) p[v] = q[v];
  cons_to_prim<ND, NF>(p, P);
  double rho = 0.0, gam = 0.0, pinf = 0.0;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    rho = rho + p[f];
    gam = gam + p[Q::ADV + f] * P.gammas[f];
    pinf = pinf + p[Q::ADV + f] * P.pi_infs[f];
  }
  const double c2 = ((gam + 1.0) * p[Q::E] + pinf) / (gam * rho);
  nonphys = !(c2 > 0.0);
  const double c = sqrt(c2);
  double rate = 0.0;
#pragma unroll
  for (int d = 0; d < ND; ++d) rate = fmax(rate, (fabs(p[Q::MOM + d]) + c) * inv_d[d]);
  const double icfl = dt * rate;
  return icfl != icfl ? __longlong_as_double(0x7ff8000000000000ll) : icfl;
}

__device__ __forceinline__ void monitor_max(unsigned long long* w, double v) {
  // NaN (all exponent bits, nonzero mantissa) orders above +inf as unsigned bits
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_down_sync(0xffffffffu, b, o);
    b = other > b ? other : b;
  }
  if ((threadIdx.x & 31) == 0 && b) atomicMax(w, b);
}

// cons -> prim for the split-precision path.  Only what cancels stays FP64:
// E - Pi (Pi = sum alpha_i pi_inf_i), where the stiffened-gas EOS of water
// cancels ~4-5 digits (E and Pi ~ 1e9, Gamma p ~ 1e4).  The density, Gamma,
// the velocity and the kinetic energy rho|u|^2/2 are well conditioned and
// computed in FP32 (relative error ~1e-7 of each, so ~1e-7 of p at most where
// the kinetic energy is comparable to Gamma p), then
// p = (float)((E - Pi) - (double)KE) / Gamma.
// GB300's FP64 pipe bounds the split stage, and this conversion runs on every
// halo cell as well (1.75x the interior for 16x16 tiles).
template <int ND, int NF>
__device__ __forceinline__ void cons_to_prim_split(const double (&q)[Eqs<ND, NF>::S], const DevParams& P,
                                                   float (&out)[Eqs<ND, NF>::S]) {
  using Q = Eqs<ND, NF>;
  double pinf = 0.0;
  float rho = 0.f, gam = 0.f;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    out[f] = d2f_bits(q[f]);
    out[Q::ADV + f] = d2f_bits(q[Q::ADV + f]);
    rho = rho + out[f];
    gam = fmaf(out[Q::ADV + f], d2f_bits(P.gammas[f]), gam);
    pinf = fma(q[Q::ADV + f], P.pi_infs[f], pinf);
  }
  rho = fmaxf(rho, 1e-16f);
  const float irho = __fdividef(1.f, rho);
  float m2 = 0.f;
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const float m = d2f_bits(q[Q::MOM + d]);
    out[Q::MOM + d] = m * irho;
    m2 = fmaf(m, m, m2);
  }
  const double dE = (q[Q::E] - pinf) - f2d_bits(0.5f * m2 * irho);
  out[Q::E] = __fdividef(d2f_bits(dE), gam);
}

// ---------------------------------------------------------------------------
// Packed FP32 pairs for the split path: two lanes of one 64-bit register,
// computed by one instruction (FFMA2 / FMUL2 / FADD2 on GB300).  Each lane
// is rounded exactly as the scalar operation would round it (to nearest,
// subnormals flushed like the split units' -ftz=true), so a pair gives the
// bits of two scalar evaluations with half the issue slots.
using f32x2 = unsigned long long;
__device__ __forceinline__ f32x2 f2_pack(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 p, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(p));
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 f2_rcp(f32x2 a) {
  float x, y;
  f2_unpack(a, x, y);
  return f2_pack(rcp_approx(x), rcp_approx(y));
}

// WENO5 for the split-precision path, two variables at once (one per lane):
// the stencils, smoothness indicators and weights of weno_cell, with the
// divisions regrouped -- one reciprocal of beta_k^2 shared by the left and
// right weights and one reciprocal of sum(alpha_k) per face value.  The
// weights are still normalised before they multiply the candidate values,
// so nothing grows beyond the operands' range.  Mathematically identical to
// weno_cell; rounding differs.  C(k) returns coefficient k of the cell's
// record as a (c, c) pair.
template <class Coef>
__device__ __forceinline__ void weno5_pair_fast(const Coef& C, const f32x2 (&v)[5], f32x2 eps, f32x2& vL,
                                                f32x2& vR) {
  const f32x2 d1 = f2_sub(v[4], v[3]), d0 = f2_sub(v[3], v[2]), dm1 = f2_sub(v[2], v[1]), dm2 = f2_sub(v[1], v[0]);
  const f32x2 b0 = f2_fma(d1, f2_fma(C(kBeta + 0), d1, f2_mul(C(kBeta + 1), d0)), f2_fma(f2_mul(C(kBeta + 2), d0), d0, eps));
  const f32x2 b1 = f2_fma(d0, f2_fma(C(kBeta + 3), d0, f2_mul(C(kBeta + 4), dm1)), f2_fma(f2_mul(C(kBeta + 5), dm1), dm1, eps));
  const f32x2 b2 = f2_fma(dm1, f2_fma(C(kBeta + 6), dm1, f2_mul(C(kBeta + 7), dm2)), f2_fma(f2_mul(C(kBeta + 8), dm2), dm2, eps));
  const f32x2 r0 = f2_rcp(f2_mul(b0, b0)), r1 = f2_rcp(f2_mul(b1, b1)), r2 = f2_rcp(f2_mul(b2, b2));
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const int kP = side ? kPR : kPL, kD = side ? kDR : kDL;
    const f32x2 p0 = f2_fma(C(kP + 1), d0, f2_fma(C(kP + 0), d1, v[2]));
    const f32x2 p1 = f2_fma(C(kP + 3), dm1, f2_fma(C(kP + 2), d0, v[2]));
    const f32x2 p2 = f2_fma(C(kP + 5), dm2, f2_fma(C(kP + 4), dm1, v[2]));
    const f32x2 a0 = f2_mul(C(kD + 0), r0), a1 = f2_mul(C(kD + 1), r1), a2 = f2_mul(C(kD + 2), r2);
    const f32x2 is = f2_rcp(f2_add(f2_add(a0, a1), a2));
    const f32x2 val = f2_fma(f2_mul(a2, is), p2, f2_fma(f2_mul(a1, is), p1, f2_mul(f2_mul(a0, is), p0)));
    if (side) vR = val;
    else vL = val;
  }
}

// WENO reconstruction of one cell from its stencil, m_weno.fpp:391-536.
// c: the cell's kNumCoef coefficients; v[k] = value at offset k - 2.
// Returns the left-face (x_{j-1/2}) and right-face (x_{j+1/2}) values.
template <int WO, class RT>
__device__ __forceinline__ void weno_cell(const RT* __restrict__ c, const RT (&v)[5], RT eps, RT& vL, RT& vR) {
  if constexpr (WO == 1) {
    vL = v[2];
    vR = v[2];
  } else if constexpr (WO == 3) {
    const RT d0 = v[3] - v[2];
    const RT dm1 = v[2] - v[1];
    const RT b0 = c[kBeta + 0] * d0 * d0 + eps;
    const RT b1 = c[kBeta + 3] * dm1 * dm1 + eps;
    RT p0 = v[2] + c[kPL + 0] * d0;
    RT p1 = v[2] + c[kPL + 2] * dm1;
    const auto D0 = divisor(b0 * b0), D1 = divisor(b1 * b1);
    RT a0 = div_rn(c[kDL + 0], D0), a1 = div_rn(c[kDL + 1], D1);
    auto S = divisor(a0 + a1);
    vL = div_rn(a0, S) * p0 + div_rn(a1, S) * p1;
    p0 = v[2] + c[kPR + 0] * d0;
    p1 = v[2] + c[kPR + 2] * dm1;
    a0 = div_rn(c[kDR + 0], D0);
    a1 = div_rn(c[kDR + 1], D1);
    S = divisor(a0 + a1);
    vR = div_rn(a0, S) * p0 + div_rn(a1, S) * p1;
  } else {
    const RT d1 = v[4] - v[3];
    const RT d0 = v[3] - v[2];
    const RT dm1 = v[2] - v[1];
    const RT dm2 = v[1] - v[0];
    const RT b0 = c[kBeta + 0] * d1 * d1 + c[kBeta + 1] * d1 * d0 + c[kBeta + 2] * d0 * d0 + eps;
    const RT b1 = c[kBeta + 3] * d0 * d0 + c[kBeta + 4] * d0 * dm1 + c[kBeta + 5] * dm1 * dm1 + eps;
    const RT b2 = c[kBeta + 6] * dm1 * dm1 + c[kBeta + 7] * dm1 * dm2 + c[kBeta + 8] * dm2 * dm2 + eps;
    // b_k^2 is the divisor of both faces' alpha_k, sum(alpha) of the three omega_k of a face
    const auto D0 = divisor(b0 * b0), D1 = divisor(b1 * b1), D2 = divisor(b2 * b2);
    {
      const RT p0 = v[2] + c[kPL + 0] * d1 + c[kPL + 1] * d0;
      const RT p1 = v[2] + c[kPL + 2] * d0 + c[kPL + 3] * dm1;
      const RT p2 = v[2] + c[kPL + 4] * dm1 + c[kPL + 5] * dm2;
      const RT a0 = div_rn(c[kDL + 0], D0), a1 = div_rn(c[kDL + 1], D1), a2 = div_rn(c[kDL + 2], D2);
      const auto S = divisor(a0 + a1 + a2);
      vL = div_rn(a0, S) * p0 + div_rn(a1, S) * p1 + div_rn(a2, S) * p2;
    }
    {
      const RT p0 = v[2] + c[kPR + 0] * d1 + c[kPR + 1] * d0;
      const RT p1 = v[2] + c[kPR + 2] * d0 + c[kPR + 3] * dm1;
      const RT p2 = v[2] + c[kPR + 4] * dm1 + c[kPR + 5] * dm2;
      const RT a0 = div_rn(c[kDR + 0], D0), a1 = div_rn(c[kDR + 1], D1), a2 = div_rn(c[kDR + 2], D2);
      const auto S = divisor(a0 + a1 + a2);
      vR = div_rn(a0, S) * p0 + div_rn(a1, S) * p1 + div_rn(a2, S) * p2;
    }
  }
}

// One face value of weno_cell (SIDE 0: left face x_{j-1/2}, 1: right face
// x_{j+1/2}), for a cell whose other face value nobody reads: the smoothness
// indicators, divisors and the chosen side are the same operations as in
// weno_cell, so the value has the same bits.
template <int WO, int SIDE, class RT>
__device__ __forceinline__ RT weno_cell_side(const RT* __restrict__ c, const RT (&v)[5], RT eps) {
  constexpr int kP = SIDE ? kPR : kPL, kD = SIDE ? kDR : kDL;
  if constexpr (WO == 1) {
    return v[2];
  } else if constexpr (WO == 3) {
    const RT d0 = v[3] - v[2];
    const RT dm1 = v[2] - v[1];
    const RT b0 = c[kBeta + 0] * d0 * d0 + eps;
    const RT b1 = c[kBeta + 3] * dm1 * dm1 + eps;
    const RT p0 = v[2] + c[kP + 0] * d0;
    const RT p1 = v[2] + c[kP + 2] * dm1;
    const auto D0 = divisor(b0 * b0), D1 = divisor(b1 * b1);
    const RT a0 = div_rn(c[kD + 0], D0), a1 = div_rn(c[kD + 1], D1);
    const auto S = divisor(a0 + a1);
    return div_rn(a0, S) * p0 + div_rn(a1, S) * p1;
  } else {
    const RT d1 = v[4] - v[3];
    const RT d0 = v[3] - v[2];
    const RT dm1 = v[2] - v[1];
    const RT dm2 = v[1] - v[0];
    const RT b0 = c[kBeta + 0] * d1 * d1 + c[kBeta + 1] * d1 * d0 + c[kBeta + 2] * d0 * d0 + eps;
    const RT b1 = c[kBeta + 3] * d0 * d0 + c[kBeta + 4] * d0 * dm1 + c[kBeta + 5] * dm1 * dm1 + eps;
    const RT b2 = c[kBeta + 6] * dm1 * dm1 + c[kBeta + 7] * dm1 * dm2 + c[kBeta + 8] * dm2 * dm2 + eps;
    const auto D0 = divisor(b0 * b0), D1 = divisor(b1 * b1), D2 = divisor(b2 * b2);
    const RT p0 = v[2] + c[kP + 0] * d1 + c[kP + 1] * d0;
    const RT p1 = v[2] + c[kP + 2] * d0 + c[kP + 3] * dm1;
    const RT p2 = v[2] + c[kP + 4] * dm1 + c[kP + 5] * dm2;
    const RT a0 = div_rn(c[kD + 0], D0), a1 = div_rn(c[kD + 1], D1), a2 = div_rn(c[kD + 2], D2);
    const auto S = divisor(a0 + a1 + a2);
    return div_rn(a0, S) * p0 + div_rn(a1, S) * p1 + div_rn(a2, S) * p2;
  }
}

// HLLC flux across one face, m_riemann_solvers.fpp:132-327, for sweep
// direction DIR.  qL/qR are the primitive states left and right of the face
// (the reference's vR(j) and vL(j+1), after its argument swap at
// m_rhs.fpp:545-556).  F receives the S fluxes, ustar the interface velocity
// (vel_src(dir_idx(1)) -> flux_src(advxb)).
//
// xi_M and xi_P of the reference are exactly 1/0 or 0/1 (0.5 +- sign(0.5,
// s_S)), so the flux is the upwind side's term alone; evaluating only that
// side gives the same values and halves the arithmetic.
//
// VS: also return vel_src of every component, m_riemann_solvers.fpp:314-324,
// with both sides' terms exactly as the reference writes them (the viscous
// energy flux needs the tangential components).
template <int ND, int NF, int DIR, class RT, bool VS = false>
__device__ __forceinline__ void hllc_face(const RT (&qL)[Eqs<ND, NF>::S], const RT (&qR)[Eqs<ND, NF>::S],
                                          const RT (&gam_i)[NF], const RT (&pi_i)[NF], RT (&F)[Eqs<ND, NF>::S],
                                          RT& ustar, RT* vsrc = nullptr) {
  using Q = Eqs<ND, NF>;
  RT rmsL = RT(0), rmsR = RT(0);
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    rmsL = rmsL + qL[Q::MOM + d] * qL[Q::MOM + d];
    rmsR = rmsR + qR[Q::MOM + d] * qR[Q::MOM + d];
  }
  const RT pL = qL[Q::E], pR = qR[Q::E];
  RT rhoL = RT(0), gamL = RT(0), piL = RT(0), rhoR = RT(0), gamR = RT(0), piR = RT(0);
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    rhoL = rhoL + qL[f];
    gamL = gamL + qL[Q::ADV + f] * gam_i[f];
    piL = piL + qL[Q::ADV + f] * pi_i[f];
    rhoR = rhoR + qR[f];
    gamR = gamR + qR[Q::ADV + f] * gam_i[f];
    piR = piR + qR[Q::ADV + f] * pi_i[f];
  }
  const RT EL = gamL * pL + piL + RT(0.5) * rhoL * rmsL;
  const RT ER = gamR * pR + piR + RT(0.5) * rhoR * rmsR;
  const RT HL = div_rn(EL + pL, divisor(rhoL));
  const RT HR = div_rn(ER + pR, divisor(rhoR));
  const RT cL = sqrt(div_rn(HL - RT(0.5) * rmsL, divisor(gamL)));
  const RT cR = sqrt(div_rn(HR - RT(0.5) * rmsR, divisor(gamR)));
  const RT uL = qL[Q::MOM + DIR], uR = qR[Q::MOM + DIR];
  const RT sL = fmin(uL - cL, uR - cR);
  const RT sR = fmax(uR + cR, uL + cL);
  const RT sS = div_rn(pR - pL + rhoL * uL * (sL - uL) - rhoR * uR * (sR - uR),
                      divisor(rhoL * (sL - uL) - rhoR * (sR - uR)));
  if constexpr (VS) {
    const RT sM = fmin(RT(0), sL), sP = fmax(RT(0), sR);
    const RT xiL = div_rn(sL - uL, divisor(sL - sS));
    const RT xiR = div_rn(sR - uR, divisor(sR - sS));
    const RT xiM = RT(0.5) + copysign(RT(0.5), sS);
    const RT xiP = RT(0.5) - copysign(RT(0.5), sS);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      const RT flg = d == DIR ? RT(1) : RT(0);
      vsrc[d] = xiM * (qL[Q::MOM + d] + flg * sM * (xiL - RT(1))) + xiP * (qR[Q::MOM + d] + flg * sP * (xiR - RT(1)));
    }
  }
  if (!signbit(sS)) {  // xi_M = 1, xi_P = 0
    const RT sM = fmin(RT(0), sL);
    const RT xi = div_rn(sL - uL, divisor(sL - sS));
    const RT w = uL + sM * (xi - RT(1));
#pragma unroll
    for (int f = 0; f < NF; ++f) F[f] = qL[f] * w;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      const RT vd = qL[Q::MOM + d];
      if (d == DIR) F[Q::MOM + d] = rhoL * (uL * vd + sM * (xi * sS - vd)) + pL;
      else F[Q::MOM + d] = rhoL * (uL * vd + sM * (xi * vd - vd));
    }
    F[Q::E] = uL * (EL + pL) + sM * (xi * (EL + (sS - uL) * (rhoL * sS + div_rn(pL, divisor(sL - uL)))) - EL);
#pragma unroll
    for (int f = 0; f < NF; ++f) F[Q::ADV + f] = qL[Q::ADV + f] * w;
    ustar = w;
  } else {  // xi_M = 0, xi_P = 1
    const RT sP = fmax(RT(0), sR);
    const RT xi = div_rn(sR - uR, divisor(sR - sS));
    const RT w = uR + sP * (xi - RT(1));
#pragma unroll
    for (int f = 0; f < NF; ++f) F[f] = qR[f] * w;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      const RT vd = qR[Q::MOM + d];
      if (d == DIR) F[Q::MOM + d] = rhoR * (uR * vd + sP * (xi * sS - vd)) + pR;
      else F[Q::MOM + d] = rhoR * (uR * vd + sP * (xi * vd - vd));
    }
    F[Q::E] = uR * (ER + pR) + sP * (xi * (ER + (sS - uR) * (rhoR * sS + div_rn(pR, divisor(sR - uR)))) - ER);
#pragma unroll
    for (int f = 0; f < NF; ++f) F[Q::ADV + f] = qR[Q::ADV + f] * w;
    ustar = w;
  }
}

// r + a*b: one fused multiply-add on the split path; on the FP64 path the
// reference's rounded product followed by the rounded sum.
__device__ __forceinline__ float mul_add(float a, float b, float r) { return fmaf(a, b, r); }
__device__ __forceinline__ double mul_add(double a, double b, double r) { return r + a * b; }

// HLLC for the split-precision path: the same wave speeds, star state and
// upwind flux as hllc_face (same cases, same sign test on s_S), in FP32 with
// every fused multiply-add written out as fmaf and the quotients as fast
// reciprocal divisions.  The split units are compiled without automatic
// contraction, so every tile shape and code path rounds identically.
// Tangential momentum flux: rho v_d (u + s_M (xi - 1)) = rho v_d w.
template <int ND, int NF, int DIR>
__device__ __forceinline__ void hllc_face_fast(const float (&qL)[Eqs<ND, NF>::S], const float (&qR)[Eqs<ND, NF>::S],
                                               const float (&gam_i)[NF], const float (&pi_i)[NF],
                                               float (&F)[Eqs<ND, NF>::S], float& ustar) {
  using Q = Eqs<ND, NF>;
  float rmsL = qL[Q::MOM] * qL[Q::MOM], rmsR = qR[Q::MOM] * qR[Q::MOM];
#pragma unroll
  for (int d = 1; d < ND; ++d) {
    rmsL = fmaf(qL[Q::MOM + d], qL[Q::MOM + d], rmsL);
    rmsR = fmaf(qR[Q::MOM + d], qR[Q::MOM + d], rmsR);
  }
  const float pL = qL[Q::E], pR = qR[Q::E];
  float rhoL = qL[0], gamL = qL[Q::ADV] * gam_i[0], piL = qL[Q::ADV] * pi_i[0];
  float rhoR = qR[0], gamR = qR[Q::ADV] * gam_i[0], piR = qR[Q::ADV] * pi_i[0];
#pragma unroll
  for (int f = 1; f < NF; ++f) {
    rhoL = rhoL + qL[f];
    gamL = fmaf(qL[Q::ADV + f], gam_i[f], gamL);
    piL = fmaf(qL[Q::ADV + f], pi_i[f], piL);
    rhoR = rhoR + qR[f];
    gamR = fmaf(qR[Q::ADV + f], gam_i[f], gamR);
    piR = fmaf(qR[Q::ADV + f], pi_i[f], piR);
  }
  const float EL = fmaf(0.5f * rhoL, rmsL, fmaf(gamL, pL, piL));
  const float ER = fmaf(0.5f * rhoR, rmsR, fmaf(gamR, pR, piR));
  const float HL = __fdividef(EL + pL, rhoL), HR = __fdividef(ER + pR, rhoR);
  const float cL = sqrtf(__fdividef(fmaf(-0.5f, rmsL, HL), gamL));
  const float cR = sqrtf(__fdividef(fmaf(-0.5f, rmsR, HR), gamR));
  const float uL = qL[Q::MOM + DIR], uR = qR[Q::MOM + DIR];
  const float sL = fminf(uL - cL, uR - cR);
  const float sR = fmaxf(uR + cR, uL + cL);
  const float mL = rhoL * (sL - uL), mR = rhoR * (sR - uR);
  const float sS = __fdividef(fmaf(-mR, uR, fmaf(mL, uL, pR - pL)), mL - mR);
  const bool left = !signbit(sS);  // xi_M = 1, xi_P = 0
  const float rho = left ? rhoL : rhoR, u = left ? uL : uR, p = left ? pL : pR, E = left ? EL : ER;
  const float s = left ? fminf(0.f, sL) : fmaxf(0.f, sR);  // s_M or s_P
  const float sk = left ? sL : sR;
  const float xi = __fdividef(sk - u, sk - sS);
  const float w = fmaf(s, xi - 1.f, u);
  const float(&q)[Eqs<ND, NF>::S] = left ? qL : qR;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    F[f] = q[f] * w;
    F[Q::ADV + f] = q[Q::ADV + f] * w;
  }
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const float vd = q[Q::MOM + d];
    if (d == DIR) F[Q::MOM + d] = fmaf(rho, fmaf(u, vd, s * fmaf(xi, sS, -vd)), p);
    else F[Q::MOM + d] = rho * vd * w;
  }
  const float t = fmaf(rho, sS, __fdividef(p, sk - u));
  F[Q::E] = fmaf(s, fmaf(xi, fmaf(sS - u, t, E), -E), u * (E + p));
  ustar = w;
}

// Viscous source flux of one face, s_compute_viscous_source_flux
// (m_riemann_solvers.fpp:683-902), from the face's left/right states (for the
// mixture Reynolds numbers, :169-230), vel_src vs and the face velocity
// gradients dx[c] = d u_c/dx, dy[c] = d u_c/dy (m_viscous.fpp:159-370).
// out: the x-momentum, y-momentum and energy source fluxes.
template <int ND, int NF, int DIR, class RT>
__device__ __forceinline__ void viscous_face_flux(const RT (&qL)[Eqs<ND, NF>::S], const RT (&qR)[Eqs<ND, NF>::S],
                                                  const ViscParams& V, const RT (&vs)[ND], const RT (&dx)[2],
                                                  const RT (&dy)[2], RT (&out)[3]) {
  using Q = Eqs<ND, NF>;
  RT re_avg[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    RT reL = RT(-1e6), reR = RT(-1e6);
    if (V.re_size[r] > 0) reL = reR = RT(0);
    for (int q = 0; q < V.re_size[r]; ++q) {
      const int f = V.re_idx[r][q];
      const auto D = divisor(RT(V.res[r][f]));
      reL = div_rn(qL[Q::ADV + f], D) + reL;
      reR = div_rn(qR[Q::ADV + f], D) + reR;
    }
    reL = div_rn(RT(1), divisor(reL < RT(1e-16) ? RT(1e-16) : reL));
    reR = div_rn(RT(1), divisor(reR < RT(1e-16) ? RT(1e-16) : reR));
    re_avg[r] = div_rn(RT(2), divisor(div_rn(RT(1), divisor(reL)) + div_rn(RT(1), divisor(reR))));
  }
  const bool shear = V.re_size[0] > 0, bulk = V.re_size[1] > 0;
  RT fm[2] = {RT(0), RT(0)}, fe = RT(0);
  if (DIR == 0) {
    if (shear) {
      const RT tau = div_rn(RT(4.0 / 3.0) * dx[0], divisor(re_avg[0]));
      fm[0] = fm[0] - tau;
      fe = fe - vs[0] * tau;
    }
    if (bulk) {
      const RT tau = div_rn(dx[0], divisor(re_avg[1]));
      fm[0] = fm[0] - tau;
      fe = fe - vs[0] * tau;
    }
    if constexpr (ND > 1) {
      if (shear) {
        const RT t0 = -div_rn(RT(2.0 / 3.0) * dy[1], divisor(re_avg[0]));
        const RT t1 = div_rn(dy[0] + dx[1], divisor(re_avg[0]));
        fm[0] = fm[0] - t0;
        fe = fe - vs[0] * t0;
        fm[1] = fm[1] - t1;
        fe = fe - vs[1] * t1;
      }
      if (bulk) {
        const RT tau = div_rn(dy[1], divisor(re_avg[1]));
        fm[0] = fm[0] - tau;
        fe = fe - vs[0] * tau;
      }
    }
  } else if constexpr (ND > 1) {
    if (shear) {
      const RT t0 = div_rn(dy[0] + dx[1], divisor(re_avg[0]));
      const RT t1 = div_rn(RT(4) * dy[1] - RT(2) * dx[0], divisor(RT(3) * re_avg[0]));
      fm[0] = fm[0] - t0;
      fe = fe - vs[0] * t0;
      fm[1] = fm[1] - t1;
      fe = fe - vs[1] * t1;
    }
    if (bulk) {
      const RT tau = div_rn(dx[0] + dy[1], divisor(re_avg[1]));
      fm[1] = fm[1] - tau;
      fe = fe - vs[1] * tau;
    }
  }
  out[0] = fm[0];
  out[1] = fm[1];
  out[2] = fe;
}

// RK stage combinations, m_time_steppers.fpp:163-348, in the reference's
// operation order.  base = q_cons_ts(1), in = the stage's input register.
enum RkKind : int {
  kRkEuler = 0,   // base + dt*rhs          (RK1; stage 1 of RK2/RK3)
  kRk2Final = 1,  // (base + in + dt*rhs)/2
  kRk3Mid = 2,    // (3*base + in + dt*rhs)/4
  kRk3Final = 3,  // (base + 2*in + 2*dt*rhs)/3
  kRhsOnly = 4,   // store rhs itself (s_compute_rhs)
};

// A stage kind as a type: the kernels' last phase is compiled once per kind
// and chosen once per block.
template <int K>
struct KindC {
  static constexpr int value = K;
};

// A run-time flag that is the same for a whole block, as a type (a phase is
// compiled for both values and chosen once per block).
template <bool B>
struct FlagC {
  static constexpr bool value = B;
};

__device__ __forceinline__ double rk_combine(int kind, double base, double in, double dt, double r) {
  switch (kind) {
    case kRkEuler: return base + dt * r;
    case kRk2Final: return (base + in + dt * r) / 2.0;
    case kRk3Mid: return (3.0 * base + in + dt * r) / 4.0;
    case kRk3Final: {
      // divisor(3.0), spelled out: significand 1.5, 2^64 / 1.5 rounded down, exponent 1024
      constexpr DivisorF64 kThree{3.0, 0x18000000000000ULL, 0xaaaaaaaaaaaaaaaaULL, 0x400u, true};
      return div_rn(base + 2.0 * in + 2.0 * dt * r, kThree);
    }
    default: return r;
  }
}

// The same combinations for the split-precision path, written as q^n plus
// the stage's increment: (q1 - q0 + dt r)/2 for RK2, (q1 - q0 + dt r)/4 and
// 2 (q2 - q0 + dt r)/3 for RK3.  The increment is small next to the state,
// so it is formed in FP32 from the FP32 right-hand side and the FP64
// difference of the registers, and the state accumulates in FP64: one or two
// FP64 operations per value instead of two or three.
__device__ __forceinline__ double rk_combine_split(int kind, double base, double in, float dt, float r) {
  switch (kind) {
    case kRkEuler: return base + f2d_bits(dt * r);
    case kRk2Final: return base + f2d_bits(0.5f * fmaf(dt, r, d2f_bits(in - base)));
    case kRk3Mid: return base + f2d_bits(0.25f * fmaf(dt, r, d2f_bits(in - base)));
    case kRk3Final: return base + f2d_bits((2.0f / 3.0f) * fmaf(dt, r, d2f_bits(in - base)));
    default: return f2d_bits(r);
  }
}

}  // namespace mfc
