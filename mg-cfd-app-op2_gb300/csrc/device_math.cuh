// Device arithmetic of the MG-CFD hot path, shared by the per-loop entry
// points and the fused solver kernels.
//
// The reference evaluates everything per edge (flux.h:41-208): both end
// nodes' velocities (3 divisions each), speeds and speeds of sound (2 square
// roots each) and the full 4x3 flux tensors, then writes fluxes_b with a
// separately computed factor_b.  On GB300, FP64 issue (about 1.2 TFLOP/s,
// with one division or square root costing about ten FMAs) rather than HBM
// bounds that form, so the arithmetic here is the same algebra arranged to
// issue fewer FP64 instructions:
//
//   * per node, once per RK stage: r = 1/rho, u = m*r, p, s = |u| + c
//     (NodePrim); the edge reads them instead of recomputing them;
//   * per edge: the tensor contractions collapse to m.w, (m.w)/rho and
//     p*w (u_i m_j w_j = m_i (u.w) since m = rho*u), so
//       F_rho = m.w,  F_m = m (u.w) + p w,  F_E = (rhoE + p)(u.w);
//   * factor_a == factor_b up to association order, so the edge flux is
//     computed once and added to node a and subtracted from node b (the
//     negation is a sign-bit flip on the integer pipe);
//   * the dissipation fac * (x_a - x_b) joins the central terms' per-end
//     coefficients: x_a * (u_a.h + fac) + x_b * (u_b.h - fac), two FMAs per
//     variable instead of a subtraction, a multiplication and two FMAs;
//   * |w| and -|w|*smoothing*0.5 are constant after setup and precomputed,
//     and the weight is kept as h = -w/2 so the central term needs no
//     multiplication by -1/2 (exact: a power-of-two scaling).
//
// Every operation is an FP64 operation; all are IEEE-rounded except the two
// square roots of node_prim (x * rsqrt(x), within about two ulp).  Results
// differ from the reference only by rounding (relative 1e-16 per operation),
// far inside the 1e-10 parity bar.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mgcfd {

constexpr double kGammaD = 1.4;
constexpr double kGammaM1 = 1.4 - 1.0;  // (double(GAMMA)-double(1.0)), inlined_funcs.h:103-106

struct NodePrim {
  double rho, mx, my, mz, rhoE;  // conserved variables
  double p;                      // pressure
  double s;                      // |u| + speed of sound
  double rinv;                   // 1 / rho
};

// sqrt(x) as x * rsqrt(x) for positive finite x: about 8 FMA-equivalents on
// GB300 instead of about 10 for the correctly rounded square root, accurate
// to about two ulp.  Zero, negative, infinite and NaN inputs (recognised from
// the bit pattern on the integer pipe) take the IEEE square root, so the
// special cases are exactly those of sqrt().
__device__ __forceinline__ double sqrt_fast(double x) {
  const long long b = __double_as_longlong(x);
  return (b > 0 && b < 0x7ff0000000000000ll) ? x * rsqrt(x) : sqrt(x);
}

// inlined_funcs.h:98-130 with one reciprocal instead of three divisions, and
// without forming the velocity: with m2 = |m|^2,
//   rho |u|^2 = m2 / rho,   |u| = sqrt(m2) / rho,
// so p = (gamma - 1)(rhoE - m2/(2 rho)) and |u| = sqrt(m2) * (1/rho) take
// five FP64 operations fewer than u = m/rho, |u|^2 = u.u (about 33 FMA
// equivalents per node instead of 35).
__device__ __forceinline__ NodePrim node_prim(double rho, double mx, double my, double mz, double rhoE) {
  NodePrim n;
  n.rho = rho; n.mx = mx; n.my = my; n.mz = mz; n.rhoE = rhoE;
  n.rinv = 1.0 / rho;
  const double m2 = fma(mz, mz, fma(my, my, mx * mx));
  n.p = kGammaM1 * fma(-0.5 * m2, n.rinv, rhoE);
  n.s = sqrt_fast(m2) * n.rinv + sqrt_fast(kGammaD * n.p * n.rinv);
  return n;
}

// flux.h:41-208 for one edge: returns the increment f of node a; node b
// receives -f.  h = -w/2 for the edge weight w, wfac = -|w| * smoothing_coefficient * 0.5.
// With fac = wfac (s_a + s_b) the dissipation factor, ga = u_a.h + fac and
// gb = u_b.h - fac:
//   f_rho = rho_a ga + rho_b gb                    (rho_a u_a.h = m_a.h)
//   f_m   = m_a ga + m_b gb + (p_a + p_b) h
//   f_E   = E_a ga + E_b gb + p_a u_a.h + p_b u_b.h
// 27 FP64 operations, each written as the FMA or operation it issues, so no
// kernel that inlines this can contract it differently.
__device__ __forceinline__ void edge_flux(const NodePrim& a, const NodePrim& b, double hx, double hy, double hz,
                                          double wfac, double f[5]) {
  const double mha = fma(a.mz, hz, fma(a.my, hy, a.mx * hx));  // -(m_a . w)/2
  const double mhb = fma(b.mz, hz, fma(b.my, hy, b.mx * hx));
  const double uha = mha * a.rinv, uhb = mhb * b.rinv;          // -(u . w)/2
  const double sab = a.s + b.s;
  const double ga = fma(wfac, sab, uha), gb = fma(-wfac, sab, uhb);
  const double pp = a.p + b.p;
  f[0] = fma(a.rho, ga, b.rho * gb);
  f[1] = fma(a.mx, ga, fma(b.mx, gb, pp * hx));
  f[2] = fma(a.my, ga, fma(b.my, gb, pp * hy));
  f[3] = fma(a.mz, ga, fma(b.mz, gb, pp * hz));
  f[4] = fma(a.rhoE, ga, fma(b.rhoE, gb, fma(a.p, uha, b.p * uhb)));
}

// -x by flipping the sign bit of the high word with an integer instruction.
// Written as inline PTX so the compiler cannot turn it back into a
// floating-point negation, which would issue on the FP64 pipe.
__device__ __forceinline__ double negate(double x) {
  int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  asm("xor.b32 %0, %0, 0x80000000;" : "+r"(hi));
  return __hiloint2double(hi, lo);
}

// flux_wall.elem_func:49-76 (far field, groups 3..7) for one boundary entry:
// increment 0.5 * w.(F_ff + F_b); ffw[k] = w . F_ff row k (precomputable).
__device__ __forceinline__ void farfield_flux(const NodePrim& b, double wx, double wy, double wz,
                                              const double ffw[5], double f[5]) {
  const double mw = b.mx * wx + b.my * wy + b.mz * wz;
  const double uw = mw * b.rinv;
  f[0] = 0.5 * (ffw[0] + mw);
  f[1] = 0.5 * (ffw[1] + (b.mx * uw + b.p * wx));
  f[2] = 0.5 * (ffw[2] + (b.my * uw + b.p * wy));
  f[3] = 0.5 * (ffw[3] + (b.mz * uw + b.p * wz));
  f[4] = 0.5 * (ffw[4] + (b.rhoE + b.p) * uw);
}

// IEEE 754 binary32 <-> binary64 conversions on the integer pipe.
//
// On GB300 a cvt between float and double issues on the FP64 pipe at about
// 1.6 FMA-equivalents each, which makes the mixed-precision path's format
// changes cost as much as its FP64 arithmetic.  These build the result's bit
// pattern from the operand's fields with integer operations instead
// (IEEE 754-2008 section 3.4 encodings; binary64 exponent = binary32
// exponent + 896), and give the same bits as the hardware conversion:
//   f2d_bits: exact widening; zeros, subnormals (renormalised with a leading
//             zero count), infinities and NaNs (payload kept, quiet bit kept)
//             included;
//   d2f_bits: narrowing with round-to-nearest-even on the 29 dropped bits;
//             overflow rounds to infinity, NaNs keep the top payload bits and
//             become quiet; results in the binary32 subnormal range are
//             rounded with the same rule from the full 53-bit significand.
// The 64-bit register is packed and unpacked with PTX moves, which the
// compiler cannot fold back into a floating-point conversion.
__device__ __forceinline__ double pack_words(uint32_t hi, uint32_t lo) {
  double d;
  asm("mov.b64 %0, {%1, %2};" : "=d"(d) : "r"(lo), "r"(hi));
  return d;
}

__device__ __forceinline__ void unpack_words(double d, uint32_t& hi, uint32_t& lo) {
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(d));
}

// Zero, subnormal, infinity and NaN inputs: a separate, rarely taken call, so
// the common path issues only its own integer instructions.  A subnormal is
// first scaled by 2^24 in FP32 (exact) and its exponent corrected after.
static __device__ __noinline__ double f2d_bits_special(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t sign = u & 0x80000000u;
  const uint32_t a = u & 0x7fffffffu;
  if (a == 0u) return pack_words(sign, 0u);
  if (a >= 0x7f800000u) return pack_words(sign | 0x7ff00000u | ((a & 0x7fffffu) >> 3), u << 29);
  const uint32_t g = __float_as_uint(__fmul_rn(__uint_as_float(a), 16777216.0f));  // normal now
  return pack_words(sign | (((g >> 3) + (896u << 20)) - (24u << 20)), g << 29);
}

__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t a = u & 0x7fffffffu;
  if (a - 0x00800000u >= 0x7f000000u) return f2d_bits_special(f);  // not a normal number
  return pack_words((u & 0x80000000u) | ((a >> 3) + (896u << 20)), u << 29);
}

__device__ __forceinline__ float d2f_bits(double d) {
  uint32_t hi, lo;
  unpack_words(d, hi, lo);
  const uint32_t sign = hi & 0x80000000u;
  const int de = (int)((hi >> 20) & 0x7ffu);
  const uint32_t mhi = hi & 0xfffffu;    // top 20 of the 52 significand bits
  uint32_t r;
  if (de > 896 && de < 1151) {           // binary32 normal range before rounding
    const uint32_t rest = lo & 0x1fffffffu;
    r = ((uint32_t)(de - 896) << 23) | (mhi << 3) | (lo >> 29);
    r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;  // carries into the exponent
  } else if (de == 2047) {               // infinity or NaN
    r = 0x7f800000u | ((mhi | lo) ? (0x400000u | (mhi << 3) | (lo >> 29)) : 0u);
  } else if (de >= 1151) {               // beyond binary32: infinity
    r = 0x7f800000u;
  } else {                               // subnormal or zero in binary32
    const int k = 926 - de;              // value / 2^-149 = full >> k, k >= 30
    const unsigned long long full = ((unsigned long long)(de ? (mhi | 0x100000u) : mhi) << 32) | lo;
    if (k >= 64) {
      r = 0u;
    } else {
      const unsigned long long q = full >> k, rem = full & ((1ull << k) - 1ull), half = 1ull << (k - 1);
      r = (uint32_t)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u);
    }
  }
  return __uint_as_float(sign | r);
}

// Order-preserving map from double to uint64 (for atomicMin on doubles).
__device__ __forceinline__ unsigned long long dkey(double v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
  if (k == ~0ull) return 1.7976931348623157e308;  // nothing reduced yet: DBL_MAX
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

// hi + lo += x with Knuth's error-free TwoSum (TAOCP vol. 2, 4.2.2,
// theorem B): s = hi + x exactly equals s + e, and e joins lo.  Plain FP32
// adds (no contraction or reassociation applies to adds).
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  const float e = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += e;
}

// Order-preserving map from float to uint32 and back.
__device__ __forceinline__ unsigned int fkey(float v) {
  const unsigned int u = __float_as_uint(v);
  return (u >> 31) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(unsigned int k) {
  return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}

// Key of a dt value for the min_dt reduction, or ~0 when the value takes no
// part: get_min_dt_kernel (time_stepping_kernels.h:34-41) keeps its DBL_MAX
// start unless dt < it, so NaN, +inf and DBL_MAX itself never win.  Integer
// operations only.
__device__ __forceinline__ unsigned long long dt_candidate_key(double dt) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(dt);
  const unsigned long long k = dkey(dt);
  const bool nan = (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
  return (!nan && k < 0xffefffffffffffffull) ? k : ~0ull;  // 0xffef.. = dkey(DBL_MAX)
}

// NaN or infinity, from the exponent field (count_bad_vals, validation.h:102-115).
__device__ __forceinline__ bool not_finite(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

__device__ __forceinline__ double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w < v) ? w : v;
  }
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sum_int(int v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace mgcfd
