// Double-word ("float-float") arithmetic for the DW precision form.
//
// GB300 issues about two FP64 operations per clock per SM against 128 FP32
// or integer ones, so the FP64 edge flux (27 FP64 operations per edge) is
// bound by FP64 issue at about a fifth of HBM bandwidth.  The DW form keeps
// the state, the node sums, the time step and the norms in FP64. It holds
// the edge flux's inputs -- the node primitives and the edge weights -- as
// unevaluated pairs of binary32 numbers x = h + l, and evaluates the flux on
// the FP32 pipes with error-free transformations:
//
//   * TwoSum (Knuth, TAOCP vol. 2, 4.2.2, theorem B): s + e == a + b exactly;
//   * Fast2Sum (Dekker 1971, "A floating-point technique for extending the
//     available precision"): the same in three operations when the exponent
//     of a is at least that of b;
//   * TwoProd with a fused multiply-add: p + e == a * b exactly;
//   * dot products accumulated as in Dot2 (Ogita, Rump and Oishi, "Accurate
//     sum and dot product", SIAM J. Sci. Comput. 26(6), 2005): the rounded
//     high parts of the products are summed through TwoSum, and every error
//     term and the cross products h*l' + l*h' collect in one FP32 word.
//
// A pair carries 48 significand bits; an operation's result is within about
// n * 2^-47 of the exact value relative to the sum of its terms' magnitudes
// (n the number of terms), where an FP64 operation is within 2^-53 of it.
// The same absolute-error behaviour as FP64 arithmetic, with a constant about
// 64 times larger: the final flow state stays well inside the 1e-10 relative
// bar of the FP64 path.  The exponent range is binary32's: values below about
// 2^-100 in magnitude keep only their high word's precision (their low word
// would be subnormal), and values above 2^127 are not representable.
//
// Every FP32 operation is written as an IEEE intrinsic (__fadd_rn, __fmul_rn,
// __fmaf_rn), which the compiler neither contracts nor reassociates: the
// error-free transformations depend on each rounding happening as written.
#pragma once

#include "device_math.cuh"

namespace mgcfd {

struct dwf {
  float h, l;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// A sum of DW products in progress: s holds the TwoSum chain of the products'
// high parts, c everything else.
struct dwacc {
  float s, c;
};

// x * y for DW x and y, as the start of a sum.  The dropped x.l * y.l is
// below 2^-48 of |x y|.
__device__ __forceinline__ dwacc acc_prod(dwf x, dwf y) {
  float p, e;
  two_prod(x.h, y.h, p, e);
  e = __fmaf_rn(x.h, y.l, e);
  e = __fmaf_rn(x.l, y.h, e);
  return dwacc{p, e};
}

// acc += x * y.
__device__ __forceinline__ void acc_add_prod(dwacc& a, dwf x, dwf y) {
  float p, e, s, q;
  two_prod(x.h, y.h, p, e);
  two_sum(a.s, p, s, q);
  e = __fmaf_rn(x.h, y.l, e);
  e = __fmaf_rn(x.l, y.h, e);
  a.s = s;
  a.c = __fadd_rn(a.c, __fadd_rn(q, e));
}

// acc += x.
__device__ __forceinline__ void acc_add(dwacc& a, dwf x) {
  float s, q;
  two_sum(a.s, x.h, s, q);
  a.s = s;
  a.c = __fadd_rn(a.c, __fadd_rn(q, x.l));
}

// The accumulated value as a normalised pair (|l| at most half an ulp of h
// when |c| <= |s|; under cancellation, where c may exceed s, the pair is
// still within 2^-24 |c| of s + c, and |c| is itself of the order of the
// terms' magnitudes times 2^-23).
__device__ __forceinline__ dwf acc_dw(dwacc a) {
  dwf r;
  fast_two_sum(a.s, a.c, r.h, r.l);
  return r;
}

__device__ __forceinline__ dwf dw_mul(dwf x, dwf y) { return acc_dw(acc_prod(x, y)); }

__device__ __forceinline__ dwf dw_add(dwf x, dwf y) {
  dwacc a{x.h, x.l};
  acc_add(a, y);
  return acc_dw(a);
}

__device__ __forceinline__ dwf dw_neg(dwf x) { return dwf{-x.h, -x.l}; }

// The accumulated value in binary64: both words widened on the integer pipe
// and added in FP64 (one FP64 operation; exact when the two words' bits fit
// in 53 bits, otherwise correctly rounded).
__device__ __forceinline__ double acc_to_double(dwacc a) { return f2d_bits(a.s) + f2d_bits(a.c); }

// d = h + l with h = d rounded to binary32 (d2f_bits) and l = d - h rounded
// to binary32, from the bit patterns.  For |d| in [2^-74, 2^127) the
// difference d - h, in units of d's last place, is the difference of the low
// 32-bit words of d and of h widened to binary64: it is at most 2^28 in
// magnitude, also when h rounded up to the next power of two (the bit
// pattern of 2^(e+1) is one step above that of the largest double below it),
// so the 32-bit difference is exact.  l is that count converted to binary32
// and scaled by 2^(e-52), a normal binary32 power of two in this range.  Other
// inputs (zeros, subnormals, tiny or huge values, infinities and NaNs) take
// one FP64 subtraction instead.
__device__ __forceinline__ dwf dw_split(double d) {
  uint32_t dh, dl;
  unpack_words(d, dh, dl);
  const float h = d2f_bits(d);
  const int de = (int)((dh >> 20) & 0x7ffu);
  if (de >= 949 && de < 1150) {
    const uint32_t hb = __float_as_uint(h);
    const int delta = (int)(dl - ((hb & 7u) << 29));
    const float scale = __uint_as_float((uint32_t)(de - 948) << 23);  // 2^(de - 1075)
    // d - h = +-delta ulps (the sign of d); a zero difference is +0 as in IEEE subtraction
    return dwf{h, __fmul_rn(__int2float_rn((dh >> 31) ? -delta : delta), scale)};
  }
  const uint32_t ha = __float_as_uint(h) & 0x7fffffffu;
  return dwf{h, ha >= 0x7f800000u ? 0.0f : d2f_bits(d - f2d_bits(h))};
}

// Pairs stored as one 64-bit word: h in the low half (the lower address), l
// in the high half.
__device__ __forceinline__ double dw_pack(dwf x) { return pack_words(__float_as_uint(x.l), __float_as_uint(x.h)); }

__device__ __forceinline__ dwf dw_unpack(double w) {
  uint32_t hi, lo;
  unpack_words(w, hi, lo);
  return dwf{__uint_as_float(lo), __uint_as_float(hi)};
}

// The node primitives of the edge flux as pairs (the NodePrim fields).
struct NodePrimDW {
  dwf rho, mx, my, mz, rhoE, p, s, rinv;
};

// One node's DW primitives as a 64-byte row of 8 pair words.
__device__ __forceinline__ NodePrimDW load_prim_dw(const double* rec2, int64_t i) {
  const double4_32a* r = reinterpret_cast<const double4_32a*>(rec2 + 8 * i);
  const double4_32a x = r[0], y = r[1];
  return NodePrimDW{dw_unpack(x.x), dw_unpack(x.y), dw_unpack(x.z), dw_unpack(x.w),
                    dw_unpack(y.x), dw_unpack(y.y), dw_unpack(y.z), dw_unpack(y.w)};
}

__device__ __forceinline__ void store_prim_dw(double* rec2, int64_t i, const NodePrimDW& q) {
  double4_32a* r = reinterpret_cast<double4_32a*>(rec2 + 8 * i);
  r[0] = make_double4_32a(dw_pack(q.rho), dw_pack(q.mx), dw_pack(q.my), dw_pack(q.mz));
  r[1] = make_double4_32a(dw_pack(q.rhoE), dw_pack(q.p), dw_pack(q.s), dw_pack(q.rinv));
}

// 1/x for a DW x of normal magnitude: the correctly rounded FP32 reciprocal
// r0 of x.h, then one Newton step r0 (1 + e) with e = 1 - x r0 formed by
// FMAs (e is about 2^-24, so its rounding and the dropped e^2 are about
// 2^-48 relative).  Zeros, infinities and NaNs give r0's own result.
__device__ __forceinline__ dwf dw_rcp(dwf x) {
  const float r0 = __frcp_rn(x.h);
  float e = __fmaf_rn(-x.h, r0, 1.0f);
  e = __fmaf_rn(-x.l, r0, e);
  dwf r;
  fast_two_sum(r0, __fmul_rn(r0, e), r.h, r.l);
  return (__float_as_uint(r0) & 0x7f800000u) == 0x7f800000u || r0 == 0.0f ? dwf{r0, 0.0f} : r;
}

// sqrt(x) for a DW x >= 0: the correctly rounded FP32 root s0 of x.h, then
// one Newton step s0 + (x - s0^2) / (2 s0), with x - s0^2 formed exactly by
// TwoProd (x.h - s0^2 is exact by Sterbenz's lemma) and the quotient, a
// correction of about 2^-24 s0, taken to FP32 accuracy.  x.h <= 0,
// infinities and NaNs give s0's own result (a negative x gives NaN, as the
// FP64 square root does).
__device__ __forceinline__ dwf dw_sqrt(dwf x) {
  const float s0 = __fsqrt_rn(x.h);
  if (!(x.h > 0.0f) || (__float_as_uint(x.h) & 0x7f800000u) == 0x7f800000u) return dwf{s0, 0.0f};
  float p, e;
  two_prod(s0, s0, p, e);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(x.h, p), e), x.l);
  dwf out;
  fast_two_sum(s0, __fmul_rn(0.5f, __fdividef(r, s0)), out.h, out.l);
  return out;
}

__device__ __forceinline__ dwf dw_scale(dwf x, float pow2) { return dwf{__fmul_rn(x.h, pow2), __fmul_rn(x.l, pow2)}; }

// The binary64 constants of node_prim as pairs.
constexpr float kGammaM1H = (float)kGammaM1;
constexpr float kGammaM1L = (float)(kGammaM1 - (double)kGammaM1H);
constexpr float kGammaDH = (float)kGammaD;
constexpr float kGammaDL = (float)(kGammaD - (double)kGammaDH);

// node_prim (device_math.cuh) in DW arithmetic from the binary64 state: the
// same formula, r = 1/rho, p = (gamma-1)(rhoE - |m|^2 r / 2), s = sqrt(|m|^2) r
// + sqrt(gamma p r), with the five conserved values split into pairs (on the
// integer pipe) and no FP64 instruction.  The conserved values are returned
// as pairs too, for the edge flux.
__device__ __forceinline__ NodePrimDW node_prim_dw(double rho, double mx, double my, double mz, double rhoE) {
  NodePrimDW n;
  n.rho = dw_split(rho); n.mx = dw_split(mx); n.my = dw_split(my); n.mz = dw_split(mz); n.rhoE = dw_split(rhoE);
  n.rinv = dw_rcp(n.rho);
  dwacc t = acc_prod(n.mx, n.mx);
  acc_add_prod(t, n.my, n.my);
  acc_add_prod(t, n.mz, n.mz);
  const dwf m2 = acc_dw(t);
  const dwf ke = dw_scale(dw_mul(m2, n.rinv), -0.5f);  // -|m|^2 / (2 rho)
  n.p = dw_mul(dwf{kGammaM1H, kGammaM1L}, dw_add(n.rhoE, ke));
  const dwf u = dw_mul(dw_sqrt(m2), n.rinv);
  const dwf c = dw_sqrt(dw_mul(dw_mul(dwf{kGammaDH, kGammaDL}, n.p), n.rinv));
  n.s = dw_add(u, c);
  return n;
}

__device__ __forceinline__ double dw_to_double(dwf x) { return f2d_bits(x.h) + f2d_bits(x.l); }

// edge_flux (device_math.cuh) in DW arithmetic: the same terms, with
// h = -w/2 and wfac = -|w| * smoothing * 0.5 as pairs; the five increments of
// node a (node b receives their negation) as accumulators.  About 265 FP32
// operations per edge and no FP64 instruction.
__device__ __forceinline__ void edge_flux_dw_acc(const NodePrimDW& a, const NodePrimDW& b, dwf hx, dwf hy, dwf hz,
                                                 dwf wfac, dwacc F[5]) {
  dwacc t = acc_prod(a.mx, hx);
  acc_add_prod(t, a.my, hy);
  acc_add_prod(t, a.mz, hz);
  const dwf mha = acc_dw(t);  // -(m_a . w)/2
  t = acc_prod(b.mx, hx);
  acc_add_prod(t, b.my, hy);
  acc_add_prod(t, b.mz, hz);
  const dwf mhb = acc_dw(t);
  const dwf uha = dw_mul(mha, a.rinv), uhb = dw_mul(mhb, b.rinv);  // -(u . w)/2
  const dwf fac = dw_mul(wfac, dw_add(a.s, b.s));
  const dwf ga = dw_add(uha, fac), gb = dw_add(uhb, dw_neg(fac));
  const dwf pp = dw_add(a.p, b.p);
  F[0] = acc_prod(a.rho, ga);
  acc_add_prod(F[0], b.rho, gb);
  F[1] = acc_prod(a.mx, ga);
  acc_add_prod(F[1], b.mx, gb);
  acc_add_prod(F[1], pp, hx);
  F[2] = acc_prod(a.my, ga);
  acc_add_prod(F[2], b.my, gb);
  acc_add_prod(F[2], pp, hy);
  F[3] = acc_prod(a.mz, ga);
  acc_add_prod(F[3], b.mz, gb);
  acc_add_prod(F[3], pp, hz);
  F[4] = acc_prod(a.rhoE, ga);
  acc_add_prod(F[4], b.rhoE, gb);
  acc_add_prod(F[4], a.p, uha);
  acc_add_prod(F[4], b.p, uhb);
}

// The same with the increments in binary64 (5 FP64 additions).
__device__ __forceinline__ void edge_flux_dw(const NodePrimDW& a, const NodePrimDW& b, dwf hx, dwf hy, dwf hz,
                                             dwf wfac, double f[5]) {
  dwacc F[5];
  edge_flux_dw_acc(a, b, hx, hy, hz, wfac, F);
#pragma unroll
  for (int k = 0; k < 5; k++) f[k] = acc_to_double(F[k]);
}

// The node-centric sum of edge_flux_dw over one node's edges (the fused DW
// stage), with the node ("me") as end a of every edge -- its b-side edges
// taken as f(b, a; -h) = -f(a, b; h).  In
//   f_rho = rho_a ga + rho_b gb,  f_m = m_a ga + m_b gb + (p_a + p_b) h,
//   f_E = E_a ga + E_b gb + p_a (u_a.h) + p_b (u_b.h),
// with ga = u_a.h + fac and gb = u_b.h - fac, the node's own terms factor out
// of the sum over its edges: sum(ga) = u_me.H + FAC and sum(p_a h) = p_me H,
// with H = sum(h) and FAC = sum(fac).  So each edge adds only the
// neighbour's terms and its h and fac to pair accumulators
// (node_flux_dw_edge), and the node's own terms are added once
// (node_flux_dw_finish): about 207 FP32 operations per edge instead of the
// 307 of edge_flux_dw_acc plus the pair sum, and 166 per node.  The same
// algebra; the roundings differ, within the pairs' 2^-47.
struct NodeFluxDW {
  dwacc S[5];             // the node's increments
  dwacc hx, hy, hz, fac;  // H and FAC
};

__device__ __forceinline__ void node_flux_dw_init(NodeFluxDW& A) {
#pragma unroll
  for (int k = 0; k < 5; k++) A.S[k] = dwacc{0.0f, 0.0f};
  A.hx = A.hy = A.hz = A.fac = dwacc{0.0f, 0.0f};
}

__device__ __forceinline__ void node_flux_dw_edge(NodeFluxDW& A, dwf s_me, const NodePrimDW& o, dwf hx, dwf hy,
                                                  dwf hz, dwf wfac) {
  const dwf fac = dw_mul(wfac, dw_add(s_me, o.s));
  dwacc t = acc_prod(o.mx, hx);
  acc_add_prod(t, o.my, hy);
  acc_add_prod(t, o.mz, hz);
  const dwf uhb = dw_mul(acc_dw(t), o.rinv);  // -(u_b . w)/2
  const dwf gb = dw_add(uhb, dw_neg(fac));
  acc_add_prod(A.S[0], o.rho, gb);
  acc_add_prod(A.S[1], o.mx, gb);
  acc_add_prod(A.S[1], o.p, hx);
  acc_add_prod(A.S[2], o.my, gb);
  acc_add_prod(A.S[2], o.p, hy);
  acc_add_prod(A.S[3], o.mz, gb);
  acc_add_prod(A.S[3], o.p, hz);
  acc_add_prod(A.S[4], o.rhoE, gb);
  acc_add_prod(A.S[4], o.p, uhb);
  acc_add(A.hx, hx);
  acc_add(A.hy, hy);
  acc_add(A.hz, hz);
  acc_add(A.fac, fac);
}

// The node's own terms, then the five sums in binary64.
__device__ __forceinline__ void node_flux_dw_finish(NodeFluxDW& A, const NodePrimDW& me, double F[5]) {
  const dwf hx = acc_dw(A.hx), hy = acc_dw(A.hy), hz = acc_dw(A.hz);
  dwacc t = acc_prod(me.mx, hx);
  acc_add_prod(t, me.my, hy);
  acc_add_prod(t, me.mz, hz);
  const dwf uh = dw_mul(acc_dw(t), me.rinv);  // u_me . H
  const dwf g = dw_add(uh, acc_dw(A.fac));    // sum of ga
  acc_add_prod(A.S[0], me.rho, g);
  acc_add_prod(A.S[1], me.mx, g);
  acc_add_prod(A.S[1], me.p, hx);
  acc_add_prod(A.S[2], me.my, g);
  acc_add_prod(A.S[2], me.p, hy);
  acc_add_prod(A.S[3], me.mz, g);
  acc_add_prod(A.S[3], me.p, hz);
  acc_add_prod(A.S[4], me.rhoE, g);
  acc_add_prod(A.S[4], me.p, uh);
#pragma unroll
  for (int k = 0; k < 5; k++) F[k] = acc_to_double(A.S[k]);
}

}  // namespace mgcfd
