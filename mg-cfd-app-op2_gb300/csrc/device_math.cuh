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
//   * |w| and -|w|*smoothing*0.5 are constant after setup and precomputed,
//     and the weight is kept as h = -w/2 so the central term needs no
//     multiplication by -1/2 (exact: a power-of-two scaling).
//
// Every operation is still an IEEE FP64 operation; results differ from the
// reference only by rounding (relative 1e-16 per operation), far inside the
// 1e-10 parity bar.
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

// inlined_funcs.h:98-130 with one reciprocal instead of three divisions.
__device__ __forceinline__ NodePrim node_prim(double rho, double mx, double my, double mz, double rhoE) {
  NodePrim n;
  n.rho = rho; n.mx = mx; n.my = my; n.mz = mz; n.rhoE = rhoE;
  n.rinv = 1.0 / rho;
  const double ux = mx * n.rinv, uy = my * n.rinv, uz = mz * n.rinv;
  const double q2 = ux * ux + uy * uy + uz * uz;
  n.p = kGammaM1 * (rhoE - 0.5 * rho * q2);
  n.s = sqrt(q2) + sqrt(kGammaD * n.p * n.rinv);
  return n;
}

// flux.h:41-208 for one edge: returns the increment f of node a; node b
// receives -f.  h = -w/2 for the edge weight w, wfac = -|w| * smoothing_coefficient * 0.5.
// About 35 FP64 operations.
__device__ __forceinline__ void edge_flux(const NodePrim& a, const NodePrim& b, double hx, double hy, double hz,
                                          double wfac, double f[5]) {
  const double mha = a.mx * hx + a.my * hy + a.mz * hz;  // -(m_a . w)/2
  const double mhb = b.mx * hx + b.my * hy + b.mz * hz;
  const double uha = mha * a.rinv, uhb = mhb * b.rinv;    // -(u . w)/2
  const double fac = wfac * (a.s + b.s);
  const double pp = a.p + b.p;
  f[0] = fac * (a.rho - b.rho) + (mha + mhb);
  f[1] = fac * (a.mx - b.mx) + (a.mx * uha + b.mx * uhb + pp * hx);
  f[2] = fac * (a.my - b.my) + (a.my * uha + b.my * uhb + pp * hy);
  f[3] = fac * (a.mz - b.mz) + (a.mz * uha + b.mz * uhb + pp * hz);
  f[4] = fac * (a.rhoE - b.rhoE) + ((a.rhoE + a.p) * uha + (b.rhoE + b.p) * uhb);
}

// -x by flipping the sign bit with an integer operation.
__device__ __forceinline__ double negate(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
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
