// Device forms of the reference's upwind schemes.  Expressions keep the
// reference's association order; the translation unit that instantiates the
// FP64 versions is compiled with --fmad=false so that they round exactly as the
// reference's FP64 CPU code (ADVECTION_METHOD_2D.h).
#pragma once

#include <cuda_runtime.h>

#include "gb2d_internal.cuh"

namespace gb2d {

// IEEE comparisons with zero.  FP64: on the integer pipes (an FP64 compare takes
// one of the part's few FP64 issue slots), exact for every input, NaN and
// infinities included.  FP32: the native compare.
constexpr long long kAbsBits = 0x7fffffffffffffffLL, kInfBits = 0x7ff0000000000000LL;
__device__ __forceinline__ bool gtz(double x) {  // x > 0
  const long long b = __double_as_longlong(x);
  return b > 0 && b <= kInfBits;
}
__device__ __forceinline__ bool gez(double x) {  // x >= 0
  const long long b = __double_as_longlong(x);
  return (b >= 0 && b <= kInfBits) || b == (long long)0x8000000000000000ull;
}
__device__ __forceinline__ bool lez(double x) {  // x <= 0
  const long long b = __double_as_longlong(x);
  return b == 0 || (b < 0 && (b & kAbsBits) <= kInfBits);
}
__device__ __forceinline__ bool ltz(double x) {  // x < 0
  const long long b = __double_as_longlong(x), m = b & kAbsBits;
  return b < 0 && m != 0 && m <= kInfBits;
}
// |a| <= |b| (false when either is NaN), on the integer pipes.
__device__ __forceinline__ bool abs_le(double a, double b) {
  const long long ma = __double_as_longlong(a) & kAbsBits, mb = __double_as_longlong(b) & kAbsBits;
  return ma <= mb && mb <= kInfBits;
}
// x < -e and x > e for a finite e > 0, on the integer pipes (false for NaN).
__device__ __forceinline__ bool lt_neg(double x, double e) {
  const long long b = __double_as_longlong(x), m = b & kAbsBits;
  return b < 0 && m > __double_as_longlong(e) && m <= kInfBits;
}
__device__ __forceinline__ bool gt_pos(double x, double e) {
  const long long b = __double_as_longlong(x);
  return b > __double_as_longlong(e) && b <= kInfBits;
}

// Smeared Heaviside inside its band |phi| <= eps (HeavisideFunction,
// PROJECTION_2D.h:1441-1461 and VISCOSITY_2D.h:688-708), with the reference's
// PI = 3.141592 (MACROS.h:5); oe = 1/eps taken on the host.
__device__ __forceinline__ double heaviside_band(double phi, double oe) {
  const double PI_REF = 3.141592, opi = 1.0 / PI_REF;
  return 0.5 + phi * oe * 0.5 + 0.5 * opi * sin(PI_REF * phi * oe);
}
__device__ __forceinline__ double heaviside(double phi, double eps, double oe) {
  if (lt_neg(phi, eps)) return 0;
  if (gt_pos(phi, eps)) return 1;
  return heaviside_band(phi, oe);
}

// Maximum of non-negative doubles by their bit patterns (which order as
// integers): a warp's maximum, then one atomicMax into *out.
__device__ __forceinline__ void block_max_bits(unsigned long long b, unsigned long long* out) {
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, b, o);
    b = w > b ? w : b;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, b);
}
// max(|x|, m) as the reference's `if (m <= |x|) m = |x|`: NaN never replaces m.
__device__ __forceinline__ unsigned long long abs_max_bits(double x, unsigned long long m) {
  const unsigned long long ab = (unsigned long long)(__double_as_longlong(x) & kAbsBits);
  return (ab > m && ab <= (unsigned long long)kInfBits) ? ab : m;
}

__device__ __forceinline__ bool gtz(float x) { return x > 0.0f; }
__device__ __forceinline__ bool gez(float x) { return x >= 0.0f; }
__device__ __forceinline__ bool lez(float x) { return x <= 0.0f; }
__device__ __forceinline__ bool ltz(float x) { return x < 0.0f; }

// a / 3 and a / 6, correctly rounded (IEEE binary64, round to nearest), in three
// FP64 operations instead of a division: with z = RN(1/d), q = RN(a z) lies within
// two ulps of a/d; the residual r = a - d q is then exactly representable and the
// FMA forms it exactly; RN(q + r z) has an error below 1e-15 ulp against a/d
// (the FMA correction step of P. Markstein, IBM J. Res. Dev. 34(1), 1990).  Since
// a is a multiple of 2 (d = 3) or 4 (d = 6) ulps of the quotient's binade, a/d
// sits at 0, 1/3 or 2/3 of an ulp from a representable number, never within 1/6
// ulp of a rounding midpoint, so that RN is the correctly rounded quotient.
// Magnitudes that could leave the normal range, zeros, infinities and NaN take
// the division.
template <int D>
__device__ __forceinline__ double div_by(double a) {
  static_assert(D == 3 || D == 6, "exact for 3 and 6");
  constexpr double z = D == 3 ? 0.33333333333333331483 : 0.16666666666666665741;  // RN(1/D)
  const int e = (int)((__double_as_longlong(a) >> 52) & 0x7ff);
  if (e < 64 || e > 1984) return a / (double)D;
  const double q = __dmul_rn(a, z);
  const double r = __fma_rn(-q, (double)D, a);
  return __fma_rn(r, z, q);
}

// Divisions in the type of the expression.  The exact FP64 path keeps IEEE
// quotients (div_by for the constants 3 and 6).  The FP32 flux path is an
// approximation of the scheme anyway: constants become reciprocal multiplies and
// the weights use the fast division (about 2 ulp).
__device__ __forceinline__ double cdiv3(double a) { return div_by<3>(a); }
__device__ __forceinline__ double cdiv6(double a) { return div_by<6>(a); }
__device__ __forceinline__ float cdiv3(float a) { return a * (1.0f / 3.0f); }
__device__ __forceinline__ float cdiv6(float a) { return a * (1.0f / 6.0f); }
__device__ __forceinline__ double vdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float vdiv(float a, float b) { return __fdividef(a, b); }

// WENO5 one-sided derivative from five first differences (ADVECTION_METHOD_2D.h:545-619).
template <typename R>
__device__ __forceinline__ R weno5_side(R a1, R a2, R a3, R a4, R a5, R eps) {
  const R c13 = R(13.0 / 12.0);
  const R q = R(0.25);
  R A1 = a1 - R(2) * a2 + a3, B1 = a1 - R(4) * a2 + R(3) * a3;
  R A2 = a2 - R(2) * a3 + a4, B2 = a2 - a4;
  R A3 = a3 - R(2) * a4 + a5, B3 = R(3) * a3 - R(4) * a4 + a5;
  R s1 = c13 * A1 * A1 + q * B1 * B1;
  R s2 = c13 * A2 * A2 + q * B2 * B2;
  R s3 = c13 * A3 * A3 + q * B3 * B3;
  R al1 = vdiv(R(1.0 / 10.0), (eps + s1) * (eps + s1));
  R al2 = vdiv(R(6.0 / 10.0), (eps + s2) * (eps + s2));
  R al3 = vdiv(R(3.0 / 10.0), (eps + s3) * (eps + s3));
  R sum = al1 + al2 + al3;
  R w1 = vdiv(al1, sum), w2 = vdiv(al2, sum), w3 = vdiv(al3, sum);
  const R cm16 = R((-1.0) / 6.0);
  return w1 * (cdiv3(a1) - cdiv6(a2 * R(7)) + cdiv6(a3 * R(11))) + w2 * (a2 * cm16 + cdiv6(a3 * R(5)) + cdiv3(a4)) +
         w3 * (cdiv3(a3) + cdiv6(a4 * R(5)) - cdiv6(a5));
}

// Exact FP64 pair: q[0..6] are values at offsets -3..+3 (ADVECTION_METHOD_2D.h:521-543).
__device__ __forceinline__ void weno5_pair(const double q[7], double o, double eps, double& dm, double& dp) {
  double d[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = o * (q[k + 1] - q[k]);
  dm = weno5_side<double>(d[0], d[1], d[2], d[3], d[4], eps);
  dp = weno5_side<double>(d[5], d[4], d[3], d[2], d[1], eps);
}

// Mixed pair: differences of the FP64 state formed in FP64, everything after in
// FP32 (the FP64 -> FP32 moves by truncation on the integer pipes).
__device__ __forceinline__ void weno5_pair_f32(const double q[7], float o, float eps, float& dm, float& dp) {
  float d[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = narrow(q[k + 1] - q[k]) * o;
  dm = weno5_side<float>(d[0], d[1], d[2], d[3], d[4], eps);
  dp = weno5_side<float>(d[5], d[4], d[3], d[2], d[1], eps);
}

// Godunov selection of WENO5thReinitialization (ADVECTION_METHOD_2D.h:1505-1655).
// Returns false where the reference leaves phi unchanged (tie sss == 0 or NaN);
// otherwise h = |grad phi| - 1 over the selected one-sided derivatives.
template <typename R>
__device__ __forceinline__ bool godunov_h(R s, R mx, R px, R my, R py, R& h) {
  R smx = s * mx, spx = s * px, smy = s * my, spy = s * py;
  int xs, ys;
  if (gez(spx) && gez(smx))
    xs = 0;
  else if (lez(spx) && lez(smx))
    xs = 1;
  else if (gtz(spx) && ltz(smx))
    xs = 2;
  else if (ltz(spx) && gtz(smx)) {
    R sss = s * (fabs(px) - fabs(mx)) / (px - mx);
    if (gtz(sss))
      xs = 0;
    else if (ltz(sss))
      xs = 1;
    else
      return false;
  } else
    return false;
  if (gez(spy) && gez(smy))
    ys = 0;
  else if (lez(spy) && lez(smy))
    ys = 1;
  else if (gtz(spy) && ltz(smy))
    ys = 2;
  else if (ltz(spy) && gtz(smy)) {
    R ss = s * (fabs(py) - fabs(my)) / (py - my);
    ys = gtz(ss) ? 0 : 1;
  } else
    return false;
  R gx = xs == 0 ? mx : px, gy = ys == 0 ? my : py;
  if (xs != 2 && ys != 2)
    h = sqrt(gx * gx + gy * gy) - R(1);
  else if (xs != 2)
    h = sqrt(gx * gx) - R(1);
  else if (ys != 2)
    h = sqrt(gy * gy) - R(1);
  else
    h = R(-1);
  return true;
}

// ENO3 one-sided derivatives by divided-difference selection (ADVECTION_METHOD_2D.h:2054-2111),
// from the six first divided differences d[0..5] (offsets -3..+2).
__device__ __forceinline__ bool mag_le(double a, double b) { return abs_le(a, b); }
__device__ __forceinline__ bool mag_le(float a, float b) { return fabsf(a) <= fabsf(b); }
template <typename R>
__device__ __forceinline__ void eno3_select(const R d[6], R o2, R o3, R h, R& dm, R& dp) {
  const R d1n1 = d[2], d10 = d[3];
  R d2n2 = o2 * (d[1] - d[0]), d2n1 = o2 * (d[2] - d[1]), d20 = o2 * (d[3] - d[2]);
  R d2p1 = o2 * (d[4] - d[3]), d2p2 = o2 * (d[5] - d[4]);
  R d3n2 = o3 * (d2n1 - d2n2), d3n1 = o3 * (d20 - d2n1), d30 = o3 * (d2p1 - d20), d3p1 = o3 * (d2p2 - d2p1);
  if (mag_le(d2n1, d20)) {
    if (mag_le(d3n2, d3n1))
      dm = d1n1 + d2n1 * h + R(2) * d3n2 * h * h;
    else
      dm = d1n1 + d2n1 * h + R(2) * d3n1 * h * h;
  } else {
    if (mag_le(d3n1, d30))
      dm = d1n1 + d20 * h - d3n1 * h * h;
    else
      dm = d1n1 + d20 * h - d30 * h * h;
  }
  if (mag_le(d20, d2p1)) {
    if (mag_le(d3n1, d30))
      dp = d10 - d20 * h - d3n1 * h * h;
    else
      dp = d10 - d20 * h - d30 * h * h;
  } else {
    if (mag_le(d30, d3p1))
      dp = d10 - d2p1 * h + R(2) * d30 * h * h;
    else
      dp = d10 - d2p1 * h + R(2) * d3p1 * h * h;
  }
}

// Exact FP64 pair: q[0..6] are values at offsets -3..+3.
__device__ __forceinline__ void eno3_pair(const double q[7], double o, double o2, double o3, double h, double& dm, double& dp) {
  double d[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = o * (q[k + 1] - q[k]);
  eno3_select<double>(d, o2, o3, h, dm, dp);
}

// Mixed pair: differences of the FP64 state formed in FP64, the divided
// differences and the selection in FP32.
__device__ __forceinline__ void eno3_pair_f32(const double q[7], float o, float o2, float o3, float h, float& dm, float& dp) {
  float d[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) d[k] = narrow(q[k + 1] - q[k]) * o;
  eno3_select<float>(d, o2, o3, h, dm, dp);
}

}  // namespace gb2d
