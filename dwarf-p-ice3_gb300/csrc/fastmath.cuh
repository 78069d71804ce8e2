// fastmath.cuh — FP64 exp, exp10 and log that spend as few FP64 instructions
// as the result's 53 bits need.
//
// GB300 issues FP64 at 1/64 of its FP32 rate (a measured 1.0 TFLOP/s FMA),
// and on it an FP64 compare, min/max or conversion costs as much as an FP64
// FMA, while integer and FP32 instructions are almost free beside them.  The
// microphysics kernels need a few dozen exp/log per grid point per sub-step,
// so these functions do in FP64 only the steps that need 53 bits and move
// the rest to the integer and FP32 pipes: range checks on the bit pattern,
// the integer part of the argument reduction in FP32, int -> double by bit
// construction, and the high-order polynomial terms (whose size is below
// 2^-28 of the result, so FP32's 2^-24 suffices) in FP32.
//
//   fexp   P. T. P. Tang, "Table-driven implementation of the exponential
//          function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989:
//          x = (256 m + j) ln2/256 + r, |r| <= ln2/512; e^x = 2^m 2^(j/256) e^r,
//          2^(j/256) tabulated as a double + float pair, e^r - 1 by its Taylor
//          series (r, r^2/2 in FP64; r^3/6 and beyond in FP32).  6 FP64 ops.
//   fexp10 the same with log10(2)/256 and r scaled by ln 10.  7 FP64 ops.
//   flog   P. T. P. Tang, "Table-driven implementation of the logarithm
//          function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990,
//          with the reduction made exact: x = 2^e z, z in [1, 2) split into
//          128 intervals by its leading 7 fraction bits, intervals above
//          sqrt(2) folded to [sqrt(1/2), 1) (e + 1); invc, a reciprocal of the
//          interval's centre rounded to 8 significant bits, makes
//          r = z*invc - 1 exact in one FMA (|r| < 2^-7); log x = e ln2 -
//          log(invc) + log1p(r), log1p by its Taylor series (to r^4 in FP64,
//          r^5 .. r^8 in FP32).  9 FP64 ops.
//   frcp   1/d: a correctly rounded FP32 reciprocal of d (truncated to FP32)
//          as the seed r0 (|eps| = |1 - d r0| < 2^-22), then one Newton-
//          Raphson step with the quadratic term of 1/(1-eps) = 1 + eps +
//          eps^2 + ..., r1 = r0 (1 + eps + eps^2), leaving eps^3 < 2^-66.
//          3 FP64 ops (an IEEE FP64 divide costs ~9 on GB300).  fdiv(a, b) =
//          a * frcp(b), within 2 ulp.  Outside 2^-125 < |d| < 2^125 (and for
//          zero, inf, NaN) it falls back to the IEEE division.
//   frsqrt 1/sqrt(d): y0 = the FP32 reciprocal of the FP32 square root of d
//          (truncated to FP32; |eps| = |1 - d y0^2| < 2^-21), then
//          y0 (1 + eps/2 + 3 eps^2/8), the series of (1 - eps)^(-1/2) to its
//          quadratic term (remainder 5 eps^3/16 < 2^-63).  5 FP64 ops, within
//          1 ulp; outside 2^-120 < d < 2^120 (and for zero, negative, inf,
//          NaN) 1 / sqrt(d).
//   fatan  reduction to [0, 1] by atan(x) = pi/2 - atan(1/x), then
//          atan(y) = atan(c) + atan(r), c = j/64 the nearest table point,
//          r = (y - c)/(1 + y c) (|r| <= 1/128), atan(r) by its Taylor series
//          (r^3 in FP64, r^5 .. r^9 in FP32); atan(c) and pi/2 - atan(c)
//          tabulated.  ~15 FP64 ops.
//
// Accuracy: within 2 ulp (tests compare the host build of this code with
// 200-bit mpmath values, and the device build with the host build bit for
// bit).  Every FP64 and FP32 operation is an explicit fma or a separately
// rounded add/multiply, so host and device builds agree exactly.  Special
// inputs (NaN, infinities, zero, negative, subnormal, overflow and underflow
// ranges) leave the fast path through one integer test and get the IEEE
// results of exp/log.
#pragma once

#include <stdint.h>
#include <string.h>
#if !defined(__CUDACC__)
#include <cmath>
#endif

#include "fastmath_tables.h"

#if defined(__CUDACC__)
#define FM_HD __host__ __device__ __forceinline__
// exp, exp10, log, the reciprocal and the rounded division are called from
// dozens of sites of the large point kernels: one out-of-line copy per
// kernel keeps those kernels' code in the instruction cache (rain_ice 172.5
// -> 171.5 ms and sedimentation 46.1 -> 44.7 ms per launch at 1024x1024x90
// for exp / log; rain_ice 162.4 -> 159.2 ms for the reciprocal, 160.7 ms
// for the division)
#define FM_NI static __host__ __device__ __noinline__
#else
#define FM_HD inline
#define FM_NI static inline
#endif

namespace fm {

struct ExpEntry { double hi; float lo; int pad; };
struct AtanEntry { double hi; float lo; int pad; };
struct LogEntry { double invc, nlog_hi; float nlog_lo; int fold; double pad; };

#if defined(__CUDA_ARCH__)
__device__ const ExpEntry kExpTable[256] = FM_EXP_TABLE_INIT;
__device__ const LogEntry kLogTable[128] = FM_LOG_TABLE_INIT;
__device__ const AtanEntry kAtanTable[65] = FM_ATAN_TABLE_INIT;
__device__ const AtanEntry kAtanCTable[65] = FM_ATANC_TABLE_INIT;
__device__ __forceinline__ void atan_entry(bool comp, int j, double &hi, float &lo)
{
  const double2 v = __ldg(reinterpret_cast<const double2 *>(comp ? kAtanCTable : kAtanTable) + j);
  hi = v.x;
  lo = __int_as_float((int)(uint32_t)__double_as_longlong(v.y));
}
__device__ __forceinline__ float rcpf_(float x) { return __frcp_rn(x); }
__device__ __forceinline__ float sqrtf_(float x) { return __fsqrt_rn(x); }
__device__ __forceinline__ void exp_entry(int j, double &hi, float &lo)
{
  const double2 v = __ldg(reinterpret_cast<const double2 *>(kExpTable) + j);
  hi = v.x;
  lo = __int_as_float((int)(uint32_t)__double_as_longlong(v.y));
}
__device__ __forceinline__ void log_entry(int i, double &invc, double &nlog_hi, float &nlog_lo, int &fold)
{
  const double2 *p = reinterpret_cast<const double2 *>(kLogTable) + 2 * i;
  const double2 a = __ldg(p);
  const float2 b = __ldg(reinterpret_cast<const float2 *>(p + 1));
  invc = a.x; nlog_hi = a.y; nlog_lo = b.x; fold = __float_as_int(b.y);
}
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fmaf_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float addf_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float mulf_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ int64_t bits_(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double from_bits_(int64_t b) { return __longlong_as_double(b); }
__device__ __forceinline__ int32_t fbits_(float x) { return __float_as_int(x); }
__device__ __forceinline__ float ffrom_bits_(int32_t b) { return __int_as_float(b); }
__device__ __forceinline__ int clz32_(uint32_t v) { return __clz((int)v); }
#else
static const ExpEntry kExpTable[256] = FM_EXP_TABLE_INIT;
static const LogEntry kLogTable[128] = FM_LOG_TABLE_INIT;
static const AtanEntry kAtanTable[65] = FM_ATAN_TABLE_INIT;
static const AtanEntry kAtanCTable[65] = FM_ATANC_TABLE_INIT;
inline void atan_entry(bool comp, int j, double &hi, float &lo)
{
  const AtanEntry &e = comp ? kAtanCTable[j] : kAtanTable[j];
  hi = e.hi; lo = e.lo;
}
inline float rcpf_(float x) { volatile float r = 1.0f / x; return r; }
inline float sqrtf_(float x) { volatile float r = std::sqrt(x); return r; }
inline void exp_entry(int j, double &hi, float &lo) { hi = kExpTable[j].hi; lo = kExpTable[j].lo; }
inline void log_entry(int i, double &invc, double &nlog_hi, float &nlog_lo, int &fold)
{
  invc = kLogTable[i].invc; nlog_hi = kLogTable[i].nlog_hi; nlog_lo = kLogTable[i].nlog_lo; fold = kLogTable[i].fold;
}
inline double fma_(double a, double b, double c) { return std::fma(a, b, c); }
inline double add_(double a, double b) { volatile double s = a + b; return s; }
inline double mul_(double a, double b) { volatile double s = a * b; return s; }
inline float fmaf_(float a, float b, float c) { return std::fmaf(a, b, c); }
inline float addf_(float a, float b) { volatile float s = a + b; return s; }
inline float mulf_(float a, float b) { volatile float s = a * b; return s; }
inline int64_t bits_(double x) { int64_t b; memcpy(&b, &x, 8); return b; }
inline double from_bits_(int64_t b) { double x; memcpy(&x, &b, 8); return x; }
inline int32_t fbits_(float x) { int32_t b; memcpy(&b, &x, 4); return b; }
inline float ffrom_bits_(int32_t b) { float x; memcpy(&x, &b, 4); return x; }
inline int clz32_(uint32_t v) { return v ? __builtin_clz(v) : 32; }
#endif

// double -> float by truncation of the significand, with integer operations
// only; magnitudes below 2^-126 become zero.  For the small high-order terms
// computed in FP32 the 2^-23 relative error is far below what they need.
FM_HD float to_f32(double x)
{
  const int64_t b = bits_(x);
  const int32_t e = (int32_t)((b >> 52) & 0x7ff) - 896;        // float biased exponent
  const int32_t s = (int32_t)((uint64_t)b >> 32) & (int32_t)0x80000000;
  if (e <= 0) return ffrom_bits_(s);
  return ffrom_bits_(s | (e << 23) | (int32_t)((b >> 29) & 0x7fffff));
}

// float -> double, exact, with integer operations only (float zero and
// subnormals give zero).
FM_HD double to_f64(float x)
{
  const int32_t b = fbits_(x);
  const int32_t e = (b >> 23) & 0xff;
  const int64_t s = (int64_t)((uint64_t)((uint32_t)b & 0x80000000u) << 32);
  if (e == 0) return from_bits_(s);
  return from_bits_(s | ((int64_t)(e + 896) << 52) | ((int64_t)(b & 0x7fffff) << 29));
}

// int -> double, exact (|k| < 2^31), with integer operations only.
FM_HD double i2d(int32_t k)
{
  if (k == 0) return 0.0;
  const int64_t s = k < 0 ? (int64_t)(1ULL << 63) : 0;
  const uint32_t a = k < 0 ? (uint32_t)(-(int64_t)k) : (uint32_t)k;
  const int n = 31 - clz32_(a);                                  // index of the leading bit
  const int64_t mant = ((int64_t)a << (52 - n)) & 0x000fffffffffffffLL;
  return from_bits_(s | ((int64_t)(1023 + n) << 52) | mant);
}

// Nearest integer of a float with |t| < 2^22 (shifter trick, FP32 add).
FM_HD int32_t rint_f32(float t)
{
  const float sh = 12582912.0f;                                  // 1.5 * 2^23
  return fbits_(addf_(t, sh)) - fbits_(sh);
}

// 2^(k/256) * e^r * (1 - corr) for |r| <= ~ln2/512 and |corr| < 2^-40.
FM_HD double exp_core(int32_t k, double r, float corr)
{
  const float rf = to_f32(r);
  // (e^r - 1 - r - r^2/2) / r^3 = 1/6 + r/24 + r^2/120 (+ r^3/720 < 2^-31 of r^3/6)
  float s = fmaf_(rf, 1.0f / 120.0f, 1.0f / 24.0f);
  s = fmaf_(rf, s, 1.0f / 6.0f);
  const double q = fma_(r, to_f64(s), 0.5);
  const double p = fma_(mul_(r, r), q, r);                      // e^r - 1
  double thi;
  float tlo;
  exp_entry(k & 255, thi, tlo);
  // lo' = T_lo - T_hi*corr (both terms < 2^-38: FP32 carries them to 2^-62)
  const float lo = fmaf_(-to_f32(thi), corr, tlo);
  const double y = add_(thi, fma_(thi, p, to_f64(lo)));           // in [0.997, 2)
  const int32_t m = k >> 8;
  if (m >= -1021 && m <= 1022) return from_bits_(bits_(y) + (int64_t)m * ((int64_t)1 << 52));
  // gradual underflow / overflow edges: scale in two steps
  const double y1 = from_bits_(bits_(y) + (int64_t)(m / 2) * ((int64_t)1 << 52));
  return mul_(y1, from_bits_((int64_t)(1023 + m - m / 2) << 52));
}

// e^x.
FM_NI double fexp(double x)
{
  const int64_t ax = bits_(x) & 0x7fffffffffffffffLL;
  if (ax > 0x40861f0000000000LL) {                               // |x| > 707.875, inf, NaN
    if (ax > 0x7ff0000000000000LL) return x;                     // NaN
    if (x > 709.782712893384) return from_bits_(0x7ff0000000000000LL);
    if (x < -745.1332191019412) return 0.0;
  }
  const int32_t k = rint_f32(mulf_(to_f32(x), FM_INV_L256_F));   // |k| < 2^18; off by one at most
  const double kd = i2d(k);
  const double r = fma_(-kd, FM_L256_HI, x);                     // one rounding, < 2^-62
  return exp_core(k, r, mulf_((float)k, FM_L256_LO_F));
}

// 10^x.
FM_NI double fexp10(double x)
{
  const int64_t ax = bits_(x) & 0x7fffffffffffffffLL;
  if (ax > 0x4073300000000000LL) {                               // |x| > 307, inf, NaN
    if (ax > 0x7ff0000000000000LL) return x;
    if (x > 308.2547155599167) return from_bits_(0x7ff0000000000000LL);
    if (x < -323.60766413161369) return 0.0;
  }
  const int32_t k = rint_f32(mulf_(to_f32(x), FM_INV_LG256_F));
  const double kd = i2d(k);
  const double r10 = fma_(-kd, FM_LG256_HI, x);                  // |r10| <= ~log10(2)/512
  return exp_core(k, mul_(r10, FM_LN10), mulf_(mulf_((float)k, FM_LG256_LO_F), FM_LN10_F));
}

// Natural logarithm.
FM_NI double flog(double x)
{
  int64_t b = bits_(x);
  int ebias = 0;
  if (b < 0x0010000000000000LL || b >= 0x7ff0000000000000LL) {   // <= 0, subnormal, inf, NaN
    if (x != x) return x;
    if (x < 0.0) return from_bits_(0x7ff8000000000000LL);
    if (x == 0.0) return from_bits_((int64_t)0xfff0000000000000ULL);
    if (b >= 0x7ff0000000000000LL) return x;                      // +inf
    x = mul_(x, 18014398509481984.0);                              // subnormal: * 2^54
    b = bits_(x);
    ebias = -54;
  }
  double invc, nlog_hi;
  float nlog_lo;
  int fold;
  log_entry((int)((b >> 45) & 127), invc, nlog_hi, nlog_lo, fold);
  const int32_t e = (int32_t)(b >> 52) - 1023 + ebias + fold;
  const double z = from_bits_((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  const double r = fma_(z, invc, -1.0);                          // exact
  const double hi = fma_(i2d(e), FM_LN2_HI, nlog_hi);            // e*LN2_HI exact
  const float lo = fmaf_((float)e, FM_LN2_LO_F, nlog_lo);        // < 2^-34: FP32 suffices
  // (log1p(r) - r) / r^2 = -1/2 + r/3 - r^2/4 + r^3 s,  s = 1/5 - r/6 + r^2/7 - r^3/8
  const float rf = to_f32(r);
  float s = fmaf_(rf, -1.0f / 8.0f, 1.0f / 7.0f);
  s = fmaf_(rf, s, -1.0f / 6.0f);
  s = fmaf_(rf, s, 1.0f / 5.0f);
  double q = fma_(r, to_f64(s), -0.25);
  q = fma_(r, q, 1.0 / 3.0);
  q = fma_(r, q, -0.5);
  const double tail = fma_(mul_(r, r), q, to_f64(lo));
  return add_(hi, add_(r, tail));
}

// The IEEE 1/d and 1/sqrt(d), out of line: the rare fallbacks of frcp and
// frsqrt, which are inlined at many sites.
FM_NI double rcp_ieee_(double d) { return 1.0 / d; }
FM_NI double rsqrt_ieee_(double d) { return 1.0 / sqrt(d); }

// 1/d (see the header): FP32 seed + one Newton-Raphson step with its
// quadratic term.
FM_NI double frcp(double d)
{
  const int64_t e = (bits_(d) >> 52) & 0x7ff;
  if (e < 1023 - 125 || e > 1023 + 125) return rcp_ieee_(d);     // zero, tiny, huge, inf, NaN
  const double r0 = to_f64(rcpf_(to_f32(d)));
  const double eps = fma_(-d, r0, 1.0);
  return fma_(r0, fma_(eps, eps, eps), r0);
}
FM_HD double fdiv(double a, double b) { return mul_(a, frcp(b)); }

// a / b rounded to nearest (the IEEE quotient) for 2^-400 <= |a|, |b| <=
// 2^400, from y = frcp(b): q0 = a y, then q1 = q0 + (a - b q0) y, checked
// with the exact remainder r = a - b q1 (one fma): q1 is the rounded quotient
// iff |r| < |b| ulp(q1) / 2 (a / b is never halfway between two doubles; q1
// a power of two, whose lower neighbour is closer, is not accepted).  Where
// the check fails or the operands are out of range, the IEEE division.  4
// FP64 operations per quotient besides the reciprocal; the check is integer
// work.  fdiv_rn2 shares the reciprocal between two numerators.
// the IEEE division, out of line (the rare fallback of the paths below)
FM_NI double div_ieee_(double a, double b) { return a / b; }
FM_HD bool div_rn_range_(double x)
{
  const int64_t e = (bits_(x) >> 52) & 0x7ff;
  return e >= 1023 - 400 && e <= 1023 + 400;
}
FM_HD double div_rn_with_(double a, double b, double y)
{
  const double q0 = mul_(a, y);
  const double q1 = fma_(fma_(-q0, b, a), y, q0);
  const double r = fma_(-q1, b, a);
  const int64_t bq = bits_(q1) & 0x7fffffffffffffffLL, bb = bits_(b) & 0x7fffffffffffffffLL;
  // |b| ulp(q1) / 2 = |b| 2^(E(q1) - 1023 - 53): add to b's exponent
  const int64_t eh = (bb >> 52) + (bq >> 52) - (1023 + 53);
  if (eh >= 1 && (bq & 0x000fffffffffffffLL) != 0 && (bits_(r) & 0x7fffffffffffffffLL) < bb + ((eh - (bb >> 52)) << 52))
    return q1;
  return div_ieee_(a, b);
}
FM_NI double fdiv_rn(double a, double b)
{
  if (!(div_rn_range_(a) && div_rn_range_(b))) return div_ieee_(a, b);
  return div_rn_with_(a, b, frcp(b));
}
FM_NI void fdiv_rn2(double a1, double a2, double b, double &q1, double &q2)
{
  if (!(div_rn_range_(a1) && div_rn_range_(a2) && div_rn_range_(b))) {
    q1 = div_ieee_(a1, b);
    q2 = div_ieee_(a2, b);
    return;
  }
  const double y = frcp(b);
  q1 = div_rn_with_(a1, b, y);
  q2 = div_rn_with_(a2, b, y);
}

// 1/sqrt(d) (see the header) for 2^-120 < d < 2^120; frsqrt_ok tells.
FM_HD bool frsqrt_ok(double d)
{
  const int64_t e = bits_(d) >> 52;                               // the sign bit makes e >= 2048
  return e >= 1023 - 120 && e <= 1023 + 120;
}
FM_HD double frsqrt(double d)
{
  if (!frsqrt_ok(d)) return rsqrt_ieee_(d);                       // zero, tiny, huge, negative, inf, NaN
  const double y0 = to_f64(rcpf_(sqrtf_(to_f32(d))));
  const double eps = fma_(-d, mul_(y0, y0), 1.0);                  // y0^2 exact (24-bit y0)
  return fma_(mul_(y0, eps), fma_(eps, 0.375, 0.5), y0);
}

// Arc tangent (see the header).
FM_HD double fatan(double x)
{
  const int64_t b = bits_(x), ab = b & 0x7fffffffffffffffLL;
  if (ab < 0x3e10000000000000LL) return x;                        // |x| < 2^-30: atan x = x (1 - x^2/3), +-0
  if (ab > 0x43b0000000000000LL) {                                // |x| > 2^60, inf, NaN
    if (ab > 0x7ff0000000000000LL) return x;
    return b < 0 ? -FM_PIO2 : FM_PIO2;
  }
  const bool comp = ab > 0x3ff0000000000000LL;                    // |x| > 1: pi/2 - atan(1/|x|)
  const double ax = from_bits_(ab);
  const double y = comp ? frcp(ax) : ax;
  const int32_t j = rint_f32(mulf_(to_f32(y), 64.0f));            // 0..64
  const double c = j == 0 ? 0.0 : from_bits_(bits_(i2d(j)) - ((int64_t)6 << 52));   // j/64, exact
  const double r = mul_(add_(y, -c), frcp(fma_(y, c, 1.0)));      // y - c exact (Sterbenz)
  const double r2 = mul_(r, r);
  const float r2f = to_f32(r2);
  // (atan r - r) / r^3 = -1/3 + r^2 (1/5 - r^2/7 + r^4/9)
  const float s = fmaf_(r2f, fmaf_(r2f, 1.0f / 9.0f, -1.0f / 7.0f), 1.0f / 5.0f);
  const double q = fma_(r2, to_f64(s), -1.0 / 3.0);
  const double at = fma_(mul_(r2, r), q, r);
  double hi;
  float lo;
  atan_entry(comp, j, hi, lo);
  const double res = comp ? add_(hi, add_(to_f64(lo), -at)) : add_(hi, add_(to_f64(lo), at));
  return b < 0 ? -res : res;
}

// x^a = e^(a log x) for x > 0 (relative error ~|a log x| ulp).
FM_HD double fpow(double x, double a) { return fexp(mul_(a, flog(x))); }
// x^a from a precomputed log x.
FM_HD double fpowl(double logx, double a) { return fexp(mul_(a, logx)); }

}  // namespace fm
