// ice3gb_device.cuh — device-side helpers shared by the ICE3 kernels.
//
// Layout: every 3-D field is [nk][nij] FP64 (ij fastest), 2-D fields [nij].
// The constants table (Ice3gbConstants, ~1.5 KB) is passed by value as a
// __grid_constant__ kernel parameter, so every lane reads it from the
// constant bank with no global-memory traffic.
#pragma once

#include <stdint.h>
#if defined(__CUDACC__)
#include <cuda_runtime.h>
#else
#include <cmath>
using std::exp; using std::log; using std::fmin; using std::fmax; using std::sqrt; using std::fabs;
using std::signbit;
#endif

#include "../../include/ice3gb.h"
#include "fastmath.cuh"

typedef Ice3gbConstants Cst;

#if defined(__CUDACC__)
#define ICE3_HD __host__ __device__ __forceinline__
#else
#define ICE3_HD inline
#endif

ICE3_HD double sq(double x) { return x * x; }
// Separately rounded multiply and add (never fused into an FMA).
ICE3_HD double mul_rn(double a, double b)
{
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  volatile double p = a * b;
  return p;
#endif
}
ICE3_HD double add_rn(double a, double b)
{
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  volatile double p = a + b;
  return p;
#endif
}
// The bit pattern of x through an inline-assembly move, which the compiler
// cannot see through: a test that equals an FP64 comparison (x == 0, x != 0)
// would otherwise be turned back into one, on the FP64 pipe.
ICE3_HD uint64_t opaque_bits(double x)
{
#if defined(__CUDA_ARCH__)
  unsigned long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
#else
  return (uint64_t)fm::bits_(x);
#endif
}
// Comparisons and clamps on the IEEE bit patterns.  On GB300 an FP64 compare
// (and so fmin/fmax) issues on the FP64 pipe at the FP64 FMA rate, while the
// same test on the 64-bit pattern runs on the integer pipe at ~30x the rate.
// Ordering key: for non-NaN doubles the signed 64-bit integer
// (sign ? -|bits| : bits) orders like the values, with -0 and +0 equal as
// IEEE compares them.  The plain versions below do not handle NaN operands
// (their callers see finite values by construction); nmin/nmax do.
ICE3_HD int64_t dkey(double x)
{
  const int64_t b = fm::bits_(x);
  return b < 0 ? -(b & 0x7fffffffffffffffLL) : b;
}
ICE3_HD bool isnan_(double a) { return (fm::bits_(a) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }

// NaN-propagating minimum/maximum/clip, as numpy's minimum/maximum/clip
// (the reference JAX lets NaN through on degenerate inputs, e.g. a negative
// vapour source with no mass flux, stencils/ice_adjust.py:293-296); CUDA's
// fmin/fmax would return the other operand instead.  Same results as
// (a < b || a != a) ? a : b, evaluated on the integer pipe.
ICE3_HD double nmin(double a, double b) { return (isnan_(a) || (!isnan_(b) && dkey(a) < dkey(b))) ? a : b; }
ICE3_HD double nmax(double a, double b) { return (isnan_(a) || (!isnan_(b) && dkey(a) > dkey(b))) ? a : b; }
ICE3_HD double nclip01(double x) { return nmin(nmax(x, 0.0), 1.0); }
// IEEE a > b / a >= b (false when either is NaN), on the integer pipe.
ICE3_HD bool fgt(double a, double b) { return !isnan_(a) && !isnan_(b) && dkey(a) > dkey(b); }
ICE3_HD bool fge(double a, double b) { return !isnan_(a) && !isnan_(b) && dkey(a) >= dkey(b); }
ICE3_HD bool gtd(double a, double b) { return dkey(a) > dkey(b); }        // a > b
ICE3_HD bool ltd(double a, double b) { return dkey(a) < dkey(b); }        // a < b
// a > b for a threshold b >= +0 (a of any sign): the raw patterns suffice.
ICE3_HD bool gtp(double a, double b) { return fm::bits_(a) > fm::bits_(b); }
// a < b for a >= +0 (b of any sign >= +0).
ICE3_HD bool ltp(double a, double b) { return fm::bits_(a) < fm::bits_(b); }
ICE3_HD bool pos(double a) { return fm::bits_(a) > 0; }                   // a > 0
ICE3_HD double pmax0(double a) { return pos(a) ? a : 0.0; }               // fmax(0, a)
ICE3_HD double dmax(double a, double b) { return gtd(a, b) ? a : b; }
ICE3_HD double dmin(double a, double b) { return gtd(a, b) ? b : a; }
// a == +-0.
ICE3_HD bool zerod_(double a) { return (opaque_bits(a) << 1) == 0; }
// x < 0 (not -0), on the bit pattern.
ICE3_HD bool negd(double x) { return fm::bits_(x) < 0 && fm::bits_(x) != INT64_MIN; }
// |a| > b for b >= +0.
ICE3_HD bool abs_gtp(double a, double b) { return (fm::bits_(a) & 0x7fffffffffffffffLL) > fm::bits_(b); }
// a != 0 (nor -0), on the bit pattern.
ICE3_HD bool nz(double a) { return (opaque_bits(a) << 1) != 0; }
// True on every lane when the predicate holds on some active lane of the warp:
// a block of arithmetic that is exact when skipped on lanes whose inputs are
// zero runs for the warp or for none of it (the host build: the lane alone).
ICE3_HD bool warp_any(bool p)
{
#if defined(__CUDA_ARCH__)
  return __any_sync(__activemask(), p);
#else
  return p;
#endif
}

// num / den to within 2^-22 relative, from the FP32 reciprocal of den
// (truncated to FP32) and one FP64 multiply; exact in sign.  0 where den is
// outside FP32's normal range.  Used to skip an IEEE division whose result
// cannot change a min / max.
ICE3_HD double quot_est(double num, double den)
{
  const int e = (int)((fm::bits_(den) >> 52) & 0x7ff);
  if (e <= 898 || e >= 1149) return 0.0;
  return num * fm::to_f64(fm::rcpf_(fm::to_f32(den)));
}
// True only if the quotient that est estimates (quot_est) is above bound
// for certain.
ICE3_HD bool est_above(double est, double bound) { return gtd(est, bound + fabs(bound) * 0x1p-18); }
ICE3_HD bool quot_above(double num, double den, double bound) { return est_above(quot_est(num, den), bound); }

// x**a evaluated as exp(a*log(x)) with the FP64-lean exp/log of
// fastmath.cuh.  For the exponents of the scheme (|a*log x| < 60) this stays
// within ~1e-14 relative of pow(), well inside the 1e-10 parity bar, at a
// fraction of the FP64 instructions; callers raising one base to several
// powers pass a shared log.
ICE3_HD double powl_(double logx, double a) { return fm::fexp(a * logx); }
ICE3_HD double fpow(double x, double a) { return fm::fexp(a * fm::flog(x)); }

// TIWMX saturation tables of OCND2 (micro/modd_tiwmx.F90, filled by
// micro/mode_ini_tiwmx.F90 from micro/mode_tiwmx_fun.F90) at T = j/100 K,
// j = 13200..37316, stored one after the other: ESTABW, ESTABI (the ice
// formula at and below 273.15 K, the water one above), A2TAB (AA2), BB3TAB
// (BB3), AM3TAB (AM3, 0 above 273.15 K), REDINTAB (REDIN).
constexpr int kTiwmxStart = 13200, kTiwmxStop = 37316, kTiwmxN = kTiwmxStop - kTiwmxStart + 1;
enum { TW_ESW = 0, TW_ESI, TW_A2, TW_BB3, TW_AM3, TW_REDIN, TW_N };

// TAB(NINT(100 T)) (micro/mode_tiwmx.F90), NINT rounding half away from
// zero; the index is clamped to the table.
ICE3_HD double tiwmx_at(const double *tab, double t)
{
  long j = (long)round(100.0 * t);
  j = j < kTiwmxStart ? kTiwmxStart : (j > kTiwmxStop ? kTiwmxStop : j);
#if defined(__CUDA_ARCH__)
  return __ldg(tab + (j - kTiwmxStart));
#else
  return tab[j - kTiwmxStart];
#endif
}

#if defined(__CUDACC__)
// 128-bit streaming accessors (LDG.128 / STG.128).
__device__ __forceinline__ double2 ld2(const double *p, long i) { return __ldg(reinterpret_cast<const double2 *>(p + i)); }
__device__ __forceinline__ void st2(double *p, long i, double a, double b)
{
  __stcs(reinterpret_cast<double2 *>(p + i), make_double2(a, b));
}
__device__ __forceinline__ double ld1(const double *p, long i) { return __ldg(p + i); }
#endif
