// FP64 elementary functions that spend few FP64-pipe instructions.
//
// On GB300 the FP64 pipe issues 2 fused multiply-adds per clock per SM, the
// FP32 pipe 128 and the integer pipe 64, so a double-precision log or
// arctangent from a generic library (tens of FP64 instructions each) dominates
// the prism kernels.  The functions below do every step that does not need 53
// bits -- exponent/mantissa splitting, table indexing, seeds, quotients and
// series on float pairs (two floats, ~46 bits) -- with integer and FP32
// instructions, and keep only the final refinement or assembly in FP64:
//
//   lm_sqrt   float-pair square root of the mantissa, one FP64 Newton step
//                                                                  3 FP64 ops
//   lm_div    FP32 reciprocal seed, one Newton step, one residual    5 FP64 ops
//   lm_log    table-driven logarithm after P. T. P. Tang, "Table-driven
//             implementation of the logarithm function in IEEE
//             floating-point arithmetic", ACM TOMS 16(4), 1990:
//             x = 2^e m, m in [0.75, 1.5); t = m c_k - 1 with c_k ~ 1/g_k
//             from a 193-entry grid; ln x = e ln2 + (-ln c_k) + log1p(t),
//             log1p by its Taylor series to t^8 (terms t^5.. in FP32)   ~10 FP64 ops
//   lm_log_quot  the same reduction for ln((p1 p2)/(q1 q2)) with the exact
//             FMA numerator near 1 and t, log1p(t) on float pairs
//                                       4 FP64 ops near 1, 7 otherwise
//   lm_arg_near  argument of a complex number, unwrapped to the 2*pi branch
//             nearest an FP32 estimate: exact rotation by quarter turns,
//             rotation by a tabulated angle, quotient and
//             arctan(u) = u - u^3/3 + u^5/5 - u^7/7 on float pairs
//                                       1 FP64 op for small angles, <= 4 otherwise
//
// Inputs outside the fast path (zero, negative, subnormal, inf, NaN) fall
// back to the generic functions, so special values behave like the library.
// All functions also compile for the host, where the FP32 approximations are
// replaced by correctly rounded float operations (used by the CPU tests).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef HG_HD
#define HG_HD __host__ __device__
#endif

#ifdef __CUDA_ARCH__
#define HG_TABLE_QUAL __device__ const
#else
#define HG_TABLE_QUAL static const
#endif

#include "lean_tables.inc"

namespace hg {
namespace lean {

// ---------------------------------------------------------------------------
// bit casts
HG_HD __forceinline__ long long d2ll(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
HG_HD __forceinline__ double ll2d(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}
HG_HD __forceinline__ unsigned f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  unsigned u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
HG_HD __forceinline__ float u2f(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

// FP32 approximations (MUFU on the device)
HG_HD __forceinline__ float rsqrt_approx(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / std::sqrt(x);
#endif
}
HG_HD __forceinline__ float rcp_approx(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}
HG_HD __forceinline__ int round_to_int(float x) {
#ifdef __CUDA_ARCH__
  return __float2int_rn(x);
#else
  return (int)std::nearbyint(x);
#endif
}
// FP32 estimate of atan2(y, x) within ~2e-5 rad, for branch selection only:
// arctan on [0, 1] by an odd degree-9 polynomial (least-squares fit on
// Chebyshev nodes, max error 1.2e-5) and the octant symmetries, with the
// sign of y (signed zeros included) as atan2.  (0, 0) gives 0.
HG_HD __forceinline__ float atan2_est(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float t = mn * rcp_approx(mx);
  const float t2 = t * t;
  float p = fmaf(t2, fmaf(t2, fmaf(t2, fmaf(t2, 0.0208451133f, -0.0851563513f), 0.180159301f),
                          -0.330304801f),
                 0.999866307f) *
            t;
  p = ay > ax ? 1.57079637f - p : p;
  p = (f2u(x) >> 31) ? 3.14159274f - p : p;
  p = (f2u(y) >> 31) ? -p : p;
  return mx == 0.0f ? 0.0f : p;
}

// Generic library functions for the inputs outside the fast paths, kept out
// of line: inlined, their code would sit between the hot instructions of every
// call site and crowd the instruction cache.
#ifdef __CUDA_ARCH__
#define HG_COLD __device__ __noinline__
#else
#define HG_COLD inline
#endif
HG_COLD double cold_sqrt(double x) { return sqrt(x); }
HG_COLD double cold_rsqrt(double x) { return 1.0 / sqrt(x); }
HG_COLD double cold_div(double n, double d) { return n / d; }
HG_COLD double cold_log(double x) { return log(x); }
HG_COLD double cold_log_quot(double p, double d) { return log(p / d); }
HG_COLD double cold_atan2(double y, double x) { return atan2(y, x); }

// double -> float by truncating the mantissa, with the exponent lowered by
// (shift - 1023): an integer-pipe conversion (no FP64 instruction).  Values
// below the float range become signed zero, above it signed infinity.
HG_HD __forceinline__ float d2f_shift(double x, int shift) {
  long long b = d2ll(x);
  unsigned hi = (unsigned)((unsigned long long)b >> 32);
  unsigned sign = hi & 0x80000000u;
  int ef = (int)((hi >> 20) & 0x7ffu);
  int e = ef - shift + 127;
  unsigned mant = (unsigned)((b >> 29) & 0x7fffff);
  unsigned out = sign | ((unsigned)e << 23) | mant;
  out = (e <= 0 || ef == 0) ? sign : out;
  out = (e >= 255) ? (sign | 0x7f800000u) : out;
  return u2f(out);
}
HG_HD __forceinline__ float d2f_trunc(double x) { return d2f_shift(x, 1023); }

// float f times 2^k as a double, built with integer instructions (exact for
// normal f and results in the normal double range; zero and subnormal f -> 0).
HG_HD __forceinline__ double f2d_scaled(float f, int k) {
  unsigned u = f2u(f);
  unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  int ef = (int)((u >> 23) & 0xffu);
  unsigned long long mant = (unsigned long long)(u & 0x7fffffu) << 29;
  unsigned long long e = (unsigned long long)(long long)(ef - 127 + 1023 + k);
  unsigned long long b = sign | (e << 52) | mant;
  return ll2d((long long)(ef == 0 ? sign : b));
}

// int -> double with one FP64 add (exact for |e| < 2^31).
HG_HD __forceinline__ double int_to_double(int e) {
  return ll2d(0x4338000000000000LL + (long long)e) - 6755399441055744.0;
}

// int -> double without an FP64 instruction (exact for |e| < 2^24).
HG_HD __forceinline__ double small_int_to_double(int e) { return f2d_scaled((float)e, 0); }

// ---------------------------------------------------------------------------
// Float pairs: a value held as h + l in two floats (about 46 significant
// bits), computed on the FP32 pipe.  Built from the error-free
// transformations two-sum (D. E. Knuth, TAOCP vol. 2, sec. 4.2.2) and the
// exact product by fused multiply-add (the FMA form of T. J. Dekker, "A
// floating-point technique for extending the available precision", Numer.
// Math. 18, 1971).  The device versions use the round-to-nearest intrinsics
// so that the compiler never contracts or reassociates them.
struct F2 {
  float h, l;
};

HG_HD __forceinline__ float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
HG_HD __forceinline__ float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
HG_HD __forceinline__ float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
HG_HD __forceinline__ float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
HG_HD __forceinline__ float u32_to_f32(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint2float_rn(u);
#else
  return (float)u;
#endif
}

// a + b = s.h + s.l exactly, any order of magnitude
HG_HD __forceinline__ F2 two_sum(float a, float b) {
  const float s = fadd(a, b);
  const float bb = fsub(s, a);
  return F2{s, fadd(fsub(a, fsub(s, bb)), fsub(b, bb))};
}
// a + b = s.h + s.l exactly, for |a| >= |b| (or a == 0)
HG_HD __forceinline__ F2 quick_two_sum(float a, float b) {
  const float s = fadd(a, b);
  return F2{s, fsub(b, fsub(s, a))};
}
// a b = p.h + p.l exactly (no underflow)
HG_HD __forceinline__ F2 two_prod(float a, float b) {
  const float p = fmul(a, b);
  return F2{p, ffma(a, b, -p)};
}
// products and sums of pairs, relative error ~2^-44 (sums without heavy
// cancellation; with cancellation the error stays ~2^-46 of the operands)
HG_HD __forceinline__ F2 f2_mul(F2 a, F2 b) {
  const F2 p = two_prod(a.h, b.h);
  return quick_two_sum(p.h, ffma(a.h, b.l, ffma(a.l, b.h, p.l)));
}
HG_HD __forceinline__ F2 f2_add(F2 a, F2 b) {
  const F2 s = two_sum(a.h, b.h);
  return quick_two_sum(s.h, fadd(s.l, fadd(a.l, b.l)));
}
// a + b for |a.h| >= |b.h| (or within a rounding of each other): Fast2Sum
// on the high parts (p2_add_big lane by lane)
HG_HD __forceinline__ F2 f2_add_big(F2 a, F2 b) {
  const F2 s = quick_two_sum(a.h, b.h);
  return quick_two_sum(s.h, fadd(s.l, fadd(a.l, b.l)));
}
HG_HD __forceinline__ F2 f2_neg(F2 a) { return F2{-a.h, -a.l}; }
HG_HD __forceinline__ F2 f2_sub(F2 a, F2 b) { return f2_add(a, f2_neg(b)); }
HG_HD __forceinline__ F2 f2_sq(F2 a) {
  const F2 p = two_prod(a.h, a.h);
  return quick_two_sum(p.h, ffma(2.0f * a.h, a.l, p.l));
}

// a / b for b > 0: FP32 reciprocal refined to float accuracy, the quotient
// rounded to a float and one correction from the exact-by-FMA residual.
HG_HD __forceinline__ F2 f2_div(F2 a, F2 b) {
  float y = rcp_approx(b.h);
  y = ffma(y, ffma(-b.h, y, 1.0f), y);
  const float qh = fmul(a.h, y);
  float r = ffma(-qh, b.h, a.h);
  r = fadd(r, a.l);
  r = ffma(-qh, b.l, r);
  return F2{qh, fmul(r, y)};
}

// sqrt(a) for a pair a > 0 (normal): FP32 rsqrt seed refined to float
// accuracy, s = a.h y, one Newton correction from the pair residual
// a - s^2 (exact product by FMA): ~2^-46.
HG_HD __forceinline__ F2 f2_sqrt(F2 a) {
  float y = rsqrt_approx(a.h);
  y = fmul(y, ffma(fmul(-0.5f, a.h), fmul(y, y), 1.5f));
  const float s = fmul(a.h, y);
  const F2 s2 = two_prod(s, s);
  const float res = fadd(fsub(fsub(a.h, s2.h), s2.l), a.l);
  return quick_two_sum(s, fmul(res, fmul(0.5f, y)));
}

// The significand of a normal double (bits b) as a pair in [1, 2):
// h = the leading 24 bits, l = the other 29 bits (rounded to a float).
HG_HD __forceinline__ F2 mant_f2(long long b) {
  const float h = u2f(0x3f800000u | (unsigned)((b >> 29) & 0x7fffff));
  const float l = fmul(u32_to_f32((unsigned)(b & 0x1fffffff)), 0x1p-52f);
  return F2{h, l};
}

// 2^k as a float, for -126 <= k <= 127
HG_HD __forceinline__ float pow2f(int k) { return u2f((unsigned)(127 + k) << 23); }

// Signed value of the double with bits b times 2^(1023 - top) as a pair,
// where top >= the double's biased exponent ef: sign * mant * 2^(ef - top).
// Zero and subnormal inputs and results below 2^-120 give 0.
HG_HD __forceinline__ F2 scaled_f2(long long b, int top) {
  const int ef = (int)((b >> 52) & 0x7ff);
  const int k = ef - top;
  F2 m = mant_f2(b);
  const float sc = pow2f(k < -120 ? -120 : k);
  m.h = fmul(m.h, sc);
  m.l = fmul(m.l, sc);
  if (b < 0) m = f2_neg(m);
  return (ef == 0 || k < -120) ? F2{0.0f, 0.0f} : m;
}

// scaled_f2 for a value that is zero or within 2^-40 of the scale (ef >=
// top - 40, as make_geom_f2 checks first): the high float assembled from the
// bits (sign, exponent 127 + ef - top, the leading 23 fraction bits), the low
// one as the other 29 fraction bits times 2^(ef - top - 52) with the same
// sign -- the same pair as scaled_f2 with fewer instructions.
HG_HD __forceinline__ F2 scaled_f2_near(long long b, int top) {
  const unsigned hi = (unsigned)((unsigned long long)b >> 32), lo = (unsigned)b;
  const int ef = (int)((hi >> 20) & 0x7ffu);
  const unsigned sign = hi & 0x80000000u;
  const unsigned frac = ((hi << 3) | (lo >> 29)) & 0x7fffffu;
  const float h = u2f(sign | ((unsigned)(127 + ef - top) << 23) | frac);
  const float l = fmul(u32_to_f32(lo & 0x1fffffffu), u2f(sign | ((unsigned)(75 + ef - top) << 23)));
  return ef == 0 ? F2{0.0f, 0.0f} : F2{h, l};
}

// The pair as a double times 2^k, assembled with integer instructions: the
// 24-bit significand of h widened to 53 bits, the significand of l shifted
// into its place and added or subtracted, one normalisation step.  For
// |l| <= 2^-8 |h| (all pairs built here) and results in the normal double
// range; within 1 ulp (the bits of l below the double's last place are
// truncated).  A zero h gives l alone.
HG_HD __forceinline__ double f2_to_double(F2 a, int k) {
  const unsigned uh = f2u(a.h), ul = f2u(a.l);
  const int eh = (int)((uh >> 23) & 0xffu), el = (int)((ul >> 23) & 0xffu);
  if (eh == 0) return f2d_scaled(a.l, k);
  long long m = (long long)((uh & 0x7fffffu) | 0x800000u) << 29;  // in [2^52, 2^53)
  int sh = el - eh + 29;  // l's significand in units of the double's last place
  sh = sh > 30 ? 30 : sh;
  long long lm = (long long)((ul & 0x7fffffu) | 0x800000u);
  lm = sh >= 0 ? (lm << sh) : (sh > -25 ? (lm >> -sh) : 0);
  lm = el == 0 ? 0 : lm;
  m = ((uh ^ ul) >> 31) ? m - lm : m + lm;
  long long e = (long long)(eh - 127 + 1023 + k);
  if (m >= (1LL << 53)) {
    m >>= 1;
    e += 1;
  } else if (m < (1LL << 52)) {
    m <<= 1;
    e -= 1;
  }
  return ll2d((long long)((unsigned long long)(uh >> 31) << 63) | (e << 52) |
              (m & ((1LL << 52) - 1)));
}

// ---------------------------------------------------------------------------
// sqrt(x): x = 4^k m with m in [1, 4) held as a float pair; sqrt(m) to
// ~2^-43 from an FP32 rsqrt seed and one FP32 Newton correction of the pair
// residual, converted to a double (one FP64 add), then one FP64 Newton step
// s + (x - s^2) / (2 s) (two FMAs).
HG_HD __forceinline__ double lm_sqrt(double x) {
  const long long b = d2ll(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return cold_sqrt(x);
  const int e = ef - 1023;
  const int odd = e & 1;
  const int k = (e - odd) / 2;
  const float mh = u2f(((unsigned)(127 + odd) << 23) | (unsigned)((b >> 29) & 0x7fffff));
  const float ml =
      fmul(u32_to_f32((unsigned)(b & 0x1fffffff)), odd ? 0x1p-51f : 0x1p-52f);
  const float y = rsqrt_approx(mh);  // ~1/sqrt(m), 2^-22
  const float sh = fmul(mh, y);
  const float hy = fmul(0.5f, y);
  const float res = fadd(ffma(-sh, sh, mh), ml);  // m - sh^2
  const double s = f2_to_double(F2{sh, fmul(res, hy)}, k);
  const double r = fma(-s, s, x);
  return fma(r, f2d_scaled(hy, -k), s);
}

// 1 / sqrt(x): FP32 seed of the mantissa and two Newton steps
// y <- y (1.5 - (x/2) y^2); other inputs take the generic path.
HG_HD __forceinline__ double lm_rsqrt(double x) {
  const long long b = d2ll(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return cold_rsqrt(x);
  const int e = ef - 1023;
  const int odd = e & 1;
  const int k = (e - odd) / 2;
  const float mf = u2f(((unsigned)(127 + odd) << 23) | (unsigned)((b >> 29) & 0x7fffff));
  double y = f2d_scaled(rsqrt_approx(mf), -k);
  const double hx = 0.5 * x;
  y = y * fma(-hx, y * y, 1.5);
  return y * fma(-hx, y * y, 1.5);
}

// n / d for d > 0 (other d fall back to the IEEE division).
HG_HD __forceinline__ double lm_div(double n, double d) {
  const long long b = d2ll(d);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef >= 0x7fe) return cold_div(n, d);
  const int e = ef - 1023;
  const float rf = rcp_approx(u2f(0x3f800000u | (unsigned)((b >> 29) & 0x7fffff)));
  double r = f2d_scaled(rf, -e);  // ~ 1/d, rel. err ~2^-22
  const double t = fma(-d, r, 1.0);
  r = fma(r, t, r);  // ~2^-44
  const double q = n * r;
  const double res = fma(-d, q, n);
  return fma(res, r, q);
}

struct Tables {
  const double* logc;
  const double* logl;
  const double* th;
  const float* csf;    // cos(th_j) as float pairs (hi, lo)
  const float* snf;    // sin(th_j) as float pairs
  const float* loglf;  // -ln(c_k) as float pairs
  const float* thf;    // th_j as float pairs
};

// Host view of the tables (the device kernels stage them in shared memory).
inline Tables host_tables() {
#ifdef __CUDA_ARCH__
  return Tables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
#else
  return Tables{kLogC, kLogL, kArgTh, kArgCosF, kArgSinF, kLogLF, kArgThF};
#endif
}

HG_HD __forceinline__ double lm_log(double x, const Tables& T) {
  const long long b = d2ll(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return cold_log(x);
  // x = 2^e0 m0, m0 in [1, 2); fold to m in [0.75, 1.5)
  const int top = (int)((b >> 51) & 1);  // m0 >= 1.5
  const int e = ef - 1023 + top;
  const double m = ll2d((b & 0x000fffffffffffffLL) | ((long long)(1023 - top) << 52));
  float mf = u2f(0x3f800000u | (unsigned)((b >> 29) & 0x7fffff));
  mf = top ? 0.5f * mf : mf;
  int k = round_to_int((mf - 0.75f) * 256.0f);
  k = k < 0 ? 0 : (k > kLogTableSize - 1 ? kLogTableSize - 1 : k);
  const double t = fma(m, T.logc[k], -1.0);  // |t| <= ~2^-8.6
  const float tf = d2f_trunc(t);
  // 1/5 - t/6 + t^2/7 - t^3/8 : contributes t^5 r2, FP32 is ample
  const float r2 = fmaf(tf, fmaf(tf, fmaf(tf, -0.125f, 0.142857143f), -0.166666672f), 0.2f);
  double a = fma(t, f2d_scaled(r2, 0), -0.25);
  a = fma(t, a, 1.0 / 3.0);
  a = fma(t, a, -0.5);
  const double p = fma(t * t, a, t);  // log1p(t)
  const double ed = int_to_double(e);
  return fma(ed, kLn2Hi, T.logl[k]) + fma(ed, kLn2Lo, p);
}

// Argument of a complex number on the 2*pi branch nearest `est` (an FP32
// estimate of the wanted angle, within ~1e-3 of it).  The vector is rotated
// by -q pi/2 exactly (q = nearest quarter turn of est) and, as a float pair,
// by -th_j (th_j = j pi/128 nearest the remainder); the residual angle
// (|u| <= ~tan(pi/256)) is arctan(u), u = im/re, by
//   u + u^3 (-1/3 + u^2/5 - u^4/7)
// with u, u^3 and 1/3 as float pairs and the tail in FP32 (~2^-46 absolute).
// FP64 work: one add to form the double, plus th_j and q pi/2 when nonzero.
HG_HD __forceinline__ void arg_plan(float est, int& q, int& j) {
  q = round_to_int(est * 0.636619772f);  // quarter turns
  const float rem = fmaf((float)(-q), 1.57079637f, est);
  j = round_to_int(rem * 40.7436654f);  // 128 / pi
  j = j < -kArgTableHalf ? -kArgTableHalf : (j > kArgTableHalf ? kArgTableHalf : j);
}

// (re, im): the vector already rotated by -q pi/2, as float pairs of
// magnitude ~1 (any common scale).
HG_HD __forceinline__ double arg_core(F2 re, F2 im, int q, int j, const Tables& T) {
  const F2 re0 = re, im0 = im;
  if (j != 0) {  // rotate by -th_j
    const int jj = 2 * (j + kArgTableHalf);
    const F2 C{T.csf[jj], T.csf[jj + 1]}, S{T.snf[jj], T.snf[jj + 1]};
    const F2 r2 = f2_add(f2_mul(re, C), f2_mul(im, S));
    im = f2_add(f2_mul(im, C), f2_neg(f2_mul(re, S)));
    re = r2;
  }
  const F2 u = f2_div(im, re);
  double delta;
  if (re.h > 0.0f && fabsf(u.h) < 0.02f) {
    F2 s2 = two_prod(u.h, u.h);
    s2.l = ffma(2.0f * u.h, u.l, s2.l);  // u^2
    F2 w = two_prod(s2.h, u.h);
    w.l = ffma(s2.h, u.l, ffma(s2.l, u.h, w.l));  // u^3
    const float tail = fmul(s2.h, ffma(s2.h, -0.142857143f, 0.2f));  // u^2/5 - u^4/7
    F2 c = two_prod(w.h, -kThirdHi);
    c.l = ffma(w.h, fsub(tail, kThirdLo), ffma(w.l, -kThirdHi, c.l));  // u^3 (-1/3 + tail)
    F2 a = quick_two_sum(u.h, c.h);
    a.l = fadd(a.l, fadd(u.l, c.l));
    delta = f2_to_double(a, 0);
  } else {
    // estimate too far off or non-finite input: generic path on the
    // quarter-turn-rotated vector
    delta = cold_atan2(f2_to_double(im0, 0), f2_to_double(re0, 0));
    j = 0;
  }
  if (q == 0) return j == 0 ? delta : T.th[j + kArgTableHalf] + delta;
  const double qd = small_int_to_double(q);
  return fma(qd, kPio2Hi, T.th[j + kArgTableHalf]) + fma(qd, kPio2Lo, delta);
}

HG_HD __forceinline__ double lm_arg_near(double pr, double pi, float est, const Tables& T) {
  int q, j;
  arg_plan(est, q, j);
  // rotate by -q pi/2 exactly: (r0, i0) as the bits of +-pr / +-pi
  const int qm = q & 3;
  const long long bpr = d2ll(pr), bpi = d2ll(pi);
  const long long kSign = (long long)0x8000000000000000ULL;
  const long long br = qm == 0 ? bpr : (qm == 1 ? bpi : (qm == 2 ? bpr ^ kSign : bpi ^ kSign));
  const long long bi = qm == 0 ? bpi : (qm == 1 ? bpr ^ kSign : (qm == 2 ? bpi ^ kSign : bpr));
  const int er = (int)((br >> 52) & 0x7ff), ei = (int)((bi >> 52) & 0x7ff);
  if (er == 0x7ff || ei == 0x7ff) return cold_atan2(pi, pr);
  const int top = (er > ei ? er : ei);
  return arg_core(scaled_f2(br, top), scaled_f2(bi, top), q, j, T);
}

// A double as a float pair (values below 2^-120 in magnitude give 0).
HG_HD __forceinline__ F2 double_to_f2(double x) { return scaled_f2(d2ll(x), 1023); }

// arg_core with the result as a float pair: theta_j and q pi/2 added on
// pairs (no FP64 instruction on the fast path).
HG_HD __forceinline__ F2 arg_core_f2(F2 re, F2 im, int q, int j, const Tables& T) {
  const F2 re0 = re, im0 = im;
  if (j != 0) {  // rotate by -th_j
    const int jj = 2 * (j + kArgTableHalf);
    const F2 C{T.csf[jj], T.csf[jj + 1]}, S{T.snf[jj], T.snf[jj + 1]};
    const F2 r2 = f2_add(f2_mul(re, C), f2_mul(im, S));
    im = f2_add(f2_mul(im, C), f2_neg(f2_mul(re, S)));
    re = r2;
  }
  const F2 u = f2_div(im, re);
  F2 a;
  if (re.h > 0.0f && fabsf(u.h) < 0.02f) {
    F2 s2 = two_prod(u.h, u.h);
    s2.l = ffma(2.0f * u.h, u.l, s2.l);  // u^2
    F2 w = two_prod(s2.h, u.h);
    w.l = ffma(s2.h, u.l, ffma(s2.l, u.h, w.l));  // u^3
    const float tail = fmul(s2.h, ffma(s2.h, -0.142857143f, 0.2f));  // u^2/5 - u^4/7
    F2 c = two_prod(w.h, -kThirdHi);
    c.l = ffma(w.h, fsub(tail, kThirdLo), ffma(w.l, -kThirdHi, c.l));  // u^3 (-1/3 + tail)
    a = quick_two_sum(u.h, c.h);
    a.l = fadd(a.l, fadd(u.l, c.l));
  } else {
    // estimate too far off or non-finite input: generic path on the
    // quarter-turn-rotated vector
    a = double_to_f2(cold_atan2(f2_to_double(im0, 0), f2_to_double(re0, 0)));
    j = 0;
  }
  if (j != 0) {
    const int jj = 2 * (j + kArgTableHalf);
    a = f2_add(a, F2{T.thf[jj], T.thf[jj + 1]});
  }
  if (q != 0) {  // q pi/2 with pi/2 in three floats (q * F1 exact)
    const float qf = (float)q;
    F2 p = two_prod(qf, kPio2F2);
    p.l = ffma(qf, kPio2F3, p.l);
    a = f2_add(a, f2_add(F2{fmul(qf, kPio2F1), 0.0f}, p));
  }
  return a;
}

// The same for a vector given as float pairs (finite, magnitude ~1).
HG_HD __forceinline__ F2 lm_arg_near_f2(F2 pr, F2 pi, float est, const Tables& T) {
  int q, j;
  arg_plan(est, q, j);
  const int qm = q & 3;
  const F2 r0 = qm == 0 ? pr : (qm == 1 ? pi : (qm == 2 ? f2_neg(pr) : f2_neg(pi)));
  const F2 i0 = qm == 0 ? pi : (qm == 1 ? f2_neg(pr) : (qm == 2 ? f2_neg(pi) : pr));
  return arg_core_f2(r0, i0, q, j, T);
}

// log1p(t) for |t| <= 2^-8.5 on float pairs:
//   t - t^2/2 + t^3 (1/3 - t/4 + t^2/5 - t^3/6)
// with t, t^2, t^3 and 1/3 as pairs and the tail in FP32 (~2^-47 relative).
HG_HD __forceinline__ F2 log1p_series_f2(F2 t) {
  F2 s2 = two_prod(t.h, t.h);
  s2.l = ffma(2.0f * t.h, t.l, s2.l);  // t^2
  F2 w = two_prod(s2.h, t.h);
  w.l = ffma(s2.h, t.l, ffma(s2.l, t.h, w.l));  // t^3
  const float tail = fmul(t.h, ffma(t.h, ffma(t.h, -0.166666672f, 0.2f), -0.25f));
  F2 c = two_prod(w.h, kThirdHi);
  c.l = ffma(w.h, fadd(tail, kThirdLo), ffma(w.l, kThirdHi, c.l));  // t^3 (1/3 + tail)
  F2 v = quick_two_sum(fmul(-0.5f, s2.h), c.h);
  v.l = fadd(v.l, ffma(-0.5f, s2.l, c.l));
  F2 lp = quick_two_sum(t.h, v.h);
  lp.l = fadd(lp.l, fadd(t.l, v.l));
  return lp;
}

// ln(1 + t) for t > -1 on float pairs (t given accurately, as from a
// cancellation-free numerator).  Small |t|: the series.  Otherwise Tang's
// reduction of w = 1 + t = 2^E m with c_k ~ 1/m from the table, the reduced
// argument formed as t c' + (c' - 1) (c' = c_k 2^-E; c' - 1 exact), so no
// digit of t is lost, then E ln2 - ln c_k + log1p(reduced) on pairs.
HG_HD __forceinline__ F2 log1p_f2(F2 t, const Tables& T) {
  if (fabsf(t.h) < 0.0026f) return log1p_series_f2(t);
  const F2 w = f2_add(F2{1.0f, 0.0f}, t);
  const unsigned uw = f2u(w.h);
  int E = (int)((uw >> 23) & 0xffu) - 127;
  float m = u2f((uw & 0x7fffffu) | 0x3f800000u);  // [1, 2)
  if (m >= 1.5f) {
    m = fmul(m, 0.5f);
    E += 1;
  }
  int k = round_to_int((m - 0.75f) * 256.0f);
  k = k < 0 ? 0 : (k > kLogTableSize - 1 ? kLogTableSize - 1 : k);
  const float cp = fmul(d2f_trunc(T.logc[k]), pow2f(-E));  // c_k is a float: exact
  const F2 red = f2_add(f2_mul(t, F2{cp, 0.0f}), two_sum(cp, -1.0f));
  const F2 lp = log1p_series_f2(red);
  const float ef = (float)E;
  F2 e2 = two_prod(ef, kLn2F2);
  e2.l = ffma(ef, kLn2F3, e2.l);
  const F2 eln2 = f2_add(F2{fmul(ef, kLn2F1), 0.0f}, e2);  // E ln 2 (E * F1 exact)
  return f2_add(f2_add(eln2, F2{T.loglf[2 * k], T.loglf[2 * k + 1]}), lp);
}

// ln((p1 p2) / (q1 q2)) for positive normal arguments, without forming the
// quotient: the FP32 estimate of the mantissa ratio selects the table entry
// c_k ~ 1/g_k and the binary exponent E, then
//   t = (p1 p2 c_k 2^-E - q1 q2) / (q1 q2)   (numerator by one FMA)
// and ln = E ln2 - ln c_k + log1p(t).  When the quotient is within half a
// table step of 1 (c_k = 1, E = 0) the numerator is the exact FMA
// p1 p2 - q1 q2 and the table/exponent terms vanish: the log of a ratio near
// 1 keeps its relative accuracy.  The division and log1p run on float pairs
// (t to ~2^-44 relative, |t| <= 2^-8.5):
//   log1p(t) = t - t^2/2 + t^3 (1/3 - t/4 + t^2/5 - t^3/6)
// with t, t^2, t^3 and 1/3 as pairs and the tail in FP32.  FP64 work: the
// products and the numerator FMA, one add to form the double, and three
// more for the table and exponent terms away from 1.  ONE_FACTOR skips the
// products (p2 = q2 = 1).  Other inputs take the generic path.
template <bool ONE_FACTOR>
HG_HD __forceinline__ double lm_log_quot(double p1, double p2, double q1, double q2,
                                         const Tables& T) {
  const long long b1 = d2ll(p1), b3 = d2ll(q1);
  const long long b2 = ONE_FACTOR ? 0x3ff0000000000000LL : d2ll(p2);
  const long long b4 = ONE_FACTOR ? 0x3ff0000000000000LL : d2ll(q2);
  const int e1 = (int)((b1 >> 52) & 0x7ff), e2 = (int)((b2 >> 52) & 0x7ff);
  const int e3 = (int)((b3 >> 52) & 0x7ff), e4 = (int)((b4 >> 52) & 0x7ff);
  const double d = ONE_FACTOR ? q1 : q1 * q2;
  const long long bd = d2ll(d);
  const int ed = (int)((bd >> 52) & 0x7ff);
  const bool ok = b1 > 0 && b2 > 0 && b3 > 0 && b4 > 0 && e1 != 0 && e2 != 0 && e3 != 0 &&
                  e4 != 0 && e1 != 0x7ff && e2 != 0x7ff && e3 != 0x7ff && e4 != 0x7ff &&
                  ed != 0 && ed < 0x7fe;
  if (!ok) return cold_log_quot(ONE_FACTOR ? p1 : p1 * p2, d);
  const auto mant = [](long long b) { return u2f(0x3f800000u | (unsigned)((b >> 29) & 0x7fffff)); };
  float rf = ONE_FACTOR ? mant(b1) * rcp_approx(mant(b3))
                        : (mant(b1) * mant(b2)) * rcp_approx(mant(b3) * mant(b4));
  int E = (e1 + e2) - (e3 + e4);
#pragma unroll
  for (int s = 0; s < 2; s++) {
    if (rf >= 1.5f) { rf *= 0.5f; E += 1; }
    if (rf < 0.75f) { rf *= 2.0f; E -= 1; }
  }
  int k = round_to_int((rf - 0.75f) * 256.0f);
  k = k < 0 ? 0 : (k > kLogTableSize - 1 ? kLogTableSize - 1 : k);
  const bool near1 = (E == 0) && (k == 64);
  if (!near1 && (E > 1000 || E < -1000)) return cold_log_quot(ONE_FACTOR ? p1 : p1 * p2, d);
  // numerator p1 p2 c_k 2^-E - q1 q2, exact when c_k 2^-E = 1
  double num;
  if (near1) {
    num = ONE_FACTOR ? p1 - d : fma(p1, p2, -d);
  } else {
    const double cp = ll2d(d2ll(T.logc[k]) - ((long long)E << 52));  // c_k 2^-E, exact
    num = fma(ONE_FACTOR ? p1 : p1 * p2, cp, -d);
  }
  const long long bn = d2ll(num);
  const int en = (int)((bn >> 52) & 0x7ff);  // 0: zero or subnormal, counted as t = 0
  if (en == 0x7ff) return cold_log_quot(ONE_FACTOR ? p1 : p1 * p2, d);
  // t = num / d: significands divided as pairs, scaled by 2^(en - ed)
  F2 t = f2_div(mant_f2(bn), mant_f2(bd));
  const int sc = en - ed;
  const float scale = pow2f(sc < -120 ? -120 : (sc > 0 ? 0 : sc));
  t.h = fmul(t.h, scale);
  t.l = fmul(t.l, scale);
  if (bn < 0) t = f2_neg(t);
  if (en == 0 || sc < -120) t = F2{0.0f, 0.0f};  // |t| < 2^-120 counts as 0
  const double p = f2_to_double(log1p_series_f2(t), 0);  // log1p(t)
  if (near1) return p;
  const double edd = small_int_to_double(E);
  return fma(edd, kLn2Hi, T.logl[k]) + fma(edd, kLn2Lo, p);
}

// FP32 angle of (re + i im) for doubles of any magnitude (joint scaling by a
// power of two with integer instructions).
HG_HD __forceinline__ float arg_f32(double re, double im) {
  const int er = (int)((d2ll(re) >> 52) & 0x7ff);
  const int ei = (int)((d2ll(im) >> 52) & 0x7ff);
  const int e = er > ei ? er : ei;
  return atan2_est(d2f_shift(im, e), d2f_shift(re, e));
}

}  // namespace lean
}  // namespace hg
