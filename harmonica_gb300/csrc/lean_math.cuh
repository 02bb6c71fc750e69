// FP64 elementary functions that spend few FP64-pipe instructions.
//
// On GB300 the FP64 pipe issues 2 fused multiply-adds per clock per SM, the
// FP32 pipe 128 and the integer pipe 64, so a double-precision log or
// arctangent from a generic library (tens of FP64 instructions each) dominates
// the prism kernels.  The functions below do every step that does not need 53
// bits -- exponent/mantissa splitting, table indexing, seeds, the high-order
// terms of series -- with integer and FP32 instructions, and keep only the
// final refinement in FP64:
//
//   lm_sqrt   FP32 rsqrt seed of the mantissa, two Newton steps     5 FP64 ops
//   lm_div    FP32 reciprocal seed, one Newton step, one residual    5 FP64 ops
//   lm_log    table-driven logarithm after P. T. P. Tang, "Table-driven
//             implementation of the logarithm function in IEEE
//             floating-point arithmetic", ACM TOMS 16(4), 1990:
//             x = 2^e m, m in [0.75, 1.5); t = m c_k - 1 with c_k ~ 1/g_k
//             from a 193-entry grid; ln x = e ln2 + (-ln c_k) + log1p(t),
//             log1p by its Taylor series to t^8 (terms t^5.. in FP32)   ~10 FP64 ops
//   lm_arg_near  argument of a complex number, unwrapped to the 2*pi branch
//             nearest an FP32 estimate: exact rotation by quarter turns,
//             rotation by a tabulated angle (cos/sin correctly rounded),
//             then arctan(u) = u - u^3/3 + (u^5/5 - u^7/7 in FP32)     ~17 FP64 ops
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
HG_HD __forceinline__ float atan2_f32(float y, float x) {
#ifdef __CUDA_ARCH__
  return atan2f(y, x);
#else
  return std::atan2(y, x);
#endif
}

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

// ---------------------------------------------------------------------------
HG_HD __forceinline__ double lm_sqrt(double x) {
  const long long b = d2ll(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return sqrt(x);
  const int e = ef - 1023;
  const int odd = e & 1;
  const int k = (e - odd) / 2;
  // mantissa in [1, 4): exponent 0 or 1
  const float mf = u2f(((unsigned)(127 + odd) << 23) | (unsigned)((b >> 29) & 0x7fffff));
  const float yf = rsqrt_approx(mf);
  const double y = f2d_scaled(yf, -k);      // ~ 1/sqrt(x), rel. err ~2^-22
  const double h = f2d_scaled(yf, -k - 1);  // y / 2
  double s = x * y;
  double r = fma(-s, s, x);
  s = fma(r, h, s);  // ~2^-44
  r = fma(-s, s, x);
  return fma(r, h, s);
}

// 1 / sqrt(x): FP32 seed of the mantissa and two Newton steps
// y <- y (1.5 - (x/2) y^2); other inputs take the generic path.
HG_HD __forceinline__ double lm_rsqrt(double x) {
  const long long b = d2ll(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return 1.0 / sqrt(x);
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
  if (b <= 0 || ef == 0 || ef >= 0x7fe) return n / d;
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
  const double* cs;
  const double* sn;
};

// Host view of the tables (the device kernels stage them in shared memory).
inline Tables host_tables() {
#ifdef __CUDA_ARCH__
  return Tables{nullptr, nullptr, nullptr, nullptr, nullptr};
#else
  return Tables{kLogC, kLogL, kArgTh, kArgCos, kArgSin};
#endif
}

HG_HD __forceinline__ double lm_log(double x, const Tables& T) {
  const long long b = d2ll(x);
  const int ef = (int)((b >> 52) & 0x7ff);
  if (b <= 0 || ef == 0 || ef == 0x7ff) return log(x);
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

// Argument of (pr + i pi) on the 2*pi branch nearest `est` (an FP32
// estimate of the wanted angle, within ~1e-3 of it).  The table rotation and
// the quarter-turn assembly are skipped for small angles (the common case for
// distant faces).
HG_HD __forceinline__ double lm_arg_near(double pr, double pi, float est, const Tables& T) {
  const int q = round_to_int(est * 0.636619772f);  // quarter turns
  const float rem = fmaf((float)(-q), 1.57079637f, est);
  int j = round_to_int(rem * 40.7436654f);  // 128 / pi
  j = j < -kArgTableHalf ? -kArgTableHalf : (j > kArgTableHalf ? kArgTableHalf : j);
  // rotate by -q pi/2 exactly
  const int qm = q & 3;
  const double r0 = qm == 0 ? pr : (qm == 1 ? pi : (qm == 2 ? -pr : -pi));
  const double i0 = qm == 0 ? pi : (qm == 1 ? -pr : (qm == 2 ? -pi : pr));
  double re = r0, im = i0;
  if (j != 0) {  // rotate by -th_j
    const double C = T.cs[j + kArgTableHalf], S = T.sn[j + kArgTableHalf];
    re = fma(i0, S, r0 * C);
    im = fma(-r0, S, i0 * C);
  }
  double delta;
  const double u = lm_div(im, re);
  const float uf = d2f_trunc(u);
  if (fabsf(uf) < 0.02f && d2ll(re) > 0) {
    const float u2f_ = uf * uf;
    const float tail = u2f_ * fmaf(u2f_, -0.142857143f, 0.2f);  // u^2/5 - u^4/7
    const double u3 = (u * u) * u;
    delta = fma(u3, f2d_scaled(tail, 0) - 1.0 / 3.0, u);
  } else {
    delta = atan2(im, re);  // estimate too far off: generic path
  }
  if (q == 0) return j == 0 ? delta : T.th[j + kArgTableHalf] + delta;
  const double qd = int_to_double(q);
  return fma(qd, kPio2Hi, T.th[j + kArgTableHalf]) + fma(qd, kPio2Lo, delta);
}

// ln((p1 p2) / (q1 q2)) for positive normal arguments, without forming the
// quotient: the FP32 estimate of the mantissa ratio selects the table entry
// c_k ~ 1/g_k and the binary exponent E, then
//   t = (p1 p2 c_k 2^-E - q1 q2) / (q1 q2)   (numerator by one FMA)
// and ln = E ln2 - ln c_k + log1p(t).  When the quotient is within half a
// table step of 1 (c_k = 1, E = 0) the numerator is the exact FMA
// p1 p2 - q1 q2 and the table/exponent terms vanish: the log of a ratio near
// 1 keeps its full relative accuracy.  ONE_FACTOR skips the products
// (p2 = q2 = 1).  Other inputs take the generic path.
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
  if (!ok) return log((ONE_FACTOR ? p1 : p1 * p2) / d);
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
  if (!near1 && (E > 1000 || E < -1000)) return log((ONE_FACTOR ? p1 : p1 * p2) / d);
  // 1/d: FP32 seed and one Newton step (~2^-44; t is small, so ample)
  double r = f2d_scaled(rcp_approx(mant(bd)), -(ed - 1023));
  r = fma(r, fma(-d, r, 1.0), r);
  double num;
  if (near1) {
    num = ONE_FACTOR ? p1 - d : fma(p1, p2, -d);
  } else {
    const double cp = ll2d(d2ll(T.logc[k]) - ((long long)E << 52));  // c_k 2^-E, exact
    num = fma(ONE_FACTOR ? p1 : p1 * p2, cp, -d);
  }
  const double t = num * r;
  const float tf = d2f_trunc(t);
  const float r2 = fmaf(tf, fmaf(tf, fmaf(tf, -0.125f, 0.142857143f), -0.166666672f), 0.2f);
  double a = fma(t, f2d_scaled(r2, 0), -0.25);
  a = fma(t, a, 1.0 / 3.0);
  a = fma(t, a, -0.5);
  const double p = fma(t * t, a, t);  // log1p(t)
  if (near1) return p;
  const double edd = int_to_double(E);
  return fma(edd, kLn2Hi, T.logl[k]) + fma(edd, kLn2Lo, p);
}

// FP32 angle of (re + i im) for doubles of any magnitude (joint scaling by a
// power of two with integer instructions).
HG_HD __forceinline__ float arg_f32(double re, double im) {
  const int er = (int)((d2ll(re) >> 52) & 0x7ff);
  const int ei = (int)((d2ll(im) >> 52) & 0x7ff);
  const int e = er > ei ? er : ei;
  return atan2_f32(d2f_shift(im, e), d2f_shift(re, e));
}

}  // namespace lean
}  // namespace hg
