// Closed-form gravitational field of a right-rectangular prism, evaluated as a
// sum over EDGES (log terms) and FACES (arctangent terms) instead of the
// 8-vertex sum.  Device code for sm_103a (also compiles for the host, where
// the tests check it against the CPU oracle).
//
// Physics (Nagy, Papp & Benedek 2000, J. Geodesy 74:552, with the 2002
// corrections; the formulation harmonica cites at
// src/harmonica/_forward/prisms/gravity.py:160-164).  With vertex coordinates
// relative to the observation point, x_i = {w,e} - easting, y_j = {s,n} -
// northing, z_k = {b,t} - upward, r = |(x,y,z)| and the signed vertex sum
// |||F||| = sum_ijk s_i s_j s_k F(x_i,y_j,z_k)   (s = +1 upper, -1 lower bound),
// the kernel of the potential is
//   K = xy ln(z+r) + yz ln(x+r) + zx ln(y+r)
//       - x^2/2 atan(yz/(xr)) - y^2/2 atan(zx/(yr)) - z^2/2 atan(xy/(zr)),
// and potential, acceleration and tensor are G rho |||K|||,
// -G rho |||dK/dx_a||| and G rho |||d2K/dx_a dx_b|||.
//
// Regrouping the vertex sum: every log term ln(a + r) whose coefficient does
// not depend on a collapses, for each of the 4 edges parallel to axis a, into
// one EDGE LOG  L = ln(a_2 + r_2) - ln(a_1 + r_1) = ln(num/den);  every
// arctangent term whose coefficient depends only on the axis normal to a face
// collapses into one FACE ANGLE  O = sum_{b,c} s_b s_c atan(b c / (a r)).
// Where a field's coefficient is shared by two edges, their logs merge into
// one log of a product of ratios; so g_z needs 4 logs and 2 face angles per
// prism (the vertex sum needs 16 logs and 8 arctangents), and all ten fields
// together need 12 logs and 6 face angles.
//
// Conventions (gravity.py:141-158): potential and acceleration are finite
// everywhere (a log or angle multiplied by a zero coefficient contributes 0);
// tensor components are NaN on the singular edges and vertices of each
// component; diagonal tensor components on a face normal to their axis take
// the limit from outside the prism.
//
// LEAN = true uses the FP64-pipe-lean functions of lean_math.cuh; LEAN = false
// the generic library functions (same formulation, used as a cross-check).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#define HG_HD __host__ __device__

#include "lean_math.cuh"
#include "lean_packed.cuh"

namespace hg {

using lean::Tables;

HG_HD __forceinline__ long long bits_of(double v) { return lean::d2ll(v); }

HG_HD __forceinline__ double quiet_nan() { return lean::ll2d(0x7ff8000000000000LL); }

constexpr double kG = 6.6743e-11;  // harmonica constants.py:12
constexpr double kHalfPi = 1.5707963267948966;

enum Field : int {
  kPotential = 0, kGe = 1, kGn = 2, kGz = 3, kGee = 4, kGnn = 5, kGzz = 6,
  kGen = 7, kGez = 8, kGnz = 9, kNumFields = 10
};
constexpr int kAll = 10;  // fused evaluation of all ten fields

// Output multiplier per field: G, harmonica's sign flip for g_z/g_ez/g_nz and
// the SI -> mGal (1e5) / Eotvos (1e9) conversion (gravity.py:227-236),
// applied to sum_j rho_j * (signed edge/face combination) where the
// combination already carries the -1 of the first derivatives.
HG_HD inline double field_scale(int f) {
  switch (f) {
    case kPotential: return kG;
    case kGe: return -kG * 1e5;
    case kGn: return -kG * 1e5;
    case kGz: return kG * 1e5;  // -(-G): upward kernel negated to downward
    case kGee: case kGnn: case kGzz: case kGen: return kG * 1e9;
    case kGez: case kGnz: return -kG * 1e9;
    default: return 0.0;
  }
}

// ---------------------------------------------------------------------------
// bit-level predicates that stay off the FP64 pipe
HG_HD __forceinline__ bool is_zero(double v) { return (bits_of(v) << 1) == 0; }
HG_HD __forceinline__ bool is_neg(double v) { return bits_of(v) < 0 && !is_zero(v); }
HG_HD __forceinline__ bool is_nonpos(double v) { return bits_of(v) < 0 || is_zero(v); }
HG_HD __forceinline__ int sgn(double v) {
  return is_zero(v) ? 0 : (bits_of(v) < 0 ? -1 : 1);
}

// Predicates and sign operations on the high word only.  An exact test of all
// 64 bits for zero is compiled into an FP64 compare (a slow-pipe
// instruction); these stay integer.  is_tiny is true for zero AND subnormal
// values: used only where a subnormal length behaves as zero within rounding
// (the exact predicates above decide the singular points).
HG_HD __forceinline__ unsigned hi_word(double v) {
  return (unsigned)((unsigned long long)bits_of(v) >> 32);
}
HG_HD __forceinline__ bool is_tiny(double v) { return (hi_word(v) & 0x7ff00000u) == 0; }
HG_HD __forceinline__ bool sign_bit(double v) { return (int)hi_word(v) < 0; }
HG_HD __forceinline__ bool neg_not_tiny(double v) { return sign_bit(v) && !is_tiny(v); }
HG_HD __forceinline__ bool nonpos_or_tiny(double v) { return sign_bit(v) || is_tiny(v); }
constexpr long long kSignBit = (long long)0x8000000000000000ULL;
HG_HD __forceinline__ double flip_sign(double v) { return lean::ll2d(bits_of(v) ^ kSignBit); }
HG_HD __forceinline__ double abs_bits(double v) { return lean::ll2d(bits_of(v) & ~kSignBit); }
// v with its sign flipped where s is negative
HG_HD __forceinline__ double times_sign_of(double v, double s) {
  return lean::ll2d(bits_of(v) ^ (bits_of(s) & kSignBit));
}

// Multiply a log/angle by a coefficient, with the limit 0 * (singular) = 0.
HG_HD __forceinline__ double cmul(double coef, double v) { return is_tiny(coef) ? 0.0 : coef * v; }
// acc + coef * v with the same limit (one FMA)
HG_HD __forceinline__ double cfma(double coef, double v, double acc) {
  return fma(coef, is_tiny(coef) ? 0.0 : v, acc);
}
// acc + (NEG ? -coef : coef) * v: the sign folds into the FMA operand (a
// negated coefficient tested as bits would cost an FP64 negation)
template <bool NEG>
HG_HD __forceinline__ double cfma_s(double coef, double v, double acc) {
  const double w = is_tiny(coef) ? 0.0 : v;
  return NEG ? fma(-coef, w, acc) : fma(coef, w, acc);
}
// the same with a run-time sign, flipped on the bits
HG_HD __forceinline__ double cfma_xs(double coef, bool neg, double v, double acc) {
  const double w = is_tiny(coef) ? 0.0 : v;
  return fma(lean::ll2d(bits_of(coef) ^ (neg ? kSignBit : 0LL)), w, acc);
}
// the same with the sign as an argument (a constant after loop unrolling)
HG_HD __forceinline__ double cfma_sgn(double coef, bool neg, double v, double acc) {
  const double w = is_tiny(coef) ? 0.0 : v;
  return neg ? fma(-coef, w, acc) : fma(coef, w, acc);
}

template <bool LEAN> struct Math;
template <> struct Math<true> {
  static HG_HD __forceinline__ double sqrt_(double x) { return lean::lm_sqrt(x); }
  static HG_HD __forceinline__ double div_(double n, double d) { return lean::lm_div(n, d); }
  static HG_HD __forceinline__ double log_(double x, const Tables& T) { return lean::lm_log(x, T); }
};
template <> struct Math<false> {
  static HG_HD __forceinline__ double sqrt_(double x) { return sqrt(x); }
  static HG_HD __forceinline__ double div_(double n, double d) { return n / d; }
  static HG_HD __forceinline__ double log_(double x, const Tables&) { return log(x); }
};

// ---------------------------------------------------------------------------
// Observation-relative bounds of one (point, prism) pair, and the prism's
// extents (east - west, north - south, top - bottom: exact, not differences
// of the relative bounds).
struct Rel {
  double x1, x2, y1, y2, z1, z2;
  double dx, dy, dz;
};

// Singular-point predicates; they mirror choclo's
// is_point_on_{easting,northing,upward}_edge as used by gravity.py:272-449
// (closed intervals, so vertices are included).
HG_HD __forceinline__ bool on_e_edge(const Rel& q) {
  return (is_zero(q.y1) || is_zero(q.y2)) && (is_zero(q.z1) || is_zero(q.z2)) && is_nonpos(q.x1) &&
         !is_neg(q.x2);
}
HG_HD __forceinline__ bool on_n_edge(const Rel& q) {
  return (is_zero(q.x1) || is_zero(q.x2)) && (is_zero(q.z1) || is_zero(q.z2)) && is_nonpos(q.y1) &&
         !is_neg(q.y2);
}
HG_HD __forceinline__ bool on_u_edge(const Rel& q) {
  return (is_zero(q.x1) || is_zero(q.x2)) && (is_zero(q.y1) || is_zero(q.y2)) && is_nonpos(q.z1) &&
         !is_neg(q.z2);
}
HG_HD __forceinline__ bool singular_for(int f, const Rel& q) {
  switch (f) {
    case kGee: return on_n_edge(q) || on_u_edge(q);
    case kGnn: return on_e_edge(q) || on_u_edge(q);
    case kGzz: return on_e_edge(q) || on_n_edge(q);
    case kGen: return on_u_edge(q);
    case kGez: return on_n_edge(q);
    case kGnz: return on_e_edge(q);
    default: return false;
  }
}

// ---------------------------------------------------------------------------
// Geometry shared by all terms: squares and the 8 vertex distances.
struct Geom {
  double x[2], y[2], z[2];
  double x2[2], y2[2], z2[2];
  double xz2[2][2];   // x_i^2 + z_k^2 (also the squared distance from y-edges)
  double r[2][2][2];  // r[i][j][k]
};

template <bool LEAN>
HG_HD __forceinline__ void make_geom(const Rel& q, Geom& g) {
  g.x[0] = q.x1; g.x[1] = q.x2;
  g.y[0] = q.y1; g.y[1] = q.y2;
  g.z[0] = q.z1; g.z[1] = q.z2;
#pragma unroll
  for (int a = 0; a < 2; a++) {
    g.x2[a] = g.x[a] * g.x[a];
    g.y2[a] = g.y[a] * g.y[a];
    g.z2[a] = g.z[a] * g.z[a];
  }
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int k = 0; k < 2; k++) g.xz2[i][k] = g.x2[i] + g.z2[k];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int k = 0; k < 2; k++) g.r[i][j][k] = Math<LEAN>::sqrt_(g.xz2[i][k] + g.y2[j]);
}

// ---------------------------------------------------------------------------
// Edge ratio along one axis: (a2 + r2) / (a1 + r1) = num / den, with a1 <= a2
// the observation-relative coordinates of the edge ends, r1, r2 their
// distances and rho2 the squared distance from the edge line, without
// cancellation:
//  * a2 <= 0: reflect a -> -a (the ratio is invariant) so that the upper end
//    is non-negative;
//  * lower end negative (the point projects inside the edge): use
//    (a1 + r1) = rho2 / (r1 - a1).
// The case depends only on the point's coordinate relative to the prism along
// this axis, so it is shared by the axis' 4 edges.
struct AxisCase {
  bool reflect;   // a2 <= 0
  bool straddle;  // after reflection, lower end < 0
};

HG_HD __forceinline__ AxisCase axis_case(double a1, double a2) {
  AxisCase c;
  c.reflect = nonpos_or_tiny(a2);
  c.straddle = neg_not_tiny(c.reflect ? flip_sign(a2) : a1);
  return c;
}

// Ratio terms of one edge before the straddle case: num = hi + r_hi and
// den = |lo| + r_lo (lo + r_lo, or r_lo - lo when lo < 0).
HG_HD __forceinline__ void edge_ratio(AxisCase c, double a1, double a2, double r1, double r2,
                                      double& num, double& den) {
  const double lo = c.reflect ? flip_sign(a2) : a1;
  const double hi = c.reflect ? flip_sign(a1) : a2;
  const double rlo = c.reflect ? r2 : r1;
  const double rhi = c.reflect ? r1 : r2;
  den = fabs(lo) + rlo;
  num = hi + rhi;
}

// The 4 edges parallel to one axis, indexed [p][s] by the other two axes in
// (x, y, z) order.
struct EdgeSet {
  double num[2][2], den[2][2];
};

// Straddle case of an axis (the point projects inside its edges):
// num / den = (hi + r_hi)(r_lo - lo) / rho2.  Taken as a branch: the point
// straddles few prisms, so most warps skip these products.
HG_HD __forceinline__ void straddle_fix(EdgeSet& E, const double rho2[2][2]) {
#pragma unroll
  for (int p = 0; p < 2; p++)
#pragma unroll
    for (int s = 0; s < 2; s++) {
      E.num[p][s] *= E.den[p][s];
      E.den[p][s] = rho2[p][s];
    }
}

// edges along x at (y_j, z_k)
HG_HD __forceinline__ void edges_x(const Geom& g, EdgeSet& E) {
  const AxisCase c = axis_case(g.x[0], g.x[1]);
#pragma unroll
  for (int j = 0; j < 2; j++)
#pragma unroll
    for (int k = 0; k < 2; k++)
      edge_ratio(c, g.x[0], g.x[1], g.r[0][j][k], g.r[1][j][k], E.num[j][k], E.den[j][k]);
  if (c.straddle) {
    double rho2[2][2];
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int k = 0; k < 2; k++) rho2[j][k] = g.y2[j] + g.z2[k];
    straddle_fix(E, rho2);
  }
}
// edges along y at (x_i, z_k)
HG_HD __forceinline__ void edges_y(const Geom& g, EdgeSet& E) {
  const AxisCase c = axis_case(g.y[0], g.y[1]);
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int k = 0; k < 2; k++)
      edge_ratio(c, g.y[0], g.y[1], g.r[i][0][k], g.r[i][1][k], E.num[i][k], E.den[i][k]);
  if (c.straddle) straddle_fix(E, g.xz2);
}
// edges along z at (x_i, y_j)
HG_HD __forceinline__ void edges_z(const Geom& g, EdgeSet& E) {
  const AxisCase c = axis_case(g.z[0], g.z[1]);
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++)
      edge_ratio(c, g.z[0], g.z[1], g.r[i][j][0], g.r[i][j][1], E.num[i][j], E.den[i][j]);
  if (c.straddle) {
    double rho2[2][2];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++) rho2[i][j] = g.x2[i] + g.y2[j];
    straddle_fix(E, rho2);
  }
}

// ln(R_a / R_b) with R = num / den: the difference of two edge logs as one log.
template <bool LEAN>
HG_HD __forceinline__ double log_ratio2(double na, double da, double nb, double db,
                                        const Tables& T) {
  if (LEAN) return lean::lm_log_quot<false>(na, db, da, nb, T);
  return log((na * db) / (da * nb));
}
template <bool LEAN>
HG_HD __forceinline__ double log_ratio1(double n, double d, const Tables& T) {
  if (LEAN) return lean::lm_log_quot<true>(n, 1.0, d, 1.0, T);
  return log(n / d);
}
// ln((p1 p2) / (q1 q2))
template <bool LEAN>
HG_HD __forceinline__ double log_quot(double p1, double p2, double q1, double q2,
                                      const Tables& T) {
  if (LEAN) return lean::lm_log_quot<false>(p1, p2, q1, q2, T);
  return log((p1 * p2) / (q1 * q2));
}

// ---------------------------------------------------------------------------
// Face angle for the face at (normal coordinate) a, with in-plane coordinates
// b_1 < b_2, c_1 < c_2 and vertex distances r_bc:
//   O = sum_{b,c} s_b s_c atan(b c / (a r)).
// For a != 0, atan(bc/(ar)) = sign(a) arg(|a| r + i bc) with a positive real
// part, so each pair of vertices along b is an argument difference in
// (-pi, pi) and equals the argument of one complex product:
//   arg(c_2c) - arg(c_1c) = arg((|a| r_2c + i b2 c)(|a| r_1c - i b1 c))
//     = atan2(|a| c (b2 r_1c - b1 r_2c), a^2 r_1c r_2c + b1 b2 c^2).
// For a distant face b2 r_1c - b1 r_2c cancels; when b1, b2 have one sign it
// is rewritten without cancellation as
//   (b2 - b1)(b2 + b1)(a^2 + c^2) / (b2 r_1c + b1 r_2c)
// and the positive denominator is moved into the real part (the argument is
// invariant under scaling by a positive number).  The face angle is then
// arg A - arg B of the two pair products, evaluated as one argument of
// A conj(B) on the branch selected by an FP32 estimate.
// For a == 0 the value is the limit from outside the prism:
// a -> 0+ for the lower face (upper == false), a -> 0- for the upper face.
HG_HD __forceinline__ void pair_complex(double aa, double asq, double b1, double b2, double c,
                                        double csq, double r1, double r2, bool same_sign,
                                        double bdiff, double& re, double& im) {
  re = asq * (r1 * r2) + (b1 * b2) * csq;
  double d;
  if (same_sign) {
    double den = b2 * r1 + b1 * r2;  // one sign, no cancellation
    d = bdiff * (asq + csq);         // bdiff = (b2 - b1)(b2 + b1)
    if (is_neg(den)) {
      den = -den;
      d = -d;
    }
    re *= den;
  } else {
    d = b2 * r1 - b1 * r2;  // b1 < 0 < b2: both terms positive
  }
  im = aa * c * d;
}

// Scales the complex number (re, im) by a power of two so that its larger
// component is in [1, 2) (zero stays zero).
HG_HD __forceinline__ void normalize_f2c(lean::F2& re, lean::F2& im) {
  using namespace lean;
  const int er = (int)((f2u(re.h) >> 23) & 0xffu), ei = (int)((f2u(im.h) >> 23) & 0xffu);
  const int e = er > ei ? er : ei;
  const float sc = u2f((unsigned)(254 - (e > 253 ? 253 : e)) << 23);  // 2^(127 - e)
  re.h = fmul(re.h, sc);
  re.l = fmul(re.l, sc);
  im.h = fmul(im.h, sc);
  im.l = fmul(im.l, sc);
}

// The same pair products on float pairs, for lengths scaled by a power of
// two so that every product stays in the float range; bdq = bdiff (a^2+c^2).
HG_HD __forceinline__ void pair_complex_f2(lean::F2 aa, lean::F2 asq, lean::F2 b1, lean::F2 b2,
                                           lean::F2 c, lean::F2 csq, lean::F2 r1, lean::F2 r2,
                                           bool same_sign, lean::F2 bdq, lean::F2& re,
                                           lean::F2& im) {
  using namespace lean;
  re = f2_add(f2_mul(asq, f2_mul(r1, r2)), f2_mul(f2_mul(b1, b2), csq));
  // same sign: den = b2 r1 + b1 r2 (one sign); straddle: d = b2 r1 - b1 r2
  F2 x = f2_add(f2_mul(b2, r1), f2_mul(same_sign ? b1 : f2_neg(b1), r2));
  F2 d = x;
  if (same_sign) {
    d = bdq;
    if (x.h < 0.0f) {
      x = f2_neg(x);
      d = f2_neg(d);
    }
    re = f2_mul(re, x);
  }
  im = f2_mul(f2_mul(aa, c), d);
}

// Face angle on float pairs, inputs already float pairs at a common scale
// where the largest of the face's vertex distances is in [1, 2): |a| (the
// caller applies the sign of a), the in-plane coordinates, the four vertex
// distances and the width b2 - b1 (given separately: no cancellation).
// A and B are each scaled by a power of two before the product A conj(B).
HG_HD __forceinline__ lean::F2 face_core_f2(lean::F2 fa, lean::F2 fb1, lean::F2 fb2,
                                            lean::F2 fc1, lean::F2 fc2, lean::F2 fr11,
                                            lean::F2 fr12, lean::F2 fr21, lean::F2 fr22,
                                            lean::F2 fw, bool same_sign, const Tables& T) {
  using namespace lean;
  F2 asq = two_prod(fa.h, fa.h);
  asq.l = ffma(2.0f * fa.h, fa.l, asq.l);
  F2 c1sq = two_prod(fc1.h, fc1.h), c2sq = two_prod(fc2.h, fc2.h);
  c1sq.l = ffma(2.0f * fc1.h, fc1.l, c1sq.l);
  c2sq.l = ffma(2.0f * fc2.h, fc2.l, c2sq.l);
  F2 bdq1{0.0f, 0.0f}, bdq2{0.0f, 0.0f};
  if (same_sign) {
    // bdiff = (b2 - b1)(b2 + b1): the width from the caller, the same-sign sum
    const F2 fbd = f2_mul(fw, f2_add(fb2, fb1));
    bdq1 = f2_mul(fbd, f2_add(asq, c1sq));
    bdq2 = f2_mul(fbd, f2_add(asq, c2sq));
  }
  F2 ar, ai, br, bi;
  pair_complex_f2(fa, asq, fb1, fb2, fc2, c2sq, fr12, fr22, same_sign, bdq2, ar, ai);
  pair_complex_f2(fa, asq, fb1, fb2, fc1, c1sq, fr11, fr21, same_sign, bdq1, br, bi);
  normalize_f2c(ar, ai);
  normalize_f2c(br, bi);
  const float est = atan2_est(ai.h, ar.h) - atan2_est(bi.h, br.h);
  const F2 pr = f2_add(f2_mul(ar, br), f2_mul(ai, bi));
  const F2 pim = f2_add(f2_mul(ai, br), f2_neg(f2_mul(ar, bi)));
  return lm_arg_near_f2(pr, pim, est, T);
}

// Face angle from FP64 inputs: every length is scaled by 2^-s, s the
// exponent of the largest vertex distance of the face (the distances bound
// all coordinates).  Returns false (and leaves o) when a nonzero coordinate
// or the face width is below 2^-16 of that scale: then a product of up to six
// scaled lengths could leave the normal float range, and the caller takes the
// FP64 path (a point within ~1e-5 face sizes of an edge line or face plane).
HG_HD __forceinline__ bool face_angle_f2(double a, double b1, double b2, double c1, double c2,
                                         double r11, double r12, double r21, double r22,
                                         bool same_sign, double width, const Tables& T,
                                         double& o) {
  using namespace lean;
  const auto ex = [](double v) { return (int)((hi_word(v) >> 20) & 0x7ffu); };
  int top = ex(r11);
  top = max(top, ex(r12));
  top = max(top, ex(r21));
  top = max(top, ex(r22));
  const int lim = top - 16;
  const auto small = [&](double v) { return !is_tiny(v) && ex(v) < lim; };
  if (small(a) || small(b1) || small(b2) || small(c1) || small(c2) || top >= 0x7fe ||
      ex(width) < lim)
    return false;
  const auto f = [&](double v) { return scaled_f2(d2ll(v), top); };
  o = f2_to_double(face_core_f2(f(abs_bits(a)), f(b1), f(b2), f(c1), f(c2), f(r11), f(r12),
                                f(r21), f(r22), f(width), same_sign, T),
                   0);
  return true;
}

// The face angle in FP64 for the faces the float-pair path declines (kept
// out of line: rarely executed).  Same pair products and argument as
// face_angle_f2; |o| for a > 0.
// O = [arg c_{2,c2} - arg c_{1,c2}] - [arg c_{2,c1} - arg c_{1,c1}] = arg A - arg B
HG_COLD double face_angle_fp64(double a, double b1, double b2, double c1, double c2, double r11,
                               double r12, double r21, double r22, bool same_sign, double width,
                               const Tables& T) {
  const double bdiff = width * (b2 + b1);
  const double aa = fabs(a);
  const double asq = a * a;
  double ar, ai, br, bi;
  pair_complex(aa, asq, b1, b2, c2, c2 * c2, r12, r22, same_sign, bdiff, ar, ai);
  pair_complex(aa, asq, b1, b2, c1, c1 * c1, r11, r21, same_sign, bdiff, br, bi);
  const float est = lean::arg_f32(ar, ai) - lean::arg_f32(br, bi);
  const double pr = fma(ar, br, ai * bi);
  const double pim = fma(ai, br, -(ar * bi));
  return lean::lm_arg_near(pr, pim, est, T);
}

// width = b2 - b1 (shared by the two faces normal to one axis).
template <bool LEAN>
HG_HD __forceinline__ double face_angle(double a, bool upper, double b1, double b2, double c1,
                                        double c2, double r11, double r12, double r21, double r22,
                                        double width, const Tables& T) {
  if (is_tiny(a)) {
    int s = sgn(b2) * sgn(c2) + sgn(b1) * sgn(c1) - sgn(b1) * sgn(c2) - sgn(b2) * sgn(c1);
    return (upper ? -kHalfPi : kHalfPi) * (double)s;
  }
  const bool same_sign = !(neg_not_tiny(b1) && !nonpos_or_tiny(b2));
  double o;
  if (LEAN) {
    if (!face_angle_f2(a, b1, b2, c1, c2, r11, r12, r21, r22, same_sign, width, T, o))
      o = face_angle_fp64(a, b1, b2, c1, c2, r11, r12, r21, r22, same_sign, width, T);
    return times_sign_of(o, a);
  }
  const double bdiff = width * (b2 + b1);
  double ar, ai, br, bi;
  pair_complex(fabs(a), a * a, b1, b2, c2, c2 * c2, r12, r22, same_sign, bdiff, ar, ai);
  pair_complex(fabs(a), a * a, b1, b2, c1, c1 * c1, r11, r21, same_sign, bdiff, br, bi);
  o = atan2(ai, ar) - atan2(bi, br);
  return times_sign_of(o, a);
}

// ---------------------------------------------------------------------------
// Rolled evaluation.  The float-pair face angle is ~1000 instructions and a
// merged log ~300; inlined once per face or log they make a loop body larger
// than the instruction cache (warps then stall on instruction fetch).  The
// helpers below evaluate the faces and logs in loops that are not unrolled,
// with the per-iteration inputs chosen by selects (registers only), so the
// kernel holds one copy of each.

// Inputs of the face normal to `axis` (0 = x, 1 = y, 2 = z) at bound k:
// x faces: b = y, c = z; y faces: b = x, c = z; z faces: b = x, c = y.
struct FaceIn {
  double a, b1, b2, c1, c2, r11, r12, r21, r22, width;
};
HG_HD __forceinline__ FaceIn face_in(const Geom& g, int axis, bool k) {
  const bool X = axis == 0, Y = axis == 1;
  FaceIn f;
  f.a = X ? (k ? g.x[1] : g.x[0]) : (Y ? (k ? g.y[1] : g.y[0]) : (k ? g.z[1] : g.z[0]));
  f.b1 = X ? g.y[0] : g.x[0];
  f.b2 = X ? g.y[1] : g.x[1];
  f.c1 = (X || Y) ? g.z[0] : g.y[0];
  f.c2 = (X || Y) ? g.z[1] : g.y[1];
  // r_{b c}: index of the vertex distance for in-plane corners (b_i, c_j)
  const auto r = [&](int bi, int cj) {
    const double rx = k ? g.r[1][bi][cj] : g.r[0][bi][cj];  // x face: r[k][b][c]
    const double ry = k ? g.r[bi][1][cj] : g.r[bi][0][cj];  // y face: r[b][k][c]
    const double rz = k ? g.r[bi][cj][1] : g.r[bi][cj][0];  // z face: r[b][c][k]
    return X ? rx : (Y ? ry : rz);
  };
  f.r11 = r(0, 0);
  f.r12 = r(0, 1);
  f.r21 = r(1, 0);
  f.r22 = r(1, 1);
  f.width = X ? g.y[1] - g.y[0] : g.x[1] - g.x[0];
  return f;
}

template <bool LEAN>
HG_HD __forceinline__ double face_of(const Geom& g, int axis, bool k, const Tables& T) {
  const FaceIn f = face_in(g, axis, k);
  return face_angle<LEAN>(f.a, k, f.b1, f.b2, f.c1, f.c2, f.r11, f.r12, f.r21, f.r22, f.width,
                          T);
}

// The two faces normal to AXIS: o0 at the lower bound, o1 at the upper.
template <int AXIS, bool LEAN>
HG_HD __forceinline__ void faces2(const Geom& g, const Tables& T, double& o0, double& o1) {
  o0 = 0.0;
  o1 = 0.0;
#pragma unroll 1
  for (int k = 0; k < 2; k++) {
    const double o = face_of<LEAN>(g, AXIS, k, T);
    o0 = k ? o0 : o;
    o1 = k ? o : o1;
  }
}

// acc + sum_k (k ? -c1 : c0) O_k over the two faces normal to AXIS, the
// product accumulated inside the loop (c0, c1 the face coefficients before
// the -s_k sign: -s_0 = +1, -s_1 = -1).
template <int AXIS, bool LEAN>
HG_HD __forceinline__ double faces2_dot(const Geom& g, double c0, double c1, const Tables& T,
                                        double acc) {
#pragma unroll 1
  for (int k = 0; k < 2; k++) {
    const double o = face_of<LEAN>(g, AXIS, k, T);
    acc = cfma_xs(k ? c1 : c0, k, o, acc);
  }
  return acc;
}

// All six faces, O[axis][k].
template <bool LEAN>
HG_HD __forceinline__ void faces6(const Geom& g, const Tables& T, double O[3][2]) {
#pragma unroll
  for (int a = 0; a < 3; a++) O[a][0] = O[a][1] = 0.0;
#pragma unroll 1
  for (int f = 0; f < 6; f++) {
    const int axis = f >> 1;
    const bool k = f & 1;
    const double o = face_of<LEAN>(g, axis, k, T);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      O[a][0] = (axis == a && !k) ? o : O[a][0];
      O[a][1] = (axis == a && k) ? o : O[a][1];
    }
  }
}

// Single edge logs of one axis, L[p][s] = ln(num/den), for the three axes in
// one rolled loop: Lx from Ex, Ly from Ey, Lz from Ez.
template <bool LEAN>
HG_HD __forceinline__ void logs12(const EdgeSet& Ex, const EdgeSet& Ey, const EdgeSet& Ez,
                                  const Tables& T, double Lx[2][2], double Ly[2][2],
                                  double Lz[2][2]) {
#pragma unroll
  for (int p = 0; p < 2; p++)
#pragma unroll
    for (int q = 0; q < 2; q++) Lx[p][q] = Ly[p][q] = Lz[p][q] = 0.0;
#pragma unroll 1
  for (int axis = 0; axis < 3; axis++) {
    const bool X = axis == 0, Y = axis == 1;
#pragma unroll
    for (int p = 0; p < 2; p++)
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const double n = X ? Ex.num[p][q] : (Y ? Ey.num[p][q] : Ez.num[p][q]);
        const double d = X ? Ex.den[p][q] : (Y ? Ey.den[p][q] : Ez.den[p][q]);
        const double l = log_ratio1<LEAN>(n, d, T);
        Lx[p][q] = X ? l : Lx[p][q];
        Ly[p][q] = Y ? l : Ly[p][q];
        Lz[p][q] = (!X && !Y) ? l : Lz[p][q];
      }
  }
}

// sum over the 4 merged logs  c_m ln(R_{m,1} / R_{m,0})  of two edge sets,
// m = 0, 1 from E0 (coefficients e0_0, e0_1) and m = 2, 3 from E1, with the
// ratio pair of entry m at [idx(m)][1] over [idx(m)][0] (T0 = false) or
// [1][idx(m)] over [0][idx(m)] (T0 = true; likewise T1 for E1); the
// coefficient signs are -, +, -, + (s_0 = -1, s_1 = +1).
template <bool LEAN, bool T0, bool T1>
HG_HD __forceinline__ double merged_logs4(const EdgeSet& E0, const EdgeSet& E1, double c00,
                                          double c01, double c10, double c11, const Tables& T,
                                          double acc) {
#pragma unroll 1
  for (int m = 0; m < 4; m++) {
    const bool b = m & 1, second = m >= 2;
    const auto pick = [&](const double (&A)[2][2], const double (&B)[2][2], bool hi) {
      const double a0 = T0 ? A[hi][0] : A[0][hi], a1 = T0 ? A[hi][1] : A[1][hi];
      const double b0 = T1 ? B[hi][0] : B[0][hi], b1 = T1 ? B[hi][1] : B[1][hi];
      return second ? (b ? b1 : b0) : (b ? a1 : a0);
    };
    const double n1 = pick(E0.num, E1.num, true), d1 = pick(E0.den, E1.den, true);
    const double n0 = pick(E0.num, E1.num, false), d0 = pick(E0.den, E1.den, false);
    const double coef = second ? (b ? c11 : c10) : (b ? c01 : c00);
    acc = cfma_xs(coef, !b, log_ratio2<LEAN>(n1, d1, n0, d0, T), acc);
  }
  return acc;
}

// ---------------------------------------------------------------------------
// g_z of one pair on float pairs.
//
// Every length of the pair is scaled by 2^-s (s: the exponent of its largest
// coordinate) and held as a float pair; vertex distances by float-pair square
// roots; the four merged edge logs from cancellation-free numerators
// (merged_t); the two face angles by face_core_f2; the combination summed on
// pairs and returned as a double (integer assembly).  No FP64 instruction on
// this path.  Pairs whose scaled geometry could leave the float range (a
// nonzero coordinate below 2^-40 of the scale, a vertex distance or extent
// below 2^-20, a face coordinate below 2^-16 of its face) take the FP64 path.

// t = R(u1) / R(u0) - 1 for the merged log of the two edges parallel to one
// axis at in-plane offset v, at u0 and u1 = u0 + du (su = u0 + u1), with edge
// ends lo < hi after reflection (lo < 0 only when the point projects inside
// the edge) and vertex distances rl0 = r(lo, u0), rl1 = r(lo, u1), rh0, rh1.
// With dQ = u1^2 - u0^2 = du su, Dl = dQ / (rl1 + rl0) = rl1 - rl0, Dh
// likewise, P_k = rl_k + rh_k, Sl = rl0 + rl1, Sh = rh0 + rh1:
//   lo >= 0: R = (hi + rh)/(lo + rl), D = lo + rl, N = hi + rh,
//       t = -dA [Dl + (hi + lo)(D0 (Dl + Dh) + Dl P1) / (P0 P1)] / (D1 N0)
//   lo < 0:  R = (hi + rh)(rl - lo)/(v^2 + u^2), M = rl - lo,
//       X = rh0 Dl - rl0 Dh - hi Sl + lo Sh,
//       t = dQ M1 X / (Sh Sl M0 (v^2 + u1^2))
// (both follow from expanding N1 D0 - D1 N0, resp. the products, in the
// differences Dl, Dh).  Every sum adds terms of one sign, so t keeps its
// relative accuracy however far the prism is; the direct numerator
// N1 D0 - D1 N0 loses it with the square of the distance.
HG_HD __forceinline__ lean::F2 merged_t(bool straddle, lean::F2 lo, lean::F2 hi, lean::F2 v,
                                        lean::F2 u1, lean::F2 rl0, lean::F2 rl1, lean::F2 rh0,
                                        lean::F2 rh1, lean::F2 dA, lean::F2 du, lean::F2 su) {
  using namespace lean;
  const F2 dQ = f2_mul(du, su);
  const F2 Sl = f2_add(rl0, rl1), Sh = f2_add(rh0, rh1);
  const F2 Dl = f2_div(dQ, Sl), Dh = f2_div(dQ, Sh);
  if (!straddle) {
    const F2 D0 = f2_add(lo, rl0), D1 = f2_add(lo, rl1), N0 = f2_add(hi, rh0);
    const F2 P0 = f2_add(rl0, rh0), P1 = f2_add(rl1, rh1);
    const F2 inner = f2_add(f2_mul(D0, f2_add(Dl, Dh)), f2_mul(Dl, P1));
    const F2 br = f2_add(Dl, f2_div(f2_mul(f2_add(hi, lo), inner), f2_mul(P0, P1)));
    return f2_neg(f2_div(f2_mul(dA, br), f2_mul(D1, N0)));
  }
  const F2 M0 = f2_sub(rl0, lo), M1 = f2_sub(rl1, lo);
  const F2 Q1 = f2_add(f2_sq(v), f2_sq(u1));
  const F2 X = f2_add(f2_add(f2_mul(rh0, Dl), f2_neg(f2_mul(rl0, Dh))),
                      f2_add(f2_neg(f2_mul(hi, Sl)), f2_mul(lo, Sh)));
  return f2_div(f2_mul(f2_mul(dQ, M1), X), f2_mul(f2_mul(Sh, Sl), f2_mul(M0, Q1)));
}

// Float-pair geometry of one pair: every length scaled by 2^(1023 - top),
// top the largest biased exponent of the six observation-relative bounds.
struct GeomF2 {
  lean::F2 c[3][2];     // bounds c[axis][0 lower, 1 upper]
  lean::F2 d[3];        // extents
  lean::F2 r[2][2][2];  // vertex distances r[i][j][k]
  int top;
};

HG_HD __forceinline__ double rel_bound(const Rel& q, int axis, int k) {
  return axis == 0 ? (k ? q.x2 : q.x1) : (axis == 1 ? (k ? q.y2 : q.y1) : (k ? q.z2 : q.z1));
}

// false: the scaled geometry could leave the float range (a nonzero bound
// below 2^-40 of the scale, an extent or a vertex distance below 2^-20);
// the pair then takes the FP64 path.
HG_HD __forceinline__ bool make_geom_f2(const Rel& q, GeomF2& g) {
  using namespace lean;
  const auto ex = [](double v) { return (int)((hi_word(v) >> 20) & 0x7ffu); };
  const int top =
      max(max(ex(q.x1), ex(q.x2)), max(max(ex(q.y1), ex(q.y2)), max(ex(q.z1), ex(q.z2))));
  // a nonzero bound below 2^-40 of the scale: 1 <= ef < top - 40, one
  // unsigned compare (zero and subnormal bounds have ef = 0)
  const unsigned lim = (unsigned)(top - 41);
  const auto tiny_nz = [&](double v) { return (unsigned)(ex(v) - 1) < lim; };
  if (top >= 0x7fe || tiny_nz(q.x1) || tiny_nz(q.x2) || tiny_nz(q.y1) || tiny_nz(q.y2) ||
      tiny_nz(q.z1) || tiny_nz(q.z2) || ex(q.dx) < top - 20 || ex(q.dy) < top - 20 ||
      ex(q.dz) < top - 20)
    return false;
  const auto f = [&](double v) { return scaled_f2_near(d2ll(v), top); };
  g.top = top;
  g.c[0][0] = f(q.x1);
  g.c[0][1] = f(q.x2);
  g.c[1][0] = f(q.y1);
  g.c[1][1] = f(q.y2);
  g.c[2][0] = f(q.z1);
  g.c[2][1] = f(q.z2);
  g.d[0] = f(q.dx);
  g.d[1] = f(q.dy);
  g.d[2] = f(q.dz);
  // squares and vertex distances two at a time (lanes: lower/upper bound)
  P2 sq[3];
#pragma unroll
  for (int a = 0; a < 3; a++) sq[a] = p2_sq(pk(g.c[a][0], g.c[a][1]));
  const F2 xs[2] = {lane0(sq[0]), lane1(sq[0])}, ys[2] = {lane0(sq[1]), lane1(sq[1])};
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const P2 xz = p2_add(pk(xs[i], xs[i]), sq[2]);  // x_i^2 + z_k^2, lanes k
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const P2 r = p2_sqrt(p2_add(xz, pk(ys[j], ys[j])));
      g.r[i][j][0] = lane0(r);
      g.r[i][j][1] = lane1(r);
      ok = ok && r.h.x >= 0x1p-20f && r.h.y >= 0x1p-20f;
    }
  }
  return ok;
}

// A sufficient test that no face of the pair declines the float-pair scale
// (face_pair_core_p2): every bound and extent within 2^14 of the largest
// bound (the face inputs must be within 2^16 of the face's largest vertex
// distance, itself below 4 x the largest bound).  The kernels that evaluate
// the edge and face parts in two launches take the FP64 path for the pairs
// that fail it, in the edge launch, and skip them in the face launch.
HG_HD __forceinline__ bool faces_fit_f2(const GeomF2& g) {
  using namespace lean;
  const auto fe = [](F2 a) { return (int)((f2u(a.h) >> 23) & 0xffu); };
  int m = min(fe(g.d[0]), min(fe(g.d[1]), fe(g.d[2])));
#pragma unroll
  for (int a = 0; a < 3; a++) m = min(m, min(fe(g.c[a][0]), fe(g.c[a][1])));
  return m >= 127 - 14;
}

// Outside limit of a face angle for a point in the face plane (face_angle):
// (upper ? -pi/2 : pi/2) * (sgn products), out of line (rare).
HG_COLD lean::F2 face_limit_f2(double b1, double b2, double c1, double c2, bool upper) {
  const int s = sgn(b2) * sgn(c2) + sgn(b1) * sgn(c1) - sgn(b1) * sgn(c2) - sgn(b2) * sgn(c1);
  const float sf = (float)(upper ? -s : s);
  return lean::F2{lean::fmul(1.57079637f, sf), lean::fmul(-4.37113883e-8f, sf)};
}

// same_sign: the in-plane b bounds have one sign (pair_complex), from the
// caller (shared by the two faces).
template <int U>
HG_HD __forceinline__ bool face_f2(const Rel& q, const GeomF2& g, bool k, bool same_sign,
                                   const Tables& T, lean::F2& o) {
  using namespace lean;
  constexpr int B = U == 0 ? 1 : 0, C = U == 2 ? 1 : 2;
  // r at in-plane corner (bi, ci) of the face at bound k (2-way select)
  const auto idx = [&](int bi, int ci) {
    int i0[3], i1[3];
    i0[U] = 0;
    i1[U] = 1;
    i0[B] = i1[B] = bi;
    i0[C] = i1[C] = ci;
    return k ? g.r[i1[0]][i1[1]][i1[2]] : g.r[i0[0]][i0[1]][i0[2]];
  };
  if (is_tiny(rel_bound(q, U, k))) {
    o = face_limit_f2(rel_bound(q, B, 0), rel_bound(q, B, 1), rel_bound(q, C, 0),
                      rel_bound(q, C, 1), k);
    return true;
  }
  const F2 r11 = idx(0, 0), r12 = idx(0, 1), r21 = idx(1, 0), r22 = idx(1, 1);
  const auto fe = [](F2 a) { return (int)((f2u(a.h) >> 23) & 0xffu); };
  const int ftop = max(max(fe(r11), fe(r12)), max(fe(r21), fe(r22)));
  const auto fsmall = [&](F2 a) { return a.h != 0.0f && fe(a) < ftop - 16; };
  const F2 a = k ? g.c[U][1] : g.c[U][0];
  if (fsmall(a) || fsmall(g.c[B][0]) || fsmall(g.c[B][1]) || fsmall(g.c[C][0]) ||
      fsmall(g.c[C][1]) || fe(g.d[B]) < ftop - 16)
    return false;
  const float sc = pow2f(127 - ftop);
  const auto h = [&](F2 v) { return F2{fmul(v.h, sc), fmul(v.l, sc)}; };
  const bool neg = a.h < 0.0f;
  o = face_core_f2(h(neg ? f2_neg(a) : a), h(g.c[B][0]), h(g.c[B][1]), h(g.c[C][0]),
                   h(g.c[C][1]), h(r11), h(r12), h(r21), h(r22), h(g.d[B]), same_sign, T);
  if (neg) o = f2_neg(o);
  return true;
}

// First derivative along axis U (U = 2: g_z, 0: g_e, 1: g_n combinations) on
// float pairs:
//   sum over the two edge families (A, V) of sum_a s_a v_a ln(R(u_1)/R(u_0))
//   - sum_k s_k u_k O_k
// where the family's edges are parallel to A at V-bound v_a and the merged
// log pairs them along U (merged_t); s_0 = -1, s_1 = +1.  Families:
// U = z: (A = y, V = x), (A = x, V = y); U = x: (A = z, V = y), (A = y, V = z);
// U = y: (A = x, V = z), (A = z, V = x).  With o_faces, the two face angles
// O_0, O_1 are returned as well (adjoint).  false: FP64 path.
template <int U>
HG_HD __forceinline__ bool pair_grad_f2(const Rel& q, const Tables& T, double& out,
                                        double* o_faces) {
  using namespace lean;
  GeomF2 g;
  if (!make_geom_f2(q, g)) return false;
  constexpr int A0 = U == 2 ? 1 : (U == 0 ? 2 : 0), V0 = 3 - U - A0;  // first family
  const AxisCase case0 = axis_case(rel_bound(q, A0, 0), rel_bound(q, A0, 1));
  const AxisCase case1 = axis_case(rel_bound(q, V0, 0), rel_bound(q, V0, 1));  // second: A = V0
  const F2 su = f2_add(g.c[U][0], g.c[U][1]);
  F2 v{0.0f, 0.0f};
#pragma unroll 1
  for (int m = 0; m < 4; m++) {
    const bool b = m & 1, second = m >= 2;
    const AxisCase c = second ? case1 : case0;
    const F2 a1 = second ? g.c[V0][0] : g.c[A0][0], a2 = second ? g.c[V0][1] : g.c[A0][1];
    const F2 lo = c.reflect ? f2_neg(a2) : a1, hi = c.reflect ? f2_neg(a1) : a2;
    // r of the vertex at A-end `end` (compile time), V-bound b, U-bound eu:
    // family 0 indexes (A0 = end, V0 = b), family 1 (V0 = end, A0 = b)
    const auto rv = [&](int end, int eu) {
      const auto at = [&](int ia, int iv) {
        int id[3] = {0, 0, 0};
        id[A0] = ia;
        id[V0] = iv;
        id[U] = eu;
        return g.r[id[0]][id[1]][id[2]];
      };
      const F2 f0 = b ? at(end, 1) : at(end, 0);
      const F2 f1 = b ? at(1, end) : at(0, end);
      return second ? f1 : f0;
    };
    const bool il = c.reflect;  // A-end of lo
    const F2 rl0 = il ? rv(1, 0) : rv(0, 0), rl1 = il ? rv(1, 1) : rv(0, 1);
    const F2 rh0 = il ? rv(0, 0) : rv(1, 0), rh1 = il ? rv(0, 1) : rv(1, 1);
    const F2 off = second ? (b ? g.c[A0][1] : g.c[A0][0]) : (b ? g.c[V0][1] : g.c[V0][0]);
    const F2 t = merged_t(c.straddle, lo, hi, off, g.c[U][1], rl0, rl1, rh0, rh1,
                          second ? g.d[V0] : g.d[A0], g.d[U], su);
    const F2 L = log1p_f2(t, T);
    if (off.h != 0.0f) v = f2_add(v, f2_mul(b ? off : f2_neg(off), L));
  }
  constexpr int B = U == 0 ? 1 : 0;
  const bool same_sign = !(neg_not_tiny(rel_bound(q, B, 0)) && !nonpos_or_tiny(rel_bound(q, B, 1)));
#pragma unroll 1
  for (int k = 0; k < 2; k++) {
    F2 o;
    if (!face_f2<U>(q, g, k, same_sign, T, o)) return false;
    if (o_faces) o_faces[k] = f2_to_double(o, 0);
    const F2 uk = k ? g.c[U][1] : g.c[U][0];
    if (uk.h != 0.0f) v = f2_add(v, f2_mul(k ? f2_neg(uk) : uk, o));  // -s_k u_k O_k
  }
  out = f2_to_double(v, g.top - 1023);
  return true;
}

// Diagonal tensor combination O_0 - O_1 of the faces normal to U on float
// pairs.  false: FP64 path.
template <int U>
HG_HD __forceinline__ bool pair_diag_f2(const Rel& q, const Tables& T, double& out) {
  using namespace lean;
  GeomF2 g;
  if (!make_geom_f2(q, g)) return false;
  constexpr int B = U == 0 ? 1 : 0;
  const bool same_sign = !(neg_not_tiny(rel_bound(q, B, 0)) && !nonpos_or_tiny(rel_bound(q, B, 1)));
  F2 v{0.0f, 0.0f};
#pragma unroll 1
  for (int k = 0; k < 2; k++) {
    F2 o;
    if (!face_f2<U>(q, g, k, same_sign, T, o)) return false;
    v = f2_add(v, k ? f2_neg(o) : o);
  }
  out = f2_to_double(v, 0);
  return true;
}

// ---------------------------------------------------------------------------
// Packed evaluation (lean_packed.cuh): the two faces normal to an axis, and
// the two merged logs of an edge family, each evaluated together in the two
// lanes of float2 registers.  Same formulas as the scalar float-pair path.

HG_HD __forceinline__ void pair_complex_p2(lean::P2 aa, lean::P2 asq, lean::P2 b1, lean::P2 b2,
                                           lean::P2 c, lean::P2 csq, lean::P2 r1, lean::P2 r2,
                                           bool same_sign, lean::P2 bdq, lean::P2& re,
                                           lean::P2& im) {
  using namespace lean;
  re = p2_add(p2_mul(asq, p2_mul(r1, r2)), p2_mul(p2_mul(b1, b2), csq));
  P2 x = p2_add(p2_mul(b2, r1), p2_mul(same_sign ? b1 : p2_neg(b1), r2));
  P2 d = x;
  if (same_sign) {
    const float2 sg = mk2(x.h.x < 0.0f ? -1.0f : 1.0f, x.h.y < 0.0f ? -1.0f : 1.0f);
    x = p2_scale(x, sg);
    d = p2_scale(bdq, sg);
    re = p2_mul(re, x);
  }
  im = p2_mul(p2_mul(aa, c), d);
}

// Scales each lane's complex number (re, im) by a power of two so that its
// larger component is in [1, 2).
HG_HD __forceinline__ void normalize_p2c(lean::P2& re, lean::P2& im) {
  using namespace lean;
  const auto sc = [](float r, float i) {
    const int er = (int)((f2u(r) >> 23) & 0xffu), ei = (int)((f2u(i) >> 23) & 0xffu);
    const int e = er > ei ? er : ei;
    return u2f((unsigned)(254 - (e > 253 ? 253 : e)) << 23);  // 2^(127 - e)
  };
  const float2 s = mk2(sc(re.h.x, im.h.x), sc(re.h.y, im.h.y));
  re = p2_scale(re, s);
  im = p2_scale(im, s);
}

// face_core_f2 for two faces at once (lanes); inputs as there.
HG_HD __forceinline__ lean::P2 face_core_p2(lean::P2 fa, lean::P2 fb1, lean::P2 fb2,
                                            lean::P2 fc1, lean::P2 fc2, lean::P2 fr11,
                                            lean::P2 fr12, lean::P2 fr21, lean::P2 fr22,
                                            lean::P2 fw, bool same_sign, const Tables& T) {
  using namespace lean;
  P2 asq = two_prod2(fa.h, fa.h);
  asq.l = fma2(add2(fa.h, fa.h), fa.l, asq.l);
  P2 c1sq = two_prod2(fc1.h, fc1.h), c2sq = two_prod2(fc2.h, fc2.h);
  c1sq.l = fma2(add2(fc1.h, fc1.h), fc1.l, c1sq.l);
  c2sq.l = fma2(add2(fc2.h, fc2.h), fc2.l, c2sq.l);
  P2 bdq1{sp2(0.0f), sp2(0.0f)}, bdq2{sp2(0.0f), sp2(0.0f)};
  if (same_sign) {
    const P2 fbd = p2_mul(fw, p2_add(fb2, fb1));
    bdq1 = p2_mul(fbd, p2_add(asq, c1sq));
    bdq2 = p2_mul(fbd, p2_add(asq, c2sq));
  }
  P2 ar, ai, br, bi;
  pair_complex_p2(fa, asq, fb1, fb2, fc2, c2sq, fr12, fr22, same_sign, bdq2, ar, ai);
  pair_complex_p2(fa, asq, fb1, fb2, fc1, c1sq, fr11, fr21, same_sign, bdq1, br, bi);
  normalize_p2c(ar, ai);
  normalize_p2c(br, bi);
  const P2 pr = p2_add(p2_mul(ar, br), p2_mul(ai, bi));
  const P2 pim = p2_add(p2_mul(ai, br), p2_neg(p2_mul(ar, bi)));
  float est0, est1;
  if (same_sign) {
    // b1 b2 >= 0: both pair products have positive real parts, so their
    // arguments differ by less than pi and the argument of A conj(B) is the
    // face angle itself (one estimate per lane instead of two)
    est0 = atan2_est(pim.h.x, pr.h.x);
    est1 = atan2_est(pim.h.y, pr.h.y);
  } else {
    est0 = atan2_est(ai.h.x, ar.h.x) - atan2_est(bi.h.x, br.h.x);
    est1 = atan2_est(ai.h.y, ar.h.y) - atan2_est(bi.h.y, br.h.y);
  }
  return arg_near_p2(pr, pim, est0, est1, T);
}

// The two faces normal to one axis (lanes: lower, upper bound), as face_f2,
// from their inputs: bounds along the normal (fa, ad), along the in-plane
// axes b and c (fb, bd, fc, cd), vertex distances fr[k][bi][ci] and the b
// width.  false: a coordinate is too small for the face's scale (FP64 path).
HG_HD __forceinline__ bool face_pair_core_p2(const lean::F2 fa[2], const lean::F2 fb[2],
                                             const lean::F2 fc[2], const lean::F2 fr[2][2][2],
                                             lean::F2 fw, bool same_sign, const Tables& T,
                                             lean::P2& o, bool fit);

HG_HD __forceinline__ bool face_pair_p2(const lean::F2 fa[2], const lean::F2 fb[2],
                                        const lean::F2 fc[2], const lean::F2 fr[2][2][2],
                                        lean::F2 fw, const double ad[2], const double bd[2],
                                        const double cd[2], const Tables& T, lean::P2& o,
                                        bool fit = false) {
  using namespace lean;
  const bool same_sign = !(neg_not_tiny(bd[0]) && !nonpos_or_tiny(bd[1]));
  if (!face_pair_core_p2(fa, fb, fc, fr, fw, same_sign, T, o, fit)) return false;
  // a point in a face plane: that face's outside limit
  if (is_tiny(ad[0]) || is_tiny(ad[1])) {
    F2 o0 = lane0(o), o1 = lane1(o);
    if (is_tiny(ad[0])) o0 = face_limit_f2(bd[0], bd[1], cd[0], cd[1], false);
    if (is_tiny(ad[1])) o1 = face_limit_f2(bd[0], bd[1], cd[0], cd[1], true);
    o = pk(o0, o1);
  }
  return true;
}

// The two faces from float-pair inputs alone (same_sign: the b bounds have
// one sign); false when a coordinate is too small for the face's scale.
// fit: the caller has established faces_fit_f2 (the checks cannot fail).
HG_HD __forceinline__ bool face_pair_core_p2(const lean::F2 fa[2], const lean::F2 fb[2],
                                             const lean::F2 fc[2], const lean::F2 fr[2][2][2],
                                             lean::F2 fw, bool same_sign, const Tables& T,
                                             lean::P2& o, bool fit) {
  using namespace lean;
  const auto fe = [](F2 a) { return (int)((f2u(a.h) >> 23) & 0xffu); };
  int ftop[2];
  bool small = false;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    ftop[k] = max(max(fe(fr[k][0][0]), fe(fr[k][0][1])), max(fe(fr[k][1][0]), fe(fr[k][1][1])));
    const auto fsmall = [&](F2 a) { return a.h != 0.0f && fe(a) < ftop[k] - 16; };
    if (!fit)
      small = small || fsmall(fa[k]) || fsmall(fb[0]) || fsmall(fb[1]) || fsmall(fc[0]) ||
              fsmall(fc[1]) || fe(fw) < ftop[k] - 16;
  }
  if (small) return false;
  const bool n0 = fa[0].h < 0.0f, n1 = fa[1].h < 0.0f;
  P2 v[10] = {pk(n0 ? f2_neg(fa[0]) : fa[0], n1 ? f2_neg(fa[1]) : fa[1]),
              pk(fb[0], fb[0]), pk(fb[1], fb[1]), pk(fc[0], fc[0]), pk(fc[1], fc[1]),
              pk(fr[0][0][0], fr[1][0][0]), pk(fr[0][0][1], fr[1][0][1]),
              pk(fr[0][1][0], fr[1][1][0]), pk(fr[0][1][1], fr[1][1][1]), pk(fw, fw)};
#ifndef HG_FACE_SCALE_ALWAYS
  // Scale so that each face's largest vertex distance is in [1, 2), unless
  // it is already in [1, 4) (the geometry's own scale puts the largest
  // bound in [1, 2): the common case of a face as far as the farthest
  // bound): the products below stay in the float range either way.
  if (ftop[0] < 127 || ftop[1] < 127)
#endif
  {
    const float2 sc = mk2(pow2f(127 - ftop[0]), pow2f(127 - ftop[1]));
#pragma unroll
    for (int k = 0; k < 10; k++) v[k] = p2_scale(v[k], sc);
  }
  o = face_core_p2(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], same_sign, T);
  F2 o0 = lane0(o), o1 = lane1(o);
  if (n0) o0 = f2_neg(o0);
  if (n1) o1 = f2_neg(o1);
  o = pk(o0, o1);
  return true;
}

// The two faces normal to U (x faces: b = y, c = z; y faces: b = x, c = z;
// z faces: b = x, c = y).
template <int U>
HG_HD __forceinline__ bool faces_p2(const Rel& q, const GeomF2& g, const Tables& T,
                                    lean::P2& o) {
  using namespace lean;
  constexpr int B = U == 0 ? 1 : 0, C = U == 2 ? 1 : 2;
  F2 fr[2][2][2];
#pragma unroll
  for (int k = 0; k < 2; k++)
#pragma unroll
    for (int bi = 0; bi < 2; bi++)
#pragma unroll
      for (int ci = 0; ci < 2; ci++) {
        int id[3];
        id[U] = k;
        id[B] = bi;
        id[C] = ci;
        fr[k][bi][ci] = g.r[id[0]][id[1]][id[2]];
      }
  const double ad[2] = {rel_bound(q, U, 0), rel_bound(q, U, 1)};
  const double bd[2] = {rel_bound(q, B, 0), rel_bound(q, B, 1)};
  const double cd[2] = {rel_bound(q, C, 0), rel_bound(q, C, 1)};
  return face_pair_p2(g.c[U], g.c[B], g.c[C], fr, g.d[B], ad, bd, cd, T, o, faces_fit_f2(g));
}

// All six faces O[axis][k] as three face pairs in a loop over the axis that
// is not unrolled (one copy of the face code; inputs chosen by selects).
HG_HD __forceinline__ bool faces_all_p2(const Rel& q, const GeomF2& g, const Tables& T,
                                        double O[3][2]) {
  using namespace lean;
#pragma unroll 1
  for (int axis = 0; axis < 3; axis++) {
    const bool X = axis == 0, Y = axis == 1;
    F2 fr[2][2][2];
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
      for (int bi = 0; bi < 2; bi++)
#pragma unroll
        for (int ci = 0; ci < 2; ci++)
          fr[k][bi][ci] = X ? g.r[k][bi][ci] : (Y ? g.r[bi][k][ci] : g.r[bi][ci][k]);
    const F2 fa[2] = {X ? g.c[0][0] : (Y ? g.c[1][0] : g.c[2][0]),
                      X ? g.c[0][1] : (Y ? g.c[1][1] : g.c[2][1])};
    const F2 fb[2] = {X ? g.c[1][0] : g.c[0][0], X ? g.c[1][1] : g.c[0][1]};
    const F2 fc[2] = {(X || Y) ? g.c[2][0] : g.c[1][0], (X || Y) ? g.c[2][1] : g.c[1][1]};
    const F2 fw = X ? g.d[1] : g.d[0];
    const double ad[2] = {rel_bound(q, axis, 0), rel_bound(q, axis, 1)};
    const double bd[2] = {X ? q.y1 : q.x1, X ? q.y2 : q.x2};
    const double cd[2] = {(X || Y) ? q.z1 : q.y1, (X || Y) ? q.z2 : q.y2};
    P2 o;
    if (!face_pair_p2(fa, fb, fc, fr, fw, ad, bd, cd, T, o)) return false;
    const double o0 = f2_to_double(lane0(o), 0), o1 = f2_to_double(lane1(o), 0);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      O[a][0] = axis == a ? o0 : O[a][0];
      O[a][1] = axis == a ? o1 : O[a][1];
    }
  }
  return true;
}

// merged_t for the two merged logs of one edge family (lanes: V-bounds 0, 1);
// the edge case is common to both lanes.
HG_HD __forceinline__ lean::P2 merged_t_p2(bool straddle, lean::P2 lo, lean::P2 hi, lean::P2 v,
                                           lean::P2 u1, lean::P2 rl0, lean::P2 rl1,
                                           lean::P2 rh0, lean::P2 rh1, lean::P2 dA,
                                           lean::P2 du, lean::P2 su) {
  using namespace lean;
  const P2 dQ = p2_mul(du, su);
  const P2 Sl = p2_add(rl0, rl1), Sh = p2_add(rh0, rh1);
  const P2 Dl = p2_div(dQ, Sl), Dh = p2_div(dQ, Sh);
  if (!straddle) {
    // 0 <= lo <= hi, so r_lo >= lo, r_hi >= hi, r_hi >= r_lo and |Dl| >= |Dh|
    // (one sign): those sums take the ordered addition
    const P2 D0 = p2_add_big(rl0, lo), D1 = p2_add_big(rl1, lo), N0 = p2_add_big(rh0, hi);
    const P2 P0 = p2_add_big(rh0, rl0), P1 = p2_add_big(rh1, rl1);
    const P2 inner = p2_add(p2_mul(D0, p2_add_big(Dl, Dh)), p2_mul(Dl, P1));
    const P2 br = p2_add(Dl, p2_div(p2_mul(p2_add_big(hi, lo), inner), p2_mul(P0, P1)));
    return p2_neg(p2_div(p2_mul(dA, br), p2_mul(D1, N0)));
  }
  const P2 M0 = p2_sub(rl0, lo), M1 = p2_sub(rl1, lo);
  const P2 Q1 = p2_add(p2_sq(v), p2_sq(u1));
  const P2 X = p2_add(p2_add(p2_mul(rh0, Dl), p2_neg(p2_mul(rl0, Dh))),
                      p2_add(p2_neg(p2_mul(hi, Sl)), p2_mul(lo, Sh)));
  return p2_div(p2_mul(p2_mul(dQ, M1), X), p2_mul(p2_mul(Sh, Sl), p2_mul(M0, Q1)));
}

// pair_grad_f2 with the merged logs and the faces evaluated two at a time.
template <int U>
HG_HD __forceinline__ bool pair_grad_p2(const Rel& q, const Tables& T, double& out,
                                        double* o_faces) {
  using namespace lean;
  GeomF2 g;
  if (!make_geom_f2(q, g)) return false;
  constexpr int A0 = U == 2 ? 1 : (U == 0 ? 2 : 0), V0 = 3 - U - A0;
  const AxisCase case0 = axis_case(rel_bound(q, A0, 0), rel_bound(q, A0, 1));
  const AxisCase case1 = axis_case(rel_bound(q, V0, 0), rel_bound(q, V0, 1));
  const F2 su = f2_add(g.c[U][0], g.c[U][1]);
  const auto bc = [](F2 a) { return pk(a, a); };
  P2 v2{sp2(0.0f), sp2(0.0f)};
#pragma unroll 1
  for (int fam = 0; fam < 2; fam++) {
    const bool second = fam;
    const AxisCase c = second ? case1 : case0;
    const F2 a1 = second ? g.c[V0][0] : g.c[A0][0], a2 = second ? g.c[V0][1] : g.c[A0][1];
    const F2 lo = c.reflect ? f2_neg(a2) : a1, hi = c.reflect ? f2_neg(a1) : a2;
    // r at A-end `end`, V-bound vb, U-bound eu (family 0: A0 = end, V0 = vb;
    // family 1: V0 = end, A0 = vb)
    const auto rv = [&](int end, int vb, int eu) {
      const auto at = [&](int ia, int iv) {
        int id[3] = {0, 0, 0};
        id[A0] = ia;
        id[V0] = iv;
        id[U] = eu;
        return g.r[id[0]][id[1]][id[2]];
      };
      return second ? at(vb, end) : at(end, vb);
    };
    const int il = c.reflect ? 1 : 0;
    const auto lanes = [&](int end, int eu) {
      return pk(il ? rv(1 - end, 0, eu) : rv(end, 0, eu), il ? rv(1 - end, 1, eu) : rv(end, 1, eu));
    };
    const P2 rl0 = lanes(0, 0), rl1 = lanes(0, 1), rh0 = lanes(1, 0), rh1 = lanes(1, 1);
    const F2 o0 = second ? g.c[A0][0] : g.c[V0][0], o1 = second ? g.c[A0][1] : g.c[V0][1];
    const P2 t = merged_t_p2(c.straddle, bc(lo), bc(hi), pk(o0, o1), bc(g.c[U][1]), rl0, rl1,
                             rh0, rh1, bc(second ? g.d[V0] : g.d[A0]), bc(g.d[U]), bc(su));
    P2 L = log1p_p2(t, T);
    // s_b off_b L_b (s_0 = -1); a zero coefficient gives 0 whatever L is
    if (o0.h == 0.0f) L.h.x = L.l.x = 0.0f;
    if (o1.h == 0.0f) L.h.y = L.l.y = 0.0f;
    v2 = p2_add(v2, p2_mul(pk(f2_neg(o0), o1), L));
  }
  P2 o;
  if (!faces_p2<U>(q, g, T, o)) return false;
  if (o_faces) {
    o_faces[0] = f2_to_double(lane0(o), 0);
    o_faces[1] = f2_to_double(lane1(o), 0);
  }
  // -s_k u_k O_k: +u_0 O_0, -u_1 O_1 (u_k = 0: the term vanishes)
  if (g.c[U][0].h == 0.0f) o.h.x = o.l.x = 0.0f;
  if (g.c[U][1].h == 0.0f) o.h.y = o.l.y = 0.0f;
  v2 = p2_add(v2, p2_mul(pk(g.c[U][0], f2_neg(g.c[U][1])), o));
  out = f2_to_double(f2_add(lane0(v2), lane1(v2)), g.top - 1023);
  return true;
}

// The two merged logs M_v = ln(R(v, u_1) / R(v, u_0)) of the edges parallel
// to A at the two V-bounds (lanes v = 0, 1), merged along U (merged_t).
template <int A, int V, int U>
HG_HD __forceinline__ lean::P2 merged_pair_p2(const Rel& q, const GeomF2& g, const Tables& T) {
  using namespace lean;
  const AxisCase c = axis_case(rel_bound(q, A, 0), rel_bound(q, A, 1));
  const F2 lo = c.reflect ? f2_neg(g.c[A][1]) : g.c[A][0];
  const F2 hi = c.reflect ? f2_neg(g.c[A][0]) : g.c[A][1];
  const int il = c.reflect ? 1 : 0;
  const auto rr = [&](int end, int vb, int eu) {
    int id[3];
    id[A] = end;
    id[V] = vb;
    id[U] = eu;
    return g.r[id[0]][id[1]][id[2]];
  };
  const auto lanes = [&](int end, int eu) {
    const int e = il ? 1 - end : end;
    return pk(rr(e, 0, eu), rr(e, 1, eu));
  };
  const auto bc = [](F2 a) { return pk(a, a); };
  const P2 t = merged_t_p2(c.straddle, bc(lo), bc(hi), pk(g.c[V][0], g.c[V][1]), bc(g.c[U][1]),
                           lanes(0, 0), lanes(0, 1), lanes(1, 0), lanes(1, 1), bc(g.d[A]),
                           bc(g.d[U]), bc(f2_add(g.c[U][0], g.c[U][1])));
  return log1p_p2(t, T);
}

// Off-diagonal tensor combination sum_{p,s} s_p s_s L[p][s] of the 4 edges
// parallel to A (= ln(R11 R00 / (R01 R10)), p along V, s along U) as the
// difference of the two merged logs M_1 - M_0.  Each M keeps its relative
// accuracy; the difference loses the first order of the distance (the FP64
// product of the four ratios loses the second).  false: FP64 path.
template <int A, int V, int U>
HG_HD __forceinline__ bool pair_offdiag_p2(const Rel& q, const Tables& T, double& out) {
  using namespace lean;
  GeomF2 g;
  if (!make_geom_f2(q, g)) return false;
  const P2 M = merged_pair_p2<A, V, U>(q, g, T);
  out = f2_to_double(f2_sub(lane1(M), lane0(M)), 0);
  return true;
}

// pair_diag_f2 with the two faces evaluated together.
template <int U>
HG_HD __forceinline__ bool pair_diag_p2(const Rel& q, const Tables& T, double& out) {
  using namespace lean;
  GeomF2 g;
  if (!make_geom_f2(q, g)) return false;
  P2 o;
  if (!faces_p2<U>(q, g, T, o)) return false;
  out = f2_to_double(f2_sub(lane0(o), lane1(o)), 0);
  return true;
}

// ---------------------------------------------------------------------------
// All ten fields, or the potential alone, on float pairs.
//
// The edge logs of one family (the 4 edges parallel to A, at the bounds p of
// P and q of Q, P < Q in (x, y, z) order: A = x: (y, z); A = y: (x, z);
// A = z: (x, y)) enter every field only through
//   MQ_p = L_p1 - L_p0   (merged along Q at P = p, merged_t),
//   MP_0 = L_10 - L_00   (along P at the lower Q bound),
//   L_00                 (one edge log, single_t_p2),
//   D    = MQ_1 - MQ_0   (= L_11 - L_10 - L_01 + L_00, the off-diagonal
//                         tensor combination of the family),
// since L_10 = L_00 + MP_0, L_01 = L_00 + MQ_0 and L_11 = L_10 + MQ_1:
//   sum_pq s_p s_q P_p Q_q L_pq = dP dQ L_00 + P_1 dQ MP_0 + Q_1 dP MQ_0 + P_1 Q_1 D
//   sum_pq s_p s_q Q_q L_pq     = Q_1 D + dQ MP_0
//   sum_pq s_p s_q P_p L_pq     = P_1 D + dP MQ_0
// (s_0 = -1, s_1 = +1; dP = P_1 - P_0).  Each right-hand term is of the
// order of the result, while the left-hand sums of four logs cancel to the
// second order of the distance (what limits the FP64 geometry far from the
// prism).  Likewise for the faces normal to an axis u:
//   u_0 O_0 - u_1 O_1     = u_0 (O_0 - O_1) - du O_1
//   u_0^2 O_0 - u_1^2 O_1 = u_0^2 (O_0 - O_1) - du (u_0 + u_1) O_1.
// With these, the combinations of pair_all become
//   potential = sum_fam E_fam + 1/2 sum_axis (u_0^2 O_0 - u_1^2 O_1),
//   g_e = QT_z + QT_y + F_x, g_n = QT_x + PT_z + F_y, g_z = PT_y + PT_x + F_z,
//   g_ee, g_nn, g_zz = O_0 - O_1 of the x, y, z faces,
//   g_en, g_ez, g_nz = D of the z, y, x families,
// with E the first sum above, QT and PT the second and third, F the first
// face identity (u the axis' coordinate).
//
// D multiplies P_1 Q_1 (of the order of the squared distance), so it needs
// the merged logs MQ_p: their difference keeps the relative accuracy of a
// first difference.  MP_0 multiplies P_1 dQ or dQ alone, so it is taken as
// the difference of the two single logs L_10 - L_00 (one packed single_t_p2
// for both): its rounding, ~2^-44 |L_00|, enters E as ~2^-44 |P_1| dQ |L_00|
// against |E| ~ dP dQ |L_00|, i.e. a relative error of ~2^-44 |P_1| / dP --
// 6e-10 at 1e4 prism widths, where the reference's own FP64 sum has lost
// ~1e-8 -- for one single log in place of a merged one.

// t = R - 1 of one edge log ln R, R = (hi + r_hi) / (lo + r_lo) for an edge
// beyond the point (lo >= 0 after reflection), or (hi + r_hi)(r_lo - lo) / rho2
// when the point projects inside the edge (lo < 0; rho2 = squared distance
// from the edge line), as sums of one-signed terms (r_hi - r_lo =
// dA (hi + lo) / (r_hi + r_lo), r_hi r_lo - rho2 = (hi^2 m^2 + rho2 (hi^2 +
// m^2)) / (r_hi r_lo + rho2) with m = -lo):
//   lo >= 0: t = dA (r_hi + r_lo + hi + lo) / ((r_hi + r_lo)(lo + r_lo))
//   lo < 0:  t = [hi r_lo + hi m + r_hi m + (hi^2 m^2 + rho2 (hi^2 + m^2))
//                 / (r_hi r_lo + rho2)] / rho2
// so t keeps its relative accuracy however far the edge is.
//
// Evaluated for the two edges of one family at P bounds 0 and 1 (lanes), at
// the same Q bound: same edge extent and case, own vertex distances and rho2.
HG_HD __forceinline__ lean::P2 single_t_p2(bool straddle, lean::P2 lo, lean::P2 hi, lean::P2 rl,
                                           lean::P2 rh, lean::P2 dA, lean::P2 rho2) {
  using namespace lean;
  if (!straddle) {
    // 0 <= lo <= hi: r_hi >= r_lo >= lo, S >= hi + lo (ordered additions)
    const P2 S = p2_add_big(rh, rl);
    return p2_div(p2_mul(dA, p2_add_big(S, p2_add_big(hi, lo))), p2_mul(S, p2_add_big(rl, lo)));
  }
  const P2 m = p2_neg(lo);
  const P2 h2 = p2_sq(hi), m2 = p2_sq(m);
  const P2 x = p2_div(p2_add(p2_mul(h2, m2), p2_mul(rho2, p2_add(h2, m2))),
                      p2_add(p2_mul(rh, rl), rho2));
  const P2 num = p2_add(p2_add(p2_mul(hi, rl), p2_mul(hi, m)), p2_add(p2_mul(rh, m), x));
  return p2_div(num, rho2);
}

// Float-pair bound k of axis a (a at run time, k a constant: selects only).
HG_HD __forceinline__ lean::F2 bound_f2(const GeomF2& g, int a, int k) {
  return a == 0 ? g.c[0][k] : (a == 1 ? g.c[1][k] : g.c[2][k]);
}
HG_HD __forceinline__ lean::F2 extent_f2(const GeomF2& g, int a) {
  return a == 0 ? g.d[0] : (a == 1 ? g.d[1] : g.d[2]);
}
HG_HD __forceinline__ lean::F2 f2_sel(bool c, lean::F2 a, lean::F2 b) { return c ? a : b; }

// The logs of edge family `fam` (= its axis A): MQ_0, MQ_1, MP_0, L_00.
// (The bounds are all nonzero here, so the case of the family's axis follows
// from the signs of the float-pair bounds: reflect when the upper bound is
// negative, straddle when the lower one is negative and the upper positive.)
HG_HD __forceinline__ void family_logs(const GeomF2& g, int fam, const Tables& T,
                                       lean::F2& mq0, lean::F2& mq1, lean::F2& mp0,
                                       lean::F2& l00) {
  using namespace lean;
  const int P = fam == 0 ? 1 : 0, Q = fam == 2 ? 1 : 2;
  const F2 a0 = bound_f2(g, fam, 0), a1 = bound_f2(g, fam, 1);
  AxisCase c;
  c.reflect = a1.h < 0.0f;
  c.straddle = !c.reflect && a0.h < 0.0f;
  const F2 lo = c.reflect ? f2_neg(a1) : a0, hi = c.reflect ? f2_neg(a0) : a1;
  // vertex distance at A-end e, P bound p, Q bound q (family layout)
  const auto R = [&](int e, int p, int qq) {
    return fam == 0 ? g.r[e][p][qq] : (fam == 1 ? g.r[p][e][qq] : g.r[p][qq][e]);
  };
  const int el = c.reflect ? 1 : 0;  // A-end of lo
  const auto RL = [&](int p, int qq) { return el ? R(1, p, qq) : R(0, p, qq); };
  const auto RH = [&](int p, int qq) { return el ? R(0, p, qq) : R(1, p, qq); };
  const F2 p0 = bound_f2(g, P, 0), p1 = bound_f2(g, P, 1);
  const F2 q0 = bound_f2(g, Q, 0), q1 = bound_f2(g, Q, 1);
  const F2 dA = extent_f2(g, fam), dP = extent_f2(g, P), dQ = extent_f2(g, Q);
  const auto bc = [](F2 v) { return pk(v, v); };
  // merged along Q, lanes P = 0, 1
  const P2 tq = merged_t_p2(c.straddle, bc(lo), bc(hi), pk(p0, p1), bc(q1),
                            pk(RL(0, 0), RL(1, 0)), pk(RL(0, 1), RL(1, 1)),
                            pk(RH(0, 0), RH(1, 0)), pk(RH(0, 1), RH(1, 1)), bc(dA), bc(dQ),
                            bc(f2_add(q0, q1)));
  (void)dP;
  const P2 q0b = bc(q0);
  const P2 ts = single_t_p2(c.straddle, bc(lo), bc(hi), pk(RL(0, 0), RL(1, 0)),
                            pk(RH(0, 0), RH(1, 0)), bc(dA),
                            p2_add(p2_sq(pk(p0, p1)), p2_sq(q0b)));
  // one copy of the logarithm for both (a smaller loop body: the fused and
  // potential kernels wait on instruction fetch)
  P2 mq, ml;
#pragma unroll 1
  for (int w = 0; w < 2; w++) {
    const P2 L = log1p_p2(w ? ts : tq, T);
    if (w) ml = L;
    else mq = L;
  }
  mq0 = lane0(mq);
  mq1 = lane1(mq);
  l00 = lane0(ml);
  mp0 = f2_sub(lane1(ml), l00);
}

// The two faces normal to `axis` as float pairs (lanes: lower, upper bound),
// for a pair with no zero bound (no face-plane limit to take); FIT as
// face_pair_core_p2.
template <bool FIT = false>
HG_HD __forceinline__ bool face_pair_f2(const GeomF2& g, int axis, const Tables& T,
                                        lean::F2& o0, lean::F2& o1) {
  using namespace lean;
  const bool X = axis == 0, Y = axis == 1;
  F2 fr[2][2][2];
#pragma unroll
  for (int k = 0; k < 2; k++)
#pragma unroll
    for (int bi = 0; bi < 2; bi++)
#pragma unroll
      for (int ci = 0; ci < 2; ci++)
        fr[k][bi][ci] = X ? g.r[k][bi][ci] : (Y ? g.r[bi][k][ci] : g.r[bi][ci][k]);
  const F2 fa[2] = {bound_f2(g, axis, 0), bound_f2(g, axis, 1)};
  const F2 fb[2] = {X ? g.c[1][0] : g.c[0][0], X ? g.c[1][1] : g.c[0][1]};
  const F2 fc[2] = {(X || Y) ? g.c[2][0] : g.c[1][0], (X || Y) ? g.c[2][1] : g.c[1][1]};
  const F2 fw = X ? g.d[1] : g.d[0];
  P2 o;
  if (!face_pair_core_p2(fa, fb, fc, fr, fw, !(fb[0].h < 0.0f && fb[1].h > 0.0f), T, o, FIT))
    return false;
  o0 = lane0(o);
  o1 = lane1(o);
  return true;
}

// out[0..9] (ALL) or out[0] (the potential alone), the raw combinations of
// pair_all.  false: a bound is zero or too small for the float-pair scale
// (the point lies in a face plane or on an edge line, where the identities
// above would add infinite logs with cancelling coefficients), or the
// geometry leaves the float range; the caller takes the FP64 geometry.
HG_HD __forceinline__ bool any_zero_bound(const Rel& q) {
  return is_tiny(q.x1) || is_tiny(q.x2) || is_tiny(q.y1) || is_tiny(q.y2) || is_tiny(q.z1) ||
         is_tiny(q.z2);
}

// pair_all_f2 on a geometry with no zero bound, already on float pairs.
// PART 0: the whole pair; 1: the edge-log terms alone; 2: the face terms
// alone (the two parts add up to part 0; see faces_fit_f2).
template <bool ALL, int PART = 0>
HG_HD __forceinline__ bool pair_all_f2_geom(const GeomF2& g, const Tables& T, double* out);


template <bool ALL>
HG_HD __forceinline__ bool pair_all_f2(const Rel& q, const Tables& T, double* out) {
  GeomF2 g;
  return !any_zero_bound(q) && make_geom_f2(q, g) && pair_all_f2_geom<ALL>(g, T, out);
}

// The potential alone.  Each family's E is taken as
//   E = dQ (dP L00 + p1 MP0) + q1 (dP MQ0 + p1 D)
// with the two brackets in the lanes of one packed pair (3 packed products,
// one packed sum, in place of eight scalar products and three sums); the
// lanes of the family sums and of the face sums are added once at the end.
// Each bracket times its factor is a sum of two of E's four terms, so its
// rounding is a rounding of those terms, as in the four-term sum.
template <int PART>
HG_HD __forceinline__ bool potential_f2_geom(const GeomF2& g, const Tables& T, lean::F2* out) {
  using namespace lean;
  P2 pot2{sp2(0.0f), sp2(0.0f)}, face2{sp2(0.0f), sp2(0.0f)};
#pragma unroll 1
  for (int fam = 0; fam < (PART == 2 ? 0 : 3); fam++) {
    F2 mq0, mq1, mp0, l00;
    family_logs(g, fam, T, mq0, mq1, mp0, l00);
    const int P = fam == 0 ? 1 : 0, Q = fam == 2 ? 1 : 2;
    const F2 p1 = bound_f2(g, P, 1), q1 = bound_f2(g, Q, 1);
    const F2 dP = extent_f2(g, P), dQ = extent_f2(g, Q);
    const F2 D = f2_sub(mq1, mq0);
    const P2 B = p2_add(p2_mul(pk(dP, dP), pk(l00, mq0)), p2_mul(pk(p1, p1), pk(mp0, D)));
    pot2 = p2_add(pot2, p2_mul(pk(dQ, q1), B));
  }
#pragma unroll 1
  for (int axis = 0; axis < (PART == 1 ? 0 : 3); axis++) {
    F2 o0, o1;
    if (!face_pair_f2<PART != 0>(g, axis, T, o0, o1)) return false;
    const F2 u0 = bound_f2(g, axis, 0), du = extent_f2(g, axis);
    // u0^2 (O0 - O1) - du (u0 + u1) O1 as the lanes (u0 u0 dO, -su du O1)
    const P2 ds = p2_add(pk(o0, u0), pk(f2_neg(o1), bound_f2(g, axis, 1)));  // (dO, su)
    const P2 T1 = p2_mul(pk(u0, du), pk(lane0(ds), o1));
    face2 = p2_add(face2, p2_mul(pk(u0, f2_neg(lane1(ds))), T1));
  }
  F2 pot;
  if constexpr (PART == 2) {
    pot = f2_add(lane0(face2), lane1(face2));
    pot = F2{fmul(0.5f, pot.h), fmul(0.5f, pot.l)};
  } else {
    pot = f2_add(lane0(pot2), lane1(pot2));
    if constexpr (PART == 0) {
      const F2 faces2 = f2_add(lane0(face2), lane1(face2));
      pot = f2_add(pot, F2{fmul(0.5f, faces2.h), fmul(0.5f, faces2.l)});
    }
  }
  out[kPotential] = pot;
  return true;
}

// pair_all_f2_geom's sums as float pairs at the pair's scale: out[f] times
// 2^(2 e1) for the potential, 2^e1 for g_e, g_n, g_z and 1 for the tensor
// components is the field (e1 = g.top - 1023, raw_exponent); the fields a
// part does not carry are zero.
template <bool ALL, int PART>
HG_HD __forceinline__ bool pair_all_f2_raw(const GeomF2& g, const Tables& T, lean::F2* out) {
  using namespace lean;
  if (!ALL) return potential_f2_geom<PART>(g, T, out);
  const F2 zero{0.0f, 0.0f};
  // The combinations below run two products or sums per packed instruction:
  // pot2 holds the potential's edge terms in two lanes (dP dQ L00 + q1 dP
  // MQ0, p1 dQ MP0 + p1 q1 D summed over the families) and its face terms in
  // face2 (lane 1; lane 0 carries the first-derivative face term F).
  P2 pot2{sp2(0.0f), sp2(0.0f)}, face2{sp2(0.0f), sp2(0.0f)};
  F2 ge = zero, gn = zero, gz = zero, Dx = zero, Dy = zero, Dz = zero;
#pragma unroll 1
  for (int fam = 0; fam < (PART == 2 ? 0 : 3); fam++) {
    F2 mq0, mq1, mp0, l00;
    family_logs(g, fam, T, mq0, mq1, mp0, l00);
    const int P = fam == 0 ? 1 : 0, Q = fam == 2 ? 1 : 2;
    const F2 p1 = bound_f2(g, P, 1), q1 = bound_f2(g, Q, 1);
    const F2 dP = extent_f2(g, P), dQ = extent_f2(g, Q);
    const F2 D = f2_sub(mq1, mq0);
    // E = dP dQ L00 + p1 dQ MP0 + q1 dP MQ0 + p1 q1 D
    const P2 X = p2_mul(pk(dP, p1), pk(dQ, dQ)), Y = p2_mul(pk(q1, p1), pk(dP, q1));
    pot2 = p2_add(pot2, p2_add(p2_mul(X, pk(l00, mp0)), p2_mul(Y, pk(mq0, D))));
    if (ALL) {
      // (QT, PT) = (q1 D + dQ MP0, p1 D + dP MQ0); g_e = QT_z + QT_y,
      // g_n = QT_x + PT_z, g_z = PT_y + PT_x (edge parts): QT goes to g_n
      // for family x, else g_e; PT to g_n for family z, else g_z
      const P2 QP = p2_add(p2_mul(pk(q1, p1), pk(D, D)), p2_mul(pk(dQ, dP), pk(mp0, mq0)));
      const bool fx = fam == 0, fz = fam == 2;
      const P2 acc = p2_add(pk(fx ? gn : ge, fz ? gn : gz), QP);
      ge = fx ? ge : lane0(acc);
      gn = fx ? lane0(acc) : (fz ? lane1(acc) : gn);
      gz = fz ? gz : lane1(acc);
      Dx = f2_sel(fx, D, Dx);
      Dy = f2_sel(fam == 1, D, Dy);
      Dz = f2_sel(fz, D, Dz);
    }
  }
  F2 diff[3] = {zero, zero, zero};
#pragma unroll 1
  for (int axis = 0; axis < (PART == 1 ? 0 : 3); axis++) {
    F2 o0, o1;
    if (!face_pair_f2<PART != 0>(g, axis, T, o0, o1)) return false;
    const F2 u0 = bound_f2(g, axis, 0), du = extent_f2(g, axis);
    // (dO, su) = (O0 - O1, u0 + u1)
    const P2 ds = p2_add(pk(o0, u0), pk(f2_neg(o1), bound_f2(g, axis, 1)));
    const F2 dO = lane0(ds);
    // T1 = (u0 dO, du O1), T2 = (u0 u0 dO, su du O1): lanes of
    // (F, face term) = (u0 dO - du O1, u0^2 dO - su du O1)
    const P2 T1 = p2_mul(pk(u0, du), pk(dO, o1));
    const P2 T2 = p2_mul(pk(u0, lane1(ds)), T1);
    const P2 FF = p2_sub(pk(lane0(T1), lane0(T2)), pk(lane1(T1), lane1(T2)));
    face2 = p2_add(face2, FF);
    if (ALL) {
      const F2 F = lane0(FF);
      const bool X = axis == 0, Y = axis == 1;
      const F2 a = f2_add(X ? ge : (Y ? gn : gz), F);
      ge = X ? a : ge;
      gn = Y ? a : gn;
      gz = (X || Y) ? gz : a;
#pragma unroll
      for (int k = 0; k < 3; k++) diff[k] = axis == k ? dO : diff[k];
    }
  }
  const F2 faces2 = lane1(face2);
  const F2 pot = f2_add(f2_add(lane0(pot2), lane1(pot2)),
                        F2{fmul(0.5f, faces2.h), fmul(0.5f, faces2.l)});
  out[kPotential] = pot;
  if (ALL) {
    out[kGe] = ge;
    out[kGn] = gn;
    out[kGz] = gz;
    // the diagonal tensor components are face terms alone, the off-diagonal
    // ones edge terms alone
    out[kGee] = PART == 1 ? zero : diff[0];
    out[kGnn] = PART == 1 ? zero : diff[1];
    out[kGzz] = PART == 1 ? zero : diff[2];
    out[kGen] = PART == 2 ? zero : Dz;
    out[kGez] = PART == 2 ? zero : Dy;
    out[kGnz] = PART == 2 ? zero : Dx;
  }
  return true;
}

// Power-of-two exponent of pair_all_f2_raw's output f (see there).
HG_HD __forceinline__ int raw_exponent(int f, int e1) {
  return f == kPotential ? 2 * e1 : ((f == kGe || f == kGn || f == kGz) ? e1 : 0);
}

template <bool ALL, int PART>
HG_HD __forceinline__ bool pair_all_f2_geom(const GeomF2& g, const Tables& T, double* out) {
  lean::F2 v[ALL ? kNumFields : 1];
  if (!pair_all_f2_raw<ALL, PART>(g, T, v)) return false;
  const int e1 = g.top - 1023;
#pragma unroll
  for (int f = 0; f < (ALL ? kNumFields : 1); f++) out[f] = f2_to_double(v[f], raw_exponent(f, e1));
  return true;
}

// FP64 evaluations for the pairs the float-pair paths decline (out of line).
template <int F>
HG_COLD double pair_field_fp64(const Rel& q, const Tables& T);

// ---------------------------------------------------------------------------
// All ten fields of one pair: the signed edge/face combinations (without G,
// rho and units).  s = -1 for index 0 (lower bound), +1 for index 1 (upper).
template <bool LEAN>
HG_HD __forceinline__ void pair_all_geom(const Rel& q, const Tables& T, double out[kNumFields]);

// The FP64 geometry for the pairs pair_all_f2 declines (out of line: rare).
HG_COLD void pair_all_fp64(const Rel& q, const Tables& T, double* out);

// All ten fields of one pair: on float pairs (pair_all_f2) with the lean
// math, else (or where that declines) on the FP64 geometry.
template <bool LEAN>
HG_HD __forceinline__ void pair_all(const Rel& q, const Tables& T, double out[kNumFields]) {
  if (!LEAN) {
    pair_all_geom<false>(q, T, out);
  } else if (!pair_all_f2<true>(q, T, out)) {
    pair_all_fp64(q, T, out);
  }
}

template <bool LEAN>
HG_HD __forceinline__ void pair_all_geom(const Rel& q, const Tables& T, double out[kNumFields]) {
  Geom g;
  make_geom<LEAN>(q, g);
  EdgeSet Ex, Ey, Ez;
  edges_x(g, Ex);
  edges_y(g, Ey);
  edges_z(g, Ez);
  double Lx[2][2], Ly[2][2], Lz[2][2];
  logs12<LEAN>(Ex, Ey, Ez, T, Lx, Ly, Lz);
  double O[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
  GeomF2 gf;
  if (!LEAN || !make_geom_f2(q, gf) || !faces_all_p2(q, gf, T, O)) faces6<LEAN>(g, T, O);
  const double* Ox = O[0];
  const double* Oy = O[1];
  const double* Oz = O[2];
  double pot = 0.0, ge = 0.0, gn = 0.0, gz = 0.0;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      // s_a s_b = +1 when a == b; Lx[j][k], Ly[i][k], Lz[i][j]
      const bool ng = a != b;
      pot = cfma_sgn(g.x[a] * g.y[b], ng, Lz[a][b], pot);
      pot = cfma_sgn(g.y[a] * g.z[b], ng, Lx[a][b], pot);
      pot = cfma_sgn(g.x[a] * g.z[b], ng, Ly[a][b], pot);
      ge = cfma_sgn(g.y[b], ng, Lz[a][b], ge);
      ge = cfma_sgn(g.z[b], ng, Ly[a][b], ge);
      gn = cfma_sgn(g.z[b], ng, Lx[a][b], gn);
      gn = cfma_sgn(g.x[a], ng, Lz[a][b], gn);
      gz = cfma_sgn(g.x[a], ng, Ly[a][b], gz);
      gz = cfma_sgn(g.y[a], ng, Lx[a][b], gz);
    }
#pragma unroll
  for (int a = 0; a < 2; a++) {
    // face terms carry -s_a (potential: -s_a / 2)
    const bool ng = a == 1;
    pot = cfma_sgn(0.5 * g.x2[a], ng, Ox[a], pot);
    pot = cfma_sgn(0.5 * g.y2[a], ng, Oy[a], pot);
    pot = cfma_sgn(0.5 * g.z2[a], ng, Oz[a], pot);
    ge = cfma_sgn(g.x[a], ng, Ox[a], ge);
    gn = cfma_sgn(g.y[a], ng, Oy[a], gn);
    gz = cfma_sgn(g.z[a], ng, Oz[a], gz);
  }
  out[kPotential] = pot;
  out[kGe] = ge;
  out[kGn] = gn;
  out[kGz] = gz;
  out[kGee] = -(Ox[1] - Ox[0]);
  out[kGnn] = -(Oy[1] - Oy[0]);
  out[kGzz] = -(Oz[1] - Oz[0]);
  out[kGen] = Lz[1][1] - Lz[0][1] - Lz[1][0] + Lz[0][0];
  out[kGez] = Ly[1][1] - Ly[0][1] - Ly[1][0] + Ly[0][0];
  out[kGnz] = Lx[1][1] - Lx[0][1] - Lx[1][0] + Lx[0][0];
}

// One field of one pair, with the edge logs merged where coefficients allow.
template <int F, bool LEAN>
HG_HD __forceinline__ double pair_field_geom(const Rel& q, const Tables& T) {
  if (F == kPotential) {
    double out[kNumFields];
    pair_all_geom<LEAN>(q, T, out);
    return out[kPotential];
  }
  Geom g;
  make_geom<LEAN>(q, g);
  if (F == kGz) {
    // sum_i s_i x_i sum_k s_k Ly[i][k] + sum_j s_j y_j sum_k s_k Lx[j][k]
    //   - sum_k s_k z_k Oz[k]
    EdgeSet Ey, Ex;
    edges_y(g, Ey);
    edges_x(g, Ex);
    const double v =
        merged_logs4<LEAN, false, false>(Ey, Ex, g.x[0], g.x[1], g.y[0], g.y[1], T, 0.0);
    return faces2_dot<2, LEAN>(g, g.z[0], g.z[1], T, v);
  } else if (F == kGe) {
    // sum_j s_j y_j sum_i s_i Lz[i][j] + sum_k s_k z_k sum_i s_i Ly[i][k]
    //   - sum_i s_i x_i Ox[i]
    EdgeSet Ez, Ey;
    edges_z(g, Ez);
    edges_y(g, Ey);
    const double v =
        merged_logs4<LEAN, true, true>(Ez, Ey, g.y[0], g.y[1], g.z[0], g.z[1], T, 0.0);
    return faces2_dot<0, LEAN>(g, g.x[0], g.x[1], T, v);
  } else if (F == kGn) {
    // sum_k s_k z_k sum_j s_j Lx[j][k] + sum_i s_i x_i sum_j s_j Lz[i][j]
    //   - sum_j s_j y_j Oy[j]
    EdgeSet Ex, Ez;
    edges_x(g, Ex);
    edges_z(g, Ez);
    const double v =
        merged_logs4<LEAN, true, false>(Ex, Ez, g.z[0], g.z[1], g.x[0], g.x[1], T, 0.0);
    return faces2_dot<1, LEAN>(g, g.y[0], g.y[1], T, v);
  } else if (F == kGee || F == kGnn || F == kGzz) {
    return faces2_dot<(F == kGee ? 0 : (F == kGnn ? 1 : 2)), LEAN>(g, 1.0, 1.0, T, 0.0);
  } else {
    // g_en / g_ez / g_nz: sum_{p,s} s_p s_s L[p][s] = ln(R11 R00 / (R01 R10))
    EdgeSet E;
    if (F == kGen) edges_z(g, E);
    if (F == kGez) edges_y(g, E);
    if (F == kGnz) edges_x(g, E);
    return log_quot<LEAN>(E.num[1][1] * E.num[0][0], E.den[0][1] * E.den[1][0],
                          E.den[1][1] * E.den[0][0], E.num[0][1] * E.num[1][0], T);
  }
}

template <int F>
HG_COLD double pair_field_fp64(const Rel& q, const Tables& T) {
  return pair_field_geom<F, true>(q, T);
}

HG_COLD void pair_all_fp64(const Rel& q, const Tables& T, double* out) {
  pair_all_geom<true>(q, T, out);
}

// One field of one pair.  With the lean math, the acceleration components and
// the diagonal tensor components run on float pairs (pair_grad_f2,
// pair_diag_f2); the rest, and the pairs those decline, on the FP64
// geometry (pair_field_geom).
template <int F, bool LEAN>
HG_HD __forceinline__ double pair_field(const Rel& q, const Tables& T) {
  if (LEAN && F == kPotential) {
    double v;
    if (pair_all_f2<false>(q, T, &v)) return v;
    return pair_field_fp64<F>(q, T);
  }
  if (LEAN && (F == kGe || F == kGn || F == kGz)) {
    double v;
    if (pair_grad_p2<(F == kGe ? 0 : (F == kGn ? 1 : 2))>(q, T, v, nullptr)) return v;
    return pair_field_fp64<F>(q, T);
  }
  if (LEAN && (F == kGee || F == kGnn || F == kGzz)) {
    double v;
    if (pair_diag_p2<(F == kGee ? 0 : (F == kGnn ? 1 : 2))>(q, T, v)) return v;
    return pair_field_fp64<F>(q, T);
  }
  if (LEAN && (F == kGen || F == kGez || F == kGnz)) {
    // edges along z at (x_i, y_j) for g_en, along y at (x_i, z_k) for g_ez,
    // along x at (y_j, z_k) for g_nz: p along the first in-plane axis
    double v;
    const bool ok = F == kGen   ? pair_offdiag_p2<2, 0, 1>(q, T, v)
                    : F == kGez ? pair_offdiag_p2<1, 0, 2>(q, T, v)
                                : pair_offdiag_p2<0, 1, 2>(q, T, v);
    if (ok) return v;
    return pair_field_fp64<F>(q, T);
  }
  return pair_field_geom<F, LEAN>(q, T);
}

// The six gradient-tensor combinations of one pair (the second derivatives
// of the unit-density potential kernel, order ee, nn, uu, en, eu, nu with
// upward u), for the magnetic field b = mu0/(4 pi) T M.  Singular points are
// not masked here (the caller decides).
template <bool LEAN>
HG_HD __forceinline__ void pair_tensor6(const Rel& q, const Tables& T, double t[6]) {
  if (LEAN) {
    // float-pair geometry: faces as three packed pairs, the off-diagonal
    // combinations as differences of merged logs (pair_offdiag_p2)
    GeomF2 gf;
    double O[3][2];
    if (make_geom_f2(q, gf) && faces_all_p2(q, gf, T, O)) {
      t[0] = O[0][0] - O[0][1];
      t[1] = O[1][0] - O[1][1];
      t[2] = O[2][0] - O[2][1];
      const auto diff = [](lean::P2 M) {
        return lean::f2_to_double(lean::f2_sub(lean::lane1(M), lean::lane0(M)), 0);
      };
      t[3] = diff(merged_pair_p2<2, 0, 1>(q, gf, T));
      t[4] = diff(merged_pair_p2<1, 0, 2>(q, gf, T));
      t[5] = diff(merged_pair_p2<0, 1, 2>(q, gf, T));
      return;
    }
  }
  Geom g;
  make_geom<LEAN>(q, g);
  double O[3][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
  GeomF2 gf;
  if (!LEAN || !make_geom_f2(q, gf) || !faces_all_p2(q, gf, T, O)) faces6<LEAN>(g, T, O);
  t[0] = O[0][0] - O[0][1];
  t[1] = O[1][0] - O[1][1];
  t[2] = O[2][0] - O[2][1];
  EdgeSet E;
  edges_z(g, E);
  t[3] = log_quot<LEAN>(E.num[1][1] * E.num[0][0], E.den[0][1] * E.den[1][0],
                        E.den[1][1] * E.den[0][0], E.num[0][1] * E.num[1][0], T);
  edges_y(g, E);
  t[4] = log_quot<LEAN>(E.num[1][1] * E.num[0][0], E.den[0][1] * E.den[1][0],
                        E.den[1][1] * E.den[0][0], E.num[0][1] * E.num[1][0], T);
  edges_x(g, E);
  t[5] = log_quot<LEAN>(E.num[1][1] * E.num[0][0], E.den[0][1] * E.den[1][0],
                        E.den[1][1] * E.den[0][0], E.num[0][1] * E.num[1][0], T);
}

// g_z combination of one pair together with its two horizontal face angles
// (the derivatives of the combination with respect to the bottom and top
// coordinates: d/dz_bottom = O_bottom, d/dz_top = -O_top), for the adjoint.
HG_COLD double pair_gz_faces_fp64(const Rel& q, const Tables& T, double* o);

template <bool LEAN>
HG_HD __forceinline__ double pair_gz_faces(const Rel& q, const Tables& T, double& o_bottom,
                                           double& o_top) {
  if (LEAN) {
    double v, o[2];
    if (!pair_grad_p2<2>(q, T, v, o)) v = pair_gz_faces_fp64(q, T, o);
    o_bottom = o[0];
    o_top = o[1];
    return v;
  }
  Geom g;
  make_geom<LEAN>(q, g);
  EdgeSet Ey, Ex;
  edges_y(g, Ey);
  edges_x(g, Ex);
  faces2<2, LEAN>(g, T, o_bottom, o_top);
  double v = merged_logs4<LEAN, false, false>(Ey, Ex, g.x[0], g.x[1], g.y[0], g.y[1], T, 0.0);
  v = cfma_s<true>(g.z[1], o_top, v);
  return cfma_s<false>(g.z[0], o_bottom, v);
}

HG_COLD double pair_gz_faces_fp64(const Rel& q, const Tables& T, double* o) {
  return pair_gz_faces<false>(q, T, o[0], o[1]);
}

}  // namespace hg
