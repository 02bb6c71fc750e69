// Closed-form gravitational field of a right-rectangular prism, evaluated as a
// sum over EDGES (log terms) and FACES (arctangent terms) instead of the
// 8-vertex sum.  Device code for sm_103a.
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
// Regrouping the vertex sum: every log term ln(a + r) with a coefficient that
// does not depend on a collapses, for each of the 4 edges parallel to axis a,
// into one EDGE LOG
//   L = ln(a_2 + r_2) - ln(a_1 + r_1)
// and every arctangent term with a coefficient depending only on the axis
// normal to a face collapses into one FACE ANGLE
//   O = sum_{b,c} s_b s_c atan(b c / (a r)).
// A prism then needs 12 edge logs and 6 face angles for all ten fields instead
// of 24 logs and 24 arctangents, and each edge log is a ratio whose argument
// tends to 1 for distant prisms instead of a difference of two large logs.
//
// Conventions (gravity.py:141-158): potential and acceleration are finite
// everywhere (a log or angle multiplied by a zero coefficient contributes 0);
// tensor components are NaN on the singular edges and vertices of each
// component; diagonal tensor components on a face normal to their axis take
// the limit from outside the prism.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

// The math is usable from host code too (the tests compile it for the CPU to
// check the formulation against the oracle without a GPU).
#define HG_HD __host__ __device__

namespace hg {

HG_HD __forceinline__ long long bits_of(double v) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(v);
#else
  long long r;
  std::memcpy(&r, &v, sizeof(r));
  return r;
#endif
}

HG_HD __forceinline__ double quiet_nan() {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(0x7ff8000000000000LL);
#else
  return std::nan("");
#endif
}

constexpr double kG = 6.6743e-11;  // harmonica constants.py:12
constexpr double kHalfPi = 1.5707963267948966;

enum Field : int {
  kPotential = 0, kGe = 1, kGn = 2, kGz = 3, kGee = 4, kGnn = 5, kGzz = 6,
  kGen = 7, kGez = 8, kGnz = 9, kNumFields = 10
};

// Output multiplier per field: G, harmonica's sign flip for g_z/g_ez/g_nz and
// the SI -> mGal (1e5) / Eotvos (1e9) conversion (gravity.py:227-236),
// applied to sum_j rho_j * (signed edge/face combination) where the
// combination already carries the -1 of the first derivatives.
HG_HD inline double field_scale(int f) {
  switch (f) {
    case kPotential: return kG;
    case kGe: return -kG * 1e5;
    case kGn: return -kG * 1e5;
    case kGz: return kG * 1e5;       // -(-G) : upward kernel negated to downward
    case kGee: case kGnn: case kGzz: case kGen: return kG * 1e9;
    case kGez: case kGnz: return -kG * 1e9;
    default: return 0.0;
  }
}

// ---------------------------------------------------------------------------
// bit-level predicates that stay off the FP64 pipe
HG_HD __forceinline__ bool is_zero(double v) {
  return (bits_of(v) << 1) == 0;  // +0 or -0
}
HG_HD __forceinline__ bool is_neg(double v) {  // strictly negative, no NaN input
  return bits_of(v) < 0 && !is_zero(v);
}
HG_HD __forceinline__ bool is_nonpos(double v) {
  return bits_of(v) < 0 || is_zero(v);
}
HG_HD __forceinline__ int sgn(double v) {
  return is_zero(v) ? 0 : (bits_of(v) < 0 ? -1 : 1);
}

// ---------------------------------------------------------------------------
// Edge log along one axis: ln((a2 + r2) / (a1 + r1)) with a1 <= a2 the
// observation-relative coordinates of the edge ends, r1, r2 their distances
// and rho2 the squared distance from the edge line.  Evaluated without
// cancellation:
//  * a2 <= 0: reflect a -> -a (the value is invariant) so that the upper end
//    is non-negative;
//  * lower end negative (the point projects inside the edge): use
//    (a1 + r1) = rho2 / (r1 - a1).
// `axis_reflect` and `axis_straddle` depend only on the point's coordinate
// relative to the prism along this axis, so they are shared by its 4 edges.
struct AxisCase {
  bool reflect;   // a2 <= 0
  bool straddle;  // after reflection, lower end < 0
};

HG_HD __forceinline__ AxisCase axis_case(double a1, double a2) {
  AxisCase c;
  c.reflect = is_nonpos(a2);
  double lo = c.reflect ? -a2 : a1;
  c.straddle = is_neg(lo);
  return c;
}

// Returns numerator and denominator of the edge ratio (both >= 0).
HG_HD __forceinline__ void edge_ratio(AxisCase c, double a1, double a2, double r1, double r2,
                                           double rho2, double& num, double& den) {
  double lo = c.reflect ? -a2 : a1;
  double hi = c.reflect ? -a1 : a2;
  double rlo = c.reflect ? r2 : r1;
  double rhi = c.reflect ? r1 : r2;
  double t = fabs(lo) + rlo;  // lo + rlo, or rlo - lo when lo < 0
  num = hi + rhi;
  if (c.straddle) {
    num = num * t;
    den = rho2;
  } else {
    den = t;
  }
}

HG_HD __forceinline__ double edge_log(AxisCase c, double a1, double a2, double r1, double r2,
                                           double rho2) {
  double num, den;
  edge_ratio(c, a1, a2, r1, r2, rho2, num, den);
  return log(num / den);
}

// ---------------------------------------------------------------------------
// Face angle for the face at (normal coordinate) a, with in-plane coordinates
// b_1 < b_2, c_1 < c_2 and vertex distances r[bi][ci]:
//   O = sum_{bi,ci} s_b s_c atan(b c / (a r)).
// For a != 0, atan(bc/(ar)) = sign(a) arg(|a| r + i bc) with a positive real
// part, so each pair of vertices along b is an argument difference in
// (-pi, pi) and equals the argument of one complex product:
//   arg(c_2c) - arg(c_1c) = arg((|a| r_2c + i b2 c)(|a| r_1c - i b1 c))
//     = atan2(|a| c (b2 r_1c - b1 r_2c), a^2 r_1c r_2c + b1 b2 c^2).
// For a distant face b2 r_1c - b1 r_2c cancels; when b1, b2 have one sign it
// is rewritten without cancellation as
//   (b2 - b1)(b2 + b1)(a^2 + c^2) / (b2 r_1c + b1 r_2c)
// and the positive denominator is moved into the real part (atan2 is
// invariant under scaling both arguments by a positive number).
// For a == 0 the value is the limit from outside the prism:
// a -> 0+ for the lower face (upper == false), a -> 0- for the upper face.
HG_HD __forceinline__ double pair_angle(double aa, double a2, double b1, double b2, double c,
                                        double c2, double r1, double r2, bool same_sign) {
  double re = a2 * r1 * r2 + b1 * b2 * c2;
  double d;
  if (same_sign) {
    double den = b2 * r1 + b1 * r2;  // one sign, no cancellation
    d = (b2 - b1) * (b2 + b1) * (a2 + c2);
    if (den < 0.0) {
      den = -den;
      d = -d;
    }
    re *= den;
  } else {
    d = b2 * r1 - b1 * r2;  // b1 < 0 < b2: both terms positive
  }
  return atan2(aa * c * d, re);
}

HG_HD __forceinline__ double face_angle(double a, bool upper, double b1, double b2, double c1,
                                        double c2, double r11, double r12, double r21,
                                        double r22) {
  if (is_zero(a)) {
    int s = sgn(b2) * sgn(c2) + sgn(b1) * sgn(c1) - sgn(b1) * sgn(c2) - sgn(b2) * sgn(c1);
    return (upper ? -kHalfPi : kHalfPi) * (double)s;
  }
  const double aa = fabs(a);
  const double asq = a * a;
  const bool same_sign = !(is_neg(b1) && !is_nonpos(b2));
  // (22 - 12) + (11 - 21) = [arg c_{2,c2} - arg c_{1,c2}] - [arg c_{2,c1} - arg c_{1,c1}]
  double o = pair_angle(aa, asq, b1, b2, c2, c2 * c2, r12, r22, same_sign) -
             pair_angle(aa, asq, b1, b2, c1, c1 * c1, r11, r21, same_sign);
  return is_neg(a) ? -o : o;
}

// ---------------------------------------------------------------------------
// Singular-point predicates on the observation-relative bounds; they mirror
// choclo's is_point_on_{easting,northing,upward}_edge as used by
// gravity.py:272-449 (closed intervals, so vertices are included).
struct Rel {
  double x1, x2, y1, y2, z1, z2;
};

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

// Multiply a log/angle by a coefficient, with the limit 0 * (singular) = 0.
HG_HD __forceinline__ double cmul(double coef, double v) {
  return is_zero(coef) ? 0.0 : coef * v;
}

// ---------------------------------------------------------------------------
// Which edge logs / face angles a field needs.
template <int F> struct Needs;
template <> struct Needs<kPotential> { static constexpr bool Lx = 1, Ly = 1, Lz = 1, Ox = 1, Oy = 1, Oz = 1; };
template <> struct Needs<kGe> { static constexpr bool Lx = 0, Ly = 1, Lz = 1, Ox = 1, Oy = 0, Oz = 0; };
template <> struct Needs<kGn> { static constexpr bool Lx = 1, Ly = 0, Lz = 1, Ox = 0, Oy = 1, Oz = 0; };
template <> struct Needs<kGz> { static constexpr bool Lx = 1, Ly = 1, Lz = 0, Ox = 0, Oy = 0, Oz = 1; };
template <> struct Needs<kGee> { static constexpr bool Lx = 0, Ly = 0, Lz = 0, Ox = 1, Oy = 0, Oz = 0; };
template <> struct Needs<kGnn> { static constexpr bool Lx = 0, Ly = 0, Lz = 0, Ox = 0, Oy = 1, Oz = 0; };
template <> struct Needs<kGzz> { static constexpr bool Lx = 0, Ly = 0, Lz = 0, Ox = 0, Oy = 0, Oz = 1; };
template <> struct Needs<kGen> { static constexpr bool Lx = 0, Ly = 0, Lz = 1, Ox = 0, Oy = 0, Oz = 0; };
template <> struct Needs<kGez> { static constexpr bool Lx = 0, Ly = 1, Lz = 0, Ox = 0, Oy = 0, Oz = 0; };
template <> struct Needs<kGnz> { static constexpr bool Lx = 1, Ly = 0, Lz = 0, Ox = 0, Oy = 0, Oz = 0; };
constexpr int kAll = 10;  // fused evaluation of all ten fields
template <> struct Needs<kAll> { static constexpr bool Lx = 1, Ly = 1, Lz = 1, Ox = 1, Oy = 1, Oz = 1; };

// Edge logs and face angles of one (observation point, prism) pair.
struct PairTerms {
  double Lx[2][2];  // edge along x at (y_j, z_k)
  double Ly[2][2];  // edge along y at (x_i, z_k)
  double Lz[2][2];  // edge along z at (x_i, y_j)
  double Ox[2], Oy[2], Oz[2];
};

template <int F>
HG_HD __forceinline__ void pair_terms(const Rel& q, PairTerms& t) {
  using N = Needs<F>;
  const double xs[2] = {q.x1, q.x2}, ys[2] = {q.y1, q.y2}, zs[2] = {q.z1, q.z2};
  double x2s[2] = {q.x1 * q.x1, q.x2 * q.x2};
  double y2s[2] = {q.y1 * q.y1, q.y2 * q.y2};
  double z2s[2] = {q.z1 * q.z1, q.z2 * q.z2};
  double r[2][2][2];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      double xy = x2s[i] + y2s[j];
#pragma unroll
      for (int k = 0; k < 2; k++) r[i][j][k] = sqrt(xy + z2s[k]);
    }
  if (N::Lx) {
    AxisCase c = axis_case(q.x1, q.x2);
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int k = 0; k < 2; k++)
        t.Lx[j][k] = edge_log(c, q.x1, q.x2, r[0][j][k], r[1][j][k], y2s[j] + z2s[k]);
  }
  if (N::Ly) {
    AxisCase c = axis_case(q.y1, q.y2);
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int k = 0; k < 2; k++)
        t.Ly[i][k] = edge_log(c, q.y1, q.y2, r[i][0][k], r[i][1][k], x2s[i] + z2s[k]);
  }
  if (N::Lz) {
    AxisCase c = axis_case(q.z1, q.z2);
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
      for (int j = 0; j < 2; j++)
        t.Lz[i][j] = edge_log(c, q.z1, q.z2, r[i][j][0], r[i][j][1], x2s[i] + y2s[j]);
  }
  if (N::Ox) {
#pragma unroll
    for (int i = 0; i < 2; i++)  // in-plane (y_j, z_k), r[i][j][k]
      t.Ox[i] = face_angle(xs[i], i == 1, ys[0], ys[1], zs[0], zs[1], r[i][0][0], r[i][0][1],
                           r[i][1][0], r[i][1][1]);
  }
  if (N::Oy) {
#pragma unroll
    for (int j = 0; j < 2; j++)  // in-plane (x_i, z_k), r[i][j][k]
      t.Oy[j] = face_angle(ys[j], j == 1, xs[0], xs[1], zs[0], zs[1], r[0][j][0], r[0][j][1],
                           r[1][j][0], r[1][j][1]);
  }
  if (N::Oz) {
#pragma unroll
    for (int k = 0; k < 2; k++)  // in-plane (x_i, y_j), r[i][j][k]
      t.Oz[k] = face_angle(zs[k], k == 1, xs[0], xs[1], ys[0], ys[1], r[0][0][k], r[0][1][k],
                           r[1][0][k], r[1][1][k]);
  }
}

// Signed combination of edge logs and face angles for one field (without
// G, rho and units): see the regrouping in the header comment.  s = -1 for
// index 0 (lower bound) and +1 for index 1 (upper bound).
HG_HD __forceinline__ double combine(int f, const Rel& q, const PairTerms& t) {
  const double xs[2] = {q.x1, q.x2}, ys[2] = {q.y1, q.y2}, zs[2] = {q.z1, q.z2};
  const double s[2] = {-1.0, 1.0};
  double v = 0.0;
  switch (f) {
    case kPotential:
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
          double sab = s[a] * s[b];
          v += sab * (cmul(xs[a] * ys[b], t.Lz[a][b]) + cmul(ys[a] * zs[b], t.Lx[a][b]) +
                      cmul(zs[b] * xs[a], t.Ly[a][b]));
        }
#pragma unroll
      for (int a = 0; a < 2; a++)
        v -= 0.5 * s[a] * (cmul(xs[a] * xs[a], t.Ox[a]) + cmul(ys[a] * ys[a], t.Oy[a]) +
                           cmul(zs[a] * zs[a], t.Oz[a]));
      return v;
    case kGe:
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
          v += s[a] * s[b] * (cmul(ys[b], t.Lz[a][b]) + cmul(zs[b], t.Ly[a][b]));
#pragma unroll
      for (int a = 0; a < 2; a++) v -= s[a] * cmul(xs[a], t.Ox[a]);
      return v;
    case kGn:
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
          v += s[a] * s[b] * (cmul(zs[b], t.Lx[a][b]) + cmul(xs[a], t.Lz[a][b]));
#pragma unroll
      for (int a = 0; a < 2; a++) v -= s[a] * cmul(ys[a], t.Oy[a]);
      return v;
    case kGz:
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++)
          v += s[a] * s[b] * (cmul(xs[a], t.Ly[a][b]) + cmul(ys[a], t.Lx[a][b]));
#pragma unroll
      for (int a = 0; a < 2; a++) v -= s[a] * cmul(zs[a], t.Oz[a]);
      return v;
    case kGee: return -(t.Ox[1] - t.Ox[0]);
    case kGnn: return -(t.Oy[1] - t.Oy[0]);
    case kGzz: return -(t.Oz[1] - t.Oz[0]);
    case kGen: return t.Lz[1][1] - t.Lz[0][1] - t.Lz[1][0] + t.Lz[0][0];
    case kGez: return t.Ly[1][1] - t.Ly[0][1] - t.Ly[1][0] + t.Ly[0][0];
    case kGnz: return t.Lx[1][1] - t.Lx[0][1] - t.Lx[1][0] + t.Lx[0][0];
    default: return 0.0;
  }
}

}  // namespace hg
