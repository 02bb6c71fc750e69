// Float pairs two at a time in the lanes of float2 registers, for the packed
// FP32 instructions of sm_100-class GPUs (FADD2 / FMUL2 / FFMA2: two FP32
// operations per lane per instruction).  On GB300 a packed FMA has the same
// FP32 throughput as two scalar ones but takes one issue slot, and the
// float-pair prism kernels are bound by instruction issue, so evaluating two
// independent float-pair quantities together (the two faces normal to an
// axis, the two merged logs of an edge family, two vertex distances) cuts
// their instruction count nearly in half.  Same algorithms and error bounds as
// the scalar float-pair functions of lean_math.cuh, lane by lane.
#pragma once
#include "lean_math.cuh"

namespace hg {
namespace lean {

// two float pairs: lane x and lane y, value = h + l per lane
struct P2 {
  float2 h, l;
};

HG_HD __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
HG_HD __forceinline__ float2 sp2(float a) { return make_float2(a, a); }
HG_HD __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
HG_HD __forceinline__ float2 add2(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
HG_HD __forceinline__ float2 sub2(float2 a, float2 b) { return add2(a, neg2(b)); }
HG_HD __forceinline__ float2 mul2(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fmul2_rn(a, b);
#else
  return make_float2(a.x * b.x, a.y * b.y);
#endif
}
HG_HD __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
#ifdef __CUDA_ARCH__
  return __ffma2_rn(a, b, c);
#else
  return make_float2(std::fmaf(a.x, b.x, c.x), std::fmaf(a.y, b.y, c.y));
#endif
}

HG_HD __forceinline__ P2 pk(F2 a, F2 b) { return P2{mk2(a.h, b.h), mk2(a.l, b.l)}; }
HG_HD __forceinline__ F2 lane0(P2 a) { return F2{a.h.x, a.l.x}; }
HG_HD __forceinline__ F2 lane1(P2 a) { return F2{a.h.y, a.l.y}; }

HG_HD __forceinline__ P2 two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  const float2 bb = sub2(s, a);
  return P2{s, add2(sub2(a, sub2(s, bb)), sub2(b, bb))};
}
HG_HD __forceinline__ P2 quick_two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  return P2{s, sub2(b, sub2(s, a))};
}
HG_HD __forceinline__ P2 two_prod2(float2 a, float2 b) {
  const float2 p = mul2(a, b);
  return P2{p, fma2(a, b, neg2(p))};
}
// product without the final renormalisation: l stays within ~1.5 ulp(h)
// (the product's rounding error plus the cross terms), which every consumer
// here tolerates; saves 3 of 7 FP32 operations.
HG_HD __forceinline__ P2 p2_mul(P2 a, P2 b) {
  const P2 p = two_prod2(a.h, b.h);
  return P2{p.h, fma2(a.h, b.l, fma2(a.l, b.h, p.l))};
}
HG_HD __forceinline__ P2 p2_add(P2 a, P2 b) {
  const P2 s = two_sum2(a.h, b.h);
  return quick_two_sum2(s.h, add2(s.l, add2(a.l, b.l)));
}
// a + b when |a.h| >= |b.h| (or the two are within a rounding of each
// other): the high parts' rounding error by Fast2Sum instead of TwoSum, 3 of
// 11 FP32 operations fewer, same result.
HG_HD __forceinline__ P2 p2_add_big(P2 a, P2 b) {
  const P2 s = quick_two_sum2(a.h, b.h);
  return quick_two_sum2(s.h, add2(s.l, add2(a.l, b.l)));
}
HG_HD __forceinline__ P2 p2_neg(P2 a) { return P2{neg2(a.h), neg2(a.l)}; }
HG_HD __forceinline__ P2 p2_sub(P2 a, P2 b) { return p2_add(a, p2_neg(b)); }
HG_HD __forceinline__ P2 p2_sq(P2 a) {
  const P2 p = two_prod2(a.h, a.h);
  return quick_two_sum2(p.h, fma2(add2(a.h, a.h), a.l, p.l));
}
// a / b for b > 0 (lane-wise f2_div)
HG_HD __forceinline__ P2 p2_div(P2 a, P2 b) {
  float2 y = mk2(rcp_approx(b.h.x), rcp_approx(b.h.y));
  y = fma2(y, fma2(neg2(b.h), y, sp2(1.0f)), y);
  const float2 qh = mul2(a.h, y);
  float2 r = fma2(neg2(qh), b.h, a.h);
  r = add2(r, a.l);
  r = fma2(neg2(qh), b.l, r);
  return P2{qh, mul2(r, y)};
}
// sqrt(a) for a > 0 normal (lane-wise f2_sqrt)
HG_HD __forceinline__ P2 p2_sqrt(P2 a) {
  float2 y = mk2(rsqrt_approx(a.h.x), rsqrt_approx(a.h.y));
  y = mul2(y, fma2(mul2(sp2(-0.5f), a.h), mul2(y, y), sp2(1.5f)));
  const float2 s = mul2(a.h, y);
  const P2 s2 = two_prod2(s, s);
  const float2 res = add2(sub2(sub2(a.h, s2.h), s2.l), a.l);
  return quick_two_sum2(s, mul2(res, mul2(sp2(0.5f), y)));
}
// both lanes times powers of two (exact)
HG_HD __forceinline__ P2 p2_scale(P2 a, float2 s) { return P2{mul2(a.h, s), mul2(a.l, s)}; }

// 1 / sqrt(x) lane by lane for x > 0 normal: FP32 seed, one Newton step with
// its second-order term, the residual 1 - x y^2 on float pairs.
HG_HD __forceinline__ P2 p2_rsqrt(P2 x) {
  const float2 y = mk2(rsqrt_approx(x.h.x), rsqrt_approx(x.h.y));
  const P2 xy2 = p2_mul(x, two_prod2(y, y));
  const float2 r = sub2(sub2(sp2(1.0f), xy2.h), xy2.l);
  const float2 c = mul2(r, fma2(sp2(0.375f), r, sp2(0.5f)));
  return P2{y, mul2(y, c)};
}

// a - b lane by lane: the rounded difference of the high parts, its exact
// rounding error plus the low parts, renormalised (the low parts of 6e6 m
// coordinates are up to 0.5 m, hundreds of ulps of a 30 km difference: left
// unnormalised, the squares below would lose their (lo)^2 terms).
HG_HD __forceinline__ P2 p2_diff(P2 a, P2 b) {
  const P2 s = two_sum2(a.h, neg2(b.h));
  return quick_two_sum2(s.h, add2(s.l, sub2(a.l, b.l)));
}

// x^2 + y^2 + z^2 lane by lane: exact squares of the high parts, their sum
// by two-sums, every low-order term added once, one renormalisation.
HG_HD __forceinline__ P2 p2_norm2(P2 x, P2 y, P2 z) {
  const P2 px = two_prod2(x.h, x.h), py = two_prod2(y.h, y.h), pz = two_prod2(z.h, z.h);
  const P2 s = two_sum2(px.h, py.h);
  const P2 t = two_sum2(s.h, pz.h);
  float2 lo = add2(add2(px.l, py.l), add2(pz.l, add2(s.l, t.l)));
  lo = fma2(x.h, add2(x.l, x.l), lo);
  lo = fma2(y.h, add2(y.l, y.l), lo);
  lo = fma2(z.h, add2(z.l, z.l), lo);
  return quick_two_sum2(t.h, lo);
}

// log1p(t) for |t| <= 2^-8.5, lane-wise log1p_series_f2
HG_HD __forceinline__ P2 log1p_series_p2(P2 t) {
  P2 s2 = two_prod2(t.h, t.h);
  s2.l = fma2(add2(t.h, t.h), t.l, s2.l);  // t^2
  // t^3 (1/3 - t/4 + t^2/5 - t^3/6) in FP32: at most |t|^2 / 3 <= 2.3e-6 of
  // the result, so its FP32 rounding stays below 1.4e-13 of ln(1 + t) (the
  // float-pair terms t and t^2/2 keep ~2^-46)
  const float2 tail =
      fma2(t.h, fma2(t.h, fma2(t.h, sp2(-0.166666672f), sp2(0.2f)), sp2(-0.25f)),
           sp2(0.333333343f));
  const float2 c = mul2(mul2(s2.h, t.h), tail);
  P2 v = quick_two_sum2(mul2(sp2(-0.5f), s2.h), c);
  v.l = fma2(sp2(-0.5f), s2.l, v.l);
  P2 lp = quick_two_sum2(t.h, v.h);
  lp.l = add2(lp.l, add2(t.l, v.l));
  return lp;
}

// ln(1 + t) lane-wise (log1p_f2), always through the table reduction: near
// 1 it selects c = 1, E = 0, so the reduced argument is t itself.
HG_HD __forceinline__ P2 log1p_p2(P2 t, const Tables& T) {
  if (fabsf(t.h.x) < 0.0026f && fabsf(t.h.y) < 0.0026f) return log1p_series_p2(t);
  const P2 w = p2_add(P2{sp2(1.0f), sp2(0.0f)}, t);
  const auto plan = [&](float wh, float& cp, int& k, float& ef) {
    const unsigned uw = f2u(wh);
    int E = (int)((uw >> 23) & 0xffu) - 127;
    float m = u2f((uw & 0x7fffffu) | 0x3f800000u);  // [1, 2)
    if (m >= 1.5f) {
      m = fmul(m, 0.5f);
      E += 1;
    }
    k = round_to_int((m - 0.75f) * 256.0f);
    k = k < 0 ? 0 : (k > kLogTableSize - 1 ? kLogTableSize - 1 : k);
    cp = fmul(d2f_trunc(T.logc[k]), pow2f(-E));  // c_k is a float: exact
    ef = (float)E;
  };
  float cp0, cp1, e0, e1;
  int k0, k1;
  plan(w.h.x, cp0, k0, e0);
  plan(w.h.y, cp1, k1, e1);
  const float2 cp = mk2(cp0, cp1);
  P2 tc = two_prod2(t.h, cp);  // t c (c a float)
  tc.l = fma2(t.l, cp, tc.l);
  const P2 red = p2_add(tc, two_sum2(cp, sp2(-1.0f)));
  const P2 lp = log1p_series_p2(red);
  const P2 lc{mk2(T.loglf[2 * k0], T.loglf[2 * k1]), mk2(T.loglf[2 * k0 + 1], T.loglf[2 * k1 + 1])};
  // 1 + t in [0.75, 1.5) in both lanes (E = 0: the far single edge logs):
  // E ln 2 is zero and (0 + lc) + lp is lc + lp, the same bits
  if (e0 == 0.0f && e1 == 0.0f) return p2_add(lc, lp);
  const float2 ef = mk2(e0, e1);
  P2 e2 = two_prod2(ef, sp2(kLn2F2));
  e2.l = fma2(ef, sp2(kLn2F3), e2.l);
  const P2 eln2 = p2_add(P2{mul2(ef, sp2(kLn2F1)), sp2(0.0f)}, e2);
  return p2_add(p2_add(eln2, lc), lp);
}

// arg_core_f2 on the quarter-turn-rotated vector, out of line: the rare lane
// whose FP32 estimate was too far off (keeps ~5 KB of code per call site out
// of the hot loops' instruction footprint).
HG_COLD F2 arg_generic_f2(F2 re, F2 im, Tables T) { return arg_core_f2(re, im, 0, 0, T); }

// Argument of two vectors (lane-wise lm_arg_near_f2) on the branches of the
// FP32 estimates est0, est1.  The table rotation runs when either lane needs
// it (the other rotates by 0: exact); a lane whose residual is not small
// takes the generic path out of line.
HG_HD __forceinline__ P2 arg_near_p2(P2 pr, P2 pi, float est0, float est1, const Tables& T) {
  int q0, j0, q1, j1;
  arg_plan(est0, q0, j0);
  arg_plan(est1, q1, j1);
  // rotate by -q pi/2 exactly, lane by lane
  const auto quarter = [](int q, F2 r, F2 i, F2& r0, F2& i0) {
    const int qm = q & 3;
    r0 = qm == 0 ? r : (qm == 1 ? i : (qm == 2 ? f2_neg(r) : f2_neg(i)));
    i0 = qm == 0 ? i : (qm == 1 ? f2_neg(r) : (qm == 2 ? f2_neg(i) : r));
  };
  P2 re = pr, im = pi;
  if (q0 != 0 || q1 != 0) {  // both lanes within pi/4 of 0: nothing to rotate
    F2 ra, ia, rb, ib;
    quarter(q0, lane0(pr), lane0(pi), ra, ia);
    quarter(q1, lane1(pr), lane1(pi), rb, ib);
    re = pk(ra, rb);
    im = pk(ia, ib);
  }
  const P2 re0 = re, im0 = im;
  const int ja = 2 * (j0 + kArgTableHalf), jb = 2 * (j1 + kArgTableHalf);
  if (j0 != 0 || j1 != 0) {  // rotate by -th_j (th_0 = 0: cos 1, sin 0)
    const P2 C{mk2(T.csf[ja], T.csf[jb]), mk2(T.csf[ja + 1], T.csf[jb + 1])};
    const P2 S{mk2(T.snf[ja], T.snf[jb]), mk2(T.snf[ja + 1], T.snf[jb + 1])};
    const P2 r2 = p2_add(p2_mul(re, C), p2_mul(im, S));
    im = p2_add(p2_mul(im, C), p2_neg(p2_mul(re, S)));
    re = r2;
  }
  const P2 u = p2_div(im, re);
  P2 s2 = two_prod2(u.h, u.h);
  s2.l = fma2(add2(u.h, u.h), u.l, s2.l);  // u^2
  P2 w = two_prod2(s2.h, u.h);
  w.l = fma2(s2.h, u.l, fma2(s2.l, u.h, w.l));  // u^3
  const float2 tail = mul2(s2.h, fma2(s2.h, sp2(-0.142857143f), sp2(0.2f)));
  P2 c = two_prod2(w.h, sp2(-kThirdHi));
  c.l = fma2(w.h, sub2(tail, sp2(kThirdLo)), fma2(w.l, sp2(-kThirdHi), c.l));
  P2 a = quick_two_sum2(u.h, c.h);
  a.l = add2(a.l, add2(u.l, c.l));
  const bool ok0 = re.h.x > 0.0f && fabsf(u.h.x) < 0.02f;
  const bool ok1 = re.h.y > 0.0f && fabsf(u.h.y) < 0.02f;
  if (!ok0 || !ok1) {
    // estimate too far off or non-finite input: generic path on the
    // quarter-turn-rotated vector for that lane, th_j then not added
    F2 a0 = lane0(a), a1 = lane1(a);
    if (!ok0) a0 = arg_generic_f2(lane0(re0), lane0(im0), T);
    if (!ok1) a1 = arg_generic_f2(lane1(re0), lane1(im0), T);
    a = pk(a0, a1);
    if (!ok0) j0 = 0;
    if (!ok1) j1 = 0;
  }
  if (j0 != 0 || j1 != 0) {  // th_j (th_0 = 0: only the renormalisation)
    const int ka = 2 * (j0 + kArgTableHalf), kb = 2 * (j1 + kArgTableHalf);
    a = p2_add(a, P2{mk2(T.thf[ka], T.thf[kb]), mk2(T.thf[ka + 1], T.thf[kb + 1])});
  } else {
    a = quick_two_sum2(a.h, a.l);
  }
  if (q0 != 0 || q1 != 0) {  // q pi/2 with pi/2 in three floats (q * F1 exact)
    const float2 qf = mk2((float)q0, (float)q1);
    P2 p = two_prod2(qf, sp2(kPio2F2));
    p.l = fma2(qf, sp2(kPio2F3), p.l);
    a = p2_add(a, p2_add(P2{mul2(qf, sp2(kPio2F1)), sp2(0.0f)}, p));
  }
  return a;
}

}  // namespace lean
}  // namespace hg
