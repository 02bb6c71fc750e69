// Host build of the edge/face prism formulation used by the CUDA kernels
// (harmonica_gb300/csrc/prism_math.cuh), for CPU tests of the formulation
// against the oracle and mpmath.  Test infrastructure only: the product
// never runs this code on the host.
#include <cstdint>

#include "../../harmonica_gb300/csrc/prism_math.cuh"
#include "../../harmonica_gb300/csrc/lean_packed.cuh"

using namespace hg;

template <bool LEAN>
static double pair_any(int f, const Rel& q) {
  const Tables T = lean::host_tables();
  switch (f) {
    case 0: return pair_field<0, LEAN>(q, T);
    case 1: return pair_field<1, LEAN>(q, T);
    case 2: return pair_field<2, LEAN>(q, T);
    case 3: return pair_field<3, LEAN>(q, T);
    case 4: return pair_field<4, LEAN>(q, T);
    case 5: return pair_field<5, LEAN>(q, T);
    case 6: return pair_field<6, LEAN>(q, T);
    case 7: return pair_field<7, LEAN>(q, T);
    case 8: return pair_field<8, LEAN>(q, T);
    case 9: return pair_field<9, LEAN>(q, T);
  }
  return 0.0;
}

extern "C" {

// Sum over prisms (AoS, 6 per row) for each point, harmonica units, with the
// kernel's null-prism skip and NaN at singular points.  mode: 0 = lean math,
// 1 = generic library math, 2 = lean math through the fused all-field path,
// 3 = the fused path as its edge-log part plus its face part.
void host_prism_gravity(int field, int64_t n_obs, const double* e, const double* n,
                        const double* u, int64_t m, const double* prisms, const double* rho,
                        double* out, int mode) {
  for (int64_t i = 0; i < n_obs; i++) {
    double acc = 0.0;
    for (int64_t j = 0; j < m; j++) {
      const double* p = prisms + 6 * j;
      if (p[0] == p[1] || p[2] == p[3] || p[4] == p[5] || rho[j] == 0.0) continue;
      Rel q{p[0] - e[i], p[1] - e[i], p[2] - n[i], p[3] - n[i], p[4] - u[i], p[5] - u[i],
            p[1] - p[0], p[3] - p[2], p[5] - p[4]};
      double v;
      if (mode == 2) {
        double all[kNumFields];
        pair_all<true>(q, lean::host_tables(), all);
        v = all[field];
      } else if (mode == 3) {
        // the two-launch form of the potential and fused all-field kernels:
        // edge-log part + face part when the faces fit, else the whole pair
        double all[kNumFields];
        GeomF2 g;
        const Tables T = lean::host_tables();
        if (!any_zero_bound(q) && make_geom_f2(q, g) && faces_fit_f2(g)) {
          double edges[kNumFields], faces[kNumFields];
          pair_all_f2_geom<true, 1>(g, T, edges);
          pair_all_f2_geom<true, 2>(g, T, faces);
          for (int f = 0; f < kNumFields; f++) all[f] = edges[f] + faces[f];
        } else {
          pair_all<true>(q, T, all);
        }
        v = all[field];
      } else {
        v = mode == 0 ? pair_any<true>(field, q) : pair_any<false>(field, q);
      }
      if (field >= kGee && singular_for(field, q)) v = quiet_nan();
      acc += rho[j] * v;
    }
    out[i] = acc * field_scale(field);
  }
}

}

extern "C" {

// Elementwise evaluation of the lean FP64 functions for the CPU tests.
// kind: 0 sqrt(a), 1 a / b, 2 log(a), 3 log((a b) / (c d)), 4 log(a / c),
//       5 arg(a + i b) on the branch nearest the float estimate c, 6 1/sqrt(a).
void host_lean(int kind, int64_t n, const double* a, const double* b, const double* c,
               const double* d, double* out) {
  const Tables T = lean::host_tables();
  for (int64_t i = 0; i < n; i++) {
    switch (kind) {
      case 0: out[i] = lean::lm_sqrt(a[i]); break;
      case 1: out[i] = lean::lm_div(a[i], b[i]); break;
      case 2: out[i] = lean::lm_log(a[i], T); break;
      case 3: out[i] = lean::lm_log_quot<false>(a[i], b[i], c[i], d[i], T); break;
      case 4: out[i] = lean::lm_log_quot<true>(a[i], 1.0, c[i], 1.0, T); break;
      case 5: out[i] = lean::lm_arg_near(a[i], b[i], (float)c[i], T); break;
      default: out[i] = lean::lm_rsqrt(a[i]); break;
    }
  }
}

}

extern "C" {

// The float-pair point-mass terms of the tesseroid and point kernels, lane 0
// of the packed helpers (lean_packed.cuh), for the CPU precision tests.
// For each i: P = (a[i], b[i], c[i]), Q = (d[3i], d[3i+1], d[3i+2]) as
// float pairs; kind 0: 1 / |P - Q| (p2_diff, p2_norm2, p2_rsqrt); kind 1:
// (P_z - Q_z) / |P - Q|^3.
void host_pairs(int kind, int64_t n, const double* a, const double* b, const double* c,
                const double* d, double* out) {
  using namespace lean;
  for (int64_t i = 0; i < n; i++) {
    const auto two = [](double v) {
      const F2 f = double_to_f2(v);
      return P2{mk2(f.h, f.h), mk2(f.l, f.l)};
    };
    const P2 dx = p2_diff(two(a[i]), two(d[3 * i]));
    const P2 dy = p2_diff(two(b[i]), two(d[3 * i + 1]));
    const P2 dz = p2_diff(two(c[i]), two(d[3 * i + 2]));
    const P2 inv = p2_rsqrt(p2_norm2(dx, dy, dz));
    const P2 v = kind == 0 ? inv : p2_mul(dz, p2_mul(p2_mul(inv, inv), inv));
    out[i] = f2_to_double(f2_add(lane0(v), F2{0.0f, 0.0f}), 0);
  }
}

}
