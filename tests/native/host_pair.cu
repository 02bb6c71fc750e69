// Host build of the edge/face prism formulation used by the CUDA kernels
// (harmonica_gb300/csrc/prism_math.cuh), for CPU tests of the formulation
// against the oracle and mpmath.  Test infrastructure only: the product
// never runs this code on the host.
#include <cstdint>

#include "../../harmonica_gb300/csrc/prism_math.cuh"

using namespace hg;

template <int F>
static double pair_value(const Rel& q) {
  PairTerms T;
  pair_terms<F>(q, T);
  return combine(F, q, T);
}

static double pair_any(int f, const Rel& q) {
  switch (f) {
    case 0: return pair_value<0>(q);
    case 1: return pair_value<1>(q);
    case 2: return pair_value<2>(q);
    case 3: return pair_value<3>(q);
    case 4: return pair_value<4>(q);
    case 5: return pair_value<5>(q);
    case 6: return pair_value<6>(q);
    case 7: return pair_value<7>(q);
    case 8: return pair_value<8>(q);
    case 9: return pair_value<9>(q);
  }
  return 0.0;
}

extern "C" {

// Sum over prisms (AoS, 6 per row) for each point, harmonica units, with the
// kernel's null-prism skip and NaN at singular points.
void host_prism_gravity(int field, int64_t n_obs, const double* e, const double* n,
                        const double* u, int64_t m, const double* prisms, const double* rho,
                        double* out) {
  for (int64_t i = 0; i < n_obs; i++) {
    double acc = 0.0;
    for (int64_t j = 0; j < m; j++) {
      const double* p = prisms + 6 * j;
      if (p[0] == p[1] || p[2] == p[3] || p[4] == p[5] || rho[j] == 0.0) continue;
      Rel q{p[0] - e[i], p[1] - e[i], p[2] - n[i], p[3] - n[i], p[4] - u[i], p[5] - u[i]};
      double v = pair_any(field, q);
      if (field >= kGee && singular_for(field, q)) v = quiet_nan();
      acc += rho[j] * v;
    }
    out[i] = acc * field_scale(field);
  }
}

}
