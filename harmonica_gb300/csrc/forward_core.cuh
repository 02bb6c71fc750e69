// Building blocks shared by the forward kernels (prism_forward.cu) and the
// batched persistent kernel (prism_batch.cu): prism sources, the staging of
// prism tiles and math tables in shared memory, and the inner loop that adds
// the field of a range of prisms to one observation point per thread.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

#include "prism_math.cuh"

namespace hg {

constexpr int kThreads = 128;  // observation points per CTA
constexpr int kTile = 128;     // prisms staged per shared-memory tile
constexpr int kSmCount = 152;

template <int F> struct NumOut { static constexpr int value = 1; };
template <> struct NumOut<kAll> { static constexpr int value = kNumFields; };

HG_HD __forceinline__ bool is_tensor(int f) { return f >= kGee && f <= kGnz; }

// Resident CTAs per SM the register allocation must allow (more warps hide
// the arithmetic latency; the fused all-field kernel needs more registers).
// Measured on the 1e6-prism layer: the tensor kernels at 6 (80 registers)
// run g_zz 3 % faster than at 5; the first-derivative kernels (g_e, g_n,
// g_z: merged logs and faces) at 5 (96 registers, less than half the
// spills) run 4 % faster than at 6.
#ifndef HG_FWD_MIN_BLOCKS
#define HG_FWD_MIN_BLOCKS 6
#endif
#ifndef HG_FWD_MIN_BLOCKS_GRAD
#define HG_FWD_MIN_BLOCKS_GRAD 5
#endif
#ifndef HG_FWD_MIN_BLOCKS_ALL
#define HG_FWD_MIN_BLOCKS_ALL 4
#endif
// the persistent batch and serving-round kernels (prism_batch.cu), tuned at 5
#ifndef HG_BATCH_MIN_BLOCKS
#define HG_BATCH_MIN_BLOCKS 5
#endif
template <int F> struct MinBlocks {
  static constexpr int value =
      (F == kGe || F == kGn || F == kGz) ? HG_FWD_MIN_BLOCKS_GRAD : HG_FWD_MIN_BLOCKS;
};
template <> struct MinBlocks<kAll> { static constexpr int value = HG_FWD_MIN_BLOCKS_ALL; };
// the potential needs every log and face angle, like the fused kernel
template <> struct MinBlocks<kPotential> { static constexpr int value = HG_FWD_MIN_BLOCKS_ALL; };
// the two launches of the potential and fused all-field forwards (PART 1, 2)
#ifndef HG_FWD_MIN_BLOCKS_PART
#define HG_FWD_MIN_BLOCKS_PART 4
#endif
template <int F, int PART> struct PartMinBlocks {
  static constexpr int value = PART == 0 ? MinBlocks<F>::value : HG_FWD_MIN_BLOCKS_PART;
};
// the tensor components' batch and round kernels at 6, like their forward
// kernels (the batched g_z/g_zz workload 1 % faster than at 5)
#ifndef HG_BATCH_MIN_BLOCKS_TENSOR
#define HG_BATCH_MIN_BLOCKS_TENSOR 6
#endif
template <int F> struct BatchMinBlocks {
  static constexpr int value = F >= kGee ? HG_BATCH_MIN_BLOCKS_TENSOR : HG_BATCH_MIN_BLOCKS;
};
template <> struct BatchMinBlocks<kAll> { static constexpr int value = HG_FWD_MIN_BLOCKS_ALL; };
template <> struct BatchMinBlocks<kPotential> {
  static constexpr int value = HG_FWD_MIN_BLOCKS_ALL;
};


// ---------------------------------------------------------------------------
// Prism sources: how a CTA loads prism p into shared memory.
struct ListSource {
  const double* soa;  // 7 rows (w, e, s, n, b, t, rho) of `stride` doubles
  int64_t stride;
  __device__ __forceinline__ void load(int64_t p, double& w, double& e, double& s, double& n,
                                       double& b, double& t, double& rho, bool& null) const {
    w = soa[p];
    e = soa[stride + p];
    s = soa[2 * stride + p];
    n = soa[3 * stride + p];
    b = soa[4 * stride + p];
    t = soa[5 * stride + p];
    rho = soa[6 * stride + p];
    // gravity.py:475-480: zero volume or zero density
    null = (w == e) || (s == n) || (b == t) || (rho == 0.0);
  }
};

struct LayerSource {
  const double* ce;
  const double* cn;
  const double* bottom;
  const double* top;
  const double* density;
  int64_t n_east;
  double threshold;
  __device__ __forceinline__ void load(int64_t p, double& w, double& e, double& s, double& n,
                                       double& b, double& t, double& rho, bool& null) const {
    // half spacings from the first two centres, as layer.py:582-583
    const double half_e = (ce[1] - ce[0]) / 2.0;
    const double half_n = (cn[1] - cn[0]) / 2.0;
    const int64_t k = p / n_east, j = p - k * n_east;
    w = ce[j] - half_e;
    e = ce[j] + half_e;
    s = cn[k] - half_n;
    n = cn[k] + half_n;
    b = bottom[p];
    t = top[p];
    rho = density[p];
    // layer.py:596-607; zero-thickness prisms add exactly zero and are skipped too
    null = (rho == 0.0) || isnan(rho) || (t - b < threshold) || isnan(t) || isnan(b) || (b == t);
  }
};

// ---------------------------------------------------------------------------
// A tile of TILE prisms staged in shared memory (structure of arrays).
template <int TILE>
struct SmemTileT {
  double w[TILE], e[TILE], s[TILE], n[TILE], b[TILE], t[TILE], rho[TILE];
  double dx[TILE], dy[TILE], dz[TILE];  // extents
  float rhoh[TILE], rhol[TILE];         // the density as a float pair
  int null[TILE];
  int rnat[TILE];                       // density within 2^-40..2^40 (nat_fields)
};

// Float-pair sums of the potential and fused all-field launches (PART 1, 2):
// each pair's fields on float pairs in natural units (times the density, a
// float pair too) are added to per-thread float-pair sums, which are added to
// the FP64 sums once per prism tile -- in place of a float-pair -> double
// conversion (~25 integer instructions) and an FP64 FMA per field and pair.
// A float-pair sum of at most one tile of terms keeps ~2^-46 of its value.
// The fields each part carries: the potential and the three first
// derivatives, then the three off-diagonal (part 1) or diagonal (part 2)
// tensor components.
template <bool ALL, int PART> struct NatFields {
  static constexpr int n = ALL ? 7 : 1;
  static HG_HD __forceinline__ int field(int k) {
    return k < 4 ? k : (PART == 1 ? kGen + (k - 4) : kGee + (k - 4));
  }
};
// Pairs whose scale exponent e1 = top - 1023 is within +-30 and whose
// density is within 2^-40..2^40 keep every natural-unit value and product
// in the normal float range (the potential scales as 2^(2 e1)).
constexpr int kNatMaxExp = 30;
using SmemTile = SmemTileT<kTile>;

struct SmemTables {
  double logc[lean::kLogTableSize], logl[lean::kLogTableSize];
  double th[lean::kArgTableSize];
  float csf[2 * lean::kArgTableSize], snf[2 * lean::kArgTableSize];
  float loglf[2 * lean::kLogTableSize], thf[2 * lean::kArgTableSize];

  // Copy the constant tables of lean_math.cuh; the caller synchronises.
  __device__ __forceinline__ Tables stage() {
    for (int t = threadIdx.x; t < lean::kLogTableSize; t += blockDim.x) {
      logc[t] = lean::kLogC[t];
      logl[t] = lean::kLogL[t];
    }
    for (int t = threadIdx.x; t < lean::kArgTableSize; t += blockDim.x) th[t] = lean::kArgTh[t];
    for (int t = threadIdx.x; t < 2 * lean::kArgTableSize; t += blockDim.x) {
      csf[t] = lean::kArgCosF[t];
      snf[t] = lean::kArgSinF[t];
      thf[t] = lean::kArgThF[t];
    }
    for (int t = threadIdx.x; t < 2 * lean::kLogTableSize; t += blockDim.x) loglf[t] = lean::kLogLF[t];
    return Tables{logc, logl, th, csf, snf, loglf, thf};
  }
};

// Adds to acc[] the field(s) F of prisms [p0, p1) of `src` at this thread's
// point (pe, pn, pu), staging TILE prisms at a time (the CTA has TILE
// threads).  Must be called by every thread of the CTA (it synchronises
// around each shared-memory tile).  With check_singular, ORs into `singular`
// whether the point is a singular point of any prism (null prisms included,
// as gravity.py:207-214 scans before discarding) for the tensor fields in
// sing_mask.  Tensor values at singular points are NaN.
// PART (all fields and the potential): 0 adds the whole pair; 1 its edge-log
// terms, and the whole pair for the pairs the float-pair form declines or
// that fail faces_fit_f2; 2 its face terms, nothing for those pairs.  Parts
// 1 and 2 run as two launches whose sums add up to part 0's, each with about
// half of the hot loop's code: the whole loop outgrows the instruction
// cache and both kernels then wait on instruction fetch.
template <int F, class Source, int TILE = kTile, int PART = 0>
__device__ __forceinline__ void accumulate(const Source& src, int64_t p0, int64_t p1, double pe,
                                           double pn, double pu, bool active, bool check_singular,
                                           uint32_t sing_mask, SmemTileT<TILE>& sh,
                                           const Tables& T, double* acc, bool& singular) {
  for (int64_t base = p0; base < p1; base += TILE) {
    const int cnt = (int)min((int64_t)TILE, p1 - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      double w, e, s, n, b, t, rho;
      bool null;
      src.load(base + threadIdx.x, w, e, s, n, b, t, rho, null);
      sh.w[threadIdx.x] = w;
      sh.e[threadIdx.x] = e;
      sh.s[threadIdx.x] = s;
      sh.n[threadIdx.x] = n;
      sh.b[threadIdx.x] = b;
      sh.t[threadIdx.x] = t;
      sh.rho[threadIdx.x] = rho;
      sh.dx[threadIdx.x] = e - w;
      sh.dy[threadIdx.x] = n - s;
      sh.dz[threadIdx.x] = t - b;
      sh.null[threadIdx.x] = null;
      if (PART != 0) {
        const long long rb = lean::d2ll(rho);
        const int re = (int)((rb >> 52) & 0x7ff);
        const lean::F2 rf = lean::scaled_f2(rb, 1023);
        sh.rhoh[threadIdx.x] = rf.h;
        sh.rhol[threadIdx.x] = rf.l;
        sh.rnat[threadIdx.x] = re >= 1023 - 40 && re <= 1023 + 40;
      }
    }
    __syncthreads();
    constexpr int NNAT = (F == kAll || F == kPotential) && PART != 0
                             ? NatFields<F == kAll, PART>::n : 1;
    lean::F2 nat[NNAT];
#pragma unroll
    for (int k = 0; k < NNAT; k++) nat[k] = lean::F2{0.0f, 0.0f};
    for (int p = 0; p < cnt; p++) {
      Rel q;
      q.x1 = sh.w[p] - pe;
      q.x2 = sh.e[p] - pe;
      q.y1 = sh.s[p] - pn;
      q.y2 = sh.n[p] - pn;
      q.z1 = sh.b[p] - pu;
      q.z2 = sh.t[p] - pu;
      q.dx = sh.dx[p];
      q.dy = sh.dy[p];
      q.dz = sh.dz[p];
      if (check_singular && active) {
#pragma unroll
        for (int f = kGee; f <= kGnz; f++)
          if ((sing_mask >> f) & 1u) singular |= singular_for(f, q);
      }
      if (sh.null[p]) continue;  // uniform across the CTA
      const double rho = sh.rho[p];
      if (F == kAll || F == kPotential) {
        // The float-pair form needs only the float-pair geometry: the FP64
        // bounds are dead after make_geom_f2 (fewer live registers through
        // the long evaluation) and are rebuilt from shared memory for the
        // rare pair it declines (a zero or tiny bound), which is also the
        // only kind of pair that can lie on a singular point.
        constexpr bool ALL = F == kAll;
        double v[ALL ? kNumFields : 1];
        GeomF2 g;
        bool fast = !any_zero_bound(q) && make_geom_f2(q, g);
        if (PART != 0) fast = fast && faces_fit_f2(g);
        if (PART != 0 && (PART == 2 || fast)) {
          // part 2 skips the pairs part 1 evaluated whole; the faces of the
          // others fit, so neither part declines them
          if (!fast) continue;
          using NF = NatFields<ALL, PART>;
          lean::F2 r[ALL ? kNumFields : 1];
          pair_all_f2_raw<ALL, PART>(g, T, r);
          const int e1 = g.top - 1023;
          if (sh.rnat[p] && e1 >= -kNatMaxExp && e1 <= kNatMaxExp) {
            using namespace lean;
            const float s1 = pow2f(e1), s2 = pow2f(2 * e1);
            const F2 rf{sh.rhoh[p], sh.rhol[p]};
            const P2 rr = pk(rf, rf);
            if constexpr (!ALL) {
              nat[0] = f2_add(nat[0], f2_mul(rf, F2{fmul(r[0].h, s2), fmul(r[0].l, s2)}));
            } else {
              // (potential, g_e), (g_n, g_z), two tensor components, then one
              const P2 a = p2_mul(rr, p2_scale(pk(r[kPotential], r[NF::field(1)]), mk2(s2, s1)));
              const P2 na = p2_add(pk(nat[0], nat[1]), a);
              nat[0] = lane0(na);
              nat[1] = lane1(na);
              const P2 b = p2_mul(rr, p2_scale(pk(r[NF::field(2)], r[NF::field(3)]), sp2(s1)));
              const P2 nb = p2_add(pk(nat[2], nat[3]), b);
              nat[2] = lane0(nb);
              nat[3] = lane1(nb);
              const P2 c = p2_mul(rr, pk(r[NF::field(4)], r[NF::field(5)]));
              const P2 nc = p2_add(pk(nat[4], nat[5]), c);
              nat[4] = lane0(nc);
              nat[5] = lane1(nc);
              nat[6] = f2_add(nat[6], f2_mul(rf, r[NF::field(6)]));
            }
          } else {
#pragma unroll
            for (int k = 0; k < NF::n; k++) {
              const int f = NF::field(k);
              acc[f] = fma(rho, f2_to_double(r[f], raw_exponent(f, e1)), acc[f]);
            }
          }
          continue;
        }
        if (!(fast && pair_all_f2_geom<ALL, PART>(g, T, v))) {
          const volatile double* vs = &sh.w[p];  // forces the reload (no reuse of q)
          Rel r;
          r.x1 = vs[0] - pe;
          r.x2 = sh.e[p] - pe;
          r.y1 = sh.s[p] - pn;
          r.y2 = sh.n[p] - pn;
          r.z1 = sh.b[p] - pu;
          r.z2 = sh.t[p] - pu;
          r.dx = sh.dx[p];
          r.dy = sh.dy[p];
          r.dz = sh.dz[p];
          if (ALL) {
            pair_all_fp64(r, T, v);
#pragma unroll
            for (int f = kGee; f <= kGnz; f++)
              if (singular_for(f, r)) v[ALL ? f : 0] = quiet_nan();
          } else {
            v[0] = pair_field_fp64<kPotential>(r, T);
          }
        }
#pragma unroll
        for (int f = 0; f < (ALL ? kNumFields : 1); f++) acc[f] = fma(rho, v[f], acc[f]);
      } else {
        double v = pair_field<(F < kNumFields ? F : 0), true>(q, T);
        if (is_tensor(F) && singular_for(F, q)) v = quiet_nan();
        acc[0] = fma(rho, v, acc[0]);
      }
    }
    if ((F == kAll || F == kPotential) && PART != 0) {
#pragma unroll
      for (int k = 0; k < NNAT; k++)
        acc[NatFields<F == kAll, PART>::field(k)] += lean::f2_to_double(nat[k], 0);
    }
  }
}

// Full waves of resident CTAs a chunked launch is cut into (HG_FWD_WAVES,
// default 32).  Short CTAs even out the SMs' progress and shrink the last,
// partial wave: on the g_z layer step 1 wave gave 1.09e10 pairs/s, 32 waves
// 1.21e10.
inline int64_t launch_waves() {
  static const int64_t waves = [] {
    const char* v = std::getenv("HG_FWD_WAVES");
    const long w = v ? std::strtol(v, nullptr, 10) : 32;
    return (int64_t)(w >= 1 && w <= 256 ? w : 32);
  }();
  return waves;
}

namespace {

// out[idx] = scale * (sum over c of part[c * stride + idx]) for idx < total:
// 32 outputs per block, thread (x, y) adds the chunks y, y + 16, ... of
// output x (coalesced rows), then the 16 group sums are added in order of y
// -- a fixed order for a given chunk count (deterministic) with 16x the
// memory parallelism of one thread walking all chunks.
constexpr int kSumGroups = 16;

__global__ void __launch_bounds__(32 * kSumGroups) chunk_sum_kernel(
    const double* __restrict__ part, int64_t n_chunks, int64_t stride, int64_t total,
    double scale, double* __restrict__ out) {
  __shared__ double group[kSumGroups][32];
  const int64_t idx = (int64_t)blockIdx.x * 32 + threadIdx.x;
  double s = 0.0;
  if (idx < total)
    for (int64_t c = threadIdx.y; c < n_chunks; c += kSumGroups) s += part[c * stride + idx];
  group[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && idx < total) {
    double t = 0.0;
#pragma unroll
    for (int g = 0; g < kSumGroups; g++) t += group[g][threadIdx.x];
    out[idx] = t * scale;
  }
}

inline void launch_chunk_sum(const double* part, int64_t n_chunks, int64_t stride, int64_t total,
                             double scale, double* out, cudaStream_t st) {
  chunk_sum_kernel<<<(unsigned)((total + 31) / 32), dim3(32, kSumGroups), 0, st>>>(
      part, n_chunks, stride, total, scale, out);
}

}  // namespace

}  // namespace hg
