// gen_rhg.cu -- threshold random hyperbolic graph generator.
//
// Stand-in for KaGen's get_rhg (benchmarks/mst_benchmarks.hpp:152-158), which
// the reference tree does not vendor; the reference exposes --gamma
// (mst_benchmarks.hpp:71).  Definition (shared with the oracle's CPU
// generator, oracle/oracle.cpp):
//   alpha = (gamma - 1) / 2, xi = alpha / (alpha - 1/2),
//   R = max(1, 2 ln(2 xi^2 n / (pi k)))  (asymptotic threshold-RHG degree
//   formula, k = target average degree);
//   point i: u, v from SplitMix64 (53-bit uniforms), r = min(R, acosh(1 +
//   u (cosh(alpha R) - 1)) / alpha), theta = 2 pi v; per point E = e^r,
//   Ei = e^-r, S = sinh r; band = min(15, floor(16 r / R));
//   ids = ranks of the points sorted by (band, bits(theta) >> 5, i);
//   p ~ q (a = lower id) iff ((2 s) s) S_a S_b <= cosh R - 0.5 (E_a Ei_b +
//   Ei_a E_b), s = hsin(d / 2), d the angular distance in [0, pi], hsin a
//   fixed degree-21 Taylor polynomial of sin.
// The per-point values use the C library's acosh / exp / sinh on the host
// (the same functions the oracle calls, built without FMA contraction); the
// pair test runs on the device with explicitly rounded double operations in
// the definition's order, so GPU and oracle agree bit for bit.
//
// Device steps: keys -> radix sort -> gather the per-point values into id
// order -> band starts -> per-vertex degree over angular windows -> scan ->
// write.  A window of band b around theta_p contains every q with
// r_q >= r_lo(b) that the test can accept: sin^2(d/2) <= cosh R /
// (2 S_p sinh r_lo(b)), widened by 1e-6 relative and 1e-9 absolute.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "common.cuh"
#include "gen_scratch.cuh"
#include "solver.cuh"
#include "sort_gen.cuh"

namespace kamsta {

namespace {

constexpr int kBands = 16;
constexpr double kTwoPiD = 6.283185307179586;
constexpr double kPiD = 3.141592653589793;

struct BandTable {
  double sh_lo[kBands];
  uint32_t start[kBands + 1];
};

__device__ __forceinline__ double hsin_rn(double x) {
  const double x2 = __dmul_rn(x, x);
  double t = __dsub_rn(1.0, __ddiv_rn(x2, 420.0));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 342.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 272.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 210.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 156.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 110.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 72.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 42.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 20.0), t));
  t = __dsub_rn(1.0, __dmul_rn(__ddiv_rn(x2, 6.0), t));
  return __dmul_rn(x, t);
}

struct RhgView {
  const double* theta;
  const double* E;
  const double* Ei;
  const double* S;
  const uint64_t* key;  // sorted keys (band << 58 | bits(theta) >> 5)
};

__device__ __forceinline__ bool rhg_edge_rn(const RhgView& v, uint32_t a, uint32_t b,
                                            double coshR) {
  const double ta = v.theta[a], tb = v.theta[b];
  double d = ta > tb ? __dsub_rn(ta, tb) : __dsub_rn(tb, ta);
  if (d > kPiD) d = __dsub_rn(kTwoPiD, d);
  const double s = hsin_rn(__dmul_rn(d, 0.5));
  const double lhs = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, s), s), v.S[a]), v.S[b]);
  const double rhs = __dsub_rn(
      coshR, __dmul_rn(0.5, __dadd_rn(__dmul_rn(v.E[a], v.Ei[b]), __dmul_rn(v.Ei[a], v.E[b]))));
  return lhs <= rhs;
}

__device__ __forceinline__ uint64_t tkey(double t) {
  return static_cast<uint64_t>(__double_as_longlong(t)) >> 5;
}

// first index in [lo, hi) with key >= x
__device__ __forceinline__ uint32_t lower_idx(const uint64_t* k, uint32_t lo, uint32_t hi,
                                              uint64_t x) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (k[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void k_rhg_place(const uint32_t* __restrict__ perm, uint32_t n,
                            const double* __restrict__ in4, double* __restrict__ out4) {
  // in4 / out4: theta, E, Ei, S arrays of n doubles each, back to back
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t i = perm[j];
#pragma unroll
    for (int f = 0; f < 4; ++f) out4[f * uint64_t(n) + j] = in4[f * uint64_t(n) + i];
  }
}

__global__ void k_rhg_bands(const uint64_t* keys, uint32_t n, uint32_t* start) {
  const int b = threadIdx.x;
  if (b > kBands) return;
  start[b] = lower_idx(keys, 0, n, static_cast<uint64_t>(b) << 58);
}

template <bool WRITE>
__global__ void __launch_bounds__(256)
    k_rhg_edges(RhgView v, uint32_t n, BandTable bt, const uint32_t* __restrict__ bstart,
                double coshR, uint32_t* __restrict__ deg, const uint32_t* __restrict__ off,
                uint64_t wseed, uint32_t max_weight, uint32_t* __restrict__ out) {
  for (uint64_t jj = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; jj < n;
       jj += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t j = static_cast<uint32_t>(jj);
    const double th = v.theta[j], Sp = v.S[j];
    uint64_t o = WRITE ? off[j] : 0;
    uint32_t d = 0;
    for (int b = 0; b < kBands; ++b) {
      const uint32_t b0 = bstart[b], b1 = bstart[b + 1];
      if (b0 == b1) continue;
      bool full = bt.sh_lo[b] <= 0.0 || Sp <= 0.0;
      double D = 0.0;
      if (!full) {
        const double s = sqrt(coshR / (2.0 * Sp * bt.sh_lo[b])) * (1.0 + 1e-6);
        if (s >= 1.0) {
          full = true;
        } else {
          D = 2.0 * asin(s) + 1e-9;
          if (D >= kPiD) full = true;
        }
      }
      uint32_t r[4] = {b0, b1, b0, b0};
      if (!full) {
        const uint64_t bk = static_cast<uint64_t>(b) << 58;
        const double lo = th - D, hi = th + D;
        auto rng = [&](double t0, double t1, uint32_t* x0, uint32_t* x1) {
          *x0 = lower_idx(v.key, b0, b1, bk | tkey(t0));
          *x1 = lower_idx(v.key, *x0, b1, (bk | tkey(t1)) + 1);
        };
        if (lo < 0.0) {
          rng(0.0, hi, &r[0], &r[1]);
          rng(lo + kTwoPiD, kTwoPiD, &r[2], &r[3]);
        } else if (hi >= kTwoPiD) {
          rng(0.0, hi - kTwoPiD, &r[0], &r[1]);
          rng(lo, kTwoPiD, &r[2], &r[3]);
        } else {
          rng(lo, hi, &r[0], &r[1]);
        }
      }
      for (int part = 0; part < 2; ++part) {
        for (uint32_t k = r[2 * part]; k < r[2 * part + 1]; ++k) {
          if (k == j) continue;
          const bool e = j < k ? rhg_edge_rn(v, j, k, coshR) : rhg_edge_rn(v, k, j, coshR);
          if (!e) continue;
          if (WRITE) {
            const uint64_t lo = j < k ? j : k, hi = j < k ? k : j;
            const uint64_t canon = (lo << 32) | hi;
            out[3 * o] = j;
            out[3 * o + 1] = k;
            out[3 * o + 2] =
                1u + static_cast<uint32_t>(__umul64hi(mix64(wseed ^ canon), max_weight));
            ++o;
          }
          ++d;
        }
      }
    }
    if (!WRITE) deg[j] = d;
  }
}

}  // namespace

kamsta_status gen_rhg(kamsta_ctx* ctx, uint32_t n, double gamma, double avg_degree, uint64_t seed,
                      uint32_t max_weight, kamsta_wedge* d_out, uint64_t capacity,
                      uint64_t* m_out, cudaStream_t st) {
  *m_out = 0;
  if (max_weight == 0 || !(gamma > 2.0) || !(avg_degree > 0.0)) {
    set_error("gen_rhg: needs gamma > 2, avg_degree > 0, max_weight >= 1");
    return KAMSTA_E_INPUT;
  }
  if (n == 0) return KAMSTA_OK;
  const double alpha = (gamma - 1.0) / 2.0;
  const double xi = alpha / (alpha - 0.5);
  double R = 2.0 * std::log(2.0 * xi * xi * n / (kPiD * avg_degree));
  if (!(R > 1.0)) R = 1.0;
  const double coshR = std::cosh(R), coshAR1 = std::cosh(alpha * R) - 1.0;
  const uint64_t base = mix64(seed ^ 0x524847ull);
  const uint64_t wseed = mix64(seed ^ 0x6a09e667f3bcc909ull);
  // ---- per-point values on the host (C library functions, as the oracle)
  std::vector<double> h4(4 * static_cast<size_t>(n));
  std::vector<uint64_t> hkey(n);
  {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < hw; ++t)
      th.emplace_back([&, t] {
        const uint64_t lo = uint64_t(n) * t / hw, hi = uint64_t(n) * (t + 1) / hw;
        for (uint64_t i = lo; i < hi; ++i) {
          const double u = static_cast<double>(mix64(base + 2 * i) >> 11) * 0x1.0p-53;
          const double v = static_cast<double>(mix64(base + 2 * i + 1) >> 11) * 0x1.0p-53;
          double r = std::acosh(1.0 + u * coshAR1) / alpha;
          if (r > R) r = R;
          const double theta = kTwoPiD * v;
          h4[i] = theta;
          h4[n + i] = std::exp(r);
          h4[2 * uint64_t(n) + i] = std::exp(-r);
          h4[3 * uint64_t(n) + i] = std::sinh(r);
          int band = static_cast<int>(std::floor(r * kBands / R));
          if (band > kBands - 1) band = kBands - 1;
          if (band < 0) band = 0;
          uint64_t tb;
          std::memcpy(&tb, &theta, sizeof(tb));
          hkey[i] = (static_cast<uint64_t>(band) << 58) | (tb >> 5);
        }
      });
    for (auto& x : th) x.join();
  }
  BandTable bt;
  for (int b = 0; b < kBands; ++b) bt.sh_lo[b] = std::sinh(R * b / kBands);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8;
  GenBuf bk, bk2, bp, bp2, bin4, bout4, bst, bdeg, boff, bcnt, bstat, bsmall;
  uint64_t *keys, *keys2, *status;
  uint32_t *perm, *perm2, *bstart, *deg, *off, *counts;
  double *in4, *out4;
  unsigned long long* small;
  GEN_CHECK(bk.alloc(ctx, st, &keys, n));
  GEN_CHECK(bk2.alloc(ctx, st, &keys2, n));
  GEN_CHECK(bp.alloc(ctx, st, &perm, n));
  GEN_CHECK(bp2.alloc(ctx, st, &perm2, n));
  GEN_CHECK(bin4.alloc(ctx, st, &in4, 4 * uint64_t(n)));
  GEN_CHECK(bout4.alloc(ctx, st, &out4, 4 * uint64_t(n)));
  GEN_CHECK(bst.alloc(ctx, st, &bstart, kBands + 1));
  const RadixScratch rs = radix_scratch_bytes(n);
  GEN_CHECK(bcnt.alloc(ctx, st, &counts, std::max<uint64_t>(rs.counts, n)));
  GEN_CHECK(bstat.alloc(ctx, st, &status, std::max<uint64_t>(rs.status, n / 2048 + 2)));
  GEN_CHECK(bsmall.alloc(ctx, st, &small, 8));
  uint32_t* ticket = reinterpret_cast<uint32_t*>(small + 4);
  uint32_t* err = reinterpret_cast<uint32_t*>(small + 5);
  GEN_CHECK(cudaMemsetAsync(small, 0, 8 * sizeof(unsigned long long), st));
  GEN_CHECK(cudaMemcpyAsync(keys, hkey.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice, st));
  GEN_CHECK(cudaMemcpyAsync(in4, h4.data(), sizeof(double) * 4 * uint64_t(n),
                          cudaMemcpyHostToDevice, st));
  {
    std::vector<uint32_t> iota(n);
    for (uint32_t i = 0; i < n; ++i) iota[i] = i;
    GEN_CHECK(cudaMemcpyAsync(perm, iota.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
    int alt = 0;
    GEN_CHECK(radix_sort_pairs_u32(st, keys, keys2, perm, perm2, n, 62, counts, status, ticket, err,
                                 &alt, sms));
    if (alt) {
      std::swap(keys, keys2);
      std::swap(perm, perm2);
    }
    GEN_CHECK(cudaStreamSynchronize(st));  // iota (pageable) is done
  }
  k_rhg_place<<<grid, 256, 0, st>>>(perm, n, in4, out4);
  k_rhg_bands<<<1, 32, 0, st>>>(keys, n, bstart);
  RhgView v{out4, out4 + n, out4 + 2 * uint64_t(n), out4 + 3 * uint64_t(n), keys};
  GEN_CHECK(bdeg.alloc(ctx, st, &deg, n));
  GEN_CHECK(boff.alloc(ctx, st, &off, n));
  k_rhg_edges<false><<<grid, 256, 0, st>>>(v, n, bt, bstart, coshR, deg, nullptr, wseed,
                                           max_weight, nullptr);
  GEN_CHECK(exclusive_scan_u32(st, deg, off, n, status, ticket, err, sms));
  GEN_CHECK(sum_u32(st, deg, n, small, sms));
  unsigned long long total = 0;
  uint32_t herr = 0;
  GEN_CHECK(cudaMemcpyAsync(&total, small, sizeof(total), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaStreamSynchronize(st));
  GEN_CHECK(cudaGetLastError());
  if (herr) {
    set_error("gen_rhg: device wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  if (total >= (1ull << 32)) {
    set_error("gen_rhg: more than 2^32 directed entries");
    return KAMSTA_E_INPUT;
  }
  *m_out = total;
  if (!d_out) return KAMSTA_OK;
  if (total > capacity) {
    set_error("gen_rhg: output capacity too small (required count in m_directed_out)");
    return KAMSTA_E_INPUT;
  }
  k_rhg_edges<true><<<grid, 256, 0, st>>>(v, n, bt, bstart, coshR, deg, off, wseed, max_weight,
                                          reinterpret_cast<uint32_t*>(d_out));
  GEN_CHECK(cudaGetLastError());
  GEN_CHECK(cudaStreamSynchronize(st));
  return KAMSTA_OK;
}

}  // namespace kamsta

extern "C" kamsta_status kamsta_gen_rhg_dev(kamsta_ctx* ctx, uint32_t n, double gamma,
                                            double avg_degree, uint64_t seed, uint32_t max_weight,
                                            kamsta_wedge* d_out, uint64_t capacity,
                                            uint64_t* m_directed_out, kamsta_stream stream) {
  if (!m_directed_out) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (ctx ? ctx->stream : nullptr);
  return kamsta::gen_rhg(ctx, n, gamma, avg_degree, seed, max_weight, d_out, capacity,
                         m_directed_out, st);
}
