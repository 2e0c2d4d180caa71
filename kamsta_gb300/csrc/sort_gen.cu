// sort_gen.cu -- host side of the radix sort and the device G(n,m) generator.
//
// The generator stands in for KaGen's get_gnm (benchmarks/mst_benchmarks.hpp:
// 126-132), which the reference tree does not vendor.  Its definition is
// shared with the oracle's CPU generator (oracle/oracle.cpp):
//   mix64 = SplitMix64's output function; base = mix64(seed);
//   candidate i: u = hi64(mix64(base + 2i) * n), v = hi64(mix64(base + 2i + 1) * n);
//   the graph = the first m distinct valid (u != v) unordered pairs in
//   candidate order; w = 1 + hi64(mix64(wseed ^ (min << 32 | max)) * max_weight),
//   wseed = mix64(seed ^ 0x6a09e667f3bcc909); both directions, (src,dst) sorted.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "radix_sort.cuh"
#include "sort_gen.cuh"
#include "solver.cuh"

namespace kamsta {

static inline uint32_t cdiv(uint64_t a, uint64_t b) { return static_cast<uint32_t>((a + b - 1) / b); }

RadixScratch radix_scratch_bytes(uint64_t n) {
  RadixScratch r;
  const uint32_t nt = cdiv(n, kRsTile);
  r.counts = static_cast<uint64_t>(nt) * 256;
  r.status = cdiv(r.counts, kScanTile) + 1;
  return r;
}

template <typename V>
static cudaError_t radix_sort_impl(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt, V* vals,
                                   V* vals_alt, uint64_t n, int bits, uint32_t* counts,
                                   uint64_t* status, uint32_t* ticket, uint32_t* err,
                                   int* result_alt, int sms) {
  *result_alt = 0;
  if (n <= 1 || bits <= 0) return cudaSuccess;
  // the per-tile digit offsets and the scan are 32-bit: refuse 2^32 or more
  // keys rather than wrap (every caller sorts fewer: lists and generators
  // stay below 2^32 entries)
  if (n >= (1ull << 32)) return cudaErrorInvalidValue;
  // the upsweep reads key pairs with 128-bit loads
  if ((reinterpret_cast<uintptr_t>(keys) | reinterpret_cast<uintptr_t>(keys_alt)) & 15u)
    return cudaErrorMisalignedAddress;
  const uint32_t nt = cdiv(n, kRsTile);
  const uint64_t ncounts = static_cast<uint64_t>(nt) * 256;
  const uint32_t nst = cdiv(ncounts, kScanTile);
  const size_t dyn = sizeof(uint64_t) * kRsTile + ValTraits<V>::kSize * kRsTile;
  cudaError_t e = cudaFuncSetAttribute(k_rs_downsweep<V>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(dyn));
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rs_downsweep<V>, kRsBlock, dyn);
  per_sm = std::max(per_sm, 1);
  const int gdown = static_cast<int>(std::min<uint64_t>(nt, uint64_t(per_sm) * sms));
  const int gup = static_cast<int>(std::min<uint64_t>(nt, uint64_t(sms) * 4));
  const int gscan = static_cast<int>(std::min<uint64_t>(nst, uint64_t(sms) * 4));
  uint64_t *kin = keys, *kout = keys_alt;
  V *vin = vals, *vout = vals_alt;
  int alt = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_upsweep<<<gup, kRsBlock, 0, st>>>(kin, n, shift, nt, counts);
    cudaMemsetAsync(status, 0, sizeof(uint64_t) * nst, st);
    cudaMemsetAsync(ticket, 0, sizeof(uint32_t), st);
    k_scan_u32<<<gscan, kRsBlock, 0, st>>>(counts, counts, ncounts, status, ticket, nst, err);
    k_rs_downsweep<V><<<gdown, kRsBlock, dyn, st>>>(kin, vin, kout, vout, n, shift, nt, counts);
    std::swap(kin, kout);
    std::swap(vin, vout);
    alt ^= 1;
  }
  *result_alt = alt;
  return cudaGetLastError();
}

cudaError_t radix_sort_keys(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt, uint64_t n,
                            int bits, uint32_t* counts, uint64_t* status, uint32_t* ticket,
                            uint32_t* err, int* result_alt, int sms) {
  return radix_sort_impl<NoVal>(st, keys, keys_alt, nullptr, nullptr, n, bits, counts, status,
                                ticket, err, result_alt, sms);
}
cudaError_t radix_sort_pairs_u32(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt,
                                 uint32_t* vals, uint32_t* vals_alt, uint64_t n, int bits,
                                 uint32_t* counts, uint64_t* status, uint32_t* ticket,
                                 uint32_t* err, int* result_alt, int sms) {
  return radix_sort_impl<uint32_t>(st, keys, keys_alt, vals, vals_alt, n, bits, counts, status,
                                   ticket, err, result_alt, sms);
}
cudaError_t radix_sort_pairs_u64(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt,
                                 uint64_t* vals, uint64_t* vals_alt, uint64_t n, int bits,
                                 uint32_t* counts, uint64_t* status, uint32_t* ticket,
                                 uint32_t* err, int* result_alt, int sms) {
  return radix_sort_impl<uint64_t>(st, keys, keys_alt, vals, vals_alt, n, bits, counts, status,
                                   ticket, err, result_alt, sms);
}

// ---------------------------------------------------------------------------
// G(n,m) generator kernels

__global__ void k_gnm_candidates(uint64_t first, uint64_t count, uint64_t base, uint32_t n,
                                 uint32_t b, uint64_t* keys, uint32_t* idx) {
  const uint64_t invalid = (b == 32) ? ~0ull : ((1ull << (2 * b)) - 1);
  for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < count;
       t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t i = first + t;
    const uint32_t u = static_cast<uint32_t>(__umul64hi(mix64(base + 2 * i), n));
    const uint32_t v = static_cast<uint32_t>(__umul64hi(mix64(base + 2 * i + 1), n));
    uint64_t key = invalid;
    if (u != v) key = (static_cast<uint64_t>(min(u, v)) << b) | max(u, v);
    keys[t] = key;
    idx[t] = static_cast<uint32_t>(i);
  }
}

// flag[idx[j]] = 1 for the first entry of every run of equal valid keys
__global__ void k_gnm_first(const uint64_t* keys, const uint32_t* idx, uint64_t K,
                            uint64_t invalid, uint32_t* flag) {
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < K;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[j];
    if (k != invalid && (j == 0 || keys[j - 1] != k)) flag[idx[j]] = 1u;
  }
}

// T = candidate index of the m-th first occurrence; total = number of them
__global__ void k_gnm_threshold(const uint32_t* flag, const uint32_t* excl, uint64_t K,
                                uint64_t m, unsigned long long* out) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < K;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    if (flag[i] && excl[i] + 1ull == m) out[0] = i;
    if (i == K - 1) out[1] = static_cast<unsigned long long>(excl[i]) + flag[i];
  }
}

// keep[j] = 1 if sorted entry j is a first occurrence with candidate index <= T
__global__ void k_gnm_keep(const uint64_t* keys, const uint32_t* idx, uint64_t K, uint64_t invalid,
                           uint64_t T, uint32_t* keep) {
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < K;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[j];
    keep[j] = (k != invalid && (j == 0 || keys[j - 1] != k) && idx[j] <= T) ? 1u : 0u;
  }
}

// selected pairs -> both directed keys
__global__ void k_gnm_directed(const uint64_t* keys, const uint32_t* keep, const uint32_t* pos,
                               uint64_t K, uint32_t b, uint64_t* dkeys) {
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < K;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    if (!keep[j]) continue;
    const uint64_t k = keys[j];
    const uint64_t u = k >> b, v = k & mask;
    const uint64_t p = pos[j];
    dkeys[2 * p] = (u << b) | v;
    dkeys[2 * p + 1] = (v << b) | u;
  }
}

__global__ void k_gnm_unpack(const uint64_t* dkeys, uint64_t md, uint32_t b, uint64_t wseed,
                             uint32_t max_weight, uint32_t* out) {
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < md;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = dkeys[i];
    const uint32_t s = static_cast<uint32_t>(k >> b), d = static_cast<uint32_t>(k & mask);
    const uint64_t canon = (static_cast<uint64_t>(min(s, d)) << 32) | max(s, d);
    const uint32_t w = 1u + static_cast<uint32_t>(__umul64hi(mix64(wseed ^ canon), max_weight));
    out[3 * i] = s;
    out[3 * i + 1] = d;
    out[3 * i + 2] = w;
  }
}

// Generator scratch: stream-ordered allocations from the context's pool when
// a generator runs with a context (set by PoolScope), plain cudaMalloc
// otherwise.
struct GenPool {
  kamsta_ctx* ctx = nullptr;
  cudaMemPool_t pool = nullptr;
  cudaStream_t st = nullptr;
};
thread_local GenPool g_gen_pool;

struct PoolScope {
  GenPool saved;
  PoolScope(kamsta_ctx* ctx, cudaStream_t st) : saved(g_gen_pool) {
    g_gen_pool = ctx ? GenPool{ctx, ctx->pool, st} : GenPool{};
  }
  ~PoolScope() { g_gen_pool = saved; }
};

struct Tmp {
  void* p = nullptr;
  GenPool gp = g_gen_pool;
  ~Tmp() { reset(); }
  void reset() {
    if (p) {
      if (gp.pool) cudaFreeAsync(p, gp.st);
      else cudaFree(p);
    }
    p = nullptr;
  }
  template <typename T>
  cudaError_t alloc(T** out, uint64_t count) {
    reset();
    const size_t bytes = std::max<uint64_t>(count, 1) * sizeof(T);
    cudaError_t e = gp.ctx ? ctx_alloc(gp.ctx, &p, bytes, gp.st) : cudaMalloc(&p, bytes);
    *out = static_cast<T*>(p);
    return e;
  }
};

#define GEN_TRY(x)                                        \
  do {                                                    \
    const cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return cuda_status(e_, #x);    \
  } while (0)


kamsta_status gen_gnm(kamsta_ctx* ctx, uint32_t n, uint64_t m, uint64_t seed, uint32_t max_weight,
                      kamsta_wedge* d_out, uint64_t* m_out, cudaStream_t st) {
  *m_out = 0;
  PoolScope scope(ctx, st);
  const uint64_t pairs = static_cast<uint64_t>(n) * (n - 1ull) / 2;
  if (m == 0) return KAMSTA_OK;
  if (n < 2 || m > pairs || max_weight == 0) {
    set_error("gen_gnm: m exceeds n(n-1)/2 or bad arguments");
    return KAMSTA_E_INPUT;
  }
  if (2 * m >= (1ull << 32) - kRsTile) {
    set_error("gen_gnm: 2m must be < 2^32");
    return KAMSTA_E_INPUT;
  }
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint32_t b = n <= 1 ? 1u : 32u - static_cast<uint32_t>(__builtin_clz(n - 1));
  if (2 * b > 64) {
    set_error("gen_gnm: n too large");
    return KAMSTA_E_INPUT;
  }
  const uint64_t invalid = (b == 32) ? ~0ull : ((1ull << (2 * b)) - 1);
  const uint64_t base = mix64(seed);
  const uint64_t wseed = mix64(seed ^ 0x6a09e667f3bcc909ull);
  const int grid = sms * 8;
  uint64_t K = m + m / 1024 + 4096;
  unsigned long long* d_small = nullptr;
  Tmp tsmall;
  GEN_TRY(tsmall.alloc(&d_small, 8));
  uint32_t* d_ticket = reinterpret_cast<uint32_t*>(d_small + 4);
  uint32_t* d_err = reinterpret_cast<uint32_t*>(d_small + 5);
  GEN_TRY(cudaMemsetAsync(d_small, 0, 8 * sizeof(unsigned long long), st));
  for (int attempt = 0; attempt < 64; ++attempt) {
    if (K >= (1ull << 32) - kRsTile) {
      set_error("gen_gnm: candidate stream too long (graph too dense)");
      return KAMSTA_E_INPUT;
    }
    Tmp tk, tk2, ti, ti2, tc, ts, tf;
    uint64_t *keys, *keys2;
    uint32_t *idx, *idx2, *counts, *flag;
    uint64_t* status;
    const RadixScratch rs = radix_scratch_bytes(K);
    GEN_TRY(tk.alloc(&keys, K));
    GEN_TRY(tk2.alloc(&keys2, K));
    GEN_TRY(ti.alloc(&idx, K));
    GEN_TRY(ti2.alloc(&idx2, K));
    GEN_TRY(tc.alloc(&counts, std::max<uint64_t>(rs.counts, K)));
    GEN_TRY(ts.alloc(&status, std::max<uint64_t>(rs.status, cdiv(K, kScanTile) + 1)));
    GEN_TRY(tf.alloc(&flag, K));
    k_gnm_candidates<<<grid, 256, 0, st>>>(0, K, base, n, b, keys, idx);
    int alt = 0;
    GEN_TRY(radix_sort_pairs_u32(st, keys, keys2, idx, idx2, K, 2 * b, counts, status, d_ticket,
                                 d_err, &alt, sms));
    if (alt) {
      std::swap(keys, keys2);
      std::swap(idx, idx2);
    }
    GEN_TRY(cudaMemsetAsync(flag, 0, sizeof(uint32_t) * K, st));
    k_gnm_first<<<grid, 256, 0, st>>>(keys, idx, K, invalid, flag);
    // exclusive prefix of the first-occurrence flags in candidate order
    const uint32_t nst = cdiv(K, kScanTile);
    GEN_TRY(cudaMemsetAsync(status, 0, sizeof(uint64_t) * nst, st));
    GEN_TRY(cudaMemsetAsync(d_ticket, 0, sizeof(uint32_t), st));
    k_scan_u32<<<std::min<uint32_t>(nst, sms * 4), kRsBlock, 0, st>>>(flag, counts, K, status,
                                                                       d_ticket, nst, d_err);
    GEN_TRY(cudaMemsetAsync(d_small, 0xff, sizeof(unsigned long long) * 2, st));
    k_gnm_threshold<<<grid, 256, 0, st>>>(flag, counts, K, m, d_small);
    unsigned long long h[2];
    GEN_TRY(cudaMemcpyAsync(h, d_small, sizeof(h), cudaMemcpyDeviceToHost, st));
    GEN_TRY(cudaStreamSynchronize(st));
    const uint64_t total = h[1];
    if (total < m) {
      K = K + (m - total) * 2 + 4096;
      continue;
    }
    const uint64_t T = h[0];
    // keep flags over the sorted list, their positions, directed keys
    uint32_t* keep = flag;  // reuse
    k_gnm_keep<<<grid, 256, 0, st>>>(keys, idx, K, invalid, T, keep);
    GEN_TRY(cudaMemsetAsync(status, 0, sizeof(uint64_t) * nst, st));
    GEN_TRY(cudaMemsetAsync(d_ticket, 0, sizeof(uint32_t), st));
    k_scan_u32<<<std::min<uint32_t>(nst, sms * 4), kRsBlock, 0, st>>>(keep, counts, K, status,
                                                                       d_ticket, nst, d_err);
    const uint64_t md = 2 * m;
    Tmp td, td2;
    uint64_t *dk, *dk2;
    GEN_TRY(td.alloc(&dk, md));
    GEN_TRY(td2.alloc(&dk2, md));
    k_gnm_directed<<<grid, 256, 0, st>>>(keys, keep, counts, K, b, dk);
    // free the candidate buffers before the big sort
    GEN_TRY(cudaStreamSynchronize(st));
    tk.reset();
    tk2.reset();
    ti.reset();
    ti2.reset();
    const RadixScratch rs2 = radix_scratch_bytes(md);
    Tmp tc2, ts2;
    uint32_t* counts2;
    uint64_t* status2;
    GEN_TRY(tc2.alloc(&counts2, rs2.counts));
    GEN_TRY(ts2.alloc(&status2, rs2.status));
    GEN_TRY(radix_sort_keys(st, dk, dk2, md, 2 * b, counts2, status2, d_ticket, d_err, &alt, sms));
    if (alt) std::swap(dk, dk2);
    k_gnm_unpack<<<grid, 256, 0, st>>>(dk, md, b, wseed, max_weight,
                                        reinterpret_cast<uint32_t*>(d_out));
    uint32_t herr = 0;
    GEN_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GEN_TRY(cudaStreamSynchronize(st));
    GEN_TRY(cudaGetLastError());
    if (herr) {
      set_error("gen_gnm: device scan wait cap reached");
      return KAMSTA_E_NOCONVERGE;
    }
    *m_out = md;
    return KAMSTA_OK;
  }
  set_error("gen_gnm: did not reach m distinct pairs");
  return KAMSTA_E_NOCONVERGE;
}

// ---------------------------------------------------------------------------
// 2-D random geometric graph.  Stand-in for KaGen's get_rgg2D
// (benchmarks/mst_benchmarks.hpp:133-139); the definition is shared with the
// oracle's CPU generator (oracle/oracle.cpp):
//   base = mix64(seed ^ 0x5247473244); point i: x = mix64(base + 2i) >> 33,
//   y = mix64(base + 2i + 1) >> 33 (31-bit integers); R = floor(radius * 2^31);
//   u ~ v iff u != v and dx^2 + dy^2 <= R^2 (exact 64-bit arithmetic);
//   G = min(floor(2^31 / R), isqrt(n), 65536) >= 1 cells per side;
//   vertex ids = ranks of the points sorted by (cell, i); GNM weights.
// Device steps: cell keys -> radix sort -> per-cell first rank -> per-vertex
// degree over the 3x3 cell block -> scan -> write.  Each vertex's neighbours
// come out in id order because cells are visited in row-major order and ids
// follow the cells.

__device__ __forceinline__ uint32_t rgg_coord(uint64_t base, uint64_t k) {
  return static_cast<uint32_t>(mix64(base + k) >> 33);
}

__global__ void k_rgg_keys(uint32_t n, uint64_t base, uint64_t G, uint64_t* keys) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t x = rgg_coord(base, 2 * i), y = rgg_coord(base, 2 * i + 1);
    const uint64_t cell = ((y * G) >> 31) * G + ((x * G) >> 31);
    keys[i] = (cell << 32) | i;
  }
}

__global__ void k_rgg_place(const uint64_t* keys, uint32_t n, uint64_t base, uint32_t* px,
                            uint32_t* py) {
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t i = keys[j] & 0xffffffffull;
    px[j] = rgg_coord(base, 2 * i);
    py[j] = rgg_coord(base, 2 * i + 1);
  }
}

// cbeg[c] = first rank in cell c (c in [0, cells])
__global__ void k_rgg_cells(const uint64_t* keys, uint32_t n, uint64_t cells, uint32_t* cbeg) {
  for (uint64_t c = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; c <= cells;
       c += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t x = c << 32;
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < x) lo = mid + 1; else hi = mid;
    }
    cbeg[c] = static_cast<uint32_t>(lo);
  }
}

template <bool WRITE>
__global__ void k_rgg_edges(uint32_t n, const uint32_t* __restrict__ px,
                            const uint32_t* __restrict__ py, const uint32_t* __restrict__ cbeg,
                            uint64_t G, uint64_t R2, uint32_t* __restrict__ deg,
                            const uint32_t* __restrict__ off, uint64_t wseed, uint32_t max_weight,
                            uint32_t mode, uint32_t* __restrict__ out) {
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t xj = px[j], yj = py[j];
    const uint64_t cx = (xj * G) >> 31, cy = (yj * G) >> 31;
    uint64_t o = WRITE ? off[j] : 0;
    uint32_t d = 0;
    const uint64_t y0 = cy ? cy - 1 : 0, y1 = min(cy + 1, G - 1);
    const uint64_t x0 = cx ? cx - 1 : 0, x1 = min(cx + 1, G - 1);
    for (uint64_t ny = y0; ny <= y1; ++ny) {
      // cells (ny, x0..x1) are contiguous: one rank range
      const uint32_t kb = cbeg[ny * G + x0], ke = cbeg[ny * G + x1 + 1];
      for (uint32_t k = kb; k < ke; ++k) {
        if (k == j) continue;
        const uint64_t xk = px[k], yk = py[k];
        const uint64_t dx = xj > xk ? xj - xk : xk - xj;
        const uint64_t dy = yj > yk ? yj - yk : yk - yj;
        const uint64_t d2 = dx * dx + dy * dy;
        if (d2 <= R2) {
          if (WRITE) {
            const uint64_t lo = j < k ? j : k, hi = j < k ? k : j;
            out[3 * o] = static_cast<uint32_t>(j);
            out[3 * o + 1] = k;
            out[3 * o + 2] = geo_weight(mode, d2, R2, wseed, (lo << 32) | hi, max_weight);
            ++o;
          }
          ++d;
        }
      }
    }
    if (!WRITE) deg[j] = d;
  }
}

__global__ void k_sum_u32(const uint32_t* v, uint64_t n, unsigned long long* out) {
  uint64_t s = 0;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    s += v[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, static_cast<unsigned long long>(s));
}

cudaError_t exclusive_scan_u32(cudaStream_t st, const uint32_t* in, uint32_t* out, uint64_t n,
                               uint64_t* status, uint32_t* ticket, uint32_t* err, int sms) {
  if (n == 0) return cudaSuccess;
  const uint32_t nst = cdiv(n, kScanTile);
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(uint64_t) * nst, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(ticket, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_scan_u32<<<std::min<uint32_t>(nst, sms * 4), kRsBlock, 0, st>>>(in, out, n, status, ticket,
                                                                     nst, err);
  return cudaGetLastError();
}

cudaError_t sum_u32(cudaStream_t st, const uint32_t* v, uint64_t n, unsigned long long* out,
                    int sms) {
  k_sum_u32<<<sms * 8, 256, 0, st>>>(v, n, out);
  return cudaGetLastError();
}

static uint64_t isqrt64(uint64_t n) {
  uint64_t s = static_cast<uint64_t>(std::sqrt(static_cast<double>(n)));
  while (s * s > n) --s;
  while ((s + 1) * (s + 1) <= n) ++s;
  return s;
}

kamsta_status gen_rgg2d(kamsta_ctx* ctx, uint32_t n, double radius, uint64_t seed,
                        uint32_t max_weight, uint32_t distance, kamsta_wedge* d_out,
                        uint64_t capacity, uint64_t* m_out, cudaStream_t st) {
  *m_out = 0;
  if (max_weight == 0 || distance > KAMSTA_DISTANCE_SQUARED_EUCLIDEAN) {
    set_error("gen_rgg2d: max_weight must be >= 1 and distance a KAMSTA_DISTANCE_* value");
    return KAMSTA_E_INPUT;
  }
  if (n == 0) return KAMSTA_OK;
  PoolScope scope(ctx, st);
  uint64_t R = 0;
  if (!(radius > 0)) R = 0;
  else if (radius >= 1) R = 1ull << 31;
  else R = static_cast<uint64_t>(radius * 2147483648.0);
  const uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(isqrt64(n), 1), 65536);
  const uint64_t G = R == 0 ? cap : std::max<uint64_t>(1, std::min<uint64_t>((1ull << 31) / R, cap));
  const uint64_t cells = G * G;
  const uint64_t base = mix64(seed ^ 0x5247473244ull);
  const uint64_t wseed = mix64(seed ^ 0x6a09e667f3bcc909ull);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8;
  Tmp tsmall, tk, tk2, tx, ty, tcb, tdeg, toff, tcnt, tst;
  unsigned long long* d_small = nullptr;
  uint64_t *keys, *keys2, *status;
  uint32_t *px, *py, *cbeg, *deg, *off, *counts;
  GEN_TRY(tsmall.alloc(&d_small, 8));
  uint32_t* d_ticket = reinterpret_cast<uint32_t*>(d_small + 4);
  uint32_t* d_err = reinterpret_cast<uint32_t*>(d_small + 5);
  GEN_TRY(cudaMemsetAsync(d_small, 0, 8 * sizeof(unsigned long long), st));
  GEN_TRY(tk.alloc(&keys, n));
  GEN_TRY(tk2.alloc(&keys2, n));
  const RadixScratch rs = radix_scratch_bytes(n);
  GEN_TRY(tcnt.alloc(&counts, std::max<uint64_t>(rs.counts, n)));
  GEN_TRY(tst.alloc(&status, std::max<uint64_t>(rs.status, cdiv(n, kScanTile) + 1)));
  k_rgg_keys<<<grid, 256, 0, st>>>(n, base, G, keys);
  int alt = 0;
  uint32_t cbits = 1;
  while (cbits < 32 && (1ull << cbits) < cells) ++cbits;
  GEN_TRY(radix_sort_keys(st, keys, keys2, n, 32 + static_cast<int>(cbits), counts, status,
                          d_ticket, d_err, &alt, sms));
  if (alt) std::swap(keys, keys2);
  GEN_TRY(tx.alloc(&px, n));
  GEN_TRY(ty.alloc(&py, n));
  GEN_TRY(tcb.alloc(&cbeg, cells + 1));
  k_rgg_place<<<grid, 256, 0, st>>>(keys, n, base, px, py);
  k_rgg_cells<<<grid, 256, 0, st>>>(keys, n, cells, cbeg);
  tk.reset();
  tk2.reset();
  GEN_TRY(tdeg.alloc(&deg, n));
  GEN_TRY(toff.alloc(&off, n));
  k_rgg_edges<false><<<grid, 256, 0, st>>>(n, px, py, cbeg, G, R * R, deg, nullptr, wseed,
                                           max_weight, distance, nullptr);
  const uint32_t nst = cdiv(n, kScanTile);
  GEN_TRY(cudaMemsetAsync(status, 0, sizeof(uint64_t) * nst, st));
  GEN_TRY(cudaMemsetAsync(d_ticket, 0, sizeof(uint32_t), st));
  k_scan_u32<<<std::min<uint32_t>(nst, sms * 4), kRsBlock, 0, st>>>(deg, off, n, status,
                                                                     d_ticket, nst, d_err);
  // exact 64-bit degree sum (the u32 prefix is only valid below 2^32)
  k_sum_u32<<<grid, 256, 0, st>>>(deg, n, d_small);
  unsigned long long h_total = 0;
  uint32_t h_err = 0;
  GEN_TRY(cudaMemcpyAsync(&h_total, d_small, sizeof(h_total), cudaMemcpyDeviceToHost, st));
  GEN_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  GEN_TRY(cudaStreamSynchronize(st));
  if (h_err) {
    set_error("gen_rgg2d: device scan wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  const uint64_t total = h_total;
  if (total >= (1ull << 32)) {
    set_error("gen_rgg2d: more than 2^32 directed entries");
    return KAMSTA_E_INPUT;
  }
  *m_out = total;
  if (!d_out || total > capacity) {
    if (d_out) {
      set_error("gen_rgg2d: output capacity too small (required count in m_directed_out)");
      return KAMSTA_E_INPUT;
    }
    return KAMSTA_OK;
  }
  k_rgg_edges<true><<<grid, 256, 0, st>>>(n, px, py, cbeg, G, R * R, deg, off, wseed,
                                          max_weight, distance, reinterpret_cast<uint32_t*>(d_out));
  GEN_TRY(cudaGetLastError());
  GEN_TRY(cudaStreamSynchronize(st));
  return KAMSTA_OK;
}

}  // namespace kamsta

extern "C" kamsta_status kamsta_gen_rgg2d_dev(kamsta_ctx* ctx, uint32_t n, double radius,
                                              uint64_t seed, uint32_t max_weight,
                                              uint32_t distance, kamsta_wedge* d_out,
                                              uint64_t capacity, uint64_t* m_directed_out,
                                              kamsta_stream stream) {
  if (!m_directed_out) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (ctx ? ctx->stream : nullptr);
  return kamsta::gen_rgg2d(ctx, n, radius, seed, max_weight, distance, d_out, capacity,
                           m_directed_out, st);
}

extern "C" kamsta_status kamsta_gen_gnm_dev(kamsta_ctx* ctx, uint32_t n, uint64_t m, uint64_t seed,
                                            uint32_t max_weight, kamsta_wedge* d_out,
                                            uint64_t* m_directed_out, kamsta_stream stream) {
  if (!m_directed_out || (m && !d_out)) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : (ctx ? ctx->stream : nullptr);
  return kamsta::gen_gnm(ctx, n, m, seed, max_weight, d_out, m_directed_out, st);
}
