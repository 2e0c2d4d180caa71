// gen_grid_rmat.cu -- lattice, 3-D random geometric and R-MAT generators.
//
// Stand-ins for KaGen's get_grid2D / get_grid3D (benchmarks/
// mst_benchmarks.hpp:159-180), get_rgg3D (:140-146) and
// get_rmat_edges_evenly_distributed (:147-151), which the reference tree does
// not vendor.  Each definition is shared with the oracle's CPU generators
// (oracle/gen_grid_rmat.cpp).  Weights are the G(n,m) generator's:
//   w = 1 + hi64(mix64(wseed ^ (min << 32 | max)) * max_weight),
//   wseed = mix64(seed ^ 0x6a09e667f3bcc909);
// the output holds both directions, sorted by (src, dst), without self loops
// or duplicates.
//
// Grid, X x Y x Z vertices (Z = 1: the 2-D grid).  Vertex (x, y, z) has id
// (z Y + y) X + x.  Its candidates are the -1 and +1 steps along each axis,
// taken modulo the side when `periodic` and dropped at the border otherwise.
// A candidate pair {u, v}, u != v, is an edge iff p >= 1 or
// (mix64(pseed ^ canon) >> 11) < floor(p 2^53), pseed = mix64(seed ^
// 0x47524944).
//
// RGG-3D.  base = mix64(seed ^ 0x5247473344); point i has 31-bit integer
// coordinates x, y, z = mix64(base + 3i + {0, 1, 2}) >> 33; R = floor(radius
// 2^31) (radius clamped to [0, 1]); u ~ v iff u != v and dx^2 + dy^2 + dz^2
// <= R^2 (exact in 64 bits: 3 (2^31)^2 < 2^64); G = min(floor(2^31 / R),
// icbrt(n), 1024) >= 1 cells per side; cell = ((z G >> 31) G + (y G >> 31))
// G + (x G >> 31); vertex ids = ranks of the points sorted by (cell, i).
//
// R-MAT.  n = 2^L (1 <= L <= 31); sample i descends L levels, the first level
// choosing the most significant id bit.  Level l reads the 32-bit half r
// (high for even l, low for odd l) of mix64(base + i ceil(L/2) + l/2), base =
// mix64(seed ^ 0x524d4154), and takes quadrant (0,0) if r < ta, (0,1) if r <
// tab, (1,0) if r < tabc and (1,1) otherwise, ta = floor(a 2^32), tab =
// floor((a + b) 2^32), tabc = floor((a + b + c) 2^32) (host doubles).  The
// graph = the distinct unordered pairs u != v among the samples; ids are not
// permuted, so the heaviest hubs have the smallest ids.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "gen_scratch.cuh"
#include "sort_gen.cuh"

namespace kamsta {

namespace {

constexpr uint64_t kWeightSalt = 0x6a09e667f3bcc909ull;
// the radix sort takes fewer than 2^32 - kRmatSortSlack keys
constexpr uint64_t kRmatSortSlack = 4096;

__device__ __forceinline__ uint32_t gen_weight(uint64_t wseed, uint64_t lo, uint64_t hi,
                                               uint32_t max_weight) {
  return 1u + static_cast<uint32_t>(__umul64hi(mix64(wseed ^ ((lo << 32) | hi)), max_weight));
}

#define GRID_STRIDE_LOOP(i, count)                                                      \
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; \
       i < (count); i += static_cast<uint64_t>(gridDim.x) * blockDim.x)

// ---------------------------------------------------------------------------
// Grid

struct GridDef {
  uint32_t X, Y, Z;
  uint32_t periodic;
  uint64_t pthr;  // kept iff all or (mix64(pseed ^ canon) >> 11) < pthr
  uint64_t pseed;
  uint32_t all;
};

// The kept neighbours of v, ascending and distinct; returns their number.
__device__ __forceinline__ int grid_neighbours(const GridDef& g, uint64_t v, uint32_t nb[6]) {
  const uint64_t XY = static_cast<uint64_t>(g.X) * g.Y;
  const uint64_t coord[3] = {v % g.X, (v / g.X) % g.Y, v / XY};
  const uint64_t side[3] = {g.X, g.Y, g.Z};
  const uint64_t stride[3] = {1, g.X, XY};
  uint64_t c[6];
  int k = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const uint64_t s = side[a], q = coord[a], t = stride[a];
    if (q > 0) c[k++] = v - t;
    else if (g.periodic && s > 1) c[k++] = v + (s - 1) * t;
    if (q + 1 < s) c[k++] = v + t;
    else if (g.periodic && s > 1) c[k++] = v - (s - 1) * t;
  }
  // insertion sort of at most 6 ids
  for (int i = 1; i < k; ++i) {
    const uint64_t x = c[i];
    int j = i - 1;
    while (j >= 0 && c[j] > x) {
      c[j + 1] = c[j];
      --j;
    }
    c[j + 1] = x;
  }
  int d = 0;
  for (int i = 0; i < k; ++i) {
    if (c[i] == v || (i > 0 && c[i] == c[i - 1])) continue;
    if (!g.all) {
      const uint64_t lo = v < c[i] ? v : c[i], hi = v < c[i] ? c[i] : v;
      if ((mix64(g.pseed ^ ((lo << 32) | hi)) >> 11) >= g.pthr) continue;
    }
    nb[d++] = static_cast<uint32_t>(c[i]);
  }
  return d;
}

template <bool WRITE>
__global__ void k_grid_edges(GridDef g, uint64_t n, uint32_t* __restrict__ deg,
                             const uint32_t* __restrict__ off, uint64_t wseed,
                             uint32_t max_weight, uint32_t* __restrict__ out) {
  GRID_STRIDE_LOOP(v, n) {
    uint32_t nb[6];
    const int d = grid_neighbours(g, v, nb);
    if (!WRITE) {
      deg[v] = static_cast<uint32_t>(d);
      continue;
    }
    const uint64_t o = off[v];
    for (int i = 0; i < d; ++i) {
      const uint64_t u = nb[i];
      out[3 * (o + i)] = static_cast<uint32_t>(v);
      out[3 * (o + i) + 1] = nb[i];
      out[3 * (o + i) + 2] = gen_weight(wseed, v < u ? v : u, v < u ? u : v, max_weight);
    }
  }
}

// ---------------------------------------------------------------------------
// RGG-3D

__device__ __forceinline__ uint64_t coord31(uint64_t base, uint64_t k) {
  return mix64(base + k) >> 33;
}

__global__ void k_rgg3_keys(uint32_t n, uint64_t base, uint64_t G, uint64_t* keys) {
  GRID_STRIDE_LOOP(i, n) {
    const uint64_t x = coord31(base, 3 * i), y = coord31(base, 3 * i + 1),
                   z = coord31(base, 3 * i + 2);
    const uint64_t cell = (((z * G) >> 31) * G + ((y * G) >> 31)) * G + ((x * G) >> 31);
    keys[i] = (cell << 32) | i;
  }
}

__global__ void k_rgg3_place(const uint64_t* keys, uint32_t n, uint64_t base, uint32_t* px,
                             uint32_t* py, uint32_t* pz) {
  GRID_STRIDE_LOOP(j, n) {
    const uint64_t i = keys[j] & 0xffffffffull;
    px[j] = static_cast<uint32_t>(coord31(base, 3 * i));
    py[j] = static_cast<uint32_t>(coord31(base, 3 * i + 1));
    pz[j] = static_cast<uint32_t>(coord31(base, 3 * i + 2));
  }
}

// cbeg[c] = first rank in cell c, c in [0, cells]
__global__ void k_cell_starts(const uint64_t* keys, uint32_t n, uint64_t cells, uint32_t* cbeg) {
  GRID_STRIDE_LOOP(c, cells + 1) {
    const uint64_t x = c << 32;
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < x) lo = mid + 1;
      else hi = mid;
    }
    cbeg[c] = static_cast<uint32_t>(lo);
  }
}

__device__ __forceinline__ uint64_t absdiff(uint64_t a, uint64_t b) { return a > b ? a - b : b - a; }

// Degree (WRITE = false) or edges (WRITE = true) of every point.  Cells are
// visited in increasing index order and ranks follow the cells, so each
// vertex's neighbours come out ascending.
template <bool WRITE>
__global__ void k_rgg3_edges(uint32_t n, const uint32_t* __restrict__ px,
                             const uint32_t* __restrict__ py, const uint32_t* __restrict__ pz,
                             const uint32_t* __restrict__ cbeg, uint64_t G, uint64_t R2,
                             uint32_t* __restrict__ deg, const uint32_t* __restrict__ off,
                             uint64_t wseed, uint32_t max_weight, uint32_t mode,
                             uint32_t* __restrict__ out) {
  GRID_STRIDE_LOOP(j, n) {
    const uint64_t xj = px[j], yj = py[j], zj = pz[j];
    const uint64_t cx = (xj * G) >> 31, cy = (yj * G) >> 31, cz = (zj * G) >> 31;
    const uint64_t x0 = cx ? cx - 1 : 0, x1 = min(cx + 1, G - 1);
    const uint64_t y0 = cy ? cy - 1 : 0, y1 = min(cy + 1, G - 1);
    const uint64_t z0 = cz ? cz - 1 : 0, z1 = min(cz + 1, G - 1);
    uint64_t o = WRITE ? off[j] : 0;
    uint32_t d = 0;
    for (uint64_t nz = z0; nz <= z1; ++nz)
      for (uint64_t ny = y0; ny <= y1; ++ny) {
        const uint64_t row = (nz * G + ny) * G;
        const uint32_t kb = cbeg[row + x0], ke = cbeg[row + x1 + 1];
        for (uint32_t k = kb; k < ke; ++k) {
          if (k == j) continue;
          const uint64_t dx = absdiff(xj, px[k]), dy = absdiff(yj, py[k]),
                         dz = absdiff(zj, pz[k]);
          const uint64_t d2 = dx * dx + dy * dy + dz * dz;
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

// ---------------------------------------------------------------------------
// R-MAT

__global__ void k_rmat_keys(uint64_t K, uint64_t base, uint32_t L, uint64_t ta, uint64_t tab,
                            uint64_t tabc, uint64_t* keys) {
  const uint64_t invalid = (1ull << (2 * L)) - 1;
  const uint64_t P = (L + 1) / 2;
  GRID_STRIDE_LOOP(i, K) {
    uint64_t u = 0, v = 0, h = 0;
    for (uint32_t l = 0; l < L; ++l) {
      uint64_t r;
      if ((l & 1) == 0) {
        h = mix64(base + i * P + (l >> 1));
        r = h >> 32;
      } else {
        r = h & 0xffffffffull;
      }
      const uint32_t q = r < ta ? 0u : r < tab ? 1u : r < tabc ? 2u : 3u;
      u = (u << 1) | (q >> 1);
      v = (v << 1) | (q & 1u);
    }
    keys[i] = u == v ? invalid : (((u < v ? u : v) << L) | (u < v ? v : u));
  }
}

// keep[j] = 1 for the first entry of every run of equal valid keys
__global__ void k_first_of_run(const uint64_t* keys, uint64_t K, uint64_t invalid,
                               uint32_t* keep) {
  GRID_STRIDE_LOOP(j, K) {
    const uint64_t k = keys[j];
    keep[j] = (k != invalid && (j == 0 || keys[j - 1] != k)) ? 1u : 0u;
  }
}

// kept pairs -> both directed keys at 2 pos, 2 pos + 1
__global__ void k_pairs_directed(const uint64_t* keys, const uint32_t* keep, const uint32_t* pos,
                                 uint64_t K, uint32_t b, uint64_t* dkeys) {
  const uint64_t mask = (1ull << b) - 1;
  GRID_STRIDE_LOOP(j, K) {
    if (!keep[j]) continue;
    const uint64_t k = keys[j], u = k >> b, v = k & mask, p = pos[j];
    dkeys[2 * p] = (u << b) | v;
    dkeys[2 * p + 1] = (v << b) | u;
  }
}

__global__ void k_pairs_unpack(const uint64_t* dkeys, uint64_t md, uint32_t b, uint64_t wseed,
                               uint32_t max_weight, uint32_t* out) {
  const uint64_t mask = (1ull << b) - 1;
  GRID_STRIDE_LOOP(i, md) {
    const uint64_t k = dkeys[i], s = k >> b, d = k & mask;
    out[3 * i] = static_cast<uint32_t>(s);
    out[3 * i + 1] = static_cast<uint32_t>(d);
    out[3 * i + 2] = gen_weight(wseed, s < d ? s : d, s < d ? d : s, max_weight);
  }
}

#undef GRID_STRIDE_LOOP

int sm_count() {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

uint32_t cdiv32(uint64_t a, uint64_t b) { return static_cast<uint32_t>((a + b - 1) / b); }

// Shared tail of the per-vertex generators: degrees -> offsets -> total;
// with room in d_out, `write` fills it.  *m_out = the directed entry count.
template <typename CountFn, typename WriteFn>
kamsta_status count_then_write(kamsta_ctx* ctx, cudaStream_t st, uint64_t n, const char* name,
                               kamsta_wedge* d_out, uint64_t capacity, uint64_t* m_out,
                               CountFn&& count, WriteFn&& write) {
  const int sms = sm_count();
  GenBuf bdeg, boff, bstat, bsmall;
  uint32_t *deg, *off;
  uint64_t* status;
  unsigned long long* small;
  GEN_CHECK(bdeg.alloc(ctx, st, &deg, n));
  GEN_CHECK(boff.alloc(ctx, st, &off, n));
  GEN_CHECK(bstat.alloc(ctx, st, &status, cdiv32(n, 2048) + 2));
  GEN_CHECK(bsmall.alloc(ctx, st, &small, 4));
  uint32_t* ticket = reinterpret_cast<uint32_t*>(small + 2);
  uint32_t* err = reinterpret_cast<uint32_t*>(small + 3);
  GEN_CHECK(cudaMemsetAsync(small, 0, 4 * sizeof(unsigned long long), st));
  count(deg);
  GEN_CHECK(cudaGetLastError());
  GEN_CHECK(exclusive_scan_u32(st, deg, off, n, status, ticket, err, sms));
  GEN_CHECK(sum_u32(st, deg, n, small, sms));
  unsigned long long total = 0;
  uint32_t herr = 0;
  GEN_CHECK(cudaMemcpyAsync(&total, small, sizeof(total), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaStreamSynchronize(st));
  if (herr) {
    set_error(std::string(name) + ": device scan wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  if (total >= (1ull << 32)) {
    set_error(std::string(name) + ": more than 2^32 directed entries");
    return KAMSTA_E_INPUT;
  }
  *m_out = total;
  if (!d_out) return KAMSTA_OK;
  if (total > capacity) {
    set_error(std::string(name) + ": output capacity too small (required count in m_directed_out)");
    return KAMSTA_E_INPUT;
  }
  write(deg, off, reinterpret_cast<uint32_t*>(d_out));
  GEN_CHECK(cudaGetLastError());
  GEN_CHECK(cudaStreamSynchronize(st));
  return KAMSTA_OK;
}

}  // namespace

kamsta_status gen_grid(kamsta_ctx* ctx, uint32_t X, uint32_t Y, uint32_t Z, double p,
                       int periodic, uint64_t seed, uint32_t max_weight, kamsta_wedge* d_out,
                       uint64_t capacity, uint64_t* m_out, cudaStream_t st) {
  *m_out = 0;
  if (max_weight == 0) {
    set_error("gen_grid: max_weight must be >= 1");
    return KAMSTA_E_INPUT;
  }
  const uint64_t n = static_cast<uint64_t>(X) * Y * Z;
  if (n >= (1ull << 32)) {
    set_error("gen_grid: X * Y * Z must be < 2^32");
    return KAMSTA_E_INPUT;
  }
  if (n == 0) return KAMSTA_OK;
  GridDef g;
  g.X = X;
  g.Y = Y;
  g.Z = Z;
  g.periodic = periodic ? 1u : 0u;
  g.all = p >= 1.0 ? 1u : 0u;
  g.pthr = p > 0.0 && p < 1.0 ? static_cast<uint64_t>(p * 9007199254740992.0) : 0;
  g.pseed = mix64(seed ^ 0x47524944ull);
  const uint64_t wseed = mix64(seed ^ kWeightSalt);
  const int grid = sm_count() * 8;
  return count_then_write(
      ctx, st, n, "gen_grid", d_out, capacity, m_out,
      [&](uint32_t* deg) {
        k_grid_edges<false><<<grid, 256, 0, st>>>(g, n, deg, nullptr, wseed, max_weight, nullptr);
      },
      [&](uint32_t* deg, uint32_t* off, uint32_t* out) {
        k_grid_edges<true><<<grid, 256, 0, st>>>(g, n, deg, off, wseed, max_weight, out);
      });
}

static uint64_t icbrt64(uint64_t n) {
  uint64_t s = static_cast<uint64_t>(std::cbrt(static_cast<double>(n)));
  while (s > 0 && s * s * s > n) --s;
  while ((s + 1) * (s + 1) * (s + 1) <= n) ++s;
  return s;
}

kamsta_status gen_rgg3d(kamsta_ctx* ctx, uint32_t n, double radius, uint64_t seed,
                        uint32_t max_weight, uint32_t distance, kamsta_wedge* d_out,
                        uint64_t capacity, uint64_t* m_out, cudaStream_t st) {
  *m_out = 0;
  if (max_weight == 0 || distance > KAMSTA_DISTANCE_SQUARED_EUCLIDEAN) {
    set_error("gen_rgg3d: max_weight must be >= 1 and distance a KAMSTA_DISTANCE_* value");
    return KAMSTA_E_INPUT;
  }
  if (n == 0) return KAMSTA_OK;
  uint64_t R = 0;
  if (!(radius > 0)) R = 0;
  else if (radius >= 1) R = 1ull << 31;
  else R = static_cast<uint64_t>(radius * 2147483648.0);
  const uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(icbrt64(n), 1), 1024);
  const uint64_t G = R == 0 ? cap : std::max<uint64_t>(1, std::min<uint64_t>((1ull << 31) / R, cap));
  const uint64_t cells = G * G * G;
  const uint64_t base = mix64(seed ^ 0x5247473344ull);
  const uint64_t wseed = mix64(seed ^ kWeightSalt);
  const int sms = sm_count();
  const int grid = sms * 8;
  GenBuf bk, bk2, bcnt, bstat, bsmall, bx, by, bz, bcb;
  uint64_t *keys, *keys2, *status;
  uint32_t *counts, *px, *py, *pz, *cbeg;
  unsigned long long* small;
  GEN_CHECK(bsmall.alloc(ctx, st, &small, 4));
  uint32_t* ticket = reinterpret_cast<uint32_t*>(small + 2);
  uint32_t* err = reinterpret_cast<uint32_t*>(small + 3);
  GEN_CHECK(cudaMemsetAsync(small, 0, 4 * sizeof(unsigned long long), st));
  GEN_CHECK(bk.alloc(ctx, st, &keys, n));
  GEN_CHECK(bk2.alloc(ctx, st, &keys2, n));
  const RadixScratch rs = radix_scratch_bytes(n);
  GEN_CHECK(bcnt.alloc(ctx, st, &counts, rs.counts));
  GEN_CHECK(bstat.alloc(ctx, st, &status, rs.status));
  k_rgg3_keys<<<grid, 256, 0, st>>>(n, base, G, keys);
  uint32_t cbits = 1;
  while (cbits < 32 && (1ull << cbits) < cells) ++cbits;
  int alt = 0;
  GEN_CHECK(radix_sort_keys(st, keys, keys2, n, 32 + static_cast<int>(cbits), counts, status,
                            ticket, err, &alt, sms));
  if (alt) std::swap(keys, keys2);
  GEN_CHECK(bx.alloc(ctx, st, &px, n));
  GEN_CHECK(by.alloc(ctx, st, &py, n));
  GEN_CHECK(bz.alloc(ctx, st, &pz, n));
  GEN_CHECK(bcb.alloc(ctx, st, &cbeg, cells + 1));
  k_rgg3_place<<<grid, 256, 0, st>>>(keys, n, base, px, py, pz);
  k_cell_starts<<<grid, 256, 0, st>>>(keys, n, cells, cbeg);
  uint32_t herr = 0;
  GEN_CHECK(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaStreamSynchronize(st));
  if (herr) {
    set_error("gen_rgg3d: device scan wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  bk.reset();
  bk2.reset();
  bcnt.reset();
  bstat.reset();
  const uint64_t R2 = R * R;
  return count_then_write(
      ctx, st, n, "gen_rgg3d", d_out, capacity, m_out,
      [&](uint32_t* deg) {
        k_rgg3_edges<false><<<grid, 256, 0, st>>>(n, px, py, pz, cbeg, G, R2, deg, nullptr, wseed,
                                                  max_weight, distance, nullptr);
      },
      [&](uint32_t* deg, uint32_t* off, uint32_t* out) {
        k_rgg3_edges<true><<<grid, 256, 0, st>>>(n, px, py, pz, cbeg, G, R2, deg, off, wseed,
                                                 max_weight, distance, out);
      });
}

kamsta_status gen_rmat(kamsta_ctx* ctx, uint32_t log_n, uint64_t samples, double a, double b,
                       double c, uint64_t seed, uint32_t max_weight, kamsta_wedge* d_out,
                       uint64_t capacity, uint64_t* m_out, cudaStream_t st) {
  *m_out = 0;
  if (max_weight == 0 || log_n > 31 || !(a >= 0) || !(b >= 0) || !(c >= 0) || a + b + c > 1.0) {
    set_error("gen_rmat: needs log_n <= 31, a, b, c >= 0 with a + b + c <= 1, max_weight >= 1");
    return KAMSTA_E_INPUT;
  }
  if (samples >= (1ull << 32) - kRmatSortSlack) {
    set_error("gen_rmat: samples must be < 2^32 - 4096");
    return KAMSTA_E_INPUT;
  }
  if (log_n == 0 || samples == 0) return KAMSTA_OK;
  const auto thr = [](double x) {
    const double t = std::floor(x * 4294967296.0);
    return t >= 4294967296.0 ? (1ull << 32) : static_cast<uint64_t>(t);
  };
  const uint64_t ta = thr(a), tab = thr(a + b), tabc = thr(a + b + c);
  const uint64_t base = mix64(seed ^ 0x524d4154ull);
  const uint64_t wseed = mix64(seed ^ kWeightSalt);
  const uint64_t K = samples;
  const uint32_t L = log_n;
  GenBuf bk;
  uint64_t* keys;
  GEN_CHECK(bk.alloc(ctx, st, &keys, K));
  k_rmat_keys<<<sm_count() * 8, 256, 0, st>>>(K, base, L, ta, tab, tabc, keys);
  GEN_CHECK(cudaGetLastError());
  return pairs_to_edges(ctx, st, bk, K, L, wseed, max_weight, "gen_rmat", d_out, capacity, m_out);
}

kamsta_status pairs_to_edges(kamsta_ctx* ctx, cudaStream_t st, GenBuf& bk, uint64_t K, uint32_t L,
                             uint64_t wseed, uint32_t max_weight, const char* name,
                             kamsta_wedge* d_out, uint64_t capacity, uint64_t* m_out) {
  *m_out = 0;
  if (K == 0) return KAMSTA_OK;
  if (L == 0 || L > 31 || K >= (1ull << 32) - kRmatSortSlack) {
    set_error(std::string(name) + ": needs 1 <= id bits <= 31 and fewer than 2^32 - 4096 pairs");
    return KAMSTA_E_INPUT;
  }
  uint64_t* keys = static_cast<uint64_t*>(bk.p);
  const uint64_t invalid = (1ull << (2 * L)) - 1;
  const int sms = sm_count();
  const int grid = sms * 8;
  GenBuf bk2, bkeep, bpos, bcnt, bstat, bsmall;
  uint64_t *keys2, *status;
  uint32_t *keep, *pos, *counts;
  unsigned long long* small;
  GEN_CHECK(bsmall.alloc(ctx, st, &small, 4));
  uint32_t* ticket = reinterpret_cast<uint32_t*>(small + 2);
  uint32_t* err = reinterpret_cast<uint32_t*>(small + 3);
  GEN_CHECK(cudaMemsetAsync(small, 0, 4 * sizeof(unsigned long long), st));
  GEN_CHECK(bk2.alloc(ctx, st, &keys2, K));
  const RadixScratch rs = radix_scratch_bytes(K);
  GEN_CHECK(bcnt.alloc(ctx, st, &counts, rs.counts));
  GEN_CHECK(bstat.alloc(ctx, st, &status, std::max<uint64_t>(rs.status, cdiv32(K, 2048) + 2)));
  int alt = 0;
  GEN_CHECK(radix_sort_keys(st, keys, keys2, K, 2 * static_cast<int>(L), counts, status, ticket,
                            err, &alt, sms));
  if (alt) {
    std::swap(keys, keys2);
    std::swap(bk.p, bk2.p);  // bk owns the sorted keys
  }
  bk2.reset();
  GEN_CHECK(bkeep.alloc(ctx, st, &keep, K));
  GEN_CHECK(bpos.alloc(ctx, st, &pos, K));
  k_first_of_run<<<grid, 256, 0, st>>>(keys, K, invalid, keep);
  GEN_CHECK(exclusive_scan_u32(st, keep, pos, K, status, ticket, err, sms));
  GEN_CHECK(sum_u32(st, keep, K, small, sms));
  unsigned long long pairs = 0;
  uint32_t herr = 0;
  GEN_CHECK(cudaMemcpyAsync(&pairs, small, sizeof(pairs), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaStreamSynchronize(st));
  if (herr) {
    set_error(std::string(name) + ": device scan wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  const uint64_t md = 2 * pairs;
  if (md >= (1ull << 32) - kRmatSortSlack) {
    set_error(std::string(name) + ": more than 2^32 - 4096 directed entries");
    return KAMSTA_E_INPUT;
  }
  *m_out = md;
  if (!d_out) return KAMSTA_OK;
  if (md > capacity) {
    set_error(std::string(name) + ": output capacity too small (required count in m_directed_out)");
    return KAMSTA_E_INPUT;
  }
  GenBuf bd, bd2, bcnt2, bstat2;
  uint64_t *dk, *dk2, *status2;
  uint32_t* counts2;
  GEN_CHECK(bd.alloc(ctx, st, &dk, md));
  GEN_CHECK(bd2.alloc(ctx, st, &dk2, md));
  k_pairs_directed<<<grid, 256, 0, st>>>(keys, keep, pos, K, L, dk);
  const RadixScratch rs2 = radix_scratch_bytes(md);
  GEN_CHECK(bcnt2.alloc(ctx, st, &counts2, rs2.counts));
  GEN_CHECK(bstat2.alloc(ctx, st, &status2, rs2.status));
  GEN_CHECK(radix_sort_keys(st, dk, dk2, md, 2 * static_cast<int>(L), counts2, status2, ticket,
                            err, &alt, sms));
  if (alt) std::swap(dk, dk2);
  k_pairs_unpack<<<grid, 256, 0, st>>>(dk, md, L, wseed, max_weight,
                                       reinterpret_cast<uint32_t*>(d_out));
  GEN_CHECK(cudaMemcpyAsync(&herr, err, sizeof(herr), cudaMemcpyDeviceToHost, st));
  GEN_CHECK(cudaStreamSynchronize(st));
  GEN_CHECK(cudaGetLastError());
  if (herr) {
    set_error(std::string(name) + ": device scan wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  return KAMSTA_OK;
}

}  // namespace kamsta

namespace {
cudaStream_t gen_stream(kamsta_ctx* ctx, kamsta_stream stream) {
  return stream ? static_cast<cudaStream_t>(stream) : (ctx ? ctx->stream : nullptr);
}
}  // namespace

extern "C" kamsta_status kamsta_gen_grid_dev(kamsta_ctx* ctx, uint32_t x, uint32_t y, uint32_t z,
                                             double p, int periodic, uint64_t seed,
                                             uint32_t max_weight, kamsta_wedge* d_out,
                                             uint64_t capacity, uint64_t* m_directed_out,
                                             kamsta_stream stream) {
  if (!m_directed_out) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return kamsta::gen_grid(ctx, x, y, z, p, periodic, seed, max_weight, d_out, capacity,
                          m_directed_out, gen_stream(ctx, stream));
}

extern "C" kamsta_status kamsta_gen_rgg3d_dev(kamsta_ctx* ctx, uint32_t n, double radius,
                                              uint64_t seed, uint32_t max_weight,
                                              uint32_t distance, kamsta_wedge* d_out,
                                              uint64_t capacity, uint64_t* m_directed_out,
                                              kamsta_stream stream) {
  if (!m_directed_out) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return kamsta::gen_rgg3d(ctx, n, radius, seed, max_weight, distance, d_out, capacity,
                           m_directed_out, gen_stream(ctx, stream));
}

extern "C" kamsta_status kamsta_gen_rmat_dev(kamsta_ctx* ctx, uint32_t log_n, uint64_t samples,
                                             double a, double b, double c, uint64_t seed,
                                             uint32_t max_weight, kamsta_wedge* d_out,
                                             uint64_t capacity, uint64_t* m_directed_out,
                                             kamsta_stream stream) {
  if (!m_directed_out) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return kamsta::gen_rmat(ctx, log_n, samples, a, b, c, seed, max_weight, d_out, capacity,
                          m_directed_out, gen_stream(ctx, stream));
}
