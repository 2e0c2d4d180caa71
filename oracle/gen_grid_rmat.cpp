// gen_grid_rmat.cpp -- the oracle's lattice, 3-D random geometric and R-MAT
// generators (test infrastructure, not the product).
//
// Stand-ins for KaGen's get_grid2D / get_grid3D (benchmarks/
// mst_benchmarks.hpp:159-180), get_rgg3D (:140-146) and
// get_rmat_edges_evenly_distributed (:147-151), which the reference tree does
// not vendor.  The definitions are the device generators' (kamsta_gen_grid_dev,
// kamsta_gen_rgg3d_dev, kamsta_gen_rmat_dev); this file restates them with
// plain enumeration and std::sort, so the two sides share no code:
//
// Grid X x Y x Z: id (z Y + y) X + x; candidates are the -1 / +1 steps along
// each axis (modulo the side when periodic, dropped at the border
// otherwise); {u, v}, u != v, is an edge iff p >= 1 or (mix64(pseed ^ (lo <<
// 32 | hi)) >> 11) < floor(p 2^53), pseed = mix64(seed ^ 0x47524944).
//
// RGG-3D: base = mix64(seed ^ 0x5247473344); point i: x, y, z = mix64(base +
// 3i + {0,1,2}) >> 33; R = floor(radius 2^31); u ~ v iff dx^2 + dy^2 + dz^2
// <= R^2; G = min(floor(2^31 / R), icbrt(n), 1024) >= 1; ids = ranks by
// (cell, i), cell = ((z G >> 31) G + (y G >> 31)) G + (x G >> 31).
//
// R-MAT: n = 2^L; sample i, level l: r = 32-bit half (high for even l) of
// mix64(base + i ceil(L/2) + l/2), base = mix64(seed ^ 0x524d4154); quadrant
// by r against floor(a 2^32), floor((a+b) 2^32), floor((a+b+c) 2^32); the
// first level sets the top id bit; the graph = the distinct pairs u != v.
//
// All: weights gen::weight(mix64(seed ^ 0x6a09e667f3bcc909), ...), both
// directions, sorted by (src, dst).
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <parallel/algorithm>
#include <vector>

#include "gen_common.h"
#include "oracle.h"

namespace {

using gen::mix64;

// Writes the sorted, distinct directed keys (src << 32 | dst) as edges.
int emit_sorted(const std::vector<uint64_t>& dkeys, uint64_t wseed, uint32_t max_weight,
                kamsta_wedge* out, uint64_t capacity, uint64_t* m_directed_out) {
  *m_directed_out = dkeys.size();
  if (dkeys.size() > capacity) return 2;
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < dkeys.size(); ++i) {
    const uint64_t s = dkeys[i] >> 32, d = dkeys[i] & 0xffffffffull;
    out[i] = kamsta_wedge{static_cast<uint32_t>(s), static_cast<uint32_t>(d),
                          gen::weight(wseed, std::min(s, d), std::max(s, d), max_weight)};
  }
  return 0;
}

uint64_t icbrt(uint64_t n) {
  uint64_t s = static_cast<uint64_t>(std::cbrt(static_cast<double>(n)));
  while (s > 0 && s * s * s > n) --s;
  while ((s + 1) * (s + 1) * (s + 1) <= n) ++s;
  return s;
}

}  // namespace

extern "C" int oracle_gen_grid(uint32_t X, uint32_t Y, uint32_t Z, double p, int periodic,
                               uint64_t seed, uint32_t max_weight, kamsta_wedge* out,
                               uint64_t capacity, uint64_t* m_directed_out) {
  *m_directed_out = 0;
  const uint64_t n = static_cast<uint64_t>(X) * Y * Z;
  if (max_weight == 0 || n >= (1ull << 32)) return 1;
  if (n == 0) return 0;
  const bool all = p >= 1.0;
  const uint64_t pthr = p > 0.0 && p < 1.0 ? static_cast<uint64_t>(p * 9007199254740992.0) : 0;
  const uint64_t pseed = mix64(seed ^ 0x47524944ull);
  const uint64_t side[3] = {X, Y, Z};
  std::vector<uint64_t> dk;
  dk.reserve(6 * n);
  for (uint64_t z = 0; z < Z; ++z)
    for (uint64_t y = 0; y < Y; ++y)
      for (uint64_t x = 0; x < X; ++x) {
        const uint64_t c[3] = {x, y, z};
        const uint64_t v = (z * Y + y) * X + x;
        for (int a = 0; a < 3; ++a)
          for (int step = -1; step <= 1; step += 2) {
            uint64_t q[3] = {c[0], c[1], c[2]};
            const int64_t t = static_cast<int64_t>(c[a]) + step;
            if (t < 0 || t >= static_cast<int64_t>(side[a])) {
              if (!periodic) continue;
              q[a] = static_cast<uint64_t>((t + static_cast<int64_t>(side[a])) %
                                           static_cast<int64_t>(side[a]));
            } else {
              q[a] = static_cast<uint64_t>(t);
            }
            const uint64_t u = (q[2] * Y + q[1]) * X + q[0];
            if (u == v) continue;
            const uint64_t lo = std::min(u, v), hi = std::max(u, v);
            if (!all && (mix64(pseed ^ ((lo << 32) | hi)) >> 11) >= pthr) continue;
            dk.push_back((v << 32) | u);
          }
      }
  std::sort(dk.begin(), dk.end());
  dk.erase(std::unique(dk.begin(), dk.end()), dk.end());
  return emit_sorted(dk, mix64(seed ^ gen::kWeightSalt), max_weight, out, capacity,
                     m_directed_out);
}

extern "C" int oracle_gen_rgg3d(uint32_t n, double radius, uint64_t seed, uint32_t max_weight,
                                uint32_t distance, kamsta_wedge* out, uint64_t capacity,
                                uint64_t* m_directed_out) {
  *m_directed_out = 0;
  if (max_weight == 0 || distance > 2) return 1;
  if (n == 0) return 0;
  uint64_t R = 0;
  if (!(radius > 0)) R = 0;
  else if (radius >= 1) R = 1ull << 31;
  else R = static_cast<uint64_t>(radius * 2147483648.0);
  const uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(icbrt(n), 1), 1024);
  const uint64_t G = R == 0 ? cap : std::max<uint64_t>(1, std::min<uint64_t>((1ull << 31) / R, cap));
  const uint64_t base = mix64(seed ^ 0x5247473344ull);
  auto coord = [&](uint64_t i, int a) { return mix64(base + 3 * i + a) >> 33; };
  auto cell_of = [&](uint64_t x, uint64_t y, uint64_t z) {
    return (((z * G) >> 31) * G + ((y * G) >> 31)) * G + ((x * G) >> 31);
  };
  std::vector<std::pair<uint64_t, uint64_t>> key(n);  // (cell, point)
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < n; ++i) key[i] = {cell_of(coord(i, 0), coord(i, 1), coord(i, 2)), i};
  std::sort(key.begin(), key.end());
  std::vector<uint64_t> px(n), py(n), pz(n);
  const uint64_t cells = G * G * G;
  std::vector<uint64_t> cbeg(cells + 1, 0);
  for (uint64_t j = 0; j < n; ++j) {
    const uint64_t i = key[j].second;
    px[j] = coord(i, 0);
    py[j] = coord(i, 1);
    pz[j] = coord(i, 2);
    cbeg[key[j].first + 1]++;
  }
  for (uint64_t c = 0; c < cells; ++c) cbeg[c + 1] += cbeg[c];
  const uint64_t R2 = R * R;
  auto ad = [](uint64_t a, uint64_t b) { return a > b ? a - b : b - a; };
  std::vector<std::vector<uint64_t>> per(omp_get_max_threads());
#pragma omp parallel
  {
    auto& mine = per[omp_get_thread_num()];
#pragma omp for schedule(dynamic, 1024)
    for (uint64_t j = 0; j < n; ++j) {
      const uint64_t cx = (px[j] * G) >> 31, cy = (py[j] * G) >> 31, cz = (pz[j] * G) >> 31;
      for (uint64_t nz = cz ? cz - 1 : 0; nz <= std::min(cz + 1, G - 1); ++nz)
        for (uint64_t ny = cy ? cy - 1 : 0; ny <= std::min(cy + 1, G - 1); ++ny)
          for (uint64_t nx = cx ? cx - 1 : 0; nx <= std::min(cx + 1, G - 1); ++nx) {
            const uint64_t c = (nz * G + ny) * G + nx;
            for (uint64_t k = cbeg[c]; k < cbeg[c + 1]; ++k) {
              if (k == j) continue;
              const uint64_t dx = ad(px[j], px[k]), dy = ad(py[j], py[k]), dz = ad(pz[j], pz[k]);
              if (dx * dx + dy * dy + dz * dz <= R2) mine.push_back((j << 32) | k);
            }
          }
    }
  }
  std::vector<uint64_t> dk;
  for (auto& v : per) dk.insert(dk.end(), v.begin(), v.end());
  __gnu_parallel::sort(dk.begin(), dk.end());
  if (distance == 0)
    return emit_sorted(dk, mix64(seed ^ gen::kWeightSalt), max_weight, out, capacity,
                       m_directed_out);
  *m_directed_out = dk.size();
  if (dk.size() > capacity) return 2;
  const uint64_t wseed = mix64(seed ^ gen::kWeightSalt);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < dk.size(); ++i) {
    const uint64_t j = dk[i] >> 32, k = dk[i] & 0xffffffffull;
    const uint64_t d2 = ad(px[j], px[k]) * ad(px[j], px[k]) + ad(py[j], py[k]) * ad(py[j], py[k]) +
                        ad(pz[j], pz[k]) * ad(pz[j], pz[k]);
    out[i] = kamsta_wedge{static_cast<uint32_t>(j), static_cast<uint32_t>(k),
                          gen::geo_weight(distance, d2, R2, wseed, std::min(j, k),
                                          std::max(j, k), max_weight)};
  }
  return 0;
}

extern "C" int oracle_gen_rmat(uint32_t log_n, uint64_t samples, double a, double b, double c,
                               uint64_t seed, uint32_t max_weight, kamsta_wedge* out,
                               uint64_t capacity, uint64_t* m_directed_out) {
  *m_directed_out = 0;
  if (max_weight == 0 || log_n > 31 || !(a >= 0) || !(b >= 0) || !(c >= 0) || a + b + c > 1.0)
    return 1;
  if (log_n == 0 || samples == 0) return 0;
  auto thr = [](double x) {
    const double t = std::floor(x * 4294967296.0);
    return t >= 4294967296.0 ? (1ull << 32) : static_cast<uint64_t>(t);
  };
  const uint64_t t1 = thr(a), t2 = thr(a + b), t3 = thr(a + b + c);
  const uint64_t base = mix64(seed ^ 0x524d4154ull);
  const uint64_t per_sample = (log_n + 1) / 2;
  std::vector<uint64_t> pairs(samples);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < samples; ++i) {
    uint64_t u = 0, v = 0;
    for (uint32_t l = 0; l < log_n; ++l) {
      const uint64_t h = mix64(base + i * per_sample + l / 2);
      const uint64_t r = (l % 2 == 0) ? (h >> 32) : (h & 0xffffffffull);
      const int bu = r < t2 ? 0 : 1;              // quadrants (0,0), (0,1) | (1,0), (1,1)
      const int bv = (r < t1 || (r >= t2 && r < t3)) ? 0 : 1;
      u = 2 * u + bu;
      v = 2 * v + bv;
    }
    pairs[i] = u == v ? ~0ull : ((std::min(u, v) << 32) | std::max(u, v));
  }
  __gnu_parallel::sort(pairs.begin(), pairs.end());
  pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
  if (!pairs.empty() && pairs.back() == ~0ull) pairs.pop_back();
  std::vector<uint64_t> dk(2 * pairs.size());
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < pairs.size(); ++i) {
    const uint64_t u = pairs[i] >> 32, v = pairs[i] & 0xffffffffull;
    dk[2 * i] = (u << 32) | v;
    dk[2 * i + 1] = (v << 32) | u;
  }
  __gnu_parallel::sort(dk.begin(), dk.end());
  return emit_sorted(dk, mix64(seed ^ gen::kWeightSalt), max_weight, out, capacity,
                     m_directed_out);
}
