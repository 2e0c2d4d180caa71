// oracle.cpp -- CPU oracle and CPU baseline for the GB300 MSF solver.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h).  Reference citations are paths in
// the KaMSTa source tree.
#include "oracle.h"
#include "gen_common.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <parallel/algorithm>
#include <random>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Union-find with union by size and path compression, as
// include/datastructures/union_find.hpp:9-32 (sizes stored as negatives).
struct UnionFind {
  std::vector<int64_t> data;
  explicit UnionFind(size_t n) : data(n, -1) {}
  uint32_t find(uint32_t a) {
    uint32_t root = a;
    while (data[root] >= 0) root = static_cast<uint32_t>(data[root]);
    while (data[a] >= 0) {  // compress
      uint32_t next = static_cast<uint32_t>(data[a]);
      data[a] = root;
      a = next;
    }
    return root;
  }
  void unify(uint32_t a, uint32_t b) {
    uint32_t ra = find(a), rb = find(b);
    if (ra == rb) return;
    if (data[rb] < data[ra]) std::swap(ra, rb);
    data[ra] += data[rb];
    data[rb] = ra;
  }
};

}  // namespace

extern "C" int oracle_max_threads(void) { return omp_get_max_threads(); }

// ---------------------------------------------------------------------------
// Kruskal, restating base_case_mst_algos.hpp:91-112: sort all entries by
// WeightSrcDstOrder (utils.hpp:81-86), scan, keep an entry iff its endpoints
// are in different sets.  For an undirected edge {u<v} the (u,v) copy sorts
// before (v,u) under equal weight, so the (v,u) copy is always rejected;
// sorting only the src<dst copies therefore gives the same forest.  The
// src<dst copies arrive in (src,dst) order, so a stable sort by weight alone
// yields the (w, src, dst) order.
extern "C" int oracle_kruskal(const kamsta_wedge* edges, uint64_t m_directed,
                              uint32_t n, kamsta_wedge* out,
                              uint64_t* out_count, uint64_t* total_weight) {
  // the src<dst copies in input order (a blocked, order-preserving filter)
  const uint64_t nb = 256, bs = (m_directed + nb - 1) / nb;
  std::vector<uint64_t> cnts(nb + 1, 0);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
  for (uint64_t b = 0; b < nb; ++b) {
    uint64_t c = 0;
    for (uint64_t i = b * bs; i < std::min(m_directed, (b + 1) * bs); ++i) {
      if (edges[i].src < edges[i].dst) {
        bad |= edges[i].dst >= n;
        ++c;
      }
    }
    cnts[b + 1] = c;
  }
  if (bad) return 1;
  for (uint64_t b = 0; b < nb; ++b) cnts[b + 1] += cnts[b];
  std::vector<kamsta_wedge> und(cnts[nb]);
#pragma omp parallel for schedule(dynamic, 1)
  for (uint64_t b = 0; b < nb; ++b) {
    uint64_t o = cnts[b];
    for (uint64_t i = b * bs; i < std::min(m_directed, (b + 1) * bs); ++i)
      if (edges[i].src < edges[i].dst) und[o++] = edges[i];
  }
  // stable by weight: ties keep the (src, dst) input order, i.e. the
  // (w, min, max) order of the reference's WeightSrcDstOrder
  __gnu_parallel::stable_sort(und.begin(), und.end(),
                              [](const kamsta_wedge& a, const kamsta_wedge& b) {
                                return a.w < b.w;
                              });
  UnionFind uf(n);
  uint64_t cnt = 0, weight = 0;
  for (const auto& e : und) {
    if (uf.find(e.src) == uf.find(e.dst)) continue;
    uf.unify(e.src, e.dst);
    out[cnt++] = e;
    weight += e.w;
  }
  *out_count = cnt;
  *total_weight = weight;
  return 0;
}

// ---------------------------------------------------------------------------
// Restatement of the reference's single-rank local filter-Boruvka.
//
// On one rank the reference's hybridMST::boruvka spends its time in
// local_contraction -> execute_contraction -> boruvka_filter
// (local_contraction.hpp:114-188, local_mst_respecting_cut_edges.hpp:262-302).
// With the whole graph in one process every vertex is local, so the cut-edge
// constraints (min_cut_weights, mst_utils_cut_edges.hpp:198-225) never bind
// and are left out; everything else follows the reference step by step.
namespace port {

constexpr uint32_t kUndef = 0xffffffffu;
constexpr uint32_t kMsb = 0x80000000u;  // self-loop tag (MSD<LocalEdgeId>)

struct LocalEdge {  // WEdgeId_4_1_7-like: labels, weight, global edge id
  uint32_t src, dst, w, gid;
};

// Parallel stable pack: out[k++] = in[i] for every i with keep(i).
template <typename T, typename Keep>
size_t pack(const T* in, size_t n, T* out, Keep keep) {
  int nt = omp_get_max_threads();
  std::vector<size_t> cnt(nt + 1, 0);
#pragma omp parallel num_threads(nt)
  {
    int t = omp_get_thread_num();
    size_t lo = n * t / nt, hi = n * (t + 1) / nt, c = 0;
    for (size_t i = lo; i < hi; ++i) c += keep(i) ? 1 : 0;
    cnt[t + 1] = c;
#pragma omp barrier
#pragma omp single
    for (int k = 0; k < nt; ++k) cnt[k + 1] += cnt[k];
    size_t o = cnt[t];
    for (size_t i = lo; i < hi; ++i)
      if (keep(i)) out[o++] = in[i];
  }
  return cnt[nt];
}

// CAS-min on a packed (weight << 32 | edge id) word: the EdgeIdWeight order
// of EdgeIdWeightBaseComparator (mst_utils_common.hpp:76-81) and
// write_min_gbbs (util/atomic_ops.hpp:30-38).
inline void write_min(std::atomic<uint64_t>& a, uint64_t v) {
  uint64_t cur = a.load(std::memory_order_relaxed);
  while (v < cur && !a.compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
  }
}

struct State {
  uint32_t n_initial = 0;
  std::vector<uint32_t> parents;             // parents over all vertices
  std::vector<std::atomic<uint64_t>> min_edges;
  std::vector<uint32_t> vertices, vertices_tmp;  // SwapStorage<VId> vertices_
  std::vector<uint32_t> mst;                 // global edge ids of forest edges
  uint32_t rounds = 0;
};

struct Result {
  size_t num_mst_edges;
  size_t num_active_vertices;
};

// boruvka3, local_mst_respecting_cut_edges.hpp:101-207.
Result boruvka3(State& st, std::vector<LocalEdge>& edges, size_t n) {
  size_t m = edges.size();
  std::vector<uint32_t> edge_ids(m), edge_ids_tmp(m);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < m; ++i) edge_ids[i] = static_cast<uint32_t>(i);
  std::vector<uint32_t> exhausted;
  std::vector<uint32_t> new_mst(n, kUndef), new_mst_packed(n);
  std::vector<uint8_t> can_be_reactivated(n, 0), is_active(n, 1);
  size_t nb_mst = 0;
  uint32_t* V = st.vertices.data();
  while (n > 0 && m > 0) {
    st.rounds++;
    // compute_min_edges, mst_utils_common.hpp:84-105
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
      st.min_edges[V[i]].store(~0ull, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < m; ++i) {
      const uint32_t e = edge_ids[i];
      const LocalEdge& ed = edges[e];
      const uint64_t key = (static_cast<uint64_t>(ed.w) << 32) | e;
      write_min(st.min_edges[ed.src], key);
      write_min(st.min_edges[ed.dst], key);
    }
    // determine_mst_edges_exhausted, mst_utils_cut_edges.hpp:102-166 (no
    // cut edges: both min-cut tests pass)
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
      const uint32_t v = V[i];
      const uint64_t k = st.min_edges[v].load(std::memory_order_relaxed);
      if (k == ~0ull) {
        is_active[i] = 0;
        can_be_reactivated[i] = 1;
        new_mst[i] = kUndef;
        continue;
      }
      const uint32_t e = static_cast<uint32_t>(k);
      const uint32_t u = edges[e].src ^ edges[e].dst ^ v;
      const uint64_t ku = st.min_edges[u].load(std::memory_order_relaxed);
      if (u > v && static_cast<uint32_t>(ku) == e) {  // pseudo root: lower id
        st.parents[v] = v;
        is_active[i] = 1;
        new_mst[i] = kUndef;
      } else {
        st.parents[v] = u;
        is_active[i] = 0;
        new_mst[i] = e;
      }
    }
    // add_new_mst_edges_to_mst_array, gbbs_reimplementation.hpp:137-159
    size_t added = pack(new_mst.data(), n, new_mst_packed.data(),
                        [&](size_t i) { return new_mst[i] != kUndef; });
    size_t base = st.mst.size();
    st.mst.resize(base + added);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < added; ++i) st.mst[base + i] = edges[new_mst_packed[i]].gid;
    nb_mst += added;
    // update_parents_min_cut_weights, mst_utils_cut_edges.hpp:168-196
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
      const uint32_t v = V[i];
      while (st.parents[v] != st.parents[st.parents[v]])
        st.parents[v] = st.parents[st.parents[v]];
    }
    // identify_exhausted_vertices / compactify_vertices,
    // mst_utils_common.hpp:106-132
    {
      size_t old = exhausted.size();
      exhausted.resize(old + n);
      size_t k = pack(V, n, exhausted.data() + old,
                      [&](size_t i) { return can_be_reactivated[i] != 0; });
      exhausted.resize(old + k);
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < n; ++i) can_be_reactivated[i] = 0;
      n = pack(V, n, st.vertices_tmp.data(),
               [&](size_t i) { return is_active[i] != 0; });
      std::swap(st.vertices, st.vertices_tmp);
      V = st.vertices.data();
    }
    // relabel_edges, gbbs_reimplementation.hpp:182-203
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < m; ++i) {
      LocalEdge& ed = edges[edge_ids[i]];
      const uint32_t pu = st.parents[ed.src], pv = st.parents[ed.dst];
      ed.src = pu;
      ed.dst = pv;
      if (pu == pv) edge_ids[i] |= kMsb;
    }
    // filter_out_self_loops, mst_utils_common.hpp:157-175
    m = pack(edge_ids.data(), m, edge_ids_tmp.data(),
             [&](size_t i) { return (edge_ids[i] & kMsb) == 0; });
    std::swap(edge_ids, edge_ids_tmp);
  }
  // append exhausted vertices, final shortcut (local_mst...:195-203)
  for (size_t i = 0; i < exhausted.size(); ++i) V[n + i] = exhausted[i];
  n += exhausted.size();
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < st.n_initial; ++i)
    while (st.parents[i] != st.parents[st.parents[i]])
      st.parents[i] = st.parents[st.parents[i]];
  return Result{nb_mst, n};
}

// localMST::get_pivot, mst_utils_filter.hpp:13-30: 50 samples drawn by
// std::mt19937(0) / uniform_int_distribution<>, 25% quantile by weight.
uint32_t get_pivot(const std::vector<LocalEdge>& edges) {
  if (edges.empty()) return 1;
  if (edges.size() <= 2) return edges[0].w;
  std::mt19937 gen(0);
  std::uniform_int_distribution<> distrib(0, static_cast<int>(edges.size() - 1));
  const size_t num_samples = 50;
  std::vector<uint32_t> samples(num_samples);
  for (size_t i = 0; i < num_samples; ++i) samples[i] = edges[distrib(gen)].w;
  std::sort(samples.begin(), samples.end());
  return samples[static_cast<size_t>(num_samples * 0.25)];
}

// localMST::is_unbalanced, mst_utils_filter.hpp:32-37.
bool is_unbalanced(size_t num_edges, size_t num_light) {
  const double diff = static_cast<double>(num_edges - num_light);
  return std::abs(0.5 - diff / static_cast<double>(num_edges)) > 0.4;
}

// boruvka_filter_rec, local_mst_respecting_cut_edges.hpp:209-260.
Result filter_rec(State& st, std::vector<LocalEdge>& edges, size_t n) {
  if (n <= 1) return Result{0, n};
  if (edges.size() <= 3 * n) return boruvka3(st, edges, n);
  // localMST::partition, mst_utils_filter.hpp:39-99
  const uint32_t pivot = get_pivot(edges);
  size_t num_light = 0;
#pragma omp parallel for reduction(+ : num_light) schedule(static)
  for (size_t i = 0; i < edges.size(); ++i) num_light += edges[i].w <= pivot;
  if (is_unbalanced(edges.size(), num_light)) return boruvka3(st, edges, n);
  std::vector<LocalEdge> light(num_light);
  pack(edges.data(), edges.size(), light.data(),
       [&](size_t i) { return edges[i].w <= pivot; });
  const Result lr = filter_rec(st, light, n);
  // localMST::filter, mst_utils_filter.hpp:102-126: relabel by the final
  // parents, zero the light edges, drop self loops (stable).
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < edges.size(); ++i) {
    LocalEdge& e = edges[i];
    const bool small = e.w <= pivot;
    e.src = small ? 0 : st.parents[e.src];
    e.dst = small ? 0 : st.parents[e.dst];
  }
  std::vector<LocalEdge> heavy(edges.size());
  size_t k = pack(edges.data(), edges.size(), heavy.data(),
                  [&](size_t i) { return edges[i].src != edges[i].dst; });
  heavy.resize(k);
  Result hr = boruvka3(st, heavy, lr.num_active_vertices);
  hr.num_mst_edges += lr.num_mst_edges;
  return hr;
}

}  // namespace port

extern "C" int oracle_boruvka_filter(const kamsta_wedge* edges,
                                     uint64_t m_directed, uint32_t n,
                                     int threads, kamsta_wedge* out,
                                     uint64_t* out_count,
                                     uint64_t* total_weight,
                                     uint32_t* rounds_out) {
  using namespace port;
  if (threads > 0) omp_set_num_threads(threads);
  // get_WEdgeIds + get_local_edges (uncompressed_graph.hpp:38-51,
  // local_contraction/utils.hpp:30-36): keep the src<dst copies, global id =
  // index in the input.
  std::vector<LocalEdge> local(m_directed / 2 + 1);
  {
    int nt = omp_get_max_threads();
    std::vector<size_t> cnt(nt + 1, 0);
#pragma omp parallel num_threads(nt)
    {
      int t = omp_get_thread_num();
      size_t lo = m_directed * t / nt, hi = m_directed * (t + 1) / nt, c = 0;
      for (size_t i = lo; i < hi; ++i) c += edges[i].src < edges[i].dst;
      cnt[t + 1] = c;
#pragma omp barrier
#pragma omp single
      for (int k = 0; k < nt; ++k) cnt[k + 1] += cnt[k];
      size_t o = cnt[t];
      for (size_t i = lo; i < hi; ++i)
        if (edges[i].src < edges[i].dst)
          local[o++] = LocalEdge{edges[i].src, edges[i].dst, edges[i].w,
                                 static_cast<uint32_t>(i)};
    }
    local.resize(cnt[nt]);
  }
  State st;
  st.n_initial = n;
  st.parents.resize(n);
  st.min_edges = std::vector<std::atomic<uint64_t>>(n);
  st.vertices.resize(n);
  st.vertices_tmp.resize(n);
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n; ++i) {
    st.parents[i] = static_cast<uint32_t>(i);
    st.vertices[i] = static_cast<uint32_t>(i);
  }
  filter_rec(st, local, n);
  uint64_t weight = 0;
  const size_t k = st.mst.size();
#pragma omp parallel for reduction(+ : weight) schedule(static)
  for (size_t i = 0; i < k; ++i) {
    const kamsta_wedge& e = edges[st.mst[i]];
    out[i] = e;
    weight += e.w;
  }
  *out_count = k;
  *total_weight = weight;
  if (rounds_out) *rounds_out = st.rounds;
  return 0;
}

// ---------------------------------------------------------------------------
// Seeded G(n,m) generator.  KaGen (the reference's generator library) is not
// vendored, so both this CPU version and the device version implement the
// same definition:
//   mix64     = SplitMix64's output function (Steele, Lea, Flood 2014);
//   candidate i: h1 = mix64(base + 2i), h2 = mix64(base + 2i + 1),
//                u = hi64(h1 * n), v = hi64(h2 * n), valid iff u != v,
//                key = min << 32 | max,       base = mix64(seed);
//   the graph   = the first m distinct valid keys in candidate order (a
//                uniform m-subset of all unordered pairs);
//   weight      = 1 + hi64(mix64(wseed ^ key) * max_weight),
//                wseed = mix64(seed ^ 0x6a09e667f3bcc909).

extern "C" int oracle_gen_gnm(uint32_t n, uint64_t m, uint64_t seed,
                              uint32_t max_weight, kamsta_wedge* out,
                              uint64_t* m_directed_out) {
  using namespace gen;
  const uint64_t pairs = static_cast<uint64_t>(n) * (n - 1ull) / 2;
  if (n < 2 || m > pairs || max_weight == 0) {
    if (m == 0) {
      *m_directed_out = 0;
      return 0;
    }
    return 1;
  }
  const uint64_t base = mix64(seed);
  const uint64_t wseed = mix64(seed ^ 0x6a09e667f3bcc909ull);
  uint64_t K = m + m / 1024 + 4096;
  std::vector<uint64_t> sel;
  for (;;) {
    // (key, candidate index) for every valid candidate, sorted by key then
    // index; the first entry of each key run is its first occurrence.
    std::vector<std::pair<uint64_t, uint64_t>> c(K);
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < K; ++i) {
      uint32_t u = static_cast<uint32_t>(hi64(mix64(base + 2 * i), n));
      uint32_t v = static_cast<uint32_t>(hi64(mix64(base + 2 * i + 1), n));
      uint64_t key = ~0ull;
      if (u != v) key = (static_cast<uint64_t>(std::min(u, v)) << 32) | std::max(u, v);
      c[i] = {key, i};
    }
    __gnu_parallel::sort(c.begin(), c.end());
    // first occurrence of every key: the head of its run (invalid keys, ~0,
    // sort last and are no pair)
    std::vector<uint8_t> first(K, 0);
#pragma omp parallel for schedule(static)
    for (uint64_t j = 0; j < K; ++j) {
      if (c[j].first == ~0ull) continue;
      if (j == 0 || c[j].first != c[j - 1].first) first[c[j].second] = 1;
    }
    // T = the candidate index of the m-th first occurrence (blocked count)
    const uint64_t nb = 256;
    const uint64_t bs = (K + nb - 1) / nb;
    std::vector<uint64_t> bc(nb, 0);
#pragma omp parallel for schedule(dynamic, 1)
    for (uint64_t b = 0; b < nb; ++b) {
      uint64_t k = 0;
      for (uint64_t i = b * bs; i < std::min(K, (b + 1) * bs); ++i) k += first[i];
      bc[b] = k;
    }
    uint64_t cnt = 0, T = K;
    for (uint64_t b = 0; b < nb && T == K; ++b) {
      if (cnt + bc[b] < m) {
        cnt += bc[b];
        continue;
      }
      for (uint64_t i = b * bs; i < std::min(K, (b + 1) * bs); ++i) {
        cnt += first[i];
        if (cnt == m) {
          T = i;
          break;
        }
      }
    }
    if (T == K) {  // not enough distinct pairs yet: draw more
      K = K + (m - cnt) * 2 + 4096;
      continue;
    }
    // the selected keys in key order: run heads with candidate index <= T
    auto take = [&](uint64_t j) {
      return c[j].first != ~0ull && (j == 0 || c[j].first != c[j - 1].first) && c[j].second <= T;
    };
    std::vector<uint64_t> sc(nb, 0);
#pragma omp parallel for schedule(dynamic, 1)
    for (uint64_t b = 0; b < nb; ++b) {
      uint64_t k = 0;
      for (uint64_t j = b * bs; j < std::min(K, (b + 1) * bs); ++j) k += take(j);
      sc[b] = k;
    }
    uint64_t tot = 0;
    for (auto& x : sc) {
      const uint64_t y = x;
      x = tot;
      tot += y;
    }
    sel.resize(tot);
#pragma omp parallel for schedule(dynamic, 1)
    for (uint64_t b = 0; b < nb; ++b) {
      uint64_t o = sc[b];
      for (uint64_t j = b * bs; j < std::min(K, (b + 1) * bs); ++j)
        if (take(j)) sel[o++] = c[j].first;
    }
    break;
  }
  // Both directions sorted by (src, dst): row x = lower neighbours (pairs
  // (u, x), in increasing u) followed by upper neighbours (pairs (x, v), in
  // increasing v).  sel is sorted by (u, v); the reversed keys (v << 32 | u),
  // sorted, give every row's lower neighbours in order.
  const uint64_t ms = sel.size();
  std::vector<uint64_t> rev(ms);
#pragma omp parallel for schedule(static)
  for (uint64_t j = 0; j < ms; ++j) rev[j] = (sel[j] << 32) | (sel[j] >> 32);
  __gnu_parallel::sort(rev.begin(), rev.end());
  std::vector<uint64_t> updeg(n + 1, 0), lowdeg(n + 1, 0);
#pragma omp parallel for schedule(static)
  for (uint64_t j = 0; j < ms; ++j) {
    __atomic_fetch_add(&updeg[sel[j] >> 32], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&lowdeg[rev[j] >> 32], 1, __ATOMIC_RELAXED);
  }
  // row offsets, and the first index of each row's run in sel and in rev
  std::vector<uint64_t> row(n + 1), up0(n + 1), low0(n + 1);
  uint64_t off = 0, a = 0, b = 0;
  for (uint32_t x = 0; x < n; ++x) {
    row[x] = off;
    up0[x] = a;
    low0[x] = b;
    off += lowdeg[x] + updeg[x];
    a += updeg[x];
    b += lowdeg[x];
  }
#pragma omp parallel for schedule(static)
  for (uint64_t j = 0; j < ms; ++j) {
    const uint64_t key = sel[j];
    const uint32_t u = static_cast<uint32_t>(key >> 32), v = static_cast<uint32_t>(key);
    const uint32_t w = 1 + static_cast<uint32_t>(hi64(mix64(wseed ^ key), max_weight));
    out[row[u] + lowdeg[u] + (j - up0[u])] = kamsta_wedge{u, v, w};
    const uint64_t rk = rev[j];
    const uint32_t rv = static_cast<uint32_t>(rk >> 32), ru = static_cast<uint32_t>(rk);
    const uint64_t ckey = (static_cast<uint64_t>(ru) << 32) | rv;
    const uint32_t rw = 1 + static_cast<uint32_t>(hi64(mix64(wseed ^ ckey), max_weight));
    out[row[rv] + (j - low0[rv])] = kamsta_wedge{rv, ru, rw};
  }
  *m_directed_out = 2 * sel.size();
  return 0;
}

// ---------------------------------------------------------------------------
// Seeded 2-D random geometric graph (stand-in for KaGen's get_rgg2D,
// benchmarks/mst_benchmarks.hpp:133-139, which the reference tree does not
// vendor).  The definition, shared with the device generator
// kamsta_gen_rgg2d_dev:
//   base = mix64(seed ^ 0x5247473244ull); point i (i < n) has 31-bit integer
//   coordinates x = mix64(base + 2i) >> 33, y = mix64(base + 2i + 1) >> 33;
//   R = floor(radius * 2^31) (radius clamped to [0, 1]); u ~ v iff u != v and
//   dx^2 + dy^2 <= R^2 (exact in 64-bit integers);
//   G = cells per side = min(floor(2^31 / R), isqrt(n), 65536), at least 1
//   (cells at least R wide); cell = (y*G >> 31) * G + (x*G >> 31);
//   vertex ids = ranks of the points sorted by (cell, i);
//   weights as in the G(n,m) generator, both directions, (src,dst) sorted.
namespace gen {

struct RggParams {
  uint64_t R;
  uint64_t G;
};

inline uint64_t isqrt64(uint64_t n) {
  uint64_t s = static_cast<uint64_t>(std::sqrt(static_cast<double>(n)));
  while (s * s > n) --s;
  while ((s + 1) * (s + 1) <= n) ++s;
  return s;
}

inline RggParams rgg_params(uint32_t n, double radius) {
  RggParams p;
  if (!(radius > 0)) p.R = 0;
  else if (radius >= 1) p.R = 1ull << 31;
  else p.R = static_cast<uint64_t>(radius * 2147483648.0);
  uint64_t cap = std::min<uint64_t>(std::max<uint64_t>(isqrt64(n), 1), 65536);
  p.G = p.R == 0 ? cap : std::max<uint64_t>(1, std::min<uint64_t>((1ull << 31) / p.R, cap));
  return p;
}

}  // namespace gen

extern "C" int oracle_gen_rgg2d(uint32_t n, double radius, uint64_t seed, uint32_t max_weight,
                                uint32_t distance, kamsta_wedge* out, uint64_t capacity,
                                uint64_t* m_directed_out) {
  using namespace gen;
  *m_directed_out = 0;
  if (max_weight == 0 || distance > 2) return 1;
  if (n == 0) return 0;
  const RggParams P = rgg_params(n, radius);
  const uint64_t base = mix64(seed ^ 0x5247473244ull);
  const uint64_t wseed = mix64(seed ^ 0x6a09e667f3bcc909ull);
  const uint64_t G = P.G, R2 = P.R * P.R;
  std::vector<uint64_t> key(n);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t x = mix64(base + 2 * i) >> 33, y = mix64(base + 2 * i + 1) >> 33;
    const uint64_t cell = ((y * G) >> 31) * G + ((x * G) >> 31);
    key[i] = (cell << 32) | i;
  }
  std::sort(key.begin(), key.end());
  std::vector<uint64_t> px(n), py(n);
  const uint64_t cells = G * G;
  std::vector<uint64_t> cbeg(cells + 1, 0);
  for (uint64_t j = 0; j < n; ++j) {
    const uint64_t i = key[j] & 0xffffffffull;
    px[j] = mix64(base + 2 * i) >> 33;
    py[j] = mix64(base + 2 * i + 1) >> 33;
    cbeg[(key[j] >> 32) + 1]++;
  }
  for (uint64_t c = 0; c < cells; ++c) cbeg[c + 1] += cbeg[c];
  auto visit = [&](uint64_t j, auto&& emit) {
    const uint64_t cx = (px[j] * G) >> 31, cy = (py[j] * G) >> 31;
    for (uint64_t ny = cy ? cy - 1 : 0; ny <= std::min(cy + 1, G - 1); ++ny)
      for (uint64_t nx = cx ? cx - 1 : 0; nx <= std::min(cx + 1, G - 1); ++nx) {
        const uint64_t c = ny * G + nx;
        for (uint64_t k = cbeg[c]; k < cbeg[c + 1]; ++k) {
          if (k == j) continue;
          const uint64_t dx = px[j] > px[k] ? px[j] - px[k] : px[k] - px[j];
          const uint64_t dy = py[j] > py[k] ? py[j] - py[k] : py[k] - py[j];
          if (dx * dx + dy * dy <= R2) emit(k, dx * dx + dy * dy);
        }
      }
  };
  std::vector<uint64_t> off(static_cast<uint64_t>(n) + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t j = 0; j < n; ++j) {
    uint64_t d = 0;
    visit(j, [&](uint64_t, uint64_t) { ++d; });
    off[j + 1] = d;
  }
  for (uint64_t j = 0; j < n; ++j) off[j + 1] += off[j];
  *m_directed_out = off[n];
  if (off[n] > capacity) return 2;
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint64_t j = 0; j < n; ++j) {
    uint64_t o = off[j];
    visit(j, [&](uint64_t k, uint64_t d2) {
      const uint32_t w = geo_weight(distance, d2, R2, wseed, std::min(j, k), std::max(j, k),
                                    max_weight);
      out[o++] = kamsta_wedge{static_cast<uint32_t>(j), static_cast<uint32_t>(k), w};
    });
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Seeded threshold random hyperbolic graph (stand-in for KaGen's get_rhg,
// benchmarks/mst_benchmarks.hpp:152-158).  The definition, shared with the
// device generator kamsta_gen_rhg_dev:
//   alpha = (gamma - 1) / 2 (gamma > 2), xi = alpha / (alpha - 1/2),
//   disk radius R = max(1, 2 ln(2 xi^2 n / (pi k))) (the asymptotic
//   threshold-RHG degree formula, k = target average degree);
//   base = mix64(seed ^ 0x524847); point i: u = (mix64(base + 2i) >> 11) 2^-53,
//   v = (mix64(base + 2i + 1) >> 11) 2^-53,
//   r = min(R, acosh(1 + u (cosh(alpha R) - 1)) / alpha), theta = 2 pi v;
//   per point E = exp(r), Ei = exp(-r), S = sinh(r) (C library functions on
//   the host), band = min(15, floor(16 r / R));
//   ids = ranks of the points sorted by (band, bits(theta) >> 5, i);
//   p ~ q (a = lower id, b = higher id) iff
//     ((2 s) s) S_a S_b <= cosh R - 0.5 (E_a Ei_b + Ei_a E_b),
//   s = hsin(d / 2), d = |theta_a - theta_b| folded to [0, pi], hsin the
//   degree-21 Taylor polynomial of sin in the fixed Horner order below; all
//   arithmetic in double, round to nearest, no fused multiply-add.
// Candidates come from per-band angular windows that contain every pair the
// test can accept (derived from sin^2(d/2) <= cosh R / (2 S_p sinh(b_lo))
// with generous margins), so the edge set does not depend on the window.
namespace gen {

constexpr int kRhgBands = 16;
constexpr double kTwoPi = 6.283185307179586;
constexpr double kPi = 3.141592653589793;

inline double rhg_hsin(double x) {
  const double x2 = x * x;
  double t = 1.0 - x2 / 420.0;
  t = 1.0 - x2 / 342.0 * t;
  t = 1.0 - x2 / 272.0 * t;
  t = 1.0 - x2 / 210.0 * t;
  t = 1.0 - x2 / 156.0 * t;
  t = 1.0 - x2 / 110.0 * t;
  t = 1.0 - x2 / 72.0 * t;
  t = 1.0 - x2 / 42.0 * t;
  t = 1.0 - x2 / 20.0 * t;
  t = 1.0 - x2 / 6.0 * t;
  return x * t;
}

struct RhgPoint {
  double theta, E, Ei, S;
  uint64_t key;  // band << 58 | bits(theta) >> 5
};

inline double rhg_radius(uint32_t n, double gamma, double k) {
  const double alpha = (gamma - 1.0) / 2.0;
  const double xi = alpha / (alpha - 0.5);
  const double R = 2.0 * std::log(2.0 * xi * xi * n / (kPi * k));
  return R > 1.0 ? R : 1.0;  // tiny graphs: at least a unit disk
}

inline RhgPoint rhg_point(uint64_t base, uint64_t i, double alpha, double R, double coshAR1) {
  const double u = static_cast<double>(mix64(base + 2 * i) >> 11) * 0x1.0p-53;
  const double v = static_cast<double>(mix64(base + 2 * i + 1) >> 11) * 0x1.0p-53;
  double r = std::acosh(1.0 + u * coshAR1) / alpha;
  if (r > R) r = R;
  RhgPoint p;
  p.theta = kTwoPi * v;
  p.E = std::exp(r);
  p.Ei = std::exp(-r);
  p.S = std::sinh(r);
  int band = static_cast<int>(std::floor(r * kRhgBands / R));
  if (band > kRhgBands - 1) band = kRhgBands - 1;
  if (band < 0) band = 0;
  uint64_t tb;
  std::memcpy(&tb, &p.theta, sizeof(tb));
  p.key = (static_cast<uint64_t>(band) << 58) | (tb >> 5);
  return p;
}

inline bool rhg_edge(const RhgPoint& a, const RhgPoint& b, double coshR) {
  double d = a.theta > b.theta ? a.theta - b.theta : b.theta - a.theta;
  if (d > kPi) d = kTwoPi - d;
  const double s = rhg_hsin(d * 0.5);
  const double lhs = 2.0 * s * s * a.S * b.S;
  const double rhs = coshR - 0.5 * (a.E * b.Ei + a.Ei * b.E);
  return lhs <= rhs;
}

}  // namespace gen

extern "C" int oracle_gen_rhg(uint32_t n, double gamma, double avg_degree, uint64_t seed,
                              uint32_t max_weight, kamsta_wedge* out, uint64_t capacity,
                              uint64_t* m_directed_out) {
  using namespace gen;
  *m_directed_out = 0;
  if (max_weight == 0 || !(gamma > 2.0) || !(avg_degree > 0)) return 1;
  if (n == 0) return 0;
  const double alpha = (gamma - 1.0) / 2.0;
  const double R = rhg_radius(n, gamma, avg_degree);
  if (!(R > 0)) return 1;
  const double coshR = std::cosh(R), coshAR1 = std::cosh(alpha * R) - 1.0;
  const uint64_t base = mix64(seed ^ 0x524847ull);
  const uint64_t wseed = mix64(seed ^ 0x6a09e667f3bcc909ull);
  std::vector<RhgPoint> pt(n);
  std::vector<std::pair<uint64_t, uint32_t>> order(n);
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < n; ++i) {
    pt[i] = rhg_point(base, i, alpha, R, coshAR1);
    order[i] = {pt[i].key, static_cast<uint32_t>(i)};
  }
  std::sort(order.begin(), order.end());
  std::vector<RhgPoint> P(n);
  for (uint64_t j = 0; j < n; ++j) P[j] = pt[order[j].second];
  std::vector<uint64_t> bstart(kRhgBands + 1, 0);
  for (int b = 0; b <= kRhgBands; ++b) {
    const uint64_t x = static_cast<uint64_t>(b) << 58;
    bstart[b] = std::lower_bound(order.begin(), order.end(), std::make_pair(x, 0u)) - order.begin();
  }
  std::vector<double> sh_lo(kRhgBands);
  for (int b = 0; b < kRhgBands; ++b) sh_lo[b] = std::sinh(R * b / kRhgBands);
  auto tkey = [](double t) {
    uint64_t tb;
    std::memcpy(&tb, &t, sizeof(tb));
    return tb >> 5;
  };
  // index range [lo, hi) of band b whose (truncated) angle lies in [t0, t1]
  auto range = [&](int b, double t0, double t1, uint64_t* lo, uint64_t* hi) {
    const uint64_t bk = static_cast<uint64_t>(b) << 58;
    auto first = order.begin() + bstart[b], last = order.begin() + bstart[b + 1];
    *lo = std::lower_bound(first, last, std::make_pair(bk | tkey(t0), 0u)) - order.begin();
    *hi = std::upper_bound(first, last, std::make_pair(bk | tkey(t1), 0xffffffffu)) -
          order.begin();
  };
  auto visit = [&](uint64_t j, auto&& emit) {
    const RhgPoint& p = P[j];
    for (int b = 0; b < kRhgBands; ++b) {
      if (bstart[b] == bstart[b + 1]) continue;
      bool full = sh_lo[b] <= 0.0 || p.S <= 0.0;
      double D = 0;
      if (!full) {
        const double s = std::sqrt(coshR / (2.0 * p.S * sh_lo[b])) * (1.0 + 1e-6);
        if (s >= 1.0) full = true;
        else {
          D = 2.0 * std::asin(s) + 1e-9;
          if (D >= kPi) full = true;
        }
      }
      uint64_t r0 = bstart[b], r1 = bstart[b], r2 = bstart[b], r3 = bstart[b];
      if (full) {
        r1 = bstart[b + 1];
      } else {
        const double lo = p.theta - D, hi = p.theta + D;
        if (lo < 0) {
          range(b, 0.0, hi, &r0, &r1);
          range(b, lo + kTwoPi, kTwoPi, &r2, &r3);
        } else if (hi >= kTwoPi) {
          range(b, 0.0, hi - kTwoPi, &r0, &r1);
          range(b, lo, kTwoPi, &r2, &r3);
        } else {
          range(b, lo, hi, &r0, &r1);
        }
      }
      for (int part = 0; part < 2; ++part) {
        const uint64_t a0 = part ? r2 : r0, a1 = part ? r3 : r1;
        for (uint64_t k = a0; k < a1; ++k) {
          if (k == j) continue;
          const bool e = j < k ? rhg_edge(P[j], P[k], coshR) : rhg_edge(P[k], P[j], coshR);
          if (e) emit(k);
        }
      }
    }
  };
  std::vector<uint64_t> off(static_cast<uint64_t>(n) + 1, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (uint64_t j = 0; j < n; ++j) {
    uint64_t d = 0;
    visit(j, [&](uint64_t) { ++d; });
    off[j + 1] = d;
  }
  for (uint64_t j = 0; j < n; ++j) off[j + 1] += off[j];
  *m_directed_out = off[n];
  if (off[n] > capacity) return 2;
#pragma omp parallel for schedule(dynamic, 256)
  for (uint64_t j = 0; j < n; ++j) {
    uint64_t o = off[j];
    visit(j, [&](uint64_t k) {
      const uint64_t canon = (std::min(j, k) << 32) | std::max(j, k);
      const uint32_t w = 1 + static_cast<uint32_t>(hi64(mix64(wseed ^ canon), max_weight));
      out[o++] = kamsta_wedge{static_cast<uint32_t>(j), static_cast<uint32_t>(k), w};
    });
  }
  return 0;
}
