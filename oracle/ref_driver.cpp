// ref_driver.cpp -- runs KaMSTa's OWN single-rank local filter-Boruvka.
//
// THIS IS TEST INFRASTRUCTURE (the oracle's reference build), NOT THE
// PRODUCT.  Only tests/ and bench.py's CPU-baseline / reference arms load
// the library built from it (oracle/_ref/libkamsta_ref.so).
//
// The reference's headers are compiled unchanged from their own source tree
// (oracle/ref_build.py); the MPI, parlay, KaGen-interface and IPS4o names
// they use come from oracle/ref_shim/ (single rank, OpenMP).  This file only
// drives them, in the order the reference's single-rank preprocessing does:
//   UncompressedGraph<WEdge_4_1, WEdgeId_4_1_7>::get_WEdgeIds
//       (hybrid_boruvka.hpp:277-285, uncompressed_graph.hpp:38-51; the
//       edge types the benchmark picks for n < 2^32 and weights <= 255,
//       benchmarks/mst.cpp:295-301)
//   execute_contraction (local_contraction.hpp:114-150):
//       compute_min_cut_weights (mst_utils_cut_edges.hpp:198-225)
//       get_local_edges          (local_contraction/utils.hpp:38-56)
//       boruvka_filter           (local_mst_respecting_cut_edges.hpp:262-302)
// On one rank the first and the last vertex count as cut vertices
// (is_true_local, local_contraction/utils.hpp:10-13), so the local phase
// leaves the edges at those two vertices, and edges heavier than both
// endpoints' lightest cut edge, to the reference's distributed rounds
// (boruvka_core, hybrid_boruvka.hpp:108-222), which need MPI exchanges.  Those
// few edges are finished here by Kruskal over the contracted graph under the
// (w, min(u,v), max(u,v)) order (base_case_mst_algos.hpp:91-112); the count
// is reported (finish_edges) so a caller can see how little that is.
//
// A second entry point runs the same boruvka_filter with every vertex local
// (no cut vertices, no cut-edge weights): the algorithm oracle.cpp's
// port::filter_rec restates, so the two can be compared bit for bit.
#include "algorithms/gbbs_reimplementation.hpp"
#include "algorithms/local_contraction/local_boruvka/local_mst_respecting_cut_edges.hpp"
#include "algorithms/local_contraction/utils.hpp"
#include "datastructures/compression/uncompressed_graph.hpp"

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <iostream>
#include <numeric>
#include <sstream>
#include <vector>

namespace {

struct Edge12 {  // the layout of kamsta_wedge: u32 src, dst, w
  uint32_t src, dst, w;
};

using EdgeType = hybridMST::WEdge_4_1;
using EdgeIdType = hybridMST::WEdgeId_4_1_7;

// The reference prints progress on rank 0 (boruvka3's `print`, the pivot,
// the local timer); a caller's stdout stays clean.
struct MuteStdout {
  std::ostringstream sink;
  std::streambuf* old;
  MuteStdout() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~MuteStdout() { std::cout.rdbuf(old); }
};

struct UnionFind {
  std::vector<uint64_t> p;
  explicit UnionFind(size_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
  uint64_t find(uint64_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct RunOut {
  std::vector<uint64_t> forest;  // input positions (src < dst copies)
  uint64_t local_forest = 0;     // found by the reference's local phase
  uint64_t finish_edges = 0;     // edges left to the distributed rounds
  double local_s = 0, finish_s = 0;
};

// all_local: every vertex local, no cut-edge weights (the port's algorithm);
// otherwise the reference's single-rank local_contraction.  The clock starts
// once the input std::vector<WEdge> exists, as the reference benchmark's
// "mst_complete" timer does (benchmarks/mst.cpp:210-229).
// The benchmark's input edges, built before its timer starts (kept between
// runs on the same input: the reference only reads them).
struct Input {
  const Edge12* in = nullptr;
  uint64_t m = 0;
  hybridMST::non_init_vector<hybridMST::WEdge> wedges;
};
Input g_input;

int set_input(const Edge12* in, uint64_t m) {
  using namespace hybridMST;
  uint64_t wide = 0;
#pragma omp parallel for schedule(static) reduction(+ : wide)
  for (uint64_t i = 0; i < m; ++i) wide += in[i].w > 255;
  if (wide) return 2;  // WEdge_4_1 holds 8-bit weights
  g_input.in = in;
  g_input.m = m;
  g_input.wedges = non_init_vector<WEdge>(m);
  parallel_for(0, m, [&](size_t i) { g_input.wedges[i] = WEdge(in[i].src, in[i].dst, in[i].w); });
  return 0;
}

int run(bool all_local, RunOut& r) {
  using namespace hybridMST;
  const Edge12* in = g_input.in;
  const uint64_t m = g_input.m;
  if (m == 0) return 0;
  MuteStdout mute;
  auto& input = g_input.wedges;
  const double t0 = now_s();
  // boruvka(): the edge container and the edges with global ids
  // (hybrid_boruvka.hpp:277-285, :230)
  UncompressedGraph<EdgeType, EdgeIdType> container(std::move(input), 0);
  auto edges = container.get_WEdgeIds();
  const VertexRange_ range(edges.front().get_src(), edges.back().get_src() + 1);
  const auto normal = [&](VId v) { return normalize_v(v, range); };

  non_init_vector<std::atomic<EdgeIdWeight>> min_cut;
  parlay::sequence<EdgeIdType> local_edges;
  if (all_local) {
    min_cut = non_init_vector<std::atomic<EdgeIdWeight>>(range.n());
    parallel_for(0, range.n(), [&](size_t i) {
      min_cut[i] = EdgeIdWeight{LOCAL_EDGEID_UNDEFINED, WEIGHT_MAX};
    });
    local_edges = parlay::filter(edges, [](const EdgeIdType& e) { return e.get_src() < e.get_dst(); });
  } else {
    // local_contraction(): the share of true-local edges decides whether the
    // local phase runs at all (threshold 0.1, local_contraction.hpp:237-263)
    const size_t nb_local = parlay::count_if(
        edges, [&](const auto& e) { return is_true_local(e, range); });
    if (static_cast<double>(nb_local) / static_cast<double>(edges.size()) <= 0.1) {
      min_cut = non_init_vector<std::atomic<EdgeIdWeight>>(range.n());
      parallel_for(0, range.n(), [&](size_t i) {
        min_cut[i] = EdgeIdWeight{LOCAL_EDGEID_UNDEFINED, WEIGHT_MAX};
      });
    } else {
      // execute_contraction() (local_contraction.hpp:114-150)
      min_cut = compute_min_cut_weights(
          Span<EdgeIdType>(edges.data(), edges.size()), range,
          [&range](const auto& e) { return is_true_local(e, range); });
      local_edges = get_local_edges(edges, range, min_cut);
    }
  }
  auto parents = parlay::sequence<VId>::from_function(
      range.n(), [&](size_t i) { return range.v_begin + i; });
  non_init_vector<GlobalEdgeId> mst_ids(range.n());
  size_t found = 0;
  if (local_edges.size())
    found = boruvka_filter(
        range, Span<EdgeIdType>(local_edges.data(), local_edges.size()),
        Span<EdgeIdType>(edges.data(), edges.size()),
        Span<std::atomic<EdgeIdWeight>>(min_cut.data(), min_cut.size()),
        Span<VId>(parents.data(), parents.size()), mst_ids.data());
  const double t1 = now_s();
  r.local_forest = found;
  r.forest.assign(mst_ids.begin(), mst_ids.begin() + found);

  // The edges the local phase left: endpoints in different components.
  // Stand-in for the distributed rounds: nearly every vertex ends in one
  // giant component, so only the rows of the vertices outside it are
  // scanned (an edge between two components has an endpoint outside the
  // giant); when many vertices are outside, every entry is checked.  Then
  // Kruskal over the candidates under the (w, min, max) order.
  const size_t nr = range.n();
  const VId giant = parents[nr / 2];
  auto outside = parlay::filter(
      parlay::delayed_seq<uint64_t>(nr, [](size_t i) { return static_cast<uint64_t>(i); }),
      [&](uint64_t i) { return parents[i] != giant; });
  std::vector<uint64_t> rest;
  auto differ = [&](uint64_t i) {
    return parents[normal(in[i].src)] != parents[normal(in[i].dst)];
  };
  if (outside.size() <= nr / 16) {
    std::vector<std::vector<uint64_t>> part(omp_get_max_threads());
#pragma omp parallel for schedule(dynamic, 64)
    for (size_t k = 0; k < outside.size(); ++k) {
      const uint64_t v = range.v_begin + outside[k];
      const Edge12* row = std::lower_bound(in, in + m, v, [](const Edge12& e, uint64_t x) {
        return e.src < x;
      });
      auto& mine = part[omp_get_thread_num()];
      for (const Edge12* e = row; e < in + m && e->src == v; ++e) {
        const bool u_out = parents[normal(e->dst)] != giant;
        // an edge between two outside vertices is taken from its src < dst copy
        if (differ(static_cast<uint64_t>(e - in)) && (!u_out || e->src < e->dst))
          mine.push_back(static_cast<uint64_t>(e - in));
      }
    }
    for (auto& p : part) rest.insert(rest.end(), p.begin(), p.end());
  } else {
    auto rest_seq = parlay::filter(
        parlay::delayed_seq<uint64_t>(m, [](size_t i) { return static_cast<uint64_t>(i); }),
        [&](uint64_t i) { return in[i].src < in[i].dst && differ(i); });
    rest.assign(rest_seq.begin(), rest_seq.end());
  }
  r.finish_edges = rest.size();
  auto key = [&](uint64_t i) {
    return std::make_tuple(in[i].w, std::min(in[i].src, in[i].dst),
                           std::max(in[i].src, in[i].dst));
  };
  ips4o::parallel::sort(rest.begin(), rest.end(),
                        [&](uint64_t a, uint64_t b) { return key(a) < key(b); });
  UnionFind uf(nr);
  for (uint64_t i : rest) {
    const uint64_t a = uf.find(normal(parents[normal(in[i].src)]));
    const uint64_t b = uf.find(normal(parents[normal(in[i].dst)]));
    if (a == b) continue;
    uf.p[a] = b;
    r.forest.push_back(i);
  }
  r.finish_s = now_s() - t1;
  r.local_s = t1 - t0;
  return 0;
}

int emit(const Edge12* in, const RunOut& r, Edge12* out, uint64_t* out_count,
         uint64_t* total_weight) {
  uint64_t w = 0;
  for (size_t k = 0; k < r.forest.size(); ++k) {
    out[k] = in[r.forest[k]];
    w += in[r.forest[k]].w;
  }
  *out_count = r.forest.size();
  *total_weight = w;
  return 0;
}

}  // namespace

extern "C" {

// Keeps the input (the caller's array must stay valid until the next call
// of ref_set_input or ref_clear_input) and its std::vector<WEdge> copy.
// Returns 2 for weights > 255.
int ref_set_input(const Edge12* in, uint64_t m) { return set_input(in, m); }

void ref_clear_input() {
  g_input.in = nullptr;
  g_input.m = 0;
  hybridMST::non_init_vector<hybridMST::WEdge>().swap(g_input.wedges);
}

// One run on the kept input.  all_local = 0: the reference's single-rank
// MODIFIED_BORUVKA preprocessing, finished as described above; 1: its
// boruvka_filter with every vertex local.  out needs room for n - 1 entries.
// info (optional, 4 doubles): local-phase forest edges, edges left to the
// distributed rounds, seconds of the reference's part, seconds of the finish.
int ref_run(int threads, int all_local, Edge12* out, uint64_t* out_count,
            uint64_t* total_weight, double* info) {
  if (threads > 0) omp_set_num_threads(threads);
  RunOut r;
  const int rc = run(all_local != 0, r);
  if (rc) return rc;
  if (info) {
    info[0] = static_cast<double>(r.local_forest);
    info[1] = static_cast<double>(r.finish_edges);
    info[2] = r.local_s;
    info[3] = r.finish_s;
  }
  return emit(g_input.in, r, out, out_count, total_weight);
}

// ref_set_input + ref_run + ref_clear_input.
int ref_local_contraction(const Edge12* in, uint64_t m, int threads, Edge12* out,
                          uint64_t* out_count, uint64_t* total_weight, double* info) {
  int rc = set_input(in, m);
  if (rc == 0) rc = ref_run(threads, 0, out, out_count, total_weight, info);
  ref_clear_input();
  return rc;
}

int ref_boruvka_filter_all_local(const Edge12* in, uint64_t m, int threads, Edge12* out,
                                 uint64_t* out_count, uint64_t* total_weight, double* info) {
  int rc = set_input(in, m);
  if (rc == 0) rc = ref_run(threads, 1, out, out_count, total_weight, info);
  ref_clear_input();
  return rc;
}

int ref_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
