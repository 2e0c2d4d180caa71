// kamsta_gpu.hpp -- header-only C++ adapter over the C ABI (kamsta_gpu.h).
//
// Gives a caller of KaMSTa the shape of its API:
//   hybridMST::boruvka(std::vector<WEdge>, const AlgorithmConfig&)
//       include/algorithms/hybrid_boruvka.hpp:263-301
//   hybridMST::filter_boruvka(std::vector<WEdge>, const AlgorithmConfig&)
//       include/algorithms/hybrid_boruvka_edgefilter.hpp:420-462
// for any edge type with get_src()/get_dst()/get_weight() and a (src, dst,
// weight) constructor (WEdge, definitions.hpp:66-84), and any config with
// local_preprocessing / compression / filter_threshold members
// (AlgorithmConfig, algorithm_configurations.hpp:27-34).  Errors are thrown
// as kamsta_gpu::error (the reference aborts the process instead).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "kamsta_gpu.h"

namespace kamsta_gpu {

struct error : std::runtime_error {
  kamsta_status status;
  error(kamsta_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

template <typename Cfg>
kamsta_cfg to_cfg(const Cfg& c) {
  kamsta_cfg k;
  kamsta_cfg_default(&k);
  k.local_preprocessing = static_cast<int32_t>(c.local_preprocessing);
  k.compression = static_cast<int32_t>(c.compression);
  k.filter_threshold = static_cast<uint64_t>(c.filter_threshold);
  return k;
}

namespace detail {
using Entry = kamsta_status (*)(const kamsta_wedge*, uint64_t, uint32_t, const kamsta_cfg*,
                                kamsta_wedge*, uint64_t*, kamsta_stats*);

template <typename Edge, typename Cfg>
std::vector<Edge> solve(Entry entry, const std::vector<Edge>& input, const Cfg& cfg) {
  uint64_t n = 0;
  std::vector<kamsta_wedge> packed(input.size());
  for (size_t i = 0; i < input.size(); ++i) {
    const uint64_t s = input[i].get_src(), d = input[i].get_dst();
    if (s > 0xfffffffeull || d > 0xfffffffeull)
      throw error(KAMSTA_E_INPUT, "kamsta_gpu: vertex id does not fit 32 bits");
    packed[i] = kamsta_wedge{static_cast<uint32_t>(s), static_cast<uint32_t>(d),
                             static_cast<uint32_t>(input[i].get_weight())};
    if (s + 1 > n) n = s + 1;
    if (d + 1 > n) n = d + 1;
  }
  const kamsta_cfg k = to_cfg(cfg);
  std::vector<kamsta_wedge> out(n > 0 ? n : 1);
  uint64_t count = 0;
  const kamsta_status s = entry(packed.data(), packed.size(), static_cast<uint32_t>(n), &k,
                                out.data(), &count, nullptr);
  if (s != KAMSTA_OK) throw error(s, kamsta_last_error());
  std::vector<Edge> mst;
  mst.reserve(count);
  for (uint64_t i = 0; i < count; ++i) mst.emplace_back(out[i].src, out[i].dst, out[i].w);
  return mst;
}
}  // namespace detail

// The forest as (min, max, w) edges; input taken by value like the reference.
template <typename Edge, typename Cfg>
std::vector<Edge> boruvka(std::vector<Edge> input, const Cfg& cfg) {
  return detail::solve(&kamsta_mst_boruvka, input, cfg);
}

template <typename Edge, typename Cfg>
std::vector<Edge> filter_boruvka(std::vector<Edge> input, const Cfg& cfg) {
  return detail::solve(&kamsta_mst_filter_boruvka, input, cfg);
}

}  // namespace kamsta_gpu
