// graphs/interface.hpp -- the names KaMSTa takes from its graph-generator
// wrapper (submodule external/graphs around KaGen, pin unknown, empty here),
// for the oracle's reference build: 64-bit vertex ids, a vertex range as a
// (first, last) pair and a weighted edge with accessors.
#pragma once
#include <cstdint>
#include <utility>

namespace graphs {
using VId = std::uint64_t;
using Weight = std::uint32_t;
using VertexRange = std::pair<VId, VId>;

struct WEdge {
  VId src;
  VId dst;
  Weight weight;
  VId get_src() const { return src; }
  VId get_dst() const { return dst; }
  Weight get_weight() const { return weight; }
};
}  // namespace graphs
