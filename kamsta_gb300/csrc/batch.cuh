// batch.cuh -- batched solve (many graphs per launch sequence) and its wave
// planner, shared by the batch entry points and the serving loop.
#pragma once
#include <cstdint>
#include <utility>
#include <vector>

#include "solver.cuh"

namespace kamsta {

// Union ids and the forest sort keys (min << b | max) must fit: b <= 31.
constexpr uint64_t kBatchMaxVertices = 1ull << 31;
constexpr uint64_t kBatchDefaultBudget = 32ull << 30;

struct BatchWaveStats {
  uint64_t entries = 0;
  uint64_t vertices = 0;
  uint32_t launches = 0;
  double solve_ms = 0;
};

// Graphs the persistent single-CTA path takes (n <= 32768, m_directed <=
// 262144).
bool is_small_graph(const kamsta_ctx* ctx, const kamsta_graph_desc& g);

// Device bytes a graph adds to a wave at its peak (input copy, edge lists,
// forest sort, vertex arrays); used for wave planning and serving admission.
uint64_t batch_graph_bytes(uint64_t m_directed, uint32_t n);

// Device bytes the serving loop admits a device-buffer job for: one scratch
// slot of the persistent small-graph kernel when the graph goes there (its
// input is read in place), batch_graph_bytes otherwise.
uint64_t serve_job_bytes(const kamsta_ctx* ctx, const kamsta_graph_desc& g);

// Consecutive runs [first, last) of graphs whose summed bytes fit `budget`
// (a graph larger than the budget forms a wave of its own).
std::vector<std::pair<uint32_t, uint32_t>> plan_waves(const kamsta_graph_desc* g, uint32_t count,
                                                      uint64_t budget);

// One wave.  Small graphs (n <= 32768, m_directed <= 262144; device
// buffers only) go to one persistent launch on the context's auxiliary
// stream, one CTA per graph from a work queue; the others are solved as
// their disjoint union on `st`, the forest split back per graph.  Either
// way each forest is sorted by (src, dst).  host_buffers: edges/out are host
// pointers.
kamsta_status solve_wave(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t G,
                         const kamsta_cfg& cfg, bool host_buffers, cudaStream_t st,
                         BatchWaveStats* ws);

kamsta_status solve_batch(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t count,
                          const kamsta_cfg& cfg, uint64_t budget, bool host_buffers,
                          kamsta_batch_stats* st, cudaStream_t stream);

kamsta_status batch_autotune(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t count,
                             const kamsta_cfg& cfg, cudaStream_t st, kamsta_tuning* out);

}  // namespace kamsta
