// batch.cu -- many graphs per solve.
//
// A wave of graphs is solved as ONE graph: their disjoint union, with graph
// g's vertex ids shifted by voff_g = n_0 + ... + n_{g-1}.  The minimum
// spanning forest of a disjoint union is the union of the forests, and the
// shift is monotone, so the (w, min, max) order inside every graph -- and
// with it each graph's canonical forest -- is unchanged.  The union goes
// through the same kernels as one large graph (full-width launches instead
// of thousands of tiny ones), and the forest is then split back per graph:
//   k_batch_gather   copy the wave's inputs into one union array, adding
//                    voff to src/dst (u32 words, coalesced); an id >= n_g is
//                    replaced by an id the solver skips and flags graph g
//   k_batch_order    (KAMSTA_FLAG_VALIDATE) per-graph (src,dst) order check
//   solve_device     the single-graph solver over the union
//   k_batch_keys     forest edges -> 64-bit (min, max) keys + weights
//   radix sort       by (min, max): groups the forest by graph (voff is
//                    monotone) and orders each graph's edges by (src, dst)
//   k_batch_bounds   first forest entry of every graph (binary search)
//   k_batch_scatter  un-shift and write to each graph's output; per-graph
//                    weight sums
// The reference has no batch API: its benchmark solves one graph per MPI
// job (benchmarks/mst.cpp:215-228); the result of each graph here equals a
// kamsta_mst_boruvka call on that graph alone, sorted by (src, dst).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "sort_gen.cuh"
#include "solver.cuh"
#include "batch.cuh"

namespace kamsta {

namespace {

constexpr int kBatchBlock = 256;
constexpr int kGatherWords = 16;  // u32 words per thread in k_batch_gather
constexpr uint32_t kSkipId = 0xffffffffu;

// Device-side wave table (structure of arrays, one allocation).
struct WaveTable {
  const uint32_t** edges;  // [G] graph input as u32 words
  uint32_t** out;          // [G] graph output as u32 words
  uint64_t* eoff;          // [G+1] first union entry of graph g
  uint64_t* voff;          // [G+1] first union vertex of graph g
  uint32_t* n;             // [G]
  uint64_t* begin;         // [G+1] first sorted forest entry of graph g
  uint64_t* weight;        // [G]
  uint32_t* err;           // [G] bit 0: id out of range, bit 1: order
  uint32_t G;
};

__device__ __forceinline__ uint32_t upper_graph(const uint64_t* off, uint32_t G, uint64_t x) {
  // last g with off[g] <= x (off[0] == 0, off is non-decreasing)
  uint32_t lo = 0, hi = G;  // answer in [lo, hi)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// Union words [c0, c1) per CTA; thread-strided inside the chunk so that each
// warp reads and writes 128 contiguous bytes per step.  Words 0 and 1 of an
// entry are ids (shifted by voff), word 2 the weight.
__global__ void __launch_bounds__(kBatchBlock)
    k_batch_gather(WaveTable t, uint32_t* __restrict__ uni, uint64_t words) {
  __shared__ uint32_t s_g0;
  const uint64_t chunk = static_cast<uint64_t>(kBatchBlock) * kGatherWords;
  for (uint64_t c0 = blockIdx.x * chunk; c0 < words; c0 += static_cast<uint64_t>(gridDim.x) * chunk) {
    __syncthreads();
    if (threadIdx.x == 0) {
      // graph of entry c0 / 3: last g with eoff[g] <= entry, skipping empty graphs
      s_g0 = upper_graph(t.eoff, t.G, c0 / 3);
    }
    __syncthreads();
    uint32_t g = s_g0;
    uint64_t gend = 3 * t.eoff[g + 1];
    uint64_t gbeg = 3 * t.eoff[g];
#pragma unroll 4
    for (int j = 0; j < kGatherWords; ++j) {
      const uint64_t q = c0 + static_cast<uint64_t>(j) * kBatchBlock + threadIdx.x;
      if (q >= words) break;
      while (q >= gend) {
        ++g;
        gbeg = gend;
        gend = 3 * t.eoff[g + 1];
      }
      const uint64_t local = q - gbeg;
      uint32_t v = t.edges[g][local];
      if (local % 3 != 2) {
        if (v >= t.n[g]) {
          atomicOr(&t.err[g], 1u);
          v = kSkipId;
        } else {
          v += static_cast<uint32_t>(t.voff[g]);
        }
      }
      uni[q] = v;
    }
  }
}

// Per-graph (src, dst) strictly-increasing check over the graph's own input.
__global__ void __launch_bounds__(kBatchBlock)
    k_batch_order(WaveTable t, uint64_t entries) {
  for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < entries;
       e += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t g = upper_graph(t.eoff, t.G, e);
    const uint64_t i = e - t.eoff[g];
    if (i == 0) continue;
    const uint32_t* p = t.edges[g] + 3 * i;
    const uint32_t s = p[0], d = p[1], ps = p[-3], pd = p[-2];
    if (s < ps || (s == ps && d <= pd)) atomicOr(&t.err[g], 2u);
  }
}

__global__ void k_batch_keys(const kamsta_wedge* __restrict__ f, uint64_t K, uint32_t b,
                             uint64_t* __restrict__ keys, uint32_t* __restrict__ w) {
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < K;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const kamsta_wedge e = f[j];
    const uint32_t lo = min(e.src, e.dst), hi = max(e.src, e.dst);
    keys[j] = (static_cast<uint64_t>(lo) << b) | hi;
    w[j] = e.w;
  }
}

// begin[g] = first sorted key whose min id is >= voff[g]
__global__ void k_batch_bounds(WaveTable t, const uint64_t* __restrict__ keys, uint64_t K,
                               uint32_t b) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g > t.G) return;
  const uint64_t x = t.voff[g] << b;
  uint64_t lo = 0, hi = K;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (keys[mid] < x) lo = mid + 1; else hi = mid;
  }
  t.begin[g] = lo;
}

__global__ void __launch_bounds__(kBatchBlock)
    k_batch_scatter(WaveTable t, const uint64_t* __restrict__ keys,
                    const uint32_t* __restrict__ w, uint64_t K, uint32_t b) {
  const uint64_t mask = (1ull << b) - 1;
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x);
       base < K; base += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t j = base + threadIdx.x;
    const bool live = j < K;
    uint32_t g = 0;
    uint64_t wt = 0;
    if (live) {
      const uint64_t key = keys[j];
      const uint64_t lo = key >> b, hi = key & mask;
      g = upper_graph(t.voff, t.G, lo);
      const uint64_t v = t.voff[g];
      uint32_t* o = t.out[g] + 3 * (j - t.begin[g]);
      o[0] = static_cast<uint32_t>(lo - v);
      o[1] = static_cast<uint32_t>(hi - v);
      o[2] = w[j];
      wt = w[j];
    }
    // one atomic per warp when the warp's live entries share a graph
    const uint32_t live_mask = __ballot_sync(kFull, live);
    const uint32_t leader = __ffs(live_mask) - 1;
    const uint32_t g0 = __shfl_sync(kFull, g, leader);
    if (__all_sync(kFull, !live || g == g0)) {
      const uint64_t s = warp_sum(wt);
      if (lane == leader) atomicAdd(reinterpret_cast<unsigned long long*>(&t.weight[g0]),
                                    static_cast<unsigned long long>(s));
    } else if (live) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&t.weight[g]),
                static_cast<unsigned long long>(wt));
    }
  }
}

inline uint32_t bits_for(uint64_t x) {  // bits to hold values < x (x >= 1)
  uint32_t b = 1;
  while (b < 64 && (1ull << b) < x) ++b;
  return b;
}

inline size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// Stream-ordered allocation from the context's pool, freed on scope exit.
struct PoolBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~PoolBuf() { reset(); }
  void reset() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
  }
  cudaError_t alloc(kamsta_ctx* ctx, size_t bytes, cudaStream_t s) {
    reset();
    st = s;
    return cudaMallocFromPoolAsync(&p, std::max<size_t>(bytes, 256), ctx->pool, s);
  }
};

#define B_TRY(x)                                         \
  do {                                                   \
    const cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) return cuda_status(e_, #x);   \
  } while (0)
#define B_KTRY(x)                                        \
  do {                                                   \
    const kamsta_status s_ = (x);                        \
    if (s_ != KAMSTA_OK) return s_;                      \
  } while (0)

}  // namespace

uint64_t batch_graph_bytes(uint64_t m_directed, uint32_t n) {
  // union copy (12 B) + first-pass lists and round lists (about 32 B per
  // directed entry at the peak) + forest sort + vertex arrays
  return 48ull * m_directed + 96ull * n + 4096;
}

std::vector<std::pair<uint32_t, uint32_t>> plan_waves(const kamsta_graph_desc* g, uint32_t count,
                                                      uint64_t budget) {
  std::vector<std::pair<uint32_t, uint32_t>> waves;
  uint32_t i = 0;
  while (i < count) {
    uint32_t j = i;
    uint64_t bytes = 0, verts = 0;
    while (j < count) {
      const uint64_t b = batch_graph_bytes(g[j].m_directed, g[j].n);
      const uint64_t v = verts + g[j].n;
      if (j > i && (bytes + b > budget || v >= kBatchMaxVertices)) break;
      bytes += b;
      verts = v;
      ++j;
    }
    waves.emplace_back(i, j);
    i = j;
  }
  return waves;
}

kamsta_status solve_wave(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t G,
                         const kamsta_cfg& cfg, bool host_buffers, cudaStream_t st,
                         BatchWaveStats* ws) {
  // ---- host side of the wave table
  std::vector<uint64_t> eoff(G + 1, 0), voff(G + 1, 0);
  for (uint32_t i = 0; i < G; ++i) {
    eoff[i + 1] = eoff[i] + g[i].m_directed;
    voff[i + 1] = voff[i] + g[i].n;
  }
  const uint64_t M = eoff[G], N = voff[G];
  if (N >= kBatchMaxVertices) {
    set_error("batch: a wave holds too many vertices");
    return KAMSTA_E_INPUT;
  }
  ws->entries = M;
  ws->vertices = N;
  // table layout in one device block
  const size_t o_edges = 0;
  const size_t o_out = o_edges + up256(sizeof(void*) * G);
  const size_t o_eoff = o_out + up256(sizeof(void*) * G);
  const size_t o_voff = o_eoff + up256(sizeof(uint64_t) * (G + 1));
  const size_t o_n = o_voff + up256(sizeof(uint64_t) * (G + 1));
  const size_t o_begin = o_n + up256(sizeof(uint32_t) * G);
  const size_t o_weight = o_begin + up256(sizeof(uint64_t) * (G + 1));
  const size_t o_err = o_weight + up256(sizeof(uint64_t) * G);
  const size_t tbytes = o_err + up256(sizeof(uint32_t) * G);
  std::vector<unsigned char> h(tbytes, 0);
  PoolBuf tbuf, ubuf, fbuf, obuf;
  B_TRY(tbuf.alloc(ctx, tbytes, st));
  B_TRY(ubuf.alloc(ctx, std::max<uint64_t>(M, 1) * sizeof(kamsta_wedge), st));
  kamsta_wedge* uni = static_cast<kamsta_wedge*>(ubuf.p);
  unsigned char* d = static_cast<unsigned char*>(tbuf.p);
  // host buffers: outputs are staged in one device buffer, graph g at the
  // offset of its vertex range (a forest of n_g vertices has < n_g edges)
  kamsta_wedge* stage = nullptr;
  if (host_buffers) {
    B_TRY(obuf.alloc(ctx, std::max<uint64_t>(N, 1) * sizeof(kamsta_wedge), st));
    stage = static_cast<kamsta_wedge*>(obuf.p);
  }
  {
    const uint32_t** he = reinterpret_cast<const uint32_t**>(h.data() + o_edges);
    uint32_t** ho = reinterpret_cast<uint32_t**>(h.data() + o_out);
    for (uint32_t i = 0; i < G; ++i) {
      if (host_buffers) {
        // the graph is copied into its union slot and shifted in place
        he[i] = reinterpret_cast<const uint32_t*>(uni + eoff[i]);
        ho[i] = reinterpret_cast<uint32_t*>(stage + voff[i]);
      } else {
        he[i] = reinterpret_cast<const uint32_t*>(g[i].edges);
        ho[i] = reinterpret_cast<uint32_t*>(g[i].out);
      }
      reinterpret_cast<uint32_t*>(h.data() + o_n)[i] = g[i].n;
    }
    std::memcpy(h.data() + o_eoff, eoff.data(), sizeof(uint64_t) * (G + 1));
    std::memcpy(h.data() + o_voff, voff.data(), sizeof(uint64_t) * (G + 1));
  }
  B_TRY(cudaMemcpyAsync(d, h.data(), tbytes, cudaMemcpyHostToDevice, st));
  WaveTable t;
  t.edges = reinterpret_cast<const uint32_t**>(d + o_edges);
  t.out = reinterpret_cast<uint32_t**>(d + o_out);
  t.eoff = reinterpret_cast<uint64_t*>(d + o_eoff);
  t.voff = reinterpret_cast<uint64_t*>(d + o_voff);
  t.n = reinterpret_cast<uint32_t*>(d + o_n);
  t.begin = reinterpret_cast<uint64_t*>(d + o_begin);
  t.weight = reinterpret_cast<uint64_t*>(d + o_weight);
  t.err = reinterpret_cast<uint32_t*>(d + o_err);
  t.G = G;
  if (host_buffers)
    for (uint32_t i = 0; i < G; ++i)
      if (g[i].m_directed)
        B_TRY(cudaMemcpyAsync(uni + eoff[i], g[i].edges, g[i].m_directed * sizeof(kamsta_wedge),
                              cudaMemcpyHostToDevice, st));
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  uint32_t launches = 0;
  if (cfg.flags & KAMSTA_FLAG_VALIDATE) {
    if (M) {
      const uint64_t blocks = std::min<uint64_t>((M + kBatchBlock - 1) / kBatchBlock, sms * 8ull);
      k_batch_order<<<static_cast<uint32_t>(blocks), kBatchBlock, 0, st>>>(t, M);
      ++launches;
    }
  }
  if (M) {
    const uint64_t words = 3 * M;
    const uint64_t chunk = static_cast<uint64_t>(kBatchBlock) * kGatherWords;
    const uint64_t blocks = std::min<uint64_t>((words + chunk - 1) / chunk, sms * 16ull);
    k_batch_gather<<<static_cast<uint32_t>(blocks), kBatchBlock, 0, st>>>(
        t, reinterpret_cast<uint32_t*>(uni), words);
    ++launches;
  }
  B_TRY(cudaGetLastError());
  // ---- one solve over the union (validation already done per graph)
  kamsta_cfg ucfg = cfg;
  ucfg.flags &= ~(KAMSTA_FLAG_VALIDATE | KAMSTA_FLAG_SORT_OUTPUT);
  B_TRY(fbuf.alloc(ctx, std::max<uint64_t>(N, 1) * sizeof(kamsta_wedge), st));
  kamsta_wedge* forest = static_cast<kamsta_wedge*>(fbuf.p);
  SolveOut so;
  kamsta_stats sst;
  B_KTRY(solve_device(ctx, algo, uni, M, static_cast<uint32_t>(N), ucfg, forest, &so, &sst, st));
  launches += sst.gpu_launches;
  ws->solve_ms = sst.device_ms;
  ubuf.reset();  // the union input is no longer needed
  // ---- split the forest per graph
  const uint64_t K = so.count;
  const uint32_t b = bits_for(std::max<uint64_t>(N, 2));
  PoolBuf kb, vb, cb, sb;
  uint64_t *keys = nullptr, *keys2 = nullptr;
  uint32_t *w = nullptr, *w2 = nullptr;
  if (K) {
    const RadixScratch rs = radix_scratch_bytes(K);
    const size_t kbytes = up256(sizeof(uint64_t) * K);
    const size_t vbytes = up256(sizeof(uint32_t) * K);
    B_TRY(kb.alloc(ctx, 2 * kbytes, st));
    B_TRY(vb.alloc(ctx, 2 * vbytes, st));
    B_TRY(cb.alloc(ctx, sizeof(uint32_t) * rs.counts + 256, st));
    B_TRY(sb.alloc(ctx, sizeof(uint64_t) * rs.status + 256, st));
    keys = static_cast<uint64_t*>(kb.p);
    keys2 = reinterpret_cast<uint64_t*>(static_cast<char*>(kb.p) + kbytes);
    w = static_cast<uint32_t*>(vb.p);
    w2 = reinterpret_cast<uint32_t*>(static_cast<char*>(vb.p) + vbytes);
    const uint32_t blocks = static_cast<uint32_t>(
        std::min<uint64_t>((K + kBatchBlock - 1) / kBatchBlock, sms * 8ull));
    k_batch_keys<<<blocks, kBatchBlock, 0, st>>>(forest, K, b, keys, w);
    ++launches;
    int alt = 0;
    uint32_t* ticket = &ctx->d_counters[kCMisc].ticket;
    B_TRY(radix_sort_pairs_u32(st, keys, keys2, w, w2, K, 2 * b, static_cast<uint32_t*>(cb.p),
                               static_cast<uint64_t*>(sb.p), ticket, ctx->d_err, &alt, sms));
    launches += 3 * ((2 * b + 7) / 8);
    if (alt) {
      std::swap(keys, keys2);
      std::swap(w, w2);
    }
  }
  B_TRY(cudaMemsetAsync(d + o_weight, 0, sizeof(uint64_t) * G, st));
  k_batch_bounds<<<(G + 1 + kBatchBlock - 1) / kBatchBlock, kBatchBlock, 0, st>>>(t, keys, K, b);
  ++launches;
  if (K) {
    const uint32_t blocks = static_cast<uint32_t>(
        std::min<uint64_t>((K + kBatchBlock - 1) / kBatchBlock, sms * 8ull));
    k_batch_scatter<<<blocks, kBatchBlock, 0, st>>>(t, keys, w, K, b);
    ++launches;
  }
  B_TRY(cudaGetLastError());
  // ---- per-graph results back to the host descriptors
  std::vector<unsigned char> back(tbytes - o_begin);
  B_TRY(cudaMemcpyAsync(back.data(), d + o_begin, back.size(), cudaMemcpyDeviceToHost, st));
  uint32_t derr = 0;
  B_TRY(cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  B_TRY(cudaStreamSynchronize(st));
  derr = *ctx->h_err;
  if (derr) {
    set_error("batch: device wait cap reached in the forest sort");
    return KAMSTA_E_NOCONVERGE;
  }
  const uint64_t* hb = reinterpret_cast<const uint64_t*>(back.data());
  const uint64_t* hw = reinterpret_cast<const uint64_t*>(back.data() + (o_weight - o_begin));
  const uint32_t* he = reinterpret_cast<const uint32_t*>(back.data() + (o_err - o_begin));
  for (uint32_t i = 0; i < G; ++i) {
    const uint64_t cnt = hb[i + 1] - hb[i];
    if (he[i]) {
      g[i].status = KAMSTA_E_INPUT;
      g[i].out_count = 0;
      g[i].total_weight = 0;
      continue;
    }
    g[i].status = KAMSTA_OK;
    g[i].out_count = cnt;
    g[i].total_weight = hw[i];
    if (host_buffers && cnt)
      B_TRY(cudaMemcpyAsync(g[i].out, stage + voff[i], cnt * sizeof(kamsta_wedge),
                            cudaMemcpyDeviceToHost, st));
  }
  if (host_buffers) B_TRY(cudaStreamSynchronize(st));
  ws->launches = launches;
  return KAMSTA_OK;
}

kamsta_status solve_batch(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t count,
                          const kamsta_cfg& cfg, uint64_t budget, bool host_buffers,
                          kamsta_batch_stats* st, cudaStream_t stream) {
  if (st) std::memset(st, 0, sizeof(*st));
  for (uint32_t i = 0; i < count; ++i) {
    g[i].status = KAMSTA_E_INPUT;
    g[i].out_count = 0;
    g[i].total_weight = 0;
    if ((g[i].m_directed && !g[i].edges) || (g[i].n > 1 && !g[i].out) ||
        g[i].n >= kBatchMaxVertices) {
      set_error("batch: graph " + std::to_string(i) + ": null pointer or n too large");
      return KAMSTA_E_INPUT;
    }
  }
  if (budget == 0) budget = kBatchDefaultBudget;
  const auto waves = plan_waves(g, count, budget);
  // own events: the solver records the context's events inside each wave
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  B_TRY(cudaEventCreate(&e0));
  B_TRY(cudaEventCreate(&e1));
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } guard{e0, e1};
  cudaEventRecord(e0, stream);
  uint32_t launches = 0;
  uint64_t entries = 0, verts = 0;
  double solve_ms = 0;
  for (const auto& w : waves) {
    BatchWaveStats ws;
    B_KTRY(solve_wave(ctx, algo, g + w.first, w.second - w.first, cfg, host_buffers, stream, &ws));
    launches += ws.launches;
    entries += ws.entries;
    verts += ws.vertices;
    solve_ms += ws.solve_ms;
  }
  cudaEventRecord(e1, stream);
  cudaEventSynchronize(e1);
  if (st) {
    st->graphs = count;
    st->waves = static_cast<uint32_t>(waves.size());
    st->gpu_launches = launches;
    st->entries = entries;
    st->vertices = verts;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    st->device_ms = ms;
    st->solve_ms = solve_ms;
    for (uint32_t i = 0; i < count; ++i) st->forest_edges += g[i].out_count;
  }
  return KAMSTA_OK;
}

}  // namespace kamsta
