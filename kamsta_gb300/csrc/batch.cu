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
//   solve_device     the single-graph solver over the union; the forest comes
//                    back as one bit per union entry (its src<dst copy)
//   k_batch_rank     rank of every set bit (word popcounts, one scan pass)
//   k_batch_bounds   first rank of every graph
//   k_batch_scatter  each forest edge, un-shifted, to its graph's output at
//                    its rank: input order, i.e. sorted by (src, dst); per-
//                    graph weight sums
// Small graphs skip the union (k_small_batch, one CTA per graph).
// The reference has no batch API: its benchmark solves one graph per MPI
// job (benchmarks/mst.cpp:215-228); the result of each graph here equals a
// kamsta_mst_boruvka call on that graph alone, sorted by (src, dst).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "sort_gen.cuh"
#include "solver.cuh"
#include "small_solve.cuh"
#include "batch.cuh"

namespace kamsta {

namespace {

constexpr int kBatchBlock = 256;
constexpr int kGatherWords = 16;  // u32 words per thread and step in k_batch_gather
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

// Union words [c0, c0 + chunk) per CTA; thread-strided inside the chunk so
// that each warp reads and writes 128 contiguous bytes per step.  Words 0
// and 1 of an entry are ids (shifted by voff), word 2 the weight.  A chunk
// inside one graph (nearly all: the union's graphs hold tens of thousands
// of words or more) issues all of a thread's kGatherWords loads before the
// first store; a chunk across graph boundaries resolves each word's graph
// on the way.  The union offset of a graph is a multiple of 3 words, so a
// word's place in its entry is q mod 3.
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
    uint64_t gbeg = 3 * t.eoff[g];
    uint64_t gend = 3 * t.eoff[g + 1];
    const uint64_t q0 = c0 + threadIdx.x;
    const uint32_t r0 = static_cast<uint32_t>(q0 % 3);  // kBatchBlock = 1 (mod 3)
    if (c0 + chunk <= gend) {  // the whole chunk in graph g (the same in every thread)
      const uint32_t* src = t.edges[g] + (q0 - gbeg);
      const uint32_t add = static_cast<uint32_t>(t.voff[g]), lim = t.n[g];
      uint32_t v[kGatherWords];
#pragma unroll
      for (int j = 0; j < kGatherWords; ++j) v[j] = __ldcs(src + j * kBatchBlock);
      uint32_t r = r0;
      bool bad = false;
#pragma unroll
      for (int j = 0; j < kGatherWords; ++j) {
        uint32_t x = v[j];
        if (r != 2) {
          bad |= x >= lim;
          x = x >= lim ? kSkipId : x + add;
        }
        uni[q0 + j * kBatchBlock] = x;
        r = r == 2 ? 0u : r + 1u;
      }
      if (bad) atomicOr(&t.err[g], 1u);
      continue;
    }
    uint32_t r = r0;
    for (int j = 0; j < kGatherWords; ++j, r = r == 2 ? 0u : r + 1u) {
      const uint64_t q = q0 + static_cast<uint64_t>(j) * kBatchBlock;
      if (q >= words) break;
      while (q >= gend) {
        ++g;
        gbeg = gend;
        gend = 3 * t.eoff[g + 1];
      }
      uint32_t v = t.edges[g][q - gbeg];
      if (r != 2) {
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

// pre[q] = set bits in words [0, q) of the forest bitmap: one pass, the word
// popcounts scanned with a decoupled look-back over tiles of kRankTile words
// taken in ticket order.  A thread reads 16 consecutive words as four
// 16-byte loads (the bitmap and every tile start are 64-byte aligned).
constexpr int kRankItems = 16;
constexpr uint32_t kRankTile = kBatchBlock * kRankItems;

__global__ void __launch_bounds__(kBatchBlock)
    k_batch_rank(const uint32_t* __restrict__ bits, uint64_t W, uint32_t* __restrict__ pre,
                 uint64_t* status, uint32_t* ticket, uint32_t ntiles, uint32_t* err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[kBatchBlock / 32];
  __shared__ uint64_t s_pre;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    const uint64_t base = static_cast<uint64_t>(tile) * kRankTile + threadIdx.x * kRankItems;
    uint32_t v[kRankItems];
    if (base + kRankItems <= W) {
      const uint4* p = reinterpret_cast<const uint4*>(bits + base);
#pragma unroll
      for (int k = 0; k < kRankItems / 4; ++k) {
        const uint4 x = p[k];
        v[4 * k] = __popc(x.x);
        v[4 * k + 1] = __popc(x.y);
        v[4 * k + 2] = __popc(x.z);
        v[4 * k + 3] = __popc(x.w);
      }
    } else {
#pragma unroll
      for (int j = 0; j < kRankItems; ++j) v[j] = base + j < W ? __popc(bits[base + j]) : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kRankItems; ++j) sum += v[j];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (lane >= static_cast<uint32_t>(o)) incl += y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t wv = lane < kBatchBlock / 32 ? s_warp[lane] : 0u;
      uint32_t wi = wv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, wi, o);
        if (lane >= static_cast<uint32_t>(o)) wi += y;
      }
      const uint32_t total = __shfl_sync(kFull, wi, kBatchBlock / 32 - 1);
      if (lane < kBatchBlock / 32) s_warp[lane] = wi - wv;
      const uint64_t tpre = lookback(status, tile, total, err);
      if (lane == 0) s_pre = tpre;
    }
    __syncthreads();
    uint32_t run = static_cast<uint32_t>(s_pre) + s_warp[warp] + (incl - sum);
    if (base + kRankItems <= W) {
      uint4* o = reinterpret_cast<uint4*>(pre + base);
#pragma unroll
      for (int k = 0; k < kRankItems / 4; ++k) {
        uint4 x;
        x.x = run;
        run += v[4 * k];
        x.y = run;
        run += v[4 * k + 1];
        x.z = run;
        run += v[4 * k + 2];
        x.w = run;
        run += v[4 * k + 3];
        o[k] = x;
      }
    } else {
#pragma unroll
      for (int j = 0; j < kRankItems; ++j) {
        if (base + j < W) pre[base + j] = run;
        run += v[j];
      }
    }
  }
}

// begin[g] = forest edges of the graphs before g: set bits before eoff[g]
__global__ void k_batch_bounds(WaveTable t, const uint32_t* __restrict__ bits,
                               const uint32_t* __restrict__ pre) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g > t.G) return;
  const uint64_t e = t.eoff[g];
  const uint32_t low = static_cast<uint32_t>(e & 31);
  t.begin[g] = pre[e >> 5] + (low ? __popc(bits[e >> 5] & ((1u << low) - 1)) : 0u);
}

// One thread per bitmap word: each set bit is a forest edge (the union entry
// at that position); it goes, un-shifted, to its graph's output at its rank
// minus the graph's first rank, so every graph's forest is in input order,
// i.e. sorted by (src, dst).  Weights are summed per graph (one atomic per
// warp when the warp's edges share a graph).  The graph of the block's first
// position is searched once per block step; a thread walks on from it (the
// union's graphs are larger than a step's 8192 positions, so a step crosses
// at most a boundary or two).
__global__ void __launch_bounds__(kBatchBlock)
    k_batch_scatter(WaveTable t, const uint32_t* __restrict__ uni,
                    const uint32_t* __restrict__ bits, const uint32_t* __restrict__ pre,
                    uint64_t W) {
  __shared__ uint32_t s_g;
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x); base < W;
       base += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    __syncthreads();
    if (threadIdx.x == 0) s_g = upper_graph(t.eoff, t.G, base * 32);
    __syncthreads();
    const uint64_t q = base + threadIdx.x;
    uint32_t f = q < W ? bits[q] : 0u;
    uint32_t g0 = 0xffffffffu;
    uint64_t w0 = 0;
    if (f) {
      uint32_t rank = pre[q];
      uint64_t pos = q * 32 + (__ffs(f) - 1);
      uint32_t g = s_g;
      while (pos >= t.eoff[g + 1]) ++g;
      g0 = g;
      while (f) {
        // up to four of the word's edges with their entry loads in flight
        constexpr int kB = 4;
        uint64_t ps[kB];
        uint32_t e0[kB], e1[kB], e2[kB];
        int c = 0;
#pragma unroll
        for (int k = 0; k < kB; ++k) {
          if (!f) break;
          ps[k] = q * 32 + (__ffs(f) - 1);
          f &= f - 1;
          c = k + 1;
        }
#pragma unroll
        for (int k = 0; k < kB; ++k) {
          if (k >= c) break;
          const uint32_t* e = uni + 3 * ps[k];
          e0[k] = e[0];
          e1[k] = e[1];
          e2[k] = e[2];
        }
#pragma unroll
        for (int k = 0; k < kB; ++k) {
          if (k >= c) break;
          while (ps[k] >= t.eoff[g + 1]) ++g;
          const uint32_t v = static_cast<uint32_t>(t.voff[g]);
          const uint32_t wt = e2[k];
          uint32_t* o = t.out[g] + 3 * (rank - t.begin[g]);
          o[0] = e0[k] - v;
          o[1] = e1[k] - v;
          o[2] = wt;
          ++rank;
          if (g == g0) {
            w0 += wt;
          } else {
            atomicAdd(reinterpret_cast<unsigned long long*>(&t.weight[g]),
                      static_cast<unsigned long long>(wt));
          }
        }
      }
    }
    // the first graph's sum: one atomic per warp when the warp agrees
    const uint32_t have = __ballot_sync(kFull, g0 != 0xffffffffu);
    if (!have) continue;
    const uint32_t leader = __ffs(have) - 1;
    const uint32_t gl = __shfl_sync(kFull, g0, leader);
    if (__all_sync(kFull, g0 == 0xffffffffu || g0 == gl)) {
      const uint64_t sum = warp_sum(w0);
      if (lane == leader) atomicAdd(reinterpret_cast<unsigned long long*>(&t.weight[gl]),
                                    static_cast<unsigned long long>(sum));
    } else if (g0 != 0xffffffffu) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&t.weight[g0]),
                static_cast<unsigned long long>(w0));
    }
  }
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
    return ctx_alloc(ctx, &p, std::max<size_t>(bytes, 256), s);
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

uint64_t serve_job_bytes(const kamsta_ctx* ctx, const kamsta_graph_desc& g) {
  kamsta_graph_desc d = g;
  d.edges = nullptr;
  if (is_small_graph(ctx, d)) return small::kScratchBytes + 4096;
  return batch_graph_bytes(g.m_directed, g.n);
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

namespace {

// ---------------------------------------------------------------------------
// Small graphs (n <= 32768, m_directed <= 262144): one persistent launch.
// Each CTA takes the next graph from a work queue (largest first) and solves
// it entirely on its own (small_solve.cuh) in its own scratch slot; the
// forest comes out sorted by (src, dst), like the union path's.

// CTA sizes the persistent kernel is built for; the context's tuning picks
// one (kamsta_batch_autotune), 512 by default.
constexpr int kSmallThreadsDefault = 512;

struct SmallTable {
  const uint32_t* const* edges;
  uint32_t* const* out;
  const uint32_t* md;
  const uint32_t* n;
  const uint32_t* order;  // graph indices, largest first
  small::Result* res;
  uint32_t G;
  uint32_t check_order;
};

template <int THREADS>
__global__ void __launch_bounds__(THREADS)
    k_small_batch(SmallTable t, unsigned char* __restrict__ scratch, uint32_t* queue) {
  __shared__ uint32_t s_q;
  unsigned char* mine = scratch + static_cast<size_t>(blockIdx.x) * small::kScratchBytes;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_q = atomicAdd(queue, 1u);
    __syncthreads();
    const uint32_t q = s_q;
    if (q >= t.G) return;
    const uint32_t g = t.order[q];
    small::solve<THREADS, small::Out::kSorted>(t.edges[g], t.md[g], t.n[g], mine, t.out[g],
                                                      &t.res[g], true, t.check_order != 0);
  }
}

uint32_t small_max_n(const kamsta_ctx* ctx) {
  return ctx->tune_small_max_n ? std::min<uint32_t>(ctx->tune_small_max_n, small::kMaxN)
                               : small::kMaxN;
}

bool is_small(const kamsta_ctx* ctx, const kamsta_graph_desc& g) {
  return g.n <= small_max_n(ctx) && g.m_directed <= small::kMaxMd;
}

template <int THREADS>
cudaError_t launch_small_kernel(const SmallTable& t, unsigned char* scratch, uint32_t* queue,
                                uint32_t grid, cudaStream_t st) {
  k_small_batch<THREADS><<<grid, THREADS, 0, st>>>(t, scratch, queue);
  return cudaGetLastError();
}

int small_per_sm(int threads) {
  int per_sm = 1;
  if (threads == 256)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_small_batch<256>, 256, 0);
  else if (threads == 1024)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_small_batch<1024>, 1024, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_small_batch<512>, 512, 0);
  return std::max(per_sm, 1);
}

// Launches the small graphs on `st` and returns; `res` (host) is valid after
// the stream synchronises.  Device buffers stay alive in `keep`.
kamsta_status launch_small(kamsta_ctx* ctx, kamsta_graph_desc* g, const std::vector<uint32_t>& idx,
                           const kamsta_cfg& cfg, cudaStream_t st, PoolBuf* tab, PoolBuf* scr,
                           small::Result** d_res, uint32_t* launches) {
  const uint32_t S = static_cast<uint32_t>(idx.size());
  std::vector<uint32_t> order(S);
  for (uint32_t i = 0; i < S; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    return g[idx[a]].m_directed + g[idx[a]].n > g[idx[b]].m_directed + g[idx[b]].n;
  });
  const size_t o_edges = 0;
  const size_t o_out = o_edges + up256(sizeof(void*) * S);
  const size_t o_md = o_out + up256(sizeof(void*) * S);
  const size_t o_n = o_md + up256(sizeof(uint32_t) * S);
  const size_t o_order = o_n + up256(sizeof(uint32_t) * S);
  const size_t o_res = o_order + up256(sizeof(uint32_t) * S);
  const size_t o_queue = o_res + up256(sizeof(small::Result) * S);
  const size_t bytes = o_queue + 256;
  std::vector<unsigned char> h(bytes, 0);
  for (uint32_t i = 0; i < S; ++i) {
    const kamsta_graph_desc& d = g[idx[i]];
    reinterpret_cast<const void**>(h.data() + o_edges)[i] = d.edges;
    reinterpret_cast<void**>(h.data() + o_out)[i] = d.out;
    reinterpret_cast<uint32_t*>(h.data() + o_md)[i] = static_cast<uint32_t>(d.m_directed);
    reinterpret_cast<uint32_t*>(h.data() + o_n)[i] = d.n;
  }
  std::memcpy(h.data() + o_order, order.data(), sizeof(uint32_t) * S);
  B_TRY(tab->alloc(ctx, bytes, st));
  unsigned char* d = static_cast<unsigned char*>(tab->p);
  B_TRY(cudaMemcpyAsync(d, h.data(), bytes, cudaMemcpyHostToDevice, st));
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = ctx->tune_small_threads ? static_cast<int>(ctx->tune_small_threads)
                                              : kSmallThreadsDefault;
  uint32_t grid = std::max<uint32_t>(
      1, std::min<uint32_t>(S, static_cast<uint32_t>(small_per_sm(threads) * sms)));
  if (ctx->mem_limit) {
    // under a memory limit, only as many scratch slots as the limit leaves
    // room for; the work queue spreads the graphs over however many CTAs run
    const uint64_t used = ctx_device_bytes(ctx);
    const uint64_t room = ctx->mem_limit > used ? ctx->mem_limit - used : 0;
    const uint64_t slots = room / (small::kScratchBytes + 4096);
    grid = std::max<uint32_t>(1, static_cast<uint32_t>(std::min<uint64_t>(grid, slots)));
  }
  B_TRY(scr->alloc(ctx, static_cast<size_t>(grid) * small::kScratchBytes, st));
  SmallTable t;
  t.edges = reinterpret_cast<const uint32_t* const*>(d + o_edges);
  t.out = reinterpret_cast<uint32_t* const*>(d + o_out);
  t.md = reinterpret_cast<const uint32_t*>(d + o_md);
  t.n = reinterpret_cast<const uint32_t*>(d + o_n);
  t.order = reinterpret_cast<const uint32_t*>(d + o_order);
  t.res = reinterpret_cast<small::Result*>(d + o_res);
  t.G = S;
  t.check_order = (cfg.flags & KAMSTA_FLAG_VALIDATE) ? 1u : 0u;
  unsigned char* scratch = static_cast<unsigned char*>(scr->p);
  uint32_t* queue = reinterpret_cast<uint32_t*>(d + o_queue);
  if (threads == 256) B_TRY(launch_small_kernel<256>(t, scratch, queue, grid, st));
  else if (threads == 1024) B_TRY(launch_small_kernel<1024>(t, scratch, queue, grid, st));
  else B_TRY(launch_small_kernel<512>(t, scratch, queue, grid, st));
  *d_res = t.res;
  ++*launches;
  return KAMSTA_OK;
}

// The union path for the graphs g[0..G).
kamsta_status solve_union(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t G,
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
  PoolBuf tbuf, ubuf, obuf;
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
  // the forest comes back as one bit per union entry (its src<dst copy)
  const uint64_t W = (M + 31) / 32;
  PoolBuf bb, preb, stb;
  B_TRY(bb.alloc(ctx, sizeof(uint32_t) * (W + 1), st));
  uint32_t* bits = static_cast<uint32_t*>(bb.p);
  B_TRY(cudaMemsetAsync(bits, 0, sizeof(uint32_t) * (W + 1), st));
  SolveOut so;
  kamsta_stats sst;
  B_KTRY(solve_device(ctx, algo, uni, M, static_cast<uint32_t>(N), ucfg, nullptr, &so, &sst, st,
                      bits));
  launches += sst.gpu_launches;
  ws->solve_ms = sst.device_ms;
  // ---- split: ranks of the set bits (word popcounts + exclusive scan), the
  // first rank of every graph, then every forest edge to its graph's output
  const uint32_t ntiles = static_cast<uint32_t>((W + 1 + kRankTile - 1) / kRankTile);
  B_TRY(preb.alloc(ctx, sizeof(uint32_t) * (W + 1), st));
  B_TRY(stb.alloc(ctx, sizeof(uint64_t) * (ntiles + 1), st));
  uint32_t* pre = static_cast<uint32_t*>(preb.p);
  {
    B_TRY(cudaMemsetAsync(stb.p, 0, sizeof(uint64_t) * ntiles, st));
    B_TRY(cudaMemsetAsync(&ctx->d_counters[kCMisc].ticket, 0, sizeof(uint32_t), st));
    k_batch_rank<<<std::min<uint32_t>(ntiles, sms * 4u), kBatchBlock, 0, st>>>(
        bits, W + 1, pre, static_cast<uint64_t*>(stb.p), &ctx->d_counters[kCMisc].ticket,
        ntiles, ctx->d_err);
    ++launches;
  }
  B_TRY(cudaMemsetAsync(d + o_weight, 0, sizeof(uint64_t) * G, st));
  k_batch_bounds<<<(G + 1 + kBatchBlock - 1) / kBatchBlock, kBatchBlock, 0, st>>>(t, bits, pre);
  ++launches;
  if (so.count) {
    const uint32_t blocks = static_cast<uint32_t>(
        std::min<uint64_t>((W + kBatchBlock - 1) / kBatchBlock, sms * 16ull));
    k_batch_scatter<<<blocks, kBatchBlock, 0, st>>>(t, reinterpret_cast<const uint32_t*>(uni),
                                                    bits, pre, W);
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
    set_error("batch: device wait cap reached in the forest split");
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

}  // namespace

bool is_small_graph(const kamsta_ctx* ctx, const kamsta_graph_desc& g) { return is_small(ctx, g); }

kamsta_status solve_wave(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t G,
                         const kamsta_cfg& cfg, bool host_buffers, cudaStream_t st,
                         BatchWaveStats* ws) {
  std::vector<uint32_t> sm, lg;
  for (uint32_t i = 0; i < G; ++i)
    ((!host_buffers && is_small(ctx, g[i])) ? sm : lg).push_back(i);
  if (sm.empty()) return solve_union(ctx, algo, g, G, cfg, host_buffers, st, ws);
  // small graphs on the auxiliary stream, overlapping the union solve (the
  // forest is the same for boruvka and filter_boruvka)
  B_TRY(cudaEventRecord(ctx->ev_fork, st));
  B_TRY(cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0));
  PoolBuf tab, scr;
  small::Result* d_res = nullptr;
  uint32_t launches = 0;
  B_KTRY(launch_small(ctx, g, sm, cfg, ctx->aux, &tab, &scr, &d_res, &launches));
  std::vector<small::Result> h_res(sm.size());
  B_TRY(cudaMemcpyAsync(h_res.data(), d_res, sizeof(small::Result) * sm.size(),
                        cudaMemcpyDeviceToHost, ctx->aux));
  BatchWaveStats us;
  kamsta_status s = KAMSTA_OK;
  if (!lg.empty()) {
    std::vector<kamsta_graph_desc> sub(lg.size());
    for (size_t k = 0; k < lg.size(); ++k) sub[k] = g[lg[k]];
    s = solve_union(ctx, algo, sub.data(), static_cast<uint32_t>(lg.size()), cfg, host_buffers,
                    st, &us);
    for (size_t k = 0; k < lg.size(); ++k) g[lg[k]] = sub[k];
  }
  B_TRY(cudaEventRecord(ctx->ev_join, ctx->aux));
  B_TRY(cudaStreamWaitEvent(st, ctx->ev_join, 0));
  B_TRY(cudaStreamSynchronize(ctx->aux));
  if (s != KAMSTA_OK) return s;
  uint64_t entries = 0, verts = 0;
  for (size_t k = 0; k < sm.size(); ++k) {
    kamsta_graph_desc& d = g[sm[k]];
    const small::Result& r = h_res[k];
    entries += d.m_directed;
    verts += d.n;
    if (r.err) {
      d.status = (r.err & ~(kErrRange | kErrOrder)) ? KAMSTA_E_NOCONVERGE : KAMSTA_E_INPUT;
      d.out_count = 0;
      d.total_weight = 0;
    } else {
      d.status = KAMSTA_OK;
      d.out_count = r.count;
      d.total_weight = r.weight;
    }
  }
  ws->entries = us.entries + entries;
  ws->vertices = us.vertices + verts;
  ws->launches = us.launches + launches;
  ws->solve_ms = us.solve_ms;
  return KAMSTA_OK;
}

// Autotuner of the batch path: times the persistent small-graph kernel at
// each CTA size on the sample's small graphs, then the small/union cutoff on
// the whole sample, and keeps the fastest in the context.
kamsta_status batch_autotune(kamsta_ctx* ctx, Algo algo, kamsta_graph_desc* g, uint32_t count,
                             const kamsta_cfg& cfg, cudaStream_t st, kamsta_tuning* out) {
  static const uint32_t kThreads[3] = {256, 512, 1024};
  static const uint32_t kCut[4] = {4096, 8192, 16384, 32768};
  std::memset(out, 0, sizeof(*out));
  auto timed = [&](kamsta_graph_desc* gg, uint32_t cnt, double* ms) -> kamsta_status {
    double best = 1e300;
    for (int rep = 0; rep < 3; ++rep) {  // the first run warms the pool
      const auto t0 = std::chrono::steady_clock::now();
      kamsta_status s = solve_batch(ctx, algo, gg, cnt, cfg, 0, false, nullptr, st);
      if (s != KAMSTA_OK) return s;
      const double t = std::chrono::duration<double, std::milli>(
                           std::chrono::steady_clock::now() - t0).count();
      if (rep > 0) best = std::min(best, t);
    }
    *ms = best;
    return KAMSTA_OK;
  };
  std::vector<kamsta_graph_desc> smalls;
  for (uint32_t i = 0; i < count; ++i)
    if (g[i].n <= small::kMaxN && g[i].m_directed <= small::kMaxMd) smalls.push_back(g[i]);
  ctx->tune_small_max_n = small::kMaxN;
  uint32_t best_t = kSmallThreadsDefault;
  double best_ms = 1e300;
  if (!smalls.empty()) {
    for (int i = 0; i < 3; ++i) {
      ctx->tune_small_threads = kThreads[i];
      B_KTRY(timed(smalls.data(), static_cast<uint32_t>(smalls.size()), &out->threads_ms[i]));
      if (out->threads_ms[i] < best_ms) {
        best_ms = out->threads_ms[i];
        best_t = kThreads[i];
      }
    }
  }
  ctx->tune_small_threads = best_t;
  uint32_t best_c = small::kMaxN;
  best_ms = 1e300;
  for (int i = 0; i < 4; ++i) {
    ctx->tune_small_max_n = kCut[i];
    B_KTRY(timed(g, count, &out->cutoff_ms[i]));
    if (out->cutoff_ms[i] < best_ms) {
      best_ms = out->cutoff_ms[i];
      best_c = kCut[i];
    }
  }
  ctx->tune_small_max_n = best_c;
  out->small_threads = best_t;
  out->small_max_n = best_c;
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
