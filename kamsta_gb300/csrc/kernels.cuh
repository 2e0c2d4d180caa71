// kernels.cuh -- device kernels of the Boruvka / filter-Boruvka hot path.
//
// Reference steps (KaMSTa tree) and the kernel that replaces each:
//   compute_min_edges             mst_utils_common.hpp:84-105     -> fused into k_edge_pass
//   determine_mst_edges(_exhausted) mst_utils_cut_edges.hpp:102-166 -> k_hook
//   update_parents                gbbs_reimplementation.hpp:161-169 -> k_jump
//   add_new_mst_edges_to_mst_array gbbs_reimplementation.hpp:137-159 -> k_vertex_scan
//   compactify_vertices           mst_utils_common.hpp:122-132    -> k_vertex_scan
//   relabel_edges + filter_out_self_loops  mst_utils_plain.hpp:7-29,
//                                 mst_utils_common.hpp:157-175    -> k_edge_pass
//   localMST::partition / filter  mst_utils_filter.hpp:39-126     -> k_edge_pass
//   final parent shortcut         local_mst_respecting_cut_edges.hpp:199-203
//                                                                  -> k_chase + k_relabel_all
#pragma once
#include "common.cuh"

namespace kamsta {

constexpr int kBlock = 256;
constexpr int kItemsDir = 12;   // directed 12-byte records per thread
constexpr int kItemsRec = 8;    // 16-byte records per thread
constexpr int kItemsVtx = 8;    // vertices per thread in the vertex scans
constexpr int kMaxOut = 3;      // weight classes materialised by one pass

// Parameters of one edge pass.  Items are kept when their weight lies in
// [wmin, wmax], their relabelled endpoints differ, and (for the directed
// input) src < dst.  The class of a kept item is the first c with w <= thr[c]
// (c < nout-1), else nout-1.  Class 0 optionally feeds the next round's
// minimum (minval) with the value (w << 32 | output position).
struct EdgePassArgs {
  const uint32_t* map;  // label map; nullptr = identity
  uint32_t wmin, wmax;  // keep wmin <= w <= wmax
  uint32_t thr[kMaxOut];
  Rec* out[kMaxOut];
  uint64_t cap[kMaxOut];  // capacity of out[c]; overflow sets kErrOverflow
  uint64_t* status[kMaxOut];
  uint64_t* minval;      // nullptr = no fused minimum
  unsigned long long* counts;  // [kMaxOut] kept per class, [kMaxOut] dropped by weight
  uint32_t* ticket;
  uint32_t* err;
  uint32_t n;            // ids must be < n (directed source)
  uint32_t validate;     // check id range and (src,dst) order
  uint32_t aligned16;    // directed source base is 16-byte aligned
  uint32_t ntiles;
};

template <int NOUT>
__device__ __forceinline__ uint8_t weight_class(uint32_t w, const EdgePassArgs& p) {
  uint8_t c = NOUT - 1;
#pragma unroll
  for (int k = NOUT - 2; k >= 0; --k)
    if (w <= p.thr[k]) c = static_cast<uint8_t>(k);
  return c;
}

// Publish per-class look-back and counts, then scatter.  Shared by both
// sources.  a/b/w/oid/cls hold the tile's items.
template <int NOUT, int ITEMS>
__device__ __forceinline__ void edge_pass_finish(
    uint32_t tile, const uint32_t (&a)[ITEMS], const uint32_t (&b)[ITEMS],
    const uint32_t (&w)[ITEMS], const uint32_t (&oid)[ITEMS],
    const uint8_t (&cls)[ITEMS], uint32_t dropped_w, const EdgePassArgs& p) {
  __shared__ uint32_t s_rank[NOUT * ITEMS * (kBlock / 32)];
  __shared__ uint32_t s_tot[NOUT];
  __shared__ uint64_t s_pre[NOUT];
  uint32_t offs[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) offs[j] = 0;
  tile_rank<NOUT, ITEMS, kBlock>(cls, offs, s_rank, s_tot);
  const uint32_t warp = threadIdx.x >> 5;
  if (warp < NOUT) {
    const uint64_t pre = lookback(p.status[warp], tile, s_tot[warp], p.err);
    if (lane_id() == 0) {
      s_pre[warp] = pre;
      if (s_tot[warp]) atomicAdd(&p.counts[warp], static_cast<unsigned long long>(s_tot[warp]));
    }
  }
  // weight-dropped count (for the unmaterialised class)
  const uint32_t dsum = warp_sum(dropped_w);
  if (lane_id() == 0 && dsum) atomicAdd(&p.counts[kMaxOut], static_cast<unsigned long long>(dsum));
  __syncthreads();
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    if (cls[j] == 0xff) continue;
    const uint64_t pos = s_pre[cls[j]] + offs[j];
    if (pos >= p.cap[cls[j]]) {
      atomicOr(p.err, kErrOverflow);
      continue;
    }
    Rec r;
    r.a = a[j];
    r.b = b[j];
    r.w = w[j];
    r.oid = oid[j];
    p.out[cls[j]][pos] = r;
    if (cls[j] == 0 && p.minval != nullptr) {
      const uint64_t v = (static_cast<uint64_t>(w[j]) << 32) | pos;
      min_update(&p.minval[a[j]], v);
      min_update(&p.minval[b[j]], v);
    }
  }
}

__device__ __forceinline__ uint32_t next_tile(uint32_t* ticket) {
  __shared__ uint32_t s_tile;
  __syncthreads();  // previous tile fully done with shared memory
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  return s_tile;
}

// Edge pass over the caller's directed input (12-byte records, (src,dst)
// sorted, both directions).  Only src < dst copies are candidates; the
// record's oid is its index in the input.  The tile is staged through shared
// memory with 16-byte loads (coalesced), then read back per item.
template <int NOUT>
__global__ void __launch_bounds__(kBlock)
    k_edge_pass_dir(const uint32_t* __restrict__ in, uint64_t m, EdgePassArgs p) {
  constexpr int TILE = kItemsDir * kBlock;
  __shared__ __align__(16) uint32_t s_words[TILE * 3];
  for (;;) {
    const uint32_t tile = next_tile(p.ticket);
    if (tile >= p.ntiles) return;
    const uint64_t base = static_cast<uint64_t>(tile) * TILE;
    const uint32_t cnt = static_cast<uint32_t>(m - base < TILE ? m - base : TILE);
    const uint32_t words = cnt * 3;
    const uint32_t* src = in + base * 3;
    if (p.aligned16) {
      const uint32_t nvec = words >> 2;
      const uint4* src4 = reinterpret_cast<const uint4*>(src);
      uint4* dst4 = reinterpret_cast<uint4*>(s_words);
      for (uint32_t i = threadIdx.x; i < nvec; i += kBlock) dst4[i] = __ldcs(src4 + i);
      for (uint32_t i = (nvec << 2) + threadIdx.x; i < words; i += kBlock) s_words[i] = src[i];
    } else {
      for (uint32_t i = threadIdx.x; i < words; i += kBlock) s_words[i] = src[i];
    }
    __syncthreads();
    uint32_t a[kItemsDir], b[kItemsDir], w[kItemsDir], oid[kItemsDir];
    uint8_t cls[kItemsDir];
    uint32_t dropped_w = 0;
#pragma unroll
    for (int j = 0; j < kItemsDir; ++j) {
      const uint32_t t = j * kBlock + threadIdx.x;
      cls[j] = 0xff;
      a[j] = b[j] = w[j] = 0;
      oid[j] = static_cast<uint32_t>(base + t);
      if (t >= cnt) continue;
      const uint32_t s = s_words[3 * t], d = s_words[3 * t + 1], wt = s_words[3 * t + 2];
      if (p.validate) {
        if (s >= p.n || d >= p.n) atomicOr(p.err, kErrRange);
        uint32_t ps, pd;
        bool have_prev = true;
        if (t > 0) {
          ps = s_words[3 * (t - 1)];
          pd = s_words[3 * (t - 1) + 1];
        } else if (base > 0) {
          ps = in[(base - 1) * 3];
          pd = in[(base - 1) * 3 + 1];
        } else {
          have_prev = false;
          ps = pd = 0;
        }
        if (have_prev && (s < ps || (s == ps && d <= pd))) atomicOr(p.err, kErrOrder);
      }
      if (!(s < d) || d >= p.n) continue;
      if (wt < p.wmin || wt > p.wmax) {
        dropped_w += (wt > p.wmax) ? 1u : 0u;
        continue;
      }
      const uint32_t la = p.map ? p.map[s] : s;
      const uint32_t lb = p.map ? p.map[d] : d;
      if (la == lb) continue;
      a[j] = la;
      b[j] = lb;
      w[j] = wt;
      cls[j] = weight_class<NOUT>(wt, p);
    }
    edge_pass_finish<NOUT, kItemsDir>(tile, a, b, w, oid, cls, dropped_w, p);
  }
}

// Edge pass over a Rec list (kept in canonical order).
template <int NOUT>
__global__ void __launch_bounds__(kBlock)
    k_edge_pass_rec(const Rec* __restrict__ in, uint64_t m, EdgePassArgs p) {
  constexpr int TILE = kItemsRec * kBlock;
  for (;;) {
    const uint32_t tile = next_tile(p.ticket);
    if (tile >= p.ntiles) return;
    const uint64_t base = static_cast<uint64_t>(tile) * TILE;
    uint32_t a[kItemsRec], b[kItemsRec], w[kItemsRec], oid[kItemsRec];
    uint8_t cls[kItemsRec];
    uint32_t dropped_w = 0;
    Rec r[kItemsRec];
#pragma unroll
    for (int j = 0; j < kItemsRec; ++j) {
      const uint64_t i = base + j * kBlock + threadIdx.x;
      if (i < m) r[j] = in[i];
    }
#pragma unroll
    for (int j = 0; j < kItemsRec; ++j) {
      const uint64_t i = base + j * kBlock + threadIdx.x;
      cls[j] = 0xff;
      a[j] = b[j] = w[j] = oid[j] = 0;
      if (i >= m) continue;
      const uint32_t wt = r[j].w;
      if (wt < p.wmin || wt > p.wmax) {
        dropped_w += (wt > p.wmax) ? 1u : 0u;
        continue;
      }
      const uint32_t la = p.map ? p.map[r[j].a] : r[j].a;
      const uint32_t lb = p.map ? p.map[r[j].b] : r[j].b;
      if (la == lb) continue;
      a[j] = la;
      b[j] = lb;
      w[j] = wt;
      oid[j] = r[j].oid;
      cls[j] = weight_class<NOUT>(wt, p);
    }
    edge_pass_finish<NOUT, kItemsRec>(tile, a, b, w, oid, cls, dropped_w, p);
  }
}

// ---------------------------------------------------------------------------
// Hook (determine_mst_edges, mst_utils_cut_edges.hpp:102-166, without cut
// edges): every live vertex hooks onto the other endpoint of its minimum
// edge; of a mutual pair the lower label stays root.  Vertices without an
// incident edge are finished ("exhausted") and stay their own root.
__global__ void k_hook(uint32_t n, const uint64_t* __restrict__ minval,
                       const Rec* __restrict__ list, uint32_t* __restrict__ parent,
                       uint32_t* __restrict__ msfoid, uint32_t* err) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += gridDim.x * blockDim.x) {
    const uint64_t val = minval[v];
    if (val == kInf64) {
      parent[v] = v;
      msfoid[v] = kNone;
      continue;
    }
    const Rec r = list[static_cast<uint32_t>(val)];
    if (r.a != v && r.b != v) {
      atomicOr(err, kErrHook);
      parent[v] = v;
      msfoid[v] = kNone;
      continue;
    }
    const uint32_t u = r.a ^ r.b ^ v;
    if (minval[u] == val && v < u) {
      parent[v] = v;
      msfoid[v] = kNone;
    } else {
      parent[v] = u;
      msfoid[v] = r.oid;
    }
  }
}

// Pointer jumping to the roots (update_parents, gbbs_reimplementation.hpp:
// 161-169) with path halving; every write stores an ancestor, so concurrent
// updates stay correct.  Capped; the cap reports kErrJump.
__global__ void k_jump(uint32_t n, uint32_t* parent, uint32_t* err) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += gridDim.x * blockDim.x) {
    uint32_t x = v;
    uint32_t p = ld_relaxed(parent + x);
    if (p == x) continue;
    uint32_t steps = 0;
    for (;;) {
      const uint32_t gp = ld_relaxed(parent + p);
      if (gp == p) break;
      st_relaxed(parent + x, gp);
      x = gp;
      p = ld_relaxed(parent + x);
      ++steps;
      // a cycle (never produced by a correct hook) must not keep the device
      // busy: one thread reaching the cap stops all others within 1024 steps
      if ((steps & 1023u) == 0 && (steps > kJumpCap || (ld_relaxed(err) & kErrJump))) {
        atomicOr(err, kErrJump);
        break;
      }
    }
    st_relaxed(parent + v, p);
  }
}

// Renumbering and forest-edge emission (compactify_vertices +
// add_new_mst_edges_to_mst_array).  Class 0: live roots -> dense new ids,
// carry their original representative and reset the next minimum.  Class 1:
// hooked vertices -> append the edge id of their minimum edge to the forest.
struct VertexScanArgs {
  uint32_t n;
  const uint32_t* parent;
  const uint64_t* minval;
  const uint32_t* msfoid;
  const uint32_t* orig_cur;
  uint32_t* orig_next;
  uint32_t* newid;
  uint64_t* minval_next;
  uint32_t* msf_out;  // already offset by the forest edges found so far
  uint64_t msf_cap;   // entries available at msf_out
  uint64_t orig_cap;  // entries available at orig_next / minval_next
  uint64_t* status[2];
  unsigned long long* counts;  // [0] roots, [1] forest edges
  uint32_t* ticket;
  uint32_t* err;
  uint32_t ntiles;
};

__global__ void __launch_bounds__(kBlock) k_vertex_scan(VertexScanArgs p) {
  constexpr int TILE = kItemsVtx * kBlock;
  __shared__ uint32_t s_rank[2 * kItemsVtx * (kBlock / 32)];
  __shared__ uint32_t s_tot[2];
  __shared__ uint64_t s_pre[2];
  for (;;) {
    const uint32_t tile = next_tile(p.ticket);
    if (tile >= p.ntiles) return;
    const uint64_t base = static_cast<uint64_t>(tile) * TILE;
    uint8_t cls[kItemsVtx];
    uint32_t offs[kItemsVtx];
#pragma unroll
    for (int j = 0; j < kItemsVtx; ++j) {
      const uint64_t v = base + j * kBlock + threadIdx.x;
      cls[j] = 0xff;
      offs[j] = 0;
      if (v >= p.n) continue;
      const uint32_t par = p.parent[v];
      if (par != v)
        cls[j] = 1;
      else if (p.minval[v] != kInf64)
        cls[j] = 0;
    }
    tile_rank<2, kItemsVtx, kBlock>(cls, offs, s_rank, s_tot);
    const uint32_t warp = threadIdx.x >> 5;
    if (warp < 2) {
      const uint64_t pre = lookback(p.status[warp], tile, s_tot[warp], p.err);
      if (lane_id() == 0) {
        s_pre[warp] = pre;
        if (s_tot[warp]) atomicAdd(&p.counts[warp], static_cast<unsigned long long>(s_tot[warp]));
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kItemsVtx; ++j) {
      const uint64_t v = base + j * kBlock + threadIdx.x;
      if (cls[j] == 0) {
        const uint64_t id = s_pre[0] + offs[j];
        if (id >= p.orig_cap) {
          atomicOr(p.err, kErrOverflow);
          continue;
        }
        p.newid[v] = static_cast<uint32_t>(id);
        p.orig_next[id] = p.orig_cur[v];
        p.minval_next[id] = kInf64;
      } else if (cls[j] == 1) {
        const uint64_t k = s_pre[1] + offs[j];
        if (k >= p.msf_cap) {
          atomicOr(p.err, kErrOverflow);
          continue;
        }
        p.msf_out[k] = p.msfoid[v];
      }
    }
  }
}

// Label map of one round: dense id in round r -> dense id in round r+1, or
// kNone for a finished vertex.
__global__ void k_map(uint32_t n, const uint64_t* __restrict__ minval,
                      const uint32_t* __restrict__ parent,
                      const uint32_t* __restrict__ newid, uint32_t* __restrict__ R) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += gridDim.x * blockDim.x) {
    R[v] = (minval[v] == kInf64 && parent[v] == v) ? kNone : newid[parent[v]];
  }
}

// Final labels of one Boruvka call: follow the round maps of every round-0
// vertex to its finished component and write that component's original
// representative into P.
constexpr int kMaxRounds = 40;
struct ChaseArgs {
  uint32_t n0;
  uint32_t rounds;
  const uint32_t* R[kMaxRounds];
  const uint32_t* orig[kMaxRounds + 1];
  uint32_t* P;
  uint32_t* err;
};

__global__ void k_chase(ChaseArgs p) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n0;
       i += gridDim.x * blockDim.x) {
    uint32_t x = i;
    uint32_t rep = kNone;
    for (uint32_t r = 0; r < p.rounds; ++r) {
      const uint32_t y = p.R[r][x];
      if (y == kNone) {
        rep = p.orig[r][x];
        break;
      }
      x = y;
    }
    if (rep == kNone) rep = p.orig[p.rounds][x];
    p.P[p.orig[0][i]] = rep;
  }
}

// New representative list of the call (V' = {v in V : P[v] == v}, stable)
// and the dense numbering of those representatives.
struct RepScanArgs {
  uint32_t n;
  const uint32_t* V;
  const uint32_t* P;
  uint32_t* Vout;
  uint32_t* dense_of;
  uint64_t* status;
  unsigned long long* counts;
  uint32_t* ticket;
  uint32_t* err;
  uint32_t ntiles;
};

__global__ void __launch_bounds__(kBlock) k_rep_scan(RepScanArgs p) {
  constexpr int TILE = kItemsVtx * kBlock;
  __shared__ uint32_t s_rank[kItemsVtx * (kBlock / 32)];
  __shared__ uint32_t s_tot[1];
  __shared__ uint64_t s_pre;
  for (;;) {
    const uint32_t tile = next_tile(p.ticket);
    if (tile >= p.ntiles) return;
    const uint64_t base = static_cast<uint64_t>(tile) * TILE;
    uint8_t cls[kItemsVtx];
    uint32_t offs[kItemsVtx], val[kItemsVtx];
#pragma unroll
    for (int j = 0; j < kItemsVtx; ++j) {
      const uint64_t i = base + j * kBlock + threadIdx.x;
      cls[j] = 0xff;
      offs[j] = 0;
      val[j] = 0;
      if (i >= p.n) continue;
      val[j] = p.V[i];
      if (p.P[val[j]] == val[j]) cls[j] = 0;
    }
    tile_rank<1, kItemsVtx, kBlock>(cls, offs, s_rank, s_tot);
    if ((threadIdx.x >> 5) == 0) {
      const uint64_t pre = lookback(p.status, tile, s_tot[0], p.err);
      if (lane_id() == 0) {
        s_pre = pre;
        if (s_tot[0]) atomicAdd(&p.counts[0], static_cast<unsigned long long>(s_tot[0]));
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kItemsVtx; ++j) {
      if (cls[j] != 0) continue;
      const uint32_t k = static_cast<uint32_t>(s_pre + offs[j]);
      p.Vout[k] = val[j];
      p.dense_of[val[j]] = k;
    }
  }
}

// Shortcut every original vertex to its new representative and compute its
// dense label for the next call: P[x] = P[P[x]], D[x] = dense_of[P[x]].
__global__ void k_relabel_all(uint32_t n, uint32_t* __restrict__ P,
                              const uint32_t* __restrict__ dense_of,
                              uint32_t* __restrict__ D) {
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += gridDim.x * blockDim.x) {
    const uint32_t p = P[P[x]];
    P[x] = p;
    D[x] = dense_of[p];
  }
}

__global__ void k_iota(uint32_t n, uint32_t* __restrict__ a) {
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += gridDim.x * blockDim.x)
    a[x] = x;
}

__global__ void k_fill64(uint64_t n, uint64_t* __restrict__ a, uint64_t v) {
  for (uint64_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    a[x] = v;
}

// Forest output: gather the src<dst input copy of every forest edge and sum
// the weights.
__global__ void k_emit(uint64_t k, const uint32_t* __restrict__ msf,
                       const uint32_t* __restrict__ in_words,
                       uint32_t* __restrict__ out_words,
                       unsigned long long* weight) {
  uint64_t local = 0;
  for (uint64_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t o = static_cast<uint64_t>(msf[i]) * 3;
    const uint32_t s = in_words[o], d = in_words[o + 1], w = in_words[o + 2];
    out_words[3 * i] = s;
    out_words[3 * i + 1] = d;
    out_words[3 * i + 2] = w;
    local += w;
  }
  local = warp_sum(local);
  if (lane_id() == 0 && local) atomicAdd(weight, static_cast<unsigned long long>(local));
}

// Weight samples for pivot selection: sample i reads the weight of the input
// entry at hi64(mix64(seed + i) * m).  Both copies of an undirected edge
// carry its weight, so sampling the directed list samples edge weights.
__global__ void k_sample_weights(const uint32_t* __restrict__ in_words, uint64_t m,
                                 uint64_t seed, uint32_t count, uint32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += gridDim.x * blockDim.x) {
    const uint64_t pos = __umul64hi(mix64(seed + i), m);
    out[i] = in_words[pos * 3 + 2];
  }
}

__global__ void k_sample_weights_rec(const Rec* __restrict__ in, uint64_t m,
                                     uint64_t seed, uint32_t count, uint32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += gridDim.x * blockDim.x) {
    const uint64_t pos = __umul64hi(mix64(seed + i), m);
    out[i] = in[pos].w;
  }
}

}  // namespace kamsta
