// kernels.cuh -- device kernels of the Boruvka / filter-Boruvka hot path.
//
// Reference steps (KaMSTa tree) and the kernel that replaces each:
//   compute_min_edges             mst_utils_common.hpp:84-105     -> fused into k_pass_*
//   determine_mst_edges(_exhausted) mst_utils_cut_edges.hpp:102-166 -> k_hook
//   update_parents                gbbs_reimplementation.hpp:161-169 -> k_jump_label
//                                    (k_jump + k_map beyond 2^31 vertices)
//   add_new_mst_edges_to_mst_array gbbs_reimplementation.hpp:137-159 -> k_hook (counts) + k_vertex_write
//   compactify_vertices           mst_utils_common.hpp:122-132    -> k_hook (counts) + k_vertex_write
//   relabel_edges + filter_out_self_loops  mst_utils_plain.hpp:7-29,
//                                 mst_utils_common.hpp:157-175    -> k_pass_seg
//   localMST::partition / filter  mst_utils_filter.hpp:39-126     -> k_pass_dir / k_pass_seg
//   final parent shortcut         local_mst_respecting_cut_edges.hpp:199-203
//                                                                  -> k_compose(_last) + k_rep_write + k_relabel_all
#pragma once
#include "common.cuh"

namespace kamsta {

constexpr int kBlock = 256;
constexpr int kItemsDir = 6;    // directed 12-byte records per thread (default tile)
constexpr int kItemsRec = 2;    // 16-byte records per thread (default tile)
constexpr int kMaxOut = 3;      // weight classes materialised by one pass

// ---------------------------------------------------------------------------
// Segmented edge lists.
//
// An edge pass splits its (logical) input into one contiguous chunk per CTA
// and every CTA appends the records it keeps to its own output segment,
// `segment * cap + running offset`.  No CTA waits on another (there is no
// cross-CTA scan), so a pass is a plain stream: the next input tile of a
// CTA is known in advance and is prefetched by a bulk asynchronous copy
// (TMA, cp.async.bulk) while the current one is processed.  Segments are
// laid out in chunk order, so the physical index of a record -- its
// "position" -- grows with the input's (min, max) order; (w << 32 | position)
// therefore keeps ordering edges exactly like the reference's (weight,
// local edge index) key (mst_utils_common.hpp:76-81), gaps and all, and the
// hook finds a record directly at its position.
constexpr int kMaxSeg = 1024;  // segments per list (= CTAs of the producing pass)

struct SegIn {  // a list produced by an edge pass
  const Rec* base;
  const uint32_t* count;  // records per segment
  uint64_t cap;           // physical records per segment
  uint32_t nseg;
};
struct SegOut {
  Rec* base;
  uint64_t cap;     // records per segment (overflow sets kErrOverflow)
  uint32_t* count;  // written at the end: records kept per segment
};

// Parameters of one edge pass.  Items are kept when their weight lies in
// [wmin, wmax], their relabelled endpoints differ, and (for the directed
// input) src < dst.  The class of a kept item is the first c with w <= thr[c]
// (c < nout-1), else nout-1.  Class 0 optionally feeds the next round's
// minimum (minval) with the value (w << 32 | position).
struct PassArgs {
  const uint32_t* map;  // label map; nullptr = identity
  // Optional membership bitmap of the largest component (bit x set iff
  // map[x] == big_label): an edge with both endpoints inside is dropped
  // without gathering map[], and one inside endpoint needs no gather.
  const uint32_t* big;
  uint32_t big_label;
  uint32_t wmin, wmax;
  uint32_t thr[kMaxOut];
  SegOut out[kMaxOut];
  uint64_t* minval;
  uint32_t min_checked;  // filter minimum updates by a cached read (hub-heavy passes)
  // Minimum keys (w << 32 | partner) instead of (w << 32 | list position):
  // the first pass over original ids, without parallel edges, where a
  // vertex's canonical (w, min, max) order is its (w, partner) order.  Both
  // directions are stored, so every copy (v, u, w) feeds v's minimum from
  // v's own row: the updates follow the (src, dst) order of the stream
  // instead of scattering to both endpoints of the kept record.
  uint32_t min_partner;
  uint64_t total;  // logical input items
  uint64_t chunk;  // logical items per CTA (a multiple of the tile size)
  unsigned long long* counts;  // [1] items that reached the label map ([0] unused)
  uint32_t* err;
  uint32_t n;         // ids must be < n (directed source)
  uint32_t validate;  // check id range and (src,dst) order (directed source)
  uint32_t aligned16; // directed source base is 16-byte aligned
  uint32_t cta_base;  // segment / chunk index of block 0 (a pass launched in groups)
  // List passes of late rounds, whose next round has few labels: the
  // minimum of labels [0, smin_n) is taken per CTA in shared memory and
  // flushed with one reduction per label at the end (0 = off).  With few
  // labels left, every record's update would otherwise hit one of a handful
  // of L2 addresses.
  uint32_t smin_n;
};

// The segment (and input chunk) this CTA owns.
__device__ __forceinline__ uint32_t seg_id(const PassArgs& p) { return blockIdx.x + p.cta_base; }

// Relabel a thread's ITEMS items with all label reads in flight together:
// membership bits first (one load per endpoint), then the map for the
// endpoints outside the largest component.  Writing the labels back to
// shared memory only afterwards keeps the compiler from ordering each
// item's loads behind the previous item's store.  keep[j] is cleared for
// items whose endpoints land in the same component.
template <int ITEMS>
__device__ __forceinline__ void relabel_batch(const PassArgs& p, const uint32_t (&a)[ITEMS],
                                              const uint32_t (&b)[ITEMS], bool (&keep)[ITEMS],
                                              uint32_t (&la)[ITEMS], uint32_t (&lb)[ITEMS]) {
  bool ina[ITEMS], inb[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    ina[j] = inb[j] = false;
    if (p.big && keep[j]) {
      ina[j] = (__ldg(p.big + (a[j] >> 5)) >> (a[j] & 31)) & 1u;
      inb[j] = (__ldg(p.big + (b[j] >> 5)) >> (b[j] & 31)) & 1u;
    }
  }
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    if (!keep[j]) continue;
    if (ina[j] && inb[j]) {
      keep[j] = false;
      continue;
    }
    la[j] = ina[j] ? p.big_label : p.map[a[j]];
    lb[j] = inb[j] ? p.big_label : p.map[b[j]];
  }
#pragma unroll
  for (int j = 0; j < ITEMS; ++j)
    if (keep[j] && la[j] == lb[j]) keep[j] = false;
}

template <int NOUT>
__device__ __forceinline__ uint8_t weight_class(uint32_t w, const PassArgs& p) {
  uint8_t c = NOUT - 1;
#pragma unroll
  for (int k = NOUT - 2; k >= 0; --k)
    if (w <= p.thr[k]) c = static_cast<uint8_t>(k);
  return c;
}

__device__ __forceinline__ uint32_t next_tile(uint32_t* ticket) {
  __shared__ uint32_t s_tile;
  __syncthreads();  // previous tile fully done with shared memory
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  return s_tile;
}

// A next-round minimum update into the CTA's shared minima; a label beyond
// them (not expected: the host sizes them for every label the round can
// produce) goes to the global word.  The shared word is read first: with a
// handful of labels left, every lane of a warp updates one of a few words,
// and the atomics on one word serialise, while once a CTA has seen a few
// tiles nearly every candidate is above its minimum.
__device__ __forceinline__ void smin_update(const PassArgs& p, uint64_t* smin, uint32_t x,
                                            uint64_t v) {
  if (x < p.smin_n) {
    unsigned long long* s = reinterpret_cast<unsigned long long*>(smin + x);
    if (v < *reinterpret_cast<volatile unsigned long long*>(s))
      atomicMin(s, static_cast<unsigned long long>(v));
  } else {
    red_min(&p.minval[x], v);
  }
}

// A kept record to its output segment with an L2 evict-first hint: the
// lists are streamed once per pass, and the gathered label and minimum arrays
// of the same pass keep the L2.
__device__ __forceinline__ void st_stream(Rec* dst, const Rec& r) {
  __stcs(reinterpret_cast<uint4*>(dst), make_uint4(r.a, r.b, r.w, r.oid));
}

// Rank the tile's kept items (stable), append them to this CTA's output
// segments and feed the fused minimum.  rec(t) returns tile item t from
// shared memory; run[] holds the CTA's running segment sizes (the same in
// every thread).  Two steps: the ranks place every kept item's tile index in
// a shared list (class by class, tile order), then the whole CTA writes the
// records and feeds the minimum from that list -- one kept item per thread
// and step instead of one predicated slot per item.  Few items of a pass
// over the directed input are kept (an eighth in the GNM first pass), so
// this halved its instructions per entry (first pass 8.15 -> 7.27 ms at
// 2^26/2^30; the list passes gained 0.3 ms).  Minimum updates of a checked
// pass read the current value first and reduce only when smaller.
template <int NOUT, int ITEMS, typename RecAt>
__device__ __forceinline__ void seg_tile_finish(const uint8_t (&cls)[ITEMS],
                                                      uint64_t (&run)[NOUT], const PassArgs& p,
                                                      RecAt rec, uint64_t* smin = nullptr) {
  __shared__ uint32_t s_rank[NOUT * ITEMS * (kBlock / 32)];
  __shared__ uint32_t s_tot[NOUT];
  __shared__ uint16_t s_dense[ITEMS * kBlock];
  uint32_t offs[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) offs[j] = 0;
  tile_rank<NOUT, ITEMS, kBlock>(cls, offs, s_rank, s_tot);
  uint32_t cbase[NOUT], tot[NOUT];
#pragma unroll
  for (int c = 0; c < NOUT; ++c) {
    tot[c] = s_tot[c];
    cbase[c] = c == 0 ? 0u : cbase[c - 1] + tot[c - 1];
  }
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint8_t c = cls[j];
    if (c == 0xff) continue;
    uint32_t b = cbase[0];
#pragma unroll
    for (int k = 1; k < NOUT; ++k)
      if (c == k) b = cbase[k];
    s_dense[b + offs[j]] = static_cast<uint16_t>(j * kBlock + threadIdx.x);
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < NOUT; ++c) {
    Rec* sg = p.out[c].base + static_cast<uint64_t>(seg_id(p)) * p.out[c].cap;
    const uint32_t cap = static_cast<uint32_t>(p.out[c].cap);
    const uint32_t run0 = static_cast<uint32_t>(run[c]);
    const uint64_t seg0 = static_cast<uint64_t>(seg_id(p)) * p.out[c].cap + run0;
    if constexpr (ITEMS <= 2) {
      // a class holds at most the tile's ITEMS * kBlock items: item k of
      // this thread is i = threadIdx.x + k * kBlock.  Every checking read of
      // the thread is in flight before the first compare, instead of one
      // read latency per item (wider tiles keep the per-item loop below:
      // their records would not fit in registers).
      bool has[ITEMS];
      Rec r[ITEMS];
#pragma unroll
      for (int k = 0; k < ITEMS; ++k) {
        const uint32_t i = threadIdx.x + k * kBlock;
        has[k] = i < tot[c];
        if (!has[k]) continue;
        if (run0 + i >= cap) {
          atomicOr(p.err, kErrOverflow);
          has[k] = false;
          continue;
        }
        r[k] = rec(s_dense[cbase[c] + i]);
        st_stream(sg + run0 + i, r[k]);
      }
      if (c != 0 || p.minval == nullptr || p.min_partner) continue;
      if (smin) {  // per-CTA minima (labels < p.smin_n)
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
          if (!has[k]) continue;
          const uint64_t v =
              (static_cast<uint64_t>(r[k].w) << 32) | (seg0 + threadIdx.x + k * kBlock);
          smin_update(p, smin, r[k].a, v);
          smin_update(p, smin, r[k].b, v);
        }
        continue;
      }
      uint64_t ca[ITEMS], cb[ITEMS];
#pragma unroll
      for (int k = 0; k < ITEMS; ++k) {
        ca[k] = cb[k] = ~0ull;
        if (has[k] && p.min_checked) {
          ca[k] = ld_weak(&p.minval[r[k].a]);
          cb[k] = ld_weak(&p.minval[r[k].b]);
        }
      }
#pragma unroll
      for (int k = 0; k < ITEMS; ++k) {
        if (!has[k]) continue;
        const uint64_t v =
            (static_cast<uint64_t>(r[k].w) << 32) | (seg0 + threadIdx.x + k * kBlock);
        if (v < ca[k]) red_min(&p.minval[r[k].a], v);
        if (v < cb[k]) red_min(&p.minval[r[k].b], v);
      }
    } else {
      for (uint32_t i = threadIdx.x; i < tot[c]; i += kBlock) {
        const uint32_t local = run0 + i;
        if (local >= cap) {
          atomicOr(p.err, kErrOverflow);
          continue;
        }
        const Rec r = rec(s_dense[cbase[c] + i]);
        st_stream(sg + local, r);
        if (c != 0 || p.minval == nullptr || p.min_partner) continue;
        const uint64_t v = (static_cast<uint64_t>(r.w) << 32) | (seg0 + i);
        if (smin) {
          smin_update(p, smin, r.a, v);
          smin_update(p, smin, r.b, v);
        } else if (p.min_checked) {
          const uint64_t ca = ld_weak(&p.minval[r.a]), cb = ld_weak(&p.minval[r.b]);
          if (v < ca) red_min(&p.minval[r.a], v);
          if (v < cb) red_min(&p.minval[r.b], v);
        } else {
          red_min(&p.minval[r.a], v);
          red_min(&p.minval[r.b], v);
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < NOUT; ++c) run[c] += tot[c];
}

template <int NOUT>
__device__ __forceinline__ void seg_pass_end(const uint64_t (&run)[NOUT], uint32_t cand,
                                             const PassArgs& p) {
  __shared__ uint32_t s_red;
  if (threadIdx.x == 0) s_red = 0;
  __syncthreads();
  const uint32_t c = warp_sum(cand);
  if (lane_id() == 0 && c) atomicAdd(&s_red, c);
  __syncthreads();
  if (threadIdx.x == 0 && s_red) atomicAdd(&p.counts[1], static_cast<unsigned long long>(s_red));
  // unclamped: a count above cap tells the host the exact size to retry with
  if (threadIdx.x < NOUT) p.out[threadIdx.x].count[seg_id(p)] = static_cast<uint32_t>(run[threadIdx.x]);
}

// Edge pass over the caller's directed input (12-byte records, (src,dst)
// sorted, both directions).  Only src < dst copies are candidates; a
// record's oid is its index in the input.  Copies need 16-byte multiples:
// the last tile's ragged tail is read with plain loads; a source that is
// not 16-byte aligned is read with plain loads throughout.  Striped layout:
// item j of thread t is tile item j*kBlock + t, so consecutive lanes read
// consecutive records (conflict-free) and write consecutive output slots.
// Items per thread is a tile-size knob (kamsta_cfg.items_per_thread: 6, 8
// or 12; 6 by default, the fastest on GB300 at 2^26/2^30).
constexpr uint32_t dir_tile(int items) { return static_cast<uint32_t>(items) * kBlock; }
constexpr size_t dir_dyn_smem(int items) { return 2ull * dir_tile(items) * 3 * sizeof(uint32_t); }
constexpr uint32_t kDirTile = dir_tile(kItemsDir);
constexpr size_t kDirDynSmem = dir_dyn_smem(kItemsDir);

template <int NOUT, int ITEMS = kItemsDir, bool MAPPED = false>
__global__ void __launch_bounds__(kBlock, ITEMS <= 8 ? 4 : 3)
    k_pass_dir(const uint32_t* __restrict__ in, PassArgs p) {
  constexpr uint32_t kDirTile = dir_tile(ITEMS);
  constexpr uint32_t kDirStageWords = kDirTile * 3;
  constexpr int kItemsDir = ITEMS;
  extern __shared__ __align__(128) uint32_t s_words[];  // two stages
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ uint32_t s_ok;
  const uint64_t lo = static_cast<uint64_t>(seg_id(p)) * p.chunk;
  const uint64_t hi = lo + p.chunk < p.total ? lo + p.chunk : p.total;
  const uint32_t ntile = lo < hi ? static_cast<uint32_t>((hi - lo + kDirTile - 1) / kDirTile) : 0u;
  const bool tma = p.aligned16 != 0;
  auto tile_items = [&](uint32_t k) -> uint32_t {
    const uint64_t b = lo + static_cast<uint64_t>(k) * kDirTile;
    return static_cast<uint32_t>(hi - b < kDirTile ? hi - b : kDirTile);
  };
  auto issue = [&](uint32_t k, int stage) {  // thread 0 only
    const uint32_t bytes16 = (tile_items(k) * 12u) & ~15u;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&s_bar[stage], bytes16);
    if (bytes16)
      bulk_load(s_words + stage * kDirStageWords,
                in + (lo + static_cast<uint64_t>(k) * kDirTile) * 3, bytes16, &s_bar[stage]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
    if (tma && ntile > 0) issue(0, 0);
  }
  __syncthreads();
  uint64_t run[NOUT];
#pragma unroll
  for (int c = 0; c < NOUT; ++c) run[c] = 0;
  uint32_t cand = 0;  // items that reached the label map (mapped passes)
  for (uint32_t k = 0; k < ntile; ++k) {
    const int stage = k & 1;
    uint32_t* words = s_words + stage * kDirStageWords;
    const uint64_t base = lo + static_cast<uint64_t>(k) * kDirTile;
    const uint32_t cnt = tile_items(k);
    uint32_t first_plain = 0;
    if (tma) {
      if (threadIdx.x == 0) s_ok = mbar_wait(&s_bar[stage], (k >> 1) & 1u, p.err) ? 1u : 0u;
      __syncthreads();  // also: every thread is done with tile k-1 and its stage
      if (!s_ok) return;
      if (threadIdx.x == 0 && k + 1 < ntile) issue(k + 1, stage ^ 1);
      first_plain = ((cnt * 12u) & ~15u) / 4u;
    } else {
      __syncthreads();
    }
    if (first_plain < cnt * 3) {
      for (uint32_t i = first_plain + threadIdx.x; i < cnt * 3; i += kBlock)
        words[i] = in[base * 3 + i];
      __syncthreads();
    }
    if (p.validate) {
#pragma unroll 1
      for (int j = 0; j < kItemsDir; ++j) {
        const uint32_t t = j * kBlock + threadIdx.x;
        if (t >= cnt) continue;
        const uint32_t s = words[3 * t], d = words[3 * t + 1];
        if (s >= p.n || d >= p.n) atomicOr(p.err, kErrRange);
        uint32_t ps = 0, pd = 0;
        bool have_prev = true;
        if (t > 0) {
          ps = words[3 * (t - 1)];
          pd = words[3 * (t - 1) + 1];
        } else if (base > 0) {
          ps = in[(base - 1) * 3];
          pd = in[(base - 1) * 3 + 1];
        } else {
          have_prev = false;
        }
        if (have_prev && (s < ps || (s == ps && d <= pd))) atomicOr(p.err, kErrOrder);
      }
    }
    uint8_t cls[kItemsDir];
    if constexpr (!MAPPED) {  // original ids: no label reads
#pragma unroll
      for (int j = 0; j < kItemsDir; ++j) {
        const uint32_t t = j * kBlock + threadIdx.x;
        const uint32_t s = words[3 * t], d = words[3 * t + 1], wt = words[3 * t + 2];
        cls[j] = 0xff;
        if (t >= cnt || s == d || s >= p.n || d >= p.n) continue;
        const bool in_w = wt >= p.wmin && wt <= p.wmax;
        // partner keys: every copy feeds its own row's minimum, so a
        // tile's updates go to a few consecutive addresses
        if (p.min_partner && in_w && weight_class<NOUT>(wt, p) == 0)
          red_min(&p.minval[s], (static_cast<uint64_t>(wt) << 32) | d);
        if (!(s < d) || !in_w) continue;
        cls[j] = weight_class<NOUT>(wt, p);
      }
    } else {
      uint32_t ss[kItemsDir], dd[kItemsDir], ww[kItemsDir];
      bool keep[kItemsDir];
#pragma unroll
      for (int j = 0; j < kItemsDir; ++j) {
        const uint32_t t = j * kBlock + threadIdx.x;
        ss[j] = words[3 * t];
        dd[j] = words[3 * t + 1];
        ww[j] = words[3 * t + 2];
        keep[j] = false;
        if (t >= cnt || !(ss[j] < dd[j]) || dd[j] >= p.n) continue;
        if (ww[j] < p.wmin || ww[j] > p.wmax) continue;
        ++cand;
        keep[j] = true;
      }
      uint32_t la[kItemsDir], lb[kItemsDir];
      relabel_batch<kItemsDir>(p, ss, dd, keep, la, lb);
#pragma unroll
      for (int j = 0; j < kItemsDir; ++j) {
        cls[j] = 0xff;
        if (!keep[j]) continue;
        const uint32_t t = j * kBlock + threadIdx.x;
        words[3 * t] = la[j];  // item t belongs to this thread alone
        words[3 * t + 1] = lb[j];
        cls[j] = weight_class<NOUT>(ww[j], p);
      }
    }
    auto rec_at = [&](uint32_t t) {
      Rec r;
      r.a = words[3 * t];
      r.b = words[3 * t + 1];
      r.w = words[3 * t + 2];
      r.oid = static_cast<uint32_t>(base + t);
      return r;
    };
    seg_tile_finish<NOUT, kItemsDir>(cls, run, p, rec_at);
  }
  seg_pass_end<NOUT>(run, cand, p);
}

// Edge pass over a segmented Rec list.  Tile k of a CTA covers logical
// items [lo + k*T, ...); thread 0 maps them to physical runs (at most a few,
// as segments hold thousands of records) and copies each run with one bulk
// copy into the tile's stage.
constexpr uint32_t rec_tile(int items) { return static_cast<uint32_t>(items) * kBlock; }
constexpr size_t rec_dyn_smem(int items) { return 2ull * rec_tile(items) * sizeof(Rec); }
constexpr uint32_t kRecTile = rec_tile(kItemsRec);
constexpr size_t kRecDynSmem = rec_dyn_smem(kItemsRec);
constexpr int kMaxRuns = 16;

// prefix[s] = records in segments < s (shared memory), built by the block
__device__ __forceinline__ void seg_prefix(const SegIn& in, uint64_t* prefix) {
  __shared__ uint64_t s_part[kBlock / 32];
  const uint32_t per = (in.nseg + kBlock - 1) / kBlock;  // <= kMaxSeg / kBlock
  uint64_t loc = 0;
  for (uint32_t i = 0; i < per; ++i) {
    const uint32_t s = threadIdx.x * per + i;
    if (s < in.nseg) loc += in.count[s];
  }
  uint64_t incl = loc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t y = __shfl_up_sync(kFull, incl, o);
    if (lane_id() >= static_cast<uint32_t>(o)) incl += y;
  }
  if (lane_id() == 31) s_part[threadIdx.x >> 5] = incl;
  __syncthreads();
  uint64_t wpre = 0;
  for (uint32_t w = 0; w < (threadIdx.x >> 5); ++w) wpre += s_part[w];
  uint64_t run = wpre + incl - loc;
  for (uint32_t i = 0; i < per; ++i) {
    const uint32_t s = threadIdx.x * per + i;
    if (s < in.nseg) {
      prefix[s] = run;
      run += in.count[s];
    }
  }
  if (threadIdx.x == kBlock - 1) prefix[in.nseg] = run;
  __syncthreads();
}

// first segment s with prefix[s+1] > x
__device__ __forceinline__ uint32_t seg_find(const uint64_t* prefix, uint32_t nseg, uint64_t x) {
  uint32_t lo = 0, hi = nseg;  // answer in [lo, hi)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (prefix[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// ITEMS (records per thread, 2, 4 or 8) is a tile knob: smaller tiles give
// more resident CTAs for the latency-bound relabel passes.
template <int NOUT, int ITEMS = kItemsRec>
__global__ void __launch_bounds__(kBlock, ITEMS <= 2 ? 5 : ITEMS <= 4 ? 4 : 3)
    k_pass_seg(SegIn in, PassArgs p) {
  constexpr uint32_t kRecTile = rec_tile(ITEMS);
  constexpr int kItemsRec = ITEMS;
  extern __shared__ __align__(128) Rec s_rec[];  // two stages, then p.smin_n minima
  uint64_t* s_min = p.smin_n ? reinterpret_cast<uint64_t*>(s_rec + 2 * kRecTile) : nullptr;
  __shared__ uint64_t s_prefix[kMaxSeg + 1];
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ uint32_t s_ok, s_plain[2];
  seg_prefix(in, s_prefix);
  const uint64_t lo = static_cast<uint64_t>(seg_id(p)) * p.chunk;
  const uint64_t hi = lo + p.chunk < p.total ? lo + p.chunk : p.total;
  const uint32_t ntile = lo < hi ? static_cast<uint32_t>((hi - lo + kRecTile - 1) / kRecTile) : 0u;
  auto tile_items = [&](uint32_t k) -> uint32_t {
    const uint64_t b = lo + static_cast<uint64_t>(k) * kRecTile;
    return static_cast<uint32_t>(hi - b < kRecTile ? hi - b : kRecTile);
  };
  // thread 0: copy logical [b, b+cnt) into stage; falls back to plain loads
  // (s_plain) when the range spans more than kMaxRuns segments
  auto issue = [&](uint32_t k, int stage) {
    const uint64_t b = lo + static_cast<uint64_t>(k) * kRecTile;
    const uint32_t cnt = tile_items(k);
    uint32_t s = seg_find(s_prefix, in.nseg, b);
    uint32_t runs = 0;
    {
      uint64_t x = b, left = cnt;
      uint32_t ss = s;
      while (left > 0 && runs <= kMaxRuns) {
        const uint64_t take0 = s_prefix[ss + 1] - x;
        const uint64_t take = take0 < left ? take0 : left;
        if (take) ++runs;
        x += take;
        left -= take;
        ++ss;
      }
    }
    s_plain[stage] = runs > kMaxRuns ? 1u : 0u;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&s_bar[stage], runs > kMaxRuns ? 0u : cnt * static_cast<uint32_t>(sizeof(Rec)));
    if (runs > kMaxRuns) return;
    uint64_t x = b, left = cnt;
    Rec* dst = s_rec + stage * kRecTile;
    while (left > 0) {
      const uint64_t off = x - s_prefix[s];
      const uint64_t take0 = s_prefix[s + 1] - x;
      const uint64_t take = take0 < left ? take0 : left;
      if (take) {
        bulk_load(dst, in.base + static_cast<uint64_t>(s) * in.cap + off,
                  static_cast<uint32_t>(take * sizeof(Rec)), &s_bar[stage]);
        dst += take;
      }
      x += take;
      left -= take;
      ++s;
    }
  };
  if (threadIdx.x == 0) {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
    if (ntile > 0) issue(0, 0);
  }
  for (uint32_t x = threadIdx.x; x < p.smin_n; x += kBlock) s_min[x] = kInf64;
  __syncthreads();
  uint64_t run[NOUT];
#pragma unroll
  for (int c = 0; c < NOUT; ++c) run[c] = 0;
  uint32_t cand = 0;  // items that reached the label map
  for (uint32_t k = 0; k < ntile; ++k) {
    const int stage = k & 1;
    Rec* recs = s_rec + stage * kRecTile;
    const uint64_t b = lo + static_cast<uint64_t>(k) * kRecTile;
    const uint32_t cnt = tile_items(k);
    if (threadIdx.x == 0) s_ok = mbar_wait(&s_bar[stage], (k >> 1) & 1u, p.err) ? 1u : 0u;
    __syncthreads();  // also: every thread is done with tile k-1 and its stage
    if (!s_ok) return;
    if (threadIdx.x == 0 && k + 1 < ntile) issue(k + 1, stage ^ 1);
    if (s_plain[stage]) {
      for (uint32_t t = threadIdx.x; t < cnt; t += kBlock) {
        const uint64_t x = b + t;
        const uint32_t s = seg_find(s_prefix, in.nseg, x);
        recs[t] = in.base[static_cast<uint64_t>(s) * in.cap + (x - s_prefix[s])];
      }
      __syncthreads();
    }
    uint8_t cls[kItemsRec];
    uint32_t ra[kItemsRec], rb[kItemsRec], rw[kItemsRec];
    bool keep[kItemsRec];
#pragma unroll
    for (int j = 0; j < kItemsRec; ++j) {
      const uint32_t t = j * kBlock + threadIdx.x;
      keep[j] = false;
      ra[j] = rb[j] = rw[j] = 0;
      if (t >= cnt) continue;
      const Rec r = recs[t];
      ra[j] = r.a;
      rb[j] = r.b;
      rw[j] = r.w;
      if (r.w < p.wmin || r.w > p.wmax) continue;
      ++cand;
      keep[j] = true;
    }
    if (p.map) {
      uint32_t la[kItemsRec], lb[kItemsRec];
      relabel_batch<kItemsRec>(p, ra, rb, keep, la, lb);
#pragma unroll
      for (int j = 0; j < kItemsRec; ++j) {
        if (!keep[j]) continue;
        const uint32_t t = j * kBlock + threadIdx.x;
        recs[t].a = la[j];
        recs[t].b = lb[j];
      }
    }
#pragma unroll
    for (int j = 0; j < kItemsRec; ++j) cls[j] = keep[j] ? weight_class<NOUT>(rw[j], p) : 0xff;
    seg_tile_finish<NOUT, kItemsRec>(cls, run, p, [&](uint32_t t) { return recs[t]; }, s_min);
  }
  if (s_min) {  // one reduction per label this CTA touched
    __syncthreads();
    for (uint32_t x = threadIdx.x; x < p.smin_n; x += kBlock) {
      const uint64_t v = s_min[x];
      if (v != kInf64) red_min(&p.minval[x], v);
    }
  }
  seg_pass_end<NOUT>(run, cand, p);
}

// ---------------------------------------------------------------------------
// Parallel-edge removal (EdgeProcessor::remove_duplicates_impl,
// duplicate_detection.hpp:25-64: sort by (src, dst, w), keep the lightest).
// Keys over the physical slots of a segmented list:
//   ((min label << bb | max label) << wbits) | w,  value = slot position;
// empty slots get ~0 and sort last.  After a stable LSD radix sort over the
// key bits, the head of every (min, max) run is its lightest edge, ties
// broken by the lower position, i.e. the survivor under the (w, min, max)
// order.  Every other slot of the run is marked dead in place by turning it
// into a self loop (b = a), which the next relabel pass drops.  A vertex's
// minimum edge is always a run head, so fused minima and the hook are
// unaffected.
__global__ void k_list_wmax(SegIn in, uint32_t* out) {
  const uint64_t phys = static_cast<uint64_t>(in.nseg) * in.cap;
  uint32_t mx = 0;
  for (uint64_t q = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; q < phys;
       q += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t seg = static_cast<uint32_t>(q / in.cap);
    if (q - static_cast<uint64_t>(seg) * in.cap < in.count[seg]) mx = max(mx, in.base[q].w);
  }
  mx = __reduce_max_sync(kFull, mx);
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(out, mx);
}

__global__ void k_dedupe_keys(SegIn in, uint32_t bb, uint32_t wbits, uint64_t* __restrict__ keys,
                              uint32_t* __restrict__ vals) {
  const uint64_t phys = static_cast<uint64_t>(in.nseg) * in.cap;
  for (uint64_t q = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; q < phys;
       q += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t seg = static_cast<uint32_t>(q / in.cap);
    uint64_t key = ~0ull;
    if (q - static_cast<uint64_t>(seg) * in.cap < in.count[seg]) {
      const Rec r = in.base[q];
      const uint64_t lo = min(r.a, r.b), hi = max(r.a, r.b);
      key = (((lo << bb) | hi) << wbits) | r.w;
    }
    keys[q] = key;
    vals[q] = static_cast<uint32_t>(q);
  }
}

__global__ void k_dedupe_mark(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                              uint64_t phys, uint32_t wbits, Rec* base,
                              unsigned long long* dead) {
  uint32_t d = 0;
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < phys;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[j];
    if (j == 0 || k == ~0ull) continue;
    if ((k >> wbits) == (keys[j - 1] >> wbits)) {
      Rec* r = base + vals[j];
      r->b = r->a;
      ++d;
    }
  }
  d = __reduce_add_sync(kFull, d);
  if ((threadIdx.x & 31) == 0 && d) atomicAdd(dead, static_cast<unsigned long long>(d));
}

// ---------------------------------------------------------------------------
// Hook (determine_mst_edges, mst_utils_cut_edges.hpp:102-166, without cut
// edges): every live vertex hooks onto the other endpoint of its minimum
// edge; of a mutual pair the lower label stays root.  Vertices without an
// incident edge are finished ("exhausted") and stay their own root.
// Each thread takes kIlp vertices per step (stride apart) and issues their
// loads level by level -- all minima, then all records, then all partner
// minima -- so several independent random reads are in flight per thread.
constexpr int kIlp = 4;

// Hook every vertex along its minimum edge (determine_mst_edges,
// mst_utils_plain.hpp:31-64); a mutual minimum roots the lower id.  With
// `partner_keys` (the first round over original ids, whose minima are
// (w << 32 | partner) keys) the partner comes from the key and no record is
// gathered; otherwise the key's low word is the record's list position and
// msfoid receives the record's input position.
__global__ void k_hook(uint32_t n, const uint64_t* __restrict__ minval,
                       const Rec* __restrict__ list, uint32_t* __restrict__ parent,
                       uint32_t* __restrict__ msfoid, uint32_t partner_keys, uint32_t chunk,
                       uint32_t* __restrict__ cta_counts, unsigned long long* counts,
                       uint32_t* err) {
  // CTA b hooks vertices [b * chunk, ...) -- the compaction's chunks -- and
  // counts its live roots and hooked vertices for the compaction
  const uint32_t lo = blockIdx.x * chunk;
  const uint32_t hi = static_cast<uint32_t>(min(static_cast<uint64_t>(lo) + chunk, uint64_t(n)));
  uint32_t c0 = 0, c1 = 0;
  for (uint64_t base = lo + threadIdx.x; base < hi; base += kIlp * kBlock) {
    uint64_t val[kIlp], mu[kIlp];
    Rec r[kIlp];
    uint32_t u[kIlp];
    bool live[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * kBlock;
      val[k] = v < hi ? minval[v] : kInf64;
      live[k] = val[k] != kInf64;
    }
    if (!partner_keys) {
#pragma unroll
      for (int k = 0; k < kIlp; ++k)
        if (val[k] != kInf64) r[k] = list[static_cast<uint32_t>(val[k])];
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      mu[k] = kInf64;
      u[k] = 0;
      if (val[k] == kInf64) continue;
      const uint32_t v = static_cast<uint32_t>(base + k * kBlock);
      if (partner_keys) {
        u[k] = static_cast<uint32_t>(val[k]);
        if (u[k] >= n) {
          val[k] = kInf64;  // reported, hooks nowhere
          atomicOr(err, kErrHook);
          continue;
        }
      } else {
        if (r[k].a != v && r[k].b != v) {
          val[k] = kInf64;  // reported, hooks nowhere
          atomicOr(err, kErrHook);
          continue;
        }
        u[k] = r[k].a ^ r[k].b ^ v;
      }
      mu[k] = minval[u[k]];
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      if (base + k * kBlock >= hi) continue;
      const uint32_t v = static_cast<uint32_t>(base + k * kBlock);
      if (partner_keys) {
        const uint64_t back = (val[k] & 0xffffffff00000000ull) | v;  // u's key if mutual
        const bool mutual = mu[k] == back;
        if (val[k] == kInf64 || (mutual && v < u[k])) {
          parent[v] = v;
          c0 += live[k] ? 1u : 0u;
          continue;
        }
        // v hooks on u, and u on its own partner x (the low word of u's
        // key) unless u is the root of a mutual pair, in which case x hooks
        // on u.  Either way x is in v's tree and one step nearer its root
        // pair, so v points at x directly: a pointer-jumping step for free.
        // The mutual pair's upper vertex keeps its root u.
        const uint32_t x = static_cast<uint32_t>(mu[k]);
        parent[v] = (mutual || mu[k] == kInf64 || x == v || x >= n) ? u[k] : x;
        ++c1;
      } else if (val[k] == kInf64 || (mu[k] == val[k] && v < u[k])) {
        parent[v] = v;
        msfoid[v] = kNone;
        c0 += live[k] ? 1u : 0u;
      } else {
        parent[v] = u[k];
        msfoid[v] = r[k].oid;
        ++c1;
      }
    }
  }
  __shared__ uint32_t s_c[2];
  if (threadIdx.x < 2) s_c[threadIdx.x] = 0;
  __syncthreads();
  c0 = warp_sum(c0);
  c1 = warp_sum(c1);
  if (lane_id() == 0) {
    if (c0) atomicAdd(&s_c[0], c0);
    if (c1) atomicAdd(&s_c[1], c1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    cta_counts[2 * blockIdx.x] = s_c[0];
    cta_counts[2 * blockIdx.x + 1] = s_c[1];
    if (s_c[0]) atomicAdd(&counts[0], static_cast<unsigned long long>(s_c[0]));
    if (s_c[1]) atomicAdd(&counts[1], static_cast<unsigned long long>(s_c[1]));
  }
}

// Pointer jumping to the roots (update_parents, gbbs_reimplementation.hpp:
// 161-169) with path halving; every write stores an ancestor, so concurrent
// updates stay correct.  Capped; the cap reports kErrJump.
// Each walk ends at its start vertex's root (the walk stops on a vertex that
// is its own parent), which is written to root_out[v] -- by v's thread
// alone, so unlike parent[v] it is never overwritten with a nearer ancestor
// by another walk.
__global__ void k_jump(uint32_t n, uint32_t* parent, uint32_t* __restrict__ root_out,
                       uint32_t* err) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; base < n;
       base += kIlp * stride) {
    // kIlp halving walks side by side, one step at a time
    uint32_t x[kIlp], p[kIlp];
    bool run[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      x[k] = static_cast<uint32_t>(v);
      p[k] = v < n ? ld_relaxed(parent + v) : x[k];
      run[k] = v < n && p[k] != x[k];
    }
    uint32_t steps = 0;
    for (;;) {
      bool any = false;
      uint32_t gp[kIlp];
#pragma unroll
      for (int k = 0; k < kIlp; ++k) gp[k] = run[k] ? ld_relaxed(parent + p[k]) : 0u;
#pragma unroll
      for (int k = 0; k < kIlp; ++k) {
        if (!run[k]) continue;
        if (gp[k] == p[k]) {
          run[k] = false;
          continue;
        }
        st_relaxed(parent + x[k], gp[k]);
        x[k] = gp[k];
        any = true;
      }
      if (!any) break;
#pragma unroll
      for (int k = 0; k < kIlp; ++k)
        if (run[k]) p[k] = ld_relaxed(parent + x[k]);
      ++steps;
      // a cycle (never produced by a correct hook) must not keep the device
      // busy: one thread reaching the cap stops all others within 1024 steps
      if ((steps & 1023u) == 0 && (steps > kJumpCap || (ld_relaxed(err) & kErrJump))) {
        atomicOr(err, kErrJump);
        break;
      }
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      if (v >= n) continue;
      if (p[k] != static_cast<uint32_t>(v)) st_relaxed(parent + v, p[k]);
      root_out[v] = p[k];
    }
  }
}

// Renumbering and forest-edge emission (compactify_vertices +
// add_new_mst_edges_to_mst_array), without a cross-CTA scan: CTA c owns the
// vertex chunk [c*chunk, (c+1)*chunk).  k_hook, which hooks the same
// chunks, counts each chunk's live roots (class 0: dense new ids, original
// representative carried, next minimum reset) and hooked vertices (class 1:
// forest edge appended); k_vertex_write sums the counts of the CTAs before
// it and writes, in vertex order, so ids and the forest order are
// deterministic.
// Root tags: bit 31 marks a root's parent entry, the low bits carry its new
// id; kRootTagNone marks a finished root (no new id).  Needs n < 2^31.
constexpr uint32_t kRootTag = 0x80000000u;
constexpr uint32_t kRootTagNone = 0xffffffffu;

struct VertexScanArgs {
  uint32_t n;
  uint32_t chunk;  // vertices per CTA (multiple of kBlock)
  const uint32_t* parent;
  const uint64_t* minval;
  const uint32_t* msfoid;
  const uint32_t* orig_cur;
  uint32_t* orig_next;
  uint32_t* newid;
  uint64_t* minval_next;
  uint32_t* msf_out;   // already offset by the forest edges found so far
  uint64_t msf_cap;    // entries available at msf_out
  uint64_t orig_cap;   // entries available at orig_next / minval_next
  uint32_t* cta_counts;  // 2 per CTA: roots, hooked
  unsigned long long* counts;  // [0] roots, [1] forest edges (totals)
  uint32_t* err;
  // direct emission (first round over original ids, minima as (w << 32 |
  // partner) keys): forest edge k of the round is written as (min, max, w)
  // at direct_out[3k..] from the hooked vertex's key, and the weights are
  // summed into direct_weight.  Null: msf_out receives input positions.
  uint32_t* direct_out;
  unsigned long long* direct_weight;
  // Root tags (k_jump_label): when set (the parent array, n < 2^31), each
  // root's entry receives kRootTag | its new id (kRootTagNone when finished)
  // instead of newid[v], so the walks that end at it read its label.
  uint32_t* root_tag;
};

// Vertices per thread per step of the compaction kernels: the loads of a
// step's vertices are all in flight before any is used, and one ranking
// (two barriers) covers kScanItems * kBlock vertices.
constexpr int kScanItems = 4;

// Class of vertex v from its parent and minimum: 0 = live root, 1 = hooked,
// 0xff = finished (a root without edges) or outside the range.
__device__ __forceinline__ uint8_t vertex_class(uint32_t v, uint32_t par, uint64_t minv) {
  if (par != v) return 1;
  return minv != kInf64 ? 0 : 0xff;
}

// Loads and classes of one step: item j of thread t is vertex r0 + j*kBlock
// + t (so ranking by (j, t) is vertex order).  The minimum is read for the
// roots, and for every vertex when `all_min` is set.
__device__ __forceinline__ void vertex_step(const VertexScanArgs& p, uint32_t r0, uint32_t hi,
                                            bool all_min, uint8_t (&cls)[kScanItems],
                                            uint64_t (&mv)[kScanItems]) {
  uint32_t par[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t v = r0 + j * kBlock + threadIdx.x;
    par[j] = v < hi ? p.parent[v] : v;
  }
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t v = r0 + j * kBlock + threadIdx.x;
    mv[j] = (v < hi && (all_min || par[j] == v)) ? p.minval[v] : kInf64;
  }
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t v = r0 + j * kBlock + threadIdx.x;
    cls[j] = v < hi ? vertex_class(v, par[j], mv[j]) : 0xff;
  }
}

__global__ void __launch_bounds__(kBlock) k_vertex_write(VertexScanArgs p) {
  __shared__ uint32_t s_base[2];
  __shared__ uint32_t s_rank[2 * kScanItems * (kBlock / 32)];
  __shared__ uint32_t s_tot[2];
  if (threadIdx.x < 32) {  // bases: counts of the CTAs before this one
    uint32_t b0 = 0, b1 = 0;
    for (uint32_t c = threadIdx.x; c < blockIdx.x; c += 32) {
      b0 += p.cta_counts[2 * c];
      b1 += p.cta_counts[2 * c + 1];
    }
    b0 = warp_sum(b0);
    b1 = warp_sum(b1);
    if (threadIdx.x == 0) {
      s_base[0] = b0;
      s_base[1] = b1;
    }
  }
  __syncthreads();
  const uint32_t lo = blockIdx.x * p.chunk;
  const uint32_t hi =
      static_cast<uint32_t>(min(static_cast<uint64_t>(lo) + p.chunk, uint64_t(p.n)));
  const bool direct = p.direct_out != nullptr;
  uint32_t run0 = s_base[0], run1 = s_base[1];
  uint64_t wsum = 0;
  for (uint32_t r0 = lo; r0 < hi; r0 += kScanItems * kBlock) {  // steps in vertex order
    uint8_t cls[kScanItems];
    uint64_t mv[kScanItems];
    vertex_step(p, r0, hi, direct, cls, mv);
    uint32_t offs[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) offs[j] = 0;
    tile_rank<2, kScanItems, kBlock>(cls, offs, s_rank, s_tot);
    const uint32_t tot0 = s_tot[0], tot1 = s_tot[1];
    // the per-class loads of all items first, then the writes
    uint32_t carry[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      const uint32_t v = r0 + j * kBlock + threadIdx.x;
      carry[j] = cls[j] == 0 ? p.orig_cur[v] : (cls[j] == 1 && !direct) ? p.msfoid[v] : 0u;
    }
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      const uint32_t v = r0 + j * kBlock + threadIdx.x;
      if (cls[j] == 0) {
        const uint32_t id = run0 + offs[j];
        if (id < p.orig_cap) {
          if (p.root_tag) p.root_tag[v] = kRootTag | id;
          else p.newid[v] = id;
          p.orig_next[id] = carry[j];
          p.minval_next[id] = kInf64;
        } else {
          if (p.root_tag) p.root_tag[v] = kRootTagNone;
          atomicOr(p.err, kErrOverflow);
        }
      } else if (cls[j] == 0xff) {
        if (p.root_tag && v < hi) p.root_tag[v] = kRootTagNone;  // finished root
      } else if (cls[j] == 1) {
        const uint32_t k = run1 + offs[j];
        if (k >= p.msf_cap) {
          atomicOr(p.err, kErrOverflow);
        } else if (direct) {
          const uint32_t u = static_cast<uint32_t>(mv[j]), w = static_cast<uint32_t>(mv[j] >> 32);
          uint32_t* o = p.direct_out + 3ull * k;
          o[0] = v < u ? v : u;
          o[1] = v < u ? u : v;
          o[2] = w;
          wsum += w;
        } else {
          p.msf_out[k] = carry[j];
        }
      }
    }
    run0 += tot0;
    run1 += tot1;
    __syncthreads();  // s_rank / s_tot are reused by the next step
  }
  if (direct) {
    wsum = warp_sum(wsum);
    if (lane_id() == 0 && wsum) atomicAdd(p.direct_weight, static_cast<unsigned long long>(wsum));
  }
}

// Pointer jumping and the round's label map in one walk: the roots' parent
// entries carry kRootTag | new id (k_vertex_write ran first), so the walk
// that reaches a root reads its label with the same load that tells it the
// walk is over -- no gather of newid[root] afterwards.  Path halving as in
// k_jump, writing only non-root entries (the tags are never overwritten),
// then parent[v] = root.  label[v] = the new id of v's root, or kNone when
// that root is finished.  Capped like k_jump.
__global__ void k_jump_label(uint32_t n, uint32_t* parent, uint32_t* __restrict__ label,
                             uint32_t* err) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  auto decode = [](uint32_t t) { return t == kRootTagNone ? kNone : (t & ~kRootTag); };
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; base < n;
       base += kIlp * stride) {
    // kIlp walks side by side; x: current vertex (never a root while a walk
    // runs), p: x's parent entry, root / lab: the result
    uint32_t x[kIlp], p[kIlp], root[kIlp], lab[kIlp];
    bool run[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      x[k] = static_cast<uint32_t>(v);
      p[k] = v < n ? ld_weak_u32(parent + v) : kRootTagNone;
      run[k] = !(p[k] & kRootTag);
      root[k] = x[k];
      lab[k] = run[k] ? kNone : decode(p[k]);
    }
    uint32_t steps = 0;
    for (;;) {
      bool any = false;
      uint32_t gp[kIlp];
#pragma unroll
      for (int k = 0; k < kIlp; ++k) gp[k] = run[k] ? ld_weak_u32(parent + p[k]) : 0u;
#pragma unroll
      for (int k = 0; k < kIlp; ++k) {
        if (!run[k]) continue;
        if (gp[k] & kRootTag) {  // p is the root
          root[k] = p[k];
          lab[k] = decode(gp[k]);
          run[k] = false;
          continue;
        }
        st_relaxed(parent + x[k], gp[k]);  // halving: x skips its parent
        x[k] = gp[k];
        any = true;
      }
      if (!any) break;
#pragma unroll
      for (int k = 0; k < kIlp; ++k) {
        if (!run[k]) continue;
        p[k] = ld_weak_u32(parent + x[k]);
        if (p[k] & kRootTag) {  // x is the root
          root[k] = x[k];
          lab[k] = decode(p[k]);
          run[k] = false;
        }
      }
      ++steps;
      if ((steps & 1023u) == 0 && (steps > kJumpCap || (ld_relaxed(err) & kErrJump))) {
        atomicOr(err, kErrJump);
        break;
      }
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      if (v >= n) continue;
      if (root[k] != static_cast<uint32_t>(v)) st_relaxed(parent + v, root[k]);
      label[v] = lab[k];
    }
  }
}

// Label map of one round: dense id in round r -> dense id in round r+1, or
// kNone for a finished vertex (a root without edges).  R holds each
// vertex's root on entry (k_jump) and its new label on return: one gather
// of the root's new id per hooked vertex.
__global__ void k_map(uint32_t n, const uint64_t* __restrict__ minval,
                      const uint32_t* __restrict__ newid, uint32_t* __restrict__ R) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; base < n;
       base += kIlp * stride) {
    uint32_t rt[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      rt[k] = v < n ? R[v] : 0u;
    }
    uint32_t q[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      q[k] = kNone;
      if (v >= n) continue;
      if (rt[k] != static_cast<uint32_t>(v) || minval[v] != kInf64) q[k] = newid[rt[k]];
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t v = base + k * stride;
      if (v < n) R[v] = q[k];
    }
  }
}

// Final labels of one Boruvka call, composed backwards over the round maps.
// For round r (vertices x < n_r), the map R_r holds x's round-(r+1) label or
// kNone once x's component is finished; afterwards R_r[x] holds the original
// representative of x's final component:
//   F_r[x] = R_r[x] == kNone ? orig_r[x] : F_{r+1}[R_r[x]],
// with F_rounds = orig_rounds (the components left after the last round).
// Launched for r = rounds-1 down to 1, so each map is read and gathered
// once (sum of n_r gathers, not n_0 walks through every round); r = 0 is
// k_compose_last, which writes the result to P at each vertex's original
// id instead.
constexpr int kMaxRounds = 40;
__global__ void k_compose(uint32_t n, uint32_t* __restrict__ R, const uint32_t* __restrict__ next,
                          const uint32_t* __restrict__ orig) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; base < n;
       base += kIlp * stride) {
    uint32_t y[kIlp], o[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t x = base + k * stride;
      y[k] = x < n ? R[x] : kNone;
      o[k] = x < n ? orig[x] : 0u;
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k)
      if (y[k] != kNone) y[k] = next[y[k]];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t x = base + k * stride;
      if (x >= n) continue;
      R[x] = y[k] == kNone ? o[k] : y[k];
    }
  }
}

// The last composition step (round 0, P set) over the compaction's chunks
// (RepScanArgs::chunk): besides P[orig[x]] = x's final representative it
// counts, per chunk, the level vertices that are their own representative
// -- the count half of the representatives' compaction (k_rep_write).
__global__ void k_compose_last(uint32_t n, const uint32_t* __restrict__ R,
                               const uint32_t* __restrict__ next,
                               const uint32_t* __restrict__ orig, uint32_t* __restrict__ P,
                               uint32_t chunk, uint32_t* __restrict__ cta_counts,
                               unsigned long long* counts) {
  const uint32_t lo = blockIdx.x * chunk;
  const uint32_t hi = static_cast<uint32_t>(min(static_cast<uint64_t>(lo) + chunk, uint64_t(n)));
  uint32_t c0 = 0;
  for (uint64_t base = lo + threadIdx.x; base < hi; base += kIlp * kBlock) {
    uint32_t y[kIlp], o[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      const uint64_t x = base + k * kBlock;
      y[k] = x < hi ? R[x] : kNone;
      o[k] = x < hi ? orig[x] : 0u;
    }
#pragma unroll
    for (int k = 0; k < kIlp; ++k)
      if (y[k] != kNone) y[k] = next[y[k]];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      if (base + k * kBlock >= hi) continue;
      const uint32_t f = y[k] == kNone ? o[k] : y[k];
      P[o[k]] = f;
      c0 += f == o[k] ? 1u : 0u;
    }
  }
  __shared__ uint32_t s_c;
  if (threadIdx.x == 0) s_c = 0;
  __syncthreads();
  c0 = warp_sum(c0);
  if (lane_id() == 0 && c0) atomicAdd(&s_c, c0);
  __syncthreads();
  if (threadIdx.x == 0) {
    cta_counts[blockIdx.x] = s_c;
    if (s_c) atomicAdd(counts, static_cast<unsigned long long>(s_c));
  }
}

struct RepScanArgs {
  uint32_t n;
  uint32_t chunk;
  const uint32_t* V;
  const uint32_t* P;
  uint32_t* Vout;
  uint32_t* dense_of;
  uint32_t* cta_counts;
  unsigned long long* counts;
  uint32_t* err;
};

// Representatives of one step (kScanItems vertices per thread, item j of
// thread t = entry r0 + j*kBlock + t): keep[j] iff V[i] is still its own
// final label.
__device__ __forceinline__ void rep_step(const RepScanArgs& p, uint32_t r0, uint32_t hi,
                                         uint8_t (&cls)[kScanItems],
                                         uint32_t (&v)[kScanItems]) {
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t i = r0 + j * kBlock + threadIdx.x;
    v[j] = i < hi ? p.V[i] : 0u;
  }
  uint32_t pv[kScanItems];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t i = r0 + j * kBlock + threadIdx.x;
    pv[j] = i < hi ? p.P[v[j]] : ~v[j];
  }
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) cls[j] = pv[j] == v[j] ? 0 : 0xff;
}

__global__ void __launch_bounds__(kBlock) k_rep_write(RepScanArgs p) {
  __shared__ uint32_t s_base;
  __shared__ uint32_t s_rank[kScanItems * (kBlock / 32)];
  __shared__ uint32_t s_tot[1];
  if (threadIdx.x < 32) {
    uint32_t b = 0;
    for (uint32_t c = threadIdx.x; c < blockIdx.x; c += 32) b += p.cta_counts[c];
    b = warp_sum(b);
    if (threadIdx.x == 0) s_base = b;
  }
  __syncthreads();
  const uint32_t lo = blockIdx.x * p.chunk;
  const uint32_t hi =
      static_cast<uint32_t>(min(static_cast<uint64_t>(lo) + p.chunk, uint64_t(p.n)));
  uint32_t run = s_base;
  for (uint32_t r0 = lo; r0 < hi; r0 += kScanItems * kBlock) {
    uint8_t cls[kScanItems];
    uint32_t v[kScanItems];
    rep_step(p, r0, hi, cls, v);
    uint32_t offs[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) offs[j] = 0;
    tile_rank<1, kScanItems, kBlock>(cls, offs, s_rank, s_tot);
    const uint32_t tot = s_tot[0];
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      if (cls[j] != 0) continue;
      const uint32_t k = run + offs[j];
      p.Vout[k] = v[j];
      p.dense_of[v[j]] = k;
    }
    run += tot;
    __syncthreads();  // s_rank / s_tot are reused by the next step
  }
}

// Membership bitmap of component `g`: bit x set iff D[x] == g.
__global__ void k_big_bitmap(uint32_t n, const uint32_t* __restrict__ D, uint32_t g,
                             uint32_t* __restrict__ bits) {
  const uint32_t words = (n + 31) / 32;
  for (uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < words;
       wi += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t x = wi * 32 + lane_id();
    const uint32_t b = __ballot_sync(kFull, x < n && D[x] == g);
    if (lane_id() == 0) bits[wi] = b;
  }
}

// ---------------------------------------------------------------------------
// Heavy-class contraction by row scans.  When the largest component holds
// all but a few vertices, an edge of the directed input survives the
// relabel pass (endpoint labels differ) only if one endpoint lies outside
// that component.  Those edges are found by scanning the input rows of the
// outside vertices -- the input is (src, dst)-sorted, so a row is one
// search away -- instead of streaming the whole input.  A record carries
// the position of either copy of its edge (the emit writes (min, max, w)
// whichever it is) and a key (min id << b | max id); sorting by the key
// restores the streaming pass's order, which is the order of the src < dst
// copies.  With `canon` set (the batch's forest bitmap, which needs the
// src < dst copy's position) the position of that copy is searched for.

// Vertices outside the largest component (bit 0 in `big`), any order; one
// counter atomic per warp and step.
__global__ void k_outside_big(uint32_t n, const uint32_t* __restrict__ big, uint32_t* __restrict__ out,
                             uint32_t cap, unsigned long long* count) {
  const uint32_t words = (n + 31) / 32;
  const uint32_t lane = lane_id();
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t start = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t w0 = start - lane; w0 < words; w0 += stride) {  // warp-uniform loop
    const uint32_t wi = w0 + lane;
    uint32_t f = 0;
    const uint32_t base = wi * 32;
    if (wi < words) {
      f = ~big[wi];
      if (base + 32 > n) f &= (n - base >= 32) ? ~0u : ((1u << (n - base)) - 1);
    }
    const uint32_t c = __popc(f);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (lane >= static_cast<uint32_t>(o)) incl += y;
    }
    unsigned long long wbase = 0;
    if (lane == 31 && incl) wbase = atomicAdd(count, static_cast<unsigned long long>(incl));
    wbase = __shfl_sync(kFull, wbase, 31);
    uint64_t k = wbase + incl - c;
    while (f) {
      const uint32_t b = __ffs(f) - 1;
      f &= f - 1;
      if (k < cap) out[k] = base + b;
      ++k;
    }
  }
}

// Fence index of the (src, dst)-sorted input: fence[i] = src of entry
// i * kFenceStep (i < ceil(md / kFenceStep)).  A row search then runs on the
// fences (a few MB, L2-resident) and then inside one kFenceStep window.
constexpr uint32_t kFenceStep = 1024;
__global__ void k_fences(const uint32_t* __restrict__ in, uint64_t md, uint32_t* __restrict__ fence) {
  const uint64_t nf = (md + kFenceStep - 1) / kFenceStep;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < nf;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    fence[i] = in[3 * i * kFenceStep];
}

// first directed entry with src >= v (entries [0, md) sorted by src); one
// thread
__device__ __forceinline__ uint64_t row_begin(const uint32_t* __restrict__ in, uint64_t md,
                                              uint32_t v) {
  uint64_t lo = 0, hi = md;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (in[3 * mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// The same with the whole warp: 32 probes per step shrink the range 33-fold.
// The fences narrow the range to one kFenceStep window first (their steps
// hit L2), so only two steps read the input.  Called by all 32 lanes with
// the same v; every lane returns the answer.
__device__ __forceinline__ uint64_t row_begin_warp(const uint32_t* __restrict__ in, uint64_t md,
                                                   const uint32_t* __restrict__ fence,
                                                   uint32_t v) {
  const uint32_t lane = lane_id();
  uint64_t lo = 0, hi = md;  // the answer lies in [lo, hi]
  {
    // first fence with src >= v: the answer lies in ((f - 1) step, f step]
    const uint64_t nf = (md + kFenceStep - 1) / kFenceStep;
    uint64_t flo = 0, fhi = nf;
    while (fhi - flo > 32) {
      const uint64_t span = fhi - flo;
      const uint64_t p = flo + span * (lane + 1) / 33;
      const uint32_t c = __popc(__ballot_sync(kFull, fence[p] < v));
      const uint64_t below = __shfl_sync(kFull, p, c == 0 ? 0 : c - 1);
      const uint64_t above = __shfl_sync(kFull, p, c == 32 ? 31 : c);
      if (c == 0) fhi = above;
      else if (c == 32) flo = below + 1;
      else {
        flo = below + 1;
        fhi = above;
      }
    }
    const uint64_t q = flo + lane;
    const uint64_t f = flo + __popc(__ballot_sync(kFull, q < fhi && fence[q] < v));
    lo = f == 0 ? 0 : (f - 1) * kFenceStep;
    hi = f * kFenceStep < md ? f * kFenceStep : md;
  }
  while (hi - lo > 32) {
    const uint64_t span = hi - lo;
    const uint64_t p = lo + span * (lane + 1) / 33;  // in [lo, hi), increasing in lane
    const uint32_t c = __popc(__ballot_sync(kFull, in[3 * p] < v));  // a prefix of lanes
    const uint64_t below = __shfl_sync(kFull, p, c == 0 ? 0 : c - 1);
    const uint64_t above = __shfl_sync(kFull, p, c == 32 ? 31 : c);
    if (c == 0) hi = above;
    else if (c == 32) lo = below + 1;
    else {
      lo = below + 1;
      hi = above;
    }
  }
  const uint64_t q = lo + lane;
  const bool less = q < hi && in[3 * q] < v;
  return lo + __popc(__ballot_sync(kFull, less));
}

// One warp per outside vertex v: every entry (v, d, w) of its row with w in
// [wmin, wmax] whose relabelled endpoints differ; d outside too and d < v:
// reported from d's row.  WRITE = false counts and stores each row's start
// in row_lo; WRITE = true writes records and keys at atomic slots.
template <bool WRITE>
__global__ void k_row_scan(const uint32_t* __restrict__ in, uint64_t md, uint32_t n,
                           const uint32_t* __restrict__ S, uint32_t ns, uint32_t* __restrict__ row_lo,
                           const uint32_t* __restrict__ fence,
                           const uint32_t* __restrict__ D, const uint32_t* __restrict__ big,
                           uint32_t big_label, uint32_t wmin, uint32_t wmax, uint32_t canon,
                           uint32_t key_bits, Rec* __restrict__ out, uint64_t* __restrict__ keys,
                           uint64_t cap, unsigned long long* count, uint32_t* err) {
  const uint32_t lane = lane_id();
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < ns; k += warps) {
    const uint32_t v = S[k];
    uint64_t lo;
    if (WRITE) {
      lo = row_lo[k];
    } else {
      lo = row_begin_warp(in, md, fence, v);
      if (lane == 0) row_lo[k] = static_cast<uint32_t>(lo);
    }
    const uint32_t la = D[v];
    for (uint64_t i0 = lo;; i0 += 32) {
      const uint64_t i = i0 + lane;
      const bool in_row = i < md && in[3 * i] == v;  // a prefix of lanes
      if (!__any_sync(kFull, in_row)) break;
      bool keep = false;
      Rec r;
      uint64_t key = 0;
      if (in_row) {
        const uint32_t d = in[3 * i + 1], w = in[3 * i + 2];
        if (d < n && d != v && w >= wmin && w <= wmax) {
          const bool d_big = (__ldg(big + (d >> 5)) >> (d & 31)) & 1u;
          const uint32_t lb = d_big ? big_label : D[d];
          if (la != lb) {
            if (v < d) {
              keep = true;
              r = Rec{la, lb, w, static_cast<uint32_t>(i)};
              key = (static_cast<uint64_t>(v) << key_bits) | d;
            } else if (d_big) {
              keep = true;
              r = Rec{lb, la, w, static_cast<uint32_t>(i)};
              key = (static_cast<uint64_t>(d) << key_bits) | v;
              if (WRITE && canon) {
                // the src<dst copy (d, v) sits in d's row, sorted by dst
                uint64_t a = row_begin(in, md, d), b = row_begin(in, md, d + 1);
                while (a < b) {
                  const uint64_t mid = (a + b) >> 1;
                  if (in[3 * mid + 1] < v) a = mid + 1; else b = mid;
                }
                if (a < md && in[3 * a] == d && in[3 * a + 1] == v) r.oid = static_cast<uint32_t>(a);
                else atomicOr(err, kErrRange);  // the input lacks (d, v)
              }
            }
          }
        }
      }
      const uint32_t bal = __ballot_sync(kFull, keep);
      if (!bal) continue;
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(count, static_cast<unsigned long long>(__popc(bal)));
      base = __shfl_sync(kFull, base, 0);
      if (WRITE && keep) {
        const uint64_t slot = base + __popc(bal & lanemask_lt());
        if (slot < cap) {
          out[slot] = r;
          keys[slot] = key;
        } else {
          atomicOr(err, kErrOverflow);
        }
      }
    }
  }
}

__global__ void k_set_u32(uint32_t* p, uint32_t v) { *p = v; }

// out[p] = in[idx[p]] and the round-0 minimum with position p.  Nearly every
// record has the largest component (`hub`) as one endpoint: its minimum is
// reduced in registers and per warp, one atomic per warp; the other
// endpoints' updates are filtered by a read.
__global__ void k_rec_place_min(const Rec* __restrict__ in, const uint32_t* __restrict__ idx,
                                uint64_t k, Rec* __restrict__ out, uint64_t* minval,
                                uint32_t hub) {
  uint64_t hub_min = kInf64;
  for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < k;
       p += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const Rec r = in[idx[p]];
    out[p] = r;
    const uint64_t v = (static_cast<uint64_t>(r.w) << 32) | p;
    if (r.a == hub) hub_min = v < hub_min ? v : hub_min;
    else if (v < ld_weak(&minval[r.a])) red_min(&minval[r.a], v);
    if (r.b == hub) hub_min = v < hub_min ? v : hub_min;
    else if (v < ld_weak(&minval[r.b])) red_min(&minval[r.b], v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t y = __shfl_xor_sync(kFull, hub_min, o);
    hub_min = y < hub_min ? y : hub_min;
  }
  if (lane_id() == 0 && hub_min != kInf64) red_min(&minval[hub], hub_min);
}

// D at `count` pseudo-random vertices (for picking the largest component).
__global__ void k_sample_labels(uint32_t n, const uint32_t* __restrict__ D, uint64_t seed,
                                uint32_t count, uint32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    out[i] = D[__umul64hi(mix64(seed ^ (0x9e3779b97f4a7c15ull * (i + 1))), n)];
}

// Shortcut every original vertex to its new representative and compute its
// dense label for the next call: P[x] = P[P[x]], D[x] = dense_of[P[x]].
__global__ void k_relabel_all(uint32_t n, uint32_t* __restrict__ P,
                              const uint32_t* __restrict__ dense_of,
                              uint32_t* __restrict__ D) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; base < n;
       base += kIlp * stride) {
    uint32_t p[kIlp], d[kIlp];
#pragma unroll
    for (int k = 0; k < kIlp; ++k) p[k] = base + k * stride < n ? P[base + k * stride] : 0u;
#pragma unroll
    for (int k = 0; k < kIlp; ++k) p[k] = base + k * stride < n ? P[p[k]] : 0u;
#pragma unroll
    for (int k = 0; k < kIlp; ++k) d[k] = base + k * stride < n ? dense_of[p[k]] : 0u;
#pragma unroll
    for (int k = 0; k < kIlp; ++k) {
      if (base + k * stride >= n) continue;
      P[base + k * stride] = p[k];
      D[base + k * stride] = d[k];
    }
  }
}

__global__ void k_iota(uint32_t n, uint32_t* __restrict__ a) {
  for (uint64_t x = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; x < n;
       x += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    a[x] = static_cast<uint32_t>(x);
}

__global__ void k_fill64(uint64_t n, uint64_t* __restrict__ a, uint64_t v) {
  for (uint64_t x = blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    a[x] = v;
}

// Forest output: gather the input copy of every forest edge (the src<dst
// copy, or for row-scan records possibly the other one), write it as
// (min, max, w) and sum the weights.
__global__ void k_emit(uint64_t k, const uint32_t* __restrict__ msf,
                       const uint32_t* __restrict__ in_words,
                       uint32_t* __restrict__ out_words,
                       unsigned long long* weight,
                       const unsigned long long* __restrict__ add_weight) {
  // add_weight: the weight of forest edges written elsewhere (direct emission)
  if (add_weight && blockIdx.x == 0 && threadIdx.x == 0 && *add_weight)
    atomicAdd(weight, *add_weight);
  uint64_t local = 0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t base = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; base < k;
       base += kIlp * stride) {
    uint32_t s[kIlp], d[kIlp], w[kIlp];
    uint64_t o[kIlp];
#pragma unroll
    for (int j = 0; j < kIlp; ++j)
      o[j] = base + j * stride < k ? static_cast<uint64_t>(msf[base + j * stride]) * 3 : ~0ull;
#pragma unroll
    for (int j = 0; j < kIlp; ++j) {
      if (o[j] == ~0ull) continue;
      s[j] = in_words[o[j]];
      d[j] = in_words[o[j] + 1];
      w[j] = in_words[o[j] + 2];
    }
#pragma unroll
    for (int j = 0; j < kIlp; ++j) {
      if (o[j] == ~0ull) continue;
      const uint64_t i = base + j * stride;
      out_words[3 * i] = s[j] < d[j] ? s[j] : d[j];  // either copy of the edge
      out_words[3 * i + 1] = s[j] < d[j] ? d[j] : s[j];
      out_words[3 * i + 2] = w[j];
      local += w[j];
    }
  }
  local = warp_sum(local);
  if (lane_id() == 0 && local) atomicAdd(weight, static_cast<unsigned long long>(local));
}

// Forest as a bitmap over input positions (batch split): bit oid of every
// forest edge is set.  The caller's split reads each marked entry anyway and
// sums the weights per graph, so no weight is gathered here.
__global__ void k_mark_forest(uint64_t k, const uint32_t* __restrict__ msf,
                              uint32_t* __restrict__ bits) {
  for (uint64_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t oid = msf[i];
    atomicOr(&bits[oid >> 5], 1u << (oid & 31));
  }
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

// Same over a segmented list; prefix[s] = records in segments < s.
__global__ void k_sample_weights_seg(SegIn in, const uint64_t* __restrict__ prefix, uint64_t m,
                                     uint64_t seed, uint32_t count, uint32_t* out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += gridDim.x * blockDim.x) {
    const uint64_t x = __umul64hi(mix64(seed + i), m);
    const uint32_t sg = seg_find(prefix, in.nseg, x);
    out[i] = in.base[static_cast<uint64_t>(sg) * in.cap + (x - prefix[sg])].w;
  }
}

}  // namespace kamsta
