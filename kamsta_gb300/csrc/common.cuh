// common.cuh -- shared device helpers of the GB300 MSF solver.
//
// Everything here is integer work: records, relaxed loads/stores for the
// single-pass (decoupled look-back) scans, stable in-tile ranking by warp
// ballots, and the bounded spin used by every wait.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/kamsta_gpu.h"

namespace kamsta {

constexpr uint64_t kInf64 = ~0ull;
constexpr uint32_t kNone = 0xffffffffu;
constexpr uint32_t kFull = 0xffffffffu;

// A live undirected edge inside the solver.  Lists of Rec are always kept in
// the input's (min, max) order, so (w << 32 | position) orders edges exactly
// like the reference's (weight, local edge index) key
// (mst_utils_common.hpp:76-81) and like its checker's (w, src, dst) order.
struct __align__(16) Rec {
  uint32_t a;    // current label of one endpoint
  uint32_t b;    // current label of the other endpoint
  uint32_t w;    // weight
  uint32_t oid;  // index of the src<dst copy in the directed input
};
static_assert(sizeof(Rec) == 16, "Rec must be 16 bytes");

// Device error bits (ORed into a device word, read by the host).
enum : uint32_t {
  kErrRange = 1u,     // id >= n in the input
  kErrOrder = 2u,     // input not sorted by (src, dst)
  kErrLookback = 4u,  // a look-back spin hit its cap
  kErrJump = 8u,      // pointer jumping hit its cap
  kErrHook = 16u,     // min edge not incident to its vertex (corruption)
  kErrChase = 32u,    // label chase longer than the round count
  kErrSpin = 64u,     // generic bounded wait expired
  kErrOverflow = 128u,  // an output buffer was too small (retry sized)
};

// Bounded spins: every wait in a kernel gives up after this many polls and
// reports kErrLookback instead of hanging the device.
constexpr uint32_t kSpinCap = 1u << 22;
// Pointer-jumping steps per vertex (a legal hook chain is shorter than n).
constexpr uint32_t kJumpCap = 1u << 26;

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// 64-bit minimum as a fire-and-forget reduction (red.min): the issuing
// thread never waits for the L2 round trip.  Right when few updates share
// an address (original vertex ids).
__device__ __forceinline__ void red_min(uint64_t* p, uint64_t v) {
  asm volatile("red.relaxed.gpu.global.min.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Weak (L1-cacheable) read of a minimum word.  Used only as a filter before
// red_min: the stored value never increases, so a stale read is an upper
// bound and can only let through an unnecessary update, never drop a
// needed one.  Contracted graphs have hub components (degree up to m), and
// without the filter their updates would serialise on one L2 address.
__device__ __forceinline__ uint64_t ld_weak(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.weak.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

// Weak (L1-cacheable) read of a parent entry during pointer jumping.  Parent
// entries only ever move to ancestors and root entries do not change within
// the walk kernel, so a stale value is still an ancestor: the walk stays
// correct and only may take an extra step.
__device__ __forceinline__ uint32_t ld_weak_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.weak.global.ca.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// SplitMix64's output function (Steele, Lea, Flood 2014): the counter-based
// hash behind weight sampling and the seeded graph generators.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// floor(sqrt(x)) for any 64-bit x (a double estimate, corrected exactly).
__host__ __device__ __forceinline__ uint64_t isqrt_u64(uint64_t x) {
  uint64_t s = static_cast<uint64_t>(sqrt(static_cast<double>(x)));
  if (s > 0xffffffffull) s = 0xffffffffull;
  while (s > 0 && s * s > x) --s;
  while (s < 0xffffffffull && (s + 1) * (s + 1) <= x) ++s;
  return s;
}

// Weight of a geometric generator's edge from its squared integer distance
// d2 <= R2 (the reference's distance types, benchmarks/mst_benchmarks.hpp:
// 59-64): random = the hash weight 1 + hi64(mix64(wseed ^ canon) *
// max_weight); squared Euclidean = 1 + floor((max_weight - 1) d2 / R2);
// Euclidean = 1 + floor(sqrt(floor((max_weight - 1)^2 d2 / R2))), i.e.
// 1 + floor((max_weight - 1) d / R).  Exact integer arithmetic, the same on
// host and device.
__host__ __device__ __forceinline__ uint32_t geo_weight(uint32_t mode, uint64_t d2, uint64_t R2,
                                                        uint64_t wseed, uint64_t canon,
                                                        uint32_t max_weight) {
  if (mode == KAMSTA_DISTANCE_RANDOM) {
    const unsigned __int128 p =
        static_cast<unsigned __int128>(mix64(wseed ^ canon)) * max_weight;
    return 1u + static_cast<uint32_t>(p >> 64);
  }
  if (R2 == 0) return 1u;
  const uint64_t k = max_weight - 1ull;
  if (mode == KAMSTA_DISTANCE_SQUARED_EUCLIDEAN)
    return 1u + static_cast<uint32_t>(static_cast<unsigned __int128>(d2) * k / R2);
  const unsigned __int128 q = static_cast<unsigned __int128>(d2) * k * k / R2;  // <= k^2
  return 1u + static_cast<uint32_t>(isqrt_u64(static_cast<uint64_t>(q)));
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Decoupled look-back (Merrill & Garland, "Single-pass Parallel Prefix Scan
// with Decoupled Look-back", 2016).  One 64-bit status word per tile:
// bits 63:62 flag (0 empty, 1 aggregate, 2 inclusive prefix), 61:0 value.
// Tiles are numbered by an atomic ticket, so every predecessor of a tile has
// started before the tile looks back; the spin is still capped.
constexpr uint64_t kLbAgg = 1ull << 62;
constexpr uint64_t kLbInc = 2ull << 62;
constexpr uint64_t kLbVal = (1ull << 62) - 1;

// Called by all 32 lanes of one warp.  Returns the exclusive prefix of
// `tile` (same value in every lane) and publishes its inclusive prefix.
// Each poll reads 256 predecessors (8 per lane, nearest first), so a tile
// usually reaches an inclusive prefix of the previous wave of CTAs in one
// or two polls instead of walking back 32 tiles at a time.
__device__ __forceinline__ uint64_t lookback(uint64_t* status, uint32_t tile,
                                             uint64_t local, uint32_t* err) {
  constexpr int kPer = 8;
  const uint32_t lane = lane_id();
  if (tile == 0) {
    if (lane == 0) st_relaxed(&status[0], kLbInc | local);
    return 0;
  }
  if (lane == 0) st_relaxed(&status[tile], kLbAgg | local);
  uint64_t excl = 0;
  int64_t window = static_cast<int64_t>(tile) - 1;
  uint32_t spins = 0;
  for (;;) {
    uint64_t s[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      const int64_t idx = window - static_cast<int64_t>(lane) * kPer - k;
      s[k] = idx >= 0 ? ld_relaxed(&status[idx]) : kLbInc;
    }
    int first_inc = kPer;
    bool empty_before = false;
    uint64_t partial = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
      if (first_inc == kPer) {
        const uint32_t flag = static_cast<uint32_t>(s[k] >> 62);
        if (flag == 0) empty_before = true;
        partial += s[k] & kLbVal;
        if (flag == 2) first_inc = k;
      }
    }
    const uint32_t inc = __ballot_sync(kFull, first_inc < kPer);
    const uint32_t limit = inc ? static_cast<uint32_t>(__ffs(inc) - 1) : 31u;
    const uint32_t relevant = limit == 31u ? kFull : ((2u << limit) - 1u);
    const uint32_t bad = __ballot_sync(kFull, empty_before) & relevant;
    if (bad) {
      if (++spins > kSpinCap) {
        if (lane == 0) atomicOr(err, kErrLookback);
        break;
      }
      __nanosleep(32);
      continue;
    }
    excl += warp_sum(lane <= limit ? partial : 0ull);
    if (inc) break;
    window -= 32 * kPer;
  }
  if (lane == 0) st_relaxed(&status[tile], kLbInc | (excl + local));
  return excl;
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (TMA, cp.async.bulk) into shared memory, completed
// on an mbarrier.  Used to stream input tiles: one elected thread issues the
// copy of the next tile while the CTA works on the current one.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same buffer
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// Bulk copy of a streamed-once tile into shared memory (bytes and both
// addresses multiples of 16), with an L2 evict-first policy: the stream leaves L2 to the randomly gathered label
// and minimum arrays of the same pass (measured 0.1 ms of 25.4 per solve at
// 2^26/2^30).
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                          uint64_t* bar) {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of `bar`; false (and kErrSpin) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* err) {
  for (uint32_t i = 0; i < kSpinCap; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  atomicOr(err, kErrSpin);
  return false;
}

// ---------------------------------------------------------------------------
// Stable in-tile ranking for up to NC output classes.
//
// Tile layout ("striped"): item j of thread t sits at tile position
// j * BLOCK + t, so the (j, warp, lane) order is the input order and a warp
// ballot per (j, warp) gives each kept item its rank inside its row.
// cls[j] = class in [0, NC) or 0xff for "dropped".  On return offs[j] is the
// item's rank among the tile's items of the same class, and tot[c] (shared)
// is the tile's count of class c.  smem must hold NC * ITEMS * WARPS words.
template <int NC, int ITEMS, int BLOCK>
__device__ __forceinline__ void tile_rank(const uint8_t (&cls)[ITEMS],
                                          uint32_t (&offs)[ITEMS],
                                          uint32_t* smem, uint32_t* tot) {
  constexpr int WARPS = BLOCK / 32;
  constexpr int ROWS = ITEMS * WARPS;
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    uint32_t mine = 0;  // the ballot of this item's class
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const uint32_t b = __ballot_sync(kFull, cls[j] == c);
      if (cls[j] == c) mine = b;
      if (lane == 0) smem[c * ROWS + j * WARPS + warp] = __popc(b);
    }
    offs[j] = __popc(mine & lt);
  }
  __syncthreads();
  // exclusive scan of each class row-list, one warp per class
  if (warp < NC) {
    const int c = warp;
    constexpr int PER = (ROWS + 31) / 32;
    uint32_t vals[PER];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int r = lane * PER + k;
      vals[k] = r < ROWS ? smem[c * ROWS + r] : 0u;
      s += vals[k];
    }
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (lane >= static_cast<uint32_t>(o)) incl += y;
    }
    uint32_t run = incl - s;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int r = lane * PER + k;
      if (r < ROWS) smem[c * ROWS + r] = run;
      run += vals[k];
    }
    if (lane == 31) tot[c] = incl;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < ITEMS; ++j)
    if (cls[j] != 0xff) offs[j] += smem[cls[j] * ROWS + j * WARPS + warp];
}

}  // namespace kamsta
