// radix_sort.cuh -- stable LSD radix sort of 64-bit keys (optional values).
//
// Used for parallel-edge removal (the reference sorts surviving edges with
// ips4o by (src, dst, w) and keeps the lightest, duplicate_detection.hpp:
// 25-64) and by the device graph generators.
//
// Per 8-bit digit: (1) k_rs_upsweep: per-tile digit histograms in shared
// memory from 128-bit key loads, stored digit major; (2) k_scan_u32: one
// exclusive scan of all histograms (decoupled look-back) -> every (digit,
// tile) output offset; (3) k_rs_downsweep: each warp ranks its rows of 32
// keys stably (8 ballots give the lanes sharing a digit), the tile is
// reordered by digit in shared memory and written out in digit runs
// (coalesced).  The downsweep loads one key per lane (a warp load moves 256
// contiguous bytes) because its ranking needs lane order = input order.
#pragma once
#include "common.cuh"

namespace kamsta {

constexpr int kRsBlock = 256;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsBlock * kRsItems;  // 4096 keys
constexpr int kScanItems = 8;
constexpr int kScanTile = kRsBlock * kScanItems;

struct NoVal {};

template <typename V>
struct ValTraits {
  static constexpr bool kHas = true;
  static constexpr size_t kSize = sizeof(V);
};
template <>
struct ValTraits<NoVal> {
  static constexpr bool kHas = false;
  static constexpr size_t kSize = 0;
};

__global__ void __launch_bounds__(kRsBlock)
    k_rs_upsweep(const uint64_t* __restrict__ keys, uint64_t n, uint32_t shift,
                 uint32_t ntiles, uint32_t* __restrict__ counts) {
  __shared__ uint32_t hist[256];
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    hist[threadIdx.x] = 0;
    __syncthreads();
    // 128-bit loads: thread t reads key pairs (2q, 2q+1) of the tile, q =
    // j * kRsBlock + t; a tile starts on a 32 KB boundary of the key array
    // (pool memory, 256-byte aligned), so every pair is 16-byte aligned
    const uint64_t base = static_cast<uint64_t>(tile) * kRsTile;
    const ulonglong2* pairs = reinterpret_cast<const ulonglong2*>(keys + base);
#pragma unroll 4
    for (int j = 0; j < kRsItems / 2; ++j) {
      const uint64_t q = static_cast<uint64_t>(j) * kRsBlock + threadIdx.x;
      const uint64_t i = base + 2 * q;
      uint64_t k0 = ~0ull, k1 = ~0ull;  // pads sort last
      if (i + 1 < n) {
        const ulonglong2 kk = pairs[q];
        k0 = kk.x;
        k1 = kk.y;
      } else if (i < n) {
        k0 = keys[i];
      }
      atomicAdd(&hist[(k0 >> shift) & 255u], 1u);
      atomicAdd(&hist[(k1 >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[static_cast<uint64_t>(threadIdx.x) * ntiles + tile] = hist[threadIdx.x];
    __syncthreads();
  }
}

// Exclusive scan of a u32 array (in place allowed), single pass.
__global__ void __launch_bounds__(kRsBlock)
    k_scan_u32(const uint32_t* in, uint32_t* out, uint64_t n, uint64_t* status,
               uint32_t* ticket, uint32_t ntiles, uint32_t* err) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[kRsBlock / 32];
  __shared__ uint64_t s_pre;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= ntiles) return;
    // blocked per thread: items [t*ITEMS, (t+1)*ITEMS) of the tile
    const uint64_t base = static_cast<uint64_t>(tile) * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      v[j] = base + j < n ? in[base + j] : 0u;
      sum += v[j];
    }
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
      uint32_t wv = lane < kRsBlock / 32 ? s_warp[lane] : 0u;
      uint32_t wi = wv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, wi, o);
        if (lane >= static_cast<uint32_t>(o)) wi += y;
      }
      const uint32_t total = __shfl_sync(kFull, wi, kRsBlock / 32 - 1);
      if (lane < kRsBlock / 32) s_warp[lane] = wi - wv;
      const uint64_t pre = lookback(status, tile, total, err);
      if (lane == 0) s_pre = pre;
    }
    __syncthreads();
    uint64_t run = s_pre + s_warp[warp] + (incl - sum);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      if (base + j < n) out[base + j] = static_cast<uint32_t>(run);
      run += v[j];
    }
  }
}

template <typename V>
__global__ void __launch_bounds__(kRsBlock)
    k_rs_downsweep(const uint64_t* __restrict__ keys_in, const V* __restrict__ vals_in,
                   uint64_t* __restrict__ keys_out, V* __restrict__ vals_out, uint64_t n,
                   uint32_t shift, uint32_t ntiles, const uint32_t* __restrict__ offsets) {
  constexpr int WARPS = kRsBlock / 32;
  constexpr bool HV = ValTraits<V>::kHas;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* s_keys = reinterpret_cast<uint64_t*>(smem_raw);
  V* s_vals = reinterpret_cast<V*>(smem_raw + sizeof(uint64_t) * kRsTile);
  __shared__ uint32_t s_whist[WARPS][256];
  __shared__ uint32_t s_start[256];
  __shared__ uint32_t s_goff[256];
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  const uint32_t lt = lanemask_lt();
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    for (int d = threadIdx.x; d < WARPS * 256; d += kRsBlock) (&s_whist[0][0])[d] = 0;
    s_goff[threadIdx.x] = offsets[static_cast<uint64_t>(threadIdx.x) * ntiles + tile];
    __syncthreads();
    const uint64_t base = static_cast<uint64_t>(tile) * kRsTile + warp * 32 * kRsItems;
    uint64_t k[kRsItems];
    V v[kRsItems];
    uint32_t rank[kRsItems];
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
      const uint64_t i = base + j * 32 + lane;
      k[j] = i < n ? keys_in[i] : ~0ull;
      if constexpr (HV) {
        if (i < n) v[j] = vals_in[i];
      }
    }
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
      const uint32_t dg = static_cast<uint32_t>(k[j] >> shift) & 255u;
      uint32_t peers = kFull;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const uint32_t bal = __ballot_sync(kFull, (dg >> b) & 1u);
        peers &= ((dg >> b) & 1u) ? bal : ~bal;
      }
      const uint32_t before = s_whist[warp][dg];
      rank[j] = before + __popc(peers & lt);
      __syncwarp();
      if ((__ffs(peers) - 1) == static_cast<int>(lane)) s_whist[warp][dg] = before + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    {  // per digit: exclusive over warps, tile count
      const uint32_t d = threadIdx.x;
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const uint32_t t = s_whist[w][d];
        s_whist[w][d] = run;
        run += t;
      }
      // exclusive scan of tile counts over digits (block-wide)
      uint32_t incl = run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += y;
      }
      __shared__ uint32_t s_wsum[WARPS];
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      uint32_t wpre = 0;
      for (uint32_t w = 0; w < warp; ++w) wpre += s_wsum[w];
      s_start[d] = wpre + incl - run;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
      const uint32_t dg = static_cast<uint32_t>(k[j] >> shift) & 255u;
      const uint32_t pos = s_start[dg] + s_whist[warp][dg] + rank[j];
      s_keys[pos] = k[j];
      if constexpr (HV) s_vals[pos] = v[j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kRsTile; i += kRsBlock) {
      const uint64_t key = s_keys[i];
      const uint32_t dg = static_cast<uint32_t>(key >> shift) & 255u;
      const uint64_t g = static_cast<uint64_t>(s_goff[dg]) + (i - s_start[dg]);
      if (g < n) {
        keys_out[g] = key;
        if constexpr (HV) vals_out[g] = s_vals[i];
      }
    }
    __syncthreads();
  }
}

}  // namespace kamsta
