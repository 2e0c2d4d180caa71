// codec.cu -- 7-bit varint difference encoding of the directed input
// (Compression::SEVEN_BIT_DIFF_ENCODING, algorithm_configurations.hpp:18-25).
//
// Per edge the reference stores varint(src - prev_src), varint(dst),
// varint(w) (DifferenceEncodedGraph::encode_edges,
// difference_encoded_graph.hpp:175-205) with its 7-bit little-endian
// varint, continuation bit 0x80 (encode_value / decode_value,
// variable_length_encoding.hpp:6-167); the edge list is cut into chunks, each
// starting with a raw first edge and a byte offset.  The byte stream of a
// chunk here is exactly that; chunks are small (<= 4096 edges) so that the
// device decodes one chunk per CTA:
//   1. the chunk's bytes go to shared memory;
//   2. a block scan over "last byte of a value" flags gives every byte its
//      value index; the thread holding a value's last byte assembles it;
//   3. a block scan over the src deltas restores src; edges are written out.
// The host encoder runs on all host cores.  A decoded input feeds the normal
// solver, so a compressed graph costs about half the bytes to keep resident
// or to copy to the device.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "codec.cuh"
#include "common.cuh"
#include "solver.cuh"

namespace kamsta {

namespace {

constexpr int kDecBlock = 512;

inline uint32_t varint_len(uint64_t v) {
  uint32_t n = 1;
  while (v >= 128) {
    v >>= 7;
    ++n;
  }
  return n;
}

inline uint8_t* varint_put(uint64_t v, uint8_t* o) {
  while (v >= 128) {
    *o++ = static_cast<uint8_t>((v & 0x7f) | 0x80);
    v >>= 7;
  }
  *o++ = static_cast<uint8_t>(v);
  return o;
}

// Block-wide exclusive scan of one u32 per thread; returns the total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* excl, uint32_t* s_warp) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t wv = lane < kDecBlock / 32 ? s_warp[lane] : 0u;
    uint32_t wi = wv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, wi, o);
      if (lane >= static_cast<uint32_t>(o)) wi += y;
    }
    if (lane < kDecBlock / 32) s_warp[lane] = wi - wv;
    if (lane == kDecBlock / 32 - 1) s_warp[kDecBlock / 32] = wi;
  }
  __syncthreads();
  *excl = s_warp[warp] + incl - v;
  const uint32_t total = s_warp[kDecBlock / 32];
  __syncthreads();
  return total;
}

// Continuation-bit positions (bit 7 of each byte) of window word q that
// belong to the chunk, whose bytes are window bytes [skip, wend).
__device__ __forceinline__ uint32_t chunk_bits(uint32_t q, uint32_t skip, uint32_t wend) {
  uint32_t mask = 0x80808080u;
  const uint32_t b = 4 * q;
  if (b < skip) mask = skip - b >= 4 ? 0u : mask << (8 * (skip - b));
  if (b + 4 > wend) mask &= wend <= b ? 0u : 0x80808080u >> (8 * (b + 4 - wend));
  return mask;
}

// One chunk per CTA step:
//   1. its bytes into shared memory (16-byte loads for the aligned middle);
//   2. each thread counts the value terminators (bytes without bit 7) in its
//      run of 4-byte words, and a block scan numbers the values;
//   3. each thread walks its bytes once, in order, assembling values and
//      emitting each at its terminator; the value whose first bytes belong
//      to the thread before is completed from up to 9 bytes looked back;
//   4. the srcs are restored from the deltas (a block scan of per-thread
//      delta sums) in place of the deltas;
//   5. the chunk's 3 * C words go out coalesced, 16 bytes per store where the
//      output is aligned.
// Two CTAs per SM at most (each holds up to 27 * C bytes of shared memory),
// so up to 64 registers per thread are free.
__global__ void __launch_bounds__(kDecBlock, 2)
    k_decode_7bit(const uint64_t* __restrict__ chunk_off, const kamsta_wedge* __restrict__ first,
                  const uint8_t* __restrict__ data, uint64_t m, uint32_t C, uint64_t nchunks,
                  uint32_t* __restrict__ out, uint32_t* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* vals = reinterpret_cast<uint32_t*>(smem);  // 3 * C values
  // the chunk's bytes, placed as in a window that starts at the 16-byte
  // boundary at or below the chunk's first byte (<= 15 * C + 16 bytes)
  uint8_t* win = smem + ((sizeof(uint32_t) * 3 * C + 15) & ~size_t(15));
  const uint32_t* wwin = reinterpret_cast<const uint32_t*>(win);
  __shared__ uint32_t s_warp[kDecBlock / 32 + 1];
  for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const uint64_t e0 = c * C;
    const uint32_t ce = static_cast<uint32_t>(m - e0 < C ? m - e0 : C);  // edges in chunk
    const uint64_t b0 = chunk_off[c];
    const uint32_t nb = static_cast<uint32_t>(chunk_off[c + 1] - b0);
    const uint32_t nv = 3 * (ce - 1);
    if (nb > 15u * C) {  // cannot come from sorted 32-bit input
      if (threadIdx.x == 0) atomicOr(err, kErrRange);
      continue;
    }
    // 16-byte loads for the aligned middle of the byte range, single bytes
    // for its ragged ends; every load lies inside [b0, b0 + nb)
    const uint64_t b1 = b0 + nb, a0 = b0 & ~15ull;
    const uint64_t m0 = (b0 + 15) & ~15ull, m1 = b1 & ~15ull;
    if (m0 < m1) {
      const uint4* src = reinterpret_cast<const uint4*>(data + m0);
      uint4* dst = reinterpret_cast<uint4*>(win + (m0 - a0));
      for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>((m1 - m0) / 16); q += kDecBlock)
        dst[q] = src[q];
      for (uint64_t x = b0 + threadIdx.x; x < m0; x += kDecBlock) win[x - a0] = data[x];
      for (uint64_t x = m1 + threadIdx.x; x < b1; x += kDecBlock) win[x - a0] = data[x];
    } else {
      for (uint64_t x = b0 + threadIdx.x; x < b1; x += kDecBlock) win[x - a0] = data[x];
    }
    __syncthreads();
    const uint32_t skip = static_cast<uint32_t>(b0 - a0), wend = skip + nb;
    const uint32_t nw = (wend + 3) / 4;
    const uint32_t perw = (nw + kDecBlock - 1) / kDecBlock;
    const uint32_t w_lo = min(nw, threadIdx.x * perw), w_hi = min(nw, w_lo + perw);
    uint32_t cnt = 0;
    for (uint32_t q = w_lo; q < w_hi; ++q)
      cnt += __popc(~wwin[q] & chunk_bits(q, skip, wend));
    uint32_t vbase = 0;
    const uint32_t total = block_excl_scan(cnt, &vbase, s_warp);
    if (total != nv) {
      if (threadIdx.x == 0) atomicOr(err, kErrRange);
      continue;
    }
    if (w_lo < w_hi) {
      // ids and weights are 32-bit: a value is kept mod 2^32, so only its
      // first five groups of 7 bits matter
      uint32_t acc = 0, sh = 0;
      // bytes of the value that runs into this thread's words from before
      const uint32_t s0 = 4 * w_lo;
      uint32_t p = s0;
      while (p > skip && (win[p - 1] & 0x80) && s0 - p < 9) --p;
      for (uint32_t k = p; k < s0; ++k, sh += 7)
        if (sh < 32) acc |= static_cast<uint32_t>(win[k] & 0x7f) << sh;
      uint32_t v = vbase;
      for (uint32_t q = w_lo; q < w_hi; ++q) {
        const uint32_t w = wwin[q];
        const uint32_t in = chunk_bits(q, skip, wend);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (!((in >> (8 * j + 7)) & 1u)) continue;  // not a chunk byte
          const uint32_t by = (w >> (8 * j)) & 0xffu;
          if (sh < 32) acc |= (by & 0x7fu) << sh;
          sh += 7;
          if (!(by & 0x80u)) {
            vals[v++] = acc;
            acc = 0;
            sh = 0;
          }
        }
      }
    }
    __syncthreads();
    // src = first src + running sum of the deltas; thread t owns edges
    // [1 + t*pe, 1 + (t+1)*pe) and overwrites their deltas with their srcs
    // (pe odd: the threads' words are 3 * pe apart, on distinct banks)
    const uint32_t pe = ((ce - 1 + kDecBlock - 1) / kDecBlock) | 1u;
    const uint32_t a = 1 + threadIdx.x * pe, z = min(ce, a + pe);
    uint32_t dsum = 0;
    for (uint32_t e = a; e < z; ++e) dsum += vals[3 * (e - 1)];
    uint32_t dpre = 0;
    block_excl_scan(dsum, &dpre, s_warp);
    const kamsta_wedge f = first[c];
    uint32_t src = f.src + dpre;
    for (uint32_t e = a; e < z; ++e) {
      src += vals[3 * (e - 1)];
      vals[3 * (e - 1)] = src;
    }
    __syncthreads();
    // the chunk's entries: its raw first edge, then the values
    uint32_t* o = out + 3 * e0;
    const uint32_t nwords = 3 * ce;
    auto word = [&](uint32_t i) -> uint32_t {
      return i >= 3 ? vals[i - 3] : i == 0 ? f.src : i == 1 ? f.dst : f.w;
    };
    uint32_t done = 0;
    if ((reinterpret_cast<uintptr_t>(o) & 15) == 0) {
      done = nwords & ~3u;
      for (uint32_t q = threadIdx.x; q < nwords / 4; q += kDecBlock)
        reinterpret_cast<uint4*>(o)[q] =
            make_uint4(word(4 * q), word(4 * q + 1), word(4 * q + 2), word(4 * q + 3));
    }
    for (uint32_t i = done + threadIdx.x; i < nwords; i += kDecBlock) o[i] = word(i);
    __syncthreads();
  }
}

}  // namespace

kamsta_status encode_7bit(const kamsta_wedge* e, uint64_t m, uint32_t C, uint64_t* off,
                          kamsta_wedge* first, uint8_t* data, uint64_t cap, uint64_t* bytes) {
  *bytes = 0;
  if (C == 0 || C > kMaxChunkEdges) {
    set_error("encode_7bit: chunk_edges must be in [1, 4096]");
    return KAMSTA_E_INPUT;
  }
  const uint64_t nch = (m + C - 1) / C;
  std::vector<uint64_t> len(nch, 0);
  const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  auto par = [&](auto&& fn) {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < hw; ++t)
      th.emplace_back([&, t] {
        for (uint64_t c = nch * t / hw; c < nch * (t + 1) / hw; ++c) fn(c);
      });
    for (auto& x : th) x.join();
  };
  std::atomic<bool> bad{false};
  par([&](uint64_t c) {
    uint64_t l = 0;
    const uint64_t a = c * C, z = std::min<uint64_t>(m, a + C);
    for (uint64_t i = a + 1; i < z; ++i) {
      if (e[i].src < e[i - 1].src) bad = true;  // deltas must be non-negative
      l += varint_len(static_cast<uint64_t>(e[i].src) - e[i - 1].src) + varint_len(e[i].dst) +
           varint_len(e[i].w);
    }
    len[c] = l;
  });
  if (bad) {
    set_error("encode_7bit: input must be sorted by src");
    return KAMSTA_E_INPUT;
  }
  uint64_t total = 0;
  for (uint64_t c = 0; c < nch; ++c) {
    if (off) off[c] = total;
    total += len[c];
  }
  if (off) off[nch] = total;
  *bytes = total;
  if (!data) return KAMSTA_OK;
  if (!off || !first) {
    set_error("encode_7bit: chunk_offset and chunk_first are required");
    return KAMSTA_E_INPUT;
  }
  if (total > cap) {
    set_error("encode_7bit: data capacity too small (required bytes in data_bytes)");
    return KAMSTA_E_INPUT;
  }
  par([&](uint64_t c) {
    const uint64_t a = c * C, z = std::min<uint64_t>(m, a + C);
    first[c] = e[a];
    uint8_t* o = data + off[c];
    for (uint64_t i = a + 1; i < z; ++i) {
      o = varint_put(static_cast<uint64_t>(e[i].src) - e[i - 1].src, o);
      o = varint_put(e[i].dst, o);
      o = varint_put(e[i].w, o);
    }
  });
  return KAMSTA_OK;
}

kamsta_status decode_7bit(const kamsta_cgraph& g, kamsta_wedge* d_out, uint32_t* d_err,
                          cudaStream_t st) {
  if (g.m_directed == 0) return KAMSTA_OK;
  if (g.chunk_edges == 0 || g.chunk_edges > kMaxChunkEdges ||
      g.num_chunks != (g.m_directed + g.chunk_edges - 1) / g.chunk_edges) {
    set_error("decode_7bit: inconsistent chunk layout");
    return KAMSTA_E_INPUT;
  }
  const size_t smem = ((12ull * g.chunk_edges + 15) & ~15ull) + 15ull * g.chunk_edges + 64;
  cudaError_t e = cudaFuncSetAttribute(k_decode_7bit, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(k_decode_7bit)");
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t grid = std::min<uint64_t>(g.num_chunks, uint64_t(sms) * 8);
  k_decode_7bit<<<static_cast<uint32_t>(grid), kDecBlock, smem, st>>>(
      g.chunk_offset, g.chunk_first, g.data, g.m_directed, g.chunk_edges, g.num_chunks,
      reinterpret_cast<uint32_t*>(d_out), d_err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e, "k_decode_7bit");
  return KAMSTA_OK;
}

}  // namespace kamsta
