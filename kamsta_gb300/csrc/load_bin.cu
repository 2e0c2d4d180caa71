// load_bin.cu -- the reference's binary weighted edge files, streamed to the
// device and turned into the solver's input contract.
//
// Format (evaluation/README.md:21-22; read by graphs::read_weighted_binaries
// (files, 4, 1), benchmarks/mst_benchmarks.hpp:185-190): a possibly unsorted
// edge list of 9-byte records -- 4-byte source, 4-byte destination, 1-byte
// weight, little endian -- over one or more files.
//
// Pipeline: the files are read in 36 MB pieces into two pinned staging
// buffers while the previous piece is copied to the device (read and copy
// overlap); on the device the 9-byte records are unpacked into 64-bit keys
// ((src << b | dst) << 8 | w), optionally with every reverse record added,
// radix sorted, and compacted: self loops are dropped and of each (src, dst)
// run only the first -- the lightest -- entry is kept.  The result is sorted
// by (src, dst), duplicate free and, when symmetrised, holds both directions.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "solver.cuh"
#include "sort_gen.cuh"

namespace kamsta {

namespace {

constexpr uint64_t kPieceRecords = 4ull << 20;  // 36 MB per staged piece
constexpr uint32_t kLoadSym = 0x1u;

__global__ void k_bin_maxid(const uint8_t* __restrict__ raw, uint64_t R, uint32_t* out) {
  uint32_t mx = 0;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < R;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint8_t* p = raw + 9 * i;
    const uint32_t s = p[0] | (p[1] << 8) | (p[2] << 16) | (uint32_t(p[3]) << 24);
    const uint32_t d = p[4] | (p[5] << 8) | (p[6] << 16) | (uint32_t(p[7]) << 24);
    mx = max(mx, max(s, d));
  }
  mx = __reduce_max_sync(kFull, mx);
  if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

__global__ void k_bin_keys(const uint8_t* __restrict__ raw, uint64_t R, uint32_t b, int sym,
                           uint64_t* __restrict__ keys) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < R;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint8_t* p = raw + 9 * i;
    const uint64_t s = p[0] | (p[1] << 8) | (p[2] << 16) | (uint64_t(p[3]) << 24);
    const uint64_t d = p[4] | (p[5] << 8) | (p[6] << 16) | (uint64_t(p[7]) << 24);
    const uint64_t w = p[8];
    keys[i] = (((s << b) | d) << 8) | w;
    if (sym) keys[R + i] = (((d << b) | s) << 8) | w;
  }
}

// keep[j] = 1 for the first entry of each (src, dst) run that is not a loop
__global__ void k_bin_keep(const uint64_t* __restrict__ keys, uint64_t K, uint32_t b,
                           uint32_t* __restrict__ keep) {
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < K;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[j] >> 8;
    const bool loop = (k >> b) == (k & mask);
    keep[j] = (!loop && (j == 0 || (keys[j - 1] >> 8) != k)) ? 1u : 0u;
  }
}

__global__ void k_bin_write(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ keep,
                            const uint32_t* __restrict__ pos, uint64_t K, uint32_t b,
                            uint32_t* __restrict__ out) {
  const uint64_t mask = (1ull << b) - 1;
  for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < K;
       j += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    if (!keep[j]) continue;
    const uint64_t k = keys[j];
    const uint64_t o = pos[j];
    out[3 * o] = static_cast<uint32_t>((k >> 8) >> b);
    out[3 * o + 1] = static_cast<uint32_t>((k >> 8) & mask);
    out[3 * o + 2] = static_cast<uint32_t>(k & 255u);
  }
}

struct PoolMem {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~PoolMem() { reset(); }
  void reset() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
  }
  cudaError_t alloc(kamsta_ctx* ctx, cudaStream_t s, size_t bytes) {
    st = s;
    return ctx_alloc(ctx, &p, std::max<size_t>(bytes, 256), s);
  }
};

struct Pinned {  // staging buffer; waits for copies out of it before freeing
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~Pinned() {
    if (p) {
      cudaStreamSynchronize(st);
      cudaFreeHost(p);
    }
  }
};

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

#define LB_TRY(x)                                         \
  do {                                                    \
    const cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return cuda_status(e_, #x);    \
  } while (0)

kamsta_status file_records(const char* path, uint64_t* records) {
  File f;
  f.f = fopen(path, "rb");
  if (!f.f) {
    set_error(std::string("cannot open ") + path);
    return KAMSTA_E_INPUT;
  }
  if (fseeko(f.f, 0, SEEK_END) != 0) {
    set_error(std::string("cannot seek ") + path);
    return KAMSTA_E_INPUT;
  }
  const off_t sz = ftello(f.f);
  if (sz < 0 || sz % 9 != 0) {
    set_error(std::string(path) + ": size is not a multiple of 9 bytes");
    return KAMSTA_E_INPUT;
  }
  *records = static_cast<uint64_t>(sz) / 9;
  return KAMSTA_OK;
}

}  // namespace

kamsta_status wedge9_capacity(const char* const* paths, uint32_t num, uint32_t flags,
                              uint64_t* cap) {
  uint64_t total = 0;
  for (uint32_t i = 0; i < num; ++i) {
    uint64_t r = 0;
    const kamsta_status s = file_records(paths[i], &r);
    if (s != KAMSTA_OK) return s;
    total += r;
  }
  *cap = (flags & kLoadSym) ? 2 * total : total;
  return KAMSTA_OK;
}

kamsta_status load_wedge9(kamsta_ctx* ctx, const char* const* paths, uint32_t num, uint32_t flags,
                          kamsta_wedge* d_out, uint64_t capacity, uint64_t* m_out, uint32_t* n_out,
                          cudaStream_t st) {
  *m_out = 0;
  *n_out = 0;
  uint64_t R = 0;
  std::vector<uint64_t> recs(num);
  for (uint32_t i = 0; i < num; ++i) {
    const kamsta_status s = file_records(paths[i], &recs[i]);
    if (s != KAMSTA_OK) return s;
    R += recs[i];
  }
  if (R == 0) return KAMSTA_OK;
  const int sym = (flags & kLoadSym) ? 1 : 0;
  const uint64_t K = sym ? 2 * R : R;
  if (K >= (1ull << 32) - 8192) {
    set_error("load_wedge9: more than 2^32 directed entries");
    return KAMSTA_E_UNSUPPORTED;
  }
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8;
  // ---- stream the files: read piece i+1 while piece i is copied
  PoolMem raw;
  LB_TRY(raw.alloc(ctx, st, 9 * R));
  Pinned stage[2];
  cudaEvent_t done[2] = {nullptr, nullptr};
  stage[0].st = stage[1].st = st;
  LB_TRY(cudaMallocHost(&stage[0].p, 9 * kPieceRecords));
  LB_TRY(cudaMallocHost(&stage[1].p, 9 * kPieceRecords));
  LB_TRY(cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming));
  LB_TRY(cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming));
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      cudaEventDestroy(e[0]);
      cudaEventDestroy(e[1]);
    }
  } eg{done};
  uint64_t dst_off = 0;
  int slot = 0;
  bool used[2] = {false, false};
  for (uint32_t fi = 0; fi < num; ++fi) {
    File f;
    f.f = fopen(paths[fi], "rb");
    if (!f.f) {
      set_error(std::string("cannot open ") + paths[fi]);
      return KAMSTA_E_INPUT;
    }
    uint64_t left = recs[fi];
    while (left > 0) {
      const uint64_t take = std::min(left, kPieceRecords);
      if (used[slot]) LB_TRY(cudaEventSynchronize(done[slot]));  // staging buffer free again
      if (fread(stage[slot].p, 9, take, f.f) != take) {
        set_error(std::string("short read from ") + paths[fi]);
        return KAMSTA_E_INPUT;
      }
      LB_TRY(cudaMemcpyAsync(static_cast<uint8_t*>(raw.p) + 9 * dst_off, stage[slot].p, 9 * take,
                             cudaMemcpyHostToDevice, st));
      LB_TRY(cudaEventRecord(done[slot], st));
      used[slot] = true;
      slot ^= 1;
      dst_off += take;
      left -= take;
    }
  }
  // ---- id range -> key width
  PoolMem small;
  LB_TRY(small.alloc(ctx, st, 64));
  uint32_t* d_max = static_cast<uint32_t*>(small.p);
  uint32_t* ticket = d_max + 1;
  uint32_t* err = d_max + 2;
  LB_TRY(cudaMemsetAsync(small.p, 0, 64, st));
  k_bin_maxid<<<grid, 256, 0, st>>>(static_cast<const uint8_t*>(raw.p), R, d_max);
  uint32_t maxid = 0;
  LB_TRY(cudaMemcpyAsync(&maxid, d_max, sizeof(maxid), cudaMemcpyDeviceToHost, st));
  LB_TRY(cudaStreamSynchronize(st));
  if (maxid == 0xffffffffu) {
    set_error("load_wedge9: vertex id 2^32-1 is reserved");
    return KAMSTA_E_INPUT;
  }
  const uint64_t n = static_cast<uint64_t>(maxid) + 1;
  uint32_t b = 1;
  while (b < 32 && (1ull << b) < n) ++b;
  if (2 * b + 8 > 64) {
    set_error("load_wedge9: more than 2^28 vertices are not supported");
    return KAMSTA_E_UNSUPPORTED;
  }
  // ---- keys, sort, keep the lightest of each (src, dst), drop loops
  PoolMem kb, kb2, cnt, stat, keep, pos;
  LB_TRY(kb.alloc(ctx, st, 8 * K));
  LB_TRY(kb2.alloc(ctx, st, 8 * K));
  uint64_t* keys = static_cast<uint64_t*>(kb.p);
  uint64_t* keys2 = static_cast<uint64_t*>(kb2.p);
  k_bin_keys<<<grid, 256, 0, st>>>(static_cast<const uint8_t*>(raw.p), R, b, sym, keys);
  raw.reset();
  const RadixScratch rs = radix_scratch_bytes(K);
  LB_TRY(cnt.alloc(ctx, st, 4 * std::max<uint64_t>(rs.counts, K)));
  LB_TRY(stat.alloc(ctx, st, 8 * std::max<uint64_t>(rs.status, K / 2048 + 2)));
  int alt = 0;
  LB_TRY(radix_sort_keys(st, keys, keys2, K, static_cast<int>(2 * b + 8),
                         static_cast<uint32_t*>(cnt.p), static_cast<uint64_t*>(stat.p), ticket,
                         err, &alt, sms));
  if (alt) std::swap(keys, keys2);
  LB_TRY(keep.alloc(ctx, st, 4 * K));
  LB_TRY(pos.alloc(ctx, st, 4 * K));
  k_bin_keep<<<grid, 256, 0, st>>>(keys, K, b, static_cast<uint32_t*>(keep.p));
  LB_TRY(exclusive_scan_u32(st, static_cast<uint32_t*>(keep.p), static_cast<uint32_t*>(pos.p), K,
                            static_cast<uint64_t*>(stat.p), ticket, err, sms));
  uint32_t last_pos = 0, last_keep = 0, herr = 0;
  LB_TRY(cudaMemcpyAsync(&last_pos, static_cast<uint32_t*>(pos.p) + (K - 1), 4,
                         cudaMemcpyDeviceToHost, st));
  LB_TRY(cudaMemcpyAsync(&last_keep, static_cast<uint32_t*>(keep.p) + (K - 1), 4,
                         cudaMemcpyDeviceToHost, st));
  LB_TRY(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
  LB_TRY(cudaStreamSynchronize(st));
  if (herr) {
    set_error("load_wedge9: device wait cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  const uint64_t m = static_cast<uint64_t>(last_pos) + last_keep;
  *m_out = m;
  *n_out = static_cast<uint32_t>(n);
  if (!d_out) return KAMSTA_OK;
  if (m > capacity) {
    set_error("load_wedge9: output capacity too small (required count in m_directed_out)");
    return KAMSTA_E_INPUT;
  }
  k_bin_write<<<grid, 256, 0, st>>>(keys, static_cast<uint32_t*>(keep.p),
                                    static_cast<uint32_t*>(pos.p), K, b,
                                    reinterpret_cast<uint32_t*>(d_out));
  LB_TRY(cudaGetLastError());
  LB_TRY(cudaStreamSynchronize(st));
  return KAMSTA_OK;
}

}  // namespace kamsta

extern "C" kamsta_status kamsta_wedge9_capacity(const char* const* paths, uint32_t num_paths,
                                                uint32_t flags, uint64_t* capacity) {
  if (!capacity || (num_paths && !paths)) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return kamsta::wedge9_capacity(paths, num_paths, flags, capacity);
}

extern "C" kamsta_status kamsta_load_wedge9_dev(kamsta_ctx* ctx, const char* const* paths,
                                                uint32_t num_paths, uint32_t flags,
                                                kamsta_wedge* d_out, uint64_t capacity,
                                                uint64_t* m_directed_out, uint32_t* n_out,
                                                kamsta_stream stream) {
  if (!ctx || !m_directed_out || !n_out || (num_paths && !paths)) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return kamsta::load_wedge9(ctx, paths, num_paths, flags, d_out, capacity, m_directed_out, n_out,
                             st);
}
