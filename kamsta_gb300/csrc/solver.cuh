// solver.cuh -- host-side driver of the GB300 MSF solver (C++ over CUDA).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/kamsta_gpu.h"
#include "common.cuh"

namespace kamsta {

// Grow-only device arena.  A solve carves its buffers from it; the memory
// stays with the context between calls (the reference's analogue is the
// per-call std::vector scratch of boruvka3, re-created every call).
struct Arena {
  char* base = nullptr;
  size_t cap = 0;
  size_t off = 0;
  cudaError_t reserve(size_t bytes);
  void release();
  void reset() { off = 0; }
  template <typename T>
  T* take(size_t count) {
    const size_t bytes = (count * sizeof(T) + 255) & ~static_cast<size_t>(255);
    if (off + bytes > cap) return nullptr;
    T* p = reinterpret_cast<T*>(base + off);
    off += bytes;
    return p;
  }
};

// Per-kernel counter block in device memory (zeroed before each round).
struct DevCounters {
  unsigned long long cnt[8];
  unsigned long long weight;
  uint32_t ticket;
  uint32_t err;
  uint32_t pad[12];
};
static_assert(sizeof(DevCounters) == 128, "counter block size");

enum CounterSlot : int { kCVertex = 0, kCEdge = 1, kCRep = 2, kCMisc = 3, kCSlots = 4 };
constexpr uint32_t kSampleCap = 4096;
constexpr int kTimerEvents = 64;
constexpr int kInputPieces = 16;  // host input copied in this many pieces

}  // namespace kamsta

struct kamsta_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;    // second stream: small graphs of a batch wave
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // batch tuning (kamsta_batch_autotune); 0 = built-in default
  uint32_t tune_small_threads = 0;  // CTA size of the persistent small-graph kernel
  uint32_t tune_small_max_n = 0;    // largest n taken by that kernel
  // single-graph tiles (kamsta_autotune_tiles); 0 = built-in default
  uint32_t tune_dir_items = 0;      // entries per thread of the first pass
  uint32_t tune_seg_items = 0;      // records per thread of the list passes
  kamsta::Arena fixed;   // vertex arrays and look-back words
  cudaMemPool_t pool = nullptr;  // edge lists (stream-ordered, cached between calls)
  kamsta::DevCounters* d_counters = nullptr;  // kCSlots blocks
  uint32_t* d_samples = nullptr;               // weight samples (kSampleCap)
  uint32_t* d_err = nullptr;
  kamsta::DevCounters* h_counters = nullptr;  // pinned mirror
  uint32_t* h_err = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t tev[kamsta::kTimerEvents] = {};  // per-phase timing events
  kamsta::Arena io;      // host-buffer entry points: device copies of in/out
  cudaEvent_t piece_ev[kamsta::kInputPieces] = {};  // host input piece k is on the device
  cudaEvent_t ev_early = nullptr;  // the first round's forest edges are written
  uint64_t mem_limit = 0;          // kamsta_ctx_set_memory_limit; 0 = none
  std::mutex mu;
};

namespace kamsta {

struct SolveOut {
  uint64_t count = 0;
  uint64_t weight = 0;
};

// Which reference entry point a call mirrors.
enum class Algo { kBoruvka, kFilterBoruvka };

// The host-buffer entry point overlaps its copies with the solve.  The input
// arrives in pieces on copy_stream: entries [0, piece_end[k]) are on the
// device once piece_ev[k] has completed (the events are recorded in order).
// The first pass starts on each chunk as soon as it has landed, and the
// weight sample of the class plan is drawn from the first piece.  When
// host_out is set, the forest edges that the first round writes directly
// are copied back to host_out[0, early) on copy_stream while the rest of the
// solve runs.
struct HostIo {
  int pieces = 0;
  uint64_t piece_end[kInputPieces] = {};
  const cudaEvent_t* piece_ev = nullptr;
  cudaStream_t copy_stream = nullptr;
  kamsta_wedge* host_out = nullptr;
  cudaEvent_t ev_early = nullptr;
  uint64_t early = 0;  // out
};

// Solves one graph whose directed, (src,dst)-sorted input lies in device
// memory.  Writes the forest to d_out (device, capacity >= n-1), or, when
// d_forest_bits is given (zeroed, one bit per input entry), sets the bit of
// the src<dst input copy of every forest edge instead (out->weight is then
// 0: the caller reads the marked entries).
kamsta_status solve_device(kamsta_ctx* ctx, Algo algo, const kamsta_wedge* d_in,
                           uint64_t m_directed, uint32_t n, const kamsta_cfg& cfg,
                           kamsta_wedge* d_out, SolveOut* out, kamsta_stats* st,
                           cudaStream_t stream, uint32_t* d_forest_bits = nullptr,
                           HostIo* io = nullptr);

void set_error(const std::string& msg);
kamsta_status cuda_status(cudaError_t e, const char* what);
// Device memory of a context under its limit (mem_limit): stream-ordered
// scratch from its pool and the growth of its arenas.  Going over the limit
// fails like a device allocation (cudaErrorMemoryAllocation -> KAMSTA_E_OOM).
uint64_t ctx_device_bytes(const kamsta_ctx* ctx);
cudaError_t ctx_alloc(kamsta_ctx* ctx, void** p, size_t bytes, cudaStream_t st);
cudaError_t ctx_reserve(kamsta_ctx* ctx, Arena& a, size_t bytes);

}  // namespace kamsta
