// noalloc.cu -- minimum spanning forest of a small graph without allocating.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's fixed memory budget, an allocator-less runtime, or a plugin
// that is handed a stream and buffers and must not touch the device heap.
// kamsta_mst_boruvka_noalloc serves them: it runs the Boruvka rounds of
// kamsta_mst_boruvka_dev (hook, pointer jumping, renumbering, relabel +
// self-loop removal + stable compaction) fused into one single-CTA kernel,
// and every scratch byte it needs lives in the file-scope array below.
//
// Limits: n <= kNoallocMaxN vertices and m_directed <= kNoallocMaxMd input
// entries.  The array (about 5 MB) is part of the library image, so every
// GPU that loads the library holds it until the process exits.  All calls
// share it and it keeps the last call's contents; the kernel clears what must
// start at zero or infinity.  Calls that overlap on the GPU (two streams,
// two threads) race on the array and must be serialised by the caller.
#include <mutex>
#include <string>

#include "../../include/kamsta_gpu.h"
#include "common.cuh"

namespace kamsta {
namespace noalloc {

constexpr uint32_t kMaxN = 1u << 15;
constexpr uint64_t kMaxMd = 1ull << 18;
constexpr uint32_t kMaxMu = static_cast<uint32_t>(kMaxMd / 2);  // src<dst copies
constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kMaxRoundsNa = 40;

// Scratch layout (bytes, 256-aligned).
constexpr size_t kHdr = 256;                         // NaResult
constexpr size_t kListBytes = size_t(kMaxMu) * sizeof(Rec);
constexpr size_t kOffL0 = kHdr;
constexpr size_t kOffL1 = kOffL0 + kListBytes;
constexpr size_t kOffMin0 = kOffL1 + kListBytes;
constexpr size_t kOffMin1 = kOffMin0 + size_t(kMaxN) * 8;
constexpr size_t kOffParent = kOffMin1 + size_t(kMaxN) * 8;
constexpr size_t kOffMsfoid = kOffParent + size_t(kMaxN) * 4;
constexpr size_t kOffNewid = kOffMsfoid + size_t(kMaxN) * 4;
constexpr size_t kOffR = kOffNewid + size_t(kMaxN) * 4;
constexpr size_t kOffMsf = kOffR + size_t(kMaxN) * 4;
constexpr size_t kScratchBytes = kOffMsf + size_t(kMaxN) * 4;

struct NaResult {
  unsigned long long count;
  unsigned long long weight;
  uint32_t err;
  uint32_t rounds;
};

}  // namespace noalloc
}  // namespace kamsta

// The scratch array.  Host code sees only a host-side stand-in for this
// symbol; the device address comes from cudaGetSymbolAddress (see below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kamsta::noalloc::kScratchBytes];

namespace kamsta {
namespace noalloc {

// Stable block-wide ranks of this thread's item for two flags (one item per
// thread, items in thread order): r = rank among the block's items with
// the same flag, t = block totals.
__device__ __forceinline__ void block_rank2(bool f0, bool f1, uint32_t& r0, uint32_t& r1,
                                            uint32_t& t0, uint32_t& t1, uint32_t* s_w) {
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, lt = lanemask_lt();
  const uint32_t b0 = __ballot_sync(kFull, f0), b1 = __ballot_sync(kFull, f1);
  if (lane == 0) {
    s_w[warp] = __popc(b0);
    s_w[kWarps + warp] = __popc(b1);
  }
  __syncthreads();
  uint32_t p0 = 0, p1 = 0, a0 = 0, a1 = 0;
#pragma unroll 8
  for (int w = 0; w < kWarps; ++w) {
    const uint32_t x0 = s_w[w], x1 = s_w[kWarps + w];
    if (static_cast<uint32_t>(w) < warp) {
      p0 += x0;
      p1 += x1;
    }
    a0 += x0;
    a1 += x1;
  }
  __syncthreads();
  r0 = p0 + __popc(b0 & lt);
  r1 = p1 + __popc(b1 & lt);
  t0 = a0;
  t1 = a1;
}

// The whole solve in one CTA: first pass (src<dst copies, fused round-0
// minimum), then Boruvka rounds until no edge is left, then the forest
// output.  Same tie-break as the multi-kernel solver: lists stay in input
// order, so (w << 32 | position) orders edges by (w, min, max).
__global__ void __launch_bounds__(kThreads, 1)
    k_noalloc_boruvka(const uint32_t* __restrict__ in, uint32_t md, uint32_t n,
                      unsigned char* __restrict__ scratch, uint32_t* __restrict__ out) {
  NaResult* res = reinterpret_cast<NaResult*>(scratch);
  Rec* L[2] = {reinterpret_cast<Rec*>(scratch + kOffL0), reinterpret_cast<Rec*>(scratch + kOffL1)};
  uint64_t* mv[2] = {reinterpret_cast<uint64_t*>(scratch + kOffMin0),
                     reinterpret_cast<uint64_t*>(scratch + kOffMin1)};
  uint32_t* parent = reinterpret_cast<uint32_t*>(scratch + kOffParent);
  uint32_t* msfoid = reinterpret_cast<uint32_t*>(scratch + kOffMsfoid);
  uint32_t* newid = reinterpret_cast<uint32_t*>(scratch + kOffNewid);
  uint32_t* R = reinterpret_cast<uint32_t*>(scratch + kOffR);
  uint32_t* msf = reinterpret_cast<uint32_t*>(scratch + kOffMsf);
  __shared__ uint32_t s_w[2 * kWarps];
  __shared__ uint32_t s_err;
  __shared__ unsigned long long s_weight;
  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
    s_err = 0;
    s_weight = 0;
  }
  for (uint32_t v = tid; v < n; v += kThreads) mv[0][v] = kInf64;
  __syncthreads();
  // first pass: keep the src<dst copies, in input order
  uint32_t m = 0;
  for (uint32_t base = 0; base < md; base += kThreads) {
    const uint32_t i = base + tid;
    uint32_t s = 0, d = 0, w = 0;
    bool keep = false;
    if (i < md) {
      s = in[3ull * i];
      d = in[3ull * i + 1];
      w = in[3ull * i + 2];
      keep = s < d && d < n;
    }
    uint32_t r0, r1, t0, t1;
    block_rank2(keep, false, r0, r1, t0, t1, s_w);
    if (keep) {
      const uint32_t pos = m + r0;
      if (pos < kMaxMu) {
        Rec x;
        x.a = s;
        x.b = d;
        x.w = w;
        x.oid = i;
        L[0][pos] = x;
        const uint64_t key = (static_cast<uint64_t>(w) << 32) | pos;
        atomicMin(reinterpret_cast<unsigned long long*>(&mv[0][s]), key);
        atomicMin(reinterpret_cast<unsigned long long*>(&mv[0][d]), key);
      } else {
        atomicOr(&s_err, kErrOverflow);
      }
    }
    m += t0;
  }
  __syncthreads();
  uint32_t nr = n, cur = 0, msf_count = 0, round = 0;
  while (m > 0) {
    if (s_err != 0) break;
    if (round >= kMaxRoundsNa) {
      if (tid == 0) s_err |= kErrChase;
      break;
    }
    const Rec* Lc = L[cur];
    Rec* Ln = L[cur ^ 1];
    const uint64_t* mc = mv[cur];
    uint64_t* mn = mv[cur ^ 1];
    // hook: along the minimum edge; of a mutual pair the lower label stays root
    for (uint32_t v = tid; v < nr; v += kThreads) {
      const uint64_t val = mc[v];
      uint32_t par = v, eid = kNone;
      if (val != kInf64) {
        const Rec x = Lc[static_cast<uint32_t>(val)];
        if (x.a != v && x.b != v) {
          atomicOr(&s_err, kErrHook);
        } else {
          const uint32_t u = x.a ^ x.b ^ v;
          if (!(mc[u] == val && v < u)) {
            par = u;
            eid = x.oid;
          }
        }
      }
      parent[v] = par;
      msfoid[v] = eid;
    }
    __syncthreads();
    // pointer jumping with path halving, then a read-only pass that fixes
    // pointers another thread's halving left one level short
    for (uint32_t v = tid; v < nr; v += kThreads) {
      uint32_t x = v, p = ld_relaxed(parent + x), steps = 0;
      if (p == x) continue;
      for (;;) {
        const uint32_t gp = ld_relaxed(parent + p);
        if (gp == p) break;
        st_relaxed(parent + x, gp);
        x = gp;
        p = ld_relaxed(parent + x);
        if (++steps > 2 * kMaxN) {
          atomicOr(&s_err, kErrJump);
          break;
        }
      }
    }
    __syncthreads();
    for (uint32_t v = tid; v < nr; v += kThreads) {
      uint32_t p = ld_relaxed(parent + v), steps = 0;
      if (p == v) continue;
      for (;;) {
        const uint32_t gp = ld_relaxed(parent + p);
        if (gp == p || ++steps > 2 * kMaxN) break;
        p = gp;
      }
      st_relaxed(parent + v, p);
    }
    __syncthreads();
    if (s_err != 0) break;
    // renumber live roots, append the forest edges of hooked vertices
    uint32_t n_next = 0;
    for (uint32_t vb = 0; vb < nr; vb += kThreads) {
      const uint32_t v = vb + tid;
      uint32_t c = 2;
      if (v < nr) {
        if (parent[v] != v)
          c = 1;
        else if (mc[v] != kInf64)
          c = 0;
      }
      uint32_t r0, r1, t0, t1;
      block_rank2(c == 0, c == 1, r0, r1, t0, t1, s_w);
      if (c == 0) {
        newid[v] = n_next + r0;
        mn[n_next + r0] = kInf64;
      } else if (c == 1) {
        if (msf_count + r1 < kMaxN)
          msf[msf_count + r1] = msfoid[v];
        else
          atomicOr(&s_err, kErrOverflow);
      }
      n_next += t0;
      msf_count += t1;
    }
    __syncthreads();
    for (uint32_t v = tid; v < nr; v += kThreads)
      R[v] = (mc[v] == kInf64 && parent[v] == v) ? kNone : newid[parent[v]];
    __syncthreads();
    // relabel, drop self loops, compact (stable), feed the next minimum
    uint32_t m_next = 0;
    for (uint32_t eb = 0; eb < m; eb += kThreads) {
      const uint32_t e = eb + tid;
      bool keep = false;
      Rec x;
      uint32_t a = 0, b = 0;
      if (e < m) {
        x = Lc[e];
        a = R[x.a];
        b = R[x.b];
        keep = a != b;
      }
      uint32_t r0, r1, t0, t1;
      block_rank2(keep, false, r0, r1, t0, t1, s_w);
      if (keep) {
        const uint32_t pos = m_next + r0;
        Rec y;
        y.a = a;
        y.b = b;
        y.w = x.w;
        y.oid = x.oid;
        Ln[pos] = y;
        const uint64_t key = (static_cast<uint64_t>(x.w) << 32) | pos;
        atomicMin(reinterpret_cast<unsigned long long*>(&mn[a]), key);
        atomicMin(reinterpret_cast<unsigned long long*>(&mn[b]), key);
      }
      m_next += t0;
    }
    __syncthreads();
    m = m_next;
    nr = n_next;
    cur ^= 1;
    ++round;
  }
  __syncthreads();
  // forest output: the src<dst input copy of every forest edge
  unsigned long long local = 0;
  if (s_err == 0) {
    for (uint32_t k = tid; k < msf_count; k += kThreads) {
      const uint64_t o = 3ull * msf[k];
      const uint32_t s = in[o], d = in[o + 1], w = in[o + 2];
      out[3ull * k] = s;
      out[3ull * k + 1] = d;
      out[3ull * k + 2] = w;
      local += w;
    }
  }
  local = warp_sum(local);
  if (lane_id() == 0 && local) atomicAdd(&s_weight, local);
  __syncthreads();
  if (tid == 0) {
    res->count = s_err == 0 ? msf_count : 0;
    res->weight = s_weight;
    res->err = s_err;
    res->rounds = round;
  }
}

}  // namespace noalloc
}  // namespace kamsta

namespace kamsta {
void set_error(const std::string& msg);
kamsta_status cuda_status(cudaError_t e, const char* what);
}  // namespace kamsta

namespace {

// Device address of g_noalloc_scratch per device, looked up once per device
// (with that device current) on the first call made there.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

kamsta_status scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return kamsta::cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    kamsta::set_error("kamsta_mst_boruvka_noalloc: device ordinal out of range");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return kamsta::cuda_status(e, "cudaGetSymbolAddress(scratch)");
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  return KAMSTA_OK;
}

}  // namespace

extern "C" kamsta_status kamsta_mst_boruvka_noalloc(const kamsta_wedge* d_edges,
                                                    uint64_t m_directed, uint32_t n,
                                                    kamsta_wedge* d_out, uint64_t* out_count,
                                                    uint64_t* total_weight,
                                                    kamsta_stream stream) {
  using namespace kamsta::noalloc;
  if (!out_count || (m_directed && !d_edges) || (n > 1 && !d_out)) {
    kamsta::set_error("kamsta_mst_boruvka_noalloc: null pointer argument");
    return KAMSTA_E_INPUT;
  }
  *out_count = 0;
  if (total_weight) *total_weight = 0;
  if (n > kMaxN || m_directed > kMaxMd) {
    kamsta::set_error("kamsta_mst_boruvka_noalloc: graph exceeds the fixed scratch limits "
                      "(n <= 32768 vertices, m_directed <= 262144 entries)");
    return KAMSTA_E_INPUT;
  }
  if (n == 0 || m_directed == 0) return KAMSTA_OK;
  unsigned char* scratch = nullptr;
  kamsta_status s = scratch_for_current_device(&scratch);
  if (s != KAMSTA_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_noalloc_boruvka<<<1, kThreads, 0, st>>>(reinterpret_cast<const uint32_t*>(d_edges),
                                            static_cast<uint32_t>(m_directed), n, scratch,
                                            reinterpret_cast<uint32_t*>(d_out));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return kamsta::cuda_status(e, "k_noalloc_boruvka launch");
  NaResult h{};
  e = cudaMemcpyAsync(&h, scratch, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return kamsta::cuda_status(e, "kamsta_mst_boruvka_noalloc result");
  if (h.err) {
    kamsta::set_error("kamsta_mst_boruvka_noalloc: device check failed (code " +
                      std::to_string(h.err) + ")");
    return (h.err & kamsta::kErrJump) ? KAMSTA_E_NOCONVERGE : KAMSTA_E_INPUT;
  }
  *out_count = h.count;
  if (total_weight) *total_weight = h.weight;
  return KAMSTA_OK;
}
