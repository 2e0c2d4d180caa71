// noalloc.cu -- minimum spanning forest of a small graph without allocating.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's fixed memory budget, an allocator-less runtime, or a plugin
// that is handed a stream and buffers and must not touch the device heap.
// kamsta_mst_boruvka_noalloc serves them: it runs the Boruvka rounds of
// kamsta_mst_boruvka_dev (hook, pointer jumping, renumbering, relabel +
// self-loop removal + stable compaction) fused into one single-CTA kernel
// (small_solve.cuh), and every scratch byte it needs lives in the file-scope
// array below.
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
#include "small_solve.cuh"

namespace kamsta {
namespace noalloc {

constexpr uint32_t kMaxN = small::kMaxN;
constexpr uint64_t kMaxMd = small::kMaxMd;
constexpr int kThreads = 1024;
constexpr size_t kScratchBytes = small::kScratchBytes;
using NaResult = small::Result;

}  // namespace noalloc
}  // namespace kamsta

// The scratch array.  Host code sees only a host-side stand-in for this
// symbol; the device address comes from cudaGetSymbolAddress (see below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kamsta::noalloc::kScratchBytes];

namespace kamsta {
namespace noalloc {

// The whole solve in one CTA (small_solve.cuh), forest edges in the order
// the rounds find them; the result header sits at the start of the scratch.
// Ids are always checked against n (one compare per entry in the pass that
// reads them anyway), so an id >= n is reported instead of skipped.
__global__ void __launch_bounds__(kThreads, 1)
    k_noalloc_boruvka(const uint32_t* __restrict__ in, uint32_t md, uint32_t n,
                      unsigned char* __restrict__ scratch, uint32_t* __restrict__ out) {
  small::solve<kThreads, small::Out::kFound>(in, md, n, scratch, out,
                                             reinterpret_cast<NaResult*>(scratch), true);
}

}  // namespace noalloc
}  // namespace kamsta

namespace kamsta {
void set_error(const std::string& msg);
kamsta_status cuda_status(cudaError_t e, const char* what);
}  // namespace kamsta

namespace {

// Device address of g_noalloc_scratch per device, looked up once per device
// (with that device current) on the first call made there.  The address
// belongs to the device's primary context: after cudaDeviceReset the module
// may load elsewhere, so the library must not be used across a reset.
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
  if (h.err & kamsta::kErrRange) {
    kamsta::set_error("kamsta_mst_boruvka_noalloc: input: vertex id >= n");
    return KAMSTA_E_INPUT;
  }
  if (h.err) {
    kamsta::set_error("kamsta_mst_boruvka_noalloc: device check failed (code " +
                      std::to_string(h.err) + ")");
    return (h.err & kamsta::kErrJump) ? KAMSTA_E_NOCONVERGE : KAMSTA_E_INPUT;
  }
  *out_count = h.count;
  if (total_weight) *total_weight = h.weight;
  return KAMSTA_OK;
}
