// gen_scratch.cuh -- scratch buffers of the device graph generators.
//
// Stream-ordered allocations from the context's pool when the generator runs
// with a context, plain cudaMalloc otherwise; freed when the buffer goes out
// of scope (stream ordered as well).
#pragma once
#include <algorithm>

#include "solver.cuh"

namespace kamsta {

struct GenBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  cudaMemPool_t pool = nullptr;
  GenBuf() = default;
  GenBuf(const GenBuf&) = delete;
  GenBuf& operator=(const GenBuf&) = delete;
  ~GenBuf() { reset(); }
  void reset() {
    if (p) {
      if (pool) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
    p = nullptr;
  }
  template <typename T>
  cudaError_t alloc(kamsta_ctx* ctx, cudaStream_t s, T** out, uint64_t count) {
    reset();
    st = s;
    pool = ctx ? ctx->pool : nullptr;
    const size_t bytes = std::max<uint64_t>(count, 1) * sizeof(T);
    cudaError_t e = ctx ? ctx_alloc(ctx, &p, bytes, s) : cudaMalloc(&p, bytes);
    *out = static_cast<T*>(p);
    return e;
  }
};

#define GEN_CHECK(x)                                      \
  do {                                                    \
    const cudaError_t e_ = (x);                           \
    if (e_ != cudaSuccess) return cuda_status(e_, #x);    \
  } while (0)

}  // namespace kamsta
