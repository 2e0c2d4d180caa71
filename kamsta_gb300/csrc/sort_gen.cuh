// sort_gen.cuh -- radix sort entry points and the device graph generators.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/kamsta_gpu.h"

namespace kamsta {

// Scratch element counts of one radix sort of n keys: `counts` u32 words and
// `status` u64 words.
struct RadixScratch {
  uint64_t counts = 0;
  uint64_t status = 0;
};
RadixScratch radix_scratch_bytes(uint64_t n);

// Stable LSD radix sorts over the low `bits` bits of 64-bit keys (n < 2^32 -
// 4096).  The result is in the *_alt buffers when *result_alt == 1.
cudaError_t radix_sort_keys(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt, uint64_t n,
                            int bits, uint32_t* counts, uint64_t* status, uint32_t* ticket,
                            uint32_t* err, int* result_alt, int sms);
cudaError_t radix_sort_pairs_u32(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt,
                                 uint32_t* vals, uint32_t* vals_alt, uint64_t n, int bits,
                                 uint32_t* counts, uint64_t* status, uint32_t* ticket,
                                 uint32_t* err, int* result_alt, int sms);
cudaError_t radix_sort_pairs_u64(cudaStream_t st, uint64_t* keys, uint64_t* keys_alt,
                                 uint64_t* vals, uint64_t* vals_alt, uint64_t n, int bits,
                                 uint32_t* counts, uint64_t* status, uint32_t* ticket,
                                 uint32_t* err, int* result_alt, int sms);

// Exclusive prefix sum of n u32 values (single pass, decoupled look-back);
// `status` needs ceil(n / 2048) + 1 words.  Sum of n u32 values into *out
// (added to its current value).
cudaError_t exclusive_scan_u32(cudaStream_t st, const uint32_t* in, uint32_t* out, uint64_t n,
                               uint64_t* status, uint32_t* ticket, uint32_t* err, int sms);
cudaError_t sum_u32(cudaStream_t st, const uint32_t* v, uint64_t n, unsigned long long* out,
                    int sms);

kamsta_status gen_gnm(kamsta_ctx* ctx, uint32_t n, uint64_t m, uint64_t seed,
                      uint32_t max_weight, kamsta_wedge* d_out, uint64_t* m_out,
                      cudaStream_t st);

kamsta_status gen_rgg2d(kamsta_ctx* ctx, uint32_t n, double radius, uint64_t seed,
                        uint32_t max_weight, uint32_t distance, kamsta_wedge* d_out,
                        uint64_t capacity, uint64_t* m_out, cudaStream_t st);
kamsta_status gen_rhg(kamsta_ctx* ctx, uint32_t n, double gamma, double avg_degree, uint64_t seed,
                      uint32_t max_weight, kamsta_wedge* d_out, uint64_t capacity,
                      uint64_t* m_out, cudaStream_t st);

struct GenBuf;
// Distinct undirected pairs -> the solver's input: bk holds K keys (min id
// << L | max id, or (1 << 2L) - 1 for "no pair") in device memory, in any
// order.  Writes both directions of every distinct pair, (src, dst)-sorted,
// with the generators' weight 1 + hi64(mix64(wseed ^ (min << 32 | max)) *
// max_weight).  Counting / capacity convention of the generators; `name`
// prefixes error messages.  bk may be swapped with scratch (it stays owned).
kamsta_status pairs_to_edges(kamsta_ctx* ctx, cudaStream_t st, GenBuf& bk, uint64_t K, uint32_t L,
                             uint64_t wseed, uint32_t max_weight, const char* name,
                             kamsta_wedge* d_out, uint64_t capacity, uint64_t* m_out);

}  // namespace kamsta
