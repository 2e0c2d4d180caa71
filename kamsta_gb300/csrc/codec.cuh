// codec.cuh -- 7-bit varint difference encoding (host encoder, device decoder).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/kamsta_gpu.h"

namespace kamsta {

constexpr uint32_t kMaxChunkEdges = 4096;  // edges per chunk at most

kamsta_status encode_7bit(const kamsta_wedge* e, uint64_t m, uint32_t chunk_edges, uint64_t* off,
                          kamsta_wedge* first, uint8_t* data, uint64_t cap, uint64_t* bytes);
// Decodes g (device pointers) into d_out (m_directed entries); stream ordered.
kamsta_status decode_7bit(const kamsta_cgraph& g, kamsta_wedge* d_out, uint32_t* d_err,
                          cudaStream_t st);

}  // namespace kamsta
