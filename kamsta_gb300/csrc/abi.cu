// abi.cu -- extern "C" entry points declared in include/kamsta_gpu.h.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "batch.cuh"
#include "codec.cuh"
#include "solver.cuh"

namespace kamsta {
const char* last_error_cstr();

namespace {

kamsta_status check_cfg(const kamsta_cfg* cfg) {
  if (!cfg) return KAMSTA_OK;
  if (cfg->compression != KAMSTA_NO_COMPRESSION &&
      cfg->compression != KAMSTA_SEVEN_BIT_DIFF_ENCODING) {
    set_error("compression: unknown value");
    return KAMSTA_E_INPUT;
  }
  if (cfg->items_per_thread != 0 && cfg->items_per_thread != 6 && cfg->items_per_thread != 8 &&
      cfg->items_per_thread != 12) {
    set_error("items_per_thread: 0, 6, 8 or 12");
    return KAMSTA_E_INPUT;
  }
  if (cfg->seg_items_per_thread != 0 && cfg->seg_items_per_thread != 2 &&
      cfg->seg_items_per_thread != 4 && cfg->seg_items_per_thread != 8) {
    set_error("seg_items_per_thread: 0, 2, 4 or 8");
    return KAMSTA_E_INPUT;
  }
  if (cfg->local_preprocessing < KAMSTA_NO_PREPROCESSING ||
      cfg->local_preprocessing > KAMSTA_REDUCE_EDGES_THEN_BORUVKA) {
    set_error("local_preprocessing: unknown value");
    return KAMSTA_E_INPUT;
  }
  return KAMSTA_OK;
}

kamsta_cfg cfg_or_default(const kamsta_cfg* cfg) {
  kamsta_cfg c;
  kamsta_cfg_default(&c);
  return cfg ? *cfg : c;
}

// Per-thread default context for the host-buffer entry points, one per
// device the thread has used.
struct DefaultCtx {
  std::vector<std::pair<int, kamsta_ctx*>> ctxs;
  ~DefaultCtx() {
    for (auto& p : ctxs) kamsta_ctx_destroy(p.second);
  }
  kamsta_status get(kamsta_ctx** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    for (auto& p : ctxs)
      if (p.first == dev) {
        *out = p.second;
        return KAMSTA_OK;
      }
    kamsta_ctx* c = nullptr;
    kamsta_status s = kamsta_ctx_create(dev, &c);
    if (s != KAMSTA_OK) return s;
    ctxs.emplace_back(dev, c);
    *out = c;
    return KAMSTA_OK;
  }
};
thread_local DefaultCtx g_default;

kamsta_status solve_host_7bit(Algo algo, const kamsta_wedge* edges, uint64_t m, uint32_t n,
                              kamsta_cfg c, kamsta_wedge* out, uint64_t* out_count,
                              kamsta_stats* stats);

// Host-to-device copy of a large input in pieces on the context's second
// stream, an event after each: the first pass's CTA groups wait only for the
// piece that holds their chunks (one stream is enough: the host link gives
// the same rate to one copy as to several).
kamsta_status solve_host(Algo algo, const kamsta_wedge* edges, uint64_t m, uint32_t n,
                         const kamsta_cfg* cfg, kamsta_wedge* out, uint64_t* out_count,
                         kamsta_stats* stats) {
  if (!out_count || (m && !edges) || (n > 1 && !out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  kamsta_status s = check_cfg(cfg);
  if (s != KAMSTA_OK) return s;
  kamsta_cfg c = cfg_or_default(cfg);
  if (c.compression == KAMSTA_SEVEN_BIT_DIFF_ENCODING)
    return solve_host_7bit(algo, edges, m, n, c, out, out_count, stats);
  kamsta_ctx* ctx = nullptr;
  s = g_default.get(&ctx);
  if (s != KAMSTA_OK) return s;
  std::lock_guard<std::mutex> lock(ctx->mu);
  *out_count = 0;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (m == 0 || n == 0) return KAMSTA_OK;
  // device copies of input and output live in the context's grow-only io pool
  const size_t in_bytes = (m * sizeof(kamsta_wedge) + 255) & ~size_t(255);
  const size_t out_bytes = std::max<uint64_t>(n, 1) * sizeof(kamsta_wedge);
  cudaError_t e = ctx_reserve(ctx, ctx->io, in_bytes + out_bytes + 256);
  if (e != cudaSuccess) return cuda_status(e, "device buffers for host input");
  kamsta_wedge* din = ctx->io.take<kamsta_wedge>(m);
  kamsta_wedge* dout = ctx->io.take<kamsta_wedge>(std::max<uint64_t>(n, 1));
  // the input in pieces on the aux stream, so the solve can start on the
  // first ones (the solve's stream waits for each piece's event)
  HostIo io;
  io.pieces = kInputPieces;
  io.piece_ev = ctx->piece_ev;
  io.copy_stream = ctx->aux;
  io.host_out = out;
  io.ev_early = ctx->ev_early;
  const uint64_t per = (m + kInputPieces - 1) / kInputPieces;
  for (int k = 0; k < kInputPieces; ++k) {
    const uint64_t b = std::min<uint64_t>(m, k * per), en = std::min<uint64_t>(m, b + per);
    io.piece_end[k] = en;
    if (en > b)
      e = cudaMemcpyAsync(din + b, edges + b, (en - b) * sizeof(kamsta_wedge),
                          cudaMemcpyHostToDevice, ctx->aux);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->piece_ev[k], ctx->aux);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(ctx->aux);  // no copy from the caller's memory outlives the call
      return cuda_status(e, "cudaMemcpyAsync(H2D)");
    }
  }
  SolveOut so;
  s = solve_device(ctx, algo, din, m, n, c, dout, &so, stats, ctx->stream, nullptr, &io);
  if (s != KAMSTA_OK) {
    cudaStreamSynchronize(ctx->aux);  // no copy may outlive the call
    return s;
  }
  // the edges not sent early (the first round's went out during the solve)
  if (so.count > io.early) {
    e = cudaMemcpyAsync(out + io.early, dout + io.early,
                        (so.count - io.early) * sizeof(kamsta_wedge), cudaMemcpyDeviceToHost,
                        ctx->stream);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(ctx->aux);
      return cuda_status(e, "cudaMemcpyAsync(D2H)");
    }
  }
  e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->aux);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
  if (c.flags & KAMSTA_FLAG_SORT_OUTPUT)
    std::sort(out, out + so.count, [](const kamsta_wedge& a, const kamsta_wedge& b) {
      return a.src != b.src ? a.src < b.src : a.dst < b.dst;
    });
  *out_count = so.count;
  return KAMSTA_OK;
}

kamsta_status solve_dev(Algo algo, kamsta_ctx* ctx, const kamsta_wedge* d_edges, uint64_t m,
                        uint32_t n, const kamsta_cfg* cfg, kamsta_wedge* d_out,
                        uint64_t* out_count, kamsta_stats* stats, kamsta_stream stream) {
  if (!ctx || !out_count || (m && !d_edges) || (n > 1 && !d_out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  kamsta_status s = check_cfg(cfg);
  if (s != KAMSTA_OK) return s;
  kamsta_cfg c = cfg_or_default(cfg);
  std::lock_guard<std::mutex> lock(ctx->mu);
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != ctx->device) {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  }
  SolveOut so;
  s = solve_device(ctx, algo, d_edges, m, n, c, d_out, &so, stats,
                   static_cast<cudaStream_t>(stream));
  if (cur != ctx->device) cudaSetDevice(cur);
  *out_count = so.count;
  return s;
}

// Decode a compressed graph (device pointers) into pool scratch and solve it.
kamsta_status solve_7bit_locked(kamsta_ctx* ctx, const kamsta_cgraph& g, kamsta_cfg c,
                                kamsta_wedge* d_out, uint64_t* out_count, kamsta_stats* stats,
                                cudaStream_t st, Algo algo = Algo::kBoruvka) {
  *out_count = 0;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (g.m_directed == 0 || g.n == 0) return KAMSTA_OK;
  void* buf = nullptr;
  cudaError_t e = ctx_alloc(ctx, &buf, g.m_directed * sizeof(kamsta_wedge), st);
  if (e != cudaSuccess) return cuda_status(e, "decode buffer");
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } fr{buf, st};
  e = cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_status(e, "cudaMemsetAsync");
  kamsta_status s = decode_7bit(g, static_cast<kamsta_wedge*>(buf), ctx->d_err, st);
  if (s != KAMSTA_OK) return s;
  e = cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "decode");
  if (*ctx->h_err) {
    set_error("decode_7bit: malformed chunk (value count or length)");
    return KAMSTA_E_INPUT;
  }
  c.compression = KAMSTA_NO_COMPRESSION;
  SolveOut so;
  s = solve_device(ctx, algo, static_cast<kamsta_wedge*>(buf), g.m_directed, g.n, c, d_out, &so,
                   stats, st);
  *out_count = so.count;
  return s;
}

kamsta_status check_cgraph(const kamsta_cgraph* g) {
  if (!g || (g->m_directed && (!g->chunk_offset || !g->chunk_first ||
                               (g->data_bytes && !g->data)))) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return KAMSTA_OK;
}

kamsta_status batch_call(kamsta_ctx* ctx, kamsta_graph_desc* graphs, uint32_t count,
                         const kamsta_cfg* cfg, uint64_t budget, kamsta_batch_stats* stats,
                         bool host_buffers, kamsta_stream stream) {
  if (count && !graphs) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  kamsta_status s = check_cfg(cfg);
  if (s != KAMSTA_OK) return s;
  kamsta_cfg c = cfg_or_default(cfg);
  if (!ctx) {
    s = g_default.get(&ctx);
    if (s != KAMSTA_OK) return s;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != ctx->device) {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  }
  const Algo algo = (c.flags & KAMSTA_FLAG_FILTER) ? Algo::kFilterBoruvka : Algo::kBoruvka;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  s = solve_batch(ctx, algo, graphs, count, c, budget, host_buffers, stats, st);
  if (cur != ctx->device) cudaSetDevice(cur);
  return s;
}

// A compressed graph in host memory: only the compressed bytes cross to the
// device, where they are decoded and solved (kamsta_mst_boruvka_7bit).
kamsta_status solve_cgraph_host(Algo algo, const kamsta_cgraph* g, kamsta_cfg c,
                                kamsta_wedge* out, uint64_t* out_count, kamsta_stats* stats) {
  kamsta_status s = check_cgraph(g);
  if (s != KAMSTA_OK) return s;
  if (!out_count || (g->n > 1 && !out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  c.compression = KAMSTA_NO_COMPRESSION;
  s = check_cfg(&c);
  if (s != KAMSTA_OK) return s;
  kamsta_ctx* ctx = nullptr;
  s = g_default.get(&ctx);
  if (s != KAMSTA_OK) return s;
  std::lock_guard<std::mutex> lock(ctx->mu);
  *out_count = 0;
  if (g->m_directed == 0 || g->n == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return KAMSTA_OK;
  }
  // compressed bytes, chunk table, the forest and a decode error word in the
  // context's io arena
  const size_t ob = (sizeof(uint64_t) * (g->num_chunks + 1) + 255) & ~size_t(255);
  const size_t fb = (sizeof(kamsta_wedge) * g->num_chunks + 255) & ~size_t(255);
  const size_t db = (g->data_bytes + 255) & ~size_t(255);
  const size_t outb = std::max<uint64_t>(g->n, 1) * sizeof(kamsta_wedge);
  cudaError_t e = ctx_reserve(ctx, ctx->io, ob + fb + db + outb + 2048);
  if (e != cudaSuccess) return cuda_status(e, "device buffers for compressed input");
  // the chunk table is on the host: every chunk's bytes must lie inside data
  bool layout = g->chunk_edges != 0 && g->chunk_edges <= kMaxChunkEdges &&
                g->num_chunks == (g->m_directed + g->chunk_edges - 1) / g->chunk_edges &&
                g->chunk_offset[g->num_chunks] <= g->data_bytes;
  for (uint64_t k = 0; layout && k < g->num_chunks; ++k)
    layout = g->chunk_offset[k] <= g->chunk_offset[k + 1];
  if (!layout) {
    set_error("decode_7bit: inconsistent chunk layout");
    return KAMSTA_E_INPUT;
  }
  kamsta_cgraph dg = *g;
  uint64_t* doff = ctx->io.take<uint64_t>(g->num_chunks + 1);
  kamsta_wedge* dfirst = ctx->io.take<kamsta_wedge>(g->num_chunks);
  uint8_t* ddata = ctx->io.take<uint8_t>(std::max<uint64_t>(g->data_bytes, 1));
  kamsta_wedge* dout = ctx->io.take<kamsta_wedge>(std::max<uint64_t>(g->n, 1));
  uint32_t* derr = ctx->io.take<uint32_t>(64);
  cudaStream_t st = ctx->stream, cp = ctx->aux;
  void* buf = nullptr;
  e = ctx_alloc(ctx, &buf, g->m_directed * sizeof(kamsta_wedge), st);
  if (e != cudaSuccess) return cuda_status(e, "decode buffer");
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } fr{buf, st};
  kamsta_wedge* dec = static_cast<kamsta_wedge*>(buf);
  dg.chunk_offset = doff;
  dg.chunk_first = dfirst;
  dg.data = ddata;
  // the compressed bytes in pieces on the second stream, an event after
  // each; the solve's stream decodes piece k as soon as it has landed, while
  // the next pieces are still being copied
  e = cudaMemsetAsync(derr, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_fork, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cp, ctx->ev_fork, 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(doff, g->chunk_offset, sizeof(uint64_t) * (g->num_chunks + 1),
                        cudaMemcpyHostToDevice, cp);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dfirst, g->chunk_first, sizeof(kamsta_wedge) * g->num_chunks,
                        cudaMemcpyHostToDevice, cp);
  if (e != cudaSuccess) {
    cudaStreamSynchronize(cp);  // no copy from the caller's memory outlives the call
    return cuda_status(e, "cudaMemcpyAsync(H2D)");
  }
  const uint64_t nch = g->num_chunks, C = g->chunk_edges;
  for (int k = 0; k < kInputPieces; ++k) {
    const uint64_t c0 = nch * k / kInputPieces, c1 = nch * (k + 1) / kInputPieces;
    const uint64_t b0 = g->chunk_offset[c0], b1 = g->chunk_offset[c1];
    if (b1 > b0) e = cudaMemcpyAsync(ddata + b0, g->data + b0, b1 - b0, cudaMemcpyHostToDevice, cp);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->piece_ev[k], cp);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(cp);
      return cuda_status(e, "cudaMemcpyAsync(H2D)");
    }
  }
  for (int k = 0; k < kInputPieces; ++k) {
    const uint64_t c0 = nch * k / kInputPieces, c1 = nch * (k + 1) / kInputPieces;
    e = cudaStreamWaitEvent(st, ctx->piece_ev[k], 0);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(cp);
      return cuda_status(e, "cudaStreamWaitEvent");
    }
    if (c1 <= c0) continue;
    kamsta_cgraph pg = dg;
    pg.chunk_offset = doff + c0;
    pg.chunk_first = dfirst + c0;
    pg.num_chunks = c1 - c0;
    pg.m_directed = std::min<uint64_t>(g->m_directed, c1 * C) - c0 * C;
    s = decode_7bit(pg, dec + c0 * C, derr, st);
    if (s != KAMSTA_OK) {
      cudaStreamSynchronize(cp);
      return s;
    }
  }
  e = cudaMemcpyAsync(ctx->h_err, derr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "decode");
  if (*ctx->h_err) {
    set_error("decode_7bit: malformed chunk (value count or length)");
    return KAMSTA_E_INPUT;
  }
  // the decoded input is complete; the forest edges of the first round go
  // back on the second stream while the solve goes on
  HostIo io;
  io.pieces = 0;
  io.copy_stream = cp;
  io.host_out = out;
  io.ev_early = ctx->ev_early;
  SolveOut so;
  s = solve_device(ctx, algo, dec, g->m_directed, g->n, c, dout, &so, stats, st, nullptr, &io);
  if (s != KAMSTA_OK) {
    cudaStreamSynchronize(cp);  // no copy may outlive the call
    return s;
  }
  if (so.count > io.early) {
    e = cudaMemcpyAsync(out + io.early, dout + io.early,
                        (so.count - io.early) * sizeof(kamsta_wedge), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(cp);
      return cuda_status(e, "cudaMemcpyAsync(D2H)");
    }
  }
  e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cp);
  if (e != cudaSuccess) return cuda_status(e, "cudaStreamSynchronize");
  *out_count = so.count;
  return KAMSTA_OK;
}

// AlgorithmConfig::compression = SEVEN_BIT_DIFF_ENCODING on the plain
// host-buffer entry points: as the reference's boruvka() compresses its
// input itself (hybrid_boruvka.hpp:277-299), the input is encoded here on
// the host cores (chunks of 4096 edges), only the compressed bytes are
// copied to the device, and the device decodes and solves them.
kamsta_status solve_host_7bit(Algo algo, const kamsta_wedge* edges, uint64_t m, uint32_t n,
                              kamsta_cfg c, kamsta_wedge* out, uint64_t* out_count,
                              kamsta_stats* stats) {
  constexpr uint32_t kChunk = 4096;
  kamsta_cgraph g{};
  g.m_directed = m;
  g.n = n;
  g.chunk_edges = kChunk;
  g.num_chunks = (m + kChunk - 1) / kChunk;
  std::vector<uint64_t> off(g.num_chunks + 1);
  std::vector<kamsta_wedge> first(std::max<uint64_t>(g.num_chunks, 1));
  uint64_t bytes = 0;
  kamsta_status s = encode_7bit(edges, m, kChunk, off.data(), first.data(), nullptr, 0, &bytes);
  if (s != KAMSTA_OK) return s;
  std::unique_ptr<uint8_t[]> data(new uint8_t[std::max<uint64_t>(bytes, 1)]);
  s = encode_7bit(edges, m, kChunk, off.data(), first.data(), data.get(), bytes, &bytes);
  if (s != KAMSTA_OK) return s;
  g.data_bytes = bytes;
  g.chunk_offset = off.data();
  g.chunk_first = first.data();
  g.data = data.get();
  s = solve_cgraph_host(algo, &g, c, out, out_count, stats);
  if (s != KAMSTA_OK) return s;
  if (c.flags & KAMSTA_FLAG_SORT_OUTPUT)
    std::sort(out, out + *out_count, [](const kamsta_wedge& a, const kamsta_wedge& b) {
      return a.src != b.src ? a.src < b.src : a.dst < b.dst;
    });
  return KAMSTA_OK;
}

}  // namespace
}  // namespace kamsta

using namespace kamsta;

extern "C" {

kamsta_status kamsta_cfg_default(kamsta_cfg* cfg) {
  if (!cfg) return KAMSTA_E_INPUT;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->local_preprocessing = KAMSTA_NO_PREPROCESSING;
  cfg->compression = KAMSTA_NO_COMPRESSION;
  cfg->filter_threshold = 4;
  cfg->dedupe_ratio = 0;
  cfg->seed = 0x243f6a8885a308d3ull;
  return KAMSTA_OK;
}

const char* kamsta_version(void) { return "kamsta-gb300 0.1 (sm_103a)"; }

const char* kamsta_last_error(void) { return last_error_cstr(); }

kamsta_status kamsta_ctx_create(int device, kamsta_ctx** out) {
  if (!out) return KAMSTA_E_INPUT;
  *out = nullptr;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  std::unique_ptr<kamsta_ctx> c(new kamsta_ctx());
  c->device = device;
  kamsta_status s = KAMSTA_OK;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_early, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_counters, sizeof(DevCounters) * kCSlots)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_err, sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_samples, sizeof(uint32_t) * kSampleCap)) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_counters, sizeof(DevCounters) * kCSlots)) != cudaSuccess ||
      (e = cudaMallocHost(&c->h_err, sizeof(uint32_t))) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
    s = cuda_status(e, "kamsta_ctx_create");
  }
  for (int i = 0; s == KAMSTA_OK && i < kTimerEvents; ++i)
    if ((e = cudaEventCreate(&c->tev[i])) != cudaSuccess) s = cuda_status(e, "cudaEventCreate");
  for (int i = 0; s == KAMSTA_OK && i < kInputPieces; ++i)
    if ((e = cudaEventCreateWithFlags(&c->piece_ev[i], cudaEventDisableTiming)) != cudaSuccess)
      s = cuda_status(e, "cudaEventCreate");
  if (s == KAMSTA_OK) {
    // a private stream-ordered pool for edge lists; it keeps its memory
    // between calls (release threshold = unlimited) until kamsta_ctx_trim
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if ((e = cudaMemPoolCreate(&c->pool, &props)) != cudaSuccess) {
      s = cuda_status(e, "cudaMemPoolCreate");
    } else {
      uint64_t thr = ~0ull;
      cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  cudaSetDevice(prev);
  if (s != KAMSTA_OK) {
    kamsta_ctx_destroy(c.release());
    return s;
  }
  *out = c.release();
  return KAMSTA_OK;
}

kamsta_status kamsta_ctx_destroy(kamsta_ctx* ctx) {
  if (!ctx) return KAMSTA_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->aux) cudaStreamSynchronize(ctx->aux);
  ctx->fixed.release();
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  if (ctx->d_counters) cudaFree(ctx->d_counters);
  if (ctx->d_err) cudaFree(ctx->d_err);
  if (ctx->d_samples) cudaFree(ctx->d_samples);
  if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
  if (ctx->h_err) cudaFreeHost(ctx->h_err);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (int i = 0; i < kTimerEvents; ++i)
    if (ctx->tev[i]) cudaEventDestroy(ctx->tev[i]);
  ctx->io.release();
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_early) cudaEventDestroy(ctx->ev_early);
  for (int i = 0; i < kInputPieces; ++i)
    if (ctx->piece_ev[i]) cudaEventDestroy(ctx->piece_ev[i]);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  cudaSetDevice(prev);
  delete ctx;
  return KAMSTA_OK;
}

kamsta_status kamsta_ctx_trim(kamsta_ctx* ctx) {
  if (!ctx) return KAMSTA_E_INPUT;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->fixed.release();
  ctx->io.release();
  if (ctx->pool) {
    cudaStreamSynchronize(ctx->stream);
    cudaMemPoolTrimTo(ctx->pool, 0);
  }
  return KAMSTA_OK;
}

kamsta_status kamsta_ctx_set_memory_limit(kamsta_ctx* ctx, uint64_t bytes) {
  if (!ctx) {
    set_error("null context");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->mem_limit = bytes;
  return KAMSTA_OK;
}

uint64_t kamsta_ctx_pool_bytes(const kamsta_ctx* ctx) {
  if (!ctx) return 0;
  uint64_t pool = 0;
  if (ctx->pool) cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &pool);
  return ctx->fixed.cap + ctx->io.cap + pool;
}

kamsta_status kamsta_mst_boruvka(const kamsta_wedge* edges, uint64_t m, uint32_t n,
                                 const kamsta_cfg* cfg, kamsta_wedge* out,
                                 uint64_t* out_count, kamsta_stats* stats) {
  return solve_host(Algo::kBoruvka, edges, m, n, cfg, out, out_count, stats);
}

kamsta_status kamsta_mst_filter_boruvka(const kamsta_wedge* edges, uint64_t m, uint32_t n,
                                        const kamsta_cfg* cfg, kamsta_wedge* out,
                                        uint64_t* out_count, kamsta_stats* stats) {
  return solve_host(Algo::kFilterBoruvka, edges, m, n, cfg, out, out_count, stats);
}

kamsta_status kamsta_mst_boruvka_wedge64(const kamsta_wedge64* edges, uint64_t m, uint64_t n,
                                         const kamsta_cfg* cfg, kamsta_wedge64* out,
                                         uint64_t* out_count, kamsta_stats* stats) {
  if (!out_count || (m && !edges)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  if (n > 0xffffffffull) {
    set_error("input: n must be < 2^32 for the packed layout");
    return KAMSTA_E_INPUT;
  }
  std::vector<kamsta_wedge> packed(m);
  for (uint64_t i = 0; i < m; ++i) {
    if (edges[i].src >= n || edges[i].dst >= n) {
      set_error("input: vertex id >= n");
      return KAMSTA_E_INPUT;
    }
    packed[i] = kamsta_wedge{static_cast<uint32_t>(edges[i].src),
                             static_cast<uint32_t>(edges[i].dst), edges[i].w};
  }
  std::vector<kamsta_wedge> res(std::max<uint64_t>(n, 1));
  kamsta_status s = solve_host(Algo::kBoruvka, packed.data(), m, static_cast<uint32_t>(n), cfg,
                               res.data(), out_count, stats);
  if (s != KAMSTA_OK) return s;
  for (uint64_t i = 0; i < *out_count; ++i)
    out[i] = kamsta_wedge64{res[i].src, res[i].dst, res[i].w, 0};
  return KAMSTA_OK;
}

kamsta_status kamsta_mst_boruvka_dev(kamsta_ctx* ctx, const kamsta_wedge* d_edges, uint64_t m,
                                     uint32_t n, const kamsta_cfg* cfg, kamsta_wedge* d_out,
                                     uint64_t* out_count, kamsta_stats* stats,
                                     kamsta_stream stream) {
  return solve_dev(Algo::kBoruvka, ctx, d_edges, m, n, cfg, d_out, out_count, stats, stream);
}

kamsta_status kamsta_mst_filter_boruvka_dev(kamsta_ctx* ctx, const kamsta_wedge* d_edges,
                                            uint64_t m, uint32_t n, const kamsta_cfg* cfg,
                                            kamsta_wedge* d_out, uint64_t* out_count,
                                            kamsta_stats* stats, kamsta_stream stream) {
  return solve_dev(Algo::kFilterBoruvka, ctx, d_edges, m, n, cfg, d_out, out_count, stats,
                   stream);
}

kamsta_status kamsta_encode_7bit(const kamsta_wedge* edges, uint64_t m_directed,
                                 uint32_t chunk_edges, uint64_t* chunk_offset,
                                 kamsta_wedge* chunk_first, uint8_t* data,
                                 uint64_t data_capacity, uint64_t* data_bytes) {
  if (!data_bytes || (m_directed && !edges)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return encode_7bit(edges, m_directed, chunk_edges, chunk_offset, chunk_first, data,
                     data_capacity, data_bytes);
}

kamsta_status kamsta_decode_7bit_dev(kamsta_ctx* ctx, const kamsta_cgraph* g,
                                     kamsta_wedge* d_out, kamsta_stream stream) {
  kamsta_status s = check_cgraph(g);
  if (s != KAMSTA_OK) return s;
  if (!ctx || (g->m_directed && !d_out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  cudaError_t e = cudaMemsetAsync(ctx->d_err, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return cuda_status(e, "cudaMemsetAsync");
  s = decode_7bit(*g, d_out, ctx->d_err, st);
  if (s != KAMSTA_OK) return s;
  e = cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_status(e, "decode");
  if (*ctx->h_err) {
    set_error("decode_7bit: malformed chunk (value count or length)");
    return KAMSTA_E_INPUT;
  }
  return KAMSTA_OK;
}

kamsta_status kamsta_mst_boruvka_7bit_dev(kamsta_ctx* ctx, const kamsta_cgraph* g,
                                          const kamsta_cfg* cfg, kamsta_wedge* d_out,
                                          uint64_t* out_count, kamsta_stats* stats,
                                          kamsta_stream stream) {
  kamsta_status s = check_cgraph(g);
  if (s != KAMSTA_OK) return s;
  if (!ctx || !out_count || (g->n > 1 && !d_out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  kamsta_cfg c = cfg_or_default(cfg);
  c.compression = KAMSTA_NO_COMPRESSION;
  s = check_cfg(&c);
  if (s != KAMSTA_OK) return s;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return solve_7bit_locked(ctx, *g, c, d_out, out_count, stats, st);
}

kamsta_status kamsta_mst_boruvka_7bit(const kamsta_cgraph* g, const kamsta_cfg* cfg,
                                      kamsta_wedge* out, uint64_t* out_count,
                                      kamsta_stats* stats) {
  return solve_cgraph_host(Algo::kBoruvka, g, cfg_or_default(cfg), out, out_count, stats);
}

kamsta_status kamsta_mst_batch_dev(kamsta_ctx* ctx, kamsta_graph_desc* graphs, uint32_t count,
                                   const kamsta_cfg* cfg, uint64_t budget_bytes,
                                   kamsta_batch_stats* stats, kamsta_stream stream) {
  if (!ctx) {
    set_error("null context");
    return KAMSTA_E_INPUT;
  }
  return batch_call(ctx, graphs, count, cfg, budget_bytes, stats, false, stream);
}

kamsta_status kamsta_batch_autotune(kamsta_ctx* ctx, kamsta_graph_desc* graphs, uint32_t count,
                                    const kamsta_cfg* cfg, kamsta_tuning* out,
                                    kamsta_stream stream) {
  if (!ctx || !out || (count && !graphs)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  kamsta_status s = check_cfg(cfg);
  if (s != KAMSTA_OK) return s;
  kamsta_cfg c = cfg_or_default(cfg);
  std::lock_guard<std::mutex> lock(ctx->mu);
  const Algo algo = (c.flags & KAMSTA_FLAG_FILTER) ? Algo::kFilterBoruvka : Algo::kBoruvka;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return batch_autotune(ctx, algo, graphs, count, c, st, out);
}

kamsta_status kamsta_ctx_set_tuning(kamsta_ctx* ctx, const kamsta_tuning* t) {
  if (!ctx) {
    set_error("null context");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (t && t->small_threads && t->small_threads != 256 && t->small_threads != 512 &&
      t->small_threads != 1024) {
    set_error("tuning: small_threads must be 256, 512 or 1024");
    return KAMSTA_E_INPUT;
  }
  ctx->tune_small_threads = t ? t->small_threads : 0;
  ctx->tune_small_max_n = t ? t->small_max_n : 0;
  return KAMSTA_OK;
}

kamsta_status kamsta_ctx_set_tiles(kamsta_ctx* ctx, uint32_t items, uint32_t seg_items) {
  if (!ctx) {
    set_error("null context");
    return KAMSTA_E_INPUT;
  }
  if ((items != 0 && items != 6 && items != 8 && items != 12) ||
      (seg_items != 0 && seg_items != 2 && seg_items != 4 && seg_items != 8)) {
    set_error("tiles: items_per_thread 0, 6, 8 or 12; seg_items_per_thread 0, 2, 4 or 8");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->tune_dir_items = items;
  ctx->tune_seg_items = seg_items;
  return KAMSTA_OK;
}

kamsta_status kamsta_autotune_tiles(kamsta_ctx* ctx, const kamsta_wedge* d_edges,
                                    uint64_t m, uint32_t n, const kamsta_cfg* cfg,
                                    kamsta_wedge* d_out, kamsta_tile_tuning* out,
                                    kamsta_stream stream) {
  if (!ctx || !out || (m && !d_edges) || (n > 1 && !d_out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  kamsta_status s = check_cfg(cfg);
  if (s != KAMSTA_OK) return s;
  const kamsta_cfg base = cfg_or_default(cfg);
  const Algo algo = (base.flags & KAMSTA_FLAG_FILTER) ? Algo::kFilterBoruvka : Algo::kBoruvka;
  static const uint32_t kPairs[6][2] = {{6, 2}, {8, 2}, {12, 2}, {6, 4}, {8, 4}, {12, 4}};
  std::memset(out, 0, sizeof(*out));
  std::lock_guard<std::mutex> lock(ctx->mu);
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != ctx->device) {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  }
  const cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  int best = -1;
  for (int i = -1; i < 6 && s == KAMSTA_OK; ++i) {  // i = -1: the untimed warm-up
    kamsta_cfg c = base;
    c.items_per_thread = kPairs[i < 0 ? 0 : i][0];
    c.seg_items_per_thread = kPairs[i < 0 ? 0 : i][1];
    c.flags &= ~static_cast<uint32_t>(KAMSTA_FLAG_SORT_OUTPUT);
    SolveOut so;
    kamsta_stats stt;
    s = solve_device(ctx, algo, d_edges, m, n, c, d_out, &so, &stt, st);
    if (s != KAMSTA_OK || i < 0) continue;
    out->ms[i] = stt.device_ms;
    if (best < 0 || stt.device_ms < out->ms[best]) best = i;
  }
  if (cur != ctx->device) cudaSetDevice(cur);
  if (s != KAMSTA_OK) return s;
  if (best >= 0) {
    out->items_per_thread = kPairs[best][0];
    out->seg_items_per_thread = kPairs[best][1];
    ctx->tune_dir_items = out->items_per_thread;
    ctx->tune_seg_items = out->seg_items_per_thread;
  }
  return KAMSTA_OK;
}

kamsta_status kamsta_mst_batch(kamsta_ctx* ctx, kamsta_graph_desc* graphs, uint32_t count,
                               const kamsta_cfg* cfg, uint64_t budget_bytes,
                               kamsta_batch_stats* stats) {
  return batch_call(ctx, graphs, count, cfg, budget_bytes, stats, true, nullptr);
}

}  // extern "C"
