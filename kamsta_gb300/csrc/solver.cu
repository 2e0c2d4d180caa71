// solver.cu -- round driver of the GB300 MSF solver.
//
// Structure (reference, KaMSTa tree -> here):
//   boruvka_filter_rec  local_mst_respecting_cut_edges.hpp:209-260
//       -> plan_classes(): the light-first recursion is unrolled into weight
//          classes up front (same 25%-quantile pivots, same "m <= 3n" and
//          balance stop rules, estimated from a device weight sample), then
//          classes are contracted lightest first.
//   boruvka3            local_mst_respecting_cut_edges.hpp:101-207
//       -> Solve::rounds(): hook, jump, renumber, map, relabel+compact.
//   localMST::filter    mst_utils_filter.hpp:102-126
//       -> Solve::contract(): heavier classes are relabelled by the current
//          components and internal edges dropped on the way into rounds().
//   boruvka_recursive   hybrid_boruvka_edgefilter.hpp:227-330
//       -> Solve::filter_rec(): host recursion over device edge lists.
//
// Edge lists are segmented (see kernels.cuh): every edge pass writes one
// segment per CTA, so no pass has a cross-CTA scan on its critical path.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "kernels.cuh"
#include "solver.cuh"
#include "sort_gen.cuh"

namespace kamsta {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }

kamsta_status cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return KAMSTA_OK;
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? KAMSTA_E_OOM : KAMSTA_E_CUDA;
}

cudaError_t Arena::reserve(size_t bytes) {
  off = 0;
  if (bytes <= cap) return cudaSuccess;
  release();
  cudaError_t e = cudaMalloc(&base, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    base = nullptr;
    cap = 0;
    return e;
  }
  cap = bytes;
  return cudaSuccess;
}

uint64_t ctx_device_bytes(const kamsta_ctx* ctx) {
  uint64_t used = 0;
  if (ctx->pool) cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemCurrent, &used);
  return used + ctx->fixed.cap + ctx->io.cap;
}

cudaError_t ctx_alloc(kamsta_ctx* ctx, void** p, size_t bytes, cudaStream_t st) {
  *p = nullptr;
  if (ctx->mem_limit && ctx_device_bytes(ctx) + bytes > ctx->mem_limit)
    return cudaErrorMemoryAllocation;
  return cudaMallocFromPoolAsync(p, bytes, ctx->pool, st);
}

cudaError_t ctx_reserve(kamsta_ctx* ctx, Arena& a, size_t bytes) {
  // growing releases the old buffer first
  if (bytes > a.cap && ctx->mem_limit &&
      ctx_device_bytes(ctx) - a.cap + bytes > ctx->mem_limit) {
    a.reset();
    return cudaErrorMemoryAllocation;
  }
  return a.reserve(bytes);
}

void Arena::release() {
  if (base) cudaFree(base);
  base = nullptr;
  cap = 0;
  off = 0;
}

#define KS_TRY(x)                   \
  do {                              \
    const kamsta_status s_ = (x);   \
    if (s_ != KAMSTA_OK) return s_; \
  } while (0)
#define CU_TRY(x)                                      \
  do {                                                 \
    const cudaError_t e_ = (x);                        \
    if (e_ != cudaSuccess) return cuda_status(e_, #x); \
  } while (0)

static inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
// Entries per thread of the mapped (relabelling) passes over the directed
// input when the first pass uses 8: 6 (R-MAT 2^24 class pass 1.98 -> 1.36
// ms, RHG 1.55 -> 1.35 ms, when the 8-entry kernel still spilled; 8 gains
// nothing since).
constexpr int kMappedDirItems = 6;
static inline uint32_t ceil_div(uint64_t a, uint64_t b) {
  return static_cast<uint32_t>((a + b - 1) / b);
}

constexpr uint32_t kSamples = 4096;
// Round passes over at most this many vertices use 4-record tiles.
constexpr uint32_t kWideRoundN = 1u << 16;
// Largest next-round label count whose minima a list pass keeps per CTA in
// shared memory (32 KB).
constexpr uint32_t kSminMax = 4096;

template <typename K>
static int blocks_per_sm(K kernel, size_t dyn_smem) {
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, dyn_smem);
  return per_sm < 1 ? 1 : per_sm;
}

// A segmented edge list in pool memory (see kernels.cuh).
struct SegList {
  Rec* base = nullptr;
  uint64_t cap = 0;  // records per segment
  uint32_t nseg = 0;
  uint32_t* d_count = nullptr;  // kMaxSeg entries, written by the pass
  std::vector<uint32_t> h_count;
  uint64_t total = 0;
  void* mem = nullptr;
  SegIn in() const { return SegIn{base, d_count, cap, nseg}; }
};

class Solve {
 public:
  Solve(kamsta_ctx* ctx, cudaStream_t st, const kamsta_wedge* in, uint64_t md, uint32_t n,
        const kamsta_cfg& cfg, kamsta_stats* stats)
      : ctx_(ctx), st_(st), in_(reinterpret_cast<const uint32_t*>(in)), md_(md), n_(n),
        cfg_(cfg), stats_(stats) {}
  ~Solve() {
    for (SegList* L : owned_) {
      free_list(L);
      delete L;
    }
  }

  kamsta_status run(Algo algo, kamsta_wedge* d_out, SolveOut* out);
  // forest as a bitmap over input positions instead of edges (batch split)
  uint32_t* forest_bits_ = nullptr;
  // host input arriving in pieces / early forest copy (host entry point)
  HostIo* io_ = nullptr;

 private:
  // ---- memory
  kamsta_status alloc_fixed();
  SegList* new_list() {
    owned_.push_back(new SegList());
    return owned_.back();
  }
  kamsta_status alloc_list(SegList* L, uint32_t nseg, uint64_t cap);
  void free_list(SegList* L);
  // ---- sync / errors
  kamsta_status fetch_counters();
  kamsta_status check_err();
  void fill_inf(uint64_t* p, uint64_t count);
  int grid_for(uint64_t items) const {
    const uint64_t g = (items + kBlock - 1) / kBlock;
    return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(g, uint64_t(sms_) * 8)));
  }
  // One edge pass (src == nullptr: the directed input).  frac[c] bounds the
  // share of a chunk's items that can land in class c (1 = all); outputs are
  // (re)allocated here and resized exactly once on overflow.  minval (with
  // minval_n entries) receives the class-0 minimum.
  // vertices of the round whose relabel pass runs (0 outside the rounds)
  uint32_t round_nr_ = 0;
  template <int NOUT>
  kamsta_status pass(int phase, const SegList* src, const uint32_t* map, uint32_t wmin,
                     uint32_t wmax, const uint32_t* thr, SegList* const* outs, const double* frac,
                     uint64_t* minval, uint64_t minval_n, bool validate);
  // Boruvka rounds on list L (dense labels in [0, nreps_)); minA_ holds the
  // round-0 minima.  Frees L if `own` is set.
  kamsta_status rounds(SegList* L, bool own);
  // Parallel-edge removal on L (labels < nr): marks every edge but the
  // lightest of each endpoint pair dead (a self loop) for the next pass.
  kamsta_status dedupe(SegList* L, uint32_t nr);
  // Relabel `L` (or the directed input when L == nullptr, weights in
  // [wmin, wmax], a share `frac` of the entries) into the current dense
  // labels, fuse the round-0 minimum and contract the result.
  kamsta_status contract(const SegList* L, uint32_t wmin, uint32_t wmax, double frac);
  // contract()'s pass over the directed input done by row scans of the
  // vertices outside the largest component (done = false: too many of them)
  kamsta_status contract_rows(uint32_t wmin, uint32_t wmax, SegList* E, bool* done);
  // Largest current component (mode of sampled labels); when it holds at
  // least half the vertices, its membership bitmap is built into big_ and
  // the next D-relabelling pass skips gathers for edges inside it.
  kamsta_status pick_big(uint32_t* label, bool* use);
  bool use_big_ = false;
  uint32_t big_label_ = 0;
  std::vector<uint32_t> plan_classes();
  kamsta_status sample_weights(const SegList* L, uint32_t count, std::vector<uint32_t>* out);
  kamsta_status filter_rec(SegList* L, bool own, bool stop, int depth);
  kamsta_status run_boruvka();
  kamsta_status run_filter_boruvka();
  // ---- debugging (KAMSTA_DEBUG_CHECKS=1): host-side invariant checks
  kamsta_status debug_list(const char* where, const SegList& L, uint64_t nlabels);
  kamsta_status debug_forest(const char* where, uint64_t count);

  void trace(uint64_t m, uint64_t n) {
    if (stats_ && (cfg_.flags & KAMSTA_FLAG_TRACE) && stats_->trace_len < KAMSTA_TRACE_MAX) {
      stats_->trace_m[stats_->trace_len] = m;
      stats_->trace_n[stats_->trace_len] = n;
      stats_->trace_len++;
    }
  }
  // phase timing: event pairs recorded on st_, resolved after each host sync
  struct Pending {
    int phase, ev_a, ev_b;
  };
  int tick() {
    const int e = next_ev_;
    next_ev_ = (next_ev_ + 1) % kTimerEvents;
    cudaEventRecord(ctx_->tev[e], st_);
    return e;
  }
  void tock(int phase, int ev_a) { pending_.push_back({phase, ev_a, tick()}); }
  void resolve() {
    for (const Pending& q : pending_) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ctx_->tev[q.ev_a], ctx_->tev[q.ev_b]) == cudaSuccess)
        phase_ms_[q.phase] += ms;
    }
    pending_.clear();
    cudaGetLastError();
  }
  void account(int phase, uint64_t bytes, uint32_t launches) {
    phase_bytes_[phase] += bytes;
    phase_launches_[phase] += launches;
    alg_bytes_ += bytes;
    launches_ += launches;
  }

  kamsta_ctx* ctx_;
  cudaStream_t st_;
  const uint32_t* in_;  // directed input as 32-bit words (3 per entry)
  uint64_t md_;
  uint32_t n_;
  kamsta_cfg cfg_;
  kamsta_stats* stats_;
  int sms_ = 1;
  bool aligned16_ = false;
  bool debug_ = false;
  bool tolerate_overflow_ = false;
  uint32_t launches_ = 0, rounds_ = 0, levels_ = 0, dedupe_passes_ = 0, row_scans_ = 0;
  bool final_contraction_ = false;  // rounds() of the last contraction (boruvka)
  int dir_items_ = kItemsDir;        // items per thread of k_pass_dir (6, 8, 12)
  int seg_items_ = kItemsRec;        // records per thread of k_pass_seg (2, 4, 8)
  uint64_t alg_bytes_ = 0;
  double phase_ms_[KAMSTA_PHASES] = {};
  uint64_t phase_bytes_[KAMSTA_PHASES] = {};
  uint32_t phase_launches_[KAMSTA_PHASES] = {};
  std::vector<Pending> pending_;
  int next_ev_ = 0;
  std::vector<SegList*> owned_;

  // vertex-side buffers (n_ entries unless noted)
  uint32_t *P_ = nullptr, *D_ = nullptr, *V_ = nullptr, *Vn_ = nullptr;
  uint32_t *dense_of_ = nullptr, *parent_ = nullptr, *msfoid_ = nullptr, *newid_ = nullptr;
  uint32_t *Rbuf_ = nullptr, *Obuf_ = nullptr, *msf_ = nullptr, *samples_ = nullptr;
  uint64_t *minA_ = nullptr, *minB_ = nullptr, *prefix_ = nullptr;
  uint32_t* cta_counts_ = nullptr;  // per-CTA counts of the vertex scans
  uint32_t* big_ = nullptr;         // membership bitmap of the largest component
  uint32_t nreps_ = 0;
  uint64_t msf_count_ = 0;
  bool input_complete_ = true;  // every later input reader is ordered after the last piece
  kamsta_status wait_input(int piece) {
    if (io_ && io_->pieces > 0)
      CU_TRY(cudaStreamWaitEvent(st_, io_->piece_ev[piece < io_->pieces ? piece : io_->pieces - 1], 0));
    return KAMSTA_OK;
  }
  // Direct emission: the first round over original ids (the first pass's
  // lightest class) writes its forest edges to the output itself, so the
  // final emit gathers only the later rounds' edges from the input.
  kamsta_wedge* d_out_ = nullptr;
  unsigned long long* dweight_ = nullptr;  // weight of the directly written edges
  bool direct_emit_ = false;  // the first pass keys minima by partner; round 0 emits
  uint64_t direct_count_ = 0;           // forest edges written directly
  std::vector<uint32_t> bounds_;        // ascending weight-class bounds
  std::vector<uint32_t> samples_host_;  // sorted weight sample of the input
};

// ---------------------------------------------------------------------------
// memory

kamsta_status Solve::alloc_fixed() {
  const uint64_t n = n_;
  size_t bytes = 0;
  auto add = [&](uint64_t count, size_t sz) { bytes += round_up(count * sz, 256); };
  for (int i = 0; i < 9; ++i) add(n + 1, 4);  // P D V Vn dense parent msfoid newid msf
  add(2 * n + 64, 4);                         // Rbuf
  add(n + 64, 4);                             // Obuf
  add(n + 1, 8);
  add(n + 1, 8);  // minA minB
  add(kMaxSeg + 1, 8);
  add(2 * kMaxSeg, 4);
  add(n / 32 + 2, 4);
  add(4, 8);  // dweight
  CU_TRY(ctx_reserve(ctx_, ctx_->fixed, bytes + 4096));
  Arena& A = ctx_->fixed;
  P_ = A.take<uint32_t>(n + 1);
  D_ = A.take<uint32_t>(n + 1);
  V_ = A.take<uint32_t>(n + 1);
  Vn_ = A.take<uint32_t>(n + 1);
  dense_of_ = A.take<uint32_t>(n + 1);
  parent_ = A.take<uint32_t>(n + 1);
  msfoid_ = A.take<uint32_t>(n + 1);
  newid_ = A.take<uint32_t>(n + 1);
  msf_ = A.take<uint32_t>(n + 1);
  Rbuf_ = A.take<uint32_t>(2 * n + 64);
  Obuf_ = A.take<uint32_t>(n + 64);
  minA_ = A.take<uint64_t>(n + 1);
  minB_ = A.take<uint64_t>(n + 1);
  prefix_ = A.take<uint64_t>(kMaxSeg + 1);
  cta_counts_ = A.take<uint32_t>(2 * kMaxSeg);
  big_ = A.take<uint32_t>(n / 32 + 2);
  dweight_ = A.take<unsigned long long>(4);
  if (!big_ || !dweight_) {
    set_error("internal: fixed arena too small");
    return KAMSTA_E_OOM;
  }
  return KAMSTA_OK;
}

kamsta_status Solve::alloc_list(SegList* L, uint32_t nseg, uint64_t cap) {
  free_list(L);
  cap = std::max<uint64_t>(cap, 1);
  const size_t cnt_bytes = round_up(sizeof(uint32_t) * kMaxSeg, 256);
  const size_t bytes = cnt_bytes + static_cast<size_t>(nseg) * cap * sizeof(Rec);
  void* mem = nullptr;
  CU_TRY(ctx_alloc(ctx_, &mem, bytes, st_));
  L->mem = mem;
  L->d_count = static_cast<uint32_t*>(mem);
  L->base = reinterpret_cast<Rec*>(static_cast<char*>(mem) + cnt_bytes);
  L->cap = cap;
  L->nseg = nseg;
  L->h_count.assign(nseg, 0);
  L->total = 0;
  return KAMSTA_OK;
}

void Solve::free_list(SegList* L) {
  if (L && L->mem) cudaFreeAsync(L->mem, st_);
  if (L) {
    L->mem = nullptr;
    L->base = nullptr;
    L->d_count = nullptr;
    L->total = 0;
    L->nseg = 0;
  }
}

// ---------------------------------------------------------------------------
// sync, errors, debugging

kamsta_status Solve::check_err() {
  uint32_t e = *ctx_->h_err;
  if (tolerate_overflow_) e &= ~static_cast<uint32_t>(kErrOverflow);
  if (e == 0) return KAMSTA_OK;
  if (e & kErrRange) {
    set_error("input: vertex id >= n");
    return KAMSTA_E_INPUT;
  }
  if (e & kErrOrder) {
    set_error("input: entries not strictly sorted by (src, dst)");
    return KAMSTA_E_INPUT;
  }
  if (e & (kErrLookback | kErrJump | kErrSpin)) {
    set_error("device wait or pointer-jumping cap reached");
    return KAMSTA_E_NOCONVERGE;
  }
  if (e & kErrOverflow) {
    set_error("internal: device output buffer overflow");
    return KAMSTA_E_CUDA;
  }
  set_error("internal consistency check failed on the device (code " + std::to_string(e) + ")");
  return KAMSTA_E_CUDA;
}

kamsta_status Solve::fetch_counters() {
  CU_TRY(cudaMemcpyAsync(ctx_->h_counters, ctx_->d_counters, sizeof(DevCounters) * kCSlots,
                         cudaMemcpyDeviceToHost, st_));
  CU_TRY(cudaMemcpyAsync(ctx_->h_err, ctx_->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
  CU_TRY(cudaStreamSynchronize(st_));
  resolve();
  return check_err();
}

kamsta_status Solve::debug_list(const char* where, const SegList& L, uint64_t nlabels) {
  if (!debug_ || L.total == 0) return KAMSTA_OK;
  uint32_t prev = 0;
  bool first = true;
  for (uint32_t s = 0; s < L.nseg; ++s) {
    const uint32_t c = L.h_count[s];
    if (!c) continue;
    std::vector<Rec> h(c);
    CU_TRY(cudaMemcpyAsync(h.data(), L.base + s * L.cap, c * sizeof(Rec), cudaMemcpyDeviceToHost,
                           st_));
    CU_TRY(cudaStreamSynchronize(st_));
    for (uint32_t i = 0; i < c; ++i) {
      const bool ok = (first || h[i].oid > prev) && h[i].a < nlabels && h[i].b < nlabels &&
                      h[i].a != h[i].b;
      if (!ok) {
        fprintf(stderr,
                "[kamsta debug] %s: bad record seg %u idx %u: a=%u b=%u w=%u oid=%u prev=%u "
                "nlabels=%llu\n",
                where, s, i, h[i].a, h[i].b, h[i].w, h[i].oid, prev, (unsigned long long)nlabels);
        set_error(std::string("debug check failed: ") + where);
        return KAMSTA_E_CUDA;
      }
      prev = h[i].oid;
      first = false;
    }
  }
  return KAMSTA_OK;
}

kamsta_status Solve::debug_forest(const char* where, uint64_t count) {
  // input positions are recorded after the directly written edges only
  if (!debug_ || count <= direct_count_) return KAMSTA_OK;
  std::vector<uint32_t> h(count - direct_count_);
  CU_TRY(cudaMemcpyAsync(h.data(), msf_ + direct_count_, h.size() * 4, cudaMemcpyDeviceToHost,
                         st_));
  CU_TRY(cudaStreamSynchronize(st_));
  std::sort(h.begin(), h.end());
  for (size_t i = 1; i < h.size(); ++i)
    if (h[i] == h[i - 1]) {
      fprintf(stderr, "[kamsta debug] %s: forest edge id %u appears twice\n", where, h[i]);
      set_error(std::string("debug check failed: ") + where);
      return KAMSTA_E_CUDA;
    }
  return KAMSTA_OK;
}

void Solve::fill_inf(uint64_t* p, uint64_t count) {
  if (!count) return;
  k_fill64<<<grid_for(count), kBlock, 0, st_>>>(count, p, kInf64);
  account(KAMSTA_PHASE_FINALIZE, count * 8, 1);
}

// ---------------------------------------------------------------------------
// edge passes

template <int NOUT>
kamsta_status Solve::pass(int phase, const SegList* src, const uint32_t* map, uint32_t wmin,
                          uint32_t wmax, const uint32_t* thr, SegList* const* outs,
                          const double* frac, uint64_t* minval, uint64_t minval_n,
                          bool validate) {
  const bool dir = src == nullptr;
  const uint64_t total = dir ? md_ : src->total;
  const int items = (map != nullptr && dir_items_ == 8) ? kMappedDirItems : dir_items_;
  int sitems = seg_items_;
  uint32_t smin_n = 0;
  if (!dir && phase == KAMSTA_PHASE_ROUND_EDGES && round_nr_ > 0) {
    // late rounds: their label map and minima sit in the L2, and a wider
    // tile (4 records per thread) gained 0.1 ms per solve at 2^26/2^30
    if (round_nr_ <= kWideRoundN && sitems < 4) sitems = 4;
    // a round's live roots are at most half its vertices, so the next
    // labels are below round_nr_ / 2: few enough to keep per CTA
    if (minval && round_nr_ / 2 <= kSminMax) smin_n = std::max<uint32_t>(1, round_nr_ / 2);
  }
  const uint32_t tile = dir ? dir_tile(items) : rec_tile(sitems);
  const size_t dyn = dir ? dir_dyn_smem(items)
                         : rec_dyn_smem(sitems) + round_up(size_t(smin_n) * 8, 16);
  const bool mapped = map != nullptr;
  const int per_sm =
      !dir ? (sitems == 2 ? blocks_per_sm(k_pass_seg<NOUT, 2>, dyn)
              : sitems == 4 ? blocks_per_sm(k_pass_seg<NOUT, 4>, dyn)
                          : blocks_per_sm(k_pass_seg<NOUT, 8>, dyn))
      : mapped ? (items == 8    ? blocks_per_sm(k_pass_dir<NOUT, 8, true>, dyn)
                  : items == 6  ? blocks_per_sm(k_pass_dir<NOUT, 6, true>, dyn)
                                : blocks_per_sm(k_pass_dir<NOUT, 12, true>, dyn))
               : (items == 8    ? blocks_per_sm(k_pass_dir<NOUT, 8, false>, dyn)
                  : items == 6  ? blocks_per_sm(k_pass_dir<NOUT, 6, false>, dyn)
                                : blocks_per_sm(k_pass_dir<NOUT, 12, false>, dyn));
  const uint64_t gmax = std::min<uint64_t>(kMaxSeg, uint64_t(per_sm) * sms_);
  uint64_t chunk = std::max<uint64_t>(1, (total + gmax - 1) / gmax);
  chunk = round_up(chunk, tile);
  const uint32_t G = std::max<uint32_t>(1, ceil_div(total, chunk));
  uint64_t cap[kMaxOut];
  for (int c = 0; c < NOUT; ++c) {
    const double f = std::min(1.0, std::max(0.0, frac ? frac[c] : 1.0));
    const double est = f * chunk * 1.1 + 6.0 * std::sqrt(f * chunk) + tile;
    cap[c] = std::min<uint64_t>(chunk, static_cast<uint64_t>(est));
  }
  if (!dir && src->nseg > static_cast<uint32_t>(kMaxSeg)) {
    set_error("internal: too many segments");
    return KAMSTA_E_CUDA;
  }
  for (int attempt = 0;; ++attempt) {
    for (int c = 0; c < NOUT; ++c) KS_TRY(alloc_list(outs[c], G, cap[c]));
    if (total == 0) return KAMSTA_OK;
    CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCEdge, 0, sizeof(DevCounters), st_));
    PassArgs a{};
    a.map = map;
    if (use_big_ && map == D_) {
      a.big = big_;
      a.big_label = big_label_;
    }
    a.wmin = wmin;
    a.wmax = wmax;
    for (int c = 0; c < NOUT - 1; ++c) a.thr[c] = thr[c];
    for (int c = 0; c < NOUT; ++c) a.out[c] = SegOut{outs[c]->base, cap[c], outs[c]->d_count};
    a.minval = minval;
    // original ids (no map): few updates per address, reductions go straight
    // out; relabelled lists have hub components, so updates are filtered
    a.min_checked = map != nullptr ? 1u : 0u;
    a.min_partner = (direct_emit_ && src == nullptr && map == nullptr) ? 1u : 0u;
    a.total = total;
    a.chunk = chunk;
    a.counts = ctx_->d_counters[kCEdge].cnt;
    a.err = ctx_->d_err;
    a.n = n_;
    a.validate = validate ? 1 : 0;
    a.aligned16 = aligned16_ ? 1 : 0;
    a.smin_n = smin_n;
    const int t0 = tick();
    bool launched = false;
    if (dir && !mapped && !input_complete_ && attempt == 0) {
      // the input is still arriving: launch the CTAs whose chunks have landed
      uint32_t b0 = 0;
      for (int k = 0; k < io_->pieces && b0 < G; ++k) {
        const uint32_t b1 =
            k + 1 == io_->pieces
                ? G
                : static_cast<uint32_t>(std::min<uint64_t>(G, io_->piece_end[k] / chunk));
        if (b1 <= b0) continue;
        KS_TRY(wait_input(k));
        a.cta_base = b0;
        if (items == 8) k_pass_dir<NOUT, 8, false><<<b1 - b0, kBlock, dyn, st_>>>(in_, a);
        else if (items == 6) k_pass_dir<NOUT, 6, false><<<b1 - b0, kBlock, dyn, st_>>>(in_, a);
        else k_pass_dir<NOUT, 12, false><<<b1 - b0, kBlock, dyn, st_>>>(in_, a);
        b0 = b1;
      }
      a.cta_base = 0;
      KS_TRY(wait_input(io_->pieces - 1));
      input_complete_ = true;
      launched = true;
    } else if (!input_complete_) {
      KS_TRY(wait_input(io_->pieces - 1));
      input_complete_ = true;
    }
    if (launched) {
      // the first pass ran in groups above
    } else if (dir && mapped && items == 8)
      k_pass_dir<NOUT, 8, true><<<G, kBlock, dyn, st_>>>(in_, a);
    else if (dir && mapped && items == 6)
      k_pass_dir<NOUT, 6, true><<<G, kBlock, dyn, st_>>>(in_, a);
    else if (dir && mapped)
      k_pass_dir<NOUT, 12, true><<<G, kBlock, dyn, st_>>>(in_, a);
    else if (dir && items == 8)
      k_pass_dir<NOUT, 8, false><<<G, kBlock, dyn, st_>>>(in_, a);
    else if (dir && items == 6)
      k_pass_dir<NOUT, 6, false><<<G, kBlock, dyn, st_>>>(in_, a);
    else if (dir)
      k_pass_dir<NOUT, 12, false><<<G, kBlock, dyn, st_>>>(in_, a);
    else if (sitems == 2)
      k_pass_seg<NOUT, 2><<<G, kBlock, dyn, st_>>>(src->in(), a);
    else if (sitems == 4)
      k_pass_seg<NOUT, 4><<<G, kBlock, dyn, st_>>>(src->in(), a);
    else
      k_pass_seg<NOUT, 8><<<G, kBlock, dyn, st_>>>(src->in(), a);
    tock(phase, t0);
    CU_TRY(cudaGetLastError());
    for (int c = 0; c < NOUT; ++c)
      CU_TRY(cudaMemcpyAsync(outs[c]->h_count.data(), outs[c]->d_count, sizeof(uint32_t) * G,
                             cudaMemcpyDeviceToHost, st_));
    tolerate_overflow_ = true;
    const kamsta_status fs = fetch_counters();
    tolerate_overflow_ = false;
    KS_TRY(fs);
    bool overflow = false;
    uint64_t kept = 0;
    for (int c = 0; c < NOUT; ++c) {
      uint64_t sum = 0, mx = 0;
      for (uint32_t s = 0; s < G; ++s) {
        sum += outs[c]->h_count[s];
        mx = std::max<uint64_t>(mx, outs[c]->h_count[s]);
      }
      outs[c]->total = sum;
      kept += sum;
      if (mx > cap[c]) {
        overflow = true;
        cap[c] = mx;
      }
    }
    const DevCounters& h = ctx_->h_counters[kCEdge];
    // read every item, two label gathers per candidate, write kept records,
    // one 8-byte minimum per endpoint of a class-0 record
    account(phase,
            total * (dir ? 12 : sizeof(Rec)) + (map ? h.cnt[1] * 8 : 0) + kept * sizeof(Rec) +
                (minval ? outs[0]->total * 16 : 0),
            1);
    if (!overflow) return KAMSTA_OK;
    if (attempt > 0) {
      set_error("internal: edge-pass output overflow after exact resize");
      return KAMSTA_E_CUDA;
    }
    CU_TRY(cudaMemsetAsync(ctx_->d_err, 0, sizeof(uint32_t), st_));
    if (minval) fill_inf(minval, minval_n);  // the failed attempt fed stale positions
  }
}

// ---------------------------------------------------------------------------
// Boruvka rounds (boruvka3).  One host read per round: the new edge, vertex
// and forest-edge counts.
kamsta_status Solve::dedupe(SegList* L, uint32_t nr) {
  if (L->total < 2 || nr < 2) return KAMSTA_OK;
  const uint64_t phys = uint64_t(L->nseg) * L->cap;
  if (phys >= (1ull << 32) - 8192) return KAMSTA_OK;  // positions ride in 32 bits
  uint32_t bb = 1;
  while (bb < 32 && (1ull << bb) < nr) ++bb;
  const int t0 = tick();
  uint32_t* d_wmax = reinterpret_cast<uint32_t*>(&ctx_->d_counters[kCMisc].cnt[2]);
  CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCMisc, 0, sizeof(DevCounters), st_));
  k_list_wmax<<<grid_for(phys), kBlock, 0, st_>>>(L->in(), d_wmax);
  KS_TRY(fetch_counters());
  const uint32_t wmax = static_cast<uint32_t>(ctx_->h_counters[kCMisc].cnt[2]);
  const uint32_t wbits = wmax ? 32u - static_cast<uint32_t>(__builtin_clz(wmax)) : 1u;
  if (2 * bb + wbits > 64) return KAMSTA_OK;  // key does not fit: keep the duplicates
  const int bits = static_cast<int>(2 * bb + wbits);
  const RadixScratch rs = radix_scratch_bytes(phys);
  const size_t kb = round_up(phys * sizeof(uint64_t), 256), vb = round_up(phys * sizeof(uint32_t), 256);
  const size_t cb = round_up(rs.counts * sizeof(uint32_t), 256);
  const size_t sb = round_up(rs.status * sizeof(uint64_t), 256);
  void* mem = nullptr;
  CU_TRY(ctx_alloc(ctx_, &mem, 2 * kb + 2 * vb + cb + sb, st_));
  char* m = static_cast<char*>(mem);
  uint64_t* keys = reinterpret_cast<uint64_t*>(m);
  uint64_t* keys2 = reinterpret_cast<uint64_t*>(m + kb);
  uint32_t* vals = reinterpret_cast<uint32_t*>(m + 2 * kb);
  uint32_t* vals2 = reinterpret_cast<uint32_t*>(m + 2 * kb + vb);
  uint32_t* counts = reinterpret_cast<uint32_t*>(m + 2 * kb + 2 * vb);
  uint64_t* status = reinterpret_cast<uint64_t*>(m + 2 * kb + 2 * vb + cb);
  k_dedupe_keys<<<grid_for(phys), kBlock, 0, st_>>>(L->in(), bb, wbits, keys, vals);
  int alt = 0;
  cudaError_t e = radix_sort_pairs_u32(st_, keys, keys2, vals, vals2, phys, bits, counts, status,
                                       &ctx_->d_counters[kCMisc].ticket, ctx_->d_err, &alt, sms_);
  if (e != cudaSuccess) {
    cudaFreeAsync(mem, st_);
    return cuda_status(e, "radix sort (dedupe)");
  }
  if (alt) {
    std::swap(keys, keys2);
    std::swap(vals, vals2);
  }
  k_dedupe_mark<<<grid_for(phys), kBlock, 0, st_>>>(keys, vals, phys, wbits, L->base,
                                                   &ctx_->d_counters[kCMisc].cnt[3]);
  CU_TRY(cudaFreeAsync(mem, st_));
  tock(KAMSTA_PHASE_DEDUPE, t0);
  const uint32_t passes = static_cast<uint32_t>((bits + 7) / 8);
  // wmax read; keys: record read + key/value write; per digit pass: upsweep
  // read, downsweep read + write of keys and values; mark: keys + values
  account(KAMSTA_PHASE_DEDUPE,
          phys * (16 + 16 + 12 + uint64_t(passes) * (8 + 24) + 12), 3 + 3 * passes);
  dedupe_passes_++;
  return KAMSTA_OK;
}

kamsta_status Solve::rounds(SegList* L, bool own) {
  levels_++;
  const uint32_t n0 = nreps_;
  SegList* cur = L;
  bool cur_owned = own;
  uint32_t nr = n0;
  uint64_t* minv = minA_;
  uint64_t* minn = minB_;
  // per round: its map, its vertices' original representatives, its size
  uint32_t* maps[kMaxRounds];
  const uint32_t* origs[kMaxRounds + 1];
  uint32_t sizes[kMaxRounds];
  origs[0] = V_;
  size_t roff = 0, ooff = 0;
  uint32_t r = 0;
  const uint32_t* orig_cur = V_;
  while (cur->total > 0) {
    if (r >= static_cast<uint32_t>(kMaxRounds)) {
      set_error("round cap reached");
      return KAMSTA_E_NOCONVERGE;
    }
    trace(cur->total, nr);
    const uint64_t m = cur->total;
    if (!(cfg_.flags & KAMSTA_FLAG_DEDUPE_NEVER) &&
        ((cfg_.flags & KAMSTA_FLAG_DEDUPE_ALWAYS) ||
         (cfg_.dedupe_ratio && m > uint64_t(cfg_.dedupe_ratio) * nr)))
      KS_TRY(dedupe(cur, nr));
    CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCVertex, 0, sizeof(DevCounters), st_));
    const int gv = grid_for(nr);
    const int tv = tick();
    // the first round of the first contraction: original ids, minima keyed
    // by partner (first pass), forest edges written directly
    const bool direct = direct_emit_ && r == 0;
    VertexScanArgs va{};
    va.n = nr;
    {
      const uint32_t g = std::max<uint32_t>(
          1, std::min<uint32_t>(ceil_div(nr, kBlock * 8u), static_cast<uint32_t>(sms_) * 4));
      va.chunk = static_cast<uint32_t>(round_up(ceil_div(nr, g), kBlock));
    }
    const uint32_t gvs = std::max<uint32_t>(1, ceil_div(nr, va.chunk));
    // the hook also counts each chunk's roots and hooked vertices
    k_hook<<<gvs, kBlock, 0, st_>>>(nr, minv, cur->base, parent_, msfoid_, direct ? 1u : 0u,
                                    va.chunk, cta_counts_, ctx_->d_counters[kCVertex].cnt,
                                    ctx_->d_err);
    uint32_t* R = Rbuf_ + roff;
    // below 2^31 vertices the compaction runs first and tags the roots, and
    // one walk per vertex yields its label (k_jump_label); otherwise the
    // walk finds the roots and k_map gathers their new ids
    const bool tagged = nr < kRootTag;
    if (!tagged) k_jump<<<gv, kBlock, 0, st_>>>(nr, parent_, R, ctx_->d_err);
    uint32_t* onext = Obuf_ + ooff;
    va.parent = parent_;
    va.minval = minv;
    va.msfoid = msfoid_;
    va.orig_cur = orig_cur;
    va.orig_next = onext;
    va.newid = newid_;
    va.minval_next = minn;
    va.msf_out = msf_ + msf_count_;
    va.msf_cap = (n_ + 1) - msf_count_;
    va.orig_cap = std::min<uint64_t>((n_ + 64) - ooff, n_ + 1);
    va.cta_counts = cta_counts_;
    va.counts = ctx_->d_counters[kCVertex].cnt;
    va.err = ctx_->d_err;
    if (direct) {
      va.direct_out = reinterpret_cast<uint32_t*>(d_out_);
      va.direct_weight = dweight_;
      va.msf_cap = n_ - 1;  // the caller's output capacity
    }
    va.root_tag = tagged ? parent_ : nullptr;
    k_vertex_write<<<gvs, kBlock, 0, st_>>>(va);
    if (tagged) k_jump_label<<<gv, kBlock, 0, st_>>>(nr, parent_, R, ctx_->d_err);
    else k_map<<<gv, kBlock, 0, st_>>>(nr, minv, newid_, R);
    tock(KAMSTA_PHASE_ROUND_VERTS, tv);
    // relabel + self-loop removal + compaction + next-round minimum
    SegList* nxt = new_list();
    SegList* outs[1] = {nxt};
    round_nr_ = nr;
    const kamsta_status ps = pass<1>(KAMSTA_PHASE_ROUND_EDGES, cur, R, 0, 0xffffffffu, nullptr,
                                     outs, nullptr, minn, 0, false);
    round_nr_ = 0;
    KS_TRY(ps);
    const uint64_t n_next = ctx_->h_counters[kCVertex].cnt[0];
    const uint64_t added = ctx_->h_counters[kCVertex].cnt[1];
    // hook: minimum, record gather, partner minimum, parent + edge id;
    // jump: parent reads/writes; scan: parent, minimum, orig per vertex and
    // id/orig/minimum per root, edge id per hooked vertex; map: 3 reads + 1
    // write, or with root tags only the label write.
    // The direct first round gathers no record and writes no edge id; it
    // reads each hooked vertex's key and writes its 12-byte forest edge.
    account(KAMSTA_PHASE_ROUND_VERTS,
            uint64_t(nr) * ((8 + 16 + 8 + 8) + 16 + (4 + 8 + 4) + (tagged ? 4 : 8 + 4 + 4)) +
                n_next * 16 + added * (direct ? 8 + 12 : 8) - (direct ? uint64_t(nr) * 20 : 0),
            tagged ? 4 : 5);
    if (direct) {
      direct_count_ = added;
      if (io_ && io_->host_out && added > 0) {
        // final already: send them to the host while the solve goes on
        CU_TRY(cudaEventRecord(io_->ev_early, st_));
        CU_TRY(cudaStreamWaitEvent(io_->copy_stream, io_->ev_early, 0));
        CU_TRY(cudaMemcpyAsync(io_->host_out, d_out_, added * sizeof(kamsta_wedge),
                               cudaMemcpyDeviceToHost, io_->copy_stream));
        io_->early = added;
      }
    }
    if (debug_) {
      fprintf(stderr, "[kamsta debug] round %u: m=%llu n=%u -> m'=%llu n'=%llu forest+=%llu\n", r,
              (unsigned long long)m, nr, (unsigned long long)nxt->total,
              (unsigned long long)n_next, (unsigned long long)added);
      KS_TRY(debug_forest("after vertex scan", msf_count_ + added));
      KS_TRY(debug_list("after relabel pass", *nxt, n_next));
    }
    msf_count_ += added;
    if (msf_count_ > n_) {
      set_error("internal: forest larger than n-1");
      return KAMSTA_E_CUDA;
    }
    maps[r] = R;
    sizes[r] = nr;
    origs[r + 1] = onext;
    roff += nr;
    ooff += n_next;
    orig_cur = onext;
    if (cur_owned) free_list(cur);
    cur = nxt;
    cur_owned = true;
    nr = static_cast<uint32_t>(n_next);
    std::swap(minv, minn);
    ++r;
  }
  if (cur_owned) free_list(cur);
  rounds_ += r;
  if (r == 0) return KAMSTA_OK;  // nothing contracted; labels unchanged
  if (final_contraction_) return KAMSTA_OK;  // no later pass needs the labels
  const int tf = tick();
  CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCRep, 0, sizeof(DevCounters), st_));
  RepScanArgs ra{};
  ra.n = n0;
  {
    const uint32_t g = std::max<uint32_t>(
        1, std::min<uint32_t>(ceil_div(n0, kBlock * 8u), static_cast<uint32_t>(sms_) * 4));
    ra.chunk = static_cast<uint32_t>(round_up(ceil_div(n0, g), kBlock));
  }
  const uint32_t gr = std::max<uint32_t>(1, ceil_div(n0, ra.chunk));
  uint64_t composed = 0;
  for (int k = static_cast<int>(r) - 1; k >= 0; --k) {
    const uint32_t* next = k + 1 == static_cast<int>(r) ? origs[r] : maps[k + 1];
    if (k > 0)
      k_compose<<<grid_for(sizes[k]), kBlock, 0, st_>>>(sizes[k], maps[k], next, origs[k]);
    else  // also counts the representatives per chunk for k_rep_write
      k_compose_last<<<gr, kBlock, 0, st_>>>(sizes[0], maps[0], next, origs[0], P_, ra.chunk,
                                             cta_counts_, &ctx_->d_counters[kCRep].cnt[0]);
    composed += sizes[k];
  }
  ra.V = V_;
  ra.P = P_;
  ra.Vout = Vn_;
  ra.dense_of = dense_of_;
  ra.cta_counts = cta_counts_;
  ra.counts = ctx_->d_counters[kCRep].cnt;
  ra.err = ctx_->d_err;
  k_rep_write<<<gr, kBlock, 0, st_>>>(ra);
  k_relabel_all<<<grid_for(n_), kBlock, 0, st_>>>(n_, P_, dense_of_, D_);
  tock(KAMSTA_PHASE_FINALIZE, tf);
  CU_TRY(cudaGetLastError());
  KS_TRY(fetch_counters());
  // compose: map + orig read, one gather, one write per round vertex; rep
  // scan: 16 per level vertex; relabel_all: 16 per vertex
  account(KAMSTA_PHASE_FINALIZE, composed * 16 + uint64_t(n0) * 16 + uint64_t(n_) * 16,
          static_cast<uint32_t>(r) + 2);
  nreps_ = static_cast<uint32_t>(ctx_->h_counters[kCRep].cnt[0]);
  std::swap(V_, Vn_);
  return KAMSTA_OK;
}

// ---------------------------------------------------------------------------
// sampling and planning

kamsta_status Solve::sample_weights(const SegList* L, uint32_t count, std::vector<uint32_t>* out) {
  out->clear();
  uint64_t m = L ? L->total : md_;
  if (!L && !input_complete_) {  // only the first piece of the input is there yet
    KS_TRY(wait_input(0));
    m = io_->piece_end[0];
  }
  if (m == 0) return KAMSTA_OK;
  count = std::min<uint32_t>(count, kSamples);
  const int g = grid_for(count);
  const int tp = tick();
  if (L) {
    std::vector<uint64_t> pre(L->nseg + 1, 0);
    for (uint32_t s = 0; s < L->nseg; ++s) pre[s + 1] = pre[s] + L->h_count[s];
    CU_TRY(cudaMemcpyAsync(prefix_, pre.data(), sizeof(uint64_t) * (L->nseg + 1),
                           cudaMemcpyHostToDevice, st_));
    k_sample_weights_seg<<<g, kBlock, 0, st_>>>(L->in(), prefix_, m, cfg_.seed, count, samples_);
  } else {
    k_sample_weights<<<g, kBlock, 0, st_>>>(in_, m, cfg_.seed, count, samples_);
  }
  tock(KAMSTA_PHASE_PLAN, tp);
  account(KAMSTA_PHASE_PLAN, uint64_t(count) * 8, 1);
  out->resize(count);
  CU_TRY(cudaMemcpyAsync(out->data(), samples_, count * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                         st_));
  CU_TRY(cudaStreamSynchronize(st_));
  resolve();
  std::sort(out->begin(), out->end());
  return KAMSTA_OK;
}

// Pivots of the light-first recursion of boruvka_filter_rec
// (local_mst_respecting_cut_edges.hpp:209-260): recurse while the level has
// more than 3n edges and its 25%-quantile split (mst_utils_filter.hpp:13-30)
// is balanced (mst_utils_filter.hpp:32-37).  Returned in descending order.
std::vector<uint32_t> Solve::plan_classes() {
  std::vector<uint32_t> thr;
  if (cfg_.local_preprocessing == KAMSTA_NO_PREPROCESSING) return thr;
  std::vector<uint32_t>& s = samples_host_;
  if (sample_weights(nullptr, kSamples, &s) != KAMSTA_OK) return thr;
  double m_est = static_cast<double>(md_) / 2.0;
  const double nv = static_cast<double>(n_);
  size_t len = s.size();
  // The split stops once the light part has at most 3n edges, the
  // reference's rule; any stop gives the same forest.  The batch's disjoint
  // unions (the only solves that mark the forest in a bitmap) stop at 2n:
  // on 1024 mixed graphs 78.6 against 86.0 ms, while single graphs are
  // fastest at 3n (GNM 2^26 deg 32 / deg 16, RGG-2D, RHG, R-MAT 2^24: 0-20%
  // slower at 2n).
  const double stop = forest_bits_ != nullptr ? 2.0 : 3.0;
  while (m_est > stop * nv && len >= 16) {
    const uint32_t pivot = s[static_cast<size_t>(len * 0.25)];
    const size_t light =
        static_cast<size_t>(std::upper_bound(s.begin(), s.begin() + len, pivot) - s.begin());
    const double frac = static_cast<double>(light) / static_cast<double>(len);
    if (std::abs(0.5 - (1.0 - frac)) > 0.4) break;  // is_unbalanced
    if (!thr.empty() && pivot >= thr.back()) break;
    thr.push_back(pivot);
    m_est *= frac;
    len = light;
  }
  return thr;
}

static double sample_share(const std::vector<uint32_t>& s, uint32_t lo, uint32_t hi) {
  if (s.empty()) return 1.0;
  const double k = static_cast<double>(std::upper_bound(s.begin(), s.end(), hi) -
                                       std::lower_bound(s.begin(), s.end(), lo));
  return k / static_cast<double>(s.size()) + 4.0 / static_cast<double>(s.size());
}

// ---------------------------------------------------------------------------
// contraction drivers

kamsta_status Solve::pick_big(uint32_t* label, bool* use) {
  *use = false;
  if (n_ < (1u << 16) || nreps_ <= 1) return KAMSTA_OK;
  const uint32_t count = kSamples;
  k_sample_labels<<<grid_for(count), kBlock, 0, st_>>>(n_, D_, cfg_.seed ^ launches_, count,
                                                       samples_);
  std::vector<uint32_t> h(count);
  CU_TRY(cudaMemcpyAsync(h.data(), samples_, count * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                         st_));
  CU_TRY(cudaStreamSynchronize(st_));
  std::sort(h.begin(), h.end());
  uint32_t best = 0, best_len = 0;
  for (size_t i = 0; i < h.size();) {
    size_t j = i;
    while (j < h.size() && h[j] == h[i]) ++j;
    if (j - i > best_len) {
      best_len = static_cast<uint32_t>(j - i);
      best = h[i];
    }
    i = j;
  }
  if (best_len * 2 < count) return KAMSTA_OK;  // no dominant component
  k_big_bitmap<<<grid_for(n_), kBlock, 0, st_>>>(n_, D_, best, big_);
  account(KAMSTA_PHASE_CLASS_PASS, uint64_t(n_) * 4 + n_ / 8 + count * 8, 2);
  *label = best;
  *use = true;
  return KAMSTA_OK;
}

kamsta_status Solve::contract_rows(uint32_t wmin, uint32_t wmax, SegList* E, bool* done) {
  *done = false;
  // the vertices outside the largest component
  const uint32_t cap_s = std::max<uint32_t>(1u << 16, n_ / 32);
  // outside vertices, their row starts, then the input's fence index
  const uint64_t nfence = (md_ + kFenceStep - 1) / kFenceStep;
  void* smem = nullptr;
  CU_TRY(ctx_alloc(ctx_, &smem, sizeof(uint32_t) * (2 * uint64_t(cap_s) + nfence + 1), st_));
  struct Free {
    void* p;
    cudaStream_t s;
    ~Free() {
      if (p) cudaFreeAsync(p, s);
    }
  } fs{smem, st_};
  uint32_t* S = static_cast<uint32_t*>(smem);
  uint32_t* row_lo = S + cap_s;
  uint32_t* fence = row_lo + cap_s;
  const int t0 = tick();
  CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCMisc, 0, sizeof(DevCounters), st_));
  unsigned long long* cnt = &ctx_->d_counters[kCMisc].cnt[0];
  k_outside_big<<<grid_for((n_ + 31) / 32), kBlock, 0, st_>>>(n_, big_, S, cap_s, cnt);
  KS_TRY(fetch_counters());
  const uint64_t ns = ctx_->h_counters[kCMisc].cnt[0];
  if (ns > cap_s) return KAMSTA_OK;  // too many: stream the input instead
  const int grid = grid_for(std::max<uint64_t>(ns * 32, 1));
  // records are ordered by (min id << key_bits | max id); the batch's forest
  // bitmap needs the src<dst copy's position in each record
  uint32_t key_bits = 1;
  while (key_bits < 32 && (1ull << key_bits) < n_) ++key_bits;
  const uint32_t canon = forest_bits_ != nullptr ? 1u : 0u;
  // count (and find the rows), then write the surviving edges
  k_fences<<<grid_for(nfence), kBlock, 0, st_>>>(in_, md_, fence);
  k_row_scan<false><<<grid, kBlock, 0, st_>>>(in_, md_, n_, S, static_cast<uint32_t>(ns), row_lo,
                                              fence, D_, big_, big_label_, wmin, wmax, canon,
                                              key_bits,
                                              nullptr, nullptr, 0,
                                              &ctx_->d_counters[kCMisc].cnt[1], ctx_->d_err);
  KS_TRY(fetch_counters());
  const uint64_t k = ctx_->h_counters[kCMisc].cnt[1];
  KS_TRY(alloc_list(E, 1, std::max<uint64_t>(k, 1)));
  if (k > 0) {
    void* tmem = nullptr;
    const RadixScratch rs = radix_scratch_bytes(k);
    const size_t rb = round_up(k * sizeof(Rec), 256), kb = round_up(k * 8, 256),
                 ib = round_up(k * 4, 256), cb = round_up(rs.counts * 4, 256),
                 sb = round_up(rs.status * 8, 256);
    CU_TRY(ctx_alloc(ctx_, &tmem, rb + 2 * kb + 2 * ib + cb + sb, st_));
    Free ft{tmem, st_};
    char* m = static_cast<char*>(tmem);
    Rec* tmp = reinterpret_cast<Rec*>(m);
    uint64_t* keys = reinterpret_cast<uint64_t*>(m + rb);
    uint64_t* keys2 = reinterpret_cast<uint64_t*>(m + rb + kb);
    uint32_t* idx = reinterpret_cast<uint32_t*>(m + rb + 2 * kb);
    uint32_t* idx2 = reinterpret_cast<uint32_t*>(m + rb + 2 * kb + ib);
    uint32_t* counts = reinterpret_cast<uint32_t*>(m + rb + 2 * kb + 2 * ib);
    uint64_t* status = reinterpret_cast<uint64_t*>(m + rb + 2 * kb + 2 * ib + cb);
    k_row_scan<true><<<grid, kBlock, 0, st_>>>(in_, md_, n_, S, static_cast<uint32_t>(ns), row_lo,
                                               fence, D_, big_, big_label_, wmin, wmax, canon,
                                               key_bits,
                                               tmp, keys, k, &ctx_->d_counters[kCMisc].cnt[2],
                                               ctx_->d_err);
    k_iota<<<grid_for(k), kBlock, 0, st_>>>(static_cast<uint32_t>(k), idx);
    int alt = 0;
    cudaError_t e = radix_sort_pairs_u32(st_, keys, keys2, idx, idx2, k,
                                         static_cast<int>(2 * key_bits), counts, status,
                                         &ctx_->d_counters[kCMisc].ticket, ctx_->d_err, &alt,
                                         sms_);
    if (e != cudaSuccess) return cuda_status(e, "radix sort (row scan)");
    if (alt) std::swap(idx, idx2);
    k_rec_place_min<<<grid_for(k), kBlock, 0, st_>>>(tmp, idx, k, E->base, minA_, big_label_);
    k_set_u32<<<1, 1, 0, st_>>>(E->d_count, static_cast<uint32_t>(k));
    KS_TRY(fetch_counters());  // also: the scratch above is released after use
  }
  E->h_count.assign(1, static_cast<uint32_t>(k));
  E->total = k;
  tock(KAMSTA_PHASE_CLASS_PASS, t0);
  // outside set, rows (entries of the scanned rows twice), kept records,
  // sort and placement
  account(KAMSTA_PHASE_CLASS_PASS, uint64_t(n_) / 8 + ns * 4 + k * (16 + 12 + 16 + 16 + 16), 6);
  ++row_scans_;
  *done = true;
  return KAMSTA_OK;
}

kamsta_status Solve::contract(const SegList* L, uint32_t wmin, uint32_t wmax, double frac) {
  if ((L && L->total == 0) || nreps_ <= 1) return KAMSTA_OK;
  fill_inf(minA_, nreps_);
  KS_TRY(pick_big(&big_label_, &use_big_));
  if (!L && use_big_) {  // heaviest class of the directed input: row scans
    SegList* E = new_list();
    bool done = false;
    KS_TRY(contract_rows(wmin, wmax, E, &done));
    if (done) {
      use_big_ = false;
      return rounds(E, true);
    }
  }
  SegList* E = new_list();
  SegList* outs[1] = {E};
  const double f[1] = {frac};
  const kamsta_status s = pass<1>(KAMSTA_PHASE_CLASS_PASS, L, D_, wmin, wmax, nullptr, outs, f,
                                  minA_, nreps_, false);
  use_big_ = false;
  KS_TRY(s);
  return rounds(E, true);
}

kamsta_status Solve::run_boruvka() {
  const std::vector<uint32_t>& b = bounds_;  // ascending class bounds
  const int K = static_cast<int>(b.size());
  const int nmat = std::max(1, std::min(K, kMaxOut));
  const uint32_t wmax0 = K == 0 ? 0xffffffffu : b[nmat - 1];
  // first pass: classes 0..nmat-1, class 0 with identity labels and the
  // round-0 minimum fused in
  fill_inf(minA_, n_);
  SegList* C[kMaxOut] = {new_list(), new_list(), new_list()};
  double frac[kMaxOut] = {1.0, 1.0, 1.0};
  if (K > 0)
    for (int c = 0; c < nmat; ++c)
      frac[c] = sample_share(samples_host_, c == 0 ? 0u : b[c - 1] + 1, b[c]);
  const bool validate = (cfg_.flags & KAMSTA_FLAG_VALIDATE) != 0;
  // direct emission: the first pass keys the round-0 minima by partner and
  // the first round writes its forest edges to the output
  direct_emit_ = d_out_ != nullptr && forest_bits_ == nullptr && n_ >= 2 && msf_count_ == 0;
  switch (nmat) {
    case 1:
      KS_TRY(pass<1>(KAMSTA_PHASE_FIRST_PASS, nullptr, nullptr, 0, wmax0, nullptr, C, frac, minA_,
                     n_, validate));
      break;
    case 2:
      KS_TRY(pass<2>(KAMSTA_PHASE_FIRST_PASS, nullptr, nullptr, 0, wmax0, b.data(), C, frac,
                     minA_, n_, validate));
      break;
    default:
      KS_TRY(pass<3>(KAMSTA_PHASE_FIRST_PASS, nullptr, nullptr, 0, wmax0, b.data(), C, frac,
                     minA_, n_, validate));
      break;
  }
  for (int c = 0; c < nmat; ++c) KS_TRY(debug_list("after first pass", *C[c], n_));
  // the last contraction skips the final label update (nothing reads it)
  const int steps = nmat + std::max(0, K - nmat + 1);
  int step = 0;
  final_contraction_ = ++step == steps;
  const kamsta_status first = rounds(C[0], true);
  direct_emit_ = false;
  KS_TRY(first);
  for (int c = 1; c < nmat; ++c) {
    final_contraction_ = ++step == steps;
    KS_TRY(contract(C[c], 0, 0xffffffffu, 1.0));
    free_list(C[c]);
  }
  for (int c = nmat; c <= K; ++c) {
    const uint32_t lo = b[c - 1] + 1;
    const uint32_t hi = c < K ? b[c] : 0xffffffffu;
    final_contraction_ = ++step == steps;
    KS_TRY(contract(nullptr, lo, hi, sample_share(samples_host_, lo, hi)));
  }
  final_contraction_ = false;
  return KAMSTA_OK;
}

// filter_boruvka's recursion (boruvka_recursive, hybrid_boruvka_edgefilter.hpp:
// 227-330): contract directly when the average degree is at most
// filter_threshold, the recursion was told to stop, or the graph is small;
// otherwise split at the median sampled weight (select_pivot,
// distributed_partitioning.hpp:91-119), recurse on the light part, relabel
// the heavy part by the components found and drop its internal edges
// (boruvka_recursive_setup, :173-225), recurse on what is left.  A light
// share above 85% stops the next level (partition_edges,
// filter_helpers.hpp:130-133).  L == nullptr is the directed input.
kamsta_status Solve::filter_rec(SegList* L, bool own, bool stop, int depth) {
  const uint64_t m_und = L ? L->total : md_ / 2;  // the input holds m_directed/2 edges
  if (m_und == 0 || nreps_ <= 1) {
    if (own) free_list(L);
    return KAMSTA_OK;
  }
  const double avg_degree = 2.0 * static_cast<double>(m_und) / static_cast<double>(n_);
  if (avg_degree <= static_cast<double>(cfg_.filter_threshold) || stop || 2 * m_und <= 1000 ||
      depth >= 48) {
    KS_TRY(contract(L, 0, 0xffffffffu, 1.0));
    if (own) free_list(L);
    return KAMSTA_OK;
  }
  std::vector<uint32_t> s;
  KS_TRY(sample_weights(L, kSamples, &s));
  const uint32_t pivot = s[s.size() / 2];
  SegList* light = new_list();
  SegList* heavy = new_list();
  SegList* outs[2] = {light, heavy};
  const double frac[2] = {sample_share(s, 0, pivot), 1.0};
  const uint32_t thr[1] = {pivot};
  KS_TRY(pass<2>(KAMSTA_PHASE_CLASS_PASS, L, nullptr, 0, 0xffffffffu, thr, outs, frac, nullptr, 0,
                 false));
  if (own) free_list(L);
  const uint64_t tot = light->total + heavy->total;
  const bool stop_next = tot == 0 || static_cast<double>(light->total) / tot > 0.85;
  KS_TRY(filter_rec(light, true, stop_next, depth + 1));
  if (nreps_ <= 1 || heavy->total == 0) {
    free_list(heavy);
    return KAMSTA_OK;
  }
  SegList* kept = new_list();
  SegList* kouts[1] = {kept};
  KS_TRY(pass<1>(KAMSTA_PHASE_CLASS_PASS, heavy, P_, 0, 0xffffffffu, nullptr, kouts, nullptr,
                 nullptr, 0, false));
  free_list(heavy);
  return filter_rec(kept, true, false, depth + 1);
}

kamsta_status Solve::run_filter_boruvka() { return filter_rec(nullptr, false, false, 0); }

// ---------------------------------------------------------------------------

kamsta_status Solve::run(Algo algo, kamsta_wedge* d_out, SolveOut* out) {
  out->count = 0;
  out->weight = 0;
  if (md_ >= (1ull << 32)) {
    set_error("input: more than 2^32-1 directed entries");
    return KAMSTA_E_INPUT;
  }
  if (n_ == 0 || md_ == 0) return KAMSTA_OK;
  int dev = 0;
  CU_TRY(cudaGetDevice(&dev));
  CU_TRY(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
  aligned16_ = (reinterpret_cast<uintptr_t>(in_) & 15u) == 0;
  // tiles: the call's cfg, else the context's tuned pair, else the defaults
  const uint32_t di = cfg_.items_per_thread ? cfg_.items_per_thread : ctx_->tune_dir_items;
  const uint32_t si = cfg_.seg_items_per_thread ? cfg_.seg_items_per_thread : ctx_->tune_seg_items;
  if (di == 6 || di == 8 || di == 12) dir_items_ = static_cast<int>(di);
  if (si == 2 || si == 4 || si == 8) seg_items_ = static_cast<int>(si);
  samples_ = ctx_->d_samples;
  {
    const char* dbg = std::getenv("KAMSTA_DEBUG_CHECKS");
    debug_ = dbg && dbg[0] == '1';
  }
  {  // per device context; cheap
    const int dr = static_cast<int>(rec_dyn_smem(8)), dr4 = static_cast<int>(rec_dyn_smem(4));
    const int d8 = static_cast<int>(dir_dyn_smem(8)), d12 = static_cast<int>(dir_dyn_smem(12)),
              d6 = static_cast<int>(dir_dyn_smem(6));
    const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
#define KAMSTA_DIR_ATTR(N, I, M, D) \
  CU_TRY(cudaFuncSetAttribute(k_pass_dir<N, I, M>, attr, D))
    KAMSTA_DIR_ATTR(1, 8, false, d8);
    KAMSTA_DIR_ATTR(2, 8, false, d8);
    KAMSTA_DIR_ATTR(3, 8, false, d8);
    KAMSTA_DIR_ATTR(1, 12, false, d12);
    KAMSTA_DIR_ATTR(2, 12, false, d12);
    KAMSTA_DIR_ATTR(3, 12, false, d12);
    KAMSTA_DIR_ATTR(1, 6, false, d6);
    KAMSTA_DIR_ATTR(2, 6, false, d6);
    KAMSTA_DIR_ATTR(3, 6, false, d6);
    KAMSTA_DIR_ATTR(1, 8, true, d8);
    KAMSTA_DIR_ATTR(2, 8, true, d8);
    KAMSTA_DIR_ATTR(3, 8, true, d8);
    KAMSTA_DIR_ATTR(1, 12, true, d12);
    KAMSTA_DIR_ATTR(2, 12, true, d12);
    KAMSTA_DIR_ATTR(3, 12, true, d12);
    KAMSTA_DIR_ATTR(1, 6, true, d6);
    KAMSTA_DIR_ATTR(2, 6, true, d6);
    KAMSTA_DIR_ATTR(3, 6, true, d6);
#undef KAMSTA_DIR_ATTR
    // the round passes (one output) may add up to kSminMax shared minima
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<1, 8>, attr, dr + int(kSminMax) * 8));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<2, 8>, attr, dr));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<3, 8>, attr, dr));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<1, 4>, attr, dr4 + int(kSminMax) * 8));
    const int dr2 = static_cast<int>(rec_dyn_smem(2));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<1, 2>, attr, dr2 + int(kSminMax) * 8));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<2, 2>, attr, dr2));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<3, 2>, attr, dr2));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<2, 4>, attr, dr4));
    CU_TRY(cudaFuncSetAttribute(k_pass_seg<3, 4>, attr, dr4));
  }
  KS_TRY(alloc_fixed());
  CU_TRY(cudaEventRecord(ctx_->ev0, st_));
  // filter_boruvka runs the local contraction first when local preprocessing
  // is requested (filter_boruvka_setup_and_preprocessing,
  // hybrid_boruvka_edgefilter.hpp:375-418); on one device that contraction
  // covers every edge, so the distributed recursion has nothing left.
  if (algo == Algo::kFilterBoruvka && cfg_.local_preprocessing != KAMSTA_NO_PREPROCESSING)
    algo = Algo::kBoruvka;
  // host input still arriving: the boruvka plan samples the first piece and
  // its first pass follows the pieces; everything else waits for all of it
  input_complete_ = !(io_ && io_->pieces > 0);
  if (!input_complete_ && algo != Algo::kBoruvka) {
    KS_TRY(wait_input(io_->pieces - 1));
    input_complete_ = true;
  }
  if (algo == Algo::kBoruvka) {
    std::vector<uint32_t> thr_desc = plan_classes();
    bounds_.assign(thr_desc.rbegin(), thr_desc.rend());
  }
  k_iota<<<grid_for(n_), kBlock, 0, st_>>>(n_, P_);
  k_iota<<<grid_for(n_), kBlock, 0, st_>>>(n_, V_);
  k_iota<<<grid_for(n_), kBlock, 0, st_>>>(n_, D_);
  account(KAMSTA_PHASE_FINALIZE, uint64_t(n_) * 12, 3);
  nreps_ = n_;
  msf_count_ = 0;
  d_out_ = d_out;
  direct_count_ = 0;
  CU_TRY(cudaMemsetAsync(dweight_, 0, sizeof(unsigned long long), st_));
  CU_TRY(cudaMemsetAsync(ctx_->d_err, 0, sizeof(uint32_t), st_));
  KS_TRY(algo == Algo::kBoruvka ? run_boruvka() : run_filter_boruvka());
  // forest output
  CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCMisc, 0, sizeof(DevCounters), st_));
  if (msf_count_ > 0 && forest_bits_) {
    const int tm = tick();
    // the weight stays 0 here: the caller's split sums it per graph
    k_mark_forest<<<grid_for(msf_count_), kBlock, 0, st_>>>(msf_count_, msf_, forest_bits_);
    tock(KAMSTA_PHASE_EMIT, tm);
    account(KAMSTA_PHASE_EMIT, msf_count_ * (4 + 4 + 4), 1);
  } else if (msf_count_ > 0) {
    // edges [0, direct_count_) are in d_out already; k_emit adds their weight
    const uint64_t k0 = direct_count_;
    const int tm = tick();
    k_emit<<<grid_for(msf_count_ - k0), kBlock, 0, st_>>>(
        msf_count_ - k0, msf_ + k0, in_, reinterpret_cast<uint32_t*>(d_out) + 3 * k0,
        &ctx_->d_counters[kCMisc].weight, k0 ? dweight_ : nullptr);
    tock(KAMSTA_PHASE_EMIT, tm);
    account(KAMSTA_PHASE_EMIT, (msf_count_ - k0) * (4 + 12 + 12), 1);
  }
  CU_TRY(cudaEventRecord(ctx_->ev1, st_));
  KS_TRY(fetch_counters());
  out->count = msf_count_;
  out->weight = ctx_->h_counters[kCMisc].weight;
  if (stats_) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx_->ev0, ctx_->ev1);
    stats_->num_mst_edges = out->count;
    stats_->total_weight = out->weight;
    stats_->rounds = rounds_;
    stats_->levels = levels_;
    stats_->dedupe_passes = dedupe_passes_;
    stats_->row_scans = row_scans_;
    stats_->gpu_launches = launches_;
    stats_->device_ms = ms;
    stats_->alg_bytes = alg_bytes_;
    for (int k = 0; k < KAMSTA_PHASES; ++k) {
      stats_->phase_ms[k] = phase_ms_[k];
      stats_->phase_bytes[k] = phase_bytes_[k];
      stats_->phase_launches[k] = phase_launches_[k];
    }
  }
  return KAMSTA_OK;
}

kamsta_status solve_device(kamsta_ctx* ctx, Algo algo, const kamsta_wedge* d_in,
                           uint64_t m_directed, uint32_t n, const kamsta_cfg& cfg,
                           kamsta_wedge* d_out, SolveOut* out, kamsta_stats* st,
                           cudaStream_t stream, uint32_t* d_forest_bits, HostIo* io) {
  if (st) std::memset(st, 0, sizeof(*st));
  Solve s(ctx, stream ? stream : ctx->stream, d_in, m_directed, n, cfg, st);
  s.forest_bits_ = d_forest_bits;
  s.io_ = io;
  return s.run(algo, d_out, out);
}

}  // namespace kamsta
