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
//       -> Solve::edge_pass(): heavier classes are relabelled by the current
//          components and internal edges dropped on the way into rounds().
//   boruvka_recursive   hybrid_boruvka_edgefilter.hpp:227-330
//       -> Solve::filter_rec(): host recursion over device edge lists.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "kernels.cuh"
#include "solver.cuh"

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

void Arena::release() {
  if (base) cudaFree(base);
  base = nullptr;
  cap = 0;
  off = 0;
}

#define KS_TRY(x)                          \
  do {                                     \
    const kamsta_status s_ = (x);          \
    if (s_ != KAMSTA_OK) return s_;        \
  } while (0)
#define CU_TRY(x)                                        \
  do {                                                   \
    const cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) return cuda_status(e_, #x);   \
  } while (0)

static inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
static inline uint32_t ceil_div(uint64_t a, uint64_t b) {
  return static_cast<uint32_t>((a + b - 1) / b);
}

constexpr uint32_t kTileDir = kItemsDir * kBlock;
constexpr uint32_t kTileRec = kItemsRec * kBlock;
constexpr uint32_t kTileVtx = kItemsVtx * kBlock;
constexpr uint32_t kSamples = 4096;

// Occupancy-derived persistent grid for the tile kernels.
template <typename K>
static int persistent_grid(K kernel, int sms, uint32_t ntiles) {
  static int per_sm = 0;  // one cache per kernel type K
  if (per_sm == 0) {
    int v = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, kBlock, 0);
    per_sm = v < 1 ? 1 : v;
  }
  const uint64_t g = static_cast<uint64_t>(per_sm) * sms;
  return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(g, ntiles)));
}

class Solve {
 public:
  Solve(kamsta_ctx* ctx, cudaStream_t st, const kamsta_wedge* in, uint64_t md,
        uint32_t n, const kamsta_cfg& cfg, kamsta_stats* stats)
      : ctx_(ctx), st_(st), in_(reinterpret_cast<const uint32_t*>(in)), md_(md),
        n_(n), cfg_(cfg), stats_(stats) {}

  kamsta_status run(Algo algo, kamsta_wedge* d_out, SolveOut* out);

 private:
  kamsta_status alloc_fixed();
  kamsta_status ensure_edges(uint64_t cap);
  kamsta_status fetch_counters(int first, int count);
  kamsta_status check_err();
  void fill_inf(uint64_t* p, uint64_t count);
  int grid_for(uint64_t items) const {
    const uint64_t g = (items + kBlock - 1) / kBlock;
    return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(g, uint64_t(sms_) * 8)));
  }
  // Edge passes.  Counts of the pass land in counts_[0..nout) (kept per class)
  // and counts_[kMaxOut] (dropped above wmax).
  template <int NOUT>
  kamsta_status pass_dir(uint64_t m, const uint32_t* map, uint32_t wmin, uint32_t wmax,
                         const uint32_t* thr, Rec* const* out, const uint64_t* cap,
                         uint64_t* minval, bool validate, uint64_t* counts);
  template <int NOUT>
  kamsta_status pass_rec(const Rec* in, uint64_t m, const uint32_t* map, uint32_t wmin,
                         uint32_t wmax, const uint32_t* thr, Rec* const* out,
                         const uint64_t* cap, uint64_t* minval, uint64_t* counts);
  // Boruvka rounds on list L (m0 edges, dense labels in [0, nreps_),
  // canonical order).  minA_ must hold the round-0 minima.
  kamsta_status rounds(Rec* L, uint64_t m0);
  // Relabel `L` (or the directed input when L == nullptr, weights in
  // [wmin, wmax]) into the current dense space and run rounds on the result.
  kamsta_status contract_list(const Rec* L, uint64_t m, uint32_t wmin, uint32_t wmax);
  std::vector<uint32_t> plan_classes();
  kamsta_status sample_weights(const Rec* L, uint64_t m, uint32_t count,
                               std::vector<uint32_t>* out);
  kamsta_status filter_rec(Rec* L, uint64_t m, bool stop, int depth);
  kamsta_status run_boruvka();
  kamsta_status run_filter_boruvka();
  void trace(uint64_t m, uint64_t n) {
    if (stats_ && (cfg_.flags & KAMSTA_FLAG_TRACE) && stats_->trace_len < KAMSTA_TRACE_MAX) {
      stats_->trace_m[stats_->trace_len] = m;
      stats_->trace_n[stats_->trace_len] = n;
      stats_->trace_len++;
    }
  }

  kamsta_ctx* ctx_;
  cudaStream_t st_;
  const uint32_t* in_;  // directed input as 32-bit words (3 per entry)
  uint64_t md_;
  uint32_t n_;
  kamsta_cfg cfg_;
  kamsta_stats* stats_;
  int sms_ = 1;
  uint32_t launches_ = 0;
  uint32_t rounds_ = 0;
  uint32_t levels_ = 0;
  uint64_t alg_bytes_ = 0;

  // vertex-side buffers (n_ entries unless noted)
  uint32_t *P_ = nullptr, *D_ = nullptr, *V_ = nullptr, *Vn_ = nullptr;
  uint32_t *dense_of_ = nullptr, *parent_ = nullptr, *msfoid_ = nullptr, *newid_ = nullptr;
  uint32_t *Rbuf_ = nullptr, *Obuf_ = nullptr, *msf_ = nullptr, *samples_ = nullptr;
  uint64_t *minA_ = nullptr, *minB_ = nullptr;
  uint64_t* status_[6] = {};
  uint32_t status_words_ = 0;  // capacity of each status array (tiles)
  Rec* C_[kMaxOut] = {};       // materialised weight classes
  uint64_t Ccap_[kMaxOut] = {};
  Rec *E1_ = nullptr, *E2_ = nullptr;
  uint64_t Ecap_ = 0;
  uint32_t nreps_ = 0;
  uint64_t msf_count_ = 0;
  bool aligned16_ = false;
  std::vector<uint32_t> bounds_;        // ascending weight-class bounds
  std::vector<uint32_t> samples_host_;  // sorted weight sample of the input
  bool tolerate_overflow_ = false;  // first pass: overflow means "resize"
  static constexpr kamsta_status kRetry = 1000;
};

kamsta_status Solve::alloc_fixed() {
  const uint64_t n = n_;
  const uint64_t mu = md_ / 2 + 1;
  const uint32_t tiles = std::max({ceil_div(md_, kTileDir), ceil_div(mu, kTileRec),
                                   ceil_div(n, kTileVtx), 1u});
  status_words_ = tiles;
  size_t bytes = 0;
  auto add = [&](uint64_t count, size_t sz) { bytes += round_up(count * sz, 256); };
  for (int i = 0; i < 9; ++i) add(n + 1, 4);        // P D V Vn dense parent msfoid newid msf
  add(2 * n + 64, 4);                               // Rbuf
  add(n + 64, 4);                                   // Obuf
  add(n + 1, 8);
  add(n + 1, 8);                                    // minA minB
  for (int i = 0; i < 6; ++i) add(tiles, 8);
  // class lists are estimated later; reserve a generous first guess here
  // and grow (re-run) if the first pass overflows.
  for (int i = 0; i < kMaxOut; ++i) add(Ccap_[i], sizeof(Rec));
  CU_TRY(ctx_->fixed.reserve(bytes + 4096));
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
  for (int i = 0; i < 6; ++i) status_[i] = A.take<uint64_t>(tiles);
  for (int i = 0; i < kMaxOut; ++i) C_[i] = Ccap_[i] ? A.take<Rec>(Ccap_[i]) : nullptr;
  if (!status_[5]) {
    set_error("internal: fixed arena too small");
    return KAMSTA_E_OOM;
  }
  return KAMSTA_OK;
}

kamsta_status Solve::ensure_edges(uint64_t cap) {
  cap = std::max<uint64_t>(cap, 1);
  const size_t bytes = 2 * round_up(cap * sizeof(Rec), 256) + 1024;
  CU_TRY(ctx_->edges.reserve(bytes));
  E1_ = ctx_->edges.take<Rec>(cap);
  E2_ = ctx_->edges.take<Rec>(cap);
  Ecap_ = cap;
  return KAMSTA_OK;
}

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

kamsta_status Solve::fetch_counters(int first, int count) {
  CU_TRY(cudaMemcpyAsync(ctx_->h_counters + first, ctx_->d_counters + first,
                         sizeof(DevCounters) * count, cudaMemcpyDeviceToHost, st_));
  CU_TRY(cudaMemcpyAsync(ctx_->h_err, ctx_->d_err, sizeof(uint32_t),
                         cudaMemcpyDeviceToHost, st_));
  CU_TRY(cudaStreamSynchronize(st_));
  return check_err();
}

void Solve::fill_inf(uint64_t* p, uint64_t count) {
  k_fill64<<<grid_for(count), kBlock, 0, st_>>>(count, p, kInf64);
  launches_++;
}

template <int NOUT>
kamsta_status Solve::pass_dir(uint64_t m, const uint32_t* map, uint32_t wmin, uint32_t wmax,
                              const uint32_t* thr, Rec* const* out, const uint64_t* cap,
                              uint64_t* minval, bool validate, uint64_t* counts) {
  const uint32_t ntiles = ceil_div(m, kTileDir);
  if (ntiles == 0) {
    for (int c = 0; c <= kMaxOut; ++c) counts[c] = 0;
    return KAMSTA_OK;
  }
  DevCounters* dc = ctx_->d_counters + kCEdge;
  CU_TRY(cudaMemsetAsync(dc, 0, sizeof(DevCounters), st_));
  for (int c = 0; c < NOUT; ++c)
    CU_TRY(cudaMemsetAsync(status_[c], 0, sizeof(uint64_t) * ntiles, st_));
  EdgePassArgs a{};
  a.map = map;
  a.wmin = wmin;
  a.wmax = wmax;
  for (int c = 0; c < NOUT - 1; ++c) a.thr[c] = thr[c];
  for (int c = 0; c < NOUT; ++c) {
    a.out[c] = out[c];
    a.cap[c] = cap[c];
    a.status[c] = status_[c];
  }
  a.minval = minval;
  a.counts = dc->cnt;
  a.ticket = &dc->ticket;
  a.err = ctx_->d_err;
  a.n = n_;
  a.validate = validate ? 1 : 0;
  a.aligned16 = aligned16_ ? 1 : 0;
  a.ntiles = ntiles;
  const int grid = persistent_grid(k_edge_pass_dir<NOUT>, sms_, ntiles);
  k_edge_pass_dir<NOUT><<<grid, kBlock, 0, st_>>>(in_, m, a);
  launches_++;
  CU_TRY(cudaGetLastError());
  KS_TRY(fetch_counters(kCEdge, 1));
  const DevCounters& h = ctx_->h_counters[kCEdge];
  uint64_t kept = 0;
  for (int c = 0; c <= kMaxOut; ++c) counts[c] = (c < NOUT || c == kMaxOut) ? h.cnt[c] : 0;
  for (int c = 0; c < NOUT; ++c) kept += counts[c];
  alg_bytes_ += m * 12 + kept * sizeof(Rec) + (map ? kept * 8 : 0) + (minval ? counts[0] * 16 : 0);
  return KAMSTA_OK;
}

template <int NOUT>
kamsta_status Solve::pass_rec(const Rec* in, uint64_t m, const uint32_t* map, uint32_t wmin,
                              uint32_t wmax, const uint32_t* thr, Rec* const* out,
                              const uint64_t* cap, uint64_t* minval, uint64_t* counts) {
  const uint32_t ntiles = ceil_div(m, kTileRec);
  if (ntiles == 0) {
    for (int c = 0; c <= kMaxOut; ++c) counts[c] = 0;
    return KAMSTA_OK;
  }
  DevCounters* dc = ctx_->d_counters + kCEdge;
  CU_TRY(cudaMemsetAsync(dc, 0, sizeof(DevCounters), st_));
  for (int c = 0; c < NOUT; ++c)
    CU_TRY(cudaMemsetAsync(status_[c], 0, sizeof(uint64_t) * ntiles, st_));
  EdgePassArgs a{};
  a.map = map;
  a.wmin = wmin;
  a.wmax = wmax;
  for (int c = 0; c < NOUT - 1; ++c) a.thr[c] = thr[c];
  for (int c = 0; c < NOUT; ++c) {
    a.out[c] = out[c];
    a.cap[c] = cap[c];
    a.status[c] = status_[c];
  }
  a.minval = minval;
  a.counts = dc->cnt;
  a.ticket = &dc->ticket;
  a.err = ctx_->d_err;
  a.n = n_;
  a.ntiles = ntiles;
  const int grid = persistent_grid(k_edge_pass_rec<NOUT>, sms_, ntiles);
  k_edge_pass_rec<NOUT><<<grid, kBlock, 0, st_>>>(in, m, a);
  launches_++;
  CU_TRY(cudaGetLastError());
  KS_TRY(fetch_counters(kCEdge, 1));
  const DevCounters& h = ctx_->h_counters[kCEdge];
  uint64_t kept = 0;
  for (int c = 0; c <= kMaxOut; ++c) counts[c] = (c < NOUT || c == kMaxOut) ? h.cnt[c] : 0;
  for (int c = 0; c < NOUT; ++c) kept += counts[c];
  alg_bytes_ += m * sizeof(Rec) + kept * sizeof(Rec) + (map ? m * 8 : 0) +
                (minval ? counts[0] * 16 : 0);
  return KAMSTA_OK;
}

// Boruvka rounds (boruvka3).  One host read per round: the new edge count,
// vertex count and forest-edge count.
kamsta_status Solve::rounds(Rec* L, uint64_t m0) {
  levels_++;
  const uint32_t n0 = nreps_;
  Rec* cur = L;
  Rec* bufs[2] = {E1_, E2_};
  int nb = (cur == E1_) ? 1 : 0;
  uint64_t m = m0;
  uint32_t nr = n0;
  uint64_t* minv = minA_;
  uint64_t* minn = minB_;
  ChaseArgs ca{};
  ca.n0 = n0;
  ca.orig[0] = V_;
  size_t roff = 0, ooff = 0;
  uint32_t r = 0;
  const uint32_t* orig_cur = V_;
  while (m > 0) {
    if (r >= static_cast<uint32_t>(kMaxRounds)) {
      set_error("round cap reached");
      return KAMSTA_E_NOCONVERGE;
    }
    trace(m, nr);
    CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCVertex, 0, 2 * sizeof(DevCounters), st_));
    const int gv = grid_for(nr);
    k_hook<<<gv, kBlock, 0, st_>>>(nr, minv, cur, parent_, msfoid_, ctx_->d_err);
    k_jump<<<gv, kBlock, 0, st_>>>(nr, parent_, ctx_->d_err);
    const uint32_t ntv = ceil_div(nr, kTileVtx);
    CU_TRY(cudaMemsetAsync(status_[3], 0, sizeof(uint64_t) * ntv, st_));
    CU_TRY(cudaMemsetAsync(status_[4], 0, sizeof(uint64_t) * ntv, st_));
    uint32_t* onext = Obuf_ + ooff;
    VertexScanArgs va{};
    va.n = nr;
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
    va.status[0] = status_[3];
    va.status[1] = status_[4];
    va.counts = ctx_->d_counters[kCVertex].cnt;
    va.ticket = &ctx_->d_counters[kCVertex].ticket;
    va.err = ctx_->d_err;
    va.ntiles = ntv;
    k_vertex_scan<<<persistent_grid(k_vertex_scan, sms_, ntv), kBlock, 0, st_>>>(va);
    uint32_t* R = Rbuf_ + roff;
    k_map<<<gv, kBlock, 0, st_>>>(nr, minv, parent_, newid_, R);
    launches_ += 4;
    // relabel + self-loop removal + compaction + next-round minimum
    const uint32_t ntiles = ceil_div(m, kTileRec);
    CU_TRY(cudaMemsetAsync(status_[0], 0, sizeof(uint64_t) * ntiles, st_));
    Rec* nxt = bufs[nb];
    EdgePassArgs a{};
    a.map = R;
    a.wmin = 0;
    a.wmax = 0xffffffffu;
    a.out[0] = nxt;
    a.cap[0] = Ecap_;
    a.status[0] = status_[0];
    a.minval = minn;
    a.counts = ctx_->d_counters[kCEdge].cnt;
    a.ticket = &ctx_->d_counters[kCEdge].ticket;
    a.err = ctx_->d_err;
    a.ntiles = ntiles;
    k_edge_pass_rec<1><<<persistent_grid(k_edge_pass_rec<1>, sms_, ntiles), kBlock, 0, st_>>>(
        cur, m, a);
    launches_++;
    CU_TRY(cudaGetLastError());
    KS_TRY(fetch_counters(kCVertex, 2));
    const uint64_t n_next = ctx_->h_counters[kCVertex].cnt[0];
    const uint64_t added = ctx_->h_counters[kCVertex].cnt[1];
    const uint64_t m_next = ctx_->h_counters[kCEdge].cnt[0];
    alg_bytes_ += uint64_t(nr) * (40 + 8 + 16 + 20) + n_next * 16 + added * 4;
    alg_bytes_ += m * (sizeof(Rec) + 8) + m_next * (sizeof(Rec) + 16);
    msf_count_ += added;
    if (msf_count_ > n_) {
      set_error("internal: forest larger than n-1");
      return KAMSTA_E_CUDA;
    }
    ca.R[r] = R;
    ca.orig[r + 1] = onext;
    roff += nr;
    ooff += n_next;
    orig_cur = onext;
    cur = nxt;
    nb ^= 1;
    m = m_next;
    nr = static_cast<uint32_t>(n_next);
    std::swap(minv, minn);
    ++r;
  }
  rounds_ += r;
  if (r == 0) return KAMSTA_OK;  // nothing contracted; labels unchanged
  ca.rounds = r;
  ca.P = P_;
  ca.err = ctx_->d_err;
  k_chase<<<grid_for(n0), kBlock, 0, st_>>>(ca);
  const uint32_t ntv = ceil_div(n0, kTileVtx);
  CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCRep, 0, sizeof(DevCounters), st_));
  CU_TRY(cudaMemsetAsync(status_[5], 0, sizeof(uint64_t) * ntv, st_));
  RepScanArgs ra{};
  ra.n = n0;
  ra.V = V_;
  ra.P = P_;
  ra.Vout = Vn_;
  ra.dense_of = dense_of_;
  ra.status = status_[5];
  ra.counts = ctx_->d_counters[kCRep].cnt;
  ra.ticket = &ctx_->d_counters[kCRep].ticket;
  ra.err = ctx_->d_err;
  ra.ntiles = ntv;
  k_rep_scan<<<persistent_grid(k_rep_scan, sms_, ntv), kBlock, 0, st_>>>(ra);
  k_relabel_all<<<grid_for(n_), kBlock, 0, st_>>>(n_, P_, dense_of_, D_);
  launches_ += 3;
  CU_TRY(cudaGetLastError());
  KS_TRY(fetch_counters(kCRep, 1));
  alg_bytes_ += uint64_t(n0) * (4 * r + 12) + uint64_t(n0) * 16 + uint64_t(n_) * 16;
  nreps_ = static_cast<uint32_t>(ctx_->h_counters[kCRep].cnt[0]);
  std::swap(V_, Vn_);
  return KAMSTA_OK;
}

kamsta_status Solve::sample_weights(const Rec* L, uint64_t m, uint32_t count,
                                    std::vector<uint32_t>* out) {
  out->clear();
  if (m == 0) return KAMSTA_OK;
  count = std::min<uint32_t>(count, kSamples);
  const int g = grid_for(count);
  if (L)
    k_sample_weights_rec<<<g, kBlock, 0, st_>>>(L, m, cfg_.seed, count, samples_);
  else
    k_sample_weights<<<g, kBlock, 0, st_>>>(in_, m, cfg_.seed, count, samples_);
  launches_++;
  out->resize(count);
  CU_TRY(cudaMemcpyAsync(out->data(), samples_, count * sizeof(uint32_t),
                         cudaMemcpyDeviceToHost, st_));
  CU_TRY(cudaStreamSynchronize(st_));
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
  if (sample_weights(nullptr, md_, kSamples, &s) != KAMSTA_OK) return thr;
  double m_est = static_cast<double>(md_) / 2.0;
  const double nv = static_cast<double>(n_);
  size_t len = s.size();
  while (m_est > 3.0 * nv && len >= 16) {
    const uint32_t pivot = s[static_cast<size_t>(len * 0.25)];
    const size_t light = static_cast<size_t>(
        std::upper_bound(s.begin(), s.begin() + len, pivot) - s.begin());
    const double frac = static_cast<double>(light) / static_cast<double>(len);
    if (std::abs(0.5 - (1.0 - frac)) > 0.4) break;  // is_unbalanced
    if (!thr.empty() && pivot >= thr.back()) break;
    thr.push_back(pivot);
    m_est *= frac;
    len = light;
  }
  return thr;
}

// Relabel a list (or the directed input) into the current dense labels with
// the next minimum fused in, then contract it.
kamsta_status Solve::contract_list(const Rec* L, uint64_t m, uint32_t wmin, uint32_t wmax) {
  if (m == 0 || nreps_ <= 1) return KAMSTA_OK;
  fill_inf(minA_, nreps_);
  uint64_t counts[kMaxOut + 1];
  Rec* out[1] = {E1_};
  const uint64_t cap[1] = {Ecap_};
  if (L)
    KS_TRY(pass_rec<1>(L, m, D_, wmin, wmax, nullptr, out, cap, minA_, counts));
  else
    KS_TRY(pass_dir<1>(md_, D_, wmin, wmax, nullptr, out, cap, minA_, false, counts));
  if (counts[0] == 0) return KAMSTA_OK;
  return rounds(E1_, counts[0]);
}

kamsta_status Solve::run_boruvka() {
  const std::vector<uint32_t>& b = bounds_;  // ascending class bounds
  const int K = static_cast<int>(b.size());
  const int nmat = std::max(1, std::min(K, kMaxOut));
  const uint32_t wmax0 = K == 0 ? 0xffffffffu : b[nmat - 1];
  // first pass: classes 0..nmat-1, class 0 with identity labels and the
  // round-0 minimum fused in
  fill_inf(minA_, n_);
  uint64_t counts[kMaxOut + 1];
  const bool validate = (cfg_.flags & KAMSTA_FLAG_VALIDATE) != 0;
  tolerate_overflow_ = true;
  switch (nmat) {
    case 1:
      KS_TRY(pass_dir<1>(md_, nullptr, 0, wmax0, nullptr, C_, Ccap_, minA_, validate, counts));
      break;
    case 2:
      KS_TRY(pass_dir<2>(md_, nullptr, 0, wmax0, b.data(), C_, Ccap_, minA_, validate, counts));
      break;
    default:
      KS_TRY(pass_dir<3>(md_, nullptr, 0, wmax0, b.data(), C_, Ccap_, minA_, validate, counts));
      break;
  }
  tolerate_overflow_ = false;
  bool overflow = false;
  for (int c = 0; c < nmat; ++c) overflow |= counts[c] > Ccap_[c];
  if (overflow) {  // the sample under-estimated a class: rerun with exact sizes
    for (int c = 0; c < nmat; ++c) Ccap_[c] = counts[c];
    return kRetry;
  }
  uint64_t ecap = counts[kMaxOut];
  for (int c = 0; c < nmat; ++c) ecap = std::max(ecap, counts[c]);
  KS_TRY(ensure_edges(ecap));
  KS_TRY(rounds(C_[0], counts[0]));
  for (int c = 1; c < nmat; ++c)
    KS_TRY(contract_list(C_[c], counts[c], 0, 0xffffffffu));
  for (int c = nmat; c <= K; ++c) {
    const uint32_t lo = b[c - 1] + 1;
    const uint32_t hi = c < K ? b[c] : 0xffffffffu;
    KS_TRY(contract_list(nullptr, md_, lo, hi));
  }
  return KAMSTA_OK;
}

kamsta_status Solve::filter_rec(Rec* L, uint64_t m, bool stop, int depth) {
  (void)L;
  (void)m;
  (void)stop;
  (void)depth;
  set_error("filter_boruvka: not built yet");
  return KAMSTA_E_UNSUPPORTED;
}

kamsta_status Solve::run_filter_boruvka() { return filter_rec(nullptr, md_ / 2, false, 0); }

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
  samples_ = ctx_->d_samples;
  CU_TRY(cudaEventRecord(ctx_->ev0, st_));
  const uint64_t mu = md_ / 2 + 1;
  if (algo == Algo::kBoruvka) {
    // class bounds (ascending) and class-list capacities from the sample
    std::vector<uint32_t> thr_desc = plan_classes();
    bounds_.assign(thr_desc.rbegin(), thr_desc.rend());
    const int K = static_cast<int>(bounds_.size());
    const int nmat = std::max(1, std::min(K, kMaxOut));
    for (int c = 0; c < kMaxOut; ++c) Ccap_[c] = 0;
    if (K == 0) {
      Ccap_[0] = mu;
    } else {
      const double S = static_cast<double>(std::max<size_t>(samples_host_.size(), 1));
      for (int c = 0; c < nmat; ++c) {
        const uint32_t lo = c == 0 ? 0u : bounds_[c - 1] + 1;
        const uint32_t hi = bounds_[c];
        const double k = static_cast<double>(
            std::upper_bound(samples_host_.begin(), samples_host_.end(), hi) -
            std::lower_bound(samples_host_.begin(), samples_host_.end(), lo));
        const double f = k / S;
        const double est = f + 6.0 * std::sqrt(f * (1.0 - f) / S + 1.0 / (S * S)) + 4.0 / S;
        Ccap_[c] = std::min<uint64_t>(mu, static_cast<uint64_t>(est * static_cast<double>(mu)) + 4096);
      }
    }
  }
  for (int attempt = 0;; ++attempt) {
    KS_TRY(alloc_fixed());
    k_iota<<<grid_for(n_), kBlock, 0, st_>>>(n_, P_);
    k_iota<<<grid_for(n_), kBlock, 0, st_>>>(n_, V_);
    k_iota<<<grid_for(n_), kBlock, 0, st_>>>(n_, D_);
    launches_ += 3;
    nreps_ = n_;
    msf_count_ = 0;
    CU_TRY(cudaMemsetAsync(ctx_->d_err, 0, sizeof(uint32_t), st_));
    const kamsta_status s = algo == Algo::kBoruvka ? run_boruvka() : run_filter_boruvka();
    if (s == kRetry && attempt == 0) continue;
    if (s == kRetry) {
      set_error("internal: class buffer overflow after resize");
      return KAMSTA_E_CUDA;
    }
    KS_TRY(s);
    break;
  }
  // forest output
  CU_TRY(cudaMemsetAsync(ctx_->d_counters + kCMisc, 0, sizeof(DevCounters), st_));
  if (msf_count_ > 0) {
    k_emit<<<grid_for(msf_count_), kBlock, 0, st_>>>(
        msf_count_, msf_, in_, reinterpret_cast<uint32_t*>(d_out),
        &ctx_->d_counters[kCMisc].weight);
    launches_++;
  }
  CU_TRY(cudaEventRecord(ctx_->ev1, st_));
  KS_TRY(fetch_counters(kCMisc, 1));
  alg_bytes_ += msf_count_ * (4 + 12 + 12);
  out->count = msf_count_;
  out->weight = ctx_->h_counters[kCMisc].weight;
  if (stats_) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx_->ev0, ctx_->ev1);
    stats_->num_mst_edges = out->count;
    stats_->total_weight = out->weight;
    stats_->rounds = rounds_;
    stats_->levels = levels_;
    stats_->gpu_launches = launches_;
    stats_->device_ms = ms;
    stats_->alg_bytes = alg_bytes_;
  }
  return KAMSTA_OK;
}

kamsta_status solve_device(kamsta_ctx* ctx, Algo algo, const kamsta_wedge* d_in,
                           uint64_t m_directed, uint32_t n, const kamsta_cfg& cfg,
                           kamsta_wedge* d_out, SolveOut* out, kamsta_stats* st,
                           cudaStream_t stream) {
  if (st) {
    std::memset(st, 0, sizeof(*st));
  }
  Solve s(ctx, stream ? stream : ctx->stream, d_in, m_directed, n, cfg, st);
  return s.run(algo, d_out, out);
}

}  // namespace kamsta
