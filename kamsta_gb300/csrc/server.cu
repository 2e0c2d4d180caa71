// server.cu -- continuous-batching request loop for MST jobs.
//
// Clients submit jobs (device edge arrays, device output buffers) at any
// time; worker threads, each with its own context and stream, repeatedly
// take whatever is queued, in arrival order, as long as the summed device
// footprint of the admitted jobs stays under the memory budget, and solve
// them as one wave (batch.cu: disjoint union -> one solve -> per-graph
// split).  The budget is enforced, not only estimated: each worker's
// context carries a memory limit of budget / workers (every pool
// allocation and arena growth is checked against it), a wave is admitted
// only within that share, and the peak each worker's context held is
// recorded per wave (kamsta_server_memory).  A job that arrives while a wave is on the GPU joins the next wave
// of the first worker that frees up, so with two or more workers waves
// overlap on the device.  Completions carry submit / start / finish times
// (steady clock) for latency accounting.
//
// The reference has no serving loop (its benchmark runs one graph per MPI
// job, benchmarks/mst.cpp:215-228); per job the result equals the batch
// entry point on that graph alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.cuh"
#include "solver.cuh"

struct kamsta_server {
  struct Job {
    kamsta_request req;
    uint64_t ticket;
    uint64_t bytes;
    double submit_us;
  };
  int device = 0;
  kamsta_server_cfg cfg{};
  kamsta_cfg scfg{};
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work;  // jobs queued / stop
  std::condition_variable cv_done;  // completions / memory freed
  std::deque<Job> queue;
  std::deque<kamsta_completion> done;
  uint64_t next_ticket = 1;
  uint64_t bytes_in_use = 0;
  uint64_t in_flight = 0;
  uint64_t waves = 0;
  uint64_t worker_limit = 0;  // budget / workers: each worker context's memory limit
  uint64_t peak_worker_bytes = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  std::vector<kamsta_ctx*> ctxs;

  double now_us() const {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0)
        .count();
  }
  void worker(int w);
};

namespace kamsta {
namespace {
constexpr uint64_t kServerDefaultBudget = 64ull << 30;
constexpr uint32_t kServerDefaultMaxBatch = 4096;

// The most device memory the context held during the last wave (pool
// high-water mark plus its arenas); resets the pool's high-water mark.
uint64_t wave_peak_bytes(kamsta_ctx* ctx) {
  uint64_t high = 0, zero = 0;
  if (ctx->pool) {
    cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemHigh, &high);
    cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrUsedMemHigh, &zero);
  }
  return high + ctx->fixed.cap + ctx->io.cap;
}
}  // namespace
}  // namespace kamsta

void kamsta_server::worker(int w) {
  using namespace kamsta;
  cudaSetDevice(device);
  kamsta_ctx* ctx = ctxs[w];
  const Algo algo = (scfg.flags & KAMSTA_FLAG_FILTER) ? Algo::kFilterBoruvka : Algo::kBoruvka;
  std::vector<Job> batch;
  std::vector<kamsta_graph_desc> descs;
  for (;;) {
    batch.clear();
    uint64_t bytes = 0;
    bool more = false;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] {
        if (stop && queue.empty()) return true;
        // admit the queue head once its footprint fits the free budget
        return !queue.empty() && bytes_in_use + queue.front().bytes <= cfg.budget_bytes;
      });
      if (queue.empty()) return;  // stop requested and drained
      // take jobs in arrival order while they fit the free budget and this
      // worker's share of it (the head always fits the share: submit checks)
      while (!queue.empty() && batch.size() < cfg.max_batch &&
             bytes_in_use + bytes + queue.front().bytes <= cfg.budget_bytes &&
             bytes + queue.front().bytes <= worker_limit) {
        bytes += queue.front().bytes;
        batch.push_back(queue.front());
        queue.pop_front();
      }
      bytes_in_use += bytes;
      in_flight += batch.size();
      ++waves;
      more = !queue.empty();
    }
    if (more) cv_work.notify_one();  // more work for another worker
    // small jobs first (one persistent launch, finished in well under a
    // millisecond), then the rest as one union solve; each group completes
    // as soon as it is done
    std::stable_partition(batch.begin(), batch.end(), [ctx](const Job& j) {
      kamsta_graph_desc d{};
      d.m_directed = j.req.m_directed;
      d.n = j.req.n;
      return is_small_graph(ctx, d);
    });
    size_t first_large = 0;
    while (first_large < batch.size()) {
      kamsta_graph_desc d{};
      d.m_directed = batch[first_large].req.m_directed;
      d.n = batch[first_large].req.n;
      if (!is_small_graph(ctx, d)) break;
      ++first_large;
    }
    const size_t groups[3] = {0, first_large, batch.size()};
    for (int grp = 0; grp < 2; ++grp) {
      const size_t a = groups[grp], z = groups[grp + 1];
      if (a == z) continue;
      const double start = now_us();
      descs.resize(z - a);
      uint64_t gbytes = 0;
      for (size_t i = a; i < z; ++i) {
        kamsta_graph_desc& d = descs[i - a];
        d = kamsta_graph_desc{};
        d.edges = batch[i].req.d_edges;
        d.m_directed = batch[i].req.m_directed;
        d.n = batch[i].req.n;
        d.out = batch[i].req.d_out;
        gbytes += batch[i].bytes;
      }
      BatchWaveStats ws;
      kamsta_status s;
      uint64_t peak = 0;
      {
        std::lock_guard<std::mutex> clk(ctx->mu);
        s = solve_wave(ctx, algo, descs.data(), static_cast<uint32_t>(descs.size()), scfg, false,
                       ctx->stream, &ws);
        peak = wave_peak_bytes(ctx);
      }
      if (s == KAMSTA_E_OOM && z - a > 1) {
        // the estimate was short for this mix: give the cached arenas back
        // and solve the jobs one at a time under the same limit
        kamsta_ctx_trim(ctx);
        s = KAMSTA_OK;
        for (auto& d : descs) {
          std::lock_guard<std::mutex> clk(ctx->mu);
          const kamsta_status s1 = solve_wave(ctx, algo, &d, 1, scfg, false, ctx->stream, &ws);
          if (s1 != KAMSTA_OK) d.status = s1;
          peak = std::max(peak, wave_peak_bytes(ctx));
        }
      }
      const double finish = now_us();
      std::lock_guard<std::mutex> lk(mu);
      peak_worker_bytes = std::max(peak_worker_bytes, peak);
      for (size_t i = a; i < z; ++i) {
        const kamsta_graph_desc& d = descs[i - a];
        kamsta_completion c{};
        c.ticket = batch[i].ticket;
        c.user_tag = batch[i].req.user_tag;
        c.status = s != KAMSTA_OK ? s : d.status;
        c.out_count = s == KAMSTA_OK ? d.out_count : 0;
        c.total_weight = s == KAMSTA_OK ? d.total_weight : 0;
        c.batch_size = static_cast<uint32_t>(batch.size());
        c.submit_us = batch[i].submit_us;
        c.start_us = start;
        c.finish_us = finish;
        done.push_back(c);
      }
      bytes_in_use -= gbytes;
      in_flight -= z - a;
      cv_done.notify_all();
    }
    cv_done.notify_all();
    cv_work.notify_all();
  }
}

using namespace kamsta;

extern "C" {

kamsta_status kamsta_server_cfg_default(kamsta_server_cfg* cfg) {
  if (!cfg) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->budget_bytes = kServerDefaultBudget;
  cfg->max_batch = kServerDefaultMaxBatch;
  cfg->workers = 2;
  kamsta_cfg_default(&cfg->solver);
  return KAMSTA_OK;
}

kamsta_status kamsta_server_create(int device, const kamsta_server_cfg* cfg,
                                   kamsta_server** out) {
  if (!out) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  *out = nullptr;
  kamsta_server_cfg c;
  kamsta_server_cfg_default(&c);
  if (cfg) c = *cfg;
  if (c.budget_bytes == 0) c.budget_bytes = kServerDefaultBudget;
  if (c.max_batch == 0) c.max_batch = kServerDefaultMaxBatch;
  if (c.workers == 0) c.workers = 1;
  if (c.workers > 8) {
    set_error("server: at most 8 workers");
    return KAMSTA_E_INPUT;
  }
  if (c.solver.compression != KAMSTA_NO_COMPRESSION &&
      c.solver.compression != KAMSTA_SEVEN_BIT_DIFF_ENCODING) {
    set_error("compression: unknown value");
    return KAMSTA_E_INPUT;
  }
  auto* s = new kamsta_server();
  s->device = device;
  s->cfg = c;
  s->worker_limit = c.budget_bytes / c.workers;
  s->scfg = c.solver;
  s->scfg.flags &= ~KAMSTA_FLAG_SORT_OUTPUT;
  s->t0 = std::chrono::steady_clock::now();
  for (uint32_t w = 0; w < c.workers; ++w) {
    kamsta_ctx* ctx = nullptr;
    const kamsta_status st = kamsta_ctx_create(device, &ctx);
    if (st != KAMSTA_OK) {
      for (auto* p : s->ctxs) kamsta_ctx_destroy(p);
      delete s;
      return st;
    }
    // the worker's share of the budget is a hard limit on what its context
    // holds; cached pool memory above it goes back to the device at the
    // wave's synchronisation points
    uint64_t keep = c.budget_bytes / c.workers;
    kamsta_ctx_set_memory_limit(ctx, keep);
    cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    kamsta_tuning tune{};
    tune.small_threads = c.small_threads;
    tune.small_max_n = c.small_max_n;
    if (kamsta_ctx_set_tuning(ctx, &tune) != KAMSTA_OK) {
      for (auto* p : s->ctxs) kamsta_ctx_destroy(p);
      kamsta_ctx_destroy(ctx);
      delete s;
      return KAMSTA_E_INPUT;
    }
    s->ctxs.push_back(ctx);
  }
  for (uint32_t w = 0; w < c.workers; ++w)
    s->workers.emplace_back([s, w] { s->worker(static_cast<int>(w)); });
  *out = s;
  return KAMSTA_OK;
}

kamsta_status kamsta_server_submit(kamsta_server* s, const kamsta_request* req,
                                   uint64_t* ticket) {
  if (!s || !req || (req->m_directed && !req->d_edges) || (req->n > 1 && !req->d_out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  if (req->n >= kBatchMaxVertices) {
    set_error("server: n too large");
    return KAMSTA_E_INPUT;
  }
  kamsta_graph_desc g{};
  g.m_directed = req->m_directed;
  g.n = req->n;
  const uint64_t bytes = serve_job_bytes(s->ctxs[0], g);
  if (bytes > s->worker_limit) {
    set_error("server: request needs more device memory than one worker's share of the "
              "budget (budget_bytes / workers)");
    return KAMSTA_E_BUDGET;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
      set_error("server: shutting down");
      return KAMSTA_E_INPUT;
    }
    kamsta_server::Job j{*req, s->next_ticket++, bytes, s->now_us()};
    if (ticket) *ticket = j.ticket;
    s->queue.push_back(j);
  }
  s->cv_work.notify_one();
  return KAMSTA_OK;
}

kamsta_status kamsta_server_poll(kamsta_server* s, kamsta_completion* out, uint32_t cap,
                                 uint32_t* count, uint32_t timeout_us) {
  if (!s || !count || (cap && !out)) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  *count = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && timeout_us)
    s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us),
                        [&] { return !s->done.empty(); });
  uint32_t k = 0;
  while (k < cap && !s->done.empty()) {
    out[k++] = s->done.front();
    s->done.pop_front();
  }
  *count = k;
  if (k == 0) {
    set_error("server: nothing finished yet");
    return KAMSTA_E_NOTREADY;
  }
  return KAMSTA_OK;
}

kamsta_status kamsta_server_cancel(kamsta_server* s, uint64_t ticket) {
  if (!s) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = std::find_if(s->queue.begin(), s->queue.end(),
                         [ticket](const kamsta_server::Job& j) { return j.ticket == ticket; });
  if (it == s->queue.end()) {
    set_error("ticket not queued (in a wave, finished or unknown)");
    return KAMSTA_E_NOTREADY;
  }
  kamsta_completion c{};
  c.ticket = it->ticket;
  c.user_tag = it->req.user_tag;
  c.status = KAMSTA_E_CANCELLED;
  c.submit_us = it->submit_us;
  c.start_us = c.finish_us = s->now_us();
  s->queue.erase(it);
  s->done.push_back(c);
  s->cv_done.notify_all();
  s->cv_work.notify_all();  // the queue head may fit the budget now
  return KAMSTA_OK;
}

kamsta_status kamsta_server_stats(kamsta_server* s, uint64_t* queued, uint64_t* in_flight,
                                  uint64_t* bytes_in_use, uint64_t* waves) {
  if (!s) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = s->queue.size();
  if (in_flight) *in_flight = s->in_flight;
  if (bytes_in_use) *bytes_in_use = s->bytes_in_use;
  if (waves) *waves = s->waves;
  return KAMSTA_OK;
}

kamsta_status kamsta_server_memory(kamsta_server* s, uint64_t* worker_limit,
                                   uint64_t* peak_worker_bytes) {
  if (!s) {
    set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (worker_limit) *worker_limit = s->worker_limit;
  if (peak_worker_bytes) *peak_worker_bytes = s->peak_worker_bytes;
  return KAMSTA_OK;
}

kamsta_status kamsta_server_destroy(kamsta_server* s) {
  if (!s) return KAMSTA_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  for (auto* c : s->ctxs) kamsta_ctx_destroy(c);
  delete s;
  return KAMSTA_OK;
}

}  // extern "C"
