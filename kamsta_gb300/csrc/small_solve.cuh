// small_solve.cuh -- the whole MSF solve of a small graph inside one CTA.
//
// Used by kamsta_mst_boruvka_noalloc (one CTA, a static scratch array) and by
// the batched path (a persistent kernel whose CTAs take small graphs from a
// work queue, each CTA with its own scratch slot).  The rounds are those of
// the multi-kernel solver -- hook along the minimum edge (of a mutual pair the
// lower label stays root), pointer jumping, renumbering of live roots,
// relabel + self-loop removal + stable compaction with the fused next-round
// minimum -- and the tie-break is the same: lists stay in input order, so
// (w << 32 | position) orders edges by (w, min, max).
#pragma once
#include "common.cuh"

namespace kamsta {
namespace small {

constexpr uint32_t kMaxN = 1u << 15;
constexpr uint64_t kMaxMd = 1ull << 18;
constexpr uint32_t kMaxMu = static_cast<uint32_t>(kMaxMd / 2);  // src<dst copies
constexpr uint32_t kMaxRounds = 40;

// Scratch layout (bytes, 256-aligned).
constexpr size_t kHdr = 256;  // Result
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
constexpr size_t kOffFlags = kOffMsf + size_t(kMaxN) * 4;  // one bit per input entry
constexpr size_t kScratchBytes = kOffFlags + size_t(kMaxMd / 32) * 4;

struct Result {
  unsigned long long count;
  unsigned long long weight;
  uint32_t err;
  uint32_t rounds;
};

// Output order of the forest.
enum class Out {
  kFound,   // in the order the rounds find the edges
  kSorted,  // sorted by (src, dst): the input order of the src<dst copies
};

// Stable block-wide ranks of this thread's item for two flags (one item per
// thread, items in thread order): r = rank among the block's items with
// the same flag, t = block totals.
template <int THREADS>
__device__ __forceinline__ void block_rank2(bool f0, bool f1, uint32_t& r0, uint32_t& r1,
                                            uint32_t& t0, uint32_t& t1, uint32_t* s_w) {
  constexpr int kWarps = THREADS / 32;
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

// The whole solve by the calling CTA (THREADS threads): first pass (src<dst
// copies, fused round-0 minimum), Boruvka rounds until no edge is left, the
// forest output.  Requires n <= kMaxN and md <= kMaxMd.  check_ids: entries
// with an id >= n set kErrRange (they are skipped either way); check_order:
// entries not strictly (src, dst)-increasing set kErrOrder.  The result
// is written by thread 0 to *res; the caller's threads are synchronised on
// return.
template <int THREADS, Out OUT>
__device__ void solve(const uint32_t* __restrict__ in, uint32_t md, uint32_t n,
                      unsigned char* __restrict__ scratch, uint32_t* __restrict__ out,
                      Result* res, bool check_ids, bool check_order = false) {
  constexpr int kWarps = THREADS / 32;
  Rec* L[2] = {reinterpret_cast<Rec*>(scratch + kOffL0), reinterpret_cast<Rec*>(scratch + kOffL1)};
  uint64_t* mv[2] = {reinterpret_cast<uint64_t*>(scratch + kOffMin0),
                     reinterpret_cast<uint64_t*>(scratch + kOffMin1)};
  uint32_t* parent = reinterpret_cast<uint32_t*>(scratch + kOffParent);
  uint32_t* msfoid = reinterpret_cast<uint32_t*>(scratch + kOffMsfoid);
  uint32_t* newid = reinterpret_cast<uint32_t*>(scratch + kOffNewid);
  uint32_t* R = reinterpret_cast<uint32_t*>(scratch + kOffR);
  uint32_t* msf = reinterpret_cast<uint32_t*>(scratch + kOffMsf);
  uint32_t* flags = reinterpret_cast<uint32_t*>(scratch + kOffFlags);
  __shared__ uint32_t s_w[2 * kWarps];
  __shared__ uint32_t s_err;
  __shared__ unsigned long long s_weight;
  const uint32_t tid = threadIdx.x;
  // Error bits this thread raised.  Every break decision is taken with
  // __syncthreads_or over these, so all threads leave the rounds together;
  // s_err only collects the codes for the result.
  uint32_t terr = 0;
  auto flag_err = [&](uint32_t code) {
    terr |= code;
    atomicOr(&s_err, code);
  };
  if (tid == 0) {
    s_err = 0;
    s_weight = 0;
  }
  for (uint32_t v = tid; v < n; v += THREADS) mv[0][v] = kInf64;
  __syncthreads();
  // first pass: keep the src<dst copies, in input order
  uint32_t m = 0;
  for (uint32_t base = 0; base < md; base += THREADS) {
    const uint32_t i = base + tid;
    uint32_t s = 0, d = 0, w = 0;
    bool keep = false;
    if (i < md) {
      s = in[3ull * i];
      d = in[3ull * i + 1];
      w = in[3ull * i + 2];
      keep = s < d && d < n;
      if (check_ids && (s >= n || d >= n)) flag_err(kErrRange);
      if (check_order && i > 0) {
        const uint32_t ps = in[3ull * (i - 1)], pd = in[3ull * (i - 1) + 1];
        if (s < ps || (s == ps && d <= pd)) flag_err(kErrOrder);
      }
    }
    uint32_t r0, r1, t0, t1;
    block_rank2<THREADS>(keep, false, r0, r1, t0, t1, s_w);
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
        flag_err(kErrOverflow);
      }
    }
    m += t0;
  }
  uint32_t nr = n, cur = 0, msf_count = 0, round = 0;
  while (m > 0) {
    if (__syncthreads_or((terr & ~kErrRange) != 0)) break;
    if (round >= kMaxRounds) {  // round is the same in every thread
      terr |= kErrChase;
      if (tid == 0) s_err |= kErrChase;
      break;
    }
    const Rec* Lc = L[cur];
    Rec* Ln = L[cur ^ 1];
    const uint64_t* mc = mv[cur];
    uint64_t* mn = mv[cur ^ 1];
    // hook: along the minimum edge; of a mutual pair the lower label stays root
    for (uint32_t v = tid; v < nr; v += THREADS) {
      const uint64_t val = mc[v];
      uint32_t par = v, eid = kNone;
      if (val != kInf64) {
        const Rec x = Lc[static_cast<uint32_t>(val)];
        if (x.a != v && x.b != v) {
          flag_err(kErrHook);
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
    // (weak, L1-cacheable reads: entries only move to ancestors and roots
    // never change, so a stale entry is still an ancestor)
    for (uint32_t v = tid; v < nr; v += THREADS) {
      uint32_t x = v, p = ld_weak_u32(parent + x), steps = 0;
      if (p == x) continue;
      for (;;) {
        const uint32_t gp = ld_weak_u32(parent + p);
        if (gp == p) break;
        st_relaxed(parent + x, gp);
        x = gp;
        p = ld_weak_u32(parent + x);
        if (++steps > 2 * kMaxN) {
          flag_err(kErrJump);
          break;
        }
      }
    }
    __syncthreads();
    for (uint32_t v = tid; v < nr; v += THREADS) {
      uint32_t p = ld_weak_u32(parent + v), steps = 0;
      if (p == v) continue;
      for (;;) {
        const uint32_t gp = ld_weak_u32(parent + p);
        if (gp == p || ++steps > 2 * kMaxN) break;
        p = gp;
      }
      st_relaxed(parent + v, p);
    }
    if (__syncthreads_or((terr & ~kErrRange) != 0)) break;
    // renumber live roots, append the forest edges of hooked vertices
    uint32_t n_next = 0;
    for (uint32_t vb = 0; vb < nr; vb += THREADS) {
      const uint32_t v = vb + tid;
      uint32_t c = 2;
      if (v < nr) {
        if (parent[v] != v)
          c = 1;
        else if (mc[v] != kInf64)
          c = 0;
      }
      uint32_t r0, r1, t0, t1;
      block_rank2<THREADS>(c == 0, c == 1, r0, r1, t0, t1, s_w);
      if (c == 0) {
        newid[v] = n_next + r0;
        mn[n_next + r0] = kInf64;
      } else if (c == 1) {
        if (msf_count + r1 < kMaxN)
          msf[msf_count + r1] = msfoid[v];
        else
          flag_err(kErrOverflow);
      }
      n_next += t0;
      msf_count += t1;
    }
    __syncthreads();
    for (uint32_t v = tid; v < nr; v += THREADS)
      R[v] = (mc[v] == kInf64 && parent[v] == v) ? kNone : newid[parent[v]];
    __syncthreads();
    // relabel, drop self loops, compact (stable), feed the next minimum
    uint32_t m_next = 0;
    for (uint32_t eb = 0; eb < m; eb += THREADS) {
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
      block_rank2<THREADS>(keep, false, r0, r1, t0, t1, s_w);
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
  // forest output: the src<dst input copy of every forest edge
  unsigned long long local = 0;
  const bool ok = !__syncthreads_or((terr & ~kErrRange) != 0);
  if (OUT == Out::kFound) {
    if (ok) {
      for (uint32_t k = tid; k < msf_count; k += THREADS) {
        const uint64_t o = 3ull * msf[k];
        const uint32_t s = in[o], d = in[o + 1], w = in[o + 2];
        out[3ull * k] = s;
        out[3ull * k + 1] = d;
        out[3ull * k + 2] = w;
        local += w;
      }
    }
  } else if (ok) {
    // mark the forest's input positions, then write them in input order
    const uint32_t words = (md + 31) / 32;
    for (uint32_t k = tid; k < words; k += THREADS) flags[k] = 0;
    __syncthreads();
    for (uint32_t k = tid; k < msf_count; k += THREADS)
      atomicOr(&flags[msf[k] >> 5], 1u << (msf[k] & 31));
    __syncthreads();
    uint32_t written = 0;
    for (uint32_t wb = 0; wb < words; wb += THREADS) {
      const uint32_t k = wb + tid;
      const uint32_t f = k < words ? flags[k] : 0u;
      // exclusive prefix of the set bits over the block's words
      const uint32_t c = __popc(f);
      uint32_t incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane_id() >= static_cast<uint32_t>(o)) incl += y;
      }
      if (lane_id() == 31) s_w[threadIdx.x >> 5] = incl;
      __syncthreads();
      uint32_t wpre = 0, tot = 0;
      for (int w = 0; w < kWarps; ++w) {
        const uint32_t x = s_w[w];
        if (static_cast<uint32_t>(w) < (threadIdx.x >> 5)) wpre += x;
        tot += x;
      }
      __syncthreads();
      uint32_t o = written + wpre + incl - c;
      uint32_t bits = f;
      while (bits) {
        const uint32_t b = __ffs(bits) - 1;
        bits &= bits - 1;
        const uint64_t p = 3ull * (k * 32 + b);
        const uint32_t s = in[p], d = in[p + 1], w = in[p + 2];
        out[3ull * o] = s;
        out[3ull * o + 1] = d;
        out[3ull * o + 2] = w;
        local += w;
        ++o;
      }
      written += tot;
    }
  }
  local = warp_sum(local);
  if (lane_id() == 0 && local) atomicAdd(&s_weight, local);
  __syncthreads();
  if (tid == 0) {
    res->count = ok ? msf_count : 0;
    res->weight = s_weight;
    res->err = s_err;
    res->rounds = round;
  }
  __syncthreads();
}

}  // namespace small
}  // namespace kamsta
