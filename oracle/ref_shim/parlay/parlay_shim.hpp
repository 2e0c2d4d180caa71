// parlay_shim.hpp -- the subset of ParlayLib that KaMSTa's single-rank hot
// path uses, written for the oracle's reference build (test infrastructure).
//
// KaMSTa vendors its parlay fork as a git submodule (external/parlay, pin
// unknown) that is empty here, so this header restates the published
// semantics of the calls the reference makes, in plain C++17 + OpenMP:
//   sequence<T>      owning array; begin()/end() are T* (bridge.hpp's filterf
//                    deduces T from them); sequence<bool> is a real bool array
//   slice, make_slice, delayed_seq
//   filter, filter_into, count_if, pack, pack_out, pack_into, scan_inplace,
//   reduce: order-preserving (stable) and parallel by blocks: count per
//   block, exclusive scan of the counts, write per block
//   hashtable<hash_numeric<T>>: a concurrent set of integers
// Calls that the reference's headers name but the single-rank local
// contraction never instantiates (sample_sort, binary_search, I/O helpers)
// are declared or given simple sequential definitions.
#pragma once

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <iostream>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <unordered_set>
#include <utility>
#include <vector>

namespace parlay {

enum flags { no_flag = 0, fl_sequential = 1, fl_debug = 2, fl_time = 4, fl_conservative = 8,
             fl_inplace = 16 };

inline size_t num_workers() { return static_cast<size_t>(omp_get_max_threads()); }
inline size_t worker_id() { return static_cast<size_t>(omp_get_thread_num()); }

template <typename F>
inline void parallel_for(size_t start, size_t end, F&& f, long granularity = 0,
                         bool /*conservative*/ = false) {
  if (end <= start) return;
  if (granularity > 0) {
#pragma omp parallel for schedule(dynamic, granularity)
    for (size_t i = start; i < end; ++i) f(i);
  } else {
#pragma omp parallel for schedule(static)
    for (size_t i = start; i < end; ++i) f(i);
  }
}

template <typename Lf, typename Rf>
inline void par_do(Lf&& left, Rf&& right, bool /*conservative*/ = false) {
  left();
  right();
}

// f(block, begin, end) over [0, n) in blocks of block_size
template <typename F>
inline void sliced_for(size_t n, size_t block_size, F&& f) {
  const size_t blocks = (n + block_size - 1) / block_size;
  parallel_for(0, blocks, [&](size_t i) {
    const size_t s = i * block_size;
    f(i, s, std::min(s + block_size, n));
  }, 1);
}

template <typename T>
struct allocator : std::allocator<T> {
  allocator() = default;
  template <typename U>
  allocator(const allocator<U>&) {}
  template <typename U>
  struct rebind {
    using other = allocator<U>;
  };
};

// ---------------------------------------------------------------- sequence
template <typename T>
class sequence {
 public:
  using value_type = T;
  using iterator = T*;
  using const_iterator = const T*;
  using reference = T&;
  using const_reference = const T&;
  using size_type = size_t;

  sequence() = default;
  explicit sequence(size_t n) : n_(n), p_(alloc(n)) {
    parallel_for(0, n, [&](size_t i) { new (p_.get() + i) T(); });
  }
  sequence(size_t n, const T& v) : n_(n), p_(alloc(n)) {
    parallel_for(0, n, [&](size_t i) { new (p_.get() + i) T(v); });
  }
  sequence(std::initializer_list<T> l) : n_(l.size()), p_(alloc(l.size())) {
    std::copy(l.begin(), l.end(), p_.get());
  }
  template <typename It, typename = decltype(*std::declval<It>())>
  sequence(It b, It e) : n_(static_cast<size_t>(e - b)), p_(alloc(n_)) {
    parallel_for(0, n_, [&](size_t i) { new (p_.get() + i) T(b[i]); });
  }
  sequence(const sequence& o) : n_(o.n_), p_(alloc(o.n_)) {
    parallel_for(0, n_, [&](size_t i) { new (p_.get() + i) T(o[i]); });
  }
  sequence(sequence&& o) noexcept : n_(o.n_), p_(std::move(o.p_)) { o.n_ = 0; }
  sequence& operator=(const sequence& o) {
    if (this != &o) {
      sequence t(o);
      swap(t);
    }
    return *this;
  }
  sequence& operator=(sequence&& o) noexcept {
    swap(o);
    return *this;
  }
  void swap(sequence& o) noexcept {
    std::swap(n_, o.n_);
    std::swap(p_, o.p_);
  }

  template <typename F>
  static sequence from_function(size_t n, F&& f, size_t /*granularity*/ = 0) {
    sequence s = uninitialized(n);
    parallel_for(0, n, [&](size_t i) { new (s.p_.get() + i) T(f(i)); });
    return s;
  }
  static sequence uninitialized(size_t n) {
    sequence s;
    s.n_ = n;
    s.p_ = alloc(n);
    return s;
  }

  size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }
  T* data() { return p_.get(); }
  const T* data() const { return p_.get(); }
  T* begin() { return p_.get(); }
  T* end() { return p_.get() + n_; }
  const T* begin() const { return p_.get(); }
  const T* end() const { return p_.get() + n_; }
  T& operator[](size_t i) { return p_[i]; }
  const T& operator[](size_t i) const { return p_[i]; }
  T& back() { return p_[n_ - 1]; }
  const T& back() const { return p_[n_ - 1]; }
  void resize(size_t n) {
    sequence t(n);
    const size_t k = std::min(n, n_);
    for (size_t i = 0; i < k; ++i) t[i] = std::move((*this)[i]);
    swap(t);
  }
  void clear() { *this = sequence(); }
  sequence cut(size_t a, size_t b) const { return sequence(begin() + a, begin() + b); }

 private:
  struct Free {
    void operator()(T* p) const { ::operator delete(static_cast<void*>(p)); }
  };
  static std::unique_ptr<T[], Free> alloc(size_t n) {
    return std::unique_ptr<T[], Free>(
        static_cast<T*>(::operator new(std::max<size_t>(n, 1) * sizeof(T))));
  }
  size_t n_ = 0;
  std::unique_ptr<T[], Free> p_;
};

// ------------------------------------------------------------------- slice
template <typename It, typename S = It>
struct slice {
  using value_type = std::decay_t<decltype(*std::declval<It>())>;
  using iterator = It;
  It s;
  S e;
  slice(It a, S b) : s(a), e(b) {}
  size_t size() const { return static_cast<size_t>(e - s); }
  bool empty() const { return size() == 0; }
  decltype(auto) operator[](size_t i) const { return s[i]; }
  It begin() const { return s; }
  S end() const { return e; }
  slice cut(size_t a, size_t b) const { return slice(s + a, s + b); }
};
template <typename It, typename S>
slice(It, S) -> slice<It, S>;

template <typename It, typename S>
inline slice<It, S> make_slice(It a, S b) {
  return slice<It, S>(a, b);
}
template <typename R, typename = decltype(std::declval<R&>().begin())>
inline auto make_slice(R&& r) {
  return make_slice(r.begin(), r.end());
}

// ------------------------------------------------------------ delayed_seq
template <typename T, typename F>
struct delayed_sequence {
  using value_type = T;
  size_t n;
  F f;
  size_t size() const { return n; }
  T operator[](size_t i) const { return f(i); }
};
template <typename T, typename F>
inline delayed_sequence<T, F> delayed_seq(size_t n, F f) {
  return delayed_sequence<T, F>{n, std::move(f)};
}
template <typename F>
inline auto delayed_tabulate(size_t n, F f) {
  using T = std::decay_t<decltype(f(size_t{0}))>;
  return delayed_seq<T>(n, std::move(f));
}

// ----------------------------------------------------------------- monoids
template <typename T>
struct addm {
  T identity = 0;
  T f(const T& a, const T& b) const { return a + b; }
  T operator()(const T& a, const T& b) const { return a + b; }
};
template <typename T>
struct maxm {
  T identity = std::numeric_limits<T>::lowest();
  T f(const T& a, const T& b) const { return std::max(a, b); }
  T operator()(const T& a, const T& b) const { return std::max(a, b); }
};
template <typename T>
struct minm {
  T identity = std::numeric_limits<T>::max();
  T f(const T& a, const T& b) const { return std::min(a, b); }
  T operator()(const T& a, const T& b) const { return std::min(a, b); }
};
template <typename T>
struct xorm {
  T identity = 0;
  T f(const T& a, const T& b) const { return a ^ b; }
  T operator()(const T& a, const T& b) const { return a ^ b; }
};

namespace internal {
constexpr size_t kBlock = 1 << 14;
inline size_t blocks_of(size_t n) { return (n + kBlock - 1) / kBlock; }

// Exclusive prefix of per-block counts; returns the total.
inline size_t scan_counts(std::vector<size_t>& c) {
  size_t t = 0;
  for (auto& x : c) {
    const size_t y = x;
    x = t;
    t += y;
  }
  return t;
}

// Stable pack: out[k] = in[i] for the k-th i with keep(i).  keep is
// evaluated once per element (into a byte per element), as ParlayLib's
// blocked pack does.
template <typename In, typename Keep, typename Put>
size_t stable_pack(size_t n, In&& in, Keep&& keep, Put&& put) {
  const size_t nb = blocks_of(n);
  std::vector<size_t> cnt(nb, 0);
  std::unique_ptr<uint8_t[]> fl(new uint8_t[std::max<size_t>(n, 1)]);
  parallel_for(0, nb, [&](size_t b) {
    size_t c = 0;
    const size_t e = std::min(n, (b + 1) * kBlock);
    for (size_t i = b * kBlock; i < e; ++i) {
      fl[i] = keep(i) ? 1 : 0;
      c += fl[i];
    }
    cnt[b] = c;
  }, 1);
  const size_t total = scan_counts(cnt);
  parallel_for(0, nb, [&](size_t b) {
    size_t o = cnt[b];
    const size_t e = std::min(n, (b + 1) * kBlock);
    for (size_t i = b * kBlock; i < e; ++i)
      if (fl[i]) put(o++, in(i));
  }, 1);
  return total;
}

template <typename In_Seq, typename Bool_Seq, typename Out_Seq>
size_t pack_out(In_Seq const& in, Bool_Seq const& fl, Out_Seq&& out, flags = no_flag) {
  return stable_pack(
      in.size(), [&](size_t i) { return in[i]; }, [&](size_t i) { return static_cast<bool>(fl[i]); },
      [&](size_t k, auto&& v) { out[k] = v; });
}

template <typename... A>
void filter_out(A&&...);
template <typename... A>
void split_two(A&&...);
template <typename... A>
void binary_search(A&&...);
template <typename... A>
void chars_to_int_t(A&&...);
template <typename... A>
void get_counts(A&&...);

template <typename Seq, typename Less>
auto sample_sort(Seq const& s, Less less, bool = false) {
  using T = std::decay_t<decltype(s[0])>;
  sequence<T> r(s.begin(), s.end());
  std::stable_sort(r.begin(), r.end(), less);
  return r;
}
template <typename Seq, typename Less>
void sample_sort_inplace(Seq&& s, Less less, bool = false) {
  std::stable_sort(s.begin(), s.end(), less);
}

struct timer {
  explicit timer(std::string name = "", bool start_now = true) : name_(std::move(name)) {
    if (start_now) start();
  }
  void start() {
    on_ = true;
    t0_ = std::chrono::steady_clock::now();
  }
  double stop() {
    if (!on_) return 0;
    on_ = false;
    const double d = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    total_ += d;
    return d;
  }
  double next_time() {
    const double d = stop();
    start();
    return d;
  }
  void next(const std::string&) { next_time(); }
  double total_time() const { return total_; }
  void report(double, const std::string&) {}

 private:
  std::string name_;
  bool on_ = false;
  double total_ = 0;
  std::chrono::steady_clock::time_point t0_;
};
}  // namespace internal

using internal::pack_out;

// ---------------------------------------------------------------- primitives
template <typename R, typename P>
size_t count_if(R const& r, P p) {
  const size_t n = r.size();
  size_t total = 0;
#pragma omp parallel for schedule(static) reduction(+ : total)
  for (size_t i = 0; i < n; ++i) total += p(r[i]) ? 1 : 0;
  return total;
}

template <typename R, typename P>
auto filter(R const& r, P p, flags = no_flag) {
  using T = std::decay_t<decltype(r[0])>;
  const size_t n = r.size();
  const size_t nb = internal::blocks_of(n);
  std::vector<size_t> cnt(nb, 0);
  std::unique_ptr<uint8_t[]> fl(new uint8_t[std::max<size_t>(n, 1)]);
  parallel_for(0, nb, [&](size_t b) {
    size_t c = 0;
    const size_t e = std::min(n, (b + 1) * internal::kBlock);
    for (size_t i = b * internal::kBlock; i < e; ++i) {
      fl[i] = p(r[i]) ? 1 : 0;
      c += fl[i];
    }
    cnt[b] = c;
  }, 1);
  const size_t total = internal::scan_counts(cnt);
  auto out = sequence<T>::uninitialized(total);
  parallel_for(0, nb, [&](size_t b) {
    size_t o = cnt[b];
    const size_t e = std::min(n, (b + 1) * internal::kBlock);
    for (size_t i = b * internal::kBlock; i < e; ++i)
      if (fl[i]) new (out.data() + o++) T(r[i]);
  }, 1);
  return out;
}

template <typename In, typename Out, typename P>
size_t filter_into(In const& in, Out&& out, P p) {
  return internal::stable_pack(
      in.size(), [&](size_t i) { return in[i]; }, [&](size_t i) { return static_cast<bool>(p(in[i])); },
      [&](size_t k, auto&& v) { out[k] = v; });
}

template <typename In_Seq, typename Bool_Seq>
auto pack(In_Seq const& in, Bool_Seq const& fl, flags = no_flag) {
  using T = std::decay_t<decltype(in[0])>;
  const size_t n = in.size();
  size_t total = count_if(fl, [](bool b) { return b; });
  auto out = sequence<T>::uninitialized(total);
  internal::stable_pack(
      n, [&](size_t i) { return in[i]; }, [&](size_t i) { return static_cast<bool>(fl[i]); },
      [&](size_t k, auto&& v) { new (out.data() + k) T(v); });
  return out;
}

template <typename In_Seq, typename Bool_Seq, typename Out_Seq>
size_t pack_into(In_Seq const& in, Bool_Seq const& fl, Out_Seq&& out) {
  return internal::pack_out(in, fl, std::forward<Out_Seq>(out));
}

// Exclusive scan in place; returns the total.
template <typename R, typename M = addm<std::decay_t<decltype(std::declval<R&>()[0])>>>
auto scan_inplace(R&& r, M m = M()) {
  using T = std::decay_t<decltype(r[0])>;
  T acc = m.identity;
  for (size_t i = 0; i < r.size(); ++i) {
    const T v = r[i];
    r[i] = acc;
    acc = m.f(acc, v);
  }
  return acc;
}

template <typename R, typename M = addm<std::decay_t<decltype(std::declval<R&>()[0])>>>
auto reduce(R const& r, M m = M()) {
  using T = std::decay_t<decltype(r[0])>;
  T acc = m.identity;
  for (size_t i = 0; i < r.size(); ++i) acc = m.f(acc, r[i]);
  return acc;
}

template <typename Seq, typename Out, typename Less>
void pack_serial_at(Seq const& in, Out const& fl, Less&& out) {
  size_t k = 0;
  for (size_t i = 0; i < in.size(); ++i)
    if (fl[i]) out[k++] = in[i];
}

// ------------------------------------------------------------------ random
struct random {
  explicit random(size_t seed = 0) : state_(seed) {}
  random next() const { return random(hash(state_ + 1)); }
  size_t ith_rand(size_t i) const { return hash(state_ * 0x9e3779b97f4a7c15ull + i); }
  size_t operator[](size_t i) const { return ith_rand(i); }

 private:
  static size_t hash(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return static_cast<size_t>(x ^ (x >> 31));
  }
  size_t state_;
};

// --------------------------------------------------------------- hashtable
template <typename T>
struct hash_numeric {
  using eType = T;
  using kType = T;
  eType empty() const { return static_cast<T>(-1); }
  kType getKey(eType v) const { return v; }
  size_t hash(kType v) const { return std::hash<T>{}(v); }
};

template <typename H>
class hashtable {
 public:
  using eType = typename H::eType;
  hashtable(size_t size, H h, double = 1.5) : h_(h) { set_.reserve(size); }
  bool insert(eType v) {
    std::lock_guard<std::mutex> lk(mu_);
    return set_.insert(v).second;
  }
  bool find(eType v) {
    std::lock_guard<std::mutex> lk(mu_);
    return set_.count(v) != 0;
  }
  sequence<eType> entries() {
    std::lock_guard<std::mutex> lk(mu_);
    std::vector<eType> v(set_.begin(), set_.end());
    return sequence<eType>(v.data(), v.data() + v.size());
  }

 private:
  H h_;
  std::mutex mu_;
  std::unordered_set<eType> set_;
};

}  // namespace parlay
