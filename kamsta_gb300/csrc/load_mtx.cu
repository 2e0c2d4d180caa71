// load_mtx.cu -- MatrixMarket coordinate files as solver input.
//
// The reference reads unweighted graphs in MatrixMarket format
// (graphs::read_unweighted_graph(file, GraphFormat::MatrixMarket),
// benchmarks/mst_benchmarks.hpp:181-184; the graphs library is not
// vendored).  Here: "%%MatrixMarket matrix coordinate <field> <symmetry>"
// with any field (values are ignored: the graph is unweighted) and any
// symmetry; '%' lines are comments; the size line gives rows, cols and the
// number of stored entries; entry (i, j) (1-based) is the undirected edge
// {i-1, j-1}.  Self loops are dropped and repeated pairs merged; vertices
// are 0 .. max(rows, cols) - 1; every edge gets the generators' weight
// 1 + hi64(mix64(mix64(seed ^ 0x6a09e667f3bcc909) ^ (min << 32 | max)) *
// max_weight).
//
// The file is read whole and its entry lines are parsed by host threads
// (one line-aligned piece each) into pair keys; the device sorts them,
// drops duplicates and writes both directions (pairs_to_edges).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "gen_scratch.cuh"
#include "sort_gen.cuh"

namespace kamsta {

namespace {

struct MtxFile {
  std::vector<char> text;
  uint64_t rows = 0, cols = 0, entries = 0;
  size_t body = 0;  // offset of the first entry line
};

bool read_all(const char* path, std::vector<char>* out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  bool ok = fseeko(f, 0, SEEK_END) == 0;
  const off_t sz = ok ? ftello(f) : -1;
  ok = ok && sz >= 0 && fseeko(f, 0, SEEK_SET) == 0;
  if (ok) {
    out->resize(static_cast<size_t>(sz) + 1);
    ok = fread(out->data(), 1, static_cast<size_t>(sz), f) == static_cast<size_t>(sz);
    (*out)[static_cast<size_t>(sz)] = '\n';  // every line ends with a newline
  }
  fclose(f);
  return ok;
}

std::string lower(std::string s) {
  for (char& c : s) c = static_cast<char>(c >= 'A' && c <= 'Z' ? c - 'A' + 'a' : c);
  return s;
}

// Parses the banner and the size line.
kamsta_status parse_header(const char* path, MtxFile* m) {
  if (!read_all(path, &m->text)) {
    set_error(std::string("cannot read ") + path);
    return KAMSTA_E_INPUT;
  }
  const char* t = m->text.data();
  const size_t len = m->text.size();
  size_t p = 0;
  auto line_end = [&](size_t q) {
    while (q < len && t[q] != '\n') ++q;
    return q;
  };
  size_t e = line_end(0);
  char w[5][64] = {};
  const std::string banner(t, e);
  if (sscanf(banner.c_str(), "%63s %63s %63s %63s %63s", w[0], w[1], w[2], w[3], w[4]) != 5 ||
      lower(w[0]) != "%%matrixmarket" || lower(w[1]) != "matrix") {
    set_error(std::string(path) + ": not a MatrixMarket matrix file");
    return KAMSTA_E_INPUT;
  }
  if (lower(w[2]) != "coordinate") {
    set_error(std::string(path) + ": only the coordinate format is supported");
    return KAMSTA_E_UNSUPPORTED;
  }
  p = e + 1;
  while (p < len) {  // comments and blank lines up to the size line
    e = line_end(p);
    size_t q = p;
    while (q < e && (t[q] == ' ' || t[q] == '\t' || t[q] == '\r')) ++q;
    if (q < e && t[q] != '%') break;
    p = e + 1;
  }
  if (p >= len) {
    set_error(std::string(path) + ": no size line");
    return KAMSTA_E_INPUT;
  }
  e = line_end(p);
  const std::string size_line(t + p, e - p);
  unsigned long long r = 0, c = 0, nz = 0;
  if (sscanf(size_line.c_str(), "%llu %llu %llu", &r, &c, &nz) != 3) {
    set_error(std::string(path) + ": bad size line");
    return KAMSTA_E_INPUT;
  }
  m->rows = r;
  m->cols = c;
  m->entries = nz;
  m->body = e + 1;
  return KAMSTA_OK;
}

// Parses entry lines of [b, e) (whole lines) into pair keys.  Returns false
// on a malformed line or an index out of range.
bool parse_piece(const char* t, size_t b, size_t e, uint64_t rows, uint64_t cols, uint32_t L,
                 std::vector<uint64_t>* keys) {
  const uint64_t none = (1ull << (2 * L)) - 1;
  size_t p = b;
  while (p < e) {
    while (p < e && (t[p] == ' ' || t[p] == '\t' || t[p] == '\r')) ++p;
    if (p < e && (t[p] == '\n' || t[p] == '%')) {  // blank line or comment
      while (p < e && t[p] != '\n') ++p;
      ++p;
      continue;
    }
    if (p >= e) break;
    uint64_t v[2] = {0, 0};
    for (int k = 0; k < 2; ++k) {
      while (p < e && (t[p] == ' ' || t[p] == '\t')) ++p;
      if (p >= e || t[p] < '0' || t[p] > '9') return false;
      uint64_t x = 0;
      while (p < e && t[p] >= '0' && t[p] <= '9') {
        x = x * 10 + static_cast<uint64_t>(t[p] - '0');
        if (x > (1ull << 40)) return false;
        ++p;
      }
      v[k] = x;
    }
    if (v[0] < 1 || v[0] > rows || v[1] < 1 || v[1] > cols) return false;
    const uint64_t a = v[0] - 1, c = v[1] - 1;
    keys->push_back(a == c ? none : ((std::min(a, c) << L) | std::max(a, c)));
    while (p < e && t[p] != '\n') ++p;  // values (ignored)
    ++p;
  }
  return true;
}

}  // namespace

kamsta_status mtx_header(const char* path, uint64_t* rows, uint64_t* cols, uint64_t* entries) {
  MtxFile m;
  const kamsta_status s = parse_header(path, &m);
  if (s != KAMSTA_OK) return s;
  *rows = m.rows;
  *cols = m.cols;
  *entries = m.entries;
  return KAMSTA_OK;
}

kamsta_status load_mtx(kamsta_ctx* ctx, const char* path, uint64_t seed, uint32_t max_weight,
                       kamsta_wedge* d_out, uint64_t capacity, uint64_t* m_out, uint32_t* n_out,
                       cudaStream_t st) {
  *m_out = 0;
  *n_out = 0;
  if (max_weight == 0) {
    set_error("load_mtx: max_weight must be >= 1");
    return KAMSTA_E_INPUT;
  }
  MtxFile m;
  kamsta_status s = parse_header(path, &m);
  if (s != KAMSTA_OK) return s;
  const uint64_t n = std::max(m.rows, m.cols);
  if (n >= (1ull << 31)) {
    set_error("load_mtx: more than 2^31 - 1 vertices are not supported");
    return KAMSTA_E_UNSUPPORTED;
  }
  *n_out = static_cast<uint32_t>(n);
  if (n < 2 || m.entries == 0) return KAMSTA_OK;
  uint32_t L = 1;
  while ((1ull << L) < n) ++L;
  // line-aligned pieces of the body, one host thread each
  const char* t = m.text.data();
  const size_t len = m.text.size();
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<size_t> cut(hw + 1, len);
  cut[0] = m.body;
  for (unsigned k = 1; k < hw; ++k) {
    size_t q = m.body + (len - m.body) * k / hw;
    while (q < len && t[q - 1] != '\n') ++q;
    cut[k] = std::max(q, cut[k - 1]);
  }
  std::vector<std::vector<uint64_t>> part(hw);
  std::vector<char> ok(hw, 1);
  {
    std::vector<std::thread> th;
    for (unsigned k = 0; k < hw; ++k)
      th.emplace_back([&, k] {
        part[k].reserve((cut[k + 1] - cut[k]) / 8 + 16);
        ok[k] = parse_piece(t, cut[k], cut[k + 1], m.rows, m.cols, L, &part[k]) ? 1 : 0;
      });
    for (auto& x : th) x.join();
  }
  uint64_t K = 0;
  for (unsigned k = 0; k < hw; ++k) {
    if (!ok[k]) {
      set_error(std::string(path) + ": malformed entry line or index out of range");
      return KAMSTA_E_INPUT;
    }
    K += part[k].size();
  }
  if (K != m.entries) {
    set_error(std::string(path) + ": entry count differs from the size line");
    return KAMSTA_E_INPUT;
  }
  GenBuf bk;
  uint64_t* keys;
  GEN_CHECK(bk.alloc(ctx, st, &keys, K));
  uint64_t off = 0;
  for (unsigned k = 0; k < hw; ++k) {
    if (!part[k].empty())
      GEN_CHECK(cudaMemcpyAsync(keys + off, part[k].data(), part[k].size() * sizeof(uint64_t),
                                cudaMemcpyHostToDevice, st));
    off += part[k].size();
  }
  GEN_CHECK(cudaStreamSynchronize(st));  // the host pieces may go now
  return pairs_to_edges(ctx, st, bk, K, L, mix64(seed ^ 0x6a09e667f3bcc909ull), max_weight,
                        "load_mtx", d_out, capacity, m_out);
}

}  // namespace kamsta

extern "C" kamsta_status kamsta_mtx_header(const char* path, uint64_t* rows, uint64_t* cols,
                                           uint64_t* entries) {
  if (!path || !rows || !cols || !entries) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  return kamsta::mtx_header(path, rows, cols, entries);
}

extern "C" kamsta_status kamsta_load_mtx_dev(kamsta_ctx* ctx, const char* path, uint64_t seed,
                                             uint32_t max_weight, kamsta_wedge* d_out,
                                             uint64_t capacity, uint64_t* m_directed_out,
                                             uint32_t* n_out, kamsta_stream stream) {
  if (!ctx || !path || !m_directed_out || !n_out) {
    kamsta::set_error("null pointer argument");
    return KAMSTA_E_INPUT;
  }
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return kamsta::load_mtx(ctx, path, seed, max_weight, d_out, capacity, m_directed_out, n_out, st);
}
