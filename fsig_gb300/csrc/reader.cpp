// t/v/e reader with the reference reader's semantics
// (IO/graph_reader.cc:12-55, graph/graph.cc:12-33):
//   - the first record must be "t V E" (V and E are not used);
//   - "v id label deg": the vertex count is the largest id + 1, the label is
//     kept (0 when unlabeled), deg is ignored;
//   - "e a b": one undirected edge, duplicates and self-loops kept;
//   - any other character is skipped one at a time;
//   - the loop tests end-of-file before each record, so a file ending in
//     whitespace applies its last record twice (a duplicated last edge).
// The whole file is read at once; files of 64 MiB and more are parsed by one
// thread per core when every line is a plain record (below), others by a
// single sequential scan.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "reader.h"

namespace fsig {
namespace {

constexpr size_t kParallelBytes = size_t(64) << 20;

struct Scan {
  const char* p;
  const char* end;
  bool fail = false, eof = false;
  static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }
  bool skip() {
    if (fail) return false;
    while (p < end && space(*p)) p++;
    if (p >= end) { fail = eof = true; return false; }
    return true;
  }
  void get(char& c) {
    if (!skip()) return;
    c = *p++;
  }
  template <class T>
  void num(T& out) {
    if (!skip()) return;
    bool neg = false;
    const char* q = p;
    if (*q == '+' || *q == '-') { neg = *q == '-'; q++; }
    const char* d0 = q;
    unsigned long long v = 0;
    while (q < end && *q >= '0' && *q <= '9') v = v * 10 + unsigned(*q++ - '0');
    if (q == d0) { fail = true; out = 0; return; }
    p = q;
    if (p >= end) eof = true;
    out = T(neg ? 0ull - v : v);
  }
};

// ---------------------------------------------------------------------------
// Parallel path for large files: the body after the t record is cut at line
// starts into one range per thread; each range is parsed line by line under
// the assumption that every line is blank or one complete "v id label deg" /
// "e a b" record of unsigned decimals.  Any other line makes the whole file
// go through the sequential scanner, so the result is always the one the
// sequential reading defines.  The ranges' records are merged in file order;
// the duplicated last record of a file ending in whitespace is applied after
// the merge.
// ---------------------------------------------------------------------------
struct Part {
  std::vector<uint32_t> vid;
  std::vector<int32_t> vlab;
  std::vector<uint32_t> edges;
  char last = 0;  // type of the range's last record
  bool ok = true;
};

bool is_space(char c) { return Scan::space(c); }

bool parse_uint(const char*& p, const char* end, uint64_t& v) {
  const char* d0 = p;
  v = 0;
  while (p < end && *p >= '0' && *p <= '9') {
    v = v * 10 + unsigned(*p - '0');
    if (v > 0xffffffffull) return false;
    p++;
  }
  return p != d0;
}

void parse_range(const char* p, const char* end, Part& out) {
  while (p < end) {
    while (p < end && *p != '\n' && is_space(*p)) p++;
    if (p >= end) break;
    if (*p == '\n') { p++; continue; }
    const char type = *p++;
    const int fields = type == 'v' ? 3 : type == 'e' ? 2 : -1;
    if (fields < 0) { out.ok = false; return; }
    uint64_t f[3] = {0, 0, 0};
    for (int i = 0; i < fields; i++) {
      const char* q = p;
      while (q < end && *q != '\n' && is_space(*q)) q++;
      if (q == p || !parse_uint(q, end, f[i])) { out.ok = false; return; }  // fields need separating blanks
      p = q;
    }
    while (p < end && *p != '\n' && is_space(*p)) p++;
    if (p < end && *p != '\n') { out.ok = false; return; }
    if (type == 'v') {
      if (f[1] > 0x7fffffffull) { out.ok = false; return; }
      out.vid.push_back(uint32_t(f[0]));
      out.vlab.push_back(int32_t(f[1]));
    } else {
      out.edges.push_back(uint32_t(f[0]));
      out.edges.push_back(uint32_t(f[1]));
    }
    out.last = type;
  }
}

bool read_parallel(const std::vector<char>& buf, int is_labeled, TveGraph& g) {
  const char* b = buf.data();
  const char* e = b + buf.size();
  // the t record: "t V E" on the first line
  const char* p = b;
  while (p < e && is_space(*p)) p++;
  if (p >= e || *p != 't') return false;
  while (p < e && *p != '\n') p++;
  if (p >= e) return false;
  p++;
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt ? nt : 4u, 32u));
  std::vector<const char*> cut(nt + 1, e);
  cut[0] = p;
  for (unsigned t = 1; t < nt; t++) {
    const char* c = p + size_t(e - p) * t / nt;
    if (c < cut[t - 1]) c = cut[t - 1];
    while (c < e && c[-1] != '\n') c++;
    cut[t] = c;
  }
  std::vector<Part> parts(nt);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++) th.emplace_back(parse_range, cut[t], cut[t + 1], std::ref(parts[t]));
  for (auto& x : th) x.join();
  for (auto& x : parts)
    if (!x.ok) return false;
  g.labels.clear();
  g.edges.clear();
  g.num_vertices = 0;
  uint32_t vmax = 0;
  bool anyv = false;
  size_t ne = 0;
  for (auto& x : parts) {
    for (uint32_t v : x.vid) { vmax = std::max(vmax, v); anyv = true; }
    ne += x.edges.size();
  }
  if (anyv) {
    g.labels.assign(size_t(vmax) + 1, -1);
    g.num_vertices = vmax + 1;
  }
  g.edges.reserve(ne + 2);
  char last = 0;
  for (auto& x : parts) {
    for (size_t i = 0; i < x.vid.size(); i++) g.labels[x.vid[i]] = is_labeled ? x.vlab[i] : 0;
    g.edges.insert(g.edges.end(), x.edges.begin(), x.edges.end());
    if (x.last) last = x.last;
  }
  // a file ending in whitespace applies its last record again
  if (!buf.empty() && is_space(buf.back()) && last == 'e') {
    const uint32_t a = g.edges[g.edges.size() - 2], c = g.edges[g.edges.size() - 1];
    g.edges.push_back(a);
    g.edges.push_back(c);
  }
  return true;
}

int read_tve_sequential(const std::vector<char>& buf, int is_labeled, TveGraph& g, std::string& err) {
  Scan s{buf.data(), buf.data() + buf.size()};
  char type = 0;
  s.get(type);
  if (type != 't') { err = "graph file does not start with a t record"; return -2; }
  uint32_t nv = 0, ne = 0;
  s.num(nv);
  s.num(ne);
  g.labels.clear();
  g.edges.clear();
  g.num_vertices = 0;
  uint32_t vid = 0, vdeg = 0, ea = 0, eb = 0;
  int32_t vlabel = 0;
  while (!s.eof) {
    s.get(type);
    if (type == 'v') {
      s.num(vid);
      s.num(vlabel);
      s.num(vdeg);
      if (g.labels.size() <= vid) {
        g.labels.resize(size_t(vid) + 1, -1);
        g.num_vertices = vid + 1;
      }
      g.labels[vid] = is_labeled ? vlabel : 0;
    } else if (type == 'e') {
      s.num(ea);
      s.num(eb);
      g.edges.push_back(ea);
      g.edges.push_back(eb);
    }
    if (s.fail && !s.eof) { err = "malformed record"; return -3; }
  }
  return 0;
}

}  // namespace

int read_tve(const char* path, int is_labeled, TveGraph& g, std::string& err, uint64_t parallel_from) {
  FILE* f = std::fopen(path, "rb");
  if (!f) { err = std::string("cannot open ") + path; return -1; }
  std::vector<char> buf;
  if (std::fseek(f, 0, SEEK_END) == 0) {
    const long size = std::ftell(f);
    if (size > 0) buf.reserve(size_t(size));
    std::fseek(f, 0, SEEK_SET);
  }
  char chunk[1 << 16];
  size_t k;
  while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + k);
  std::fclose(f);
  if (buf.size() >= (parallel_from ? parallel_from : kParallelBytes) && read_parallel(buf, is_labeled, g)) return 0;
  return read_tve_sequential(buf, is_labeled, g, err);
}

}  // namespace fsig
