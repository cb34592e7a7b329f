// t/v/e reader with the reference reader's semantics
// (IO/graph_reader.cc:12-55, graph/graph.cc:12-33):
//   - the first record must be "t V E" (V and E are not used);
//   - "v id label deg": the vertex count is the largest id + 1, the label is
//     kept (0 when unlabeled), deg is ignored;
//   - "e a b": one undirected edge, duplicates and self-loops kept;
//   - any other character is skipped one at a time;
//   - the loop tests end-of-file before each record, so a file ending in
//     whitespace applies its last record twice (a duplicated last edge).
// The whole file is read at once and scanned in a single pass.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "reader.h"

namespace fsig {
namespace {

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

}  // namespace

int read_tve(const char* path, int is_labeled, TveGraph& g, std::string& err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) { err = std::string("cannot open ") + path; return -1; }
  std::vector<char> buf;
  char chunk[1 << 16];
  size_t k;
  while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + k);
  std::fclose(f);
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

}  // namespace fsig
