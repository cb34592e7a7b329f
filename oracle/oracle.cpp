// CPU oracle for the FSIG subgraph-matching path -- TEST INFRASTRUCTURE ONLY.
// See oracle.h for what is restated and how it is pinned.  Every function
// names the reference lines it follows.
#include "oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kInvalid = 0xffffffffu;  // utility/defines.h:22 INVALID
constexpr uint32_t kHashSeed = 17;          // utility/defines.h:29 HASHSEED
constexpr int kSigWords = 16;               // utility/defines.h:31 SIGNUM (512 bits)

// ----------------------------------------------------------------------------
// Plain graph: restates UndirectedPlainGraph (graph/graph.h:50-69, graph.cc:12-67)
// ----------------------------------------------------------------------------
struct Plain {
  uint32_t num_vertices = 0;
  uint32_t num_edges = 0;
  int32_t num_labels = 0;
  uint32_t min_degree = 0;
  std::vector<int32_t> labels;
  std::vector<std::vector<uint32_t>> adj;

  // graph.cc:12-21: grow the label array (new slots hold INVALID_LABEL) and
  // raise num_labels to label+1.
  void add_vertex(uint32_t id, int32_t label) {
    if (labels.size() <= id) {
      labels.resize(size_t(id) + 1, int32_t(kInvalid));
      num_vertices = id + 1;
    }
    if (num_labels <= label) num_labels = label + 1;
    labels[id] = label;
  }
  // graph.cc:23-33: both directions pushed, no de-duplication.
  void add_edge(uint32_t a, uint32_t b) {
    if (adj.size() <= a) adj.resize(size_t(a) + 1);
    if (adj.size() <= b) adj.resize(size_t(b) + 1);
    adj[a].push_back(b);
    adj[b].push_back(a);
    num_edges++;
  }
  // graph.cc:60-67 (rows past the edge array count as degree 0 here; the
  // reference reads past its vector in that case).
  void set_min_degree() {
    min_degree = num_vertices;
    for (uint32_t i = 0; i < num_vertices; i++) {
      uint32_t d = i < adj.size() ? uint32_t(adj[i].size()) : 0;
      if (d < min_degree) min_degree = d;
    }
  }
};

// A minimal std::istream stand-in: the reader below mirrors the reference's
// sequence of `>>` extractions, including that a failed extraction leaves
// its target unchanged.
struct Tokens {
  std::string buf;
  size_t pos = 0;
  bool fail = false, eof = false;

  static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }
  bool skip_ws() {
    if (fail) return false;
    while (pos < buf.size() && space(buf[pos])) pos++;
    if (pos >= buf.size()) { fail = eof = true; return false; }
    return true;
  }
  void get(char& c) {
    if (!skip_ws()) return;
    c = buf[pos++];
  }
  template <class T>
  void get_int(T& out) {
    if (!skip_ws()) return;
    bool neg = false;
    size_t p = pos;
    if (buf[p] == '+' || buf[p] == '-') { neg = buf[p] == '-'; p++; }
    size_t d0 = p;
    unsigned long long v = 0;
    while (p < buf.size() && buf[p] >= '0' && buf[p] <= '9') { v = v * 10 + unsigned(buf[p] - '0'); p++; }
    if (p == d0) { fail = true; out = 0; return; }
    pos = p;
    if (pos >= buf.size()) eof = true;  // the number ran into end-of-file
    out = T(neg ? (0ull - v) : v);
  }
};

// Restates UndirectedSurveyPlainReader::read (IO/graph_reader.cc:12-55).
// The loop tests eof() before each record, so when the file ends in
// whitespace one more pass runs in which every extraction fails and the
// previous record's values are applied again (a duplicated last edge).
Plain* read_tve(const char* path, int is_labeled) {
  FILE* f = fopen(path, "rb");
  if (!f) return nullptr;
  Tokens t;
  char chunk[1 << 16];
  size_t n;
  while ((n = fread(chunk, 1, sizeof(chunk), f)) > 0) t.buf.append(chunk, n);
  fclose(f);

  auto* g = new Plain();
  char type = 0;
  t.get(type);
  if (type != 't') { delete g; return nullptr; }
  uint32_t nv = 0, ne = 0;
  t.get_int(nv);
  t.get_int(ne);
  // Locals kept across passes: the failed pass reuses them.
  uint32_t vid = 0, vdeg = 0, ea = 0, eb = 0;
  int32_t vlabel = 0;
  while (!t.eof) {
    t.get(type);
    if (type == 'v') {
      t.get_int(vid);
      t.get_int(vlabel);
      t.get_int(vdeg);
      g->add_vertex(vid, is_labeled ? vlabel : 0);
    } else if (type == 'e') {
      t.get_int(ea);
      t.get_int(eb);
      g->add_edge(ea, eb);
    }
    if (t.fail && !t.eof) break;  // malformed token: stop (the reference would spin)
  }
  g->set_min_degree();
  return g;
}

// MurmurHash2, 32-bit (Austin Appleby, public domain), as used for PCSR
// buckets and signature slots (graph_format_transformer.h:59-93).
uint32_t murmur2(const void* key, int len, uint32_t seed) {
  const uint32_t m = 0x5bd1e995u;
  const unsigned char* p = static_cast<const unsigned char*>(key);
  uint32_t h = seed ^ uint32_t(len);
  while (len >= 4) {
    uint32_t k = uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
    k *= m;
    k ^= k >> 24;
    k *= m;
    h = (h * m) ^ k;
    p += 4;
    len -= 4;
  }
  if (len == 3) h ^= uint32_t(p[2]) << 16;
  if (len >= 2) h ^= uint32_t(p[1]) << 8;
  if (len >= 1) { h ^= uint32_t(p[0]); h *= m; }
  h ^= h >> 13;
  h *= m;
  h ^= h >> 15;
  return h;
}

inline uint32_t murmur_u32(uint32_t x) { return murmur2(&x, 4, kHashSeed); }

// MurmurHash3 64-bit finaliser (public, Appleby) -- the embedding hash mixer.
inline uint64_t fmix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// UndirectedPCSRGraph::get_edge_label (graph/graph.h:107-122).
inline int32_t edge_label(int32_t a, int32_t b) {
  int32_t hi = a >= b ? a : b, lo = a >= b ? b : a;
  return hi == 0 ? lo : ((hi - 1) * hi) / 2 + lo;
}

}  // namespace

extern "C" {

void* orc_read_tve(const char* path, int is_labeled) { return read_tve(path, is_labeled); }

void orc_plain_sizes(void* h, uint32_t* nv, uint32_t* ne, int32_t* nl, uint64_t* nadj, uint32_t* mind) {
  auto* g = static_cast<Plain*>(h);
  *nv = g->num_vertices;
  *ne = g->num_edges;
  *nl = g->num_labels;
  uint64_t s = 0;
  for (uint32_t i = 0; i < g->num_vertices && i < g->adj.size(); i++) s += g->adj[i].size();
  *nadj = s;
  *mind = g->min_degree;
}

// UndirectedPlainToCSRTransformer::transform (graph_format_transformer.cc:12-37):
// per-row ascending sort, offsets by prefix sum, duplicates kept.
void orc_plain_to_csr(void* h, int32_t* labels, uint32_t* offsets, uint32_t* edges) {
  auto* g = static_cast<Plain*>(h);
  std::copy(g->labels.begin(), g->labels.end(), labels);
  offsets[0] = 0;
  for (uint32_t i = 0; i < g->num_vertices; i++) {
    std::vector<uint32_t> row = i < g->adj.size() ? g->adj[i] : std::vector<uint32_t>();
    std::sort(row.begin(), row.end());
    offsets[i + 1] = offsets[i] + uint32_t(row.size());
    std::copy(row.begin(), row.end(), edges + offsets[i]);
  }
}

void orc_free(void* h) { delete static_cast<Plain*>(h); }

uint32_t orc_murmur2(const void* key, int len, uint32_t seed) { return murmur2(key, len, seed); }
uint64_t orc_fmix64(uint64_t k) { return fmix64(k); }

// build_signature (graph_format_transformer.cc:217-281).  Word 0 holds the
// label; 240 two-bit saturating counters (0 -> 1 -> 3) are indexed by the
// MurmurHash2 of each neighbour's label.  The reference shifts by 2*b with b
// in [0,30], i.e. by up to 60 bits; x86-64 and AArch64 both reduce a 32-bit
// shift count modulo 32, so the effective shift is (2*b) & 31 and only eight
// counter positions per word are reachable.  That behaviour is kept.
void orc_build_signature(uint32_t V, const int32_t* labels, const uint32_t* offsets,
                         const uint32_t* edges, int column_oriented, uint32_t* out) {
  std::vector<uint32_t> sig(size_t(V) * kSigWords, 0);
  const uint32_t slots = (kSigWords * 32 - 32) / 2;  // 240
  for (uint32_t i = 0; i < V; i++) {
    uint32_t* s = &sig[size_t(i) * kSigWords];
    s[0] = uint32_t(labels[i]);
    for (uint32_t e = offsets[i]; e < offsets[i + 1]; e++) {
      uint32_t hp = murmur_u32(uint32_t(labels[edges[e]])) % slots;
      uint32_t a = 2 * hp / 32, b = 2 * hp % 32;
      uint32_t sh = (2 * b) & 31;
      uint32_t t = s[1 + a];
      uint32_t c = (t >> sh) & 3u;
      c = (c == 0) ? 1u : 3u;
      s[1 + a] = t | (c << sh);
    }
  }
  if (!column_oriented) {
    std::copy(sig.begin(), sig.end(), out);
  } else {
    for (int j = 0; j < kSigWords; j++)
      for (uint32_t k = 0; k < V; k++) out[size_t(j) * V + k] = sig[size_t(k) * kSigWords + j];
  }
}

uint32_t orc_pcsr_num_units(int32_t L) { return uint32_t(L) * uint32_t(L + 1) / 2; }
int32_t orc_edge_label(int32_t a, int32_t b) { return edge_label(a, b); }

namespace {
// Partition of graph_format_transformer.cc:84-107: per unit, the keys in
// ascending vertex order and each key's neighbours in row order.
struct Units {
  std::vector<std::vector<uint32_t>> keys;
  std::vector<std::vector<std::vector<uint32_t>>> lists;
};
Units partition_units(uint32_t V, int32_t L, const int32_t* labels, const uint32_t* off, const uint32_t* adj) {
  Units u;
  uint32_t U = orc_pcsr_num_units(L);
  u.keys.resize(U);
  u.lists.resize(U);
  for (uint32_t i = 0; i < V; i++) {
    for (uint32_t e = off[i]; e < off[i + 1]; e++) {
      int32_t el = edge_label(labels[i], labels[adj[e]]);
      auto& ks = u.keys[el];
      if (ks.empty() || ks.back() != i) {
        ks.push_back(i);
        u.lists[el].emplace_back();
      }
      u.lists[el].back().push_back(adj[e]);
    }
  }
  return u;
}
}  // namespace

void orc_pcsr_sizes(uint32_t V, int32_t L, const int32_t* labels, const uint32_t* off, const uint32_t* adj,
                    uint32_t* unit_keys, uint32_t* unit_edges) {
  Units u = partition_units(V, L, labels, off, adj);
  for (size_t i = 0; i < u.keys.size(); i++) {
    unit_keys[i] = uint32_t(u.keys[i].size());
    uint64_t s = 0;
    for (auto& l : u.lists[i]) s += l.size();
    unit_edges[i] = uint32_t(s);
  }
}

// UndirectedPlainToPCSRTransformer::transform (graph_format_transformer.cc:39-215):
// per unit, 32-word buckets of up to 15 (key, start) pairs; bucket = MurmurHash2
// of the key mod num_keys; a full group of 15 chains (word 30) to the next
// empty bucket in ascending order; word 31 closes the last list.  Lists are
// laid out in bucket-slot order.  The reference finds each key's list with a
// linear `find`; this uses a binary search over the ascending key array,
// which returns the same index.
void orc_build_pcsr(uint32_t V, int32_t L, const int32_t* labels, const uint32_t* off, const uint32_t* adj,
                    uint32_t* offsets_out, uint32_t* edges_out) {
  Units u = partition_units(V, L, labels, off, adj);
  size_t obase = 0, ebase = 0;
  for (size_t unit = 0; unit < u.keys.size(); unit++) {
    const auto& keys = u.keys[unit];
    const auto& lists = u.lists[unit];
    const uint32_t nk = uint32_t(keys.size());
    uint32_t ne = 0;
    for (auto& l : lists) ne += uint32_t(l.size());
    uint32_t* o = offsets_out + obase;
    uint32_t* ed = edges_out + ebase;
    for (uint64_t j = 0; j < uint64_t(nk) * 16; j++) { o[2 * j] = kInvalid; o[2 * j + 1] = 0; }
    for (uint32_t j = 0; j < ne; j++) ed[j] = kInvalid;
    std::vector<std::vector<uint32_t>> buckets(nk);
    for (uint32_t k : keys) buckets[murmur_u32(k) % nk].push_back(k);
    std::deque<uint32_t> empty;
    for (uint32_t j = 0; j < nk; j++)
      if (buckets[j].empty()) empty.push_back(j);
    for (uint32_t j = 0; j < nk; j++) {
      const auto& b = buckets[j];
      if (b.empty()) continue;
      uint32_t full = uint32_t(b.size()) / 15, rest = uint32_t(b.size()) % 15, slot = j;
      for (uint32_t g = 0; g < full; g++) {
        for (uint32_t l = 0; l < 15; l++) o[32 * size_t(slot) + 2 * l] = b[g * 15 + l];
        uint32_t nxt = empty.front();
        empty.pop_front();
        o[32 * size_t(slot) + 30] = nxt;
        slot = nxt;
      }
      for (uint32_t l = 0; l < rest; l++) o[32 * size_t(slot) + 2 * l] = b[full * 15 + l];
    }
    uint32_t pos = 0;
    for (uint32_t j = 0; j < nk; j++) {
      for (uint32_t k = 0; k < 15; k++) {
        uint32_t vid = o[32 * size_t(j) + 2 * k];
        if (vid == kInvalid) break;
        size_t idx = size_t(std::lower_bound(keys.begin(), keys.end(), vid) - keys.begin());
        const auto& nl = lists[idx];
        o[32 * size_t(j) + 2 * k + 1] = pos;
        o[32 * size_t(j) + 2 * (k + 1) + 1] = pos + uint32_t(nl.size());
        for (uint32_t x : nl) ed[pos++] = x;
      }
    }
    obase += size_t(nk) * 32;
    ebase += ne;
  }
}

// filter_kernel (match/GSI_kernels.cuh:8-24): word 0 equal (the label), and
// words 1..15 of the query signature a bit-subset of the data signature.
void orc_gsi_filter(uint32_t V, const uint32_t* ds, const uint32_t* qs, uint8_t* flags) {
  for (uint32_t v = 0; v < V; v++) {
    const uint32_t* d = ds + size_t(v) * kSigWords;
    bool ok = d[0] == qs[0];
    for (int i = 1; ok && i < kSigWords; i++) ok = (qs[i] & d[i]) == qs[i];
    flags[v] = ok ? 1 : 0;
  }
}

// initialise_kernel (match/MMatch_kernels.cuh:6-16): label equal, degree >= query degree.
void orc_mmatch_init(uint32_t V, const int32_t* labels, const uint32_t* off, int32_t label,
                     uint32_t degree, uint8_t* flags) {
  for (uint32_t v = 0; v < V; v++) flags[v] = (labels[v] == label && off[v + 1] - off[v] >= degree) ? 1 : 0;
}

uint64_t orc_simplify(uint32_t V, const uint32_t* off, const uint32_t* adj, uint32_t* oo, uint32_t* oe) {
  uint64_t w = 0;
  oo[0] = 0;
  for (uint32_t v = 0; v < V; v++) {
    std::vector<uint32_t> row(adj + off[v], adj + off[v + 1]);
    std::sort(row.begin(), row.end());
    uint32_t prev = kInvalid;
    for (uint32_t x : row) {
      if (x == v || x == prev) continue;
      oe[w++] = x;
      prev = x;
    }
    oo[v + 1] = uint32_t(w);
  }
  return w;
}

// Neighbour-support refinement, one Jacobi step per iteration, with
// per-class thresholds: u's query neighbours are grouped by class (cls[w],
// null = every vertex its own class); for each group S, v stays in C(u) only
// if some data neighbour of v is in C(w) for every w in S, and at least |S|
// adjacency entries of v are in the union of C(w), w in S, as they stood at
// the start of the step.  This is the pull-mode check of MMatch
// (count_neighbors_kernel + check_re_kernel, MMatch_kernels.cuh:28-117,
// 190-214) with the class counts of its refine plan (MMatch.cu:317-541) as
// the thresholds; with every vertex its own class every threshold is one.
void orc_refine(uint32_t V, const int32_t* labels, const uint32_t* off, const uint32_t* adj,
                uint32_t n, const uint32_t* qadj, const uint32_t* cls, int iterations, uint8_t* cand) {
  (void)labels;
  std::vector<uint8_t> next(size_t(n) * V);
  for (int it = 0; it < iterations; it++) {
    for (uint32_t u = 0; u < n; u++) {
      // groups of u's neighbours
      std::vector<std::vector<uint32_t>> groups;
      for (uint32_t w = 0; w < n; w++) {
        if (!((qadj[u] >> w) & 1u)) continue;
        bool placed = false;
        for (auto& gr : groups)
          if (cls && cls[gr[0]] == cls[w]) { gr.push_back(w); placed = true; break; }
        if (!placed) groups.push_back(std::vector<uint32_t>(1, w));
      }
      for (uint32_t v = 0; v < V; v++) {
        uint8_t keep = cand[size_t(u) * V + v];
        for (size_t gi = 0; keep && gi < groups.size(); gi++) {
          const std::vector<uint32_t>& gr = groups[gi];
          uint64_t in_union = 0;
          for (uint32_t e = off[v]; e < off[v + 1]; e++) {
            bool any = false;
            for (uint32_t w : gr) any = any || cand[size_t(w) * V + adj[e]] != 0;
            in_union += any ? 1 : 0;
          }
          keep = in_union >= gr.size();
          for (uint32_t w : gr) {
            bool found = false;
            for (uint32_t e = off[v]; e < off[v + 1] && !found; e++) found = cand[size_t(w) * V + adj[e]] != 0;
            keep = keep && found;
          }
        }
        next[size_t(u) * V + v] = keep;
      }
    }
    std::copy(next.begin(), next.end(), cand);
  }
}

namespace {
struct MatchCtx {
  uint32_t V;
  const int32_t* labels;
  const uint32_t* off;
  const uint32_t* adj;
  uint32_t n;
  uint64_t seed;
  std::vector<int32_t> plabel;    // label of the query vertex at each position
  std::vector<uint32_t> pdeg;     // its query degree
  std::vector<uint32_t> pvert;    // query vertex id at each position
  std::vector<std::vector<uint32_t>> bwd;  // backward-neighbour positions
};

struct Local {
  uint64_t count = 0, hash = 0;
  uint64_t levels[32] = {0};
};

void dfs(const MatchCtx& c, uint32_t depth, uint32_t* f, uint64_t S, Local& out) {
  const auto& b = c.bwd[depth];
  // Driver: the shortest backward neighbour list.
  uint32_t drv = 0;
  uint32_t best = kInvalid;
  for (uint32_t j : b) {
    uint32_t len = c.off[f[j] + 1] - c.off[f[j]];
    if (len < best) { best = len; drv = j; }
  }
  const uint32_t* dl = c.adj + c.off[f[drv]];
  const int32_t lab = c.plabel[depth];
  const uint32_t dq = c.pdeg[depth];
  const uint64_t term_base = uint64_t(c.pvert[depth]) << 32;
  for (uint32_t i = 0; i < best; i++) {
    uint32_t x = dl[i];
    if (c.labels[x] != lab || c.off[x + 1] - c.off[x] < dq) continue;
    bool ok = true;
    for (uint32_t j : b) {
      if (j == drv) continue;
      const uint32_t* l = c.adj + c.off[f[j]];
      const uint32_t* e = c.adj + c.off[f[j] + 1];
      if (!std::binary_search(l, e, x)) { ok = false; break; }
    }
    if (!ok) continue;
    for (uint32_t j = 0; j < depth && ok; j++) ok = f[j] != x;
    if (!ok) continue;
    uint64_t S2 = S + fmix64(term_base | x);
    out.levels[depth]++;
    if (depth + 1 == c.n) {
      out.count++;
      out.hash += fmix64(c.seed + S2);
    } else {
      f[depth] = x;
      dfs(c, depth + 1, f, S2, out);
    }
  }
}
}  // namespace

int orc_match(uint32_t V, const int32_t* labels, const uint32_t* off, const uint32_t* adj,
              uint32_t n, const int32_t* qlabels, uint32_t m, const uint32_t* qedges,
              const uint32_t* order, int num_threads, uint64_t seed,
              uint64_t* count, uint64_t* hash, uint64_t* level_counts) {
  if (n == 0 || n > 32) return -1;
  std::vector<uint32_t> qadj(n, 0), qdeg(n, 0);
  for (uint32_t e = 0; e < m; e++) {
    uint32_t a = qedges[2 * e], b = qedges[2 * e + 1];
    if (a >= n || b >= n) return -2;
    if (a == b) continue;  // query self-loops never constrain an injective map
    if (!((qadj[a] >> b) & 1u)) { qdeg[a]++; qdeg[b]++; }
    qadj[a] |= 1u << b;
    qadj[b] |= 1u << a;
  }
  std::vector<uint32_t> ord(n);
  if (order) {
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t i = 0; i < n; i++) {
      if (order[i] >= n || seen[order[i]]) return -3;
      seen[order[i]] = 1;
      ord[i] = order[i];
    }
  } else {
    // Default: the rule of GSI::generate_join_order (match/GSI.cu:105-149)
    // over candidate counts from the label and degree test: the vertex with
    // the fewest candidates first, then repeatedly the unplaced neighbour of
    // the placed ones with the lowest score, a vertex's score shrinking by
    // 0.9 for every placed neighbour (lowest id on ties).  Any order gives the
    // same count and hash; this one keeps the search small.
    std::vector<uint32_t> qlab_idx(n);
    std::vector<int32_t> distinct;
    for (uint32_t u = 0; u < n; u++) {
      auto it = std::find(distinct.begin(), distinct.end(), qlabels[u]);
      qlab_idx[u] = uint32_t(it - distinct.begin());
      if (it == distinct.end()) distinct.push_back(qlabels[u]);
    }
    // hist[k][d]: data vertices of the k-th query label with degree d (d capped at 32)
    std::vector<std::array<uint64_t, 33>> hist(distinct.size());
    for (auto& h : hist) h.fill(0);
    for (uint32_t v = 0; v < V; v++) {
      auto it = std::find(distinct.begin(), distinct.end(), labels[v]);
      if (it == distinct.end()) continue;
      const uint32_t d = std::min<uint32_t>(off[v + 1] - off[v], 32u);
      hist[size_t(it - distinct.begin())][d]++;
    }
    std::vector<double> score(n);
    for (uint32_t u = 0; u < n; u++) {
      uint64_t cnt = 0;
      for (uint32_t d = std::min<uint32_t>(qdeg[u], 32u); d <= 32; d++) cnt += hist[qlab_idx[u]][d];
      score[u] = double(cnt);
    }
    uint32_t placed = 0;
    for (uint32_t i = 0; i < n; i++) {
      uint32_t bu = n;
      for (uint32_t u = 0; u < n; u++) {
        if ((placed >> u) & 1u) continue;
        if (i > 0 && !(qadj[u] & placed)) continue;
        if (bu == n || score[u] < score[bu]) bu = u;
      }
      if (bu == n) return -4;  // disconnected query
      ord[i] = bu;
      placed |= 1u << bu;
      for (uint32_t w = 0; w < n; w++)
        if (((qadj[bu] >> w) & 1u) && !((placed >> w) & 1u)) score[w] *= 0.9;
    }
  }
  MatchCtx c;
  c.V = V; c.labels = labels; c.off = off; c.adj = adj; c.n = n; c.seed = seed;
  c.plabel.resize(n); c.pdeg.resize(n); c.pvert.resize(n); c.bwd.resize(n);
  std::vector<uint32_t> pos(n);
  for (uint32_t i = 0; i < n; i++) pos[ord[i]] = i;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t u = ord[i];
    c.plabel[i] = qlabels[u];
    c.pdeg[i] = qdeg[u];
    c.pvert[i] = u;
    for (uint32_t w = 0; w < n; w++)
      if (((qadj[u] >> w) & 1u) && pos[w] < i) c.bwd[i].push_back(pos[w]);
    if (i > 0 && c.bwd[i].empty()) return -4;  // disconnected query or order
  }
  std::vector<uint32_t> roots;
  for (uint32_t v = 0; v < V; v++)
    if (labels[v] == c.plabel[0] && off[v + 1] - off[v] >= c.pdeg[0]) roots.push_back(v);

  if (num_threads <= 0) num_threads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<size_t> next{0};
  std::vector<Local> locals(static_cast<size_t>(num_threads));
  auto worker = [&](int t) {
    uint32_t f[32];
    Local& L = locals[size_t(t)];
    const uint64_t tb = uint64_t(c.pvert[0]) << 32;
    for (;;) {
      size_t i = next.fetch_add(1);
      if (i >= roots.size()) break;
      uint32_t r = roots[i];
      uint64_t S = fmix64(tb | r);
      L.levels[0]++;
      if (n == 1) { L.count++; L.hash += fmix64(seed + S); continue; }
      f[0] = r;
      dfs(c, 1, f, S, L);
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < num_threads; t++) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();
  uint64_t C = 0, H = 0, lv[32] = {0};
  for (auto& L : locals) {
    C += L.count;
    H += L.hash;
    for (int d = 0; d < 32; d++) lv[d] += L.levels[d];
  }
  *count = C;
  *hash = H;
  if (level_counts)
    for (uint32_t d = 0; d < n; d++) level_counts[d] = lv[d];
  return 0;
}

// K4 subgraphs of a simple graph, listed once each: every edge oriented
// towards the endpoint of higher (degree, id) rank, then for every oriented
// edge (u, v) the common out-neighbours W of u and v, and for every w in W
// its out-neighbours in W.  Also returns the number of embeddings of K4 plus
// a pendant vertex at query vertex 0 (the K4+pendant identity): each K4
// subgraph has 24 embeddings, each of its vertices the image of vertex 0 in
// 6 of them, and the pendant is any neighbour of that image outside the
// other three, so the count is 6 * sum over K4 subgraphs of the sum of
// (deg - 3) over their vertices.  A cross-check for counting at scales the
// backtracking matcher cannot finish; returns 0, negative on bad input.
int orc_k4_pendant(uint32_t V, const uint32_t* off, const uint32_t* adj, int num_threads, uint64_t* k4,
                   uint64_t* pendant) {
  if (!off || !k4 || !pendant || (off[V] && !adj)) return -1;
  auto before = [&](uint32_t a, uint32_t b) {
    const uint32_t da = off[a + 1] - off[a], db = off[b + 1] - off[b];
    return da < db || (da == db && a < b);
  };
  std::vector<uint64_t> oo(size_t(V) + 1, 0);
  for (uint32_t v = 0; v < V; v++) {
    uint64_t c = 0;
    for (uint32_t i = off[v]; i < off[v + 1]; i++) c += before(v, adj[i]) ? 1 : 0;
    oo[v + 1] = oo[v] + c;
  }
  std::vector<uint32_t> oe(oo[V]);
  for (uint32_t v = 0; v < V; v++) {
    uint64_t k = oo[v];
    for (uint32_t i = off[v]; i < off[v + 1]; i++)
      if (before(v, adj[i])) oe[k++] = adj[i];
  }
  if (num_threads <= 0) num_threads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<uint32_t> next{0};
  std::vector<uint64_t> cnt(size_t(num_threads), 0), wsum(size_t(num_threads), 0);
  auto worker = [&](int t) {
    std::vector<uint32_t> m1(V, 0), m2(V, 0), W;
    uint32_t stamp2 = 0;
    uint64_t c = 0, s = 0;
    for (;;) {
      const uint32_t u0 = next.fetch_add(64);
      if (u0 >= V) break;
      for (uint32_t u = u0; u < std::min(V, u0 + 64); u++) {
        for (uint64_t i = oo[u]; i < oo[u + 1]; i++) m1[oe[i]] = u + 1;
        const uint64_t du = off[u + 1] - off[u];
        for (uint64_t i = oo[u]; i < oo[u + 1]; i++) {
          const uint32_t v = oe[i];
          W.clear();
          for (uint64_t j = oo[v]; j < oo[v + 1]; j++)
            if (m1[oe[j]] == u + 1) W.push_back(oe[j]);
          if (W.size() < 2) continue;
          if (++stamp2 == 0) {  // wrapped: clear and restart the stamps
            std::fill(m2.begin(), m2.end(), 0u);
            stamp2 = 1;
          }
          for (uint32_t w : W) m2[w] = stamp2;
          const uint64_t duv = du + (off[v + 1] - off[v]);
          for (uint32_t w : W) {
            const uint64_t duvw = duv + (off[w + 1] - off[w]);
            for (uint64_t j = oo[w]; j < oo[w + 1]; j++) {
              const uint32_t x = oe[j];
              if (m2[x] == stamp2) {
                c++;
                s += duvw + (off[x + 1] - off[x]) - 12;
              }
            }
          }
        }
      }
    }
    cnt[size_t(t)] = c;
    wsum[size_t(t)] = s;
  };
  std::vector<std::thread> th;
  for (int t = 1; t < num_threads; t++) th.emplace_back(worker, t);
  worker(0);
  for (auto& t : th) t.join();
  uint64_t C = 0, S = 0;
  for (int t = 0; t < num_threads; t++) {
    C += cnt[size_t(t)];
    S += wsum[size_t(t)];
  }
  *k4 = C;
  *pendant = 6 * S;
  return 0;
}

}  // extern "C"
