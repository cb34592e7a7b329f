// Seeded synthetic workloads: R-MAT and Chung-Lu data graphs, uniform and
// Zipf labels, random-walk queries, and a t/v/e writer.  Host code only.
//
// The same source gives bit-identical graphs on x86-64 and AArch64: the RNG is
// integer, the floating point uses only +, -, *, / and sqrt (correctly
// rounded on both), the powers in the Chung-Lu weights and Zipf labels come
// from det_pow below instead of libm (whose last bit may differ between
// platforms), and the file is compiled with -ffp-contract=off so that no
// multiply-add is fused on one platform and not the other.
#include "../../include/fsig_gen.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

// x^y for x >= 1 and moderate |y|, from the series definitions alone:
//   ln x = e ln 2 + 2 atanh(t),  t = (m - 1) / (m + 1),  x = m 2^e, m in [1/sqrt2, sqrt2)
//   atanh t = sum t^(2k+1) / (2k+1)                   (|t| < 0.172, 16 terms)
//   exp z   = 2^k exp(r),  r = z - k ln 2, |r| <= ln2/2, exp r = sum r^j / j!  (24 terms)
// Relative error about 1e-15, which is ample for weights; what matters is
// that every step is a basic IEEE operation, so both platforms agree bit for
// bit.
double det_pow(double x, double y) {
  constexpr double kLn2 = 0.693147180559945309417232121458;
  constexpr double kSqrtHalf = 0.707106781186547524400844362105;
  int e = 0;
  double m = std::frexp(x, &e);  // exact: x = m 2^e, m in [0.5, 1)
  if (m < kSqrtHalf) {
    m *= 2.0;
    e -= 1;
  }
  const double t = (m - 1.0) / (m + 1.0), t2 = t * t;
  double term = t, s = 0.0;
  for (int k = 0; k < 16; k++) {
    s += term / double(2 * k + 1);
    term *= t2;
  }
  const double z = y * (double(e) * kLn2 + 2.0 * s);
  const double kf = std::floor(z / kLn2 + 0.5);
  const double r = z - kf * kLn2;
  double p = 1.0, acc = 1.0;
  for (int j = 1; j < 24; j++) {
    p = p * r / double(j);
    acc += p;
  }
  return std::ldexp(acc, int(kf));  // exact scaling by a power of two
}

inline uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// xoshiro256** (Blackman & Vigna, public domain).
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    for (auto& x : s) x = splitmix64(seed);
  }
  static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  inline uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
  }
  inline double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }
  inline uint32_t below(uint32_t n) { return uint32_t((uint64_t(uint32_t(next() >> 32)) * n) >> 32); }
};

// Open-addressing set of canonical edge keys (lo << 32 | hi).
struct EdgeSet {
  std::vector<uint64_t> slot;
  uint64_t mask;
  explicit EdgeSet(uint64_t expected) {
    uint64_t cap = 16;
    while (cap < expected * 2) cap <<= 1;
    slot.assign(cap, ~0ull);
    mask = cap - 1;
  }
  bool insert(uint64_t k) {
    uint64_t h = k * 0x9e3779b97f4a7c15ull;
    uint64_t i = (h ^ (h >> 29)) & mask;
    for (;;) {
      if (slot[i] == ~0ull) { slot[i] = k; return true; }
      if (slot[i] == k) return false;
      i = (i + 1) & mask;
    }
  }
};

// Shared driver: candidate edges are produced in blocks of kBlock; block b is
// generated from its own RNG stream (seed, b), several blocks in parallel, and
// consumed in block order, keeping the first E distinct edges.
constexpr uint64_t kBlock = 1u << 18;

template <class Sampler>
int distinct_edges(uint64_t E, uint64_t seed, int threads, uint32_t* edges, Sampler sample) {
  if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
  EdgeSet set(E);
  uint64_t have = 0, block = 0;
  std::vector<std::vector<uint64_t>> buf(static_cast<size_t>(threads), std::vector<uint64_t>(kBlock));
  uint64_t rounds = 0;
  while (have < E) {
    if (++rounds > 1000000) return FSIG_GEN_EGIVEUP;
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) {
      th.emplace_back([&, t] {
        uint64_t s = seed ^ (0xa0761d6478bd642full * (block + uint64_t(t) + 1));
        Rng r(splitmix64(s));
        for (uint64_t i = 0; i < kBlock; i++) buf[size_t(t)][i] = sample(r);
      });
    }
    for (auto& x : th) x.join();
    for (int t = 0; t < threads && have < E; t++) {
      for (uint64_t i = 0; i < kBlock && have < E; i++) {
        uint64_t k = buf[size_t(t)][i];
        if (k == ~0ull) continue;
        if (set.insert(k)) {
          edges[2 * have] = uint32_t(k >> 32);
          edges[2 * have + 1] = uint32_t(k);
          have++;
        }
      }
    }
    block += uint64_t(threads);
  }
  return 0;
}

inline uint64_t canon(uint32_t a, uint32_t b) {
  if (a > b) std::swap(a, b);
  return (uint64_t(a) << 32) | b;
}

}  // namespace

extern "C" {

int fsig_gen_rmat(uint32_t V, uint64_t E, double a, double b, double c, uint64_t seed, int threads,
                  uint32_t* edges) {
  if (V < 2 || !edges || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return FSIG_GEN_EINVAL;
  if (E > uint64_t(V) * (V - 1) / 2) return FSIG_GEN_EINVAL;
  int scale = 0;
  while ((1ull << scale) < V) scale++;
  const double ab = a + b, abc = a + b + c;
  auto sample = [=](Rng& r) -> uint64_t {
    for (int tries = 0; tries < 64; tries++) {
      uint64_t u = 0, v = 0;
      for (int l = 0; l < scale; l++) {
        double x = r.uniform();
        u <<= 1; v <<= 1;
        if (x < a) {
        } else if (x < ab) { v |= 1; }
        else if (x < abc) { u |= 1; }
        else { u |= 1; v |= 1; }
      }
      if (u < V && v < V && u != v) return canon(uint32_t(u), uint32_t(v));
    }
    return ~0ull;
  };
  return distinct_edges(E, seed, threads, edges, sample);
}

int fsig_gen_chung_lu(uint32_t V, uint64_t E, double gamma, uint64_t seed, int threads, uint32_t* edges) {
  if (V < 2 || !edges || gamma <= 1.0) return FSIG_GEN_EINVAL;
  if (E > uint64_t(V) * (V - 1) / 2) return FSIG_GEN_EINVAL;
  const double alpha = 1.0 / (gamma - 1.0);
  std::vector<double> w(V);
  double sum = 0;
  for (uint32_t i = 0; i < V; i++) sum += (w[i] = det_pow(double(i) + 1.0, -alpha));
  const double target = 2.0 * double(E), cap = std::sqrt(target);
  // Scale to the target total degree; cap at sqrt(2E) and rescale the rest.
  for (int it = 0; it < 8; it++) {
    double capped = 0, free_sum = 0;
    const double scale = target / sum;
    for (uint32_t i = 0; i < V; i++) {
      double x = w[i] * scale;
      if (x >= cap) capped += cap; else free_sum += x;
    }
    for (uint32_t i = 0; i < V; i++) {
      double x = w[i] * scale;
      w[i] = x >= cap ? cap : x * ((target - capped) / std::max(free_sum, 1e-300));
    }
    sum = 0;
    for (uint32_t i = 0; i < V; i++) sum += (w[i] = std::min(w[i], cap));
  }
  // Vose alias table over the weights.
  std::vector<double> prob(V);
  std::vector<uint32_t> alias(V, 0);
  {
    std::vector<uint32_t> small, large;
    std::vector<double> p(V);
    for (uint32_t i = 0; i < V; i++) {
      p[i] = w[i] * double(V) / sum;
      (p[i] < 1.0 ? small : large).push_back(i);
    }
    while (!small.empty() && !large.empty()) {
      uint32_t s = small.back(); small.pop_back();
      uint32_t l = large.back();
      prob[s] = p[s];
      alias[s] = l;
      p[l] = (p[l] + p[s]) - 1.0;
      if (p[l] < 1.0) { large.pop_back(); small.push_back(l); }
    }
    for (uint32_t i : large) prob[i] = 1.0;
    for (uint32_t i : small) prob[i] = 1.0;
  }
  const double* pp = prob.data();
  const uint32_t* al = alias.data();
  auto pick = [=](Rng& r) -> uint32_t {
    uint32_t i = r.below(V);
    return r.uniform() < pp[i] ? i : al[i];
  };
  auto sample = [=](Rng& r) -> uint64_t {
    for (int tries = 0; tries < 64; tries++) {
      uint32_t u = pick(r), v = pick(r);
      if (u != v) return canon(u, v);
    }
    return ~0ull;
  };
  return distinct_edges(E, seed, threads, edges, sample);
}

int fsig_gen_labels_uniform(uint32_t V, uint32_t L, uint64_t seed, int32_t* labels) {
  if (!labels || L == 0) return FSIG_GEN_EINVAL;
  Rng r(seed);
  for (uint32_t i = 0; i < V; i++) labels[i] = int32_t(r.below(L));
  return 0;
}

int fsig_gen_labels_zipf(uint32_t V, uint32_t L, double s, uint64_t seed, int32_t* labels) {
  if (!labels || L == 0) return FSIG_GEN_EINVAL;
  std::vector<double> cdf(L);
  double acc = 0;
  for (uint32_t k = 0; k < L; k++) cdf[k] = (acc += 1.0 / det_pow(double(k) + 1.0, s));
  Rng r(seed);
  for (uint32_t i = 0; i < V; i++) {
    double x = r.uniform() * acc;
    uint32_t k = uint32_t(std::upper_bound(cdf.begin(), cdf.end(), x) - cdf.begin());
    labels[i] = int32_t(k < L ? k : L - 1);
  }
  return 0;
}

int fsig_gen_csr(uint32_t V, uint64_t E, const uint32_t* edges, uint32_t* offsets, uint32_t* adj,
                 uint64_t* num_adj) {
  if (!edges || !offsets || !adj) return FSIG_GEN_EINVAL;
  std::vector<uint64_t> deg(size_t(V) + 1, 0);
  for (uint64_t e = 0; e < E; e++) {
    uint32_t a = edges[2 * e], b = edges[2 * e + 1];
    if (a >= V || b >= V) return FSIG_GEN_EINVAL;
    if (a == b) continue;
    deg[a]++; deg[b]++;
  }
  std::vector<uint64_t> pos(size_t(V) + 1, 0);
  for (uint32_t v = 0; v < V; v++) pos[v + 1] = pos[v] + deg[v];
  if (pos[V] > 0xffffffffull) return FSIG_GEN_EINVAL;
  std::vector<uint64_t> cur(pos.begin(), pos.end() - 1);
  for (uint64_t e = 0; e < E; e++) {
    uint32_t a = edges[2 * e], b = edges[2 * e + 1];
    if (a == b) continue;
    adj[cur[a]++] = b;
    adj[cur[b]++] = a;
  }
  // Sort and de-duplicate rows in parallel, then compact in one pass.
  std::vector<uint32_t> uniq(V, 0);
  const unsigned T = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; t++) {
    th.emplace_back([&, t] {
      for (uint32_t v = t; v < V; v += T) {
        uint32_t* row = adj + pos[v];
        const size_t len = size_t(pos[v + 1] - pos[v]);
        std::sort(row, row + len);
        uint32_t u = 0, prev = 0xffffffffu;
        for (size_t i = 0; i < len; i++) {
          if (row[i] == prev) continue;
          row[u++] = prev = row[i];
        }
        uniq[v] = u;
      }
    });
  }
  for (auto& x : th) x.join();
  uint64_t w = 0;
  offsets[0] = 0;
  for (uint32_t v = 0; v < V; v++) {
    const uint32_t* row = adj + pos[v];
    if (w != pos[v]) std::memmove(adj + w, row, sizeof(uint32_t) * uniq[v]);
    w += uniq[v];
    offsets[v + 1] = uint32_t(w);
  }
  if (num_adj) *num_adj = w;
  return 0;
}

int fsig_gen_query(uint32_t V, const uint32_t* off, const uint32_t* adj, const int32_t* labels, uint32_t n,
                   int mode, uint64_t seed, int32_t* qlabels, uint32_t* qedges, uint32_t* m, uint32_t* src) {
  return fsig_gen_query_ex(V, off, adj, labels, n, mode, seed, INT32_MIN, qlabels, qedges, m, src);
}

int fsig_gen_query_ex(uint32_t V, const uint32_t* off, const uint32_t* adj, const int32_t* labels, uint32_t n,
                      int mode, uint64_t seed, int32_t min_label, int32_t* qlabels, uint32_t* qedges, uint32_t* m,
                      uint32_t* src) {
  if (n < 2 || n > 32 || !off || !adj || !labels || !qlabels || !qedges || !m || !src) return FSIG_GEN_EINVAL;
  if (mode != FSIG_QUERY_INDUCED && mode != FSIG_QUERY_DENSE && mode != FSIG_QUERY_SPARSE) return FSIG_GEN_EINVAL;
  Rng r(seed);
  std::vector<uint32_t> set;
  std::vector<std::pair<uint32_t, uint32_t>> walk_edges;
  for (int attempt = 0; attempt < 4000; attempt++) {
    uint32_t start = r.below(V);
    if (off[start + 1] == off[start] || labels[start] < min_label) continue;
    set.assign(1, start);
    walk_edges.clear();
    uint32_t cur = start;
    auto index_of = [&](uint32_t v) -> int {
      for (size_t i = 0; i < set.size(); i++)
        if (set[i] == v) return int(i);
      return -1;
    };
    if (mode == FSIG_QUERY_DENSE) {
      // Randomised greedy walk: with probability 3/4 step to a frontier
      // vertex with the most edges into the set (ties at random), otherwise
      // to a uniformly random frontier vertex.  Frontier edge counts are
      // kept incrementally as vertices join.
      std::vector<std::pair<uint32_t, uint32_t>> front;  // (vertex, edges into set), by first appearance
      std::unordered_map<uint32_t, uint32_t> where;       // vertex -> index in front
      auto add = [&](uint32_t v) {
        for (uint32_t k = off[v]; k < off[v + 1]; k++) {
          const uint32_t c = adj[k];
          if (labels[c] < min_label) continue;
          auto it = where.find(c);
          if (it == where.end()) {
            where.emplace(c, uint32_t(front.size()));
            front.emplace_back(c, 1u);
          } else if (front[it->second].second != 0xffffffffu) {
            front[it->second].second++;
          }
        }
        auto it = where.find(v);
        if (it == where.end()) {
          where.emplace(v, uint32_t(front.size()));
          front.emplace_back(v, 0xffffffffu);
        } else {
          front[it->second].second = 0xffffffffu;  // in the set
        }
      };
      add(start);
      while (set.size() < n) {
        uint32_t pick = 0xffffffffu;
        if ((r.next() & 3) != 0) {
          uint32_t best = 0, ties = 0;
          for (auto& fc : front) {
            if (fc.second == 0xffffffffu) continue;
            if (fc.second > best) { best = fc.second; ties = 1; pick = fc.first; }
            else if (fc.second == best && r.below(++ties) == 0) pick = fc.first;
          }
        } else {
          uint32_t live = 0;
          for (auto& fc : front) live += fc.second != 0xffffffffu;
          if (live) {
            uint32_t k = r.below(live);
            for (auto& fc : front) {
              if (fc.second == 0xffffffffu) continue;
              if (k-- == 0) { pick = fc.first; break; }
            }
          }
        }
        if (pick == 0xffffffffu) break;
        set.push_back(pick);
        add(pick);
      }
    }
    for (uint32_t step = 0; step < 64 * n && set.size() < n; step++) {
      uint32_t d = off[cur + 1] - off[cur];
      if (d == 0) break;
      uint32_t nxt = adj[off[cur] + r.below(d)];
      if (labels[nxt] < min_label) {
        // resample among the qualifying neighbours (bounded tries)
        bool found = false;
        for (int t = 0; t < 32 && !found; t++) {
          nxt = adj[off[cur] + r.below(d)];
          found = labels[nxt] >= min_label;
        }
        if (!found) continue;
      }
      int ci = index_of(cur), ni = index_of(nxt);
      if (ni < 0) { set.push_back(nxt); ni = int(set.size()) - 1; }
      uint32_t a = uint32_t(ci), b = uint32_t(ni);
      if (a > b) std::swap(a, b);
      if (a != b) walk_edges.emplace_back(a, b);
      cur = nxt;
    }
    if (set.size() < n) continue;
    std::vector<std::pair<uint32_t, uint32_t>> es;
    if (mode == FSIG_QUERY_SPARSE) {
      es = walk_edges;
    } else {
      for (uint32_t i = 0; i < n; i++) {
        const uint32_t* b = adj + off[set[i]];
        const uint32_t* e = adj + off[set[i] + 1];
        for (uint32_t j = i + 1; j < n; j++)
          if (std::binary_search(b, e, set[j])) es.emplace_back(i, j);
      }
    }
    std::sort(es.begin(), es.end());
    es.erase(std::unique(es.begin(), es.end()), es.end());
    // dense: average degree above 3, or above 0.75 (n - 1) where 3 is out of
    // reach (n = 4 has at most average degree 3)
    if (mode == FSIG_QUERY_DENSE && !(8 * es.size() > std::min<size_t>(12 * size_t(n), 3 * size_t(n) * (n - 1))))
      continue;
    if (mode == FSIG_QUERY_SPARSE && !(2 * es.size() <= 3 * size_t(n))) continue;
    for (uint32_t i = 0; i < n; i++) {
      src[i] = set[i];
      qlabels[i] = labels[set[i]];
    }
    for (size_t i = 0; i < es.size(); i++) {
      qedges[2 * i] = es[i].first;
      qedges[2 * i + 1] = es[i].second;
    }
    *m = uint32_t(es.size());
    return 0;
  }
  return FSIG_GEN_EGIVEUP;
}

int fsig_write_tve(const char* path, uint32_t V, const int32_t* labels, uint64_t E, const uint32_t* edges) {
  if (!path || !labels || (E && !edges)) return FSIG_GEN_EINVAL;
  std::vector<uint32_t> deg(V, 0);
  for (uint64_t e = 0; e < E; e++) {
    if (edges[2 * e] >= V || edges[2 * e + 1] >= V) return FSIG_GEN_EINVAL;
    deg[edges[2 * e]]++;
    deg[edges[2 * e + 1]]++;
  }
  FILE* f = fopen(path, "wb");
  if (!f) return FSIG_GEN_EIO;
  std::vector<char> out;
  out.reserve(1 << 20);
  char line[96];
  auto flush = [&](bool force) {
    if (force || out.size() > (1u << 20)) {
      fwrite(out.data(), 1, out.size(), f);
      out.clear();
    }
  };
  int k = snprintf(line, sizeof line, "t %u %llu", V, (unsigned long long)E);
  out.insert(out.end(), line, line + k);
  for (uint32_t v = 0; v < V; v++) {
    k = snprintf(line, sizeof line, "\nv %u %d %u", v, labels[v], deg[v]);
    out.insert(out.end(), line, line + k);
    flush(false);
  }
  for (uint64_t e = 0; e < E; e++) {
    k = snprintf(line, sizeof line, "\ne %u %u", edges[2 * e], edges[2 * e + 1]);
    out.insert(out.end(), line, line + k);
    flush(false);
  }
  flush(true);
  return fclose(f) == 0 ? 0 : FSIG_GEN_EIO;
}

}  // extern "C"
