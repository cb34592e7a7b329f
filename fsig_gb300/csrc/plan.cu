// Host-side join orders with the reference's exact semantics, including its
// std::priority_queue tie-breaking (same container, comparator and push
// sequence), for the single-query path.  The batched path orders on the
// device with the same scores and ties broken by the lowest vertex id.
#include <algorithm>
#include <cstring>
#include <queue>
#include <utility>
#include <vector>

#include "match.h"

namespace fsig {
namespace {

// ScoredVertex (match/GSI.h:23-36): ordered by score only.
struct Scored {
  uint32_t id;
  float score;
  bool operator>(const Scored& o) const { return score > o.score; }
};
using MinQueue = std::priority_queue<Scored, std::vector<Scored>, std::greater<Scored>>;

}  // namespace

// GSI::generate_join_order (match/GSI.cu:105-149): start from the vertex with
// the fewest candidates; each later position takes the frontier vertex with
// the lowest score; the neighbours of each placed vertex have their score
// multiplied by 0.9.
void gsi_order_host(const HostQuery& q, const uint32_t* cand, uint32_t* order) {
  const uint32_t n = q.n;
  std::vector<Scored> qv(n);
  std::vector<char> visited(n, 0);
  for (uint32_t i = 0; i < n; i++) qv[i] = Scored{i, float(cand[i])};
  for (uint32_t pos = 0; pos < n; pos++) {
    MinQueue pq;
    if (pos == 0) {
      for (auto& s : qv) pq.push(s);
    } else {
      for (uint32_t j = 0; j < pos; j++)
        for (uint32_t w : q.nbr[order[j]])
          if (!visited[w]) pq.push(qv[w]);
    }
    const uint32_t u = pq.top().id;
    order[pos] = u;
    visited[u] = 1;
    for (uint32_t w : q.nbr[u]) qv[w].score = float(double(qv[w].score) * 0.9);
  }
}

namespace {

// MMatch::decompose_query_graph (match/MMatch.cu:543-607): peel degree-1
// vertices; 2 = 2-core, 1 = forest, 0 = leaf.
std::vector<uint32_t> decompose(const HostQuery& q) {
  const uint32_t n = q.n;
  std::vector<uint32_t> d(n), type(n);
  std::queue<uint32_t> leaves;
  for (uint32_t i = 0; i < n; i++) {
    d[i] = uint32_t(q.nbr[i].size());
    if (d[i] == 1) leaves.push(i);
  }
  while (!leaves.empty()) {
    const uint32_t v = leaves.front();
    for (uint32_t w : q.nbr[v]) {
      const uint32_t dw = d[w];
      if (dw == 0) continue;
      d[w]--;
      if (dw == 2) leaves.push(w);
    }
    leaves.pop();
    d[v] = 0;
  }
  for (uint32_t i = 0; i < n; i++) type[i] = d[i] >= 2 ? 2 : (q.nbr[i].size() == 1 ? 0 : 1);
  return type;
}

// MMatch::find_equivalent_classes (match/MMatch.cu:34-173): classes of equal
// (degree, label), split while no neighbour permutation maps classes and
// labels onto each other.  The permutation search is the reference's
// next_permutation walk from the current arrangement; it is skipped (the
// vertices are treated as different) above degree 10, where the reference's
// search would take minutes.
struct Classes {
  std::vector<std::vector<uint32_t>> members;
  std::vector<std::pair<uint32_t, uint32_t>> inv;  // (class, index in class)
};

bool maps(const HostQuery& q, const std::vector<uint32_t>& a, const std::vector<uint32_t>& b,
          const std::vector<std::pair<uint32_t, uint32_t>>& inv) {
  for (size_t i = 0; i < a.size(); i++)
    if (inv[a[i]].first != inv[b[i]].first || q.label[a[i]] != q.label[b[i]]) return false;
  return true;
}

bool permutation_match(const HostQuery& q, const std::vector<uint32_t>& crt, std::vector<uint32_t> tgt,
                       const std::vector<std::pair<uint32_t, uint32_t>>& inv) {
  if (crt.size() != tgt.size() || crt.size() > 10) return false;
  do {
    if (maps(q, crt, tgt, inv)) return true;
  } while (std::next_permutation(tgt.begin(), tgt.end()));
  return false;
}

Classes equivalent_classes(const HostQuery& q) {
  const uint32_t n = q.n;
  Classes c;
  c.members.push_back(std::vector<uint32_t>(1, 0));
  c.inv.assign(n, {0, 0});
  for (uint32_t i = 1; i < n; i++) {
    bool eq = false;
    for (uint32_t j = 0; j < c.members.size(); j++) {
      const uint32_t r = c.members[j][0];
      if (q.nbr[i].size() == q.nbr[r].size() && q.label[i] == q.label[r]) {
        eq = true;
        c.members[j].push_back(i);
        c.inv[i] = {j, uint32_t(c.members[j].size() - 1)};
      }
    }
    if (!eq) {
      c.members.push_back(std::vector<uint32_t>(1, i));
      c.inv[i] = {uint32_t(c.members.size() - 1), 0};
    }
  }
  std::vector<uint32_t> checked;
  for (auto& m : c.members)
    for (size_t i = 1; i < m.size(); i++) checked.push_back(m[i]);
  size_t old = c.members.size();
  while (old != n && !checked.empty()) {
    std::vector<uint32_t> next_checked;
    for (uint32_t v : checked) {
      if (c.members[c.inv[v].first].size() == 1) continue;
      const uint32_t target = c.inv[v].second == 0 ? 1 : 0;
      const std::vector<uint32_t>& crt = q.nbr[v];
      bool eq = permutation_match(q, crt, q.nbr[c.members[c.inv[v].first][target]], c.inv);
      if (!eq) {
        std::vector<uint32_t> cls = c.members[c.inv[v].first];
        cls.erase(cls.begin() + c.inv[v].second);
        c.members[c.inv[v].first] = cls;
        for (uint32_t i = 0; i < cls.size(); i++) c.inv[cls[i]] = {c.inv[v].first, i};
        for (size_t i = old; i < c.members.size(); i++) {
          if (q.label[v] != q.label[c.members[i][0]]) continue;
          c.inv[v].first = uint32_t(i);
          eq = permutation_match(q, crt, q.nbr[c.members[i][0]], c.inv);
          if (eq) {
            c.members[i].push_back(v);
            c.inv[v].second = uint32_t(c.members[i].size() - 1);
            break;
          }
        }
        if (!eq) {
          c.members.push_back(std::vector<uint32_t>(1, v));
          c.inv[v] = {uint32_t(c.members.size() - 1), 0};
        }
        for (uint32_t w : crt)
          if (std::find(next_checked.begin(), next_checked.end(), w) == next_checked.end()) next_checked.push_back(w);
      }
    }
    old = c.members.size();
    checked = next_checked;
  }
  return c;
}

// MMatch::compute_weight (match/MMatch.cu:270-296): BFS levels weighted by depth.
double bfs_weight(const HostQuery& q, uint32_t root) {
  std::vector<char> seen(q.n, 0);
  seen[root] = 1;
  uint32_t nseen = 1, level = 0;
  double w = 0;
  std::vector<uint32_t> frontier(1, root);
  while (nseen < q.n) {
    std::vector<uint32_t> next;
    for (uint32_t v : frontier)
      for (uint32_t x : q.nbr[v])
        if (!seen[x]) { next.push_back(x); seen[x] = 1; }
    if (next.empty()) break;
    w += double(next.size()) * (level + 1);
    level++;
    nseen += uint32_t(next.size());
    frontier = next;
  }
  return w;
}

}  // namespace

void mmatch_structure(const HostQuery& q, uint32_t* types, uint32_t* classes) {
  const std::vector<uint32_t> t = decompose(q);
  const Classes c = equivalent_classes(q);
  for (uint32_t i = 0; i < q.n; i++) {
    if (types) types[i] = t[i];
    if (classes) classes[i] = c.inv[i].first;
  }
}

// MMatch::generate_join_order (match/MMatch.cu:1575-1641).  Class candidate
// counts are the counts of each class's first member.  Without a 2-core the
// first position is restricted to the class of the forest vertex of least BFS
// weight (select_min_spanning_tree, MMatch.cu:298-315).
void mmatch_order_host(const HostQuery& q, const uint32_t* cand, uint32_t* order) {
  const uint32_t n = q.n;
  const std::vector<uint32_t> vtype = decompose(q);
  const Classes c = equivalent_classes(q);
  const uint32_t nc = uint32_t(c.members.size());
  std::vector<uint32_t> ctype(nc), ccount(nc);
  for (uint32_t i = 0; i < nc; i++) {
    ctype[i] = vtype[c.members[i][0]];
    ccount[i] = cand[c.members[i][0]];
  }
  float max_core = 0, max_forest = 0;
  bool has_core = false;
  for (uint32_t i = 0; i < nc; i++) {
    if (ctype[i] == 2) has_core = true;
    if (ctype[i] == 2 && float(ccount[i]) > max_core) max_core = float(ccount[i]);
    else if (ctype[i] == 1 && float(ccount[i]) > max_forest) max_forest = float(ccount[i]);
  }
  uint32_t root_class = 0xffffffffu;
  if (!has_core) {
    double best = 0;
    bool any = false;
    uint32_t root = 0;
    for (uint32_t i = 0; i < n; i++) {
      if (vtype[i] != 1) continue;
      double w = bfs_weight(q, i);
      if (!any || w < best) { best = w; root = i; any = true; }
    }
    if (any) root_class = c.inv[root].first;
  }
  std::vector<Scored> qv(n);
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t k = c.inv[i].first;
    float s;
    if (ctype[k] == 0) s = (float(ccount[k]) + max_forest) + max_core;
    else if (ctype[k] == 1) s = float(ccount[k]) + max_core;
    else s = float(ccount[k]);
    qv[i] = Scored{i, s};
  }
  std::vector<char> visited(n, 0);
  for (uint32_t pos = 0; pos < n; pos++) {
    MinQueue pq;
    if (pos == 0) {
      for (uint32_t i = 0; i < n; i++)
        if (root_class == 0xffffffffu || c.inv[i].first == root_class) pq.push(qv[i]);
    } else {
      for (uint32_t j = 0; j < pos; j++)
        for (uint32_t w : q.nbr[order[j]])
          if (!visited[w]) pq.push(qv[w]);
    }
    const uint32_t u = pq.top().id;
    order[pos] = u;
    visited[u] = 1;
  }
}

// Refinement classes: the coarsest partition of the query vertices that keeps
// apart vertices whose filter inputs differ (label, degree, signature) and is
// equitable (members of a class have as many query neighbours as each other
// in every class).  MMatch::find_equivalent_classes (match/MMatch.cu:44-173)
// looks for such classes with a permutation search over each vertex's
// neighbours; colour refinement reaches the coarsest one in polynomial time:
// each round splits the classes by the multiset of neighbour classes, until a
// round splits nothing.  Members of a class then have equal candidate sets
// after the filter and after every refinement step (by induction on the
// steps), so they share one bitmap.  cls[u] = the smallest member of u's class.
//
// dom[u], for a class's smallest member u: a class j != cls[u] of the same
// label with degree and signature bits within u's and at most as many
// neighbours as u in every class (the most constrained such j, lowest id on
// ties), else kNoClass.  Every condition on j is then implied by one on u, so
// C(u) stays within C(j) through the refinement, and a test of v in C(j)
// rejects early without changing any outcome (the optimised operators of
// MMatch::generate_refine_plan, match/MMatch.cu:317-541).
void refine_classes(const HostQuery& q, uint8_t* cls, uint8_t* dom) {
  const uint32_t n = q.n;
  uint32_t col[kMaxQ], next[kMaxQ], members[kMaxQ], reps;
  for (uint32_t u = 0; u < n; u++) {
    col[u] = u;
    for (uint32_t v = 0; v < u; v++)
      if (q.label[v] == q.label[u] && q.deg[v] == q.deg[u] &&
          std::memcmp(q.sig[v], q.sig[u], sizeof(q.sig[u])) == 0) {
        col[u] = v;
        break;
      }
  }
  // neighbours of u in the class with member mask m
  auto in_class = [&](uint32_t u, uint32_t m) { return uint32_t(__builtin_popcount(q.adj[u] & m)); };
  for (;;) {
    reps = 0;
    for (uint32_t u = 0; u < n; u++) members[u] = 0;
    for (uint32_t u = 0; u < n; u++) {
      members[col[u]] |= 1u << u;
      if (col[u] == u) reps |= 1u << u;
    }
    bool split = false;
    for (uint32_t u = 0; u < n; u++) {
      next[u] = u;
      for (uint32_t v = 0; v < u; v++) {
        if (col[v] != col[u]) continue;
        bool same = true;
        for (uint32_t r = reps; r && same; r &= r - 1) {
          const uint32_t m = members[__builtin_ctz(r)];
          same = in_class(u, m) == in_class(v, m);
        }
        if (same) { next[u] = v; break; }
      }
      split |= next[u] != col[u];
    }
    for (uint32_t u = 0; u < n; u++) col[u] = next[u];
    if (!split) break;
  }
  for (uint32_t u = 0; u < n; u++) {
    cls[u] = uint8_t(col[u]);
    dom[u] = uint8_t(kNoClass);
    if (col[u] != u) continue;
    uint32_t best = kNoClass;
    for (uint32_t r = reps; r; r &= r - 1) {
      const uint32_t j = __builtin_ctz(r);
      if (j == u || q.label[j] != q.label[u] || q.deg[j] > q.deg[u]) continue;
      if (best != kNoClass && q.deg[j] <= q.deg[best]) continue;
      bool implied = true;
      for (int k = 1; k < kSigWords && implied; k++) implied = (q.sig[j][k] & ~q.sig[u][k]) == 0;
      for (uint32_t y = reps; y && implied; y &= y - 1) {
        const uint32_t m = members[__builtin_ctz(y)];
        implied = in_class(j, m) <= in_class(u, m);
      }
      if (implied) best = j;
    }
    dom[u] = uint8_t(best);
  }
}

}  // namespace fsig
