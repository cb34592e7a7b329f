// Batch matching: candidate filter, neighbour-support refinement, candidate
// counts, device-side ordering, root compaction and the DFS enumerator.
//
// Reference counterparts:
//   filter_kernel / scatter_kernel            match/GSI_kernels.cuh:8-36
//   initialise_kernel / scatter_kernel        match/MMatch_kernels.cuh:6-26
//   count_neighbors_kernel + check_re_kernel  match/MMatch_kernels.cuh:28-117, 190-214
//   GSI::generate_join_order                  match/GSI.cu:105-149
//   MMatch::generate_join_order               match/MMatch.cu:1575-1641
//   GSI join kernels                          match/GSI_kernels.cuh:95-560
//   MMatch join kernels                       match/MMatch_kernels.cuh:374-820
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "match.h"
#include "mpnn.h"
#include "scan.cuh"

namespace fsig {

struct GraphView {
  uint32_t V;
  int32_t L;
  const int32_t* __restrict__ label;
  const uint32_t* __restrict__ off;
  const uint32_t* __restrict__ adj;
  const uint32_t* __restrict__ lseg;
  const uint4* __restrict__ sig;
  const uint32_t* __restrict__ old_of_new;
  const uint32_t* __restrict__ adj_old;  // null when lseg is
  const uint32_t* __restrict__ base;     // [L+1] first id of each label class
};

namespace {

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kChunk = 32;  // driver elements examined per refill (one per lane)

GraphView view_of(const DeviceGraph& g) {
  return GraphView{g.V, g.L, g.label, g.off, g.adj, g.lseg, g.sig, g.old_of_new, g.adj_old, g.base};
}

// Segment [lo, hi) of row v's neighbours with label l (0 <= l < L), from the
// dense table when the store has one, else by two binary searches in the row.
__device__ __forceinline__ void segment_of(const GraphView& g, uint32_t v, int32_t l, uint32_t& lo, uint32_t& hi) {
  if (g.lseg) {
    const uint32_t* s = g.lseg + uint64_t(v) * (uint64_t(g.L) + 1) + l;
    lo = s[0];
    hi = s[1];
  } else {
    const uint32_t b = __ldg(g.off + v), e = __ldg(g.off + v + 1);
    lo = lower_bound_u32(g.adj, b, e, __ldg(g.base + l));
    hi = lower_bound_u32(g.adj, lo, e, __ldg(g.base + l + 1));
  }
}

// ---------------------------------------------------------------------------
// Filter: one warp per aligned group of 32 (renumbered) data vertices, lane i
// holding vertex i of the group.  The group's vertices carry one or a few
// labels (ids are label-sorted).  The warp turns its 32 signatures around
// once: after a 32 x 32 bit transpose of each signature word (five rounds of
// shuffles), lane b holds, for word w, the mask of the group's vertices whose
// word w has bit b set, kept in shared memory.  The query vertices of each of
// the group's labels are then taken 32 at a time, one per lane: a lane ANDs
// the masks of the signature bits its query vertex requires (subset test,
// GSI_kernels.cuh:8-24), the label mask and the mask of vertices of at least
// its degree (initialise_kernel, MMatch_kernels.cuh:6-16), which is the
// query vertex's bitmap word for this group, written once.  Every bitmap word
// is written exactly once, so no clearing pass is needed.
// ---------------------------------------------------------------------------
constexpr uint32_t kFilterWarps = 8;

__device__ __forceinline__ uint32_t transpose_step(uint32_t x, uint32_t lane, uint32_t j, uint32_t m) {
  const uint32_t y = __shfl_xor_sync(kFull, x, j);
  return (lane & j) ? ((x & ~m) | ((y >> j) & m)) : ((x & m) | ((y << j) & ~m));
}

// Lane b receives bit b of every lane's x: bit i of the result = bit b of
// lane i's x (32 x 32 bit-matrix transpose).
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, uint32_t lane) {
  x = transpose_step(x, lane, 16, 0x0000ffffu);
  x = transpose_step(x, lane, 8, 0x00ff00ffu);
  x = transpose_step(x, lane, 4, 0x0f0f0f0fu);
  x = transpose_step(x, lane, 2, 0x33333333u);
  x = transpose_step(x, lane, 1, 0x55555555u);
  return x;
}

__global__ void __launch_bounds__(kFilterWarps * 32, 8) filter_kernel(GraphView g, const QVert* __restrict__ qv,
                                                                   const uint32_t* __restrict__ lab_gidx,
                                                                   const uint32_t* __restrict__ lab_begin,
                                                                   uint32_t mode, uint32_t* __restrict__ pool) {
  __shared__ uint32_t cols[kFilterWarps][kSigWords - 1][32];
  const uint32_t lane = threadIdx.x & 31;
  uint32_t (*col)[32] = cols[threadIdx.x >> 5];
  const uint32_t nwt = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ngroups = (g.V + 31) >> 5;
  const bool use_sig = mode & kFilterSignature, use_deg = mode & kFilterDegree;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < ngroups; w += nwt) {
    const uint32_t v = (w << 5) + lane;
    const bool live = v < g.V;
    const int32_t l = live ? g.label[v] : -1;
    // lane t: the group's vertices of degree >= t (query degrees are < 32)
    uint32_t atleast = kFull;
    if (use_deg) {
      const uint32_t deg = live ? g.off[v + 1] - g.off[v] : 0;
#pragma unroll 4
      for (uint32_t t = 0; t < 32; t++) {
        const uint32_t m = __ballot_sync(kFull, deg >= t);
        if (lane == t) atleast = m;
      }
    }
    if (use_sig) {
      uint4 s0 = make_uint4(0, 0, 0, 0), s1 = s0, s2 = s0, s3 = s0;
      if (live) {
        const uint4* p = g.sig + uint64_t(v) * 4;
        s0 = p[0]; s1 = p[1]; s2 = p[2]; s3 = p[3];
      }
      __syncwarp();
      // word 0 is the label; words 1..15 hold the neighbour-label counters
      col[0][lane] = warp_transpose32(s0.y, lane);
      col[1][lane] = warp_transpose32(s0.z, lane);
      col[2][lane] = warp_transpose32(s0.w, lane);
      col[3][lane] = warp_transpose32(s1.x, lane);
      col[4][lane] = warp_transpose32(s1.y, lane);
      col[5][lane] = warp_transpose32(s1.z, lane);
      col[6][lane] = warp_transpose32(s1.w, lane);
      col[7][lane] = warp_transpose32(s2.x, lane);
      col[8][lane] = warp_transpose32(s2.y, lane);
      col[9][lane] = warp_transpose32(s2.z, lane);
      col[10][lane] = warp_transpose32(s2.w, lane);
      col[11][lane] = warp_transpose32(s3.x, lane);
      col[12][lane] = warp_transpose32(s3.y, lane);
      col[13][lane] = warp_transpose32(s3.z, lane);
      col[14][lane] = warp_transpose32(s3.w, lane);
      __syncwarp();
    }
    const int32_t lfirst = __shfl_sync(kFull, l, 0);
    const uint32_t last_lane = min(31u, g.V - 1 - (w << 5));
    const int32_t llast = __shfl_sync(kFull, l, last_lane);
    for (int32_t lab = lfirst; lab <= llast; lab++) {
      const uint32_t lmask = __ballot_sync(kFull, l == lab);
      const uint32_t b = lab_begin[lab], e = lab_begin[lab + 1];
      for (uint32_t i0 = b; i0 < e; i0 += 32) {
        const uint32_t i = i0 + lane;
        uint32_t word = 0, qdeg = 0;
        const QVert* q = nullptr;
        if (i < e) {
          q = qv + lab_gidx[i];
          word = lmask;
          qdeg = min(q->deg, 31u);
          if (use_sig) {
            // word 0 (the label) is covered by the label mask
#pragma unroll
            for (int k = 1; k < kSigWords; k++) {
              uint32_t need = q->sig[k];
              while (need) {
                const uint32_t bit = __ffs(need) - 1;
                need &= need - 1;
                word &= col[k - 1][bit];
              }
            }
          }
        }
        const uint32_t dm = __shfl_sync(kFull, atleast, qdeg);
        if (i < e) {
          if (use_deg) word &= dm;
          if (q->words) pool[q->bmoff + (w - (q->bmbase >> 5))] = word;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// One Jacobi step of neighbour-support refinement.  The query neighbours of u
// are grouped by refinement class; v stays in C(u) only if, for every group
// of k neighbours in class y, at least k entries of v's label-l(y) neighbour
// segment are in C(y) as read from src (k distinct query neighbours need k
// distinct data neighbours; the count of entries with repeated edges is an
// upper bound, so the test never drops a true image).  This is the pull-mode
// check of MMatch (count_neighbors_kernel + check_re_kernel,
// MMatch_kernels.cuh:28-117, 190-214) with its per-class thresholds.  With
// every vertex its own class every k is one.  A class dominated by u's (dom)
// is tested first: C(u) stays within C(dom) through the refinement, so a v
// outside C(dom) fails one of the counts anyway.  Warps take runs of bitmap
// words (lane = candidate); class members other than the smallest own no
// words.  A candidate's segment of at most coop_min entries is scanned by its
// own lane; a longer one by the whole warp, 32 consecutive entries per step
// (coalesced loads, one ballot per step), one such candidate after another.
// ---------------------------------------------------------------------------
constexpr uint32_t kRefineRun = 8;

__global__ void __launch_bounds__(256) refine_kernel(GraphView g, const QVert* __restrict__ qv, uint32_t G,
                                                     const uint64_t* __restrict__ gword, uint64_t total_words,
                                                     const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                                     uint32_t coop_min) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nwt = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t run = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; run * kRefineRun < total_words;
       run += nwt) {
    uint64_t W = run * kRefineRun;
    const uint64_t Wend = min(W + kRefineRun, total_words);
    // query vertex owning word W: last g with gword[g] <= W
    uint32_t lo = 0, hi = G;
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (gword[mid] <= W) lo = mid; else hi = mid;
    }
    uint32_t gi = lo;
    for (; W < Wend; W++) {
      while (gword[gi + 1] <= W) gi++;
      const QVert* q = qv + gi;
      const uint32_t word = src[W];
      if (word == 0 || q->adj == 0) {
        if (lane == 0) dst[W] = word;
        continue;
      }
      const uint32_t bit0 = uint32_t((W - q->bmoff) << 5) + lane;  // bit of v in every bitmap of u's label
      const uint32_t v = q->bmbase + bit0;
      bool alive = (word >> lane) & 1u;
      const uint32_t gbase = gi - q->u;
      if (q->dom != kNoClass) {
        const QVert* qd = qv + gbase + q->dom;
        alive = alive && ((src[qd->bmoff + (bit0 >> 5)] >> (bit0 & 31)) & 1u);
      }
      uint32_t m = q->adj;
      while (m && __any_sync(kFull, alive)) {
        const uint32_t wv = __ffs(m) - 1;
        const QVert* qw = qv + gbase + wv;
        const uint32_t grp = m & qw->cmask;
        m &= ~grp;
        const uint32_t need = __popc(grp);
        if (qw->words == 0) {  // no data vertex carries the neighbour's label
          alive = false;
          continue;
        }
        const uint32_t* __restrict__ nb = src + qw->bmoff;
        const uint32_t nbase = qw->bmbase;
        uint32_t k = 0, e = 0;
        if (alive) segment_of(g, v, qw->label, k, e);
        const bool coop = alive && e - k > coop_min;
        if (alive && !coop) {
          uint32_t have = 0;
          for (; k < e && have < need; k++) {
            const uint32_t bit = g.adj[k] - nbase;
            have += (nb[bit >> 5] >> (bit & 31)) & 1u;
          }
          alive = have >= need;
        }
        uint32_t cm = __ballot_sync(kFull, coop);
        while (cm) {
          const uint32_t c = __ffs(cm) - 1;
          cm &= cm - 1;
          const uint32_t ck = __shfl_sync(kFull, k, c), ce = __shfl_sync(kFull, e, c);
          uint32_t have = 0;
          for (uint32_t p = ck; p < ce && have < need; p += 32) {
            const uint32_t idx = p + lane;
            bool hit = false;
            if (idx < ce) {
              const uint32_t bit = g.adj[idx] - nbase;
              hit = (nb[bit >> 5] >> (bit & 31)) & 1u;
            }
            have += __popc(__ballot_sync(kFull, hit));
          }
          if (lane == c) alive = have >= need;
        }
      }
      const uint32_t nw = __ballot_sync(kFull, alive);
      if (lane == 0) dst[W] = nw;
    }
  }
}

// Candidates per query vertex (popcount of its bitmap).
__global__ void __launch_bounds__(256) popcount_kernel(const QVert* __restrict__ qv, uint32_t G,
                                                       const uint32_t* __restrict__ pool, uint32_t* counts) {
  __shared__ uint32_t red[8];
  for (uint32_t gi = blockIdx.x; gi < G; gi += gridDim.x) {
    const QVert* q = qv + gi;
    uint32_t c = 0;
    for (uint32_t i = threadIdx.x; i < q->words; i += blockDim.x) c += __popc(pool[q->bmoff + i]);
    c = warp_sum(c);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int i = 0; i < int(blockDim.x >> 5); i++) t += red[i];
      counts[gi] = t;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Ordering: one warp per query, lane u = query vertex u.  Greedy frontier
// argmin of a score with ties to the lowest vertex id.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t warp_argmin(float s, uint32_t id) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float s2 = __shfl_xor_sync(kFull, s, o);
    uint32_t i2 = __shfl_xor_sync(kFull, id, o);
    if (s2 < s || (s2 == s && i2 < id)) { s = s2; id = i2; }
  }
  return id;
}

// With scores (kOrderScores), the first `lprefix` positions are chosen by the
// scores and the rest by the GSI rule from that prefix on (candidate count,
// times 0.9 per placed neighbour, the prefix's vertices included).
__global__ void order_kernel(const QVert* __restrict__ qv, const uint32_t* __restrict__ qoff, uint32_t Q,
                             const uint32_t* __restrict__ counts, uint32_t mode, const float* __restrict__ scores,
                             const uint32_t* __restrict__ given, Plan* plans, uint32_t* root_count,
                             uint32_t* orders_out, uint32_t lprefix = kMaxQ) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < Q; q += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t g0 = qoff[q], n = qoff[q + 1] - g0;
    const bool live = lane < n;
    const uint32_t all = n == 32 ? kFull : ((1u << n) - 1);
    const QVert* me = qv + g0 + (live ? lane : 0);
    const uint32_t cnt = live ? counts[g0 + lane] : 0;
    const uint32_t adj = live ? me->adj : 0;
    const int32_t lab = live ? me->label : -1;
    const uint32_t deg = live ? me->deg : 0;
    const bool ok = n > 0 && __ballot_sync(kFull, live && cnt == 0) == 0;

    float score = float(cnt);
    float gscore = float(cnt);   // GSI-rule score that continues a scored prefix
    uint32_t root_only = kFull;  // position 0 restricted to this vertex when != kFull
    if (mode == kOrderMMatch) {
      // 2-core by peeling vertices of degree <= 1 (match/MMatch.cu:543-607)
      uint32_t alive = all;
      for (int it = 0; it < 32; it++) {
        const bool in = live && ((alive >> lane) & 1u) && __popc(adj & alive) <= 1;
        const uint32_t peel = __ballot_sync(kFull, in);
        if (!peel) break;
        alive &= ~peel;
      }
      const uint32_t type = ((alive >> lane) & 1u) ? 2u : (deg == 1 ? 0u : 1u);
      float maxc = 0.f, maxf = 0.f;
      float myc = (live && type == 2) ? float(cnt) : 0.f, myf = (live && type == 1) ? float(cnt) : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        myc = fmaxf(myc, __shfl_xor_sync(kFull, myc, o));
        myf = fmaxf(myf, __shfl_xor_sync(kFull, myf, o));
      }
      maxc = myc;
      maxf = myf;
      if (type == 0) score = (float(cnt) + maxf) + maxc;
      else if (type == 1) score = float(cnt) + maxc;
      if (alive == 0) {
        // no core: root = forest vertex of least BFS weight (MMatch.cu:270-315)
        uint32_t visited = 1u << lane, frontier = visited, weight = 0;
        for (uint32_t level = 0; level < n; level++) {
          uint32_t next = 0;
          for (uint32_t j = 0; j < n; j++) {
            uint32_t mj = __shfl_sync(kFull, adj, j);
            if ((frontier >> j) & 1u) next |= mj;
          }
          next &= ~visited & all;
          weight += __popc(next) * (level + 1);
          visited |= next;
          frontier = next;
        }
        const bool cand = live && type == 1;
        const uint32_t any = __ballot_sync(kFull, cand);
        if (any) root_only = warp_argmin(cand ? float(weight) : INFINITY, cand ? lane : 0xffffu);
      }
    } else if (mode == kOrderScores) {
      score = live ? scores[g0 + lane] : 0.f;
    }

    uint32_t myord = 0, placed = 0;
    if (mode == kOrderGiven) {
      myord = live ? given[g0 + lane] : 0;
    } else {
      for (uint32_t i = 0; i < n; i++) {
        bool elig = live && !((placed >> lane) & 1u);
        if (i == 0) elig = elig && (root_only == kFull || lane == root_only);
        else elig = elig && (adj & placed) != 0;
        const float sc = (mode == kOrderScores && i >= lprefix) ? gscore : score;
        const uint32_t u = warp_argmin(elig ? sc : INFINITY, elig ? lane : 0xffffu);
        if (u >= n) break;  // cannot happen for connected queries
        placed |= 1u << u;
        if (lane == i) myord = u;
        if (mode == kOrderGSI && live && ((adj >> u) & 1u)) score = float(double(score) * 0.9);
        if (mode == kOrderScores && live && ((adj >> u) & 1u)) gscore = float(double(gscore) * 0.9);
      }
    }
    // Plan for position i = lane.
    const uint32_t u = myord;
    const uint32_t adj_u = __shfl_sync(kFull, adj, u);
    const int32_t lab_u = __shfl_sync(kFull, lab, u);
    uint32_t bwd = 0, same = 0;
    for (uint32_t j = 0; j < n; j++) {
      const uint32_t uj = __shfl_sync(kFull, myord, j);
      const int32_t lj = __shfl_sync(kFull, lab, uj);
      if (j < lane) {
        if ((adj_u >> uj) & 1u) bwd |= 1u << j;
        if (lj == lab_u) same |= 1u << j;
      }
    }
    Plan* p = plans + q;
    if (live) {
      const QVert* qu = qv + g0 + u;
      p->qv[lane] = u;
      p->lab[lane] = lab_u;
      p->bwd[lane] = bwd;
      p->same[lane] = same;
      p->bmbase[lane] = qu->bmbase;
      p->bmoff[lane] = qu->bmoff;
      orders_out[uint64_t(q) * kMaxQ + lane] = u;
    }
    if (lane == 0) {
      p->n = n;
      p->ok = ok ? 1u : 0u;
      p->g0 = g0;
      root_count[q] = ok ? counts[g0 + u] : 0u;
    }
  }
}

// Roots of each query in ascending vertex order (block scan of word popcounts).
__global__ void __launch_bounds__(256) roots_kernel(const QVert* __restrict__ qv, const Plan* __restrict__ plans,
                                                    uint32_t Q, const uint32_t* __restrict__ root_off,
                                                    const uint32_t* __restrict__ pool, uint32_t* roots,
                                                    uint32_t* root_q) {
  __shared__ uint32_t sw[33];
  for (uint32_t q = blockIdx.x; q < Q; q += gridDim.x) {
    const Plan* p = plans + q;
    if (!p->ok) continue;
    const QVert* r = qv + p->g0 + p->qv[0];
    uint32_t outp = root_off[q];
    for (uint32_t b = 0; b < r->words; b += blockDim.x) {
      const uint32_t i = b + threadIdx.x;
      const uint32_t word = i < r->words ? pool[r->bmoff + i] : 0u;
      uint32_t total;
      uint32_t ex = block_exclusive_scan<uint32_t>(__popc(word), sw, total);
      uint32_t wbits = word;
      uint32_t k = outp + ex;
      while (wbits) {
        const uint32_t bit = __ffs(wbits) - 1;
        wbits &= wbits - 1;
        root_q[k] = q;
        roots[k++] = r->bmbase + (i << 5) + bit;
      }
      outp += total;
    }
  }
}

// Number of pass-0 tasks per root: its depth-1 driver range in chunks of
// `split` entries (at least one task per root, so every root is counted).
__global__ void root_chunks_kernel(GraphView g, const Plan* __restrict__ plans, const uint32_t* __restrict__ roots,
                                   const uint32_t* __restrict__ root_q, const uint32_t* __restrict__ total_roots,
                                   uint32_t split, uint32_t* chunks) {
  const uint32_t nr = *total_roots;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nr; i += gridDim.x * blockDim.x) {
    const Plan* p = plans + root_q[i];
    uint32_t c = 1;
    if (p->n > 1) {
      uint32_t lo, hi;
      segment_of(g, roots[i], p->lab[1], lo, hi);
      c = max(1u, (hi - lo + split - 1) / split);
    }
    chunks[i] = c;
  }
}

}  // namespace
}  // namespace fsig

#include "enumerate.cuh"

namespace fsig {
namespace {

inline unsigned grid_cap(uint64_t n, int threads, int sms, int per_sm) {
  uint64_t b = (n + threads - 1) / threads;
  uint64_t cap = uint64_t(sms) * per_sm;
  if (b > cap) b = cap;
  return unsigned(b ? b : 1);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int prepare_query(const fsig_query& q, int32_t num_labels, HostQuery& h) {
  (void)num_labels;
  h = HostQuery();
  if (q.num_vertices == 0 || q.num_vertices > uint32_t(kMaxQ)) return fail(FSIG_EQUERY, "query size must be 1..32");
  if (!q.labels || (q.num_edges && !q.edges)) return fail(FSIG_EINVAL, "query arrays missing");
  const uint32_t n = q.num_vertices;
  h.n = n;
  h.nbr.assign(n, std::vector<uint32_t>());
  for (uint32_t u = 0; u < n; u++) {
    h.label[u] = q.labels[u];
    h.adj[u] = 0;
  }
  for (uint32_t e = 0; e < q.num_edges; e++) {
    const uint32_t a = q.edges[2 * e], b = q.edges[2 * e + 1];
    if (a >= n || b >= n) return fail(FSIG_EQUERY, "query edge endpoint out of range");
    h.nbr[a].push_back(b);
    h.nbr[b].push_back(a);
    if (a == b) continue;
    h.adj[a] |= 1u << b;
    h.adj[b] |= 1u << a;
  }
  for (uint32_t u = 0; u < n; u++) h.deg[u] = uint32_t(__builtin_popcount(h.adj[u]));
  // connectivity
  uint32_t seen = 1u, frontier = 1u;
  while (frontier) {
    uint32_t next = 0;
    for (uint32_t u = 0; u < n; u++)
      if ((frontier >> u) & 1u) next |= h.adj[u];
    frontier = next & ~seen;
    seen |= next;
  }
  const uint32_t all = n == 32 ? 0xffffffffu : ((1u << n) - 1);
  if ((seen & all) != all) return fail(FSIG_EQUERY, "query graph is disconnected");
  // signature of every query vertex (graph_format_transformer.cc:217-262)
  for (uint32_t u = 0; u < n; u++) {
    std::memset(h.sig[u], 0, sizeof(h.sig[u]));
    h.sig[u][0] = uint32_t(h.label[u]);
    for (uint32_t w = 0; w < n; w++) {
      if (!((h.adj[u] >> w) & 1u)) continue;
      uint32_t word, sh;
      sig_slot(h.label[w], word, sh);
      const uint32_t cur = (h.sig[u][word] >> sh) & 3u;
      h.sig[u][word] |= (cur == 0 ? 1u : 3u) << sh;
    }
  }
  if (q.order) {
    uint32_t seenv = 0;
    for (uint32_t i = 0; i < n; i++) {
      if (q.order[i] >= n || ((seenv >> q.order[i]) & 1u)) return fail(FSIG_EQUERY, "order is not a permutation");
      seenv |= 1u << q.order[i];
      h.given[i] = q.order[i];
    }
    // every position after the first needs a placed neighbour
    uint32_t placed = 1u << h.given[0];
    for (uint32_t i = 1; i < n; i++) {
      if (!(h.adj[h.given[i]] & placed)) return fail(FSIG_EQUERY, "order is not connected");
      placed |= 1u << h.given[i];
    }
    h.has_given = true;
  }
  return FSIG_OK;
}

namespace {
struct BatchLayout {
  uint32_t Q = 0, G = 0;
  uint64_t words = 0;
  uint64_t root_cap = 0;
  std::vector<QVert> qv;
  std::vector<uint32_t> qoff, lab_gidx, lab_begin;
  std::vector<uint64_t> gword;
};

// Bitmap layout of a batch: one bitmap per query vertex over its label's id
// range, except that members of a refinement class (classes on) use the
// bitmap of the class's smallest member and own no words.  Callers turn
// classes on only when the refinement runs: without it, sharing saves a few
// bitmap words of filter output, less than the classes cost on the host.
void layout_batch(const DeviceGraph& g, const std::vector<HostQuery>& qs, BatchLayout& b, bool classes) {
  b.Q = uint32_t(qs.size());
  b.qoff.assign(size_t(b.Q) + 1, 0);
  for (uint32_t q = 0; q < b.Q; q++) b.qoff[q + 1] = b.qoff[q] + qs[q].n;
  b.G = b.qoff[b.Q];
  b.qv.assign(b.G, QVert());
  b.gword.assign(size_t(b.G) + 1, 0);
  std::vector<std::vector<uint32_t>> by_label(size_t(g.L));
  uint64_t w = 0, rc = 0;
  for (uint32_t q = 0; q < b.Q; q++) {
    const HostQuery& h = qs[q];
    uint64_t qmax = 0;
    uint8_t cls[kMaxQ], dom[kMaxQ];
    if (classes) {
      refine_classes(h, cls, dom);
    } else {
      for (uint32_t u = 0; u < h.n; u++) { cls[u] = uint8_t(u); dom[u] = uint8_t(kNoClass); }
    }
    for (uint32_t u = 0; u < h.n; u++) {
      const uint32_t gi = b.qoff[q] + u;
      QVert& x = b.qv[gi];
      std::memset(&x, 0, sizeof(x));
      x.label = h.label[u];
      x.deg = h.deg[u];
      x.adj = h.adj[u];
      x.q = q;
      x.u = u;
      x.cls = cls[u];
      x.dom = dom[u];
      for (uint32_t v = 0; v < h.n; v++)
        if (cls[v] == cls[u]) x.cmask |= 1u << v;
      std::memcpy(x.sig, h.sig[u], sizeof(x.sig));
      const int32_t l = h.label[u];
      uint32_t lo = 0, hi = 0;
      if (l >= 0 && l < g.L) { lo = g.h_base[l]; hi = g.h_base[l + 1]; }
      b.gword[gi] = w;
      if (hi > lo) {
        x.bmbase = lo & ~31u;
        x.words = ((hi + 31) >> 5) - (lo >> 5);
        qmax = std::max<uint64_t>(qmax, hi - lo);
        if (cls[u] != u) {  // same label, so the same extent as the class's bitmap
          x.alias = 1;
          x.bmoff = b.qv[b.qoff[q] + cls[u]].bmoff;
          continue;
        }
        by_label[size_t(l)].push_back(gi);
      } else {
        x.bmbase = 0;
        x.words = 0;
      }
      x.bmoff = w;
      w += x.words;
    }
    rc += qmax;
  }
  b.gword[b.G] = w;
  b.words = w;
  b.root_cap = rc;
  b.lab_begin.assign(size_t(g.L) + 1, 0);
  b.lab_gidx.clear();
  for (int32_t l = 0; l < g.L; l++) {
    b.lab_begin[size_t(l)] = uint32_t(b.lab_gidx.size());
    b.lab_gidx.insert(b.lab_gidx.end(), by_label[size_t(l)].begin(), by_label[size_t(l)].end());
  }
  b.lab_begin[size_t(g.L)] = uint32_t(b.lab_gidx.size());
}

template <class T>
T* upload(Engine& e, const std::vector<T>& v, int& rc) {
  T* d = e.arena.take<T>(std::max<size_t>(v.size(), 1));
  if (!d) { rc = fail(FSIG_EADMISSION, "batch does not fit the device arena"); return nullptr; }
  if (!v.empty()) {
    cudaError_t err = cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, e.stream);
    if (err != cudaSuccess) { rc = fail_cuda(err, "cudaMemcpyAsync", __FILE__, __LINE__); return nullptr; }
    e.cur_h2d += sizeof(T) * v.size();
  }
  return d;
}

// Filter + refine + popcount on the device.  Returns the final pool.
int filter_stage(Engine& e, const BatchLayout& b, uint32_t mode, int refine_iters, QVert* d_qv, uint64_t* d_gword,
                 uint32_t* d_lab_gidx, uint32_t* d_lab_begin, uint32_t*& pool, uint32_t* d_counts,
                 uint32_t* launches = nullptr, uint32_t coop_min = kRefineCoopDefault) {
  uint32_t nl = 1;
  const DeviceGraph& g = e.g;
  cudaStream_t s = e.stream;
  uint32_t* p0 = e.arena.take<uint32_t>(std::max<uint64_t>(b.words, 1));
  uint32_t* p1 = refine_iters > 0 ? e.arena.take<uint32_t>(std::max<uint64_t>(b.words, 1)) : nullptr;
  if (!p0 || (refine_iters > 0 && !p1)) return fail(FSIG_EADMISSION, "candidate bitmaps do not fit the arena");
  const GraphView gv = view_of(g);
  filter_kernel<<<grid_cap(uint64_t(g.V), kFilterWarps * 32, e.num_sms, 8), kFilterWarps * 32, 0, s>>>(
      gv, d_qv, d_lab_gidx, d_lab_begin, mode, p0);
  FSIG_CUDA_TRY(cudaGetLastError());
  uint32_t* cur = p0;
  uint32_t* nxt = p1;
  for (int it = 0; it < refine_iters && b.words; it++) {
    const uint64_t runs = (b.words + kRefineRun - 1) / kRefineRun;
    refine_kernel<<<grid_cap(runs * 32, 256, e.num_sms, 16), 256, 0, s>>>(gv, d_qv, b.G, d_gword, b.words, cur, nxt,
                                                                           coop_min);
    FSIG_CUDA_TRY(cudaGetLastError());
    std::swap(cur, nxt);
    nl++;
  }
  if (b.G) {
    popcount_kernel<<<std::min<uint32_t>(b.G, e.num_sms * 8), 256, 0, s>>>(d_qv, b.G, cur, d_counts);
    FSIG_CUDA_TRY(cudaGetLastError());
    nl++;
  }
  if (launches) *launches += nl;
  pool = cur;
  return FSIG_OK;
}
}  // namespace

namespace {
constexpr uint32_t kOverflowCap = 1u << 20;  // task records per overflow queue

// Records ev on s.  Inside a stream capture an ordinary record only orders
// the capture; the external form makes it a node of the graph.
cudaError_t record(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const cudaError_t err = cudaStreamIsCapturing(s, &cs);
  if (err != cudaSuccess) return err;
  return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                             : cudaEventRecord(ev, s);
}

// Milliseconds between two recorded events, or -1 when the runtime cannot
// time them (the error is cleared so that no later call reports it).
float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return -1.f;
  }
  return ms;
}

// Keeps the network's order near the heuristic one: the score of the vertex
// at heuristic position i is clamped to positions [i - window, i + window]
// (scores are positions / (n - 1)); thread per query.
__global__ void order_window_kernel(const uint32_t* __restrict__ qoff, uint32_t Q,
                                    const uint32_t* __restrict__ horders, uint32_t window, float* scores) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < Q; q += gridDim.x * blockDim.x) {
    const uint32_t g0 = qoff[q], n = qoff[q + 1] - g0;
    if (n < 2) continue;
    const float scale = float(n - 1);
    for (uint32_t i = 0; i < n; i++) {
      const uint32_t u = horders[uint64_t(q) * kMaxQ + i];
      const float lo = float(i > window ? i - window : 0u), hi = float(i + window);
      scores[g0 + u] = fminf(fmaxf(scores[g0 + u] * scale, lo), hi) / scale;
    }
  }
}

// In a learned-order batch, queries that carry their own order keep it: their
// scores become the positions of that order (thread per query).
__global__ void given_scores_kernel(const uint32_t* __restrict__ qoff, uint32_t Q,
                                    const uint32_t* __restrict__ has_given, const uint32_t* __restrict__ given,
                                    float* scores) {
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < Q; q += gridDim.x * blockDim.x) {
    if (!has_given[q]) continue;
    const uint32_t g0 = qoff[q], n = qoff[q + 1] - g0;
    for (uint32_t i = 0; i < n; i++) scores[g0 + given[g0 + i]] = float(i);
  }
}

__global__ void ctr_init_kernel(uint32_t* ctr, uint32_t first_task, uint32_t active) {
  for (uint32_t i = threadIdx.x; i < 8 * kCtrStride; i += blockDim.x)
    ctr[i] = i == 0 ? first_task : (i == 5 * kCtrStride ? active : 0u);
}

// The enumeration passes of one batch: pass 0 over the implicit root tasks,
// then passes over the records each pass leaves in its overflow queue, until
// none are left.  Launching a pass is stream-ordered work only (capturable);
// deciding whether another pass is needed reads the counters the pass copied
// to pinned host memory, after the stream has reached them.
struct EnumRun {
  EnumArgs A;
  TaskRec *out = nullptr, *other = nullptr;
  uint32_t *ready = nullptr, *other_ready = nullptr, *ctr = nullptr;
  unsigned long long* d_ev = nullptr;
  uint32_t* h_ctr = nullptr;  // pinned, 4 counters kCtrStride apart
  uint32_t grid = 0, block = 0, active = 0, first_task = 0, pass = 0;
  size_t smem = 0;
  bool timed = true;  // every pass's kernel time was measured
};

// One-time kernel attributes and occupancy (host calls, kept out of captures).
template <bool kRows>
int enum_configure_one(int* per_sm) {
  FSIG_CUDA_TRY(cudaFuncSetAttribute(enumerate_kernel<kRows>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(sizeof(WarpSmem) * kEnumWarps)));
  for (uint32_t w = 1; w <= kEnumWarps; w++) {
    int per = 0;
    FSIG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, enumerate_kernel<kRows>, int(w * 32),
                                                                sizeof(WarpSmem) * w));
    per_sm[w] = std::max(per, 1);
  }
  return FSIG_OK;
}

int enum_configure(Engine& e) {
  if (e.enum_per_sm[kEnumWarps]) return FSIG_OK;
  int rc = enum_configure_one<false>(e.enum_per_sm);
  if (!rc) rc = enum_configure_one<true>(e.enum_per_sm_rows);
  if (rc) e.enum_per_sm[kEnumWarps] = 0;
  return rc;
}

int enum_prepare(Engine& e, const BatchOptions& opt, const GraphView& gv, const Plan* d_plans, const uint32_t* pool,
                 uint32_t Q, const uint32_t* d_roots, const uint32_t* d_root_q, const uint32_t* d_chunk_off,
                 const uint32_t* d_nroots, uint32_t split, QueryResult* d_res, unsigned long long* d_misc,
                 uint32_t* d_emit, unsigned long long* d_emit_ctr, uint32_t* h_ctr, EnumRun& R) {
  cudaStream_t s = e.stream;
  TaskRec* qa = e.arena.take<TaskRec>(kOverflowCap);
  TaskRec* qb = e.arena.take<TaskRec>(kOverflowCap);
  uint32_t* ra = e.arena.take<uint32_t>(kOverflowCap);
  uint32_t* rb = e.arena.take<uint32_t>(kOverflowCap);
  R.ctr = e.arena.take<uint32_t>(8 * kCtrStride);
  R.d_ev = e.arena.take<unsigned long long>(8);
  if (!qa || !qb || !ra || !rb || !R.ctr || !R.d_ev)
    return fail(FSIG_EADMISSION, "work queues do not fit the device arena");
  FSIG_CUDA_TRY(cudaMemsetAsync(ra, 0, sizeof(uint32_t) * kOverflowCap, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(rb, 0, sizeof(uint32_t) * kOverflowCap, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(R.d_ev, 0, 64, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(d_misc + 1, 0, sizeof(unsigned long long), s));
  const uint32_t wpb = std::max<uint32_t>(1, std::min<uint32_t>(opt.warps_per_block, kEnumWarps));
  const int per_sm = gv.lseg ? e.enum_per_sm[wpb] : e.enum_per_sm_rows[wpb];
  R.smem = sizeof(WarpSmem) * wpb;
  R.grid = uint32_t(e.num_sms * per_sm);
  R.block = wpb * 32;
  R.active = R.grid * wpb;  // every warp starts active; idle warps are counted as they wait
  R.first_task = opt.task_begin;
  R.h_ctr = h_ctr;
  R.pass = 0;
  EnumArgs& A = R.A;
  A.g = gv;
  A.plans = d_plans;
  A.pool = pool;
  A.Q = Q;
  A.roots = d_roots;
  A.root_q = d_root_q;
  A.chunk_off = d_chunk_off;
  A.nroots_ptr = d_nroots;
  A.split = split;
  A.t_end = opt.task_end;
  A.emit = d_emit;
  A.emit_cap = d_emit ? opt.emit_cap : 0;
  A.emit_ctr = d_emit_ctr;
  A.in_tasks = nullptr;
  A.in_count = 0;
  A.out_cap = kOverflowCap;
  A.ctr = R.ctr;
  A.chunk = std::max<uint32_t>(opt.chunk, 1);
  A.budget = (long long)opt.budget_cycles;
  A.res = d_res;
  A.work_cap = opt.max_work;
  A.algo_bytes = d_misc + 1;
  A.ev = R.d_ev;
  A.seed = FSIG_HASH_SEED;
  A.ready_wait_ns = e.ready_wait_ns;
  A.idle_wait_ns = e.idle_wait_ns;
  A.unpublished = e.inject_unpublished;
  A.isect = opt.isect;
  R.out = qa;
  R.ready = ra;
  R.other = qb;
  R.other_ready = rb;
  return FSIG_OK;
}

int enum_launch(Engine& e, EnumRun& R) {
  cudaStream_t s = e.stream;
  R.A.out_tasks = R.out;
  R.A.out_ready = R.ready;
  R.A.tag = R.pass + 1;
  ctr_init_kernel<<<1, 256, 0, s>>>(R.ctr, R.pass == 0 ? R.first_task : 0u, R.active);
  FSIG_CUDA_TRY(cudaGetLastError());
  FSIG_CUDA_TRY(record(e.ev_enum[0], s));
  if (R.A.g.lseg) enumerate_kernel<false><<<R.grid, R.block, R.smem, s>>>(R.A);
  else enumerate_kernel<true><<<R.grid, R.block, R.smem, s>>>(R.A);
  FSIG_CUDA_TRY(cudaGetLastError());
  FSIG_CUDA_TRY(record(e.ev_enum[1], s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(R.h_ctr, R.ctr, sizeof(uint32_t) * 4 * kCtrStride, cudaMemcpyDeviceToHost, s));
  return FSIG_OK;
}

// Call once the stream has passed the pass's counter copy.  Sets more when
// records are left for another pass, and readies that pass.
int enum_after(Engine& e, EnumRun& R, bool& more, float& ms_enum, uint64_t& d2h) {
  const float ms = elapsed(e.ev_enum[0], e.ev_enum[1]);
  if (ms < 0.f) R.timed = false;
  else ms_enum += ms;
  d2h += sizeof(uint32_t) * 4 * kCtrStride;
  const uint32_t* hc = R.h_ctr;
  if (hc[3 * kCtrStride] & kErrTimeout) return fail(FSIG_ETIMEOUT, "a work-queue record was not published in time");
  const uint32_t head = hc[2 * kCtrStride], tail = std::min(hc[1 * kCtrStride], kOverflowCap);
  more = head < tail;
  if (!more) return FSIG_OK;
  // unconsumed records become the next pass's input
  R.A.in_tasks = R.out + head;
  R.A.in_count = tail - head;
  std::swap(R.out, R.other);
  std::swap(R.ready, R.other_ready);
  if (++R.pass > 4096) return fail(FSIG_EOVERFLOW, "enumeration did not converge");
  return FSIG_OK;
}

// Page-locked host staging of one batch (inputs, then outputs), grown on
// demand; graph-captured copies read and write it at replay.
struct Stage {
  uint8_t* base = nullptr;
  size_t used = 0;
  template <class T>
  T* take(size_t n) {
    used = (used + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + used);
    used += sizeof(T) * n;
    return p;
  }
};

int reserve_pinned(Engine& e, size_t bytes) {
  if (e.pinned_bytes >= bytes) return FSIG_OK;
  if (e.pinned) cudaFreeHost(e.pinned);
  e.pinned = nullptr;
  e.pinned_bytes = 0;
  const size_t want = std::max<size_t>(bytes + bytes / 4, size_t(1) << 20);
  FSIG_CUDA_TRY(cudaHostAlloc(&e.pinned, want, cudaHostAllocDefault));
  e.pinned_bytes = want;
  return FSIG_OK;
}

template <class T>
T* stage_upload(Engine& e, Stage& st, const std::vector<T>& v, int& rc) {
  T* d = e.arena.take<T>(std::max<size_t>(v.size(), 1));
  if (!d) { rc = fail(FSIG_EADMISSION, "batch does not fit the device arena"); return nullptr; }
  T* h = st.take<T>(v.size());
  if (!v.empty()) {
    std::memcpy(h, v.data(), sizeof(T) * v.size());
    cudaError_t err = cudaMemcpyAsync(d, h, sizeof(T) * v.size(), cudaMemcpyHostToDevice, e.stream);
    if (err != cudaSuccess) { rc = fail_cuda(err, "cudaMemcpyAsync", __FILE__, __LINE__); return nullptr; }
    e.cur_h2d += sizeof(T) * v.size();
  }
  return d;
}

size_t stage_bytes(const BatchLayout& b) {
  const size_t a = 256;
  const size_t Q = b.Q, G = b.G;
  return 20 * a + sizeof(QVert) * G + 4 * (Q + 1) + 4 * b.lab_gidx.size() + 4 * b.lab_begin.size() +
         8 * b.gword.size() + 4 * G + 4 * G + 4 * Q + sizeof(QueryResult) * Q + 4 * G + 4 * Q * kMaxQ + sizeof(Plan) * Q +
         8 + 4 * 4 * kCtrStride + 64;
}
}  // namespace

int run_batch(Engine& e, const std::vector<HostQuery>& qs, const BatchOptions& opt, BatchOutput& out) {
  if (!e.has_graph) return fail(FSIG_ENOGRAPH, "no data graph loaded");
  const DeviceGraph& g = e.g;
  cudaStream_t s = e.stream;
  BatchLayout b;
  layout_batch(g, qs, b, opt.classes && opt.refine_iters > 0);
  const uint32_t Q = b.Q;
  out.res.assign(Q, QueryResult());
  out.counts.assign(b.G, 0);
  out.orders.assign(size_t(Q) * kMaxQ, 0);
  out.ok.assign(Q, 0);
  if (Q == 0) return FSIG_OK;
  if (b.root_cap + 1 > 0xffffffffull) return fail(FSIG_EADMISSION, "batch has more than 2^32 root candidates");
  if ((opt.emit_cap || opt.want_tasks) && Q != 1)
    return fail(FSIG_EINVAL, "embedding output and task ranges are for one query at a time");
  // One CUDA graph per batch when every step is stream-ordered: orders chosen
  // on the device and no embedding output.
  const bool graph = opt.use_graph && !opt.host_order && !opt.emit_cap && !opt.want_tasks;
  // The host writes this batch into the page-locked staging area that earlier
  // calls' copies read from the stream: wait until the stream has drained
  // (every call also drains it before it returns, errors included).
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  e.arena.release(g.arena_mark);
  e.cur_h2d = 0;
  uint64_t d2h = 0;
  uint32_t launches = 0;
  int rc = enum_configure(e);
  if (rc) return rc;
  if (opt.learned) {
    rc = mpnn_configure(e);
    if (rc) return rc;
  }
  rc = reserve_pinned(e, stage_bytes(b));
  if (rc) return rc;
  Stage st;
  st.base = static_cast<uint8_t*>(e.pinned);

  std::vector<uint32_t> given(b.G, 0);
  std::vector<float> scores(b.G, 0.f);
  std::vector<uint32_t> has_given(Q, 0);
  bool any_given = false;
  for (uint32_t q = 0; q < Q; q++) {
    has_given[q] = qs[q].has_given ? 1u : 0u;
    any_given |= qs[q].has_given;
  }
  for (uint32_t q = 0; q < Q; q++)
    for (uint32_t i = 0; i < qs[q].n; i++) {
      given[b.qoff[q] + i] = qs[q].has_given ? qs[q].given[i] : i;
      if (opt.scores) scores[b.qoff[q] + i] = opt.scores[b.qoff[q] + i];
    }

  cudaGraph_t cg = nullptr;
  if (graph) FSIG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  EnumRun R;
  QueryResult* h_res = nullptr;
  uint32_t *h_counts = nullptr, *h_orders = nullptr, *d_chunk_off = nullptr, *d_rootoff = nullptr;
  Plan* h_plans = nullptr;
  unsigned long long* h_misc = nullptr;
  unsigned long long* h_ev = nullptr;
  QueryResult* d_res = nullptr;
  unsigned long long* d_misc = nullptr;
  Plan* d_plans = nullptr;
  uint32_t *d_counts = nullptr, *d_orders = nullptr, *d_emit = nullptr;
  unsigned long long* d_emit_ctr = nullptr;

  // Everything from the uploads to the results' copy back, in stream order.
  auto enqueue = [&]() -> int {
    int rc = FSIG_OK;
    FSIG_CUDA_TRY(record(e.ev[0], s));
    QVert* d_qv = stage_upload(e, st, b.qv, rc);
    if (rc) return rc;
    uint32_t* d_qoff = stage_upload(e, st, b.qoff, rc);
    if (rc) return rc;
    uint32_t* d_lab_gidx = stage_upload(e, st, b.lab_gidx, rc);
    if (rc) return rc;
    uint32_t* d_lab_begin = stage_upload(e, st, b.lab_begin, rc);
    if (rc) return rc;
    uint64_t* d_gword = stage_upload(e, st, b.gword, rc);
    if (rc) return rc;
    uint32_t* d_given = stage_upload(e, st, given, rc);
    if (rc) return rc;
    float* d_scores = stage_upload(e, st, scores, rc);
    if (rc) return rc;
    d_counts = e.arena.take<uint32_t>(std::max<uint32_t>(b.G, 1));
    d_plans = e.arena.take<Plan>(Q);
    uint32_t* d_rootcnt = e.arena.take<uint32_t>(uint64_t(Q) + 1);
    d_rootoff = e.arena.take<uint32_t>(uint64_t(Q) + 1);
    d_orders = e.arena.take<uint32_t>(uint64_t(Q) * kMaxQ);
    d_res = e.arena.take<QueryResult>(Q);
    d_misc = e.arena.take<unsigned long long>(4);  // [1] modelled bytes
    if (!d_counts || !d_plans || !d_rootcnt || !d_rootoff || !d_orders || !d_res || !d_misc)
      return fail(FSIG_EADMISSION, "batch does not fit the device arena");
    h_res = st.take<QueryResult>(Q);
    h_counts = st.take<uint32_t>(b.G);
    h_orders = st.take<uint32_t>(size_t(Q) * kMaxQ);
    h_plans = st.take<Plan>(Q);
    h_misc = st.take<unsigned long long>(1);
    uint32_t* h_ctr = st.take<uint32_t>(4 * kCtrStride);
    h_ev = st.take<unsigned long long>(8);

    uint32_t* pool = nullptr;
    rc = filter_stage(e, b, opt.filter_mode, opt.refine_iters, d_qv, d_gword, d_lab_gidx, d_lab_begin, pool,
                      d_counts, &launches, opt.refine_coop);
    if (rc) return rc;
    FSIG_CUDA_TRY(record(e.ev[1], s));

    uint32_t order_mode = opt.order_mode;
    if (opt.host_order) {
      // Reference-exact orders are computed on the host from the counts.
      FSIG_CUDA_TRY(cudaMemcpyAsync(out.counts.data(), d_counts, sizeof(uint32_t) * b.G, cudaMemcpyDeviceToHost, s));
      FSIG_CUDA_TRY(cudaStreamSynchronize(s));
      d2h += sizeof(uint32_t) * b.G;
      for (uint32_t q = 0; q < Q; q++) {
        bool any_zero = false;
        for (uint32_t u = 0; u < qs[q].n; u++) any_zero |= out.counts[b.qoff[q] + u] == 0;
        if (qs[q].has_given) continue;
        if (any_zero) {  // nothing to enumerate; any connected order will do
          for (uint32_t i = 0; i < qs[q].n; i++) given[b.qoff[q] + i] = i;
          uint32_t placed = 1u;
          for (uint32_t i = 1; i < qs[q].n; i++)
            for (uint32_t u = 0; u < qs[q].n; u++)
              if (!((placed >> u) & 1u) && (qs[q].adj[u] & placed)) { given[b.qoff[q] + i] = u; placed |= 1u << u; break; }
          continue;
        }
        opt.host_order(qs[q], out.counts.data() + b.qoff[q], given.data() + b.qoff[q]);
      }
      FSIG_CUDA_TRY(cudaMemcpyAsync(d_given, given.data(), sizeof(uint32_t) * b.G, cudaMemcpyHostToDevice, s));
      e.cur_h2d += sizeof(uint32_t) * b.G;
      order_mode = kOrderGiven;
    }
    const float* d_score_src = d_scores;
    if (opt.learned) {
      // Order-network scores from the filtered candidate counts, on the
      // device; the algorithm's own heuristic order is one of the inputs.
      float* d_feat = e.arena.take<float>(uint64_t(std::max<uint32_t>(b.G, 1)) * kFeat);
      uint32_t* d_nbr = e.arena.take<uint32_t>(std::max<uint32_t>(b.G, 1));
      float* d_lscores = e.arena.take<float>(std::max<uint32_t>(b.G, 1));
      if (!d_feat || !d_nbr || !d_lscores) return fail(FSIG_EADMISSION, "order-network inputs do not fit the arena");
      order_kernel<<<(Q + 7) / 8, 256, 0, s>>>(d_qv, d_qoff, Q, d_counts, order_mode, d_scores, d_given, d_plans,
                                               d_rootcnt, d_orders);
      FSIG_CUDA_TRY(cudaGetLastError());
      rc = mpnn_features_device(e, d_qv, b.G, d_qoff, Q, d_counts, d_orders, d_feat, d_nbr);
      if (rc) return rc;
      rc = mpnn_forward_device(e, Q, d_qoff, d_feat, d_nbr, d_lscores);
      if (rc) return rc;
      launches += 3;
      if (opt.learned_window < kMaxQ) {
        order_window_kernel<<<std::max<uint32_t>(1, (Q + 127) / 128), 128, 0, s>>>(d_qoff, Q, d_orders,
                                                                                 opt.learned_window, d_lscores);
        FSIG_CUDA_TRY(cudaGetLastError());
        launches++;
      }
      if (any_given) {
        uint32_t* d_has_given = stage_upload(e, st, has_given, rc);
        if (rc) return rc;
        given_scores_kernel<<<std::max<uint32_t>(1, (Q + 127) / 128), 128, 0, s>>>(d_qoff, Q, d_has_given, d_given,
                                                                                 d_lscores);
        FSIG_CUDA_TRY(cudaGetLastError());
        launches++;
      }
      d_score_src = d_lscores;
      order_mode = kOrderScores;
    }
    uint32_t* d_roots = e.arena.take<uint32_t>(std::max<uint64_t>(b.root_cap, 1));
    uint32_t* d_root_q = e.arena.take<uint32_t>(std::max<uint64_t>(b.root_cap, 1));
    uint32_t* d_chunks = e.arena.take<uint32_t>(b.root_cap + 1);
    d_chunk_off = e.arena.take<uint32_t>(b.root_cap + 1);
    if (!d_roots || !d_root_q || !d_chunks || !d_chunk_off)
      return fail(FSIG_EADMISSION, "root list does not fit the device arena");
    FSIG_CUDA_TRY(cudaMemsetAsync(d_rootcnt, 0, sizeof(uint32_t) * (uint64_t(Q) + 1), s));
    order_kernel<<<(Q + 7) / 8, 256, 0, s>>>(d_qv, d_qoff, Q, d_counts, order_mode, d_score_src, d_given, d_plans,
                                             d_rootcnt, d_orders, opt.learned ? opt.learned_prefix : kMaxQ);
    FSIG_CUDA_TRY(cudaGetLastError());
    rc = device_exclusive_scan<uint32_t>(e.arena, d_rootcnt, d_rootoff, uint64_t(Q) + 1, nullptr, s, &launches);
    if (rc) return rc;
    roots_kernel<<<std::min<uint32_t>(Q, e.num_sms * 8), 256, 0, s>>>(d_qv, d_plans, Q, d_rootoff, pool, d_roots,
                                                                       d_root_q);
    FSIG_CUDA_TRY(cudaGetLastError());
    launches += 2;
    // Pass-0 task space: depth-1 chunks of every root.  Sized by the bound
    // on the number of roots (the count itself stays on the device).
    // (embedding output may cut the depth-1 ranges as finely as one entry)
    const uint32_t split = std::max<uint32_t>(opt.split, opt.emit_cap ? 1u : 32u);
    FSIG_CUDA_TRY(cudaMemsetAsync(d_chunks, 0, sizeof(uint32_t) * (b.root_cap + 1), s));
    if (b.root_cap) {
      root_chunks_kernel<<<grid_cap(b.root_cap, 256, e.num_sms, 8), 256, 0, s>>>(view_of(g), d_plans, d_roots,
                                                                                  d_root_q, d_rootoff + Q, split,
                                                                                  d_chunks);
      FSIG_CUDA_TRY(cudaGetLastError());
      launches++;
    }
    rc = device_exclusive_scan<uint32_t>(e.arena, d_chunks, d_chunk_off, b.root_cap + 1, nullptr, s, &launches);
    if (rc) return rc;
    FSIG_CUDA_TRY(cudaMemsetAsync(d_res, 0, sizeof(QueryResult) * Q, s));
    if (opt.emit_cap) {
      d_emit_ctr = e.arena.take<unsigned long long>(1);
      d_emit = e.arena.take<uint32_t>(opt.emit_cap * qs[0].n);
      if (!d_emit || !d_emit_ctr) return fail(FSIG_EADMISSION, "embedding buffer does not fit the device arena");
      FSIG_CUDA_TRY(cudaMemsetAsync(d_emit_ctr, 0, sizeof(unsigned long long), s));
    }
    rc = enum_prepare(e, opt, view_of(g), d_plans, pool, Q, d_roots, d_root_q, d_chunk_off, d_rootoff + Q, split,
                      d_res, d_misc, d_emit, d_emit_ctr, h_ctr, R);
    if (rc) return rc;
    return enum_launch(e, R);
  };
  // The results' copy back (after the last pass).
  auto copy_back = [&]() -> int {
    FSIG_CUDA_TRY(record(e.ev[2], s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(h_res, d_res, sizeof(QueryResult) * Q, cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(h_counts, d_counts, sizeof(uint32_t) * b.G, cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(h_orders, d_orders, sizeof(uint32_t) * Q * kMaxQ, cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(h_misc, d_misc + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(h_plans, d_plans, sizeof(Plan) * Q, cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(h_ev, R.d_ev, sizeof(e.last_ev), cudaMemcpyDeviceToHost, s));
    return FSIG_OK;
  };

  bool more = false;
  out.passes = 0;
  out.ms_enum = 0;
  if (graph) {
    rc = enqueue();
    if (!rc) rc = copy_back();
    const cudaError_t end = cudaStreamEndCapture(s, &cg);
    if (rc) {
      if (cg) cudaGraphDestroy(cg);
      return rc;
    }
    if (end != cudaSuccess) return fail_cuda(end, "cudaStreamEndCapture", __FILE__, __LINE__);
    if (e.gexec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(e.gexec, cg, &info) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphExecDestroy(e.gexec);
        e.gexec = nullptr;
      }
    }
    if (!e.gexec) {
      const cudaError_t err = cudaGraphInstantiate(&e.gexec, cg, 0);
      if (err != cudaSuccess) {
        cudaGraphDestroy(cg);
        e.gexec = nullptr;
        return fail_cuda(err, "cudaGraphInstantiate", __FILE__, __LINE__);
      }
    }
    cudaGraphDestroy(cg);
    FSIG_CUDA_TRY(cudaEventRecord(e.ev_outer[0], s));
    FSIG_CUDA_TRY(cudaGraphLaunch(e.gexec, s));
    FSIG_CUDA_TRY(cudaEventRecord(e.ev_outer[1], s));
    FSIG_CUDA_TRY(cudaStreamSynchronize(s));
    out.passes = 1;
    rc = enum_after(e, R, more, out.ms_enum, d2h);
    if (rc) return rc;
    if (more) {  // records left over: further passes run as ordinary launches
      while (more) {
        rc = enum_launch(e, R);
        if (rc) return rc;
        FSIG_CUDA_TRY(cudaStreamSynchronize(s));
        out.passes++;
        rc = enum_after(e, R, more, out.ms_enum, d2h);
        if (rc) return rc;
      }
      rc = copy_back();
      if (rc) return rc;
      FSIG_CUDA_TRY(cudaEventRecord(e.ev_outer[1], s));
      FSIG_CUDA_TRY(cudaStreamSynchronize(s));
    }
  } else {
    rc = enqueue();
    if (rc) {
      // work queued before the failure still reads the staging area and the
      // arena: let it finish before they are reused
      cudaStreamSynchronize(s);
      return rc;
    }
    do {
      FSIG_CUDA_TRY(cudaStreamSynchronize(s));
      out.passes++;
      rc = enum_after(e, R, more, out.ms_enum, d2h);
      if (rc) return rc;
      if (more) {
        rc = enum_launch(e, R);
        if (rc) return rc;
      }
    } while (more);
    if (opt.emit_cap || opt.want_tasks) {
      uint32_t nroots = 0;
      FSIG_CUDA_TRY(cudaMemcpyAsync(&nroots, d_rootoff + Q, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      if (opt.emit_cap)
        FSIG_CUDA_TRY(cudaMemcpyAsync(&out.emit_total, d_emit_ctr, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
      FSIG_CUDA_TRY(cudaStreamSynchronize(s));
      FSIG_CUDA_TRY(cudaMemcpyAsync(&out.tasks_total, d_chunk_off + nroots, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      FSIG_CUDA_TRY(cudaStreamSynchronize(s));
      d2h += 8;
    }
    if (opt.emit_cap) {
      const uint64_t rows = std::min<uint64_t>(out.emit_total, opt.emit_cap);
      out.rows.resize(rows * qs[0].n);
      if (rows)
        FSIG_CUDA_TRY(cudaMemcpyAsync(out.rows.data(), d_emit, sizeof(uint32_t) * rows * qs[0].n,
                                      cudaMemcpyDeviceToHost, s));
      d2h += 8 + sizeof(uint32_t) * rows * qs[0].n;
    }
    rc = copy_back();
    if (rc) return rc;
    FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  launches += out.passes * 2;  // counter reset + enumeration per pass
  std::memcpy(out.res.data(), h_res, sizeof(QueryResult) * Q);
  std::memcpy(out.counts.data(), h_counts, sizeof(uint32_t) * b.G);
  std::memcpy(out.orders.data(), h_orders, sizeof(uint32_t) * Q * kMaxQ);
  std::memcpy(e.last_ev, h_ev, sizeof(e.last_ev));
  out.algo_bytes = *h_misc;
  for (uint32_t q = 0; q < Q; q++) out.ok[q] = h_plans[q].ok;
  out.ms_filter = elapsed(e.ev[0], e.ev[1]);
  out.ms_join = elapsed(e.ev[1], e.ev[2]);
  if (out.ms_filter < 0.f || out.ms_join < 0.f) {
    // the phases inside the graph could not be timed: the whole launch counts as join
    out.ms_filter = 0.f;
    out.ms_join = graph ? std::max(elapsed(e.ev_outer[0], e.ev_outer[1]), 0.f) : 0.f;
  }
  if (!R.timed) out.ms_enum = -1.f;
  d2h += sizeof(QueryResult) * Q + sizeof(uint32_t) * b.G + sizeof(uint32_t) * Q * kMaxQ +
         sizeof(unsigned long long) + sizeof(Plan) * Q + sizeof(e.last_ev);
  out.h2d_bytes = e.cur_h2d;
  out.d2h_bytes = d2h;
  out.launches = launches;
  out.graph = graph;
  e.last.h2d_bytes = out.h2d_bytes;
  e.last.d2h_bytes = out.d2h_bytes;
  e.last.enum_bytes = out.algo_bytes;
  e.last.kernel_launches = out.launches;
  e.last.enum_passes = out.passes;
  e.last.ms_filter = out.ms_filter;
  e.last.ms_join = out.ms_join;
  e.last.ms_enum = out.ms_enum;
  e.last.enum_tasks = e.last_ev[0];
  e.last.enum_pops = e.last_ev[1];
  e.last.enum_handoffs = e.last_ev[2];
  e.last.enum_records = e.last_ev[3];
  e.last.enum_examines = e.last_ev[4];
  e.last.graph = graph ? 1u : 0u;
  e.arena.release(g.arena_mark);
  return FSIG_OK;
}

int run_embeddings(Engine& e, const HostQuery& q, BatchOptions opt, uint64_t buffer_rows,
                   int (*sink)(void*, const uint32_t*, uint64_t, uint32_t), void* user, BatchOutput& first) {
  if (!buffer_rows) return fail(FSIG_EINVAL, "embedding buffer of zero rows");
  const std::vector<HostQuery> qs(1, q);
  opt.emit_cap = buffer_rows;
  opt.task_begin = 0;
  opt.task_end = 0xffffffffu;
  int rc = run_batch(e, qs, opt, first);
  if (rc) return rc;
  if (!first.ok[0] || first.res[0].aborted) return FSIG_OK;
  if (first.emit_total <= buffer_rows) {
    if (first.emit_total) sink(user, first.rows.data(), first.emit_total, q.n);
    return FSIG_OK;
  }
  // More embeddings than one buffer holds: cut the task space into ranges,
  // matched one after the other, halving a range whose rows still overflow.
  // Tasks are made as small as they go (one depth-1 entry under one root) so
  // that a range of one task is unlikely to overflow; an empty range gives
  // their number.
  first.rows.clear();
  const uint64_t total = first.res[0].count;
  opt.split = 1;
  opt.task_begin = 0;
  opt.task_end = 0;
  BatchOutput probe;
  rc = run_batch(e, qs, opt, probe);
  if (rc) return rc;
  const uint32_t T = probe.tasks_total;
  const uint64_t parts = std::max<uint64_t>(1, std::min<uint64_t>(T, 2 * ((total + buffer_rows - 1) / buffer_rows)));
  std::vector<std::pair<uint32_t, uint32_t>> todo;
  for (uint64_t i = parts; i-- > 0;) todo.push_back({uint32_t(T * i / parts), uint32_t(T * (i + 1) / parts)});
  uint64_t seen = 0;
  while (!todo.empty()) {
    const auto [t0, t1] = todo.back();
    todo.pop_back();
    if (t0 >= t1) continue;
    BatchOutput o;
    opt.task_begin = t0;
    opt.task_end = t1;
    rc = run_batch(e, qs, opt, o);
    if (rc) return rc;
    if (o.emit_total > buffer_rows) {
      if (t1 - t0 == 1) return fail(FSIG_EADMISSION, "the embeddings under one root chunk exceed the row buffer");
      const uint32_t mid = t0 + (t1 - t0) / 2;
      todo.push_back({mid, t1});
      todo.push_back({t0, mid});
      continue;
    }
    seen += o.emit_total;
    if (o.emit_total && sink(user, o.rows.data(), o.emit_total, q.n)) return FSIG_OK;
  }
  if (seen != total) return fail(FSIG_ECUDA, "task ranges found a different number of embeddings");
  return FSIG_OK;
}

int run_features(Engine& e, const std::vector<HostQuery>& qs, const uint32_t* counts, uint32_t order_mode,
                 float* features) {
  if (!e.has_graph) return fail(FSIG_ENOGRAPH, "no data graph loaded");
  BatchLayout b;
  layout_batch(e.g, qs, b, false);
  const uint64_t mark = e.arena.mark();
  int rc = FSIG_OK;
  QVert* d_qv = upload(e, b.qv, rc);
  if (rc) return rc;
  uint32_t* d_qoff = upload(e, b.qoff, rc);
  if (rc) return rc;
  std::vector<uint32_t> hc(counts, counts + b.G);
  uint32_t* d_counts = upload(e, hc, rc);
  if (rc) return rc;
  float* d_feat = e.arena.take<float>(uint64_t(std::max<uint32_t>(b.G, 1)) * kFeat);
  uint32_t* d_nbr = e.arena.take<uint32_t>(std::max<uint32_t>(b.G, 1));
  Plan* d_plans = e.arena.take<Plan>(std::max<uint32_t>(b.Q, 1));
  uint32_t* d_rootcnt = e.arena.take<uint32_t>(uint64_t(b.Q) + 1);
  uint32_t* d_orders = e.arena.take<uint32_t>(uint64_t(std::max<uint32_t>(b.Q, 1)) * kMaxQ);
  if (!d_feat || !d_nbr || !d_plans || !d_rootcnt || !d_orders) return fail(FSIG_EADMISSION, "arena");
  if (b.Q) {
    order_kernel<<<(b.Q + 7) / 8, 256, 0, e.stream>>>(d_qv, d_qoff, b.Q, d_counts, order_mode, nullptr, nullptr,
                                                      d_plans, d_rootcnt, d_orders);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  rc = mpnn_features_device(e, d_qv, b.G, d_qoff, b.Q, d_counts, d_orders, d_feat, d_nbr);
  if (rc) return rc;
  if (b.G)
    FSIG_CUDA_TRY(cudaMemcpyAsync(features, d_feat, sizeof(float) * kFeat * b.G, cudaMemcpyDeviceToHost, e.stream));
  FSIG_CUDA_TRY(cudaStreamSynchronize(e.stream));
  e.arena.release(mark);
  return FSIG_OK;
}

int run_filter_probe(Engine& e, const HostQuery& q, uint32_t filter_mode, int refine_iters, bool classes,
                     uint8_t* flags) {
  if (!e.has_graph) return fail(FSIG_ENOGRAPH, "no data graph loaded");
  const DeviceGraph& g = e.g;
  std::vector<HostQuery> qs(1, q);
  BatchLayout b;
  layout_batch(g, qs, b, classes && refine_iters > 0);
  e.arena.release(g.arena_mark);
  int rc = FSIG_OK;
  QVert* d_qv = upload(e, b.qv, rc);
  if (rc) return rc;
  uint32_t* d_lab_gidx = upload(e, b.lab_gidx, rc);
  if (rc) return rc;
  uint32_t* d_lab_begin = upload(e, b.lab_begin, rc);
  if (rc) return rc;
  uint64_t* d_gword = upload(e, b.gword, rc);
  if (rc) return rc;
  uint32_t* d_counts = e.arena.take<uint32_t>(std::max<uint32_t>(b.G, 1));
  if (!d_counts) return fail(FSIG_EADMISSION, "arena");
  uint32_t* pool = nullptr;
  rc = filter_stage(e, b, filter_mode, refine_iters, d_qv, d_gword, d_lab_gidx, d_lab_begin, pool, d_counts);
  if (rc) return rc;
  std::vector<uint32_t> hpool(b.words);
  std::vector<uint32_t> old_of_new(g.V);
  if (b.words)
    FSIG_CUDA_TRY(cudaMemcpyAsync(hpool.data(), pool, sizeof(uint32_t) * b.words, cudaMemcpyDeviceToHost, e.stream));
  FSIG_CUDA_TRY(cudaMemcpyAsync(old_of_new.data(), g.old_of_new, sizeof(uint32_t) * g.V, cudaMemcpyDeviceToHost,
                                e.stream));
  FSIG_CUDA_TRY(cudaStreamSynchronize(e.stream));
  e.arena.release(g.arena_mark);
  std::memset(flags, 0, size_t(q.n) * g.V);
  for (uint32_t u = 0; u < q.n; u++) {
    const QVert& x = b.qv[u];
    for (uint32_t w = 0; w < x.words; w++) {
      uint32_t word = hpool[x.bmoff + w];
      while (word) {
        const uint32_t bit = uint32_t(__builtin_ctz(word));
        word &= word - 1;
        const uint32_t v = x.bmbase + (w << 5) + bit;
        if (v < g.V) flags[size_t(u) * g.V + old_of_new[v]] = 1;
      }
    }
  }
  return FSIG_OK;
}

}  // namespace fsig

namespace fsig {

// ---------------------------------------------------------------------------
// Allocation-free candidate filter.
//
// Some callers cannot allocate device memory when they filter: a process whose
// device memory is all handed to its own pool allocator up front has nothing
// left for cudaMalloc, and code on a latency-critical path cannot accept the
// device-wide synchronisation that cudaFree implies.  For them the filter can
// run with its candidate bitmaps in the fixed array below instead of the
// engine arena; nothing is allocated on the device or the host per call.
//
// The array is a file-scope device variable, so every GPU that loads this
// library holds it until the process exits: 2^21 bitmap words (8 MiB) plus a
// small region for the query's descriptors.  A query whose bitmaps need more
// words is rejected with FSIG_EADMISSION.  All calls share the array and it
// keeps the previous call's contents; each bitmap word is rewritten before it
// is read, and the caller's flag buffer is cleared by the call.  Calls whose
// work overlaps on the GPU (different engines or streams on one device) race
// on the array.  The first call on a device looks up the array's address
// (cudaGetSymbolAddress) with that device current; that first call should
// come before any stream capture.
// ---------------------------------------------------------------------------
namespace {
constexpr uint64_t kNoAllocPoolWords = 1ull << 21;
constexpr uint64_t kNoAllocMetaWords = 8192;
// The metadata region holds the label group table (L + 1 words), the query's
// vertex list (<= 32 words) and its descriptors (32 x 28 words), with slack
// for their 16-byte alignment: 7199 labels fit, more than a loaded graph has.
constexpr uint64_t kNoAllocMaxLabels = kNoAllocMetaWords - 1 - kMaxQ - sizeof(QVert) / 4 * kMaxQ - 64;
static_assert(kMaxLabels <= kNoAllocMaxLabels, "every loadable graph's label table fits the metadata region");
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocPoolWords + kNoAllocMetaWords];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// Device address of the scratch array on `device` (current), looked up once.
int noalloc_scratch(int device, uint32_t** out) {
  if (device < 0 || device >= kNoAllocMaxDevices) return fail(FSIG_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return fail_cuda(err, "cudaGetSymbolAddress", __FILE__, __LINE__);
    g_noalloc_addr[device] = static_cast<uint32_t*>(p);
  }
  *out = g_noalloc_addr[device];
  return FSIG_OK;
}

// Bitmap words -> one flag byte per (query vertex, caller vertex id).
__global__ void bitmap_to_flags_kernel(const QVert* __restrict__ qv, uint32_t n, const uint32_t* __restrict__ pool,
                                       uint64_t total_words, const uint32_t* __restrict__ old_of_new, uint32_t V,
                                       uint8_t* __restrict__ flags) {
  for (uint64_t W = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; W < total_words;
       W += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t u = 0;
    while (u + 1 < n && qv[u + 1].bmoff <= W) u++;
    uint32_t word = pool[W];
    while (word) {
      const uint32_t bit = __ffs(word) - 1;
      word &= word - 1;
      const uint32_t v = qv[u].bmbase + uint32_t((W - qv[u].bmoff) << 5) + bit;
      if (v < V) flags[uint64_t(u) * V + old_of_new[v]] = 1;
    }
  }
}
}  // namespace

int run_filter_noalloc(Engine& e, const fsig_query& q, uint32_t filter_mode, uint8_t* d_flags) {
  if (!e.has_graph) return fail(FSIG_ENOGRAPH, "no data graph loaded");
  const DeviceGraph& g = e.g;
  if (q.num_vertices == 0 || q.num_vertices > uint32_t(kMaxQ)) return fail(FSIG_EQUERY, "query size must be 1..32");
  if (!q.labels || (q.num_edges && !q.edges) || !d_flags) return fail(FSIG_EINVAL, "null argument");
  if (uint64_t(g.L) > kNoAllocMaxLabels)  // guard; a loaded graph has at most kMaxLabels
    return fail(FSIG_EADMISSION, "the allocation-free filter's label table holds " +
                                     std::to_string(kNoAllocMaxLabels) + " labels; the graph has " + std::to_string(g.L));
  const uint32_t n = q.num_vertices;
  // Query descriptors on the stack (no host allocation either).
  QVert qv[kMaxQ];
  uint32_t adj[kMaxQ] = {0};
  for (uint32_t e2 = 0; e2 < q.num_edges; e2++) {
    const uint32_t a = q.edges[2 * e2], b = q.edges[2 * e2 + 1];
    if (a >= n || b >= n) return fail(FSIG_EQUERY, "query edge endpoint out of range");
    if (a == b) continue;
    adj[a] |= 1u << b;
    adj[b] |= 1u << a;
  }
  uint64_t words = 0;
  for (uint32_t u = 0; u < n; u++) {
    QVert& x = qv[u];
    std::memset(&x, 0, sizeof(x));
    x.label = q.labels[u];
    x.adj = adj[u];
    x.deg = uint32_t(__builtin_popcount(adj[u]));
    x.u = u;
    x.cls = uint8_t(u);
    x.cmask = 1u << u;
    x.dom = uint8_t(kNoClass);
    x.sig[0] = uint32_t(x.label);
    for (uint32_t w = 0; w < n; w++) {
      if (!((adj[u] >> w) & 1u)) continue;
      uint32_t word, sh;
      sig_slot(q.labels[w], word, sh);
      const uint32_t cur = (x.sig[word] >> sh) & 3u;
      x.sig[word] |= (cur == 0 ? 1u : 3u) << sh;
    }
    const int32_t l = x.label;
    const uint32_t lo = (l >= 0 && l < g.L) ? g.h_base[l] : 0, hi = (l >= 0 && l < g.L) ? g.h_base[l + 1] : 0;
    x.bmoff = words;
    if (hi > lo) {
      x.bmbase = lo & ~31u;
      x.words = ((hi + 31) >> 5) - (lo >> 5);
    }
    words += x.words;
  }
  if (words > kNoAllocPoolWords)
    return fail(FSIG_EADMISSION, "the query's candidate bitmaps need " + std::to_string(words) +
                                     " words; the allocation-free filter holds 2^21");
  // Label groups: query vertices sorted by label (labels present in the graph).
  uint32_t meta[kNoAllocMetaWords];
  uint32_t* lab_begin = meta;                 // [L + 1]
  uint32_t* lab_gidx = meta + g.L + 1;        // [n]
  uint32_t k = 0;
  for (int32_t l = 0; l < g.L; l++) {
    lab_begin[l] = k;
    for (uint32_t u = 0; u < n; u++)
      if (qv[u].label == l && qv[u].words) lab_gidx[k++] = u;
  }
  lab_begin[g.L] = k;
  uint32_t* scratch = nullptr;
  int rc = noalloc_scratch(e.device, &scratch);
  if (rc) return rc;
  uint32_t* pool = scratch;
  // descriptors at a 16-byte aligned offset of the metadata region
  const uint64_t meta_words = (uint64_t(g.L) + 1 + n + 3) & ~3ull;
  uint32_t* d_meta = scratch + kNoAllocPoolWords;
  QVert* d_qv = reinterpret_cast<QVert*>(d_meta + meta_words);
  cudaStream_t s = e.stream;
  FSIG_CUDA_TRY(cudaMemcpyAsync(d_meta, meta, sizeof(uint32_t) * (uint64_t(g.L) + 1 + n), cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(d_qv, qv, sizeof(QVert) * n, cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(d_flags, 0, uint64_t(n) * g.V, s));
  filter_kernel<<<grid_cap(uint64_t(g.V), kFilterWarps * 32, e.num_sms, 8), kFilterWarps * 32, 0, s>>>(
      view_of(g), d_qv, d_meta + g.L + 1, d_meta, filter_mode, pool);
  FSIG_CUDA_TRY(cudaGetLastError());
  if (words) {
    bitmap_to_flags_kernel<<<grid_cap(words, 256, e.num_sms, 16), 256, 0, s>>>(d_qv, n, pool, words, g.old_of_new,
                                                                                g.V, d_flags);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  return FSIG_OK;
}

}  // namespace fsig
