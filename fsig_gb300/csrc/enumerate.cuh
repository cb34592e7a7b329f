// Enumeration kernel: depth-first extension of partial embeddings, one warp
// per task, with work stealing.  Included by match.cu.
//
// A task is (query q, depth d, mapped vertices f[0..d), driver range
// [lo, hi) at depth d).  Pass 0 takes implicit tasks: every root candidate of
// every query, with its depth-1 driver range cut into chunks of `split`
// entries.  Later passes (normally none) take explicit task records.
//
// Level state lives in registers distributed over lanes: lane j holds, for
// depth j, the mapped vertex f_j, the partial hash S_j (sum of fmix64 terms of
// depths 0..j), the driver cursor (dpos_j, dend_j, drv_j) and the candidate
// buffer cursor (cnt_j, it_j).  The candidate buffers (32 per depth) and the
// current query's plan are in shared memory.
//
// Candidates at depth i come from the driver -- the shortest label-l(i)
// segment among the rows of the backward neighbours -- 32 entries at a time,
// one per lane, filtered by injectivity (against earlier same-label depths),
// the candidate bitmap of depth i, and membership in every other backward
// segment.  Membership is decided by the launch's strategy (kIsect*): by
// default every surviving lane binary-searches the segments alone, two at a
// time in lockstep (two independent loads in flight per step); otherwise
// the warp finds the window of that segment spanned by the 32 driver entries
// with a 32-ary search (all lanes probe 32 pivots per round, about log32 of
// the segment length rounds), loads a window of at most 32 entries once and
// searches it in registers by shuffles, a longer one by a per-lane binary
// search inside the window.
//
// Work stealing: warps that run out of input wait for work.  A busy warp
// checks every 64 steps whether idle warps outnumber the queued records; if
// so it hands its shallowest pending depth (buffered candidates and the
// remaining driver range) to the queue as task records and carries on with
// the rest.  Waiting is bounded: a warp that waits too long simply leaves,
// which never loses work -- records still queued when the pass ends are the
// next pass's input.  Every value that steers a warp's control flow is read
// by lane 0 and broadcast.
#pragma once

namespace fsig {
namespace {

struct TaskRec {
  uint32_t f[kMaxQ];
  uint32_t q, d, lo, hi;  // lo == hi == kInvalid: the whole driver range
};

struct EnumArgs {
  GraphView g;
  const Plan* __restrict__ plans;
  const uint32_t* __restrict__ pool;
  uint32_t Q;
  // pass-0 implicit tasks
  const uint32_t* __restrict__ roots;
  const uint32_t* __restrict__ root_q;
  const uint32_t* __restrict__ chunk_off;  // [nroots + 1]
  const uint32_t* __restrict__ nroots_ptr;  // number of roots (device)
  uint32_t split;
  uint32_t t_end;  // pass-0 tasks [initial ctr[0], t_end) (a range of the task space)
  // explicit input tasks (passes >= 1)
  const TaskRec* __restrict__ in_tasks;
  uint32_t in_count;
  // work queue
  TaskRec* out_tasks;
  uint32_t* out_ready;
  uint32_t out_cap;
  uint32_t tag;
  uint32_t* ctr;  // counters, kCtrStride apart: [0] input grab, [1] queue tail (reserved),
                  // [2] queue head, [3] error bits, [4] idle warps, [5] active warps
  uint32_t chunk;
  long long budget;  // cycles on a task before it may be split while warps are idle
  QueryResult* res;
  unsigned long long work_cap;  // per-query limit on examined driver entries (0: none)
  unsigned long long* algo_bytes;
  unsigned long long* ev;       // event counters: tasks, records popped, hand-offs, records written, examines
  unsigned long long seed;
  // optional embedding output (single-query batches): rows of n caller ids,
  // column u = the data vertex of query vertex u; emit_ctr counts every
  // embedding found, rows past emit_cap are not written
  uint32_t* emit;
  unsigned long long emit_cap;
  unsigned long long* emit_ctr;
  // bounded waits (nanoseconds of the GPU's global timer): how long a warp
  // waits for a record it took to be published, and how long an idle warp
  // waits for hand-offs before it leaves (its queued work runs in a later pass)
  unsigned long long ready_wait_ns;
  unsigned long long idle_wait_ns;
  // fault injection for tests: the first record handed off in the pass is
  // written but never published, so the warp that takes it waits out
  // ready_wait_ns and the pass reports a timeout
  uint32_t unpublished;
  // set-intersection strategy (kIsect*)
  uint32_t isect;
};

// Membership of a window's entries in a backward segment:
constexpr uint32_t kIsectBinary = 0;    // every lane binary-searches the segments alone, two in lockstep (default)
constexpr uint32_t kIsectSearch = 1;    // 32-ary window search from the cursor (galloping-like)
constexpr uint32_t kIsectAdaptive = 2;  // the 32 entries after the cursor first (merge-like), else window search
constexpr uint32_t kIsectHybrid = 3;    // the tile when the segment's rest fits 32 entries, else as kIsectBinary

// Backward segments searched in lockstep by the default strategy (three
// spill at 64 registers and run slower).
constexpr int kGroup = 2;

constexpr uint32_t kErrTimeout = 1u;
constexpr uint32_t kCtrStride = 32;        // one 128-byte line per counter
constexpr uint32_t kMaxWaiters = 2048;     // warps beyond this many idle ones leave instead of waiting

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

struct WarpSmem {
  Plan plan;
  uint32_t cand[kMaxQ][kChunk];
};

// Segment [lo, hi) of row v's neighbours with label l (0 <= l < L): two loads
// from the dense table, or, in a graph store without one (kRows), two binary
// searches in the row for the first ids of label classes l and l + 1.
template <bool kRows>
__device__ __forceinline__ void row_segment(const GraphView& g, uint32_t v, int32_t l, uint64_t W1, uint32_t& lo,
                                            uint32_t& hi) {
  if constexpr (kRows) {
    const uint32_t b = __ldg(g.off + v), e = __ldg(g.off + v + 1);
    lo = lower_bound_u32(g.adj, b, e, __ldg(g.base + l));
    hi = lower_bound_u32(g.adj, lo, e, __ldg(g.base + l + 1));
  } else {
    const uint32_t* s = g.lseg + uint64_t(v) * W1 + l;
    lo = s[0];
    hi = s[1];
  }
}

__device__ __forceinline__ bool bsearch_range(const uint32_t* __restrict__ a, uint32_t lo, uint32_t hi, uint32_t x,
                                              uint32_t& bytes) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const uint32_t y = __ldg(a + mid);
    bytes += 4;
    if (y < x) lo = mid + 1;
    else if (y > x) hi = mid;
    else return true;
  }
  return false;
}

// Whether x lies in each of the K sorted ranges a[lo[k], hi[k]): the K binary
// searches run in lockstep, so each step has up to K independent loads in
// flight; it stops as soon as one search ends without x.
template <int K>
__device__ __forceinline__ bool bsearch_all(const uint32_t* __restrict__ a, uint32_t (&lo)[K], uint32_t (&hi)[K],
                                            uint32_t x, uint32_t& bytes) {
  bool in[K];
#pragma unroll
  for (int k = 0; k < K; k++) in[k] = false;
  for (;;) {
    bool s[K], any = false;
#pragma unroll
    for (int k = 0; k < K; k++) {
      s[k] = !in[k] && lo[k] < hi[k];
      if (!in[k] && !s[k]) return false;
      any |= s[k];
    }
    if (!any) return true;
    uint32_t m[K], y[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      m[k] = (lo[k] + hi[k]) >> 1;
      y[k] = s[k] ? __ldg(a + m[k]) : 0u;
      bytes += s[k] ? 4u : 0u;
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (!s[k]) continue;
      if (y[k] < x) lo[k] = m[k] + 1;
      else if (y[k] > x) hi[k] = m[k];
      else in[k] = true;
    }
  }
}

// First index in [lo, hi) of sorted a[] with a[i] >= key (warp-uniform key
// and range): 32 pivots per round, then one 32-entry tile.
__device__ __forceinline__ uint32_t warp_lower_bound(const uint32_t* __restrict__ a, uint32_t lo, uint32_t hi,
                                                     uint32_t key, uint32_t lane, uint32_t& bytes) {
  while (hi - lo > 32) {
    const uint32_t step = (hi - lo + 31) >> 5;
    const uint32_t idx = lo + lane * step;
    const bool in = idx < hi;
    const uint32_t v = in ? __ldg(a + idx) : 0xffffffffu;
    if (in) bytes += 4;
    const uint32_t t = __popc(__ballot_sync(kFull, in && v < key));
    if (t == 0) return lo;
    const uint32_t nlo = lo + (t - 1) * step + 1;
    const uint32_t nhi = min(hi, lo + t * step);
    lo = nlo;
    hi = nhi;
  }
  const uint32_t idx = lo + lane;
  const bool in = idx < hi;
  const uint32_t v = in ? __ldg(a + idx) : 0xffffffffu;
  if (in) bytes += 4;
  return lo + __popc(__ballot_sync(kFull, in && v < key));
}

// kRows: the graph store has no segment table (GraphView::lseg is null) and
// no caller-id copy of the adjacency (adj_old); segments are found in the
// rows and a leaf's caller id is looked up once it survives.
template <bool kRows>
__global__ void __launch_bounds__(kEnumWarps * 32, kEnumMinBlocks) enumerate_kernel(EnumArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem& ws = reinterpret_cast<WarpSmem*>(smem_raw)[threadIdx.x >> 5];
  const uint32_t lane = threadIdx.x & 31;
  const GraphView& g = A.g;
  const uint64_t W1 = uint64_t(g.L) + 1;
  const uint32_t nroots = A.in_tasks ? 0u : *A.nroots_ptr;
  const uint32_t T_in = A.in_tasks ? A.in_count : min(A.chunk_off[nroots], A.t_end);

  // lane-distributed level state
  uint32_t f = 0, dpos = 0, dend = 0, drv = 0, cnt = 0, it = 0;
  unsigned long long S = 0, my_hash = 0;
  // per-lane counters in 32 bits, drained into the 64-bit device totals
  // before any lane's can reach 2^31 (drain, at every periodic check)
  uint32_t lc = 0, my_count = 0, bytes = 0;
  uint32_t pend = 0;  // driver entries examined, not yet published to res.work (lane 0; flushed every 64 windows)
  // event counters (lane 0); a warp's share of one launch fits 32 bits
  uint32_t n_tasks = 0, n_pops = 0, n_handoffs = 0, n_recs = 0, n_examine = 0;
  uint32_t cur_q = kInvalid;

  auto flush = [&]() {
    if (cur_q == kInvalid) return;
    const unsigned long long c = warp_sum((unsigned long long)my_count), h = warp_sum(my_hash);
    if (lane == 0 && (c | h)) {
      atomicAdd(&A.res[cur_q].count, c);
      atomicAdd(&A.res[cur_q].hash, h);
    }
    if (lane < ws.plan.n && lc) atomicAdd(&A.res[cur_q].levels[lane], (unsigned long long)lc);
    my_count = my_hash = 0;
    lc = 0;
  };

  // Publishes the driver entries this warp examined for the current query and
  // reports (warp-uniformly) whether the query is over its limit.  The total
  // a query examines does not depend on how its work was split (ranges are
  // cut at multiples of 32 from the same origins), so whether it exceeds the
  // limit does not either.
  // Also stops the warp's work (true) once the pass has recorded an error:
  // the call will fail anyway, so it returns without finishing the pass.
  auto over_limit = [&]() -> bool {
    if (__any_sync(kFull, (lc | my_count | bytes) >= (1u << 30))) {
      flush();
      const unsigned long long b = warp_sum((unsigned long long)bytes);
      if (lane == 0) atomicAdd(A.algo_bytes, b);
      bytes = 0;
    }
    int stop = 0;
    if (lane == 0) {
      if (A.work_cap) {
        if (pend) {
          const unsigned long long tot = atomicAdd(&A.res[cur_q].work, (unsigned long long)pend) + pend;
          pend = 0;
          if (tot > A.work_cap) atomicExch(&A.res[cur_q].aborted, 1u);
        }
        stop = *(volatile unsigned int*)&A.res[cur_q].aborted != 0;
      }
      stop |= *(volatile uint32_t*)&A.ctr[3 * kCtrStride] != 0;
    }
    return __shfl_sync(kFull, stop, 0) != 0;
  };

  auto use_query = [&](uint32_t q) {
    if (q == cur_q) return;
    if (cur_q != kInvalid) over_limit();  // publish the previous query's work
    flush();
    __syncwarp();
    const uint32_t* src = reinterpret_cast<const uint32_t*>(A.plans + q);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&ws.plan);
    for (uint32_t i = lane; i < sizeof(Plan) / 4; i += 32) dst[i] = src[i];
    __syncwarp();
    cur_q = q;
  };

  // Driver of depth lv from the backward neighbours' rows; stored in lane lv.
  // Backward segment bounds loaded by the last enter(), kept for the scan
  // that follows it at the same depth (lane j: segment j; c_lv: that depth).
  uint32_t c_lo = 0, c_hi = 0, c_lv = kInvalid;

  auto enter = [&](uint32_t lv, uint32_t lo_set, uint32_t hi_set) {
    const uint32_t bw = ws.plan.bwd[lv];
    const int32_t lab = ws.plan.lab[lv];
    uint32_t lo = 0, hi = 0, len = kInvalid;
    if ((bw >> lane) & 1u) {
      row_segment<kRows>(g, f, lab, W1, lo, hi);
      len = hi - lo;
      bytes += 8;
    }
    c_lo = lo;
    c_hi = hi;
    c_lv = lv;
    const bool empty = __ballot_sync(kFull, len == 0) != 0;
    // shortest segment, lowest lane on ties: one warp reduction of (length, lane)
    const uint32_t key = len == kInvalid ? 0xffffffffu : (min(len, (1u << 27) - 1u) << 5) | lane;
    const uint32_t j = __reduce_min_sync(kFull, key) & 31u;
    const uint32_t dlo = __shfl_sync(kFull, lo, j), dhi = __shfl_sync(kFull, hi, j);
    if (lane == lv) {
      if (lo_set != kInvalid) {
        dpos = lo_set;
        dend = hi_set;
      } else {
        dpos = dlo;
        dend = empty ? dlo : dhi;
      }
      drv = j;
      cnt = 0;
      it = 0;
    }
  };

  // Membership of the window's surviving entries (x, lanes in pred) in every
  // backward segment of bw, lane j holding segment j as [seg_lo, seg_hi).
  // Windows of one scan are examined in ascending order, so seg_lo doubles as
  // a cursor: no later window's entries lie below the end of the last window
  // found there.  The 32 entries after the cursor are loaded first; when the
  // window lies among them it is searched there by shuffles (merge-like),
  // otherwise found by 32-ary searches and searched by shuffles (<= 32
  // entries) or per-lane binary search (galloping-like).
  auto member = [&](uint32_t bw, uint32_t x, bool pred, uint32_t& seg_lo, uint32_t seg_hi) -> bool {
    const uint32_t alive = __ballot_sync(kFull, pred);
    if (!bw || !alive) return pred;
    if (A.isect == kIsectBinary) {
      // each surviving lane searches alone, kGroup segments at a time
      while (bw) {
        uint32_t lo[kGroup], hi[kGroup], k = 0;
#pragma unroll
        for (int t = 0; t < kGroup; t++) {
          lo[t] = hi[t] = 0;
          if (bw) {
            const uint32_t j = __ffs(bw) - 1;
            bw &= bw - 1;
            lo[t] = __shfl_sync(kFull, seg_lo, j);
            hi[t] = __shfl_sync(kFull, seg_hi, j);
            k = t + 1;
          }
        }
        if (pred) {
          if (k == kGroup) {
            pred = bsearch_all<kGroup>(g.adj, lo, hi, x, bytes);
          } else if (kGroup > 2 && k == 2) {
            uint32_t l2[2] = {lo[0], lo[1]}, h2[2] = {hi[0], hi[1]};
            pred = bsearch_all<2>(g.adj, l2, h2, x, bytes);
          } else {
            pred = bsearch_range(g.adj, lo[0], hi[0], x, bytes);
          }
        }
        if (__ballot_sync(kFull, pred) == 0) break;
      }
      return pred;
    }
    const uint32_t xfirst = __shfl_sync(kFull, x, __ffs(alive) - 1);
    const uint32_t xlast = __shfl_sync(kFull, x, 31 - __clz(alive));
    while (bw) {
      const uint32_t j = __ffs(bw) - 1;
      bw &= bw - 1;
      const uint32_t lo = __shfl_sync(kFull, seg_lo, j), hi = __shfl_sync(kFull, seg_hi, j);
      if (A.isect == kIsectBinary || (A.isect == kIsectHybrid && hi - lo > 32)) {
        // no cooperation and no cursor: each surviving lane searches alone
        if (pred) pred = bsearch_range(g.adj, lo, hi, x, bytes);
        if (__ballot_sync(kFull, pred) == 0) break;
        continue;
      }
      uint32_t v = 0xffffffffu, ta = 0, tb = 32;
      if (A.isect != kIsectSearch) {
        const uint32_t idx = lo + lane;
        v = idx < hi ? __ldg(g.adj + idx) : 0xffffffffu;
        if (idx < hi) bytes += 4;
        ta = __popc(__ballot_sync(kFull, v < xfirst));
        tb = __popc(__ballot_sync(kFull, v <= xlast));
      }
      uint32_t a, b;
      if (A.isect != kIsectSearch && (tb < 32 || lo + 32 >= hi)) {
        // window [lo + ta, lo + tb) lies in this tile: shuffle search
        b = lo + tb;
        uint32_t l2 = ta, h2 = tb;
#pragma unroll
        for (int step = 0; step < 6; step++) {
          const uint32_t mid = (l2 + h2) >> 1;
          const uint32_t y = __shfl_sync(kFull, v, mid & 31);
          if (l2 < h2) {
            if (y < x) l2 = mid + 1; else h2 = mid;
          }
        }
        const uint32_t y = __shfl_sync(kFull, v, l2 & 31);
        pred = pred && l2 < tb && y == x;
      } else {
        if (A.isect == kIsectSearch) {
          a = warp_lower_bound(g.adj, lo, hi, xfirst, lane, bytes);
          b = warp_lower_bound(g.adj, a, hi, xlast + 1, lane, bytes);
        } else if (ta < 32) {
          a = lo + ta;
          b = warp_lower_bound(g.adj, lo + 32, hi, xlast + 1, lane, bytes);
        } else {
          a = warp_lower_bound(g.adj, lo + 32, hi, xfirst, lane, bytes);
          b = warp_lower_bound(g.adj, a, hi, xlast + 1, lane, bytes);
        }
        const uint32_t w = b - a;
        if (w == 0) {
          pred = false;
        } else if (w <= 32) {
          const uint32_t tile = lane < w ? __ldg(g.adj + a + lane) : 0xffffffffu;
          bytes += lane < w ? 4 : 0;
          uint32_t l2 = 0, h2 = w;
#pragma unroll
          for (int step = 0; step < 6; step++) {
            const uint32_t mid = (l2 + h2) >> 1;
            const uint32_t y = __shfl_sync(kFull, tile, mid & 31);
            if (l2 < h2) {
              if (y < x) l2 = mid + 1; else h2 = mid;
            }
          }
          const uint32_t y = __shfl_sync(kFull, tile, l2 & 31);
          pred = pred && l2 < w && y == x;
        } else if (pred) {
          pred = bsearch_range(g.adj, a, b, x, bytes);
        }
      }
      if (lane == j) seg_lo = b;
      if (__ballot_sync(kFull, pred) == 0) break;
    }
    return pred;
  };

  // Hands the shallowest depth in [d0, lv] that still has work (buffered
  // candidates and the rest of its driver range) to the queue and marks that
  // depth done here.  Returns false when the queue has no room.
  auto donate = [&](uint32_t d0, uint32_t lv) -> bool {
    const uint32_t n = ws.plan.n;
    const uint32_t hand = max(A.split, 32u);  // driver entries per handed-off range
    uint32_t mine = 0;
    if (lane >= d0 && lane <= lv) {
      if (lane + 1 < n && cnt > it) mine += cnt - it;
      if (dend > dpos) mine += (dend - dpos + hand - 1) / hand;
    }
    const uint32_t has = __ballot_sync(kFull, mine > 0);
    if (!has) return true;
    const uint32_t l = __ffs(has) - 1;
    const uint32_t total = __shfl_sync(kFull, mine, l);
    uint32_t base = 0;
    if (lane == 0) {
      base = kInvalid;
      uint32_t r = *(volatile uint32_t*)&A.ctr[1 * kCtrStride];
      while (r + total <= A.out_cap) {
        const uint32_t prev = atomicCAS(&A.ctr[1 * kCtrStride], r, r + total);
        if (prev == r) { base = r; break; }
        r = prev;
      }
    }
    base = __shfl_sync(kFull, base, 0);
    if (base == kInvalid) return false;
    uint32_t slot = base;
    const uint32_t c_l = __shfl_sync(kFull, cnt, l), i_l = __shfl_sync(kFull, it, l);
    const uint32_t p_l = __shfl_sync(kFull, dpos, l), e_l = __shfl_sync(kFull, dend, l);
    if (l + 1 < n) {
      for (uint32_t k = i_l; k < c_l; k++) {
        TaskRec* r = A.out_tasks + slot++;
        const uint32_t cv = ws.cand[l][k];
        if (lane < l) r->f[lane] = f;
        if (lane == l) r->f[lane] = cv;
        if (lane == 0) { r->q = cur_q; r->d = l + 1; r->lo = kInvalid; r->hi = kInvalid; }
      }
    }
    for (uint32_t p = p_l; p < e_l; p += hand) {
      TaskRec* r = A.out_tasks + slot++;
      if (lane < l) r->f[lane] = f;
      if (lane == 0) { r->q = cur_q; r->d = l; r->lo = p; r->hi = min(p + hand, e_l); }
    }
    if (lane == l) {
      it = cnt;
      dpos = dend;
    }
    __threadfence();
    __syncwarp();
    int hold = 0;  // test hook: keep the pass's first handed-off record unpublished
    if (A.unpublished && lane == 0) hold = atomicCAS(&A.ctr[6 * kCtrStride], 0u, 1u) == 0u;
    hold = __shfl_sync(kFull, hold, 0);
    for (uint32_t s = base + lane; s < base + total; s += 32)
      if (!(hold && s == base)) atomicExch(&A.out_ready[s], A.tag);
    if (lane == 0) { n_handoffs++; n_recs += total; }
    return true;
  };

  // Whether idle warps are waiting for more work than the queue holds.
  // Decided by lane 0 alone and broadcast.
  auto should_split = [&](uint32_t t_start) -> bool {
    int w = 0;
    if (lane == 0 && A.out_cap) {
      const uint32_t idle = *(volatile uint32_t*)&A.ctr[4 * kCtrStride];
      if (idle) {
        const uint32_t tail = *(volatile uint32_t*)&A.ctr[1 * kCtrStride], head = *(volatile uint32_t*)&A.ctr[2 * kCtrStride];
        w = (tail - min(head, tail) < idle) && (long long)(uint32_t(clock()) - t_start) > A.budget;
      }
    }
    return __shfl_sync(kFull, w, 0) != 0;
  };

  // Writes the embeddings completed by one leaf examine step: lanes in m hold
  // a leaf's caller id in xo, lanes < lv the shared prefix (f).
  auto emit_rows = [&](uint32_t m, uint32_t lv, uint32_t xo) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(A.emit_ctr, (unsigned long long)__popc(m));
    base = __shfl_sync(kFull, base, 0);
    const uint32_t n = lv + 1;
    const uint32_t col = lane < n ? uint32_t(ws.plan.qv[lane]) : 0u;
    const uint32_t fo = lane < lv ? __ldg(g.old_of_new + f) : 0u;
    uint32_t k = 0;
    while (m) {
      const uint32_t b = __ffs(m) - 1;
      m &= m - 1;
      const uint32_t leaf = __shfl_sync(kFull, xo, b);
      const unsigned long long row = base + k++;
      if (row < A.emit_cap) {
        uint32_t* dst = A.emit + row * n;
        if (lane < lv) dst[col] = fo;
        else if (lane == lv) dst[col] = leaf;
      }
    }
  };

  // Scans the driver windows of depth lv, 32 entries at a time, one per lane:
  // the depth's candidate bitmap, injectivity against earlier depths of the
  // same label, then membership in the other backward segments.  What does not
  // change from window to window -- the bitmap's place, the driver range's
  // end, the backward segments' bounds (with their cursors), and at the leaf
  // the positions of the same-label mapped vertices in the driver range -- is
  // read once per scan.  A non-leaf scan stops at the first window that leaves
  // candidates (they go to the depth's buffer); a leaf scan consumes the whole
  // range, adding embeddings.  Every 64 windows the query's work limit and the
  // idle warps are checked.  Returns false when the query is over its limit.
  auto scan = [&](uint32_t d, uint32_t lv, bool leaf, uint32_t t_start, uint32_t& steps) -> bool {
    const uint32_t dv = __shfl_sync(kFull, drv, lv);
    const uint32_t de = __shfl_sync(kFull, dend, lv);
    uint32_t dp = __shfl_sync(kFull, dpos, lv);
    const uint32_t bmbase = ws.plan.bmbase[lv];
    const uint32_t* __restrict__ bm = A.pool + ws.plan.bmoff[lv];
    const uint32_t bw = ws.plan.bwd[lv] & ~(1u << dv);
    const uint32_t same = ws.plan.same[lv];
    uint32_t seg_lo = c_lo, seg_hi = c_hi;
    if (c_lv != lv) {  // not the scan right after this depth's enter(): load again
      if ((bw >> lane) & 1u) {
        row_segment<kRows>(g, f, ws.plan.lab[lv], W1, seg_lo, seg_hi);
        bytes += 8;
      }
    }
    c_lv = kInvalid;
    // Leaf ranges of more than two windows: lane j of the same-label depths
    // holds the position of f_j in the driver range (kInvalid when absent); the
    // range has no repeated entry, so f_j can only be the entry at that
    // position.  Shorter ranges compare by shuffles, window by window.
    uint32_t same_pos = kInvalid;
    unsigned long long Sp = 0;
    uint64_t tq = 0;
    const bool by_pos = leaf && de - dp > 2 * kChunk;
    if (leaf) {
      if (by_pos && ((same >> lane) & 1u)) {
        uint32_t lo = dp, hi = de;
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          const uint32_t y = __ldg(g.adj + mid);
          bytes += 4;
          if (y < f) lo = mid + 1;
          else if (y > f) hi = mid;
          else { same_pos = mid; break; }
        }
      }
      Sp = __shfl_sync(kFull, S, lv - 1);
      tq = uint64_t(ws.plan.qv[lv]) << 32;
    }
    while (dp < de) {
      const uint32_t nvalid = min(32u, de - dp);
      const uint32_t k = dp + lane;
      bool pred = lane < nvalid;
      const uint32_t x = pred ? __ldg(g.adj + k) : 0xffffffffu;
      uint32_t xo = (!kRows && pred && leaf) ? __ldg(g.adj_old + k) : 0u;
      if (pred) bytes += leaf ? 8 : 4;
      if (pred) {
        const uint32_t bit = x - bmbase;
        pred = (__ldg(bm + (bit >> 5)) >> (bit & 31)) & 1u;
        bytes += 4;
      }
      if (by_pos) {
        uint32_t hit = __ballot_sync(kFull, same_pos - dp < nvalid);
        while (hit) {
          const uint32_t j = __ffs(hit) - 1;
          hit &= hit - 1;
          if (lane == __shfl_sync(kFull, same_pos, j) - dp) pred = false;
        }
      } else {
        uint32_t sm = same;
        while (sm) {
          const uint32_t j = __ffs(sm) - 1;
          sm &= sm - 1;
          const uint32_t fj = __shfl_sync(kFull, f, j);  // every lane shuffles; then the test
          pred = pred && x != fj;
        }
      }
      pred = member(bw, x, pred, seg_lo, seg_hi);
      if (kRows && leaf && pred) xo = __ldg(g.old_of_new + x);
      if (lane == 0) {
        n_examine++;
        if (A.work_cap) pend += nvalid;
      }
      dp += kChunk;
      const uint32_t m = __ballot_sync(kFull, pred);
      if (leaf) {
        if (pred) {
          my_count += 1;
          my_hash += fmix64(A.seed + Sp + fmix64(tq | xo));
        }
        if (A.emit && m) emit_rows(m, lv, xo);
        if (lane == lv) lc += __popc(m);
      } else if (m) {
        __syncwarp();
        if (pred) ws.cand[lv][__popc(m & lanemask_lt())] = x;
        __syncwarp();
        if (lane == lv) {
          dpos = dp;
          cnt = __popc(m);
          it = 0;
          lc += __popc(m);
        }
        return true;
      }
      if ((++steps & 63u) == 0) {
        if (lane == lv) dpos = dp;
        if (over_limit()) return false;
        if (should_split(t_start)) {
          donate(d, lv);
          dp = __shfl_sync(kFull, dpos, lv);  // this depth's range may have been handed off
        }
      }
    }
    if (lane == lv) dpos = dp;
    return true;
  };

  // Runs one task: depth d, mapped f (lane-distributed, lanes < d), driver
  // range override [lo, hi) at depth d.
  auto run = [&](uint32_t d, uint32_t lo_set, uint32_t hi_set) {
    const uint32_t n = ws.plan.n;
    if (lane == 0) n_tasks++;
    // partial hashes of depths < d by an inclusive warp scan of the terms
    unsigned long long term = 0;
    if (lane < d) {
      term = fmix64((uint64_t(ws.plan.qv[lane]) << 32) | __ldg(g.old_of_new + f));
      bytes += 4;
    }
    unsigned long long incl = term;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFull, incl, o);
      if (lane >= uint32_t(o)) incl += y;
    }
    S = incl;
    if (d == n) {  // a complete embedding (single-vertex queries)
      const unsigned long long Sn = __shfl_sync(kFull, S, n - 1);
      if (lane == 0) {
        my_count += 1;
        my_hash += fmix64(A.seed + Sn);
        if (A.emit) {
          const unsigned long long row = atomicAdd(A.emit_ctr, 1ull);
          if (row < A.emit_cap) A.emit[row] = __ldg(g.old_of_new + f);
        }
      }
      return;
    }
    if (over_limit()) return;
    const uint32_t t_start = uint32_t(clock());
    uint32_t lv = d;
    enter(d, lo_set, hi_set);
    uint32_t steps = 0;
    while (true) {
      if ((++steps & 63u) == 0) {
        if (over_limit()) return;
        if (should_split(t_start)) donate(d, lv);
      }
      if (lv == n - 1) {
        if (!scan(d, lv, true, t_start, steps)) return;
        if (lv == d) return;
        lv--;
        continue;
      }
      const uint32_t i = __shfl_sync(kFull, it, lv), c = __shfl_sync(kFull, cnt, lv);
      if (i < c) {
        const uint32_t x = ws.cand[lv][i];
        const unsigned long long Sp = __shfl_sync(kFull, S, lv - 1);
        if (lane == lv) {
          it = i + 1;
          f = x;
          S = Sp + fmix64((uint64_t(ws.plan.qv[lv]) << 32) | __ldg(g.old_of_new + x));
          bytes += 4;
        }
        lv++;
        enter(lv, kInvalid, kInvalid);
        continue;
      }
      if (__shfl_sync(kFull, dpos, lv) < __shfl_sync(kFull, dend, lv)) {
        if (!scan(d, lv, false, t_start, steps)) return;
        continue;
      }
      if (lv == d) return;
      lv--;
    }
  };

  // The header is read by lane 0 and broadcast, like every other value that
  // steers the warp's control flow; records popped in this launch were
  // written by another SM, so they are read through L2 (ld.cg).
  auto run_record = [&](const TaskRec* r) {
    uint32_t q = 0, d = 0, lo = 0, hi = 0;
    if (lane == 0) {
      q = __ldcg(&r->q);
      d = __ldcg(&r->d);
      lo = __ldcg(&r->lo);
      hi = __ldcg(&r->hi);
    }
    q = __shfl_sync(kFull, q, 0);
    d = __shfl_sync(kFull, d, 0);
    lo = __shfl_sync(kFull, lo, 0);
    hi = __shfl_sync(kFull, hi, 0);
    use_query(q);
    if (lane < d) f = __ldcg(&r->f[lane]);
    run(d, lo, hi);
  };

  for (;;) {
    // 1. input tasks (after an error every task returns at once: over_limit)
    uint32_t t0 = T_in;
    if (lane == 0 && *(volatile uint32_t*)&A.ctr[0 * kCtrStride] < T_in) t0 = atomicAdd(&A.ctr[0 * kCtrStride], A.chunk);
    t0 = __shfl_sync(kFull, t0, 0);
    if (t0 < T_in) {
      const uint32_t t1 = min(t0 + A.chunk, T_in);
      for (uint32_t t = t0; t < t1; t++) {
        if (A.in_tasks) {
          run_record(A.in_tasks + t);
        } else {
          // implicit: root i, chunk c of its depth-1 driver range
          uint32_t lo = 0, hi = nroots;  // last i with chunk_off[i] <= t
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (A.chunk_off[mid] <= t) lo = mid; else hi = mid;
          }
          const uint32_t i = lo, c = t - A.chunk_off[i];
          use_query(A.root_q[i]);
          const uint32_t r = A.roots[i];
          if (lane == 0) f = r;
          if (ws.plan.n == 1) {
            run(1, kInvalid, kInvalid);
          } else {
            uint32_t b0, e0;
            row_segment<kRows>(g, r, ws.plan.lab[1], W1, b0, e0);
            const uint32_t clo = b0 + c * A.split;
            if (lane == 0) lc += (c == 0);  // the root itself, once
            run(1, clo, min(clo + A.split, e0));
          }
        }
      }
      continue;
    }
    // 2. input exhausted: take queued records, waiting while others work
    uint32_t slot = kInvalid;
    if (lane == 0) {
      atomicSub(&A.ctr[5 * kCtrStride], 1u);
      const uint32_t waiting = atomicAdd(&A.ctr[4 * kCtrStride], 1u);
      uint32_t sleep_ns = 256;
      // enough warps already wait: leave at once (queued work is never lost)
      const unsigned long long t_idle = global_ns();
      const unsigned long long idle_ns = waiting >= kMaxWaiters ? 0ull : A.idle_wait_ns;
      for (;;) {
        const uint32_t tail = min(*(volatile uint32_t*)&A.ctr[1 * kCtrStride], A.out_cap);
        uint32_t h = *(volatile uint32_t*)&A.ctr[2 * kCtrStride];
        bool got = false;
        while (h < tail) {
          const uint32_t prev = atomicCAS(&A.ctr[2 * kCtrStride], h, h + 1);
          if (prev == h) { slot = h; got = true; break; }
          h = prev;
        }
        if (got) break;
        // finished when nobody works and nothing is queued (active read first)
        if (*(volatile uint32_t*)&A.ctr[5 * kCtrStride] == 0 &&
            *(volatile uint32_t*)&A.ctr[2 * kCtrStride] >= min(*(volatile uint32_t*)&A.ctr[1 * kCtrStride], A.out_cap))
          break;
        if (global_ns() - t_idle >= idle_ns || *(volatile uint32_t*)&A.ctr[3 * kCtrStride]) break;
        __nanosleep(sleep_ns);
        if (sleep_ns < 8192) sleep_ns <<= 1;
      }
      atomicSub(&A.ctr[4 * kCtrStride], 1u);
      if (slot != kInvalid) {
        atomicAdd(&A.ctr[5 * kCtrStride], 1u);
        const unsigned long long t_ready = global_ns();
        while (*(volatile uint32_t*)&A.out_ready[slot] != A.tag) {
          if (global_ns() - t_ready > A.ready_wait_ns) {
            atomicOr(&A.ctr[3 * kCtrStride], kErrTimeout);
            slot = kInvalid - 1;
            break;
          }
          __nanosleep(64);
        }
        if (slot == kInvalid - 1) atomicSub(&A.ctr[5 * kCtrStride], 1u);
      }
    }
    slot = __shfl_sync(kFull, slot, 0);
    if (slot >= kInvalid - 1) break;
    __threadfence();
    if (lane == 0) n_pops++;
    run_record(A.out_tasks + slot);
  }
  if (cur_q != kInvalid) over_limit();
  flush();
  const unsigned long long all_bytes = warp_sum((unsigned long long)bytes);
  if (lane == 0) {
    atomicAdd(A.algo_bytes, all_bytes);
    atomicAdd(&A.ev[0], (unsigned long long)n_tasks);
    atomicAdd(&A.ev[1], (unsigned long long)n_pops);
    atomicAdd(&A.ev[2], (unsigned long long)n_handoffs);
    atomicAdd(&A.ev[3], (unsigned long long)n_recs);
    atomicAdd(&A.ev[4], (unsigned long long)n_examine);
  }
}

}  // namespace
}  // namespace fsig
