// Device-side graph transforms: the resident matching store (renumbered CSR,
// label segments, signatures) and the reference-layout CSR and signature
// tables.  Replaces the host loops of graph_format_transformer.cc:12-37 and
// :217-281 and the per-buffer copies of match/MMatch.cu:14-32.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "engine.h"
#include "scan.cuh"

namespace fsig {
namespace {

constexpr int kRenumTile = 1024;

// ---- label validation --------------------------------------------------------
__global__ void label_range_kernel(const int32_t* __restrict__ lab, uint32_t V, int32_t* out_max,
                                   uint32_t* out_bad) {
  int32_t mx = -1;
  uint32_t bad = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < V; i += uint64_t(gridDim.x) * blockDim.x) {
    int32_t l = lab[i];
    if (l < 0) bad = 1; else mx = max(mx, l);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out_max, mx);
    if (bad) atomicOr(out_bad, 1u);
  }
}

// ---- stable counting sort of vertices by label ---------------------------------
__global__ void __launch_bounds__(kRenumTile) label_tile_hist_kernel(const int32_t* __restrict__ lab, uint32_t V,
                                                                     int32_t L, uint32_t T, uint32_t* counts) {
  extern __shared__ uint32_t h[];
  for (int i = threadIdx.x; i < L; i += blockDim.x) h[i] = 0;
  __syncthreads();
  uint64_t v = uint64_t(blockIdx.x) * kRenumTile + threadIdx.x;
  if (v < V) atomicAdd(&h[lab[v]], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < L; i += blockDim.x) counts[uint64_t(i) * T + blockIdx.x] = h[i];
}

// counts scanned in (label, tile) order give each tile's first slot per label;
// within a tile, warps take turns so that ranks follow caller ids.
__global__ void __launch_bounds__(kRenumTile) label_tile_rank_kernel(const int32_t* __restrict__ lab, uint32_t V,
                                                                     int32_t L, uint32_t T,
                                                                     const uint32_t* __restrict__ starts,
                                                                     uint32_t* new_of_old, uint32_t* old_of_new,
                                                                     int32_t* label_new) {
  extern __shared__ uint32_t run[];
  for (int i = threadIdx.x; i < L; i += blockDim.x) run[i] = 0;
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t v = uint64_t(blockIdx.x) * kRenumTile + threadIdx.x;
  const bool live = v < V;
  const int32_t l = live ? lab[v] : -1;
  const uint32_t nw = blockDim.x >> 5;
  for (uint32_t w = 0; w < nw; w++) {
    if (warp == w) {
      uint32_t peers = __match_any_sync(0xffffffffu, l);
      uint32_t before = 0;
      if (live) before = run[l];
      __syncwarp();
      if (live) {
        uint32_t rank = __popc(peers & lanemask_lt());
        uint32_t leader = __ffs(peers) - 1;
        uint32_t nid = starts[uint64_t(l) * T + blockIdx.x] + before + rank;
        new_of_old[v] = nid;
        old_of_new[nid] = uint32_t(v);
        label_new[nid] = l;
        if (lane == leader) run[l] = before + __popc(peers);
      }
    }
    __syncthreads();
  }
}

__global__ void base_from_starts_kernel(const uint32_t* __restrict__ starts, int32_t L, uint32_t T, uint32_t V,
                                        uint32_t* base) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < L) base[i] = starts[uint64_t(i) * T];
  if (i == L) base[L] = V;
}

// ---- adjacency -----------------------------------------------------------------
// Degree histogram.  map == nullptr keeps caller ids; drop_loops removes
// self-loops (the matching store) or keeps both copies (the reference CSR).
__global__ void degree_kernel(const uint2* __restrict__ edges, uint64_t E, uint32_t V,
                              const uint32_t* __restrict__ map, bool drop_loops, uint32_t* deg, uint32_t* bad) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < E; i += uint64_t(gridDim.x) * blockDim.x) {
    uint2 e = edges[i];
    if (e.x >= V || e.y >= V) { atomicOr(bad, 2u); continue; }
    if (drop_loops && e.x == e.y) continue;
    uint32_t a = map ? map[e.x] : e.x, b = map ? map[e.y] : e.y;
    atomicAdd(&deg[a], 1u);
    atomicAdd(&deg[b], 1u);
  }
}

__global__ void scatter_kernel(const uint2* __restrict__ edges, uint64_t E, uint32_t V,
                               const uint32_t* __restrict__ map, bool drop_loops, uint32_t* cursor, uint32_t* adj) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < E; i += uint64_t(gridDim.x) * blockDim.x) {
    uint2 e = edges[i];
    if (e.x >= V || e.y >= V) continue;
    if (drop_loops && e.x == e.y) continue;
    uint32_t a = map ? map[e.x] : e.x, b = map ? map[e.y] : e.y;
    adj[atomicAdd(&cursor[a], 1u)] = b;
    adj[atomicAdd(&cursor[b], 1u)] = a;
  }
}

// ---- segmented sort of rows ------------------------------------------------------
constexpr uint32_t kWarpRow = 32, kBlockRow = 2048, kSmemRow = 16384;

__global__ void classify_rows_kernel(const uint32_t* __restrict__ off, uint32_t V, uint32_t* lists,
                                     uint32_t* counts, uint32_t* max_len) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    uint32_t len = off[v + 1] - off[v];
    if (len > 0) atomicMax(max_len, len);
    if (len <= 1) continue;
    int c = len <= kWarpRow ? 0 : (len <= kBlockRow ? 1 : (len <= kSmemRow ? 2 : 3));
    uint32_t p = atomicAdd(&counts[c], 1u);
    lists[uint64_t(c) * V + p] = v;
  }
}

__global__ void sort_rows_warp_kernel(const uint32_t* __restrict__ rows, const uint32_t* __restrict__ count,
                                      const uint32_t* __restrict__ off, uint32_t* adj) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t n = *count;
  for (uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += (gridDim.x * blockDim.x) >> 5) {
    uint32_t v = rows[r];
    uint32_t b = off[v], len = off[v + 1] - b;
    uint32_t x = lane < len ? adj[b + lane] : kInvalid;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
        bool up = (lane & k) == 0;
        bool lower = (lane & j) == 0;
        x = (lower == up) ? min(x, y) : max(x, y);
      }
    }
    if (lane < len) adj[b + lane] = x;
  }
}

__device__ void block_bitonic(uint32_t* s, uint32_t n) {
  for (uint32_t k = 2; k <= n; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t p = i ^ j;
        if (p > i) {
          uint32_t a = s[i], b = s[p];
          bool up = (i & k) == 0;
          if ((a > b) == up) { s[i] = b; s[p] = a; }
        }
      }
      __syncthreads();
    }
  }
}

// One block per row; rows of class c are sorted in shared memory (padded to a
// power of two) or, for the longest rows, in a global scratch buffer.
__global__ void sort_rows_block_kernel(const uint32_t* __restrict__ rows, const uint32_t* __restrict__ count,
                                       const uint32_t* __restrict__ off, uint32_t* adj, uint32_t* gscratch) {
  extern __shared__ uint32_t sm[];
  const uint32_t n = *count;
  for (uint32_t r = blockIdx.x; r < n; r += gridDim.x) {
    uint32_t v = rows[r];
    uint32_t b = off[v], len = off[v + 1] - b;
    uint32_t p2 = 1;
    while (p2 < len) p2 <<= 1;
    uint32_t* s = gscratch ? gscratch + uint64_t(blockIdx.x) * 0 : sm;
    if (gscratch) s = gscratch;  // a single block handles the global class
    for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) s[i] = i < len ? adj[b + i] : kInvalid;
    __syncthreads();
    block_bitonic(s, p2);
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) adj[b + i] = s[i];
    __syncthreads();
  }
}

// Unique entries per sorted row.
__global__ void unique_count_kernel(const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj, uint32_t V,
                                    uint32_t* ucount) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    uint32_t b = off[v], e = off[v + 1], c = 0, prev = kInvalid;
    for (uint32_t i = b; i < e; i++) {
      uint32_t x = adj[i];
      c += x != prev;
      prev = x;
    }
    ucount[v] = c;
  }
}

__global__ void unique_copy_kernel(const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj, uint32_t V,
                                   const uint32_t* __restrict__ noff, uint32_t* out) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    uint32_t b = off[v], e = off[v + 1], w = noff[v], prev = kInvalid;
    for (uint32_t i = b; i < e; i++) {
      uint32_t x = adj[i];
      if (x != prev) out[w++] = x;
      prev = x;
    }
  }
}

// lseg[v*(L+1)+l] = first entry of row v with id >= base[l].
__global__ void label_segments_kernel(const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj,
                                      const uint32_t* __restrict__ base, uint32_t V, int32_t L, uint32_t* lseg) {
  const uint64_t W = uint64_t(L) + 1;
  const uint64_t total = uint64_t(V) * W;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < total; i += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t v = uint32_t(i / W), l = uint32_t(i % W);
    uint32_t b = off[v], e = off[v + 1];
    lseg[i] = (l == uint32_t(L)) ? e : lower_bound_u32(adj, b, e, base[l]);
  }
}

// Signature of every vertex from its label segments: each segment of c > 0
// neighbours applies min(c, 2) saturating increments to its label's counter.
__global__ void signature_from_segments_kernel(const int32_t* __restrict__ label, const uint32_t* __restrict__ lseg,
                                               uint32_t V, int32_t L, uint4* sig) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    uint32_t w[kSigWords];
#pragma unroll
    for (int i = 0; i < kSigWords; i++) w[i] = 0;
    w[0] = uint32_t(label[v]);
    const uint32_t* s = lseg + uint64_t(v) * (uint32_t(L) + 1);
    for (int32_t l = 0; l < L; l++) {
      uint32_t c = s[l + 1] - s[l];
      if (!c) continue;
      uint32_t word, sh;
      sig_slot(l, word, sh);
      for (uint32_t k = 0; k < min(c, 2u); k++) {
        // registers cannot be indexed dynamically without spilling; select.
#pragma unroll
        for (int i = 1; i < kSigWords; i++) {
          if (uint32_t(i) == word) {
            uint32_t cur = (w[i] >> sh) & 3u;
            w[i] |= (cur == 0 ? 1u : 3u) << sh;
          }
        }
      }
    }
    uint4* o = sig + uint64_t(v) * 4;
    o[0] = make_uint4(w[0], w[1], w[2], w[3]);
    o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    o[2] = make_uint4(w[8], w[9], w[10], w[11]);
    o[3] = make_uint4(w[12], w[13], w[14], w[15]);
  }
}

// Reference-layout signature: one saturating increment per adjacency entry
// (duplicates counted as the reference counts them).
__global__ void signature_from_rows_kernel(const int32_t* __restrict__ label, const uint32_t* __restrict__ off,
                                           const uint32_t* __restrict__ adj, uint32_t V, int column_oriented,
                                           uint32_t* out) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    uint32_t w[kSigWords];
#pragma unroll
    for (int i = 0; i < kSigWords; i++) w[i] = 0;
    w[0] = uint32_t(label[v]);
    for (uint32_t e = off[v]; e < off[v + 1]; e++) {
      uint32_t word, sh;
      sig_slot(label[adj[e]], word, sh);
#pragma unroll
      for (int i = 1; i < kSigWords; i++) {
        if (uint32_t(i) == word) {
          uint32_t cur = (w[i] >> sh) & 3u;
          w[i] |= (cur == 0 ? 1u : 3u) << sh;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < kSigWords; i++) {
      if (column_oriented) out[uint64_t(i) * V + v] = w[i];
      else out[uint64_t(v) * kSigWords + i] = w[i];
    }
  }
}

__global__ void gather_kernel(const uint32_t* __restrict__ idx, uint64_t n, const uint32_t* __restrict__ table,
                              uint32_t* out) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    out[i] = table[idx[i]];
}

inline unsigned grid_for(uint64_t n, int threads, int sms) {
  uint64_t b = (n + threads - 1) / threads;
  uint64_t cap = uint64_t(sms) * 32;
  if (b > cap) b = cap;
  return unsigned(b ? b : 1);
}

// Builds offsets/adjacency (rows sorted) from an edge list already on the
// device.  map == nullptr keeps caller ids.  Returns the row data in adj.
int build_rows(Engine& e, const uint2* d_edges, uint64_t E, uint32_t V, const uint32_t* map, bool drop_loops,
               uint32_t* off, uint32_t* adj, uint32_t* d_flags) {
  cudaStream_t s = e.stream;
  uint64_t m = e.arena.mark();
  uint32_t* deg = e.arena.take<uint32_t>(uint64_t(V) + 1);
  uint32_t* lists = e.arena.take<uint32_t>(uint64_t(V) * 4);
  uint32_t* small = e.arena.take<uint32_t>(8);
  if (!deg || !lists || !small) return fail(FSIG_EADMISSION, "graph build scratch does not fit the arena");
  FSIG_CUDA_TRY(cudaMemsetAsync(deg, 0, sizeof(uint32_t) * (uint64_t(V) + 1), s));
  FSIG_CUDA_TRY(cudaMemsetAsync(small, 0, sizeof(uint32_t) * 8, s));
  const int T = 256;
  degree_kernel<<<grid_for(E, T, e.num_sms), T, 0, s>>>(d_edges, E, V, map, drop_loops, deg, d_flags);
  FSIG_CUDA_TRY(cudaGetLastError());
  int rc = device_exclusive_scan<uint32_t>(e.arena, deg, off, uint64_t(V) + 1, nullptr, s);
  if (rc) return rc;
  FSIG_CUDA_TRY(cudaMemcpyAsync(deg, off, sizeof(uint32_t) * V, cudaMemcpyDeviceToDevice, s));
  scatter_kernel<<<grid_for(E, T, e.num_sms), T, 0, s>>>(d_edges, E, V, map, drop_loops, deg, adj);
  FSIG_CUDA_TRY(cudaGetLastError());
  classify_rows_kernel<<<grid_for(V, T, e.num_sms), T, 0, s>>>(off, V, lists, small, small + 4);
  FSIG_CUDA_TRY(cudaGetLastError());
  uint32_t h[8];
  FSIG_CUDA_TRY(cudaMemcpyAsync(h, small, sizeof(h), cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  if (h[0]) {
    sort_rows_warp_kernel<<<grid_for(uint64_t(h[0]) * 32, T, e.num_sms), T, 0, s>>>(lists, small + 0, off, adj);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  if (h[1]) {
    sort_rows_block_kernel<<<std::min<uint32_t>(h[1], e.num_sms * 8), 256, kBlockRow * 4, s>>>(
        lists + uint64_t(V), small + 1, off, adj, nullptr);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  if (h[2]) {
    FSIG_CUDA_TRY(cudaFuncSetAttribute(sort_rows_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kSmemRow * 4));
    sort_rows_block_kernel<<<std::min<uint32_t>(h[2], e.num_sms * 2), 1024, kSmemRow * 4, s>>>(
        lists + 2 * uint64_t(V), small + 2, off, adj, nullptr);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  if (h[3]) {
    uint32_t p2 = 1;
    while (p2 < h[4]) p2 <<= 1;
    uint32_t* gs = e.arena.take<uint32_t>(p2);
    if (!gs) return fail(FSIG_EADMISSION, "row sort scratch does not fit the arena");
    sort_rows_block_kernel<<<1, 1024, 0, s>>>(lists + 3 * uint64_t(V), small + 3, off, adj, gs);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  e.arena.release(m);
  return FSIG_OK;
}

}  // namespace

bool use_segment_table(int mode, uint32_t V, int32_t L, uint64_t nadj) {
  if (mode == FSIG_SEGMENTS_TABLE) return true;
  if (mode == FSIG_SEGMENTS_ROWS) return false;
  return uint64_t(V) * (uint64_t(L) + 1) <= 4 * std::max<uint64_t>(nadj, V);
}

uint64_t store_bytes(const DeviceGraph& g) {
  const uint64_t V = g.V, L1 = uint64_t(g.L) + 1;
  uint64_t b = 4 * V * 3 + 4 * L1 + 4 * (V + 1) + 4 * g.nadj + 64 * V;  // label, id maps, base, off, adj, sig
  if (g.lseg) b += 4 * V * L1 + 4 * g.nadj;                           // lseg, adj_old
  return b;
}

int build_device_graph(Engine& e, uint32_t V, const int32_t* h_labels, uint64_t E, const uint32_t* h_edges) {
  cudaStream_t s = e.stream;
  if (V == 0) return fail(FSIG_EINVAL, "graph has no vertices");
  if (2 * E > 0xffffffffull) return fail(FSIG_EINVAL, "graph has 2^31 or more edges");
  // Reset any previous graph.
  e.arena.release(0);
  e.has_graph = false;
  DeviceGraph g;
  g.V = V;

  // Persistent arrays whose sizes do not depend on L.
  g.label = e.arena.take<int32_t>(V);
  g.old_of_new = e.arena.take<uint32_t>(V);
  g.new_of_old = e.arena.take<uint32_t>(V);
  g.off = e.arena.take<uint32_t>(uint64_t(V) + 1);
  g.adj = e.arena.take<uint32_t>(std::max<uint64_t>(2 * E, 1));
  uint32_t* flags = e.arena.take<uint32_t>(4);
  if (!g.label || !g.old_of_new || !g.new_of_old || !g.off || !g.adj || !flags)
    return fail(FSIG_EADMISSION, "graph does not fit the device arena");
  uint64_t mark_tmp = e.arena.mark();
  int32_t* lab_old = e.arena.take<int32_t>(V);
  uint2* d_edges = e.arena.take<uint2>(std::max<uint64_t>(E, 1));
  if (!lab_old || !d_edges) return fail(FSIG_EADMISSION, "graph staging does not fit the device arena");
  FSIG_CUDA_TRY(cudaMemcpyAsync(lab_old, h_labels, sizeof(int32_t) * V, cudaMemcpyHostToDevice, s));
  if (E) FSIG_CUDA_TRY(cudaMemcpyAsync(d_edges, h_edges, sizeof(uint2) * E, cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(flags, 0, 16, s));
  int32_t init_max = -1;
  FSIG_CUDA_TRY(cudaMemcpyAsync(flags + 1, &init_max, 4, cudaMemcpyHostToDevice, s));
  label_range_kernel<<<grid_for(V, 256, e.num_sms), 256, 0, s>>>(lab_old, V, reinterpret_cast<int32_t*>(flags + 1),
                                                                 flags);
  FSIG_CUDA_TRY(cudaGetLastError());
  uint32_t hf[2];
  FSIG_CUDA_TRY(cudaMemcpyAsync(hf, flags, 8, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hf[0] & 1u) return fail(FSIG_EINVAL, "negative vertex label");
  const int32_t L = int32_t(hf[1]) + 1;
  if (L > int32_t(kMaxLabels)) return fail(FSIG_EINVAL, "more than 4096 distinct labels");
  g.L = L;

  // Renumber by (label, caller id).
  const uint32_t T = (V + kRenumTile - 1) / kRenumTile;
  uint32_t* counts = e.arena.take<uint32_t>(uint64_t(L) * T);
  if (!counts) return fail(FSIG_EADMISSION, "renumbering scratch does not fit the arena");
  label_tile_hist_kernel<<<T, kRenumTile, L * 4, s>>>(lab_old, V, L, T, counts);
  FSIG_CUDA_TRY(cudaGetLastError());
  int rc = device_exclusive_scan<uint32_t>(e.arena, counts, counts, uint64_t(L) * T, nullptr, s);
  if (rc) return rc;
  label_tile_rank_kernel<<<T, kRenumTile, L * 4, s>>>(lab_old, V, L, T, counts, g.new_of_old, g.old_of_new, g.label);
  FSIG_CUDA_TRY(cudaGetLastError());
  uint32_t* base_tmp = e.arena.take<uint32_t>(uint64_t(L) + 1);
  if (!base_tmp) return fail(FSIG_EADMISSION, "arena");
  base_from_starts_kernel<<<(L + 1 + 255) / 256, 256, 0, s>>>(counts, L, T, V, base_tmp);
  FSIG_CUDA_TRY(cudaGetLastError());
  g.h_base.resize(size_t(L) + 1);
  FSIG_CUDA_TRY(cudaMemcpyAsync(g.h_base.data(), base_tmp, sizeof(uint32_t) * (L + 1), cudaMemcpyDeviceToHost, s));

  // Rows in new-id space, self-loops dropped, then duplicates removed.
  rc = build_rows(e, d_edges, E, V, g.new_of_old, true, g.off, g.adj, flags);
  if (rc) return rc;
  uint32_t* ucount = e.arena.take<uint32_t>(uint64_t(V) + 1);
  uint32_t* noff = e.arena.take<uint32_t>(uint64_t(V) + 1);
  uint32_t* totals = e.arena.take<uint32_t>(2);
  if (!ucount || !noff || !totals) return fail(FSIG_EADMISSION, "arena");
  FSIG_CUDA_TRY(cudaMemsetAsync(ucount, 0, sizeof(uint32_t) * (uint64_t(V) + 1), s));
  unique_count_kernel<<<grid_for(V, 256, e.num_sms), 256, 0, s>>>(g.off, g.adj, V, ucount);
  FSIG_CUDA_TRY(cudaGetLastError());
  rc = device_exclusive_scan<uint32_t>(e.arena, ucount, noff, uint64_t(V) + 1, totals, s);
  if (rc) return rc;
  uint32_t h_tot[2] = {0, 0};
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_tot, totals, 4, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_tot + 1, g.off + V, 4, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(hf, flags, 4, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  if (hf[0] & 2u) return fail(FSIG_EINVAL, "edge endpoint out of range");
  if (h_tot[0] != h_tot[1]) {
    uint32_t* tmp = e.arena.take<uint32_t>(std::max<uint32_t>(h_tot[0], 1));
    if (!tmp) return fail(FSIG_EADMISSION, "arena");
    unique_copy_kernel<<<grid_for(V, 256, e.num_sms), 256, 0, s>>>(g.off, g.adj, V, noff, tmp);
    FSIG_CUDA_TRY(cudaGetLastError());
    FSIG_CUDA_TRY(cudaMemcpyAsync(g.adj, tmp, sizeof(uint32_t) * h_tot[0], cudaMemcpyDeviceToDevice, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(g.off, noff, sizeof(uint32_t) * (uint64_t(V) + 1), cudaMemcpyDeviceToDevice, s));
  }
  g.nadj = h_tot[0];
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  e.arena.release(mark_tmp);

  // Persistent label table, segments and signatures.
  const bool table = use_segment_table(e.seg_index, V, L, g.nadj);
  g.base = e.arena.take<uint32_t>(uint64_t(L) + 1);
  g.sig = e.arena.take<uint4>(uint64_t(V) * 4);
  if (table) {
    g.lseg = e.arena.take<uint32_t>(uint64_t(V) * (uint64_t(L) + 1));
    g.adj_old = e.arena.take<uint32_t>(std::max<uint64_t>(g.nadj, 1));
  }
  if (!g.base || !g.sig || (table && (!g.lseg || !g.adj_old)))
    return fail(FSIG_EADMISSION, "graph tables do not fit the device arena");
  FSIG_CUDA_TRY(cudaMemcpyAsync(g.base, g.h_base.data(), sizeof(uint32_t) * (L + 1), cudaMemcpyHostToDevice, s));
  if (table) {
    if (g.nadj) {
      gather_kernel<<<grid_for(g.nadj, 256, e.num_sms), 256, 0, s>>>(g.adj, g.nadj, g.old_of_new, g.adj_old);
      FSIG_CUDA_TRY(cudaGetLastError());
    }
    label_segments_kernel<<<grid_for(uint64_t(V) * (L + 1), 256, e.num_sms), 256, 0, s>>>(g.off, g.adj, g.base, V,
                                                                                         L, g.lseg);
    FSIG_CUDA_TRY(cudaGetLastError());
    signature_from_segments_kernel<<<grid_for(V, 128, e.num_sms), 128, 0, s>>>(g.label, g.lseg, V, L, g.sig);
  } else {
    // one saturating increment per neighbour (rows have no duplicates) gives
    // every label segment's min(count, 2) increments
    signature_from_rows_kernel<<<grid_for(V, 128, e.num_sms), 128, 0, s>>>(g.label, g.off, g.adj, V, 0,
                                                                           reinterpret_cast<uint32_t*>(g.sig));
  }
  FSIG_CUDA_TRY(cudaGetLastError());
  // Maximum degree.
  uint32_t* mx = e.arena.take<uint32_t>(1);
  if (!mx) return fail(FSIG_EADMISSION, "arena");
  FSIG_CUDA_TRY(cudaMemsetAsync(mx, 0, 4, s));
  {
    uint64_t mm = e.arena.mark();
    uint32_t* lists = e.arena.take<uint32_t>(uint64_t(V) * 4);
    uint32_t* small = e.arena.take<uint32_t>(8);
    if (!lists || !small) return fail(FSIG_EADMISSION, "arena");
    FSIG_CUDA_TRY(cudaMemsetAsync(small, 0, 32, s));
    classify_rows_kernel<<<grid_for(V, 256, e.num_sms), 256, 0, s>>>(g.off, V, lists, small, mx);
    FSIG_CUDA_TRY(cudaGetLastError());
    FSIG_CUDA_TRY(cudaMemcpyAsync(&g.max_deg, mx, 4, cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaStreamSynchronize(s));
    e.arena.release(mm);
  }
  g.arena_mark = e.arena.mark();
  e.g = g;
  e.has_graph = true;
  return FSIG_OK;
}

// ---------------------------------------------------------------------------
// Binary cache of the resident graph store: a header, then the device arrays
// as they are (renumbered ids, CSR, caller ids, label segments, signatures),
// so that a later load is a file read and host-to-device copies, with no
// parsing, sorting or segment building.
// ---------------------------------------------------------------------------
namespace {
constexpr char kCacheMagic[8] = {'F', 'S', 'I', 'G', 'G', 'S', '0', '1'};

constexpr uint32_t kCacheRows = 1u;  // CacheHeader::flags: a store without lseg and adj_old

struct CacheHeader {
  char magic[8];
  uint32_t V;
  int32_t L;
  uint64_t nadj;
  uint32_t max_deg;
  uint32_t flags;
};

struct CacheArray {
  void* dev;
  uint64_t bytes;
};

std::vector<CacheArray> cache_arrays(const DeviceGraph& g, bool table) {
  const uint64_t V = g.V, L1 = uint64_t(g.L) + 1;
  return {{g.label, 4 * V},
          {g.old_of_new, 4 * V},
          {g.new_of_old, 4 * V},
          {g.base, 4 * L1},
          {g.off, 4 * (V + 1)},
          {g.adj, 4 * g.nadj},
          {g.adj_old, table ? 4 * g.nadj : 0},
          {g.lseg, table ? 4 * V * L1 : 0},
          {g.sig, 64 * V}};
}
}  // namespace

int save_graph_cache(Engine& e, const char* path) {
  if (!e.has_graph) return fail(FSIG_ENOGRAPH, "no data graph loaded");
  const DeviceGraph& g = e.g;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(FSIG_EIO, std::string("cannot open ") + path);
  CacheHeader h{};
  std::memcpy(h.magic, kCacheMagic, 8);
  h.V = g.V;
  h.L = g.L;
  h.nadj = g.nadj;
  h.max_deg = g.max_deg;
  h.flags = g.lseg ? 0u : kCacheRows;
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
  std::vector<char> buf;
  for (const CacheArray& a : cache_arrays(g, g.lseg != nullptr)) {
    if (!ok) break;
    buf.resize(a.bytes);
    if (a.bytes) {
      const cudaError_t err = cudaMemcpy(buf.data(), a.dev, a.bytes, cudaMemcpyDeviceToHost);
      if (err != cudaSuccess) {
        std::fclose(f);
        return fail_cuda(err, "cudaMemcpy", __FILE__, __LINE__);
      }
      ok = std::fwrite(buf.data(), 1, a.bytes, f) == a.bytes;
    }
  }
  if (std::fclose(f) != 0) ok = false;
  return ok ? FSIG_OK : fail(FSIG_EIO, std::string("cannot write ") + path);
}

int load_graph_cache(Engine& e, const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(FSIG_EIO, std::string("cannot open ") + path);
  CacheHeader h{};
  if (std::fread(&h, sizeof h, 1, f) != 1 || std::memcmp(h.magic, kCacheMagic, 8) != 0 || h.V == 0 || h.L < 1 ||
      h.L > int32_t(kMaxLabels) || (h.flags & ~kCacheRows) != 0) {
    std::fclose(f);
    return fail(FSIG_EIO, std::string(path) + " is not a graph cache of this engine");
  }
  e.arena.release(0);
  e.has_graph = false;
  DeviceGraph g;
  g.V = h.V;
  g.L = h.L;
  g.nadj = h.nadj;
  g.max_deg = h.max_deg;
  const uint64_t V = g.V, L1 = uint64_t(g.L) + 1;
  g.label = e.arena.take<int32_t>(V);
  g.old_of_new = e.arena.take<uint32_t>(V);
  g.new_of_old = e.arena.take<uint32_t>(V);
  g.off = e.arena.take<uint32_t>(V + 1);
  g.adj = e.arena.take<uint32_t>(std::max<uint64_t>(g.nadj, 1));
  const bool table = (h.flags & kCacheRows) == 0;
  g.base = e.arena.take<uint32_t>(L1);
  g.sig = e.arena.take<uint4>(V * 4);
  if (table) {
    g.lseg = e.arena.take<uint32_t>(V * L1);
    g.adj_old = e.arena.take<uint32_t>(std::max<uint64_t>(g.nadj, 1));
  }
  if (!g.label || !g.old_of_new || !g.new_of_old || !g.off || !g.adj || !g.base || !g.sig ||
      (table && (!g.lseg || !g.adj_old))) {
    std::fclose(f);
    e.arena.release(0);
    return fail(FSIG_EADMISSION, "graph does not fit the device arena");
  }
  std::vector<char> buf;
  for (const CacheArray& a : cache_arrays(g, table)) {
    buf.resize(a.bytes);
    if (a.bytes && std::fread(buf.data(), 1, a.bytes, f) != a.bytes) {
      std::fclose(f);
      e.arena.release(0);
      return fail(FSIG_EIO, std::string(path) + " is truncated");
    }
    if (a.bytes) FSIG_CUDA_TRY(cudaMemcpy(a.dev, buf.data(), a.bytes, cudaMemcpyHostToDevice));
  }
  std::fclose(f);
  g.h_base.resize(L1);
  FSIG_CUDA_TRY(cudaMemcpy(g.h_base.data(), g.base, 4 * L1, cudaMemcpyDeviceToHost));
  g.arena_mark = e.arena.mark();
  e.g = g;
  e.has_graph = true;
  return FSIG_OK;
}

int build_reference_csr(Engine& e, uint32_t V, uint64_t E, const uint32_t* h_edges, uint32_t* h_off,
                        uint32_t* h_adj) {
  cudaStream_t s = e.stream;
  if (2 * E > 0xffffffffull) return fail(FSIG_EINVAL, "graph has 2^31 or more edges");
  uint64_t m = e.arena.mark();
  uint32_t* off = e.arena.take<uint32_t>(uint64_t(V) + 1);
  uint32_t* adj = e.arena.take<uint32_t>(std::max<uint64_t>(2 * E, 1));
  uint2* d_edges = e.arena.take<uint2>(std::max<uint64_t>(E, 1));
  uint32_t* flags = e.arena.take<uint32_t>(4);
  if (!off || !adj || !d_edges || !flags) { e.arena.release(m); return fail(FSIG_EADMISSION, "CSR does not fit the arena"); }
  if (E) FSIG_CUDA_TRY(cudaMemcpyAsync(d_edges, h_edges, sizeof(uint2) * E, cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(flags, 0, 16, s));
  int rc = build_rows(e, d_edges, E, V, nullptr, false, off, adj, flags);
  if (rc) { e.arena.release(m); return rc; }
  uint32_t hf = 0;
  FSIG_CUDA_TRY(cudaMemcpyAsync(&hf, flags, 4, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_off, off, sizeof(uint32_t) * (uint64_t(V) + 1), cudaMemcpyDeviceToHost, s));
  if (E) FSIG_CUDA_TRY(cudaMemcpyAsync(h_adj, adj, sizeof(uint32_t) * 2 * E, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  e.arena.release(m);
  if (hf & 2u) return fail(FSIG_EINVAL, "edge endpoint out of range");
  return FSIG_OK;
}

int build_reference_signature(Engine& e, uint32_t V, const int32_t* h_labels, const uint32_t* h_off,
                              const uint32_t* h_adj, int column_oriented, uint32_t* h_sig) {
  cudaStream_t s = e.stream;
  uint64_t nadj = h_off[V];
  uint64_t m = e.arena.mark();
  int32_t* lab = e.arena.take<int32_t>(V);
  uint32_t* off = e.arena.take<uint32_t>(uint64_t(V) + 1);
  uint32_t* adj = e.arena.take<uint32_t>(std::max<uint64_t>(nadj, 1));
  uint32_t* sig = e.arena.take<uint32_t>(uint64_t(V) * kSigWords);
  if (!lab || !off || !adj || !sig) { e.arena.release(m); return fail(FSIG_EADMISSION, "signature does not fit the arena"); }
  FSIG_CUDA_TRY(cudaMemcpyAsync(lab, h_labels, sizeof(int32_t) * V, cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(off, h_off, sizeof(uint32_t) * (uint64_t(V) + 1), cudaMemcpyHostToDevice, s));
  if (nadj) FSIG_CUDA_TRY(cudaMemcpyAsync(adj, h_adj, sizeof(uint32_t) * nadj, cudaMemcpyHostToDevice, s));
  signature_from_rows_kernel<<<grid_for(V, 128, e.num_sms), 128, 0, s>>>(lab, off, adj, V, column_oriented, sig);
  FSIG_CUDA_TRY(cudaGetLastError());
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_sig, sig, sizeof(uint32_t) * kSigWords * V, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  e.arena.release(m);
  return FSIG_OK;
}

}  // namespace fsig
