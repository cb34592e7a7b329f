// The reference's PCSR layout built on the device
// (UndirectedPlainToPCSRTransformer::transform, graph_format_transformer.cc:39-215;
// PCSRUnit and get_edge_label, graph/graph.h:90-123).
//
// One unit per edge label el = get_edge_label(label(v), label(w)) (colliding as
// the reference's does).  A unit's keys are the vertices with at least one
// neighbour in it, in ascending order; key v's list is those neighbours in row
// order.  The unit's offset table has 32 words per key slot: up to 15
// (key, start) pairs, word 30 a chain to an overflow slot, word 31 closing the
// last list.  A key goes to bucket MurmurHash2(key) mod (number of keys);
// keys of a bucket fill its slot in ascending order, every full group of 15
// continues in the next empty bucket (empty buckets taken in ascending order
// as buckets are filled in ascending order); lists are laid out slot by slot.
//
// The engine itself does not use this layout (label segments serve the same
// lookups); it is built for callers of the reference format.  Every step is a
// data-parallel kernel: stable one-bit partitions (scan + scatter) sort the
// entries by unit and the keys by (unit, bucket), and scans place the
// overflow slots and the lists.
#include <algorithm>
#include <vector>

#include "engine.h"
#include "scan.cuh"

namespace fsig {
namespace {

constexpr uint32_t kNone = 0xffffffffu;

__device__ __forceinline__ uint32_t edge_label(int32_t a, int32_t b) {
  const int32_t hi = a >= b ? a : b, lo = a >= b ? b : a;
  return uint32_t(hi == 0 ? lo : ((hi - 1) * hi) / 2 + lo);
}

__global__ void rows_kernel(const uint32_t* __restrict__ off, uint32_t V, uint32_t* __restrict__ row) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < V; v += (gridDim.x * blockDim.x) >> 5)
    for (uint32_t e = off[v] + lane; e < off[v + 1]; e += 32) row[e] = v;
}

__global__ void units_kernel(const int32_t* __restrict__ lab, const uint32_t* __restrict__ row,
                             const uint32_t* __restrict__ adj, uint32_t n, uint32_t* __restrict__ unit) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    unit[e] = edge_label(lab[row[e]], lab[adj[e]]);
}

__global__ void iota_kernel(uint32_t* __restrict__ p, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = i;
}

// zero[t] = 1 when bit `bit` of the sort key of element perm[t] is 0.  The
// key is lo[x] below lo_bits and hi[x] above (hi may be null).
__global__ void zero_flags_kernel(const uint32_t* __restrict__ perm, uint32_t n, const uint32_t* __restrict__ lo,
                                  const uint32_t* __restrict__ hi, uint32_t lo_bits, uint32_t bit,
                                  uint32_t* __restrict__ zero) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t x = perm[t];
    const uint32_t v = bit < lo_bits ? (lo[x] >> bit) : (hi[x] >> (bit - lo_bits));
    zero[t] = (v & 1u) ? 0u : 1u;
  }
}

// Stable partition step: zeros keep their order in front, ones after them.
__global__ void partition_kernel(const uint32_t* __restrict__ perm, uint32_t n, const uint32_t* __restrict__ zero,
                                 const uint32_t* __restrict__ zpos, const uint32_t* __restrict__ zeros_total,
                                 uint32_t* __restrict__ out) {
  const uint32_t Z = *zeros_total;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    out[zero[t] ? zpos[t] : Z + (t - zpos[t])] = perm[t];
}

// Key starts among the entries sorted by (unit, row).
__global__ void key_flags_kernel(const uint32_t* __restrict__ perm, uint32_t n, const uint32_t* __restrict__ unit,
                                 const uint32_t* __restrict__ row, uint32_t* __restrict__ flag) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t x = perm[t];
    bool s = t == 0;
    if (!s) {
      const uint32_t y = perm[t - 1];
      s = unit[x] != unit[y] || row[x] != row[y];
    }
    flag[t] = s ? 1u : 0u;
  }
}

__global__ void keys_kernel(const uint32_t* __restrict__ perm, uint32_t n, const uint32_t* __restrict__ flag,
                            const uint32_t* __restrict__ kid, const uint32_t* __restrict__ unit,
                            const uint32_t* __restrict__ row, uint32_t* __restrict__ kpos,
                            uint32_t* __restrict__ kunit, uint32_t* __restrict__ kvert) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    if (!flag[t]) continue;
    const uint32_t k = kid[t], x = perm[t];
    kpos[k] = t;
    kunit[k] = unit[x];
    kvert[k] = row[x];
  }
}

__global__ void key_sizes_kernel(const uint32_t* __restrict__ kpos, uint32_t K, uint32_t n,
                                 const uint32_t* __restrict__ kunit, uint32_t* __restrict__ klen,
                                 uint32_t* __restrict__ unit_keys, uint32_t* __restrict__ unit_edges) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    const uint32_t len = (k + 1 < K ? kpos[k + 1] : n) - kpos[k];
    klen[k] = len;
    atomicAdd(&unit_keys[kunit[k]], 1u);
    atomicAdd(&unit_edges[kunit[k]], len);
  }
}

__global__ void buckets_kernel(const uint32_t* __restrict__ kvert, const uint32_t* __restrict__ kunit, uint32_t K,
                               const uint32_t* __restrict__ unit_keys, uint32_t* __restrict__ bucket) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
    bucket[k] = murmur2_u32(kvert[k]) % unit_keys[kunit[k]];
}

// Group starts among keys sorted by (unit, bucket), and each group's first
// position; bucket sizes by flat index ubase[unit] + bucket.
__global__ void group_flags_kernel(const uint32_t* __restrict__ q, uint32_t K, const uint32_t* __restrict__ kunit,
                                   const uint32_t* __restrict__ bucket, uint32_t* __restrict__ flag) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < K; t += gridDim.x * blockDim.x) {
    const uint32_t x = q[t];
    bool s = t == 0;
    if (!s) {
      const uint32_t y = q[t - 1];
      s = kunit[x] != kunit[y] || bucket[x] != bucket[y];
    }
    flag[t] = s ? 1u : 0u;
  }
}

__global__ void group_first_kernel(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ gid, uint32_t K,
                                   uint32_t* __restrict__ gfirst) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < K; t += gridDim.x * blockDim.x)
    if (flag[t]) gfirst[gid[t]] = t;
}

// Group id of each position: starts up to and including it, minus one.
__global__ void group_ids_kernel(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ excl, uint32_t K,
                                 uint32_t* __restrict__ gid) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < K; t += gridDim.x * blockDim.x)
    gid[t] = excl[t] + flag[t] - 1;
}

__global__ void ranks_kernel(const uint32_t* __restrict__ q, uint32_t K, const uint32_t* __restrict__ gid,
                             const uint32_t* __restrict__ gfirst, const uint32_t* __restrict__ kunit,
                             const uint32_t* __restrict__ bucket, const uint32_t* __restrict__ ubase,
                             uint32_t* __restrict__ rank, uint32_t* __restrict__ size) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < K; t += gridDim.x * blockDim.x) {
    const uint32_t x = q[t];
    rank[x] = t - gfirst[gid[t]];
    atomicAdd(&size[ubase[kunit[x]] + bucket[x]], 1u);
  }
}

// Per flat bucket: overflow groups (full) and emptiness.
__global__ void bucket_flags_kernel(const uint32_t* __restrict__ size, uint32_t K, uint32_t* __restrict__ full,
                                    uint32_t* __restrict__ empty) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    full[i] = size[i] / 15u;
    empty[i] = size[i] == 0 ? 1u : 0u;
  }
}

// unit of each flat bucket (ubase is ascending)
__device__ __forceinline__ uint32_t unit_of(const uint32_t* __restrict__ ubase, uint32_t U, uint32_t i) {
  uint32_t lo = 0, hi = U;  // last u with ubase[u] <= i
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (ubase[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// empty_list[ubase[u] + r] = local index of the unit's r-th empty bucket.
__global__ void empty_list_kernel(const uint32_t* __restrict__ empty, const uint32_t* __restrict__ epos, uint32_t K,
                                  const uint32_t* __restrict__ ubase, uint32_t U, uint32_t* __restrict__ elist) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    if (!empty[i]) continue;
    const uint32_t u = unit_of(ubase, U, i);
    elist[ubase[u] + (epos[i] - epos[ubase[u]])] = i - ubase[u];
  }
}

__device__ __forceinline__ uint32_t chain_slot(uint32_t j, uint32_t g, uint32_t base, const uint32_t* ovb,
                                               const uint32_t* elist) {
  return g == 0 ? j : elist[base + (ovb[base + j] - ovb[base]) + g - 1];
}

__global__ void table_init_kernel(uint32_t* __restrict__ table, uint64_t words) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < words; i += uint64_t(gridDim.x) * blockDim.x)
    table[i] = (i & 1) ? 0u : kNone;
}

// Chain words of full groups, thread per flat bucket.
__global__ void chains_kernel(const uint32_t* __restrict__ full, const uint32_t* __restrict__ ovb, uint32_t K,
                              const uint32_t* __restrict__ ubase, uint32_t U, const uint32_t* __restrict__ elist,
                              uint32_t* __restrict__ table) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    if (!full[i]) continue;
    const uint32_t u = unit_of(ubase, U, i), base = ubase[u], j = i - base;
    for (uint32_t g = 0; g < full[i]; g++) {
      const uint32_t from = chain_slot(j, g, base, ovb, elist), to = chain_slot(j, g + 1, base, ovb, elist);
      table[32ull * (base + from) + 30] = to;
    }
  }
}

// Slot of every key; list lengths per (slot, position) for the in-slot prefix.
__global__ void key_slots_kernel(uint32_t K, const uint32_t* __restrict__ kunit, const uint32_t* __restrict__ bucket,
                                 const uint32_t* __restrict__ rank, const uint32_t* __restrict__ klen,
                                 const uint32_t* __restrict__ ubase, const uint32_t* __restrict__ ovb,
                                 const uint32_t* __restrict__ elist, uint32_t* __restrict__ kslot,
                                 uint32_t* __restrict__ slot_len15, uint32_t* __restrict__ slot_total) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    const uint32_t base = ubase[kunit[k]];
    const uint32_t s = base + chain_slot(bucket[k], rank[k] / 15u, base, ovb, elist);
    kslot[k] = s;
    slot_len15[15ull * s + rank[k] % 15u] = klen[k];
    atomicAdd(&slot_total[s], klen[k]);
  }
}

// Keys into the table and lists into the edge array, thread per key.
__global__ void place_kernel(uint32_t K, const uint32_t* __restrict__ kunit, const uint32_t* __restrict__ kvert,
                             const uint32_t* __restrict__ kpos, const uint32_t* __restrict__ klen,
                             const uint32_t* __restrict__ rank, const uint32_t* __restrict__ kslot,
                             const uint32_t* __restrict__ slot_len15, const uint32_t* __restrict__ slot_start,
                             const uint32_t* __restrict__ ubase, const uint32_t* __restrict__ perm,
                             const uint32_t* __restrict__ adj, uint32_t* __restrict__ table,
                             uint32_t* __restrict__ edges) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    const uint32_t s = kslot[k], l = rank[k] % 15u;
    uint32_t start = slot_start[s];
    for (uint32_t i = 0; i < l; i++) start += slot_len15[15ull * s + i];
    const uint32_t local = start - slot_start[ubase[kunit[k]]];  // lists are numbered within the unit
    uint32_t* w = table + 32ull * s;
    w[2 * l] = kvert[k];
    w[2 * l + 1] = local;
    w[2 * (l + 1) + 1] = local + klen[k];
    for (uint32_t t = 0; t < klen[k]; t++) edges[start + t] = adj[perm[kpos[k] + t]];
  }
}

unsigned grid_of(uint64_t n, unsigned per, int sms) {
  return unsigned(std::max<uint64_t>(1, std::min<uint64_t>((n + per - 1) / per, uint64_t(sms) * 32)));
}

// Stable sort of perm by the (lo, hi) key bits, one bit per pass.
int bit_sort(Engine& e, uint32_t*& perm, uint32_t*& other, uint32_t n, const uint32_t* lo, const uint32_t* hi,
             uint32_t lo_bits, uint32_t bits, uint32_t* zero, uint32_t* zpos, uint32_t* ztot) {
  cudaStream_t s = e.stream;
  for (uint32_t b = 0; b < bits; b++) {
    zero_flags_kernel<<<grid_of(n, 256, e.num_sms), 256, 0, s>>>(perm, n, lo, hi, lo_bits, b, zero);
    FSIG_CUDA_TRY(cudaGetLastError());
    int rc = device_exclusive_scan<uint32_t>(e.arena, zero, zpos, n, ztot, s);
    if (rc) return rc;
    partition_kernel<<<grid_of(n, 256, e.num_sms), 256, 0, s>>>(perm, n, zero, zpos, ztot, other);
    FSIG_CUDA_TRY(cudaGetLastError());
    std::swap(perm, other);
  }
  return FSIG_OK;
}

uint32_t bit_length(uint64_t x) {
  uint32_t b = 0;
  while (x) { b++; x >>= 1; }
  return std::max(b, 1u);
}

}  // namespace

int build_reference_pcsr(Engine& e, uint32_t V, int32_t L, const int32_t* h_labels, const uint32_t* h_off,
                         const uint32_t* h_adj, uint32_t* h_unit_keys, uint32_t* h_unit_edges, uint32_t* h_table,
                         uint32_t* h_edges) {
  if (V == 0 || L < 1) return fail(FSIG_EINVAL, "graph without vertices or labels");
  for (uint32_t v = 0; v < V; v++)
    if (h_labels[v] < 0 || h_labels[v] >= L) return fail(FSIG_EINVAL, "label outside [0, num_labels)");
  const uint64_t n64 = h_off[V];
  if (n64 >= 0xffffffffull) return fail(FSIG_EINVAL, "too many adjacency entries");
  const uint32_t n = uint32_t(n64);
  const uint32_t U = uint32_t(uint64_t(L) * uint64_t(L + 1) / 2);
  cudaStream_t s = e.stream;
  const uint64_t mark = e.arena.mark();
  auto bail = [&](int rc) {
    cudaStreamSynchronize(s);
    e.arena.release(mark);
    return rc;
  };
  const uint32_t N = std::max(n, 1u);
  int32_t* lab = e.arena.take<int32_t>(V);
  uint32_t* off = e.arena.take<uint32_t>(uint64_t(V) + 1);
  uint32_t* adj = e.arena.take<uint32_t>(N);
  uint32_t* row = e.arena.take<uint32_t>(N);
  uint32_t* unit = e.arena.take<uint32_t>(N);
  uint32_t* pa = e.arena.take<uint32_t>(N);
  uint32_t* pb = e.arena.take<uint32_t>(N);
  uint32_t* zero = e.arena.take<uint32_t>(N);
  uint32_t* zpos = e.arena.take<uint32_t>(N);
  uint32_t* ztot = e.arena.take<uint32_t>(1);
  uint32_t* unit_keys = e.arena.take<uint32_t>(U);
  uint32_t* unit_edges = e.arena.take<uint32_t>(U);
  uint32_t* ubase = e.arena.take<uint32_t>(uint64_t(U) + 1);
  if (!lab || !off || !adj || !row || !unit || !pa || !pb || !zero || !zpos || !ztot || !unit_keys || !unit_edges ||
      !ubase)
    return bail(fail(FSIG_EADMISSION, "PCSR build does not fit the device arena"));
  FSIG_CUDA_TRY(cudaMemcpyAsync(lab, h_labels, sizeof(int32_t) * V, cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(off, h_off, sizeof(uint32_t) * (uint64_t(V) + 1), cudaMemcpyHostToDevice, s));
  if (n) FSIG_CUDA_TRY(cudaMemcpyAsync(adj, h_adj, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(unit_keys, 0, sizeof(uint32_t) * U, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(unit_edges, 0, sizeof(uint32_t) * U, s));
  uint32_t K = 0;
  uint32_t *kpos = nullptr, *kunit = nullptr, *kvert = nullptr, *klen = nullptr;
  if (n) {
    rows_kernel<<<grid_of(uint64_t(V) * 32, 256, e.num_sms), 256, 0, s>>>(off, V, row);
    units_kernel<<<grid_of(n, 256, e.num_sms), 256, 0, s>>>(lab, row, adj, n, unit);
    iota_kernel<<<grid_of(n, 256, e.num_sms), 256, 0, s>>>(pa, n);
    FSIG_CUDA_TRY(cudaGetLastError());
    // entries by unit, stably (rows and row order kept)
    int rc = bit_sort(e, pa, pb, n, unit, nullptr, 32, bit_length(U - 1), zero, zpos, ztot);
    if (rc) return bail(rc);
    key_flags_kernel<<<grid_of(n, 256, e.num_sms), 256, 0, s>>>(pa, n, unit, row, zero);
    FSIG_CUDA_TRY(cudaGetLastError());
    rc = device_exclusive_scan<uint32_t>(e.arena, zero, zpos, n, ztot, s);
    if (rc) return bail(rc);
    FSIG_CUDA_TRY(cudaMemcpyAsync(&K, ztot, 4, cudaMemcpyDeviceToHost, s));
    FSIG_CUDA_TRY(cudaStreamSynchronize(s));
    kpos = e.arena.take<uint32_t>(K);
    kunit = e.arena.take<uint32_t>(K);
    kvert = e.arena.take<uint32_t>(K);
    klen = e.arena.take<uint32_t>(K);
    if (!kpos || !kunit || !kvert || !klen) return bail(fail(FSIG_EADMISSION, "PCSR build does not fit the device arena"));
    keys_kernel<<<grid_of(n, 256, e.num_sms), 256, 0, s>>>(pa, n, zero, zpos, unit, row, kpos, kunit, kvert);
    key_sizes_kernel<<<grid_of(K, 256, e.num_sms), 256, 0, s>>>(kpos, K, n, kunit, klen, unit_keys, unit_edges);
    FSIG_CUDA_TRY(cudaGetLastError());
  }
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_unit_keys, unit_keys, sizeof(uint32_t) * U, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_unit_edges, unit_edges, sizeof(uint32_t) * U, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  if (!h_table || !h_edges || K == 0) return bail(FSIG_OK);

  // keys by (unit, bucket), stably (ascending vertex within a bucket)
  int rc = device_exclusive_scan<uint32_t>(e.arena, unit_keys, ubase, U, ubase + U, s);
  if (rc) return bail(rc);
  uint32_t max_keys = 0;
  for (uint32_t u = 0; u < U; u++) max_keys = std::max(max_keys, h_unit_keys[u]);
  uint32_t* bucket = e.arena.take<uint32_t>(K);
  uint32_t* qa = e.arena.take<uint32_t>(K);
  uint32_t* qb = e.arena.take<uint32_t>(K);
  uint32_t* gid = e.arena.take<uint32_t>(K);
  uint32_t* gfirst = e.arena.take<uint32_t>(K);
  uint32_t* rank = e.arena.take<uint32_t>(K);
  uint32_t* size = e.arena.take<uint32_t>(K);
  uint32_t* full = e.arena.take<uint32_t>(K);
  uint32_t* ovb = e.arena.take<uint32_t>(K);
  uint32_t* empty = e.arena.take<uint32_t>(K);
  uint32_t* epos = e.arena.take<uint32_t>(K);
  uint32_t* elist = e.arena.take<uint32_t>(K);
  uint32_t* kslot = e.arena.take<uint32_t>(K);
  uint32_t* slot_len15 = e.arena.take<uint32_t>(uint64_t(K) * 15);
  uint32_t* slot_total = e.arena.take<uint32_t>(K);
  uint32_t* slot_start = e.arena.take<uint32_t>(K);
  uint32_t* table = e.arena.take<uint32_t>(uint64_t(K) * 32);
  uint32_t* edges_out = e.arena.take<uint32_t>(n);
  if (!bucket || !qa || !qb || !gid || !gfirst || !rank || !size || !full || !ovb || !empty || !epos || !elist ||
      !kslot || !slot_len15 || !slot_total || !slot_start || !table || !edges_out)
    return bail(fail(FSIG_EADMISSION, "PCSR build does not fit the device arena"));
  const unsigned gk = grid_of(K, 256, e.num_sms);
  buckets_kernel<<<gk, 256, 0, s>>>(kvert, kunit, K, unit_keys, bucket);
  iota_kernel<<<gk, 256, 0, s>>>(qa, K);
  FSIG_CUDA_TRY(cudaGetLastError());
  const uint32_t bb = bit_length(max_keys > 0 ? max_keys - 1 : 0);
  rc = bit_sort(e, qa, qb, K, bucket, kunit, bb, bb + bit_length(U - 1), zero, zpos, ztot);
  if (rc) return bail(rc);
  group_flags_kernel<<<gk, 256, 0, s>>>(qa, K, kunit, bucket, zero);
  FSIG_CUDA_TRY(cudaGetLastError());
  rc = device_exclusive_scan<uint32_t>(e.arena, zero, zpos, K, ztot, s);
  if (rc) return bail(rc);
  // a start's exclusive count of starts is its group id
  group_first_kernel<<<gk, 256, 0, s>>>(zero, zpos, K, gfirst);
  group_ids_kernel<<<gk, 256, 0, s>>>(zero, zpos, K, gid);
  FSIG_CUDA_TRY(cudaMemsetAsync(size, 0, sizeof(uint32_t) * K, s));
  FSIG_CUDA_TRY(cudaGetLastError());
  ranks_kernel<<<gk, 256, 0, s>>>(qa, K, gid, gfirst, kunit, bucket, ubase, rank, size);
  bucket_flags_kernel<<<gk, 256, 0, s>>>(size, K, full, empty);
  FSIG_CUDA_TRY(cudaGetLastError());
  rc = device_exclusive_scan<uint32_t>(e.arena, full, ovb, K, ztot, s);
  if (rc) return bail(rc);
  rc = device_exclusive_scan<uint32_t>(e.arena, empty, epos, K, ztot, s);
  if (rc) return bail(rc);
  empty_list_kernel<<<gk, 256, 0, s>>>(empty, epos, K, ubase, U, elist);
  table_init_kernel<<<grid_of(uint64_t(K) * 32, 256, e.num_sms), 256, 0, s>>>(table, uint64_t(K) * 32);
  chains_kernel<<<gk, 256, 0, s>>>(full, ovb, K, ubase, U, elist, table);
  FSIG_CUDA_TRY(cudaMemsetAsync(slot_total, 0, sizeof(uint32_t) * K, s));
  FSIG_CUDA_TRY(cudaMemsetAsync(slot_len15, 0, sizeof(uint32_t) * uint64_t(K) * 15, s));
  key_slots_kernel<<<gk, 256, 0, s>>>(K, kunit, bucket, rank, klen, ubase, ovb, elist, kslot, slot_len15, slot_total);
  FSIG_CUDA_TRY(cudaGetLastError());
  rc = device_exclusive_scan<uint32_t>(e.arena, slot_total, slot_start, K, ztot, s);
  if (rc) return bail(rc);
  place_kernel<<<gk, 256, 0, s>>>(K, kunit, kvert, kpos, klen, rank, kslot, slot_len15, slot_start, ubase, pa, adj,
                                  table, edges_out);
  FSIG_CUDA_TRY(cudaGetLastError());
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_table, table, sizeof(uint32_t) * 32 * uint64_t(K), cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaMemcpyAsync(h_edges, edges_out, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  return bail(FSIG_OK);
}

}  // namespace fsig
