// Device exclusive prefix sum (reduce-then-scan), used by the graph builder
// and the batch planner in place of cub::DeviceScan::ExclusiveSum
// (match/GSI.cu:15-32, match/MMatch.cu:645-675).  Temporary block sums come
// from the engine arena, so a scan never calls cudaMalloc and never syncs the
// host; the total is left in device memory for the next kernel to read.
#pragma once
#include "common.cuh"

namespace fsig {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint64_t kScanTile = uint64_t(kScanThreads) * kScanItems;

template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* smem_warp, T& total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  T incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= uint32_t(o)) incl += y;
  }
  if (lane == 31) smem_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t nw = blockDim.x >> 5;
    T w = lane < nw ? smem_warp[lane] : T(0);
    T wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= uint32_t(o)) wi += y;
    }
    if (lane < nw) smem_warp[lane] = wi - w;
    if (lane == 31) smem_warp[32] = wi;
  }
  __syncthreads();
  total = smem_warp[32];
  T r = smem_warp[warp] + incl - v;
  __syncthreads();
  return r;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const T* __restrict__ in, uint64_t n,
                                                                  T* __restrict__ block_sums) {
  __shared__ T sw[33];
  const uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++)
    if (base + i < n) s += in[base + i];
  T total;
  block_exclusive_scan<T>(s, sw, total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// out[i] = offset + sum(in[0..i)); in may equal out.  total_out (optional)
// receives the grand total when this is the top-level single-block pass.
template <class T>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const T* in, T* out, uint64_t n,
                                                                 const T* __restrict__ block_offsets,
                                                                 T* total_out) {
  __shared__ T sw[33];
  const uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
  T v[kScanItems];
  T s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    v[i] = (base + i < n) ? in[base + i] : T(0);
    s += v[i];
  }
  T total;
  T ex = block_exclusive_scan<T>(s, sw, total);
  T off = block_offsets ? block_offsets[blockIdx.x] : T(0);
  T run = off + ex;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (total_out && threadIdx.x == 0 && blockIdx.x == gridDim.x - 1) *total_out = off + total;
}

// Exclusive scan of n elements; *total (device pointer, may be null) gets the
// sum.  Block-sum scratch comes from the arena and is released on return.
template <class T>
int device_exclusive_scan(Arena& arena, const T* in, T* out, uint64_t n, T* total, cudaStream_t s,
                          uint32_t* launches = nullptr) {
  if (n == 0) {
    if (total) FSIG_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(T), s));
    return FSIG_OK;
  }
  const uint64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    scan_apply_kernel<T><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, total);
    FSIG_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 1;
    return FSIG_OK;
  }
  uint64_t m = arena.mark();
  T* sums = arena.take<T>(nb);
  if (!sums) return fail(FSIG_EADMISSION, "scan scratch does not fit the arena");
  scan_reduce_kernel<T><<<unsigned(nb), kScanThreads, 0, s>>>(in, n, sums);
  FSIG_CUDA_TRY(cudaGetLastError());
  int rc = device_exclusive_scan<T>(arena, sums, sums, nb, total, s, launches);
  if (rc != FSIG_OK) return rc;
  scan_apply_kernel<T><<<unsigned(nb), kScanThreads, 0, s>>>(in, out, n, sums, nullptr);
  FSIG_CUDA_TRY(cudaGetLastError());
  if (launches) *launches += 2;
  arena.release(m);
  return FSIG_OK;
}

}  // namespace fsig
