// Shared device helpers, the device arena and error plumbing for libfsig.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/fsig.h"

namespace fsig {

constexpr uint32_t kInvalid = 0xffffffffu;
constexpr int kSigWords = 16;          // 512-bit signature, word 0 = label
constexpr uint32_t kMurmurSeed = 17;   // HASHSEED of the reference

// ---------------------------------------------------------------------------
// hashing
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t fmix64(uint64_t k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// MurmurHash2 (Appleby) of one little-endian 32-bit word with seed 17, the
// key hash of the reference's PCSR buckets and signature slots.
__host__ __device__ __forceinline__ uint32_t murmur2_u32(uint32_t k) {
  const uint32_t m = 0x5bd1e995u;
  uint32_t h = kMurmurSeed ^ 4u;
  k *= m;
  k ^= k >> 24;
  k *= m;
  h = (h * m) ^ k;
  h ^= h >> 13;
  h *= m;
  h ^= h >> 15;
  return h;
}

// Signature counter position for a neighbour label: word 1 + a, shift s.
// The shift is (2*b) & 31 with b = (2*slot) % 32 (see the signature builder).
__host__ __device__ __forceinline__ void sig_slot(int32_t label, uint32_t& word, uint32_t& shift) {
  uint32_t hp = murmur2_u32(uint32_t(label)) % 240u;
  word = 1u + (2u * hp) / 32u;
  shift = (2u * ((2u * hp) % 32u)) & 31u;
}

// ---------------------------------------------------------------------------
// device arena: one cudaMalloc, bump allocation with marks
// ---------------------------------------------------------------------------
struct Arena {
  char* base = nullptr;
  uint64_t cap = 0;
  uint64_t top = 0;
  uint64_t peak = 0;

  static constexpr uint64_t kAlign = 256;
  // Returns nullptr when the request does not fit (admission failure).
  template <class T>
  T* take(uint64_t count) {
    uint64_t bytes = (count * sizeof(T) + kAlign - 1) & ~(kAlign - 1);
    if (bytes == 0) bytes = kAlign;
    if (top + bytes > cap) return nullptr;
    T* p = reinterpret_cast<T*>(base + top);
    top += bytes;
    if (top > peak) peak = top;
    return p;
  }
  uint64_t mark() const { return top; }
  void release(uint64_t m) { top = m; }
  uint64_t free_bytes() const { return cap - top; }
};

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// first index in [lo, hi) of sorted a[] with a[i] >= key
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* __restrict__ a, uint32_t lo, uint32_t hi,
                                                    uint32_t key) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

}  // namespace fsig

#define FSIG_CUDA_TRY(expr)                                                        \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) {                                                        \
      return ::fsig::fail_cuda(_e, #expr, __FILE__, __LINE__);                      \
    }                                                                               \
  } while (0)

namespace fsig {
// Records the CUDA error text in a thread-local slot; the C ABI copies it to
// the engine's last-error string.
int fail_cuda(cudaError_t e, const char* what, const char* file, int line);
int fail(int status, const std::string& msg);
const std::string& thread_error();
void clear_thread_error();
}  // namespace fsig
