// Order-scoring network kernels: features, forward, backward, weight
// gradients and Adam, all hand-written; matrix products on the tensor cores
// with mma.sync m16n8k16 (BF16 operands, FP32 accumulation), one warp per
// query graph (at most 32 vertices = two 16-row tiles).
//
//   h0 = relu(x W_in + b_in)                        x: 8 features, padded to 16
//   h_{l+1} = relu(h_l W_s[l] + (D^-1 A h_l) W_n[l] + b[l]),  l = 0, 1, 2
//   score = h3 . w_out + b_out
//
// Rows of absent vertices (index >= n) are kept at zero.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "match.h"
#include "mpnn.h"

namespace fsig {
namespace {

constexpr int kWarpsPerBlock = 2;
constexpr int kWBf = kPB;  // BF16 weight copy covers [0, kPB): W_in, b_in (unused), W_s, W_n

__device__ __forceinline__ uint16_t f2bf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf2f(uint16_t x) { return __bfloat162float(__ushort_as_bfloat16(x)); }
__device__ __forceinline__ uint32_t pack2(uint16_t lo, uint16_t hi) { return uint32_t(lo) | (uint32_t(hi) << 16); }

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// acc (C[32][64], fragment layout of m16n8k16) += sum_k A(r, k) B(k, n).
// A and B return BF16 bit patterns; K is a multiple of 16.
template <class FA, class FB>
__device__ __forceinline__ void warp_gemm(int K, FA A, FB B, float acc[2][8][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
  for (int kk = 0; kk < K; kk += 16) {
    const int k0 = kk + 2 * c;
    uint32_t a[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      const int r0 = mt * 16 + g, r1 = r0 + 8;
      a[mt][0] = pack2(A(r0, k0), A(r0, k0 + 1));
      a[mt][1] = pack2(A(r1, k0), A(r1, k0 + 1));
      a[mt][2] = pack2(A(r0, k0 + 8), A(r0, k0 + 9));
      a[mt][3] = pack2(A(r1, k0 + 8), A(r1, k0 + 9));
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int n = nt * 8 + g;
      const uint32_t b[2] = {pack2(B(k0, n), B(k0 + 1, n)), pack2(B(k0 + 8, n), B(k0 + 9, n))};
      mma_bf16(acc[0][nt], a[0], b);
      mma_bf16(acc[1][nt], a[1], b);
    }
  }
}

__device__ __forceinline__ void zero_acc(float acc[2][8][4]) {
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
      for (int k = 0; k < 4; k++) acc[i][j][k] = 0.f;
}

// Visits every accumulator element as (row, col, value&).
template <class F>
__device__ __forceinline__ void for_acc(float acc[2][8][4], F f) {
  const int lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int j = 0; j < 4; j++) f(mt * 16 + g + (j >= 2 ? 8 : 0), nt * 8 + 2 * c + (j & 1), acc[mt][nt][j]);
}

struct BlockW {
  uint16_t win[kFeatPad * kHid];
  uint16_t ws[kLayers][kHid * kHid];
  uint16_t wn[kLayers][kHid * kHid];
};

struct WarpBuf {
  uint16_t x[32 * kFeatPad];
  uint16_t h[kLayers + 1][32 * kHid];
  uint16_t m[kLayers][32 * kHid];
  uint16_t dz[32 * kHid];
  float dh[32 * kHid];
  float q[32 * kHid];
  uint32_t nbr[32];
  float invdeg[32];
};

// Per-node record of what the weight-gradient kernel needs (BF16).
constexpr int kActX = 0, kActH = kFeatPad, kActM = kActH + kLayers * kHid, kActDz = kActM + kLayers * kHid,
              kActW = kActDz + (kLayers + 1) * kHid;

// One warp per graph.  Train: also the loss, the bias and output gradients,
// and per-node activations and pre-activation gradients for the weight
// gradients.
template <bool kTrain>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) mpnn_graph_kernel(
    const uint16_t* __restrict__ wbf, const float* __restrict__ master, uint32_t num_graphs,
    const uint32_t* __restrict__ goff, const float* __restrict__ feat, const uint32_t* __restrict__ nbr,
    float* __restrict__ scores, const float* __restrict__ target, float inv_count, float* __restrict__ grad,
    float* __restrict__ loss, uint16_t* __restrict__ acts) {
  extern __shared__ __align__(16) unsigned char smem[];
  BlockW& W = *reinterpret_cast<BlockW*>(smem);
  WarpBuf& B = reinterpret_cast<WarpBuf*>(smem + sizeof(BlockW))[threadIdx.x >> 5];
  for (int i = threadIdx.x; i < kFeatPad * kHid; i += blockDim.x) W.win[i] = wbf[kPWin + i];
  for (int i = threadIdx.x; i < kLayers * kHid * kHid; i += blockDim.x) {
    W.ws[0][i] = wbf[kPWs + i];
    W.wn[0][i] = wbf[kPWn + i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const float* b_in = master + kPBin;
  const float* b_l = master + kPB;
  const float* w_out = master + kPWout;
  const float b_out = master[kPBout];
  float acc[2][8][4];
  for (uint32_t q = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); q < num_graphs;
       q += gridDim.x * kWarpsPerBlock) {
    const uint32_t g0 = goff[q];
    const int n = int(goff[q + 1] - g0);
    // inputs
    for (int r = 0; r < 32; r++) {
      if (lane < kFeatPad) B.x[r * kFeatPad + lane] = (r < n && lane < kFeat) ? f2bf(feat[(g0 + r) * kFeat + lane]) : 0;
    }
    const uint32_t my_nbr = lane < n ? nbr[g0 + lane] : 0u;
    B.nbr[lane] = my_nbr;
    B.invdeg[lane] = my_nbr ? 1.f / float(__popc(my_nbr)) : 0.f;
    __syncwarp();
    // input layer
    zero_acc(acc);
    warp_gemm(kFeatPad, [&](int r, int k) { return B.x[r * kFeatPad + k]; },
              [&](int k, int c) { return W.win[k * kHid + c]; }, acc);
    for_acc(acc, [&](int r, int c, float& v) { B.h[0][r * kHid + c] = r < n ? f2bf(fmaxf(v + b_in[c], 0.f)) : 0; });
    __syncwarp();
    for (int l = 0; l < kLayers; l++) {
      // mean over neighbours, two columns per lane
      for (int r = 0; r < 32; r++) {
        const uint32_t nb = B.nbr[r];
        float s0 = 0.f, s1 = 0.f;
        uint32_t m = nb;
        while (m) {
          const int j = __ffs(m) - 1;
          m &= m - 1;
          s0 += bf2f(B.h[l][j * kHid + 2 * lane]);
          s1 += bf2f(B.h[l][j * kHid + 2 * lane + 1]);
        }
        const float id = B.invdeg[r];
        B.m[l][r * kHid + 2 * lane] = f2bf(s0 * id);
        B.m[l][r * kHid + 2 * lane + 1] = f2bf(s1 * id);
      }
      __syncwarp();
      zero_acc(acc);
      warp_gemm(kHid, [&](int r, int k) { return B.h[l][r * kHid + k]; },
                [&](int k, int c) { return W.ws[l][k * kHid + c]; }, acc);
      warp_gemm(kHid, [&](int r, int k) { return B.m[l][r * kHid + k]; },
                [&](int k, int c) { return W.wn[l][k * kHid + c]; }, acc);
      const float* bl = b_l + l * kHid;
      for_acc(acc, [&](int r, int c, float& v) {
        B.h[l + 1][r * kHid + c] = r < n ? f2bf(fmaxf(v + bl[c], 0.f)) : 0;
      });
      __syncwarp();
    }
    // scores: lane r
    float s = 0.f;
    if (lane < n) {
      s = b_out;
      for (int c = 0; c < kHid; c++) s += bf2f(B.h[kLayers][lane * kHid + c]) * w_out[c];
      scores[g0 + lane] = s;
    }
    if (!kTrain) continue;

    // ---- backward ----
    const float ds = lane < n ? 2.f * inv_count * (s - target[g0 + lane]) : 0.f;
    float lsum = lane < n ? (s - target[g0 + lane]) * (s - target[g0 + lane]) * inv_count : 0.f;
    lsum = warp_sum(lsum);
    const float dsum = warp_sum(ds);
    if (lane == 0) {
      atomicAdd(loss, lsum);
      atomicAdd(grad + kPBout, dsum);
    }
    // d w_out[c] = sum_r h3[r][c] ds_r ; d h3[r][c] = ds_r w_out[c]
    for (int c = lane; c < kHid; c += 32) {
      float gw = 0.f;
      for (int r = 0; r < n; r++) gw += bf2f(B.h[kLayers][r * kHid + c]) * __shfl_sync(0xffffffffu, ds, r);
      atomicAdd(grad + kPWout + c, gw);
    }
    for (int r = 0; r < 32; r++) {
      const float dr = __shfl_sync(0xffffffffu, ds, r);
      B.dh[r * kHid + lane] = dr * w_out[lane];
      B.dh[r * kHid + lane + 32] = dr * w_out[lane + 32];
    }
    __syncwarp();
    for (int l = kLayers - 1; l >= -1; l--) {
      // dz = dh * relu'(h_{l+1}); bias gradient
      const uint16_t* hl1 = B.h[l + 1];
      float db0 = 0.f, db1 = 0.f;
      for (int r = 0; r < 32; r++) {
        const int c0 = lane, c1 = lane + 32;
        const float z0 = (r < n && bf2f(hl1[r * kHid + c0]) > 0.f) ? B.dh[r * kHid + c0] : 0.f;
        const float z1 = (r < n && bf2f(hl1[r * kHid + c1]) > 0.f) ? B.dh[r * kHid + c1] : 0.f;
        B.dz[r * kHid + c0] = f2bf(z0);
        B.dz[r * kHid + c1] = f2bf(z1);
        db0 += z0;
        db1 += z1;
      }
      float* gb = grad + (l >= 0 ? kPB + l * kHid : kPBin);
      atomicAdd(gb + lane, db0);
      atomicAdd(gb + lane + 32, db1);
      __syncwarp();
      // save per-node records for the weight gradients
      for (int r = 0; r < n; r++) {
        uint16_t* rec = acts + uint64_t(g0 + r) * kActW;
        rec[kActDz + (l + 1) * kHid + lane] = B.dz[r * kHid + lane];
        rec[kActDz + (l + 1) * kHid + lane + 32] = B.dz[r * kHid + lane + 32];
        if (l >= 0) {
          rec[kActH + l * kHid + lane] = B.h[l][r * kHid + lane];
          rec[kActH + l * kHid + lane + 32] = B.h[l][r * kHid + lane + 32];
          rec[kActM + l * kHid + lane] = B.m[l][r * kHid + lane];
          rec[kActM + l * kHid + lane + 32] = B.m[l][r * kHid + lane + 32];
        } else if (lane < kFeatPad) {
          rec[kActX + lane] = B.x[r * kFeatPad + lane];
        }
      }
      if (l < 0) break;
      // dh_l = dz W_s^T + A_norm^T (dz W_n^T)
      zero_acc(acc);
      warp_gemm(kHid, [&](int r, int k) { return B.dz[r * kHid + k]; },
                [&](int k, int c) { return W.wn[l][c * kHid + k]; }, acc);
      for_acc(acc, [&](int r, int c, float& v) { B.q[r * kHid + c] = v * B.invdeg[r]; });
      zero_acc(acc);
      warp_gemm(kHid, [&](int r, int k) { return B.dz[r * kHid + k]; },
                [&](int k, int c) { return W.ws[l][c * kHid + k]; }, acc);
      __syncwarp();
      for_acc(acc, [&](int r, int c, float& v) {
        // (A_norm^T Q)[r] = sum over i with r in nbr(i) of Q[i] / deg_i (already scaled)
        float t = v;
        const uint32_t nb = B.nbr[r];  // symmetric adjacency: i in nbr(r) <=> r in nbr(i)
        uint32_t m = nb;
        while (m) {
          const int i = __ffs(m) - 1;
          m &= m - 1;
          t += B.q[i * kHid + c];
        }
        B.dh[r * kHid + c] = r < n ? t : 0.f;
      });
      __syncwarp();
    }
  }
}

// Weight gradients: for matrix id (0: W_in, 1..3: W_s, 4..6: W_n),
// G[i][c] = sum over nodes of A_node[i] * dZ_node[c]; K-split over blocks,
// one warp per 32 output rows.
__global__ void __launch_bounds__(64) mpnn_wgrad_kernel(const uint16_t* __restrict__ acts, uint32_t nodes,
                                                        uint32_t nodes_per_block, float* __restrict__ grad) {
  const int mat = blockIdx.y;
  const int warp = threadIdx.x >> 5;
  const int rows = mat == 0 ? kFeatPad : kHid;
  if (warp * 32 >= rows) return;
  int asrc, dzsrc, gdst;
  if (mat == 0) { asrc = kActX; dzsrc = kActDz; gdst = kPWin; }
  else if (mat <= kLayers) { asrc = kActH + (mat - 1) * kHid; dzsrc = kActDz + mat * kHid; gdst = kPWs + (mat - 1) * kHid * kHid; }
  else { asrc = kActM + (mat - 1 - kLayers) * kHid; dzsrc = kActDz + (mat - kLayers) * kHid; gdst = kPWn + (mat - 1 - kLayers) * kHid * kHid; }
  const uint32_t k_begin = blockIdx.x * nodes_per_block;
  const uint32_t k_end = min(nodes, k_begin + nodes_per_block);
  if (k_begin >= k_end) return;
  float acc[2][8][4];
  zero_acc(acc);
  const int r_base = warp * 32;
  for (uint32_t kb = k_begin; kb < k_end; kb += 16) {
    auto A = [&](int r, int k) -> uint16_t {
      const uint32_t node = kb + k;
      const int i = r_base + r;
      return (node < k_end && i < rows) ? acts[uint64_t(node) * kActW + asrc + i] : uint16_t(0);
    };
    auto Bf = [&](int k, int c) -> uint16_t {
      const uint32_t node = kb + k;
      return node < k_end ? acts[uint64_t(node) * kActW + dzsrc + c] : uint16_t(0);
    };
    warp_gemm(16, A, Bf, acc);
  }
  for_acc(acc, [&](int r, int c, float& v) {
    const int i = r_base + r;
    if (i < rows && v != 0.f) atomicAdd(grad + gdst + i * kHid + c, v);
  });
}

__global__ void mpnn_adam_kernel(float* p, const float* g, float* m1, float* m2, uint16_t* wbf, int n, float lr,
                                 float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float v = p[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    p[i] = v;
    if (i < kWBf) wbf[i] = f2bf(v);
  }
}

__global__ void mpnn_to_bf16_kernel(const float* p, uint16_t* wbf, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) wbf[i] = f2bf(p[i]);
}

// Features (see fsig_mpnn_features in include/fsig.h); thread per query vertex.
__global__ void mpnn_features_kernel(const QVert* __restrict__ qv, uint32_t G, const uint32_t* __restrict__ qoff,
                                     uint32_t Q, const uint32_t* __restrict__ counts,
                                     const uint32_t* __restrict__ orders, const uint32_t* __restrict__ base,
                                     int32_t L, float* __restrict__ feat, uint32_t* __restrict__ nbr) {
  for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < G; gi += gridDim.x * blockDim.x) {
    const QVert& x = qv[gi];
    uint32_t lo = 0, hi = Q;  // query of gi: last q with qoff[q] <= gi
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (qoff[mid] <= gi) lo = mid; else hi = mid;
    }
    const uint32_t g0 = qoff[lo], n = qoff[lo + 1] - g0;
    const uint32_t deg = __popc(x.adj), cnt = counts[gi];
    const uint32_t cls = (x.label >= 0 && x.label < L) ? base[x.label + 1] - base[x.label] : 0u;
    uint32_t sigbits = 0;
    for (int i = 1; i < kSigWords; i++) sigbits += __popc(x.sig[i]);
    float nsum = 0.f;
    for (uint32_t w = 0; w < n; w++)
      if ((x.adj >> w) & 1u) nsum += plog2(counts[g0 + w]);
    uint32_t pos = 0;  // position of this vertex in the heuristic order
    const uint32_t u = gi - g0;
    for (uint32_t i = 0; i < n; i++)
      if (orders[uint64_t(lo) * kMaxQ + i] == u) pos = i;
    float* f = feat + uint64_t(gi) * kFeat;
    f[0] = n > 1 ? float(pos) / float(n - 1) : 0.f;
    f[1] = float(deg) / 8.f;
    f[2] = plog2(cnt) / 20.f;
    f[3] = plog2(cls) / 20.f;
    f[4] = cls ? float(cnt) / float(cls) : 0.f;
    f[5] = float(sigbits) / 16.f;
    f[6] = float(n) / 32.f;
    f[7] = deg ? nsum / float(20u * deg) : 0.f;
    nbr[gi] = x.adj;
  }
}

size_t graph_kernel_smem() { return sizeof(BlockW) + kWarpsPerBlock * sizeof(WarpBuf); }

int launch_graph_kernel(Engine& e, bool train, uint32_t num_graphs, const uint32_t* d_goff, const float* d_feat,
                        const uint32_t* d_nbr, float* d_scores, const float* d_target, float inv_count,
                        float* d_loss, uint16_t* d_acts) {
  MpnnState& M = *e.mpnn;
  if (!num_graphs) return FSIG_OK;
  const size_t smem = graph_kernel_smem();
  const unsigned grid = std::max(1u, std::min<unsigned>((num_graphs + kWarpsPerBlock - 1) / kWarpsPerBlock,
                                                       unsigned(e.num_sms) * 4));
  int rc = mpnn_configure(e);
  if (rc) return rc;
  if (train) {
    mpnn_graph_kernel<true><<<grid, 32 * kWarpsPerBlock, smem, e.stream>>>(
        M.wbf, M.master, num_graphs, d_goff, d_feat, d_nbr, d_scores, d_target, inv_count, M.grad, d_loss, d_acts);
  } else {
    mpnn_graph_kernel<false><<<grid, 32 * kWarpsPerBlock, smem, e.stream>>>(
        M.wbf, M.master, num_graphs, d_goff, d_feat, d_nbr, d_scores, nullptr, 0.f, nullptr, nullptr, nullptr);
  }
  FSIG_CUDA_TRY(cudaGetLastError());
  return FSIG_OK;
}

}  // namespace

int mpnn_configure(Engine& e) {
  if (e.mpnn_configured) return FSIG_OK;
  const int smem = int(graph_kernel_smem());
  FSIG_CUDA_TRY(cudaFuncSetAttribute(mpnn_graph_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  FSIG_CUDA_TRY(cudaFuncSetAttribute(mpnn_graph_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  e.mpnn_configured = true;
  return FSIG_OK;
}

int mpnn_init(Engine& e) {
  if (e.mpnn) return FSIG_OK;
  auto* M = new MpnnState();
  const size_t pb = sizeof(float) * kParams;
  // One-time state outside the arena (the arena is reset when a graph loads).
  if (cudaMalloc(&M->master, pb) != cudaSuccess || cudaMalloc(&M->grad, pb) != cudaSuccess ||
      cudaMalloc(&M->m1, pb) != cudaSuccess || cudaMalloc(&M->m2, pb) != cudaSuccess ||
      cudaMalloc(&M->wbf, sizeof(uint16_t) * kWBf) != cudaSuccess) {
    cudaFree(M->master);
    cudaFree(M->grad);
    cudaFree(M->m1);
    cudaFree(M->m2);
    cudaFree(M->wbf);
    delete M;
    return fail(FSIG_EADMISSION, "cannot reserve the order network's state");
  }
  e.mpnn = M;
  FSIG_CUDA_TRY(cudaMemsetAsync(M->master, 0, pb, e.stream));
  FSIG_CUDA_TRY(cudaMemsetAsync(M->grad, 0, pb, e.stream));
  FSIG_CUDA_TRY(cudaMemsetAsync(M->m1, 0, pb, e.stream));
  FSIG_CUDA_TRY(cudaMemsetAsync(M->m2, 0, pb, e.stream));
  FSIG_CUDA_TRY(cudaMemsetAsync(M->wbf, 0, sizeof(uint16_t) * kWBf, e.stream));
  return FSIG_OK;
}

void mpnn_free(Engine& e) {
  if (!e.mpnn) return;
  cudaFree(e.mpnn->master);
  cudaFree(e.mpnn->grad);
  cudaFree(e.mpnn->m1);
  cudaFree(e.mpnn->m2);
  cudaFree(e.mpnn->wbf);
  delete e.mpnn;
  e.mpnn = nullptr;
}

int mpnn_set_params(Engine& e, const float* params) {
  int rc = mpnn_init(e);
  if (rc) return rc;
  MpnnState& M = *e.mpnn;
  FSIG_CUDA_TRY(cudaMemcpyAsync(M.master, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, e.stream));
  FSIG_CUDA_TRY(cudaMemsetAsync(M.m1, 0, sizeof(float) * kParams, e.stream));
  FSIG_CUDA_TRY(cudaMemsetAsync(M.m2, 0, sizeof(float) * kParams, e.stream));
  mpnn_to_bf16_kernel<<<64, 256, 0, e.stream>>>(M.master, M.wbf, kWBf);
  FSIG_CUDA_TRY(cudaGetLastError());
  FSIG_CUDA_TRY(cudaStreamSynchronize(e.stream));
  M.step = 0;
  M.loaded = true;
  return FSIG_OK;
}

int mpnn_get_params(Engine& e, float* params) {
  if (!e.mpnn || !e.mpnn->loaded) return fail(FSIG_EINVAL, "no order network loaded");
  FSIG_CUDA_TRY(cudaMemcpyAsync(params, e.mpnn->master, sizeof(float) * kParams, cudaMemcpyDeviceToHost, e.stream));
  FSIG_CUDA_TRY(cudaStreamSynchronize(e.stream));
  return FSIG_OK;
}

int mpnn_features_device(Engine& e, const QVert* d_qv, uint32_t G, const uint32_t* d_qoff, uint32_t Q,
                         const uint32_t* d_counts, const uint32_t* d_orders, float* d_feat, uint32_t* d_nbr) {
  if (!e.has_graph) return fail(FSIG_ENOGRAPH, "no data graph loaded");
  if (!G) return FSIG_OK;
  mpnn_features_kernel<<<std::min<uint32_t>((G + 127) / 128, e.num_sms * 8), 128, 0, e.stream>>>(
      d_qv, G, d_qoff, Q, d_counts, d_orders, e.g.base, e.g.L, d_feat, d_nbr);
  FSIG_CUDA_TRY(cudaGetLastError());
  return FSIG_OK;
}

int mpnn_forward_device(Engine& e, uint32_t num_graphs, const uint32_t* d_goff, const float* d_feat,
                        const uint32_t* d_nbr, float* d_scores) {
  if (!e.mpnn || !e.mpnn->loaded) return fail(FSIG_EINVAL, "no order network loaded");
  return launch_graph_kernel(e, false, num_graphs, d_goff, d_feat, d_nbr, d_scores, nullptr, 0.f, nullptr, nullptr);
}

// Host-array entry used by the C ABI: scores, and with targets one training
// step (loss, gradients, Adam update when lr > 0).
int mpnn_run(Engine& e, uint32_t num_graphs, const uint32_t* goff, const float* feat, const uint32_t* nbr,
             const float* target, float lr, float* scores, float* loss, float* grads_out) {
  if (!e.mpnn || !e.mpnn->loaded) return fail(FSIG_EINVAL, "no order network loaded");
  MpnnState& M = *e.mpnn;
  cudaStream_t s = e.stream;
  for (uint32_t q = 0; q < num_graphs; q++)
    if (goff[q + 1] < goff[q] || goff[q + 1] - goff[q] > 32) return fail(FSIG_EINVAL, "graphs have 0..32 vertices");
  const uint32_t nodes = goff[num_graphs];
  const uint64_t mark = e.arena.mark();
  uint32_t* d_goff = e.arena.take<uint32_t>(num_graphs + 1);
  float* d_feat = e.arena.take<float>(std::max<uint64_t>(uint64_t(nodes) * kFeat, 1));
  uint32_t* d_nbr = e.arena.take<uint32_t>(std::max<uint32_t>(nodes, 1));
  float* d_scores = e.arena.take<float>(std::max<uint32_t>(nodes, 1));
  float* d_target = target ? e.arena.take<float>(std::max<uint32_t>(nodes, 1)) : nullptr;
  uint16_t* d_acts = target ? e.arena.take<uint16_t>(std::max<uint64_t>(uint64_t(nodes) * kActW, 1)) : nullptr;
  float* d_loss = e.arena.take<float>(1);
  if (!d_goff || !d_feat || !d_nbr || !d_scores || !d_loss || (target && (!d_target || !d_acts))) {
    e.arena.release(mark);
    return fail(FSIG_EADMISSION, "order-network batch does not fit the arena");
  }
  FSIG_CUDA_TRY(cudaMemcpyAsync(d_goff, goff, sizeof(uint32_t) * (num_graphs + 1), cudaMemcpyHostToDevice, s));
  if (nodes) {
    FSIG_CUDA_TRY(cudaMemcpyAsync(d_feat, feat, sizeof(float) * nodes * kFeat, cudaMemcpyHostToDevice, s));
    FSIG_CUDA_TRY(cudaMemcpyAsync(d_nbr, nbr, sizeof(uint32_t) * nodes, cudaMemcpyHostToDevice, s));
    if (target) FSIG_CUDA_TRY(cudaMemcpyAsync(d_target, target, sizeof(float) * nodes, cudaMemcpyHostToDevice, s));
  }
  int rc;
  if (!target) {
    rc = launch_graph_kernel(e, false, num_graphs, d_goff, d_feat, d_nbr, d_scores, nullptr, 0.f, nullptr, nullptr);
  } else {
    FSIG_CUDA_TRY(cudaMemsetAsync(M.grad, 0, sizeof(float) * kParams, s));
    FSIG_CUDA_TRY(cudaMemsetAsync(d_loss, 0, sizeof(float), s));
    rc = launch_graph_kernel(e, true, num_graphs, d_goff, d_feat, d_nbr, d_scores, d_target,
                             nodes ? 1.f / float(nodes) : 0.f, d_loss, d_acts);
    if (!rc && nodes) {
      const uint32_t per_block = 512;
      dim3 grid((nodes + per_block - 1) / per_block, 1 + 2 * kLayers);
      mpnn_wgrad_kernel<<<grid, 64, 0, s>>>(d_acts, nodes, per_block, M.grad);
      FSIG_CUDA_TRY(cudaGetLastError());
    }
    if (!rc && lr > 0.f) {
      M.step++;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f - std::pow(b1, float(M.step)), c2 = 1.f - std::pow(b2, float(M.step));
      mpnn_adam_kernel<<<64, 256, 0, s>>>(M.master, M.grad, M.m1, M.m2, M.wbf, kParams, lr, b1, b2, 1e-8f, c1, c2);
      FSIG_CUDA_TRY(cudaGetLastError());
    }
  }
  if (rc) { e.arena.release(mark); return rc; }
  if (scores && nodes) FSIG_CUDA_TRY(cudaMemcpyAsync(scores, d_scores, sizeof(float) * nodes, cudaMemcpyDeviceToHost, s));
  if (loss) FSIG_CUDA_TRY(cudaMemcpyAsync(loss, d_loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  if (grads_out) FSIG_CUDA_TRY(cudaMemcpyAsync(grads_out, M.grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s));
  FSIG_CUDA_TRY(cudaStreamSynchronize(s));
  e.arena.release(mark);
  return FSIG_OK;
}

}  // namespace fsig
