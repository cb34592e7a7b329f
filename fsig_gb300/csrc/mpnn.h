// Order-scoring network: a 3-layer message-passing network over the query
// graph (hidden 64, BF16 weights and activations, FP32 accumulation), scoring
// each query vertex; the matching order takes the frontier vertex of lowest
// score.  No reference counterpart (the reference orders by heuristics only,
// match/GSI.cu:105-149, match/MMatch.cu:1575-1641).
#pragma once
#include <stdint.h>

#include "engine.h"

namespace fsig {

constexpr int kFeat = 8;     // input features per query vertex
constexpr int kFeatPad = 16; // padded to one k-step of the tensor-core tile
constexpr int kHid = 64;
constexpr int kLayers = 3;

// Flat parameter layout (FP32 master copy).
constexpr int kPWin = 0;                                  // [16][64]
constexpr int kPBin = kPWin + kFeatPad * kHid;            // [64]
constexpr int kPWs = kPBin + kHid;                        // [3][64][64]
constexpr int kPWn = kPWs + kLayers * kHid * kHid;        // [3][64][64]
constexpr int kPB = kPWn + kLayers * kHid * kHid;         // [3][64]
constexpr int kPWout = kPB + kLayers * kHid;              // [64]
constexpr int kPBout = kPWout + kHid;                     // [1]
constexpr int kParams = kPBout + 1;

struct MpnnState {
  float* master = nullptr;   // [kParams]
  float* grad = nullptr;     // [kParams]
  float* m1 = nullptr;       // Adam moments
  float* m2 = nullptr;
  uint16_t* wbf = nullptr;   // BF16 copies of W_in, W_s, W_n (same offsets as master, up to kPB)
  int step = 0;
  bool loaded = false;
};

// Piecewise-linear log2: e + (x / 2^e - 1) with e = floor(log2 x); exact in
// float for x < 2^24 and identical on host and device.  plog2(0) = 0.
__host__ __device__ inline float plog2(uint32_t x) {
  if (x == 0) return 0.f;
  int e = 31;
  while (!((x >> e) & 1u)) e--;
  return float(e) + (float(x) / float(1u << e) - 1.f);
}

struct QVert;
int mpnn_init(Engine& e);
// Shared-memory attributes of the network kernels (once per engine, before
// any stream capture).
int mpnn_configure(Engine& e);
void mpnn_free(Engine& e);
// Features of the batch's query vertices from their candidate counts and the
// heuristic order (d_orders: Q x 32 vertex ids by position), on the device;
// also copies each vertex's neighbour mask to d_nbr.
int mpnn_features_device(Engine& e, const QVert* d_qv, uint32_t G, const uint32_t* d_qoff, uint32_t Q,
                         const uint32_t* d_counts, const uint32_t* d_orders, float* d_feat, uint32_t* d_nbr);
int mpnn_run(Engine& e, uint32_t num_graphs, const uint32_t* goff, const float* feat, const uint32_t* nbr,
             const float* target, float lr, float* scores, float* loss, float* grads_out);
int mpnn_set_params(Engine& e, const float* params);
int mpnn_get_params(Engine& e, float* params);
// Scores for a batch of graphs already on the device.
int mpnn_forward_device(Engine& e, uint32_t num_graphs, const uint32_t* d_goff, const float* d_feat,
                        const uint32_t* d_nbr, float* d_scores);

}  // namespace fsig
