// Engine state shared by the libfsig translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace fsig {

constexpr uint32_t kMaxLabels = 4096;  // labels 0..4095 in a loaded data graph

// The resident data graph, renumbered so that every label class occupies a
// contiguous id range: new ids are sorted by (label, caller id).  In this id
// space a row of the adjacency sorted by id is also sorted by neighbour
// label, so the neighbours of v with label l are one contiguous segment
// [lseg[v*(L+1)+l], lseg[v*(L+1)+l+1]) -- the label-partitioned layout that
// replaces the reference's hashed PCSR units.  A store built without the
// table (FSIG_SEGMENTS_ROWS: V x (L+1) words is large next to the adjacency)
// finds the same segment by binary search in the row, between the first ids
// of classes l and l+1 (base).
struct DeviceGraph {
  uint32_t V = 0;
  int32_t L = 0;
  uint64_t nadj = 0;
  uint32_t max_deg = 0;
  int32_t* label = nullptr;        // [V]   label of each new id
  uint32_t* old_of_new = nullptr;  // [V]
  uint32_t* new_of_old = nullptr;  // [V]
  uint32_t* base = nullptr;        // [L+1] first new id of each label class
  uint32_t* off = nullptr;         // [V+1]
  uint32_t* adj = nullptr;         // [nadj] new ids, rows ascending, no duplicates
  uint32_t* adj_old = nullptr;     // [nadj] caller id of each adj entry (for the result hash); null without lseg
  uint32_t* lseg = nullptr;        // [V*(L+1)]; null: segments are found by binary search in the rows
  uint4* sig = nullptr;            // [V*4] 64-byte signature per vertex
  std::vector<uint32_t> h_base;    // host copy of base
  uint64_t arena_mark = 0;         // arena top after the graph store
};

struct Engine {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  Arena arena;
  DeviceGraph g;
  bool has_graph = false;
  std::string last_error;
  // pinned host staging for batches
  void* pinned = nullptr;
  uint64_t pinned_bytes = 0;
  // enumeration kernel: resident blocks per SM (0 until first queried)
  int enum_per_sm[9] = {0};       // resident blocks per SM at 1..8 warps per block (0 until queried)
  int enum_per_sm_rows[9] = {0};  // the same for a graph store without a segment table
  int seg_index = 0;              // segment index of the next graph build (FSIG_SEGMENTS_*)
  // timing events
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev_enum[2] = {nullptr, nullptr};
  cudaEvent_t ev_outer[2] = {nullptr, nullptr};  // around a graph launch
  fsig_batch_stats last{};
  uint64_t cur_h2d = 0;  // host-to-device bytes of the call in progress
  unsigned long long last_ev[8] = {0};  // enumeration event counters of the last call
  struct MpnnState* mpnn = nullptr;      // order-scoring network (mpnn.cu), created on first use
  bool mpnn_configured = false;          // its kernels' shared-memory attributes are set
  cudaGraphExec_t gexec = nullptr;       // the last batch's executable graph, updated in place
  // bounded waits of the enumeration's work queue (fsig_set_queue_waits)
  uint64_t ready_wait_ns = 200000000ull;   // a taken record's publication: 200 ms
  uint64_t idle_wait_ns = 2000000000ull;   // an idle warp waiting for hand-offs: 2 s
  uint32_t inject_unpublished = 0;         // test hook: leave each pass's first hand-off unpublished
};

// graph_store.cu
int build_device_graph(Engine& e, uint32_t V, const int32_t* labels, uint64_t E, const uint32_t* edges);
bool use_segment_table(int mode, uint32_t V, int32_t L, uint64_t nadj);
uint64_t store_bytes(const DeviceGraph& g);
int save_graph_cache(Engine& e, const char* path);
// pcsr.cu
int build_reference_pcsr(Engine& e, uint32_t V, int32_t L, const int32_t* labels, const uint32_t* off,
                         const uint32_t* adj, uint32_t* unit_keys, uint32_t* unit_edges, uint32_t* table,
                         uint32_t* edges);
int load_graph_cache(Engine& e, const char* path);
int build_reference_csr(Engine& e, uint32_t V, uint64_t E, const uint32_t* edges, uint32_t* offsets,
                        uint32_t* adj);
int build_reference_signature(Engine& e, uint32_t V, const int32_t* labels, const uint32_t* offsets,
                              const uint32_t* adj, int column_oriented, uint32_t* sig);

}  // namespace fsig
