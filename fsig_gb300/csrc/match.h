// Batch matching pipeline shared between the C ABI and the planner.
#pragma once
#include <stdint.h>

#include <vector>

#include "engine.h"

namespace fsig {

constexpr int kMaxQ = FSIG_MAX_QUERY;
constexpr uint32_t kNoClass = FSIG_NO_CLASS;  // no dominated class

// Filter tests (bit flags).
constexpr uint32_t kFilterDegree = 1u;
constexpr uint32_t kFilterSignature = 2u;

// Device order modes.
constexpr uint32_t kOrderGSI = 0;      // candidate count, 0.9 decay of neighbours (match/GSI.cu:105-149)
constexpr uint32_t kOrderMMatch = 1;   // core < forest < leaf offsets, then count (match/MMatch.cu:1575-1641)
constexpr uint32_t kOrderScores = 2;   // externally supplied scores (learned), frontier argmin
constexpr uint32_t kOrderGiven = 3;    // fixed order

// One validated query, in host form.
struct HostQuery {
  uint32_t n = 0;
  // neighbour lists in the caller's edge order (both directions, duplicates
  // kept), as UndirectedPlainGraph::add_edge builds them (graph/graph.cc:23-33);
  // the reference orders iterate these lists.
  std::vector<std::vector<uint32_t>> nbr;
  int32_t label[kMaxQ];
  uint32_t adj[kMaxQ];   // neighbour bitmask (no self-loops, no duplicates)
  uint32_t deg[kMaxQ];
  uint32_t sig[kMaxQ][kSigWords];
  uint32_t given[kMaxQ];
  bool has_given = false;
  int status = FSIG_OK;
};

int prepare_query(const fsig_query& q, int32_t num_labels, HostQuery& out);

// Per-query-vertex descriptor on the device (16-byte aligned for the
// vector loads of the signature).
struct alignas(16) QVert {
  uint32_t sig[kSigWords];
  int32_t label;
  uint32_t deg;
  uint32_t adj;        // neighbours, as local ids of the same query
  uint32_t q;          // query index in the batch
  uint32_t u;          // local id
  uint32_t words;      // bitmap words (0: no data vertex carries this label)
  uint32_t bmbase;     // first new id covered by bitmap word 0 (multiple of 32)
  uint32_t cmask;      // members of its refinement class (local ids)
  uint8_t cls;         // refinement class: local id of its smallest member
  uint8_t dom;         // class whose candidate set contains this class's (kNoClass: none)
  uint8_t alias;       // 1: uses the bitmap of vertex cls (no words of its own)
  uint8_t pad;
  uint64_t bmoff;      // word offset of the bitmap in the pool
};

// Per-query matching plan, built on the device from the chosen order.
struct Plan {
  uint32_t n;
  uint32_t ok;         // 0: some vertex has no candidate, nothing to enumerate
  uint32_t g0;         // first query-vertex descriptor of this query
  uint32_t pad;
  uint32_t qv[kMaxQ];      // query vertex at position i
  int32_t lab[kMaxQ];      // its label
  uint32_t bwd[kMaxQ];     // positions j < i adjacent to position i
  uint32_t same[kMaxQ];    // positions j < i with the same label
  uint32_t bmbase[kMaxQ];
  uint64_t bmoff[kMaxQ];
};

struct QueryResult {
  unsigned long long count;
  unsigned long long hash;
  unsigned long long levels[kMaxQ];
  unsigned long long work;   // driver entries examined so far (with a limit)
  unsigned int aborted;      // 1: the limit was exceeded
  unsigned int pad;
};

// Refinement: candidate segments longer than this are scanned by the whole
// warp, shorter ones by the candidate's own lane.
constexpr uint32_t kRefineCoopDefault = 32;

// Enumeration launch shape: at most kEnumWarps warps per block, compiled for
// kEnumMinBlocks resident blocks per SM (which caps registers per thread).
constexpr uint32_t kEnumWarps = 8;
constexpr uint32_t kEnumMinBlocks = 4;

struct BatchOptions {
  uint32_t filter_mode = kFilterDegree | kFilterSignature;
  int refine_iters = 0;
  uint32_t order_mode = kOrderGSI;
  uint32_t chunk = 1;        // tasks per grab
  uint32_t split = 256;      // driver entries per task range
  long long budget_cycles = 4000;     // cycles on a task before it may be split for idle warps
  unsigned long long max_work = 0;  // per-query limit on examined driver entries (0: none)
  uint32_t warps_per_block = kEnumWarps;
  const float* scores = nullptr;  // host scores per query vertex (kOrderScores), batch order
  bool learned = false;           // score with the loaded order network (kOrderScores)
  uint32_t learned_window = 32;   // positions a vertex may move from the heuristic order (32: any)
  uint32_t learned_prefix = 32;   // positions chosen by the network; the rest by the GSI rule (32: all)
  // Refinement classes (refine_classes), when refine_iters > 0: members
  // share one bitmap, a vertex needs as many data neighbours in a query
  // neighbour class as it has query neighbours there, and dominated classes
  // are tested first.  Off: every vertex its own class (per-vertex support,
  // every count one).
  bool classes = true;
  // Single-query batches only: write up to emit_cap embeddings to
  // BatchOutput::rows, and enumerate only pass-0 tasks [task_begin, task_end).
  uint64_t emit_cap = 0;
  uint32_t task_begin = 0, task_end = 0xffffffffu;
  // Single-query batches: report the size of the pass-0 task space in
  // BatchOutput::tasks_total (ordinary launches, not a CUDA graph).
  bool want_tasks = false;
  // Set-intersection strategy of the enumeration (kIsect* in enumerate.cuh)
  // and the refinement's lane/warp split (kRefineCoopDefault).
  uint32_t isect = 0;
  uint32_t refine_coop = kRefineCoopDefault;
  // Run the batch as one CUDA graph (uploads, filter, order, roots, first
  // enumeration pass, results back) when orders are chosen on the device.
  bool use_graph = false;
  // When set, candidate counts are brought to the host after filtering and
  // this function chooses each query's order (the reference-exact orders).
  void (*host_order)(const HostQuery&, const uint32_t* cand, uint32_t* order) = nullptr;
};

struct BatchOutput {
  std::vector<QueryResult> res;
  std::vector<uint32_t> counts;    // candidates per query vertex (batch order)
  std::vector<uint32_t> orders;    // kMaxQ per query
  std::vector<uint32_t> ok;
  float ms_filter = 0, ms_join = 0;
  unsigned long long algo_bytes = 0;  // bytes the enumerator's loads request
  uint32_t passes = 0;                // enumeration passes run
  uint64_t h2d_bytes = 0, d2h_bytes = 0;
  uint32_t launches = 0;
  float ms_enum = 0;
  std::vector<uint32_t> rows;   // emitted embeddings, n per row (emit_cap > 0)
  uint64_t emit_total = 0;      // embeddings found in the task range
  uint32_t tasks_total = 0;     // size of the pass-0 task space (emit_cap > 0 or want_tasks)
  bool graph = false;           // ran as a CUDA graph
};

// Runs filter -> refine -> order -> roots -> enumerate for a batch.
int run_batch(Engine& e, const std::vector<HostQuery>& qs, const BatchOptions& opt, BatchOutput& out);

// All embeddings of one query, handed to sink in chunks of at most
// buffer_rows rows (n caller ids per row, column u = query vertex u).  When
// they do not fit one buffer the pass-0 task space is cut into ranges that
// each fit, each range matched separately.  A non-zero sink return stops.
int run_embeddings(Engine& e, const HostQuery& q, BatchOptions opt, uint64_t buffer_rows,
                   int (*sink)(void*, const uint32_t*, uint64_t, uint32_t), void* user, BatchOutput& first);

// Features of the given queries from host candidate counts and the device
// heuristic order of order_mode (device kernels).
int run_features(Engine& e, const std::vector<HostQuery>& qs, const uint32_t* counts, uint32_t order_mode,
                 float* features);

// Filter (+ refinement) only; flags[n*V] in caller vertex ids, for one query.
int run_filter_probe(Engine& e, const HostQuery& q, uint32_t filter_mode, int refine_iters, bool classes,
                     uint8_t* flags);

// Filter without any allocation: bitmaps in a fixed device array, flags
// written to the caller's device buffer (n * V bytes).
int run_filter_noalloc(Engine& e, const fsig_query& q, uint32_t filter_mode, uint8_t* d_flags);

// Host-side reference orders (plan.cpp).
void gsi_order_host(const HostQuery& q, const uint32_t* cand, uint32_t* order);
void mmatch_order_host(const HostQuery& q, const uint32_t* cand, uint32_t* order);
void mmatch_structure(const HostQuery& q, uint32_t* types, uint32_t* classes);
// Refinement classes and dominated classes of one query (kNoClass: none).
void refine_classes(const HostQuery& q, uint8_t* cls, uint8_t* dom);

}  // namespace fsig
