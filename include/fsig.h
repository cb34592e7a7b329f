/* FSIG-GB300: C ABI of the subgraph-matching engine (libfsig.so).
 *
 * This is the drop-in boundary for the reference's matching path.  Each entry
 * point names the reference interface it replaces.  Conventions:
 *   - opaque handles; every function returns an int status (FSIG_OK == 0,
 *     negative on error) and never exits the process;
 *   - the caller owns every host buffer; the engine owns one device arena;
 *   - one engine per host thread (engines are independent; a single engine is
 *     not safe to call from two threads at once);
 *   - the engine runs only on the GPU: there is no CPU fallback.  A process
 *     without a usable sm_103 device gets FSIG_ENODEV from fsig_create.
 *
 * Matching semantics (both algorithms, as in the reference): an embedding is
 * an injective map f from query vertices to data vertices with
 * label(f(u)) == label(u) and (u,w) in E(q) => (f(u),f(w)) in E(G); it is
 * non-induced and automorphic images count separately
 * (match/GSI_kernels.cuh:199-213, match/MMatch_kernels.cuh:641-654).  The data
 * graph is matched as a simple graph: duplicate edges and self-loops are
 * collapsed when it is loaded.
 *
 * Result hash: h(f) = fmix64(FSIG_HASH_SEED + sum_u fmix64((u << 32) | f(u)))
 * with fmix64 the MurmurHash3 64-bit finaliser; the set hash is the sum of
 * h(f) over all embeddings, modulo 2^64.  It does not depend on the order in
 * which embeddings are found.
 */
#ifndef FSIG_H
#define FSIG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSIG_HASH_SEED 0x46534947b3000001ull
#define FSIG_MAX_QUERY 32

/* status codes */
#define FSIG_OK 0
#define FSIG_EINVAL (-1)        /* bad argument                                  */
#define FSIG_ENODEV (-2)        /* no usable CUDA device                         */
#define FSIG_ECUDA (-3)         /* a CUDA call failed (see fsig_last_error)      */
#define FSIG_EADMISSION (-4)    /* request does not fit the device arena         */
#define FSIG_ENOGRAPH (-5)      /* no data graph loaded                          */
#define FSIG_EQUERY (-6)        /* query too large, disconnected or malformed    */
#define FSIG_EIO (-7)           /* file could not be read or parsed              */
#define FSIG_ETIMEOUT (-8)      /* a bounded device wait gave up                 */
#define FSIG_EOVERFLOW (-9)     /* a device work queue overflowed                */
#define FSIG_ELIMIT (-10)       /* the query exceeded its work limit              */

/* algorithms (argv[3] of the reference CLI, main/run.cc:31) */
#define FSIG_ALGO_FSIG 1  /* label+degree filter, neighbour-support refinement, core/forest/leaf order (MMatch) */
#define FSIG_ALGO_GSI 2   /* label+signature filter, candidate-count order with 0.9 decay (GSI)                  */
#define FSIG_ALGO_FUSED 3 /* all filters + refinement, candidate-count order                                      */

/* segment index of the resident graph store (fsig_set_segment_index) */
#define FSIG_SEGMENTS_AUTO 0  /* TABLE when it takes at most 4 words per adjacency entry, else ROWS */
#define FSIG_SEGMENTS_TABLE 1 /* dense table of every row's label-segment starts, V x (L+1) words,
                                 plus the caller id of every adjacency entry: one load per lookup  */
#define FSIG_SEGMENTS_ROWS 2  /* no table: a segment is found by binary search in its row, a
                                 leaf's caller id by one lookup once it survives                    */

/* order sources */
#define FSIG_ORDER_HEURISTIC 0 /* the algorithm's own order                         */
#define FSIG_ORDER_LEARNED 1   /* the loaded order-scoring network (fsig_mpnn_*)    */
#define FSIG_ORDER_GIVEN 2     /* fsig_query.order                                   */

typedef struct fsig_engine fsig_engine;

/* A query graph: n <= 32 vertices, m undirected edges (pairs of vertex ids). */
typedef struct {
  uint32_t num_vertices;
  uint32_t num_edges;
  const int32_t* labels;  /* [num_vertices]   */
  const uint32_t* edges;  /* [2 * num_edges]  */
  const uint32_t* order;  /* [num_vertices] or NULL; used with FSIG_ORDER_GIVEN */
} fsig_query;

typedef struct {
  uint64_t count;                       /* number of embeddings (exact, 64-bit)        */
  uint64_t hash;                        /* order-independent set hash                   */
  int32_t status;                       /* FSIG_OK or the query's own error             */
  uint32_t num_vertices;
  uint32_t order[FSIG_MAX_QUERY];       /* matching order used (query vertex ids)      */
  uint32_t candidates[FSIG_MAX_QUERY];  /* |C(u)| after filtering, by query vertex id   */
  uint64_t level_counts[FSIG_MAX_QUERY];/* partial embeddings of length d+1, d=0..n-1   */
  float ms_filter;                      /* device time: filter + refinement            */
  float ms_join;                        /* device time: enumeration                    */
  uint64_t work;                        /* driver entries examined (when max_work set)  */
} fsig_result;

typedef struct {
  int algo;            /* FSIG_ALGO_*                                     */
  int order_source;    /* FSIG_ORDER_*                                    */
  int refine_iters;    /* neighbour-support refinement steps (-1: default) */
  int use_graph;       /* capture/replay the batch as one CUDA graph       */
  uint32_t chunk;      /* tasks taken per warp grab (0: default)                  */
  uint32_t split_len;  /* driver entries per task range (0: default)              */
  uint64_t split_cycles; /* SM cycles on one task before its unexplored frontier
                            is handed to idle warps (0: default)                   */
  uint64_t max_work;     /* per-query limit on driver entries examined (all
                            depths); a query over it stops with status
                            FSIG_ELIMIT.  The outcome does not depend on
                            scheduling: it is set iff the query's total work
                            under its order exceeds the limit (0: no limit)     */
  uint32_t warps_per_block; /* enumeration block size in warps, 1..8 (0: default 8) */
  uint32_t learned_window;  /* FSIG_ORDER_LEARNED: positions a vertex may move away
                               from the heuristic order (0: any)                 */
  uint32_t no_classes;      /* 1: filter and refine every query vertex on its own,
                               with every neighbour count one; 0 (default):
                               refinement classes (see fsig_refine_classes)      */
  uint32_t isect;           /* set-intersection strategy of the enumeration:
                               0 (default) every lane binary-searches the
                               segments alone, two in lockstep; 1 warp-
                               cooperative 32-ary window search (galloping-
                               like); 2 adaptive: the 32 entries after a
                               segment's cursor first (merge-like), else the
                               window search; 3 the tile search when the
                               segment's rest fits 32 entries, else a lane's
                               own binary search                          */
  uint32_t refine_coop;     /* refinement: a candidate's neighbour segment
                               longer than this is scanned by the whole warp
                               (warp per candidate), shorter ones by the
                               candidate's own lane (0: default 32;
                               0xffffffff: always a lane)                    */
  uint32_t learned_prefix;  /* FSIG_ORDER_LEARNED: the network chooses the first
                               this many positions, the heuristic rule (GSI's:
                               candidate count, 0.9 per placed neighbour)
                               continues from them (0: all positions)        */
} fsig_batch_opts;

/* ---- engine lifetime; replaces GPUSubgraphMatcher::init_GPU (match/subgraph_match.h:51-80)
 *      and MemoryManager (memory_manager/memory_manager.h:16-265): one device arena of
 *      arena_bytes (0 = a quarter of the device's memory), admission-checked. ---- */
int fsig_create(int device, uint64_t arena_bytes, fsig_engine** out);
int fsig_destroy(fsig_engine* e);
const char* fsig_last_error(const fsig_engine* e);
const char* fsig_status_string(int status);

/* ---- data graph; replaces GraphReader::read (IO/graph_reader.h:27-34) followed by
 *      GraphFormatTransformer::transform (graph_format_transformer/graph_format_transformer.h:37-40)
 *      and MMatch::copy_graph_to_GPU (match/MMatch.cu:14-32).  The CSR, the
 *      label-partitioned adjacency and the signature table are built on the device.
 *      Labels are 0..4095 (more distinct labels: FSIG_EINVAL). ---- */
int fsig_load_graph(fsig_engine* e, uint32_t num_vertices, const int32_t* labels,
                    uint64_t num_edges, const uint32_t* edges);
/* Reads a t/v/e file with the reference reader's semantics (graph_reader.cc:12-55);
 * is_labeled == 0 sets every label to 0 (argv[4] of main/run.cc:32). */
int fsig_load_graph_file(fsig_engine* e, const char* path, int is_labeled);
int fsig_graph_info(const fsig_engine* e, uint32_t* num_vertices, uint64_t* num_adj,
                    int32_t* num_labels, uint32_t* max_degree);
/* Segment index (FSIG_SEGMENTS_*) of the graphs the engine builds from now on
 * (fsig_load_graph, fsig_load_graph_file; a cache keeps the index it was
 * saved with).  Results do not depend on it.  The dense table costs
 * 4 V (L+1) + 4 x adjacency bytes; without it a graph of many labels fits in
 * about half the memory of its adjacency and signatures, and lookups cost
 * two binary searches in a row.  Replaces nothing in the reference, whose
 * PCSR units are sized per label pair (graph_format_transformer.cc:39-215). */
int fsig_set_segment_index(fsig_engine* e, int mode);
/* The resident store's index (FSIG_SEGMENTS_TABLE or _ROWS) and its device
 * bytes (every array kept for matching). */
int fsig_graph_layout(const fsig_engine* e, int* segment_index, uint64_t* store_bytes);

/* Binary cache of the resident graph store (the device arrays as built: the
 * renumbered CSR, caller ids, label segments and signatures), in place of the
 * reference's commented-out binary PCSR dump (graph_format_transformer.cc:47-74,
 * 197-213): a load is a file read and copies, no parsing or building.  A
 * load replaces the resident graph; when it fails no graph is resident. */
int fsig_save_graph_cache(fsig_engine* e, const char* path);
int fsig_load_graph_cache(fsig_engine* e, const char* path);

/* ---- host reader; replaces UndirectedSurveyPlainReader::read (IO/graph_reader.cc:12-55)
 *      for callers that want the parsed graph itself (query files, the CLI).
 *      The handle owns labels[num_vertices] (-1 for ids without a v record) and
 *      edges[2 * num_edges] (file order, duplicates kept). ---- */
typedef struct fsig_graph_file fsig_graph_file;
int fsig_read_graph_file(const char* path, int is_labeled, fsig_graph_file** out);
/* The same, parsing with one thread per core from parallel_min_bytes of file
 * size on (0: 64 MiB) when every line is blank or one plain v/e record; the
 * result is always the sequential reading's. */
int fsig_read_graph_file_threads(const char* path, int is_labeled, uint64_t parallel_min_bytes, fsig_graph_file** out);
int fsig_graph_file_data(const fsig_graph_file* f, uint32_t* num_vertices, const int32_t** labels,
                         uint64_t* num_edges, const uint32_t** edges);
void fsig_free_graph_file(fsig_graph_file* f);

/* ---- matching; replaces GPUSubgraphMatcher::match (match/subgraph_match.h:46),
 *      i.e. MMatch::match (match/MMatch.cu:2077-2121, algo 1) and GSI::match
 *      (match/GSI.cu:329-358, algo 2), for one query. ---- */
int fsig_match(fsig_engine* e, const fsig_query* q, int algo, fsig_result* out);
/* ---- one query over a range of its root tasks; the block split of
 *      MMatch::extend_embeddings_recursively (match/MMatch.cu:1834-1985,
 *      memory_manager.h:220-242) cuts the work of one query into pieces too,
 *      there to bound memory.  The task space of a query is its root
 *      candidates in ascending order, each root's first-level driver range in
 *      chunks of split_len entries (0: 256; at least 32), under the
 *      algorithm's heuristic order (or q->order).  The call enumerates tasks
 *      [task_begin, task_end) (task_end may exceed the space) and returns their
 *      count and set hash in out (level_counts likewise); *tasks_total
 *      receives the size of the space.  Results of ranges that partition
 *      [0, tasks_total) add up (counts exactly, hashes modulo 2^64) to the
 *      query's, so a query can be split across calls, processes or GPUs. ---- */
int fsig_match_range(fsig_engine* e, const fsig_query* q, int algo, uint32_t split_len, uint32_t task_begin,
                     uint32_t task_end, fsig_result* out, uint32_t* tasks_total);
/* Many queries against the resident data graph in one persistent launch.
 * With order_source FSIG_ORDER_LEARNED, a query that carries an order
 * (fsig_query.order) keeps it; the others are ordered by the network. */
int fsig_match_batch(fsig_engine* e, uint32_t num_queries, const fsig_query* qs,
                     const fsig_batch_opts* opts, fsig_result* out);

/* ---- embeddings; the output the reference's EmbeddingWriter::write
 *      (IO/embedding_writer.h:12-20, an empty stub there) was meant to produce.
 *      sink receives rows[num_rows * width]: one embedding per row, column u =
 *      the data vertex (caller id) matched to query vertex u.  Rows come in
 *      chunks of at most buffer_rows (0: 2^20); a non-zero return stops.  When
 *      a query has more embeddings than one buffer holds, its root tasks are
 *      cut into ranges matched one after the other.  out gets the count and
 *      hash of the whole set, as fsig_match. ---- */
typedef int (*fsig_embedding_sink)(void* user, const uint32_t* rows, uint64_t num_rows, uint32_t width);
int fsig_match_embeddings(fsig_engine* e, const fsig_query* q, int algo, uint64_t buffer_rows,
                          fsig_embedding_sink sink, void* user, fsig_result* out);
/* PlainEmbeddingWriter: the embeddings as text, one per line, the data ids of
 * query vertices 0..n-1 separated by spaces. */
int fsig_write_embeddings(fsig_engine* e, const fsig_query* q, int algo, const char* path, fsig_result* out);

/* ---- order-scoring network (no counterpart in the reference, which orders by
 *      the heuristics of match/GSI.cu:105-149 and match/MMatch.cu:1575-1641).
 *      A 3-layer message-passing network over the query graph, hidden 64, BF16
 *      weights and activations with FP32 accumulation, scoring each query
 *      vertex from 8 features; FSIG_ORDER_LEARNED orders by lowest score among
 *      the frontier.  Graphs are passed as node offsets (graph g has nodes
 *      [node_offsets[g], node_offsets[g+1]), at most 32), 8 features per node
 *      and a neighbour bitmask per node (local ids).  Parameters are FP32, in
 *      the layout documented in fsig_gb300/csrc/mpnn.h. ---- */
uint32_t fsig_mpnn_param_count(void);
int fsig_mpnn_set_params(fsig_engine* e, const float* params, uint32_t count);
int fsig_mpnn_get_params(fsig_engine* e, float* params, uint32_t count);
/* Features of each query vertex given its candidate count (candidates[] in
 * query order, vertex order), computed on the device as the batched path does:
 * position in algo's heuristic order/(n-1), degree/8, plog2(candidates)/20,
 * plog2(label class size)/20, candidates/class size, signature bits/16, n/32,
 * mean plog2 of neighbours' candidates/20, where plog2(x) = e + x/2^e - 1,
 * e = floor(log2 x).  features[8 * total vertices]. */
int fsig_mpnn_features(fsig_engine* e, uint32_t num_queries, const fsig_query* qs, int algo,
                       const uint32_t* candidates, float* features);
int fsig_mpnn_forward(fsig_engine* e, uint32_t num_graphs, const uint32_t* node_offsets, const float* features,
                      const uint32_t* neighbours, float* scores);
/* One training step on the mean squared error against targets: loss, the
 * gradients (grads may be NULL) and, when lr > 0, an Adam update. */
int fsig_mpnn_train_step(fsig_engine* e, uint32_t num_graphs, const uint32_t* node_offsets, const float* features,
                         const uint32_t* neighbours, const float* targets, float lr, float* loss, float* grads);

/* ---- statistics of the engine's last fsig_match / fsig_match_batch call ----
 * (no reference counterpart: the reference prints phase timings with its
 * TimeRecorder, utility/time_recorder.h:26-57) */
typedef struct {
  uint64_t h2d_bytes;        /* host-to-device bytes copied for the call        */
  uint64_t d2h_bytes;        /* device-to-host bytes copied back                */
  uint64_t enum_bytes;       /* bytes the enumeration kernel's loads requested  */
  uint32_t kernel_launches;  /* libfsig kernels launched by the call             */
  uint32_t enum_passes;      /* enumeration kernel launches (work-splitting passes) */
  float ms_filter;           /* device time, filter + refinement + counts       */
  float ms_join;             /* device time, ordering + roots + enumeration     */
  float ms_enum;             /* device time of the enumeration kernel launches
                                (-1 when a graph launch left it unmeasurable)  */
  uint32_t graph;            /* 1 when the batch ran as one CUDA graph          */
  uint64_t enum_tasks;       /* tasks run by the enumeration kernel             */
  uint64_t enum_pops;        /* handed-off records taken within the same pass   */
  uint64_t enum_handoffs;    /* frontier hand-offs                              */
  uint64_t enum_records;     /* task records written by hand-offs               */
  uint64_t enum_examines;    /* 32-entry driver chunks examined                 */
} fsig_batch_stats;
int fsig_last_stats(const fsig_engine* e, fsig_batch_stats* out);

/* ---- bounded waits of the enumeration's work queue (no reference counterpart:
 *      the reference has no device work queue and ends the process on any
 *      failure, e.g. memory_manager/memory_manager.h:31-61).  A warp that took
 *      a handed-off record waits at most ready_wait_ns for it to be published,
 *      then records FSIG_ETIMEOUT for the call and leaves (0: 200 ms); an idle
 *      warp waits at most idle_wait_ns for hand-offs before it leaves, its
 *      share of the queue then running in a later pass (0: 2 s).  unpublished
 *      = 1 is fault injection for tests: the first record handed off in each
 *      enumeration pass of later calls is written but never published, so the
 *      warp that takes it waits out ready_wait_ns and the call returns
 *      FSIG_ETIMEOUT without faulting the GPU; 0 turns it off.  Waits are
 *      limited to 60 s. ---- */
int fsig_set_queue_waits(fsig_engine* e, uint64_t ready_wait_ns, uint64_t idle_wait_ns, int unpublished);

/* ---- transforms with the reference's output layout, built on the device ---- */
/* UndirectedPlainToCSRTransformer::transform (graph_format_transformer.cc:12-37):
 * offsets[V+1], adj[2E]; rows ascending, duplicate edges kept as the reference keeps them. */
int fsig_build_csr(fsig_engine* e, uint32_t num_vertices, uint64_t num_edges,
                   const uint32_t* edges, uint32_t* offsets, uint32_t* adj);
/* UndirectedPlainToPCSRTransformer::build_signature (graph_format_transformer.cc:217-281)
 * over a CSR: 16 words per vertex; column-major [16][V] when column_oriented != 0. */
int fsig_build_signature(fsig_engine* e, uint32_t num_vertices, const int32_t* labels,
                         const uint32_t* offsets, const uint32_t* adj, int column_oriented,
                         uint32_t* signature);
/* UndirectedPlainToPCSRTransformer::transform (graph_format_transformer.cc:39-215)
 * over a CSR with labels in [0, num_labels): U = num_labels (num_labels + 1) / 2
 * units (get_edge_label, graph/graph.h:107-122); unit_keys[U] and unit_edges[U]
 * give each unit's keys and list entries.  When table and edges are given they
 * receive every unit's 32-word slot table (32 x keys words) and its lists,
 * units concatenated in order.  Computed on the device; call once with
 * table = edges = NULL for the sizes. */
int fsig_build_pcsr(fsig_engine* e, uint32_t num_vertices, int32_t num_labels, const int32_t* labels,
                    const uint32_t* offsets, const uint32_t* adj, uint32_t* unit_keys, uint32_t* unit_edges,
                    uint32_t* table, uint32_t* edges);

/* ---- join order on the host, no device work; replaces GSI::generate_join_order
 *      (match/GSI.cu:105-149, algo 2 and 3) and MMatch::decompose_query_graph +
 *      find_equivalent_classes + generate_join_order (match/MMatch.cu:543-607,
 *      44-173, 1575-1641, algo 1), with the reference's priority-queue
 *      tie-breaking.  candidates[n] are the per-vertex candidate counts.
 *      vertex_types (2 core, 1 forest, 0 leaf) and classes (equivalence class
 *      per vertex) may be NULL; they are filled for algo 1 only. ---- */
int fsig_plan_order(const fsig_query* q, int algo, const uint32_t* candidates, uint32_t* order,
                    uint32_t* vertex_types, uint32_t* classes);

/* ---- refinement classes of a query, no device work; the classes of
 *      MMatch::find_equivalent_classes (match/MMatch.cu:44-173) as the coarsest
 *      partition that keeps apart vertices of different label, degree or
 *      signature and in which members of a class have as many neighbours as
 *      each other in every class.  Members share one candidate bitmap; a
 *      vertex keeps candidate v only while v has at least k data neighbours
 *      in C(y) for each class y holding k of its query neighbours (the
 *      thresholds of MMatch's refine plan, match/MMatch.cu:317-541).
 *      classes[u] = the smallest member of u's class.  dominated[u] (for the
 *      smallest member of a class, else FSIG_NO_CLASS): a class whose every
 *      condition is implied by u's, so C(u) stays within it and the
 *      refinement tests it first (MMatch's optimised operators); FSIG_NO_CLASS
 *      when there is none.  Either output may be NULL. ---- */
#define FSIG_NO_CLASS 0xffu
int fsig_refine_classes(const fsig_query* q, uint32_t* classes, uint32_t* dominated);

/* ---- candidate filter probe: signature_filter (match/GSI.cu:34-103) and
 *      kernel_initialise + refinement (match/MMatch.cu:609-1227) on the loaded graph.
 *      flags[n * V] (1 = candidate), in the caller's vertex ids.  fsig_filter
 *      refines with refinement classes; fsig_filter_classes chooses
 *      (classes = 0: every vertex its own class, every neighbour count one). ---- */
int fsig_filter(fsig_engine* e, const fsig_query* q, int algo, int refine_iters, uint8_t* flags);
int fsig_filter_classes(fsig_engine* e, const fsig_query* q, int algo, int refine_iters, int classes,
                        uint8_t* flags);

/* ---- candidate filter that allocates nothing (no counterpart in the reference).
 *      For callers that cannot allocate device memory when they filter: a
 *      process whose device memory is all handed to its own pool allocator,
 *      or code on a latency-critical path that cannot accept the device-wide
 *      synchronisation cudaFree implies.  Same result as fsig_filter with
 *      refine_iters = 0 (no refinement), written to the caller's DEVICE buffer
 *      d_flags[n * V] (1 = candidate, caller vertex ids); the call clears it
 *      first.  The candidate bitmaps live in a fixed device array of 2^21
 *      words (8 MiB) that every GPU loading the library holds until exit; a
 *      query whose bitmaps need more returns FSIG_EADMISSION and leaves
 *      d_flags untouched.  Every graph fsig_load_graph accepts (up to 4096
 *      labels) fits its label table.  All calls share
 *      the array: calls whose work overlaps on the GPU race.  The first call
 *      on a device looks up the array's address and should come before any
 *      stream capture.  Synchronous: the flags are complete on return. ---- */
int fsig_filter_noalloc(fsig_engine* e, const fsig_query* q, int algo, uint8_t* d_flags);

#ifdef __cplusplus
}
#endif
#endif /* FSIG_H */
