// CPU oracle for the FSIG subgraph-matching path.
//
// TEST INFRASTRUCTURE ONLY.  This library is the checker: tests, the smoke
// check and the CPU-baseline leg of the benchmark link it; the product
// (libfsig.so, the CLI, the Python package) never does.
//
// It restates, in plain single-file C++, what the reference computes on the
// path: the t/v/e reader (IO/graph_reader.cc:12-55), the CSR and PCSR
// transforms (graph_format_transformer/graph_format_transformer.cc:12-215),
// the neighbour-label signature (graph_format_transformer.cc:217-281), the two
// candidate filters (match/GSI_kernels.cuh:8-24, match/MMatch_kernels.cuh:6-16)
// and the semantics both matchers enumerate: label-preserving injective
// (non-induced) embeddings, automorphic images counted separately
// (match/GSI_kernels.cuh:199-213, match/MMatch_kernels.cuh:641-654).
//
// Parity status: the reader, CSR, PCSR and signature restatements are pinned
// against the reference's own CPU sources compiled from the reference tree
// (oracle/ref_dump.cc, fixtures in tests/golden/).  Embedding counts are pinned
// by closed-form known-answer tests; the reference's GPU matchers were not run.
#pragma once
#include <cstdint>

#ifdef __cplusplus
extern "C" {
#endif

// ---- plain graph read with the reference reader's semantics ----
// Returns an opaque handle (nullptr on open/format failure).
void* orc_read_tve(const char* path, int is_labeled);
void orc_plain_sizes(void* h, uint32_t* num_vertices, uint32_t* num_edges, int32_t* num_labels,
                     uint64_t* num_adj_entries, uint32_t* min_degree);
// labels[V]; offsets[V+1]; edges[2E] -- the CSR transform (rows sorted, duplicates kept).
void orc_plain_to_csr(void* h, int32_t* labels, uint32_t* offsets, uint32_t* edges);
void orc_free(void* h);

// ---- hashes ----
uint32_t orc_murmur2(const void* key, int len, uint32_t seed);
uint64_t orc_fmix64(uint64_t k);

// ---- signature (16 x u32 per vertex) ----
// Row-major [V][16] when column_oriented == 0, column-major [16][V] otherwise.
void orc_build_signature(uint32_t V, const int32_t* labels, const uint32_t* offsets,
                         const uint32_t* edges, int column_oriented, uint32_t* out);

// ---- PCSR ----
// Sizes first: num_units, then per unit num_keys / num_edges.
uint32_t orc_pcsr_num_units(int32_t num_labels);
int32_t orc_edge_label(int32_t a, int32_t b);
// unit_keys[U], unit_edges[U]: filled.  Returns total words needed for offsets and edges.
void orc_pcsr_sizes(uint32_t V, int32_t num_labels, const int32_t* labels, const uint32_t* offsets,
                    const uint32_t* edges, uint32_t* unit_keys, uint32_t* unit_edges);
// offsets_out: concatenation over units of 32*num_keys words; edges_out: of num_edges words.
void orc_build_pcsr(uint32_t V, int32_t num_labels, const int32_t* labels, const uint32_t* offsets,
                    const uint32_t* edges, uint32_t* offsets_out, uint32_t* edges_out);

// ---- candidate filters: flags[V] in {0,1} ----
void orc_gsi_filter(uint32_t V, const uint32_t* data_sig_rowmajor, const uint32_t* query_sig16,
                    uint8_t* flags);
void orc_mmatch_init(uint32_t V, const int32_t* labels, const uint32_t* offsets, int32_t label,
                     uint32_t degree, uint8_t* flags);

// ---- simple graph (rows sorted, duplicates and self-loops removed) ----
// out_offsets[V+1]; returns the number of entries written to out_edges (<= offsets[V]).
uint64_t orc_simplify(uint32_t V, const uint32_t* offsets, const uint32_t* edges,
                      uint32_t* out_offsets, uint32_t* out_edges);

// ---- candidate refinement (Jacobi iterations of the neighbour-support rule) ----
// cand: n x V flags, in/out.  qadj_mask[u] = bitmask of u's query neighbours.
// classes[u] = u's refinement class (null: every vertex its own class).
void orc_refine(uint32_t V, const int32_t* labels, const uint32_t* offsets, const uint32_t* edges,
                uint32_t n, const uint32_t* qadj_mask, const uint32_t* classes, int iterations, uint8_t* cand);

// ---- matcher ----
// Counts injective label-preserving embeddings of the query (n <= 32 vertices,
// m undirected edges qedges[2m]) into the simple data graph.  order may be null:
// then the order follows GSI::generate_join_order (match/GSI.cu:105-149) over
// label-and-degree candidate counts (results never depend on the order).  level_counts (may be null) receives, per
// depth d in [0,n), the number of partial embeddings of length d+1.
// Returns 0 on success, negative on bad input.
int orc_match(uint32_t V, const int32_t* labels, const uint32_t* offsets, const uint32_t* edges,
              uint32_t n, const int32_t* qlabels, uint32_t m, const uint32_t* qedges,
              const uint32_t* order, int num_threads, uint64_t hash_seed,
              uint64_t* count, uint64_t* hash, uint64_t* level_counts);

// K4 subgraphs of a simple graph (symmetric CSR, no duplicates or
// self-loops) and the number of embeddings of K4 plus a pendant at query
// vertex 0, by the identity 6 * sum over K4s of sum of (deg - 3).
int orc_k4_pendant(uint32_t V, const uint32_t* offsets, const uint32_t* edges, int num_threads, uint64_t* k4,
                   uint64_t* pendant);

#ifdef __cplusplus
}
#endif
