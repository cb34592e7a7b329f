/* Synthetic workload generators and the t/v/e writer (host C ABI).
 *
 * The reference ships no datasets, so seeded synthetic graphs and random-walk
 * queries stand in for them.  None of these entry points has a counterpart in
 * the reference; fsig_write_tve emits the format the reference reads
 * (README.md:24-35, IO/graph_reader.cc:12-55), with no trailing newline so the
 * reference reader does not duplicate the last record.
 *
 * All functions return 0 on success and a negative FSIG_GEN_E* code on error.
 */
#ifndef FSIG_GEN_H
#define FSIG_GEN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSIG_GEN_EINVAL (-1)
#define FSIG_GEN_ENOMEM (-2)
#define FSIG_GEN_EIO (-3)
#define FSIG_GEN_EGIVEUP (-4)

/* Query extraction modes. */
#define FSIG_QUERY_INDUCED 0 /* induced subgraph on a random walk's vertex set */
#define FSIG_QUERY_DENSE 1   /* greedy walk, induced, average degree > 3 (n = 4: > 2.25) */
#define FSIG_QUERY_SPARSE 2  /* the walk's own edges, average degree <= 3        */

/* R-MAT (a, b, c, d = 1-a-b-c) over V vertices: edges[2E] receives exactly E
 * distinct undirected edges without self-loops, the first E distinct ones of a
 * seeded candidate stream (endpoints >= V are resampled). */
int fsig_gen_rmat(uint32_t V, uint64_t E, double a, double b, double c, uint64_t seed,
                  int threads, uint32_t* edges);

/* Chung-Lu: expected degree of vertex i proportional to (i+1)^(-1/(gamma-1)),
 * capped at sqrt(2E); E distinct undirected edges without self-loops. */
int fsig_gen_chung_lu(uint32_t V, uint64_t E, double gamma, uint64_t seed, int threads,
                      uint32_t* edges);

/* Labels in [0, L): uniform, or Zipf with exponent s (P(k) ~ 1/(k+1)^s). */
int fsig_gen_labels_uniform(uint32_t V, uint32_t L, uint64_t seed, int32_t* labels);
int fsig_gen_labels_zipf(uint32_t V, uint32_t L, double s, uint64_t seed, int32_t* labels);

/* Build a CSR (rows sorted, duplicates and self-loops dropped) from an edge
 * list; offsets[V+1], adj[2E].  Returns the number of adjacency entries in
 * *num_adj. */
int fsig_gen_csr(uint32_t V, uint64_t E, const uint32_t* edges, uint32_t* offsets, uint32_t* adj,
                 uint64_t* num_adj);

/* Extract one connected query of n vertices (2 <= n <= 32) from the data
 * graph by random walk.  qlabels[n]; qedges[2*n*(n-1)/2] max; *m edges;
 * src[n] = the data vertex each query vertex was taken from (the identity
 * embedding).  Returns FSIG_GEN_EGIVEUP when no walk met the mode's density
 * rule within the attempt budget. */
int fsig_gen_query(uint32_t V, const uint32_t* offsets, const uint32_t* adj, const int32_t* labels,
                   uint32_t n, int mode, uint64_t seed, int32_t* qlabels, uint32_t* qedges,
                   uint32_t* m, uint32_t* src);

/* As fsig_gen_query, with the walk confined to data vertices whose label is
 * at least min_label (with Zipf labels: the less frequent ones). */
int fsig_gen_query_ex(uint32_t V, const uint32_t* offsets, const uint32_t* adj, const int32_t* labels,
                      uint32_t n, int mode, uint64_t seed, int32_t min_label, int32_t* qlabels,
                      uint32_t* qedges, uint32_t* m, uint32_t* src);

/* Write a graph in t/v/e form: "t V E", one "v id label degree" per vertex,
 * one "e u v" per edge, no trailing newline. */
int fsig_write_tve(const char* path, uint32_t V, const int32_t* labels, uint64_t E,
                   const uint32_t* edges);

#ifdef __cplusplus
}
#endif
#endif /* FSIG_GEN_H */
