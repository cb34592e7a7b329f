// The FSIG command line, on the C ABI (include/fsig.h):
//
//   FSIG <data graph> <query graph> [algorithm 1|2|3] [graph type 0|1] [output file] [device]
//
// Same arguments and defaults as the reference's main/run.cc:28-64 (algorithm
// 1 = FSIG, 2 = GSI; graph type 0 = unlabeled; device 0).  Prints the phase
// times in the reference's TimeRecorder format (utility/time_recorder.h:54),
// the embedding count as MMatch (match/MMatch.cu:2047, "#embedding: N") or
// GSI (match/GSI.cu:280, "#embeddings: N") prints it, and the set hash.  The
// reference never writes its output file (its EmbeddingWriter is a stub); here
// the embeddings are written to it, one per line in query-vertex order, when
// it is named on the command line.  Algorithm 3 is the fused filter of both.
// Errors print a message and return non-zero instead of exit(0).
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "fsig.h"

namespace {

double ms_since(std::chrono::steady_clock::time_point t) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

int fail(fsig_engine* e, const char* what, int rc) {
  std::printf("Error: %s: %s (%s)\n", what, fsig_status_string(rc), fsig_last_error(e));
  return 1;
}

}  // namespace

int main(int argc, const char* argv[]) {
  if (argc < 3) {
    std::printf("invalid arguments!\n");
    std::printf("usage: %s <data graph> <query graph> [algorithm 1|2|3] [graph type 0|1] [output file] [device]\n",
                argv[0]);
    return -1;
  }
  const char* data_file = argv[1];
  const char* query_file = argv[2];
  const int algo = argc >= 4 ? std::atoi(argv[3]) : 1;
  const int is_labeled = (argc >= 5 && std::atoi(argv[4]) == 0) ? 0 : 1;
  const char* out_file = argc >= 6 ? argv[5] : nullptr;
  const int dev = argc >= 7 ? std::atoi(argv[6]) : 0;
  if (algo < 1 || algo > 3) {
    std::printf("invalid arguments! algorithm must be 1, 2 or 3\n");
    return -1;
  }

  auto t = std::chrono::steady_clock::now();
  fsig_graph_file* data = nullptr;
  int rc = fsig_read_graph_file(data_file, is_labeled, &data);
  if (rc) return fail(nullptr, data_file, rc);
  const double t_read_data = ms_since(t);

  t = std::chrono::steady_clock::now();
  fsig_graph_file* query = nullptr;
  rc = fsig_read_graph_file(query_file, is_labeled, &query);
  if (rc) return fail(nullptr, query_file, rc);
  const double t_read_query = ms_since(t);

  fsig_engine* e = nullptr;
  rc = fsig_create(dev, 0, &e);
  if (rc) return fail(nullptr, "fsig_create", rc);

  t = std::chrono::steady_clock::now();
  uint32_t V = 0;
  uint64_t E = 0;
  const int32_t* labels = nullptr;
  const uint32_t* edges = nullptr;
  fsig_graph_file_data(data, &V, &labels, &E, &edges);
  for (uint32_t v = 0; v < V; v++)
    if (labels[v] < 0) {
      std::printf("Error: data vertex %u has no v record\n", v);
      return 1;
    }
  rc = fsig_load_graph(e, V, labels, E, edges);
  if (rc) return fail(e, "organise graph", rc);
  const double t_organise = ms_since(t);
  fsig_free_graph_file(data);

  std::printf("time cost(read data): %gms\n", t_read_data);
  std::printf("time cost(read query): %gms\n", t_read_query);
  std::printf("time cost(organise graph): %gms\n", t_organise);

  uint32_t n = 0;
  uint64_t m = 0;
  const int32_t* qlabels = nullptr;
  const uint32_t* qedges = nullptr;
  fsig_graph_file_data(query, &n, &qlabels, &m, &qedges);
  for (uint32_t u = 0; u < n; u++)
    if (qlabels[u] < 0) {
      std::printf("Error: query vertex %u has no v record\n", u);
      return 1;
    }
  fsig_query q{n, uint32_t(m), qlabels, qedges, nullptr};
  fsig_result r{};
  t = std::chrono::steady_clock::now();
  rc = out_file ? fsig_write_embeddings(e, &q, algo, out_file, &r) : fsig_match(e, &q, algo, &r);
  if (rc) return fail(e, "match", rc);
  const double t_match = ms_since(t);
  std::printf("%s: %" PRIu64 "\n", algo == 2 ? "#embeddings" : "#embedding", r.count);
  std::printf("hash: 0x%016" PRIx64 "\n", r.hash);
  std::printf("time cost(filter): %gms\n", double(r.ms_filter));
  std::printf("time cost(join): %gms\n", double(r.ms_join));
  std::printf("time cost(match): %gms\n", t_match);
  fsig_free_graph_file(query);
  fsig_destroy(e);
  return 0;
}
