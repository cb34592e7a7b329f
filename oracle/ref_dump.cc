// Test-infrastructure driver linked against the reference's own sources (see
// oracle/build.py).  It runs the reference's CPU-side code paths and prints
// their outputs as text, for the parity fixtures under tests/golden/:
//
//   ref_dump csr   <graph> <labeled>        reader + CSR transform
//   ref_dump pcsr  <graph> <labeled>        reader + PCSR transform
//   ref_dump sig   <graph> <labeled> <col>  reader + build_signature
//   ref_dump gsiorder <query> <labeled> <c0> <c1> ...      GSI::generate_join_order
//   ref_dump mmorder  <query> <labeled> <c0> <c1> ...      MMatch decomposition, classes, order
//
// Only host code of the reference runs; no kernel is launched.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "IO/graph_reader.h"
#include "graph/graph.h"
#include "graph_format_transformer/graph_format_transformer.h"
#include "match/GSI.h"
#include "match/MMatch.h"
#include "utility/inverted_index.h"

static UndirectedPlainGraph* read_plain(const char* path, bool labeled) {
  Graph* g = nullptr;
  UndirectedSurveyPlainReader reader;
  reader.read(path, g, labeled);
  return dynamic_cast<UndirectedPlainGraph*>(g);
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: ref_dump mode file labeled [...]\n");
    return 2;
  }
  const std::string mode = argv[1];
  const bool labeled = std::atoi(argv[3]) != 0;
  UndirectedPlainGraph* pg = read_plain(argv[2], labeled);
  if (!pg) return 3;
  if (mode == "csr") {
    Graph* out = nullptr;
    UndirectedPlainToCSRTransformer t;
    std::printf("@plain %u %u %d %u\n", pg->num_vertices(), pg->num_edges(), pg->num_labels(), pg->min_degree);
    t.transform(pg, out);
    auto* c = dynamic_cast<UndirectedCSRGraph*>(out);
    std::printf("@labels");
    for (Vertex i = 0; i < c->num_vertices(); i++) std::printf(" %d", c->labels_[i]);
    std::printf("\n@offsets");
    for (Vertex i = 0; i <= c->num_vertices(); i++) std::printf(" %u", c->offset_[i]);
    std::printf("\n@edges");
    for (Edge i = 0; i < 2 * c->num_edges(); i++) std::printf(" %u", c->edges_[i]);
    std::printf("\n");
  } else if (mode == "pcsr") {
    Graph* out = nullptr;
    UndirectedPlainToPCSRTransformer t;
    t.transform(pg, out);
    auto* p = dynamic_cast<UndirectedPCSRGraph*>(out);
    std::printf("@units %u\n", p->num_units_);
    for (Vertex u = 0; u < p->num_units_; u++) {
      PCSRUnit* x = p->units_[u];
      std::printf("@unit %u %u %u\n@offset", u, x->num_keys_, x->num_edges_);
      for (Vertex i = 0; i < 32 * x->num_keys_; i++) std::printf(" %u", x->offset_[i]);
      std::printf("\n@uedges");
      for (Vertex i = 0; i < x->num_edges_; i++) std::printf(" %u", x->edges_[i]);
      std::printf("\n");
    }
  } else if (mode == "sig") {
    const bool col = argc > 4 && std::atoi(argv[4]) != 0;
    // The CLI sorts the rows (transform) before building signatures
    // (main/run.cc:111, 134-135); the signature does not depend on row order.
    Vertex* table = nullptr;
    UndirectedPlainToPCSRTransformer::build_signature(col, table, pg);
    std::printf("@sig");
    for (Vertex i = 0; i < 16 * pg->num_vertices(); i++) std::printf(" %u", table[i]);
    std::printf("\n");
  } else if (mode == "gsiorder" || mode == "mmorder") {
    const Vertex n = pg->num_vertices();
    if (argc < 4 + int(n)) return 4;
    std::vector<unsigned> cnt(n);
    for (Vertex i = 0; i < n; i++) cnt[i] = unsigned(std::strtoul(argv[4 + i], nullptr, 10));
    if (mode == "gsiorder") {
      UndirectedPCSRGraph* data = new UndirectedPCSRGraph();
      GSI m(pg, data, nullptr, nullptr, nullptr, 0);
      m.size_candidate_sets_ = new unsigned[n];
      for (Vertex i = 0; i < n; i++) m.size_candidate_sets_[i] = cnt[i];
      m.id_to_pos_ = new Vertex[n];
      m.pos_to_id_ = new Vertex[n];
      m.generate_join_order();
      std::printf("@order");
      for (Vertex i = 0; i < n; i++) std::printf(" %u", m.pos_to_id_[i]);
      std::printf("\n");
    } else {
      UndirectedCSRGraph* data = new UndirectedCSRGraph();
      data->labels_ = nullptr;
      data->offset_ = nullptr;
      data->edges_ = nullptr;
      MMatch m(pg, data, nullptr, 0);
      m.decompose_query_graph();
      m.generate_refine_plan();
      m.num_candidates_array_ = new unsigned[m.num_equivalent_classes_];
      for (Vertex c = 0; c < m.num_equivalent_classes_; c++) m.num_candidates_array_[c] = cnt[m.equivalent_classes_[c][0]];
      m.generate_join_order();
      std::printf("@types");
      for (Vertex i = 0; i < n; i++) std::printf(" %u", m.query_vertex_type_[i]);
      std::printf("\n@classes");
      for (Vertex i = 0; i < n; i++) std::printf(" %u", m.inversed_classes_[i].first);
      std::printf("\n@order");
      for (Vertex i = 0; i < n; i++) std::printf(" %u", m.join_order_[i]);
      std::printf("\n");
    }
  } else {
    return 5;
  }
  return 0;
}
