// FsigMatcher: the reference's matcher interface (GPUSubgraphMatcher,
// match/subgraph_match.h:39-81) implemented on libfsig's C ABI, the adapter a
// maintainer adds next to match/MMatch.h.  It takes the graphs the reference's
// own pipeline builds (main/run.cc:72-138): the query as an
// UndirectedPlainGraph, the data graph as an UndirectedCSRGraph
// (graph/graph.h:50-85), and prints the count line MMatch prints
// (match/MMatch.cu:2047) or GSI's (match/GSI.cu:280), plus the set hash.
// Unlike the reference it reports failures instead of exiting.
#ifndef FSIG_MATCHER_H
#define FSIG_MATCHER_H

#include <cstdint>
#include <iostream>
#include <vector>

#include "fsig.h"
#include "match/subgraph_match.h"

class FsigMatcher : public GPUSubgraphMatcher {
 public:
  FsigMatcher(UndirectedPlainGraph* query, UndirectedCSRGraph* data, int algo, int dev_id)
      : GPUSubgraphMatcher(query, data), algo_(algo) {
    status_ = fsig_create(dev_id, 0, &eng_);
    if (status_ != FSIG_OK) return;
    // CSR rows -> each undirected edge once (the engine collapses the
    // duplicates the reference's CSR keeps)
    std::vector<uint32_t> e;
    for (Vertex v = 0; v < data->num_vertices(); v++)
      for (Edge k = data->offset_[v]; k < data->offset_[v + 1]; k++)
        if (v < data->edges_[k]) {
          e.push_back(v);
          e.push_back(data->edges_[k]);
        }
    status_ = fsig_load_graph(eng_, data->num_vertices(), data->labels_, e.size() / 2, e.data());
  }
  ~FsigMatcher() {
    if (eng_) fsig_destroy(eng_);
  }

  void match() override {
    if (status_ != FSIG_OK) {
      std::cout << "Error: " << (eng_ ? fsig_last_error(eng_) : fsig_status_string(status_)) << std::endl;
      return;
    }
    auto* q = dynamic_cast<UndirectedPlainGraph*>(query_graph_);
    std::vector<uint32_t> qe;
    for (Vertex u = 0; u < q->num_vertices(); u++)
      for (Vertex w : q->edges_[u])
        if (u < w) {
          qe.push_back(u);
          qe.push_back(w);
        }
    fsig_query fq{q->num_vertices(), uint32_t(qe.size() / 2), q->labels_.data(), qe.data(), nullptr};
    status_ = fsig_match(eng_, &fq, algo_, &result_);
    if (status_ != FSIG_OK) {
      std::cout << "Error: " << fsig_last_error(eng_) << std::endl;
      return;
    }
    std::cout << (algo_ == FSIG_ALGO_GSI ? "#embeddings: " : "#embedding: ") << result_.count << std::endl;
    std::cout << "hash: 0x" << std::hex << result_.hash << std::dec << std::endl;
  }

  int status() const { return status_; }
  const fsig_result& result() const { return result_; }

 private:
  fsig_engine* eng_ = nullptr;
  int algo_;
  int status_ = FSIG_OK;
  fsig_result result_{};
};

#endif
