// The reference's own ingest (main/run.cc:72-111: UndirectedSurveyPlainReader,
// UndirectedPlainToCSRTransformer) feeding the engine through FsigMatcher.
//   adapter_main <data graph> <query graph> [algo 1|2|3] [labeled 0|1] [device]
// Exit status: 0 matched, 2 the engine reported an error.
#include <cstdlib>
#include <string>

#include "IO/graph_reader.h"
#include "fsig_matcher.h"
#include "graph_format_transformer/graph_format_transformer.h"

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cout << "usage: adapter_main data query [algo] [labeled] [device]" << std::endl;
    return 1;
  }
  const int algo = argc > 3 ? std::atoi(argv[3]) : FSIG_ALGO_FSIG;
  const bool labeled = argc > 4 ? std::atoi(argv[4]) != 0 : true;
  const int dev = argc > 5 ? std::atoi(argv[5]) : 0;
  Graph* data = nullptr;
  Graph* query = nullptr;
  UndirectedSurveyPlainReader reader;
  reader.read(argv[1], data, labeled);
  reader.read(argv[2], query, labeled);
  auto* plain_data = dynamic_cast<UndirectedPlainGraph*>(data);
  auto* plain_query = dynamic_cast<UndirectedPlainGraph*>(query);
  if (!plain_data || !plain_query) return 1;
  UndirectedPlainToCSRTransformer to_csr;
  Graph* csr = nullptr;
  to_csr.transform(plain_data, csr);
  auto* csr_data = dynamic_cast<UndirectedCSRGraph*>(csr);
  if (!csr_data) return 1;
  FsigMatcher matcher(plain_query, csr_data, algo, dev);
  GPUSubgraphMatcher* m = &matcher;  // used through the reference's interface
  m->match();
  return matcher.status() == FSIG_OK ? 0 : 2;
}
