#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace fsig {

struct TveGraph {
  uint32_t num_vertices = 0;
  std::vector<int32_t> labels;   // -1 for ids without a v record
  std::vector<uint32_t> edges;   // pairs, file order
};

// parallel_from: files of at least this many bytes are parsed with one thread
// per core when every line is a plain record (0: 64 MiB).
int read_tve(const char* path, int is_labeled, TveGraph& g, std::string& err, uint64_t parallel_from = 0);

}  // namespace fsig
