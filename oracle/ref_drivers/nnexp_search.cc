// Test infrastructure only: a program written against the reference's public C++ API that makes
// the same calls, in the same order and with the same arguments, as the reference's command-line
// search (samples/efanna_search.cc:31-64): FIndex over Matrix<float> views with
// KDTreeUbIndexParams(true, 8, 8, 10, 25, 30, 10), loadTrees, loadGraph,
// setSearchParams(epochs, pool, extend, trees, method) -- the method lands in the search_lv slot
// there too -- knnSearch and saveResults.
//
// It is compiled twice: against the reference's headers (`make -C oracle ref`, where the reference
// sources are) and against this library's facade (include/efanna_gb300/efanna.hpp), which has no
// reference sources to read and so also builds where they are absent.  Both builds must write the
// reference's own results file byte for byte on the same trees and graph files.
//
//   nnexp_search data.fvecs trees graph queries.fvecs results.ivecs trees epochs pool extend k [method]
#include <malloc.h>

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>

#include "efanna.hpp"

using namespace efanna;

// fvecs rows into a zero-padded buffer: row stride rounded up to 8 floats, 32-byte aligned (the
// layout Matrix<float> expects under AVX).
static float* read_rows(const char* path, size_t& n, int& dim) {
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    std::cerr << "cannot open " << path << "\n";
    std::exit(2);
  }
  in.read(reinterpret_cast<char*>(&dim), 4);
  in.seekg(0, std::ios::end);
  const size_t bytes = (size_t)in.tellg();
  n = bytes / ((size_t)dim + 1) / 4;
  const size_t stride = ((size_t)dim + 7) / 8 * 8;
  float* rows = static_cast<float*>(memalign(32, n * stride * sizeof(float)));
  std::memset(rows, 0, n * stride * sizeof(float));
  in.seekg(0, std::ios::beg);
  for (size_t i = 0; i < n; ++i) {
    int d = 0;
    in.read(reinterpret_cast<char*>(&d), 4);
    in.read(reinterpret_cast<char*>(rows + i * stride), (std::streamsize)dim * 4);
  }
  return rows;
}

int main(int argc, char** argv) {
  if (argc != 11 && argc != 12) {
    std::cerr << "usage: " << argv[0] << " data trees graph queries results trees epochs pool extend k [method]\n";
    return 1;
  }
  size_t n = 0, nq = 0;
  int dim = 0, qdim = 0;
  float* base_rows = read_rows(argv[1], n, dim);
  float* query_rows = read_rows(argv[4], nq, qdim);
  Matrix<float> base(n, dim, base_rows);
  Matrix<float> queries(nq, qdim, query_rows);
  FIndex<float> index(base, new L2DistanceAVX<float>(), KDTreeUbIndexParams(true, 8, 8, 10, 25, 30, 10));
  index.loadTrees(argv[2]);
  index.loadGraph(argv[3]);
  const int method = argc == 12 ? std::atoi(argv[11]) : 0;
  index.setSearchParams(std::atoi(argv[7]), std::atoi(argv[8]), std::atoi(argv[9]), std::atoi(argv[6]), method);
  index.knnSearch(std::atoi(argv[10]), queries);
  index.saveResults(argv[5]);
  return 0;
}
