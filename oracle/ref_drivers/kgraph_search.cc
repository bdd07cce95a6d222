// Test infrastructure only: a driver that runs the reference's kgraph search (search method 1),
// which its own command-line programs cannot reach (they pass the method in the search_lv slot).
// Compiled against the reference's headers by `make -C oracle ref`; it goes through the public
// FIndex API exactly as a C++ user of the reference would.
//
//   kgraph_search data.fvecs trees graph queries.fvecs results.ivecs trees epochs pool extend k [calls]
//
// With calls = 2 the search runs twice on the same index and results.ivecs.2 receives the second
// call's ids (the first call may enlarge the stored pool size, kdtreeub_index.hpp:510-514).
#include <malloc.h>

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "efanna.hpp"

using namespace efanna;

// fvecs rows into a zero-padded buffer: row stride rounded up to 8 floats, 32-byte aligned (the
// layout Matrix<float> expects under AVX).
static float* read_fvecs_padded(const char* path, size_t& n, int& dim) {
  std::ifstream in(path, std::ios::binary);
  if (!in) {
    std::cerr << "cannot open " << path << "\n";
    std::exit(2);
  }
  in.read(reinterpret_cast<char*>(&dim), 4);
  in.seekg(0, std::ios::end);
  size_t bytes = (size_t)in.tellg();
  n = bytes / ((size_t)dim + 1) / 4;
  size_t stride = ((size_t)dim + 7) / 8 * 8;
  float* buf = static_cast<float*>(memalign(32, n * stride * sizeof(float)));
  std::memset(buf, 0, n * stride * sizeof(float));
  in.seekg(0, std::ios::beg);
  for (size_t i = 0; i < n; ++i) {
    int d = 0;
    in.read(reinterpret_cast<char*>(&d), 4);
    in.read(reinterpret_cast<char*>(buf + i * stride), (std::streamsize)dim * 4);
  }
  return buf;
}

int main(int argc, char** argv) {
  if (argc != 11 && argc != 12) {
    std::cerr << "usage: " << argv[0]
              << " data trees graph queries results trees epochs pool extend k [calls]\n";
    return 1;
  }
  size_t n = 0, nq = 0;
  int dim = 0, qdim = 0;
  float* data = read_fvecs_padded(argv[1], n, dim);
  float* qdata = read_fvecs_padded(argv[4], nq, qdim);
  Matrix<float> base(n, dim, data);
  Matrix<float> queries(nq, qdim, qdata);
  FIndex<float> index(base, new L2DistanceAVX<float>(), KDTreeUbIndexParams(true, 8, 8, 10, 25, 30, 10));
  index.loadTrees(argv[2]);
  index.loadGraph(argv[3]);
  index.setSearchParams(std::atoi(argv[7]), std::atoi(argv[8]), std::atoi(argv[9]), std::atoi(argv[6]), -1, 1);
  int calls = argc == 12 ? std::atoi(argv[11]) : 1;
  int k = std::atoi(argv[10]);
  index.knnSearch(k, queries);
  index.saveResults(argv[5]);
  if (calls > 1) {
    index.knnSearch(k, queries);
    std::string second = std::string(argv[5]) + ".2";
    index.saveResults(&second[0]);  // saveResults takes a char*
  }
  return 0;
}
