// Test infrastructure only: a driver that runs the reference's hashing-seeded searches (HASHINGIndex,
// search method 1: getNeighborsIEH32_nnexp / getNeighborsIEH64_nnexp; method 0: the kgraph search
// getNeighborsIEH32_kgraph / getNeighborsIEH64_kgraph), which have no sample program in the
// reference tree.  Compiled against the reference's headers by
// `make -C oracle ref`; it goes through the public FIndex API as a C++ user of the reference would:
// HASHINGIndexParams, buildIndex (the hash tables), loadGraph, setSearchParams, knnSearch.
//
//   hashing_search data.fvecs graph queries.fvecs base_codes query_codes results.ivecs
//                  codelen tables upbits radius shift epochs pool extend k [method]
//
// base_codes / query_codes are code-file prefixes (files <prefix>_1 ... <prefix>_<tables>).  A graph
// argument of "-" loads no graph: the index then runs its graph-less bucket search (getNeighbors32).
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
  if (argc != 16 && argc != 17) {
    std::cerr << "usage: " << argv[0]
              << " data graph queries base_codes query_codes results codelen tables upbits radius shift"
                 " epochs pool extend k [method]\n";
    return 1;
  }
  size_t n = 0, nq = 0;
  int dim = 0, qdim = 0;
  float* data = read_fvecs_padded(argv[1], n, dim);
  float* qdata = read_fvecs_padded(argv[3], nq, qdim);
  Matrix<float> base(n, dim, data);
  Matrix<float> queries(nq, qdim, qdata);
  char* bcf = argv[4];
  char* qcf = argv[5];
  FIndex<float> index(base, new L2DistanceAVX<float>(),
                      HASHINGIndexParams(std::atoi(argv[7]), std::atoi(argv[8]), std::atoi(argv[9]),
                                         std::atoi(argv[10]), bcf, qcf, std::atoi(argv[11])));
  index.buildIndex();
  if (std::strcmp(argv[2], "-") != 0) index.loadGraph(argv[2]);
  index.setSearchParams(std::atoi(argv[12]), std::atoi(argv[13]), std::atoi(argv[14]), 0, -1,
                        argc == 17 ? std::atoi(argv[16]) : 1);
  index.knnSearch(std::atoi(argv[15]), queries);
  index.saveResults(argv[6]);
  index.outputVisitBucketNum();  // the per-radius histogram of the search (stdout)
  return 0;
}
