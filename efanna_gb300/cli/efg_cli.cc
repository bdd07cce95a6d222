// Command-line front ends with the argv shapes of the reference's sample programs, written
// against the drop-in FIndex facade (include/efanna_gb300/efanna.hpp).  One binary; the tool is
// chosen by the name it is invoked as (or by its first argument):
//
//   efanna_index_buildgraph data.fvecs out.graph trees level epoch L K kNN S
//       (samples/efanna_index_buildgraph.cc:30-59)
//   efanna_index_buildtrees data.fvecs out.trees trees          (samples/efanna_index_buildtrees.cc:29-49)
//   efanna_index_buildall   data.fvecs out.graph out.trees trees level epoch L K kNN S
//       (samples/efanna_index_buildall.cc:28-62)
//   efanna_search base.fvecs in.trees in.graph query.fvecs out.ivecs trees epoch pool extend k [method]
//       (samples/efanna_search.cc:31-66; the method lands in search_lv as in the reference)
//   evaluate result.ivecs groundtruth.ivecs k                   (samples/evaluate.cc:24-64)
//
// Rows are read into buffers padded to the facade Matrix's stride.
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <vector>

#include "efanna.hpp"

using namespace efanna;

namespace {

size_t padded(size_t dim) {
#ifdef __AVX__
  return (dim + 7) / 8 * 8;
#else
#ifdef __SSE2__
  return (dim + 3) / 4 * 4;
#else
  return dim;
#endif
#endif
}

// fvecs -> rows padded to the Matrix stride; returns false when the file cannot be opened.
bool read_fvecs(const char* path, std::vector<float>& data, size_t& num, int& dim) {
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) return false;
  in.read((char*)&dim, 4);
  in.seekg(0, std::ios::end);
  size_t fsize = (size_t)in.tellg();
  num = fsize / (dim + 1) / 4;
  size_t cols = padded(dim);
  data.assign(num * cols, 0.0f);
  in.seekg(0, std::ios::beg);
  for (size_t i = 0; i < num; i++) {
    in.seekg(4, std::ios::cur);
    in.read((char*)(data.data() + i * cols), dim * 4);
  }
  return true;
}

bool read_ivecs(const char* path, std::vector<int>& data, int& num, int& dim) {
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) return false;
  in.read((char*)&dim, 4);
  in.seekg(0, std::ios::end);
  size_t fsize = (size_t)in.tellg();
  num = (int)(fsize / (dim + 1) / 4);
  data.assign((size_t)num * dim, 0);
  in.seekg(0, std::ios::beg);
  for (int i = 0; i < num; i++) {
    in.seekg(4, std::ios::cur);
    in.read((char*)(data.data() + (size_t)i * dim), dim * 4);
  }
  return true;
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int buildgraph(int argc, char** argv, bool all) {
  int need = all ? 11 : 10;
  if (argc != need) {
    std::cout << argv[0] << (all ? " data_file save_graph_file save_trees_file" : " data_file save_graph_file")
              << " trees level epoch L K kNN S" << std::endl;
    return -1;
  }
  std::vector<float> data;
  size_t num;
  int dim;
  if (!read_fvecs(argv[1], data, num, dim)) {
    std::cout << "open file error" << std::endl;
    return -1;
  }
  std::cout << "data dimension: " << dim << std::endl;
  int o = all ? 4 : 3;
  int trees = atoi(argv[o]), mlevel = atoi(argv[o + 1]), epochs = atoi(argv[o + 2]), L = atoi(argv[o + 3]),
      checkK = atoi(argv[o + 4]), kNN = atoi(argv[o + 5]), S = atoi(argv[o + 6]);
  Matrix<float> dataset(num, dim, data.data());
  FIndex<float> index(dataset, new L2DistanceAVX<float>(),
                      KDTreeUbIndexParams(true, trees, mlevel, epochs, checkK, L, kNN, trees, S));
  double t0 = now_s();
  index.buildIndex();
  std::cout << (now_s() - t0) << std::endl;
  index.saveGraph(argv[2]);
  if (all) index.saveTrees(argv[3]);
  return 0;
}

int buildtrees(int argc, char** argv) {
  if (argc != 4) {
    std::cout << argv[0] << " data_file save_trees_file trees" << std::endl;
    return -1;
  }
  std::vector<float> data;
  size_t num;
  int dim;
  if (!read_fvecs(argv[1], data, num, dim)) {
    std::cout << "open file error" << std::endl;
    return -1;
  }
  Matrix<float> dataset(num, dim, data.data());
  FIndex<float> index(dataset, new L2DistanceAVX<float>(),
                      KDTreeUbIndexParams(true, atoi(argv[3]), 8, 8, 25, 30, 10, 8, 10));
  double t0 = now_s();
  index.buildTrees();
  std::cout << "Index building time : " << (now_s() - t0) << " seconds" << std::endl;
  index.saveTrees(argv[2]);
  return 0;
}

int search(int argc, char** argv) {
  if (argc != 11 && argc != 12) {
    std::cout << argv[0]
              << " data_file tree_index graph_index query_file result_file tree epoch initsz extend querNN "
                 "search_method(optional)"
              << std::endl;
    return -1;
  }
  std::vector<float> data, queries;
  size_t num, qnum;
  int dim, qdim;
  if (!read_fvecs(argv[1], data, num, dim) || !read_fvecs(argv[4], queries, qnum, qdim)) {
    std::cout << "open file error" << std::endl;
    return -1;
  }
  Matrix<float> dataset(num, dim, data.data());
  Matrix<float> query(qnum, qdim, queries.data());
  FIndex<float> index(dataset, new L2DistanceAVX<float>(), KDTreeUbIndexParams(true, 8, 8, 10, 25, 30, 10));
  index.loadTrees(argv[2]);
  index.loadGraph(argv[3]);
  int method = argc == 12 ? atoi(argv[11]) : 0;
  // the reference passes the method into the search_lv slot (samples/efanna_search.cc:54)
  index.setSearchParams(atoi(argv[7]), atoi(argv[8]), atoi(argv[9]), atoi(argv[6]), method);
  double t0 = now_s();
  index.knnSearch(atoi(argv[10]), query);
  std::cout << (now_s() - t0) << std::endl;
  index.saveResults(argv[5]);
  return 0;
}

int evaluate(int argc, char** argv) {
  if (argc != 4) {
    std::cout << argv[0] << " resultfile gound_truth kNN" << std::endl;
    return -1;
  }
  std::vector<int> res, gt;
  int p1, p2, d1, d2;
  if (!read_ivecs(argv[1], res, p1, d1) || !read_ivecs(argv[2], gt, p2, d2)) {
    std::cout << "open file error" << std::endl;
    return -1;
  }
  if (p1 != p2) {
    std::cout << "result file and groundtruth don't match" << std::endl;
    return -1;
  }
  int k = atoi(argv[3]);
  if (k > d1) {
    std::cout << "result file not enough for k=" << k << std::endl;
    return -1;
  }
  for (int i = 0; i < p1; i++) {
    std::set<int> s(res.begin() + (size_t)i * d1, res.begin() + (size_t)i * d1 + k);
    if ((int)s.size() < k) std::cout << "query " << i << " result index not unique!" << std::endl;
  }
  long miss = 0;
  for (int i = 0; i < p1; i++) {
    for (int j = 0; j < k; j++) {
      int v = res[(size_t)i * d1 + j], m = 0;
      for (; m < k; m++)
        if (v == gt[(size_t)i * d2 + m]) break;
      if (m == k) miss++;
    }
  }
  std::cout << k << "NN accuracy: " << 1 - (float)miss / ((float)p1 * k) << std::endl;
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::string name = argv[0];
  size_t sl = name.find_last_of('/');
  if (sl != std::string::npos) name = name.substr(sl + 1);
  if (name == "efg_cli" && argc > 1) {  // efg_cli <tool> args...
    name = argv[1];
    ++argv;
    --argc;
  }
  try {
    if (name == "efanna_index_buildgraph") return buildgraph(argc, argv, false);
    if (name == "efanna_index_buildall") return buildgraph(argc, argv, true);
    if (name == "efanna_index_buildtrees") return buildtrees(argc, argv);
    if (name == "efanna_search") return search(argc, argv);
    if (name == "evaluate") return evaluate(argc, argv);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 2;
  }
  std::cerr << "usage: efg_cli {efanna_index_buildgraph|efanna_index_buildtrees|efanna_index_buildall|"
               "efanna_search|evaluate} args..."
            << std::endl;
  return 1;
}
