// Drop-in replacement for the reference's efanna.hpp (ZJULearning/efanna): the same namespace,
// classes and signatures -- FIndex<float>, KDTreeUbIndexParams, IndexParams, SearchParams,
// Matrix<T>, Distance<T> and the L2Distance* tags -- over the efanna_gb300 C ABI
// (include/efanna_gb300.h), so code written against the reference compiles unchanged with
// `-I include/efanna_gb300` and links with `-lefanna_gb300`.
//
// Reference interfaces mirrored:
//   FIndex                efanna.hpp:9-75
//   IndexParams / SearchParams / init_algorithm / ValueType / ExtraParamsMap
//                         general/params.hpp:7-42
//   KDTreeUbIndexParams   algorithm/kdtreeub_index.hpp:14-35
//   HASHINGIndexParams    algorithm/hashing_index.hpp:19-46 (the hashing initialiser: its code
//                         files, hash tables and the searches seeded from them: over a loaded
//                         graph method 1 pool/extend and method 0 kgraph, without a graph the
//                         bucket search)
//   Matrix                general/matrix.hpp:12-72
//   Distance, L2Distance, L2DistanceSSE, L2DistanceAVX, L2DistanceAVXr4
//                         general/distance.hpp:46-379 (here plain C++; the GPU computes the
//                         squared L2 itself, the object only names the metric)
// Error behaviour follows the reference: unopenable files print "open file error" and exit with
// the reference's codes, an over-deep merge level prints the reference's message and leaves no
// graph, too many search trees prints "wrong tree number"; other failures throw
// std::runtime_error with efg_last_error().
#ifndef EFANNA_GB300_EFANNA_HPP
#define EFANNA_GB300_EFANNA_HPP

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>
#include <algorithm>

#include "../efanna_gb300.h"

#ifdef __GNUC__
#ifdef __AVX__
#define KGRAPH_MATRIX_ALIGN 32
#else
#ifdef __SSE2__
#define KGRAPH_MATRIX_ALIGN 16
#else
#define KGRAPH_MATRIX_ALIGN 4
#endif
#endif
#endif

namespace efanna {

// ---- distances (general/distance.hpp) ----------------------------------------------------------
template <typename T>
struct Candidate {
  size_t row_id;
  T distance;
  Candidate(const size_t row_id, const T distance) : row_id(row_id), distance(distance) {}
  bool operator>(const Candidate& rhs) const {
    if (this->distance == rhs.distance) return this->row_id > rhs.row_id;
    return this->distance > rhs.distance;
  }
  bool operator<(const Candidate& rhs) const {
    if (this->distance == rhs.distance) return this->row_id < rhs.row_id;
    return this->distance < rhs.distance;
  }
};

template <typename T>
class Distance {
 public:
  virtual T compare(const T* a, const T* b, size_t length) const = 0;
  virtual T norm(const T* a, size_t length) const = 0;
  virtual T dot(const T* a, const T* b, size_t length) const = 0;
  virtual ~Distance() {}
};

// Squared L2 on the host (used by Matrix::brute_force_search and by callers); the index itself
// always measures squared L2 on the GPU whichever of these tags it is given.
template <typename T>
class L2Distance : public Distance<T> {
 public:
  T compare(const T* a, const T* b, size_t size) const {
    T r = T();
    for (size_t i = 0; i < size; ++i) {
      T d = a[i] - b[i];
      r += d * d;
    }
    return r;
  }
  T norm(const T* a, size_t size) const {
    T r = T();
    for (size_t i = 0; i < size; ++i) r += a[i] * a[i];
    return r;
  }
  T dot(const T* a, const T* b, size_t size) const {
    T r = T();
    for (size_t i = 0; i < size; ++i) r += a[i] * b[i];
    return r;
  }
};
template <typename T>
class L2DistanceSSE : public L2Distance<T> {};
template <typename T>
class L2DistanceAVX : public L2Distance<T> {};
template <typename T>
class L2DistanceAVXr4 : public L2Distance<T> {};

// ---- parameters (general/params.hpp, algorithm/kdtreeub_index.hpp:14-35) ------------------------
enum init_algorithm { KDTREE_UB, HASHING };
union ValueType {
  int int_val;
  float float_val;
  char* str_pt;
};
typedef std::map<std::string, ValueType> ExtraParamsMap;
struct IndexParams {
  init_algorithm init_index_type;
  size_t K;
  size_t S;
  size_t L = 30;
  size_t TNS = 10;
  size_t Check_K = 40;
  int build_epoches;
  int extend_num;
  size_t pool_size = 100;
  size_t init_num = 100;
  ExtraParamsMap extra_params;
  bool reverse_nn_used;
};
struct SearchParams {
  int search_init_num;
  int search_epoches;
  int search_method;
  unsigned extend_to;
  unsigned tree_num;
  unsigned search_depth;
};
struct KDTreeUbIndexParams : public IndexParams {
  KDTreeUbIndexParams(bool rnn_used, int tree_num_total, int merge_level = 4, int epoches = 4, int check = 25,
                      int myL = 30, int building_use_k = 10, int tree_num_build = 0, int myS = 10) {
    reverse_nn_used = rnn_used;
    init_index_type = KDTREE_UB;
    K = building_use_k;
    build_epoches = epoches;
    S = myS;
    ValueType v;
    v.int_val = tree_num_total;
    extra_params.insert(std::make_pair("trees", v));
    v.int_val = tree_num_build > 0 ? tree_num_build : tree_num_total;
    extra_params.insert(std::make_pair("treesb", v));
    v.int_val = merge_level;
    extra_params.insert(std::make_pair("ml", v));
    L = myL;
    Check_K = check;
  }
};

struct HASHINGIndexParams : public IndexParams {
  HASHINGIndexParams(int codelen, int TableNum, int UpperBits, int HashRadius, char*& BaseCodeFile,
                     char*& QueryCodeFile, int codelenShift = 0) {
    init_index_type = HASHING;
    ValueType v;
    v.int_val = codelen;
    extra_params.insert(std::make_pair("codelen", v));
    v.int_val = TableNum;
    extra_params.insert(std::make_pair("tablenum", v));
    v.int_val = UpperBits;
    extra_params.insert(std::make_pair("upbits", v));
    v.int_val = HashRadius;
    extra_params.insert(std::make_pair("radius", v));
    v.str_pt = BaseCodeFile;
    extra_params.insert(std::make_pair("bcfile", v));
    v.str_pt = QueryCodeFile;
    extra_params.insert(std::make_pair("qcfile", v));
    v.int_val = codelenShift;
    extra_params.insert(std::make_pair("lenshift", v));
  }
};

// ---- Matrix (general/matrix.hpp): a non-owning row view with the reference's padding rule -------
template <typename T>
class Matrix {
 public:
  Matrix(const size_t rows, const size_t cols, const void* data) : rows_(rows), cols_(cols), data_(data) {
#ifdef __AVX__
    align_cols_ = (cols + 7) / 8 * 8;
#else
#ifdef __SSE2__
    align_cols_ = (cols + 3) / 4 * 4;
#else
    align_cols_ = cols;
#endif
#endif
  }
  size_t get_cols() const { return cols_; }
  size_t get_rows() const { return rows_; }
  size_t get_stride() const { return align_cols_; }
  const T* data() const { return reinterpret_cast<const T*>(data_); }
  const T* get_row(const size_t index) const {
    if (index >= rows_) throw std::runtime_error("index out of range");
    return reinterpret_cast<const T*>(data_) + align_cols_ * index;
  }
  std::vector<std::pair<T, size_t> > brute_force_search(size_t idx, size_t k, Distance<T>* distance) const {
    std::vector<std::pair<T, size_t> > result;
    for (size_t i = 0; i < rows_; i++) result.push_back(std::make_pair(distance->compare(get_row(i), get_row(idx), cols_), i));
    std::partial_sort(result.begin(), result.begin() + k, result.end());
    result.resize(k);
    return result;
  }

 private:
  size_t rows_, cols_, align_cols_;
  const void* data_;
};

// ---- FIndex (efanna.hpp) ------------------------------------------------------------------------
template <typename DataType>
class FIndex {
 public:
  FIndex(const Matrix<DataType>& features, Distance<DataType>* d, const IndexParams& params)
      : index_params_(params), distance_(d), idx_(nullptr) {
    static_assert(sizeof(DataType) == 4, "efanna_gb300 indexes float vectors");
    efg_build_params p;
    efg_default_build_params(&p);
    if (params.init_index_type == HASHING) {
      init_hashing(features, params, p);
      return;
    }
    if (params.init_index_type != KDTREE_UB) throw std::runtime_error("unknown initialisation type");
    p.K = (uint32_t)params.K;
    p.S = (uint32_t)params.S;
    p.L = (uint32_t)params.L;
    p.check_k = (uint32_t)params.Check_K;
    p.epochs = (uint32_t)params.build_epoches;
    p.leaf_size = (uint32_t)params.TNS;
    ExtraParamsMap::const_iterator it = params.extra_params.find("trees");
    p.trees = it != params.extra_params.end() ? (uint32_t)it->second.int_val : 4;
    it = params.extra_params.find("treesb");
    p.trees_build = it != params.extra_params.end() ? (uint32_t)it->second.int_val : p.trees;
    it = params.extra_params.find("ml");
    p.merge_level = it != params.extra_params.end() ? (uint32_t)it->second.int_val : 0;
    check(efg_index_create(reinterpret_cast<const float*>(features.data()), features.get_rows(),
                           (uint32_t)features.get_cols(), features.get_stride(), &p, &idx_));
  }
  virtual ~FIndex() {
    efg_hash_destroy(hash_);
    efg_index_destroy(idx_);
  }

  void buildIndex() {
    if (hashing_) {  // HASHINGIndex::buildIndexImpl: the hash tables (hashing_index.hpp:872-886)
      efg_hash_destroy(hash_);
      hash_ = nullptr;
      check(efg_hash_create(idx_, base_codes_.data(), (uint32_t)tables_, (uint32_t)bits_, (uint32_t)radius_, &hash_));
      return;
    }
    int rc = efg_build_graph(idx_);
    if (rc == EFG_ERR_MERGE_LEVEL) {
      efg_build_stats s;
      efg_get_build_stats(idx_, &s);
      std::cout << "merge level deeper than tree, max merge deepth is" << s.max_merge_depth << std::endl;
      return;
    }
    check(rc);
  }
  void buildTrees() {
    if (!hashing_) check(efg_build_trees(idx_));  // the hashing initialiser has no trees
  }
  void knnSearch(int k, const Matrix<DataType>& query) {
    if (hashing_) {
      hashing_search(k, query);
      return;
    }
    std::vector<int32_t> out((size_t)query.get_rows() * (size_t)k);
    int rc = efg_knn_search(idx_, reinterpret_cast<const float*>(query.data()), query.get_rows(),
                            (uint32_t)query.get_cols(), query.get_stride(), (uint32_t)k, out.data());
    if (rc == EFG_ERR_TREE_COUNT) {
      std::cout << "wrong tree number" << std::endl;
      return;
    }
    check(rc);
  }
  // the hashing index's index, trees and graph writers and index/trees loaders do nothing in the
  // reference (hashing_index.hpp:1628-1655); only its loadGraph reads a file
  void saveIndex(char* filename) {
    if (!hashing_) file(efg_save_index(idx_, filename), -10086);
  }
  void loadIndex(char* filename) {
    if (!hashing_) file(efg_load_index(idx_, filename), -10087);
  }
  void saveTrees(char* filename) {
    if (!hashing_) file(efg_save_trees(idx_, filename), -10086);
  }
  void loadTrees(char* filename) {
    if (!hashing_) file(efg_load_trees(idx_, filename), -10087);
  }
  void saveGraph(char* filename) {
    if (hashing_) return;
    int rc = efg_save_graph(idx_, filename);
    if (rc != EFG_ERR_STATE) file(rc, -10086);  // no graph: the reference writes an empty file
  }
  void loadGraph(char* filename) { file(efg_load_graph(idx_, filename), -10087); }
  void saveResults(char* filename) { file(efg_save_results(idx_, filename), -10086); }
  void setSearchParams(int epochs, int init_num, int extend_to, int search_trees = 0, int search_lv = -1,
                       int search_method = 0) {
    method_ = search_method;
    sp_epochs_ = epochs;
    sp_init_ = init_num;
    sp_extend_ = extend_to > init_num ? init_num : extend_to;
    check(efg_set_search_params(idx_, epochs, init_num, extend_to, search_trees, search_lv, search_method));
  }
  size_t getGraphSize() { return (size_t)efg_graph_size(idx_); }
  std::vector<unsigned> getGraphRow(unsigned row_id) {
    std::vector<unsigned> row;
    int64_t len = efg_graph_row(idx_, row_id, nullptr, 0);
    if (len > 0) {
      row.resize((size_t)len);
      efg_graph_row(idx_, row_id, reinterpret_cast<uint32_t*>(row.data()), (uint64_t)len);
    }
    return row;
  }
  // The hashing index's histogram of the last search (hashing_index.hpp:1618-1626, counted at
  // :1133-1143): per radius, the masks it holds and the queries whose pool filled within it
  // (a pool that filled at the first mask of the next radius counts for the smaller one, as in
  // the reference), then the queries whose pool the Hamming ball could not fill.  Recomputed here
  // on the host from the codes; the KD-tree index prints nothing, as in the reference.
  void outputVisitBucketNum() {
    if (!hashing_ || !last_nq_) return;
    if (vb_maps_.empty()) {
      const size_t n = base_codes_.size() / (size_t)tables_;
      vb_maps_.resize((size_t)tables_);
      for (int h = 0; h < tables_; ++h)
        for (size_t i = 0; i < n; ++i) vb_maps_[(size_t)h][base_codes_[(size_t)h * n + i]].push_back((uint32_t)i);
    }
    const size_t n = base_codes_.size() / (size_t)tables_;
    std::vector<uint64_t> masks(1, 0);
    std::vector<uint64_t> radius_end(1, 1);  // HammingRadius
    std::vector<int> pos;
    for (int r = 1; r <= radius_; ++r) {
      pos.assign((size_t)r, 0);
      for (int t = 0; t < r; ++t) pos[(size_t)t] = t;
      for (;;) {
        uint64_t m = 0;
        for (int t = 0; t < r; ++t) m |= 1ull << pos[(size_t)t];
        masks.push_back(m);
        int t = r - 1;
        while (t >= 0 && pos[(size_t)t] == bits_ - r + t) --t;
        if (t < 0) break;
        ++pos[(size_t)t];
        for (int u = t + 1; u < r; ++u) pos[(size_t)u] = pos[(size_t)u - 1] + 1;
      }
      radius_end.push_back(masks.size());
    }
    std::vector<unsigned> visit((size_t)radius_ + 2, 0);
    std::vector<uint32_t> stamp(n, 0);
    const size_t nq = last_nq_;
    for (size_t q = 0; q < nq; ++q) {
      unsigned p = 0;
      size_t j = 0;
      for (; j < masks.size(); ++j) {
        for (int h = 0; h < tables_ && p < last_pool_; ++h) {
          auto it = vb_maps_[(size_t)h].find(query_codes_[(size_t)h * nq + q] ^ masks[j]);
          if (it == vb_maps_[(size_t)h].end()) continue;
          for (size_t e = 0; e < it->second.size() && p < last_pool_; ++e) {
            uint32_t id = it->second[e];
            if (stamp[id] == (uint32_t)q + 1) continue;
            stamp[id] = (uint32_t)q + 1;
            ++p;
          }
        }
        if (p >= last_pool_) break;
      }
      if (p < last_pool_) {
        ++visit[(size_t)radius_ + 1];
      } else {
        for (int r = 0; r <= radius_; ++r)
          if (j <= radius_end[(size_t)r]) {
            ++visit[(size_t)r];
            break;
          }
      }
    }
    std::cout << "Radius 0 bucket num: " << radius_end[0] << " points num: " << visit[0] << std::endl;
    size_t i = 1;
    for (; i < radius_end.size(); ++i)
      std::cout << "Radius " << i << " bucket num: " << radius_end[i] - radius_end[i - 1]
                << " points num: " << visit[i] << std::endl;
    std::cout << "Radius larger, points num: " << visit[i] << std::endl;
  }

 private:
  static void check(int rc) {
    if (rc != EFG_OK) throw std::runtime_error(std::string("efanna_gb300: ") + efg_last_error());
  }
  static void file(int rc, int exit_code) {
    if (rc == EFG_ERR_OPEN) {
      std::cout << "open file error" << std::endl;
      std::exit(exit_code);
    }
    if (rc == EFG_ERR_FORMAT) {
      std::cout << efg_last_error() << std::endl;
      std::exit(-11);
    }
    check(rc);
  }
  // HASHINGIndex's constructor (hashing_index.hpp:66-198): parameters, the radius limit per code
  // length, and the base and query code files read at construction.
  void init_hashing(const Matrix<DataType>& features, const IndexParams& params, efg_build_params& p) {
    hashing_ = true;
    auto get = [&](const char* key) -> const ValueType* {
      ExtraParamsMap::const_iterator it = params.extra_params.find(key);
      return it == params.extra_params.end() ? nullptr : &it->second;
    };
    const ValueType *len = get("codelen"), *tab = get("tablenum"), *up = get("upbits"), *rad = get("radius"),
                    *bcf = get("bcfile"), *qcf = get("qcfile"), *sh = get("lenshift");
    if (!len || !tab || !up || !rad || !bcf || !qcf)
      throw std::runtime_error("HASHINGIndexParams: code length, tables, upper bits, radius and code files are required");
    int codelen = len->int_val, shift = sh ? sh->int_val : 0;
    tables_ = tab->int_val;
    if (codelen > 64 || codelen < 1) throw std::runtime_error("code length not supported yet!");
    if (tables_ < 1) throw std::runtime_error("Total hash table num error!");
    if (codelen - shift <= 0) throw std::runtime_error("lenShift error: could not be larger than the code length!");
    if (up->int_val >= codelen - shift) throw std::runtime_error("upbits should be smaller than the actual codelength!");
    int actual = codelen - shift;
    int cap = actual <= 32 ? 13 : actual <= 36 ? 11 : actual <= 40 ? 10 : actual <= 48 ? 9 : actual <= 60 ? 8 : 7;
    radius_ = std::min(rad->int_val, cap);
    int file_len = 0;
    base_codes_ = load_codes(bcf->str_pt, codelen, shift, features.get_rows(), file_len);
    query_codes_ = load_codes(qcf->str_pt, codelen, shift, 0, file_len);
    bits_ = file_len - shift;  // the files' code length, as the reference's loader takes it
    if (bits_ < 1 || bits_ > 64) throw std::runtime_error("code length not supported yet!");
    if (radius_ > bits_) radius_ = bits_;
    check(efg_index_create(reinterpret_cast<const float*>(features.data()), features.get_rows(),
                           (uint32_t)features.get_cols(), features.get_stride(), &p, &idx_));
  }
  // LoadCode32 / LoadCode64 (hashing_index.hpp:206-300): files <prefix>_1 .. <prefix>_<tables>, each
  // int32 1, int32 code length, int32 count, then count codes of 32 (code length <= 32) or 64 bits,
  // shifted right by the shift and bounded by codelen - shift bits.  Returns tables x count codes.
  std::vector<uint64_t> load_codes(const char* prefix, int codelen, int shift, size_t expect, int& file_len) {
    std::vector<uint64_t> all;
    size_t count = 0;
    const uint64_t maxv = codelen - shift >= 64 ? ~0ull : (1ull << (codelen - shift)) - 1;
    for (int t = 0; t < tables_; ++t) {
      std::string path = std::string(prefix) + "_" + std::to_string(t + 1);
      std::ifstream in(path.c_str(), std::ios::binary);
      if (!in.is_open()) throw std::runtime_error("open file " + path + " error");
      int head[3] = {0, 0, 0};
      in.read(reinterpret_cast<char*>(head), sizeof(head));
      if (!in || head[0] != 1 || head[2] < 0) throw std::runtime_error("codefile " + path + " error!");
      file_len = head[1];
      if (t == 0) count = (size_t)head[2];
      if ((size_t)head[2] != count || (expect && count != expect))
        throw std::runtime_error("codefile " + path + ": wrong number of codes");
      for (size_t i = 0; i < count; ++i) {
        uint64_t c = 0;
        if (codelen <= 32) {
          uint32_t w = 0;
          in.read(reinterpret_cast<char*>(&w), 4);
          c = w;
        } else {
          in.read(reinterpret_cast<char*>(&c), 8);
        }
        if (!in) throw std::runtime_error("codefile " + path + " truncated");
        c >>= shift;
        if (c > maxv) throw std::runtime_error("codefile " + path + " error! Exceed maximum value");
        all.push_back(c);
      }
    }
    return all;
  }
  void hashing_search(int k, const Matrix<DataType>& query) {
    if (efg_graph_size(idx_) != 0 && method_ != 0 && method_ != 1) {
      std::cout << "no such searching method" << std::endl;
      return;
    }
    if (!hash_) throw std::runtime_error("buildIndex() builds the hash tables before searching");
    const size_t nq = query.get_rows();
    if (query_codes_.size() != nq * (size_t)tables_)
      throw std::runtime_error("the query code files hold a different number of queries");
    std::vector<int32_t> out(nq * (size_t)k);
    // the pool size this search fills (the kgraph search raises the stored size to epochs *
    // extend_to first, as the reference does) -- kept for outputVisitBucketNum
    unsigned pool = (unsigned)sp_init_;
    if (efg_graph_size(idx_) != 0 && method_ == 0 && (unsigned)(sp_epochs_ * sp_extend_) >= pool) {
      pool = (unsigned)(sp_epochs_ * sp_extend_);
      sp_init_ = (int)pool;
    }
    check(efg_hash_search(idx_, hash_, reinterpret_cast<const float*>(query.data()), nq, (uint32_t)query.get_cols(),
                          query.get_stride(), query_codes_.data(), (uint32_t)k, out.data()));
    last_nq_ = nq;
    last_pool_ = pool;
  }

  IndexParams index_params_;
  Distance<DataType>* distance_;
  efg_index* idx_ = nullptr;
  efg_hash* hash_ = nullptr;
  bool hashing_ = false;
  int method_ = 0, tables_ = 0, bits_ = 0, radius_ = 0;
  int sp_epochs_ = 0, sp_init_ = 0, sp_extend_ = 0;
  size_t last_nq_ = 0;
  unsigned last_pool_ = 0;
  std::vector<uint64_t> base_codes_, query_codes_;
  std::vector<std::unordered_map<uint64_t, std::vector<uint32_t> > > vb_maps_;
};

}  // namespace efanna
#endif
