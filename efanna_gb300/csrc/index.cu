#include <algorithm>
// efg_index lifecycle, parameters, file formats and the C ABI front door.
//
// The file formats are the reference's (ZJULearning/efanna):
//   graph   per row: u32 k, k x u32 id                       (kdtreeub_index.hpp:243-312)
//   trees   header u32 K, u32 trees, u64 N, u64 dim; per tree i32 node_num, i32 node_size(48),
//           node_num post-order 40-byte records {i32 DivDim, f32 DivVal, u64 Start, u64 End,
//           u64 Lchild, u64 Rchild}; then trees x N u32 leaf lists (kdtreeub_index.hpp:139-242)
//   index   trees file followed by N x K i32 graph ids        (kdtreeub_index.hpp:701-825)
//   results ivecs                                             (base_index.hpp:136-151)
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "internal.cuh"

namespace efg {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

static int check_params(const efg_build_params* p, uint64_t n) {
  if (!p) return fail(EFG_ERR_ARG, "null build params");
  if (p->S < 1 || p->S > 16) return fail(EFG_ERR_ARG, "S must be in [1, 16]");
  if (p->L < p->S || p->L > 255) return fail(EFG_ERR_ARG, "L must be in [S, 255]");
  if (p->K < 1 || p->K > p->L) return fail(EFG_ERR_ARG, "K must be in [1, L]");
  if (p->trees < 1 || p->trees > 1024) return fail(EFG_ERR_ARG, "trees must be in [1, 1024]");
  if (p->trees_build > p->trees) return fail(EFG_ERR_ARG, "trees_build must be <= trees");
  if (p->leaf_size < 1) return fail(EFG_ERR_ARG, "leaf_size must be >= 1");
  if (p->reverse_cap < 1 || p->reverse_cap > 4096) return fail(EFG_ERR_ARG, "reverse_cap must be in [1, 4096]");
  if (n < 2 * (uint64_t)p->S + 2) return fail(EFG_ERR_ARG, "need at least 2*S+2 points");
  if (n >= (1ULL << 30)) return fail(EFG_ERR_ARG, "at most 2^30 - 1 points");
  return EFG_OK;
}

static int make_index(uint64_t n, uint32_t dim, const efg_build_params* params, efg_index** out) {
  if (!out) return fail(EFG_ERR_ARG, "null output handle");
  *out = nullptr;
  if (n == 0 || dim == 0) return fail(EFG_ERR_ARG, "empty data");
  efg_build_params p;
  if (params) p = *params;
  else efg_default_build_params(&p);
  if (p.trees_build == 0) p.trees_build = p.trees;
  EFG_TRY(check_params(&p, n));
  efg_index* idx = new efg_index();
  idx->n = n;
  idx->dim = dim;
  idx->ld = (uint32_t)round_up(dim, 4);
  idx->bp = p;
  idx->sp.search_trees = (int)p.trees;  // SP.tree_num = TreeNum (kdtreeub_index.hpp:59)
  cudaError_t e = cudaMalloc((void**)&idx->d_base, n * idx->ld * sizeof(float));
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete idx;
    return fail(EFG_ERR_NOMEM, std::string("cannot allocate base vectors: ") + cudaGetErrorString(e));
  }
  e = cudaMemset(idx->d_base, 0, n * idx->ld * sizeof(float));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&idx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cudaFree(idx->d_base);
    delete idx;
    return fail(EFG_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = idx;
  return EFG_OK;
}

// ---- trees file ------------------------------------------------------------------------------
static void write_post(std::ofstream& out, const std::vector<HNode>& nodes, int32_t ni, int& cnt) {
  // Iterative post-order (trees can be deep).
  std::vector<std::pair<int32_t, int>> st{{ni, 0}};
  while (!st.empty()) {
    auto& top = st.back();
    const HNode& nd = nodes[top.first];
    if (nd.left >= 0 && top.second == 0) {
      top.second = 1;
      st.push_back({nd.left, 0});
      continue;
    }
    if (nd.right >= 0 && top.second == 1) {
      top.second = 2;
      st.push_back({nd.right, 0});
      continue;
    }
    int dd = nd.div_dim;
    float dv = nd.div_val;
    uint64_t s = nd.start, e = nd.end;
    uint64_t lp = nd.left >= 0 ? 1 : 0, rp = nd.right >= 0 ? 1 : 0;
    out.write((const char*)&dd, 4);
    out.write((const char*)&dv, 4);
    out.write((const char*)&s, 8);
    out.write((const char*)&e, 8);
    out.write((const char*)&lp, 8);
    out.write((const char*)&rp, 8);
    ++cnt;
    st.pop_back();
  }
}

static int write_trees(efg_index* idx, std::ofstream& out) {
  std::vector<HNode> nodes;
  std::vector<uint32_t> leaves;
  EFG_TRY(download_forest(idx, nodes, leaves));
  uint32_t K = idx->bp.K, tn = idx->forest.ntrees;
  uint64_t num = idx->n, dim = idx->dim;
  out.write((const char*)&K, 4);
  out.write((const char*)&tn, 4);
  out.write((const char*)&num, 8);
  out.write((const char*)&dim, 8);
  for (uint32_t t = 0; t < tn; ++t) {
    std::streampos pos = out.tellp();
    int zero = 0, nsz = 48;
    out.write((const char*)&zero, 4);
    out.write((const char*)&nsz, 4);
    int cnt = 0;
    write_post(out, nodes, idx->forest.roots[t], cnt);
    std::streampos endp = out.tellp();
    out.seekp(pos);
    out.write((const char*)&cnt, 4);
    out.seekp(endp);
  }
  out.write((const char*)leaves.data(), (std::streamsize)(leaves.size() * 4));
  return out.good() ? EFG_OK : fail(EFG_ERR_OPEN, "write failed");
}

// Reads the trees section; DepthFirstBuildTree's stack merge (kdtreeub_index.hpp:672-700) links
// the post-order records back into trees.
static int read_trees(efg_index* idx, std::ifstream& in, uint32_t* K_out) {
  uint32_t K, tn;
  uint64_t num, dim;
  in.read((char*)&K, 4);
  in.read((char*)&tn, 4);
  in.read((char*)&num, 8);
  in.read((char*)&dim, 8);
  if (!in) return fail(EFG_ERR_FORMAT, "truncated trees header");
  if (num != idx->n) return fail(EFG_ERR_FORMAT, "trees file is for " + std::to_string(num) + " points");
  if (tn == 0 || tn > 4096) return fail(EFG_ERR_FORMAT, "bad tree count");
  std::vector<HNode> nodes;
  std::vector<int32_t> roots;
  for (uint32_t t = 0; t < tn; ++t) {
    int node_num, node_size;
    in.read((char*)&node_num, 4);
    in.read((char*)&node_size, 4);
    if (!in || node_num <= 0 || (uint64_t)node_num > 2 * num + 1) return fail(EFG_ERR_FORMAT, "bad node count");
    std::vector<int32_t> stack;
    for (int j = 0; j < node_num; ++j) {
      HNode nd;
      uint64_t lp, rp;
      in.read((char*)&nd.div_dim, 4);
      in.read((char*)&nd.div_val, 4);
      in.read((char*)&nd.start, 8);
      in.read((char*)&nd.end, 8);
      in.read((char*)&lp, 8);
      in.read((char*)&rp, 8);
      if (!in) return fail(EFG_ERR_FORMAT, "truncated tree nodes");
      if (nd.start > nd.end || nd.end > num) return fail(EFG_ERR_FORMAT, "node range out of bounds");
      nd.left = nd.right = -1;
      nd.level = 0;
      nodes.push_back(nd);
      int32_t cur = (int32_t)nodes.size() - 1;
      size_t rs = stack.size();
      if (rs >= 2) {
        HNode& l1 = nodes[stack[rs - 1]];
        HNode& l2 = nodes[stack[rs - 2]];
        if (l1.end == nodes[cur].end && l2.start == nodes[cur].start) {
          nodes[cur].right = stack[rs - 1];
          nodes[cur].left = stack[rs - 2];
          stack.pop_back();
          stack.pop_back();
        }
      }
      stack.push_back(cur);
    }
    if (stack.size() != 1) return fail(EFG_ERR_FORMAT, "Error constructing trees");
    roots.push_back(stack[0]);
  }
  for (size_t i = 0; i < nodes.size(); ++i)
    if (nodes[i].left >= 0 && (nodes[i].div_dim < 0 || (uint32_t)nodes[i].div_dim >= idx->dim))
      return fail(EFG_ERR_FORMAT, "split dimension out of range");
  std::vector<uint32_t> leaves((size_t)tn * num);
  in.read((char*)leaves.data(), (std::streamsize)(leaves.size() * 4));
  if (!in) return fail(EFG_ERR_FORMAT, "truncated leaf lists");
  for (uint32_t v : leaves)
    if (v >= num) return fail(EFG_ERR_FORMAT, "leaf id out of range");
  // node levels (depth from the root), used by the merge-level check
  for (uint32_t t = 0; t < tn; ++t) {
    std::vector<int32_t> st{roots[t]};
    nodes[roots[t]].level = 0;
    while (!st.empty()) {
      int32_t v = st.back();
      st.pop_back();
      if (nodes[v].left >= 0) {
        nodes[nodes[v].left].level = nodes[v].level + 1;
        nodes[nodes[v].right].level = nodes[v].level + 1;
        st.push_back(nodes[v].left);
        st.push_back(nodes[v].right);
      }
    }
  }
  if (K_out) *K_out = K;
  return upload_forest(idx, nodes, roots, leaves, tn);
}

// ---- graph -----------------------------------------------------------------------------------
static int upload_graph(efg_index* idx, const std::vector<uint64_t>& ptr, const std::vector<uint32_t>& ids) {
  Graph& g = idx->graph;
  g.release();
  g.n = ptr.size() - 1;
  g.nnz = ids.size();
  EFG_TRY(g.ptr.reserve(ptr.size()));
  EFG_TRY(g.ids.reserve(ids.size() + 1));
  EFG_CUDA(cudaMemcpy(g.ptr.p, ptr.data(), ptr.size() * 8, cudaMemcpyHostToDevice));
  if (!ids.empty()) EFG_CUDA(cudaMemcpy(g.ids.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice));
  g.fixed_k = 0;
  if (g.n > 0) {
    uint64_t k0 = ptr[1] - ptr[0];
    bool fixed = true;
    for (uint64_t i = 0; i < g.n && fixed; ++i) fixed = (ptr[i + 1] - ptr[i]) == k0;
    if (fixed) g.fixed_k = (uint32_t)k0;
  }
  g.max_deg = 0;
  for (uint64_t i = 0; i < g.n; ++i) g.max_deg = std::max<uint32_t>(g.max_deg, (uint32_t)(ptr[i + 1] - ptr[i]));
  g.valid = true;
  return EFG_OK;
}

static int download_graph(const efg_index* idx, std::vector<uint64_t>& ptr, std::vector<uint32_t>& ids) {
  const Graph& g = idx->graph;
  ptr.resize(g.n + 1);
  ids.resize(g.nnz);
  EFG_CUDA(cudaMemcpy(ptr.data(), g.ptr.p, ptr.size() * 8, cudaMemcpyDeviceToHost));
  if (g.nnz) EFG_CUDA(cudaMemcpy(ids.data(), g.ids.p, g.nnz * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

}  // namespace efg

using namespace efg;

// Argument checks shared by the exact k-NN entry points.
namespace efg {
int bf_check_args(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q, uint64_t nq,
                  uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row, const int32_t* d_ids) {
  if (!d_base || (!d_q && nq) || (!d_ids && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (k == 0 || k > 256) return fail(EFG_ERR_ARG, "k must be in [1, 256]");
  if ((uint64_t)k + (exclude_self ? 1 : 0) > n) return fail(EFG_ERR_ARG, "k larger than the base");
  if (n > (uint64_t)INT32_MAX) return fail(EFG_ERR_ARG, "base larger than 2^31 - 1 rows (ids are int32)");
  if (exclude_self && (first_row > n || nq > n - first_row))
    return fail(EFG_ERR_ARG, "exclude_self: queries first_row .. first_row + nq must be base rows");
  if (dim == 0) return fail(EFG_ERR_ARG, "dim must be positive");
  if (row_stride < dim || q_stride < dim || (row_stride % 4) || (q_stride % 4) || (((uintptr_t)d_base) & 15) ||
      (((uintptr_t)d_q) & 15))
    return fail(EFG_ERR_ARG, "rows must be 16-byte aligned: strides a multiple of 4 floats");
  return EFG_OK;
}

}  // namespace efg

extern "C" {

const char* efg_last_error(void) { return g_last_error.c_str(); }
const char* efg_version(void) { return "efanna_gb300 0.1 (sm_103a)"; }

void efg_default_build_params(efg_build_params* p) {
  if (!p) return;
  p->K = 10;
  p->S = 10;
  p->L = 30;
  p->check_k = 25;
  p->epochs = 4;
  p->trees = 4;
  p->trees_build = 0;
  p->merge_level = 4;
  p->leaf_size = 10;
  p->reverse_cap = 100;
  p->seed = 1998;
}

int efg_index_create(const float* data, uint64_t n, uint32_t dim, uint64_t row_stride,
                     const efg_build_params* params, efg_index** out) {
  if (!data) return fail(EFG_ERR_ARG, "null data");
  if (row_stride < dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  EFG_TRY(make_index(n, dim, params, out));
  efg_index* idx = *out;
  cudaError_t e = cudaMemcpy2D(idx->d_base, idx->ld * sizeof(float), data, row_stride * sizeof(float),
                               dim * sizeof(float), n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    efg_index_destroy(idx);
    *out = nullptr;
    return fail(EFG_ERR_CUDA, std::string("copying base vectors: ") + cudaGetErrorString(e));
  }
  return EFG_OK;
}

int efg_index_create_device(const float* d_data, uint64_t n, uint32_t dim, uint64_t row_stride,
                            const efg_build_params* params, efg_index** out) {
  if (!d_data) return fail(EFG_ERR_ARG, "null data");
  if (row_stride < dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  EFG_TRY(make_index(n, dim, params, out));
  efg_index* idx = *out;
  cudaError_t e = cudaMemcpy2D(idx->d_base, idx->ld * sizeof(float), d_data, row_stride * sizeof(float),
                               dim * sizeof(float), n, cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) {
    efg_index_destroy(idx);
    *out = nullptr;
    return fail(EFG_ERR_CUDA, std::string("copying base vectors: ") + cudaGetErrorString(e));
  }
  return EFG_OK;
}

void efg_index_destroy(efg_index* idx) {
  if (!idx) return;
  if (idx->stream) cudaStreamSynchronize(idx->stream);
  idx->forest.release();
  idx->graph.release();
  idx->q_buf.release();
  idx->out_buf.release();
  idx->eval_counter.release();
  idx->ht_scratch.release();
  idx->ovf_list.release();
  idx->base16.release();
  idx->base8.release();
  idx->scale8.release();
  idx->kg_keys.release();
  idx->qp_buf.release();
  idx->kg_bits.release();
  if (idx->d_base) cudaFree(idx->d_base);
  if (idx->stream) cudaStreamDestroy(idx->stream);
  delete idx;
}

int efg_build_trees(efg_index* idx) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  return build_forest(idx, idx->bp.trees);
}

int efg_build_trees_count(efg_index* idx, uint32_t ntrees) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  if (ntrees < 1 || ntrees > 1024) return fail(EFG_ERR_ARG, "trees must be in [1, 1024]");
  EFG_TRY(build_forest(idx, ntrees));
  idx->sp.search_trees = (int)ntrees;
  return EFG_OK;
}

int efg_build_graph(efg_index* idx) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  return build_graph_device(idx);
}

int efg_get_build_stats(const efg_index* idx, efg_build_stats* out) {
  if (!idx || !out) return fail(EFG_ERR_ARG, "null argument");
  *out = idx->bstats;
  return EFG_OK;
}

int efg_get_search_stats(const efg_index* idx, efg_search_stats* out) {
  if (!idx || !out) return fail(EFG_ERR_ARG, "null argument");
  *out = idx->sstats;
  return EFG_OK;
}

int efg_set_search_params(efg_index* idx, int epochs, int init_num, int extend_to, int search_trees, int search_lv,
                          int search_method) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  SearchParams& sp = idx->sp;
  sp.epochs = epochs;
  sp.init_num = init_num;
  sp.extend_to = extend_to > init_num ? init_num : extend_to;
  sp.search_lv = search_lv;
  sp.search_trees = search_trees;
  sp.method = search_method;
  return EFG_OK;
}

int efg_set_search_candidate_cap(efg_index* idx, uint32_t cap) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  idx->candidate_cap = cap;
  return EFG_OK;
}

int efg_set_search_precision(efg_index* idx, int precision) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  if (precision != EFG_PRECISION_FP32 && precision != EFG_PRECISION_BF16 && precision != EFG_PRECISION_FP8)
    return fail(EFG_ERR_ARG, "precision must be EFG_PRECISION_FP32, EFG_PRECISION_BF16 or EFG_PRECISION_FP8");
  if (precision == EFG_PRECISION_BF16 && !idx->base16.p) EFG_TRY(make_base16(idx));
  if (precision == EFG_PRECISION_FP8 && !idx->base8.p) EFG_TRY(make_base8(idx));
  idx->precision = precision;
  return EFG_OK;
}

int efg_set_build_precision(efg_index* idx, int precision) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  if (precision != EFG_PRECISION_FP32 && precision != EFG_PRECISION_BF16)
    return fail(EFG_ERR_ARG, "build precision must be EFG_PRECISION_FP32 or EFG_PRECISION_BF16");
  idx->build_precision = precision;
  return EFG_OK;
}

int efg_screen_distances(efg_index* idx, int precision, const float* d_q, uint64_t nq, uint64_t row_stride,
                         const uint32_t* d_ids, uint32_t m, float* d_out, void* stream) {
  if (!idx || ((!d_q || !d_ids || !d_out) && nq && m)) return fail(EFG_ERR_ARG, "null argument");
  if (row_stride < idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  return screen_pairs(idx, precision, d_q, nq, row_stride, d_ids, m, d_out, (cudaStream_t)stream);
}

int efg_knn_search_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t row_stride, uint32_t k,
                          int32_t* d_out, void* stream) {
  if (!idx || (!d_q && nq) || (!d_out && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (row_stride < idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  return search_device(idx, d_q, nq, row_stride, k, d_out, (cudaStream_t)stream, false);
}

int efg_knn_search_batch_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t row_stride,
                                const efg_query_params* d_params, const efg_query_params* limits, int32_t* d_out,
                                const uint32_t* d_nq, void* stream) {
  if (!idx || !limits || ((!d_q || !d_params || !d_out) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (row_stride < idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (idx->sp.method != 0) return fail(EFG_ERR_ARG, "per-query parameters are supported by search method 0 only");
  return search_device_ex(idx, d_q, nq, row_stride, *limits, d_params, d_nq, d_out, (cudaStream_t)stream, false);
}

int efg_knn_search_seeded_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t row_stride,
                                 const efg_query_params* d_params, const efg_query_params* limits,
                                 const uint32_t* d_seeds, uint32_t seeds_per_query, int use_trees, int32_t* d_out,
                                 void* stream) {
  if (!idx || !limits || ((!d_q || !d_out || (!d_seeds && seeds_per_query)) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (row_stride < idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (idx->sp.method != 0) return fail(EFG_ERR_ARG, "seeded search uses search method 0");
  return search_device_ex(idx, d_q, nq, row_stride, *limits, d_params, nullptr, d_out, (cudaStream_t)stream, false,
                          d_seeds, seeds_per_query, use_trees != 0);
}

int efg_knn_search_batch(efg_index* idx, const float* q, uint64_t nq, uint32_t dim, uint64_t row_stride,
                         const efg_query_params* params, uint32_t k_max, int32_t* out_ids) {
  if (!idx || ((!q || !params || !out_ids) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (dim != idx->dim) return fail(EFG_ERR_ARG, "query dimension differs from the base");
  if (row_stride < dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (idx->sp.method != 0) return fail(EFG_ERR_ARG, "per-query parameters are supported by search method 0 only");
  if (k_max == 0) return fail(EFG_ERR_ARG, "k_max must be positive");
  if (nq == 0) return EFG_OK;
  efg_query_params lim{0, 1, 0, k_max};
  for (uint64_t i = 0; i < nq; ++i) {
    const efg_query_params& p = params[i];
    if (p.init_num <= 0 || (uint64_t)p.init_num > idx->n) return fail(EFG_ERR_ARG, "pool size must be in [1, n]");
    if (p.epochs < 0 || p.extend_to < 0) return fail(EFG_ERR_ARG, "negative epochs or extend");
    if (p.k == 0 || p.k > k_max || (int)p.k > p.init_num) return fail(EFG_ERR_ARG, "k must be in [1, min(k_max, pool)]");
    lim.epochs = std::max(lim.epochs, p.epochs);
    lim.init_num = std::max(lim.init_num, p.init_num);
    lim.extend_to = std::max(lim.extend_to, std::min(p.extend_to, p.init_num));
  }
  if ((int)k_max > lim.init_num) lim.k = (uint32_t)lim.init_num;
  EFG_TRY(idx->q_buf.reserve(nq * idx->ld));
  EFG_TRY(idx->out_buf.reserve(nq * (uint64_t)lim.k));
  EFG_TRY(idx->qp_buf.reserve(nq));
  EFG_CUDA(cudaMemsetAsync(idx->q_buf.p, 0, nq * idx->ld * sizeof(float), idx->stream));
  EFG_CUDA(cudaMemcpy2DAsync(idx->q_buf.p, idx->ld * sizeof(float), q, row_stride * sizeof(float), dim * sizeof(float),
                             nq, cudaMemcpyHostToDevice, idx->stream));
  EFG_CUDA(cudaMemcpyAsync(idx->qp_buf.p, params, nq * sizeof(efg_query_params), cudaMemcpyHostToDevice,
                           idx->stream));
  EFG_TRY(search_device_ex(idx, idx->q_buf.p, nq, idx->ld, lim, idx->qp_buf.p, nullptr, idx->out_buf.p, idx->stream,
                           true));
  if (lim.k == k_max) {
    EFG_CUDA(cudaMemcpyAsync(out_ids, idx->out_buf.p, nq * (uint64_t)k_max * sizeof(int32_t), cudaMemcpyDeviceToHost,
                             idx->stream));
  } else {  // every pool is smaller than k_max: rows of lim.k ids, padded with -1
    EFG_CUDA(cudaMemcpy2DAsync(out_ids, k_max * sizeof(int32_t), idx->out_buf.p, lim.k * sizeof(int32_t),
                               lim.k * sizeof(int32_t), nq, cudaMemcpyDeviceToHost, idx->stream));
  }
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  if (lim.k != k_max)
    for (uint64_t i = 0; i < nq; ++i)
      for (uint32_t j = lim.k; j < k_max; ++j) out_ids[i * k_max + j] = -1;
  return EFG_OK;
}

int efg_knn_search(efg_index* idx, const float* q, uint64_t nq, uint32_t dim, uint64_t row_stride, uint32_t k,
                   int32_t* out_ids) {
  if (!idx || (!q && nq) || (!out_ids && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (dim != idx->dim) return fail(EFG_ERR_ARG, "query dimension differs from the base");
  if (row_stride < dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (nq == 0) {
    idx->last_results.clear();
    idx->last_nq = 0;
    idx->last_k = k;
    return EFG_OK;
  }
  EFG_TRY(idx->q_buf.reserve(nq * idx->ld));
  EFG_TRY(idx->out_buf.reserve(nq * (uint64_t)k));
  EFG_CUDA(cudaMemsetAsync(idx->q_buf.p, 0, nq * idx->ld * sizeof(float), idx->stream));
  EFG_CUDA(cudaMemcpy2DAsync(idx->q_buf.p, idx->ld * sizeof(float), q, row_stride * sizeof(float), dim * sizeof(float),
                             nq, cudaMemcpyHostToDevice, idx->stream));
  EFG_TRY(search_device(idx, idx->q_buf.p, nq, idx->ld, k, idx->out_buf.p, idx->stream, true));
  EFG_CUDA(cudaMemcpyAsync(out_ids, idx->out_buf.p, nq * (uint64_t)k * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           idx->stream));
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  idx->last_results.assign(out_ids, out_ids + nq * (uint64_t)k);
  idx->last_nq = nq;
  idx->last_k = k;
  return EFG_OK;
}

int efg_save_results(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ofstream out(path, std::ios::binary);
  if (!out.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  int dim = (int)idx->last_k;
  for (uint64_t i = 0; i < idx->last_nq; ++i) {
    out.write((const char*)&dim, 4);
    out.write((const char*)&idx->last_results[i * idx->last_k], 4 * (std::streamsize)idx->last_k);
  }
  return out.good() ? EFG_OK : fail(EFG_ERR_OPEN, "write failed");
}

int efg_save_graph(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ofstream out(path, std::ios::binary);
  if (!out.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph to save (empty file written)");
  std::vector<uint64_t> ptr;
  std::vector<uint32_t> ids;
  EFG_TRY(download_graph(idx, ptr, ids));
  for (uint64_t i = 0; i < idx->graph.n; ++i) {
    uint32_t k = (uint32_t)(ptr[i + 1] - ptr[i]);
    out.write((const char*)&k, 4);
    out.write((const char*)&ids[ptr[i]], 4 * (std::streamsize)k);
  }
  return out.good() ? EFG_OK : fail(EFG_ERR_OPEN, "write failed");
}

int efg_load_graph(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  in.seekg(0, std::ios::end);
  uint64_t fsize = (uint64_t)in.tellg();
  in.seekg(0, std::ios::beg);
  int first = 0;
  in.read((char*)&first, 4);
  if (!in || first < 0) return fail(EFG_ERR_FORMAT, "empty or malformed graph file");
  uint64_t N = fsize / ((uint64_t)first + 1) / 4;  // loadGraph's row count (kdtreeub_index.hpp:253)
  in.seekg(0, std::ios::beg);
  std::vector<uint64_t> ptr{0};
  std::vector<uint32_t> ids;
  for (uint64_t i = 0; i < N; ++i) {
    uint32_t k;
    in.read((char*)&k, 4);
    if (!in) return fail(EFG_ERR_FORMAT, "truncated graph file");
    size_t off = ids.size();
    ids.resize(off + k);
    in.read((char*)&ids[off], 4 * (std::streamsize)k);
    if (!in) return fail(EFG_ERR_FORMAT, "truncated graph file");
    ptr.push_back(ids.size());
  }
  if (N != idx->n) return fail(EFG_ERR_FORMAT, "graph has " + std::to_string(N) + " rows, index has " +
                                                   std::to_string(idx->n));
  for (uint32_t v : ids)
    if (v >= idx->n) return fail(EFG_ERR_FORMAT, "graph id out of range");
  return upload_graph(idx, ptr, ids);
}

int efg_save_trees(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ofstream out(path, std::ios::binary);
  if (!out.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  if (idx->forest.ntrees == 0) return fail(EFG_ERR_STATE, "no trees to save");
  return write_trees(idx, out);
}

int efg_load_trees(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  EFG_TRY(read_trees(idx, in, nullptr));
  idx->sp.search_trees = (int)idx->forest.ntrees;  // SP.tree_num = tree_num (kdtreeub_index.hpp:151)
  return EFG_OK;
}

// saveIndex writes the trees and then N x K graph ids.  (The reference's save_data writes its
// knn_graph sets, which buildIndex has already cleared, so it exits; this writes the graph the
// build produced, first K ids of each row.)
int efg_save_index(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ofstream out(path, std::ios::binary);
  if (!out.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  if (idx->forest.ntrees == 0 || !idx->graph.valid) return fail(EFG_ERR_STATE, "index needs trees and a graph");
  EFG_TRY(write_trees(idx, out));
  std::vector<uint64_t> ptr;
  std::vector<uint32_t> ids;
  EFG_TRY(download_graph(idx, ptr, ids));
  uint32_t K = idx->bp.K;
  for (uint64_t i = 0; i < idx->graph.n; ++i) {
    for (uint32_t j = 0; j < K; ++j) {
      int32_t v = j < ptr[i + 1] - ptr[i] ? (int32_t)ids[ptr[i] + j] : -1;
      out.write((const char*)&v, 4);
    }
  }
  return out.good() ? EFG_OK : fail(EFG_ERR_OPEN, "write failed");
}

int efg_load_index(efg_index* idx, const char* path) {
  if (!idx || !path) return fail(EFG_ERR_ARG, "null argument");
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) return fail(EFG_ERR_OPEN, std::string("open file error: ") + path);
  uint32_t K = 0;
  EFG_TRY(read_trees(idx, in, &K));
  idx->sp.search_trees = (int)idx->forest.ntrees;
  std::vector<int32_t> raw((size_t)idx->n * K);
  in.read((char*)raw.data(), (std::streamsize)(raw.size() * 4));
  if (!in) return fail(EFG_ERR_FORMAT, "truncated graph section");
  std::vector<uint64_t> ptr{0};
  std::vector<uint32_t> ids;
  ids.reserve(raw.size());
  for (uint64_t i = 0; i < idx->n; ++i) {
    for (uint32_t j = 0; j < K; ++j) {
      int32_t v = raw[i * K + j];
      if (v < 0) continue;
      if ((uint64_t)v >= idx->n) return fail(EFG_ERR_FORMAT, "graph id out of range");
      ids.push_back((uint32_t)v);
    }
    ptr.push_back(ids.size());
  }
  return upload_graph(idx, ptr, ids);
}

uint64_t efg_graph_size(const efg_index* idx) { return (idx && idx->graph.valid) ? idx->graph.n : 0; }

int64_t efg_graph_row(const efg_index* idx, uint64_t row, uint32_t* out, uint64_t cap) {
  if (!idx) return fail(EFG_ERR_ARG, "null index"), -1;
  if (!idx->graph.valid || row >= idx->graph.n) return 0;  // getGraphRow returns an empty row
  uint64_t pr[2];
  if (cudaMemcpy(pr, idx->graph.ptr.p + row, 16, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  uint64_t len = pr[1] - pr[0];
  if (out && cap) {
    uint64_t m = len < cap ? len : cap;
    if (m && cudaMemcpy(out, idx->graph.ids.p + pr[0], m * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  }
  return (int64_t)len;
}

int efg_graph_csr(const efg_index* idx, uint64_t* row_ptr, uint32_t* ids, uint64_t* nnz) {
  if (!idx) return fail(EFG_ERR_ARG, "null index");
  if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph");
  if (nnz) *nnz = idx->graph.nnz;
  if (row_ptr) EFG_CUDA(cudaMemcpy(row_ptr, idx->graph.ptr.p, (idx->graph.n + 1) * 8, cudaMemcpyDeviceToHost));
  if (ids && idx->graph.nnz) EFG_CUDA(cudaMemcpy(ids, idx->graph.ids.p, idx->graph.nnz * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

int efg_csr_transpose(uint64_t n, const uint64_t* row_ptr, const uint32_t* ids, uint64_t* col_ptr,
                      uint32_t* row_ids) {
  if (!row_ptr || !col_ptr || (!ids && row_ptr[n]) || (!row_ids && row_ptr[n])) return fail(EFG_ERR_ARG, "null argument");
  if (row_ptr[0] != 0) return fail(EFG_ERR_ARG, "row_ptr[0] must be 0");
  for (uint64_t i = 0; i < n; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return fail(EFG_ERR_ARG, "row_ptr must be ascending");
  const uint64_t nnz = row_ptr[n];
  // counting sort by column; sources visited in ascending order keep each column's rows ascending
  std::vector<uint64_t> cnt(n + 1, 0);
  for (uint64_t e = 0; e < nnz; ++e) {
    if (ids[e] >= n) return fail(EFG_ERR_ARG, "graph id " + std::to_string(ids[e]) + " >= n");
    ++cnt[ids[e] + 1];
  }
  for (uint64_t j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
  for (uint64_t j = 0; j <= n; ++j) col_ptr[j] = cnt[j];
  for (uint64_t i = 0; i < n; ++i)
    for (uint64_t e = row_ptr[i]; e < row_ptr[i + 1]; ++e) row_ids[cnt[ids[e]]++] = (uint32_t)i;
  return EFG_OK;
}

int efg_graph_csc(const efg_index* idx, uint64_t* col_ptr, uint32_t* row_ids) {
  if (!idx || !col_ptr) return fail(EFG_ERR_ARG, "null argument");
  if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph");
  const uint64_t n = idx->graph.n, nnz = idx->graph.nnz;
  if (nnz && !row_ids) return fail(EFG_ERR_ARG, "null argument");
  std::vector<uint64_t> ptr(n + 1);
  std::vector<uint32_t> ids(nnz);
  EFG_TRY(efg_graph_csr(idx, ptr.data(), ids.data(), nullptr));
  return efg_csr_transpose(n, ptr.data(), ids.data(), col_ptr, row_ids);
}

uint32_t efg_tree_count(const efg_index* idx) { return idx ? idx->forest.ntrees : 0; }

int efg_l2_pairs(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const uint32_t* d_a,
                 const uint32_t* d_b, uint64_t m, float* d_out, void* stream) {
  if (!d_base || ((!d_a || !d_b || !d_out) && m)) return fail(EFG_ERR_ARG, "null argument");
  if (dim == 0 || row_stride < dim || (row_stride % 4) != 0 || (((uintptr_t)d_base) & 15))
    return fail(EFG_ERR_ARG, "rows must be 16-byte aligned: row_stride a multiple of 4 floats");
  (void)n;
  return launch_l2_pairs(d_base, dim, (uint32_t)row_stride, d_a, d_b, m, d_out, (cudaStream_t)stream);
}

int efg_brute_force_knn(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q,
                        uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row,
                        int32_t* d_ids, float* d_dists, void* stream) {
  EFG_TRY(efg::bf_check_args(d_base, n, dim, row_stride, d_q, nq, q_stride, k, exclude_self, first_row, d_ids));
  return exact_knn(d_base, n, dim, (uint32_t)row_stride, d_q, nq, (uint32_t)q_stride, k, exclude_self, first_row,
                   d_ids, d_dists, (cudaStream_t)stream);
}

int efg_get_knn_stats(efg_knn_stats* out) {
  if (!out) return fail(EFG_ERR_ARG, "null argument");
  *out = g_knn_stats;
  return EFG_OK;
}

int efg_brute_force_knn_fp32(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q,
                             uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row,
                             int32_t* d_ids, float* d_dists, void* stream) {
  EFG_TRY(efg::bf_check_args(d_base, n, dim, row_stride, d_q, nq, q_stride, k, exclude_self, first_row, d_ids));
  return brute_force_knn(d_base, n, dim, (uint32_t)row_stride, d_q, nq, (uint32_t)q_stride, k, exclude_self,
                         first_row, d_ids, d_dists, (cudaStream_t)stream);
}

int efg_brute_force_knn_split(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q,
                              uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row,
                              int32_t* d_ids, float* d_dists, void* stream) {
  EFG_TRY(efg::bf_check_args(d_base, n, dim, row_stride, d_q, nq, q_stride, k, exclude_self, first_row, d_ids));
  if (k > tc_knn_max_k()) return fail(EFG_ERR_ARG, "k above the tensor-core path's limit");
  return brute_force_knn_tc(d_base, n, dim, (uint32_t)row_stride, d_q, nq, (uint32_t)q_stride, k, exclude_self,
                            first_row, d_ids, d_dists, (cudaStream_t)stream, 1);
}

int efg_nnd_init(efg_index* idx, efg_nnd_host_state* st) {
  if (!idx || !st) return fail(EFG_ERR_ARG, "null argument");
  return nnd_init_host(idx, st);
}

int efg_nnd_iterate(efg_index* idx, efg_nnd_host_state* st, uint32_t iter, uint64_t* pairs) {
  if (!idx || !st) return fail(EFG_ERR_ARG, "null argument");
  return nnd_iterate_host(idx, st, iter, pairs);
}

}  // extern "C"
