// Internal declarations shared by the efanna_gb300 translation units.
#pragma once
#include <cuda_bf16.h>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace efg {

// A device buffer that grows on demand (never shrinks until freed).
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;  // elements
  int reserve(size_t n) {
    if (n <= cap) return EFG_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = n + n / 8 + 64;
    cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(EFG_ERR_NOMEM, "cudaMalloc of " + std::to_string(want * sizeof(T)) + " bytes failed");
    }
    cap = want;
    return EFG_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// An NVTX range over a scope (named phases for Nsight Systems / Nsight Compute; free when no tool
// is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// CUDA events owned by a scope (destroyed on every return path).
template <int N>
struct ScopedEvents {
  cudaEvent_t e[N];
  ScopedEvents() {
    for (auto& x : e) cudaEventCreate(&x);
  }
  ~ScopedEvents() {
    for (auto& x : e) cudaEventDestroy(x);
  }
  ScopedEvents(const ScopedEvents&) = delete;
  ScopedEvents& operator=(const ScopedEvents&) = delete;
};

// A function-local device buffer: freed when it goes out of scope (also on early error returns).
template <typename T>
struct LocalBuf : DevBuf<T> {
  LocalBuf() = default;
  LocalBuf(const LocalBuf&) = delete;
  LocalBuf& operator=(const LocalBuf&) = delete;
  ~LocalBuf() { this->release(); }
};

// Host-side tree node (load/save and the merge-level check).
struct HNode {
  int32_t div_dim;
  float div_val;
  uint64_t start, end;
  int32_t left, right;  // global node indices, -1 for leaves
  int32_t level;
};

// Trees held by an index.  Nodes of all trees share one index space; leaf lists are tree-major
// (tree t's list is leaves[t*n .. t*n+n)).
struct Forest {
  uint32_t ntrees = 0;
  uint64_t n = 0;
  std::vector<int32_t> roots;           // per tree, global node index
  std::vector<uint32_t> tree_of_root;   // unused placeholder for symmetry
  DevBuf<DNode> nodes;                  // search layout
  uint64_t nnodes = 0;
  DevBuf<int32_t> d_roots;
  DevBuf<uint32_t> leaves;              // ntrees * n
  // SoA build-side arrays (kept after a device build; used by the leaf merge)
  DevBuf<int32_t> n_left, n_right, n_level, n_tree;
  DevBuf<uint32_t> n_start, n_end;
  DevBuf<int32_t> nleaf;                // leaves in each node's subtree (search descent ranks)
  DevBuf<uint2> cnl;                    // per internal node: (nleaf[left], nleaf[right]), loaded with the node
  bool has_soa = false;
  void release() {
    nodes.release(); d_roots.release(); leaves.release(); nleaf.release(); cnl.release();
    n_left.release(); n_right.release(); n_level.release(); n_tree.release(); n_start.release(); n_end.release();
    ntrees = 0; nnodes = 0; roots.clear(); has_soa = false;
  }
};

struct Graph {
  uint64_t n = 0, nnz = 0;
  uint32_t fixed_k = 0;  // 0 when rows have different lengths
  uint32_t max_deg = 0;  // longest row
  DevBuf<uint64_t> ptr;  // n + 1
  DevBuf<uint32_t> ids;  // nnz
  bool valid = false;
  void release() { ptr.release(); ids.release(); valid = false; n = nnz = 0; fixed_k = 0; max_deg = 0; }
};

struct SearchParams {
  int epochs = 4, init_num = 100, extend_to = 10, search_trees = 0, search_lv = -1, method = 0;
};

}  // namespace efg

struct efg_index {
  uint64_t n = 0;
  uint32_t dim = 0, ld = 0;  // ld: padded row stride in floats (multiple of 4)
  float* d_base = nullptr;
  efg_build_params bp{};
  efg::Forest forest;
  efg::Graph graph;
  efg::SearchParams sp;
  cudaStream_t stream = nullptr;
  std::vector<int32_t> last_results;
  uint32_t last_k = 0;
  uint64_t last_nq = 0;
  efg_build_stats bstats{};
  efg_search_stats sstats{};
  // search scratch
  efg::DevBuf<float> q_buf;
  efg::DevBuf<int32_t> out_buf;
  efg::DevBuf<unsigned long long> eval_counter;
  efg::DevBuf<uint32_t> ht_scratch;  // per-CTA visited sets when they do not fit in shared memory
  efg::DevBuf<uint32_t> ovf_list;    // queries handed from the first search pass to the overflow pass
  // search precision: 0 = FP32 rows, 1 = BF16 screening copy (base16, ld16 values per row) + FP32 re-rank
  int precision = 0;
  int build_precision = 0;  // NN-descent join: EFG_PRECISION_FP32 or EFG_PRECISION_BF16 (tensor cores)
  efg::DevBuf<uint16_t> base16;
  uint32_t ld16 = 0;
  efg::DevBuf<uint8_t> base8;   // FP8 e4m3 screening copy (ld8 bytes per row) and per-row scales
  efg::DevBuf<float> scale8;
  uint32_t ld8 = 0;
  // kgraph search scratch: pool keys per query, visited bitsets per warp
  efg::DevBuf<uint64_t> kg_keys;
  efg::DevBuf<uint32_t> kg_bits;
  efg::DevBuf<efg_query_params> qp_buf;  // per-query parameters of a host batch
  int search_threads = 0;                  // nnexp block size forced by a plan's autotuner (0: by occupancy)
  int search_ctas_per_sm = 0;              // cap on resident nnexp CTAs per SM (0: as many as fit)
  int search_ht_pct = 0;                   // shared visited-set size, percent of the default (0: 100)
  uint32_t candidate_cap = 0;              // bound on the nnexp candidate buffer (0: extend_to x degree)
};

namespace efg {

// distance.cu
int launch_l2_pairs(const float* base, uint32_t dim, uint32_t ld, const uint32_t* a, const uint32_t* b, uint64_t m,
                    float* out, cudaStream_t s);
int brute_force_knn(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                    uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                    cudaStream_t s);
// index.cu: argument checks of the exact k-NN entry points (null pointers, k, sizes, alignment).
int bf_check_args(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q, uint64_t nq,
                  uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row, const int32_t* d_ids);
// gram_tc.cu: the same results with the screening on the tensor cores (k <= tc_knn_max_k());
// force_split uses the hi + lo BF16 products even when BF16 holds the data exactly.
uint32_t tc_knn_max_k();
extern thread_local efg_knn_stats g_knn_stats;  // the calling thread's last tensor-core k-NN call
int brute_force_knn_tc(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                       uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                       cudaStream_t s, int force_split = 0);
// join_tc.cu: the NN-descent join's pass 0 on the tensor cores.  tc_join_prepare converts the base
// to BF16 hi / lo rows of round_up(dim, 64) values with FP32 norms and sets *inexact when some lo is
// not zero; tc_join scores every node in three launches (tiles of 128 rows over all nodes, tiles of
// 256 rows over the nodes listed in mid, the nodes listed in big tile by tile; counters: three node
// counters); err is set when a wait ran out or a list holds an id >= n.
int tc_join_prepare(const float* base, uint64_t n, uint32_t dim, uint32_t ld, __nv_bfloat16* hi, __nv_bfloat16* lo,
                    float* norms, int* inexact, cudaStream_t s);
int tc_join(const __nv_bfloat16* hi, const __nv_bfloat16* lo, const float* norms, uint64_t n, uint32_t dim,
            uint32_t terms, uint32_t cap, uint32_t P, uint32_t check_k, const uint32_t* new_ids,
            const uint32_t* new_cnt, const uint32_t* old_ids, const uint32_t* old_cnt, const uint64_t* pair_off,
            const float* bound, float* pairdist, uint32_t* cnt, uint8_t* found, uint32_t* counters, uint32_t* mid,
            uint32_t* big, int* err, cudaStream_t s);
// mlp_tc.cu: the learned form's dense layers on the tensor cores, C = act(A W^T + bias) (A: M x K,
// W: N x K, BF16 row-major; C FP32 and / or Cb BF16, M x N); EFG_ERR_ARG when the shape does not fit.
int tc_gemm_bf16(uint32_t M, uint32_t N, uint32_t K, const __nv_bfloat16* A, const __nv_bfloat16* W,
                 const float* bias, int relu, float* C, __nv_bfloat16* Cb, int* err, cudaStream_t s);
// The exact k-NN of the library: tensor-core screening where k allows, else the FP32 kernels.
inline int exact_knn(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                     uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                     cudaStream_t s) {
  if (k <= tc_knn_max_k())
    return brute_force_knn_tc(base, n, dim, ld, q, nq, qld, k, exclude_self, first_row, ids, dists, s);
  return brute_force_knn(base, n, dim, ld, q, nq, qld, k, exclude_self, first_row, ids, dists, s);
}

// trees.cu: builds `ntrees` canonical trees over the index's base (fills idx->forest).
int build_forest(efg_index* idx, uint32_t ntrees);
// Uploads a host forest (after loadTrees) into the device search layout.
int upload_forest(efg_index* idx, const std::vector<HNode>& nodes, const std::vector<int32_t>& roots,
                  const std::vector<uint32_t>& leaves, uint32_t ntrees);
// Copies the device forest into host nodes (global indices) + leaves.
int download_forest(efg_index* idx, std::vector<HNode>& nodes, std::vector<uint32_t>& leaves);

// search.cu
int search_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, uint32_t k, int32_t* d_out,
                  cudaStream_t s, bool count_evals);
// nnexp over a batch whose queries carry their own parameters (d_params, bounded by lim), or all
// use lim when d_params is null; d_nq optionally holds the batch size on the device.
int search_device_ex(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, const efg_query_params& lim,
                     const efg_query_params* d_params, const uint32_t* d_nq, int32_t* d_out, cudaStream_t s,
                     bool count_evals, const uint32_t* d_seeds = nullptr, uint32_t seeds_per_query = 0,
                     bool use_trees = true, bool bucket_only = false, const uint32_t* d_seed_counts = nullptr);
// Builds the BF16 screening copy of the base (round to nearest even, rows padded with zeros).
int make_base16(efg_index* idx);
// Builds the FP8 e4m3 screening copy of the base with one FP32 scale per row.
int make_base8(efg_index* idx);
// Screening distances of (query, id) pairs in a given precision (the search's gather).
int screen_pairs(efg_index* idx, int precision, const float* d_q, uint64_t nq, uint64_t qld, const uint32_t* d_ids,
                 uint32_t m, float* d_out, cudaStream_t s);
// kgraph.cu: search method 1 (getNeighbors_kgraph).  With a seed source the pool comes from the
// hash tables' probe sequence instead of the trees, and expansions visit whole graph rows (the
// hashing initialiser's kgraph search, getNeighborsIEH32_kgraph).
struct KgSeedSource {
  efg_hash* h;
  const uint64_t* d_qcodes;  // tables x qstride
  uint64_t qstride;
  uint32_t tables;
  DevBuf<uint32_t>* buf;  // seed rows, grown as needed
  DevBuf<uint32_t>* cnt;  // entries present per seed row
};
// hashing.cu: the probe sequences of nq queries into seed rows of seeds_per_query entries; with
// d_counts, the entries present per row (the row's rest untouched), else rows padded with 0xffffffff.
int hash_seed_rows(efg_hash* h, const uint64_t* d_qcodes, uint64_t qcode_stride, uint64_t nq,
                   uint32_t seeds_per_query, uint32_t* d_seeds, uint32_t* d_counts, cudaStream_t s);
int kgraph_search_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, uint32_t k, int32_t* d_out,
                         cudaStream_t s, bool count_evals, const KgSeedSource* hs = nullptr);

// nndescent.cu
struct NNDState;
int build_graph_device(efg_index* idx);
int nnd_init_host(efg_index* idx, efg_nnd_host_state* st);
int nnd_iterate_host(efg_index* idx, efg_nnd_host_state* st, uint32_t iter, uint64_t* pairs);

}  // namespace efg
