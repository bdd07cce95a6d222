// Randomised truncated KD-trees, built level-synchronously for all trees at once.
//
// Reference: buildTrees / the tree part of initGraph (algorithm/kdtreeub_index.hpp:1192-1276,
// 1295-1363), meanSplit (:902-953), selectDivision (:974-999), planeSplit (:954-973),
// DFSbuild (:1138-1167).  Per node, as in the reference:
//   * mean and variance over the first min(101, count) ids of the node's id range, summed in id
//     order (FP32, no fused multiply-add);
//   * the split dimension is one of the (up to) 5 largest variances, ranked by (variance desc,
//     dimension asc) — the order selectDivision's insertion produces — picked at random;
//   * the cut is the mean in that dimension; ids with value < cut, == cut, > cut are laid out in
//     that order and the split index follows meanSplit's balancing rule;
//   * while fewer than 1100 nodes are active (all trees together) every active node is split and
//     children with more than S ids stay active (the BFS phase); afterwards nodes split while they
//     hold more than TNS ids (the DFS phase).
// Where the reference draws from std::rand()/mt19937 and partitions with Hoare swaps, this build
// uses a Feistel permutation per tree, a counter hash for the split choice and a stable
// three-way partition, so the trees are a pure function of (data, seed): the oracle's canonical
// mode builds identical trees.
//
// Layout during the build: ids[t*n + pos] (tree-major leaf lists, double-buffered),
// owner[t*n + pos] = node holding position pos; node records in structure-of-arrays form.
#include <algorithm>
#include <vector>

#include "scan.cuh"

namespace efg {

static constexpr int T_SAMPLE = 101;  // SAMPLE_NUM + 1 (kdtreeub_index.hpp:912)
static constexpr int T_RAND_DIM = 5;  // RAND_DIM (kdtreeub_index.hpp:1102)

struct NodeArrays {
  uint32_t *start, *end;
  int32_t *tree, *level, *left, *right, *dim, *split_at;  // split_at = level + 1 when split
  float* val;
};

__global__ void perm_init_kernel(uint32_t* ids, int32_t* owner, uint64_t n, uint32_t ntrees, uint64_t seed) {
  uint64_t total = n * ntrees;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t t = (uint32_t)(g / n), i = (uint32_t)(g % n);
    ids[g] = feistel_perm(i, (uint32_t)n, hash4(seed, TAG_PERM, t, 0, 0));
    owner[g] = (int32_t)t;  // node t is tree t's root
  }
}

__global__ void roots_init_kernel(NodeArrays na, uint32_t ntrees, uint64_t n) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntrees) return;
  na.start[t] = 0;
  na.end[t] = (uint32_t)n;
  na.tree[t] = (int32_t)t;
  na.level[t] = 0;
  na.left[t] = na.right[t] = -1;
  na.dim[t] = -1;
  na.val[t] = 0.f;
  na.split_at[t] = 0;
}

// (value desc, index asc): the rank order of selectDivision.
__device__ __forceinline__ bool var_better(float va, int32_t ia, float vb, int32_t ib) {
  return va > vb || (va == vb && ia < ib);
}

// One warp per active node: statistics, split dimension and cut value.
__global__ void split_stats_kernel(const float* __restrict__ base, uint32_t dim, uint32_t ld, uint64_t n,
                                   const uint32_t* __restrict__ ids, NodeArrays na, const int32_t* __restrict__ active,
                                   uint32_t nactive, int32_t level, int phaseB, uint32_t tns, uint64_t seed,
                                   uint32_t* __restrict__ split_flag) {
  extern __shared__ float smean[];  // (blockDim.x / 32) * dim
  uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t a = blockIdx.x * (blockDim.x >> 5) + wib;
  if (a >= nactive) return;
  float* mean = smean + (size_t)wib * dim;
  int32_t v = active[a];
  uint32_t s = na.start[v], e = na.end[v], count = e - s;
  int32_t t = na.tree[v];
  if (phaseB && count <= tns) {  // DFSbuild leaf (kdtreeub_index.hpp:1142-1149)
    if (lane == 0) {
      na.dim[v] = -1;
      split_flag[a] = 0;
    }
    return;
  }
  const uint32_t* seg = ids + (uint64_t)t * n + s;
  uint32_t cnt = min((uint32_t)T_SAMPLE, count);
  float inv = __fdiv_rn(1.0f, (float)cnt);
  // running top-5, identical on all lanes
  float tv[T_RAND_DIM];
  int32_t ti[T_RAND_DIM];
#pragma unroll
  for (int r = 0; r < T_RAND_DIM; ++r) {
    tv[r] = -1.0f;
    ti[r] = 0x7fffffff;
  }
  for (uint32_t kb = 0; kb < dim; kb += 32) {
    uint32_t k = kb + lane;
    float m = 0.f, var = 0.f;
    if (k < dim) {
      for (uint32_t j = 0; j < cnt; ++j) m = __fadd_rn(m, __ldg(base + (uint64_t)seg[j] * ld + k));
      m = __fmul_rn(m, inv);
      for (uint32_t j = 0; j < cnt; ++j) {
        float dd = __fsub_rn(__ldg(base + (uint64_t)seg[j] * ld + k), m);
        var = __fadd_rn(var, __fmul_rn(dd, dd));
      }
      mean[k] = m;
    }
    // merge this block's 32 candidates into the running top-5
    float cv = k < dim ? var : -1.0f;
    int32_t ci = k < dim ? (int32_t)k : 0x7fffffff;
    bool taken_c = k >= dim;
    bool taken_r[T_RAND_DIM];
#pragma unroll
    for (int r = 0; r < T_RAND_DIM; ++r) taken_r[r] = ti[r] == 0x7fffffff;
    float nv[T_RAND_DIM];
    int32_t ni[T_RAND_DIM];
#pragma unroll
    for (int r = 0; r < T_RAND_DIM; ++r) {
      // best remaining running entry (uniform) vs best remaining lane candidate (warp argmax)
      float bv = -1.0f;
      int32_t bi = 0x7fffffff;
      int br = -1;
#pragma unroll
      for (int q = 0; q < T_RAND_DIM; ++q)
        if (!taken_r[q] && (br < 0 || var_better(tv[q], ti[q], bv, bi))) {
          bv = tv[q];
          bi = ti[q];
          br = q;
        }
      float lv = taken_c ? -1.0f : cv;
      int32_t li = taken_c ? 0x7fffffff : ci;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float ov = __shfl_xor_sync(0xffffffffu, lv, o);
        int32_t oi = __shfl_xor_sync(0xffffffffu, li, o);
        if (var_better(ov, oi, lv, li)) {
          lv = ov;
          li = oi;
        }
      }
      bool lane_wins = li != 0x7fffffff && (br < 0 || var_better(lv, li, bv, bi));
      if (lane_wins) {
        nv[r] = lv;
        ni[r] = li;
        if (!taken_c && ci == li) taken_c = true;
      } else if (br >= 0) {
        nv[r] = bv;
        ni[r] = bi;
#pragma unroll
        for (int q = 0; q < T_RAND_DIM; ++q)
          if (q == br) taken_r[q] = true;
      } else {
        nv[r] = -1.0f;
        ni[r] = 0x7fffffff;
      }
    }
#pragma unroll
    for (int r = 0; r < T_RAND_DIM; ++r) {
      tv[r] = nv[r];
      ti[r] = ni[r];
    }
  }
  __syncwarp();
  int num = 0;
#pragma unroll
  for (int r = 0; r < T_RAND_DIM; ++r) num += ti[r] != 0x7fffffff;
  uint32_t rnd = (uint32_t)(hash4(seed, TAG_DIM, (uint64_t)t, (uint64_t)level, (uint64_t)s) % (uint64_t)num);
  int32_t cutdim = ti[0];
#pragma unroll
  for (int r = 0; r < T_RAND_DIM; ++r)
    if ((uint32_t)r == rnd) cutdim = ti[r];
  if (lane == 0) {
    na.dim[v] = cutdim;
    na.val[v] = mean[cutdim];
    na.split_at[v] = level + 1;
    split_flag[a] = 1;
  }
}

// Packed class counters per position: (is_less << 32) | is_equal, zero outside split nodes.
__global__ void classify_kernel(const float* __restrict__ base, uint32_t ld, uint64_t n, uint32_t ntrees,
                                const uint32_t* __restrict__ ids, const int32_t* __restrict__ owner, NodeArrays na,
                                int32_t level, uint64_t* __restrict__ flags) {
  uint64_t total = n * ntrees;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
    int32_t v = owner[g];
    uint64_t f = 0;
    if (na.split_at[v] == level + 1) {
      float x = __ldg(base + (uint64_t)ids[g] * ld + na.dim[v]);
      float c = na.val[v];
      if (x < c) f = 1ULL << 32;
      else if (x <= c) f = 1ULL;
    }
    flags[g] = f;
  }
}

// One thread per active node: split index, children, and the next level's activity flags.
__global__ void finish_nodes_kernel(NodeArrays na, uint64_t n, const int32_t* __restrict__ active, uint32_t nactive,
                                    const uint32_t* __restrict__ child_off, const uint64_t* __restrict__ pref,
                                    int32_t base_node, int32_t level, int phaseB, uint32_t S,
                                    uint32_t* __restrict__ mids, uint32_t* __restrict__ next_flag,
                                    int32_t* __restrict__ next_cand) {
  uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nactive) return;
  int32_t v = active[a];
  next_flag[2 * a] = next_flag[2 * a + 1] = 0;
  if (na.split_at[v] != level + 1) return;
  uint32_t s = na.start[v], e = na.end[v], count = e - s;
  uint64_t g0 = (uint64_t)na.tree[v] * n + s, g1 = g0 + count;
  uint64_t d = pref[g1] - pref[g0];
  uint32_t nless = (uint32_t)(d >> 32), neq = (uint32_t)(d & 0xffffffffu);
  uint32_t lim1 = nless, lim2 = nless + neq;
  uint32_t index;  // meanSplit's split-index rule (kdtreeub_index.hpp:942-950)
  if (lim1 > count / 2) index = lim1;
  else if (lim2 < count / 2) index = lim2;
  else index = count / 2;
  if ((lim1 == count) || (lim2 == 0)) index = count / 2;
  mids[a] = index;
  int32_t L = base_node + 2 * (int32_t)child_off[a], R = L + 1;
  na.left[v] = L;
  na.right[v] = R;
  int32_t t = na.tree[v];
  na.start[L] = s;
  na.end[L] = s + index;
  na.start[R] = s + index;
  na.end[R] = e;
  na.tree[L] = na.tree[R] = t;
  na.level[L] = na.level[R] = level + 1;
  na.left[L] = na.right[L] = na.left[R] = na.right[R] = -1;
  na.dim[L] = na.dim[R] = 0;  // value-initialised Node (kdtreeub_index.hpp:1249)
  na.val[L] = na.val[R] = 0.f;
  na.split_at[L] = na.split_at[R] = 0;
  next_cand[2 * a] = L;
  next_cand[2 * a + 1] = R;
  if (phaseB) {
    next_flag[2 * a] = next_flag[2 * a + 1] = 1;
  } else {
    next_flag[2 * a] = index > S;
    next_flag[2 * a + 1] = count - index > S;
  }
}

// Stable three-way scatter of the ids of split nodes; owner[] switches to the children.
__global__ void scatter_kernel(uint64_t n, uint32_t ntrees, const uint32_t* __restrict__ ids_in,
                               uint32_t* __restrict__ ids_out, int32_t* __restrict__ owner, NodeArrays na,
                               int32_t level, const uint64_t* __restrict__ pref) {
  uint64_t total = n * ntrees;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
    int32_t v = owner[g];
    uint32_t id = ids_in[g];
    if (na.split_at[v] != level + 1) {
      ids_out[g] = id;
      continue;
    }
    uint32_t s = na.start[v], count = na.end[v] - s;
    uint64_t g0 = (uint64_t)na.tree[v] * n + s;
    uint64_t pg = pref[g] - pref[g0], pt = pref[g0 + count] - pref[g0];
    uint32_t rl = (uint32_t)(pg >> 32), re = (uint32_t)pg, nl = (uint32_t)(pt >> 32), ne = (uint32_t)pt;
    uint32_t off = (uint32_t)(g - g0);
    uint64_t fg = pref[g + 1] - pref[g];
    uint32_t np;
    if (fg >> 32) np = rl;
    else if (fg & 0xffffffffu) np = nl + re;
    else np = nl + ne + (off - rl - re);
    ids_out[g0 + np] = id;
    uint32_t mid = na.end[na.left[v]] - s;
    owner[g] = off < mid ? na.left[v] : na.right[v];
  }
}

__global__ void compact_kernel(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                               const int32_t* __restrict__ cand, uint32_t m, int32_t* __restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m && flag[i]) out[pos[i]] = cand[i];
}

__global__ void to_dnodes_kernel(NodeArrays na, uint32_t nnodes, DNode* __restrict__ out) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nnodes) return;
  DNode d;
  d.div_dim = na.dim[v];
  d.div_val = na.val[v];
  if (na.left[v] >= 0) {
    d.left = na.left[v];
    d.right = na.right[v];
  } else {
    d.left = -(int32_t)na.start[v] - 1;
    d.right = (int32_t)na.end[v];
  }
  out[v] = d;
}

// Leaves per subtree for the nodes [lo, hi) of one level; deeper levels are already done.
// Children's leaf counts next to each node, so that the search descent gets them with the node.
__global__ void child_counts_kernel(const DNode* __restrict__ nodes, const int32_t* __restrict__ nleaf, uint32_t m,
                                    uint2* __restrict__ cnl) {
  uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= m) return;
  DNode d = nodes[v];
  cnl[v] = d.left < 0 ? make_uint2(0, 0) : make_uint2((uint32_t)nleaf[d.left], (uint32_t)nleaf[d.right]);
}

__global__ void leaf_count_kernel(const int32_t* __restrict__ left, const int32_t* __restrict__ right, int32_t lo,
                                  int32_t hi, int32_t* __restrict__ nleaf) {
  int32_t v = lo + (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (v >= hi) return;
  nleaf[v] = left[v] < 0 ? 1 : nleaf[left[v]] + nleaf[right[v]];
}

static unsigned grid_for(uint64_t total, int threads) {
  return (unsigned)std::min<uint64_t>((total + threads - 1) / threads, 152ull * 32);
}

int build_forest(efg_index* idx, uint32_t ntrees) {
  cudaStream_t s = idx->stream;
  Forest& F = idx->forest;
  F.release();
  const uint64_t n = idx->n;
  const uint64_t total = n * ntrees;
  const uint32_t S = idx->bp.S, tns = idx->bp.leaf_size;
  const uint64_t seed = idx->bp.seed;
  const uint64_t cap_nodes = 2 * total + ntrees;  // each split adds two nodes; at most n-1 splits per tree

  EFG_TRY(F.leaves.reserve(total));
  LocalBuf<uint32_t> ids_b;
  LocalBuf<int32_t> owner;
  LocalBuf<uint64_t> flags, pref, scan_tmp;
  EFG_TRY(ids_b.reserve(total));
  EFG_TRY(owner.reserve(total));
  EFG_TRY(flags.reserve(total));
  EFG_TRY(pref.reserve(total + 1));
  EFG_TRY(scan_tmp.reserve(scan_tmp_elems<uint64_t>(total) + 1));
  EFG_TRY(F.n_start.reserve(cap_nodes));
  EFG_TRY(F.n_end.reserve(cap_nodes));
  EFG_TRY(F.n_tree.reserve(cap_nodes));
  EFG_TRY(F.n_level.reserve(cap_nodes));
  EFG_TRY(F.n_left.reserve(cap_nodes));
  EFG_TRY(F.n_right.reserve(cap_nodes));
  LocalBuf<int32_t> n_dim, n_split;
  LocalBuf<float> n_val;
  EFG_TRY(n_dim.reserve(cap_nodes));
  EFG_TRY(n_split.reserve(cap_nodes));
  EFG_TRY(n_val.reserve(cap_nodes));
  NodeArrays na{F.n_start.p, F.n_end.p, F.n_tree.p, F.n_level.p, F.n_left.p, F.n_right.p, n_dim.p, n_split.p, n_val.p};

  // active lists and per-level scratch (active count <= total)
  uint64_t cap_act = std::max<uint64_t>(total, 2048);
  LocalBuf<int32_t> act, next_cand;
  LocalBuf<uint32_t> split_flag, child_off, mids, next_flag, next_pos, tmp32;
  EFG_TRY(act.reserve(cap_act));
  EFG_TRY(next_cand.reserve(2 * cap_act));
  EFG_TRY(split_flag.reserve(cap_act));
  EFG_TRY(child_off.reserve(cap_act + 1));
  EFG_TRY(mids.reserve(cap_act));
  EFG_TRY(next_flag.reserve(2 * cap_act));
  EFG_TRY(next_pos.reserve(2 * cap_act + 1));
  EFG_TRY(tmp32.reserve(scan_tmp_elems<uint32_t>(2 * cap_act) + 1));

  ScopedEvents<2> evs;
  cudaEvent_t e0 = evs.e[0], e1 = evs.e[1];
  cudaEventRecord(e0, s);
  perm_init_kernel<<<grid_for(total, 256), 256, 0, s>>>(F.leaves.p, owner.p, n, ntrees, seed);
  roots_init_kernel<<<(ntrees + 255) / 256, 256, 0, s>>>(na, ntrees, n);
  std::vector<int32_t> roots(ntrees);
  for (uint32_t t = 0; t < ntrees; ++t) roots[t] = (int32_t)t;
  EFG_CUDA(cudaMemcpyAsync(act.p, roots.data(), ntrees * 4, cudaMemcpyHostToDevice, s));
  EFG_CUDA(cudaGetLastError());

  uint32_t nactive = ntrees;
  int32_t nnodes = (int32_t)ntrees;
  std::vector<std::pair<int32_t, int32_t>> level_ranges{{0, (int32_t)ntrees}};
  bool phaseA = true;
  int32_t level = 0;
  uint32_t* cur = F.leaves.p;
  uint32_t* other = ids_b.p;
  const int wpb = 8;
  size_t smem = (size_t)wpb * idx->dim * sizeof(float);
  if (smem > 48 * 1024)
    EFG_CUDA(cudaFuncSetAttribute(split_stats_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  while (nactive > 0) {
    if (phaseA && nactive >= 1100) phaseA = false;
    int phaseB = phaseA ? 0 : 1;
    split_stats_kernel<<<(nactive + wpb - 1) / wpb, wpb * 32, smem, s>>>(idx->d_base, idx->dim, idx->ld, n, cur, na,
                                                                         act.p, nactive, level, phaseB, tns, seed,
                                                                         split_flag.p);
    EFG_CUDA(cudaGetLastError());
    EFG_TRY(device_scan<uint32_t>(split_flag.p, nactive, child_off.p, tmp32.p, s));
    classify_kernel<<<grid_for(total, 256), 256, 0, s>>>(idx->d_base, idx->ld, n, ntrees, cur, owner.p, na, level,
                                                         flags.p);
    EFG_CUDA(cudaGetLastError());
    EFG_TRY(device_scan<uint64_t>(flags.p, total, pref.p, scan_tmp.p, s));
    uint32_t nsplit = 0;
    EFG_CUDA(cudaMemcpyAsync(&nsplit, child_off.p + nactive, 4, cudaMemcpyDeviceToHost, s));
    finish_nodes_kernel<<<(nactive + 255) / 256, 256, 0, s>>>(na, n, act.p, nactive, child_off.p, pref.p, nnodes,
                                                              level, phaseB, S, mids.p, next_flag.p, next_cand.p);
    EFG_CUDA(cudaGetLastError());
    scatter_kernel<<<grid_for(total, 256), 256, 0, s>>>(n, ntrees, cur, other, owner.p, na, level, pref.p);
    EFG_CUDA(cudaGetLastError());
    std::swap(cur, other);
    EFG_TRY(device_scan<uint32_t>(next_flag.p, 2ull * nactive, next_pos.p, tmp32.p, s));
    compact_kernel<<<(2 * nactive + 255) / 256, 256, 0, s>>>(next_flag.p, next_pos.p, next_cand.p, 2 * nactive,
                                                             act.p);
    EFG_CUDA(cudaGetLastError());
    uint32_t nnext = 0;
    EFG_CUDA(cudaMemcpyAsync(&nnext, next_pos.p + 2ull * nactive, 4, cudaMemcpyDeviceToHost, s));
    EFG_CUDA(cudaStreamSynchronize(s));
    level_ranges.push_back({nnodes, nnodes + 2 * (int32_t)nsplit});
    nnodes += 2 * (int32_t)nsplit;
    nactive = nnext;
    ++level;
    if ((uint64_t)nnodes + 2ull * nactive > cap_nodes || level > 4096)
      return fail(EFG_ERR_DEVICE_LIMIT, "tree build exceeded its node capacity");
  }
  if (cur != F.leaves.p)
    EFG_CUDA(cudaMemcpyAsync(F.leaves.p, cur, total * 4, cudaMemcpyDeviceToDevice, s));
  EFG_TRY(F.nodes.reserve(nnodes));
  to_dnodes_kernel<<<(nnodes + 255) / 256, 256, 0, s>>>(na, (uint32_t)nnodes, F.nodes.p);
  EFG_TRY(F.nleaf.reserve(nnodes));
  for (size_t l = level_ranges.size(); l-- > 0;) {
    int32_t lo = level_ranges[l].first, hi = level_ranges[l].second;
    if (hi > lo) leaf_count_kernel<<<(hi - lo + 255) / 256, 256, 0, s>>>(na.left, na.right, lo, hi, F.nleaf.p);
  }
  EFG_TRY(F.cnl.reserve(nnodes));
  child_counts_kernel<<<(nnodes + 255) / 256, 256, 0, s>>>(F.nodes.p, F.nleaf.p, (uint32_t)nnodes, F.cnl.p);
  EFG_CUDA(cudaGetLastError());
  // keep dim/val in the DNode array; the SoA start/end/tree/level/left/right stay for the merge
  EFG_TRY(F.d_roots.reserve(ntrees));
  EFG_CUDA(cudaMemcpyAsync(F.d_roots.p, roots.data(), ntrees * 4, cudaMemcpyHostToDevice, s));
  cudaEventRecord(e1, s);
  EFG_CUDA(cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  idx->bstats.trees_ms = ms;
  F.ntrees = ntrees;
  F.n = n;
  F.nnodes = (uint64_t)nnodes;
  F.roots = roots;
  F.has_soa = true;
  ids_b.release();
  owner.release();
  flags.release();
  pref.release();
  scan_tmp.release();
  n_dim.release();
  n_split.release();
  n_val.release();
  return EFG_OK;
}

int upload_forest(efg_index* idx, const std::vector<HNode>& nodes, const std::vector<int32_t>& roots,
                  const std::vector<uint32_t>& leaves, uint32_t ntrees) {
  Forest& F = idx->forest;
  F.release();
  std::vector<DNode> dn(nodes.size());
  std::vector<int32_t> lvl(nodes.size()), tr(nodes.size(), 0), l(nodes.size()), r(nodes.size());
  std::vector<uint32_t> st(nodes.size()), en(nodes.size());
  for (size_t i = 0; i < nodes.size(); ++i) {
    const HNode& h = nodes[i];
    dn[i].div_dim = h.div_dim;
    dn[i].div_val = h.div_val;
    if (h.left >= 0) {
      dn[i].left = h.left;
      dn[i].right = h.right;
    } else {
      dn[i].left = -(int32_t)h.start - 1;
      dn[i].right = (int32_t)h.end;
    }
    lvl[i] = h.level;
    l[i] = h.left;
    r[i] = h.right;
    st[i] = (uint32_t)h.start;
    en[i] = (uint32_t)h.end;
  }
  for (uint32_t t = 0; t < ntrees; ++t) {  // tree id of every node
    std::vector<int32_t> stack{roots[t]};
    while (!stack.empty()) {
      int32_t v = stack.back();
      stack.pop_back();
      tr[v] = (int32_t)t;
      if (l[v] >= 0) {
        stack.push_back(l[v]);
        stack.push_back(r[v]);
      }
    }
  }
  size_t m = nodes.size();
  std::vector<int32_t> nl(m, 0);
  for (uint32_t t = 0; t < ntrees; ++t) {  // post-order leaf counts
    std::vector<std::pair<int32_t, bool>> stack{{roots[t], false}};
    while (!stack.empty()) {
      auto [v, done] = stack.back();
      stack.pop_back();
      if (l[v] < 0) {
        nl[v] = 1;
      } else if (done) {
        nl[v] = nl[l[v]] + nl[r[v]];
      } else {
        stack.push_back({v, true});
        stack.push_back({l[v], false});
        stack.push_back({r[v], false});
      }
    }
  }
  EFG_TRY(F.nleaf.reserve(m));
  EFG_CUDA(cudaMemcpy(F.nleaf.p, nl.data(), m * 4, cudaMemcpyHostToDevice));
  EFG_TRY(F.nodes.reserve(m));
  EFG_TRY(F.d_roots.reserve(ntrees));
  EFG_TRY(F.leaves.reserve(leaves.size()));
  EFG_TRY(F.n_left.reserve(m));
  EFG_TRY(F.n_right.reserve(m));
  EFG_TRY(F.n_level.reserve(m));
  EFG_TRY(F.n_tree.reserve(m));
  EFG_TRY(F.n_start.reserve(m));
  EFG_TRY(F.n_end.reserve(m));
  EFG_CUDA(cudaMemcpy(F.nodes.p, dn.data(), m * sizeof(DNode), cudaMemcpyHostToDevice));
  EFG_TRY(F.cnl.reserve(m));
  child_counts_kernel<<<(unsigned)((m + 255) / 256), 256>>>(F.nodes.p, F.nleaf.p, (uint32_t)m, F.cnl.p);
  EFG_CUDA(cudaGetLastError());
  EFG_CUDA(cudaStreamSynchronize(0));  // searches run on a non-blocking stream
  EFG_CUDA(cudaMemcpy(F.d_roots.p, roots.data(), ntrees * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.leaves.p, leaves.data(), leaves.size() * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.n_left.p, l.data(), m * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.n_right.p, r.data(), m * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.n_level.p, lvl.data(), m * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.n_tree.p, tr.data(), m * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.n_start.p, st.data(), m * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(F.n_end.p, en.data(), m * 4, cudaMemcpyHostToDevice));
  F.ntrees = ntrees;
  F.n = idx->n;
  F.nnodes = m;
  F.roots = roots;
  F.has_soa = true;
  return EFG_OK;
}

int download_forest(efg_index* idx, std::vector<HNode>& nodes, std::vector<uint32_t>& leaves) {
  Forest& F = idx->forest;
  size_t m = F.nnodes;
  std::vector<DNode> dn(m);
  std::vector<int32_t> l(m), r(m), lvl(m);
  std::vector<uint32_t> st(m), en(m);
  EFG_CUDA(cudaMemcpy(dn.data(), F.nodes.p, m * sizeof(DNode), cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(l.data(), F.n_left.p, m * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(r.data(), F.n_right.p, m * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(lvl.data(), F.n_level.p, m * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st.data(), F.n_start.p, m * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(en.data(), F.n_end.p, m * 4, cudaMemcpyDeviceToHost));
  nodes.resize(m);
  for (size_t i = 0; i < m; ++i) {
    nodes[i].div_dim = dn[i].div_dim;
    nodes[i].div_val = dn[i].div_val;
    nodes[i].start = st[i];
    nodes[i].end = en[i];
    nodes[i].left = l[i];
    nodes[i].right = r[i];
    nodes[i].level = lvl[i];
  }
  leaves.resize((size_t)F.ntrees * F.n);
  EFG_CUDA(cudaMemcpy(leaves.data(), F.leaves.p, leaves.size() * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

}  // namespace efg
