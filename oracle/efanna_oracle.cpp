// TEST INFRASTRUCTURE ONLY — the CPU oracle for the efanna_gb300 hot path.
//
// This file restates, on the CPU, the algorithms of EFANNA's kNN-graph hot path so that the
// CUDA implementation in efanna_gb300/ can be checked against it.  Nothing in the product links
// or loads this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
//
// Two modes are restated:
//
//   ORC_SEQ   — the reference exactly as its single-threaded OpenMP build runs it: the same
//               std::rand()/random_shuffle and std::mt19937 draws, the same Hoare partition,
//               the same arrival order of neighbour-list inserts, and the same quirks (zeroed
//               pool slots beyond L feeding `radius`, the reused rank `r` in join's found test).
//               Its graph, tree and result files are pinned byte-for-byte against the reference
//               compiled from its own sources (oracle/Makefile, OMP_NUM_THREADS=1).
//   ORC_CANON — the order-independent restatement that a data-parallel implementation can
//               reproduce exactly: counter-hash random numbers instead of global generators,
//               stable three-way partitions instead of Hoare swaps, and every neighbour-list
//               insert applied in ascending (dist, id, source, side) order per target node.
//               The CUDA build is required to match this mode bit-for-bit.
//
// Reference files cited below are paths inside the ZJULearning/efanna project.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <random>
#include <set>
#include <unordered_map>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

enum { MODE_SEQ = 0, MODE_CANON = 1, MODE_OMP = 2 };

// ----------------------------------------------------------------------------------------------
// Squared L2 distances.
// ----------------------------------------------------------------------------------------------

// L2DistanceAVX::compare (general/distance.hpp:299-323): eight running lane sums, the (single)
// 8-float tail block first, then 16-float blocks, then a left-to-right horizontal add.  Only 8
// tail floats are summed even when the padded tail holds 16 or 24 (the reference's behaviour for
// d mod 32 in {9..24}).  Elements past `size` (row padding) count as zero here.
static float l2_avx(const float* a, const float* b, size_t size) {
  unsigned D = (unsigned)((size + 7) & ~7U);
  unsigned DR = D % 32;
  unsigned DD = D - DR;
  float sum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  auto lane = [&](unsigned base) {
    if (base + 8 <= size) {  // full block: no padding involved
      for (unsigned k = 0; k < 8; ++k) {
        float t = a[base + k] - b[base + k];
        t = t * t;
        sum[k] = sum[k] + t;
      }
      return;
    }
    for (unsigned k = 0; k < 8; ++k) {
      unsigned idx = base + k;
      float x = idx < size ? a[idx] : 0.0f;
      float y = idx < size ? b[idx] : 0.0f;
      float t = x - y;
      t = t * t;
      sum[k] = sum[k] + t;
    }
  };
  if (DR) lane(DD);
  for (unsigned i = 0; i < DD; i += 16) {
    lane(i);
    lane(i + 8);
  }
  return sum[0] + sum[1] + sum[2] + sum[3] + sum[4] + sum[5] + sum[6] + sum[7];
}

// L2Distance::compare (general/distance.hpp:125-147): groups of four, then the 0-3 tail.
static float l2_scalar(const float* a, const float* b, size_t size) {
  float result = 0.0f;
  size_t i = 0;
  for (; i + 3 < size; i += 4) {
    float d0 = a[i] - b[i], d1 = a[i + 1] - b[i + 1], d2 = a[i + 2] - b[i + 2], d3 = a[i + 3] - b[i + 3];
    result += d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
  }
  for (; i < size; ++i) {
    float d0 = a[i] - b[i];
    result += d0 * d0;
  }
  return result;
}

// Sequential mode measures with L2DistanceAVX, the class every reference sample uses; canonical
// mode with the plain squared L2 (L2Distance), which the CUDA kernels compute (in any summation
// order the two agree exactly on integer-valued data).  They differ beyond rounding only for
// d mod 32 in {9..24}, where L2DistanceAVX drops part of the tail.
struct Data {
  const float* p;
  size_t n, d, ld;
  int mode;
  const float* row(size_t i) const { return p + i * ld; }
  float distq(const float* a, const float* b) const { return mode != 1 ? l2_avx(a, b, d) : l2_scalar(a, b, d); }
  float dist(size_t i, size_t j) const { return distq(row(i), row(j)); }
};

// ----------------------------------------------------------------------------------------------
// Counter-hash random numbers (canonical mode).  The CUDA build implements the same functions.
// ----------------------------------------------------------------------------------------------
enum : uint64_t {
  TAG_PERM = 1, TAG_DIM = 2, TAG_EXTRA = 3, TAG_GENRAND = 4, TAG_TOPUP = 5,
  TAG_RNEW = 6, TAG_ROLD = 7, TAG_SFILL = 8
};
static inline uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline uint64_t hash4(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b, uint64_t c) {
  return mix64(mix64(mix64(mix64(seed ^ (tag * 0x9E3779B97F4A7C15ULL)) ^ a) ^ b) ^ c);
}
struct CRng {  // a counter stream: next() = high 32 bits of mix64(key ^ ctr * odd constant)
  uint64_t key, ctr;
  CRng(uint64_t k) : key(k), ctr(0) {}
  uint32_t next() { ++ctr; return (uint32_t)(mix64(key ^ (ctr * 0xD1B54A32D192ED03ULL)) >> 32); }
};
// Balanced 4-round Feistel permutation of [0, 2^b) with cycle walking onto [0, n).
static uint32_t feistel_perm(uint32_t i, uint32_t n, uint64_t key) {
  unsigned b = 2;
  while ((1ULL << b) < (uint64_t)n) b += 2;
  unsigned half = b / 2;
  uint32_t mask = (uint32_t)((1ULL << half) - 1);
  uint32_t x = i;
  do {
    uint32_t L = x >> half, R = x & mask;
    for (uint32_t r = 0; r < 4; ++r) {
      uint32_t F = (uint32_t)mix64(key ^ ((uint64_t)r << 48) ^ R) & mask;
      uint32_t nl = R, nr = L ^ F;
      L = nl; R = nr;
    }
    x = (L << half) | R;
  } while (x >= n);
  return x;
}

// ----------------------------------------------------------------------------------------------
// Randomised truncated KD-trees.
// ----------------------------------------------------------------------------------------------
struct Node {
  int div_dim;
  float div_val;
  uint64_t start, end;
  int32_t left, right;  // -1 for a leaf
};
struct Forest {
  uint64_t n = 0, dim = 0;
  std::vector<std::vector<Node>> nodes;  // per tree
  std::vector<int32_t> roots;
  std::vector<std::vector<uint32_t>> leaves;  // LeafLists
};

static const unsigned SAMPLE_NUM = 100, RAND_DIM = 5;  // kdtreeub_index.hpp:1094,1102

// selectDivision (kdtreeub_index.hpp:974-999): top RAND_DIM variances, strict comparisons.
static int top_dims(const float* v, size_t d, size_t* topind) {
  int num = 0;
  for (size_t i = 0; i < d; ++i) {
    if ((num < (int)RAND_DIM) || (v[i] > v[topind[num - 1]])) {
      if (num < (int)RAND_DIM) topind[num++] = i;
      else topind[num - 1] = i;
      int j = num - 1;
      while (j > 0 && v[topind[j]] > v[topind[j - 1]]) {
        std::swap(topind[j], topind[j - 1]);
        --j;
      }
    }
  }
  return num;
}

// meanSplit's statistics (kdtreeub_index.hpp:902-937): mean and variance over the first
// min(SAMPLE_NUM+1, count) ids, summed in id order, mean scaled by the float reciprocal.
static void sample_stats(const Data& X, const unsigned* ids, unsigned count, std::vector<float>& mean,
                         std::vector<float>& var) {
  size_t d = X.d;
  mean.assign(d, 0.0f);
  var.assign(d, 0.0f);
  unsigned cnt = std::min((unsigned)SAMPLE_NUM + 1, count);
  for (unsigned j = 0; j < cnt; ++j) {
    const float* v = X.row(ids[j]);
    for (size_t k = 0; k < d; ++k) mean[k] += v[k];
  }
  float div_factor = 1.0f / (float)cnt;
  for (size_t k = 0; k < d; ++k) mean[k] *= div_factor;
  for (unsigned j = 0; j < cnt; ++j) {
    const float* v = X.row(ids[j]);
    for (size_t k = 0; k < d; ++k) {
      float dist = v[k] - mean[k];
      var[k] += dist * dist;
    }
  }
}

// Split index rule of meanSplit (kdtreeub_index.hpp:942-950).
static unsigned split_index(unsigned count, unsigned lim1, unsigned lim2) {
  unsigned index;
  if (lim1 > count / 2) index = lim1;
  else if (lim2 < count / 2) index = lim2;
  else index = count / 2;
  if ((lim1 == count) || (lim2 == 0)) index = count / 2;
  return index;
}

// planeSplit (kdtreeub_index.hpp:954-973): the two-pass Hoare partition.
static void plane_split_hoare(const Data& X, unsigned* indices, unsigned count, unsigned cutdim, float cutval,
                              unsigned& lim1, unsigned& lim2) {
  int left = 0;
  int right = (int)count - 1;
  for (;;) {
    while (left <= right && X.row(indices[left])[cutdim] < cutval) ++left;
    while (left <= right && X.row(indices[right])[cutdim] >= cutval) --right;
    if (left > right) break;
    std::swap(indices[left], indices[right]);
    ++left;
    --right;
  }
  lim1 = left;
  right = (int)count - 1;
  for (;;) {
    while (left <= right && X.row(indices[left])[cutdim] <= cutval) ++left;
    while (left <= right && X.row(indices[right])[cutdim] > cutval) --right;
    if (left > right) break;
    std::swap(indices[left], indices[right]);
    ++left;
    --right;
  }
  lim2 = left;
}

// meanSplit (kdtreeub_index.hpp:902-953) with the reference's generator and partition.
static void mean_split_seq(const Data& X, std::mt19937& rng, unsigned* indices, unsigned count, unsigned& index,
                           unsigned& cutdim, float& cutval) {
  std::vector<float> mean, var;
  sample_stats(X, indices, count, mean, var);
  size_t topind[RAND_DIM];
  int num = top_dims(var.data(), X.d, topind);
  int rnd = rng() % num;
  cutdim = (unsigned)topind[rnd];
  cutval = mean[cutdim];
  unsigned lim1, lim2;
  plane_split_hoare(X, indices, count, cutdim, cutval, lim1, lim2);
  index = split_index(count, lim1, lim2);
}

static int32_t new_node(std::vector<Node>& v, int div_dim, uint64_t s, uint64_t e) {
  Node nd;
  nd.div_dim = div_dim;
  nd.div_val = 0.0f;
  nd.start = s;
  nd.end = e;
  nd.left = nd.right = -1;
  v.push_back(nd);
  return (int32_t)v.size() - 1;
}

// DFSbuild (kdtreeub_index.hpp:1138-1167).
static void dfs_build(const Data& X, std::vector<Node>& nodes, int32_t node, std::mt19937& rng, unsigned* indices,
                      unsigned count, unsigned offset, unsigned tns) {
  if (count <= tns) {
    nodes[node].div_dim = -1;
    nodes[node].left = nodes[node].right = -1;
    nodes[node].start = offset;
    nodes[node].end = offset + count;
    return;
  }
  unsigned idx, cutdim;
  float cutval;
  mean_split_seq(X, rng, indices, count, idx, cutdim, cutval);
  nodes[node].div_dim = (int)cutdim;
  nodes[node].div_val = cutval;
  nodes[node].start = offset;
  nodes[node].end = offset + count;
  int32_t l = new_node(nodes, 0, 0, 0);
  int32_t r = new_node(nodes, 0, 0, 0);
  nodes[node].left = l;
  nodes[node].right = r;
  dfs_build(X, nodes, l, rng, indices, idx, offset, tns);
  dfs_build(X, nodes, r, rng, indices + idx, count - idx, offset + idx, tns);
}

// The tree part of buildTrees / initGraph (kdtreeub_index.hpp:1192-1276, 1295-1363), run as the
// single-threaded OpenMP build runs it: per-tree random_shuffle with std::rand(), BFS levels while
// fewer than 1100 nodes are active (each node reseeds mt19937(1998 ^ thread 0)), then DFSbuild.
static void build_forest_seq(const Data& X, unsigned T, unsigned S, unsigned tns, Forest& F) {
  unsigned N = (unsigned)X.n;
  const unsigned seed = 1998;
  F.n = X.n;
  F.dim = X.d;
  F.nodes.assign(T, {});
  F.roots.assign(T, 0);
  F.leaves.assign(T, {});
  std::vector<std::pair<unsigned, int32_t>> active, next;
  for (unsigned t = 0; t < T; ++t) {
    F.roots[t] = new_node(F.nodes[t], -1, 0, N);
    active.push_back({t, F.roots[t]});
  }
  for (unsigned t = 0; t < T; ++t) {
    std::vector<unsigned>& ids = F.leaves[t];
    ids.resize(N);
    for (unsigned i = 0; i < N; ++i) ids[i] = i;
    std::random_shuffle(ids.begin(), ids.end());
  }
  while (!active.empty() && active.size() < 1100) {
    next.clear();
    for (auto& a : active) {
      unsigned t = a.first;
      int32_t ni = a.second;
      std::mt19937 rng(seed ^ 0);
      std::vector<Node>& nodes = F.nodes[t];
      unsigned mid, cutdim;
      float cutval;
      uint64_t s = nodes[ni].start, e = nodes[ni].end;
      mean_split_seq(X, rng, &F.leaves[t][0] + s, (unsigned)(e - s), mid, cutdim, cutval);
      nodes[ni].div_dim = (int)cutdim;
      nodes[ni].div_val = cutval;
      int32_t l = new_node(nodes, 0, s, s + mid);
      int32_t r = new_node(nodes, 0, s + mid, e);
      nodes[ni].left = l;
      nodes[ni].right = r;
      if (mid > S) next.push_back({t, l});
      if (e - (s + mid) > S) next.push_back({t, r});
    }
    active.swap(next);
  }
  for (auto& a : active) {
    unsigned t = a.first;
    int32_t ni = a.second;
    std::mt19937 rng(seed ^ 0);
    uint64_t s = F.nodes[t][ni].start, e = F.nodes[t][ni].end;
    dfs_build(X, F.nodes[t], ni, rng, &F.leaves[t][0] + s, (unsigned)(e - s), (unsigned)s, tns);
  }
}

// Canonical tree build: the same level structure (BFS rule while < 1100 nodes are active, then
// split-while-larger-than-TNS), the same statistics and split-index rule, but a Feistel
// permutation per tree, a counter-hash choice among the top variances, and a stable three-way
// partition (< cut, == cut, > cut) of each node's id range.
static void build_forest_canon(const Data& X, unsigned T, unsigned S, unsigned tns, uint64_t seed, Forest& F) {
  uint32_t N = (uint32_t)X.n;
  F.n = X.n;
  F.dim = X.d;
  F.nodes.assign(T, {});
  F.roots.assign(T, 0);
  F.leaves.assign(T, {});
  std::vector<std::pair<unsigned, int32_t>> active, next;
  for (unsigned t = 0; t < T; ++t) {
    F.roots[t] = new_node(F.nodes[t], -1, 0, N);
    active.push_back({t, F.roots[t]});
    uint64_t key = hash4(seed, TAG_PERM, t, 0, 0);
    F.leaves[t].resize(N);
    for (uint32_t i = 0; i < N; ++i) F.leaves[t][i] = feistel_perm(i, N, key);
  }
  bool phaseA = true;
  uint64_t level = 0;
  std::vector<float> mean, var;
  std::vector<unsigned> tmp;
  while (!active.empty()) {
    if (phaseA && active.size() >= 1100) phaseA = false;
    next.clear();
    for (auto& a : active) {
      unsigned t = a.first;
      int32_t ni = a.second;
      std::vector<Node>& nodes = F.nodes[t];
      uint64_t s = nodes[ni].start, e = nodes[ni].end;
      unsigned count = (unsigned)(e - s);
      if (!phaseA && count <= tns) {
        nodes[ni].div_dim = -1;
        continue;
      }
      unsigned* ids = &F.leaves[t][0] + s;
      sample_stats(X, ids, count, mean, var);
      size_t topind[RAND_DIM];
      int num = top_dims(var.data(), X.d, topind);
      uint32_t rnd = (uint32_t)(hash4(seed, TAG_DIM, t, level, s) % (uint64_t)num);
      unsigned cutdim = (unsigned)topind[rnd];
      float cutval = mean[cutdim];
      tmp.clear();
      unsigned nless = 0, neq = 0;
      for (unsigned j = 0; j < count; ++j) {
        float v = X.row(ids[j])[cutdim];
        if (v < cutval) ++nless;
        else if (v <= cutval) ++neq;
      }
      tmp.resize(count);
      unsigned pl = 0, pe = nless, pg = nless + neq;
      for (unsigned j = 0; j < count; ++j) {
        float v = X.row(ids[j])[cutdim];
        if (v < cutval) tmp[pl++] = ids[j];
        else if (v <= cutval) tmp[pe++] = ids[j];
        else tmp[pg++] = ids[j];
      }
      std::copy(tmp.begin(), tmp.end(), ids);
      unsigned mid = split_index(count, nless, nless + neq);
      nodes[ni].div_dim = (int)cutdim;
      nodes[ni].div_val = cutval;
      int32_t l = new_node(nodes, 0, s, s + mid);
      int32_t r = new_node(nodes, 0, s + mid, e);
      nodes[ni].left = l;
      nodes[ni].right = r;
      if (phaseA) {
        if (mid > S) next.push_back({t, l});
        if (count - mid > S) next.push_back({t, r});
      } else {
        next.push_back({t, l});
        next.push_back({t, r});
      }
    }
    active.swap(next);
    ++level;
  }
}

// Trees file (kdtreeub_index.hpp:197-242, 658-671): header {u32 K, u32 trees, u64 N, u64 dim};
// per tree {i32 node_num, i32 node_size=48, node_num post-order 40-byte records}; then the leaf
// lists.  Child pointers are written as 0 for leaves and 1 for internal nodes (the loader ignores
// them; the reference writes raw addresses).
static void write_post(std::ofstream& out, const std::vector<Node>& nodes, int32_t ni, int& cnt) {
  const Node& nd = nodes[ni];
  if (nd.left >= 0) write_post(out, nodes, nd.left, cnt);
  if (nd.right >= 0) write_post(out, nodes, nd.right, cnt);
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
}
static int save_forest(const Forest& F, const char* path, uint32_t K) {
  std::ofstream out(path, std::ios::binary);
  if (!out.is_open()) return -1;
  uint32_t tn = (uint32_t)F.nodes.size();
  out.write((const char*)&K, 4);
  out.write((const char*)&tn, 4);
  out.write((const char*)&F.n, 8);
  out.write((const char*)&F.dim, 8);
  for (uint32_t t = 0; t < tn; ++t) {
    std::streampos pos = out.tellp();
    int zero = 0, nsz = 48;
    out.write((const char*)&zero, 4);
    out.write((const char*)&nsz, 4);
    int cnt = 0;
    write_post(out, F.nodes[t], F.roots[t], cnt);
    std::streampos endp = out.tellp();
    out.seekp(pos);
    out.write((const char*)&cnt, 4);
    out.seekp(endp);
  }
  for (uint32_t t = 0; t < tn; ++t) out.write((const char*)F.leaves[t].data(), 4 * F.n);
  return out.good() ? 0 : -1;
}
// loadTrees (kdtreeub_index.hpp:139-196) with DepthFirstBuildTree's stack merge (:672-700).
static Forest* load_forest(const char* path) {
  std::ifstream in(path, std::ios::binary);
  if (!in.is_open()) return nullptr;
  uint32_t K, tn;
  uint64_t num, dim;
  in.read((char*)&K, 4);
  in.read((char*)&tn, 4);
  in.read((char*)&num, 8);
  in.read((char*)&dim, 8);
  if (!in) return nullptr;
  Forest* F = new Forest();
  F->n = num;
  F->dim = dim;
  F->nodes.assign(tn, {});
  F->roots.assign(tn, -1);
  for (uint32_t t = 0; t < tn; ++t) {
    int node_num, node_size;
    in.read((char*)&node_num, 4);
    in.read((char*)&node_size, 4);
    std::vector<Node>& nodes = F->nodes[t];
    std::vector<int32_t> stack;
    for (int j = 0; j < node_num; ++j) {
      Node nd;
      uint64_t lp, rp;
      in.read((char*)&nd.div_dim, 4);
      in.read((char*)&nd.div_val, 4);
      in.read((char*)&nd.start, 8);
      in.read((char*)&nd.end, 8);
      in.read((char*)&lp, 8);
      in.read((char*)&rp, 8);
      nd.left = nd.right = -1;
      nodes.push_back(nd);
      int32_t cur = (int32_t)nodes.size() - 1;
      size_t rs = stack.size();
      if (rs >= 2) {
        Node& l1 = nodes[stack[rs - 1]];
        Node& l2 = nodes[stack[rs - 2]];
        if (l1.end == nodes[cur].end && l2.start == nodes[cur].start) {
          nodes[cur].right = stack[rs - 1];
          nodes[cur].left = stack[rs - 2];
          stack.pop_back();
          stack.pop_back();
        }
      }
      stack.push_back(cur);
    }
    if (!in || stack.size() != 1) {
      delete F;
      return nullptr;
    }
    F->roots[t] = stack[0];
  }
  F->leaves.assign(tn, std::vector<uint32_t>(num));
  for (uint32_t t = 0; t < tn; ++t) in.read((char*)F->leaves[t].data(), 4 * num);
  if (!in) {
    delete F;
    return nullptr;
  }
  return F;
}

// ----------------------------------------------------------------------------------------------
// NN-descent state (base_index.hpp:24-109).
// ----------------------------------------------------------------------------------------------
struct Point {
  uint32_t id;
  float dist;
  bool flag;
};
struct Params {
  uint32_t K, S, L, check_k, epochs, trees, trees_build, merge_level, tns, reverse_cap;
  uint64_t seed;
};
struct State {
  size_t n = 0;
  uint32_t P = 0;  // pool capacity = L + 1 (the last slot is InsertIntoKnn's overflow slot)
  std::vector<Point> pool;  // n * P, zero-initialised like the reference's freshly allocated pools
  std::vector<uint32_t> L, Range;
  std::vector<float> radius, radiusM;
  std::vector<uint8_t> found;
  std::vector<std::vector<uint32_t>> nn_new, nn_old;
  Point* row(size_t i) { return &pool[i * P]; }
  void init(size_t n_, uint32_t Lcap) {
    n = n_;
    P = Lcap + 1;
    pool.assign(n * P, Point{0, 0.0f, false});
    L.assign(n, 0);
    Range.assign(n, 0);
    radius.assign(n, FLT_MAX);
    radiusM.assign(n, 0.0f);
    found.assign(n, 0);
    nn_new.assign(n, {});
    nn_old.assign(n, {});
  }
};

// InsertIntoKnn (base_index.hpp:37-62).
static inline unsigned insert_into_knn(Point* addr, unsigned K, Point nn) {
  unsigned j;
  unsigned i = K;
  while (i > 0) {
    j = i - 1;
    if (addr[j].dist <= nn.dist) break;
    i = j;
  }
  unsigned l = i;
  while (l > 0) {
    j = l - 1;
    if (addr[j].dist < nn.dist) break;
    if (addr[j].id == nn.id) return K + 1;
    l = j;
  }
  j = K;
  while (j > i) {
    addr[j] = addr[j - 1];
    --j;
  }
  addr[i] = nn;
  return i;
}
// Neighbor::insert (base_index.hpp:80-93).
static inline unsigned nb_insert(State& st, size_t t, uint32_t id, float dist) {
  if (dist > st.radius[t]) return st.P;
  Point* pool = st.row(t);
  unsigned l = insert_into_knn(pool, st.L[t], Point{id, dist, true});
  if (l <= st.L[t]) {
    if (st.L[t] + 1 < st.P) ++st.L[t];
    else st.radius[t] = pool[st.L[t] - 1].dist;
  }
  return l;
}

// ---- join ----
// InitIndex::join (base_index.hpp:328-371), nodes in order, pairs in the callback order.
static uint64_t join_seq(const Data& X, State& st, const Params& p) {
  uint64_t cc = 0;
  for (size_t i = 0; i < st.n; ++i) {
    size_t uu = 0;
    st.found[i] = 0;
    auto cb = [&](unsigned a, unsigned b) {
      float dist = X.dist(a, b);
      ++cc;
      unsigned r = nb_insert(st, a, b, dist);
      if (r < p.check_k) ++uu;
      nb_insert(st, b, a, dist);
      if (r < p.check_k) ++uu;
    };
    const std::vector<uint32_t>& nw = st.nn_new[i];
    const std::vector<uint32_t>& od = st.nn_old[i];
    for (unsigned a : nw) {
      for (unsigned b : nw)
        if (a < b) cb(a, b);
      for (unsigned b : od) cb(a, b);
    }
    st.found[i] = uu > 0;
  }
  return cc;
}

struct Rec {
  float d;
  uint32_t cand, src;
  uint8_t side;  // 0: the insert whose rank feeds `found`, 1: the reverse insert
};
static inline bool rec_less(const Rec& x, const Rec& y) {
  if (x.d != y.d) return x.d < y.d;
  if (x.cand != y.cand) return x.cand < y.cand;
  if (x.src != y.src) return x.src < y.src;
  return x.side < y.side;
}
// Canonical join: the same pairs and the same per-insert semantics, but each target node applies
// its inserts in ascending (dist, candidate id, source node, side) order.
static uint64_t join_canon(const Data& X, State& st, const Params& p) {
  std::vector<std::vector<Rec>> recs(st.n);
  uint64_t cc = 0;
  for (size_t i = 0; i < st.n; ++i) {
    const std::vector<uint32_t>& nw = st.nn_new[i];
    const std::vector<uint32_t>& od = st.nn_old[i];
    for (size_t a = 0; a < nw.size(); ++a) {
      for (size_t b = a + 1; b < nw.size(); ++b) {
        uint32_t x = nw[a], y = nw[b];
        if (x == y) continue;
        uint32_t lo = std::min(x, y), hi = std::max(x, y);
        float d = X.dist(lo, hi);
        ++cc;
        recs[lo].push_back(Rec{d, hi, (uint32_t)i, 0});
        recs[hi].push_back(Rec{d, lo, (uint32_t)i, 1});
      }
      for (size_t b = 0; b < od.size(); ++b) {
        uint32_t x = nw[a], y = od[b];
        float d = X.dist(x, y);
        ++cc;
        recs[x].push_back(Rec{d, y, (uint32_t)i, 0});
        recs[y].push_back(Rec{d, x, (uint32_t)i, 1});
      }
    }
  }
  std::fill(st.found.begin(), st.found.end(), 0);
  for (size_t t = 0; t < st.n; ++t) {
    std::vector<Rec>& R = recs[t];
    std::sort(R.begin(), R.end(), rec_less);
    for (const Rec& r : R) {
      unsigned rank = nb_insert(st, t, r.cand, r.d);
      if (r.side == 0 && rank < p.check_k) st.found[r.src] = 1;
    }
  }
  return cc;
}

// ---- update ----
// InitIndex::update (base_index.hpp:373-437).  In sequential mode reverse lists are cut with
// random_shuffle; in canonical mode they are sorted by source id and, when longer than the cap,
// reduced to the `cap` sources with the smallest (high 32 bits of the counter hash, source),
// in that order.
static void update(State& st, const Params& p, int mode, uint32_t iter) {
  size_t n = st.n;
  std::vector<std::vector<uint32_t>> rnn_new(n), rnn_old(n);
  for (size_t i = 0; i < n; ++i) {
    st.nn_new[i].clear();
    st.nn_old[i].clear();
    st.radius[i] = st.row(i)[st.P - 1].dist;
  }
  for (size_t i = 0; i < n; ++i) {
    Point* pool = st.row(i);
    if (st.found[i]) {
      unsigned maxl = st.Range[i] + p.S < st.L[i] ? st.Range[i] + p.S : st.L[i];
      unsigned c = 0, l = 0;
      while ((l < maxl) && (c < p.S)) {
        if (pool[l].flag) ++c;
        ++l;
      }
      st.Range[i] = l;
    }
    st.radiusM[i] = pool[st.Range[i] - 1].dist;
  }
  for (size_t nn = 0; nn < n; ++nn) {
    Point* pool = st.row(nn);
    for (unsigned l = 0; l < st.Range[nn]; ++l) {
      Point& e = pool[l];
      if (e.flag) {
        st.nn_new[nn].push_back(e.id);
        if (e.dist > st.radiusM[e.id]) rnn_new[e.id].push_back((uint32_t)nn);
        e.flag = false;
      } else {
        st.nn_old[nn].push_back(e.id);
        if (e.dist > st.radiusM[e.id]) rnn_old[e.id].push_back((uint32_t)nn);
      }
    }
  }
  unsigned cap = p.reverse_cap;
  for (size_t i = 0; i < n; ++i) {
    for (int which = 0; which < 2; ++which) {
      std::vector<uint32_t>& R = which == 0 ? rnn_new[i] : rnn_old[i];
      if (mode == MODE_SEQ) {
        if (cap && R.size() > cap) {
          std::random_shuffle(R.begin(), R.end());
          R.resize(cap);
        }
      } else if (cap && R.size() > cap) {
        uint64_t tag = which == 0 ? TAG_RNEW : TAG_ROLD;
        std::vector<std::pair<uint64_t, uint32_t>> h;
        for (uint32_t s : R) h.push_back({hash4(p.seed, tag, iter, i, s) >> 32, s});
        std::sort(h.begin(), h.end());
        R.clear();
        for (unsigned k = 0; k < cap; ++k) R.push_back(h[k].second);
      }
      std::vector<uint32_t>& dst = which == 0 ? st.nn_new[i] : st.nn_old[i];
      dst.insert(dst.end(), R.begin(), R.end());
    }
  }
}

// ---- initial graph from the leaves ----
struct Cand {  // efanna::Candidate ordering (general/distance.hpp:26-44)
  size_t row_id;
  float distance;
  bool operator>(const Cand& r) const {
    if (distance == r.distance) return row_id > r.row_id;
    return distance > r.distance;
  }
  bool operator<(const Cand& r) const {
    if (distance == r.distance) return row_id < r.row_id;
    return distance < r.distance;
  }
};
typedef std::set<Cand, std::greater<Cand>> CandHeap;

// getMergeLevelNodeList (kdtreeub_index.hpp:1000-1011).
static void merge_level_nodes(const Forest& F, unsigned t, int32_t ni, int depth, int ml,
                              std::vector<std::pair<int32_t, unsigned>>& out, bool& err, int& maxd) {
  const Node& nd = F.nodes[t][ni];
  if (nd.left >= 0 && nd.right >= 0 && depth < ml) {
    ++depth;
    merge_level_nodes(F, t, nd.left, depth, ml, out, err, maxd);
    merge_level_nodes(F, t, nd.right, depth, ml, out, err, maxd);
  } else if (depth == ml) {
    out.push_back({ni, t});
  } else {
    err = true;
    if (depth < maxd) maxd = depth;
  }
}
// SearchToLeaf (kdtreeub_index.hpp:1012-1021).
static int32_t search_to_leaf(const Forest& F, const Data& X, unsigned t, int32_t ni, size_t id) {
  const std::vector<Node>& nodes = F.nodes[t];
  while (nodes[ni].left >= 0 && nodes[ni].right >= 0) {
    const Node& nd = nodes[ni];
    ni = X.row(id)[nd.div_dim] < nd.div_val ? nd.left : nd.right;
  }
  return ni;
}
// mergeSubGraphs (kdtreeub_index.hpp:1022-1081), sequential.
static void merge_subgraphs_seq(const Forest& F, const Data& X, unsigned t, int32_t ni, const Params& p,
                                std::vector<CandHeap>& knn, State& st) {
  const Node& nd = F.nodes[t][ni];
  if (!(nd.left >= 0 && nd.right >= 0)) return;
  merge_subgraphs_seq(F, X, t, nd.left, p, knn, st);
  merge_subgraphs_seq(F, X, t, nd.right, p, knn, st);
  const Node& L = F.nodes[t][nd.left];
  const Node& R = F.nodes[t][nd.right];
  size_t numL = L.end - L.start, numR = R.end - R.start;
  size_t start, end;
  int32_t root;
  if (numL < numR) {
    root = nd.right;
    start = L.start;
    end = L.end;
  } else {
    root = nd.left;
    start = R.start;
    end = R.end;
  }
  for (; start < end; start++) {
    size_t fid = F.leaves[t][start];
    int32_t leaf = search_to_leaf(F, X, t, root, fid);
    const Node& lf = F.nodes[t][leaf];
    for (size_t i = lf.start; i < lf.end; i++) {
      size_t tf = F.leaves[t][i];
      float dist = X.dist(tf, fid);
      auto offer = [&](size_t tgt, size_t cand) {
        CandHeap& h = knn[tgt];
        if (h.size() < p.S || dist < h.begin()->distance) {
          h.insert(Cand{cand, dist});
          if (h.size() > p.S) h.erase(h.begin());
        } else if (st.nn_new[tgt].size() < p.S * 2) {
          st.nn_new[tgt].push_back((uint32_t)cand);
        }
      };
      offer(tf, fid);
      offer(fid, tf);
    }
  }
}

// GenRandom (kdtreeub_index.hpp:1121-1135), templated on the generator.
template <typename G>
static void gen_random(G& rng, unsigned* addr, unsigned size, unsigned N) {
  for (unsigned i = 0; i < size; ++i) addr[i] = rng() % (N - size);
  std::sort(addr, addr + size);
  for (unsigned i = 1; i < size; ++i)
    if (addr[i] <= addr[i - 1]) addr[i] = addr[i - 1] + 1;
  unsigned off = rng() % N;
  for (unsigned i = 0; i < size; ++i) addr[i] = (addr[i] + off) % N;
}
struct CRngFn {  // adapts CRng to the rng() call syntax
  CRng r;
  uint32_t operator()() { return r.next(); }
};

// initGraph's merge and pool seeding (kdtreeub_index.hpp:1367-1424).  Returns 0, or 3 when a
// leaf of a graph tree is shallower than the merge level (error_flag, :108-111).
static int init_graph(const Data& X, const Forest& F, const Params& p, int mode, State& st, int* max_depth) {
  size_t N = X.n;
  st.init(N, p.L);
  std::vector<std::pair<int32_t, unsigned>> ml_nodes;
  bool err = false;
  int maxd = 0x0fffffff;
  for (unsigned t = 0; t < p.trees_build; ++t)
    merge_level_nodes(F, t, F.roots[t], 0, (int)p.merge_level, ml_nodes, err, maxd);
  if (max_depth) *max_depth = maxd;
  if (err) return 3;
  if (mode == MODE_SEQ) {
    std::vector<CandHeap> knn(N);
    for (auto& mn : ml_nodes) merge_subgraphs_seq(F, X, mn.second, mn.first, p, knn, st);
    std::mt19937 rng(1998 ^ 0);
    std::vector<unsigned> random(p.S + 1);
    for (unsigned nn = 0; nn < (unsigned)N; ++nn) {
      std::vector<uint32_t>& nw = st.nn_new[nn];
      if (nw.size() < p.S * 2) {
        nw.resize(p.S * 2);
        gen_random(rng, &nw[0], (unsigned)nw.size(), (unsigned)N);
      }
      gen_random(rng, &random[0], (unsigned)random.size(), (unsigned)N);
      st.L[nn] = p.S;
      st.Range[nn] = p.S;
      while (knn[nn].size() < p.S) {
        unsigned rid = rng() % (unsigned)N;
        float dist = X.dist(nn, rid);
        knn[nn].insert(Cand{rid, dist});
      }
      Point* pool = st.row(nn);
      auto it = knn[nn].rbegin();
      for (unsigned l = 0; l < st.L[nn]; ++l) {
        pool[l].id = (uint32_t)it->row_id;
        nw[l] = (uint32_t)it->row_id;
        pool[l].dist = it->distance;
        pool[l].flag = true;
        ++it;
      }
      std::sort(pool, pool + st.L[nn], [](const Point& a, const Point& b) { return a.dist < b.dist; });
    }
    return 0;
  }
  // Canonical: every offer becomes a (target, dist, candidate) record; each target keeps its S
  // smallest distinct (dist, id) keys, and takes its S extra join candidates from the rest by
  // counter hash when at least 2S distinct others exist (else from gen_random, as the reference
  // does when its overflow list is short).
  std::vector<std::vector<std::pair<float, uint32_t>>> recs(N);
  for (auto& mn : ml_nodes) {
    unsigned t = mn.second;
    std::vector<int32_t> stack{mn.first};
    while (!stack.empty()) {
      int32_t ni = stack.back();
      stack.pop_back();
      const Node& nd = F.nodes[t][ni];
      if (!(nd.left >= 0 && nd.right >= 0)) continue;
      stack.push_back(nd.left);
      stack.push_back(nd.right);
      const Node& L = F.nodes[t][nd.left];
      const Node& R = F.nodes[t][nd.right];
      size_t numL = L.end - L.start, numR = R.end - R.start;
      int32_t root = numL < numR ? nd.right : nd.left;
      const Node& small = numL < numR ? L : R;
      for (size_t s = small.start; s < small.end; ++s) {
        uint32_t fid = F.leaves[t][s];
        int32_t leaf = search_to_leaf(F, X, t, root, fid);
        const Node& lf = F.nodes[t][leaf];
        for (size_t i = lf.start; i < lf.end; ++i) {
          uint32_t tf = F.leaves[t][i];
          float dist = X.dist(tf, fid);
          recs[tf].push_back({dist, fid});
          recs[fid].push_back({dist, tf});
        }
      }
    }
  }
  for (size_t nn = 0; nn < N; ++nn) {
    std::vector<std::pair<float, uint32_t>>& R = recs[nn];
    std::sort(R.begin(), R.end());
    R.erase(std::unique(R.begin(), R.end()), R.end());
    std::vector<std::pair<float, uint32_t>> knn(R.begin(), R.begin() + std::min<size_t>(R.size(), p.S));
    std::vector<uint32_t> extra;
    if (R.size() >= p.S + 2 * (size_t)p.S) {
      std::vector<std::pair<uint64_t, uint32_t>> h;
      for (size_t k = p.S; k < R.size(); ++k)
        h.push_back({hash4(p.seed, TAG_EXTRA, nn, R[k].second, 0) >> 32, R[k].second});
      std::sort(h.begin(), h.end());
      for (unsigned k = 0; k < p.S; ++k) extra.push_back(h[k].second);
    } else {
      CRngFn g{CRng(hash4(p.seed, TAG_GENRAND, nn, 0, 0))};
      std::vector<unsigned> tmp(2 * p.S);
      gen_random(g, &tmp[0], 2 * p.S, (unsigned)N);
      for (unsigned k = p.S; k < 2 * p.S; ++k) extra.push_back(tmp[k]);
    }
    if (knn.size() < p.S) {
      CRng g(hash4(p.seed, TAG_TOPUP, nn, 0, 0));
      while (knn.size() < p.S) {
        uint32_t rid = g.next() % (uint32_t)N;
        std::pair<float, uint32_t> c{X.dist(nn, rid), rid};
        auto pos = std::lower_bound(knn.begin(), knn.end(), c);
        if (pos != knn.end() && *pos == c) continue;
        knn.insert(pos, c);
      }
    }
    Point* pool = st.row(nn);
    std::vector<uint32_t>& nw = st.nn_new[nn];
    nw.clear();
    for (unsigned l = 0; l < p.S; ++l) {
      pool[l] = Point{knn[l].second, knn[l].first, true};
      nw.push_back(knn[l].second);
    }
    for (uint32_t e : extra) nw.push_back(e);
    st.L[nn] = p.S;
    st.Range[nn] = p.S;
  }
  return 0;
}

// ----------------------------------------------------------------------------------------------
// Multi-threaded restatement (ORC_OMP): the reference's OpenMP build with its parallel loops and
// per-node spin locks, used only as the CPU timing baseline (its output depends on thread timing,
// as the reference's does).  kdtreeub_index.hpp:1311-1423, base_index.hpp:328-437.
// ----------------------------------------------------------------------------------------------
struct Spin {
  std::atomic_flag f = ATOMIC_FLAG_INIT;
  void lock() { while (f.test_and_set(std::memory_order_acquire)) { } }
  void unlock() { f.clear(std::memory_order_release); }
};
static inline int thread_id() {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

static void dfs_build_local(const Data& X, std::vector<Node>& sub, int32_t node, std::mt19937& rng,
                            unsigned* indices, unsigned count, unsigned offset, unsigned tns) {
  dfs_build(X, sub, node, rng, indices, count, offset, tns);
}

static void build_forest_omp(const Data& X, unsigned T, unsigned S, unsigned tns, Forest& F) {
  unsigned N = (unsigned)X.n;
  F.n = X.n;
  F.dim = X.d;
  F.nodes.assign(T, {});
  F.roots.assign(T, 0);
  F.leaves.assign(T, {});
  std::vector<std::pair<unsigned, int32_t>> active, next;
  for (unsigned t = 0; t < T; ++t) {
    F.roots[t] = new_node(F.nodes[t], -1, 0, N);
    active.push_back({t, F.roots[t]});
    F.leaves[t].resize(N);
  }
#pragma omp parallel for
  for (int t = 0; t < (int)T; ++t) {
    std::vector<unsigned>& ids = F.leaves[t];
    for (unsigned i = 0; i < N; ++i) ids[i] = i;
    std::random_shuffle(ids.begin(), ids.end());
  }
  struct Split { unsigned mid, dim; float val; };
  while (!active.empty() && active.size() < 1100) {
    std::vector<Split> sp(active.size());
#pragma omp parallel for
    for (long a = 0; a < (long)active.size(); ++a) {
      std::mt19937 rng(1998 ^ thread_id());
      const Node& nd = F.nodes[active[a].first][active[a].second];
      mean_split_seq(X, rng, &F.leaves[active[a].first][0] + nd.start, (unsigned)(nd.end - nd.start), sp[a].mid,
                     sp[a].dim, sp[a].val);
    }
    next.clear();
    for (size_t a = 0; a < active.size(); ++a) {
      unsigned t = active[a].first;
      int32_t ni = active[a].second;
      std::vector<Node>& nodes = F.nodes[t];
      uint64_t s = nodes[ni].start, e = nodes[ni].end;
      nodes[ni].div_dim = (int)sp[a].dim;
      nodes[ni].div_val = sp[a].val;
      int32_t l = new_node(nodes, 0, s, s + sp[a].mid);
      int32_t r = new_node(nodes, 0, s + sp[a].mid, e);
      nodes[ni].left = l;
      nodes[ni].right = r;
      if (sp[a].mid > S) next.push_back({t, l});
      if (e - (s + sp[a].mid) > S) next.push_back({t, r});
    }
    active.swap(next);
  }
  std::vector<std::vector<Node>> subs(active.size());
#pragma omp parallel for schedule(dynamic, 4)
  for (long a = 0; a < (long)active.size(); ++a) {
    std::mt19937 rng(1998 ^ thread_id());
    const Node& nd = F.nodes[active[a].first][active[a].second];
    std::vector<Node>& sub = subs[a];
    sub.push_back(nd);
    dfs_build_local(X, sub, 0, rng, &F.leaves[active[a].first][0] + nd.start, (unsigned)(nd.end - nd.start),
                    (unsigned)nd.start, tns);
  }
  for (size_t a = 0; a < active.size(); ++a) {  // splice the subtrees in
    std::vector<Node>& nodes = F.nodes[active[a].first];
    int32_t base = (int32_t)nodes.size() - 1;
    std::vector<Node>& sub = subs[a];
    for (size_t j = 0; j < sub.size(); ++j) {
      Node nd = sub[j];
      if (nd.left >= 0) {
        nd.left = nd.left == 0 ? active[a].second : nd.left + base;
        nd.right = nd.right == 0 ? active[a].second : nd.right + base;
      }
      if (j == 0) nodes[active[a].second] = nd;
      else nodes.push_back(nd);
    }
  }
}

static void merge_subgraphs_omp(const Forest& F, const Data& X, unsigned t, int32_t ni, const Params& p,
                                std::vector<CandHeap>& knn, State& st, std::vector<Spin>& locks) {
  const Node& nd = F.nodes[t][ni];
  if (!(nd.left >= 0 && nd.right >= 0)) return;
  merge_subgraphs_omp(F, X, t, nd.left, p, knn, st, locks);
  merge_subgraphs_omp(F, X, t, nd.right, p, knn, st, locks);
  const Node& L = F.nodes[t][nd.left];
  const Node& R = F.nodes[t][nd.right];
  size_t numL = L.end - L.start, numR = R.end - R.start;
  int32_t root = numL < numR ? nd.right : nd.left;
  size_t start = numL < numR ? L.start : R.start, end = numL < numR ? L.end : R.end;
  for (; start < end; start++) {
    size_t fid = F.leaves[t][start];
    int32_t leaf = search_to_leaf(F, X, t, root, fid);
    const Node& lf = F.nodes[t][leaf];
    for (size_t i = lf.start; i < lf.end; i++) {
      size_t tf = F.leaves[t][i];
      float dist = X.dist(tf, fid);
      auto offer = [&](size_t tgt, size_t cand) {
        locks[tgt].lock();
        CandHeap& h = knn[tgt];
        if (h.size() < p.S || dist < h.begin()->distance) {
          h.insert(Cand{cand, dist});
          if (h.size() > p.S) h.erase(h.begin());
        } else if (st.nn_new[tgt].size() < p.S * 2) {
          st.nn_new[tgt].push_back((uint32_t)cand);
        }
        locks[tgt].unlock();
      };
      offer(tf, fid);
      offer(fid, tf);
    }
  }
}

static int init_graph_omp(const Data& X, const Forest& F, const Params& p, State& st, std::vector<Spin>& locks,
                          int* max_depth) {
  size_t N = X.n;
  st.init(N, p.L);
  std::vector<std::pair<int32_t, unsigned>> ml_nodes;
  bool err = false;
  int maxd = 0x0fffffff;
  for (unsigned t = 0; t < p.trees_build; ++t)
    merge_level_nodes(F, t, F.roots[t], 0, (int)p.merge_level, ml_nodes, err, maxd);
  if (max_depth) *max_depth = maxd;
  if (err) return 3;
  std::vector<CandHeap> knn(N);
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = 0; i < (long)ml_nodes.size(); ++i)
    merge_subgraphs_omp(F, X, ml_nodes[i].second, ml_nodes[i].first, p, knn, st, locks);
#pragma omp parallel
  {
    std::mt19937 rng(1998 ^ thread_id());
    std::vector<unsigned> random(p.S + 1);
#pragma omp for
    for (long nn = 0; nn < (long)N; ++nn) {
      std::vector<uint32_t>& nw = st.nn_new[nn];
      if (nw.size() < p.S * 2) {
        nw.resize(p.S * 2);
        gen_random(rng, &nw[0], (unsigned)nw.size(), (unsigned)N);
      }
      gen_random(rng, &random[0], (unsigned)random.size(), (unsigned)N);
      st.L[nn] = p.S;
      st.Range[nn] = p.S;
      while (knn[nn].size() < p.S) {
        unsigned rid = rng() % (unsigned)N;
        knn[nn].insert(Cand{rid, X.dist(nn, rid)});
      }
      Point* pool = st.row(nn);
      auto it = knn[nn].rbegin();
      for (unsigned l = 0; l < st.L[nn]; ++l, ++it) {
        pool[l] = Point{(uint32_t)it->row_id, it->distance, true};
        nw[l] = (uint32_t)it->row_id;
      }
      std::sort(pool, pool + st.L[nn], [](const Point& a, const Point& b) { return a.dist < b.dist; });
    }
  }
  return 0;
}

static uint64_t join_omp(const Data& X, State& st, const Params& p, std::vector<Spin>& locks) {
  uint64_t cc = 0;
  auto ins = [&](size_t t, uint32_t id, float dist) -> unsigned {
    if (dist > st.radius[t]) return st.P;  // unlocked read, as Neighbor::insert
    locks[t].lock();
    unsigned r = nb_insert(st, t, id, dist);
    locks[t].unlock();
    return r;
  };
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : cc)
  for (long i = 0; i < (long)st.n; ++i) {
    size_t uu = 0;
    st.found[i] = 0;
    const std::vector<uint32_t>& nw = st.nn_new[i];
    const std::vector<uint32_t>& od = st.nn_old[i];
    auto cb = [&](unsigned a, unsigned b) {
      float dist = X.dist(a, b);
      ++cc;
      unsigned r = ins(a, b, dist);
      if (r < p.check_k) ++uu;
      ins(b, a, dist);
      if (r < p.check_k) ++uu;
    };
    for (unsigned a : nw) {
      for (unsigned b : nw)
        if (a < b) cb(a, b);
      for (unsigned b : od) cb(a, b);
    }
    st.found[i] = uu > 0;
  }
  return cc;
}

static void update_omp(State& st, const Params& p, std::vector<Spin>& locks) {
  size_t n = st.n;
  std::vector<std::vector<uint32_t>> rnn_new(n), rnn_old(n);
  for (size_t i = 0; i < n; ++i) {
    st.nn_new[i].clear();
    st.nn_old[i].clear();
    st.radius[i] = st.row(i)[st.P - 1].dist;
  }
#pragma omp parallel for
  for (long i = 0; i < (long)n; ++i) {
    Point* pool = st.row(i);
    if (st.found[i]) {
      unsigned maxl = st.Range[i] + p.S < st.L[i] ? st.Range[i] + p.S : st.L[i];
      unsigned c = 0, l = 0;
      while ((l < maxl) && (c < p.S)) {
        if (pool[l].flag) ++c;
        ++l;
      }
      st.Range[i] = l;
    }
    st.radiusM[i] = pool[st.Range[i] - 1].dist;
  }
#pragma omp parallel for
  for (long nn = 0; nn < (long)n; ++nn) {
    Point* pool = st.row(nn);
    for (unsigned l = 0; l < st.Range[nn]; ++l) {
      Point& e = pool[l];
      if (e.flag) {
        st.nn_new[nn].push_back(e.id);
        if (e.dist > st.radiusM[e.id]) {
          locks[e.id].lock();
          rnn_new[e.id].push_back((uint32_t)nn);
          locks[e.id].unlock();
        }
        e.flag = false;
      } else {
        st.nn_old[nn].push_back(e.id);
        if (e.dist > st.radiusM[e.id]) {
          locks[e.id].lock();
          rnn_old[e.id].push_back((uint32_t)nn);
          locks[e.id].unlock();
        }
      }
    }
  }
  unsigned cap = p.reverse_cap;
  for (size_t i = 0; i < n; ++i) {
    for (int which = 0; which < 2; ++which) {
      std::vector<uint32_t>& R = which == 0 ? rnn_new[i] : rnn_old[i];
      if (cap && R.size() > cap) {
        std::random_shuffle(R.begin(), R.end());
        R.resize(cap);
      }
      std::vector<uint32_t>& dst = which == 0 ? st.nn_new[i] : st.nn_old[i];
      dst.insert(dst.end(), R.begin(), R.end());
    }
  }
}

static void export_graph(State& st, uint32_t K, uint32_t* gs) {
  for (size_t i = 0; i < st.n; ++i)
    for (uint32_t j = 0; j < K; ++j) gs[i * K + j] = st.row(i)[j].id;
}

// ----------------------------------------------------------------------------------------------
// Search: getNeighbors_nnexp (kdtreeub_index.hpp:363-494).
// ----------------------------------------------------------------------------------------------
// getSearchNodeList (kdtreeub_index.hpp:332-346).
static void search_node_list(const Forest& F, unsigned t, int32_t ni, const float* q, unsigned lsize,
                             std::vector<int32_t>& vn) {
  if (vn.size() >= lsize) return;
  const Node& nd = F.nodes[t][ni];
  if (nd.left >= 0 && nd.right >= 0) {
    if (q[nd.div_dim] < nd.div_val) {
      search_node_list(F, t, nd.left, q, lsize, vn);
      search_node_list(F, t, nd.right, q, lsize, vn);
    } else {
      search_node_list(F, t, nd.right, q, lsize, vn);
      search_node_list(F, t, nd.left, q, lsize, vn);
    }
  } else {
    vn.push_back(ni);
  }
}

struct SearchArgs {
  int epochs, init_num, extend_to, trees;
  uint32_t k;
  const uint32_t* seeds = nullptr;  // this query's entry seeds (learned form)
  unsigned nseeds = 0;
};

// Pool seeding shared by both search methods (kdtreeub_index.hpp:380-418 and :519-548): leaves of
// the near-first DFS of every tree, leaf rank outer and tree inner, first occurrences until
// init_num; short pools are topped up with random ids (std::rand() in sequential mode, the
// per-query counter hash in canonical mode).  tbflag marks the pool's ids.
static std::vector<int> fill_pool(const Data& X, const Forest& F, const float* q, uint64_t qi, unsigned T,
                                  unsigned lsize, unsigned init_num, int mode, uint64_t seed,
                                  std::vector<uint8_t>& tbflag, const uint32_t* seeds = nullptr,
                                  unsigned nseeds = 0) {
  size_t N = X.n;
  std::vector<std::vector<int32_t>> cand(T);
  for (unsigned t = 0; t < T; ++t) search_node_list(F, t, F.roots[t], q, lsize, cand[t]);
  std::vector<int> pool(init_num);
  unsigned pcount = 0;
  // entry seeds (learned form; no reference counterpart) ahead of the leaves, in order
  for (unsigned j = 0; j < nseeds && pcount < init_num; ++j) {
    uint32_t id = seeds[j];
    if (id >= N || tbflag[id]) continue;
    tbflag[id] = 1;
    pool[pcount++] = (int)id;
  }
  for (unsigned ni = 0; ni < lsize; ni++) {
    for (unsigned t = 0; t < T; t++) {
      if (ni >= cand[t].size()) continue;
      const Node& leaf = F.nodes[t][cand[t][ni]];
      for (size_t j = leaf.start; j < leaf.end && pcount < init_num; j++) {
        size_t id = F.leaves[t][j];
        if (tbflag[id]) continue;
        tbflag[id] = 1;
        pool[pcount++] = (int)id;
      }
      if (pcount >= init_num) break;
    }
    if (pcount >= init_num) break;
  }
  if (mode == MODE_SEQ) {
    int base_n = (int)N;
    while (pcount < init_num) {
      unsigned id = rand() % base_n;
      if (tbflag[id]) continue;
      tbflag[id] = 1;
      pool[pcount++] = (int)id;
    }
  } else {
    CRng g(hash4(seed, TAG_SFILL, qi, 0, 0));
    while (pcount < init_num) {
      uint32_t id = g.next() % (uint32_t)N;
      if (tbflag[id]) continue;
      tbflag[id] = 1;
      pool[pcount++] = (int)id;
    }
  }
  return pool;
}

static void search_one(const Data& X, const Forest& F, const uint64_t* gptr, const uint32_t* gids, const float* q,
                       uint64_t qi, const SearchArgs& a, int mode, uint64_t seed, int32_t* out, uint64_t* nd) {
  size_t N = X.n;
  std::vector<uint8_t> tbflag(N, 0), newflag(N, 1);
  unsigned T = (unsigned)a.trees;
  unsigned lsize = T ? a.init_num * 2 / (5 * T) + 1 : 0;  // T == 0: a pool from the seeds alone
  std::vector<int> pool = fill_pool(X, F, q, qi, T, lsize, (unsigned)a.init_num, mode, seed, tbflag, a.seeds,
                                    a.nseeds);
  unsigned resultSize = (unsigned)a.extend_to;
  if (a.k > resultSize) resultSize = a.k;
  std::vector<std::pair<float, size_t>> result;
  for (unsigned j = 0; j < pool.size(); ++j) result.push_back({X.distq(q, X.row(pool[j])), (size_t)pool[j]});
  uint64_t evals = pool.size();
  std::partial_sort(result.begin(), result.begin() + resultSize, result.end());
  result.resize(resultSize);
  pool.clear();
  for (unsigned j = 0; j < resultSize; j++) pool.push_back((int)result[j].second);
  std::vector<int> ids;
  for (int iter = 0; iter < a.epochs; ++iter) {
    ids.clear();
    for (unsigned j = 0; j < (unsigned)a.extend_to; j++) {
      size_t pj = (size_t)pool[j];
      if (newflag[pj]) {
        newflag[pj] = 0;
        for (uint64_t e = gptr[pj]; e < gptr[pj + 1]; ++e) {
          uint32_t id = gids[e];
          if (tbflag[id]) continue;
          tbflag[id] = 1;
          ids.push_back((int)id);
        }
      }
    }
    for (size_t j = 0; j < ids.size(); ++j) result.push_back({X.distq(q, X.row(ids[j])), (size_t)ids[j]});
    evals += ids.size();
    std::partial_sort(result.begin(), result.begin() + resultSize, result.end());
    result.resize(resultSize);
    pool.clear();
    for (unsigned j = 0; j < resultSize; j++) pool.push_back((int)result[j].second);
  }
  for (uint32_t i = 0; i < a.k; i++) out[i] = pool[i];
  if (nd) *nd = evals;
}

// ----------------------------------------------------------------------------------------------
// Search: getNeighbors_kgraph (kdtreeub_index.hpp:496-654).
// ----------------------------------------------------------------------------------------------
// Point (base_index.hpp:24-34): ordered by dist only.  `id == UINT32_MAX` stands for the
// reference's default-constructed (uninitialised) Point.
struct KPoint {
  uint32_t id;
  float dist;
  bool flag;
  bool operator<(const KPoint& o) const { return dist < o.dist; }
};
static inline bool canon_less(const KPoint& a, const KPoint& b) {
  return a.dist < b.dist || (a.dist == b.dist && a.id < b.id);
}

// InsertIntoKnn (base_index.hpp:37-62): insert after the entries of equal distance, reject a
// duplicate id among them (returns K + 1); writes addr[K] (the slot past the live list).
static unsigned insert_knn_seq(KPoint* addr, unsigned K, KPoint nn) {
  unsigned i = K;
  while (i > 0) {
    if (addr[i - 1].dist <= nn.dist) break;
    --i;
  }
  unsigned l = i;
  while (l > 0) {
    if (addr[l - 1].dist < nn.dist) break;
    if (addr[l - 1].id == nn.id) return K + 1;
    --l;
  }
  for (unsigned j = K; j > i; --j) addr[j] = addr[j - 1];
  addr[i] = nn;
  return i;
}
// Canonical counterpart: the position by (dist, id); ids are unique here, so no duplicate test.
static unsigned insert_knn_canon(KPoint* addr, unsigned K, KPoint nn) {
  unsigned i = K;
  while (i > 0 && canon_less(nn, addr[i - 1])) --i;
  for (unsigned j = K; j > i; --j) addr[j] = addr[j - 1];
  addr[i] = nn;
  return i;
}

// One query of getNeighbors_kgraph.  init_num is the pool size in effect for this call (the
// caller applies the reference's enlargement to epochs * extend_to) and lsize the per-tree leaf
// count computed from the pool size before that enlargement (:507, :510-514).
// full_rows: every graph neighbour of an expanded node is visited (the hashing initialiser's
// kgraph search, hashing_index.hpp:1306-1321) instead of the first extend_to (kdtreeub_index.hpp:599-603).
static void search_one_kgraph(const Data& X, const Forest& F, const uint64_t* gptr, const uint32_t* gids,
                              const float* q, uint64_t qi, const SearchArgs& a, unsigned lsize, bool sorted,
                              int mode, uint64_t seed, int32_t* out, uint64_t* nd, bool full_rows = false) {
  size_t N = X.n;
  const unsigned T = (unsigned)a.trees, E = (unsigned)a.extend_to, epochs = (unsigned)a.epochs;
  const unsigned searchK = a.k, pool_size = epochs * E;
  std::vector<uint8_t> flags(N, 0);
  std::vector<int> pool = fill_pool(X, F, q, qi, T, lsize, (unsigned)a.init_num, mode, seed, flags, a.seeds,
                                    a.nseeds);
  std::vector<std::pair<float, size_t>> result;  // :551-566, in pool order
  for (unsigned j = 0; j < pool.size(); ++j) result.push_back({X.distq(q, X.row(pool[j])), (size_t)pool[j]});
  uint64_t evals = pool.size();
  if (sorted) {  // :567-570
    std::partial_sort(result.begin(), result.begin() + pool_size, result.end());
    result.resize(pool_size);
  }
  std::fill(flags.begin(), flags.end(), 0);  // flags.reset() (:572)
  const bool seq = mode == MODE_SEQ;
  auto insert = seq ? insert_knn_seq : insert_knn_canon;
  std::vector<KPoint> knn(searchK + E + 1);
  std::vector<KPoint> results;
  for (unsigned iter = 0; iter < epochs; ++iter) {
    unsigned L = 0;
    for (unsigned j = 0; j < E; j++) {  // :577-585
      const auto& r = result[iter * E + j];
      if (!flags[r.second]) {
        flags[r.second] = 1;
        knn[L].id = (uint32_t)r.second;
        knn[L].dist = r.first;
        knn[L].flag = true;
        L++;
      }
    }
    if (seq) std::sort(knn.begin(), knn.begin() + L);  // `if(~bSorted)` is always true (:587-589)
    else std::sort(knn.begin(), knn.begin() + L, canon_less);
    unsigned k = 0;
    while (k < L) {  // :591-631
      unsigned nk = L;
      if (knn[k].flag) {
        knn[k].flag = false;
        unsigned n = knn[k].id;
        unsigned maxM = full_rows ? UINT32_MAX : E;
        unsigned deg = (unsigned)(gptr[n + 1] - gptr[n]);
        if (maxM > deg) maxM = deg;
        for (unsigned m = 0; m < maxM; ++m) {
          unsigned id = gids[gptr[n] + m];
          if (flags[id]) continue;
          flags[id] = 1;
          KPoint nn{id, X.distq(q, X.row(id)), true};
          ++evals;
          unsigned r = insert(&knn[0], L, nn);
          if (L + 1 < knn.size()) ++L;
          if (r < nk) nk = r;
        }
      }
      if (nk <= k) k = nk;
      else ++k;
    }
    if (L > searchK) L = searchK;
    if (results.empty()) {  // :634-646
      results.resize(L + 1, KPoint{UINT32_MAX, 0.f, false});
      std::copy(knn.begin(), knn.begin() + L, results.begin());
    } else if (seq) {
      for (unsigned l = 0; l < L; ++l) {
        unsigned r = insert_knn_seq(&results[0], (unsigned)results.size() - 1, knn[l]);
        if (r < results.size() && results.size() < searchK + 1) results.push_back(KPoint{UINT32_MAX, 0.f, false});
      }
    } else {
      for (unsigned l = 0; l < L; ++l) {
        unsigned r = insert_knn_canon(&results[0], (unsigned)results.size() - 1, knn[l]);
        if (r < results.size() && results.size() < searchK + 1) results.push_back(KPoint{UINT32_MAX, 0.f, false});
      }
    }
  }
  // :649-651; the slot past the live list holds an uninitialised Point in the reference: -1 here
  for (uint32_t i = 0; i < searchK; i++) {
    uint32_t id = i + 1 < results.size() ? results[i].id : UINT32_MAX;
    out[i] = id == UINT32_MAX ? -1 : (int32_t)id;
  }
  if (nd) *nd = evals;
}

}  // namespace orc

// ================================================================================================
// C interface used by the tests (ctypes) and by bench.py's CPU-baseline leg.
// ================================================================================================
using namespace orc;

extern "C" {

typedef struct {
  uint32_t K, S, L, check_k, epochs, trees, trees_build, merge_level, tns, reverse_cap;
  uint64_t seed;
} orc_params;

static Params to_params(const orc_params* q) {
  Params p;
  p.K = q->K; p.S = q->S; p.L = q->L; p.check_k = q->check_k; p.epochs = q->epochs; p.trees = q->trees;
  p.trees_build = q->trees_build ? q->trees_build : q->trees; p.merge_level = q->merge_level; p.tns = q->tns;
  p.reverse_cap = q->reverse_cap; p.seed = q->seed;
  return p;
}

float orc_l2_avx(const float* a, const float* b, uint64_t d) { return l2_avx(a, b, d); }
float orc_l2_scalar(const float* a, const float* b, uint64_t d) { return l2_scalar(a, b, d); }
void orc_l2_pairs(const float* base, uint64_t ld, uint64_t d, const uint32_t* ia, const uint32_t* ib, uint64_t m,
                  int order, float* out) {
  for (uint64_t i = 0; i < m; ++i) {
    const float* a = base + ia[i] * ld;
    const float* b = base + ib[i] * ld;
    out[i] = order == 0 ? l2_avx(a, b, d) : l2_scalar(a, b, d);
  }
}

void* orc_forest_build(const float* data, uint64_t n, uint32_t d, uint64_t ld, uint32_t trees, uint32_t S,
                       uint32_t tns, int mode, uint64_t seed) {
  Data X{data, n, d, ld, mode};
  Forest* F = new Forest();
  if (mode == MODE_SEQ) {
    srand(1);
    build_forest_seq(X, trees, S, tns, *F);
  } else if (mode == MODE_OMP) {
    srand(1);
    build_forest_omp(X, trees, S, tns, *F);
  } else {
    build_forest_canon(X, trees, S, tns, seed, *F);
  }
  return F;
}
int orc_forest_save(void* f, const char* path, uint32_t K) { return save_forest(*(Forest*)f, path, K); }
void* orc_forest_load(const char* path) { return load_forest(path); }
uint32_t orc_forest_trees(void* f) { return (uint32_t)((Forest*)f)->nodes.size(); }
void orc_forest_free(void* f) { delete (Forest*)f; }

// Whole buildIndex (initGraph + refineGraph, kdtreeub_index.hpp:92-113, base_index.hpp:438-481).
// Writes gs (n*K ids); *forest_out receives the trees built along the way (caller frees).
// stats[0] = join pair distances over all iterations, stats[1] = merge-depth limit on error.
int orc_build_graph(const float* data, uint64_t n, uint32_t d, uint64_t ld, const orc_params* pp, int mode,
                    uint32_t* gs_out, void** forest_out, uint64_t* stats) {
  Data X{data, n, d, ld, mode};
  Params p = to_params(pp);
  Forest* F = new Forest();
  std::vector<Spin> locks(mode == MODE_OMP ? n : 0);
  if (mode == MODE_SEQ) {
    srand(1);
    build_forest_seq(X, p.trees, p.S, p.tns, *F);
  } else if (mode == MODE_OMP) {
    srand(1);
    build_forest_omp(X, p.trees, p.S, p.tns, *F);
  } else {
    build_forest_canon(X, p.trees, p.S, p.tns, p.seed, *F);
  }
  State st;
  int maxd = 0;
  int rc = mode == MODE_OMP ? init_graph_omp(X, *F, p, st, locks, &maxd) : init_graph(X, *F, p, mode, st, &maxd);
  if (stats) stats[0] = stats[1] = 0;
  if (rc != 0) {
    if (stats) stats[1] = (uint64_t)(maxd - 1);
    if (forest_out) *forest_out = F;
    else delete F;
    return rc;
  }
  uint64_t cc = 0;
  for (uint32_t it = 0; it < p.epochs; ++it) {
    if (mode == MODE_OMP) {
      cc += join_omp(X, st, p, locks);
      update_omp(st, p, locks);
    } else {
      cc += mode == MODE_SEQ ? join_seq(X, st, p) : join_canon(X, st, p);
      update(st, p, mode, it);
    }
  }
  export_graph(st, p.K, gs_out);
  if (stats) stats[0] = cc;
  if (forest_out) *forest_out = F;
  else delete F;
  return 0;
}

// State-level entry points used by the join/update parity tests.  Arrays are n*(L+1) for the
// pool and n*cap for the lists; list order is preserved exactly.
static void state_in(State& st, uint64_t n, uint32_t Lcap, const float* pd, const uint32_t* pid, const uint8_t* pf,
                     const uint32_t* L, const uint32_t* R, const float* rad, const float* radM, const uint8_t* found,
                     const uint32_t* nid, const uint32_t* ncnt, const uint32_t* oid, const uint32_t* ocnt, uint32_t cap) {
  st.init(n, Lcap);
  for (uint64_t i = 0; i < n * st.P; ++i) st.pool[i] = Point{pid[i], pd[i], pf[i] != 0};
  for (uint64_t i = 0; i < n; ++i) {
    st.L[i] = L[i]; st.Range[i] = R[i]; st.radius[i] = rad[i]; st.radiusM[i] = radM[i]; st.found[i] = found[i];
    st.nn_new[i].assign(nid + i * cap, nid + i * cap + ncnt[i]);
    st.nn_old[i].assign(oid + i * cap, oid + i * cap + ocnt[i]);
  }
}
static int state_out(State& st, float* pd, uint32_t* pid, uint8_t* pf, uint32_t* L, uint32_t* R, float* rad,
                     float* radM, uint8_t* found, uint32_t* nid, uint32_t* ncnt, uint32_t* oid, uint32_t* ocnt,
                     uint32_t cap) {
  for (uint64_t i = 0; i < st.n * st.P; ++i) { pid[i] = st.pool[i].id; pd[i] = st.pool[i].dist; pf[i] = st.pool[i].flag; }
  for (uint64_t i = 0; i < st.n; ++i) {
    L[i] = st.L[i]; R[i] = st.Range[i]; rad[i] = st.radius[i]; radM[i] = st.radiusM[i]; found[i] = st.found[i];
    if (st.nn_new[i].size() > cap || st.nn_old[i].size() > cap) return -2;
    ncnt[i] = (uint32_t)st.nn_new[i].size();
    ocnt[i] = (uint32_t)st.nn_old[i].size();
    std::copy(st.nn_new[i].begin(), st.nn_new[i].end(), nid + i * cap);
    std::copy(st.nn_old[i].begin(), st.nn_old[i].end(), oid + i * cap);
  }
  return 0;
}

// initGraph (merge + seeding) on a given forest; fills the state arrays.
int orc_nnd_init(const float* data, uint64_t n, uint32_t d, uint64_t ld, void* forest, const orc_params* pp, int mode,
                 float* pd, uint32_t* pid, uint8_t* pf, uint32_t* L, uint32_t* R, float* rad, float* radM,
                 uint8_t* found, uint32_t* nid, uint32_t* ncnt, uint32_t* oid, uint32_t* ocnt, uint32_t cap) {
  Data X{data, n, d, ld, mode};
  Params p = to_params(pp);
  State st;
  int rc = init_graph(X, *(Forest*)forest, p, mode, st, nullptr);
  if (rc) return rc;
  return state_out(st, pd, pid, pf, L, R, rad, radM, found, nid, ncnt, oid, ocnt, cap);
}

// One refinement iteration (join then update) on the given state, in place.
int orc_nnd_iterate(const float* data, uint64_t n, uint32_t d, uint64_t ld, const orc_params* pp, int mode,
                    uint32_t iter, float* pd, uint32_t* pid, uint8_t* pf, uint32_t* L, uint32_t* R, float* rad,
                    float* radM, uint8_t* found, uint32_t* nid, uint32_t* ncnt, uint32_t* oid, uint32_t* ocnt,
                    uint32_t cap, uint64_t* pairs) {
  Data X{data, n, d, ld, mode};
  Params p = to_params(pp);
  State st;
  state_in(st, n, p.L, pd, pid, pf, L, R, rad, radM, found, nid, ncnt, oid, ocnt, cap);
  if (mode == MODE_SEQ) srand(1);
  uint64_t cc = mode == MODE_SEQ ? join_seq(X, st, p) : join_canon(X, st, p);
  update(st, p, mode, iter);
  if (pairs) *pairs = cc;
  return state_out(st, pd, pid, pf, L, R, rad, radM, found, nid, ncnt, oid, ocnt, cap);
}

// Batched nnexp search over a forest and a CSR graph.  evals receives the distance evaluations
// per query (may be null).  threads > 1 runs queries in parallel (canonical mode only: sequential
// mode's fill draws from the process-wide std::rand()).
int orc_search(const float* data, uint64_t n, uint32_t d, uint64_t ld, void* forest, const uint64_t* gptr,
               const uint32_t* gids, const float* q, uint64_t nq, uint64_t qld, int epochs, int init_num,
               int extend_to, int search_trees, uint32_t k, int mode, int threads, uint64_t seed, int32_t* out,
               uint64_t* evals) {
  Data X{data, n, d, ld, mode};
  Forest* F = (Forest*)forest;
  if (search_trees <= 0 || (size_t)search_trees > F->nodes.size()) return -1;
  if (extend_to > init_num) extend_to = init_num;  // setSearchParams (base_index.hpp:156-157)
  if ((int)k > init_num || init_num <= 0) return -1;
  SearchArgs a{epochs, init_num, extend_to, search_trees, k};
  if (mode == MODE_SEQ) srand(1);
#ifdef _OPENMP
  int nt = (mode == MODE_SEQ || threads < 1) ? 1 : threads;  // sequential fill uses std::rand()
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
  for (long long i = 0; i < (long long)nq; ++i)
    search_one(X, *F, gptr, gids, q + (uint64_t)i * qld, (uint64_t)i, a, mode, seed, out + (uint64_t)i * k,
               evals ? evals + i : nullptr);
  return 0;
}

// Batched nnexp search with per-query parameters (params: nq rows of epochs, pool, extend, k; out rows
// of k_max ids, -1 past each k) and optional entry seeds (nq rows of seeds_per_query ids).
int orc_search_batch(const float* data, uint64_t n, uint32_t d, uint64_t ld, void* forest, const uint64_t* gptr,
                     const uint32_t* gids, const float* q, uint64_t nq, uint64_t qld, const int32_t* params,
                     uint32_t k_max, int search_trees, const uint32_t* seeds, uint32_t seeds_per_query, int threads,
                     uint64_t seed, int32_t* out) {
  Data X{data, n, d, ld, MODE_CANON};
  Forest* F = (Forest*)forest;
  // search_trees == 0 (with seeds): no trees -- the hashing initialiser's search
  if (search_trees < 0 || (search_trees == 0 && !seeds) || (F && (size_t)search_trees > F->nodes.size()) ||
      (!F && search_trees > 0))
    return -1;
  Forest empty;
  if (!F) F = &empty;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads < 1 ? 1 : threads)
#endif
  for (long long i = 0; i < (long long)nq; ++i) {
    const int32_t* p = params + 4 * i;
    int init = p[1], ext = p[2] > p[1] ? p[1] : p[2];
    uint32_t k = (uint32_t)p[3];
    SearchArgs a{p[0], init, ext, search_trees, k};
    if (seeds) {
      a.seeds = seeds + (uint64_t)i * seeds_per_query;
      a.nseeds = seeds_per_query;
    }
    std::vector<int32_t> row(k);
    search_one(X, *F, gptr, gids, q + (uint64_t)i * qld, (uint64_t)i, a, MODE_CANON, seed, row.data(), nullptr);
    for (uint32_t j = 0; j < k_max; ++j) out[(uint64_t)i * k_max + j] = j < k ? row[j] : -1;
  }
  return 0;
}

// ---- hashing-seeded search (algorithm/hashing_index.hpp) ----
// Hamming-ball masks in the reference's order (generateMask32 / generateMask64, hashing_index.hpp:
// 348-860): the zero mask, then for r = 1..radius every r-tuple of bit positions i < j < ... in
// lexicographic order.
static void hamming_masks(unsigned bits, unsigned radius, std::vector<uint64_t>& out) {
  out.assign(1, 0);
  std::vector<unsigned> pos;
  for (unsigned r = 1; r <= radius && r <= bits; ++r) {
    pos.resize(r);
    for (unsigned t = 0; t < r; ++t) pos[t] = t;
    for (;;) {
      uint64_t m = 0;
      for (unsigned t = 0; t < r; ++t) m |= 1ull << pos[t];
      out.push_back(m);
      int t = (int)r - 1;  // next tuple: bump the last position that can still move
      while (t >= 0 && pos[t] == bits - r + (unsigned)t) --t;
      if (t < 0) break;
      ++pos[t];
      for (unsigned u = (unsigned)t + 1; u < r; ++u) pos[u] = pos[u - 1] + 1;
    }
  }
}

// Hash tables keyed by the full code (the reference splits it into upper and lower bits for a
// two-level lookup, BuildHashTable32/64 at hashing_index.hpp:323-346, which finds the same bucket),
// members in insertion (= id) order; probe() returns a query's first `limit` distinct ids in the
// visit order of the reference's searches: masks in order, tables inner, bucket members in order.
struct HashTabs {
  uint32_t tables;
  uint64_t n;
  std::vector<std::unordered_map<uint64_t, std::vector<uint32_t>>> tab;
  std::vector<uint64_t> masks;
  HashTabs(const uint64_t* bcodes, uint64_t n_, uint32_t tables_, uint32_t bits, uint32_t radius)
      : tables(tables_), n(n_), tab(tables_) {
    for (uint32_t h = 0; h < tables; ++h)
      for (uint64_t i = 0; i < n; ++i) tab[h][bcodes[(uint64_t)h * n + i]].push_back((uint32_t)i);
    hamming_masks(bits, radius, masks);
  }
  std::vector<uint32_t> probe(const uint64_t* qcodes, uint64_t nq, uint64_t qi, unsigned limit) const {
    std::vector<uint8_t> seen(n, 0);
    std::vector<uint32_t> prefix;
    for (size_t j = 0; j < masks.size() && prefix.size() < limit; ++j)
      for (uint32_t h = 0; h < tables && prefix.size() < limit; ++h) {
        auto it = tab[h].find(qcodes[(uint64_t)h * nq + qi] ^ masks[j]);
        if (it == tab[h].end()) continue;
        for (size_t e = 0; e < it->second.size() && prefix.size() < limit; ++e) {
          uint32_t id = it->second[e];
          if (seen[id]) continue;
          seen[id] = 1;
          prefix.push_back(id);
        }
      }
    return prefix;
  }
};

// getNeighborsIEH32_nnexp / getNeighborsIEH64_nnexp (hashing_index.hpp:1087-1200, 1354-1470):
// per query the probe's first init_num distinct ids, then the random fill and the pool / extend
// expansion of search_one with no trees.  bcodes: tables x n, qcodes: tables x nq.
int orc_search_hashed(const float* data, uint64_t n, uint32_t d, uint64_t ld, const uint64_t* gptr,
                      const uint32_t* gids, const float* q, uint64_t nq, uint64_t qld, const uint64_t* bcodes,
                      const uint64_t* qcodes, uint32_t tables, uint32_t bits, uint32_t radius, int epochs,
                      int init_num, int extend_to, uint32_t k, int mode, int threads, uint64_t seed, int32_t* out,
                      uint64_t* evals) {
  if (tables < 1 || bits < 1 || bits > 64 || init_num <= 0 || (uint64_t)init_num > n || k == 0 ||
      k > (uint32_t)init_num || epochs < 0 || extend_to < 0)
    return -1;
  if (extend_to > init_num) extend_to = init_num;  // setSearchParams (base_index.hpp:156-157)
  Data X{data, n, d, ld, mode};
  HashTabs H(bcodes, n, tables, bits, radius);
  Forest empty;
  if (mode == MODE_SEQ) srand(1);
#ifdef _OPENMP
  int nt = (mode == MODE_SEQ || threads < 1) ? 1 : threads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
  for (long long i = 0; i < (long long)nq; ++i) {
    std::vector<uint32_t> prefix = H.probe(qcodes, nq, (uint64_t)i, (unsigned)init_num);
    SearchArgs a{epochs, init_num, extend_to, 0, k};
    a.seeds = prefix.data();
    a.nseeds = (unsigned)prefix.size();
    uint64_t nd = 0;
    search_one(X, empty, gptr, gids, q + (uint64_t)i * qld, (uint64_t)i, a, mode, seed, out + (uint64_t)i * k, &nd);
    if (evals) evals[i] = nd;
  }
  return 0;
}

// getNeighborsIEH32_kgraph / getNeighborsIEH64_kgraph (hashing_index.hpp:1203-1352 and its 64-bit
// twin): the pool size is enlarged to epochs * extend_to as in the tree-seeded kgraph search
// (written back through *init_num), the pool is the probe's first init_num distinct ids plus the
// random fill, and each expanded node's whole graph row is visited.
int orc_search_hashed_kgraph(const float* data, uint64_t n, uint32_t d, uint64_t ld, const uint64_t* gptr,
                             const uint32_t* gids, const float* q, uint64_t nq, uint64_t qld, const uint64_t* bcodes,
                             const uint64_t* qcodes, uint32_t tables, uint32_t bits, uint32_t radius, int epochs,
                             int* init_num, int extend_to, uint32_t k, int mode, int threads, uint64_t seed,
                             int32_t* out, uint64_t* evals) {
  if (tables < 1 || bits < 1 || bits > 64 || !init_num || *init_num <= 0 || k == 0 || epochs < 0 || extend_to < 0)
    return -1;
  if (extend_to > *init_num) extend_to = *init_num;  // setSearchParams (base_index.hpp:156-157)
  unsigned pool_size = (unsigned)epochs * (unsigned)extend_to;
  bool sorted = true;
  if (pool_size >= (unsigned)*init_num) {  // :1212-1216
    *init_num = (int)pool_size;
    sorted = false;
  }
  if ((uint64_t)*init_num > n || *init_num <= 0) return -1;  // the random fill would not end
  Data X{data, n, d, ld, mode};
  HashTabs H(bcodes, n, tables, bits, radius);
  Forest empty;
  if (mode == MODE_SEQ) srand(1);
#ifdef _OPENMP
  int nt = (mode == MODE_SEQ || threads < 1) ? 1 : threads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
  for (long long i = 0; i < (long long)nq; ++i) {
    std::vector<uint32_t> prefix = H.probe(qcodes, nq, (uint64_t)i, (unsigned)*init_num);
    SearchArgs a{epochs, *init_num, extend_to, 0, k};
    a.seeds = prefix.data();
    a.nseeds = (unsigned)prefix.size();
    uint64_t nd = 0;
    search_one_kgraph(X, empty, gptr, gids, q + (uint64_t)i * qld, (uint64_t)i, a, 0, sorted, mode, seed,
                      out + (uint64_t)i * k, &nd, true);
    if (evals) evals[i] = nd;
  }
  return 0;
}

// getNeighbors32 / getNeighbors64 (hashing_index.hpp:929-1085, the hashing index without a graph):
// the probe's first init_num distinct ids, topped up by the random fill to k only when fewer, ranked
// by (distance, id) (partial_sort of (dist, id) pairs); the first k ids.
int orc_search_hashed_buckets(const float* data, uint64_t n, uint32_t d, uint64_t ld, const float* q, uint64_t nq,
                              uint64_t qld, const uint64_t* bcodes, const uint64_t* qcodes, uint32_t tables,
                              uint32_t bits, uint32_t radius, int init_num, uint32_t k, int mode, int threads,
                              uint64_t seed, int32_t* out) {
  if (tables < 1 || bits < 1 || bits > 64 || init_num <= 0 || k == 0 || k > (uint32_t)init_num ||
      (uint64_t)k > n)
    return -1;
  Data X{data, n, d, ld, mode};
  HashTabs H(bcodes, n, tables, bits, radius);
  if (mode == MODE_SEQ) srand(1);
#ifdef _OPENMP
  int nt = (mode == MODE_SEQ || threads < 1) ? 1 : threads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
  for (long long i = 0; i < (long long)nq; ++i) {
    std::vector<uint32_t> pool = H.probe(qcodes, nq, (uint64_t)i, (unsigned)init_num);
    if (pool.size() < k) {  // :976-985
      std::vector<uint8_t> seen(n, 0);
      for (uint32_t id : pool) seen[id] = 1;
      CRng g(hash4(seed, TAG_SFILL, (uint64_t)i, 0, 0));
      while (pool.size() < k) {
        uint32_t id = mode == MODE_SEQ ? (uint32_t)(rand() % (int)n) : g.next() % (uint32_t)n;
        if (seen[id]) continue;
        seen[id] = 1;
        pool.push_back(id);
      }
    }
    const float* qr = q + (uint64_t)i * qld;
    std::vector<std::pair<float, size_t>> result;
    for (uint32_t id : pool) result.push_back({X.distq(qr, X.row(id)), (size_t)id});
    std::partial_sort(result.begin(), result.begin() + k, result.end());
    for (uint32_t j = 0; j < k; ++j) out[(uint64_t)i * k + j] = (int32_t)result[j].second;
  }
  return 0;
}

// Batched kgraph search (getNeighbors_kgraph).  *init_num is the index's pool size; like the
// reference (kdtreeub_index.hpp:510-514) it is raised to epochs * extend_to when that is not
// smaller, and the raised value is written back for the caller's next search.
int orc_search_kgraph(const float* data, uint64_t n, uint32_t d, uint64_t ld, void* forest, const uint64_t* gptr,
                      const uint32_t* gids, const float* q, uint64_t nq, uint64_t qld, int epochs, int* init_num,
                      int extend_to, int search_trees, uint32_t k, int mode, int threads, uint64_t seed, int32_t* out,
                      uint64_t* evals) {
  Data X{data, n, d, ld, mode};
  Forest* F = (Forest*)forest;
  if (search_trees <= 0 || (size_t)search_trees > F->nodes.size()) return -1;
  if (!init_num || *init_num <= 0 || epochs < 0 || extend_to < 0) return -1;
  if (extend_to > *init_num) extend_to = *init_num;  // setSearchParams (base_index.hpp:156-157)
  unsigned lsize = (unsigned)*init_num * 2 / (5 * (unsigned)search_trees) + 1;
  unsigned pool_size = (unsigned)epochs * (unsigned)extend_to;
  bool sorted = true;
  if (pool_size >= (unsigned)*init_num) {
    *init_num = (int)pool_size;
    sorted = false;
  }
  if ((uint64_t)*init_num > n || *init_num <= 0) return -1;  // the reference's random fill would not end
  SearchArgs a{epochs, *init_num, extend_to, search_trees, k};
  if (mode == MODE_SEQ) srand(1);
#ifdef _OPENMP
  int nt = (mode == MODE_SEQ || threads < 1) ? 1 : threads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
#endif
  for (long long i = 0; i < (long long)nq; ++i)
    search_one_kgraph(X, *F, gptr, gids, q + (uint64_t)i * qld, (uint64_t)i, a, lsize, sorted, mode, seed,
                      out + (uint64_t)i * k, evals ? evals + i : nullptr);
  return 0;
}

}  // extern "C"
