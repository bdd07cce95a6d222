// NN-descent kNN-graph build: leaf-merge initial graph, then `epochs` x (join, update).
//
// Reference (ZJULearning/efanna):
//   initGraph's merge + pool seeding   algorithm/kdtreeub_index.hpp:1000-1081, 1367-1424
//   Point / InsertIntoKnn / insert      algorithm/base_index.hpp:24-93
//   join                                algorithm/base_index.hpp:328-371
//   update                              algorithm/base_index.hpp:373-437
//   refineGraph                         algorithm/base_index.hpp:438-481
//
// Order independence.  The reference applies neighbour-list inserts in whatever order its
// OpenMP threads reach them; its results depend on that order only through ties and through the
// rank an insert lands at.  Here every insert aimed at node t is first materialised as a record
// (dist, candidate, source node, side), the records of t are applied in ascending order of that
// tuple with exactly the reference's insert semantics (radius test, InsertIntoKnn with its
// equal-distance duplicate check and overflow slot, L growth, radius update, rank-based `found`),
// and everything else (reverse-list sampling, initial extra candidates, random fills) comes from
// counter hashes.  A build is therefore a pure function of (data, params), reproduced bit-for-bit
// by the oracle's canonical mode.
//
// Device state (n nodes, pool capacity P = L + 1):
//   pd[n*P]  pool distances           pid[n*P] pool ids, bit 31 = the "new" flag
//   Lc[n], Range[n], radius[n], radiusM[n], found[n]
//   new_ids/old_ids[n*cap] + counts   the sampled lists the next join reads
// Pool slots past L stay zero (dist 0, id 0) until written, as the reference's freshly
// allocated pools are; update() reads pool[L].dist as the next radius either way.
#include <algorithm>
#include <cfloat>
#include <vector>

#include "join.cuh"
#include "scan.cuh"
#include "warpsort.cuh"

namespace efg {

static constexpr uint32_t FLAG = 0x80000000u;
static constexpr uint32_t IDM = 0x7FFFFFFFu;

struct NNDev {
  uint64_t n = 0;
  uint32_t P = 0, cap = 0;
  DevBuf<float> pd, radius, radiusM;
  DevBuf<uint32_t> pid, Lc, Range, new_ids, new_cnt, old_ids, old_cnt;
  DevBuf<uint8_t> found;
  // scratch
  DevBuf<uint64_t> pair_off, rec_off64, scan64;
  DevBuf<float> pairdist;
  DevBuf<uint32_t> cnt, cursor, rec_aux, rcnt, rcur, roff, rbuf, scan32, ucnt;
  DevBuf<uint64_t> rec_key;
  // tensor-core join: BF16 rows (hi, lo), FP32 norms, flags {inexact, error}, nodes left to FP32
  DevBuf<__nv_bfloat16> jhi, jlo;
  DevBuf<float> jnorm;
  DevBuf<int> jflag;
  DevBuf<uint32_t> jmid, jbig;  // nodes of 129-256 rows, and larger ones (count in word 0)
  uint32_t jterms = 0;  // 0: not prepared; 1 or 3 products per value
  void release_all() {
    pd.release(); radius.release(); radiusM.release(); pid.release(); Lc.release(); Range.release();
    new_ids.release(); new_cnt.release(); old_ids.release(); old_cnt.release(); found.release();
    pair_off.release(); rec_off64.release(); scan64.release(); pairdist.release(); cnt.release(); cursor.release();
    rec_aux.release(); rcnt.release(); rcur.release(); roff.release(); rbuf.release(); scan32.release();
    ucnt.release(); rec_key.release(); jhi.release(); jlo.release(); jnorm.release(); jflag.release();
    jmid.release();
    jbig.release();
    jterms = 0;
  }
};

static int nn_alloc(NNDev& S, uint64_t n, uint32_t L, uint32_t cap) {
  S.n = n;
  S.P = L + 1;
  S.cap = cap;
  uint64_t np = n * S.P;
  EFG_TRY(S.pd.reserve(np));
  EFG_TRY(S.pid.reserve(np));
  EFG_TRY(S.Lc.reserve(n));
  EFG_TRY(S.Range.reserve(n));
  EFG_TRY(S.radius.reserve(n));
  EFG_TRY(S.radiusM.reserve(n));
  EFG_TRY(S.found.reserve(n));
  EFG_TRY(S.new_ids.reserve(n * cap));
  EFG_TRY(S.old_ids.reserve(n * cap));
  EFG_TRY(S.new_cnt.reserve(n));
  EFG_TRY(S.old_cnt.reserve(n));
  return EFG_OK;
}

// Warp-cooperative partial squared distance between rows a and b (lane owns float4 chunks).
__device__ __forceinline__ float lane_l2_rows(const float* __restrict__ base, uint32_t ld4, uint32_t a, uint32_t b) {
  const float4* ra = reinterpret_cast<const float4*>(base) + (uint64_t)a * ld4;
  const float4* rb = reinterpret_cast<const float4*>(base) + (uint64_t)b * ld4;
  uint32_t lane = threadIdx.x & 31;
  float acc = 0.f;
  for (uint32_t c = lane; c < ld4; c += 32) {
    float4 x = __ldg(ra + c), y = __ldg(rb + c);
    float d0 = x.x - y.x, d1 = x.y - y.y, d2 = x.z - y.z, d3 = x.w - y.w;
    acc += d0 * d0;
    acc += d1 * d1;
    acc += d2 * d2;
    acc += d3 * d3;
  }
  return acc;
}

// =============================================================================================
// Initial graph: leaf merge (mergeSubGraphs) and pool seeding.
// =============================================================================================

struct TreeView {
  const DNode* nodes;
  const int32_t *left, *right, *level, *tree;
  const uint32_t *start, *end;
  const uint32_t* leaves;
  uint64_t n;
};

// Merge tasks: internal nodes of the graph trees at depth >= ml.  len = size of the smaller child.
__global__ void merge_task_len_kernel(TreeView tv, uint64_t nnodes, uint32_t trees_build, int32_t ml,
                                      uint64_t* __restrict__ len) {
  uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nnodes) return;
  uint64_t l = 0;
  if (tv.left[v] >= 0 && (uint32_t)tv.tree[v] < trees_build && tv.level[v] >= ml) {
    int32_t L = tv.left[v], R = tv.right[v];
    uint64_t nl = tv.end[L] - tv.start[L], nr = tv.end[R] - tv.start[R];
    l = nl < nr ? nl : nr;
  }
  len[v] = l;
}

__global__ void min_leaf_level_kernel(TreeView tv, uint64_t nnodes, uint32_t trees_build, int32_t* __restrict__ out) {
  uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nnodes) return;
  if (tv.left[v] < 0 && (uint32_t)tv.tree[v] < trees_build) atomicMin(out, tv.level[v]);
}

// One warp per routed point: descend the larger child to a leaf (SearchToLeaf,
// kdtreeub_index.hpp:1012-1021) and compare with each leaf point.  pass 0 counts records per
// target, pass 1 writes them: key = (dist bits << 32) | candidate.  With task_d set, pass 0 also
// keeps each task's point, leaf and distances (maxl per task), and merge_emit_kernel writes the
// records from them instead of a second routing pass.
template <int PASS>
__global__ void __launch_bounds__(256, 3) merge_route_kernel(const float* __restrict__ base, uint32_t ld4, TreeView tv,
                                   const uint64_t* __restrict__ task_off, uint64_t nnodes, uint64_t ntasks,
                                   uint32_t* __restrict__ cnt, const uint64_t* __restrict__ off,
                                   uint32_t* __restrict__ cursor, uint64_t* __restrict__ keys,
                                   unsigned long long* __restrict__ ndist, uint32_t* __restrict__ task_p,
                                   int32_t* __restrict__ task_leaf, float* __restrict__ task_d, uint32_t maxl) {
  // a warp routes 32 consecutive tasks at once, one per lane (search and descent are chains of
  // dependent loads: the lanes run theirs side by side), then the whole warp computes each task's
  // leaf distances in turn
  const uint64_t gwarp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long local = 0;
  const float* fb = base;
  for (uint64_t wb = gwarp * 32; wb < ntasks; wb += nwarps * 32) {
    const uint64_t myw = wb + lane;
    uint32_t myp = 0, mls = 0, mle = 0;
    uint64_t mt = 0;
    if (myw < ntasks) {
      // node owning task myw: last v with task_off[v] <= myw
      uint64_t lo = 0, hi = nnodes;
      while (hi - lo > 1) {
        uint64_t mid = (lo + hi) >> 1;
        if (task_off[mid] <= myw) lo = mid;
        else hi = mid;
      }
      const uint64_t v = lo;
      int32_t L = tv.left[v], R = tv.right[v];
      uint64_t nl = tv.end[L] - tv.start[L], nr = tv.end[R] - tv.start[R];
      int32_t cur = nl < nr ? R : L;
      int32_t small = nl < nr ? L : R;
      mt = (uint64_t)tv.tree[v];
      myp = tv.leaves[mt * tv.n + tv.start[small] + (myw - task_off[v])];
      DNode nd = tv.nodes[cur];
      while (nd.left >= 0) {
        float x = __ldg(fb + (uint64_t)myp * (ld4 * 4) + nd.div_dim);
        cur = x < nd.div_val ? nd.left : nd.right;
        nd = tv.nodes[cur];
      }
      mls = (uint32_t)(-(nd.left + 1));
      mle = (uint32_t)nd.right;
      if (PASS == 0 && task_d) {
        task_p[myw] = myp;
        task_leaf[myw] = cur;
      }
    }
    const uint32_t ntask = ntasks - wb < 32 ? (uint32_t)(ntasks - wb) : 32u;
    for (uint32_t j = 0; j < ntask; ++j) {
      const uint64_t w = wb + j;
      const uint32_t p = __shfl_sync(0xffffffffu, myp, j);
      const uint32_t ls = __shfl_sync(0xffffffffu, mls, j), le = __shfl_sync(0xffffffffu, mle, j);
      const uint64_t t = __shfl_sync(0xffffffffu, mt, j);
      const uint32_t* ll = tv.leaves + t * tv.n;
      const float4* rp = reinterpret_cast<const float4*>(base) + (uint64_t)p * ld4;
      for (uint32_t i0 = ls; i0 < le; i0 += 8) {  // eight leaf points at a time, their loads in flight together
        const uint32_t cnt8 = min(8u, le - i0);
        uint32_t qq[8];
        float acc[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          qq[u] = ll[i0 + min((uint32_t)u, cnt8 - 1)];
          acc[u] = 0.f;
        }
        for (uint32_t c = lane; c < ld4; c += 32) {
          float4 y = __ldg(rp + c);
          float4 x[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) x[u] = __ldg(reinterpret_cast<const float4*>(base) + (uint64_t)qq[u] * ld4 + c);
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            float d0 = x[u].x - y.x, d1 = x[u].y - y.y, d2 = x[u].z - y.z, d3 = x[u].w - y.w;
            acc[u] += d0 * d0;
            acc[u] += d1 * d1;
            acc[u] += d2 * d2;
            acc[u] += d3 * d3;
          }
        }
        const float d = reduce8_rows(acc, lane);  // lanes 4r .. 4r+3: leaf point r's distance
        const uint32_t r = lane >> 2;
        uint32_t q = qq[0];
#pragma unroll
        for (int u = 1; u < 8; ++u)
          if (r == (uint32_t)u) q = qq[u];
        local += cnt8;
        if ((lane & 3) == 0 && r < cnt8) {
          if (PASS == 0) {
            if (task_d) task_d[w * maxl + (i0 - ls) + r] = d;
            atomicAdd(&cnt[q], 1u);
            atomicAdd(&cnt[p], 1u);
          } else {
            uint32_t a = atomicAdd(&cursor[q], 1u);
            keys[off[q] + a] = pack_key(d, p);
            uint32_t b = atomicAdd(&cursor[p], 1u);
            keys[off[p] + b] = pack_key(d, q);
          }
        }
      }
    }
  }
  if (PASS == 0 && lane == 0 && local) atomicAdd(ndist, local);
}

// Records of the leaf merge from what pass 0 kept: one thread per task.
__global__ void merge_emit_kernel(TreeView tv, uint64_t ntasks, const uint32_t* __restrict__ task_p,
                                  const int32_t* __restrict__ task_leaf, const float* __restrict__ task_d,
                                  uint32_t maxl, const uint64_t* __restrict__ off, uint32_t* __restrict__ cursor,
                                  uint64_t* __restrict__ keys) {
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < ntasks;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = task_p[w];
    const int32_t leaf = task_leaf[w];
    const DNode nd = tv.nodes[leaf];
    const uint32_t* ll = tv.leaves + (uint64_t)tv.tree[leaf] * tv.n;
    const uint32_t ls = (uint32_t)(-(nd.left + 1)), le = (uint32_t)nd.right;
    for (uint32_t i = ls; i < le; ++i) {
      const uint32_t q = ll[i];
      const float d = task_d[w * maxl + (i - ls)];
      uint32_t a = atomicAdd(&cursor[q], 1u);
      keys[off[q] + a] = pack_key(d, p);
      uint32_t b = atomicAdd(&cursor[p], 1u);
      keys[off[p] + b] = pack_key(d, q);
    }
  }
}

// Largest leaf of the forest (points per leaf).
__global__ void max_leaf_kernel(TreeView tv, uint64_t nnodes, uint32_t* __restrict__ out) {
  uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nnodes) return;
  if (tv.left[v] < 0) atomicMax(out, (uint32_t)(tv.end[v] - tv.start[v]));
}

// Position of x in the ascending warp-distributed list t (number of elements < x), or -1 if an
// element equals x.
// Every lane must call this (fixed five shuffle steps, no lane-dependent trip count).
__device__ __forceinline__ int warp_find(uint64_t t, uint64_t x) {
  int pos = 0;  // number of elements < x (branchless lower bound over 32 sorted lanes)
#pragma unroll
  for (int step = 16; step > 0; step >>= 1) {
    uint64_t v = __shfl_sync(0xffffffffu, t, pos + step - 1);
    if (v < x) pos += step;
  }
  uint64_t at = __shfl_sync(0xffffffffu, t, pos < 32 ? pos : 31);
  return (pos < 32 && at == x) ? -1 : pos;
}

// Folds one batch (one key per lane, ~0 = none) into the running ascending list of distinct keys.
__device__ __forceinline__ uint64_t fold_distinct(uint64_t run, uint64_t x) {
  uint32_t lane = threadIdx.x & 31;
  uint32_t same = __match_any_sync(0xffffffffu, x);
  if ((same & ((1u << lane) - 1)) != 0) x = ~0ULL;  // keep the lowest lane of each equal group
  int found_at = warp_find(run, x);
  if (x != ~0ULL && found_at < 0) x = ~0ULL;
  x = warp_sort32(x);
  return warp_merge_min32(run, x);
}

// One warp per node: S best distinct (dist, id) keys, S extra join candidates, pool seeding.
__global__ void init_select_kernel(const float* __restrict__ base, uint32_t ld4, uint64_t n, uint32_t S, uint32_t P,
                                   uint32_t cap, uint64_t seed, const uint32_t* __restrict__ cnt,
                                   const uint64_t* __restrict__ off, const uint64_t* __restrict__ keys,
                                   float* __restrict__ pd, uint32_t* __restrict__ pid, uint32_t* __restrict__ Lc,
                                   uint32_t* __restrict__ Range, float* __restrict__ radius,
                                   float* __restrict__ radiusM, uint8_t* __restrict__ found,
                                   uint32_t* __restrict__ new_ids, uint32_t* __restrict__ new_cnt,
                                   uint32_t* __restrict__ old_cnt) {
  uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t lane = threadIdx.x & 31;
  if (t >= n) return;
  const uint64_t* R = keys + off[t];
  uint32_t B = cnt[t];
  // 1. the smallest distinct keys (up to 32)
  uint64_t run = ~0ULL;
  for (uint32_t b = 0; b < B; b += 32) {
    uint64_t x = b + lane < B ? R[b + lane] : ~0ULL;
    run = fold_distinct(run, x);
  }
  uint32_t nvalid = __popc(__ballot_sync(0xffffffffu, run != ~0ULL));
  // 2. top up to S distinct with counter-hash random ids (kdtreeub_index.hpp:1399-1405)
  if (nvalid < S) {
    CRng g(hash4(seed, TAG_TOPUP, t, 0, 0));
    uint32_t guard = 0;
    while (nvalid < S && guard < 1000000u) {
      ++guard;
      uint32_t rid = g.next() % (uint32_t)n;
      float d = warp_sum(lane_l2_rows(base, ld4, (uint32_t)t, rid));
      uint64_t x = lane == 0 ? pack_key(d, rid) : ~0ULL;
      run = fold_distinct(run, x);
      nvalid = __popc(__ballot_sync(0xffffffffu, run != ~0ULL));
    }
  }
  uint64_t kth = __shfl_sync(0xffffffffu, run, S - 1);
  // 3. extras: S of the distinct keys beyond the S best, by smallest (hash, id); needs >= 2S
  uint64_t hrun = ~0ULL;
  if (kth != ~0ULL) {
    for (uint32_t b = 0; b < B; b += 32) {
      uint64_t x = ~0ULL;
      if (b + lane < B) {
        uint64_t k = R[b + lane];
        if (k > kth) {
          uint32_t c = (uint32_t)k;
          x = ((hash4(seed, TAG_EXTRA, t, c, 0) >> 32) << 32) | c;
        }
      }
      hrun = fold_distinct(hrun, x);
    }
  }
  uint32_t nh = __popc(__ballot_sync(0xffffffffu, hrun != ~0ULL));
  uint32_t extra = 0;  // lane l < S holds extra id l
  if (nh >= 2 * S) {
    extra = (uint32_t)hrun;
  } else if (lane == 0) {
    // GenRandom(2S) (kdtreeub_index.hpp:1121-1135) on a counter stream; keep positions S..2S-1
    uint32_t addr[32];
    uint32_t size = 2 * S, N = (uint32_t)n;
    CRng g(hash4(seed, TAG_GENRAND, t, 0, 0));
    for (uint32_t i = 0; i < size; ++i) addr[i] = g.next() % (N - size);
    for (uint32_t i = 1; i < size; ++i) {  // insertion sort
      uint32_t v = addr[i];
      int j = (int)i - 1;
      while (j >= 0 && addr[j] > v) {
        addr[j + 1] = addr[j];
        --j;
      }
      addr[j + 1] = v;
    }
    for (uint32_t i = 1; i < size; ++i)
      if (addr[i] <= addr[i - 1]) addr[i] = addr[i - 1] + 1;
    uint32_t offr = g.next() % N;
    for (uint32_t i = 0; i < S; ++i) new_ids[t * cap + S + i] = (addr[S + i] + offr) % N;
  }
  // 4. seed the pool and the first new list (lane j < S holds the j-th best key)
  uint64_t prow = t * P;
  uint64_t mine = run;
  for (uint32_t j = lane; j < P; j += 32) {
    float dd = 0.f;
    uint32_t ii = 0;
    if (j < S) {
      dd = key_dist(mine);
      ii = key_id(mine) | FLAG;
    }
    pd[prow + j] = dd;
    pid[prow + j] = ii;
  }
  if (lane < S) new_ids[t * cap + lane] = key_id(run);
  if (nh >= 2 * S && lane < S) new_ids[t * cap + S + lane] = extra;
  if (lane == 0) {
    Lc[t] = S;
    Range[t] = S;
    radius[t] = FLT_MAX;
    radiusM[t] = 0.f;
    found[t] = 0;
    new_cnt[t] = 2 * S;
    old_cnt[t] = 0;
  }
}

// =============================================================================================
// Join.
// =============================================================================================

// Pairs of node i's join: new x new with p < q (skipped when the ids are equal) and new x old.
__global__ void pair_count_kernel(uint64_t n, const uint32_t* __restrict__ new_cnt,
                                  const uint32_t* __restrict__ old_cnt, uint64_t* __restrict__ pairs) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t a = new_cnt[i], b = old_cnt[i];
  pairs[i] = a * (a - (a > 0 ? 1 : 0)) / 2 + a * b;
}

// The largest distance any insert aimed at node t can still be accepted at during this join:
// max(radius, pool[L-1].dist).  Inserts beyond it are rejected by Neighbor::insert whatever the
// order (the radius never rises above it), so their records need not be materialised.
__global__ void bound_kernel(uint64_t n, uint32_t P, const float* __restrict__ pd, const uint32_t* __restrict__ Lc,
                             const float* __restrict__ radius, float* __restrict__ bound) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float r = radius[t];
  float w = pd[t * P + Lc[t] - 1];
  bound[t] = r > w ? r : w;
}

// Join pass 0: the distances of node i's pairs, stored, and record counts per target.  One warp
// per node, nodes taken from a shared counter as warps come free (pair counts differ by an order
// of magnitude, so a fixed assignment leaves most warps of a block idle behind its longest node).
// New entries are taken two at a time: x0 = new[p] pairs with Y = new[p+1..] + old, x1 = new[p+1]
// with Y[1..], so every candidate row loaded serves both; four rows per pass, the 2 x 4 sums
// reduced together.
__global__ void __launch_bounds__(256, 4) join_dist_kernel(
    const float* __restrict__ base, uint32_t ld4, uint64_t n, uint32_t cap, uint32_t P, uint32_t check_k,
    const uint32_t* __restrict__ new_ids, const uint32_t* __restrict__ new_cnt, const uint32_t* __restrict__ old_ids,
    const uint32_t* __restrict__ old_cnt, const uint64_t* __restrict__ pair_off, const float* __restrict__ bound,
    float* __restrict__ pairdist, uint32_t* __restrict__ cnt, uint8_t* __restrict__ found,
    uint32_t* __restrict__ next_node) {
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t ii = 0;
    if (lane == 0) ii = atomicAdd(next_node, 1u);
    const uint64_t i = __shfl_sync(0xffffffffu, ii, 0);
    if (i >= n) return;
    const uint32_t nn = new_cnt[i], no = old_cnt[i];
    if (nn == 0) continue;
    const uint32_t* nw = new_ids + i * cap;
    const uint32_t* od = old_ids + i * cap;
    const uint64_t po = pair_off[i];
    bool found_drop = false;
    for (uint32_t p = 0; p < nn; p += 2) {
      const bool two = p + 1 < nn;
      const uint32_t x0 = nw[p], x1 = two ? nw[p + 1] : x0;
      const uint32_t nl = nn - 1 - p;  // new-list candidates of x0
      const uint32_t m = nl + no;      // Y positions (x1 takes positions 1..m-1)
      const float4* r0 = reinterpret_cast<const float4*>(base) + (uint64_t)x0 * ld4;
      const float4* r1 = reinterpret_cast<const float4*>(base) + (uint64_t)x1 * ld4;
      for (uint32_t cb = 0; cb < m; cb += 32) {
        const uint32_t cm = min(32u, m - cb);
        // lane l's candidate (position cb + l; the last one repeated past cm), loaded once per
        // chunk and handed to the passes by shuffles
        const uint32_t cl = cb + min(lane, cm - 1);
        const uint32_t cand = cl < nl ? nw[p + 1 + cl] : od[cl - nl];
        float mine0 = 0.f, mine1 = 0.f;
        for (uint32_t u0 = 0; u0 < cm; u0 += 4) {
          float acc[8];  // [0..4): x0 against rows u0..u0+3, [4..8): x1 against them
          const float4* ry[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            uint32_t yu = __shfl_sync(0xffffffffu, cand, min(u0 + u, cm - 1));
            ry[u] = reinterpret_cast<const float4*>(base) + (uint64_t)yu * ld4;
            acc[u] = 0.f;
            acc[u + 4] = 0.f;
          }
          for (uint32_t c4 = lane; c4 < ld4; c4 += 32) {
            const float4 a = __ldg(r0 + c4), b = __ldg(r1 + c4);
            float4 yv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) yv[u] = __ldg(ry[u] + c4);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              float d0 = a.x - yv[u].x, d1 = a.y - yv[u].y, d2 = a.z - yv[u].z, d3 = a.w - yv[u].w;
              acc[u] += d0 * d0;
              acc[u] += d1 * d1;
              acc[u] += d2 * d2;
              acc[u] += d3 * d3;
              float e0 = b.x - yv[u].x, e1 = b.y - yv[u].y, e2 = b.z - yv[u].z, e3 = b.w - yv[u].w;
              acc[u + 4] += e0 * e0;
              acc[u + 4] += e1 * e1;
              acc[u + 4] += e2 * e2;
              acc[u + 4] += e3 * e3;
            }
          }
          // lanes 4r .. 4r+3 end with sum r: r < 4 x0's row u0+r, r >= 4 x1's row u0+r-4; row
          // u's sums move to lane u0 + u
          const float tot = reduce8_rows(acc, lane);
          const uint32_t u = (lane - u0) & 3;
          const float d0 = __shfl_sync(0xffffffffu, tot, u * 4), d1 = __shfl_sync(0xffffffffu, tot, (u + 4) * 4);
          if (lane - u0 < 4u) {
            mine0 = d0;
            mine1 = d1;
          }
        }
        const uint32_t c = cb + lane;
        if (lane < cm) {
          const bool my_new = c < nl;
          found_drop |= join_lane_record<0>(i, x0, cand, my_new, mine0, join_slot(po, nn, no, p, c), P, check_k,
                                            bound, pairdist, cnt, nullptr, nullptr, nullptr, nullptr);
          if (two && c >= 1)  // x1's candidate c - 1 (new exactly when x0's candidate c is)
            found_drop |= join_lane_record<0>(i, x1, cand, my_new, mine1, join_slot(po, nn, no, p + 1, c - 1), P,
                                              check_k, bound, pairdist, cnt, nullptr, nullptr, nullptr, nullptr);
        }
      }
    }
    if (__any_sync(0xffffffffu, found_drop) && lane == 0) found[i] = 1;
  }
}

// Join pass 1: node i's records written from the stored distances (warps take nodes from a
// shared counter, as in pass 0).
__global__ void __launch_bounds__(256, 4) join_records_kernel(
    uint64_t n, uint32_t cap, uint32_t P, uint32_t check_k, const uint32_t* __restrict__ new_ids,
    const uint32_t* __restrict__ new_cnt, const uint32_t* __restrict__ old_ids, const uint32_t* __restrict__ old_cnt,
    const uint64_t* __restrict__ pair_off, const float* __restrict__ bound, float* __restrict__ pairdist,
    const uint64_t* __restrict__ rec_off, uint32_t* __restrict__ cursor, uint64_t* __restrict__ rec_key,
    uint32_t* __restrict__ rec_aux, uint32_t* __restrict__ next_node) {
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    uint32_t ii = 0;
    if (lane == 0) ii = atomicAdd(next_node, 1u);
    const uint64_t i = __shfl_sync(0xffffffffu, ii, 0);
    if (i >= n) return;
    const uint32_t nn = new_cnt[i], no = old_cnt[i];
    if (nn == 0) continue;
    const uint32_t* nw = new_ids + i * cap;
    const uint32_t* od = old_ids + i * cap;
    const uint64_t po = pair_off[i];
    for (uint32_t p = 0; p < nn; ++p) {
      const uint32_t x = nw[p], nl = nn - 1 - p, m = nl + no;
      for (uint32_t c = lane; c < m; c += 32) {
        const bool my_new = c < nl;
        const uint32_t y = my_new ? nw[p + 1 + c] : od[c - nl];
        join_lane_record<1>(i, x, y, my_new, 0.f, join_slot(po, nn, no, p, c), P, check_k, bound, pairdist, nullptr,
                            rec_off, cursor, rec_key, rec_aux);
      }
    }
  }
}

// Pool of one node held by a warp: entry e on lane e % 32, slot e / 32.
template <int NS>
struct WarpPool {
  float d[NS];
  uint32_t id[NS];  // with FLAG
};

// Next 32 records of a bucket in ascending (key, aux) order from `last` on (copies of `last`
// included: the caller skips the ones it has applied).
__device__ __forceinline__ K96 next_batch(const uint64_t* __restrict__ rk, const uint32_t* __restrict__ ra,
                                          uint32_t B, K96 last, bool first) {
  uint32_t lane = threadIdx.x & 31;
  K96 run = k96_max();
  for (uint32_t b = 0; b < B; b += 32) {
    K96 x = k96_max();
    if (b + lane < B) {
      K96 y{rk[b + lane], ra[b + lane]};
      if (first || !lt(y, last)) x = y;
    }
    if (__all_sync(0xffffffffu, is_max(x))) continue;
    x = warp_sort32(x);
    run = warp_merge_min32(run, x);
  }
  return run;
}

// Ascending bitonic sort of Bp records (keys sk, aux sa; Bp a power of two >= 32) in shared
// memory by one warp.
__device__ __forceinline__ void warp_sort_smem(uint64_t* sk, uint32_t* sa, uint32_t Bp) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint32_t k = 2; k <= Bp; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t t = lane; t < Bp / 2; t += 32) {
        const uint32_t i = ((t & ~(j - 1)) << 1) | (t & (j - 1)), l = i + j;
        const K96 x{sk[i], sa[i]}, y{sk[l], sa[l]};
        if ((i & k) == 0 ? lt(y, x) : lt(x, y)) {
          sk[i] = y.k;
          sa[i] = y.a;
          sk[l] = x.k;
          sa[l] = x.a;
        }
      }
      __syncwarp();
    }
  }
}

constexpr uint32_t MERGE_WARPS = 4;  // warps per merge block

// Lane of the smallest of the warp's 32 records (the lower lane on a tie), on every lane.
__device__ __forceinline__ uint32_t warp_argmin(K96 x) {
  uint32_t who = threadIdx.x & 31;
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    const K96 y = shfl_xor(x, m);
    const uint32_t wy = __shfl_xor_sync(0xffffffffu, who, m);
    if (lt(y, x) || (!lt(x, y) && wy < who)) {
      x = y;
      who = wy;
    }
  }
  return who;
}

// One warp per target node: applies its records in ascending (dist, id, source, side) order,
// every one of them (repeats of a record included), with Neighbor::insert / InsertIntoKnn
// semantics (base_index.hpp:37-61).  The order comes from one of three sources:
//   * 129 to msort records: sorted once in the warp's shared memory;
//   * up to 32 x msort: runs of msort sorted in shared memory and written back in place, then
//     merged 32 ways (lane l holds run l's head; msort / 32 records of each run staged in shared
//     memory);
//   * up to 128, or more than 32 x msort: pulled 32 at a time by scanning all of them.
// The reference rejects a candidate whose id sits among the entries of equal distance; a pair's
// distance is the same wherever the reference computes it, so that finds every repeat.  With
// any_dist a repeat is found at any distance: the tensor-core join's distances can differ in the
// last bits from the FP32 ones a pool entry was inserted with, and an equal-distance test would
// let the id in twice.
template <int NS>
__global__ void merge_kernel(uint64_t n, uint32_t P, uint32_t check_k, bool any_dist, uint32_t msort,
                 const uint32_t* __restrict__ cnt, const uint64_t* __restrict__ rec_off, uint64_t* __restrict__ rec_key,
                 uint32_t* __restrict__ rec_aux, float* __restrict__ pd, uint32_t* __restrict__ pid,
                 uint32_t* __restrict__ Lc, float* __restrict__ radius, uint8_t* __restrict__ found,
                 uint32_t* __restrict__ next_node) {
  extern __shared__ uint64_t merge_smem[];  // per warp: msort keys, then msort aux
  const uint32_t lane = threadIdx.x & 31;
  uint64_t* sk = merge_smem + (size_t)(threadIdx.x >> 5) * (msort + msort / 2);
  uint32_t* sa = reinterpret_cast<uint32_t*>(sk + msort);
  for (;;) {  // nodes taken from a shared counter as warps come free (their record counts differ)
  uint32_t tt = 0;
  if (lane == 0) tt = atomicAdd(next_node, 1u);
  const uint64_t t = __shfl_sync(0xffffffffu, tt, 0);
  if (t >= n) return;
  const uint32_t B = cnt[t];
  if (B == 0) continue;
  uint64_t* rk = rec_key + rec_off[t];
  uint32_t* ra = rec_aux + rec_off[t];
  WarpPool<NS> pool;
  const uint64_t prow = t * P;
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    uint32_t e = s * 32 + lane;
    pool.d[s] = e < P ? pd[prow + e] : 0.f;
    pool.id[s] = e < P ? pid[prow + e] : 0u;
  }
  uint32_t L = Lc[t];
  float rad = radius[t];
  bool rejected = false;
  K96 rej{0, 0};

  // Applies record r; true when r is rejected (every later record is too).
  auto apply = [&](const K96 r) -> bool {
    const float d = key_dist(r.k);
    const uint32_t cand = key_id(r.k);
    uint32_t rank;
    if (d > rad) {
      rejected = true;
      rej = r;
      return true;
    }
    // i = entries of [0, L) with dist <= d
    uint32_t i = 0, dup = 0;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      uint32_t e = s * 32 + lane;
      i += __popc(__ballot_sync(0xffffffffu, e < L && pool.d[s] <= d));
    }
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      uint32_t e = s * 32 + lane;
      dup |= __ballot_sync(0xffffffffu,
                           (any_dist ? e < L : (e < i && pool.d[s] == d)) && (pool.id[s] & IDM) == cand);
    }
    if (dup) {
      rank = L + 1;
    } else {
      // shift [i, L) up by one; entry L (<= P-1) receives entry L-1
#pragma unroll
      for (int s = NS - 1; s >= 0; --s) {
        float ud = __shfl_up_sync(0xffffffffu, pool.d[s], 1);
        uint32_t ui = __shfl_up_sync(0xffffffffu, pool.id[s], 1);
        if (s > 0) {
          float cd = __shfl_sync(0xffffffffu, pool.d[s > 0 ? s - 1 : 0], 31);
          uint32_t ci = __shfl_sync(0xffffffffu, pool.id[s > 0 ? s - 1 : 0], 31);
          if (lane == 0) {
            ud = cd;
            ui = ci;
          }
        }
        uint32_t e = s * 32 + lane;
        if (e > i && e <= L) {
          pool.d[s] = ud;
          pool.id[s] = ui;
        } else if (e == i) {
          pool.d[s] = d;
          pool.id[s] = cand | FLAG;
        }
      }
      rank = i;
      if (L + 1 < P) {
        ++L;
      } else {
        uint32_t e = L - 1;
        float v = 0.f;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          float w = __shfl_sync(0xffffffffu, pool.d[s], e & 31);
          if ((uint32_t)s == e / 32) v = w;
        }
        rad = v;
      }
    }
    if ((r.a & 1u) == 0 && rank < check_k && lane == 0) found[r.a >> 1] = 1;
    return false;
  };

  const uint32_t runs = (B + msort - 1) / msort;
  if (B > 128 && runs <= 32) {  // (a few batches of a small node: scanning, which stops at a rejection)
    // sort each run of msort records in shared memory (a single run stays there)
    for (uint32_t q = 0; q < runs; ++q) {
      const uint32_t b0 = q * msort, len = min(msort, B - b0);
      uint32_t Bp = 32;
      while (Bp < len) Bp <<= 1;
      for (uint32_t b = lane; b < Bp; b += 32) {
        sk[b] = b < len ? rk[b0 + b] : ~0ULL;
        sa[b] = b < len ? ra[b0 + b] : 0xffffffffu;
      }
      __syncwarp();
      warp_sort_smem(sk, sa, Bp);
      if (runs > 1) {
        for (uint32_t b = lane; b < len; b += 32) {
          rk[b0 + b] = sk[b];
          ra[b0 + b] = sa[b];
        }
        __syncwarp();
      }
    }
    if (runs == 1) {
      bool stop = false;
      for (uint32_t base = 0; base < B && !stop; base += 32) {
        const K96 batch = base + lane < B ? K96{sk[base + lane], sa[base + lane]} : k96_max();
        const uint32_t m = min(32u, B - base);
        for (uint32_t u = 0; u < m; ++u)
          if (apply(shfl_idx(batch, u))) {
            stop = true;
            break;
          }
      }
    } else {
      // 32-way merge: lane q holds run q's head; run q's records [ws, ws + SD) staged at
      // sk/sa[SD q ..]
      const uint32_t SD = msort / 32;
      const uint32_t my_len = lane < runs ? min(msort, B - lane * msort) : 0;
      uint32_t at = 0, ws = 0;  // lane q: next record of run q, first staged record of run q
      for (uint32_t q = 0; q < runs; ++q) {
        const uint32_t len = min(msort, B - q * msort);
        if (lane < SD && lane < len) {
          sk[SD * q + lane] = rk[q * msort + lane];
          sa[SD * q + lane] = ra[q * msort + lane];
        }
      }
      __syncwarp();
      for (;;) {
        const K96 head = at < my_len ? K96{sk[SD * lane + at - ws], sa[SD * lane + at - ws]} : k96_max();
        const uint32_t w = warp_argmin(head);
        const K96 r = shfl_idx(head, w);
        if (is_max(r)) break;
        if (apply(r)) break;
        if (lane == w) ++at;
        const uint32_t wat = __shfl_sync(0xffffffffu, at, w), wws = __shfl_sync(0xffffffffu, ws, w);
        const uint32_t wlen = __shfl_sync(0xffffffffu, my_len, w);
        if (wat == wws + SD && wat < wlen) {  // run w's staged records are spent: stage the next SD
          __syncwarp();
          if (lane < SD && wat + lane < wlen) {
            sk[SD * w + lane] = rk[w * msort + wat + lane];
            sa[SD * w + lane] = ra[w * msort + wat + lane];
          }
          __syncwarp();
          if (lane == w) ws = wat;
        }
      }
    }
  } else {
    // scanning: the next 32 records from the last applied one on, copies of it included
    K96 last{0, 0};
    uint32_t last_n = 0;  // copies of `last` applied so far
    bool first = true, stop = false;
    while (!stop) {
      const K96 batch = next_batch(rk, ra, B, last, first);
      first = false;
      uint32_t skip = last_n;  // the batch starts with every copy of `last`
      bool applied = false;
      for (int u = 0; u < 32; ++u) {
        const K96 r = shfl_idx(batch, u);
        if (is_max(r)) {
          stop = true;
          break;
        }
        if (skip) {
          --skip;
          continue;
        }
        applied = true;
        if (last_n && r.k == last.k && r.a == last.a) {
          ++last_n;
        } else {
          last = r;
          last_n = 1;
        }
        if (apply(r)) {
          stop = true;
          break;
        }
      }
      if (!applied) break;  // a batch of nothing but applied copies (more than 32 repeats)
    }
  }
  if (rejected && P < check_k) {
    // every record from `rej` on was rejected with rank P < check_k
    for (uint32_t b = lane; b < B; b += 32) {
      K96 y{rk[b], ra[b]};
      if (!lt(y, rej) && (y.a & 1u) == 0) found[y.a >> 1] = 1;
    }
  }
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    uint32_t e = s * 32 + lane;
    if (e < P) {
      pd[prow + e] = pool.d[s];
      pid[prow + e] = pool.id[s];
    }
  }
  if (lane == 0) {
    Lc[t] = L;
    radius[t] = rad;
  }
  }
}

// =============================================================================================
// Update.
// =============================================================================================

// radius = pool[L].dist (the overflow slot); Range grows by up to S new entries for found nodes;
// radiusM = pool[Range-1].dist.  (update(), base_index.hpp:374-395)
__global__ void update_range_kernel(uint64_t n, uint32_t P, uint32_t S, const float* __restrict__ pd,
                                    const uint32_t* __restrict__ pid, const uint32_t* __restrict__ Lc,
                                    uint32_t* __restrict__ Range, float* __restrict__ radius,
                                    float* __restrict__ radiusM, const uint8_t* __restrict__ found) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint64_t row = t * P;
  radius[t] = pd[row + P - 1];
  uint32_t R = Range[t];
  if (found[t]) {
    uint32_t L = Lc[t];
    uint32_t maxl = R + S < L ? R + S : L;
    uint32_t c = 0, l = 0;
    while (l < maxl && c < S) {
      if (pid[row + l] & FLAG) ++c;
      ++l;
    }
    R = l;
    Range[t] = R;
  }
  radiusM[t] = pd[row + R - 1];
}

// Forward lists of node t (pool order) and reverse-edge counts per target.
// PASS 0: counts; PASS 1: writes reverse edges and clears the new flags.
template <int PASS>
__global__ void update_lists_kernel(uint64_t n, uint32_t P, uint32_t cap, const float* __restrict__ pd,
                                    uint32_t* __restrict__ pid, const uint32_t* __restrict__ Range,
                                    const float* __restrict__ radiusM, uint32_t* __restrict__ new_ids,
                                    uint32_t* __restrict__ new_cnt, uint32_t* __restrict__ old_ids,
                                    uint32_t* __restrict__ old_cnt, uint32_t* __restrict__ rcnt,
                                    const uint32_t* __restrict__ roff, uint32_t* __restrict__ rcur,
                                    uint32_t* __restrict__ rbuf) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  uint64_t row = t * P;
  uint32_t R = Range[t];
  uint32_t cn = 0, co = 0;
  for (uint32_t l = 0; l < R; ++l) {
    uint32_t v = pid[row + l];
    uint32_t id = v & IDM;
    float d = pd[row + l];
    bool rev = d > radiusM[id];
    if (v & FLAG) {
      if (PASS == 0) {
        new_ids[t * cap + cn] = id;
        if (rev) atomicAdd(&rcnt[id], 1u);
      } else {
        if (rev) rbuf[roff[id] + atomicAdd(&rcur[id], 1u)] = (uint32_t)t;
        pid[row + l] = id;  // flag cleared
      }
      ++cn;
    } else {
      if (PASS == 0) {
        old_ids[t * cap + co] = id;
        if (rev) atomicAdd(&rcnt[n + id], 1u);
      } else {
        if (rev) rbuf[roff[n + id] + atomicAdd(&rcur[n + id], 1u)] = (uint32_t)t;
      }
      ++co;
    }
  }
  if (PASS == 0) {
    new_cnt[t] = cn;
    old_cnt[t] = co;
  }
}

// One warp per (target, list): the reverse sources, sorted by id, or -- when more than `rcap` --
// the rcap sources with the smallest (hash, id), in that order; appended to the list.
__global__ void update_reverse_kernel(uint64_t n, uint32_t cap, uint32_t rcap, uint64_t seed, uint32_t iter,
                                      const uint32_t* __restrict__ rcnt, const uint32_t* __restrict__ roff,
                                      const uint32_t* __restrict__ rbuf, uint32_t* __restrict__ new_ids,
                                      uint32_t* __restrict__ new_cnt, uint32_t* __restrict__ old_ids,
                                      uint32_t* __restrict__ old_cnt) {
  uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t lane = threadIdx.x & 31;
  if (w >= 2 * n) return;
  uint64_t t = w % n;
  bool is_old = w >= n;
  uint32_t B = rcnt[w];
  if (B == 0) return;
  const uint32_t* src = rbuf + roff[w];
  uint32_t* ids = (is_old ? old_ids : new_ids) + t * cap;
  uint32_t* cntp = (is_old ? old_cnt : new_cnt) + t;
  uint32_t c0 = *cntp;
  bool sample = rcap && B > rcap;
  uint32_t take = sample ? rcap : B;
  uint64_t tag = is_old ? TAG_ROLD : TAG_RNEW;
  uint64_t last = 0;
  bool first = true;
  uint32_t done = 0;
  while (done < take) {
    uint64_t run = ~0ULL;
    for (uint32_t b = 0; b < B; b += 32) {
      uint64_t x = ~0ULL;
      if (b + lane < B) {
        uint32_t sv = src[b + lane];
        uint64_t k = sample ? (((hash4(seed, tag, iter, t, sv) >> 32) << 32) | sv) : (uint64_t)sv;
        if (first || k > last) x = k;
      }
      if (__all_sync(0xffffffffu, x == ~0ULL)) continue;
      x = warp_sort32(x);
      run = warp_merge_min32(run, x);
    }
    first = false;
    // a source listed twice (a pool holding an id twice) leaves fewer distinct keys than take:
    // the list ends at the last one
    uint32_t got = min(32u, take - done);
    got = min(got, (uint32_t)__popc(__ballot_sync(0xffffffffu, run != ~0ULL)));
    if (lane < got) ids[c0 + done + lane] = (uint32_t)run;
    if (got == 0) break;
    last = __shfl_sync(0xffffffffu, run, got - 1);
    done += got;
  }
  if (lane == 0) *cntp = c0 + done;
}

__global__ void export_graph_kernel(uint64_t n, uint32_t P, uint32_t K, const uint32_t* __restrict__ pid,
                                    uint32_t* __restrict__ gids, uint64_t* __restrict__ gptr) {
  uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n * K) gids[g] = pid[(g / K) * P + (g % K)] & IDM;
  if (g <= n) gptr[g] = g * K;
}

// =============================================================================================
// Host drivers.
// =============================================================================================

static unsigned blocks_for(uint64_t threads, int per_block) {
  return (unsigned)((threads + per_block - 1) / per_block);
}

__global__ void widen_kernel(const uint32_t* __restrict__ in, uint64_t* __restrict__ out, uint64_t n) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i];
}

static int merge_level_check(efg_index* idx, int32_t* min_level) {
  Forest& F = idx->forest;
  TreeView tv{F.nodes.p, F.n_left.p, F.n_right.p, F.n_level.p, F.n_tree.p, F.n_start.p, F.n_end.p, F.leaves.p, F.n};
  LocalBuf<int32_t> d;
  EFG_TRY(d.reserve(1));
  int32_t big = 0x7fffffff;
  EFG_CUDA(cudaMemcpyAsync(d.p, &big, 4, cudaMemcpyHostToDevice, idx->stream));
  min_leaf_level_kernel<<<blocks_for(F.nnodes, 256), 256, 0, idx->stream>>>(tv, F.nnodes, idx->bp.trees_build, d.p);
  EFG_CUDA(cudaGetLastError());
  EFG_CUDA(cudaMemcpyAsync(min_level, d.p, 4, cudaMemcpyDeviceToHost, idx->stream));
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  d.release();
  return EFG_OK;
}

static int nnd_init_device(efg_index* idx, NNDev& S) {
  Forest& F = idx->forest;
  cudaStream_t s = idx->stream;
  const efg_build_params& bp = idx->bp;
  if (F.ntrees < bp.trees_build) return fail(EFG_ERR_STATE, "fewer trees than trees_build");
  int32_t minlev = 0;
  EFG_TRY(merge_level_check(idx, &minlev));
  idx->bstats.max_merge_depth = -1;
  if (minlev < (int32_t)bp.merge_level) {
    idx->bstats.max_merge_depth = minlev - 1;
    return fail(EFG_ERR_MERGE_LEVEL,
                "merge level deeper than tree, max merge deepth is" + std::to_string(minlev - 1));
  }
  uint64_t n = idx->n;
  uint32_t ld4 = idx->ld / 4;
  uint32_t cap = std::max(bp.L, 2 * bp.S) + bp.reverse_cap;
  EFG_TRY(nn_alloc(S, n, bp.L, cap));
  TreeView tv{F.nodes.p, F.n_left.p, F.n_right.p, F.n_level.p, F.n_tree.p, F.n_start.p, F.n_end.p, F.leaves.p, F.n};
  // task offsets over nodes
  EFG_TRY(S.pair_off.reserve(F.nnodes + 1));
  EFG_TRY(S.rec_off64.reserve(F.nnodes + 1));
  EFG_TRY(S.scan64.reserve(scan_tmp_elems<uint64_t>(std::max<uint64_t>(F.nnodes, n)) + 1));
  merge_task_len_kernel<<<blocks_for(F.nnodes, 256), 256, 0, s>>>(tv, F.nnodes, bp.trees_build,
                                                                   (int32_t)bp.merge_level, S.pair_off.p);
  EFG_CUDA(cudaGetLastError());
  EFG_TRY(device_scan<uint64_t>(S.pair_off.p, F.nnodes, S.rec_off64.p, S.scan64.p, s));
  uint64_t ntasks = 0;
  EFG_CUDA(cudaMemcpyAsync(&ntasks, S.rec_off64.p + F.nnodes, 8, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  // per-target record counts -> offsets
  EFG_TRY(S.cnt.reserve(n));
  EFG_TRY(S.cursor.reserve(n));
  LocalBuf<uint64_t> cnt64, off64;
  EFG_TRY(cnt64.reserve(n));
  EFG_TRY(off64.reserve(n + 1));
  LocalBuf<unsigned long long> nd;
  EFG_TRY(nd.reserve(1));
  EFG_CUDA(cudaMemsetAsync(S.cnt.p, 0, n * 4, s));
  EFG_CUDA(cudaMemsetAsync(S.cursor.p, 0, n * 4, s));
  EFG_CUDA(cudaMemsetAsync(nd.p, 0, 8, s));
  unsigned rgrid = (unsigned)std::min<uint64_t>(blocks_for(ntasks * 32, 256), 152ull * 64);
  // what pass 0 keeps for the record pass: the point, the leaf and maxl distances per task (when
  // that stays within 4 GiB; otherwise pass 1 routes again)
  uint32_t maxl = 0;
  {
    LocalBuf<uint32_t> ml;
    EFG_TRY(ml.reserve(1));
    EFG_CUDA(cudaMemsetAsync(ml.p, 0, 4, s));
    max_leaf_kernel<<<blocks_for(F.nnodes, 256), 256, 0, s>>>(tv, F.nnodes, ml.p);
    EFG_CUDA(cudaMemcpyAsync(&maxl, ml.p, 4, cudaMemcpyDeviceToHost, s));
    EFG_CUDA(cudaStreamSynchronize(s));
  }
  const bool keep = ntasks && maxl && ntasks * (uint64_t)(maxl + 2) * 4 <= (4ull << 30);
  LocalBuf<uint32_t> task_p;
  LocalBuf<int32_t> task_leaf;
  LocalBuf<float> task_d;
  if (keep) {
    EFG_TRY(task_p.reserve(ntasks));
    EFG_TRY(task_leaf.reserve(ntasks));
    EFG_TRY(task_d.reserve(ntasks * maxl));
  }
  if (ntasks) {
    merge_route_kernel<0><<<rgrid, 256, 0, s>>>(idx->d_base, ld4, tv, S.rec_off64.p, F.nnodes, ntasks, S.cnt.p,
                                                 nullptr, nullptr, nullptr, nd.p, task_p.p, task_leaf.p, task_d.p,
                                                 maxl);
    EFG_CUDA(cudaGetLastError());
  }
  widen_kernel<<<blocks_for(n, 256), 256, 0, s>>>(S.cnt.p, cnt64.p, n);
  EFG_CUDA(cudaGetLastError());
  EFG_TRY(device_scan<uint64_t>(cnt64.p, n, off64.p, S.scan64.p, s));
  uint64_t nrec = 0;
  unsigned long long ndist = 0;
  EFG_CUDA(cudaMemcpyAsync(&nrec, off64.p + n, 8, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaMemcpyAsync(&ndist, nd.p, 8, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  idx->bstats.merge_distances = ndist;
  EFG_TRY(S.rec_key.reserve(nrec + 1));
  if (keep) {
    merge_emit_kernel<<<(unsigned)std::min<uint64_t>(blocks_for(ntasks, 256), 152ull * 64), 256, 0, s>>>(
        tv, ntasks, task_p.p, task_leaf.p, task_d.p, maxl, off64.p, S.cursor.p, S.rec_key.p);
    EFG_CUDA(cudaGetLastError());
  } else if (ntasks) {
    merge_route_kernel<1><<<rgrid, 256, 0, s>>>(idx->d_base, ld4, tv, S.rec_off64.p, F.nnodes, ntasks, nullptr,
                                                off64.p, S.cursor.p, S.rec_key.p, nullptr, nullptr, nullptr, nullptr,
                                                0);
    EFG_CUDA(cudaGetLastError());
  }
  init_select_kernel<<<blocks_for(n * 32, 256), 256, 0, s>>>(
      idx->d_base, ld4, n, bp.S, S.P, cap, bp.seed, S.cnt.p, off64.p, S.rec_key.p, S.pd.p, S.pid.p, S.Lc.p,
      S.Range.p, S.radius.p, S.radiusM.p, S.found.p, S.new_ids.p, S.new_cnt.p, S.old_cnt.p);
  EFG_CUDA(cudaGetLastError());
  EFG_CUDA(cudaStreamSynchronize(s));
  cnt64.release();
  off64.release();
  nd.release();
  return EFG_OK;
}

static int nnd_iterate_device(efg_index* idx, NNDev& S, uint32_t iter, uint64_t* pairs_out, uint64_t* recs_out) {
  cudaStream_t s = idx->stream;
  const efg_build_params& bp = idx->bp;
  uint64_t n = S.n;
  uint32_t ld4 = idx->ld / 4;
  // ---- join
  EFG_TRY(S.pair_off.reserve(n + 1));
  EFG_TRY(S.rec_off64.reserve(n + 1));
  EFG_TRY(S.scan64.reserve(scan_tmp_elems<uint64_t>(2 * n) + 1));
  LocalBuf<uint64_t> tmp64;
  EFG_TRY(tmp64.reserve(2 * n + 1));
  pair_count_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, S.new_cnt.p, S.old_cnt.p, tmp64.p);
  EFG_CUDA(cudaGetLastError());
  EFG_TRY(device_scan<uint64_t>(tmp64.p, n, S.pair_off.p, S.scan64.p, s));
  uint64_t npairs = 0;
  EFG_CUDA(cudaMemcpyAsync(&npairs, S.pair_off.p + n, 8, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  EFG_TRY(S.pairdist.reserve(npairs + 1));
  EFG_TRY(S.cnt.reserve(2 * n));
  EFG_TRY(S.cursor.reserve(2 * n));
  LocalBuf<float> bound;
  EFG_TRY(bound.reserve(n));
  bound_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, S.P, S.pd.p, S.Lc.p, S.radius.p, bound.p);
  EFG_CUDA(cudaMemsetAsync(S.cnt.p, 0, n * 4, s));
  EFG_CUDA(cudaMemsetAsync(S.cursor.p, 0, n * 4, s));
  EFG_CUDA(cudaMemsetAsync(S.found.p, 0, n, s));
  LocalBuf<uint32_t> jctr;  // node counters of the two join passes, the merge, the tensor-core join's three
  EFG_TRY(jctr.reserve(6));
  EFG_CUDA(cudaMemsetAsync(jctr.p, 0, 24, s));
  int sms = 152, per0 = 1, per1 = 1, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, join_dist_kernel, 256, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, join_records_kernel, 256, 0);
  const unsigned jgrid0 = (unsigned)std::min<uint64_t>(blocks_for(n * 32, 256), (uint64_t)sms * std::max(per0, 1));
  const unsigned jgrid1 = (unsigned)std::min<uint64_t>(blocks_for(n * 32, 256), (uint64_t)sms * std::max(per1, 1));
  const bool tc = idx->build_precision == EFG_PRECISION_BF16;
  if (tc) {
    // pass 0 on the tensor cores: nodes that fit one tile packed together, then the larger ones
    if (!S.jterms) {
      const uint64_t W = (idx->dim + 63) / 64 * 64;
      EFG_TRY(S.jhi.reserve(n * W));
      EFG_TRY(S.jlo.reserve(n * W));
      EFG_TRY(S.jnorm.reserve(n));
      EFG_TRY(S.jflag.reserve(2));
      EFG_TRY(S.jmid.reserve(n + 1));
      EFG_TRY(S.jbig.reserve(n + 1));
      EFG_TRY(tc_join_prepare(idx->d_base, n, idx->dim, idx->ld, S.jhi.p, S.jlo.p, S.jnorm.p, S.jflag.p, s));
      int inexact = 0;
      EFG_CUDA(cudaMemcpyAsync(&inexact, S.jflag.p, 4, cudaMemcpyDeviceToHost, s));
      EFG_CUDA(cudaStreamSynchronize(s));
      S.jterms = inexact ? 3 : 1;
    }
    EFG_CUDA(cudaMemsetAsync(S.jflag.p + 1, 0, 4, s));
    EFG_CUDA(cudaMemsetAsync(S.jmid.p, 0, 4, s));
    EFG_CUDA(cudaMemsetAsync(S.jbig.p, 0, 4, s));
    EFG_TRY(tc_join(S.jhi.p, S.jlo.p, S.jnorm.p, n, idx->dim, S.jterms, S.cap, S.P, bp.check_k, S.new_ids.p,
                    S.new_cnt.p, S.old_ids.p, S.old_cnt.p, S.pair_off.p, bound.p, S.pairdist.p, S.cnt.p, S.found.p,
                    jctr.p + 3, S.jmid.p, S.jbig.p, S.jflag.p + 1, s));
  } else {
    join_dist_kernel<<<jgrid0, 256, 0, s>>>(idx->d_base, ld4, n, S.cap, S.P, bp.check_k, S.new_ids.p, S.new_cnt.p,
                                            S.old_ids.p, S.old_cnt.p, S.pair_off.p, bound.p, S.pairdist.p, S.cnt.p,
                                            S.found.p, jctr.p);
    EFG_CUDA(cudaGetLastError());
  }
  widen_kernel<<<blocks_for(n, 256), 256, 0, s>>>(S.cnt.p, tmp64.p, n);
  EFG_TRY(device_scan<uint64_t>(tmp64.p, n, S.rec_off64.p, S.scan64.p, s));
  uint64_t nrec = 0;
  EFG_CUDA(cudaMemcpyAsync(&nrec, S.rec_off64.p + n, 8, cudaMemcpyDeviceToHost, s));
  int jstat[2] = {0, 0};  // tensor-core join: error word, nodes larger than one tile
  if (tc) {
    EFG_CUDA(cudaMemcpyAsync(&jstat[0], S.jflag.p + 1, 4, cudaMemcpyDeviceToHost, s));
    EFG_CUDA(cudaMemcpyAsync(&jstat[1], S.jbig.p, 4, cudaMemcpyDeviceToHost, s));
  }
  EFG_CUDA(cudaStreamSynchronize(s));
  if (jstat[0] & 4) return fail(EFG_ERR_ARG, "tensor-core join: a join list holds an id >= n");
  if (jstat[0]) return fail(EFG_ERR_DEVICE_LIMIT, "tensor-core join: a wait ran out on the device");
  idx->bstats.join_large_nodes += (uint32_t)jstat[1];
  EFG_TRY(S.rec_key.reserve(nrec + 1));
  EFG_TRY(S.rec_aux.reserve(nrec + 1));
  join_records_kernel<<<jgrid1, 256, 0, s>>>(n, S.cap, S.P, bp.check_k, S.new_ids.p, S.new_cnt.p, S.old_ids.p,
                                             S.old_cnt.p, S.pair_off.p, bound.p, S.pairdist.p, S.rec_off64.p,
                                             S.cursor.p, S.rec_key.p, S.rec_aux.p, jctr.p + 1);
  EFG_CUDA(cudaGetLastError());
  // merge: a warp per target node; records of up to msort per node sorted in shared memory
  const uint32_t msort = S.P > 64 ? 1024 : 256;
  const size_t msmem = (size_t)MERGE_WARPS * msort * 12;
  auto launch_merge = [&](auto kern) -> int {
    EFG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msmem));
    int per = 1;
    EFG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, MERGE_WARPS * 32, msmem));
    const unsigned grid = (unsigned)std::min<uint64_t>(blocks_for(n * 32, MERGE_WARPS * 32),
                                                       (uint64_t)sms * std::max(per, 1));
    kern<<<grid, MERGE_WARPS * 32, msmem, s>>>(n, S.P, bp.check_k, tc, msort, S.cnt.p, S.rec_off64.p, S.rec_key.p,
                                               S.rec_aux.p, S.pd.p, S.pid.p, S.Lc.p, S.radius.p, S.found.p, jctr.p + 2);
    return EFG_OK;
  };
  if (S.P <= 32) EFG_TRY(launch_merge(merge_kernel<1>));
  else if (S.P <= 64) EFG_TRY(launch_merge(merge_kernel<2>));
  else if (S.P <= 128) EFG_TRY(launch_merge(merge_kernel<4>));
  else EFG_TRY(launch_merge(merge_kernel<8>));
  EFG_CUDA(cudaGetLastError());
  // ---- update
  update_range_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, S.P, bp.S, S.pd.p, S.pid.p, S.Lc.p, S.Range.p,
                                                         S.radius.p, S.radiusM.p, S.found.p);
  EFG_CUDA(cudaGetLastError());
  EFG_TRY(S.rcnt.reserve(2 * n));
  EFG_TRY(S.rcur.reserve(2 * n));
  EFG_TRY(S.roff.reserve(2 * n + 1));
  EFG_TRY(S.scan32.reserve(scan_tmp_elems<uint32_t>(2 * n) + 1));
  EFG_CUDA(cudaMemsetAsync(S.rcnt.p, 0, 2 * n * 4, s));
  EFG_CUDA(cudaMemsetAsync(S.rcur.p, 0, 2 * n * 4, s));
  update_lists_kernel<0><<<blocks_for(n, 128), 128, 0, s>>>(n, S.P, S.cap, S.pd.p, S.pid.p, S.Range.p, S.radiusM.p,
                                                            S.new_ids.p, S.new_cnt.p, S.old_ids.p, S.old_cnt.p,
                                                            S.rcnt.p, nullptr, nullptr, nullptr);
  EFG_CUDA(cudaGetLastError());
  EFG_TRY(device_scan<uint32_t>(S.rcnt.p, 2 * n, S.roff.p, S.scan32.p, s));
  uint32_t nrev = 0;
  EFG_CUDA(cudaMemcpyAsync(&nrev, S.roff.p + 2 * n, 4, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  EFG_TRY(S.rbuf.reserve((uint64_t)nrev + 1));
  update_lists_kernel<1><<<blocks_for(n, 128), 128, 0, s>>>(n, S.P, S.cap, S.pd.p, S.pid.p, S.Range.p, S.radiusM.p,
                                                            S.new_ids.p, S.new_cnt.p, S.old_ids.p, S.old_cnt.p,
                                                            S.rcnt.p, S.roff.p, S.rcur.p, S.rbuf.p);
  EFG_CUDA(cudaGetLastError());
  update_reverse_kernel<<<blocks_for(2 * n * 32, 256), 256, 0, s>>>(n, S.cap, bp.reverse_cap, bp.seed, iter, S.rcnt.p,
                                                                    S.roff.p, S.rbuf.p, S.new_ids.p, S.new_cnt.p,
                                                                    S.old_ids.p, S.old_cnt.p);
  EFG_CUDA(cudaGetLastError());
  EFG_CUDA(cudaStreamSynchronize(s));
  bound.release();
  tmp64.release();
  if (pairs_out) *pairs_out = npairs;
  if (recs_out) *recs_out = nrec;
  return EFG_OK;
}

int build_graph_device(efg_index* idx) {
  NvtxRange range("efg: build graph");
  cudaStream_t s = idx->stream;
  idx->bstats = efg_build_stats{};
  idx->graph.release();
  ScopedEvents<4> evs;
  cudaEvent_t* ev = evs.e;
  cudaEventRecord(ev[0], s);
  {
    NvtxRange r("efg: build trees");
    EFG_TRY(build_forest(idx, idx->bp.trees));
  }
  cudaEventRecord(ev[1], s);
  NNDev S;
  int rc;
  {
    NvtxRange r("efg: leaf-merge init");
    rc = nnd_init_device(idx, S);
  }
  if (rc != EFG_OK) {
    S.release_all();
    return rc;
  }
  cudaEventRecord(ev[2], s);
  uint64_t pairs = 0, recs = 0;
  for (uint32_t it = 0; it < idx->bp.epochs; ++it) {
    uint64_t p = 0, r = 0;
    NvtxRange range_it("efg: nn-descent iteration");
    rc = nnd_iterate_device(idx, S, it, &p, &r);
    if (rc != EFG_OK) {
      S.release_all();
      return rc;
    }
    pairs += p;
    recs += r;
  }
  // export gs: first K pool ids of every node (refineGraph, base_index.hpp:469-479)
  uint64_t n = idx->n;
  uint32_t K = idx->bp.K;
  Graph& g = idx->graph;
  EFG_TRY(g.ids.reserve(n * K));
  EFG_TRY(g.ptr.reserve(n + 1));
  export_graph_kernel<<<blocks_for(n * K + 1, 256), 256, 0, s>>>(n, S.P, K, S.pid.p, g.ids.p, g.ptr.p);
  EFG_CUDA(cudaGetLastError());
  cudaEventRecord(ev[3], s);
  EFG_CUDA(cudaStreamSynchronize(s));
  g.n = n;
  g.nnz = n * K;
  g.fixed_k = K;
  g.max_deg = K;
  g.valid = true;
  float a = 0, b = 0, c = 0;
  cudaEventElapsedTime(&a, ev[0], ev[1]);
  cudaEventElapsedTime(&b, ev[1], ev[2]);
  cudaEventElapsedTime(&c, ev[2], ev[3]);
  idx->bstats.trees_ms = a;
  idx->bstats.init_ms = b;
  idx->bstats.refine_ms = c;
  idx->bstats.total_ms = a + b + c;
  idx->bstats.join_pairs = pairs;
  idx->bstats.join_records = recs;
  S.release_all();
  return EFG_OK;
}

// ---- host-state entry points (state-level parity) ----------------------------------------------

static int state_to_device(efg_index* idx, NNDev& S, const efg_nnd_host_state* st) {
  if (st->n != idx->n || st->L != idx->bp.L) return fail(EFG_ERR_ARG, "state does not match the index");
  EFG_TRY(nn_alloc(S, st->n, st->L, st->cap));
  uint64_t n = st->n, np = n * S.P;
  std::vector<uint32_t> pid(np);
  for (uint64_t i = 0; i < np; ++i) pid[i] = st->pool_id[i] | (st->pool_flag[i] ? FLAG : 0u);
  EFG_CUDA(cudaMemcpy(S.pd.p, st->pool_dist, np * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.pid.p, pid.data(), np * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.Lc.p, st->Lcur, n * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.Range.p, st->Range, n * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.radius.p, st->radius, n * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.radiusM.p, st->radiusM, n * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.found.p, st->found, n, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.new_ids.p, st->new_ids, n * st->cap * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.new_cnt.p, st->new_cnt, n * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.old_ids.p, st->old_ids, n * st->cap * 4, cudaMemcpyHostToDevice));
  EFG_CUDA(cudaMemcpy(S.old_cnt.p, st->old_cnt, n * 4, cudaMemcpyHostToDevice));
  return EFG_OK;
}

static int state_to_host(NNDev& S, efg_nnd_host_state* st) {
  uint64_t n = S.n, np = n * S.P;
  std::vector<uint32_t> pid(np);
  EFG_CUDA(cudaMemcpy(st->pool_dist, S.pd.p, np * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(pid.data(), S.pid.p, np * 4, cudaMemcpyDeviceToHost));
  for (uint64_t i = 0; i < np; ++i) {
    st->pool_id[i] = pid[i] & IDM;
    st->pool_flag[i] = (pid[i] & FLAG) ? 1 : 0;
  }
  EFG_CUDA(cudaMemcpy(st->Lcur, S.Lc.p, n * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->Range, S.Range.p, n * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->radius, S.radius.p, n * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->radiusM, S.radiusM.p, n * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->found, S.found.p, n, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->new_ids, S.new_ids.p, n * S.cap * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->new_cnt, S.new_cnt.p, n * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->old_ids, S.old_ids.p, n * S.cap * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(st->old_cnt, S.old_cnt.p, n * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

int nnd_init_host(efg_index* idx, efg_nnd_host_state* st) {
  if (idx->forest.ntrees == 0) return fail(EFG_ERR_STATE, "no trees");
  if (st->n != idx->n || st->L != idx->bp.L) return fail(EFG_ERR_ARG, "state does not match the index");
  uint32_t need = std::max(idx->bp.L, 2 * idx->bp.S) + idx->bp.reverse_cap;
  if (st->cap != need) return fail(EFG_ERR_ARG, "state list capacity must be " + std::to_string(need));
  NNDev S;
  int rc = nnd_init_device(idx, S);
  if (rc == EFG_OK) rc = state_to_host(S, st);
  S.release_all();
  return rc;
}

int nnd_iterate_host(efg_index* idx, efg_nnd_host_state* st, uint32_t iter, uint64_t* pairs) {
  uint32_t need = std::max(idx->bp.L, 2 * idx->bp.S) + idx->bp.reverse_cap;
  if (st->cap < need) return fail(EFG_ERR_ARG, "state list capacity too small");
  NNDev S;
  int rc = state_to_device(idx, S, st);
  uint64_t p = 0, r = 0;
  if (rc == EFG_OK) rc = nnd_iterate_device(idx, S, iter, &p, &r);
  if (rc == EFG_OK) rc = state_to_host(S, st);
  if (pairs) *pairs = p;
  S.release_all();
  return rc;
}

}  // namespace efg
