// Graph search over batched queries: the "nnexp" method of getNeighbors_nnexp
// (algorithm/kdtreeub_index.hpp:363-494).
//
// One CTA (256 threads) answers one query; all per-query state lives in shared memory:
//   * the query vector;
//   * an open-addressing hash set of visited ids (the reference's N-bit `tbflag`, which it
//     allocates and clears per query), whose bit 31 doubles as the "expanded" mark (the
//     reference's `newflag`);
//   * the candidate list as packed (dist_bits << 32 | id) keys, kept sorted by bitonic sorts, which
//     orders exactly like the reference's partial_sort of pair<float, size_t>;
//   * the leaves chosen by the trees.
// Steps per query, as in the reference:
//   1. per tree, a near-first DFS collecting lsize = init_num*2/(5*trees)+1 leaves
//      (getSearchNodeList, :332-346);
//   2. leaves interleaved leaf-rank-major, tree-minor; ids deduplicated in that order until
//      init_num are collected (:396-410); a counter-hash fill if the leaves run short (:411-417);
//   3. distances to the pool, keep the resultSize = max(extend_to, k) best (:420-442);
//   4. `epochs` times: expand every not-yet-expanded id among the first extend_to through its
//      graph row, add the unvisited neighbours, keep the resultSize best (:444-484);
//   5. emit the first k ids (:486-492).
// Ids are unique in the candidate list, so the sorted order (and the output) does not depend on
// the order in which threads discover neighbours.
#include <algorithm>

#include "internal.cuh"

namespace efg {

static constexpr int S_THREADS = 256;
static constexpr int S_WARPS = S_THREADS / 32;
static constexpr int S_CHUNK = 512;      // seeding ids deduplicated per step
static constexpr int S_MAX_STACK = 64;   // DFS stack depth per tree
static constexpr uint32_t ID_MASK = 0x3FFFFFFFu;
static constexpr uint32_t EXPANDED = 0x80000000u;

enum : uint32_t { SERR_STACK = 1u, SERR_HASH = 2u };

struct SearchCfg {
  uint32_t T, lsize, init_num, extend_to, result_size, epochs, k;
  uint32_t ht_bits, keys_cap, nseq;
  uint32_t ht_global;  // visited set in a per-CTA slice of global scratch instead of shared memory
  uint64_t seed;
};

__device__ __forceinline__ uint32_t ht_slot(uint32_t id, uint32_t bits) { return (id * 2654435761u) >> (32 - bits); }

// Inserts id; true if it was not present.  Sets *err on a full table.
__device__ __forceinline__ bool ht_insert(uint32_t* ht, uint32_t bits, uint32_t id, uint32_t* err) {
  uint32_t mask = (1u << bits) - 1, h = ht_slot(id, bits);
  for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
    uint32_t cur = *reinterpret_cast<volatile const uint32_t*>(&ht[h]);
    if (cur == kEmpty) {
      uint32_t prev = atomicCAS(&ht[h], kEmpty, id);
      if (prev == kEmpty) return true;
      cur = prev;
    }
    if ((cur & ID_MASK) == id) return false;
  }
  atomicOr(err, SERR_HASH);
  return false;
}
__device__ __forceinline__ bool ht_contains(const uint32_t* ht, uint32_t bits, uint32_t id) {
  uint32_t mask = (1u << bits) - 1, h = ht_slot(id, bits);
  for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
    uint32_t cur = *reinterpret_cast<volatile const uint32_t*>(&ht[h]);
    if (cur == kEmpty) return false;
    if ((cur & ID_MASK) == id) return true;
  }
  return false;
}
// Marks id expanded; true if this call did it (id must be present).
__device__ __forceinline__ bool ht_mark_expanded(uint32_t* ht, uint32_t bits, uint32_t id) {
  uint32_t mask = (1u << bits) - 1, h = ht_slot(id, bits);
  for (uint32_t probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
    uint32_t cur = *reinterpret_cast<volatile const uint32_t*>(&ht[h]);
    if (cur == kEmpty) return false;
    if ((cur & ID_MASK) == id) return (atomicOr(&ht[h], EXPANDED) & EXPANDED) == 0;
  }
  return false;
}

__device__ void sort_keys_block(uint64_t* keys, uint32_t n) {
  for (uint32_t k = 2; k <= n; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t ixj = i ^ j;
        if (ixj > i) {
          uint64_t a = keys[i], b = keys[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Exclusive scan of one value per thread over the block; returns the thread's prefix and the total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < S_WARPS ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (uint32_t)o) t += y;
    }
    if (lane < S_WARPS) warp_tot[lane] = t;  // inclusive per warp
  }
  __syncthreads();
  uint32_t before = warp == 0 ? 0 : warp_tot[warp - 1];
  *total = warp_tot[S_WARPS - 1];
  __syncthreads();
  return before + x - v;
}

// Distances from the query (shared memory, zero padded to ld4 float4) to keys[lo..hi) whose low
// 32 bits hold ids; rewrites them as packed (dist, id) keys.  Each warp takes 4 rows at a time so
// that 4 independent row loads are in flight per lane.
__device__ __forceinline__ void pool_distances(const float4* __restrict__ qv, uint32_t ld4,
                                               const float* __restrict__ base, uint32_t ld, uint64_t* keys,
                                               uint32_t lo, uint32_t hi) {
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t i = lo + warp * 4; i < hi; i += S_WARPS * 4) {
    uint32_t id[4];
    const float4* row[4];
    float acc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      id[u] = i + u < hi ? (uint32_t)keys[i + u] : (uint32_t)keys[i];
      row[u] = reinterpret_cast<const float4*>(base + (uint64_t)id[u] * ld);
      acc[u] = 0.f;
    }
    for (uint32_t c = lane; c < ld4; c += 32) {
      float4 qc = qv[c];
      float4 x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = __ldg(row[u] + c);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float d0 = x[u].x - qc.x, d1 = x[u].y - qc.y, d2 = x[u].z - qc.z, d3 = x[u].w - qc.w;
        acc[u] += d0 * d0;
        acc[u] += d1 * d1;
        acc[u] += d2 * d2;
        acc[u] += d3 * d3;
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = warp_sum(acc[u]);
    if (lane < 4 && i + lane < hi) {
      float dv = lane == 0 ? acc[0] : lane == 1 ? acc[1] : lane == 2 ? acc[2] : acc[3];
      keys[i + lane] = pack_key(dv, id[lane]);
    }
  }
}

__global__ void __launch_bounds__(S_THREADS) nnexp_kernel(
    const float* __restrict__ base, uint64_t n, uint32_t dim, uint32_t ld, const DNode* __restrict__ nodes,
    const int32_t* __restrict__ roots, const uint32_t* __restrict__ leaves, const uint64_t* __restrict__ gptr,
    const uint32_t* __restrict__ gids, const float* __restrict__ queries, uint64_t nq, uint64_t qld, SearchCfg cfg,
    int32_t* __restrict__ out, unsigned long long* __restrict__ stats, uint32_t* __restrict__ ht_scratch) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t ld4 = ld >> 2;
  float4* qv = reinterpret_cast<float4*>(smem);
  uint64_t* keys = reinterpret_cast<uint64_t*>(qv + ld4);                  // keys_cap
  uint64_t* chunk = keys + cfg.keys_cap;                                    // S_CHUNK
  uint32_t* ht_smem = reinterpret_cast<uint32_t*>(chunk + S_CHUNK);        // 1 << ht_bits (if in smem)
  uint32_t* ht = cfg.ht_global ? ht_scratch + ((uint64_t)blockIdx.x << cfg.ht_bits) : ht_smem;
  uint32_t* lstart = ht_smem + (cfg.ht_global ? 0u : (1u << cfg.ht_bits));  // nseq
  uint32_t* lend = lstart + cfg.nseq;                                       // nseq
  uint32_t* seqoff = lend + cfg.nseq;                                       // nseq + 1
  uint8_t* firstflag = reinterpret_cast<uint8_t*>(seqoff + cfg.nseq + 1);  // S_CHUNK
  __shared__ uint32_t warp_tot[S_WARPS];
  __shared__ uint32_t s_p, s_m, s_err, s_total, s_exp;
  __shared__ uint32_t lcount[256];

  const uint32_t tid = threadIdx.x;
  const uint32_t ht_size = 1u << cfg.ht_bits;
  unsigned long long evals = 0;
  if (threadIdx.x == 0) s_exp = 0;

  for (uint64_t qi = blockIdx.x; qi < nq; qi += gridDim.x) {
    const float* qrow = queries + qi * qld;
    for (uint32_t c = tid; c < ld4; c += S_THREADS) {
      float4 v;
      uint32_t e = 4 * c;
      v.x = e < dim ? qrow[e] : 0.f;
      v.y = e + 1 < dim ? qrow[e + 1] : 0.f;
      v.z = e + 2 < dim ? qrow[e + 2] : 0.f;
      v.w = e + 3 < dim ? qrow[e + 3] : 0.f;
      qv[c] = v;
    }
    for (uint32_t i = tid; i < ht_size; i += S_THREADS) ht[i] = kEmpty;
    if (tid == 0) {
      s_p = 0;
      s_err = 0;
    }
    __syncthreads();

    // 1. near-first DFS per tree
    for (uint32_t t = tid; t < cfg.T; t += S_THREADS) {
      int32_t stack[S_MAX_STACK];
      int sp = 0;
      stack[sp++] = roots[t];
      uint32_t c = 0;
      while (sp > 0 && c < cfg.lsize) {
        int32_t v = stack[--sp];
        DNode nd = nodes[v];
        while (!dn_is_leaf(nd)) {
          int32_t nearc, farc;
          if (reinterpret_cast<const float*>(qv)[nd.div_dim] < nd.div_val) {
            nearc = nd.left;
            farc = nd.right;
          } else {
            nearc = nd.right;
            farc = nd.left;
          }
          if (sp >= S_MAX_STACK) {
            atomicOr(&s_err, SERR_STACK);
            break;
          }
          stack[sp++] = farc;
          nd = nodes[nearc];
        }
        if (!dn_is_leaf(nd)) break;
        uint32_t j = c * cfg.T + t;  // leaf-rank-major, tree-minor
        lstart[j] = (uint32_t)(-(nd.left + 1));
        lend[j] = (uint32_t)nd.right;
        ++c;
      }
      lcount[t] = c;
    }
    __syncthreads();
    // sequence offsets over (leaf rank, tree); missing leaves contribute nothing
    for (uint32_t base_j = 0; base_j < cfg.nseq; base_j += S_THREADS) {
      uint32_t j = base_j + tid;
      uint32_t sz = 0;
      if (j < cfg.nseq) {
        uint32_t t = j % cfg.T, c = j / cfg.T;
        if (c < lcount[t]) sz = lend[j] - lstart[j];
      }
      uint32_t tot;
      uint32_t ex = block_excl_scan(sz, warp_tot, &tot);
      uint32_t carry = base_j == 0 ? 0 : seqoff[base_j];
      if (j < cfg.nseq) seqoff[j] = carry + ex;
      __syncthreads();
      if (tid == 0) seqoff[min(base_j + S_THREADS, cfg.nseq)] = carry + tot;
      __syncthreads();
    }
    const uint32_t total = seqoff[cfg.nseq];

    // 2. deduplicated pool fill in sequence order, S_CHUNK ids per step
    for (uint32_t cb = 0; cb < total; cb += S_CHUNK) {
      if (s_p >= cfg.init_num) break;
      for (uint32_t i = tid; i < S_CHUNK; i += S_THREADS) {
        uint32_t e = cb + i;
        uint64_t v = ~0ULL;
        if (e < total) {
          // last j with seqoff[j] <= e
          uint32_t lo = 0, hi = cfg.nseq;
          while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (seqoff[mid] <= e) lo = mid;
            else hi = mid;
          }
          uint32_t t = lo % cfg.T;
          uint32_t pos = lstart[lo] + (e - seqoff[lo]);
          uint32_t id = leaves[(uint64_t)t * n + pos];
          v = ((uint64_t)id << 32) | i;
        }
        chunk[i] = v;
      }
      __syncthreads();
      sort_keys_block(chunk, S_CHUNK);
      for (uint32_t s = tid; s < S_CHUNK; s += S_THREADS) {
        uint64_t v = chunk[s];
        if (v == ~0ULL) continue;
        uint32_t id = (uint32_t)(v >> 32);
        bool first = (s == 0 || (uint32_t)(chunk[s - 1] >> 32) != id) && !ht_contains(ht, cfg.ht_bits, id);
        firstflag[(uint32_t)v] = first;
      }
      for (uint32_t i = tid; i < S_CHUNK; i += S_THREADS)
        if (cb + i >= total) firstflag[i] = 0;
      __syncthreads();
      // ranks in sequence order (two elements per thread)
      uint32_t i0 = 2 * tid;
      uint32_t f0 = firstflag[i0], f1 = firstflag[i0 + 1];
      uint32_t tot;
      uint32_t ex = block_excl_scan(f0 + f1, warp_tot, &tot);
      uint32_t p0 = s_p;
      uint32_t ids_i[2] = {0, 0};
      // ids of this thread's two elements: recompute from the sequence
      for (int u = 0; u < 2; ++u) {
        uint32_t e = cb + i0 + u;
        if ((u == 0 ? f0 : f1) && e < total) {
          uint32_t lo = 0, hi = cfg.nseq;
          while (hi - lo > 1) {
            uint32_t mid = (lo + hi) >> 1;
            if (seqoff[mid] <= e) lo = mid;
            else hi = mid;
          }
          uint32_t t = lo % cfg.T;
          ids_i[u] = leaves[(uint64_t)t * n + lstart[lo] + (e - seqoff[lo])];
        }
      }
      uint32_t r = p0 + ex;
      if (f0) {
        if (r < cfg.init_num) {
          keys[r] = ids_i[0];
          ht_insert(ht, cfg.ht_bits, ids_i[0], &s_err);
        }
        ++r;
      }
      if (f1 && r < cfg.init_num) {
        keys[r] = ids_i[1];
        ht_insert(ht, cfg.ht_bits, ids_i[1], &s_err);
      }
      __syncthreads();
      if (tid == 0) s_p = min(cfg.init_num, p0 + tot);
      __syncthreads();
    }
    // counter-hash fill when the leaves hold fewer than init_num distinct ids
    if (tid == 0 && s_p < cfg.init_num) {
      CRng g(hash4(cfg.seed, TAG_SFILL, qi, 0, 0));
      uint32_t p = s_p;
      uint64_t guard = 0;
      while (p < cfg.init_num && guard < 64ull * n + 1024) {
        uint32_t id = g.next() % (uint32_t)n;
        ++guard;
        if (ht_insert(ht, cfg.ht_bits, id, &s_err)) keys[p++] = id;
      }
      s_p = p;
    }
    __syncthreads();
    const uint32_t P = s_p;

    // 3. distances to the pool; keep the result_size best
    pool_distances(qv, ld4, base, ld, keys, 0, P);
    evals += P;
    uint32_t p2 = next_pow2(P);
    for (uint32_t i = P + tid; i < p2; i += S_THREADS) keys[i] = ~0ULL;
    __syncthreads();
    sort_keys_block(keys, p2);
    const uint32_t RS = cfg.result_size;

    // 4. expansion epochs
    for (uint32_t ep = 0; ep < cfg.epochs; ++ep) {
      if (tid == 0) s_m = 0;
      __syncthreads();
      for (uint32_t j = tid; j < cfg.extend_to; j += S_THREADS) {
        uint64_t kj = keys[j];
        if (kj == ~0ULL) continue;
        uint32_t id = (uint32_t)kj;
        if (!ht_mark_expanded(ht, cfg.ht_bits, id)) continue;
        atomicAdd(&s_exp, 1u);
        for (uint64_t e = gptr[id], ee = gptr[id + 1]; e < ee; ++e) {
          uint32_t nb = gids[e];
          if (ht_insert(ht, cfg.ht_bits, nb, &s_err)) {
            uint32_t pos = atomicAdd(&s_m, 1u);
            if (RS + pos < cfg.keys_cap) keys[RS + pos] = nb;
            else atomicOr(&s_err, SERR_HASH);
          }
        }
      }
      __syncthreads();
      uint32_t m = min(s_m, cfg.keys_cap - RS);
      pool_distances(qv, ld4, base, ld, keys, RS, RS + m);
      evals += m;
      uint32_t q2 = next_pow2(RS + m);
      for (uint32_t i = RS + m + tid; i < q2; i += S_THREADS) keys[i] = ~0ULL;
      __syncthreads();
      sort_keys_block(keys, q2);
    }

    // 5. output
    for (uint32_t i = tid; i < cfg.k; i += S_THREADS) {
      uint64_t kv = keys[i];
      out[qi * cfg.k + i] = kv == ~0ULL ? -1 : (int32_t)(uint32_t)kv;
    }
    if (tid == 0 && s_err) atomicOr(reinterpret_cast<unsigned int*>(stats + 1), s_err);
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd(stats, evals);
    atomicAdd(stats + 2, (unsigned long long)s_exp);
  }
}

int search_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, uint32_t k, int32_t* d_out,
                  cudaStream_t s, bool count_evals) {
  const SearchParams& sp = idx->sp;
  if (sp.method != 0) return fail(EFG_ERR_ARG, "only search method 0 (nnexp) is implemented");
  if (idx->forest.ntrees == 0) return fail(EFG_ERR_STATE, "no trees: build or load trees before searching");
  if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph: build or load a graph before searching");
  if (sp.search_trees <= 0) return fail(EFG_ERR_ARG, "search trees must be positive");
  if ((uint32_t)sp.search_trees > idx->forest.ntrees) return fail(EFG_ERR_TREE_COUNT, "wrong tree number");
  if (sp.init_num <= 0 || (uint64_t)sp.init_num > idx->n) return fail(EFG_ERR_ARG, "pool size must be in [1, n]");
  if (k == 0 || (int)k > sp.init_num) return fail(EFG_ERR_ARG, "k must be in [1, pool size]");
  if (sp.epochs < 0 || sp.extend_to < 0) return fail(EFG_ERR_ARG, "negative epochs or extend");
  if (nq == 0) return EFG_OK;

  SearchCfg cfg;
  cfg.T = (uint32_t)sp.search_trees;
  cfg.lsize = (uint32_t)sp.init_num * 2 / (5 * cfg.T) + 1;
  cfg.init_num = (uint32_t)sp.init_num;
  cfg.extend_to = (uint32_t)sp.extend_to;
  cfg.result_size = std::max<uint32_t>(cfg.extend_to, k);
  cfg.epochs = (uint32_t)sp.epochs;
  cfg.k = k;
  cfg.seed = idx->bp.seed;
  cfg.nseq = cfg.T * cfg.lsize;
  uint32_t maxdeg = idx->graph.fixed_k;
  if (!maxdeg) {
    std::vector<uint64_t> ptr(idx->graph.n + 1);
    EFG_CUDA(cudaMemcpy(ptr.data(), idx->graph.ptr.p, ptr.size() * 8, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < idx->graph.n; ++i) maxdeg = std::max<uint32_t>(maxdeg, (uint32_t)(ptr[i + 1] - ptr[i]));
  }
  uint64_t grow = (uint64_t)cfg.extend_to * maxdeg;
  uint64_t keys_need = std::max<uint64_t>(cfg.init_num, cfg.result_size + grow);
  cfg.keys_cap = next_pow2((uint32_t)std::min<uint64_t>(keys_need, 1u << 20));
  uint64_t visited = (uint64_t)cfg.init_num + (uint64_t)cfg.epochs * grow;
  uint32_t bits = 10;
  while ((1ull << bits) < visited + visited / 2 + 64 && bits < 24) ++bits;
  cfg.ht_bits = bits;
  size_t smem_rest = (size_t)(idx->ld / 4) * 16 + (size_t)cfg.keys_cap * 8 + S_CHUNK * 8 + (size_t)cfg.nseq * 12 + 4 +
                     S_CHUNK;
  size_t ht_bytes = ((size_t)1 << bits) * 4;
  cfg.ht_global = smem_rest + ht_bytes > 200 * 1024;
  size_t smem = smem_rest + (cfg.ht_global ? 0 : ht_bytes);
  if (smem > 220 * 1024)
    return fail(EFG_ERR_ARG, "search parameters need " + std::to_string(smem) +
                                 " bytes of shared memory per query (pool/extend/degree too large)");
  if (cfg.T > 256) return fail(EFG_ERR_ARG, "at most 256 search trees");
  EFG_CUDA(cudaFuncSetAttribute(nnexp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  EFG_TRY(idx->eval_counter.reserve(3));
  EFG_CUDA(cudaMemsetAsync(idx->eval_counter.p, 0, 24, s));
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nnexp_kernel, S_THREADS, smem);
  uint64_t grid = std::min<uint64_t>(nq, (uint64_t)sms * std::max(1, per_sm) * (cfg.ht_global ? 1 : 4));
  if (cfg.ht_global) EFG_TRY(idx->ht_scratch.reserve(grid << bits));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  const Forest& F = idx->forest;
  nnexp_kernel<<<(unsigned)grid, S_THREADS, smem, s>>>(idx->d_base, idx->n, idx->dim, idx->ld, F.nodes.p, F.d_roots.p,
                                                       F.leaves.p, idx->graph.ptr.p, idx->graph.ids.p, d_q, nq, qld,
                                                       cfg, d_out, idx->eval_counter.p, idx->ht_scratch.p);
  cudaError_t le = cudaGetLastError();
  cudaEventRecord(e1, s);
  if (le != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return fail(EFG_ERR_CUDA, std::string("nnexp launch: ") + cudaGetErrorString(le));
  }
  if (count_evals) {
    unsigned long long h[3];
    EFG_CUDA(cudaMemcpyAsync(h, idx->eval_counter.p, 24, cudaMemcpyDeviceToHost, s));
    EFG_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    idx->sstats.device_ms = ms;
    idx->sstats.distance_evals = h[0];
    idx->sstats.queries = nq;
    idx->sstats.expanded_nodes = h[2];
    if (h[1] & SERR_STACK) return fail(EFG_ERR_DEVICE_LIMIT, "tree deeper than the search stack");
    if (h[1] & SERR_HASH) return fail(EFG_ERR_DEVICE_LIMIT, "visited set overflow");
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return EFG_OK;
}

}  // namespace efg
