// Graph search method 1: getNeighbors_kgraph (algorithm/kdtreeub_index.hpp:496-654).
//
// Stage 1 (the nnexp kernel in pool mode): tree descent and pool fill exactly as for method 0
// (:505-548), then the distances of the pool's init_num ids, written per query in pool order.
// Stage 2 (only when epochs * extend_to < init_num): each query's pool sorted by (dist, id); its
// first epochs * extend_to keys are the reference's partial_sort (:567-570).  Otherwise the pool
// holds exactly epochs * extend_to ids and stays in pool order, as in the reference.
// Stage 3 (kgraph_kernel, one warp per query): per epoch, the segment [iter*E, (iter+1)*E) of the
// pool minus the ids already visited forms a list sorted by (dist, id) (:574-589); the best
// entry not yet expanded is expanded, again and again: its first min(E, degree) neighbours not yet
// visited are scored and merged into the list, which keeps at most k + E entries (:591-631 -- the
// reference's k/nk loop expands the list's first unexpanded entry each time, which is what the
// scan below does); when every entry is expanded, the list's first k entries are merged into the
// running top k (:632-646).
//
// Equal distances are ordered by id (the reference orders them by arrival).  The visited set is
// the reference's N-bit `flags`: one bitset per warp in global memory, cleared per query.
#include <algorithm>

#include "search.cuh"

namespace efg {
namespace {

constexpr uint64_t KEXP = 1ull << 31;     // "expanded" mark inside a list key (ids are < 2^30)
constexpr uint32_t KID_MASK = 0x3FFFFFFFu;
constexpr uint32_t KG_WARPS = 4;          // queries (warps) per CTA
constexpr uint32_t FULL = 0xffffffffu;

struct KgCfg {
  uint32_t epochs, E, k, C;  // C = k + E: list capacity (knn.size() - 1 in the reference)
  uint32_t list_slots;       // max(C + 1, next_pow2(E)): the list, and the initial sort's padding
  uint32_t key_stride;       // pool keys per query from stage 1
  uint32_t fixed_k;          // graph row length when every row has it (row start = id * fixed_k)
  uint32_t ld4, words;       // float4 per base row; bitset words per warp (multiple of 4)
  uint32_t warp_bytes;       // shared memory per warp
  uint32_t o_list, o_res, o_res2;
  uint32_t full_rows;        // 1: an expansion visits the whole graph row, else its first E ids
};

__device__ __forceinline__ uint64_t kmask(uint64_t x) { return x & ~KEXP; }

// Number of entries of a[0..n) (ascending by masked key) below key.
__device__ __forceinline__ uint32_t lower_bound_keys(const uint64_t* a, uint32_t n, uint64_t key) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (kmask(a[mid]) < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Ascending bitonic sort of n (power of two) keys in shared memory by one warp.
__device__ void warp_sort_keys(uint64_t* a, uint32_t n, uint32_t lane) {
  for (uint32_t k = 2; k <= n; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = lane; i < (n >> 1); i += 32) {
        uint32_t lo = ((i & ~(j - 1)) << 1) | (i & (j - 1));
        uint32_t hi = lo | j;
        uint64_t x = a[lo], y = a[hi];
        if ((x > y) == ((lo & k) == 0)) {
          a[lo] = y;
          a[hi] = x;
        }
      }
      __syncwarp();
    }
}

// Bitonic sort of one key per lane, ascending with the lane index.
__device__ __forceinline__ uint64_t warp_sort32(uint64_t v, uint32_t lane) {
#pragma unroll
  for (uint32_t k = 2; k <= 32; k <<= 1)
#pragma unroll
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      uint64_t o = __shfl_xor_sync(FULL, v, j);
      bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      v = keep_min ? (o < v ? o : v) : (o > v ? o : v);
    }
  return v;
}

// Sums v[0..4) over the warp's 32 lanes; lane l returns the total of v[(l >> 3) & 3].
__device__ __forceinline__ float reduce4_rows(const float* v, uint32_t lane) {
  const bool b4 = (lane >> 4) & 1, b3 = (lane >> 3) & 1;
  float h[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float keep = b4 ? v[j + 2] : v[j], send = b4 ? v[j] : v[j + 2];
    h[j] = keep + __shfl_xor_sync(FULL, send, 16);
  }
  float keep = b3 ? h[1] : h[0], send = b3 ? h[0] : h[1];
  float x = keep + __shfl_xor_sync(FULL, send, 8);
  x += __shfl_xor_sync(FULL, x, 4);
  x += __shfl_xor_sync(FULL, x, 2);
  x += __shfl_xor_sync(FULL, x, 1);
  return x;
}

// U rows (8 or 4) of the query's distances: rows u0 .. u0+U-1 of the lanes' ids (the last one
// repeated past cnt); lane u0 + u receives row u's distance in `mine`.
template <int U>
__device__ __forceinline__ void row_dists_pass(const float4* qv, uint32_t ld4, const float* __restrict__ base,
                                               uint32_t ld, uint32_t id, uint32_t cnt, uint32_t u0, uint32_t lane,
                                               float& mine) {
  uint32_t rid[U];
  float acc[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    rid[u] = __shfl_sync(FULL, id, u0 + u < cnt ? u0 + u : u0);
    acc[u] = 0.f;
  }
  for (uint32_t c = lane; c < ld4; c += 32) {
    float4 qc = qv[c];
    float4 x[U];
#pragma unroll
    for (int u = 0; u < U; ++u) x[u] = __ldg(reinterpret_cast<const float4*>(base + (uint64_t)rid[u] * ld) + c);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float d0 = x[u].x - qc.x, d1 = x[u].y - qc.y, d2 = x[u].z - qc.z, d3 = x[u].w - qc.w;
      acc[u] += d0 * d0;
      acc[u] += d1 * d1;
      acc[u] += d2 * d2;
      acc[u] += d3 * d3;
    }
  }
  // the U sums reduced together (U = 8: lanes 4r .. 4r+3 end with row r's; U = 4: lanes 8r .. 8r+7),
  // then row u's sum moves to lane u0 + u
  if (U == 8) {
    const float tot = reduce8_rows(acc, lane);
    const float t = __shfl_sync(FULL, tot, ((lane - u0) & 7) * 4);
    if (lane - u0 < 8u) mine = t;
  } else {
    const float tot = reduce4_rows(acc, lane);
    const float t = __shfl_sync(FULL, tot, ((lane - u0) & 3) * 8);
    if (lane - u0 < 4u) mine = t;
  }
}

// Squared distances from the query (shared memory, ld4 float4, zero padded) to the rows named by
// lanes 0..cnt-1 (`id`); lane u returns row u's distance.  Eight rows are in flight per pass, four
// in a last pass of at most four rows (most expansions bring fewer than five new neighbours).
__device__ __forceinline__ float warp_row_dists(const float4* qv, uint32_t ld4, const float* __restrict__ base, uint32_t ld,
                                uint32_t id, uint32_t cnt, uint32_t lane) {
  float mine = 0.f;
  for (uint32_t u0 = 0; u0 < cnt; u0 += 8) {
    if (cnt - u0 <= 4) row_dists_pass<4>(qv, ld4, base, ld, id, cnt, u0, lane, mine);
    else row_dists_pass<8>(qv, ld4, base, ld, id, cnt, u0, lane, mine);
  }
  return mine;
}

__global__ void __launch_bounds__(KG_WARPS * 32, 6) kgraph_kernel(
    const float* __restrict__ base, uint32_t dim, uint32_t ld, const uint64_t* __restrict__ gptr,
    const uint32_t* __restrict__ gids, const float* __restrict__ queries, uint64_t nq, uint64_t qld,
    const uint64_t* __restrict__ keys, KgCfg c, int32_t* __restrict__ out, uint32_t* __restrict__ bits,
    unsigned long long* __restrict__ stats, uint32_t* __restrict__ next_query) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* ws = smem + (size_t)wib * c.warp_bytes;
  float4* qv = reinterpret_cast<float4*>(ws);
  uint64_t* list = reinterpret_cast<uint64_t*>(ws + c.o_list);
  uint64_t* res = reinterpret_cast<uint64_t*>(ws + c.o_res);
  uint64_t* res2 = reinterpret_cast<uint64_t*>(ws + c.o_res2);
  const uint64_t gw = (uint64_t)blockIdx.x * KG_WARPS + wib;
  uint32_t* vis = bits + gw * c.words;
  unsigned long long evals = 0, expanded = 0;

  // queries taken from a shared counter as warps come free (their expansion counts differ)
  for (;;) {
    uint32_t qq = 0;
    if (lane == 0) qq = atomicAdd(next_query, 1u);
    const uint64_t q = __shfl_sync(FULL, qq, 0);
    if (q >= nq) break;
    const float* qrow = queries + q * qld;
    for (uint32_t i = lane; i < c.ld4; i += 32) {
      uint32_t e = 4 * i;
      float4 v;
      v.x = e < dim ? qrow[e] : 0.f;
      v.y = e + 1 < dim ? qrow[e + 1] : 0.f;
      v.z = e + 2 < dim ? qrow[e + 2] : 0.f;
      v.w = e + 3 < dim ? qrow[e + 3] : 0.f;
      qv[i] = v;
    }
    uint4* v4 = reinterpret_cast<uint4*>(vis);
    for (uint32_t i = lane; i < c.words / 4; i += 32) v4[i] = make_uint4(0, 0, 0, 0);
    __syncwarp();
    const uint64_t* seg = keys + q * c.key_stride;
    uint32_t rc = 0;
    for (uint32_t iter = 0; iter < c.epochs; ++iter) {
      // the epoch's segment of the pool, minus visited ids, sorted
      uint32_t L = 0;
      for (uint32_t j0 = 0; j0 < c.E; j0 += 32) {
        uint32_t j = j0 + lane;
        bool fresh = false;
        uint64_t key = 0;
        if (j < c.E) {
          key = seg[(uint64_t)iter * c.E + j];
          uint32_t id = (uint32_t)key & KID_MASK;
          uint32_t bit = 1u << (id & 31);
          fresh = !(atomicOr(&vis[id >> 5], bit) & bit);
        }
        uint32_t m = __ballot_sync(FULL, fresh);
        if (fresh) list[L + __popc(m & ((1u << lane) - 1))] = key;
        L += __popc(m);
      }
      uint32_t p2 = next_pow2(L < 2 ? 2 : L);
      for (uint32_t i = L + lane; i < p2; i += 32) list[i] = ~0ULL;
      __syncwarp();
      warp_sort_keys(list, p2, lane);
      // expand the first unexpanded entry until there is none
      uint32_t kpos = 0;
      while (true) {
        uint32_t p = L;
        for (uint32_t b = kpos; b < L; b += 32) {
          uint32_t i = b + lane;
          bool un = i < L && !(list[i] & KEXP);
          uint32_t m = __ballot_sync(FULL, un);
          if (m) {
            p = b + __ffs(m) - 1;
            break;
          }
        }
        if (p >= L) break;
        uint64_t pk = list[p];
        __syncwarp();
        if (lane == 0) list[p] = pk | KEXP;
        __syncwarp();
        ++expanded;
        uint32_t node = (uint32_t)pk & KID_MASK;
        uint64_t row;
        uint32_t deg;
        if (c.fixed_k) {
          row = (uint64_t)node * c.fixed_k;
          deg = c.fixed_k;
        } else {
          row = gptr[node];
          deg = (uint32_t)(gptr[node + 1] - row);
        }
        uint32_t maxM = c.full_rows ? deg : min(c.E, deg);
        uint32_t nk = L;
        for (uint32_t m0 = 0; m0 < maxM; m0 += 32) {
          uint32_t mm = m0 + lane;
          bool fresh = false;
          uint32_t nb = 0;
          if (mm < maxM) {
            nb = gids[row + mm];
            uint32_t bit = 1u << (nb & 31);
            fresh = !(atomicOr(&vis[nb >> 5], bit) & bit);
          }
          uint32_t fm = __ballot_sync(FULL, fresh);
          uint32_t cnt = __popc(fm);
          if (cnt == 0) continue;
          uint32_t src = lane < cnt ? __fns(fm, 0, lane + 1) : 0;
          uint32_t my = __shfl_sync(FULL, nb, src);
          float d = warp_row_dists(qv, c.ld4, base, ld, my, cnt, lane);
          evals += cnt;
          uint64_t dk = warp_sort32(lane < cnt ? pack_key(d, my) : ~0ULL, lane);
          // merge the cnt sorted keys into the list (capacity C)
          uint32_t lb = lane < cnt ? lower_bound_keys(list, L, dk) : L;
          uint32_t newL = min(c.C, L + cnt);
          uint32_t first = __shfl_sync(FULL, lb, 0);
          // old entries move right: those in [lb_j, lb_{j+1}) (lb_cnt = L) by j + 1, the highest
          // segment first, each copied from its top down (reads before writes within a round)
          for (int32_t j = (int32_t)cnt - 1; j >= 0; --j) {
            const uint32_t s_lo = __shfl_sync(FULL, lb, j);
            const uint32_t s_hi = __shfl_sync(FULL, lb, j + 1 < (int32_t)cnt ? j + 1 : j);
            const uint32_t top = j + 1 < (int32_t)cnt ? s_hi : L;
            for (int32_t hi = (int32_t)top; hi > (int32_t)s_lo; hi -= 32) {
              int32_t i = hi - 32 + (int32_t)lane;
              bool act = i >= (int32_t)s_lo;
              uint64_t v = act ? list[i] : 0;
              __syncwarp();
              if (act && (uint32_t)i + j + 1 < newL) list[i + j + 1] = v;
              __syncwarp();
            }
          }
          if (lane < cnt && lb + lane < newL) list[lb + lane] = dk;
          __syncwarp();
          L = newL;
          if (first < newL && first < nk) nk = first;
        }
        kpos = min(nk, p + 1);
      }
      // running top k: merge the list's first min(L, k) entries
      uint32_t Lk = min(L, c.k);
      uint32_t nr = min(c.k, rc + Lk);
      for (uint32_t i = lane; i < rc; i += 32) {
        uint64_t a = res[i];
        uint32_t pos = i + lower_bound_keys(list, Lk, a);
        if (pos < nr) res2[pos] = a;
      }
      for (uint32_t i = lane; i < Lk; i += 32) {
        uint64_t b = kmask(list[i]);
        uint32_t pos = i + lower_bound_keys(res, rc, b);
        if (pos < nr) res2[pos] = b;
      }
      __syncwarp();
      uint64_t* t = res;
      res = res2;
      res2 = t;
      rc = nr;
    }
    for (uint32_t i = lane; i < c.k; i += 32)
      out[q * c.k + i] = i < rc ? (int32_t)((uint32_t)res[i] & KID_MASK) : -1;
    __syncwarp();
  }
  if (lane == 0) {
    atomicAdd(stats, evals);
    atomicAdd(stats + 2, expanded);
  }
}

}  // namespace

int kgraph_search_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, uint32_t k, int32_t* d_out,
                         cudaStream_t s, bool count_evals, const KgSeedSource* hs) {
  NvtxRange range("efg: kgraph search");
  SearchParams& sp = idx->sp;
  if (hs) {  // pools from the hash tables: no trees needed
    if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph: build or load a graph before searching");
    if (k == 0) return fail(EFG_ERR_ARG, "k must be positive");
  } else {
    EFG_TRY(search_common_checks(idx, k));
  }
  if (sp.init_num <= 0 || (uint64_t)sp.init_num > idx->n) return fail(EFG_ERR_ARG, "pool size must be in [1, n]");
  if (sp.epochs < 0 || sp.extend_to < 0) return fail(EFG_ERR_ARG, "negative epochs or extend");
  const uint32_t T = hs ? 0 : (uint32_t)sp.search_trees, E = (uint32_t)sp.extend_to, epochs = (uint32_t)sp.epochs;
  const uint32_t lsize = T ? (uint32_t)sp.init_num * 2 / (5 * T) + 1 : 0;  // from the pool size before it grows (:507)
  const uint64_t pool_size = (uint64_t)epochs * E;
  bool sorted = true;
  uint64_t init = (uint64_t)sp.init_num;
  if (pool_size >= init) {  // :510-514
    init = pool_size;
    sorted = false;
  }
  if (init > idx->n) return fail(EFG_ERR_ARG, "kgraph search: epochs * extend_to exceeds the number of points");
  if (k > 1024) return fail(EFG_ERR_ARG, "kgraph search: k above 1024 is not supported");
  if (E > 4096) return fail(EFG_ERR_ARG, "kgraph search: extend_to above 4096 is not supported");
  if (sorted && init > 16384) return fail(EFG_ERR_ARG, "kgraph search: pools above 16384 are not supported");
  sp.init_num = (int)init;  // the reference keeps the enlarged pool size for later searches
  if (nq == 0) return EFG_OK;

  KgCfg kc{};
  kc.epochs = epochs;
  kc.E = E;
  kc.k = k;
  kc.C = k + E;
  kc.list_slots = std::max<uint32_t>(kc.C + 1, next_pow2(std::max<uint32_t>(E, 2)));
  kc.key_stride = (uint32_t)init;
  kc.fixed_k = idx->graph.fixed_k;
  kc.ld4 = idx->ld / 4;
  kc.words = (uint32_t)round_up((idx->n + 31) / 32, 4);
  kc.o_list = (uint32_t)round_up((uint64_t)kc.ld4 * 16, 16);
  kc.o_res = (uint32_t)round_up(kc.o_list + (uint64_t)kc.list_slots * 8, 16);
  kc.o_res2 = (uint32_t)round_up(kc.o_res + (uint64_t)k * 8, 16);
  kc.warp_bytes = (uint32_t)round_up(kc.o_res2 + (uint64_t)k * 8, 16);
  kc.full_rows = hs ? 1 : 0;
  size_t smem = (size_t)KG_WARPS * kc.warp_bytes;
  if (smem > 200 * 1024) return fail(EFG_ERR_ARG, "kgraph search: k + extend_to too large for shared memory");

  SearchCfg cfg{};  // stage 1: the nnexp kernel up to the pool
  cfg.T = T;
  cfg.lsize = lsize;
  cfg.init_num = (uint32_t)init;
  cfg.extend_to = 0;
  cfg.result_size = 1;
  cfg.epochs = 0;
  cfg.k = 1;
  cfg.seed = idx->bp.seed;
  cfg.nseq = T * lsize;
  uint32_t maxdeg = graph_max_degree(idx);
  // hash seeds: pool * tables entries per query hold the probe's first `pool` distinct ids
  const uint64_t cap = hs ? init * hs->tables : 0;
  if (cap > 0xffffffffull) return fail(EFG_ERR_ARG, "kgraph search: pool * tables too large");
  cfg.nseeds = (uint32_t)cap;

  uint64_t chunk = std::max<uint64_t>(1, std::min<uint64_t>(nq, (512ull << 20) / (init * 8)));
  if (hs) chunk = std::max<uint64_t>(1, std::min<uint64_t>(chunk, (512ull << 20) / (cap * 4)));
  EFG_TRY(idx->kg_keys.reserve(chunk * init));
  if (hs) {
    EFG_TRY(hs->buf->reserve(chunk * cap));
    EFG_TRY(hs->cnt->reserve(chunk));
    cfg.seed_cnt = hs->cnt->p;
  }
  EFG_CUDA(cudaFuncSetAttribute(kgraph_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kgraph_kernel, KG_WARPS * 32, smem);
  uint64_t max_warps = std::max<uint64_t>(KG_WARPS, (512ull << 20) / ((uint64_t)kc.words * 4));
  uint64_t warps = std::min<uint64_t>({round_up(chunk, KG_WARPS), (uint64_t)sms * std::max(1, per_sm) * KG_WARPS,
                                       round_up(max_warps, KG_WARPS)});
  uint64_t grid = std::max<uint64_t>(1, warps / KG_WARPS);
  EFG_TRY(idx->kg_bits.reserve(grid * KG_WARPS * kc.words));

  EFG_TRY(idx->eval_counter.reserve(8));
  EFG_CUDA(cudaMemsetAsync(idx->eval_counter.p, 0, 32, s));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  int launches = 0, rc = EFG_OK;
  const uint64_t nchunks = (nq + chunk - 1) / chunk;
  LocalBuf<uint32_t> qctr;  // one query counter per chunk launch
  EFG_TRY(qctr.reserve(nchunks));
  EFG_CUDA(cudaMemsetAsync(qctr.p, 0, nchunks * 4, s));
  for (uint64_t q0 = 0; q0 < nq && rc == EFG_OK; q0 += chunk) {
    uint64_t m = std::min(chunk, nq - q0);
    int l = 0;
    if (hs) {
      rc = hash_seed_rows(hs->h, hs->d_qcodes + q0, hs->qstride, m, (uint32_t)cap, hs->buf->p, hs->cnt->p, s);
      if (rc != EFG_OK) break;
      ++launches;
    }
    rc = launch_nnexp(idx, cfg, maxdeg, d_q + q0 * qld, m, qld, nullptr, idx->kg_keys.p, s, &l, nullptr, nullptr,
                      hs ? hs->buf->p : nullptr);
    launches += l;
    if (rc == EFG_OK && sorted) {
      rc = launch_row_sort(idx->kg_keys.p, m, (uint32_t)init, (uint32_t)init, s);
      launches += (int)((m + 65534) / 65535);
    }
    if (rc != EFG_OK) break;
    kgraph_kernel<<<(unsigned)grid, KG_WARPS * 32, smem, s>>>(idx->d_base, idx->dim, idx->ld, idx->graph.ptr.p,
                                                              idx->graph.ids.p, d_q + q0 * qld, m, qld,
                                                              idx->kg_keys.p, kc, d_out + q0 * k, idx->kg_bits.p,
                                                              idx->eval_counter.p, qctr.p + q0 / chunk);
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) rc = fail(EFG_ERR_CUDA, std::string("kgraph launch: ") + cudaGetErrorString(le));
    ++launches;
  }
  cudaEventRecord(e1, s);
  if (rc == EFG_OK && count_evals) rc = finish_search_stats(idx, s, e0, e1, nq, false, launches, 0);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

}  // namespace efg
