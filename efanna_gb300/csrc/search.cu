// Graph search over batched queries: the "nnexp" method of getNeighbors_nnexp
// (algorithm/kdtreeub_index.hpp:363-494).
//
// One CTA (256 threads) answers one query at a time; per-query state lives in shared memory.
// Steps, as in the reference:
//   1. per tree, the first lsize = init_num*2/(5*trees)+1 leaves of a near-first DFS
//      (getSearchNodeList, :332-346).  Computed as a level-by-level frontier expansion: every node
//      knows how many leaves its subtree holds, so the near child starts at its parent's DFS rank
//      and the far child at that rank plus the near subtree's leaf count; subtrees whose first
//      rank is >= lsize are dropped and a leaf's rank is its position in the DFS order.  All
//      frontier nodes of a level are expanded in parallel instead of one serial walk per tree.
//   2. leaves interleaved leaf-rank-major, tree-minor; ids deduplicated in that order until
//      init_num are collected (:396-410) -- processed 1024 sequence positions at a time with a
//      chunk-local table that keeps the first position of every id; a counter-hash fill when the
//      leaves run short (:411-417).
//   3. distances to the pool; keep the resultSize = max(extend_to, k) best (:420-442).
//   4. `epochs` times: expand every not-yet-expanded id among the first extend_to through its
//      graph row, add the unvisited neighbours, keep the resultSize best (:444-484).
//   5. emit the first k ids (:486-492).
// Candidate lists are packed (dist_bits << 32 | id) keys, which order exactly like the reference's
// pair<float, size_t>.  The resultSize best are kept as one sorted list; candidates are folded
// into it 1024 at a time: keys at or above the current worst are dropped, the rest sorted and
// merged by rank.  Ids are unique, so the result does not depend on the order threads find them.
//
// The visited set (the reference's N-bit tbflag) is a double-hashing table in shared memory sized
// for the expected number of visits; the reference's newflag ("expanded") is a bit of the result
// keys.  A query whose set reaches 80% of the table at a phase boundary moves it to a worst-case
// table in global scratch; one that fills 90% within a phase is abandoned and listed, and a second
// launch answers the listed queries with worst-case tables in global memory.
#include <algorithm>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "search.cuh"

namespace efg {

// Two builds of the kernel: 256 threads (several CTAs per SM when the per-query shared state
// is small) and 512 threads (one CTA per SM when it is large).
static constexpr int FILL_CHUNK = 1024;  // sequence positions deduplicated per step
static constexpr int FILL_TAB = 2048;    // chunk-local id table
static constexpr int SEL_CHUNK = 1024;   // candidates folded into the result list per step
static constexpr uint32_t ID_MASK = 0x3FFFFFFFu;

enum : uint32_t { SERR_FRONTIER = 1u, SERR_HASH = 2u };


__device__ __forceinline__ uint32_t ht_slot(uint32_t id, uint32_t size) { return __umulhi(id * 2654435761u, size); }
// Double hashing: a second, odd probe step that is not a multiple of 3 -- coprime with every table
// size used here (2^k or 3 * 2^k slots), so a probe sequence visits every slot; it avoids the
// long clustered runs of linear probing at high load.
__device__ __forceinline__ uint32_t ht_step(uint32_t id, uint32_t size) {
  uint32_t st = 2 * __umulhi((id ^ (id >> 15)) * 0x85EBCA6Bu, size >> 1) + 1;
  if (st % 3 == 0) st = st + 2 < size ? st + 2 : st - 2;
  return st;
}
__device__ __forceinline__ uint32_t ht_next(uint32_t h, uint32_t st, uint32_t size) {
  h += st;
  return h >= size ? h - size : h;
}

// Inserts id into the visited set; true if it was not present.  When the set already holds
// `limit` ids (*count, which callers advance by the inserts they made, a warp at a time) the insert
// is refused and *ovf is set (the query goes to the overflow pass).
__device__ __forceinline__ bool ht_insert(uint32_t* ht, uint32_t size, uint32_t limit, uint32_t* count,
                                          uint32_t* ovf, uint32_t id) {
  uint32_t h = ht_slot(id, size), st = ht_step(id, size);
  for (uint32_t probe = 0; probe < size; ++probe) {
    uint32_t cur = *reinterpret_cast<volatile const uint32_t*>(&ht[h]);
    if (cur == kEmpty) {
      if (*reinterpret_cast<volatile uint32_t*>(count) >= limit) {
        atomicOr(ovf, 1u);
        return false;
      }
      uint32_t prev = atomicCAS(&ht[h], kEmpty, id);
      if (prev == kEmpty) return true;
      cur = prev;
    }
    if ((cur & ID_MASK) == id) return false;
    h = ht_next(h, st, size);
  }
  atomicOr(ovf, 1u);
  return false;
}
// ht_insert continued from slot h after `done` probes of id's sequence.
__device__ __forceinline__ bool ht_insert_from(uint32_t* ht, uint32_t size, uint32_t limit, uint32_t* count,
                                               uint32_t* ovf, uint32_t id, uint32_t h, uint32_t done) {
  const uint32_t st = ht_step(id, size);
  for (uint32_t probe = done; probe < size; ++probe) {
    uint32_t cur = *reinterpret_cast<volatile const uint32_t*>(&ht[h]);
    if (cur == kEmpty) {
      if (*reinterpret_cast<volatile uint32_t*>(count) >= limit) {
        atomicOr(ovf, 1u);
        return false;
      }
      uint32_t prev = atomicCAS(&ht[h], kEmpty, id);
      if (prev == kEmpty) return true;
      cur = prev;
    }
    if ((cur & ID_MASK) == id) return false;
    h = ht_next(h, st, size);
  }
  atomicOr(ovf, 1u);
  return false;
}

// XR inserts of one thread with their first probes issued together: the first slots' loads, then
// the compare-and-swaps of the ids whose first slot was empty, then (rarely) the rest of a probe
// sequence.  The same outcome as XR ht_insert calls in order: an id met twice in the batch takes
// its slot once (the second CAS returns the first's id).  kEmpty entries are skipped.
template <int XR>
__device__ __forceinline__ void ht_insert_batch(uint32_t* ht, uint32_t size, uint32_t limit, uint32_t* count,
                                                uint32_t* ovf, const uint32_t (&id)[XR], bool (&fresh)[XR]) {
  uint32_t h[XR], cur[XR], prev[XR];
#pragma unroll
  for (int u = 0; u < XR; ++u) h[u] = id[u] != kEmpty ? ht_slot(id[u], size) : 0u;
#pragma unroll
  for (int u = 0; u < XR; ++u) cur[u] = id[u] != kEmpty ? *reinterpret_cast<volatile const uint32_t*>(&ht[h[u]]) : 0u;
  const bool full = *reinterpret_cast<volatile uint32_t*>(count) >= limit;
#pragma unroll
  for (int u = 0; u < XR; ++u)
    prev[u] = (id[u] != kEmpty && cur[u] == kEmpty && !full) ? atomicCAS(&ht[h[u]], kEmpty, id[u]) : cur[u];
#pragma unroll
  for (int u = 0; u < XR; ++u) {
    fresh[u] = false;
    if (id[u] == kEmpty) continue;
    uint32_t c = cur[u];
    if (c == kEmpty) {
      if (full) {
        atomicOr(ovf, 1u);
        continue;
      }
      if (prev[u] == kEmpty) {
        fresh[u] = true;
        continue;
      }
      c = prev[u];
    }
    if ((c & ID_MASK) == id[u]) continue;
    fresh[u] = ht_insert_from(ht, size, limit, count, ovf, id[u], ht_next(h[u], ht_step(id[u], size), size), 1);
  }
}

__device__ __forceinline__ bool ht_contains(const uint32_t* ht, uint32_t size, uint32_t id) {
  uint32_t h = ht_slot(id, size), st = ht_step(id, size);
  for (uint32_t probe = 0; probe < size; ++probe) {
    uint32_t cur = *reinterpret_cast<volatile const uint32_t*>(&ht[h]);
    if (cur == kEmpty) return false;
    if ((cur & ID_MASK) == id) return true;
    h = ht_next(h, st, size);
  }
  return false;
}

// Ascending bitonic sort of n (power of two) keys by the whole block.
__device__ void sort_keys_block(uint64_t* keys, uint32_t n) {
  for (uint32_t k = 2; k <= n; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < (n >> 1); i += blockDim.x) {
        uint32_t lo = ((i & ~(j - 1)) << 1) | (i & (j - 1));  // index with bit j clear
        uint32_t hi = lo | j;
        uint64_t a = keys[lo], b = keys[hi];
        bool up = (lo & k) == 0;
        if ((a > b) == up) {
          keys[lo] = b;
          keys[hi] = a;
        }
      }
      __syncthreads();
    }
  }
}

namespace s256 {
static constexpr int S_THREADS = 256;
static constexpr int S_WARPS = S_THREADS / 32;
static constexpr int S_MIN_BLOCKS = 2;  // two CTAs per SM: at most 128 registers per thread
#include "search_kernel.inc"
}  // namespace s256
namespace s512 {
static constexpr int S_THREADS = 512;
static constexpr int S_WARPS = S_THREADS / 32;
static constexpr int S_MIN_BLOCKS = 1;
#include "search_kernel.inc"
}  // namespace s512

__global__ void to_bf16_kernel(const float* __restrict__ base, uint64_t n, uint32_t dim, uint32_t ld,
                               uint16_t* __restrict__ out, uint32_t ld16) {
  uint64_t total = n * ld16;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t r = i / ld16;
    uint32_t c = (uint32_t)(i - r * ld16);
    float v = c < dim ? base[r * ld + c] : 0.f;
    out[i] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
  }
}

// FP8 e4m3 rows with one scale per row: scale = max|x| / 448 (the largest e4m3 value), values
// x / scale rounded to nearest (saturating), rows padded with zeros to ld8 bytes.  One warp per row.
__global__ void to_fp8_kernel(const float* __restrict__ base, uint64_t n, uint32_t dim, uint32_t ld,
                              uint8_t* __restrict__ out, uint32_t ld8, float* __restrict__ scale) {
  uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint32_t lane = threadIdx.x & 31;
  if (r >= n) return;
  const float* row = base + r * ld;
  float mx = 0.f;
  for (uint32_t j = lane; j < dim; j += 32) mx = fmaxf(mx, fabsf(row[j]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  float s = mx > 0.f ? mx / 448.f : 1.f;
  for (uint32_t j = lane; j < ld8; j += 32)
    out[r * ld8 + j] = j < dim ? (uint8_t)__nv_cvt_float_to_fp8(row[j] / s, __NV_SATFINITE, __NV_E4M3) : 0;
  if (lane == 0) scale[r] = s;
}

int make_base8(efg_index* idx) {
  idx->ld8 = (uint32_t)round_up(idx->dim, 16);
  EFG_TRY(idx->base8.reserve(idx->n * idx->ld8));
  EFG_TRY(idx->scale8.reserve(idx->n));
  to_fp8_kernel<<<(unsigned)((idx->n * 32 + 255) / 256), 256, 0, idx->stream>>>(idx->d_base, idx->n, idx->dim, idx->ld,
                                                                                idx->base8.p, idx->ld8, idx->scale8.p);
  EFG_CUDA(cudaGetLastError());
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  return EFG_OK;
}

int make_base16(efg_index* idx) {
  idx->ld16 = (uint32_t)round_up(idx->dim, 8);
  EFG_TRY(idx->base16.reserve(idx->n * idx->ld16));
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  to_bf16_kernel<<<sms * 8, 256, 0, idx->stream>>>(idx->d_base, idx->n, idx->dim, idx->ld, idx->base16.p, idx->ld16);
  EFG_CUDA(cudaGetLastError());
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  return EFG_OK;
}

__global__ void __launch_bounds__(512) row_sort_kernel(uint64_t* keys, uint32_t stride, uint32_t count,
                                                       uint32_t p2) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* k = reinterpret_cast<uint64_t*>(smem);
  uint64_t* row = keys + (uint64_t)blockIdx.x * stride;
  for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) k[i] = i < count ? row[i] : ~0ULL;
  __syncthreads();
  sort_keys_block(k, p2);
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) row[i] = k[i];
}

int launch_row_sort(uint64_t* keys, uint64_t nq, uint32_t stride, uint32_t count, cudaStream_t s) {
  if (nq == 0 || count < 2) return EFG_OK;
  if (count > 16384) return fail(EFG_ERR_ARG, "kgraph search: pools above 16384 are not supported");
  uint32_t p2 = next_pow2(count);
  size_t smem = (size_t)p2 * 8;
  EFG_CUDA(cudaFuncSetAttribute(row_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for (uint64_t q0 = 0; q0 < nq; q0 += 65535) {
    uint64_t m = std::min<uint64_t>(nq - q0, 65535);
    row_sort_kernel<<<(unsigned)m, 512, smem, s>>>(keys + q0 * stride, stride, count, p2);
    EFG_CUDA(cudaGetLastError());
  }
  return EFG_OK;
}

int screen_pairs(efg_index* idx, int precision, const float* d_q, uint64_t nq, uint64_t qld, const uint32_t* d_ids,
                 uint32_t m, float* d_out, cudaStream_t s) {
  if (m == 0 || nq == 0) return EFG_OK;
  if (m > 4096) return fail(EFG_ERR_ARG, "at most 4096 ids per query");
  SearchCfg cfg{};
  if (precision == EFG_PRECISION_FP8) {
    if (!idx->base8.p) EFG_TRY(make_base8(idx));
    cfg.fp8 = 1;
    cfg.screened = 1;
    cfg.ld8 = idx->ld8;
    cfg.cpr8 = idx->ld8 / 16;
    uint32_t g = std::min<uint32_t>(next_pow2(cfg.cpr8), 32);
    while ((1u << cfg.gshift8) < g) ++cfg.gshift8;
  } else if (precision == EFG_PRECISION_BF16) {
    if (!idx->base16.p) EFG_TRY(make_base16(idx));
    cfg.screened = 1;
    cfg.ld16 = idx->ld16;
    cfg.cpr16 = idx->ld16 / 8;
    uint32_t g = std::min<uint32_t>(next_pow2(cfg.cpr16), 32);
    while ((1u << cfg.gshift16) < g) ++cfg.gshift16;
  } else if (precision != EFG_PRECISION_FP32) {
    return fail(EFG_ERR_ARG, "unknown precision");
  }
  cfg.q4 = std::max<uint32_t>(std::max<uint32_t>(idx->ld / 4, cfg.screened && !cfg.fp8 ? cfg.ld16 / 4 : 0u),
                              cfg.fp8 ? cfg.ld8 / 4 : 0u);
  size_t smem = round_up((size_t)cfg.q4 * 16 + (size_t)m * 4, 16) + (size_t)m * 8;
  EFG_CUDA(cudaFuncSetAttribute(s256::screen_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for (uint64_t q0 = 0; q0 < nq; q0 += 65535) {
    uint64_t b = std::min<uint64_t>(nq - q0, 65535);
    s256::screen_pairs_kernel<<<(unsigned)b, 256, smem, s>>>(idx->d_base, idx->dim, idx->ld, idx->base16.p,
                                                             idx->base8.p, idx->scale8.p, cfg, d_q + q0 * qld, qld,
                                                             d_ids + q0 * m, m, d_out + q0 * m);
    EFG_CUDA(cudaGetLastError());
  }
  return EFG_OK;
}

// Largest graph row length (the fixed degree when every row has K ids).
uint32_t graph_max_degree(efg_index* idx) { return idx->graph.max_deg; }

// Launches the nnexp kernel for cfg's search parameters (T, lsize, init_num, extend_to,
// result_size, epochs, k, seed, nseq and the precision fields set) over nq queries: a first pass
// with visited sets in shared memory and, when the worst case does not fit there, an overflow
// pass for the queries that outgrew them.  With d_keys set the kernel stops after the pool and
// writes each query's init_num packed (dist, id) keys in pool order instead of ids.
int launch_nnexp(efg_index* idx, SearchCfg cfg, uint32_t maxdeg, const float* d_q, uint64_t nq, uint64_t qld,
                 int32_t* d_out, uint64_t* d_keys, cudaStream_t s, int* launches, const efg_query_params* d_params,
                 const uint32_t* d_nq, const uint32_t* d_seeds) {
  *launches = 0;
  cfg.ids_cap = idx->candidate_cap;  // layout() reads it as a bound, then sets the buffer's size
  if (cfg.T > 256) return fail(EFG_ERR_ARG, "at most 256 search trees");
  if (cfg.lsize >= 65536) return fail(EFG_ERR_ARG, "pool too large for the tree descent");
  cfg.emit_pool = d_keys ? 1 : 0;
  cfg.fixed_k = idx->graph.fixed_k >= 2 ? idx->graph.fixed_k : 0;
  if (cfg.fixed_k) {
    // item r * K + c -> (r, c) by a multiply-high: exact while items * K < 2^32
    uint64_t items = (uint64_t)cfg.extend_to * cfg.fixed_k;
    if (items * cfg.fixed_k >= (1ull << 32)) cfg.fixed_k = 0;
    else cfg.kmagic = (uint32_t)(((1ull << 32) + cfg.fixed_k - 1) / cfg.fixed_k);
  }
  // visited set: shared memory sized for the expected visits; worst case in global memory
  uint64_t worst = (uint64_t)cfg.init_num + (uint64_t)cfg.epochs * cfg.extend_to * maxdeg;
  uint64_t expect = (uint64_t)cfg.init_num + (uint64_t)cfg.epochs * cfg.extend_to * maxdeg / 4;
  auto nice = [](uint64_t x) {  // the next size of the form 2^k or 3 * 2^k (coprime with the probe steps)
    uint64_t p = 256;
    while (p < x && p * 3 / 2 < x) p *= 2;
    return p >= x ? p : p * 3 / 2;
  };
  uint64_t big = nice(worst * 8 / 5 + 64);
  uint64_t small = std::min<uint64_t>(std::max<uint64_t>(nice(expect * 8 / 5), 2048), 12288);
  if (idx->search_ht_pct > 0)  // a plan's autotuner scales the shared table (sets that outgrow it migrate)
    small = std::max<uint64_t>(2048, nice(small * (uint64_t)idx->search_ht_pct / 100));
  small = std::min(small, big);
  if (big > (1ull << 28)) return fail(EFG_ERR_ARG, "search parameters visit too many candidates");
  // block size: 256 threads when several CTAs fit on an SM, else 512 threads
  int per_sm = 1;
  size_t smem_probe;
  {
    SearchCfg t = cfg;
    smem_probe = s256::layout(t, idx->ld, maxdeg, false, (uint32_t)small);
    EFG_CUDA(cudaFuncSetAttribute(s256::nnexp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::min<size_t>(smem_probe, 220 * 1024)));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, s256::nnexp_kernel, 256, smem_probe);
  }
  // block size: the autotuned choice when one is set, else 256 threads when two CTAs fit on an SM
  const bool wide = idx->search_threads ? idx->search_threads == 512 : per_sm < 2;
  const int threads = wide ? 512 : 256;
  auto kernel = wide ? s512::nnexp_kernel : s256::nnexp_kernel;
  auto layout = wide ? s512::layout : s256::layout;
  SearchCfg c1 = cfg, c2 = cfg;
  size_t smem1 = layout(c1, idx->ld, maxdeg, false, (uint32_t)small);
  c1.ht_limit = (uint32_t)(small * 4 / 5);
  c1.ht_soft = c1.ht_limit;
  size_t smem2 = layout(c2, idx->ld, maxdeg, true, (uint32_t)big);
  c2.ht_limit = (uint32_t)big;
  bool two_pass = big > small;
  if (smem1 > 200 * 1024) {  // the reduced set does not fit beside the rest: one pass, global set
    c1 = c2;
    smem1 = smem2;
    two_pass = false;
  }
  if (smem1 > 220 * 1024)
    return fail(EFG_ERR_ARG, "search parameters need " + std::to_string(smem1) +
                                 " bytes of shared memory per query (pool/extend/degree too large)");
  EFG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max(smem1, smem2)));
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem1);
  if (idx->search_ctas_per_sm > 0) per_sm = std::min(per_sm, idx->search_ctas_per_sm);
  uint64_t grid1 = std::min<uint64_t>(nq, (uint64_t)sms * std::max(1, per_sm));
  uint64_t grid2 = (uint64_t)sms;
  if (c1.ht_global) EFG_TRY(idx->ht_scratch.reserve(grid1 * c1.ht_size));
  if (two_pass && !c1.ht_global && grid1 * big * 4 <= (1ull << 30)) {
    // a query whose set holds 80% of the shared table at a phase boundary continues in a
    // worst-case table in global scratch; only a set that reaches 90% within one phase is handed
    // to the overflow pass
    c1.ht_mig = 1;
    c1.mig_size = (uint32_t)big;
    c1.ht_limit = (uint32_t)(small * 9 / 10);
    EFG_TRY(idx->ht_scratch.reserve(grid1 * big));
  }
  if (two_pass) {
    EFG_TRY(idx->ht_scratch.reserve(grid2 * c2.ht_size));
    EFG_TRY(idx->ovf_list.reserve(nq + 1));
    EFG_CUDA(cudaMemsetAsync(idx->ovf_list.p, 0, 4, s));
  }
  // the two passes' query counters, after the four statistics words
  EFG_TRY(idx->eval_counter.reserve(8));
  uint32_t* qctr = reinterpret_cast<uint32_t*>(idx->eval_counter.p + 4);
  EFG_CUDA(cudaMemsetAsync(qctr, 0, 2 * sizeof(uint32_t), s));
  c1.next_q = qctr;
  c2.next_q = qctr + 1;
  const Forest& F = idx->forest;
  kernel<<<(unsigned)grid1, threads, smem1, s>>>(
      idx->d_base, idx->n, idx->dim, idx->ld, F.nodes.p, F.nleaf.p, F.cnl.p, F.d_roots.p, F.leaves.p, idx->graph.ptr.p,
      idx->graph.ids.p, d_q, nq, qld, c1, d_out, idx->eval_counter.p, idx->ht_scratch.p, nullptr,
      two_pass ? idx->ovf_list.p : nullptr, idx->base16.p, d_keys, d_params, d_nq, d_seeds, idx->base8.p,
      idx->scale8.p);
  cudaError_t le = cudaGetLastError();
  *launches = 1;
  if (le == cudaSuccess && two_pass) {
    kernel<<<(unsigned)grid2, threads, smem2, s>>>(
        idx->d_base, idx->n, idx->dim, idx->ld, F.nodes.p, F.nleaf.p, F.cnl.p, F.d_roots.p, F.leaves.p, idx->graph.ptr.p,
        idx->graph.ids.p, d_q, nq, qld, c2, d_out, idx->eval_counter.p, idx->ht_scratch.p, idx->ovf_list.p, nullptr,
        idx->base16.p, d_keys, d_params, d_nq, d_seeds, idx->base8.p, idx->scale8.p);
    le = cudaGetLastError();
    *launches = 2;
  }
  if (le != cudaSuccess) return fail(EFG_ERR_CUDA, std::string("nnexp launch: ") + cudaGetErrorString(le));
  return EFG_OK;
}

// Search parameters common to both methods: checks and the tree-descent fields of the config.
int search_common_checks(efg_index* idx, uint32_t k) {
  const SearchParams& sp = idx->sp;
  if (idx->forest.ntrees == 0) return fail(EFG_ERR_STATE, "no trees: build or load trees before searching");
  if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph: build or load a graph before searching");
  if (sp.search_trees <= 0) return fail(EFG_ERR_ARG, "search trees must be positive");
  if ((uint32_t)sp.search_trees > idx->forest.ntrees) return fail(EFG_ERR_TREE_COUNT, "wrong tree number");
  if (k == 0) return fail(EFG_ERR_ARG, "k must be positive");
  return EFG_OK;
}

// Reads the per-call counters back into the index's search statistics.
int finish_search_stats(efg_index* idx, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, uint64_t nq, bool two_pass,
                        int launches, uint64_t reranked) {
  unsigned long long h[4];
  uint32_t novf = 0;
  EFG_CUDA(cudaMemcpyAsync(h, idx->eval_counter.p, 32, cudaMemcpyDeviceToHost, s));
  if (two_pass) EFG_CUDA(cudaMemcpyAsync(&novf, idx->ovf_list.p, 4, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  idx->sstats.device_ms = ms;
  idx->sstats.distance_evals = h[0];
  idx->sstats.queries = nq;
  idx->sstats.expanded_nodes = h[2];
  idx->sstats.overflow_queries = novf;
  idx->sstats.kernel_launches = (uint64_t)launches;
  idx->sstats.reranked = reranked;
  idx->sstats.migrated_queries = h[3];
  if (h[1] & SERR_FRONTIER) return fail(EFG_ERR_DEVICE_LIMIT, "tree descent frontier overflow");
  if (h[1] & SERR_HASH) return fail(EFG_ERR_DEVICE_LIMIT, "candidate buffer overflow");
  return EFG_OK;
}

int search_device_ex(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, const efg_query_params& lim_in,
                     const efg_query_params* d_params, const uint32_t* d_nq, int32_t* d_out, cudaStream_t s,
                     bool count_evals, const uint32_t* d_seeds, uint32_t seeds_per_query, bool use_trees,
                     bool bucket_only, const uint32_t* d_seed_counts) {
  NvtxRange range("efg: nnexp search");
  const SearchParams& sp = idx->sp;
  efg_query_params lim = lim_in;
  const uint32_t k = lim.k;
  if (bucket_only) {  // the seeds ranked, topped up to k: no trees, no graph, no epochs
    if (!d_seeds && nq) return fail(EFG_ERR_ARG, "the bucket search needs seeds");
    if (k == 0) return fail(EFG_ERR_ARG, "k must be positive");
    use_trees = false;
    lim.epochs = 0;
    lim.extend_to = 0;
  } else if (use_trees) {
    EFG_TRY(search_common_checks(idx, k));
  } else {  // a pool from the seeds alone (then the random fill): no trees needed
    if (!idx->graph.valid) return fail(EFG_ERR_STATE, "no graph: build or load a graph before searching");
    if (k == 0) return fail(EFG_ERR_ARG, "k must be positive");
  }
  if (lim.init_num <= 0 || (uint64_t)lim.init_num > idx->n) return fail(EFG_ERR_ARG, "pool size must be in [1, n]");
  if (lim.epochs < 0 || lim.extend_to < 0) return fail(EFG_ERR_ARG, "negative epochs or extend");
  if ((int)k > lim.init_num) return fail(EFG_ERR_ARG, "k must be in [1, pool size]");
  if (nq == 0) return EFG_OK;

  SearchCfg cfg{};
  cfg.T = use_trees ? (uint32_t)sp.search_trees : 0;
  cfg.lsize = cfg.T ? (uint32_t)lim.init_num * 2 / (5 * cfg.T) + 1 : 0;
  cfg.init_num = (uint32_t)lim.init_num;
  cfg.extend_to = std::min<uint32_t>((uint32_t)lim.extend_to, cfg.init_num);
  cfg.result_size = std::max<uint32_t>(cfg.extend_to, k);
  cfg.epochs = (uint32_t)lim.epochs;
  cfg.k = k;
  cfg.seed = idx->bp.seed;
  cfg.nseq = cfg.T * cfg.lsize;
  cfg.nseeds = d_seeds ? seeds_per_query : 0;
  cfg.seed_cnt = d_seeds ? d_seed_counts : nullptr;
  cfg.fill_k = bucket_only ? 1 : 0;
  if (idx->precision == EFG_PRECISION_FP8) {
    if (!idx->base8.p) EFG_TRY(make_base8(idx));
    cfg.fp8 = 1;
    cfg.ld8 = idx->ld8;
    cfg.cpr8 = idx->ld8 / 16;
    uint32_t g = std::min<uint32_t>(next_pow2(cfg.cpr8), 32);
    while ((1u << cfg.gshift8) < g) ++cfg.gshift8;
  }
  if (idx->precision == EFG_PRECISION_BF16 || idx->precision == EFG_PRECISION_FP8) {
    if (idx->precision == EFG_PRECISION_BF16 && !idx->base16.p) EFG_TRY(make_base16(idx));
    cfg.screened = 1;
    cfg.ld16 = idx->ld16;
    cfg.cpr16 = idx->ld16 / 8;
    uint32_t g = std::min<uint32_t>(next_pow2(cfg.cpr16), 32);
    while ((1u << cfg.gshift16) < g) ++cfg.gshift16;
    cfg.rerank = std::min<uint32_t>(std::min<uint32_t>(std::max(2 * k, k + 32), cfg.result_size),
                                    (uint32_t)SEL_CHUNK);
    if (k > cfg.rerank) return fail(EFG_ERR_ARG, "k above 1024 is not supported with BF16 screening");
  }
  uint32_t maxdeg = graph_max_degree(idx);
  EFG_TRY(idx->eval_counter.reserve(8));
  EFG_CUDA(cudaMemsetAsync(idx->eval_counter.p, 0, 32, s));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  int launches = 0;
  int rc = launch_nnexp(idx, cfg, maxdeg, d_q, nq, qld, d_out, nullptr, s, &launches, d_params, d_nq,
                        cfg.nseeds ? d_seeds : nullptr);
  cudaEventRecord(e1, s);
  if (rc == EFG_OK && count_evals)
    rc = finish_search_stats(idx, s, e0, e1, nq, launches == 2, launches, cfg.screened ? cfg.rerank : 0);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int search_device(efg_index* idx, const float* d_q, uint64_t nq, uint64_t qld, uint32_t k, int32_t* d_out,
                  cudaStream_t s, bool count_evals) {
  const SearchParams& sp = idx->sp;
  if (sp.method == 1) return kgraph_search_device(idx, d_q, nq, qld, k, d_out, s, count_evals);
  if (sp.method != 0) return fail(EFG_ERR_ARG, "no such searching method");
  efg_query_params lim{sp.epochs, sp.init_num, sp.extend_to, k};
  return search_device_ex(idx, d_q, nq, qld, lim, nullptr, nullptr, d_out, s, count_evals);
}

}  // namespace efg
