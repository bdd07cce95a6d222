// Hashing-seeded search: the pool/extend search of the reference's hashing initialiser
// (HASHINGIndex::getNeighborsIEH32_nnexp / getNeighborsIEH64_nnexp, algorithm/hashing_index.hpp:1087-1200,
// 1354-1470).  Each base point carries one binary code per hash table (codes made outside the
// library, as in the reference); a query's pool is built by visiting its Hamming ball in the
// reference's order -- radius 0, 1, 2, ... and, inside a radius, the flipped bit positions as
// ascending tuples in lexicographic order (generateMask32/64, :348-860) -- with all tables probed at
// each mask, every bucket's points in ascending id order, first occurrences kept until the pool
// size; the random fill and the pool/extend expansion then run as in the tree-seeded search.
//
// On the device:
//   * one open-addressing table per hash table: code -> (first, count) of its bucket in an id list
//     sorted by (code, id), so a probe is one or two 16-byte loads instead of a map walk;
//   * one warp per query enumerates probes (mask j, table h) 32 at a time, unranking each lane's
//     mask from its index (no mask list in memory, so every radius the reference allows works),
//     and copies the buckets it hits, in probe order, into the query's seed row; a row of
//     pool * tables entries always holds the first `pool` distinct ids of the probe sequence (each
//     id sits in one bucket per table), and the search kernel keeps first occurrences;
//   * the pool/extend kernel with seeds and no trees (search_device_ex with use_trees = false);
//     without a graph, the same kernel with no epochs ranks the bucket ids, the random fill topping
//     the pool up to k only (the graph-less search getNeighbors32 / getNeighbors64, :929-1085).
#include <algorithm>
#include <atomic>
#include <system_error>
#include <thread>
#include <vector>

#include "internal.cuh"

using namespace efg;

struct HashSlot {
  unsigned long long code;
  uint32_t first;  // bucket start in the table's sorted id list
  uint32_t count;  // 0: an empty slot
};
static_assert(sizeof(HashSlot) == 16, "one 16-byte load per probe");

constexpr uint32_t HB_MAX_TABLES = 32;
constexpr uint32_t HB_MAX_BITS = 64;
constexpr uint32_t HB_MAX_RADIUS = 13;
constexpr uint64_t HB_MAX_PROBES = 1ull << 26;   // masks * tables per query
constexpr uint64_t HB_SEED_CHUNK = 1ull << 26;   // seed entries staged per search launch

struct efg_hash {
  efg_index* idx = nullptr;
  uint32_t tables = 0, bits = 0, radius = 0;
  uint64_t n = 0;
  uint64_t nmasks = 0;  // Hamming-ball size: sum over r <= radius of C(bits, r)
  uint32_t cap = 0;     // slots per table (a power of two)
  DevBuf<HashSlot> slots;
  DevBuf<uint32_t> ids;                // tables x n: ids sorted by (code, id)
  DevBuf<unsigned long long> binom;    // (HB_MAX_BITS + 1) x (HB_MAX_RADIUS + 1) binomials
  DevBuf<unsigned long long> rstart;   // radius r's first mask index, r = 0..radius+1
  DevBuf<uint32_t> seeds;
  DevBuf<uint32_t> counts;             // entries of each seed row before its padding
  DevBuf<unsigned long long> qcodes;   // staged query codes (host entry point)
};

namespace {

__host__ __device__ __forceinline__ uint64_t code_mix(uint64_t x) {  // splitmix64 finaliser
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

constexpr int BR = HB_MAX_RADIUS + 1;

// Probes and bucket copies, one warp per query.  qcodes[h * qstride + qi] is the query's code in
// table h; seeds[qi * cap_q + e] receives the e-th entry of the probe sequence (ids >= n pad the row).
__global__ void __launch_bounds__(256) hash_seed_kernel(const HashSlot* __restrict__ slots, uint32_t cap_mask,
                                                       const uint32_t* __restrict__ ids, uint64_t n, uint32_t H,
                                                       uint32_t bits, uint32_t radius,
                                                       const unsigned long long* __restrict__ binom_g,
                                                       const unsigned long long* __restrict__ rstart_g,
                                                       const unsigned long long* __restrict__ qcodes, uint64_t qstride,
                                                       uint64_t nq, uint32_t cap_q, uint32_t* __restrict__ seeds,
                                                       uint32_t* __restrict__ counts) {
  __shared__ unsigned long long binom[(HB_MAX_BITS + 1) * BR];
  __shared__ unsigned long long rstart[HB_MAX_RADIUS + 2];
  for (uint32_t i = threadIdx.x; i < (HB_MAX_BITS + 1) * BR; i += blockDim.x) binom[i] = binom_g[i];
  for (uint32_t i = threadIdx.x; i < radius + 2; i += blockDim.x) rstart[i] = rstart_g[i];
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t qi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (qi >= nq) return;  // whole warps leave together
  const unsigned long long myq = lane < H ? qcodes[(uint64_t)lane * qstride + qi] : 0ull;
  const uint64_t total = rstart[radius + 1] * H;
  uint32_t* row = seeds + qi * cap_q;
  uint64_t written = 0;
  for (uint64_t b = 0; b < total && written < cap_q; b += 32) {
    const uint64_t p = b + lane;
    uint32_t h = 0, first = 0, cnt = 0;
    unsigned long long mask = 0;
    if (p < total) {
      const uint64_t j = p / H;
      h = (uint32_t)(p - j * H);
      // mask j: its radius, then its rank among that radius's ascending bit tuples (lexicographic)
      uint32_t r = 0;
      while (r < radius && rstart[r + 1] <= j) ++r;
      unsigned long long m = j - rstart[r];
      uint32_t c = 0;
      for (uint32_t t = r; t > 0; --t) {
        // tuples whose next position is c: C(bits - 1 - c, t - 1)
        while (m >= binom[(bits - 1 - c) * BR + (t - 1)]) {
          m -= binom[(bits - 1 - c) * BR + (t - 1)];
          ++c;
        }
        mask |= 1ull << c;
        ++c;
      }
    }
    const unsigned long long code = __shfl_sync(0xffffffffu, myq, h) ^ mask;  // every lane takes part
    if (p < total) {
      const HashSlot* tab = slots + (uint64_t)h * (cap_mask + 1ull);
      uint32_t s = (uint32_t)code_mix(code) & cap_mask;
      for (uint32_t probe = 0; probe <= cap_mask; ++probe) {  // at most half full: ends at an empty slot
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(tab + s));
        const unsigned long long k = ((unsigned long long)v.y << 32) | v.x;
        if (v.w == 0) break;
        if (k == code) {
          first = v.z;
          cnt = v.w;
          break;
        }
        s = (s + 1) & cap_mask;
      }
    }
    // exclusive offsets of the buckets in probe order (lane order), capped at the row
    uint64_t inc = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t v = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += v;
    }
    const uint64_t off = written + inc - cnt;
    const uint64_t sum = __shfl_sync(0xffffffffu, inc, 31);
    uint32_t hits = __ballot_sync(0xffffffffu, cnt > 0 && off < cap_q);
    while (hits) {
      const int l = __ffs(hits) - 1;
      hits &= hits - 1;
      const uint64_t o = __shfl_sync(0xffffffffu, off, l);
      const uint32_t f = __shfl_sync(0xffffffffu, first, l), c = __shfl_sync(0xffffffffu, cnt, l),
                     hh = __shfl_sync(0xffffffffu, h, l);
      const uint32_t len = (uint64_t)c < cap_q - o ? c : (uint32_t)(cap_q - o);
      const uint32_t* src = ids + (uint64_t)hh * n + f;
      for (uint32_t i = lane; i < len; i += 32) row[o + i] = __ldg(src + i);
    }
    written += sum;
  }
  const uint32_t filled = written < cap_q ? (uint32_t)written : cap_q;
  if (counts) {  // the search reads only this much of the row
    if (lane == 0) counts[qi] = filled;
  } else {
    for (uint64_t e = filled + lane; e < cap_q; e += 32) row[e] = 0xffffffffu;
  }
}

}  // namespace

// Probe sequences of nq queries into rows of cap_q seeds (with counts: the entries present per row,
// the rest of the row left as it was; without: the rest padded with 0xffffffff).
int efg::hash_seed_rows(efg_hash* h, const uint64_t* d_qcodes, uint64_t qcode_stride, uint64_t nq,
                        uint32_t seeds_per_query, uint32_t* d_seeds, uint32_t* d_counts, cudaStream_t s) {
  if (nq == 0 || seeds_per_query == 0) return EFG_OK;
  const uint64_t warps_per_block = 8;
  const uint64_t blocks = (nq + warps_per_block - 1) / warps_per_block;
  if (blocks > 0x7fffffffull) return fail(EFG_ERR_ARG, "too many queries for one launch");
  hash_seed_kernel<<<(unsigned)blocks, 256, 0, s>>>(h->slots.p, h->cap - 1, h->ids.p, h->n, h->tables, h->bits,
                                                  h->radius, h->binom.p, h->rstart.p,
                                                  reinterpret_cast<const unsigned long long*>(d_qcodes),
                                                  qcode_stride, nq, seeds_per_query, d_seeds, d_counts);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

// Runs fn(h) for every table h on up to `tables` host threads (the calling one included); the
// tables are independent, so the result does not depend on the number of threads.
template <class F>
static void for_each_table(uint32_t tables, const F& fn) {
  std::atomic<uint32_t> next{0};
  auto worker = [&] {
    for (uint32_t h; (h = next.fetch_add(1)) < tables;) fn(h);
  };
  const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  for (uint32_t t = 1; t < std::min(tables, hw); ++t) {
    try {
      pool.emplace_back(worker);
    } catch (const std::system_error&) {
      break;  // fewer threads: the calling thread takes what is left
    }
  }
  worker();
  for (auto& th : pool) th.join();
}

extern "C" {

int efg_hash_create(efg_index* idx, const uint64_t* codes, uint32_t tables, uint32_t code_bits, uint32_t radius,
                    efg_hash** out) {
  if (!idx || !codes || !out) return fail(EFG_ERR_ARG, "null argument");
  *out = nullptr;
  if (tables < 1 || tables > HB_MAX_TABLES) return fail(EFG_ERR_ARG, "tables must be in [1, 32]");
  if (code_bits < 1 || code_bits > HB_MAX_BITS) return fail(EFG_ERR_ARG, "code_bits must be in [1, 64]");
  if (radius > HB_MAX_RADIUS || radius > code_bits) return fail(EFG_ERR_ARG, "radius must be <= min(13, code_bits)");
  const uint64_t n = idx->n;
  if (n >= 0xffffffffull) return fail(EFG_ERR_ARG, "too many base points for 32-bit bucket offsets");
  const uint64_t vmask = code_bits == 64 ? ~0ull : (1ull << code_bits) - 1;
  // binomials C(a, b), a <= 64, b <= 13 (C(64, 13) < 2^64), and the radius starts
  std::vector<unsigned long long> binom((HB_MAX_BITS + 1) * BR, 0);
  for (uint32_t a = 0; a <= HB_MAX_BITS; ++a) {
    binom[a * BR] = 1;
    for (uint32_t b = 1; b < (uint32_t)BR && b <= a; ++b)
      binom[a * BR + b] = binom[(a - 1) * BR + b - 1] + (b < a ? binom[(a - 1) * BR + b] : 0);
  }
  std::vector<unsigned long long> rstart(radius + 2, 0);
  for (uint32_t r = 0; r <= radius; ++r) rstart[r + 1] = rstart[r] + binom[code_bits * BR + r];
  if (rstart[radius + 1] * tables > HB_MAX_PROBES)
    return fail(EFG_ERR_ARG, "Hamming ball too large: masks * tables must be <= 2^26");
  // per table: ids sorted by (code, id), unique codes into an open-addressing table at most half
  // full; the tables are built on parallel host threads (allocations stay on the calling thread)
  std::vector<std::vector<std::pair<uint64_t, uint32_t>>> sorted(tables);
  for (auto& v : sorted) v.resize(n);
  std::vector<uint64_t> uniq(tables, 0);
  std::atomic<bool> bad_code{false};
  for_each_table(tables, [&](uint32_t h) {
    auto& v = sorted[h];
    for (uint64_t i = 0; i < n; ++i) {
      uint64_t c = codes[(uint64_t)h * n + i];
      if (c & ~vmask) {
        bad_code = true;
        return;
      }
      v[i] = {c, (uint32_t)i};
    }
    std::sort(v.begin(), v.end());
    uint64_t u = 0;
    for (uint64_t i = 0; i < n; ++i) u += i == 0 || v[i].first != v[i - 1].first;
    uniq[h] = u;
  });
  if (bad_code) return fail(EFG_ERR_ARG, "a code has bits above code_bits");
  uint64_t maxu = 1;
  for (uint64_t u : uniq) maxu = std::max(maxu, u);
  uint64_t cap = 16;
  while (cap < 2 * maxu) cap *= 2;
  if (cap > (1ull << 31)) return fail(EFG_ERR_ARG, "too many distinct codes");
  std::vector<HashSlot> hslots(cap * tables, HashSlot{0, 0, 0});
  std::vector<uint32_t> hids(n * tables);
  for_each_table(tables, [&](uint32_t h) {
    const auto& v = sorted[h];
    HashSlot* tab = hslots.data() + (uint64_t)h * cap;
    for (uint64_t i = 0; i < n;) {
      uint64_t e = i;
      while (e < n && v[e].first == v[i].first) {
        hids[(uint64_t)h * n + e] = v[e].second;
        ++e;
      }
      uint64_t s = code_mix(v[i].first) & (cap - 1);
      while (tab[s].count) s = (s + 1) & (cap - 1);
      tab[s] = HashSlot{(unsigned long long)v[i].first, (uint32_t)i, (uint32_t)(e - i)};
      i = e;
    }
  });
  efg_hash* H = new efg_hash();
  H->idx = idx;
  H->tables = tables;
  H->bits = code_bits;
  H->radius = radius;
  H->n = n;
  H->nmasks = rstart[radius + 1];
  H->cap = (uint32_t)cap;
  int rc = EFG_OK;
  if ((rc = H->slots.reserve(hslots.size())) != EFG_OK || (rc = H->ids.reserve(std::max<uint64_t>(hids.size(), 1))) != EFG_OK ||
      (rc = H->binom.reserve(binom.size())) != EFG_OK || (rc = H->rstart.reserve(rstart.size())) != EFG_OK) {
    efg_hash_destroy(H);
    return rc;
  }
  cudaStream_t s = idx->stream;
  cudaError_t e = cudaMemcpyAsync(H->slots.p, hslots.data(), hslots.size() * sizeof(HashSlot), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && n)
    e = cudaMemcpyAsync(H->ids.p, hids.data(), hids.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H->binom.p, binom.data(), binom.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(H->rstart.p, rstart.data(), rstart.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    efg_hash_destroy(H);
    return fail(EFG_ERR_CUDA, std::string("hash table upload: ") + cudaGetErrorString(e));
  }
  *out = H;
  return EFG_OK;
}

uint64_t efg_hash_ball_size(const efg_hash* h) { return h ? h->nmasks : 0; }

int efg_hash_seeds_device(efg_hash* h, const uint64_t* d_qcodes, uint64_t qcode_stride, uint64_t nq,
                          uint32_t seeds_per_query, uint32_t* d_seeds, void* stream) {
  if (!h || ((!d_qcodes || !d_seeds) && nq && seeds_per_query)) return fail(EFG_ERR_ARG, "null argument");
  if (qcode_stride < nq) return fail(EFG_ERR_ARG, "qcode_stride < nq");
  return hash_seed_rows(h, d_qcodes, qcode_stride, nq, seeds_per_query, d_seeds, nullptr, (cudaStream_t)stream);
}

int efg_hash_search_device(efg_index* idx, efg_hash* h, const float* d_q, uint64_t nq, uint64_t row_stride,
                           const uint64_t* d_qcodes, uint64_t qcode_stride, uint32_t k, int32_t* d_out, void* stream) {
  NvtxRange range("efg: hashing-seeded search");
  if (!idx || !h || ((!d_q || !d_qcodes || !d_out) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (h->idx != idx) return fail(EFG_ERR_ARG, "the hash tables belong to another index");
  if (row_stride < idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (qcode_stride < nq) return fail(EFG_ERR_ARG, "qcode_stride < nq");
  const SearchParams& sp = idx->sp;
  const bool buckets_only = !idx->graph.valid;  // getNeighbors32 / getNeighbors64 (:929-1085)
  if (!buckets_only && sp.method == 0) {  // the hashing initialiser's kgraph search (its method 0)
    KgSeedSource src{h, d_qcodes, qcode_stride, h->tables, &h->seeds, &h->counts};
    return kgraph_search_device(idx, d_q, nq, row_stride, k, d_out, (cudaStream_t)stream, false, &src);
  }
  if (!buckets_only && sp.method != 1) return fail(EFG_ERR_ARG, "no such searching method");
  if (sp.init_num <= 0 || (uint64_t)sp.init_num > idx->n) return fail(EFG_ERR_ARG, "pool size must be in [1, n]");
  if (nq == 0) return EFG_OK;
  efg_query_params lim{sp.epochs, sp.init_num, sp.extend_to, k};
  const uint32_t cap_q = (uint32_t)std::min<uint64_t>((uint64_t)sp.init_num * h->tables, 0xffffffffull);
  const uint64_t chunk = std::max<uint64_t>(1, HB_SEED_CHUNK / cap_q);
  cudaStream_t s = (cudaStream_t)stream;
  EFG_TRY(h->seeds.reserve(std::min(chunk, nq) * cap_q));
  EFG_TRY(h->counts.reserve(std::min(chunk, nq)));
  for (uint64_t q0 = 0; q0 < nq; q0 += chunk) {
    const uint64_t m = std::min(chunk, nq - q0);
    EFG_TRY(hash_seed_rows(h, d_qcodes + q0, qcode_stride, m, cap_q, h->seeds.p, h->counts.p, s));
    EFG_TRY(search_device_ex(idx, d_q + q0 * row_stride, m, row_stride, lim, nullptr, nullptr, d_out + q0 * k, s,
                             false, h->seeds.p, cap_q, false, buckets_only, h->counts.p));
  }
  return EFG_OK;
}

int efg_hash_search(efg_index* idx, efg_hash* h, const float* q, uint64_t nq, uint32_t dim, uint64_t row_stride,
                    const uint64_t* qcodes, uint32_t k, int32_t* out_ids) {
  if (!idx || !h || ((!q || !qcodes || !out_ids) && nq)) return fail(EFG_ERR_ARG, "null argument");
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
  EFG_TRY(h->qcodes.reserve(nq * h->tables));
  EFG_CUDA(cudaMemsetAsync(idx->q_buf.p, 0, nq * idx->ld * sizeof(float), idx->stream));
  EFG_CUDA(cudaMemcpy2DAsync(idx->q_buf.p, idx->ld * sizeof(float), q, row_stride * sizeof(float), dim * sizeof(float),
                             nq, cudaMemcpyHostToDevice, idx->stream));
  EFG_CUDA(cudaMemcpyAsync(h->qcodes.p, qcodes, nq * h->tables * sizeof(uint64_t), cudaMemcpyHostToDevice, idx->stream));
  EFG_TRY(efg_hash_search_device(idx, h, idx->q_buf.p, nq, idx->ld, reinterpret_cast<const uint64_t*>(h->qcodes.p), nq,
                                 k, idx->out_buf.p, idx->stream));
  EFG_CUDA(cudaMemcpyAsync(out_ids, idx->out_buf.p, nq * (uint64_t)k * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           idx->stream));
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  idx->last_results.assign(out_ids, out_ids + nq * (uint64_t)k);
  idx->last_nq = nq;
  idx->last_k = k;
  return EFG_OK;
}

void efg_hash_destroy(efg_hash* h) {
  if (!h) return;
  h->slots.release();
  h->ids.release();
  h->binom.release();
  h->rstart.release();
  h->seeds.release();
  h->counts.release();
  h->qcodes.release();
  delete h;
}

}  // extern "C"
