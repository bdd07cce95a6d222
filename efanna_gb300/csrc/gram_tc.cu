// Exact k-NN screening on the fifth-generation tensor cores (tcgen05, sm_103a).
//
// Matrix::brute_force_search (general/matrix.hpp:57-68) ranks every base row by its squared L2
// distance to the query.  Written as ||q||^2 + ||x||^2 - 2 q.x, the distances of a block of
// queries against a block of base rows are one dense Gram contraction, which this file runs as
// BF16 tcgen05.mma tiles accumulated in FP32 in tensor memory (TMEM):
//
//   * queries and base rows are converted once per call to BF16 rows padded to a multiple of 64
//     values (128 bytes, one 128-byte-swizzle row), together with their FP32 squared norms.  Data
//     whose values BF16 holds exactly (the integer-valued configurations: values in [0, 255]) use
//     one product per tile, and then every product and every FP32 partial sum is an exact integer
//     below 2^24, so the screened distances equal the exact ones.  Other data are split as
//     x = hi + lo (two BF16 values) and each tile accumulates hi.hi + hi.lo + lo.hi, which leaves
//     an error near 2^-16 of |q.x| instead of 2^-8.
//   * a CTA owns one work item at a time: 128 queries (the MMA's M, one TMEM lane each) against
//     one chunk of base rows, walked in tiles of 128 rows (N).  Warp 0 streams the operand
//     k-blocks into a ring of shared-memory stages with cp.async.bulk.tensor (TMA, 128-byte
//     swizzle), one (query block, base block) pair per stage -- in the split form three pairs per
//     k-block: (hi, hi), (hi, lo), (lo, hi); one thread of warp 1 issues the MMAs (K = 16 each) into one of two TMEM
//     accumulators and commits them to mbarriers; warps 2-5 read the other accumulator with
//     tcgen05.ld, one query per thread, turn each Gram value into a distance and keep the
//     query's best K2 = k + 16 (distance, id) keys of the chunk.  The two accumulators let the
//     MMAs of tile t + 1 run while tile t is being screened.
//   * every query starts with a bound on its K2-th distance: the K2-th distance over a strided
//     sample of the base, from a first pass of the same kernel over the sample alone (any subset's
//     K2-th distance bounds the whole base's from above).  Per group of 64 values a branch-free
//     test (one FMA, one compare per value) builds each thread's mask of values under its bound;
//     only values in some mask reach the exact test, one per lane per round, and go straight into
//     the thread's sorted list in shared memory, which tightens the bound once it holds K2 keys.
//     The base-row norms of the next tile are loaded while the current one is screened, and the
//     second half of the accumulator is read from TMEM during the first.
//
// The chunks' lists are the same per-(query, chunk) lists the FP32 kernel writes (distance.cu);
// the same merge kernel then re-ranks the K2 survivors of each query in FP64.  Every wait on an
// mbarrier is bounded: a wait that runs out sets an error word and the CTA leaves its loops,
// drains its tensor-core work and frees its TMEM; the host turns the word into
// EFG_ERR_DEVICE_LIMIT.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <mutex>

#include "internal.cuh"
#include "tcgen05.cuh"

namespace efg {

int bf_merge_launch(const float* base, uint32_t dim, uint32_t ld, const float* q, uint64_t nq, uint32_t qld,
                    uint32_t k, uint32_t K2, uint32_t nchunks, const uint64_t* part, int32_t* ids, float* dists,
                    cudaStream_t s);

namespace {

constexpr uint32_t TM = 128;           // queries per tile (MMA M, TMEM lanes)
constexpr uint32_t TN = 128;           // base rows per tile (MMA N, TMEM columns per accumulator)
constexpr uint32_t TKB = 64;           // BF16 values per k-block: one 128-byte swizzle row
constexpr uint32_t PART = TM * TKB * 2;  // bytes of one 128 x 64 BF16 operand block (16 KiB)
constexpr uint32_t GRP = 16;           // values per screening group (one any-hit vote)
// warp 0 TMA, warp 1 MMA (+TMEM), then EW screening warps: 4 (each thread one query, all 128
// columns of a tile) or 8 (two threads per query, 64 columns each, two warps per scheduler)
template <int EW>
constexpr uint32_t kThreads = 64 + 32 * EW;
constexpr uint32_t MAX_STAGES = 8;
constexpr uint32_t TMEM_COLS = 2 * TN;  // two FP32 accumulators of 128 columns

constexpr uint32_t IDESC = tc::idesc_bf16(TM, TN);
using namespace tc;

struct TcArgs {
  const float* qnorm;  // nq FP32 squared norms
  const float* xnorm;  // squared norms of the base rows, +inf past n (rounded up to a tile)
  const float* qbound; // per query an upper bound of its K2-th distance, or null (+inf)
  uint64_t* part;      // nq x nchunks x K2 keys
  int* err;
  uint64_t n, chunk, first_row;
  uint32_t nq, qtiles, nchunks, K2, kblocks, terms, stages, exclude_self;
  uint32_t o_list, o_scr, o_xn;  // byte offsets of the lists, scratch and norm copies in dynamic shared memory
};

__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64]) {
  tmem_ld16(taddr, r);
  tmem_ld16(taddr + 16, r + 16);
  tmem_ld16(taddr + 32, r + 32);
  tmem_ld16(taddr + 48, r + 48);
}

// Inserts a key into a thread's sorted list of at most K2 keys (a full list drops its last key).
// Lists are slot-major with a stride of LS (the screening threads), so the threads of a warp touch
// consecutive words.
template <uint32_t LS>
__device__ __forceinline__ void insert_key(uint64_t* list, uint32_t t, uint32_t K2, uint32_t& lcnt, uint64_t key) {
  if (lcnt == K2 && key >= list[(K2 - 1) * LS + t]) return;
  uint32_t j = lcnt < K2 ? lcnt : K2 - 1;
  while (j > 0) {
    const uint64_t prev = list[(j - 1) * LS + t];
    if (prev <= key) break;
    list[j * LS + t] = prev;
    --j;
  }
  list[j * LS + t] = key;
  if (lcnt < K2) ++lcnt;
}

template <int EW>
__global__ void __launch_bounds__(kThreads<EW>, 1)
    tc_knn_kernel(const __grid_constant__ CUtensorMap mq_hi, const __grid_constant__ CUtensorMap mq_lo,
                  const __grid_constant__ CUtensorMap mx_hi, const __grid_constant__ CUtensorMap mx_lo,
                  const TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[MAX_STAGES], bar_empty[MAX_STAGES], bar_tfull[2], bar_tempty[2],
      bar_drain;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;

  // stages start on a 1024-byte boundary (the swizzle pattern repeats every 1024 bytes)
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  unsigned char* smem = smem_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t stage_bytes = 2 * PART;  // a query block and a base block
  const uint32_t steps = a.kblocks * a.terms;  // stages per tile
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < a.stages; ++s) {
      mbar_init(smem_addr(&bar_full[s]), 1);
      mbar_init(smem_addr(&bar_empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_addr(&bar_tfull[b]), 1);
      mbar_init(smem_addr(&bar_tempty[b]), 32 * EW);
    }
    mbar_init(smem_addr(&bar_drain), 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // the whole warp allocates the two accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_sh)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = tmem_base_sh;
  volatile int* abort_flag = &abort_sh;
  const uint32_t items = a.qtiles * a.nchunks;
  bool mma_issued = false;

  if (warp == 0) {
    // ---------------------------------------------------------------- TMA producer (one lane)
    if (lane == 0) {
      uint32_t s = 0, ph = 0;
      bool ok = true;
      for (uint32_t w = blockIdx.x; ok && w < items; w += gridDim.x) {
        const uint32_t chunk = w / a.qtiles, qt = w % a.qtiles;
        const uint64_t r0 = (uint64_t)chunk * a.chunk, r1 = min(a.n, r0 + a.chunk);
        const uint32_t ntiles = (uint32_t)((r1 - r0 + TN - 1) / TN);
        for (uint32_t t = 0; ok && t < ntiles; ++t) {
          for (uint32_t step = 0; step < steps; ++step) {
            if (!mbar_wait(smem_addr(&bar_empty[s]), ph ^ 1u, abort_flag, a.err)) {
              ok = false;
              break;
            }
            const uint32_t kb = step / a.terms, term = step - kb * a.terms;  // term 0 (hi,hi), 1 (hi,lo), 2 (lo,hi)
            const uint32_t fb = smem_addr(&bar_full[s]);
            mbar_expect_tx(fb, stage_bytes);
            const uint32_t st = sbase + s * stage_bytes;
            const int x = (int)(kb * TKB), yq = (int)(qt * TM), yx = (int)(r0 + (uint64_t)t * TN);
            tma_load_2d(st, term == 2 ? &mq_lo : &mq_hi, fb, x, yq);
            tma_load_2d(st + PART, term == 1 ? &mx_lo : &mx_hi, fb, x, yx);
            if (++s == a.stages) {
              s = 0;
              ph ^= 1u;
            }
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- MMA issuer (one lane)
    if (lane == 0) {
      uint32_t s = 0, ph = 0, tcount = 0;
      bool ok = true;
      for (uint32_t w = blockIdx.x; ok && w < items; w += gridDim.x) {
        const uint32_t chunk = w / a.qtiles;
        const uint64_t r0 = (uint64_t)chunk * a.chunk, r1 = min(a.n, r0 + a.chunk);
        const uint32_t ntiles = (uint32_t)((r1 - r0 + TN - 1) / TN);
        for (uint32_t t = 0; ok && t < ntiles; ++t, ++tcount) {
          const uint32_t b = tcount & 1u, tph = (tcount >> 1) & 1u;
          if (!mbar_wait(smem_addr(&bar_tempty[b]), tph ^ 1u, abort_flag, a.err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d_tmem = tmem_base + b * TN;
          for (uint32_t step = 0; step < steps; ++step) {
            if (!mbar_wait(smem_addr(&bar_full[s]), ph, abort_flag, a.err)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t st = sbase + s * stage_bytes;
            const uint64_t dq = sw128_desc(st), dx = sw128_desc(st + PART);
#pragma unroll
            for (uint32_t j = 0; j < TKB / 16; ++j) {  // K = 16 per MMA: 32 bytes further along the row
              const uint64_t o = (uint64_t)(2 * j);
              umma_bf16(d_tmem, dq + o, dx + o, IDESC, (step | j) != 0 ? 1u : 0u);
            }
            mma_issued = true;
            umma_commit(smem_addr(&bar_empty[s]));  // frees the stage when these MMAs have read it
            if (++s == a.stages) {
              s = 0;
              ph ^= 1u;
            }
          }
          if (!ok) break;
          umma_commit(smem_addr(&bar_tfull[b]));  // accumulator b holds tile t
        }
      }
    }
  } else {
    // ---------------------------------------------------------------- screening (warps 2 ..)
    constexpr uint32_t CH = EW / 4;             // column parts of a tile (threads per query)
    constexpr uint32_t CPT = TN / CH;           // columns per thread per tile
    constexpr uint32_t LS = 32 * EW;            // list stride: all screening threads
    const uint32_t ew = warp - 2;
    const uint32_t quad = warp & 3u;            // TMEM lanes 32 * quad .. + 31
    const uint32_t et = quad * 32 + lane;       // this thread's query within the tile
    const uint32_t cp = ew / 4;                 // its column part: columns cp * CPT ..
    const uint32_t lt = cp * TM + et;           // its list
    uint64_t* list = reinterpret_cast<uint64_t*>(smem + a.o_list);
    // this thread's copy of a group's 16 values, float4 slot j4 stored at j4 ^ ((lane >> 1) & 3): the
    // eight threads of a quarter warp then write eight different 16-byte bank groups
    float* scr = reinterpret_cast<float*>(smem + a.o_scr) + (ew * 32 + lane) * GRP;
    const uint32_t sw = (lane >> 1) & 3u;
    // base-row norms of the current and the next tile, one copy per warp (warp-local hand-over)
    float* xw = reinterpret_cast<float*>(smem + a.o_xn) + ew * 2 * TN;
    uint32_t tcount = 0;
    bool ok = true;
    for (uint32_t w = blockIdx.x; ok && w < items; w += gridDim.x) {
      const uint32_t chunk = w / a.qtiles, qt = w % a.qtiles;
      const uint64_t r0 = (uint64_t)chunk * a.chunk, r1 = min(a.n, r0 + a.chunk);
      const uint32_t ntiles = (uint32_t)((r1 - r0 + TN - 1) / TN);
      const uint32_t q = qt * TM + et;
      const bool qvalid = q < a.nq;
      const float qn = qvalid ? a.qnorm[q] : 0.f;
      const uint64_t self = a.exclude_self ? a.first_row + q : ~0ull;
      uint32_t lcnt = 0;
      // distance bound: the K2-th key's once the list is full; a thread past the queries accepts nothing
      float thr = qvalid ? (a.qbound ? a.qbound[q] : INFINITY) : -1.f;
      // the group test compares xn - 2 q.x against thr - qn, widened by a few ulps so that it never
      // rejects what the exact test (d = xn - 2 q.x + qn <= thr) accepts
      auto bound = [&](float t) { return qvalid ? t - qn + (fabsf(t) + qn) * 4.8e-7f : -INFINITY; };
      float lim = bound(thr);
      reinterpret_cast<float4*>(xw + (tcount & 1u) * TN)[lane] =
          __ldg(reinterpret_cast<const float4*>(a.xnorm + r0) + lane);
      __syncwarp();
      for (uint32_t t = 0; t < ntiles; ++t, ++tcount) {
        const uint32_t b = tcount & 1u, tph = (tcount >> 1) & 1u;
        const uint64_t row0 = r0 + (uint64_t)t * TN;
        const bool more = t + 1 < ntiles;
        float4 xnext = make_float4(0.f, 0.f, 0.f, 0.f);
        if (more) xnext = __ldg(reinterpret_cast<const float4*>(a.xnorm + row0 + TN) + lane);  // in flight meanwhile
        // every lane waits; the vote keeps the warp together for the warp-wide TMEM loads
        ok = __all_sync(0xffffffffu, mbar_wait(smem_addr(&bar_tfull[b]), tph, abort_flag, a.err));
        if (!ok) break;
        tc_fence_after();
        const bool edge = row0 + TN > r1 || (self >= row0 && self < row0 + TN);
        const uint32_t taddr = tmem_base + ((quad * 32u) << 16) + b * TN + cp * CPT;
        const float* xs = xw + (tcount & 1u) * TN + cp * CPT;
        uint32_t va[64], vb[64];
        tmem_ld64(taddr, va);
        tmem_wait();
        if (CPT == 128) tmem_ld64(taddr + 64, vb);  // the second half arrives while the first is screened
#pragma unroll
        for (uint32_t half = 0; half < CPT / 64; ++half) {
          if (half == 1) tmem_wait();
          const uint32_t* v = half == 0 ? va : vb;
#pragma unroll
          for (uint32_t g = 0; g < 64 / GRP; ++g) {
            const float4* x4 = reinterpret_cast<const float4*>(xs + half * 64 + g * GRP);
            // any value of the group under the bound? (four independent chains)
            bool h0 = false, h1 = false, h2 = false, h3 = false;
#pragma unroll
            for (uint32_t j4 = 0; j4 < GRP / 4; ++j4) {
              const float4 xn = x4[j4];
              const uint32_t o = g * GRP + 4 * j4;
              h0 |= fmaf(-2.f, __uint_as_float(v[o + 0]), xn.x) <= lim;
              h1 |= fmaf(-2.f, __uint_as_float(v[o + 1]), xn.y) <= lim;
              h2 |= fmaf(-2.f, __uint_as_float(v[o + 2]), xn.z) <= lim;
              h3 |= fmaf(-2.f, __uint_as_float(v[o + 3]), xn.w) <= lim;
            }
            const bool hit = h0 | h1 | h2 | h3;
            if (__any_sync(0xffffffffu, hit)) {
              // the group's values under the bound, as a mask; this thread's values to its scratch
              uint32_t m = 0;
              if (hit) {
#pragma unroll
                for (uint32_t j4 = 0; j4 < GRP / 4; ++j4) {
                  const float4 xn = x4[j4];
                  const uint32_t o = g * GRP + 4 * j4;
                  m |= (fmaf(-2.f, __uint_as_float(v[o + 0]), xn.x) <= lim ? 1u : 0u) << (4 * j4);
                  m |= (fmaf(-2.f, __uint_as_float(v[o + 1]), xn.y) <= lim ? 2u : 0u) << (4 * j4);
                  m |= (fmaf(-2.f, __uint_as_float(v[o + 2]), xn.z) <= lim ? 4u : 0u) << (4 * j4);
                  m |= (fmaf(-2.f, __uint_as_float(v[o + 3]), xn.w) <= lim ? 8u : 0u) << (4 * j4);
                  reinterpret_cast<float4*>(scr)[j4 ^ sw] =
                      make_float4(__uint_as_float(v[o]), __uint_as_float(v[o + 1]), __uint_as_float(v[o + 2]),
                                  __uint_as_float(v[o + 3]));
                }
              }
              // one marked value per lane per round: the exact test, straight into the sorted list
              while (__any_sync(0xffffffffu, m != 0u)) {
                if (m != 0u) {
                  const uint32_t j = __ffs(m) - 1;
                  m &= m - 1;
                  const float val = scr[(((j >> 2) ^ sw) << 2) | (j & 3u)];
                  const uint32_t c = half * 64 + g * GRP + j;
                  const float d = fmaxf(fmaf(-2.f, val, xs[c]) + qn, 0.f);
                  const uint64_t row = row0 + cp * CPT + c;
                  if (d <= thr && (!edge || (row < r1 && row != self))) {
                    insert_key<LS>(list, lt, a.K2, lcnt, ((uint64_t)__float_as_uint(d) << 32) | (uint32_t)row);
                    if (lcnt == a.K2) {
                      thr = __uint_as_float((uint32_t)(list[(a.K2 - 1) * LS + lt] >> 32));
                      lim = bound(thr);
                    }
                  }
                }
              }
            }
          }
        }
        tc_fence_before();
        mbar_arrive(smem_addr(&bar_tempty[b]));  // accumulator b may be overwritten
        if (more) reinterpret_cast<float4*>(xw + ((tcount + 1) & 1u) * TN)[lane] = xnext;
        __syncwarp();
      }
      if (!ok) break;
      if (qvalid) {  // list part cp of this (query, chunk): the merge sees CH lists per chunk
        uint64_t* dst = a.part + ((uint64_t)q * a.nchunks * CH + chunk * CH + cp) * a.K2;
        for (uint32_t i = 0; i < a.K2; ++i) dst[i] = i < lcnt ? list[i * LS + lt] : ~0ull;
      }
    }
  }

  // ------------------------------------------------------------------------------ teardown
  __syncthreads();
  if (warp == 1) {
    if (lane == 0 && mma_issued) {  // every MMA this thread issued has finished before TMEM is freed
      umma_commit(smem_addr(&bar_drain));
      unsigned long long t0 = clock64();
      while (!mbar_try_wait(smem_addr(&bar_drain), 0)) {
        if (clock64() - t0 > WAIT_CYCLES) {
          atomicOr(a.err, 2);
          break;
        }
      }
    }
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS)
                 : "memory");
  }
}

// Rows floor(i * n / S) of the converted base (hi, lo, norm) into S contiguous sample rows (a warp
// per row, 16-byte copies; W BF16 values per row).
__global__ void sample_rows_kernel(const uint4* __restrict__ hi, const uint4* __restrict__ lo,
                                   const float* __restrict__ norms, uint64_t n, uint32_t W, uint32_t S,
                                   uint4* __restrict__ shi, uint4* __restrict__ slo, float* __restrict__ snorms) {
  const uint32_t lane = threadIdx.x & 31, w16 = W / 8;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < S; i += nw) {
    const uint64_t r = i * n / S;
    for (uint32_t c = lane; c < w16; c += 32) {
      shi[i * w16 + c] = hi[r * w16 + c];
      slo[i * w16 + c] = lo[r * w16 + c];
    }
    if (lane == 0) snorms[i] = norms[r];
  }
}

// Per query the distance of the rank-th smallest key over its L sorted lists of `stride` keys (L <=
// 16, ~0 padded), widened by `rel` (the split form's passes may round differently); +inf when the
// lists hold fewer keys; never above the query's previous bound `prev` (when given).
__global__ void bound_kernel(const uint64_t* __restrict__ lists, uint64_t nq, uint32_t L, uint32_t stride,
                             uint32_t rank, float rel, const float* __restrict__ prev, float* __restrict__ out) {
  for (uint64_t qi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; qi < nq; qi += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t* a = lists + qi * L * stride;
    uint32_t pos[16];
    for (uint32_t l = 0; l < L; ++l) pos[l] = 0;
    uint64_t key = ~0ull;
    for (uint32_t r = 0; r < rank; ++r) {  // merge walk up to the rank-th key
      uint32_t best = 0;
      key = ~0ull;
      for (uint32_t l = 0; l < L; ++l) {
        const uint64_t h = pos[l] < stride ? a[l * stride + pos[l]] : ~0ull;
        if (h < key) {
          key = h;
          best = l;
        }
      }
      if (key == ~0ull) break;
      pos[best] += 1;
    }
    const float d = __uint_as_float((uint32_t)(key >> 32));
    float bnd = key == ~0ull ? INFINITY : d + d * rel;
    if (prev) bnd = fminf(bnd, prev[qi]);
    out[qi] = bnd;
  }
}

}  // namespace

thread_local efg_knn_stats g_knn_stats = {};

// Largest k the tensor-core path serves (the per-thread lists of K2 = k + 16 keys and the buffers
// must fit in shared memory beside two pipeline stages of the split form).
uint32_t tc_knn_max_k() { return 104; }

int brute_force_knn_tc(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                       uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                       cudaStream_t s, int force_split) {
  if (nq == 0) return EFG_OK;
  if (n >= (1ull << 31) || nq >= (1ull << 31)) return fail(EFG_ERR_ARG, "tensor-core k-NN: more than 2^31 rows");
  if (k > tc_knn_max_k()) return fail(EFG_ERR_ARG, "tensor-core k-NN: k above " + std::to_string(tc_knn_max_k()));
  const uint32_t K2 = (uint32_t)std::min<uint64_t>(k + 16, n);
  const uint32_t W = (dim + TKB - 1) / TKB * TKB;
  const uint32_t kblocks = W / TKB;
  const uint64_t qtiles = (nq + TM - 1) / TM;
  const uint64_t nrows_pad = (n + TN - 1) / TN * TN;

  int dev = 0, sms = 148;
  EFG_CUDA(cudaGetDevice(&dev));
  EFG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int smem_max = 0;
  EFG_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));

  // operands: BF16 hi/lo rows, norms, the inexact flag and the error word
  __nv_bfloat16 *xh = nullptr, *xl = nullptr, *qh = nullptr, *ql = nullptr;
  float *xn = nullptr, *qn = nullptr;
  int* flags = nullptr;
  uint64_t* part = nullptr;
  float *sn = nullptr, *qbound = nullptr;
  auto release = [&] {
    cudaFreeAsync(sn, s);
    cudaFreeAsync(qbound, s);
    cudaFreeAsync(xh, s);
    cudaFreeAsync(xl, s);
    cudaFreeAsync(qh, s);
    cudaFreeAsync(ql, s);
    cudaFreeAsync(xn, s);
    cudaFreeAsync(qn, s);
    cudaFreeAsync(flags, s);
    cudaFreeAsync(part, s);
  };
  struct Guard {
    decltype(release)& f;
    ~Guard() { f(); }
  } guard{release};
  EFG_CUDA(cudaMallocAsync((void**)&xh, n * W * 2, s));
  EFG_CUDA(cudaMallocAsync((void**)&xl, n * W * 2, s));
  EFG_CUDA(cudaMallocAsync((void**)&qh, nq * W * 2, s));
  EFG_CUDA(cudaMallocAsync((void**)&ql, nq * W * 2, s));
  EFG_CUDA(cudaMallocAsync((void**)&xn, nrows_pad * 4, s));
  EFG_CUDA(cudaMallocAsync((void**)&qn, nq * 4, s));
  EFG_CUDA(cudaMallocAsync((void**)&flags, 8, s));
  EFG_CUDA(cudaMemsetAsync(flags, 0, 8, s));
  cudaEvent_t ev[5] = {};
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      for (int i = 0; i < 5; ++i)
        if (e[i]) cudaEventDestroy(e[i]);
    }
  } evguard{ev};
  for (auto& e : ev) EFG_CUDA(cudaEventCreate(&e));
  EFG_CUDA(cudaEventRecord(ev[0], s));
  {
    const uint64_t warps = std::min<uint64_t>(nrows_pad, (uint64_t)sms * 64);
    to_bf16_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(base, n, dim, ld, W, xh, xl, xn, nrows_pad,
                                                                        flags);
    EFG_CUDA(cudaGetLastError());
    const uint64_t qwarps = std::min<uint64_t>(nq, (uint64_t)sms * 64);
    to_bf16_kernel<<<(unsigned)((qwarps * 32 + 255) / 256), 256, 0, s>>>(q, nq, dim, qld, W, qh, ql, qn, nq, flags);
    EFG_CUDA(cudaGetLastError());
  }
  int hflags[2] = {0, 0};
  EFG_CUDA(cudaMemcpyAsync(hflags, flags, 8, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  const uint32_t terms = (hflags[0] || force_split) ? 3u : 1u;

  // shared memory: pipeline stages, then the per-thread lists, scratch and norm copies
  const uint32_t stage_bytes = 2 * PART;
  // screening warps: eight (two threads per query) while their lists fit, else four
  auto warps_for = [](uint32_t K2l) { return K2l <= 48 ? 8u : 4u; };
  auto layout = [&](uint32_t K2l, uint32_t& stages, uint32_t& o_list, uint32_t& o_scr, uint32_t& o_xn,
                    size_t& smem) -> bool {
    const uint32_t ew = warps_for(K2l);
    const uint32_t lists = 32 * ew * K2l * 8, scratch = 32 * ew * GRP * 4, norms = ew * 2 * TN * 4;
    const int64_t room = (int64_t)smem_max - 1024 - 2048 - lists - scratch - norms;  // alignment pad, barriers
    stages = (uint32_t)std::min<int64_t>(MAX_STAGES, std::max<int64_t>(0, room / stage_bytes));
    o_list = stages * stage_bytes;
    o_scr = o_list + lists;
    o_xn = o_scr + scratch;
    smem = 1024 + (size_t)o_xn + norms;
    return stages >= 2;
  };
  auto launch = [&](const CUtensorMap& mq_h, const CUtensorMap& mq_l, const CUtensorMap& mx_h,
                    const CUtensorMap& mx_l, const float* xnorm, uint64_t rows, uint64_t chunk_rows,
                    uint32_t nch, uint32_t K2l, const float* qb, uint64_t* out, int excl, unsigned* grid_out) -> int {
    TcArgs a;
    uint32_t stages, o_list, o_scr, o_xn;
    size_t smem;
    if (!layout(K2l, stages, o_list, o_scr, o_xn, smem))
      return fail(EFG_ERR_ARG, "tensor-core k-NN: k too large for shared memory");
    a.qnorm = qn;
    a.xnorm = xnorm;
    a.qbound = qb;
    a.part = out;
    a.err = flags + 1;
    a.n = rows;
    a.chunk = chunk_rows;
    a.first_row = first_row;
    a.nq = (uint32_t)nq;
    a.qtiles = (uint32_t)qtiles;
    a.nchunks = nch;
    a.K2 = K2l;
    a.kblocks = kblocks;
    a.terms = terms;
    a.stages = stages;
    a.exclude_self = excl ? 1u : 0u;
    a.o_list = o_list;
    a.o_scr = o_scr;
    a.o_xn = o_xn;
    const unsigned grid = (unsigned)std::min<uint64_t>(qtiles * nch, (uint64_t)sms);
    if (warps_for(K2l) == 8) {
      EFG_CUDA(cudaFuncSetAttribute(tc_knn_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      tc_knn_kernel<8><<<grid, kThreads<8>, smem, s>>>(mq_h, mq_l, mx_h, mx_l, a);
    } else {
      EFG_CUDA(cudaFuncSetAttribute(tc_knn_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      tc_knn_kernel<4><<<grid, kThreads<4>, smem, s>>>(mq_h, mq_l, mx_h, mx_l, a);
    }
    EFG_CUDA(cudaGetLastError());
    if (grid_out) *grid_out = grid;
    g_knn_stats.stages = stages;
    return EFG_OK;
  };
  {
    uint32_t st, o1, o2, o3;
    size_t sm;
    if (!layout(K2 + 1, st, o1, o2, o3, sm)) return fail(EFG_ERR_ARG, "tensor-core k-NN: k too large for shared memory");
  }

  CUtensorMap mqh, mql, mxh, mxl;
  EFG_TRY(make_map(&mqh, qh, nq, W));
  EFG_TRY(make_map(&mql, ql, nq, W));
  EFG_TRY(make_map(&mxh, xh, n, W));
  EFG_TRY(make_map(&mxl, xl, n, W));

  // 1. bounds from strided samples of the base: the rank-th distance of a sample bounds the whole
  // base's (rank = K2, + 1 with exclude_self: a sample may hold the query itself).  Nested samples
  // growing 8x, each holding the previous one (strides that divide), each pass starting from the
  // previous bound so that it only admits about 8 x rank candidates.
  EFG_CUDA(cudaEventRecord(ev[1], s));
  const uint32_t rank = K2 + (exclude_self ? 1u : 0u);
  const uint32_t CHb = warps_for(rank) / 4;
  uint32_t S = 0;  // rows of the last bound pass
  auto bound_pass = [&](uint32_t rows, const float* prev, float* out) -> int {
    __nv_bfloat16 *bh = nullptr, *bl = nullptr;
    float* bn = nullptr;
    uint64_t* lists = nullptr;
    struct Free {
      cudaStream_t s;
      void* p[4];
      ~Free() {
        for (void* x : p) cudaFreeAsync(x, s);
      }
    } fr{s, {nullptr, nullptr, nullptr, nullptr}};
    // chunks: enough items for the SMs, at most 16 lists per query, at least 1024 rows each
    uint32_t nch = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((sms + qtiles - 1) / qtiles, 16 / CHb));
    nch = std::min<uint32_t>(nch, std::max<uint32_t>(1, rows / 1024));
    const uint32_t crow = (rows / nch + TN - 1) / TN * TN;
    nch = (rows + crow - 1) / crow;
    EFG_CUDA(cudaMallocAsync((void**)&bh, (uint64_t)rows * W * 2, s));
    fr.p[0] = bh;
    EFG_CUDA(cudaMallocAsync((void**)&bl, (uint64_t)rows * W * 2, s));
    fr.p[1] = bl;
    EFG_CUDA(cudaMallocAsync((void**)&bn, (uint64_t)rows * 4, s));
    fr.p[2] = bn;
    EFG_CUDA(cudaMallocAsync((void**)&lists, nq * nch * CHb * rank * 8, s));
    fr.p[3] = lists;
    sample_rows_kernel<<<(unsigned)std::min<uint64_t>((rows + 7) / 8, (uint64_t)sms * 8), 256, 0, s>>>(
        reinterpret_cast<const uint4*>(xh), reinterpret_cast<const uint4*>(xl), xn, n, W, rows,
        reinterpret_cast<uint4*>(bh), reinterpret_cast<uint4*>(bl), bn);
    EFG_CUDA(cudaGetLastError());
    CUtensorMap mbh, mbl;
    EFG_TRY(make_map(&mbh, bh, rows, W));
    EFG_TRY(make_map(&mbl, bl, rows, W));
    EFG_TRY(launch(mqh, mql, mbh, mbl, bn, rows, crow, nch, rank, prev, lists, 0, nullptr));
    bound_kernel<<<(unsigned)std::min<uint64_t>((nq + 127) / 128, 4096), 128, 0, s>>>(
        lists, nq, nch * CHb, rank, rank, terms == 1 ? 0.f : 1e-5f, prev, out);
    EFG_CUDA(cudaGetLastError());
    S = rows;
    return EFG_OK;
  };
  // sample sizes: S0 = 64 x rank (at least 2048) and 8x steps up to n / 16, each a multiple of the
  // previous one (so each sample holds the previous one) and of the tile height
  uint32_t S0 = 2048;
  while (S0 < 64 * rank) S0 *= 2;
  if (n / 16 >= S0) {
    EFG_CUDA(cudaMallocAsync((void**)&qbound, nq * 4, s));
    EFG_CUDA(cudaMallocAsync((void**)&sn, nq * 4, s));
    EFG_TRY(bound_pass(S0, nullptr, qbound));
    uint64_t last = S0;
    const uint64_t cap = std::min<uint64_t>(n / 16, 1u << 20);
    for (uint64_t Si = last * 8; Si <= cap; Si *= 8) {
      EFG_TRY(bound_pass((uint32_t)Si, qbound, sn));
      std::swap(sn, qbound);
      last = Si;
    }
    if (cap / last >= 2) {  // the largest multiple of the last sample within n / 16
      EFG_TRY(bound_pass((uint32_t)(cap / last * last), qbound, sn));
      std::swap(sn, qbound);
    }
  }

  // 2. the whole base in (query tile, base chunk) items, about 8 per SM, balanced over the SMs
  uint64_t best_nc = 1;
  double best_cost = 1e300;
  const uint32_t CH = warps_for(K2) / 4;  // lists per (query, chunk)
  const uint64_t max_nc = std::max<uint64_t>(1, std::min<uint64_t>(4096 / (K2 * CH), (n + TN - 1) / TN));
  const uint64_t target = std::max<uint64_t>(1, ((uint64_t)sms * 8 + qtiles - 1) / qtiles);
  for (uint64_t nc = std::max<uint64_t>(1, target / 2); nc <= std::min(max_nc, target * 2); ++nc) {
    const uint64_t chunk = ((n + nc - 1) / nc + TN - 1) / TN * TN;
    const uint64_t real = (n + chunk - 1) / chunk, itm = qtiles * real;
    const uint64_t waves = (itm + sms - 1) / sms;
    // time ~ waves x tiles per item; a small merge cost per chunk
    const double cost = (double)waves * (double)(chunk / TN) + 0.02 * (double)real * (double)(chunk / TN);
    if (cost < best_cost) {
      best_cost = cost;
      best_nc = real;
    }
  }
  const uint64_t chunk = ((n + best_nc - 1) / best_nc + TN - 1) / TN * TN;
  const uint32_t nchunks = (uint32_t)((n + chunk - 1) / chunk);
  EFG_CUDA(cudaMallocAsync((void**)&part, nq * nchunks * CH * K2 * 8, s));
  EFG_CUDA(cudaEventRecord(ev[2], s));
  unsigned grid = 0;
  EFG_TRY(launch(mqh, mql, mxh, mxl, xn, n, chunk, nchunks, K2, S ? qbound : nullptr, part, exclude_self, &grid));
  EFG_CUDA(cudaEventRecord(ev[3], s));
  EFG_TRY(bf_merge_launch(base, dim, ld, q, nq, qld, k, K2, nchunks * CH, part, ids, dists, s));
  EFG_CUDA(cudaEventRecord(ev[4], s));
  EFG_CUDA(cudaMemcpyAsync(hflags, flags, 8, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  float ms[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
  g_knn_stats.convert_ms = ms[0];
  g_knn_stats.bound_ms = ms[1];
  g_knn_stats.screen_ms = ms[2];
  g_knn_stats.merge_ms = ms[3];
  g_knn_stats.sample_rows = S;
  g_knn_stats.screen_flops = 2.0 * (double)nq * (double)n * (double)dim;
  g_knn_stats.tile_flops = 2.0 * (double)(qtiles * TM) * (double)(nchunks * chunk) * (double)W * (double)terms;
  g_knn_stats.terms = terms;
  g_knn_stats.nchunks = nchunks;
  g_knn_stats.ctas = grid;
  if (hflags[1]) return fail(EFG_ERR_DEVICE_LIMIT, "tensor-core k-NN: a pipeline wait ran out (error word " +
                                                        std::to_string(hflags[1]) + ")");
  return EFG_OK;
}

}  // namespace efg
