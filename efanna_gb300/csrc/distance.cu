// Squared-L2 kernels: row-pair distances and exact brute-force k-NN.
//
// The reference's distance is L2DistanceAVX::compare (general/distance.hpp:299-323), a squared
// L2 in FP32 with eight running lane sums.  Here a warp computes one distance: lane l owns the
// float4 chunks l, l+32, ... of both rows (coalesced 512-byte row reads at d = 128), and the 32
// partial sums are folded by an xor butterfly.  The summation order differs from the AVX one
// only by FP32 rounding; on integer-valued data every order is exact.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "internal.cuh"

namespace efg {

// Partial squared distance of one lane's chunks; the caller reduces across the warp.
__device__ __forceinline__ float lane_l2(const float4* __restrict__ a, const float4* __restrict__ b, uint32_t dim,
                                         uint32_t lane) {
  float acc = 0.f;
  uint32_t c4n = (dim + 3) >> 2;
  for (uint32_t c = lane; c < c4n; c += 32) {
    float4 x = __ldg(a + c), y = __ldg(b + c);
    uint32_t base = c << 2;
    float d0 = x.x - y.x, d1 = x.y - y.y, d2 = x.z - y.z, d3 = x.w - y.w;
    if (base + 4 > dim) {  // ragged last chunk: the caller's padding is not assumed to be zero
      if (base + 1 > dim) d0 = 0.f;
      if (base + 2 > dim) d1 = 0.f;
      if (base + 3 > dim) d2 = 0.f;
      d3 = 0.f;
    }
    acc += d0 * d0;
    acc += d1 * d1;
    acc += d2 * d2;
    acc += d3 * d3;
  }
  return acc;
}

__global__ void l2_pairs_kernel(const float* __restrict__ base, uint32_t dim, uint32_t ld,
                                const uint32_t* __restrict__ ia, const uint32_t* __restrict__ ib, uint64_t m,
                                float* __restrict__ out) {
  uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t lane = threadIdx.x & 31;
  uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (; w < m; w += nw) {
    const float4* a = reinterpret_cast<const float4*>(base + (uint64_t)ia[w] * ld);
    const float4* b = reinterpret_cast<const float4*>(base + (uint64_t)ib[w] * ld);
    float v = warp_sum(lane_l2(a, b, dim, lane));
    if (lane == 0) out[w] = v;
  }
}

int launch_l2_pairs(const float* base, uint32_t dim, uint32_t ld, const uint32_t* a, const uint32_t* b, uint64_t m,
                    float* out, cudaStream_t s) {
  if (m == 0) return EFG_OK;
  uint64_t blocks = std::min<uint64_t>((m + 7) / 8, 152ull * 64);
  l2_pairs_kernel<<<(unsigned)blocks, 256, 0, s>>>(base, dim, ld, a, b, m, out);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

// ---------------------------------------------------------------------------------------------
// Brute-force k-NN.  A block holds QB queries and scans one chunk of base rows, one row per
// thread per step; distances below a query's current threshold go to that query's candidate
// buffer in shared memory, which is pruned (sorted, cut to K2 = k + margin) when it fills.  A
// second kernel merges the chunks' lists per query and re-ranks the K2 survivors in FP64.
// ---------------------------------------------------------------------------------------------
static constexpr int BF_QB = 16;        // queries per block
static constexpr int BF_THREADS = 256;  // rows per step
static constexpr int BF_CAP = 1024;     // candidate buffer per query
static constexpr int BF_MARGIN = 16;    // extra candidates kept for the FP64 re-rank

// Base chunks of the FP32 kernel: enough blocks for eight per SM, chunks of at least 2048 rows, and
// at most 4096 keys per query for the merge.
static uint64_t bf_chunks(uint64_t n, uint64_t nq, uint32_t K2) {
  uint64_t qblocks = (nq + BF_QB - 1) / BF_QB;
  uint64_t want = std::max<uint64_t>(1, (152ull * 8 + qblocks - 1) / qblocks);
  uint64_t nchunks = std::min<uint64_t>(want, std::max<uint64_t>(1, n / 2048));
  return std::min<uint64_t>(nchunks, std::max<uint64_t>(1, 4096 / K2));
}

// Sorts `n` (power of two) keys in shared memory with the whole block.
__device__ void block_bitonic_sort(uint64_t* keys, uint32_t n) {
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

// Sorts `n` (power of two) keys in shared memory with one warp.
__device__ void warp_bitonic_sort(uint64_t* keys, uint32_t n) {
  uint32_t lane = threadIdx.x & 31;
  for (uint32_t k = 2; k <= n; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = lane; i < n; i += 32) {
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
      __syncwarp();
    }
  }
}

__global__ void __launch_bounds__(BF_THREADS) bf_chunk_kernel(const float* __restrict__ base, uint64_t n,
                                                               uint32_t dim, uint32_t ld,
                                                               const float* __restrict__ q, uint64_t nq,
                                                               uint32_t qld, uint32_t K2, uint64_t chunk,
                                                               int exclude_self, uint64_t first_row,
                                                               uint64_t* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t ld4 = (dim + 3) >> 2;
  float4* qt = reinterpret_cast<float4*>(smem);                              // BF_QB * ld4
  uint64_t* cand = reinterpret_cast<uint64_t*>(qt + (size_t)BF_QB * ld4);   // BF_QB * BF_CAP
  __shared__ uint32_t cnt[BF_QB];
  __shared__ uint64_t thr[BF_QB];
  __shared__ int need_prune;

  uint64_t q0 = (uint64_t)blockIdx.x * BF_QB;
  uint64_t r0 = (uint64_t)blockIdx.y * chunk;
  uint64_t r1 = min(n, r0 + chunk);
  uint32_t nqb = (uint32_t)((nq - q0) < (uint64_t)BF_QB ? (nq - q0) : (uint64_t)BF_QB);
  for (uint32_t i = threadIdx.x; i < BF_QB * ld4; i += blockDim.x) {
    uint32_t qq = i / ld4, c = i % ld4;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (qq < nqb) {
      const float* src = q + (q0 + qq) * qld + 4 * c;
      v.x = src[0];
      v.y = 4 * c + 1 < dim ? src[1] : 0.f;
      v.z = 4 * c + 2 < dim ? src[2] : 0.f;
      v.w = 4 * c + 3 < dim ? src[3] : 0.f;
    }
    qt[i] = v;
  }
  if (threadIdx.x < BF_QB) {
    cnt[threadIdx.x] = 0;
    thr[threadIdx.x] = ~0ULL;
  }
  __syncthreads();

  auto prune = [&](void) {
    // warp w prunes queries w, w + 8
    uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t qq = warp; qq < BF_QB; qq += BF_THREADS / 32) {
      uint64_t* buf = cand + (size_t)qq * BF_CAP;
      uint32_t c = cnt[qq] < (uint32_t)BF_CAP ? cnt[qq] : (uint32_t)BF_CAP;
      uint32_t p2 = 1;
      while (p2 < c) p2 <<= 1;
      for (uint32_t i = c + lane; i < p2; i += 32) buf[i] = ~0ULL;
      __syncwarp();
      warp_bitonic_sort(buf, p2);
      uint32_t keep = min(c, K2);
      if (lane == 0) {
        cnt[qq] = keep;
        if (keep == K2) thr[qq] = buf[K2 - 1];
      }
      __syncwarp();
    }
  };

  // two rows per thread per step: every query chunk read from shared memory serves both
  for (uint64_t rb = r0; rb < r1; rb += 2 * BF_THREADS) {
    const uint64_t ra = rb + threadIdx.x, rc = ra + BF_THREADS;
    if (ra < r1) {
      const bool two = rc < r1;
      float acc0[BF_QB], acc1[BF_QB];
#pragma unroll
      for (int j = 0; j < BF_QB; ++j) {
        acc0[j] = 0.f;
        acc1[j] = 0.f;
      }
      const float4* row0 = reinterpret_cast<const float4*>(base + ra * ld);
      const float4* row1 = reinterpret_cast<const float4*>(base + (two ? rc : ra) * ld);
      for (uint32_t c = 0; c < ld4; ++c) {
        float4 x0 = __ldg(row0 + c), x1 = __ldg(row1 + c);
        uint32_t e = c << 2;
        if (e + 4 > dim) {
          if (e + 2 > dim) x0.y = x1.y = 0.f;
          if (e + 3 > dim) x0.z = x1.z = 0.f;
          x0.w = x1.w = 0.f;
        }
#pragma unroll
        for (int j = 0; j < BF_QB; ++j) {
          float4 y = qt[j * ld4 + c];
          float d0 = x0.x - y.x, d1 = x0.y - y.y, d2 = x0.z - y.z, d3 = x0.w - y.w;
          acc0[j] += d0 * d0;
          acc0[j] += d1 * d1;
          acc0[j] += d2 * d2;
          acc0[j] += d3 * d3;
          float e0 = x1.x - y.x, e1 = x1.y - y.y, e2 = x1.z - y.z, e3 = x1.w - y.w;
          acc1[j] += e0 * e0;
          acc1[j] += e1 * e1;
          acc1[j] += e2 * e2;
          acc1[j] += e3 * e3;
        }
      }
#pragma unroll
      for (int j = 0; j < BF_QB; ++j) {
        if ((uint32_t)j >= nqb) continue;
        if (!(exclude_self && ra == first_row + q0 + j)) {
          uint64_t key = pack_key(acc0[j], (uint32_t)ra);
          if (key < thr[j]) {
            uint32_t pos = atomicAdd(&cnt[j], 1u);
            if (pos < BF_CAP) cand[(size_t)j * BF_CAP + pos] = key;
          }
        }
        if (two && !(exclude_self && rc == first_row + q0 + j)) {
          uint64_t key = pack_key(acc1[j], (uint32_t)rc);
          if (key < thr[j]) {
            uint32_t pos = atomicAdd(&cnt[j], 1u);
            if (pos < BF_CAP) cand[(size_t)j * BF_CAP + pos] = key;
          }
        }
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int np = 0;
      for (int j = 0; j < BF_QB; ++j) np |= cnt[j] + 2 * BF_THREADS > BF_CAP;
      need_prune = np;
    }
    __syncthreads();
    if (need_prune) {
      prune();
      __syncthreads();
    }
  }
  prune();
  __syncthreads();
  for (uint32_t qq = 0; qq < nqb; ++qq) {
    uint64_t* dst = part + ((q0 + qq) * gridDim.y + blockIdx.y) * K2;
    for (uint32_t i = threadIdx.x; i < K2; i += blockDim.x)
      dst[i] = i < cnt[qq] ? cand[(size_t)qq * BF_CAP + i] : ~0ULL;
  }
}

// Merges the per-chunk lists of one query (one warp per query) and re-ranks in FP64.  Each list is
// sorted ascending (~0 padded), so the K2 smallest keys overall are taken head by head: lane l
// follows lists l, l + 32, ..., and each round the warp minimum of the lanes' best heads is taken
// and its list advanced (keys are distinct: ids differ across chunks).
__global__ void bf_merge_kernel(const float* __restrict__ base, uint32_t dim, uint32_t ld,
                                const float* __restrict__ q, uint64_t nq, uint32_t qld, uint32_t k, uint32_t K2,
                                uint32_t nlists, const uint64_t* __restrict__ part, int32_t* __restrict__ ids,
                                float* __restrict__ dists) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t wpb = blockDim.x >> 5;
  uint64_t qi = (uint64_t)blockIdx.x * wpb + warp;
  uint64_t* buf = reinterpret_cast<uint64_t*>(smem) + (size_t)warp * K2;  // the K2 selected keys
  double* d64 = reinterpret_cast<double*>(smem + (size_t)wpb * K2 * 8) + (size_t)warp * K2;
  uint32_t* pos = reinterpret_cast<uint32_t*>(smem + (size_t)wpb * K2 * 16) + (size_t)warp * nlists;
  if (qi >= nq) return;
  const uint64_t* src = part + qi * (uint64_t)nlists * K2;
  for (uint32_t l = lane; l < nlists; l += 32) pos[l] = 0;
  __syncwarp();
  uint64_t hk = ~0ULL;  // this lane's smallest head and its list
  uint32_t hl = 0;
  auto lane_best = [&]() {
    hk = ~0ULL;
    for (uint32_t l = lane; l < nlists; l += 32) {
      const uint32_t p = pos[l];
      const uint64_t h = p < K2 ? src[(uint64_t)l * K2 + p] : ~0ULL;
      if (h < hk) {
        hk = h;
        hl = l;
      }
    }
  };
  lane_best();
  for (uint32_t r = 0; r < K2; ++r) {
    uint64_t m = hk;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const uint64_t other = __shfl_xor_sync(0xffffffffu, m, o);
      m = other < m ? other : m;
    }
    if (lane == 0) buf[r] = m;
    if (m != ~0ULL && hk == m) {  // the lane holding the minimum advances that list
      pos[hl] += 1;
      lane_best();
    }
    __syncwarp();
  }
  // FP64 re-rank of the K2 selected keys
  const float* qr = q + qi * qld;
  for (uint32_t i = 0; i < K2; ++i) {
    uint64_t key = buf[i];
    double acc = 0.0;
    if (key != ~0ULL) {
      const float* br = base + (uint64_t)(uint32_t)key * ld;
      for (uint32_t c = lane; c < dim; c += 32) {
        double t = (double)br[c] - (double)qr[c];
        acc += t * t;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    } else {
      acc = INFINITY;
    }
    if (lane == 0) d64[i] = acc;
  }
  __syncwarp();
  if (lane == 0) {  // insertion sort of K2 (<= 272) entries by (d64, id)
    for (uint32_t i = 1; i < K2; ++i) {
      double dv = d64[i];
      uint64_t kv = buf[i];
      int j = (int)i - 1;
      while (j >= 0 && (d64[j] > dv || (d64[j] == dv && (uint32_t)buf[j] > (uint32_t)kv))) {
        d64[j + 1] = d64[j];
        buf[j + 1] = buf[j];
        --j;
      }
      d64[j + 1] = dv;
      buf[j + 1] = kv;
    }
  }
  __syncwarp();
  for (uint32_t i = lane; i < k; i += 32) {
    uint64_t key = buf[i];
    ids[qi * k + i] = key == ~0ULL ? -1 : (int32_t)(uint32_t)key;
    if (dists) dists[qi * k + i] = key == ~0ULL ? INFINITY : (float)d64[i];
  }
}

// Launches the merge of the per-(query, chunk) lists `part` (nq x nlists x K2 keys, each list sorted):
// per query the K2 smallest keys, re-ranked in FP64, of which the k first go to ids (and dists).
int bf_merge_launch(const float* base, uint32_t dim, uint32_t ld, const float* q, uint64_t nq, uint32_t qld,
                    uint32_t k, uint32_t K2, uint32_t nlists, const uint64_t* part, int32_t* ids, float* dists,
                    cudaStream_t s) {
  const uint32_t wpb = 4;
  size_t msmem = (size_t)wpb * K2 * 16 + (size_t)wpb * nlists * 4;
  if (msmem > 48 * 1024) EFG_CUDA(cudaFuncSetAttribute(bf_merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msmem));
  bf_merge_kernel<<<(unsigned)((nq + wpb - 1) / wpb), wpb * 32, msmem, s>>>(base, dim, ld, q, nq, qld, k, K2, nlists,
                                                                            part, ids, dists);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

// The FP32 kernels with caller-provided scratch for the per-(query, chunk) candidate lists:
// `part` holds part_cap keys; the base is cut into as many chunks as fit (at least one).  Every
// slot the merge reads is written by bf_chunk_kernel first, so the scratch needs no clearing.
int brute_force_knn_in(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                       uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                       uint64_t* part, uint64_t part_cap, cudaStream_t s) {
  if (nq == 0) return EFG_OK;
  uint32_t K2 = std::min<uint64_t>(k + BF_MARGIN, n);
  if (nq * K2 > part_cap)
    return fail(EFG_ERR_ARG, "brute force needs " + std::to_string(nq * K2) + " scratch entries (queries x (k+" +
                                 std::to_string(BF_MARGIN) + ")); the built-in scratch holds " +
                                 std::to_string(part_cap));
  uint64_t nchunks = bf_chunks(n, nq, K2);
  nchunks = std::min<uint64_t>(nchunks, std::max<uint64_t>(1, part_cap / (nq * K2)));
  uint64_t chunk = (n + nchunks - 1) / nchunks;
  nchunks = (n + chunk - 1) / chunk;
  uint32_t ld4 = (dim + 3) / 4;
  size_t smem = (size_t)BF_QB * ld4 * 16 + (size_t)BF_QB * BF_CAP * 8;
  if (smem > 48 * 1024) EFG_CUDA(cudaFuncSetAttribute(bf_chunk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)((nq + BF_QB - 1) / BF_QB), (unsigned)nchunks);
  bf_chunk_kernel<<<grid, BF_THREADS, smem, s>>>(base, n, dim, ld, q, nq, qld, K2, chunk, exclude_self, first_row,
                                                 part);
  EFG_CUDA(cudaGetLastError());
  return bf_merge_launch(base, dim, ld, q, nq, qld, k, K2, (uint32_t)nchunks, part, ids, dists, s);
}

// The FP32 path with its scratch from the stream-ordered allocator: as many chunks as the
// occupancy target asks for.
int brute_force_knn(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                    uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                    cudaStream_t s) {
  if (nq == 0) return EFG_OK;
  uint32_t K2 = std::min<uint64_t>(k + BF_MARGIN, n);
  uint64_t nchunks = bf_chunks(n, nq, K2);
  uint64_t chunk = (n + nchunks - 1) / nchunks;
  nchunks = (n + chunk - 1) / chunk;
  const uint64_t cap = nq * nchunks * K2;
  uint64_t* part = nullptr;
  EFG_CUDA(cudaMallocAsync((void**)&part, cap * sizeof(uint64_t), s));
  int rc = brute_force_knn_in(base, n, dim, ld, q, nq, qld, k, exclude_self, first_row, ids, dists, part, cap, s);
  cudaFreeAsync(part, s);
  return rc;
}

}  // namespace efg
