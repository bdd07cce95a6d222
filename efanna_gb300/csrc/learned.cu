// Learned form (no reference counterpart): a small MLP, trained on search traces the method itself
// generates, predicts for each query the k-means clusters of the base that hold its neighbours (their
// central members become entry seeds of the pool) and a search setting (an early-stop pool size);
// the plain pool/extend search runs with those, and remains the fallback.
//
// Build steps, all on the device with kernels below:
//   1. k-means over a seeded sample of the base: assignments by the exact brute-force kernel
//      (k = 1 against the centroids), updates by one CTA per cluster summing its members in sample
//      order (deterministic).  Then every base row is assigned, and each cluster keeps its
//      `entries_per_cluster` members nearest the centroid, ordered by (dist, id).
//   2. Traces (efg_learned_train): exact 10-NN of the training queries (or the plain search's ids at a
//      high reference setting, for large training sets) -> clusters of those
//      neighbours (the entry head's target distribution); plain searches at every setting of the
//      rung ladder -> per-query recall -> the smallest setting reaching min(target, best recall)
//      (the early-stop head's label).
//   3. Training: inputs standardised per dimension, H = hidden units,
//        h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), z = W3 h2 + b3,  z = [clusters | rungs],
//      loss = softmax cross-entropy of the cluster logits against the neighbour-cluster histogram
//      plus softmax cross-entropy of the rung logits against the label, averaged over the batch.
//      GEMM operands are BF16 (weights and activations; master weights FP32), accumulation FP32,
//      gradients FP32, Adam on the master weights.  The forward layers run on the tensor cores
//      (mlp_tc.cu: tcgen05 MMAs, bias and ReLU in the epilogue) where their inner size allows
//      (64 <= K <= 256, K a multiple of 8); the rest, and the gradient GEMMs, on CUDA cores.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cuda_bf16.h>

#include "internal.cuh"

using namespace efg;

namespace {

constexpr uint32_t FULLMASK = 0xffffffffu;
constexpr int GT_K = 10;  // neighbours per training query in the traces

__device__ __forceinline__ float ld_as_float(const float* p) { return *p; }
__device__ __forceinline__ float ld_as_float(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// ---------------------------------------------------------------------------------------------
// k-means and entry lists
// ---------------------------------------------------------------------------------------------
__global__ void gather_rows_kernel(const float* __restrict__ base, uint32_t ld, const uint32_t* __restrict__ rows,
                                   uint64_t m, float* __restrict__ out) {
  uint64_t total = m * ld;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t r = i / ld;
    out[i] = base[(uint64_t)rows[r] * ld + (i - r * ld)];
  }
}

// Per-dimension mean and 1/std over m rows (one thread per dimension, rows in order).
__global__ void norm_stats_kernel(const float* __restrict__ rows, uint64_t m, uint32_t dim, uint32_t ld,
                                  float* __restrict__ mean, float* __restrict__ istd) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ld) return;
  if (j >= dim) {
    mean[j] = 0.f;
    istd[j] = 0.f;
    return;
  }
  double s = 0, s2 = 0;
  for (uint64_t r = 0; r < m; ++r) {
    double v = rows[r * ld + j];
    s += v;
    s2 += v * v;
  }
  double mu = s / (double)m, var = s2 / (double)m - mu * mu;
  mean[j] = (float)mu;
  istd[j] = var > 1e-12 ? (float)(1.0 / sqrt(var)) : 0.f;
}

// One CTA per cluster: the mean of its members (sample order, so the sums are deterministic);
// an empty cluster keeps its centroid.
__global__ void kmeans_update_kernel(const float* __restrict__ rows, uint64_t m, const int32_t* __restrict__ assign,
                                     uint32_t dim, uint32_t ld, float* __restrict__ cent) {
  extern __shared__ uint32_t members[];  // blockDim.x entries
  __shared__ uint32_t wcount[32], total;
  const uint32_t c = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // accumulators: thread t owns dimensions t, t + blockDim, ... (at most 4 per thread)
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  uint64_t cnt = 0;
  for (uint64_t b0 = 0; b0 < m; b0 += blockDim.x) {
    uint64_t i = b0 + threadIdx.x;
    bool mine = i < m && assign[i] == (int32_t)c;
    uint32_t bal = __ballot_sync(FULLMASK, mine);
    if (lane == 0) wcount[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t s = 0;
      for (uint32_t w = 0; w < nw; ++w) {
        uint32_t t = wcount[w];
        wcount[w] = s;
        s += t;
      }
      total = s;
    }
    __syncthreads();
    if (mine) members[wcount[warp] + __popc(bal & ((1u << lane) - 1))] = (uint32_t)i;
    __syncthreads();
    uint32_t tc = total;
    for (uint32_t e = 0; e < tc; ++e) {  // members in sample order
      const float* row = rows + (uint64_t)members[e] * ld;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        uint32_t j = threadIdx.x + u * blockDim.x;
        if (j < dim) acc[u] += row[j];
      }
    }
    cnt += tc;
    __syncthreads();
  }
  if (cnt == 0) return;
  float inv = 1.f / (float)cnt;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    uint32_t j = threadIdx.x + u * blockDim.x;
    if (j < dim) cent[(uint64_t)c * ld + j] = acc[u] * inv;
  }
}

__device__ void block_sort_keys(uint64_t* keys, uint32_t n) {  // ascending, n a power of two
  for (uint32_t k = 2; k <= n; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < (n >> 1); i += blockDim.x) {
        uint32_t lo = ((i & ~(j - 1)) << 1) | (i & (j - 1)), hi = lo | j;
        uint64_t a = keys[lo], b = keys[hi];
        if ((a > b) == ((lo & k) == 0)) {
          keys[lo] = b;
          keys[hi] = a;
        }
      }
      __syncthreads();
    }
}

// One CTA per cluster: its `mcap` members nearest the centroid, by (dist, id).
constexpr uint32_t ENT_CAND = 4096;
__global__ void __launch_bounds__(256) entries_kernel(const int32_t* __restrict__ assign,
                                                      const float* __restrict__ dist, uint64_t n, uint32_t mcap,
                                                      uint32_t* __restrict__ entries, uint32_t* __restrict__ counts) {
  __shared__ uint64_t cand[ENT_CAND];
  __shared__ uint32_t cnt;
  const uint32_t c = blockIdx.x;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (uint64_t b0 = 0; b0 < n; b0 += (uint64_t)blockDim.x * 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      uint64_t i = b0 + (uint64_t)u * blockDim.x + threadIdx.x;
      if (i < n && assign[i] == (int32_t)c) cand[atomicAdd(&cnt, 1u)] = pack_key(dist[i], (uint32_t)i);
    }
    __syncthreads();
    if (cnt > ENT_CAND - blockDim.x * 8 || b0 + (uint64_t)blockDim.x * 8 >= n) {  // keep the mcap best
      uint32_t k = cnt, p2 = next_pow2(k < 2 ? 2 : k);
      for (uint32_t i = k + threadIdx.x; i < p2; i += blockDim.x) cand[i] = ~0ULL;
      __syncthreads();
      block_sort_keys(cand, p2);
      if (threadIdx.x == 0) cnt = k < mcap ? k : mcap;
      __syncthreads();
    }
  }
  uint32_t k = cnt;
  for (uint32_t i = threadIdx.x; i < mcap; i += blockDim.x)
    entries[(uint64_t)c * mcap + i] = i < k ? (uint32_t)cand[i] : kEmpty;
  if (threadIdx.x == 0) counts[c] = k;
}

// ---------------------------------------------------------------------------------------------
// MLP kernels
// ---------------------------------------------------------------------------------------------
// Standardised BF16 inputs: out[r][j] = (q[r][j] - mean[j]) * istd[j], j < dim.
__global__ void mlp_input_kernel(const float* __restrict__ q, uint64_t nq, uint64_t qld, uint32_t dim,
                                 const uint32_t* __restrict__ rows, const float* __restrict__ mean,
                                 const float* __restrict__ istd, __nv_bfloat16* __restrict__ out) {
  uint64_t total = nq * dim;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t r = i / dim;
    uint32_t j = (uint32_t)(i - r * dim);
    uint64_t src = rows ? rows[r] : r;
    out[i] = __float2bfloat16_rn((q[src * qld + j] - mean[j]) * istd[j]);
  }
}

// C[m][n] = sum_k A[m*sam + k*sak] * B[n*sbn + k*sbk] (+ bias[n]); then optionally relu, or a
// multiply by (mask[m][n] > 0); written as FP32 (C, row stride N) and/or BF16 (Cb).  64x64 tiles,
// 16-deep k slices staged in shared memory, 4x4 outputs per thread, FP32 accumulation.
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) gemm_kernel(uint32_t M, uint32_t N, uint32_t K, const TA* __restrict__ A,
                                                   int64_t sam, int64_t sak, const TB* __restrict__ B, int64_t sbn,
                                                   int64_t sbk, const float* __restrict__ bias, int relu,
                                                   const float* __restrict__ mask, float* __restrict__ C,
                                                   __nv_bfloat16* __restrict__ Cb) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const uint32_t tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const uint32_t m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (uint32_t k0 = 0; k0 < K; k0 += 16) {
    for (uint32_t e = threadIdx.x; e < 16 * 64; e += 256) {
      uint32_t kk = e / 64, r = e % 64;
      uint32_t gm = m0 + r, gn = n0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? ld_as_float(A + (int64_t)gm * sam + (int64_t)gk * sak) : 0.f;
      Bs[kk][r] = (gn < N && gk < K) ? ld_as_float(B + (int64_t)gn * sbn + (int64_t)gk * sbk) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint32_t gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j] + (bias ? bias[gn] : 0.f);
      if (relu) v = fmaxf(v, 0.f);
      if (mask && !(mask[(uint64_t)gm * N + gn] > 0.f)) v = 0.f;
      if (C) C[(uint64_t)gm * N + gn] = v;
      if (Cb) Cb[(uint64_t)gm * N + gn] = __float2bfloat16_rn(v);
    }
  }
}

template <typename TA, typename TB>
void gemm(uint32_t M, uint32_t N, uint32_t K, const TA* A, int64_t sam, int64_t sak, const TB* B, int64_t sbn,
          int64_t sbk, const float* bias, int relu, const float* mask, float* C, __nv_bfloat16* Cb, cudaStream_t s) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  gemm_kernel<TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, B, sbn, sbk, bias, relu, mask, C, Cb);
}

// Softmax cross-entropy of both heads, one warp per row.  Cluster target: the histogram of the row's
// GT_K neighbour clusters (tc), divided by GT_K; rung target: one-hot (tr).  dlogits = (p - t) / B.
__global__ void softmax_ce_kernel(const float* __restrict__ z, uint32_t B, uint32_t O, uint32_t Cn, uint32_t R,
                                  const uint32_t* __restrict__ tc, const uint32_t* __restrict__ rows,
                                  const uint8_t* __restrict__ tr, float* __restrict__ dz,
                                  double* __restrict__ loss) {
  uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= B) return;
  const float* zr = z + (uint64_t)warp * O;
  float* dr = dz + (uint64_t)warp * O;
  uint64_t src = rows ? rows[warp] : warp;
  const uint32_t* tcr = tc + src * GT_K;
  float invB = 1.f / (float)B;
  double l = 0;
  for (int head = 0; head < 2; ++head) {
    uint32_t off = head ? Cn : 0, len = head ? R : Cn;
    float mx = -INFINITY;
    for (uint32_t j = lane; j < len; j += 32) mx = fmaxf(mx, zr[off + j]);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULLMASK, mx, o));
    float se = 0.f;
    for (uint32_t j = lane; j < len; j += 32) se += expf(zr[off + j] - mx);
    se = warp_sum(se);
    float lse = mx + logf(se);
    for (uint32_t j = lane; j < len; j += 32) {
      float t = 0.f;
      if (head) {
        t = j == tr[src] ? 1.f : 0.f;
      } else {
#pragma unroll
        for (int g = 0; g < GT_K; ++g) t += tcr[g] == j ? 1.f / GT_K : 0.f;
      }
      float p = expf(zr[off + j] - lse);
      dr[off + j] = (p - t) * invB;
      if (t > 0.f) l -= (double)t * (double)(zr[off + j] - lse);
    }
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(FULLMASK, l, o);
  if (lane == 0) atomicAdd(loss, l);
}

// out[j] = sum over rows of X[r][j] (rows in order).
__global__ void colsum_kernel(const float* __restrict__ X, uint32_t rows, uint32_t N, float* __restrict__ out) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0.f;
  for (uint32_t r = 0; r < rows; ++r) s += X[(uint64_t)r * N + j];
  out[j] = s;
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, uint64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2, __nv_bfloat16* __restrict__ wb) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    float gi = g[i];
    float a = b1 * m1[i] + (1.f - b1) * gi, b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    float v = w[i] - lr * (a * c1) / (sqrtf(b * c2) + eps);
    w[i] = v;
    wb[i] = __float2bfloat16_rn(v);
  }
}

__global__ void to_bf16_flat_kernel(const float* __restrict__ w, uint64_t n, __nv_bfloat16* __restrict__ wb) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    wb[i] = __float2bfloat16_rn(w[i]);
}

// ---------------------------------------------------------------------------------------------
// traces and prediction
// ---------------------------------------------------------------------------------------------
// Neighbour clusters of each training query: tc[q][g] = assign[gt[q][g]].
__global__ void trace_clusters_kernel(const int32_t* __restrict__ gt, uint64_t nq, const int32_t* __restrict__ assign,
                                      uint32_t* __restrict__ tc) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nq * GT_K; i += (uint64_t)gridDim.x * blockDim.x)
    tc[i] = gt[i] >= 0 ? (uint32_t)assign[gt[i]] : 0u;
}

// recall[q] = |res[q] ∩ gt[q]| / GT_K, res rows of k ids.
__global__ void recall_kernel(const int32_t* __restrict__ res, uint32_t k, const int32_t* __restrict__ gt, uint64_t nq,
                              float* __restrict__ rec) {
  uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q >= nq) return;
  uint32_t hit = 0;
  for (int g = 0; g < GT_K; ++g)
    for (uint32_t j = 0; j < k; ++j) hit += res[q * k + j] == gt[q * GT_K + g] ? 1u : 0u;
  rec[q] = (float)hit / GT_K;
}

// label[q] = the first rung whose recall reaches min(target, best over rungs).
__global__ void rung_label_kernel(const float* __restrict__ rec, uint64_t nq, uint32_t R, float target,
                                  uint8_t* __restrict__ label) {
  uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q >= nq) return;
  float best = 0.f;
  for (uint32_t r = 0; r < R; ++r) best = fmaxf(best, rec[r * nq + q]);
  float need = fminf(best, target) - 1e-6f;
  uint8_t l = (uint8_t)(R - 1);
  for (uint32_t r = 0; r < R; ++r)
    if (rec[r * nq + q] >= need) {
      l = (uint8_t)r;
      break;
    }
  label[q] = l;
}

// Per query (one warp): the E largest cluster logits (ties by index) and the rung: the argmax, or
// with coverage > 0 the first rung whose cumulative softmax probability reaches it.
__global__ void predict_kernel(const float* __restrict__ z, uint64_t nq, uint32_t O, uint32_t Cn, uint32_t R,
                               uint32_t E, float coverage, uint32_t* __restrict__ clusters,
                               uint32_t* __restrict__ rung) {
  uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  uint32_t lane = threadIdx.x & 31;
  if (q >= nq) return;
  const float* zr = z + q * O;
  uint32_t picked[64];  // picks so far (E <= 64)
  for (uint32_t e = 0; e < E; ++e) {
    float bv = -INFINITY;
    uint32_t bi = 0xffffffffu;
    for (uint32_t j = lane; j < Cn; j += 32) {
      bool used = false;
      for (uint32_t t = 0; t < e; ++t) used |= picked[t] == j;
      float v = zr[j];
      if (!used && (v > bv || (v == bv && j < bi))) {
        bv = v;
        bi = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      float ov = __shfl_xor_sync(FULLMASK, bv, o);
      uint32_t oi = __shfl_xor_sync(FULLMASK, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    picked[e] = bi;
    if (lane == 0) clusters[q * E + e] = bi;
  }
  if (lane == 0) {
    uint32_t br = 0;
    for (uint32_t r = 1; r < R; ++r)
      if (zr[Cn + r] > zr[Cn + br]) br = r;
    if (coverage > 0.f) {
      float mx = zr[Cn + br], se = 0.f;
      for (uint32_t r = 0; r < R; ++r) se += expf(zr[Cn + r] - mx);
      float cum = 0.f;
      br = R - 1;
      for (uint32_t r = 0; r < R; ++r) {
        cum += expf(zr[Cn + r] - mx) / se;
        if (cum >= coverage) {
          br = r;
          break;
        }
      }
    }
    rung[q] = br;
  }
}

// Seeds (E clusters x m entries per query) and per-query parameters from the predictions.
__global__ void assemble_kernel(const uint32_t* __restrict__ clusters, const uint32_t* __restrict__ rung, uint64_t nq,
                                uint32_t E, const uint32_t* __restrict__ entries, uint32_t mcap, uint32_t m,
                                const efg_query_params* __restrict__ ladder, uint32_t R, int bias, uint32_t k,
                                uint32_t* __restrict__ seeds, efg_query_params* __restrict__ params) {
  uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (q >= nq) return;
  for (uint32_t e = 0; e < E; ++e)
    for (uint32_t j = 0; j < m; ++j) seeds[(q * E + e) * m + j] = entries[(uint64_t)clusters[q * E + e] * mcap + j];
  int r = (int)rung[q] + bias;
  r = r < 0 ? 0 : (r >= (int)R ? (int)R - 1 : r);
  efg_query_params p = ladder[r];
  p.k = k;
  params[q] = p;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// the learned object
// ---------------------------------------------------------------------------------------------
struct efg_learned {
  efg_index* idx = nullptr;
  efg_learned_params p{};
  uint32_t Cn = 0, R = 0, H = 0, O = 0, din = 0;
  DevBuf<float> cent, mean, istd;
  DevBuf<int32_t> assign;  // per base row
  DevBuf<float> adist;
  DevBuf<uint32_t> entries, counts;
  // parameters: flat FP32 master [W1 | b1 | W2 | b2 | W3 | b3], BF16 copy, Adam moments, gradients
  uint64_t off[7] = {};
  DevBuf<float> w, g, m1, m2;
  DevBuf<__nv_bfloat16> wb;
  uint64_t adam_t = 0;
  // traces
  DevBuf<uint32_t> tclusters;
  DevBuf<uint8_t> tlabel;
  uint64_t ntrain = 0;
  DevBuf<float> trainq;  // standardisation happens per batch from these rows
  // scratch
  DevBuf<__nv_bfloat16> xb, h1b, h2b;
  DevBuf<float> h1, h2, z, dz, dh2, dh1;
  DevBuf<double> loss;
  DevBuf<uint32_t> pred_c, pred_r, seeds, batch_rows;
  DevBuf<int> gerr;  // set by a tensor-core layer whose wait ran out (checked after training)
  DevBuf<efg_query_params> qp, ladder;
  efg_learned_stats stats{};
};

namespace {

uint64_t nparams(uint32_t H, uint32_t din, uint32_t O) {
  return (uint64_t)H * din + H + (uint64_t)H * H + H + (uint64_t)O * H + O;
}

int reserve_batch(efg_learned* L, uint64_t B) {
  EFG_TRY(L->xb.reserve(B * L->din));
  EFG_TRY(L->h1b.reserve(B * L->H));
  EFG_TRY(L->h2b.reserve(B * L->H));
  EFG_TRY(L->h1.reserve(B * L->H));
  EFG_TRY(L->h2.reserve(B * L->H));
  EFG_TRY(L->z.reserve(B * L->O));
  EFG_TRY(L->dz.reserve(B * L->O));
  EFG_TRY(L->dh2.reserve(B * L->H));
  EFG_TRY(L->dh1.reserve(B * L->H));
  return EFG_OK;
}

// One dense layer, act(A W^T + bias): on the tensor cores where the shape allows (64 <= K <= 256,
// K a multiple of 8), else the CUDA-core GEMM.
int dense(efg_learned* L, uint32_t M, uint32_t N, uint32_t K, const __nv_bfloat16* A, const __nv_bfloat16* W,
          const float* bias, int relu, float* C, __nv_bfloat16* Cb, cudaStream_t s) {
  int rc = tc_gemm_bf16(M, N, K, A, W, bias, relu, C, Cb, L->gerr.p, s);
  if (rc == EFG_OK) return EFG_OK;
  if (rc != EFG_ERR_ARG) return rc;
  gemm(M, N, K, A, K, 1, W, K, 1, bias, relu, (const float*)nullptr, C, Cb, s);
  return EFG_OK;
}

// Forward pass of B standardised rows already in L->xb: h1, h2 (FP32 and BF16) and logits z.
int forward(efg_learned* L, uint32_t B, cudaStream_t s) {
  const uint32_t H = L->H, din = L->din, O = L->O;
  const __nv_bfloat16* W1 = L->wb.p + L->off[0];
  const __nv_bfloat16* W2 = L->wb.p + L->off[2];
  const __nv_bfloat16* W3 = L->wb.p + L->off[4];
  EFG_TRY(dense(L, B, H, din, L->xb.p, W1, L->w.p + L->off[1], 1, L->h1.p, L->h1b.p, s));
  EFG_TRY(dense(L, B, H, H, L->h1b.p, W2, L->w.p + L->off[3], 1, L->h2.p, L->h2b.p, s));
  return dense(L, B, O, H, L->h2b.p, W3, L->w.p + L->off[5], 0, L->z.p, nullptr, s);
}

// Loss and gradients (into L->g) for B rows whose inputs are in L->xb and targets are trace rows
// `rows` (or 0..B-1 when rows is null).
int loss_and_grad(efg_learned* L, uint32_t B, const uint32_t* rows, cudaStream_t s, double* loss_out) {
  const uint32_t H = L->H, din = L->din, O = L->O;
  EFG_TRY(forward(L, B, s));
  EFG_CUDA(cudaMemsetAsync(L->loss.p, 0, sizeof(double), s));
  softmax_ce_kernel<<<(B * 32 + 255) / 256, 256, 0, s>>>(L->z.p, B, O, L->Cn, L->R, L->tclusters.p, rows,
                                                        L->tlabel.p, L->dz.p, L->loss.p);
  float* g = L->g.p;
  const __nv_bfloat16* W2 = L->wb.p + L->off[2];
  const __nv_bfloat16* W3 = L->wb.p + L->off[4];
  // dW3 = dz^T h2, db3 = colsum(dz), dh2 = (dz W3) * (h2 > 0)
  gemm(O, H, B, L->dz.p, 1, O, L->h2b.p, 1, H, (const float*)nullptr, 0, (const float*)nullptr, g + L->off[4],
       (__nv_bfloat16*)nullptr, s);
  colsum_kernel<<<(O + 255) / 256, 256, 0, s>>>(L->dz.p, B, O, g + L->off[5]);
  gemm(B, H, O, L->dz.p, O, 1, W3, 1, H, (const float*)nullptr, 0, L->h2.p, L->dh2.p, (__nv_bfloat16*)nullptr, s);
  // dW2 = dh2^T h1, db2, dh1 = (dh2 W2) * (h1 > 0)
  gemm(H, H, B, L->dh2.p, 1, H, L->h1b.p, 1, H, (const float*)nullptr, 0, (const float*)nullptr, g + L->off[2],
       (__nv_bfloat16*)nullptr, s);
  colsum_kernel<<<(H + 255) / 256, 256, 0, s>>>(L->dh2.p, B, H, g + L->off[3]);
  gemm(B, H, H, L->dh2.p, H, 1, W2, 1, H, (const float*)nullptr, 0, L->h1.p, L->dh1.p, (__nv_bfloat16*)nullptr, s);
  // dW1 = dh1^T x, db1
  gemm(H, din, B, L->dh1.p, 1, H, L->xb.p, 1, din, (const float*)nullptr, 0, (const float*)nullptr, g + L->off[0],
       (__nv_bfloat16*)nullptr, s);
  colsum_kernel<<<(H + 255) / 256, 256, 0, s>>>(L->dh1.p, B, H, g + L->off[1]);
  EFG_CUDA(cudaGetLastError());
  if (loss_out) {
    EFG_CUDA(cudaMemcpyAsync(loss_out, L->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    EFG_CUDA(cudaStreamSynchronize(s));
    *loss_out /= (double)B;
  }
  return EFG_OK;
}

int refresh_bf16(efg_learned* L, cudaStream_t s) {
  uint64_t n = nparams(L->H, L->din, L->O);
  to_bf16_flat_kernel<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(L->w.p, n, L->wb.p);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

// Deterministic uniform initialisation U(-a, a), a = sqrt(6 / (fan_in + fan_out)) per layer; biases 0.
void init_weights(efg_learned* L, std::vector<float>& w) {
  uint64_t n = nparams(L->H, L->din, L->O);
  w.assign(n, 0.f);
  const uint32_t fin[3] = {L->din, L->H, L->H}, fout[3] = {L->H, L->H, L->O};
  for (int layer = 0; layer < 3; ++layer) {
    uint64_t o = L->off[2 * layer], cnt = (uint64_t)fin[layer] * fout[layer];
    double a = std::sqrt(6.0 / (fin[layer] + fout[layer]));
    for (uint64_t i = 0; i < cnt; ++i) {
      uint64_t h = mix64(L->p.seed ^ (0x5eedULL + layer) * 0x9E3779B97F4A7C15ULL ^ (i * 0xD1B54A32D192ED03ULL));
      double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);
      w[o + i] = (float)((2.0 * u - 1.0) * a);
    }
  }
}

}  // namespace

void efg_learned_default_params(efg_learned_params* p) {
  if (!p) return;
  *p = efg_learned_params{};
  p->clusters = 1024;
  p->kmeans_iters = 10;
  p->kmeans_sample = 100000;
  p->entries_per_cluster = 16;
  p->entry_clusters = 8;
  p->hidden = 256;
  p->rungs = 7;
  const int lad[7][3] = {{4, 600, 60}, {6, 1200, 120}, {6, 2000, 200}, {8, 3000, 300},
                         {8, 4000, 400}, {8, 6000, 600}, {10, 9000, 900}};
  for (int r = 0; r < 7; ++r) p->rung[r] = efg_query_params{lad[r][0], lad[r][1], lad[r][2], 10};
  p->target = 0.9f;
  p->train_epochs = 8;
  p->batch = 1024;
  p->lr = 1e-3f;
  p->seed = 1998;
}

int efg_learned_create(efg_index* idx, const efg_learned_params* params, efg_learned** out) {
  if (!idx || !out) return fail(EFG_ERR_ARG, "null argument");
  *out = nullptr;
  efg_learned_params p;
  if (params) p = *params;
  else efg_learned_default_params(&p);
  if (p.clusters < 2 || p.clusters > 65536 || p.clusters > idx->n) return fail(EFG_ERR_ARG, "clusters must be in [2, min(n, 65536)]");
  if (p.rungs < 1 || p.rungs > EFG_LEARNED_MAX_RUNGS) return fail(EFG_ERR_ARG, "rungs must be in [1, 16]");
  if (p.entry_clusters > 64 || p.entry_clusters > p.clusters) return fail(EFG_ERR_ARG, "entry_clusters must be <= min(64, clusters)");
  if (p.entries_per_cluster > 1024) return fail(EFG_ERR_ARG, "entries_per_cluster must be <= 1024");
  if (p.hidden < 8 || p.hidden > 4096) return fail(EFG_ERR_ARG, "hidden must be in [8, 4096]");
  if (idx->dim > 4 * 256) return fail(EFG_ERR_ARG, "the k-means update handles at most 1024 dimensions");
  for (uint32_t r = 0; r < p.rungs; ++r)
    if (p.rung[r].init_num <= 0 || (uint64_t)p.rung[r].init_num > idx->n || p.rung[r].epochs < 0 ||
        p.rung[r].extend_to < 0)
      return fail(EFG_ERR_ARG, "invalid rung settings");
  uint64_t S = std::min<uint64_t>(std::max<uint64_t>(p.kmeans_sample, p.clusters), idx->n);
  efg_learned* L = new efg_learned();
  L->idx = idx;
  L->p = p;
  L->Cn = p.clusters;
  L->R = p.rungs;
  L->H = p.hidden;
  L->O = L->Cn + L->R;
  L->din = idx->dim;
  const uint32_t ld = idx->ld, dim = idx->dim;
  cudaStream_t s = idx->stream;
  int rc = EFG_OK;
  auto bail = [&](int code) {
    cudaStreamSynchronize(s);
    efg_learned_destroy(L);
    return code;
  };
  // 1. sample (a Feistel permutation of the base, seeded) and k-means
  std::vector<uint32_t> rows(S);
  for (uint64_t i = 0; i < S; ++i) rows[i] = feistel_perm((uint32_t)i, (uint32_t)idx->n, p.seed ^ 0x6b6d65616e73ULL);
  LocalBuf<uint32_t> drows;
  LocalBuf<float> sample;
  LocalBuf<int32_t> sassign;
  LocalBuf<float> sdist;
  if ((rc = drows.reserve(S)) || (rc = sample.reserve(S * ld)) || (rc = sassign.reserve(S)) ||
      (rc = sdist.reserve(S)) || (rc = L->cent.reserve((uint64_t)L->Cn * ld)) || (rc = L->mean.reserve(ld)) ||
      (rc = L->istd.reserve(ld)))
    return bail(rc);
  cudaMemcpy(drows.p, rows.data(), S * 4, cudaMemcpyHostToDevice);
  gather_rows_kernel<<<1024, 256, 0, s>>>(idx->d_base, ld, drows.p, S, sample.p);
  norm_stats_kernel<<<(ld + 127) / 128, 128, 0, s>>>(sample.p, S, dim, ld, L->mean.p, L->istd.p);
  cudaMemcpyAsync(L->cent.p, sample.p, (uint64_t)L->Cn * ld * 4, cudaMemcpyDeviceToDevice, s);  // first C of the sample
  for (uint32_t it = 0; it < p.kmeans_iters; ++it) {
    if ((rc = brute_force_knn(L->cent.p, L->Cn, dim, ld, sample.p, S, ld, 1, 0, 0, sassign.p, sdist.p, s)))
      return bail(rc);
    kmeans_update_kernel<<<L->Cn, 256, 256 * 4, s>>>(sample.p, S, sassign.p, dim, ld, L->cent.p);
  }
  // 2. every base row to its centroid; entry members per cluster
  if ((rc = L->assign.reserve(idx->n)) || (rc = L->adist.reserve(idx->n)) ||
      (rc = L->entries.reserve((uint64_t)L->Cn * std::max<uint32_t>(p.entries_per_cluster, 1))) ||
      (rc = L->counts.reserve(L->Cn)))
    return bail(rc);
  for (uint64_t r0 = 0; r0 < idx->n; r0 += 1u << 20) {
    uint64_t m = std::min<uint64_t>(idx->n - r0, 1u << 20);
    if ((rc = brute_force_knn(L->cent.p, L->Cn, dim, ld, idx->d_base + r0 * ld, m, ld, 1, 0, 0, L->assign.p + r0,
                              L->adist.p + r0, s)))
      return bail(rc);
  }
  if (p.entries_per_cluster)
    entries_kernel<<<L->Cn, 256, 0, s>>>(L->assign.p, L->adist.p, idx->n, p.entries_per_cluster, L->entries.p,
                                         L->counts.p);
  // 3. the network
  uint64_t np = nparams(L->H, L->din, L->O);
  L->off[0] = 0;
  L->off[1] = L->off[0] + (uint64_t)L->H * L->din;
  L->off[2] = L->off[1] + L->H;
  L->off[3] = L->off[2] + (uint64_t)L->H * L->H;
  L->off[4] = L->off[3] + L->H;
  L->off[5] = L->off[4] + (uint64_t)L->O * L->H;
  L->off[6] = L->off[5] + L->O;
  std::vector<float> w;
  init_weights(L, w);
  if ((rc = L->w.reserve(np)) || (rc = L->g.reserve(np)) || (rc = L->m1.reserve(np)) || (rc = L->m2.reserve(np)) ||
      (rc = L->wb.reserve(np)) || (rc = L->loss.reserve(1)) || (rc = L->ladder.reserve(L->R)) ||
      (rc = L->gerr.reserve(1)))
    return bail(rc);
  cudaMemsetAsync(L->gerr.p, 0, sizeof(int), s);
  cudaMemcpyAsync(L->w.p, w.data(), np * 4, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(L->m1.p, 0, np * 4, s);
  cudaMemsetAsync(L->m2.p, 0, np * 4, s);
  cudaMemcpyAsync(L->ladder.p, p.rung, L->R * sizeof(efg_query_params), cudaMemcpyHostToDevice, s);
  if ((rc = refresh_bf16(L, s))) return bail(rc);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return bail(fail(EFG_ERR_CUDA, std::string("learned build: ") + cudaGetErrorString(e)));
  e = cudaGetLastError();
  if (e != cudaSuccess) return bail(fail(EFG_ERR_CUDA, std::string("learned build: ") + cudaGetErrorString(e)));
  *out = L;
  return EFG_OK;
}

void efg_learned_destroy(efg_learned* L) {
  if (!L) return;
  if (L->idx && L->idx->stream) cudaStreamSynchronize(L->idx->stream);
  L->cent.release(); L->mean.release(); L->istd.release(); L->assign.release(); L->adist.release();
  L->entries.release(); L->counts.release(); L->w.release(); L->g.release(); L->m1.release(); L->m2.release();
  L->wb.release(); L->tclusters.release(); L->tlabel.release(); L->trainq.release(); L->xb.release();
  L->h1b.release(); L->h2b.release(); L->h1.release(); L->h2.release(); L->z.release(); L->dz.release();
  L->dh2.release(); L->dh1.release(); L->loss.release(); L->pred_c.release(); L->pred_r.release();
  L->seeds.release(); L->batch_rows.release(); L->qp.release(); L->ladder.release();
  delete L;
}

int efg_learned_train(efg_learned* L, const float* d_q, uint64_t n, uint64_t row_stride) {
  if (!L || (!d_q && n)) return fail(EFG_ERR_ARG, "null argument");
  efg_index* idx = L->idx;
  if (row_stride < idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (n == 0) return fail(EFG_ERR_ARG, "no training queries");
  if (n > 0xffffffffull) return fail(EFG_ERR_ARG, "at most 2^32 - 1 training queries");
  cudaStream_t s = idx->stream;
  const uint32_t ld = idx->ld, dim = idx->dim, R = L->R;
  // the queries, padded to the index's row stride
  EFG_TRY(L->trainq.reserve(n * ld));
  EFG_CUDA(cudaMemsetAsync(L->trainq.p, 0, n * ld * 4, s));
  EFG_CUDA(cudaMemcpy2DAsync(L->trainq.p, ld * 4, d_q, row_stride * 4, dim * 4, n, cudaMemcpyDeviceToDevice, s));
  // traces: exact neighbours, their clusters, recall per rung, labels
  LocalBuf<int32_t> gt, res;
  LocalBuf<float> gtd, rec;
  EFG_TRY(gt.reserve(n * GT_K));
  EFG_TRY(gtd.reserve(n * GT_K));
  EFG_TRY(rec.reserve(n * R));
  EFG_TRY(res.reserve(n * 10));
  EFG_TRY(L->tclusters.reserve(n * GT_K));
  EFG_TRY(L->tlabel.reserve(n));
  L->ntrain = n;
  if (L->p.trace_reference.init_num > 0) {  // the plain search at a high setting stands in for the exact 10-NN
    efg_query_params ref = L->p.trace_reference;
    ref.k = GT_K;
    EFG_TRY(search_device_ex(idx, L->trainq.p, n, ld, ref, nullptr, nullptr, gt.p, s, false));
  } else {
    for (uint64_t q0 = 0; q0 < n; q0 += 65536) {
      uint64_t m = std::min<uint64_t>(n - q0, 65536);
      EFG_TRY(exact_knn(idx->d_base, idx->n, dim, ld, L->trainq.p + q0 * ld, m, ld, GT_K, 0, 0, gt.p + q0 * GT_K,
                        gtd.p + q0 * GT_K, s));
    }
  }
  trace_clusters_kernel<<<1024, 256, 0, s>>>(gt.p, n, L->assign.p, L->tclusters.p);
  for (uint32_t r = 0; r < R; ++r) {
    efg_query_params lim = L->p.rung[r];
    lim.k = 10;
    EFG_TRY(search_device_ex(idx, L->trainq.p, n, ld, lim, nullptr, nullptr, res.p, s, false));
    recall_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(res.p, 10, gt.p, n, rec.p + (uint64_t)r * n);
  }
  rung_label_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rec.p, n, R, L->p.target, L->tlabel.p);
  std::vector<float> hrec(n * R);
  EFG_CUDA(cudaMemcpyAsync(hrec.data(), rec.p, n * R * 4, cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  for (uint32_t r = 0; r < R && r < EFG_LEARNED_MAX_RUNGS; ++r) {
    double a = 0;
    for (uint64_t q = 0; q < n; ++q) a += hrec[r * n + q];
    L->stats.rung_recall[r] = (float)(a / n);
  }
  // training: shuffled mini-batches (a Feistel permutation per pass), Adam
  const uint32_t B = (uint32_t)std::min<uint64_t>(L->p.batch ? L->p.batch : 1024, n);
  EFG_TRY(reserve_batch(L, B));
  EFG_TRY(L->batch_rows.reserve(B));
  std::vector<uint32_t> hb(B);
  const uint64_t np = nparams(L->H, L->din, L->O);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  L->stats.train_loss_first = L->stats.train_loss_last = 0;
  for (uint32_t ep = 0; ep < L->p.train_epochs; ++ep) {
    double lsum = 0;
    uint64_t nb = 0;
    for (uint64_t b0 = 0; b0 + B <= n; b0 += B) {
      for (uint32_t i = 0; i < B; ++i)
        hb[i] = feistel_perm((uint32_t)(b0 + i), (uint32_t)n, L->p.seed * 0x9E3779B97F4A7C15ULL + ep);
      EFG_CUDA(cudaMemcpyAsync(L->batch_rows.p, hb.data(), B * 4, cudaMemcpyHostToDevice, s));
      mlp_input_kernel<<<512, 256, 0, s>>>(L->trainq.p, B, ld, dim, L->batch_rows.p, L->mean.p, L->istd.p, L->xb.p);
      double l = 0;
      EFG_TRY(loss_and_grad(L, B, L->batch_rows.p, s, &l));
      ++L->adam_t;
      float c1 = 1.f / (1.f - std::pow(b1, (float)L->adam_t)), c2 = 1.f / (1.f - std::pow(b2, (float)L->adam_t));
      adam_kernel<<<(unsigned)std::min<uint64_t>((np + 255) / 256, 4096), 256, 0, s>>>(
          L->w.p, L->g.p, L->m1.p, L->m2.p, np, L->p.lr, b1, b2, eps, c1, c2, L->wb.p);
      EFG_CUDA(cudaGetLastError());
      lsum += l;
      ++nb;
    }
    double mean_loss = nb ? lsum / nb : 0;
    if (ep == 0) L->stats.train_loss_first = (float)mean_loss;
    L->stats.train_loss_last = (float)mean_loss;
  }
  L->stats.train_queries = n;
  int gerr = 0;
  EFG_CUDA(cudaMemcpyAsync(&gerr, L->gerr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  EFG_CUDA(cudaStreamSynchronize(s));
  if (gerr) return fail(EFG_ERR_DEVICE_LIMIT, "a tensor-core layer's pipeline wait ran out");
  return EFG_OK;
}

int efg_learned_predict_device(efg_learned* L, const float* d_q, uint64_t nq, uint64_t row_stride,
                               float coverage, uint32_t* d_clusters, uint32_t* d_rung, void* stream) {
  if (!L || ((!d_q || !d_rung || (!d_clusters && L->p.entry_clusters)) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (row_stride < L->idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t B = 32768;  // queries per pass through the network
  EFG_TRY(reserve_batch(L, B));
  for (uint64_t q0 = 0; q0 < nq; q0 += B) {
    uint32_t m = (uint32_t)std::min<uint64_t>(nq - q0, B);
    mlp_input_kernel<<<512, 256, 0, s>>>(d_q + q0 * row_stride, m, row_stride, L->din, nullptr, L->mean.p, L->istd.p,
                                         L->xb.p);
    EFG_TRY(forward(L, m, s));
    predict_kernel<<<(m * 32 + 255) / 256, 256, 0, s>>>(L->z.p, m, L->O, L->Cn, L->R, L->p.entry_clusters,
                                                        coverage, d_clusters ? d_clusters + q0 * L->p.entry_clusters : nullptr,
                                                        d_rung + q0);
    EFG_CUDA(cudaGetLastError());
  }
  return EFG_OK;
}

int efg_learned_search_device(efg_learned* L, const float* d_q, uint64_t nq, uint64_t row_stride, uint32_t k,
                              float coverage, int rung_bias, int32_t* d_out, void* stream) {
  if (!L || ((!d_q || !d_out) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (nq == 0) return EFG_OK;
  efg_index* idx = L->idx;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t E = L->p.entry_clusters, m = L->p.entries_per_cluster;
  efg_query_params lim{0, 1, 0, k};
  for (uint32_t r = 0; r < L->R; ++r) {
    lim.epochs = std::max(lim.epochs, L->p.rung[r].epochs);
    lim.init_num = std::max(lim.init_num, L->p.rung[r].init_num);
    lim.extend_to = std::max(lim.extend_to, std::min(L->p.rung[r].extend_to, L->p.rung[r].init_num));
  }
  if ((int)k > lim.init_num) return fail(EFG_ERR_ARG, "k above the largest pool of the ladder");
  EFG_TRY(L->pred_c.reserve(std::max<uint64_t>(nq * E, 1)));
  EFG_TRY(L->pred_r.reserve(nq));
  EFG_TRY(L->seeds.reserve(std::max<uint64_t>(nq * E * m, 1)));
  EFG_TRY(L->qp.reserve(nq));
  EFG_TRY(efg_learned_predict_device(L, d_q, nq, row_stride, coverage, E ? L->pred_c.p : nullptr, L->pred_r.p, s));
  assemble_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(L->pred_c.p, L->pred_r.p, nq, E, L->entries.p,
                                                              std::max<uint32_t>(m, 1), m, L->ladder.p, L->R,
                                                              rung_bias, k, L->seeds.p, L->qp.p);
  EFG_CUDA(cudaGetLastError());
  return search_device_ex(idx, d_q, nq, row_stride, lim, L->qp.p, nullptr, d_out, s, false,
                          (E && m) ? L->seeds.p : nullptr, E * m);
}

int efg_learned_get_stats(const efg_learned* L, efg_learned_stats* out) {
  if (!L || !out) return fail(EFG_ERR_ARG, "null argument");
  *out = L->stats;
  return EFG_OK;
}

uint64_t efg_learned_num_params(const efg_learned* L) { return L ? nparams(L->H, L->din, L->O) : 0; }

int efg_learned_get_weights(efg_learned* L, float* host) {
  if (!L || !host) return fail(EFG_ERR_ARG, "null argument");
  EFG_CUDA(cudaStreamSynchronize(L->idx->stream));
  EFG_CUDA(cudaMemcpy(host, L->w.p, nparams(L->H, L->din, L->O) * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

int efg_learned_set_weights(efg_learned* L, const float* host) {
  if (!L || !host) return fail(EFG_ERR_ARG, "null argument");
  EFG_CUDA(cudaStreamSynchronize(L->idx->stream));
  EFG_CUDA(cudaMemcpy(L->w.p, host, nparams(L->H, L->din, L->O) * 4, cudaMemcpyHostToDevice));
  EFG_TRY(refresh_bf16(L, L->idx->stream));
  EFG_CUDA(cudaStreamSynchronize(L->idx->stream));
  return EFG_OK;
}

int efg_learned_get_norm(efg_learned* L, float* mean, float* istd) {
  if (!L || !mean || !istd) return fail(EFG_ERR_ARG, "null argument");
  EFG_CUDA(cudaStreamSynchronize(L->idx->stream));
  EFG_CUDA(cudaMemcpy(mean, L->mean.p, L->idx->dim * 4, cudaMemcpyDeviceToHost));
  EFG_CUDA(cudaMemcpy(istd, L->istd.p, L->idx->dim * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

int efg_learned_grad(efg_learned* L, const float* d_x, uint32_t B, uint64_t row_stride, const uint32_t* d_tclusters,
                     const uint8_t* d_tlabel, double* loss, float* host_grad) {
  if (!L || !d_x || !d_tclusters || !d_tlabel || !host_grad || B == 0) return fail(EFG_ERR_ARG, "null argument");
  cudaStream_t s = L->idx->stream;
  EFG_TRY(reserve_batch(L, B));
  // targets for rows 0..B-1 taken from the caller's arrays
  LocalBuf<uint32_t> tc;
  LocalBuf<uint8_t> tl;
  EFG_TRY(tc.reserve((uint64_t)B * GT_K));
  EFG_TRY(tl.reserve(B));
  EFG_CUDA(cudaMemcpyAsync(tc.p, d_tclusters, (uint64_t)B * GT_K * 4, cudaMemcpyDeviceToDevice, s));
  EFG_CUDA(cudaMemcpyAsync(tl.p, d_tlabel, B, cudaMemcpyDeviceToDevice, s));
  std::swap(L->tclusters.p, tc.p);
  std::swap(L->tclusters.cap, tc.cap);
  std::swap(L->tlabel.p, tl.p);
  std::swap(L->tlabel.cap, tl.cap);
  mlp_input_kernel<<<512, 256, 0, s>>>(d_x, B, row_stride, L->din, nullptr, L->mean.p, L->istd.p, L->xb.p);
  int rc = loss_and_grad(L, B, nullptr, s, loss);
  std::swap(L->tclusters.p, tc.p);
  std::swap(L->tclusters.cap, tc.cap);
  std::swap(L->tlabel.p, tl.p);
  std::swap(L->tlabel.cap, tl.cap);
  EFG_TRY(rc);
  EFG_CUDA(cudaMemcpy(host_grad, L->g.p, nparams(L->H, L->din, L->O) * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}

int efg_learned_clusters(efg_learned* L, int32_t* host_assign, uint32_t* host_entries, uint32_t* host_counts) {
  if (!L) return fail(EFG_ERR_ARG, "null argument");
  EFG_CUDA(cudaStreamSynchronize(L->idx->stream));
  if (host_assign) EFG_CUDA(cudaMemcpy(host_assign, L->assign.p, L->idx->n * 4, cudaMemcpyDeviceToHost));
  uint32_t m = std::max<uint32_t>(L->p.entries_per_cluster, 1);
  if (host_entries && L->p.entries_per_cluster)
    EFG_CUDA(cudaMemcpy(host_entries, L->entries.p, (uint64_t)L->Cn * m * 4, cudaMemcpyDeviceToHost));
  if (host_counts && L->p.entries_per_cluster)
    EFG_CUDA(cudaMemcpy(host_counts, L->counts.p, L->Cn * 4, cudaMemcpyDeviceToHost));
  return EFG_OK;
}
