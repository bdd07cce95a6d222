// The learned form's network layers on the tensor cores: C = act(A W^T + bias) with A an M x K BF16
// activation matrix and W the N x K BF16 weight matrix (both row-major, so both operands are
// K-major), FP32 accumulation in TMEM, written as FP32 and/or BF16.  One CTA per 128 x 256 output
// tile: warp 0 loads every k-block of the tile with TMA (K <= 256: at most four 64-value blocks,
// one stage each, so nothing waits for a stage to free), one thread of warp 1 issues the MMAs
// (M = 128, N = 256, K = 16 each) and commits them, warps 2-5 read the accumulator back with
// tcgen05.ld (one output row per thread), add the bias, apply the ReLU and store 32-column slices
// through a per-warp shared-memory transpose so that global stores run along rows.  Waits are
// bounded as in the k-NN kernel: one that runs out sets an error word and the CTA leaves.
#include "tcgen05.cuh"

namespace efg {
namespace {

using namespace tc;

constexpr uint32_t GM = 128;  // output rows per tile (MMA M, TMEM lanes)
constexpr uint32_t GN = 256;  // output columns per tile (MMA N, TMEM columns)
constexpr uint32_t GKB = 64;  // BF16 values per k-block
constexpr uint32_t MAX_KB = 4;
constexpr uint32_t A_BYTES = GM * GKB * 2;  // 16 KiB
constexpr uint32_t B_BYTES = GN * GKB * 2;  // 32 KiB
constexpr uint32_t STAGE = A_BYTES + B_BYTES;
constexpr uint32_t GIDESC = idesc_bf16(GM, GN);
constexpr uint32_t GTHREADS = 192;

struct GemmArgs {
  uint32_t M, N, kblocks, relu;
  const float* bias;  // N entries or null
  float* C;           // M x N FP32 or null
  __nv_bfloat16* Cb;  // M x N BF16 or null
  int* err;
};

__global__ void __launch_bounds__(GTHREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mw, const GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[MAX_KB], bar_tfull, bar_drain;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;
  const uint32_t raw = smem_addr(smem_raw);
  const uint32_t pad = ((raw + 1023u) & ~1023u) - raw;
  const uint32_t sbase = raw + pad;
  float* xpose = reinterpret_cast<float*>(smem_raw + pad + MAX_KB * STAGE);  // 4 warps x 32 x 33 floats
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t m0 = blockIdx.x * GM, n0 = blockIdx.y * GN;

  if (threadIdx.x == 0) {
    for (uint32_t kb = 0; kb < g.kblocks; ++kb) mbar_init(smem_addr(&bar_full[kb]), 1);
    mbar_init(smem_addr(&bar_tfull), 1);
    mbar_init(smem_addr(&bar_drain), 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_sh)),
                 "r"(GN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;
  volatile int* abort_flag = &abort_sh;
  bool mma_issued = false;

  if (warp == 0) {
    if (lane == 0) {  // every k-block in its own stage
      for (uint32_t kb = 0; kb < g.kblocks; ++kb) {
        const uint32_t fb = smem_addr(&bar_full[kb]), st = sbase + kb * STAGE;
        mbar_expect_tx(fb, STAGE);
        tma_load_2d(st, &ma, fb, (int)(kb * GKB), (int)m0);
        tma_load_2d(st + A_BYTES, &mw, fb, (int)(kb * GKB), (int)n0);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      for (uint32_t kb = 0; ok && kb < g.kblocks; ++kb) {
        if (!mbar_wait(smem_addr(&bar_full[kb]), 0, abort_flag, g.err)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t st = sbase + kb * STAGE;
        const uint64_t da = sw128_desc(st), dw = sw128_desc(st + A_BYTES);
#pragma unroll
        for (uint32_t j = 0; j < GKB / 16; ++j)
          umma_bf16(tmem, da + 2 * j, dw + 2 * j, GIDESC, (kb | j) != 0 ? 1u : 0u);
        mma_issued = true;
      }
      if (ok) umma_commit(smem_addr(&bar_tfull));
    }
  } else {
    const uint32_t quad = warp & 3u;
    float* xp = xpose + (warp - 2) * 32 * 33;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(smem_addr(&bar_tfull), 0, abort_flag, g.err));
    if (ok) {
      tc_fence_after();
      const uint32_t rbase = m0 + quad * 32;  // this warp's 32 output rows
      for (uint32_t c0 = 0; c0 < GN && n0 + c0 < g.N; c0 += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((quad * 32u) << 16) + c0;
        tmem_ld16(taddr, v);
        tmem_ld16(taddr + 16, v + 16);
        tmem_wait();
        // lane l holds row rbase + l, columns c0 .. c0 + 31: into the transpose tile
#pragma unroll
        for (uint32_t j = 0; j < 32; ++j) xp[lane * 33 + j] = __uint_as_float(v[j]);
        __syncwarp();
        // row by row: lane l writes column c0 + l
        const uint32_t col = n0 + c0 + lane;
        const float b = (g.bias && col < g.N) ? g.bias[col] : 0.f;
        for (uint32_t r = 0; r < 32; ++r) {
          const uint32_t row = rbase + r;
          if (row >= g.M || col >= g.N) continue;
          float x = xp[r * 33 + lane] + b;
          if (g.relu) x = fmaxf(x, 0.f);
          if (g.C) g.C[(uint64_t)row * g.N + col] = x;
          if (g.Cb) g.Cb[(uint64_t)row * g.N + col] = __float2bfloat16_rn(x);
        }
        __syncwarp();
      }
    }
  }

  __syncthreads();
  if (warp == 1) {
    if (lane == 0 && mma_issued) {  // the MMAs have finished before TMEM is freed
      umma_commit(smem_addr(&bar_drain));
      const unsigned long long t0 = clock64();
      while (!mbar_try_wait(smem_addr(&bar_drain), 0)) {
        if (clock64() - t0 > WAIT_CYCLES) {
          atomicOr(g.err, 2);
          break;
        }
      }
    }
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(GN) : "memory");
  }
}

}  // namespace

// C = act(A W^T + bias) on the tensor cores for 64 <= K <= 256 and K a multiple of 8 (row strides of
// 16-byte multiples); EFG_ERR_ARG when the shape does not fit (the caller then uses the CUDA-core
// GEMM), another status when a CUDA call failed.
// A: M x K BF16 rows K apart; W: N x K BF16 rows K apart; C (FP32) and Cb (BF16): M x N, either may
// be null.  err: a device word the kernel sets when a wait runs out (checked by the caller).
int tc_gemm_bf16(uint32_t M, uint32_t N, uint32_t K, const __nv_bfloat16* A, const __nv_bfloat16* W,
                 const float* bias, int relu, float* C, __nv_bfloat16* Cb, int* err, cudaStream_t s) {
  if (M == 0 || N == 0) return EFG_OK;
  if (K < GKB || K > MAX_KB * GKB || K % 8) return EFG_ERR_ARG;
  CUtensorMap ma, mw;
  if (make_map(&ma, A, M, K, GM) != EFG_OK || make_map(&mw, W, N, K, GN) != EFG_OK) return EFG_ERR_ARG;
  GemmArgs g{M, N, (K + GKB - 1) / GKB, (uint32_t)(relu ? 1 : 0), bias, C, Cb, err};
  const size_t smem = 1024 + (size_t)MAX_KB * STAGE + 4 * 32 * 33 * 4;
  EFG_CUDA(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((M + GM - 1) / GM, (N + GN - 1) / GN);
  tc_gemm_kernel<<<grid, GTHREADS, smem, s>>>(ma, mw, g);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

}  // namespace efg
