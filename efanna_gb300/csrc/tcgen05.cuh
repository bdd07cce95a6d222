// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a, in inline PTX: mbarriers,
// TMA tile loads, shared-memory matrix descriptors of the 128-byte-swizzle K-major layout,
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation in TMEM), commits and TMEM loads; and on
// the host the tensor maps of BF16 row-major matrices.  Used by the exact k-NN screening
// (gram_tc.cu) and the learned form's network layers (mlp_tc.cu).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>
#include <string>

#include "internal.cuh"

namespace efg {
namespace tc {

constexpr unsigned long long WAIT_CYCLES = 4000000000ull;  // a bounded wait: about 2 s at 2 GHz

// Instruction descriptor of tcgen05.mma.kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for the phase of `parity` to complete; false when the CTA is aborting or the wait ran out
// (which also starts the abort).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err) {
  unsigned long long t0 = clock64();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 127) == 127) {
      if (*abort_flag) return false;
      if (clock64() - t0 > WAIT_CYCLES) {
        *abort_flag = 1;
        atomicOr(err, 1);
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a 128-row block of K-major BF16 rows, 128 bytes per row, in
// the 128-byte swizzle layout TMA writes: 8-row groups 1024 bytes apart (stride byte offset),
// descriptor version 1 (bits 46-47), swizzle mode 2 = 128 bytes (bits 61-63).  The block must
// start on a 1024-byte boundary; the k-th 16-value slice starts 32 * k bytes further.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// One tcgen05.mma.kind::f16 (BF16 operands from shared memory, FP32 accumulator in TMEM) with the
// given instruction descriptor; accumulate = 0 overwrites the accumulator.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 lanes x 16 consecutive FP32 columns: thread i of the warp receives the 16 values of TMEM lane
// (lane base + i) from the address's column on.  Asynchronous until tmem_wait().
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// Waits for every tcgen05.ld this thread issued.
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// FP32 rows -> BF16 hi (and lo = x - hi) rows of W values (zero padded), FP32 squared norms (+inf
// for the padding rows up to norm_rows), and a flag set when some lo is not zero.  A warp per row.
static __global__ void to_bf16_kernel(const float* __restrict__ src, uint64_t rows, uint32_t dim, uint64_t ld, uint32_t W,
                               __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                               float* __restrict__ norms, uint64_t norm_rows, int* __restrict__ inexact) {
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t r = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < norm_rows; r += nw) {
    if (r >= rows) {
      if (lane == 0) norms[r] = INFINITY;
      continue;
    }
    float acc = 0.f;
    bool any_lo = false;
    for (uint32_t c = lane; c < W; c += 32) {
      const float x = c < dim ? src[r * ld + c] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
      hi[r * W + c] = h;
      lo[r * W + c] = l;
      any_lo |= __bfloat162float(l) != 0.f;
      acc = fmaf(x, x, acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) norms[r] = acc;
    if (__any_sync(0xffffffffu, any_lo) && lane == 0) atomicOr(inexact, 1);
  }
}

// cuTensorMapEncodeTiled from the driver, found once through the runtime (no link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// Tensor map of `rows` BF16 rows of W values (W x 2 bytes a multiple of 16): boxes of 64 values x
// box_rows rows, 128-byte swizzle; rows and columns past the end read as zeros.
inline int make_map(CUtensorMap* m, const __nv_bfloat16* p, uint64_t rows, uint32_t W, uint32_t box_rows = 128) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(EFG_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  cuuint64_t dims[2] = {W, rows};
  cuuint64_t strides[1] = {(cuuint64_t)W * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(p), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(EFG_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return EFG_OK;
}


}  // namespace tc
}  // namespace efg
