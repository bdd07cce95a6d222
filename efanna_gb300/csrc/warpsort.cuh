// Warp-level sorting networks over one element per lane (bitonic), used to pull the next 32
// smallest records of a bucket in order and to keep a running sorted top-32.
#pragma once
#include "common.cuh"

namespace efg {

// 96-bit record key: (dist bits << 32 | id, aux) compared lexicographically.
struct K96 {
  uint64_t k;
  uint32_t a;
};
__device__ __forceinline__ bool lt(const K96& x, const K96& y) { return x.k < y.k || (x.k == y.k && x.a < y.a); }
__device__ __forceinline__ bool lt(uint64_t x, uint64_t y) { return x < y; }
__device__ __forceinline__ K96 shfl_xor(const K96& x, int m) {
  K96 r;
  r.k = __shfl_xor_sync(0xffffffffu, x.k, m);
  r.a = __shfl_xor_sync(0xffffffffu, x.a, m);
  return r;
}
__device__ __forceinline__ uint64_t shfl_xor(uint64_t x, int m) { return __shfl_xor_sync(0xffffffffu, x, m); }
__device__ __forceinline__ K96 shfl_idx(const K96& x, int src) {
  K96 r;
  r.k = __shfl_sync(0xffffffffu, x.k, src);
  r.a = __shfl_sync(0xffffffffu, x.a, src);
  return r;
}
__device__ __forceinline__ uint64_t shfl_idx(uint64_t x, int src) { return __shfl_sync(0xffffffffu, x, src); }
__device__ __forceinline__ K96 k96_max() { return K96{~0ULL, 0xffffffffu}; }
__device__ __forceinline__ bool is_max(const K96& x) { return x.k == ~0ULL && x.a == 0xffffffffu; }
__device__ __forceinline__ bool is_max(uint64_t x) { return x == ~0ULL; }

// Ascending bitonic sort of 32 elements, element i on lane i.
template <typename T>
__device__ __forceinline__ T warp_sort32(T x) {
  const uint32_t lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      T y = shfl_xor(x, j);
      bool asc = (lane & k) == 0;
      bool lower = (lane & j) == 0;
      bool take_min = lower == asc;
      bool ylt = lt(y, x);
      x = (take_min == ylt) ? y : x;
    }
  }
  return x;
}

// t and x ascending across lanes -> the 32 smallest of both, ascending.
template <typename T>
__device__ __forceinline__ T warp_merge_min32(T t, T x) {
  const uint32_t lane = threadIdx.x & 31;
  T xr = shfl_idx(x, 31 - lane);
  T m = lt(xr, t) ? xr : t;
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    T y = shfl_xor(m, j);
    bool lower = (lane & j) == 0;
    bool ylt = lt(y, m);
    m = (lower == ylt) ? y : m;
  }
  return m;
}

}  // namespace efg
