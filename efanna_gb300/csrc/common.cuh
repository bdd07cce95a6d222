// Shared device/host helpers for the efanna_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "efanna_gb300.h"

namespace efg {

// ---- error reporting -------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

#define EFG_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return ::efg::fail(e_ == cudaErrorMemoryAllocation ? EFG_ERR_NOMEM : EFG_ERR_CUDA, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

#define EFG_TRY(expr)        \
  do {                       \
    int rc_ = (expr);        \
    if (rc_ != EFG_OK) return rc_; \
  } while (0)

// ---- counter-hash random streams ---------------------------------------------------------------
// splitmix64 finaliser and the tagged 4-word hash that every random choice of the build derives
// from; identical on host and device so that a build is a pure function of (data, params).
enum : uint64_t {
  TAG_PERM = 1, TAG_DIM = 2, TAG_EXTRA = 3, TAG_GENRAND = 4, TAG_TOPUP = 5,
  TAG_RNEW = 6, TAG_ROLD = 7, TAG_SFILL = 8
};
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t hash4(uint64_t seed, uint64_t tag, uint64_t a, uint64_t b,
                                                   uint64_t c) {
  return mix64(mix64(mix64(mix64(seed ^ (tag * 0x9E3779B97F4A7C15ULL)) ^ a) ^ b) ^ c);
}
struct CRng {
  uint64_t key, ctr;
  __host__ __device__ explicit CRng(uint64_t k) : key(k), ctr(0) {}
  __host__ __device__ uint32_t next() {
    ++ctr;
    return (uint32_t)(mix64(key ^ (ctr * 0xD1B54A32D192ED03ULL)) >> 32);
  }
};
// Balanced 4-round Feistel permutation with cycle walking: a bijection of [0, n).
__host__ __device__ inline uint32_t feistel_perm(uint32_t i, uint32_t n, uint64_t key) {
  unsigned b = 2;
  while ((1ULL << b) < (uint64_t)n) b += 2;
  unsigned half = b / 2;
  uint32_t mask = (uint32_t)((1ULL << half) - 1);
  uint32_t x = i;
  do {
    uint32_t L = x >> half, R = x & mask;
    for (uint32_t r = 0; r < 4; ++r) {
      uint32_t F = (uint32_t)mix64(key ^ ((uint64_t)r << 48) ^ R) & mask;
      uint32_t nl = R, nr = L ^ F;
      L = nl;
      R = nr;
    }
    x = (L << half) | R;
  } while (x >= n);
  return x;
}

// ---- packed (dist, id) keys --------------------------------------------------------------------
// Distances are non-negative, so their IEEE bits order like unsigned integers; (bits << 32) | id
// orders by distance then id, the order of std::pair<float, size_t> in the reference's search.
__host__ __device__ __forceinline__ uint64_t pack_key(float d, uint32_t id) {
#ifdef __CUDA_ARCH__
  return ((uint64_t)__float_as_uint(d) << 32) | id;
#else
  uint32_t b;
  memcpy(&b, &d, 4);
  return ((uint64_t)b << 32) | id;
#endif
}
__device__ __forceinline__ float key_dist(uint64_t k) { return __uint_as_float((uint32_t)(k >> 32)); }
__device__ __forceinline__ uint32_t key_id(uint64_t k) { return (uint32_t)k; }

// ---- device layout of the trees ----------------------------------------------------------------
// One 16-byte record per node, all trees concatenated.  Internal nodes: left/right are global node
// indices.  Leaves: left = -(start + 1), right = end (a range of the tree's leaf list).
struct DNode {
  int32_t div_dim;
  float div_val;
  int32_t left;
  int32_t right;
};
__device__ __forceinline__ bool dn_is_leaf(const DNode& n) { return n.left < 0; }

__host__ __device__ __forceinline__ uint64_t round_up(uint64_t x, uint64_t m) { return (x + m - 1) / m * m; }
__host__ __device__ __forceinline__ uint32_t next_pow2(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

static constexpr int kWarp = 32;
static constexpr uint32_t kEmpty = 0xFFFFFFFFu;

// ---- squared L2 of one row pair, computed by one warp ------------------------------------------
// Lane l owns float4 chunks l, l+32, ...; lanes reduce with an xor butterfly.  All 32 lanes
// return the same value.  ld4 = row stride in float4 units, dim4 = float4 chunks per row.
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums v[0..8) over the warp's 32 lanes; lane l returns the total of v[(l >> 2) & 7].  At each
// exchange a lane keeps the half of its values that its partner sends it the other half of.
__device__ __forceinline__ float reduce8_rows(const float* v, uint32_t lane) {
  const bool b4 = (lane >> 4) & 1, b3 = (lane >> 3) & 1, b2 = (lane >> 2) & 1;
  float h[4], q[2];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float keep = b4 ? v[j + 4] : v[j], send = b4 ? v[j] : v[j + 4];
    h[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float keep = b3 ? h[j + 2] : h[j], send = b3 ? h[j] : h[j + 2];
    q[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  float keep = b2 ? q[1] : q[0], send = b2 ? q[0] : q[1];
  float x = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  return x;
}

}  // namespace efg
