// Device-wide exclusive prefix sums (three-phase: block totals, scan of totals, rescan + offset).
// Used for the segmented partitions of the tree build and the bucket offsets of NN-descent.
#pragma once
#include "internal.cuh"

namespace efg {

static constexpr int SCAN_THREADS = 1024;
static constexpr int SCAN_ITEMS = 4;
static constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T x) {
  uint32_t lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  return x;
}

// Block-wide exclusive scan of one value per thread (blockDim.x == SCAN_THREADS).
template <typename T>
__device__ __forceinline__ T block_scan_excl(T v, T* total) {
  __shared__ T wsum[32];
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = warp_incl_scan(v);
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (blockDim.x >> 5) ? wsum[lane] : T(0);
    w = warp_incl_scan(w);
    wsum[lane] = w;
  }
  __syncthreads();
  T before = warp == 0 ? T(0) : wsum[warp - 1];
  *total = wsum[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

template <typename T>
__global__ void scan_tile_sums(const T* __restrict__ in, uint64_t n, T* __restrict__ sums) {
  uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
  T s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i)
    if (base + i < n) s += in[base + i];
  T tot;
  block_scan_excl(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void scan_tile_apply(const T* __restrict__ in, uint64_t n, const T* __restrict__ offs,
                                T* __restrict__ out) {
  uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
  T v[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = base + i < n ? in[base + i] : T(0);
    s += v[i];
  }
  T tot;
  T ex = block_scan_excl(s, &tot) + (offs ? offs[blockIdx.x] : T(0));
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  // out[n] = total, written by the thread owning the last element
  if (base <= n - 1 && n - 1 < base + SCAN_ITEMS) out[n] = ex;
}

// Exclusive scan of in[0..n) into out[0..n], out[n] = total.  `tmp` must hold scan_tmp_elems(n).
template <typename T>
inline uint64_t scan_tmp_elems(uint64_t n) {
  uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles <= 1) return 0;
  return 2 * tiles + 1 + scan_tmp_elems<T>(tiles);
}

template <typename T>
int device_scan(const T* in, uint64_t n, T* out, T* tmp, cudaStream_t s) {
  if (n == 0) {
    EFG_CUDA(cudaMemsetAsync(out, 0, sizeof(T), s));
    return EFG_OK;
  }
  uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    scan_tile_apply<T><<<1, SCAN_THREADS, 0, s>>>(in, n, nullptr, out);
    EFG_CUDA(cudaGetLastError());
    return EFG_OK;
  }
  T* sums = tmp;              // tiles
  T* offs = tmp + tiles;      // tiles + 1
  T* rest = offs + tiles + 1;
  scan_tile_sums<T><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, sums);
  EFG_CUDA(cudaGetLastError());
  EFG_TRY(device_scan<T>(sums, tiles, offs, rest, s));
  scan_tile_apply<T><<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, n, offs, out);
  EFG_CUDA(cudaGetLastError());
  return EFG_OK;
}

}  // namespace efg
