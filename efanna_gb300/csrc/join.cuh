// The record side of the NN-descent join (base_index.hpp:328-371), shared by the FP32 join
// kernels (nndescent.cu) and the tensor-core join (join_tc.cu): where a pair's distance lands in the
// per-node pair array, and which of its two sides becomes a pool-insert record.
#pragma once
#include "internal.cuh"

namespace efg {

// The record side of one join pair (a lane's pair): x is the list entry being joined, y the
// candidate, my_new whether y comes from the new list, slot its pairdist index.  Pass 0 stores the
// distance and counts the records per target; pass 1 reads it back and writes the records.
// Returns whether side 0 dropped a candidate that a rank below check_k could have needed.
template <int PASS>
__device__ __forceinline__ bool join_lane_record(uint64_t i, uint32_t x, uint32_t y, bool my_new, float mine,
                                                 uint64_t slot, uint32_t P, uint32_t check_k,
                                                 const float* __restrict__ bound, float* __restrict__ pairdist,
                                                 uint32_t* __restrict__ cnt, const uint64_t* __restrict__ rec_off,
                                                 uint32_t* __restrict__ cursor, uint64_t* __restrict__ rec_key,
                                                 uint32_t* __restrict__ rec_aux) {
  const bool same = my_new && y == x;  // equal ids: no pair
  if (PASS == 0) pairdist[slot] = same ? __int_as_float(0x7fc00000) : mine;
  else mine = pairdist[slot];
  if (same) return false;
  uint32_t a = x, b = y;
  if (my_new && b < a) {
    a = y;
    b = x;
  }
  bool drop = false;
  // side 0: candidate b into node a (its rank feeds found); side 1: a into b
  if (mine <= bound[a]) {
    if (PASS == 0) atomicAdd(&cnt[a], 1u);
    else {
      uint32_t pos = atomicAdd(&cursor[a], 1u);
      rec_key[rec_off[a] + pos] = pack_key(mine, b);
      rec_aux[rec_off[a] + pos] = (uint32_t)(i << 1);
    }
  } else if (P < check_k) {
    drop = true;
  }
  if (mine <= bound[b]) {
    if (PASS == 0) atomicAdd(&cnt[b], 1u);
    else {
      uint32_t pos = atomicAdd(&cursor[b], 1u);
      rec_key[rec_off[b] + pos] = pack_key(mine, a);
      rec_aux[rec_off[b] + pos] = (uint32_t)(i << 1) | 1u;
    }
  }
  return drop;
}

// pairdist index of node i's pair (new entry p, candidate c): the pairs of p' < p come first.
__device__ __forceinline__ uint64_t join_slot(uint64_t po, uint32_t nn, uint32_t no, uint32_t p, uint32_t c) {
  uint64_t sp = p == 0 ? 0 : (uint64_t)p * (nn - 1) - (uint64_t)p * (p - 1) / 2 + (uint64_t)p * no;
  return po + sp + c;
}

}  // namespace efg
