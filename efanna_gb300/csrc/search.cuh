// Declarations shared by the two search methods (search.cu: nnexp; kgraph.cu: kgraph).
#pragma once
#include "internal.cuh"

namespace efg {

struct SearchCfg {
  uint32_t T, lsize, init_num, extend_to, result_size, epochs, k;
  uint32_t ht_size;     // visited-set slots
  uint32_t ht_limit;    // inserts allowed before the query is handed to the overflow pass
  uint32_t ht_soft;     // at a phase boundary, a set holding this many ids moves to global scratch
  uint32_t ht_mig;      // (when enabled) into a table of mig_size slots, the worst case
  uint32_t mig_size;
  uint32_t ht_global;   // visited set in a per-CTA slice of global scratch
  uint32_t ids_cap;     // candidate id buffer (u32 entries); on entry to layout(): a bound, 0 = none
  uint32_t res_cap;     // power of two >= result_size
  uint32_t nseq;        // T * lsize leaf slots
  // shared-memory byte offsets
  uint32_t o_ids, o_ht, o_u;
  uint32_t o_lstart, o_seqoff, o_tkey, o_tpos;  // fill phase (absolute)
  uint32_t o_res, o_tmp, o_newk, o_surv;                // select phase (absolute)
  uint32_t q4;          // staged query length in float4 (covers both row layouts)
  // reduced-precision screening (BF16 or FP8): BF16 rows ld16 values apart, cpr16 16-byte chunks
  // per row, 2^gshift16 lanes per row in the gather; the first `rerank` results are re-scored in
  // FP32 before the k are emitted
  uint32_t screened, ld16, cpr16, gshift16, rerank;
  // FP8 (e4m3, one FP32 scale per row) screening instead of BF16: rows ld8 bytes apart, cpr8
  // 16-byte chunks per row, 2^gshift8 lanes per row
  uint32_t fp8, ld8, cpr8, gshift8;
  uint32_t emit_pool;   // stop after the pool and write its keys (kgraph's first stage)
  uint32_t fixed_k;     // graph degree when every row has it (0: row pointers), and
  uint32_t kmagic;      // ceil(2^32 / fixed_k) for the division of item indices
  uint32_t nseeds;      // entry seeds per query placed ahead of the leaves (the seed rows' stride)
  const uint32_t* seed_cnt;  // per query, how many of its row's seeds are present (nullptr: all)
  uint32_t* next_q;          // the launch's query counter: CTAs take queries as they come free
  uint32_t fill_k;      // 1: the random fill tops the pool up to k only (the graph-less bucket search)
  uint64_t seed;
};

// Largest graph row length (the fixed degree when every row has K ids).
uint32_t graph_max_degree(efg_index* idx);
// Launches the nnexp kernel (one or two passes) for cfg's search parameters; with d_keys set it
// writes each query's pool keys (init_num per query, pool order) instead of result ids.
int launch_nnexp(efg_index* idx, SearchCfg cfg, uint32_t maxdeg, const float* d_q, uint64_t nq, uint64_t qld,
                 int32_t* d_out, uint64_t* d_keys, cudaStream_t s, int* launches,
                 const efg_query_params* d_params = nullptr, const uint32_t* d_nq = nullptr,
                 const uint32_t* d_seeds = nullptr);
// Checks shared by both methods (trees, graph, tree count, pool size, k).
int search_common_checks(efg_index* idx, uint32_t k);

// Reads the per-call device counters into the index's search statistics.
int finish_search_stats(efg_index* idx, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, uint64_t nq, bool two_pass,
                        int launches, uint64_t reranked);
// Sorts the first `count` keys of each of nq rows (rows `stride` keys apart) ascending in place;
// count <= 16384.
int launch_row_sort(uint64_t* keys, uint64_t nq, uint32_t stride, uint32_t count, cudaStream_t s);

}  // namespace efg
