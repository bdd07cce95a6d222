/*
 * efanna_gb300 — C ABI of the GB300 (sm_103a) kNN-graph build and graph search.
 *
 * Plain pointers, sizes and status codes only; no CUDA or C++ types cross this boundary
 * (streams are passed as void*, device buffers as plain pointers).  Each entry point names the
 * reference interface it replaces (paths inside the ZJULearning/efanna project).
 *
 * Conventions
 *   - Every function that can fail returns an int status (EFG_OK on success) and leaves a
 *     description in efg_last_error() (thread-local).
 *   - Host buffers are never retained: index creation copies the base vectors to the device.
 *   - "row_stride" arguments are in elements (floats), not bytes; stride >= dim.
 *   - Ids are uint32 (graph rows) or int32 (search results), as in the reference's files.
 *   - An index is single-caller: do not call into one index from two threads at once
 *     (as FIndex, efanna.hpp:9-75).
 */
#ifndef EFANNA_GB300_H
#define EFANNA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference reports these conditions by exit()/stdout
 * (kdtreeub_index.hpp:108-111,141,179,202,367-369,703,772,815); here each is a return value. */
#define EFG_OK 0
#define EFG_ERR_ARG 1          /* invalid argument (sizes, k > pool, zero trees, ...)          */
#define EFG_ERR_CUDA 2         /* a CUDA call failed; see efg_last_error()                      */
#define EFG_ERR_MERGE_LEVEL 3  /* merge level deeper than a tree leaf (kdtreeub_index.hpp:108) */
#define EFG_ERR_OPEN 4         /* file cannot be opened (exit -10086/-10087)                   */
#define EFG_ERR_FORMAT 5       /* malformed trees/graph/index file (exit -11, -6, -1)           */
#define EFG_ERR_STATE 6        /* operation needs trees/graph that the index does not hold      */
#define EFG_ERR_TREE_COUNT 7   /* more search trees requested than built ("wrong tree number")  */
#define EFG_ERR_NOMEM 8        /* device allocation failed                                      */
#define EFG_ERR_DEVICE_LIMIT 9 /* a device-side iteration limit was hit (work queue, probing)   */

/* Build parameters: KDTreeUbIndexParams (kdtreeub_index.hpp:14-35) + IndexParams
 * (general/params.hpp:19-33).  Field meaning follows the reference:
 *   K            graph degree exported to gs/saveGraph                      (IndexParams::K)
 *   S            sample size per iteration; also the BFS leaf threshold     (IndexParams::S)
 *   L            neighbour pool capacity                                    (IndexParams::L)
 *   check_k      rank below which an insert marks its source as "found"     (IndexParams::Check_K)
 *   epochs       NN-descent iterations                                      (build_epoches)
 *   trees        trees built (and kept for search)                          ("trees")
 *   trees_build  trees used for the leaf-merge initial graph, 0 = trees    ("treesb")
 *   merge_level  conquer-to depth of the leaf merge                         ("ml")
 *   leaf_size    DFS leaf size                                              (IndexParams::TNS)
 *   reverse_cap  reverse-list cap in update()                               (base_index.hpp:442)
 *   seed         seed of the counter-hash random streams                    (reference: 1998)  */
typedef struct efg_build_params {
  uint32_t K, S, L, check_k, epochs, trees, trees_build, merge_level, leaf_size, reverse_cap;
  uint64_t seed;
} efg_build_params;

/* Per-phase build statistics (the reference prints CPU clock() per phase under -DINFO,
 * kdtreeub_index.hpp:93-106, base_index.hpp:441-447; these are device times). */
typedef struct efg_build_stats {
  double trees_ms, init_ms, refine_ms, total_ms;
  uint64_t join_pairs;      /* pair distances evaluated by the join (the reference's `cc`)     */
  uint64_t join_records;    /* neighbour-list insert candidates kept after the radius filter    */
  uint64_t merge_distances; /* leaf-merge distances of the initial graph                        */
  int32_t max_merge_depth;  /* on EFG_ERR_MERGE_LEVEL: deepest usable merge level               */
  uint64_t join_large_nodes; /* BF16 build precision: node joins larger than one tensor-core tile */
} efg_build_stats;

/* Per-call search statistics. */
typedef struct efg_search_stats {
  double device_ms;         /* kernel time of the last search call                             */
  uint64_t distance_evals;  /* query-to-base distances computed by the last search call         */
  uint64_t queries;
  uint64_t expanded_nodes;  /* graph rows read by the expansion epochs of the last search call  */
  uint64_t overflow_queries; /* queries whose visited set outgrew shared memory (second pass)   */
  uint64_t kernel_launches;  /* search kernels launched by the last search call (1 or 2)         */
  uint64_t reranked;         /* FP32 re-rank distances per query under BF16 screening (0 in FP32) */
  uint64_t migrated_queries; /* queries whose visited set moved from shared to global memory      */
} efg_search_stats;

typedef struct efg_index efg_index;

/* Defaults of KDTreeUbIndexParams(true, 4) with IndexParams' member defaults. */
void efg_default_build_params(efg_build_params* p);

/* FIndex<float>(Matrix, Distance*, IndexParams) — efanna.hpp:14-20, matrix.hpp:21-39.
 * Copies n rows of dim floats (row_stride floats apart) from host memory to the device. */
int efg_index_create(const float* data, uint64_t n, uint32_t dim, uint64_t row_stride,
                     const efg_build_params* params, efg_index** out);
/* Same, from a device buffer (copied device-to-device into the index's padded layout). */
int efg_index_create_device(const float* d_data, uint64_t n, uint32_t dim, uint64_t row_stride,
                            const efg_build_params* params, efg_index** out);
void efg_index_destroy(efg_index* idx);

/* FIndex::buildTrees — efanna.hpp:28-31, kdtreeub_index.hpp:1192-1276. */
int efg_build_trees(efg_index* idx);
/* buildTrees with an explicit tree count: the trees a KDTreeUbIndexParams(true, ntrees) index
 * over the same data would build (samples/efanna_index_buildtrees.cc:42-46); the graph is kept. */
int efg_build_trees_count(efg_index* idx, uint32_t ntrees);
/* FIndex::buildIndex — efanna.hpp:24-27, kdtreeub_index.hpp:92-113 (initGraph + refineGraph). */
int efg_build_graph(efg_index* idx);
int efg_get_build_stats(const efg_index* idx, efg_build_stats* out);

/* FIndex::setSearchParams — efanna.hpp:56-58, base_index.hpp:153-161 (extend_to is clamped to
 * init_num).  search_method 0 = nnexp (kdtreeub_index.hpp:363-494), 1 = kgraph (:496-654). */
int efg_set_search_params(efg_index* idx, int epochs, int init_num, int extend_to, int search_trees,
                          int search_lv, int search_method);

/* Search precision (no reference counterpart; the reference computes in FP32 only).
 * EFG_PRECISION_FP32: every distance from the FP32 rows, results as the reference's.
 * EFG_PRECISION_BF16: the search walks the graph with distances from a BF16 copy of the base
 * (half the bytes per row; made on the first call that selects it and kept with the index), then
 * re-scores its best max(2k, k + 32) candidates (at most 1024) from the FP32 rows and emits the k
 * best of those.  Ids can differ from the FP32 search where BF16 rounding reorders candidates. */
#define EFG_PRECISION_FP32 0
#define EFG_PRECISION_BF16 1
#define EFG_PRECISION_FP8 2  /* e4m3 copy with one FP32 scale per row (max|x| / 448); same re-rank */
int efg_set_search_precision(efg_index* idx, int precision);
/* Build precision: how the NN-descent join (base_index.hpp:328-371) computes its pair distances
 * (no reference counterpart).  EFG_PRECISION_FP32, the default: FP32 rows on the CUDA cores.
 * EFG_PRECISION_BF16: per node, one Gram tile of its new x (new + old) rows on the tensor cores from
 * a BF16 copy of the base made at the start of each build, distance = |x|^2 + |y|^2 - 2 x.y; when
 * BF16 holds every value one product per value, else three (hi + lo split, a relative error near
 * 2^-17 of sum |x_k y_k|).  For integer data with squared norms below 2^23 (bytes up to 128
 * dimensions) every distance, and so the graph, equals the FP32 build's; for other data pools can
 * differ where distances tie within that error.  Several nodes share a tile of up to 128 new
 * entries x 128 (or, for larger nodes, 256) rows; a node with more than 128 new entries or 256
 * rows is scored as blocks of its new entries x chunks of its candidates
 * (efg_build_stats.join_large_nodes counts them).  A pair already in a pool is rejected as a
 * duplicate whatever its distance in this form (the reference compares ids among entries of equal
 * distance), so an id that comes back a few ulps apart is not inserted twice. */
int efg_set_build_precision(efg_index* idx, int precision);
/* Bound on the nnexp search's per-query candidate buffer (no reference counterpart; the reference's
 * candidate vector grows without bound).  0, the default, sizes it for the worst case of one
 * expansion epoch, extend_to x graph degree, which cannot overflow.  A smaller bound needs less
 * shared memory per query; it never goes below the pool size or the tree-descent frontier.  When an
 * epoch of some query appends more new candidates than the buffer holds, the extra ones are dropped
 * on the device and the search call returns EFG_ERR_DEVICE_LIMIT ("candidate buffer overflow"). */
int efg_set_search_candidate_cap(efg_index* idx, uint32_t cap);
/* The search's screening distances for given pairs: query q (device memory, row_stride floats apart)
 * against ids d_ids[q*m .. q*m + m) (m <= 4096), in `precision`; FP32 results into d_out (nq x m).
 * Used to state each precision's distance error against an FP64 reference. */
int efg_screen_distances(efg_index* idx, int precision, const float* d_queries, uint64_t nq, uint64_t row_stride,
                         const uint32_t* d_ids, uint32_t m, float* d_out, void* stream);

/* FIndex::knnSearch — efanna.hpp:32-34, base_index.hpp:311-313.  Host queries in, host ids out
 * (nq*k int32).  The ids are also kept for efg_save_results. */
int efg_knn_search(efg_index* idx, const float* queries, uint64_t nq, uint32_t dim, uint64_t row_stride,
                   uint32_t k, int32_t* out_ids);
/* Device-resident variant: queries and out_ids are device pointers; runs on `stream`
 * (a cudaStream_t, or NULL for the legacy default stream) and does not synchronise. */
int efg_knn_search_device(efg_index* idx, const float* d_queries, uint64_t nq, uint64_t row_stride,
                          uint32_t k, int32_t* d_out_ids, void* stream);
int efg_get_search_stats(const efg_index* idx, efg_search_stats* out);

/* Batching form (no reference counterpart: the reference applies one setSearchParams to a whole
 * batch).  Each query carries its own nnexp parameters; extend_to is clamped to init_num and k to
 * [1, init_num].  Method 0 (nnexp) with the index's search_trees and precision. */
typedef struct efg_query_params {
  int32_t epochs;
  int32_t init_num;  /* pool size */
  int32_t extend_to;
  uint32_t k;
} efg_query_params;
/* Host arrays: params has nq entries (init_num in [1, n], k in [1, k_max]); out_ids receives nq
 * rows of k_max ids, -1 past a query's k. */
int efg_knn_search_batch(efg_index* idx, const float* queries, uint64_t nq, uint32_t dim, uint64_t row_stride,
                         const efg_query_params* params, uint32_t k_max, int32_t* out_ids);
/* Device arrays: d_params (nq entries) and d_out_ids (nq rows of limits->k ids) in device memory;
 * `limits` (host memory) bounds every query's parameters -- larger values are clamped to it -- and
 * sizes the launch.  Runs on `stream` without synchronising.  d_nq, when not NULL, is a device
 * counter read by the kernel in place of nq (nq is then the capacity): a launch sequence captured
 * once in a CUDA graph serves batches of any size up to nq. */
int efg_knn_search_batch_device(efg_index* idx, const float* d_queries, uint64_t nq, uint64_t row_stride,
                                const efg_query_params* d_params, const efg_query_params* limits,
                                int32_t* d_out_ids, const uint32_t* d_nq, void* stream);

/* Seeded batch: like efg_knn_search_batch_device, and each query's pool starts with its
 * seeds_per_query entry ids from d_seeds (row qi, in order; ids >= n and repeats are skipped).
 * use_trees != 0: the tree leaves follow as usual until the query's pool size (the learned form's
 * search).  use_trees == 0: no trees are needed or read; a pool the seeds leave short is topped up
 * by the random fill -- the search of the hashing initialiser (getNeighborsIEH32_nnexp,
 * algorithm/hashing_index.hpp:1087-1200), whose Hamming-ball bucket visits give the seed order.
 * d_params may be NULL (every query at *limits). */
int efg_knn_search_seeded_device(efg_index* idx, const float* d_queries, uint64_t nq, uint64_t row_stride,
                                 const efg_query_params* d_params, const efg_query_params* limits,
                                 const uint32_t* d_seeds, uint32_t seeds_per_query, int use_trees,
                                 int32_t* d_out_ids, void* stream);

/* Learned form (no reference counterpart).  A two-layer MLP (d -> hidden -> hidden -> clusters +
 * rungs; BF16 weights and activations, FP32 accumulation; trained on the device by the library's own
 * forward/backward/Adam kernels) predicts per query the k-means clusters of the base that hold its
 * neighbours -- their `entries_per_cluster` members nearest the centroid become entry seeds of the
 * pool -- and a search setting from the rung ladder (the early-stop pool size).  Training traces
 * come from the method itself: exact neighbours of the training queries and the plain search's
 * recall at every rung (label: the first rung reaching min(target, best recall)).  Plain search
 * stays the fallback. */
#define EFG_LEARNED_MAX_RUNGS 16
typedef struct efg_learned_params {
  uint32_t clusters;             /* k-means clusters of the base (entry-point classes)          */
  uint32_t kmeans_iters;
  uint32_t kmeans_sample;        /* base rows used by the k-means iterations                    */
  uint32_t entries_per_cluster;  /* members nearest each centroid kept as seeds (0: no seeds)   */
  uint32_t entry_clusters;       /* clusters predicted per query (<= 64; 0: no seeds)           */
  uint32_t hidden;               /* hidden units per layer                                      */
  uint32_t rungs;                /* settings in rung[], ascending cost                          */
  efg_query_params rung[EFG_LEARNED_MAX_RUNGS];  /* k is ignored                              */
  float target;                  /* per-query recall@10 that defines the rung label             */
  uint32_t train_epochs;         /* passes over the traces                                      */
  uint32_t batch;                /* training batch                                              */
  float lr;                      /* Adam step                                                   */
  uint64_t seed;
  /* Neighbours the traces score the rungs against: the exact 10-NN of each training query when
   * trace_reference.init_num is 0 (the default), else the plain search's 10 ids at this setting
   * (epochs, pool, extend; k ignored) -- for training sets whose exact neighbours cost too much. */
  efg_query_params trace_reference;
} efg_learned_params;
typedef struct efg_learned_stats {
  uint64_t train_queries;
  float train_loss_first, train_loss_last;       /* mean batch loss of the first and last pass  */
  float rung_recall[EFG_LEARNED_MAX_RUNGS];      /* plain search's mean recall@10 per rung      */
} efg_learned_stats;
typedef struct efg_learned efg_learned;
void efg_learned_default_params(efg_learned_params* p);
/* Clusters the index's base (k-means on the device) and initialises the network. */
int efg_learned_create(efg_index* idx, const efg_learned_params* params, efg_learned** out);
/* Generates the traces for n training queries (device memory) and trains the network. */
int efg_learned_train(efg_learned* lr, const float* d_queries, uint64_t n, uint64_t row_stride);
/* Per query: entry_clusters predicted cluster ids (d_clusters, may be NULL when entry_clusters is 0)
 * and the predicted rung (d_rung): the most likely rung, or with coverage > 0 the first rung whose
 * cumulative predicted probability reaches coverage (the early stop). */
int efg_learned_predict_device(efg_learned* lr, const float* d_queries, uint64_t nq, uint64_t row_stride,
                               float coverage, uint32_t* d_clusters, uint32_t* d_rung, void* stream);
/* Learned search: prediction, then the seeded nnexp search with each query at its predicted rung
 * shifted by rung_bias (clamped to the ladder); nq rows of k ids into d_out. */
int efg_learned_search_device(efg_learned* lr, const float* d_queries, uint64_t nq, uint64_t row_stride,
                              uint32_t k, float coverage, int rung_bias, int32_t* d_out, void* stream);
int efg_learned_get_stats(const efg_learned* lr, efg_learned_stats* out);
/* Network parameters as one FP32 array [W1 | b1 | W2 | b2 | W3 | b3] (row-major, outputs x inputs). */
uint64_t efg_learned_num_params(const efg_learned* lr);
int efg_learned_get_weights(efg_learned* lr, float* host);
int efg_learned_set_weights(efg_learned* lr, const float* host);
/* Input standardisation (dim floats each): x' = (x - mean) * istd. */
int efg_learned_get_norm(efg_learned* lr, float* mean, float* istd);
/* Loss (mean over the batch) and its gradient for B query rows (device memory) with targets
 * d_tclusters (B x 10 neighbour clusters) and d_tlabel (B rungs), without updating the network. */
int efg_learned_grad(efg_learned* lr, const float* d_x, uint32_t B, uint64_t row_stride,
                     const uint32_t* d_tclusters, const uint8_t* d_tlabel, double* loss, float* host_grad);
/* Cluster of every base row (n int32), and per cluster its entry members (clusters x
 * entries_per_cluster, 0xffffffff past the count) and counts; any pointer may be NULL. */
int efg_learned_clusters(efg_learned* lr, int32_t* host_assign, uint32_t* host_entries, uint32_t* host_counts);
void efg_learned_destroy(efg_learned* lr);

/* Hashing-seeded search: the reference's hashing initialiser (HASHINGIndex).  Every base point has
 * one binary code per hash table (made outside the library, as in the reference; io.read_codes
 * reads its code files).  A query's pool is the first init_num distinct ids met while visiting its
 * Hamming ball of the given radius -- radius by radius, each radius's flipped-bit tuples in
 * ascending lexicographic order, all tables at every mask, bucket members in ascending id order --
 * topped up by the random fill, then expanded over the graph with the index's search parameters
 * (epochs, init_num, extend_to; no trees are needed).  The search method follows the hashing
 * index's numbering (efg_set_search_params' last argument): 1 = pool/extend
 * (getNeighborsIEH32_nnexp / getNeighborsIEH64_nnexp, algorithm/hashing_index.hpp:1087-1200 and
 * 1354-1470), 0 = kgraph (getNeighborsIEH32_kgraph / _64_kgraph, :1203-1352: the pool size grows
 * to epochs * extend_to as in the tree-seeded kgraph search, and expansions visit whole graph rows).
 * efg_hash_create: codes = tables x n codes (host, table-major) of code_bits bits (<= 64; the
 * reference's code length after its shift), radius <= min(13, code_bits), Hamming ball x tables <=
 * 2^26 probes.  The tables belong to idx, which must outlive them. */
typedef struct efg_hash efg_hash;
int efg_hash_create(efg_index* idx, const uint64_t* codes, uint32_t tables, uint32_t code_bits, uint32_t radius,
                    efg_hash** out);
/* Masks in the Hamming ball: sum over r <= radius of C(code_bits, r) (the reference's MaxCheck). */
uint64_t efg_hash_ball_size(const efg_hash* h);
/* Probe sequence of nq queries: d_qcodes[t * qcode_stride + q] is query q's code in table t;
 * row q of d_seeds (seeds_per_query entries) receives the probe sequence's first entries,
 * 0xffffffff past its end.  seeds_per_query = init_num * tables always holds the first init_num
 * distinct ids. */
int efg_hash_seeds_device(efg_hash* h, const uint64_t* d_qcodes, uint64_t qcode_stride, uint64_t nq,
                          uint32_t seeds_per_query, uint32_t* d_seeds, void* stream);
/* The hashing-seeded search over device queries and codes: nq rows of k ids into d_out.  Without a
 * graph on the index it is the reference's graph-less bucket search (getNeighbors32 / _64,
 * :929-1085): the pool's bucket ids, topped up by the random fill to k only, ranked by distance. */
int efg_hash_search_device(efg_index* idx, efg_hash* h, const float* d_queries, uint64_t nq, uint64_t row_stride,
                           const uint64_t* d_qcodes, uint64_t qcode_stride, uint32_t k, int32_t* d_out_ids,
                           void* stream);
/* Host-memory form (qcodes: tables x nq); the results are kept for efg_save_results. */
int efg_hash_search(efg_index* idx, efg_hash* h, const float* queries, uint64_t nq, uint32_t dim,
                    uint64_t row_stride, const uint64_t* qcodes, uint32_t k, int32_t* out_ids);
void efg_hash_destroy(efg_hash* h);

/* A search plan: the batched nnexp launch sequence for up to `capacity` queries whose parameters
 * are bounded by *limits, captured once in a CUDA graph over the plan's own device buffers (queries,
 * parameters, ids and the search's scratch) and replayed on the plan's own stream.  When
 * calibration queries are given (n_calib > 0, host memory, dim floats per row), the plan's
 * autotuner times the 256- and 512-thread kernel builds on them with the limits' parameters and
 * keeps the faster.  efg_search_plan_submit stages a batch (queries, per-query parameters) through
 * the plan's pinned buffers and queues the copies, the graph and the copy of the ids without
 * waiting; efg_search_plan_collect waits for that batch and writes its nq rows of limits->k ids;
 * efg_search_plan_run does both.  Several plans of one index may have batches in flight at once
 * (one each: a plan's batch is collected before its next submit).  A plan belongs to its index:
 * the index must outlive it, and creating a plan must not overlap other calls on the index. */
typedef struct efg_search_plan efg_search_plan;
int efg_search_plan_create(efg_index* idx, uint64_t capacity, const efg_query_params* limits,
                           const float* calib_queries, uint64_t n_calib, efg_search_plan** out);
int efg_search_plan_submit(efg_search_plan* plan, const float* queries, uint64_t nq, uint64_t row_stride,
                           const efg_query_params* params);
int efg_search_plan_collect(efg_search_plan* plan, int32_t* out_ids);
int efg_search_plan_run(efg_search_plan* plan, const float* queries, uint64_t nq, uint64_t row_stride,
                        const efg_query_params* params, int32_t* out_ids);
/* Block size the autotuner chose (256 or 512; 0 when the plan chose by occupancy). */
int efg_search_plan_threads(const efg_search_plan* plan);
/* The launch the plan's autotuner chose (all 0 when it was created without calibration queries):
 * block size (256 or 512), cap on resident CTAs per SM (0: as many as fit), shared visited-set
 * table in percent of the default size (sets that outgrow it move to global scratch; 0: 100), the
 * number of variants timed and the chosen one's time on the calibration batch.  Any pointer may be
 * NULL. */
int efg_search_plan_config(const efg_search_plan* plan, int32_t* threads, int32_t* ctas_per_sm, int32_t* ht_pct,
                           int32_t* variants, double* tuned_ms);
void efg_search_plan_destroy(efg_search_plan* plan);

/* File I/O, byte-compatible with the reference's formats. */
int efg_save_graph(efg_index* idx, const char* path);   /* saveGraph  kdtreeub_index.hpp:295-312 */
int efg_load_graph(efg_index* idx, const char* path);   /* loadGraph  kdtreeub_index.hpp:243-277 */
int efg_save_trees(efg_index* idx, const char* path);   /* saveTrees  kdtreeub_index.hpp:197-242 */
int efg_load_trees(efg_index* idx, const char* path);   /* loadTrees  kdtreeub_index.hpp:139-196 */
int efg_save_index(efg_index* idx, const char* path);   /* saveIndex  kdtreeub_index.hpp:771-825 */
int efg_load_index(efg_index* idx, const char* path);   /* loadIndex  kdtreeub_index.hpp:701-770 */
int efg_save_results(efg_index* idx, const char* path); /* saveResults base_index.hpp:136-151    */

/* getGraphSize / getGraphRow — efanna.hpp:59-64, base_index.hpp:494-501. */
uint64_t efg_graph_size(const efg_index* idx);
/* Copies row `row` into out (up to cap ids); returns the row length, or -1 on error. */
int64_t efg_graph_row(const efg_index* idx, uint64_t row, uint32_t* out, uint64_t cap);
/* Whole graph as CSR: row_ptr[n+1] and ids[nnz] (host buffers; pass NULL to query nnz). */
int efg_graph_csr(const efg_index* idx, uint64_t* row_ptr, uint32_t* ids, uint64_t* nnz);
/* The graph as the MATLAB front end's sparse matrix (findex.cc:106-150, getGraphMat): entry (i, j)
 * for every neighbour j of node i, in compressed-column form -- col_ptr[n+1], and row_ids[nnz]
 * holding for each column j the nodes i whose rows list j, ascending, once per listing.  Host
 * buffers of n + 1 and nnz (efg_graph_csr) entries. */
int efg_graph_csc(const efg_index* idx, uint64_t* col_ptr, uint32_t* row_ids);
/* The same transpose of any CSR graph over n nodes held in host memory (no GPU involved):
 * EFG_ERR_ARG when an id is >= n or row_ptr is not ascending. */
int efg_csr_transpose(uint64_t n, const uint64_t* row_ptr, const uint32_t* ids, uint64_t* col_ptr,
                      uint32_t* row_ids);
/* Trees held by the index (0 if none). */
uint32_t efg_tree_count(const efg_index* idx);

const char* efg_last_error(void);
const char* efg_version(void);

/* ---------------------------------------------------------------------------------------
 * Kernel-level entry points (device pointers).  These expose the hot-path kernels on their
 * own for integration and parity testing.
 * --------------------------------------------------------------------------------------- */

/* Squared L2 of m row pairs: out[i] = ||base[a[i]] - base[b[i]]||^2.
 * L2DistanceAVX::compare / L2Distance::compare — general/distance.hpp:125-147, 299-323. */
int efg_l2_pairs(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const uint32_t* d_a,
                 const uint32_t* d_b, uint64_t m, float* d_out, void* stream);

/* Exact k-NN by brute force (Matrix::brute_force_search, general/matrix.hpp:57-68), ordered by
 * (dist, id).  If exclude_self is nonzero, query i is base row (first_row + i) and is skipped
 * (those rows must lie in the base).  n <= 2^31 - 1.  Screening keeps, per query and base chunk,
 * the k + 16 smallest screened distances; the k + 16 best of those over all chunks are re-computed
 * in FP64 and the k smallest by (FP64 distance, id) are returned, d_dists (may be NULL) receiving
 * the FP64 distances rounded to FP32.  For k <= 104 the screening runs on the tensor cores
 * (tcgen05 BF16 Gram tiles, FP32 accumulation): exact on data BF16 holds exactly (integers up to
 * 256 in magnitude, as the byte-valued data sets), otherwise split into hi + lo BF16 parts with an
 * error near 2^-16 of |q.x|.  Larger k screen with the FP32 kernel below.  Ids are exact whenever
 * the true k nearest are among the k + 16 screened survivors of their chunk -- always on exactly
 * representable data. */
int efg_brute_force_knn(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q,
                        uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row,
                        int32_t* d_ids, float* d_dists, void* stream);
/* Timing of this thread's last tensor-core k-NN call (CUDA events on the call's stream). */
typedef struct efg_knn_stats {
  double convert_ms;    /* BF16 hi/lo rows and FP32 norms of base and queries                       */
  double bound_ms;      /* the per-query distance bounds from a strided sample of the base          */
  double screen_ms;     /* the tcgen05 screening kernel                                             */
  double merge_ms;      /* per-query merge of the chunk lists and FP64 re-rank                      */
  double screen_flops;  /* algorithmic: 2 x queries x base rows x dim (one Gram contraction)          */
  double tile_flops;    /* issued by the MMAs: whole tiles, 64-value k-blocks, x products per value  */
  uint32_t terms;       /* BF16 products per value: 1 (exact data) or 3 (hi.hi + hi.lo + lo.hi)      */
  uint32_t stages, nchunks, ctas;
  uint32_t sample_rows; /* base rows of the bound pass (0: none, small bases)                        */
} efg_knn_stats;
int efg_get_knn_stats(efg_knn_stats* out);
/* The same with the screening in FP32 on CUDA cores (squared differences, any k <= 256). */
int efg_brute_force_knn_fp32(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q,
                             uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row,
                             int32_t* d_ids, float* d_dists, void* stream);
/* The tensor-core path with the hi + lo split forced even on exactly representable data (k <= 104;
 * the lo parts are then zero and the results equal the plain tensor-core path's). */
int efg_brute_force_knn_split(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride, const float* d_q,
                              uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self, uint64_t first_row,
                              int32_t* d_ids, float* d_dists, void* stream);

/* efg_brute_force_knn without any device allocation, for callers that must not have a library
 * allocate GPU memory during the call (their device memory is owned by another allocator, or the
 * call sits in a loop that cannot afford an allocation).  No counterpart in the reference.
 * Same arguments and results as efg_brute_force_knn.  Its scratch is a fixed array compiled into
 * the library (EFG_BF_NOALLOC_SCRATCH_ENTRIES 8-byte entries = 16 MiB, held on every GPU that loads
 * the library until exit); calls needing more than nq * (k + 16) <= that many entries return
 * EFG_ERR_ARG.  The first call on a device looks up the scratch address (cudaGetSymbolAddress),
 * so make it before any stream capture; the address is kept per device and CUDA context, and a
 * call from a new context on that device (after cudaDeviceReset, or a driver-API context) looks it
 * up again -- also before any capture in that context.  All calls share the scratch: calls that
 * overlap on the GPU race and must be serialised by the caller.  Screening here is the FP32 kernel
 * of efg_brute_force_knn_fp32 (same results as efg_brute_force_knn). */
#define EFG_BF_NOALLOC_SCRATCH_ENTRIES (1ull << 21)
int efg_brute_force_knn_noalloc(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride,
                                const float* d_q, uint64_t nq, uint64_t q_stride, uint32_t k, int exclude_self,
                                uint64_t first_row, int32_t* d_ids, float* d_dists, void* stream);

/* NN-descent state on the host, for state-level parity checks (one layout with the oracle):
 * pool arrays are n*(L+1), list arrays n*cap.  efg_nnd_init runs the leaf-merge initial
 * graph on the index's trees (initGraph, kdtreeub_index.hpp:1367-1424); efg_nnd_iterate runs
 * one join + update (base_index.hpp:328-437) in place. */
typedef struct efg_nnd_host_state {
  uint64_t n;
  uint32_t L, cap;
  float* pool_dist;
  uint32_t* pool_id;
  uint8_t* pool_flag;
  uint32_t *Lcur, *Range;
  float *radius, *radiusM;
  uint8_t* found;
  uint32_t *new_ids, *new_cnt, *old_ids, *old_cnt;
} efg_nnd_host_state;
int efg_nnd_init(efg_index* idx, efg_nnd_host_state* st);
int efg_nnd_iterate(efg_index* idx, efg_nnd_host_state* st, uint32_t iter, uint64_t* pairs);

#ifdef __cplusplus
}
#endif
#endif /* EFANNA_GB300_H */
