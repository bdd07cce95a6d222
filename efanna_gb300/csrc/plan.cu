// Search plans (batching form): the nnexp launch sequence for a bounded batch, captured once in a
// CUDA graph over device buffers owned by the plan (its queries, parameters, ids and the search's
// scratch), replayed per batch on the plan's own stream -- so several plans of one index keep
// batches in flight side by side (submit / collect).  The batch size travels in
// a device counter, so one graph serves every batch size up to the plan's capacity; the kernel is
// persistent (a grid of resident CTAs looping over the batch's queries), and each query brings its
// own pool size, extend, epochs and k.  An optional autotuner times launch variants on calibration
// queries at the limits' parameters and keeps the fastest: the block size (256 or 512 threads), the
// shared visited-set table (half, the default or double size; sets that outgrow it move to global
// scratch) and the CTAs resident per SM (as many as fit, or one).  None of these changes a result.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "internal.cuh"

using namespace efg;

struct efg_search_plan {
  efg_index* idx = nullptr;
  uint64_t capacity = 0;
  efg_query_params lim{};
  int threads = 0;       // the tuned launch: block size (0: by occupancy), CTAs per SM cap (0: none),
  int ctas_per_sm = 0;   // shared visited-set size in percent of the default (0: 100)
  int ht_pct = 0;
  double tuned_ms = 0;   // the chosen variant's time on the calibration batch
  int variants = 0;      // variants timed
  cudaStream_t stream = nullptr;  // the plan's own: plans of one index run side by side
  cudaEvent_t done = nullptr;     // the last submitted batch's ids are in hout
  DevBuf<float> q;
  DevBuf<efg_query_params> params;
  DevBuf<int32_t> out;
  DevBuf<uint32_t> nq;
  // the search's scratch, the plan's own (the captured kernels name these, not the index's)
  DevBuf<uint32_t> ht_scratch, ovf_list;
  DevBuf<unsigned long long> eval_counter;
  // pinned host staging: one contiguous copy each way per batch
  float* hq = nullptr;
  efg_query_params* hparams = nullptr;
  int32_t* hout = nullptr;
  uint32_t* hnq = nullptr;
  uint64_t pending = 0;  // queries of the submitted, not yet collected batch
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

void plan_release(efg_search_plan* p) {
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->q.release();
  p->params.release();
  p->out.release();
  p->nq.release();
  p->ht_scratch.release();
  p->ovf_list.release();
  p->eval_counter.release();
  if (p->hq) cudaFreeHost(p->hq);
  if (p->hparams) cudaFreeHost(p->hparams);
  if (p->hout) cudaFreeHost(p->hout);
  if (p->hnq) cudaFreeHost(p->hnq);
  if (p->done) cudaEventDestroy(p->done);
  if (p->stream) cudaStreamDestroy(p->stream);
  p->hq = nullptr;
  p->hparams = nullptr;
  p->hout = nullptr;
  p->hnq = nullptr;
  p->done = nullptr;
  p->stream = nullptr;
}

// The index's search scratch and the plan's trade places around a search issued for the plan
// (warm-up, autotuning and the captured launch), so that the plan's kernels use its own.
struct ScratchSwap {
  efg_search_plan* p;
  explicit ScratchSwap(efg_search_plan* pl) : p(pl) { swap_all(); }
  ~ScratchSwap() { swap_all(); }
  void swap_all() {
    std::swap(p->idx->ht_scratch, p->ht_scratch);
    std::swap(p->idx->ovf_list, p->ovf_list);
    std::swap(p->idx->eval_counter, p->eval_counter);
  }
};

// Loads host queries (dim floats per row, row_stride apart) and parameters into the plan's pinned
// staging and from there into its device buffers; on the plan's stream, nothing waited for.
int stage_batch(efg_search_plan* p, const float* queries, uint64_t nq, uint64_t row_stride,
                const efg_query_params* params) {
  efg_index* idx = p->idx;
  const uint64_t ld = idx->ld, dim = idx->dim;
  for (uint64_t i = 0; i < nq; ++i) std::memcpy(p->hq + i * ld, queries + i * row_stride, dim * sizeof(float));
  std::memcpy(p->hparams, params, nq * sizeof(efg_query_params));
  *p->hnq = (uint32_t)nq;
  EFG_CUDA(cudaMemcpyAsync(p->q.p, p->hq, nq * ld * sizeof(float), cudaMemcpyHostToDevice, p->stream));
  EFG_CUDA(cudaMemcpyAsync(p->params.p, p->hparams, nq * sizeof(efg_query_params), cudaMemcpyHostToDevice,
                           p->stream));
  EFG_CUDA(cudaMemcpyAsync(p->nq.p, p->hnq, 4, cudaMemcpyHostToDevice, p->stream));
  return EFG_OK;
}

// One launch variant of the nnexp search.
struct Variant {
  int threads, ht_pct, ctas_per_sm;
};

// Times one launch variant on the calibration batch already staged (median of three runs after a
// warm-up).
int time_variant(efg_search_plan* p, const Variant& v, uint64_t n_calib, double* ms) {
  efg_index* idx = p->idx;
  idx->search_threads = v.threads;
  idx->search_ht_pct = v.ht_pct;
  idx->search_ctas_per_sm = v.ctas_per_sm;
  double best[3];
  for (int r = 0; r < 4; ++r) {
    auto t0 = std::chrono::steady_clock::now();
    EFG_TRY(search_device_ex(idx, p->q.p, n_calib, idx->ld, p->lim, p->params.p, nullptr, p->out.p, p->stream,
                             false));
    EFG_CUDA(cudaStreamSynchronize(p->stream));
    double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (r > 0) best[r - 1] = dt;  // the first run warms up
  }
  std::sort(best, best + 3);
  *ms = best[1];
  return EFG_OK;
}

// The index's launch knobs, kept aside while a plan tunes and captures its own.
struct KnobGuard {
  efg_index* idx;
  int t, h, c;
  explicit KnobGuard(efg_index* i)
      : idx(i), t(i->search_threads), h(i->search_ht_pct), c(i->search_ctas_per_sm) {}
  ~KnobGuard() {
    idx->search_threads = t;
    idx->search_ht_pct = h;
    idx->search_ctas_per_sm = c;
  }
};

int plan_build(efg_search_plan* p, const float* calib_queries, uint64_t n_calib) {
  efg_index* idx = p->idx;
  const uint64_t capacity = p->capacity;
  EFG_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  EFG_CUDA(cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming));
  EFG_TRY(p->q.reserve(capacity * idx->ld));
  EFG_TRY(p->params.reserve(capacity));
  EFG_TRY(p->out.reserve(capacity * (uint64_t)p->lim.k));
  EFG_TRY(p->nq.reserve(1));
  EFG_TRY(p->eval_counter.reserve(8));
  if (cudaMallocHost((void**)&p->hq, capacity * idx->ld * sizeof(float)) != cudaSuccess ||
      cudaMallocHost((void**)&p->hparams, capacity * sizeof(efg_query_params)) != cudaSuccess ||
      cudaMallocHost((void**)&p->hout, capacity * (uint64_t)p->lim.k * sizeof(int32_t)) != cudaSuccess ||
      cudaMallocHost((void**)&p->hnq, sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    return fail(EFG_ERR_NOMEM, "pinned staging for the plan failed");
  }
  std::memset(p->hq, 0, capacity * idx->ld * sizeof(float));  // row padding stays zero
  EFG_CUDA(cudaMemsetAsync(p->q.p, 0, capacity * idx->ld * sizeof(float), p->stream));
  EFG_CUDA(cudaStreamSynchronize(idx->stream));  // the index is built and idle
  ScratchSwap swap(p);
  KnobGuard knobs(idx);
  // autotune the launch on the calibration queries, all at the limits' parameters
  if (calib_queries && n_calib) {
    uint64_t nc = std::min(n_calib, capacity);
    std::vector<efg_query_params> cp(nc, p->lim);
    EFG_TRY(stage_batch(p, calib_queries, nc, idx->dim, cp.data()));
    const Variant variants[] = {{256, 100, 0}, {512, 100, 0}, {256, 50, 0},  {512, 50, 0}, {256, 200, 0},
                                {512, 200, 0}, {256, 100, 1}, {256, 50, 1}, {256, 200, 1}};
    double best = 1e300;
    Variant pick = variants[0];
    std::vector<int32_t> ref, got(nc * p->lim.k);
    for (const Variant& v : variants) {
      double ms = 0;
      if (time_variant(p, v, nc, &ms) != EFG_OK) {  // a variant whose state does not fit: skipped
        cudaGetLastError();
        continue;
      }
      // every variant must return the same ids (the knobs change only where and how fast)
      EFG_CUDA(cudaMemcpyAsync(got.data(), p->out.p, got.size() * 4, cudaMemcpyDeviceToHost, p->stream));
      EFG_CUDA(cudaStreamSynchronize(p->stream));
      if (ref.empty()) ref = got;
      else if (ref != got) return fail(EFG_ERR_STATE, "launch variants returned different ids");
      ++p->variants;
      if (ms < best) {
        best = ms;
        pick = v;
      }
    }
    if (!p->variants) return fail(EFG_ERR_ARG, "no launch variant fits the plan's parameter limits");
    p->threads = pick.threads;
    p->ht_pct = pick.ht_pct;
    p->ctas_per_sm = pick.ctas_per_sm;
    p->tuned_ms = best;
  }
  idx->search_threads = p->threads;
  idx->search_ht_pct = p->ht_pct;
  idx->search_ctas_per_sm = p->ctas_per_sm;
  // size every buffer and kernel attribute for the full capacity with an empty batch, then capture
  *p->hnq = 0;
  EFG_CUDA(cudaMemcpyAsync(p->nq.p, p->hnq, 4, cudaMemcpyHostToDevice, p->stream));
  EFG_TRY(search_device_ex(idx, p->q.p, capacity, idx->ld, p->lim, p->params.p, p->nq.p, p->out.p, p->stream,
                           false));
  EFG_CUDA(cudaStreamSynchronize(p->stream));
  if (cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return fail(EFG_ERR_CUDA, "cannot begin stream capture");
  int crc = search_device_ex(idx, p->q.p, capacity, idx->ld, p->lim, p->params.p, p->nq.p, p->out.p, p->stream,
                             false);
  cudaError_t ce = cudaStreamEndCapture(p->stream, &p->graph);
  if (crc != EFG_OK) return crc;
  if (ce != cudaSuccess || !p->graph)
    return fail(EFG_ERR_CUDA, std::string("stream capture failed: ") + cudaGetErrorString(ce));
  if (cudaGraphInstantiate(&p->exec, p->graph, 0) != cudaSuccess) return fail(EFG_ERR_CUDA, "graph instantiation failed");
  return EFG_OK;
}

}  // namespace

int efg_search_plan_create(efg_index* idx, uint64_t capacity, const efg_query_params* limits,
                           const float* calib_queries, uint64_t n_calib, efg_search_plan** out) {
  if (!idx || !limits || !out) return fail(EFG_ERR_ARG, "null argument");
  *out = nullptr;
  if (capacity == 0 || capacity > 0xffffffffull) return fail(EFG_ERR_ARG, "capacity must be in [1, 2^32)");
  if (idx->sp.method != 0) return fail(EFG_ERR_ARG, "search plans use search method 0");
  if (limits->k == 0 || limits->init_num <= 0 || (uint64_t)limits->init_num > idx->n || limits->epochs < 0 ||
      limits->extend_to < 0 || (int)limits->k > limits->init_num)
    return fail(EFG_ERR_ARG, "invalid parameter limits");
  efg_search_plan* p = new efg_search_plan();
  p->idx = idx;
  p->capacity = capacity;
  p->lim = *limits;
  const int saved_threads = idx->search_threads;
  int rc = plan_build(p, calib_queries, n_calib);
  idx->search_threads = saved_threads;
  if (rc != EFG_OK) {
    cudaGetLastError();
    plan_release(p);
    delete p;
    return rc;
  }
  *out = p;
  return EFG_OK;
}

int efg_search_plan_submit(efg_search_plan* p, const float* queries, uint64_t nq, uint64_t row_stride,
                           const efg_query_params* params) {
  if (!p || ((!queries || !params) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (nq > p->capacity) return fail(EFG_ERR_ARG, "batch larger than the plan's capacity");
  if (row_stride < p->idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (p->pending) return fail(EFG_ERR_STATE, "the plan's previous batch has not been collected");
  if (nq == 0) return EFG_OK;
  EFG_TRY(stage_batch(p, queries, nq, row_stride, params));
  EFG_CUDA(cudaGraphLaunch(p->exec, p->stream));
  EFG_CUDA(cudaMemcpyAsync(p->hout, p->out.p, nq * (uint64_t)p->lim.k * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           p->stream));
  EFG_CUDA(cudaEventRecord(p->done, p->stream));
  p->pending = nq;
  return EFG_OK;
}

int efg_search_plan_collect(efg_search_plan* p, int32_t* out_ids) {
  if (!p || (!out_ids && p->pending)) return fail(EFG_ERR_ARG, "null argument");
  if (!p->pending) return EFG_OK;
  EFG_CUDA(cudaEventSynchronize(p->done));
  std::memcpy(out_ids, p->hout, p->pending * (uint64_t)p->lim.k * sizeof(int32_t));
  p->pending = 0;
  return EFG_OK;
}

int efg_search_plan_run(efg_search_plan* p, const float* queries, uint64_t nq, uint64_t row_stride,
                        const efg_query_params* params, int32_t* out_ids) {
  if (!p || ((!queries || !params || !out_ids) && nq)) return fail(EFG_ERR_ARG, "null argument");
  EFG_TRY(efg_search_plan_submit(p, queries, nq, row_stride, params));
  return efg_search_plan_collect(p, out_ids);
}

int efg_search_plan_threads(const efg_search_plan* p) { return p ? p->threads : 0; }

int efg_search_plan_config(const efg_search_plan* p, int32_t* threads, int32_t* ctas_per_sm, int32_t* ht_pct,
                           int32_t* variants, double* tuned_ms) {
  if (!p) return fail(EFG_ERR_ARG, "null plan");
  if (threads) *threads = p->threads;
  if (ctas_per_sm) *ctas_per_sm = p->ctas_per_sm;
  if (ht_pct) *ht_pct = p->ht_pct;
  if (variants) *variants = p->variants;
  if (tuned_ms) *tuned_ms = p->tuned_ms;
  return EFG_OK;
}

void efg_search_plan_destroy(efg_search_plan* p) {
  if (!p) return;
  plan_release(p);  // waits for the plan's stream first
  delete p;
}
