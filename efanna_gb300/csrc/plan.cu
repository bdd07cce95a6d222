// Search plans (batching form): the nnexp launch sequence for a bounded batch, captured once in a
// CUDA graph over device buffers owned by the plan, replayed per batch.  The batch size travels in
// a device counter, so one graph serves every batch size up to the plan's capacity; the kernel is
// persistent (a grid of resident CTAs looping over the batch's queries), and each query brings its
// own pool size, extend, epochs and k.  An optional autotuner times the 256- and 512-thread builds
// on calibration queries and keeps the faster one.
#include <algorithm>
#include <chrono>
#include <vector>

#include "internal.cuh"

using namespace efg;

struct efg_search_plan {
  efg_index* idx = nullptr;
  uint64_t capacity = 0;
  efg_query_params lim{};
  int threads = 0;
  DevBuf<float> q;
  DevBuf<efg_query_params> params;
  DevBuf<int32_t> out;
  DevBuf<uint32_t> nq;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

void plan_release(efg_search_plan* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->q.release();
  p->params.release();
  p->out.release();
  p->nq.release();
}

// Loads host queries (dim floats per row, row_stride apart) and parameters into the plan's buffers.
int stage_batch(efg_search_plan* p, const float* queries, uint64_t nq, uint64_t row_stride,
                const efg_query_params* params) {
  efg_index* idx = p->idx;
  cudaStream_t s = idx->stream;
  uint32_t n32 = (uint32_t)nq;
  EFG_CUDA(cudaMemcpy2DAsync(p->q.p, idx->ld * sizeof(float), queries, row_stride * sizeof(float),
                             idx->dim * sizeof(float), nq, cudaMemcpyHostToDevice, s));
  EFG_CUDA(cudaMemcpyAsync(p->params.p, params, nq * sizeof(efg_query_params), cudaMemcpyHostToDevice, s));
  EFG_CUDA(cudaMemcpyAsync(p->nq.p, &n32, 4, cudaMemcpyHostToDevice, s));
  EFG_CUDA(cudaStreamSynchronize(s));  // n32 lives on this stack frame
  return EFG_OK;
}

// Times one block-size build on the calibration batch already staged (median of three runs).
int time_variant(efg_search_plan* p, int threads, uint64_t n_calib, double* ms) {
  efg_index* idx = p->idx;
  idx->search_threads = threads;
  double best[3];
  for (int r = 0; r < 4; ++r) {
    auto t0 = std::chrono::steady_clock::now();
    EFG_TRY(search_device_ex(idx, p->q.p, n_calib, idx->ld, p->lim, p->params.p, nullptr, p->out.p, idx->stream,
                             false));
    EFG_CUDA(cudaStreamSynchronize(idx->stream));
    double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (r > 0) best[r - 1] = dt;  // the first run warms up
  }
  std::sort(best, best + 3);
  *ms = best[1];
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
  cudaStream_t s = idx->stream;
  int rc = EFG_OK;
  const int saved_threads = idx->search_threads;
  do {
    if ((rc = p->q.reserve(capacity * idx->ld)) != EFG_OK) break;
    if ((rc = p->params.reserve(capacity)) != EFG_OK) break;
    if ((rc = p->out.reserve(capacity * (uint64_t)limits->k)) != EFG_OK) break;
    if ((rc = p->nq.reserve(1)) != EFG_OK) break;
    if (cudaMemsetAsync(p->q.p, 0, capacity * idx->ld * sizeof(float), s) != cudaSuccess) {
      rc = fail(EFG_ERR_CUDA, "plan buffer clear failed");
      break;
    }
    // autotune the block size on the calibration queries, all at the limits' parameters
    if (calib_queries && n_calib) {
      uint64_t nc = std::min(n_calib, capacity);
      std::vector<efg_query_params> cp(nc, *limits);
      if ((rc = stage_batch(p, calib_queries, nc, idx->dim, cp.data())) != EFG_OK) break;
      double t256 = 0, t512 = 0;
      if ((rc = time_variant(p, 256, nc, &t256)) != EFG_OK) break;
      if ((rc = time_variant(p, 512, nc, &t512)) != EFG_OK) break;
      p->threads = t512 < t256 ? 512 : 256;
    }
    idx->search_threads = p->threads;
    // size every buffer and kernel attribute for the full capacity with an empty batch, then capture
    uint32_t zero = 0;
    if (cudaMemcpyAsync(p->nq.p, &zero, 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      rc = fail(EFG_ERR_CUDA, "plan counter reset failed");
      break;
    }
    if ((rc = search_device_ex(idx, p->q.p, capacity, idx->ld, p->lim, p->params.p, p->nq.p, p->out.p, s, false)) !=
        EFG_OK)
      break;
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      rc = fail(EFG_ERR_CUDA, "plan warm-up failed");
      break;
    }
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      rc = fail(EFG_ERR_CUDA, "cannot begin stream capture");
      break;
    }
    int crc = search_device_ex(idx, p->q.p, capacity, idx->ld, p->lim, p->params.p, p->nq.p, p->out.p, s, false);
    cudaError_t ce = cudaStreamEndCapture(s, &p->graph);
    if (crc != EFG_OK) {
      rc = crc;
      break;
    }
    if (ce != cudaSuccess || !p->graph) {
      rc = fail(EFG_ERR_CUDA, std::string("stream capture failed: ") + cudaGetErrorString(ce));
      break;
    }
    if (cudaGraphInstantiate(&p->exec, p->graph, 0) != cudaSuccess) {
      rc = fail(EFG_ERR_CUDA, "graph instantiation failed");
      break;
    }
  } while (false);
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

int efg_search_plan_run(efg_search_plan* p, const float* queries, uint64_t nq, uint64_t row_stride,
                        const efg_query_params* params, int32_t* out_ids) {
  if (!p || ((!queries || !params || !out_ids) && nq)) return fail(EFG_ERR_ARG, "null argument");
  if (nq > p->capacity) return fail(EFG_ERR_ARG, "batch larger than the plan's capacity");
  if (row_stride < p->idx->dim) return fail(EFG_ERR_ARG, "row_stride < dim");
  if (nq == 0) return EFG_OK;
  efg_index* idx = p->idx;
  EFG_TRY(stage_batch(p, queries, nq, row_stride, params));
  EFG_CUDA(cudaGraphLaunch(p->exec, idx->stream));
  EFG_CUDA(cudaMemcpyAsync(out_ids, p->out.p, nq * (uint64_t)p->lim.k * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           idx->stream));
  EFG_CUDA(cudaStreamSynchronize(idx->stream));
  return EFG_OK;
}

int efg_search_plan_threads(const efg_search_plan* p) { return p ? p->threads : 0; }

void efg_search_plan_destroy(efg_search_plan* p) {
  if (!p) return;
  if (p->idx && p->idx->stream) cudaStreamSynchronize(p->idx->stream);
  plan_release(p);
  delete p;
}
