// Exact brute-force k-NN that allocates no device memory.
//
// efg_brute_force_knn takes the per-(query, chunk) candidate lists it needs between its two
// kernels from cudaMallocAsync.  Some callers cannot let a library allocate device memory when
// they call it: a host process whose GPU memory is handed out by its own allocator (a memory
// pool or a framework's caching allocator that has reserved the device, where a foreign
// cudaMalloc can fail or fragment what it manages), or a latency-critical loop that must not pay
// for an allocation and its implicit synchronisation.  efg_brute_force_knn_noalloc serves them:
// its scratch is a fixed array in this file, compiled into the library, so every GPU that loads
// the library holds these 16 MiB until the process exits.
//
// The array's name in host code is only a host-side stand-in, not a device address; the device
// address is looked up with cudaGetSymbolAddress on the first call made with a device (and
// context) current, and cached per device together with that context; a call from another context
// on the same device (after cudaDeviceReset, or a context made through the driver API) looks it up
// again.  That first call per device and context should come before any stream capture.
// All calls share the one array: calls that overlap on the GPU (concurrent streams, or threads
// sharing a device) race on it and must be serialised by the caller.  Nothing in it needs to start
// at zero -- every entry the second kernel reads is written by the first kernel of the same call.
#include <mutex>

#include "internal.cuh"

namespace efg {
int brute_force_knn_in(const float* base, uint64_t n, uint32_t dim, uint32_t ld, const float* q, uint64_t nq,
                       uint32_t qld, uint32_t k, int exclude_self, uint64_t first_row, int32_t* ids, float* dists,
                       uint64_t* part, uint64_t part_cap, cudaStream_t s);
}  // namespace efg

namespace {

constexpr uint64_t kScratchEntries = EFG_BF_NOALLOC_SCRATCH_ENTRIES;  // 2^21 keys x 8 B = 16 MiB
static __device__ __align__(256) uint64_t g_bf_scratch[kScratchEntries];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Per device ordinal: the context the address was looked up in, and the address.  A call made in
// another context on the same ordinal (after cudaDeviceReset, or with a context the caller created
// through the driver API) looks the address up again in that context.
void* g_ctx[kMaxDevices] = {};
uint64_t* g_dev_ptr[kMaxDevices] = {};

// cuCtxGetCurrent from the driver, found once through the runtime (no link against libcuda).
typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn ctx_get_current() {
  static std::once_flag once;
  static CtxGetCurrentFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}

// Device address of g_bf_scratch in the current device's current context.
int scratch_address(uint64_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return efg::fail(EFG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return efg::fail(EFG_ERR_ARG, "device ordinal beyond the scratch table");
  e = cudaFree(nullptr);  // makes the runtime's context current on this thread if none is
  if (e != cudaSuccess) return efg::fail(EFG_ERR_CUDA, std::string("cudaFree(0): ") + cudaGetErrorString(e));
  void* ctx = nullptr;
  CtxGetCurrentFn get = ctx_get_current();
  if (!get || get(&ctx) != 0 || !ctx) return efg::fail(EFG_ERR_CUDA, "no current CUDA context");
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_dev_ptr[dev] || g_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_bf_scratch);
    if (e != cudaSuccess || !p)
      return efg::fail(EFG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_dev_ptr[dev] = static_cast<uint64_t*>(p);
    g_ctx[dev] = ctx;
  }
  *out = g_dev_ptr[dev];
  return EFG_OK;
}

}  // namespace

extern "C" int efg_brute_force_knn_noalloc(const float* d_base, uint64_t n, uint32_t dim, uint64_t row_stride,
                                           const float* d_q, uint64_t nq, uint64_t q_stride, uint32_t k,
                                           int exclude_self, uint64_t first_row, int32_t* d_ids, float* d_dists,
                                           void* stream) {
  int rc0 = efg::bf_check_args(d_base, n, dim, row_stride, d_q, nq, q_stride, k, exclude_self, first_row, d_ids);
  if (rc0 != EFG_OK) return rc0;
  uint64_t* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != EFG_OK) return rc;
  return efg::brute_force_knn_in(d_base, n, dim, (uint32_t)row_stride, d_q, nq, (uint32_t)q_stride, k, exclude_self,
                                 first_row, d_ids, d_dists, scratch, kScratchEntries, (cudaStream_t)stream);
}
