// Systematic resampling for callers that cannot allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc at all: an XLA custom
// call or a node of a framework-built CUDA graph is handed its input and
// output buffers and must not allocate behind the framework's allocator, and
// a plugin loaded into a process whose allocator owns the device heap may be
// forbidden from creating allocations of its own.  For them,
// mgb_resample_systematic_u_noalloc keeps the scratch that systematic
// resampling needs (logsumexp partials, prefix-scan tile status words and a
// control block) in one fixed file-scope device array instead of a
// caller-provided workspace, and then runs the ordinary systematic path on it.
//
// The array holds MGB_NOALLOC_MAX_N particles' worth of scratch (256 KiB) and
// stays resident on every device that loads the library until the process
// exits.  All calls share it: each call clears what must start at zero, and
// calls whose work overlaps on the GPU (different streams, or a graph replayed
// concurrently) race on it.
#include <cuda.h>

#include <mutex>

#include "mgb_internal.cuh"

namespace mgb {

constexpr size_t kNoallocBytes = 256 * 1024;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Device addresses of the scratch array, one per CUDA context the library has
// served, keyed by the context's process-unique ID (cuCtxGetId).  A context
// created after cudaDeviceReset, or a caller's own non-primary context on the
// same device, loads the module again at another address and gets a new ID,
// so it never sees a stale entry.
constexpr int kMaxContexts = 64;
struct ScratchEntry {
  unsigned long long ctx_id;
  void *addr;
};
static ScratchEntry g_scratch_addr[kMaxContexts];
static int g_scratch_count = 0;
static std::mutex g_scratch_mu;

// Device address of the scratch array in the current context, looked up once
// per context with that context current (the host-side name is only a
// stand-in and must never be passed to a kernel).  The first call in a
// context does the lookup, so that first call should be made before any
// stream capture; later calls only read the current context's ID.
static int scratch_address(void **out) {
  // the driver's context queries, resolved through the runtime (the library
  // does not link libcuda itself)
  typedef CUresult (*GetCurrentFn)(CUcontext *);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!get_current || !get_id) {
    void *f0 = nullptr, *f1 = nullptr;
    cudaDriverEntryPointQueryResult q0, q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
      return ERR_CUDA;
    get_current = (GetCurrentFn)f0;
    get_id = (GetIdFn)f1;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS) return ERR_CUDA;
  if (!ctx) {
    // nothing current yet (no runtime call made on this thread): make the current
    // device's primary context current, as the runtime's first call would
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return ERR_CUDA;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return ERR_CUDA;
  }
  if (get_id(ctx, &id) != CUDA_SUCCESS) return ERR_CUDA;
  for (int i = 0; i < g_scratch_count; ++i)
    if (g_scratch_addr[i].ctx_id == id) {
      *out = g_scratch_addr[i].addr;
      return OK;
    }
  if (g_scratch_count == kMaxContexts) return ERR_UNSUPPORTED;
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return ERR_CUDA;
  g_scratch_addr[g_scratch_count++] = {id, p};
  *out = p;
  return OK;
}

}  // namespace mgb

using namespace mgb;

extern "C" int mgb_resample_systematic_u_noalloc(const float *lw, int64_t n, uint32_t m23, int32_t *anc,
                                                 int32_t *err, void *stream) {
  if (n < 1 || !lw || !anc || m23 >= (1u << 23)) return ERR_BAD_ARG;
  if (n > MGB_NOALLOC_MAX_N) return ERR_UNSUPPORTED;
  const size_t need = mgb_resample_workspace(n, MGB_RESAMPLE_SYSTEMATIC);
  if (need > kNoallocBytes) return ERR_UNSUPPORTED;
  void *base = nullptr;
  const int st = scratch_address(&base);
  if (st) return st;
  return mgb_resample_systematic_u(lw, n, m23, anc, base, kNoallocBytes, err, stream);
}
