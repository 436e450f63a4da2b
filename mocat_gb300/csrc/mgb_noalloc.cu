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
#include <mutex>

#include "mgb_internal.cuh"

namespace mgb {

constexpr size_t kNoallocBytes = 256 * 1024;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
static void *g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

// Device address of the scratch array on the current device, looked up once
// per device with that device current (the host-side name is only a stand-in
// and must never be passed to a kernel).  The first call on a device does the
// lookup, so that first call should be made before any stream capture.
static int scratch_address(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
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
