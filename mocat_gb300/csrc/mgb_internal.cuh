// Host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mocat_gb300.h"
#include "mgb_device.cuh"

namespace mgb {

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

inline unsigned grid_for(int64_t work, int tpb, int64_t cap = 16LL * kNumSMs) {
  int64_t g = (work + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? OK : ERR_LAUNCH;
}

// Bump allocator over a caller-provided workspace (256-byte aligned slices).
// With base == nullptr it only measures.
struct Carver {
  char *base;
  size_t off = 0;
  explicit Carver(void *b) : base((char *)b) {}
  template <class T>
  T *take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T *p = base ? (T *)(base + off) : nullptr;
    off += count * sizeof(T);
    return p;
  }
  size_t bytes() const { return (off + 255) & ~(size_t)255; }
};

}  // namespace mgb
