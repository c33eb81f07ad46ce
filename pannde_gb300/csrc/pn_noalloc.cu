// pn_noalloc.cu -- fixed device scratch for pn_batch_solve_noalloc.
//
// The batch kernels read every member's argument block and the prefix of the
// members' work tiles from device memory.  pn_batch_solve keeps that staging
// in buffers it grows with cudaMalloc; the allocation-free variant stages it
// here instead: one file-scope device array of kNoAllocScratchBytes, whose
// address is looked up once per device and then reused by every call.
#include <cuda_runtime.h>

#include <mutex>

#include "pn_noalloc.hpp"

namespace pn {
namespace {

// argument blocks + tile prefixes of one batch call (about 270 grid-form or
// 550 table-form members)
static __device__ __align__(256) unsigned char g_batch_scratch[kNoAllocScratchBytes];

std::mutex g_setup;
void *g_ptr[kNoAllocMaxDevices] = {};

}  // namespace

std::mutex &noalloc_call_lock() {
  static std::mutex m;
  return m;
}

cudaError_t noalloc_scratch(void **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_setup);
  if (!g_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_batch_scratch);
    if (e != cudaSuccess) return e;
    g_ptr[dev] = p;
  }
  *ptr = g_ptr[dev];
  return cudaSuccess;
}

}  // namespace pn
