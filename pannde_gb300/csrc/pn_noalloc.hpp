// pn_noalloc.hpp -- the fixed device scratch of pn_batch_solve_noalloc
// (pn_noalloc.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

namespace pn {

constexpr size_t kNoAllocScratchBytes = 256 * 1024;
constexpr int kNoAllocMaxDevices = 64;

// Device address of the scratch on the current device.  The first call on a
// device looks the symbol up (cudaGetSymbolAddress) and caches it; later calls
// only read the cache.  The cache lives as long as the process's context on
// that device: after cudaDeviceReset the address is stale, so a process that
// resets a device must not call the allocation-free solve on it again.
cudaError_t noalloc_scratch(void **ptr);

// Held for the whole of a pn_batch_solve_noalloc call: calls from several
// host threads take turns instead of overwriting each other's staging.
std::mutex &noalloc_call_lock();

}  // namespace pn
