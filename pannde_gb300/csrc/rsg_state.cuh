// rsg_state.cuh -- launchers of the state transfer kernels (rsg_state.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pn {

// Convert n FP64 values at src (device-accessible) to the storage type of
// `precision` and write them to dst[map[i]] (dst[i] when map is null); sets
// *nonfinite (device, when given) to 1 if any value is NaN or infinite.
cudaError_t launch_state_store(int precision, const double *src, int64_t n, const int64_t *map,
                               void *dst, cudaStream_t st, int32_t *nonfinite = nullptr);

// Read src[map[i]] (src[i] when map is null) in the storage type of
// `precision` and write it as FP64 to dst[i] (device), i < n.
cudaError_t launch_state_load(int precision, const void *src, int64_t n, const int64_t *map,
                              double *dst, cudaStream_t st);

// Halo exchange of a partitioned solve: for each entry e of ex[n]
// (dst part, dst node, src part, src node), V[e.x][c][e.y] = V[e.z][c][e.w]
// for c = 0..2, with vptr[3*part + c] the device address of that velocity
// component (vptr itself in device memory).
cudaError_t launch_halo_exchange(int precision, const int4 *ex, int64_t n, void *const *vptr, cudaStream_t st);

}  // namespace pn
