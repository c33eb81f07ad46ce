// rsg_state.cuh -- launchers of the state transfer kernels (rsg_state.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace pn {

// The FP64 form's tile flags for a state written into the voxel lattice:
// each value outside [2^(e_lo-1023), 2^(e_hi-1022)) (zero aside) or-s the bits
// the step kernel would record for it into its tile's word, flags[tile] (1
// any; 2 / 4 the tile's first / last owned column; 8 / 16 its first / last
// owned row; the last two for cells only).  Lattice index j = (layer * rows
// + y) * pitch + x, tiles of 31 x ty_own owned sites, gxc tiles along x; an
// index at or past lattice_len (a split site's copy) sets *unplaced instead.
struct StateRangeFlags {
  uint32_t *flags;
  int32_t *unplaced;
  int64_t lattice_len;
  int32_t pitch, rows, gxc, ty_own;
  uint32_t e_lo, e_hi;
  int32_t cell;
};

// Convert n FP64 values at src (device-accessible) to the storage type of
// `precision` and write them to dst[map[i]] (dst[i] when map is null); sets
// *nonfinite (device, when given) to 1 if any value is NaN or infinite; with
// rf (FP64 storage only), also flags the tiles of out-of-range values.
cudaError_t launch_state_store(int precision, const double *src, int64_t n, const int64_t *map,
                               void *dst, cudaStream_t st, int32_t *nonfinite = nullptr,
                               const StateRangeFlags *rf = nullptr);

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
