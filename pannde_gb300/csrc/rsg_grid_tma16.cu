// rsg_grid_tma16.cu -- the tensor-copy grid step (rsg_grid_tma.cuh) with
// 32 x 16 tiles for FP32 storage: half the +y apron recompute of 32 x 8
// (31 x 15 owned of 512 threads against 31 x 7 of 256) at the same threads
// per SM (two blocks in shared memory).  A translation unit of its own so it
// compiles beside rsg_grid_tma.cu.
#include "rsg_grid_tma.cuh"

namespace pn {

cudaError_t launch_grid_tma_f32_rows16(const GridArgs<float> &a, int sym, cudaStream_t st) {
  return launch_sym<float, 16>(a, sym, st);
}

cudaError_t launch_grid_tma_batch_f32_rows16(const GridBatchLaunch &b, int step, cudaStream_t st) {
  return launch_batch_sym<float, 16>(b, step, st);
}

int grid_tma_blocks_per_sm_f32_rows16() {
  int sms = 0, per_sm = 0;
  return SetupT<float, 0, 16>::ensure(sms, per_sm) == cudaSuccess ? per_sm : 0;
}

}  // namespace pn
