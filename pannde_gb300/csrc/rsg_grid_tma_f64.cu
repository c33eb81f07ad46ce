// rsg_grid_tma_f64.cu -- the FP64 form's tensor-copy grid step
// (rsg_grid_tma.cuh k_grid_tma_f64h*): double storage, each block computing
// in double-float or, where its tile's values or source terms leave that
// range, in IEEE double.  A translation unit of its own so it compiles beside
// rsg_grid_tma.cu.
#include "rsg_grid_tma.cuh"

namespace pn {

cudaError_t launch_grid_tma_f64h(const GridArgs<double> &a, int sym, cudaStream_t st) {
  return launch_sym_h(a, sym, st);
}

cudaError_t launch_grid_tma_batch_f64h(const GridBatchLaunch &b, int step, cudaStream_t st) {
  return launch_batch_sym_h(b, step, st);
}

int grid_tma_f64_launches() { return PN_F64H_TWO_LAUNCHES ? 2 : 1; }

}  // namespace pn
