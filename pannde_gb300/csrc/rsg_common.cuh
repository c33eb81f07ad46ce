// rsg_common.cuh -- argument blocks shared by the host setup and the RSG
// leapfrog kernels (velocity update at nodes, stress update at cells).
//
// Device layout (structure of arrays, one array per component):
//   V[3]     node velocities Vx,Vy,Vz                 [n_nodes]      T
//   S[6]     cell stresses Sxx,Syy,Szz,Syz,Sxz,Sxy     [n_cells]      T
//   hex      cell -> 8 corner nodes                    [n_cells] int4x2
//   ncc      node -> 8 incident cell slots (-1 none)   [n_nodes] int4x2
//   coef     dt / rho_node (0 = node not owned)        [n_nodes]      T
//   mat      cell -> material row                      [n_cells]  int32
//   ctab     per material: 36 stiffness entries         [n_mat][36]    T
//            (fast forms: dt*C; exact form: C)
// Sources and sensors are sparse lists sorted by element, with one [begin,end)
// range per tile of kTile consecutive elements, so tiles without sources or
// sensors pay nothing.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pn {

constexpr int kTile = 256;  // elements per tile == threads per block

template <typename T>
struct VelArgs {
  int32_t n_nodes;
  const int4 *__restrict__ ncc;  // [n_nodes*2]
  T *__restrict__ V0;
  T *__restrict__ V1;
  T *__restrict__ V2;
  const T *__restrict__ S0;
  const T *__restrict__ S1;
  const T *__restrict__ S2;
  const T *__restrict__ S3;
  const T *__restrict__ S4;
  const T *__restrict__ S5;
  const T *__restrict__ coef;
  // spacing factors: uniform (gx,gy,gz = 0.25/h) or per node [3][n_nodes]
  // (fast forms: 0.25/d; exact form: d)
  T gx, gy, gz;
  const T *__restrict__ gnode;
  // force sources
  const int2 *__restrict__ tile_src;  // [n_tiles] or null
  const int32_t *__restrict__ src_elem;
  const int32_t *__restrict__ src_code;  // dir | (signal << 2)
  const T *__restrict__ src_w;
  const T *__restrict__ sigval;  // signal values: row min(step, sig_rows-1) at stride sig_stride
  int32_t n_sig;
  int32_t sig_stride;            // 0 when sigval already points at this step's row
  int32_t sig_rows;
  // sensors
  const int2 *__restrict__ tile_sens;  // [n_tiles] or null
  const int32_t *__restrict__ sens_node;
  const int32_t *__restrict__ sens_idx;
  double *__restrict__ traces;  // [rec_cap][n_sens][3]
  int32_t n_sens;
  int64_t rec_base;
  int64_t rec_cap;
};

template <typename T>
struct StressArgs {
  int32_t n_cells;
  const int4 *__restrict__ hex;  // [n_cells*2]
  const T *__restrict__ V0;
  const T *__restrict__ V1;
  const T *__restrict__ V2;
  T *__restrict__ S0;
  T *__restrict__ S1;
  T *__restrict__ S2;
  T *__restrict__ S3;
  T *__restrict__ S4;
  T *__restrict__ S5;
  const int32_t *__restrict__ mat;
  const T *__restrict__ ctab;
  T gx, gy, gz;
  const T *__restrict__ gcell;  // per cell [3][n_cells] or null
  T dt;                          // exact form only (fast forms fold dt into ctab)
  // moment sources
  const int2 *__restrict__ tile_src;
  const int32_t *__restrict__ src_elem;
  const int32_t *__restrict__ src_code;  // comp | (signal << 3)
  const T *__restrict__ src_w;
  const T *__restrict__ sigval;
  int32_t n_sig;
  int32_t sig_stride;
  int32_t sig_rows;
  int32_t has_moments;
};

#ifdef __CUDACC__
// signal row of a step: sigval + min(step, sig_rows-1) * sig_stride
template <typename T>
__device__ __forceinline__ const T *signal_row(const T *sigval, int step, int stride, int rows) {
  return sigval + (int64_t)min(step, rows - 1) * stride;
}
#endif

// Launchers (defined in rsg_fast.cu / rsg_exact.cu).  step = index of this
// step inside the current solve() call (selects the signal row).
cudaError_t launch_velocity_f64(const VelArgs<double> &a, int step, bool uniform, cudaStream_t st);
cudaError_t launch_stress_f64(const StressArgs<double> &a, int step, bool uniform, cudaStream_t st);
cudaError_t launch_velocity_f32(const VelArgs<float> &a, int step, bool uniform, cudaStream_t st);
cudaError_t launch_stress_f32(const StressArgs<float> &a, int step, bool uniform, cudaStream_t st);
cudaError_t launch_velocity_df64(const VelArgs<float2> &a, int step, bool uniform, cudaStream_t st);
cudaError_t launch_stress_df64(const StressArgs<float2> &a, int step, bool uniform, cudaStream_t st);
// a batch of table-form members: device arrays of their argument blocks and
// the prefix sums of their tile counts (members own consecutive tiles)
struct BatchLaunch {
  int n_members;
  const void *vel_args;   // VelArgs<S>[n_members]
  const void *str_args;   // StressArgs<S>[n_members]
  const int *vel_start;   // [n_members + 1]
  const int *str_start;   // [n_members + 1]
  int vel_tiles, str_tiles;
  int blocks_vel, blocks_str;  // grid sizes (blocks walk the tiles)
};
// precision: PN_PREC_F64 (1), PN_PREC_F32 (2), PN_PREC_DF64 (3)
cudaError_t launch_table_batch(const BatchLaunch &b, int precision, int step, cudaStream_t st);
// one or both half steps of a batch step: halves bit 0 velocity, bit 1 stress
cudaError_t launch_table_batch_halves(const BatchLaunch &b, int precision, int step, int halves, cudaStream_t st);

cudaError_t launch_velocity_exact(const VelArgs<double> &a, int step, cudaStream_t st);
cudaError_t launch_stress_exact(const StressArgs<double> &a, int step, cudaStream_t st);

}  // namespace pn
