// rsg_energy.cu -- FP64 energy audit of a solver's state, whatever its
// storage type:
//   kinetic  1/2 sum_n m_n |V_n|^2          m_n = lumped nodal mass
//   strain   1/2 sum_c vol_c S_c . C+_c S_c  C+ = pseudo-inverse of the cell's
//                                            6x6 Voigt stiffness (engineering
//                                            shear), so S . C+ S = sigma : eps
// Every term is formed and accumulated in FP64.  Each block writes one
// partial sum; the host adds the partials in block order, so the result does
// not depend on scheduling.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pannde_gb300.h"
#include "rsg_energy.cuh"

namespace {

template <typename R> __device__ __forceinline__ double as_double(R v);
template <> __device__ __forceinline__ double as_double<double>(double v) { return v; }
template <> __device__ __forceinline__ double as_double<float>(float v) { return (double)v; }
template <> __device__ __forceinline__ double as_double<float2>(float2 v) {
  return __dadd_rn((double)v.x, (double)v.y);
}

constexpr int kThreads = 256;

__device__ __forceinline__ void block_sum_store(double v, double *part) {
  __shared__ double warp_sums[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warp_sums[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kThreads / 32; k++) s += warp_sums[k];
    part[blockIdx.x] = s;
  }
}

template <typename R>
__global__ void __launch_bounds__(kThreads) k_energy_nodes(const R *__restrict__ v0, const R *__restrict__ v1,
                                                           const R *__restrict__ v2,
                                                           const double *__restrict__ mass, int64_t n,
                                                           double *__restrict__ part) {
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double m = __ldg(mass + i);
    if (m == 0.0) continue;
    const double a = as_double(v0[i]), b = as_double(v1[i]), c = as_double(v2[i]);
    acc += 0.5 * m * (a * a + b * b + c * c);
  }
  block_sum_store(acc, part);
}

template <typename R, typename M>
__global__ void __launch_bounds__(kThreads)
    k_energy_cells(pn::EnergyCells<R> a, const M *__restrict__ mat, double *__restrict__ part) {
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const int row = (int)mat[i];
    const double vol = a.vol ? __ldg(a.vol + i) : a.vol_uniform;
    if (vol == 0.0) continue;
    double s[6];
#pragma unroll
    for (int k = 0; k < 6; k++) s[k] = as_double(a.S[k][i]);
    const double *cp = a.comp + 36 * row;
    double q = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      double r = 0.0;
#pragma unroll
      for (int j = 0; j < 6; j++) r += __ldg(cp + 6 * k + j) * s[j];
      q += s[k] * r;
    }
    acc += 0.5 * vol * q;
  }
  block_sum_store(acc, part);
}

int blocks_for(int64_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 152;
  const int64_t want = (n + kThreads - 1) / kThreads;
  const int64_t cap = (int64_t)sms * 4;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

template <typename R>
cudaError_t nodes_t(const void *const V[3], const double *mass, int64_t n, double *part, int nb, cudaStream_t st) {
  k_energy_nodes<R><<<nb, kThreads, 0, st>>>((const R *)V[0], (const R *)V[1], (const R *)V[2], mass, n, part);
  return cudaGetLastError();
}

template <typename R>
cudaError_t cells_t(const void *const S[6], const void *mat, bool mat_u8, const double *comp, const double *vol,
                    double vol_uniform, int64_t n, double *part, int nb, cudaStream_t st) {
  pn::EnergyCells<R> a;
  for (int k = 0; k < 6; k++) a.S[k] = (const R *)S[k];
  a.comp = comp;
  a.vol = vol;
  a.vol_uniform = vol_uniform;
  a.n = n;
  if (mat_u8) k_energy_cells<R, uint8_t><<<nb, kThreads, 0, st>>>(a, (const uint8_t *)mat, part);
  else k_energy_cells<R, int32_t><<<nb, kThreads, 0, st>>>(a, (const int32_t *)mat, part);
  return cudaGetLastError();
}

}  // namespace

namespace pn {

int energy_blocks(int64_t n) { return blocks_for(n); }

cudaError_t launch_energy_nodes(int precision, const void *const V[3], const double *mass, int64_t n,
                                double *part, int nb, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (precision == PN_PREC_F32) return nodes_t<float>(V, mass, n, part, nb, st);
  if (precision == PN_PREC_DF64) return nodes_t<float2>(V, mass, n, part, nb, st);
  return nodes_t<double>(V, mass, n, part, nb, st);
}

cudaError_t launch_energy_cells(int precision, const void *const S[6], const void *mat, bool mat_u8,
                                const double *comp, const double *vol, double vol_uniform, int64_t n,
                                double *part, int nb, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (precision == PN_PREC_F32) return cells_t<float>(S, mat, mat_u8, comp, vol, vol_uniform, n, part, nb, st);
  if (precision == PN_PREC_DF64) return cells_t<float2>(S, mat, mat_u8, comp, vol, vol_uniform, n, part, nb, st);
  return cells_t<double>(S, mat, mat_u8, comp, vol, vol_uniform, n, part, nb, st);
}

}  // namespace pn
