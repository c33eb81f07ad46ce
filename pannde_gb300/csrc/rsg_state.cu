// rsg_state.cu -- device-side state transfer: FP64 host layout <-> storage.
//
// The C ABI takes and returns the state as FP64 arrays in the caller's node /
// cell numbering (PanNDE's Field order).  The device keeps it in the solver's
// storage type (double, float, or the (hi, lo) float pair of the double-float
// form) and, in the grid form, at lattice positions.  Instead of converting
// and permuting on the host, the FP64 array is copied once into a device
// staging buffer and these kernels convert + scatter (store) or gather +
// convert (load) it at HBM speed.
//
// Conversions are the host's: (float)v; hi = (float)v, lo = (float)(v - hi);
// hi + lo in double -- so results are the same bits as the host path.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pannde_gb300.h"
#include "df64.cuh"
#include "rsg_state.cuh"

namespace {

template <typename R> __device__ __forceinline__ R cvt_in(double v);
template <> __device__ __forceinline__ double cvt_in<double>(double v) { return v; }
template <> __device__ __forceinline__ float cvt_in<float>(double v) { return __double2float_rn(v); }
template <> __device__ __forceinline__ float2 cvt_in<float2>(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(__dsub_rn(v, (double)hi)));
}

template <typename R> __device__ __forceinline__ double cvt_out(R v);
template <> __device__ __forceinline__ double cvt_out<double>(double v) { return v; }
template <> __device__ __forceinline__ double cvt_out<float>(float v) { return (double)v; }
template <> __device__ __forceinline__ double cvt_out<float2>(float2 v) {
  return __dadd_rn((double)v.x, (double)v.y);
}

// the tile flag bits of an out-of-range value at lattice index j
__device__ __forceinline__ void flag_value(const pn::StateRangeFlags &rf, int64_t j) {
  if (j >= rf.lattice_len) {
    *rf.unplaced = 1;
    return;
  }
  const int x = (int)(j % rf.pitch), y = (int)((j / rf.pitch) % rf.rows);
  const int bx = x / 31, tx = x - 31 * bx, by = y / rf.ty_own, ty = y - rf.ty_own * by;
  uint32_t bits = 1u | (tx == 0 ? 2u : 0u) | (ty == 0 ? 8u : 0u);
  if (rf.cell) bits |= (tx == 30 ? 4u : 0u) | (ty == rf.ty_own - 1 ? 16u : 0u);
  atomicOr(rf.flags + (int64_t)by * rf.gxc + bx, bits);
}

// dst[map ? map[i] : i] = cvt(src[i]), i < n
template <typename R>
__global__ void __launch_bounds__(256) k_state_store(const double *__restrict__ src, int64_t n,
                                                     const int64_t *__restrict__ map,
                                                     R *__restrict__ dst, int32_t *nonfinite,
                                                     const pn::StateRangeFlags rf) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t j = map ? __ldg(map + i) : i;
    const double v = __ldg(src + i);
    // NaN or infinity: every exponent bit set
    bad = bad || (__double_as_longlong(v) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
    dst[j] = cvt_in<R>(v);
    if (rf.flags && !pn::in_df64_range(v, rf.e_lo, rf.e_hi)) flag_value(rf, j);
  }
  if (bad && nonfinite) *nonfinite = 1;
}

// dst[i] = cvt(src[map ? map[i] : i]), i < n
template <typename R>
__global__ void __launch_bounds__(256) k_state_load(const R *__restrict__ src, int64_t n,
                                                    const int64_t *__restrict__ map,
                                                    double *__restrict__ dst) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int64_t j = map ? __ldg(map + i) : i;
    dst[i] = cvt_out<R>(src[j]);
  }
}

// halo exchange of a partitioned solve: V[dst part][c][dst] = V[src part][c][src]
// for every entry (dst part, dst node, src part, src node) -- the halo copy of
// a node takes its owner's freshly updated velocity
template <typename R>
__global__ void __launch_bounds__(256) k_halo(const int4 *__restrict__ ex, int64_t n, R *const *__restrict__ vptr) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int4 e = __ldg(ex + i);
#pragma unroll
    for (int c = 0; c < 3; c++) vptr[3 * e.x + c][e.y] = vptr[3 * e.z + c][e.w];
  }
}

int blocks_for(int64_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 152;
  const int64_t want = (n + 255) / 256;
  const int64_t cap = (int64_t)sms * 8;  // grid-stride beyond 8 blocks per SM
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

namespace pn {

cudaError_t launch_state_store(int precision, const double *src, int64_t n, const int64_t *map,
                               void *dst, cudaStream_t st, int32_t *nonfinite, const StateRangeFlags *rf) {
  if (n <= 0) return cudaSuccess;
  const int nb = blocks_for(n);
  StateRangeFlags f{};
  if (rf) f = *rf;
  switch (precision) {
    case PN_PREC_F32: k_state_store<float><<<nb, 256, 0, st>>>(src, n, map, (float *)dst, nonfinite, StateRangeFlags{}); break;
    case PN_PREC_DF64: k_state_store<float2><<<nb, 256, 0, st>>>(src, n, map, (float2 *)dst, nonfinite, StateRangeFlags{}); break;
    default: k_state_store<double><<<nb, 256, 0, st>>>(src, n, map, (double *)dst, nonfinite, f); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_state_load(int precision, const void *src, int64_t n, const int64_t *map,
                              double *dst, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = blocks_for(n);
  switch (precision) {
    case PN_PREC_F32: k_state_load<float><<<nb, 256, 0, st>>>((const float *)src, n, map, dst); break;
    case PN_PREC_DF64: k_state_load<float2><<<nb, 256, 0, st>>>((const float2 *)src, n, map, dst); break;
    default: k_state_load<double><<<nb, 256, 0, st>>>((const double *)src, n, map, dst); break;
  }
  return cudaGetLastError();
}

}  // namespace pn

namespace pn {

cudaError_t launch_halo_exchange(int precision, const int4 *ex, int64_t n, void *const *vptr, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int nb = blocks_for(n);
  switch (precision) {
    case PN_PREC_F32: k_halo<float><<<nb, 256, 0, st>>>(ex, n, (float *const *)vptr); break;
    case PN_PREC_DF64: k_halo<float2><<<nb, 256, 0, st>>>(ex, n, (float2 *const *)vptr); break;
    default: k_halo<double><<<nb, 256, 0, st>>>(ex, n, (double *const *)vptr); break;
  }
  return cudaGetLastError();
}

}  // namespace pn
