// rsg_exact.cu -- RSG leapfrog kernels in the reference's exact FP64
// operation order.  This translation unit is compiled with -fmad=false, so
// every product and sum is rounded separately, as the reference's C++ is;
// divisions are IEEE round-to-nearest (nvcc's default -prec-div=true).  The
// results are bit-identical to HostSolver on the same inputs.
//
//   DD*_nc (RightHex.hpp:151-192, ncDifferencer 225-231):
//     value = 0; value += (f[fwd_k] or 0) - (f[bwd_k] or 0), k = 0..3;
//     return (value*0.25)/d_node
//   DD*_cc (RightHex.hpp:100-141, ccDifferencer 241-247): the same over corners
//     with the cell spacing.
//   velocity (HostRSGTDUT.hpp:343-360):
//     V_d += coef * (((DDx + DDy) + DDz) + evalXds)
//   stress (HostRSGTDUT.hpp:284-291, HostUTModel.hpp:276-284):
//     S_k += dt * (C_k0*d00 + C_k1*d11 + C_k2*d22 + C_k3*(d12+d21)
//                  + C_k4*(d02+d20) + C_k5*(d01+d10) [+ evalMoments])
//   evalXds / evalMoments: 0.125*signal summed over the in-window
//     (element, source) pairs in the reference's loop order (kept in the
//     source list order; the weight of every entry is 0.125).
#include "rsg_common.cuh"

namespace pn {
namespace {

// forward / backward corner (or slot) sets per axis, RightHex.hpp:103-104,
// 118-119, 133-134 (the same sets index the node slots, 154-186)
__host__ __device__ constexpr int fwd_of(int a, int k) {
  return a == 0 ? (k == 0 ? 1 : k == 1 ? 2 : k == 2 ? 5 : 6)
       : a == 1 ? (k == 0 ? 2 : k == 1 ? 3 : k == 2 ? 6 : 7)
                : 4 + k;
}
__host__ __device__ constexpr int bwd_of(int a, int k) {
  return a == 0 ? (k == 0 ? 0 : k == 1 ? 3 : k == 2 ? 4 : 7)
       : a == 1 ? (k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 4 : 5)
                : k;
}

template <int A>
__device__ __forceinline__ double dd_nc(const double *__restrict__ f, const int s[8], double d) {
  double value = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int a = s[fwd_of(A, k)], b = s[bwd_of(A, k)];
    const double fa = (a == -1) ? 0. : f[a];
    const double fb = (b == -1) ? 0. : f[b];
    value += (fa - fb);
  }
  return (value * 0.25) / d;
}

template <int A>
__device__ __forceinline__ double dd_cc(const double *__restrict__ f, const int s[8], double d) {
  double value = 0.0;
#pragma unroll
  for (int k = 0; k < 4; k++) value += (f[s[fwd_of(A, k)]] - f[s[bwd_of(A, k)]]);
  return (value * 0.25) / d;
}

// sensor traces: V after this step at the sensors of this tile
__device__ __forceinline__ void record(const VelArgs<double> &a, int n, int step, double v0,
                                       double v1, double v2) {
  if (!a.tile_sens) return;
  const int2 r = a.tile_sens[blockIdx.x];
  const int64_t rec = a.rec_base + step;
  if (rec >= a.rec_cap) return;
  for (int i = r.x; i < r.y; i++) {
    if (a.sens_node[i] != n) continue;
    double *t = a.traces + (rec * a.n_sens + a.sens_idx[i]) * 3;
    t[0] = v0;
    t[1] = v1;
    t[2] = v2;
  }
}

__global__ void __launch_bounds__(kTile) k_velocity_exact(const VelArgs<double> a, int step) {
  const int n = blockIdx.x * kTile + threadIdx.x;
  if (n >= a.n_nodes) return;
  const double cf = a.coef[n];
  if (cf == 0.) {  // node owned by another partition: not updated, still recorded
    record(a, n, step, a.V0[n], a.V1[n], a.V2[n]);
    return;
  }
  const int4 lo = a.ncc[2 * n], hi = a.ncc[2 * n + 1];
  const int s[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
  const double dxn = a.gnode[n], dyn = a.gnode[a.n_nodes + n], dzn = a.gnode[2 * a.n_nodes + n];
  double xd[3] = {0., 0., 0.};
  if (a.tile_src) {
    const int2 r = a.tile_src[blockIdx.x];
    for (int i = r.x; i < r.y; i++) {
      if (a.src_elem[i] != n) continue;
      const int code = a.src_code[i];
      const double v = a.src_w[i] * a.sigval[code >> 2];
      const int d = code & 3;
      if (d == 0) xd[0] = xd[0] + v;
      else if (d == 1) xd[1] = xd[1] + v;
      else xd[2] = xd[2] + v;
    }
  }
  const double v0 = a.V0[n] + cf * (((dd_nc<0>(a.S0, s, dxn) + dd_nc<1>(a.S5, s, dyn)) +
                                     dd_nc<2>(a.S4, s, dzn)) + xd[0]);
  const double v1 = a.V1[n] + cf * (((dd_nc<0>(a.S5, s, dxn) + dd_nc<1>(a.S1, s, dyn)) +
                                     dd_nc<2>(a.S3, s, dzn)) + xd[1]);
  const double v2 = a.V2[n] + cf * (((dd_nc<0>(a.S4, s, dxn) + dd_nc<1>(a.S3, s, dyn)) +
                                     dd_nc<2>(a.S2, s, dzn)) + xd[2]);
  a.V0[n] = v0;
  a.V1[n] = v1;
  a.V2[n] = v2;
  record(a, n, step, v0, v1, v2);
}

__global__ void __launch_bounds__(kTile) k_stress_exact(const StressArgs<double> a, int step) {
  const int c = blockIdx.x * kTile + threadIdx.x;
  if (c >= a.n_cells) return;
  const int4 lo = a.hex[2 * c], hi = a.hex[2 * c + 1];
  const int s[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
  const double dxc = a.gcell[c], dyc = a.gcell[a.n_cells + c], dzc = a.gcell[2 * a.n_cells + c];
  const double *V[3] = {a.V0, a.V1, a.V2};
  double d[3][3];
#pragma unroll
  for (int k1 = 0; k1 < 3; k1++) {
    d[0][k1] = dd_cc<0>(V[k1], s, dxc);
    d[1][k1] = dd_cc<1>(V[k1], s, dyc);
    d[2][k1] = dd_cc<2>(V[k1], s, dzc);
  }
  double mom[6] = {0., 0., 0., 0., 0., 0.};
  if (a.has_moments && a.tile_src) {
    const int2 r = a.tile_src[blockIdx.x];
    for (int i = r.x; i < r.y; i++) {
      if (a.src_elem[i] != c) continue;
      const int code = a.src_code[i];
      const double v = a.src_w[i] * a.sigval[code >> 3];
      const int k = code & 7;
#pragma unroll
      for (int q = 0; q < 6; q++) if (q == k) mom[q] = mom[q] + v;
    }
  }
  const double *C = a.ctab + 36 * a.mat[c];
  double *S[6] = {a.S0, a.S1, a.S2, a.S3, a.S4, a.S5};
#pragma unroll
  for (int ks = 0; ks < 6; ks++) {
    const double *Ck = C + 6 * ks;
    double acc = Ck[0] * d[0][0] + Ck[1] * d[1][1] + Ck[2] * d[2][2] +
                 Ck[3] * (d[1][2] + d[2][1]) + Ck[4] * (d[0][2] + d[2][0]) +
                 Ck[5] * (d[0][1] + d[1][0]);
    if (a.has_moments) acc = acc + mom[ks];
    S[ks][c] = S[ks][c] + a.dt * acc;
  }
}

}  // namespace

cudaError_t launch_velocity_exact(const VelArgs<double> &a, int step, cudaStream_t st) {
  if (a.n_nodes <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((a.n_nodes + kTile - 1) / kTile);
  k_velocity_exact<<<grid, kTile, 0, st>>>(a, step);
  return cudaGetLastError();
}

cudaError_t launch_stress_exact(const StressArgs<double> &a, int step, cudaStream_t st) {
  if (a.n_cells <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((a.n_cells + kTile - 1) / kTile);
  k_stress_exact<<<grid, kTile, 0, st>>>(a, step);
  return cudaGetLastError();
}

}  // namespace pn
