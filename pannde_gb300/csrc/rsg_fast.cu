// rsg_fast.cu -- RSG leapfrog kernels, fast forms (FP64 and FP32).
//
// Velocity update at node n (HostRSGTDUT.hpp:338-362):
//   V_d += dt/rho_n * (Dx(S_dx) + Dy(S_dy) + Dz(S_dz) + force_d)
//   x: S0,S5,S4   y: S5,S1,S3   z: S4,S3,S2
// with D* the node-centred difference over the 8 incident cell slots
// (RightHex.hpp:151-192; slot k holds the cell that has this node as corner
// k^6, a missing cell (-1) contributes 0).
//
// Stress update at cell c (HostRSGTDUT.hpp:278-293, HostUTModel.hpp:270-286):
//   S_k += dt*(C_k0 exx + C_k1 eyy + C_k2 ezz + C_k3 gyz + C_k4 gxz + C_k5 gxy [+ moment_k])
// with the 3x3 velocity gradient from the 8 corners (RightHex.hpp:100-141).
//
// Both differences use one butterfly over the 8 values (corner / slot order
// 0=(0,0,0) 1=(1,0,0) 2=(1,1,0) 3=(0,1,0) 4..7 the same at +z):
//   a=f1-f0 b=f2-f3 c=f5-f4 d=f6-f7, p=f1+f0 q=f2+f3 r=f5+f4 s=f6+f7
//   Dx=(a+b)+(c+d)  Dy=(q-p)+(s-r)  Dz=(r+s)-(p+q)
// Constants are folded on the host: g = 0.25/h, coef = dt/rho_n, ctab = dt*C,
// moment weights carry dt.  This changes rounding only (<= 1e-10 rel. L2).
#include "rsg_common.cuh"

namespace pn {
namespace {

template <typename T>
__device__ __forceinline__ void diff3(const T f[8], T &dx, T &dy, T &dz) {
  const T a = f[1] - f[0], b = f[2] - f[3], c = f[5] - f[4], d = f[6] - f[7];
  const T p = f[1] + f[0], q = f[2] + f[3], r = f[5] + f[4], s = f[6] + f[7];
  dx = (a + b) + (c + d);
  dy = (q - p) + (s - r);
  dz = (r + s) - (p + q);
}

template <typename T>
__device__ __forceinline__ void gather_slots(const T *__restrict__ f, const int s[8], T out[8]) {
#pragma unroll
  for (int k = 0; k < 8; k++) out[k] = (s[k] >= 0) ? __ldg(f + s[k]) : T(0);
}

template <typename T>
__device__ __forceinline__ void gather_nodes(const T *__restrict__ f, const int s[8], T out[8]) {
#pragma unroll
  for (int k = 0; k < 8; k++) out[k] = __ldg(f + s[k]);
}

template <typename T, bool UNIFORM>
__global__ void __launch_bounds__(kTile) k_velocity(const VelArgs<T> a, int step) {
  const int n = blockIdx.x * kTile + threadIdx.x;
  if (n >= a.n_nodes) return;
  const T cf = a.coef[n];
  if (cf == T(0)) return;  // node owned by another partition
  const int4 lo = a.ncc[2 * n], hi = a.ncc[2 * n + 1];
  const int s[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};

  T f[8], dx, dy, dz;
  T ax, ay, az;
  T gx = a.gx, gy = a.gy, gz = a.gz;
  if (!UNIFORM) {
    gx = a.gnode[n];
    gy = a.gnode[a.n_nodes + n];
    gz = a.gnode[2 * a.n_nodes + n];
  }
  gather_slots(a.S0, s, f); diff3(f, dx, dy, dz);
  ax = gx * dx;
  gather_slots(a.S5, s, f); diff3(f, dx, dy, dz);
  ax += gy * dy;
  ay = gx * dx;
  gather_slots(a.S4, s, f); diff3(f, dx, dy, dz);
  ax += gz * dz;
  az = gx * dx;
  gather_slots(a.S1, s, f); diff3(f, dx, dy, dz);
  ay += gy * dy;
  gather_slots(a.S3, s, f); diff3(f, dx, dy, dz);
  ay += gz * dz;
  az += gy * dy;
  gather_slots(a.S2, s, f); diff3(f, dx, dy, dz);
  az += gz * dz;

  if (a.tile_src) {
    const int2 r = a.tile_src[blockIdx.x];
    const T *sig = a.sigval;
    for (int i = r.x; i < r.y; i++) {
      if (a.src_elem[i] != n) continue;
      const int code = a.src_code[i];
      const T v = a.src_w[i] * sig[code >> 2];
      const int d = code & 3;
      if (d == 0) ax += v; else if (d == 1) ay += v; else az += v;
    }
  }
  const T v0 = a.V0[n] + cf * ax;
  const T v1 = a.V1[n] + cf * ay;
  const T v2 = a.V2[n] + cf * az;
  a.V0[n] = v0;
  a.V1[n] = v1;
  a.V2[n] = v2;

  if (a.tile_sens) {
    const int2 r = a.tile_sens[blockIdx.x];
    const int64_t rec = a.rec_base + step;
    if (rec < a.rec_cap) {
      for (int i = r.x; i < r.y; i++) {
        if (a.sens_node[i] != n) continue;
        double *t = a.traces + (rec * a.n_sens + a.sens_idx[i]) * 3;
        t[0] = (double)v0;
        t[1] = (double)v1;
        t[2] = (double)v2;
      }
    }
  }
}

template <typename T, bool UNIFORM>
__global__ void __launch_bounds__(kTile) k_stress(const StressArgs<T> a, int step) {
  const int c = blockIdx.x * kTile + threadIdx.x;
  if (c >= a.n_cells) return;
  const int4 lo = a.hex[2 * c], hi = a.hex[2 * c + 1];
  const int s[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
  T gx = a.gx, gy = a.gy, gz = a.gz;
  if (!UNIFORM) {
    gx = a.gcell[c];
    gy = a.gcell[a.n_cells + c];
    gz = a.gcell[2 * a.n_cells + c];
  }
  T f[8];
  T d00, d10, d20, d01, d11, d21, d02, d12, d22;  // d_ij = d/dx_i V_j (unscaled)
  gather_nodes(a.V0, s, f); diff3(f, d00, d10, d20);
  gather_nodes(a.V1, s, f); diff3(f, d01, d11, d21);
  gather_nodes(a.V2, s, f); diff3(f, d02, d12, d22);
  T e[6];
  e[0] = gx * d00;
  e[1] = gy * d11;
  e[2] = gz * d22;
  e[3] = gy * d12 + gz * d21;
  e[4] = gx * d02 + gz * d20;
  e[5] = gx * d01 + gy * d10;

  const T *C = a.ctab + 36 * a.mat[c];
  T m[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
  if (a.tile_src) {
    const int2 r = a.tile_src[blockIdx.x];
    for (int i = r.x; i < r.y; i++) {
      if (a.src_elem[i] != c) continue;
      const int code = a.src_code[i];
      const T v = a.src_w[i] * a.sigval[code >> 3];
      const int k = code & 7;
#pragma unroll
      for (int q = 0; q < 6; q++) if (q == k) m[q] += v;
    }
  }
  T *S[6] = {a.S0, a.S1, a.S2, a.S3, a.S4, a.S5};
#pragma unroll
  for (int k = 0; k < 6; k++) {
    T acc = S[k][c] + m[k];
#pragma unroll
    for (int j = 0; j < 6; j++) acc += __ldg(C + 6 * k + j) * e[j];
    S[k][c] = acc;
  }
}

template <typename T>
cudaError_t launch_vel(const VelArgs<T> &a, int step, bool uniform, cudaStream_t st) {
  if (a.n_nodes <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((a.n_nodes + kTile - 1) / kTile);
  if (uniform) k_velocity<T, true><<<grid, kTile, 0, st>>>(a, step);
  else k_velocity<T, false><<<grid, kTile, 0, st>>>(a, step);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_str(const StressArgs<T> &a, int step, bool uniform, cudaStream_t st) {
  if (a.n_cells <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((a.n_cells + kTile - 1) / kTile);
  if (uniform) k_stress<T, true><<<grid, kTile, 0, st>>>(a, step);
  else k_stress<T, false><<<grid, kTile, 0, st>>>(a, step);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_velocity_f64(const VelArgs<double> &a, int step, bool uniform, cudaStream_t st) {
  return launch_vel<double>(a, step, uniform, st);
}
cudaError_t launch_stress_f64(const StressArgs<double> &a, int step, bool uniform, cudaStream_t st) {
  return launch_str<double>(a, step, uniform, st);
}
cudaError_t launch_velocity_f32(const VelArgs<float> &a, int step, bool uniform, cudaStream_t st) {
  return launch_vel<float>(a, step, uniform, st);
}
cudaError_t launch_stress_f32(const StressArgs<float> &a, int step, bool uniform, cudaStream_t st) {
  return launch_str<float>(a, step, uniform, st);
}

}  // namespace pn
