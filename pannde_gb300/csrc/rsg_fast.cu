// rsg_fast.cu -- RSG leapfrog kernels, fast forms: FP64, FP32 and
// double-float (df64: FP64-class accuracy on the FP32 pipes; GB300 issues
// about 2 FP64 FMAs per SM per clock against 128 FP32 FMAs).
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
// moment weights carry dt.  This changes rounding only.
#include <type_traits>

#include "df64.cuh"
#include "rsg_common.cuh"

namespace pn {
namespace {

// storage <-> arithmetic type
template <typename R> struct Num;
template <> struct Num<float> {
  using S = float;
  static __device__ __forceinline__ float ld(const float *p, int i) { return __ldg(p + i); }
  static __device__ __forceinline__ float get(const float *p, int i) { return p[i]; }
  static __device__ __forceinline__ void put(float *p, int i, float v) { p[i] = v; }
  static __device__ __forceinline__ float val(float v) { return v; }
  static __device__ __forceinline__ double dbl(float v) { return (double)v; }
};
template <> struct Num<double> {
  using S = double;
  static __device__ __forceinline__ double ld(const double *p, int i) { return __ldg(p + i); }
  static __device__ __forceinline__ double get(const double *p, int i) { return p[i]; }
  static __device__ __forceinline__ void put(double *p, int i, double v) { p[i] = v; }
  static __device__ __forceinline__ double val(double v) { return v; }
  static __device__ __forceinline__ double dbl(double v) { return v; }
};
template <> struct Num<df64> {
  using S = float2;  // (hi, lo)
  static __device__ __forceinline__ df64 ld(const float2 *p, int i) {
    const float2 v = __ldg(p + i);
    return df64(v.x, v.y);
  }
  static __device__ __forceinline__ df64 get(const float2 *p, int i) {
    const float2 v = p[i];
    return df64(v.x, v.y);
  }
  static __device__ __forceinline__ void put(float2 *p, int i, df64 v) { p[i] = make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ df64 val(float2 v) { return df64(v.x, v.y); }
  static __device__ __forceinline__ double dbl(df64 v) { return (double)v.hi + (double)v.lo; }
};

template <typename R>
__device__ __forceinline__ void diff3(const R f[8], R &dx, R &dy, R &dz) {
  const R a = f[1] - f[0], b = f[2] - f[3], c = f[5] - f[4], d = f[6] - f[7];
  const R p = f[1] + f[0], q = f[2] + f[3], r = f[5] + f[4], s = f[6] + f[7];
  dx = (a + b) + (c + d);
  dy = (q - p) + (s - r);
  dz = (r + s) - (p + q);
}

template <typename R>
__device__ __forceinline__ void gather_slots(const typename Num<R>::S *__restrict__ f, const int s[8],
                                             R out[8]) {
#pragma unroll
  for (int k = 0; k < 8; k++) out[k] = (s[k] >= 0) ? Num<R>::ld(f, s[k]) : R();
}

template <typename R>
__device__ __forceinline__ void gather_nodes(const typename Num<R>::S *__restrict__ f, const int s[8],
                                             R out[8]) {
#pragma unroll
  for (int k = 0; k < 8; k++) out[k] = Num<R>::ld(f, s[k]);
}

// velocity update of node n (tile = n / kTile, step within the call)
template <typename R, bool UNIFORM>
__device__ __forceinline__ void velocity_node(const VelArgs<typename Num<R>::S> &a, int n, int tile,
                                              int step) {
  using N = Num<R>;
  const R cf = N::get(a.coef, n);
  R v0 = N::get(a.V0, n), v1 = N::get(a.V1, n), v2 = N::get(a.V2, n);
  if (!(cf == R())) {  // a zero coefficient marks a node owned by another partition
    const int4 lo = a.ncc[2 * n], hi = a.ncc[2 * n + 1];
    const int s[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
    R gx = N::val(a.gx), gy = N::val(a.gy), gz = N::val(a.gz);
    if (!UNIFORM) {
      gx = N::get(a.gnode, n);
      gy = N::get(a.gnode, a.n_nodes + n);
      gz = N::get(a.gnode, 2 * a.n_nodes + n);
    }
    R f[8], dx, dy, dz, ax, ay, az;
    if constexpr (std::is_same<R, float>::value) {
      // FP32: two fields' 16 gathers at a time, at the same 32 registers (velocity
      // step 0.121 -> 0.118 ms on the 400 x 400 x 40 laminate; double-float ran
      // 2% slower so, at 60 registers instead of 54)
      R h[8];
      gather_slots<R>(a.S0, s, f);
      gather_slots<R>(a.S5, s, h);
      diff3(f, dx, dy, dz);
      ax = gx * dx;
      diff3(h, dx, dy, dz);
      ax = ax + gy * dy;
      ay = gx * dx;
      gather_slots<R>(a.S4, s, f);
      gather_slots<R>(a.S1, s, h);
      diff3(f, dx, dy, dz);
      ax = ax + gz * dz;
      az = gx * dx;
      diff3(h, dx, dy, dz);
      ay = ay + gy * dy;
      gather_slots<R>(a.S3, s, f);
      gather_slots<R>(a.S2, s, h);
      diff3(f, dx, dy, dz);
      ay = ay + gz * dz;
      az = az + gy * dy;
      diff3(h, dx, dy, dz);
      az = az + gz * dz;
    } else {
      // one field's 8 gathers at a time: grouping three fields' gathers raised
      // the registers (FP32 32 -> 40, double-float 48 -> 78) and the kernel ran
      // 8-10% slower at the lower occupancy
      gather_slots<R>(a.S0, s, f); diff3(f, dx, dy, dz);
      ax = gx * dx;
      gather_slots<R>(a.S5, s, f); diff3(f, dx, dy, dz);
      ax = ax + gy * dy;
      ay = gx * dx;
      gather_slots<R>(a.S4, s, f); diff3(f, dx, dy, dz);
      ax = ax + gz * dz;
      az = gx * dx;
      gather_slots<R>(a.S1, s, f); diff3(f, dx, dy, dz);
      ay = ay + gy * dy;
      gather_slots<R>(a.S3, s, f); diff3(f, dx, dy, dz);
      ay = ay + gz * dz;
      az = az + gy * dy;
      gather_slots<R>(a.S2, s, f); diff3(f, dx, dy, dz);
      az = az + gz * dz;
    }
    if (a.tile_src) {
      const int2 r = a.tile_src[tile];
      const typename N::S *sig = signal_row(a.sigval, step, a.sig_stride, a.sig_rows);
      for (int i = r.x; i < r.y; i++) {
        if (a.src_elem[i] != n) continue;
        const int code = a.src_code[i];
        const R v = N::get(a.src_w, i) * N::get(sig, code >> 2);
        const int d = code & 3;
        if (d == 0) ax = ax + v;
        else if (d == 1) ay = ay + v;
        else az = az + v;
      }
    }
    v0 = v0 + cf * ax;
    v1 = v1 + cf * ay;
    v2 = v2 + cf * az;
    N::put(a.V0, n, v0);
    N::put(a.V1, n, v1);
    N::put(a.V2, n, v2);
  }
  if (a.tile_sens) {  // V after this step at the sensors of this tile
    const int2 r = a.tile_sens[tile];
    const int64_t rec = a.rec_base + step;
    if (rec < a.rec_cap) {
      for (int i = r.x; i < r.y; i++) {
        if (a.sens_node[i] != n) continue;
        double *t = a.traces + (rec * a.n_sens + a.sens_idx[i]) * 3;
        t[0] = N::dbl(v0);
        t[1] = N::dbl(v1);
        t[2] = N::dbl(v2);
      }
    }
  }
}

// stress update of cell c
template <typename R, bool UNIFORM>
__device__ __forceinline__ void stress_cell(const StressArgs<typename Num<R>::S> &a, int c, int tile,
                                            int step) {
  using N = Num<R>;
  const int4 lo = a.hex[2 * c], hi = a.hex[2 * c + 1];
  const int s[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
  R gx = N::val(a.gx), gy = N::val(a.gy), gz = N::val(a.gz);
  if (!UNIFORM) {
    gx = N::get(a.gcell, c);
    gy = N::get(a.gcell, a.n_cells + c);
    gz = N::get(a.gcell, 2 * a.n_cells + c);
  }
  // the 24 corner gathers are issued together, before their arithmetic (FP32
  // stress step 0.153 -> 0.136 ms on the 400 x 400 x 40 laminate)
  R f0[8], f1[8], f2[8];
  gather_nodes<R>(a.V0, s, f0);
  gather_nodes<R>(a.V1, s, f1);
  gather_nodes<R>(a.V2, s, f2);
  R d00, d10, d20, d01, d11, d21, d02, d12, d22;  // d_ij = d/dx_i V_j (unscaled)
  diff3(f0, d00, d10, d20);
  diff3(f1, d01, d11, d21);
  diff3(f2, d02, d12, d22);
  R e[6];
  e[0] = gx * d00;
  e[1] = gy * d11;
  e[2] = gz * d22;
  e[3] = gy * d12 + gz * d21;
  e[4] = gx * d02 + gz * d20;
  e[5] = gx * d01 + gy * d10;

  const typename N::S *C = a.ctab + 36 * a.mat[c];
  R m[6];
#pragma unroll
  for (int q = 0; q < 6; q++) m[q] = R();
  if (a.tile_src) {
    const int2 r = a.tile_src[tile];
    const typename N::S *sig = signal_row(a.sigval, step, a.sig_stride, a.sig_rows);
    for (int i = r.x; i < r.y; i++) {
      if (a.src_elem[i] != c) continue;
      const int code = a.src_code[i];
      const R v = N::get(a.src_w, i) * N::get(sig, code >> 3);
      const int k = code & 7;
#pragma unroll
      for (int q = 0; q < 6; q++)
        if (q == k) m[q] = m[q] + v;
    }
  }
  typename N::S *S[6] = {a.S0, a.S1, a.S2, a.S3, a.S4, a.S5};
#pragma unroll
  for (int k = 0; k < 6; k++) {
    R acc = N::get(S[k], c) + m[k];
#pragma unroll
    for (int j = 0; j < 6; j++) acc = acc + N::ld(C, 6 * k + j) * e[j];
    N::put(S[k], c, acc);
  }
}

template <typename R, bool UNIFORM>
__global__ void __launch_bounds__(kTile) k_velocity(const VelArgs<typename Num<R>::S> a, int step) {
  const int n = blockIdx.x * kTile + threadIdx.x;
  if (n < a.n_nodes) velocity_node<R, UNIFORM>(a, n, blockIdx.x, step);
}

template <typename R, bool UNIFORM>
__global__ void __launch_bounds__(kTile) k_stress(const StressArgs<typename Num<R>::S> a, int step) {
  const int c = blockIdx.x * kTile + threadIdx.x;
  if (c < a.n_cells) stress_cell<R, UNIFORM>(a, c, blockIdx.x, step);
}

// member owning work tile t: tile_start is the members' prefix of tile counts
__device__ __forceinline__ int member_of(const int *__restrict__ tile_start, int n_members, int t) {
  int lo = 0, hi = n_members;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(tile_start + mid) <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// batches: block b takes the contiguous share [b*T/B, (b+1)*T/B) of the T
// tiles of all members (members' tiles in member order).  The argument block
// of the member being worked on sits in shared memory, copied in once when
// the share reaches the member; the member of the first tile is found by
// binary search, later ones by stepping forward.
template <typename A>
__device__ __forceinline__ void load_args(A &dst, const A *src) {
  static_assert(sizeof(A) % 8 == 0, "argument blocks are copied in 8-byte words");
  unsigned long long *d = reinterpret_cast<unsigned long long *>(&dst);
  const unsigned long long *q = reinterpret_cast<const unsigned long long *>(src);
  for (int w = threadIdx.x; w < (int)(sizeof(A) / 8); w += blockDim.x) d[w] = __ldg(q + w);
}

__device__ __forceinline__ void share_of_tiles(int total, int &t0, int &t1) {
  t0 = (int)((long long)total * blockIdx.x / gridDim.x);
  t1 = (int)((long long)total * (blockIdx.x + 1) / gridDim.x);
}

template <typename R>
__global__ void __launch_bounds__(kTile) k_velocity_batch(const VelArgs<typename Num<R>::S> *__restrict__ args,
                                                          const int *__restrict__ tile_start, int n_members,
                                                          int step) {
  __shared__ __align__(16) VelArgs<typename Num<R>::S> a;
  int t0, t1;
  share_of_tiles(__ldg(tile_start + n_members), t0, t1);
  if (t0 >= t1) return;
  int m = member_of(tile_start, n_members, t0), m_end = -1, m_begin = 0;
  for (int t = t0; t < t1; t++) {
    if (t >= m_end) {  // the share reaches member m (first tile, or the previous member ended)
      while (t >= __ldg(tile_start + m + 1)) m++;
      __syncthreads();  // every thread is done with the previous member's block
      load_args(a, args + m);
      m_begin = __ldg(tile_start + m);
      m_end = __ldg(tile_start + m + 1);
      __syncthreads();
    }
    const int tl = t - m_begin;
    const int n = tl * kTile + threadIdx.x;
    if (n >= a.n_nodes) continue;
    if (a.gnode) velocity_node<R, false>(a, n, tl, step);
    else velocity_node<R, true>(a, n, tl, step);
  }
}

template <typename R>
__global__ void __launch_bounds__(kTile) k_stress_batch(const StressArgs<typename Num<R>::S> *__restrict__ args,
                                                        const int *__restrict__ tile_start, int n_members,
                                                        int step) {
  __shared__ __align__(16) StressArgs<typename Num<R>::S> a;
  int t0, t1;
  share_of_tiles(__ldg(tile_start + n_members), t0, t1);
  if (t0 >= t1) return;
  int m = member_of(tile_start, n_members, t0), m_end = -1, m_begin = 0;
  for (int t = t0; t < t1; t++) {
    if (t >= m_end) {
      while (t >= __ldg(tile_start + m + 1)) m++;
      __syncthreads();
      load_args(a, args + m);
      m_begin = __ldg(tile_start + m);
      m_end = __ldg(tile_start + m + 1);
      __syncthreads();
    }
    const int tl = t - m_begin;
    const int c = tl * kTile + threadIdx.x;
    if (c >= a.n_cells) continue;
    if (a.gcell) stress_cell<R, false>(a, c, tl, step);
    else stress_cell<R, true>(a, c, tl, step);
  }
}

template <typename R>
cudaError_t launch_vel(const VelArgs<typename Num<R>::S> &a, int step, bool uniform, cudaStream_t st) {
  if (a.n_nodes <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((a.n_nodes + kTile - 1) / kTile);
  if (uniform) k_velocity<R, true><<<grid, kTile, 0, st>>>(a, step);
  else k_velocity<R, false><<<grid, kTile, 0, st>>>(a, step);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_str(const StressArgs<typename Num<R>::S> &a, int step, bool uniform, cudaStream_t st) {
  if (a.n_cells <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((a.n_cells + kTile - 1) / kTile);
  if (uniform) k_stress<R, true><<<grid, kTile, 0, st>>>(a, step);
  else k_stress<R, false><<<grid, kTile, 0, st>>>(a, step);
  return cudaGetLastError();
}

// blocks of the batch kernels that are resident at once on the current
// device: every block's share of tiles is worked in one wave, so a grid
// larger than this would leave a tail of blocks queued behind the others
template <typename R>
int batch_resident(int sms_blocks_wanted, bool stress) {
  static int per_sm[2][64] = {{0}};
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return sms_blocks_wanted;
  int &p = per_sm[stress ? 1 : 0][dev & 63];
  if (p == 0) {
    int v = 0;
    const cudaError_t e =
        stress ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_stress_batch<R>, kTile, 0)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_velocity_batch<R>, kTile, 0);
    p = (e == cudaSuccess && v > 0) ? v : 1;
  }
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return sms_blocks_wanted;
  return std::min(sms_blocks_wanted, p * sms);
}

template <typename R>
cudaError_t launch_batch(const BatchLaunch &b, int step, int halves, cudaStream_t st) {
  using S = typename Num<R>::S;
  if ((halves & 1) && b.vel_tiles > 0)
    k_velocity_batch<R><<<batch_resident<R>(b.blocks_vel, false), kTile, 0, st>>>(
        (const VelArgs<S> *)b.vel_args, b.vel_start, b.n_members, step);
  if ((halves & 2) && b.str_tiles > 0)
    k_stress_batch<R><<<batch_resident<R>(b.blocks_str, true), kTile, 0, st>>>(
        (const StressArgs<S> *)b.str_args, b.str_start, b.n_members, step);
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
cudaError_t launch_velocity_df64(const VelArgs<float2> &a, int step, bool uniform, cudaStream_t st) {
  return launch_vel<df64>(a, step, uniform, st);
}
cudaError_t launch_stress_df64(const StressArgs<float2> &a, int step, bool uniform, cudaStream_t st) {
  return launch_str<df64>(a, step, uniform, st);
}
cudaError_t launch_table_batch(const BatchLaunch &b, int precision, int step, cudaStream_t st) {
  return launch_table_batch_halves(b, precision, step, 3, st);
}

cudaError_t launch_table_batch_halves(const BatchLaunch &b, int precision, int step, int halves, cudaStream_t st) {
  if (precision == 2) return launch_batch<float>(b, step, halves, st);
  if (precision == 3) return launch_batch<df64>(b, step, halves, st);
  return launch_batch<double>(b, step, halves, st);
}

}  // namespace pn
