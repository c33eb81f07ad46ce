// rsg_split.cu -- the grid form's fix-up of split lattice sites.
//
// A crack modelled as disconnected faces leaves lattice sites that several
// mesh nodes share ("copies"), each joined to some of the site's eight cells.
// The fused step kernel computes one velocity per site from all eight cells,
// and the stresses of the cells around such a site from it.  After the step
// kernel, on the same stream, two small kernels redo those sites from the
// step's input buffers, which the step leaves unchanged (double buffering):
//   1. k_split_copies: every copy's velocity from the cells it joins only,
//      with its force sources and sensor records;
//   2. k_split_cells: every fix cell's stress (a cell with a corner on a split
//      site) from its own corner nodes' new velocities, with its moment sources.
// This is the reference's semantics for a node without some incident cells --
// a missing cell adds nothing to the differences (RightHex.hpp:225-231) -- and
// for a cell's corner velocities, which are its own corner nodes' values
// (RightHex.hpp:241-247, HostRSGTDUT.hpp:278-293, 338-362).
#include <cstdint>

#include "df64.cuh"
#include "rsg_grid.cuh"

namespace pn {
namespace {

template <typename S> struct SN;  // storage type -> arithmetic
template <> struct SN<float> {
  using R = float;
  static __device__ __forceinline__ float val(float v) { return v; }
  static __device__ __forceinline__ float sto(float v) { return v; }
  static __device__ __forceinline__ double dbl(float v) { return (double)v; }
};
template <> struct SN<double> {
  using R = double;
  static __device__ __forceinline__ double val(double v) { return v; }
  static __device__ __forceinline__ double sto(double v) { return v; }
  static __device__ __forceinline__ double dbl(double v) { return v; }
};
template <> struct SN<float2> {
  using R = df64;
  static __device__ __forceinline__ df64 val(float2 v) { return df64(v.x, v.y); }
  static __device__ __forceinline__ float2 sto(df64 v) { return make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ double dbl(df64 v) { return (double)v.hi + (double)v.lo; }
};

constexpr int TPB = 128;

// FP64 form (a.rflags set): a stored value outside the double-float range
// puts the tile of lattice column (i, j) on the FP64 path for the next step
// (the tensor-copy kernel's flags, rsg_grid_tma.cuh fp64_path)
template <typename S>
__device__ __forceinline__ void flag_range(const GridArgs<S> &a, double v, int64_t i, int64_t j, int step,
                                           bool stress) {
  if (!a.rflags || in_df64_range(v, (uint32_t)(stress ? a.r_elo_s : a.r_elo), (uint32_t)(stress ? a.r_ehi_s : a.r_ehi)))
    return;
  const int gxc = a.nx / (kGridTileX - 1) + 1, gyc = a.ny / (a.tile_rows - 1) + 1;
  const int64_t blk = (j / (a.tile_rows - 1)) * gxc + i / (kGridTileX - 1);
  atomicOr(a.rflags + ((a.flag_phase + step + 1) % 3) * (int64_t)gxc * gyc + blk, 0x1fu);  // the tile, every edge
}

template <typename S>
__device__ __forceinline__ const S *signal_row(const GridArgs<S> &a, int step) {
  return a.sigval ? a.sigval + (int64_t)min(step, a.sig_rows - 1) * a.sig_stride : nullptr;
}

// velocity of copy q: x differences of Sxx, Sxy, Sxz; y of Sxy, Syy, Syz; z of
// Sxz, Syz, Szz over the cells the copy joins (a cell's sign along an axis is
// + on the site's upper side)
template <typename S>
__device__ void copy_velocity(const GridArgs<S> &a, int q, int step) {
  using N = SN<S>;
  using R = typename N::R;
  const SplitCopy cp = a.copies[q];
  const int64_t cplane = (int64_t)a.pcx * a.ny;
  R x0 = R(), x5 = R(), x4 = R(), y5 = R(), y1 = R(), y3 = R(), z4 = R(), z3 = R(), z2 = R();
  for (int c = 0; c < 8; c++) {
    if (!((cp.mask >> c) & 1u)) continue;
    const int ca = c & 1, cb = (c >> 1) & 1, cc = c >> 2;
    const int64_t cell = (int64_t)(cp.k - 1 + cc) * cplane + (int64_t)(cp.j - 1 + cb) * a.pcx + (cp.i - 1 + ca);
    const R s0 = N::val(a.S_in[0][cell]), s1 = N::val(a.S_in[1][cell]), s2 = N::val(a.S_in[2][cell]);
    const R s3 = N::val(a.S_in[3][cell]), s4 = N::val(a.S_in[4][cell]), s5 = N::val(a.S_in[5][cell]);
    if (ca) { x0 = x0 + s0; x5 = x5 + s5; x4 = x4 + s4; } else { x0 = x0 - s0; x5 = x5 - s5; x4 = x4 - s4; }
    if (cb) { y5 = y5 + s5; y1 = y1 + s1; y3 = y3 + s3; } else { y5 = y5 - s5; y1 = y1 - s1; y3 = y3 - s3; }
    if (cc) { z4 = z4 + s4; z3 = z3 + s3; z2 = z2 + s2; } else { z4 = z4 - s4; z3 = z3 - s3; z2 = z2 - s2; }
  }
  const R gx = N::val(a.g[0]), gy = N::val(a.g[1]), gz = N::val(a.g[2]);
  R acc[3];
  acc[0] = madd(gz, z4, madd(gy, y5, gx * x0));
  acc[1] = madd(gz, z3, madd(gy, y1, gx * x5));
  acc[2] = madd(gz, z2, madd(gy, y3, gx * x4));
  const S *sigrow = signal_row(a, step);
  for (int e = cp.f0; e < cp.f1; e++) {
    const int d = a.cf_dir[e];
    const R w = N::val(a.cf_w[e]), sg = N::val(sigrow[a.cf_sig[e]]);
    if (d == 0) acc[0] = madd(w, sg, acc[0]);
    else if (d == 1) acc[1] = madd(w, sg, acc[1]);
    else acc[2] = madd(w, sg, acc[2]);
  }
  const R cf = N::val(a.coef[cp.v]);
  R vn[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    vn[c] = N::val(a.V_in[c][cp.v]);
    if (!(cf == R())) vn[c] = madd(cf, acc[c], vn[c]);
    a.V_out[c][cp.v] = N::sto(vn[c]);
    flag_range(a, N::dbl(vn[c]), cp.i, cp.j, step, false);
  }
  const int64_t rec = a.rec + step;
  if (rec < a.rec_cap)
    for (int e = cp.s0; e < cp.s1; e++) {
      double *tr = a.traces + (rec * a.n_sens + a.cs_idx[e]) * 3;
      tr[0] = N::dbl(vn[0]);
      tr[1] = N::dbl(vn[1]);
      tr[2] = N::dbl(vn[2]);
    }
}

// stress of fix cell q from its corners' new velocities
template <typename S>
__device__ void fix_stress(const GridArgs<S> &a, int q, int step) {
  using N = SN<S>;
  using R = typename N::R;
  const FixCell fc = a.fix[q];
  R d[3][3];  // d[axis][component]: differences of the corner velocities
#pragma unroll
  for (int m = 0; m < 3; m++)
#pragma unroll
    for (int c = 0; c < 3; c++) d[m][c] = R();
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int bx = (k == 1 || k == 2 || k == 5 || k == 6), by = (k == 2 || k == 3 || k == 6 || k == 7), bz = k >= 4;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const R v = N::val(a.V_out[c][fc.v[k]]);
      d[0][c] = bx ? d[0][c] + v : d[0][c] - v;
      d[1][c] = by ? d[1][c] + v : d[1][c] - v;
      d[2][c] = bz ? d[2][c] + v : d[2][c] - v;
    }
  }
  const R gx = N::val(a.g[0]), gy = N::val(a.g[1]), gz = N::val(a.g[2]);
  R e[6];
  e[0] = gx * d[0][0];
  e[1] = gy * d[1][1];
  e[2] = gz * d[2][2];
  e[3] = madd(gz, d[2][1], gy * d[1][2]);
  e[4] = madd(gz, d[2][0], gx * d[0][2]);
  e[5] = madd(gy, d[1][0], gx * d[0][1]);
  const S *Cm = a.ctab + 36 * (int)a.mat[fc.cell];
  R acc[6];
#pragma unroll
  for (int k = 0; k < 6; k++) acc[k] = N::val(a.S_in[k][fc.cell]);
  const S *sigrow = signal_row(a, step);
  for (int ee = fc.m0; ee < fc.m1; ee++) {
    const int comp = a.cm_comp[ee];
    const R w = N::val(a.cm_w[ee]), sg = N::val(sigrow[a.cm_sig[ee]]);
#pragma unroll
    for (int k = 0; k < 6; k++)
      if (k == comp) acc[k] = madd(w, sg, acc[k]);
  }
#pragma unroll
  for (int k = 0; k < 6; k++) {
#pragma unroll
    for (int j = 0; j < 6; j++) acc[k] = madd(N::val(Cm[6 * k + j]), e[j], acc[k]);
    a.S_out[k][fc.cell] = N::sto(acc[k]);
    flag_range(a, N::dbl(acc[k]), fc.cell % a.pcx, (fc.cell / a.pcx) % a.ny, step, true);
  }
}

template <typename S>
__global__ void __launch_bounds__(TPB) k_split_copies(const GridArgs<S> a) {
  const int q = blockIdx.x * TPB + threadIdx.x;
  if (q < a.n_copies) copy_velocity(a, q, 0);
}

template <typename S>
__global__ void __launch_bounds__(TPB) k_split_cells(const GridArgs<S> a) {
  const int q = blockIdx.x * TPB + threadIdx.x;
  if (q < a.n_fix) fix_stress(a, q, 0);
}

// member of flat item id: start[m] <= id < start[m + 1]
__device__ __forceinline__ int member_of(const int *start, int n, int id) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(start + mid) <= id) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <typename S>
__global__ void __launch_bounds__(TPB)
    k_split_copies_batch(const GridArgs<S> *__restrict__ args, const int *__restrict__ start, int n, int total,
                         int step) {
  const int id = blockIdx.x * TPB + threadIdx.x;
  if (id >= total) return;
  const int m = member_of(start, n, id);
  copy_velocity(args[m], id - __ldg(start + m), step);
}

template <typename S>
__global__ void __launch_bounds__(TPB)
    k_split_cells_batch(const GridArgs<S> *__restrict__ args, const int *__restrict__ start, int n, int total,
                        int step) {
  const int id = blockIdx.x * TPB + threadIdx.x;
  if (id >= total) return;
  const int m = member_of(start, n, id);
  fix_stress(args[m], id - __ldg(start + m), step);
}

template <typename S>
cudaError_t split_one(const GridArgs<S> &a, cudaStream_t st) {
  if (a.n_copies > 0) k_split_copies<S><<<(a.n_copies + TPB - 1) / TPB, TPB, 0, st>>>(a);
  if (a.n_fix > 0) k_split_cells<S><<<(a.n_fix + TPB - 1) / TPB, TPB, 0, st>>>(a);
  return cudaGetLastError();
}

template <typename S>
cudaError_t split_batch(const GridSplitBatch &b, int step, cudaStream_t st) {
  const GridArgs<S> *args = (const GridArgs<S> *)b.args;
  if (b.total_copies > 0)
    k_split_copies_batch<S><<<(b.total_copies + TPB - 1) / TPB, TPB, 0, st>>>(args, b.copy_start, b.n_members,
                                                                              b.total_copies, step);
  if (b.total_fix > 0)
    k_split_cells_batch<S><<<(b.total_fix + TPB - 1) / TPB, TPB, 0, st>>>(args, b.fix_start, b.n_members,
                                                                         b.total_fix, step);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_grid_split(const void *args, int precision, cudaStream_t st) {
  if (precision == 2) return split_one<float>(*(const GridArgs<float> *)args, st);
  if (precision == 3) return split_one<float2>(*(const GridArgs<float2> *)args, st);
  return split_one<double>(*(const GridArgs<double> *)args, st);
}

cudaError_t launch_grid_split_batch(const GridSplitBatch &b, int precision, int step, cudaStream_t st) {
  if (precision == 2) return split_batch<float>(b, step, st);
  if (precision == 3) return split_batch<float2>(b, step, st);
  return split_batch<double>(b, step, st);
}

}  // namespace pn
