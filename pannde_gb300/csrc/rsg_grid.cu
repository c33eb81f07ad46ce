// rsg_grid.cu -- the RSG leapfrog on voxel-grid meshes: one fused kernel per
// step that marches node layers along z through shared-memory tiles.
//
// The mesh is a lattice of nx*ny*nz cells (void sites hold zero stress and
// velocity, which is what a missing incident cell contributes in the
// reference, RightHex.hpp:225-231).  Indices are implicit: no connectivity
// table is read.  State is double-buffered (read *_in, write *_out) so that
// neighbouring tiles never see a half-updated step.
//
// A block owns a (TX-1) x (TY-1) column of cells and the same column of
// nodes over a chunk of cell layers [k0, k1) (blockIdx.z; chunks give the
// GPU enough blocks on thin plates); its TX x TY threads are the nodes of the
// column plus a one-node apron on the +x / +y side.  For each node layer
// k = k0-1 .. k1 (layer k0-1 only seeds the partial sums, layer k1 is
// recomputed for the stress of cell layer k1-1 and written by the next chunk):
//   A  stage cell layer k of S_in (a (TX+1) x (TY+1) tile with a one-cell
//      apron on the -x / -y side) in shared memory; issue the loads of layer
//      k+1 into registers (software pipelining)
//   B  velocity update of node layer k (HostRSGTDUT.hpp:338-362): the eight
//      incident cells are the four tile neighbours in cell layers k-1 and k;
//      per layer the four values give px=(B+C)-(A+D), py=(C+D)-(A+B),
//      s=(A+B)+(C+D), and Dx=px[k-1]+px[k], Dy=py[k-1]+py[k], Dz=s[k]-s[k-1]
//      with layer k-1's partial sums kept in registers.  New V goes to shared
//      memory and, for owned nodes, to V_out.
//   C  stress update of cell layer k-1 (HostRSGTDUT.hpp:278-293): the same
//      partial sums over the corner velocities of node layers k-1 and k.
// The apron node row/column is computed by both neighbouring tiles
// (identical inputs, identical result) and written only by its owner.
#include <algorithm>
#include <cstdlib>
#include <cstdint>

#include "df64.cuh"
#include "rsg_common.cuh"
#include "rsg_grid.cuh"

namespace pn {
namespace {

template <typename R> struct GNum;
template <> struct GNum<float> {
  using S = float;
  static __device__ __forceinline__ float ld(const float *p, int64_t i) { return __ldg(p + i); }
  static __device__ __forceinline__ void st(float *p, int64_t i, float v) { p[i] = v; }
  static __device__ __forceinline__ float val(float v) { return v; }
  static __device__ __forceinline__ float sto(float v) { return v; }
  static __device__ __forceinline__ double dbl(float v) { return (double)v; }
};
template <> struct GNum<double> {
  using S = double;
  static __device__ __forceinline__ double ld(const double *p, int64_t i) { return __ldg(p + i); }
  static __device__ __forceinline__ void st(double *p, int64_t i, double v) { p[i] = v; }
  static __device__ __forceinline__ double val(double v) { return v; }
  static __device__ __forceinline__ double sto(double v) { return v; }
  static __device__ __forceinline__ double dbl(double v) { return v; }
};
template <> struct GNum<df64> {
  using S = float2;
  static __device__ __forceinline__ df64 ld(const float2 *p, int64_t i) {
    const float2 v = __ldg(p + i);
    return df64(v.x, v.y);
  }
  static __device__ __forceinline__ void st(float2 *p, int64_t i, df64 v) { p[i] = make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ df64 val(float2 v) { return df64(v.x, v.y); }
  static __device__ __forceinline__ float2 sto(df64 v) { return make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ double dbl(df64 v) { return (double)v.hi + (double)v.lo; }
};

// stiffness entries kept by material symmetry class (all others are zero):
// 0 general, 1 monoclinic about z (no C14 C15 C24 C25 C34 C35 C46 C56),
// 2 orthotropic in the axes (C11..C33 block and the three shear diagonals)
__host__ __device__ constexpr bool c_used(int sym, int k, int j) {
  return sym == 0 ? true
       : sym == 2 ? ((k < 3 && j < 3) || k == j)
                  : ((k < 3 && j < 3) || k == j || (k == 5 && j < 3) || (j == 5 && k < 3) ||
                     (k == 3 && j == 4) || (k == 4 && j == 3));
}

// one block's work: tile (bx, by) of a grid with gxc tiles along x, z chunk bz
template <typename R, int TX, int TY, int SYM>
__device__ __forceinline__ void grid_block(const GridArgs<typename GNum<R>::S> &a, int bx, int by, int bz,
                                           int gxc, int step) {
  using N = GNum<R>;
  using St = typename N::S;
  constexpr int NT = TX * TY;
  constexpr int CW = TX + 1, CH = TY + 1, CT = CW * CH;  // cell tile
  constexpr int PF = (CT + NT - 1) / NT;                  // staged cells per thread
  extern __shared__ __align__(16) unsigned char smem_raw[];
  St *sS = reinterpret_cast<St *>(smem_raw);  // [3][6][CT]
  St *sV = sS + 3 * 6 * CT;                    // [2][3][NT]

  const int t = threadIdx.x;
  const int tx = t % TX, ty = t / TX;
  const int i0 = bx * (TX - 1), j0 = by * (TY - 1);
  const int blk = by * gxc + bx;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int i = i0 + tx, j = j0 + ty;
  const bool node_in = (i <= nx) && (j <= ny);
  const bool node_own = node_in && tx < TX - 1 && ty < TY - 1;
  const bool cell_own = tx < TX - 1 && ty < TY - 1 && i < nx && j < ny;
  const int64_t nplane = (int64_t)a.pnx * (ny + 1), cplane = (int64_t)a.pcx * ny;
  const int64_t nidx0 = (int64_t)j * a.pnx + i;  // node index in its layer
  const int64_t cidx0 = (int64_t)j * a.pcx + i;  // cell index in its layer
  const R gx = N::val(a.g[0]), gy = N::val(a.g[1]), gz = N::val(a.g[2]);
  const St *sigrow = a.sigval ? a.sigval + (int64_t)min(step, a.sig_rows - 1) * a.sig_stride : nullptr;
  const int64_t rec = a.rec + step;

  // staged cells of this thread: tile position and validity per layer
  int pf_off[PF];
  bool pf_ok[PF];
#pragma unroll
  for (int p = 0; p < PF; p++) {
    const int q = t + p * NT;
    const int cx = q % CW, cy = q / CW;
    const int ci = i0 - 1 + cx, cj = j0 - 1 + cy;
    pf_ok[p] = q < CT && ci >= 0 && ci < nx && cj >= 0 && cj < ny;
    pf_off[p] = pf_ok[p] ? cj * a.pcx + ci : 0;
  }
  R pf[PF][6];
  auto issue = [&](int kc) {  // loads of cell layer kc (zeros outside)
#pragma unroll
    for (int p = 0; p < PF; p++) {
      const bool ok = pf_ok[p] && kc >= 0 && kc < nz;
      const int64_t g = ok ? (int64_t)kc * cplane + pf_off[p] : 0;  // in bounds either way
#pragma unroll
      for (int f = 0; f < 6; f++) pf[p][f] = ok ? N::ld(a.S_in[f], g) : R();
    }
  };
  // this block's chunk of the column: cell layers [k0, k1), node layers [k0, k1)
  // (and node layer nz in the last chunk).  The march starts one cell layer
  // below (its partial sums only) and recomputes node layer k1, which the next
  // chunk owns, for the stress of cell layer k1-1.
  const int k0 = bz * a.kchunk, k1 = min(nz, k0 + a.kchunk);
  const bool last_chunk = k1 == nz;
  issue(k0 - 1);

  // layer k-1 partial sums: velocity (per stress field) and stress (per V comp)
  R vpx0 = R(), vpx4 = R(), vpx5 = R(), vpy1 = R(), vpy3 = R(), vpy5 = R(), vs2 = R(), vs3 = R(),
    vs4 = R();
  R spx[3], spy[3], ss[3];
#pragma unroll
  for (int c = 0; c < 3; c++) spx[c] = spy[c] = ss[c] = R();

  for (int k = k0 - 1; k <= k1; k++) {
    const int slot = (k + 1) % 3;  // cell layer k; layer -1 uses slot 0
    const bool do_vel = k >= k0;                        // node layer k is computed
    const bool own_layer = do_vel && (k < k1 || last_chunk);  // ... and written here
    St *Sk = sS + slot * 6 * CT;
    // ---- A: stage cell layer k, prefetch layer k+1
#pragma unroll
    for (int p = 0; p < PF; p++) {
      const int q = t + p * NT;
      if (q < CT) {
#pragma unroll
        for (int f = 0; f < 6; f++) Sk[f * CT + q] = N::sto(pf[p][f]);
      }
    }
    if (k < k1) issue(k + 1);
    R vold[3], cf = R();
    if (node_in && do_vel) {
      const int64_t n = (int64_t)k * nplane + nidx0;
      cf = N::ld(a.coef, n);
#pragma unroll
      for (int c = 0; c < 3; c++) vold[c] = N::ld(a.V_in[c], n);
    }
    __syncthreads();

    // ---- B: velocity of node layer k
    St *Vk = sV + (k & 1) * 3 * NT;
    if (node_in) {
      const int ia = ty * CW + tx, ib = ia + 1, ic = ia + CW + 1, id = ia + CW;
      auto cellv = [&](int f, int q) { return N::val(Sk[f * CT + q]); };
      R A, B, C, D;
      // S0: x only
      A = cellv(0, ia); B = cellv(0, ib); C = cellv(0, ic); D = cellv(0, id);
      const R px0 = (B + C) - (A + D);
      A = cellv(1, ia); B = cellv(1, ib); C = cellv(1, ic); D = cellv(1, id);
      const R py1 = (C + D) - (A + B);
      A = cellv(2, ia); B = cellv(2, ib); C = cellv(2, ic); D = cellv(2, id);
      const R s2 = (A + B) + (C + D);
      A = cellv(3, ia); B = cellv(3, ib); C = cellv(3, ic); D = cellv(3, id);
      R ab = A + B, cd = C + D;
      const R py3 = cd - ab, s3 = ab + cd;
      A = cellv(4, ia); B = cellv(4, ib); C = cellv(4, ic); D = cellv(4, id);
      R bc = B + C, ad = A + D;
      const R px4 = bc - ad, s4 = bc + ad;
      A = cellv(5, ia); B = cellv(5, ib); C = cellv(5, ic); D = cellv(5, id);
      const R px5 = (B + C) - (A + D), py5 = (C + D) - (A + B);
      // node derivatives (x: S0,S5,S4  y: S5,S1,S3  z: S4,S3,S2)
      R ax = gx * (vpx0 + px0) + gy * (vpy5 + py5) + gz * (s4 - vs4);
      R ay = gx * (vpx5 + px5) + gy * (vpy1 + py1) + gz * (s3 - vs3);
      R az = gx * (vpx4 + px4) + gy * (vpy3 + py3) + gz * (s2 - vs2);
      vpx0 = px0; vpx4 = px4; vpx5 = px5; vpy1 = py1; vpy3 = py3; vpy5 = py5;
      vs2 = s2; vs3 = s3; vs4 = s4;
      if (do_vel) {
      if (a.f_rng) {  // force sources of this block and layer
        const int2 r = a.f_rng[(int64_t)blk * (nz + 1) + k];
        for (int e = first_local(a.f_key, r.x, r.y, t); e < r.y; e++) {
          const int key = a.f_key[e];
          if ((key & 0xffff) != t) {
            if ((key & 0xffff) > t) break;
            continue;
          }
          const R v = N::val(a.f_w[e]) * N::val(sigrow[a.f_sig[e]]);
          const int d = key >> 16;
          if (d == 0) ax = ax + v;
          else if (d == 1) ay = ay + v;
          else az = az + v;
        }
      }
      R vn[3] = {vold[0], vold[1], vold[2]};
      if (!(cf == R())) {
        vn[0] = vold[0] + cf * ax;
        vn[1] = vold[1] + cf * ay;
        vn[2] = vold[2] + cf * az;
      }
#pragma unroll
      for (int c = 0; c < 3; c++) Vk[c * NT + t] = N::sto(vn[c]);
      if (node_own && own_layer) {
        const int64_t n = (int64_t)k * nplane + nidx0;
#pragma unroll
        for (int c = 0; c < 3; c++) N::st(a.V_out[c], n, vn[c]);
        if (a.s_rng && rec < a.rec_cap) {  // sensor traces
          const int2 r = a.s_rng[(int64_t)blk * (nz + 1) + k];
          for (int e = first_local(a.s_key, r.x, r.y, t); e < r.y; e++) {
            if (a.s_key[e] != t) {
              if (a.s_key[e] > t) break;
              continue;
            }
            double *tr = a.traces + (rec * a.n_sens + a.s_idx[e]) * 3;
            tr[0] = N::dbl(vn[0]);
            tr[1] = N::dbl(vn[1]);
            tr[2] = N::dbl(vn[2]);
          }
        }
      }
      }  // do_vel
    }
    __syncthreads();

    // ---- C: stress of cell layer k-1 (partial sums of node layer k first)
    if (do_vel && tx < TX - 1 && ty < TY - 1) {
      const int ia = t, ib = t + 1, ic = t + TX + 1, id = t + TX;
      R px[3], py[3], s[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const R A = N::val(Vk[c * NT + ia]), B = N::val(Vk[c * NT + ib]);
        const R C = N::val(Vk[c * NT + ic]), D = N::val(Vk[c * NT + id]);
        const R ab = A + B, cd = C + D;
        px[c] = (B + C) - (A + D);
        py[c] = cd - ab;
        s[c] = ab + cd;
      }
      if (k > k0 && cell_own) {
        // d_ij = d/dx_i V_j over the cell of layer k-1
        const R d00 = spx[0] + px[0], d10 = spy[0] + py[0], d20 = s[0] - ss[0];
        const R d01 = spx[1] + px[1], d11 = spy[1] + py[1], d21 = s[1] - ss[1];
        const R d02 = spx[2] + px[2], d12 = spy[2] + py[2], d22 = s[2] - ss[2];
        R e[6];
        e[0] = gx * d00;
        e[1] = gy * d11;
        e[2] = gz * d22;
        e[3] = gy * d12 + gz * d21;
        e[4] = gx * d02 + gz * d20;
        e[5] = gx * d01 + gy * d10;
        const int kc = k - 1;
        const int64_t cg = (int64_t)kc * cplane + cidx0;
        const St *Cm = a.ctab + 36 * (int)a.mat[cg];
        const St *Sprev = sS + (kc + 1) % 3 * 6 * CT;
        const int q = (ty + 1) * CW + tx + 1;
        R acc[6];
#pragma unroll
        for (int f = 0; f < 6; f++) acc[f] = N::val(Sprev[f * CT + q]);
        if (a.m_rng) {  // moment sources of this block and cell layer
          const int2 r = a.m_rng[(int64_t)blk * nz + kc];
          for (int ee = first_local(a.m_key, r.x, r.y, t); ee < r.y; ee++) {
            const int key = a.m_key[ee];
            if ((key & 0xffff) != t) {
              if ((key & 0xffff) > t) break;
              continue;
            }
            const R v = N::val(a.m_w[ee]) * N::val(sigrow[a.m_sig[ee]]);
            const int kk = key >> 16;
#pragma unroll
            for (int f = 0; f < 6; f++)
              if (f == kk) acc[f] = acc[f] + v;
          }
        }
#pragma unroll
        for (int kk = 0; kk < 6; kk++) {
#pragma unroll
          for (int jj = 0; jj < 6; jj++)
            if (c_used(SYM, kk, jj)) acc[kk] = acc[kk] + N::ld(Cm, 6 * kk + jj) * e[jj];
          N::st(a.S_out[kk], cg, acc[kk]);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        spx[c] = px[c];
        spy[c] = py[c];
        ss[c] = s[c];
      }
    }
  }
}

template <typename R, int TX, int TY, int SYM>
__global__ void __launch_bounds__(TX *TY) k_grid_step(const GridArgs<typename GNum<R>::S> a, int step) {
  grid_block<R, TX, TY, SYM>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x, step);
}

// a batch of grid-form members: flat block ids over all members' (x, y, z)
// block grids; block_start is the prefix of the members' block counts
template <typename R, int TX, int TY, int SYM>
__global__ void __launch_bounds__(TX *TY) k_grid_batch(const GridArgs<typename GNum<R>::S> *__restrict__ args,
                                                       const int *__restrict__ block_start, int n_members,
                                                       int step) {
  const int id = blockIdx.x;
  int lo = 0, hi = n_members;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(block_start + mid) <= id) lo = mid;
    else hi = mid;
  }
  const GridArgs<typename GNum<R>::S> a = args[lo];
  const int local = id - __ldg(block_start + lo);
  const int gxc = a.nx / (TX - 1) + 1, gyc = a.ny / (TY - 1) + 1;
  grid_block<R, TX, TY, SYM>(a, local % gxc, (local / gxc) % gyc, local / (gxc * gyc), gxc, step);
}

// per-instantiation, per-device set-up: shared-memory opt-in for the single
// and batch kernels, SM count and resident blocks per SM
template <typename R, int TX, int TY, int SYM>
struct Setup {
  using St = typename GNum<R>::S;
  static constexpr int CT = (TX + 1) * (TY + 1);
  static constexpr size_t smem = sizeof(St) * (3 * 6 * CT + 2 * 3 * TX * TY);
  static cudaError_t ensure(int &sms, int &per_sm) {
    static unsigned long long done = 0;
    static int s_sms[64] = {0}, s_per[64] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int d = dev & 63;
    if (!(done & (1ull << d))) {
      e = cudaFuncSetAttribute(k_grid_step<R, TX, TY, SYM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_grid_batch<R, TX, TY, SYM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s_sms[d], cudaDevAttrMultiProcessorCount, dev);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s_per[d], k_grid_step<R, TX, TY, SYM>, TX * TY, smem);
      if (e != cudaSuccess) return e;
      s_per[d] = s_per[d] > 0 ? s_per[d] : 1;
      done |= 1ull << d;
    }
    sms = s_sms[d];
    per_sm = s_per[d];
    return cudaSuccess;
  }
};

template <typename R, int TX, int TY, int SYM>
cudaError_t launch_t(const GridArgs<typename GNum<R>::S> &a, cudaStream_t st) {
  using S = Setup<R, TX, TY, SYM>;
  int sms = 0, per_sm = 0;
  cudaError_t e = S::ensure(sms, per_sm);
  if (e != cudaSuccess) return e;
  GridArgs<typename GNum<R>::S> b = a;
  const unsigned gx = (unsigned)(a.nx / (TX - 1) + 1), gy = (unsigned)(a.ny / (TY - 1) + 1);
  if (b.kchunk <= 0) b.kchunk = grid_chunk_for(a.nz, (long long)gx * gy, sms, per_sm);
  const dim3 grid(gx, gy, (unsigned)((a.nz + b.kchunk - 1) / b.kchunk));
  k_grid_step<R, TX, TY, SYM><<<grid, TX * TY, S::smem, st>>>(b, 0);
  return cudaGetLastError();
}

template <typename R, int TX, int TY, int SYM>
cudaError_t launch_batch_t(const GridBatchLaunch &b, int step, cudaStream_t st) {
  using S = Setup<R, TX, TY, SYM>;
  int sms = 0, per_sm = 0;
  cudaError_t e = S::ensure(sms, per_sm);
  if (e != cudaSuccess) return e;
  if (b.total_blocks <= 0) return cudaSuccess;
  k_grid_batch<R, TX, TY, SYM><<<b.total_blocks, TX * TY, S::smem, st>>>(
      (const GridArgs<typename GNum<R>::S> *)b.args, b.block_start, b.n_members, step);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_sym(const GridArgs<typename GNum<R>::S> &a, int sym, cudaStream_t st) {
  if (a.nx <= 0 || a.ny <= 0 || a.nz <= 0) return cudaSuccess;
  if (sym == 2) return launch_t<R, 32, 8, 2>(a, st);
  if (sym == 1) return launch_t<R, 32, 8, 1>(a, st);
  return launch_t<R, 32, 8, 0>(a, st);
}

template <typename R>
cudaError_t launch_batch_sym(const GridBatchLaunch &b, int step, cudaStream_t st) {
  if (b.sym == 2) return launch_batch_t<R, 32, 8, 2>(b, step, st);
  if (b.sym == 1) return launch_batch_t<R, 32, 8, 1>(b, step, st);
  return launch_batch_t<R, 32, 8, 0>(b, step, st);
}

}  // namespace


int grid_chunk_for(int nz, long long xy_blocks, int sms, int per_sm) {
  if (nz <= 0) return 1;
  // tuning override: PN_GRID_KCHUNK cell layers per chunk
  if (const char *v = std::getenv("PN_GRID_KCHUNK")) {
    const int k = std::atoi(v);
    if (k > 0) return std::min(std::min(k, kGridChunkMax), nz);
  }
  // Each chunk re-marches two layers (the partial sums below it, the node
  // layer above it), which costs more than a partly empty last wave: split
  // columns only as far as one wave of resident blocks needs.
  const long long want = (long long)sms * per_sm;
  long long chunks = (want + xy_blocks - 1) / xy_blocks;
  chunks = std::max(1LL, std::min(chunks, (long long)std::max(1, nz / 4)));
  chunks = std::max(chunks, (long long)((nz + kGridChunkMax - 1) / kGridChunkMax));
  return (int)((nz + chunks - 1) / chunks);
}

// The blocks of a one-chunk launch run in waves of `slots`; whole columns in
// the last, partial wave keep the GPU as busy as that wave is full (on the
// 400 x 400 x 40 laminate, FP32: 608 columns over 77 us, then the other 146
// alone for 50 us more).  The tiles of that wave get their columns cut into c
// chunks, the c of least modelled time: full waves x (nz + o) + waves of the
// tail's R c chunks x (nz / c + o), o = 4 layers of a block's fixed cost
// (start-up, the re-marched layers at each cut).
void grid_tail_split(int nz, int kchunk, long long tiles, long long slots, int &tail_from, int &tail_chunk) {
  tail_from = 0;
  tail_chunk = 0;
  if (nz <= 1 || kchunk < nz || slots <= 0 || tiles <= slots) return;
  const long long full = tiles / slots * slots, rest = tiles - full;
  if (rest == 0) return;
  int best = 1;
  if (const char *v = std::getenv("PN_GRID_TAIL_CHUNKS")) {
    best = std::max(1, std::min(std::atoi(v), nz));
  } else {
    constexpr double o = 4.0;
    double best_t = 0.0;
    for (int c = 1; c <= std::min(8, nz); c++) {
      const int len = (nz + c - 1) / c;
      const int cc = (nz + len - 1) / len;
      const double waves = (double)((rest * cc + slots - 1) / slots);
      const double t = waves * (len + o);
      if (c == 1 || t < best_t - 1e-9) {
        best_t = t;
        best = c;
      }
    }
  }
  if (best <= 1) return;
  tail_from = (int)full;
  tail_chunk = (nz + best - 1) / best;
}

int grid_chunk_layers(int precision, int nx, int ny, int nz, bool tma, int tile_rows) {
  int sms = 0, per_sm = 0;
  cudaError_t e = precision == 2 ? Setup<float, 32, 8, 0>::ensure(sms, per_sm)
                : precision == 3 ? Setup<df64, 32, 8, 0>::ensure(sms, per_sm)
                                 : Setup<double, 32, 8, 0>::ensure(sms, per_sm);
  if (e != cudaSuccess || nz <= 0) return std::min(std::max(nz, 1), kGridChunkMax);
  if (!tma) tile_rows = kGridTileRows;
  if (tma) {
    const int p = grid_tma_blocks_per_sm(precision, tile_rows);
    if (p > 0) per_sm = p;
  }
  const long long xy = (long long)(nx / (kGridTileX - 1) + 1) * (ny / (tile_rows - 1) + 1);
  return grid_chunk_for(nz, xy, sms, per_sm);
}

cudaError_t launch_grid_f32(const GridArgs<float> &a, int sym, cudaStream_t st) {
  return launch_sym<float>(a, sym, st);
}
cudaError_t launch_grid_f64(const GridArgs<double> &a, int sym, cudaStream_t st) {
  return launch_sym<double>(a, sym, st);
}
cudaError_t launch_grid_df64(const GridArgs<float2> &a, int sym, cudaStream_t st) {
  return launch_sym<df64>(a, sym, st);
}
cudaError_t launch_grid_batch(const GridBatchLaunch &b, int precision, int step, cudaStream_t st) {
  if (precision == 2) return launch_batch_sym<float>(b, step, st);
  if (precision == 3) return launch_batch_sym<df64>(b, step, st);
  return launch_batch_sym<double>(b, step, st);
}

}  // namespace pn
