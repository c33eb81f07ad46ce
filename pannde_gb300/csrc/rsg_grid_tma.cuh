// rsg_grid_tma.cuh -- the fused voxel-grid step with tensor-copy (TMA) staging
// (templates; rsg_grid_tma.cu instantiates 32 x 8 tiles for every storage
// type plus the dispatch and the tensor-map encoding, rsg_grid_tma16.cu 32 x 16
// tiles for FP32 storage).
//
// Same arithmetic as rsg_grid.cu (a block owns a 31 x (TY-1) column of nodes
// and cells over a chunk of layers; its 32 x TY threads are the nodes plus a
// one-node apron on +x / +y; TY = 8 or 16 rows), but every per-layer input
// tile arrives in shared memory by cp.async.bulk.tensor, issued by one thread
// one layer ahead and completed on an mbarrier:
//   slot ring (4 layers)    S_in[6] cell tile (33 x (TY+1) used, x rounded down
//                           to the 16-byte boundary), material tile (31 x (TY-1))
//   node ring (2 layers)    V_in[3] and coef node tiles (32 x TY used)
// No thread holds prefetched values in registers and the loads never stall an
// instruction stream; out-of-lattice elements arrive as zeros (the tensor
// copy's fill), which is the void-site value.
//
// One __syncthreads per layer: iteration k runs
//   B(k)    velocity of node layer k from cell layers k-1 (partial sums in
//           registers) and k (slot k), written to the computed-velocity tile
//           k&1 and, for owned nodes, to V_out (HostRSGTDUT.hpp:338-362)
//   C(k-2)  stress of cell layer k-2 from node layers k-2 (partial sums in
//           registers) and k-1 (computed tile (k-1)&1, complete since the
//           previous barrier) (HostRSGTDUT.hpp:278-293)
// and the first thread of the last warp (the tile's apron row, which has no
// stress half) first issues the copies of layer k+1 into its slot, whose
// previous layer was last read before the previous barrier.
//
// A single solver's launch is the 3D grid (x tiles, y tiles, z chunks), or,
// when whole columns leave a last partial wave of resident blocks, a 1D grid
// whose last wave's columns are cut into shorter chunks (block_coords).  The
// sparse sources and sensors of a (tile, layer) slot are sorted by node: a
// thread finds its own by a binary search in a long slot.
//
// Every wait is bounded (about one second of %globaltimer); a wait that gives
// up records an error word for the host, the block drains its own copies in
// flight (again bounded) and returns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "df64.cuh"
#include "rsg_common.cuh"
#include "rsg_grid.cuh"

namespace pn {
namespace {

constexpr int TX = 32;  // a tile row is one warp
constexpr int KC_MAX = kGridChunkMax;  // cell layers per chunk (source-range staging)
constexpr int ROWS_MAX = kGridTmaRowsMax;

struct GridMaps {
  CUtensorMap S[6];
  CUtensorMap V[3];
  CUtensorMap coef;
  CUtensorMap mat;
};

// shared-memory geometry for a storage element of ESZ bytes.  Copies run PD
// layers ahead of the layer being computed.  A layer's stress tile is read in
// its own iteration (velocity half) and, with OWN_SMEM, two iterations later
// (a cell's old stress in the stress half; without it that value comes from
// global memory, mostly L2, which needs fewer slots: the room for a third
// block per SM with 8-byte storage).  Slots per ring: stress PD + 1 (+ 2 with
// OWN_SMEM), velocity + dt/rho PD + 1, material PD + 3 (read in the stress
// half, two iterations after its layer's).
#ifndef PN_GRID_F32_OWN_STRESS
#define PN_GRID_F32_OWN_STRESS 1  // FP32: old stress from the tile (four stress slots)
#endif
#ifndef PN_GRID_F32_MIN_BLOCKS
#define PN_GRID_F32_MIN_BLOCKS 0  // FP32: resident blocks per SM the kernel is compiled for
#endif
template <int ESZ, int TY>
struct Geo {
  static constexpr int NT = TX * TY;
  static constexpr int PD = 1;
  static constexpr bool OWN_SMEM = ESZ == 4 && PN_GRID_F32_OWN_STRESS;
  static constexpr int NS = PD + 1 + (OWN_SMEM ? 2 : 0);
  static constexpr int NV = PD + 1;
  static constexpr int NM = PD + 3;
  static constexpr int A = 16 / ESZ;              // x alignment of a copy (elements)
  static constexpr int BWC = ESZ == 4 ? 36 : 34;  // cell tile width: offset (< A) + 33
  static constexpr int BWN = ESZ == 4 ? 36 : 34;  // node tile width: offset (< A) + 32
  static constexpr int BWM = 48;                  // material tile width: offset (< 16) + 31
  static constexpr int SBOX_BYTES = BWC * (TY + 1) * ESZ;
  static constexpr int SBOX = (SBOX_BYTES + 127) / 128 * 128;
  static constexpr int VBOX = BWN * TY * ESZ;
  static constexpr int MBOX_BYTES = BWM * (TY - 1);
  static constexpr int MBOX = (MBOX_BYTES + 127) / 128 * 128;
  static constexpr int SLOT = 6 * SBOX;                        // S[6] of one layer
  static constexpr int VSLOT = 4 * VBOX;                       // V[3], dt/rho of one layer
  static constexpr uint32_t TX_BYTES = 6 * SBOX_BYTES + 4 * VBOX + MBOX_BYTES;
  static constexpr int OFF_V = NS * SLOT;                      // velocity ring [NV]
  static constexpr int OFF_M = OFF_V + NV * VSLOT;             // material ring [NM]
  static constexpr int OFF_VT = OFF_M + NM * MBOX;             // computed velocity [2][3][NT]
  static constexpr int OFF_C = OFF_VT + 2 * 3 * NT * ESZ;      // dt*C rows [ROWS_MAX][36]
  static constexpr int OFF_R = OFF_C + ROWS_MAX * 36 * ESZ;    // ranges f, s [KC_MAX+2], m [KC_MAX]
  static constexpr int OFF_B = OFF_R + (3 * KC_MAX + 4) * 8;   // mbarriers [NS]
  static constexpr int BYTES = OFF_B + NS * 8;
  static constexpr size_t SMEM = BYTES + 128;                  // + base alignment
  static_assert(SLOT % 128 == 0 && VBOX % 128 == 0 && OFF_V % 128 == 0 && OFF_M % 128 == 0 && OFF_B % 8 == 0,
                "alignment");
  static_assert(SBOX % ESZ == 0 && VBOX % ESZ == 0, "element size");
};

// Kinds of step: K picks the arithmetic type R, the storage type S of global
// memory and of the tensor copies, and the type T of the shared tiles the
// block itself writes or converts (computed velocities, stiffness rows, and
// for df64d the stress slots):
//   float / double / df64   R, S and T alike (df64 stored as float2)
//   df64d                   the FP64 form's double-float path: S double, R
//                           df64, T float2 -- loads split doubles exactly
//                           (split_double), stores join them (join_double),
//                           stress tiles are split in place once per layer
struct df64d {};
template <typename K> struct GNum;
template <> struct GNum<float> {
  using S = float;
  using T = float;
  using R = float;
  static constexpr bool SPLIT = false;
  static __device__ __forceinline__ float ld(const float *p, int64_t i) { return __ldg(p + i); }
  static __device__ __forceinline__ float val(float v) { return v; }
  static __device__ __forceinline__ float tval(float v) { return v; }
  static __device__ __forceinline__ float tsto(float v) { return v; }
  static __device__ __forceinline__ void st(float *p, int64_t i, float v) { p[i] = v; }
  static __device__ __forceinline__ double dbl(float v) { return (double)v; }
};
template <> struct GNum<double> {
  using S = double;
  using T = double;
  using R = double;
  static constexpr bool SPLIT = false;
  static __device__ __forceinline__ double ld(const double *p, int64_t i) { return __ldg(p + i); }
  static __device__ __forceinline__ double val(double v) { return v; }
  static __device__ __forceinline__ double tval(double v) { return v; }
  static __device__ __forceinline__ double tsto(double v) { return v; }
  static __device__ __forceinline__ void st(double *p, int64_t i, double v) { p[i] = v; }
  static __device__ __forceinline__ double dbl(double v) { return v; }
};
template <> struct GNum<df64> {
  using S = float2;
  using T = float2;
  using R = df64;
  static constexpr bool SPLIT = false;
  static __device__ __forceinline__ df64 ld(const float2 *p, int64_t i) {
    const float2 v = __ldg(p + i);
    return df64(v.x, v.y);
  }
  static __device__ __forceinline__ df64 val(float2 v) { return df64(v.x, v.y); }
  static __device__ __forceinline__ df64 tval(float2 v) { return df64(v.x, v.y); }
  static __device__ __forceinline__ float2 tsto(df64 v) { return make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ void st(float2 *p, int64_t i, df64 v) { p[i] = make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ double dbl(df64 v) { return (double)v.hi + (double)v.lo; }
};
// stores of the FP64 form's double-float path: 1 joins on the integer and
// FP32 pipes (join_double_int), 0 on the FP64 unit (join_double)
#ifndef PN_F64H_JOIN_INT
#define PN_F64H_JOIN_INT 1
#endif
// The path's increments onto the stored doubles: PN_F64H_ADD_PAIR 1 by the
// pair's exact halves and two FP64 adds (add_pair: fewer instructions, two
// FP64-pipe operations), 0 by one join on the integer pipe and one FP64 add.
// Measured on the laminate: with no FP64-path blocks (a developed state) the
// two adds are faster (0.495 against 0.531 ms per step), with 15% of the
// blocks on the FP64 path (the burst's first steps), whose FP64 pipe is then
// busy, the join (0.571 against 0.600 ms).  Choosing per step from the
// previous step's path counts was slower than either (0.584 / 0.544 ms): the
// kernel then carries both.  With edge-aware path flags (fewer FP64 blocks)
// the join measured 0.529 / 0.531 ms against 0.588 / 0.528: the join is the
// default.
#ifndef PN_F64H_ADD_PAIR
#define PN_F64H_ADD_PAIR 0
#endif
__device__ __forceinline__ double add_increment(double base, df64 inc) {
  if (PN_F64H_ADD_PAIR) return add_pair(base, inc);
  return __dadd_rn(base, PN_F64H_JOIN_INT ? join_double_int(inc) : join_double(inc));
}
template <> struct GNum<df64d> {
  using S = double;
  using T = float2;
  using R = df64;
  static constexpr bool SPLIT = true;
  static __device__ __forceinline__ double join(df64 v) {
    return PN_F64H_JOIN_INT ? join_double_int(v) : join_double(v);
  }
  static __device__ __forceinline__ df64 ld(const double *p, int64_t i) { return split_double(__ldg(p + i)); }
  static __device__ __forceinline__ df64 val(double v) { return split_double(v); }
  static __device__ __forceinline__ df64 tval(float2 v) { return df64(v.x, v.y); }
  static __device__ __forceinline__ float2 tsto(df64 v) { return make_float2(v.hi, v.lo); }
  static __device__ __forceinline__ void st(double *p, int64_t i, df64 v) { p[i] = join(v); }
  static __device__ __forceinline__ double dbl(df64 v) { return join(v); }
};

__host__ __device__ constexpr bool c_used(int sym, int k, int j) {
  return sym == 0 ? true
       : sym == 2 ? ((k < 3 && j < 3) || k == j)
                  : ((k < 3 && j < 3) || k == j || (k == 5 && j < 3) || (j == 5 && k < 3) ||
                     (k == 3 && j == 4) || (k == 4 && j == 3));
}

// ---- PTX wrappers: mbarrier, tensor copy, timer -------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// wait for phase `parity` of the barrier; false after about one second (the
// loop out of line: the first try usually succeeds)
__device__ __noinline__ bool mbar_wait_slow(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  for (uint32_t n = 1;; n++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63) == 0 && global_ns() - t0 > 1000000000ull) return false;
  }
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  return mbar_try_wait(bar, parity) || mbar_wait_slow(bar, parity);
}
// the whole wait out of line (fewer registers live across it: the batch
// kernel, which reads its arguments through global memory)
__device__ __noinline__ bool mbar_wait_call(uint32_t bar, uint32_t parity) {
  return mbar_try_wait(bar, parity) || mbar_wait_slow(bar, parity);
}
__device__ __forceinline__ void proxy_fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_prefetch_map(const void *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void *map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ int floor_to(int v, int m) {  // largest multiple of m <= v (m > 0)
  return v >= 0 ? v / m * m : -((-v + m - 1) / m) * m;
}

// error word codes
constexpr int32_t kErrWait = 1;

// RANGE (the FP64 form's kernel): every V and S value the block stores is
// tested against the double-float range, and a block that stored one outside
// it marks its tile for the FP64 path in the next step (range_flags_write).
template <typename K, int SYM, int TY, bool BATCH = false, bool RANGE = false>
__device__ __forceinline__ void grid_block_tma(const GridArgs<typename GNum<K>::S> &a, const GridMaps *M,
                                               int bx, int by, int k0, int kc, int gxc, int step) {
  using N = GNum<K>;
  using R = typename N::R;
  using St = typename N::S;
  using Sm = typename N::T;
  static_assert(sizeof(Sm) == sizeof(St), "shared tiles hold one storage element per value");
  using G = Geo<(int)sizeof(St), TY>;
  constexpr int NT = G::NT;
  // SYM: material symmetry class (bits 0-1, see c_used) | 4 when the lattice is
  // cubic and 0.25/h has been folded into the coefficients (g = 1)
  constexpr bool CUBIC = (SYM & 4) != 0;
  constexpr int SB = G::SBOX / (int)sizeof(St);  // field stride in a slot (elements)
  constexpr int VB = G::VBOX / (int)sizeof(St);
  extern __shared__ unsigned char smem_raw[];
  // 128-byte aligned base.  A single launch derives it from smem_raw by an
  // offset, so that every tile pointer stays in the shared state space (shared
  // loads and stores, 32-bit addressing: FP32 45.4 -> 47.8, double-float 18.0
  // -> 19.3 Gcell-steps/s on the laminate).  The batch kernel, which reads its
  // arguments through global memory, spilled with that and ran slower; it keeps
  // the generic pointer.
  unsigned char *base = BATCH ? (unsigned char *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127)
                              : smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  Sm *sVt = reinterpret_cast<Sm *>(base + G::OFF_VT);
  Sm *sC = reinterpret_cast<Sm *>(base + G::OFF_C);
  int2 *sRf = reinterpret_cast<int2 *>(base + G::OFF_R);
  int2 *sRs = sRf + (KC_MAX + 2);
  int2 *sRm = sRs + (KC_MAX + 2);
  const uint32_t bars = smem_u32(base + G::OFF_B);

  const int t = threadIdx.x;
  const int tx = t % TX, ty = t / TX;
  const int i0 = bx * (TX - 1), j0 = by * (TY - 1);
  const int blk = by * gxc + bx;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int i = i0 + tx, j = j0 + ty;
  const bool node_own = (i <= nx) && (j <= ny) && tx < TX - 1 && ty < TY - 1;
  const bool cell_own = tx < TX - 1 && ty < TY - 1 && i < nx && j < ny;
  const int64_t nplane = (int64_t)a.pnx * (ny + 1), cplane = (int64_t)a.pcx * ny;
  const int64_t nidx0 = (int64_t)j * a.pnx + i;
  const int64_t cidx0 = (int64_t)j * a.pcx + i;
  const R gx = N::val(a.g[0]), gy = N::val(a.g[1]), gz = N::val(a.g[2]);
  const St *sigrow = a.sigval ? a.sigval + (int64_t)min(step, a.sig_rows - 1) * a.sig_stride : nullptr;
  const int64_t rec = a.rec + step;
  // columns of the tile (and its apron) hold no solid cell at or above ktop:
  // the march ends there, and a chunk above it has nothing to do
  const int ktop = a.ktop ? min(nz, __ldg(a.ktop + blk)) : nz;
  const int k1 = min(ktop, k0 + kc);
  if (k0 >= ktop) return;
  const bool last_chunk = k1 == ktop;

  // tile origins of the copies (x on the 16-byte boundary) and offsets in them
  const int xs_c = floor_to(i0 - 1, G::A), oc = i0 - 1 - xs_c;
  const int xs_n = floor_to(i0, G::A), on = i0 - xs_n;
  const int xs_m = floor_to(i0, 16), om = i0 - xs_m;

  // layer L is copy number u = L - k0 + 1 of the block: stress slot and
  // mbarrier u % NS (phase (u / NS) & 1), velocity slot u % NV, material slot u % NM
  auto ucount = [&](int L) { return (uint32_t)(L - k0 + 1); };
  auto sslot = [&](int L) { return base + (ucount(L) % G::NS) * G::SLOT; };
  auto vslot = [&](int L) { return base + G::OFF_V + (ucount(L) % G::NV) * G::VSLOT; };
  auto mslot = [&](int L) { return base + G::OFF_M + (ucount(L) % G::NM) * G::MBOX; };
  auto bar_of = [&](int L) { return bars + 8u * (ucount(L) % G::NS); };
  auto parity = [&](int L) { return (ucount(L) / G::NS) & 1u; };
  // The chunk's first layer k0 - 1 gives only the partial sums of its cell
  // layer (stress boxes); no node velocity or cell stress of it is computed
  // here, so its velocity, dt/rho and material boxes are not copied.  The top
  // layer k1 gives the velocity of node layer k1 but no cell stress: no
  // material box.  (A chunk above the lattice's first layer re-reads two
  // layers; these are the bytes of them it does not need.)
  auto issue = [&](int L) {  // the issuing thread: copies of layer L
    if (L == a.test_skip_layer) return;  // failure-path test: this layer's wait runs out
    const uint32_t bar = bar_of(L);
    unsigned char *sl = sslot(L), *vl = vslot(L);
    const bool first = L == k0 - 1, top = L == k1;
    mbar_expect_tx(bar, first ? 6u * G::SBOX_BYTES : top ? G::TX_BYTES - G::MBOX_BYTES : G::TX_BYTES);
#pragma unroll
    for (int f = 0; f < 6; f++) tma_load_3d(smem_u32(sl + f * G::SBOX), &M->S[f], xs_c, j0 - 1, L, bar);
    if (first) return;
#pragma unroll
    for (int c = 0; c < 3; c++) tma_load_3d(smem_u32(vl + c * G::VBOX), &M->V[c], xs_n, j0, L, bar);
    tma_load_3d(smem_u32(vl + 3 * G::VBOX), &M->coef, xs_n, j0, L, bar);
    if (!top) tma_load_3d(smem_u32(mslot(L)), &M->mat, xs_m, j0, L, bar);
  };

  if (t == 0) {
#pragma unroll
    for (int f = 0; f < 6; f++) tma_prefetch_map(&M->S[f]);
#pragma unroll
    for (int c = 0; c < 3; c++) tma_prefetch_map(&M->V[c]);
    tma_prefetch_map(&M->coef);
    tma_prefetch_map(&M->mat);
#pragma unroll
    for (int s = 0; s < G::NS; s++) mbar_init(bars + 8u * s, 1);
    mbar_init_fence();
  }
  // per-chunk tables: stiffness rows, source and sensor ranges
  for (int q = t; q < a.n_rows * 36; q += NT) sC[q] = N::tsto(N::val(a.ctab[q]));
  const int nL = k1 - k0 + 2;  // node layers k0-1 .. k1
  for (int q = t; q < nL; q += NT) {
    const int k = k0 - 1 + q;
    const bool ok = k >= 0 && k <= nz;
    sRf[q] = (a.f_rng && ok) ? a.f_rng[(int64_t)blk * (nz + 1) + k] : make_int2(0, 0);
    sRs[q] = (a.s_rng && ok) ? a.s_rng[(int64_t)blk * (nz + 1) + k] : make_int2(0, 0);
  }
  for (int q = t; q < k1 - k0; q += NT) sRm[q] = a.m_rng ? a.m_rng[(int64_t)blk * nz + k0 + q] : make_int2(0, 0);
  __syncthreads();
  // the copies are issued (and, on failure, drained) by the first thread of
  // the last warp: its row is the tile's apron, which has no stress half
  constexpr int ISSUER = (TY - 1) * TX;
  if (t == ISSUER) {
#pragma unroll
    for (int d = 0; d <= G::PD; d++)
      if (k0 - 1 + d <= k1) issue(k0 - 1 + d);
  }
  // split the stress slot of layer L in place (df64d): each stored double
  // becomes its double-float pair, so the velocity half reads pairs; the
  // slot is waited for first (false: the wait gave up).  Two elements per
  // 16-byte shared access over the whole slot (6 fields x SB elements, SB
  // even; the few padding elements past each box are split too and never read)
  auto split_slot = [&](int L) {
    if (!mbar_wait(bar_of(L), parity(L))) return false;
    double2 *sl = reinterpret_cast<double2 *>(sslot(L));
    static_assert(SB % 2 == 0, "pairs of elements");
    for (int q = t; q < 3 * SB; q += NT) {
      const double2 d = sl[q];
      const df64 u = split_double(d.x), w = split_double(d.y);
      reinterpret_cast<float4 *>(sl)[q] = make_float4(u.hi, u.lo, w.hi, w.lo);
    }
    return true;
  };

  // per cell layer: A = (x, y differences) + z sum, B = the same - z sum; a
  // node's acceleration is A of the layer above + B of the layer below
  R blx = R(), bly = R(), blz = R();  // B of the layer below
  using L = typename Lazy<R>::type;  // pair differences before renormalisation
  L spx[3], spy[3], ss[3];
#pragma unroll
  for (int c = 0; c < 3; c++) spx[c] = spy[c] = ss[c] = L();
  const int ra = ty * G::BWC + oc + tx;  // cell (i-1, j-1) in the cell tile
  const int rv = ty * G::BWN + on + tx;  // node (i, j) in the node tile
  int waited = k0 - 2;                   // last layer this thread has waited for
  bool fail = false;
  // RANGE: where this block stored values outside the double-float range, as
  // the bits its neighbours read (1 any; 2 / 4 the first / last owned column,
  // 8 / 16 the first / last owned row -- the edges inside another tile's
  // boxes: nodes are read at the first column and row, cells at all four)
  uint32_t oorb = 0;
  const uint32_t vbits = 1u | (tx == 0 ? 2u : 0u) | (ty == 0 ? 8u : 0u);
  const uint32_t sbits = vbits | (tx == TX - 2 ? 4u : 0u) | (ty == TY - 2 ? 16u : 0u);
  // a double value into double storage (RANGE: tested against the velocity
  // range, field 0, or the stress range, field 1); generic, so that it is
  // instantiated only where called (double storage)
  auto store_d = [&](auto *p, int64_t i, double d, int field) {
    if constexpr (RANGE)
      if (!in_df64_range(d, (uint32_t)(field ? a.r_elo_s : a.r_elo), (uint32_t)(field ? a.r_ehi_s : a.r_ehi)))
        oorb |= field ? sbits : vbits;
    p[i] = d;
  };
  auto store = [&](St *p, int64_t i, R v, int field) {
    if constexpr (RANGE) store_d(p, i, N::dbl(v), field);
    else N::st(p, i, v);
  };

  if constexpr (N::SPLIT) {
    bool ok = split_slot(k0 - 1);
    if (ok) waited = k0 - 1;
    if (__syncthreads_or(!ok)) {
      if (t == ISSUER) {
        if (a.err) atomicExch(a.err, kErrWait);
        for (int L = k0; L <= min(k1, k0 - 1 + G::PD); L++) (void)mbar_wait(bar_of(L), parity(L));
      }
      return;
    }
  }

  // FP32 storage: two layers per unrolled body, so the values carried from
  // one layer to the next alternate registers instead of moving
#pragma unroll(sizeof(St) == 4 ? 2 : 1)
  for (int k = k0 - 1; k <= k1 + 1; k++) {
    if (t == ISSUER && k >= k0 && k + G::PD <= k1) {
      proxy_fence_async_smem();
      issue(k + G::PD);
    }
    // ---- B: velocity of node layer k
    if (k <= k1) {
      if (BATCH ? mbar_wait_call(bar_of(k), parity(k)) : mbar_wait(bar_of(k), parity(k))) waited = k;
      else fail = true;
      const Sm *Sk = reinterpret_cast<const Sm *>(sslot(k));
      auto cellv = [&](int f, int q) { return N::tval(Sk[f * SB + q]); };
      const int ib = ra + 1, id = ra + G::BWC, ic = id + 1;
      R A, B, C, D;
      A = cellv(0, ra); B = cellv(0, ib); C = cellv(0, ic); D = cellv(0, id);
      const L px0 = diff22_u(B, C, A, D);
      A = cellv(1, ra); B = cellv(1, ib); C = cellv(1, ic); D = cellv(1, id);
      const L py1 = diff22_u(C, D, A, B);
      A = cellv(2, ra); B = cellv(2, ib); C = cellv(2, ic); D = cellv(2, id);
      const L s2 = sum22_u(A, B, C, D);
      A = cellv(3, ra); B = cellv(3, ib); C = cellv(3, ic); D = cellv(3, id);
      L py3, s3;
      diffsum22_u(A, B, C, D, py3, s3);
      A = cellv(4, ra); B = cellv(4, ib); C = cellv(4, ic); D = cellv(4, id);
      L px4, s4;
      diffsum22_u(A, D, B, C, px4, s4);
      A = cellv(5, ra); B = cellv(5, ib); C = cellv(5, ic); D = cellv(5, id);
      L px5, py5;
      diffdiff22_u(A, B, C, D, px5, py5);
      // x: Sxx along x, Sxy along y, Sxz along z; y: Sxy, Syy, Syz; z: Sxz, Syz, Szz
      R tx, ty, tz, ax, ay, az, nbx, nby, nbz;
      L axu, ayu, azu;  // A of this layer (renormalised when B of the layer below joins)
      if constexpr (CUBIC) {  // 0.25/h folded into dt/rho and the force weights
        tx = add_uu(px0, py5);
        ty = add_uu(px5, py1);
        tz = add_uu(px4, py3);
        axu = add_unnorm(to_u(tx), s4);
        ayu = add_unnorm(to_u(ty), s3);
        azu = add_unnorm(to_u(tz), s2);
        nbx = sub_uu(to_u(tx), s4);
        nby = sub_uu(to_u(ty), s3);
        nbz = sub_uu(to_u(tz), s2);
      } else {
        tx = madd(gy, norm_u(py5), gx * norm_u(px0));
        ty = madd(gy, norm_u(py1), gx * norm_u(px5));
        tz = madd(gy, norm_u(py3), gx * norm_u(px4));
        const R n4 = norm_u(s4), n3 = norm_u(s3), n2 = norm_u(s2);
        axu = to_u(madd(gz, n4, tx));
        ayu = to_u(madd(gz, n3, ty));
        azu = to_u(madd(gz, n2, tz));
        nbx = madd(-gz, n4, tx);
        nby = madd(-gz, n3, ty);
        nbz = madd(-gz, n2, tz);
      }
      if (k >= k0) {
        ax = add_uu(axu, to_u(blx));
        ay = add_uu(ayu, to_u(bly));
        az = add_uu(azu, to_u(blz));
        const int2 fr = sRf[k - k0 + 1];
        // this node's force sources (the batch kernel scans its slots whole:
        // the searches cost it registers for a fourth block per SM)
        for (int e = BATCH ? fr.x : first_local(a.f_key, fr.x, fr.y, t); e < fr.y; e++) {
          const int key = __ldg(a.f_key + e);
          if ((key & 0xffff) != t) {
            if (!BATCH && (key & 0xffff) > t) break;
            continue;
          }
          const R w = N::val(a.f_w[e]), sg = N::val(sigrow[__ldg(a.f_sig + e)]);
          const int d = key >> 16;
          if (d == 0) ax = madd(w, sg, ax);
          else if (d == 1) ay = madd(w, sg, ay);
          else az = madd(w, sg, az);
        }
        const St *Vk = reinterpret_cast<const St *>(vslot(k));
        R vn[3];
        double vd[3];  // split storage: the new velocity as stored and recorded
        // dt/rho is 0 at void and padding sites, whose differences are 0 too:
        // the update leaves them unchanged without a branch
        const R cf = N::val(Vk[3 * VB + rv]);
        if constexpr (N::SPLIT) {
          // the increment in double-float, added to the stored double by one
          // FP64 add: the old value enters exactly (a node the step leaves
          // alone keeps its bits), and only the new one is split, for the
          // stress half
          const R acc3[3] = {ax, ay, az};
#pragma unroll
          for (int c = 0; c < 3; c++) {
            vd[c] = add_increment((double)Vk[c * VB + rv], cf * acc3[c]);
            vn[c] = split_double(vd[c]);
          }
        } else {
#pragma unroll
          for (int c = 0; c < 3; c++) vn[c] = N::val(Vk[c * VB + rv]);
          vn[0] = madd(cf, ax, vn[0]);
          vn[1] = madd(cf, ay, vn[1]);
          vn[2] = madd(cf, az, vn[2]);
        }
        Sm *Vt = sVt + (k & 1) * 3 * NT;
#pragma unroll
        for (int c = 0; c < 3; c++) Vt[c * NT + t] = N::tsto(vn[c]);
        if (node_own && (k < k1 || last_chunk)) {
          const int64_t n = (int64_t)k * nplane + nidx0;
          // the value stored and recorded
          auto out = [&](int c) -> double {
            if constexpr (N::SPLIT) return vd[c];
            else return N::dbl(vn[c]);
          };
          if constexpr (N::SPLIT) {
#pragma unroll
            for (int c = 0; c < 3; c++) store_d(a.V_out[c], n, out(c), 0);
          } else {
#pragma unroll
            for (int c = 0; c < 3; c++) store(a.V_out[c], n, vn[c], 0);
          }
          const int2 sr = sRs[k - k0 + 1];
          if (rec < a.rec_cap) {
            for (int e = BATCH ? sr.x : first_local(a.s_key, sr.x, sr.y, t); e < sr.y; e++) {  // sensor traces
              const int lk = __ldg(a.s_key + e);
              if (lk != t) {
                if (!BATCH && lk > t) break;
                continue;
              }
              double *tr = a.traces + (rec * a.n_sens + __ldg(a.s_idx + e)) * 3;
              tr[0] = out(0);
              tr[1] = out(1);
              tr[2] = out(2);
            }
          }
        }
      }
      blx = nbx;
      bly = nby;
      blz = nbz;
    }

    // ---- C: partial sums of node layer k-1, stress of cell layer k-2
    if (k - 1 >= k0 && k - 1 <= k1 && tx < TX - 1 && ty < TY - 1) {
      const Sm *Vt = sVt + ((k - 1) & 1) * 3 * NT;
      const int ia = t, ib = t + 1, ic = t + TX + 1, id = t + TX;
      L px[3], py[3], s[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const R A = N::tval(Vt[c * NT + ia]), B = N::tval(Vt[c * NT + ib]);
        const R C = N::tval(Vt[c * NT + ic]), D = N::tval(Vt[c * NT + id]);
        px[c] = diff22_u(B, C, A, D);
        diffsum22_u(A, B, C, D, py[c], s[c]);
      }
      const int kc = k - 2;
      if (kc >= k0 && cell_own) {
        R e[6];
        if constexpr (CUBIC) {  // 0.25/h folded into dt*C
          e[0] = add_uu(spx[0], px[0]);
          e[1] = add_uu(spy[1], py[1]);
          e[2] = sub_uu(s[2], ss[2]);
          // shear: two layer sums, each left unnormalised, and one renormalised add
          e[3] = add_uu(add_unnorm(spy[2], py[2]), sub_unnorm(s[1], ss[1]));
          e[4] = add_uu(add_unnorm(spx[2], px[2]), sub_unnorm(s[0], ss[0]));
          e[5] = add_uu(add_unnorm(spx[1], px[1]), add_unnorm(spy[0], py[0]));
        } else {
          const R d00 = add_uu(spx[0], px[0]), d10 = add_uu(spy[0], py[0]), d20 = sub_uu(s[0], ss[0]);
          const R d01 = add_uu(spx[1], px[1]), d11 = add_uu(spy[1], py[1]), d21 = sub_uu(s[1], ss[1]);
          const R d02 = add_uu(spx[2], px[2]), d12 = add_uu(spy[2], py[2]), d22 = sub_uu(s[2], ss[2]);
          e[0] = gx * d00;
          e[1] = gy * d11;
          e[2] = gz * d22;
          e[3] = madd(gz, d21, gy * d12);
          e[4] = madd(gz, d20, gx * d02);
          e[5] = madd(gy, d10, gx * d01);
        }
        const int64_t cg = (int64_t)kc * cplane + cidx0;
        const int row = mslot(kc)[ty * G::BWM + om + tx];
        const Sm *Cm = sC + 36 * row;
        R acc[6];  // the cell's stress before the update (split storage: its increment)
        if constexpr (N::SPLIT) {  // the old stress joins at the store, by one FP64 add
#pragma unroll
          for (int f = 0; f < 6; f++) acc[f] = R();
        } else if constexpr (G::OWN_SMEM) {
          const Sm *Sc = reinterpret_cast<const Sm *>(sslot(kc));
          const int own = ra + G::BWC + 1;  // cell (i, j)
#pragma unroll
          for (int f = 0; f < 6; f++) acc[f] = N::tval(Sc[f * SB + own]);
        } else {  // in L2: its tile was copied two layers ago
#pragma unroll
          for (int f = 0; f < 6; f++) acc[f] = N::ld(a.S_in[f], cg);
        }
        const int2 mr = sRm[kc - k0];
        for (int ee = BATCH ? mr.x : first_local(a.m_key, mr.x, mr.y, t); ee < mr.y; ee++) {  // this cell's moments
          const int key = __ldg(a.m_key + ee);
          if ((key & 0xffff) != t) {
            if (!BATCH && (key & 0xffff) > t) break;
            continue;
          }
          const R w = N::val(a.m_w[ee]), sg = N::val(sigrow[__ldg(a.m_sig + ee)]);
          const int kk = key >> 16;
#pragma unroll
          for (int f = 0; f < 6; f++)
            if (f == kk) acc[f] = madd(w, sg, acc[f]);
        }
        // 8-byte arithmetic: when every active lane's row is orthotropic
        // (C11..C33 block and the shear diagonal only: a laminate's 0/90 plies
        // beside its +-45 ones), the 12-term product; the others are zero, so
        // the result is the same bits.  FP64 (bound by the FP64 pipe) 4.93 ->
        // 5.01, double-float 20.4 -> 21.0 Gcell-steps/s; FP32 measured no gain.
        bool ortho = (SYM & 3) == 2;
        if constexpr ((SYM & 3) != 2 && !std::is_same<R, float>::value)
          ortho = __all_sync(__activemask(), (a.ortho_rows >> row) & 1u);
        // one row of the stiffness product (double-float: one renormalisation per row)
        auto prod_row = [&](int kk, int cls) {
          if constexpr (std::is_same<R, df64>::value) {
            df64_acc sacc = acc_start(acc[kk]);
#pragma unroll
            for (int jj = 0; jj < 6; jj++)
              if (c_used(cls, kk, jj)) acc_madd(sacc, N::tval(Cm[6 * kk + jj]), e[jj]);
            acc[kk] = acc_end(sacc);
          } else {
#pragma unroll
            for (int jj = 0; jj < 6; jj++)
              if (c_used(cls, kk, jj)) acc[kk] = madd(N::tval(Cm[6 * kk + jj]), e[jj], acc[kk]);
          }
          if constexpr (N::SPLIT)
            store_d(a.S_out[kk], cg, add_increment(__ldg(a.S_in[kk] + cg), acc[kk]), 1);
          else store(a.S_out[kk], cg, acc[kk], 1);
        };
        if (ortho) {
#pragma unroll
          for (int kk = 0; kk < 6; kk++) prod_row(kk, 2);
        } else {
#pragma unroll
          for (int kk = 0; kk < 6; kk++) prod_row(kk, SYM & 3);
        }
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        spx[c] = px[c];
        spy[c] = py[c];
        ss[c] = s[c];
      }
    }
    if constexpr (N::SPLIT) {
      // layer k+1 (copied since the start of this iteration; its slot's
      // previous layer k-1 is no longer read) becomes pairs for the next one
      if (k + 1 <= k1) {
        if (split_slot(k + 1)) waited = max(waited, k + 1);
        else fail = true;
      }
    }
    if (__syncthreads_or(fail)) {
      // give up: record, drain this block's copies in flight, return
      if (t == ISSUER) {
        if (a.err) atomicExch(a.err, kErrWait);
        const int issued = min(k1, max(k + G::PD, k0 - 1 + G::PD));
        for (int L = waited + 1; L <= issued; L++) (void)mbar_wait(bar_of(L), parity(L));
      }
      return;
    }
  }
  if constexpr (RANGE) {  // values left the double-float range: mark the tile (and its edges)
    if (oorb) {
      const int nt = gxc * (a.ny / (TY - 1) + 1);
      atomicOr(a.rflags + ((a.flag_phase + step + 1) % 3) * nt + blk, oorb);
    }
  }
}

// The FP64 form's path for this block: the FP64 path (the tensor-copy kernel
// in IEEE double) when, in the previous step, its tile stored a value outside
// the double-float range, or a neighbour tile did so on an edge this tile's
// boxes read (the neighbour's last cell column for the tile on its right,
// its first node and cell column for the tile on its left, rows likewise, and
// a corner for a diagonal neighbour: both edge bits), or when one of this
// step's source terms of its layers lies outside the range; the double-float
// path (df64d) otherwise.  Flags rotate through three per-tile words: read
// (flag_phase + step) % 3, or-ed by this step's blocks (+1), cleared for the
// step after next by each tile's first chunk (+2).  Block-uniform.
template <int TY>
__device__ __forceinline__ bool fp64_path(const GridArgs<double> &a, int bx, int by, int k0, int kc, int gxc,
                                          int step) {
  constexpr int NT = TX * TY;
  const int t = threadIdx.x;
  const int gyc = a.ny / (TY - 1) + 1, nt = gxc * gyc;
  const int blk = by * gxc + bx;
  const int phase = (a.flag_phase + step) % 3;
  if (k0 == 0 && t == 0) a.rflags[((phase + 2) % 3) * nt + blk] = 0;
  bool f = false;
  if (t < 9) {
    const int dx = t % 3 - 1, dy = t / 3 - 1, x = bx + dx, y = by + dy;
    if (x >= 0 && x < gxc && y >= 0 && y < gyc) {
      const uint32_t m = (dx == 0 && dy == 0) ? 1u : ((dx < 0 ? 4u : dx > 0 ? 2u : 0u) | (dy < 0 ? 16u : dy > 0 ? 8u : 0u));
      f = (a.rflags[phase * nt + y * gxc + x] & m) == m;
    }
  }
  const int nz = a.nz;
  const int ktop = a.ktop ? min(nz, __ldg(a.ktop + blk)) : nz;
  const int k1 = min(ktop, k0 + kc);
  if (k0 < ktop && a.sigval) {
    const double *sigrow = a.sigval + (int64_t)min(step, a.sig_rows - 1) * a.sig_stride;
    const uint32_t lo = (uint32_t)a.r_elo_s, hi = (uint32_t)a.r_ehi_s;
    auto bad = [&](double w, double sg) { return !in_df64_range(sg, lo, hi) || !in_df64_range(w * sg, lo, hi); };
    if (a.f_rng) {  // force entries of node layers k0-1 .. k1 (contiguous per block)
      const int64_t r0 = (int64_t)blk * (nz + 1);
      const int e0 = a.f_rng[r0 + max(k0 - 1, 0)].x, e1 = a.f_rng[r0 + k1].y;
      for (int e = e0 + t; e < e1; e += NT) f = f || bad(a.f_w[e], sigrow[a.f_sig[e]]);
    }
    if (a.m_rng) {  // moment entries of cell layers k0 .. k1-1
      const int64_t r0 = (int64_t)blk * nz;
      const int e0 = a.m_rng[r0 + k0].x, e1 = a.m_rng[r0 + k1 - 1].y;
      for (int e = e0 + t; e < e1; e += NT) f = f || bad(a.m_w[e], sigrow[a.m_sig[e]]);
    }
  }
  return __syncthreads_or(f) != 0;
}

// tile (bx, by) and layer range [k0, k0 + kc) of this block of a single
// solver's launch: the 3D grid (x, y, chunk of kchunk layers), or with a
// tail split (tail_chunk > 0) the 1D grid of whole columns, then the
// remaining tiles' chunks of tail_chunk layers, chunk-major
template <int TY, typename T>
__device__ __forceinline__ void block_coords(const GridArgs<T> &a, int &bx, int &by, int &k0, int &kc, int &gxc) {
  gxc = a.nx / (TX - 1) + 1;
  if (a.tail_chunk > 0) {
    const int id = blockIdx.x, tiles = gxc * (a.ny / (TY - 1) + 1);
    int tile;
    if (id < a.tail_from) {
      tile = id;
      k0 = 0;
      kc = a.kchunk;
    } else {
      const int rest = tiles - a.tail_from, j = id - a.tail_from;
      tile = a.tail_from + j % rest;
      k0 = (j / rest) * a.tail_chunk;
      kc = a.tail_chunk;
    }
    bx = tile % gxc;
    by = tile / gxc;
  } else {
    bx = blockIdx.x;
    by = blockIdx.y;
    k0 = blockIdx.z * a.kchunk;
    kc = a.kchunk;
  }
}

// The FP64 form's kernels: MODE 0 runs each block on its path; with the two
// paths as two launches (PN_F64H_TWO_LAUNCHES), MODE 1 runs the double-float
// blocks and MODE 2 the FP64 ones (the other blocks return at once), so each
// kernel gets registers for one path only.  Both launches decide alike.
// Measured on the laminate bench step (15% FP64 blocks): one launch 0.663 ms,
// two launches 1.049 ms -- in one launch the FP64 blocks share the SMs with
// double-float ones and the two pipes work at once; alone, the FP64 blocks
// are a serial tail on a few SMs.  One launch is the default.
#ifndef PN_F64H_TWO_LAUNCHES
#define PN_F64H_TWO_LAUNCHES 0
#endif
template <typename K, int SYM, bool BATCH>
__device__ __forceinline__ void f64h_path(const GridArgs<double> &a, const GridMaps *M, int bx, int by, int k0,
                                          int kc, int gxc, int step) {
  grid_block_tma<K, SYM, 8, BATCH, true>(a, M, bx, by, k0, kc, gxc, step);
}

template <int SYM, bool BATCH, int MODE>
__device__ __forceinline__ void f64h_block(const GridArgs<double> &a, int bx, int by, int k0, int kc, int gxc,
                                           int step) {
  const GridMaps *M = reinterpret_cast<const GridMaps *>(a.tmaps);
  const bool fp64 = fp64_path<8>(a, bx, by, k0, kc, gxc, step);
  if ((MODE == 1 && fp64) || (MODE == 2 && !fp64)) return;
  if (threadIdx.x == 0 && a.path_count) atomicAdd(a.path_count + (fp64 ? 0 : 1), 1ull);
  if constexpr (MODE != 1) {
    if (fp64) {
      f64h_path<double, SYM, BATCH>(a, M, bx, by, k0, kc, gxc, step);
      return;
    }
  }
  if constexpr (MODE != 2) f64h_path<df64d, SYM, BATCH>(a, M, bx, by, k0, kc, gxc, step);
}

// resident blocks per SM the FP64 form's kernel is compiled for (its register
// cap: 3 -> 80 registers, 2 -> 128)
#ifndef PN_F64H_MIN_BLOCKS
#define PN_F64H_MIN_BLOCKS 3
#endif

template <int SYM, int MODE>
__global__ void __launch_bounds__(TX * 8, PN_F64H_MIN_BLOCKS)
    k_grid_tma_f64h(const __grid_constant__ GridArgs<double> a, int step) {
  int bx, by, k0, kc, gxc;
  block_coords<8>(a, bx, by, k0, kc, gxc);
  f64h_block<SYM, false, MODE>(a, bx, by, k0, kc, gxc, step);
}

template <int SYM, int MODE>
__global__ void __launch_bounds__(TX * 8, PN_F64H_MIN_BLOCKS)
    k_grid_tma_f64h_batch(const GridArgs<double> *__restrict__ args, const int *__restrict__ block_start,
                          const int *__restrict__ order, int n_members, int step) {
  const int id = order ? __ldg(order + blockIdx.x) : (int)blockIdx.x;
  int lo = 0, hi = n_members;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(block_start + mid) <= id) lo = mid;
    else hi = mid;
  }
  const GridArgs<double> &a = args[lo];
  const int local = id - __ldg(block_start + lo);
  const int gxc = a.nx / (TX - 1) + 1, gyc = a.ny / 7 + 1;
  f64h_block<SYM, true, MODE>(a, local % gxc, (local / gxc) % gyc, local / (gxc * gyc) * a.kchunk, a.kchunk, gxc,
                              step);
}

// minimum blocks per SM each storage type is compiled for (the register cap
// follows): 3 for 8-byte storage (80 registers; shared memory holds 3 blocks);
// none for 4-byte storage (the compiler's 62-64 registers give 4 blocks, and a
// cap of 4 blocks measured 6% slower)
// (32 x 16 tiles with 8-byte storage: shared memory holds one block per SM)
template <typename R, int TY> struct GMinBlocks { static constexpr int v = TY == 8 ? 3 : 1; };
template <int TY> struct GMinBlocks<float, TY> { static constexpr int v = PN_GRID_F32_MIN_BLOCKS; };

template <typename R, int SYM, int TY>
__global__ void __launch_bounds__(TX *TY, GMinBlocks<R, TY>::v)
    k_grid_tma(const GridArgs<typename GNum<R>::S> a, int step) {
  const GridMaps *M = reinterpret_cast<const GridMaps *>(a.tmaps);
  int bx, by, k0, kc, gxc;
  block_coords<TY>(a, bx, by, k0, kc, gxc);
  grid_block_tma<R, SYM, TY>(a, M, bx, by, k0, kc, gxc, step);
}

template <typename R, int SYM, int TY>
__global__ void __launch_bounds__(TX *TY, GMinBlocks<R, TY>::v)
    k_grid_tma_batch(const GridArgs<typename GNum<R>::S> *__restrict__ args, const int *__restrict__ block_start,
                     const int *__restrict__ order, int n_members, int step) {
  const int id = order ? __ldg(order + blockIdx.x) : (int)blockIdx.x;
  int lo = 0, hi = n_members;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(block_start + mid) <= id) lo = mid;
    else hi = mid;
  }
  const GridArgs<typename GNum<R>::S> &a = args[lo];
  const GridMaps *M = reinterpret_cast<const GridMaps *>(a.tmaps);
  const int local = id - __ldg(block_start + lo);
  const int gxc = a.nx / (TX - 1) + 1, gyc = a.ny / (TY - 1) + 1;
  grid_block_tma<R, SYM, TY, true>(a, M, local % gxc, (local / gxc) % gyc, local / (gxc * gyc) * a.kchunk, a.kchunk,
                                   gxc, step);
}

template <typename R, int SYM, int TY>
struct SetupT {
  using St = typename GNum<R>::S;
  static constexpr size_t smem = Geo<(int)sizeof(St), TY>::SMEM;
  static cudaError_t ensure(int &sms, int &per_sm) {
    static unsigned long long done = 0;
    static int s_sms[64] = {0}, s_per[64] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int d = dev & 63;
    if (!(done & (1ull << d))) {
      e = cudaFuncSetAttribute(k_grid_tma<R, SYM, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_grid_tma_batch<R, SYM, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s_sms[d], cudaDevAttrMultiProcessorCount, dev);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s_per[d], k_grid_tma<R, SYM, TY>, TX * TY, smem);
      if (e != cudaSuccess) return e;
      s_per[d] = s_per[d] > 0 ? s_per[d] : 1;
      done |= 1ull << d;
    }
    sms = s_sms[d];
    per_sm = s_per[d];
    return cudaSuccess;
  }
};

// grid of a single solver's launch: chunks (kchunk, when the caller left it
// 0) and the tail split; grid.x == 0: a chunk longer than the kernel stages
template <int TY, typename T>
dim3 single_grid(GridArgs<T> &b, int sms, int per_sm) {
  const unsigned gx = (unsigned)(b.nx / (TX - 1) + 1), gy = (unsigned)(b.ny / (TY - 1) + 1);
  if (b.kchunk <= 0) b.kchunk = grid_chunk_for(b.nz, (long long)gx * gy, sms, per_sm);
  if (b.kchunk > KC_MAX) return dim3(0, 1, 1);
  grid_tail_split(b.nz, b.kchunk, (long long)gx * gy, (long long)sms * per_sm, b.tail_from, b.tail_chunk);
  if (b.tail_chunk > 0) {
    const long long tiles = (long long)gx * gy, cuts = (b.nz + b.tail_chunk - 1) / b.tail_chunk;
    return dim3((unsigned)(b.tail_from + (tiles - b.tail_from) * cuts), 1, 1);
  }
  return dim3(gx, gy, (unsigned)((b.nz + b.kchunk - 1) / b.kchunk));
}

template <typename R, int SYM, int TY>
cudaError_t launch_t(const GridArgs<typename GNum<R>::S> &a, cudaStream_t st) {
  using S = SetupT<R, SYM, TY>;
  int sms = 0, per_sm = 0;
  cudaError_t e = S::ensure(sms, per_sm);
  if (e != cudaSuccess) return e;
  GridArgs<typename GNum<R>::S> b = a;
  const dim3 grid = single_grid<TY>(b, sms, per_sm);
  if (grid.x == 0) return cudaErrorInvalidValue;
  k_grid_tma<R, SYM, TY><<<grid, TX * TY, S::smem, st>>>(b, 0);
  return cudaGetLastError();
}

template <typename R, int SYM, int TY>
cudaError_t launch_batch_t(const GridBatchLaunch &b, int step, cudaStream_t st) {
  using S = SetupT<R, SYM, TY>;
  int sms = 0, per_sm = 0;
  cudaError_t e = S::ensure(sms, per_sm);
  if (e != cudaSuccess) return e;
  if (b.total_blocks <= 0) return cudaSuccess;
  k_grid_tma_batch<R, SYM, TY><<<b.total_blocks, TX * TY, S::smem, st>>>(
      (const GridArgs<typename GNum<R>::S> *)b.args, b.block_start, b.order, b.n_members, step);
  return cudaGetLastError();
}

// the FP64 form's kernels (k_grid_tma_f64h*): the FP64 path's shared-memory geometry
template <int SYM, int MODE>
struct SetupH {
  static constexpr size_t smem = Geo<8, 8>::SMEM;
  static cudaError_t ensure() {
    static unsigned long long done = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int d = dev & 63;
    if (!(done & (1ull << d))) {
      e = cudaFuncSetAttribute(k_grid_tma_f64h<SYM, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_grid_tma_f64h_batch<SYM, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
      if (e != cudaSuccess) return e;
      done |= 1ull << d;
    }
    return cudaSuccess;
  }
};

template <int SYM, int MODE>
cudaError_t launch_h_mode(const GridArgs<double> &b, const dim3 &grid, cudaStream_t st) {
  cudaError_t e = SetupH<SYM, MODE>::ensure();
  if (e != cudaSuccess) return e;
  k_grid_tma_f64h<SYM, MODE><<<grid, TX * 8, SetupH<SYM, MODE>::smem, st>>>(b, 0);
  return cudaGetLastError();
}

template <int SYM>
cudaError_t launch_h(const GridArgs<double> &a, cudaStream_t st) {
  int sms = 0, per_sm = 0;
  cudaError_t e = SetupT<double, SYM, 8>::ensure(sms, per_sm);
  if (e != cudaSuccess) return e;
  GridArgs<double> b = a;
  const dim3 grid = single_grid<8>(b, sms, per_sm);
  if (grid.x == 0) return cudaErrorInvalidValue;
  if constexpr (PN_F64H_TWO_LAUNCHES != 0) {
    e = launch_h_mode<SYM, 1>(b, grid, st);
    return e == cudaSuccess ? launch_h_mode<SYM, 2>(b, grid, st) : e;
  } else {
    return launch_h_mode<SYM, 0>(b, grid, st);
  }
}

template <int SYM, int MODE>
cudaError_t launch_batch_h_mode(const GridBatchLaunch &b, int step, cudaStream_t st) {
  cudaError_t e = SetupH<SYM, MODE>::ensure();
  if (e != cudaSuccess) return e;
  k_grid_tma_f64h_batch<SYM, MODE><<<b.total_blocks, TX * 8, SetupH<SYM, MODE>::smem, st>>>(
      (const GridArgs<double> *)b.args, b.block_start, b.order, b.n_members, step);
  return cudaGetLastError();
}

template <int SYM>
cudaError_t launch_batch_h(const GridBatchLaunch &b, int step, cudaStream_t st) {
  if (b.total_blocks <= 0) return cudaSuccess;
  if constexpr (PN_F64H_TWO_LAUNCHES != 0) {
    const cudaError_t e = launch_batch_h_mode<SYM, 1>(b, step, st);
    return e == cudaSuccess ? launch_batch_h_mode<SYM, 2>(b, step, st) : e;
  } else {
    return launch_batch_h_mode<SYM, 0>(b, step, st);
  }
}

template <typename T> inline bool is_one(T v) { return v == T(1); }
template <> inline bool is_one<float2>(float2 v) { return v.x == 1.0f && v.y == 0.0f; }

template <typename R, int TY>
cudaError_t launch_sym(const GridArgs<typename GNum<R>::S> &a, int sym, cudaStream_t st) {
  if (a.nx <= 0 || a.ny <= 0 || a.nz <= 0) return cudaSuccess;
  if (!a.tmaps || a.n_rows > ROWS_MAX) return cudaErrorInvalidValue;
  const bool cubic = is_one(a.g[0]) && is_one(a.g[1]) && is_one(a.g[2]);
  switch ((sym & 3) | (cubic ? 4 : 0)) {
    case 2: return launch_t<R, 2, TY>(a, st);
    case 1: return launch_t<R, 1, TY>(a, st);
    case 0: return launch_t<R, 0, TY>(a, st);
    case 6: return launch_t<R, 6, TY>(a, st);
    case 5: return launch_t<R, 5, TY>(a, st);
    default: return launch_t<R, 4, TY>(a, st);
  }
}

inline cudaError_t launch_sym_h(const GridArgs<double> &a, int sym, cudaStream_t st) {
  if (a.nx <= 0 || a.ny <= 0 || a.nz <= 0) return cudaSuccess;
  if (!a.tmaps || a.n_rows > ROWS_MAX || !a.rflags) return cudaErrorInvalidValue;
  const bool cubic = is_one(a.g[0]) && is_one(a.g[1]) && is_one(a.g[2]);
  switch ((sym & 3) | (cubic ? 4 : 0)) {
    case 2: return launch_h<2>(a, st);
    case 1: return launch_h<1>(a, st);
    case 0: return launch_h<0>(a, st);
    case 6: return launch_h<6>(a, st);
    case 5: return launch_h<5>(a, st);
    default: return launch_h<4>(a, st);
  }
}

inline cudaError_t launch_batch_sym_h(const GridBatchLaunch &b, int step, cudaStream_t st) {
  switch (b.sym) {
    case 2: return launch_batch_h<2>(b, step, st);
    case 1: return launch_batch_h<1>(b, step, st);
    case 0: return launch_batch_h<0>(b, step, st);
    case 6: return launch_batch_h<6>(b, step, st);
    case 5: return launch_batch_h<5>(b, step, st);
    default: return launch_batch_h<4>(b, step, st);
  }
}

// b.sym: the members' most general symmetry class | 4 when every member is cubic
template <typename R, int TY>
cudaError_t launch_batch_sym(const GridBatchLaunch &b, int step, cudaStream_t st) {
  switch (b.sym) {
    case 2: return launch_batch_t<R, 2, TY>(b, step, st);
    case 1: return launch_batch_t<R, 1, TY>(b, step, st);
    case 0: return launch_batch_t<R, 0, TY>(b, step, st);
    case 6: return launch_batch_t<R, 6, TY>(b, step, st);
    case 5: return launch_batch_t<R, 5, TY>(b, step, st);
    default: return launch_batch_t<R, 4, TY>(b, step, st);
  }
}

}  // namespace
}  // namespace pn
