// rsg_grid.cuh -- arguments of the fused voxel-grid step kernel (rsg_grid.cu).
//
// Layout (x fastest, padded rows): grid node (i,j,k) at (k*(ny+1)+j)*pnx+i,
// grid cell (i,j,k) at (k*ny+j)*pcx+i; pnx*sizeof(T) and pcx are multiples of
// 16 bytes (row strides a tensor copy accepts).  Block (bx,by) owns node and cell columns
// i in [bx*(TX-1), bx*(TX-1)+TX-1), j likewise with TY; its local index of the
// node / cell (i,j) is (i-i0) + TX*(j-j0).  Sparse sources and sensors are
// sorted by (block, layer, local index) with one [begin,end) range per
// (block, layer).
#pragma once
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

namespace pn {

// split lattice sites (rsg_split.cu): a copy is one mesh node of a site that
// several nodes share; a fix cell is a cell with a corner on such a site
struct SplitCopy {
  int32_t i, j, k;    // the site
  uint32_t mask;      // the site's cells (i-1+a, j-1+b, k-1+c) the copy joins: bit a + 2b + 4c
  int64_t v;          // index of the copy in the node buffers (lattice site or tail slot)
  int32_t f0, f1;     // its force entries [f0, f1)
  int32_t s0, s1;     // its sensor entries [s0, s1)
};
struct FixCell {
  int64_t cell;       // lattice cell
  int64_t v[8];       // node-buffer index of each corner (reference corner order)
  int32_t m0, m1;     // its moment entries [m0, m1)
};

template <typename T>
struct GridArgs {
  int32_t nx, ny, nz;  // cells per axis
  int32_t pnx, pcx;    // row pitch (sites) of node / cell buffers
  int32_t kchunk;      // cell layers per block along z (set by the launcher when 0)
  const T *V_in[3];
  T *V_out[3];
  const T *S_in[6];
  T *S_out[6];
  const T *coef;       // [grid nodes] dt/rho_node; 0 = void or not owned
  const uint8_t *mat;  // [grid cells] material row; the last row is zero (void)
  const T *ctab;       // [rows][36] dt*C
  T g[3];              // 0.25/h per axis
  // force sources, ranges per (block, node layer): [blocks][nz+1]
  const int2 *f_rng;
  const int32_t *f_key;  // local node | direction << 16
  const int32_t *f_sig;
  const T *f_w;
  // moment sources, ranges per (block, cell layer): [blocks][nz]
  const int2 *m_rng;
  const int32_t *m_key;  // local cell | Voigt component << 16
  const int32_t *m_sig;
  const T *m_w;          // weights carry dt
  const T *sigval;       // signal rows: row min(step, sig_rows-1) at stride sig_stride
  int32_t sig_stride;    // 0 when sigval already points at the step's row
  int32_t sig_rows;
  // sensors, ranges per (block, node layer)
  const int2 *s_rng;
  const int32_t *s_key;  // local node
  const int32_t *s_idx;  // sensor number
  double *traces;        // [records][n_sens][3]
  int32_t n_sens;
  int64_t rec;           // record written by step 0 of the launch (rec + step later)
  int64_t rec_cap;       // records beyond this are not written
  int32_t *err;          // device error word (bounded waits that gave up), or null
  const void *tmaps;     // tensor maps of this step's input buffers (rsg_grid_tma.cu), or null
  const int32_t *ktop;   // [tiles] cell layers below the tile's top solid cell + 1 (its
                         // node layers above are void; the tensor-copy kernel stops
                         // there), or null: nz
  int32_t n_rows;        // rows of ctab (materials + the void row)
  uint32_t ortho_rows;   // bit r: row r is orthotropic (tensor-copy kernel, rows < 32)
  // split sites, redone after the step kernel by the fix-up (rsg_split.cu)
  int32_t n_copies, n_fix;
  const SplitCopy *copies;
  const int32_t *cf_dir;  // copy forces: direction, signal, weight (as f_w)
  const int32_t *cf_sig;
  const T *cf_w;
  const int32_t *cs_idx;  // copy sensors: sensor number
  const FixCell *fix;
  const int32_t *cm_comp;  // fix-cell moments: Voigt component, signal, weight (as m_w)
  const int32_t *cm_sig;
  const T *cm_w;
  int32_t test_skip_layer;  // failure-path test: the layer whose copies are never issued (kNoLayer: none)
  int32_t tile_rows;        // rows TY of the 32 x TY block tile (8, or 16 with the tensor-copy kernel)
  // FP64 form with the tensor-copy kernel: per-tile path flag words [3][tiles]
  // (rsg_grid_tma.cuh fp64_path) and the double-float ranges as biased double
  // exponents, [r_elo, r_ehi] for velocities and [r_elo_s, r_ehi_s] for
  // stresses and source terms; rflags null: no path choice (the other forms)
  uint32_t *rflags;
  int32_t flag_phase;       // (step of this launch's step 0) % 3
  int32_t r_elo, r_ehi;
  int32_t r_elo_s, r_ehi_s;
  unsigned long long *path_count;  // [2] blocks that took the FP64 / double-float path, or null
  // tail split (tensor-copy kernel, one launch per solver; set by the launcher):
  // tail_chunk > 0 runs a 1D grid whose first tail_from blocks are the first
  // tail_from tiles' whole columns and whose others cut each remaining tile's
  // column into chunks of tail_chunk layers, chunk-major (the last partial wave
  // of whole columns would leave most SMs idle); 0: the 3D grid of kchunk chunks
  int32_t tail_from, tail_chunk;
};

// where a thread's scan of its (block, layer) slot starts: the entries are
// sorted by local index (key & 0xffff), so in a long slot (a transducer patch
// puts a few hundred entries in one) a binary search finds the first entry of
// local index t, or the first past them, in log2(hi - lo) loads; a short slot
// is scanned from its start.  The scan skips entries of smaller local index
// and stops at the first larger one.
#ifdef __CUDACC__
__device__ __forceinline__ int first_local(const int32_t *__restrict__ key, int lo, int hi, int t) {
  if (hi - lo <= 32) return lo;  // a short slot: scanned from its start (independent loads)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((__ldg(key + mid) & 0xffff) < t) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
#endif

constexpr int32_t kNoLayer = INT32_MIN;  // no layer index (layers run from -1 to nz)

constexpr int kGridChunkMax = 64;     // cell layers per z chunk, at most

// tail split of a one-chunk launch (GridArgs::tail_from / tail_chunk) for
// `tiles` tile columns of nz layers on `slots` resident blocks; tail_chunk 0:
// none.  PN_GRID_TAIL_CHUNKS overrides the chunks per tail column (1: none).
void grid_tail_split(int nz, int kchunk, long long tiles, long long slots, int &tail_from, int &tail_chunk);
constexpr int kGridTmaRowsMax = 32;   // stiffness rows the tensor-copy kernel stages

// block tiles: 32 x TY threads, one warp per row; TY = 8 everywhere, 16 as
// well for the tensor-copy kernel with FP32 storage
constexpr int kGridTileX = 32;
constexpr int kGridTileRows = 8;  // the classic kernel's, and the default
// cell layers per z chunk: about one wave of blocks, at least four layers,
// at most kGridChunkMax
int grid_chunk_for(int nz, long long xy_blocks, int sms, int per_sm);
// cell layers per z chunk the launcher picks for this lattice, precision and
// kernel (tma: the tensor-copy kernel of rsg_grid_tma.cu)
int grid_chunk_layers(int precision, int nx, int ny, int nz, bool tma, int tile_rows = kGridTileRows);

// a batch of grid-form members: argument blocks (kchunk set) and the prefix
// of their block counts ((nx/(TX-1)+1) * (ny/(TY-1)+1) * chunks each)
struct GridBatchLaunch {
  int n_members;
  const void *args;        // GridArgs<S>[n_members]
  const int *block_start;  // [n_members + 1]
  int total_blocks;
  int sym;                 // most general symmetry class among the members
  int tile_rows;           // TY of every member's tiles
  int range_flags;         // FP64 form: every member has path flags (rflags)
  // launch order of the blocks (tensor-copy kernel): block i of the launch is
  // block order[i] of the member-major numbering, total_blocks entries; null:
  // the numbering itself.  pn_batch_solve lists the blocks that have layers to
  // march, longest first, so that no long column starts in the last wave
  const int *order = nullptr;
};
cudaError_t launch_grid_batch(const GridBatchLaunch &b, int precision, int step, cudaStream_t st);
cudaError_t launch_grid_f32(const GridArgs<float> &a, int sym, cudaStream_t st);
cudaError_t launch_grid_f64(const GridArgs<double> &a, int sym, cudaStream_t st);
cudaError_t launch_grid_df64(const GridArgs<float2> &a, int sym, cudaStream_t st);

// tensor-copy kernel (rsg_grid_tma.cu): maps of one input parity occupy
// grid_tma_maps_bytes(); encoding fails (false) when a buffer or pitch does not
// meet the copy's alignment rules
size_t grid_tma_maps_bytes();
// tile rows the tensor-copy kernel has for this storage (8; 16 for FP32)
bool grid_tma_rows_supported(int precision, int tile_rows);
bool grid_tma_encode(int precision, int tile_rows, int nx, int ny, int nz, int pnx, int pcx,
                     const void *const V[3], const void *const S[6], const void *coef, const uint8_t *mat,
                     void *out);
int grid_tma_blocks_per_sm(int precision, int tile_rows = kGridTileRows);
cudaError_t launch_grid_tma(const void *args /* GridArgs<storage type> */, int precision, int sym,
                            cudaStream_t st);
cudaError_t launch_grid_tma_batch(const GridBatchLaunch &b, int precision, int step, cudaStream_t st);
// kernel launches of one FP64-form step (the double-float and the FP64 blocks
// in one launch or in two)
int grid_tma_f64_launches();

// fix-up of split sites after a step launch (rsg_split.cu): the copies'
// velocities, then the fix cells' stresses, from the step's input buffers
cudaError_t launch_grid_split(const void *args /* GridArgs<storage type> */, int precision, cudaStream_t st);
struct GridSplitBatch {
  int n_members;
  const void *args;         // GridArgs<S>[n_members] (device)
  const int *copy_start;    // [n_members + 1] prefix of n_copies
  const int *fix_start;     // [n_members + 1] prefix of n_fix
  int total_copies, total_fix;
};
cudaError_t launch_grid_split_batch(const GridSplitBatch &b, int precision, int step, cudaStream_t st);

}  // namespace pn
