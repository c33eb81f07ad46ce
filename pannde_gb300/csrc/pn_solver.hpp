// pn_solver.hpp -- the solver object behind the C ABI (private).
//
// Two device forms share it:
//   table form  connectivity tables (cell->8 nodes, node->8 cell slots) and
//               two kernels per step (rsg_fast.cu / rsg_exact.cu); any hex mesh
//   grid form   voxel-grid meshes (pn::detect_grid): implicit indices, one fused
//               kernel per step, double-buffered state (rsg_grid.cu)
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/pannde_gb300.h"
#include "pn_setup.hpp"
#include "rsg_common.cuh"
#include "rsg_grid.cuh"
#include "rsg_state.cuh"

namespace pn {

struct CudaError {
  cudaError_t e;
  const char *what;
};

inline void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError{e, what};
}

// Optional artificial HBM budget (bytes) for allocation-failure tests:
// PN_HBM_BUDGET_BYTES caps the device memory one solver may hold.
inline int64_t hbm_budget() {
  const char *s = std::getenv("PN_HBM_BUDGET_BYTES");
  if (!s || !*s) return -1;
  return std::strtoll(s, nullptr, 10);
}

constexpr int64_t kSigRowsCap = 1 << 16;  // signal rows uploaded at once

// a host double in the storage type T
template <typename T> inline T to_store(double v);
template <> inline double to_store<double>(double v) { return v; }
template <> inline float to_store<float>(double v) { return (float)v; }
template <> inline float2 to_store<float2>(double v) {
  float2 r;
  split_df(v, r.x, r.y);
  return r;
}

}  // namespace pn

struct pn_solver {
  int device = 0;
  int precision = PN_PREC_F64;
  int form = PN_FORM_TABLE;
  cudaStream_t stream = nullptr;
  double dt = 0., time = 0.;
  int64_t step = 0;
  size_t esz = 8;  // bytes per state value

  pn::MeshTables mesh;
  pn::MaterialTables mat;

  std::vector<void *> allocs;
  int64_t dev_bytes = 0;

  // state: V[3] over nodes, S[6] over cells (grid form: buffer `cur` of two)
  void *V[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  void *S[2][6] = {{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr},
                   {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr}};
  int cur = 0;
  void *d_coef = nullptr, *d_ctab = nullptr;

  // table form
  int4 *d_hex = nullptr, *d_ncc = nullptr;
  void *d_gnode = nullptr, *d_gcell = nullptr;
  int32_t *d_mat = nullptr;

  // grid form
  pn::GridMap grid;
  int sym = 0;             // material symmetry class of the stiffness table
  uint8_t *d_gmat = nullptr;
  void *d_tmaps = nullptr;   // tensor maps [2 input parities] (null: classic kernel)
  int32_t *d_ktop = nullptr; // [tiles] cell layers the tensor-copy kernel marches per tile
  mutable int64_t step_bytes_cached = 0;  // grid form: algorithmic bytes of one step (0: not yet)
  int tile_rows = pn::kGridTileRows;      // grid form: rows TY of the 32 x TY block tiles
  // FP64 form with the tensor-copy kernel: per-tile path flags [3][tiles] and
  // the double-float ranges (biased double exponents) of velocities and of
  // stresses, from the magnitudes of the coefficients each is multiplied by
  // (velocities: dt*C*g and g; stresses: dt/rho*g, g and source weights);
  // block counts of the two paths [fp64, df64]
  uint32_t *d_rflags = nullptr;
  int32_t r_elo = 1, r_ehi = 0, r_elo_s = 1, r_ehi_s = 0;
  double r_cmin = 1.0, r_cmax = 1.0, r_cmin_s = 1.0, r_cmax_s = 1.0;
  unsigned long long *d_pathcnt = nullptr;
  std::vector<std::pair<int32_t, int32_t>> sensor_pairs;  // grid form: (node, sensor) sorted, for re-tiling
  // cubic lattice with the tensor-copy kernel: 0.25/h folded into dt/rho, dt*C
  // and the force weights (the kernel's g is then 1); 1.0 when not folded
  double gfold = 1.0;
  int32_t *d_err = nullptr;  // device error word of the grid kernels
  uint32_t *d_rflags_stage = nullptr;  // FP64 form: set_state's tile flags before the state is accepted
  int32_t *d_nonfinite = nullptr;  // [4] set_state's NaN / infinity flags (velocity, stress), and
                                   // (FP64 form) an out-of-range value at a split site's copy
  // split sites (grid.copy_node / fix_cell): the step's fix-up tables, rebuilt
  // when sources or sensors change; host lists of the copies' forces and
  // sensors and the fix cells' moments (per copy / fix cell, in order)
  struct SplitForce { int32_t copy, dir, sig; double w; };
  struct SplitSensor { int32_t copy, idx; };
  struct FixMoment { int32_t fix, comp, sig; double w; };
  std::vector<SplitForce> split_forces;
  std::vector<SplitSensor> split_sensors;
  std::vector<FixMoment> fix_moments;
  pn::SplitCopy *d_copies = nullptr;
  pn::FixCell *d_fix = nullptr;
  int32_t *d_cf_dir = nullptr, *d_cf_sig = nullptr, *d_cs_idx = nullptr, *d_cm_comp = nullptr, *d_cm_sig = nullptr;
  void *d_cf_w = nullptr, *d_cm_w = nullptr;

  // energy audit tables (pn_energy.cpp; built on the first call)
  double *d_emass = nullptr, *d_evol = nullptr, *d_ecomp = nullptr, *d_epart = nullptr;
  int64_t e_nodes = 0, e_cells = 0;

  // sources (both forms)
  std::vector<pn_window_source> src;
  std::vector<std::vector<double>> src_t, src_v;  // owned copies of signal arrays
  std::vector<pn::Series> series;
  std::vector<std::vector<uint8_t>> src_mask;  // non-empty: window given by a caller's mask
  bool src_dirty = false;
  bool caller_signals = false;  // inside pn_solver_solve_signals

  bool has_mask_sources() const {
    for (auto &m : src_mask)
      if (!m.empty()) return true;
    return false;
  }
  std::vector<const uint8_t *> mask_ptrs() const {
    std::vector<const uint8_t *> p;
    for (auto &m : src_mask) p.push_back(m.empty() ? nullptr : m.data());
    return p;
  }
  bool has_moments = false;
  int32_t n_force = 0, n_moment = 0, n_src_nodes = 0, n_src_cells = 0;
  // table-form lists: per-tile ranges, element, code, weight
  int2 *d_ftile = nullptr, *d_mtile = nullptr;
  int32_t *d_felem = nullptr, *d_fcode = nullptr, *d_melem = nullptr, *d_mcode = nullptr;
  // grid-form lists: per (block, layer) ranges, key, signal
  int2 *d_frng = nullptr, *d_mrng = nullptr;
  int32_t *d_fkey = nullptr, *d_fsig = nullptr, *d_mkey = nullptr, *d_msig = nullptr;
  void *d_fw = nullptr, *d_mw = nullptr;
  // signal table: rows [sig_step0, sig_step0 + sig_rows) of [n_sig] values;
  // sig_hold: the last row holds for every later step
  void *d_sig = nullptr;
  int64_t sig_step0 = 0, sig_rows = 0, sig_alloc_rows = 0;
  bool sig_hold = false, sig_valid = false;

  // sensors
  int32_t n_sens = 0;
  int2 *d_stile = nullptr, *d_srng = nullptr;
  int32_t *d_snode = nullptr, *d_sidx = nullptr, *d_skey = nullptr;
  double *d_traces = nullptr;
  int64_t rec_cap = 0, rec_count = 0;

  // optional per-kernel event timing (kind 0 velocity, 1 stress, 2 fused step)
  bool timing = false;
  struct Mark {
    cudaEvent_t a, b;
    int kind;
  };
  std::vector<Mark> marks;

  bool is_df64() const { return precision == PN_PREC_DF64; }

  template <typename P>
  P *alloc(size_t bytes) {
    if (bytes == 0) bytes = 16;
    const int64_t budget = pn::hbm_budget();
    if (budget >= 0 && dev_bytes + (int64_t)bytes > budget)
      throw pn::SetupError{PN_ERR_ALLOC, "device allocation exceeds PN_HBM_BUDGET_BYTES"};
    void *p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      throw pn::SetupError{PN_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e)};
    }
    allocs.push_back(p);
    dev_bytes += (int64_t)bytes;
    return (P *)p;
  }

  template <typename P>
  void release(P *&p) {
    if (!p) return;
    auto it = std::find(allocs.begin(), allocs.end(), (void *)p);
    if (it != allocs.end()) allocs.erase(it);
    cudaFree((void *)p);
    p = nullptr;
  }

  // upload a double host array in the storage type (double, float, or the
  // (hi, lo) float pair of the double-float form)
  void upload_real(void *dst, const double *src_, size_t n) {
    if (n == 0) return;
    if (is_df64()) {
      pn::hvec<float> tmp(2 * n);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)n; i++) pn::split_df(src_[i], tmp[2 * i], tmp[2 * i + 1]);
      pn::ck(cudaMemcpyAsync(dst, tmp.data(), n * 8, cudaMemcpyHostToDevice, stream), "upload");
      pn::ck(cudaStreamSynchronize(stream), "upload sync");
    } else if (esz == 8) {
      pn::ck(cudaMemcpyAsync(dst, src_, n * 8, cudaMemcpyHostToDevice, stream), "upload");
    } else {
      pn::hvec<float> tmp(n);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)n; i++) tmp[i] = (float)src_[i];
      pn::ck(cudaMemcpyAsync(dst, tmp.data(), n * 4, cudaMemcpyHostToDevice, stream), "upload");
      pn::ck(cudaStreamSynchronize(stream), "upload sync");
    }
  }

  void upload_raw(void *dst, const void *src_, size_t bytes) {
    if (bytes == 0) return;
    pn::ck(cudaMemcpyAsync(dst, src_, bytes, cudaMemcpyHostToDevice, stream), "upload");
  }

  // State transfer through the device: one FP64 field is copied to a staging
  // buffer and converted / permuted there by rsg_state.cu.  The staging buffer
  // (8 B per node or cell, whichever is more) and the grid form's index maps
  // are allocated on the first transfer and counted in dev_bytes from then.
  double *d_stage = nullptr;
  int64_t *d_nmap = nullptr, *d_cmap = nullptr;

  double *stage() {
    if (!d_stage) d_stage = alloc<double>(8 * (size_t)std::max(mesh.n_nodes, mesh.n_cells));
    return d_stage;
  }
  // The device's address of a caller buffer in page-locked, mapped host
  // memory (cudaHostAlloc / cudaHostRegister): the conversion kernels then
  // read or write it directly over the CPU-GPU link, without the staging
  // copy.  Null for any other memory (staged through device memory).  The
  // calls that use it wait for the stream before returning.
  // PN_STATE_COPY=dma stages page-locked buffers too (copy engine, then the
  // conversion kernel on device memory): for comparing the two paths.
  static void *device_view(const void *host) {
    const char *mode = std::getenv("PN_STATE_COPY");
    if (mode && mode[0] == 'd') return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
  }
  // host FP64 field[n] -> dst[map[i]] in the storage type (map null: dst[i]);
  // *nonfinite (device, when given) becomes 1 if a value is NaN or infinite
  // (rf: the FP64 form's tile flags of out-of-range values, see rsg_state.cuh)
  void put_field(void *dst, const double *host, size_t n, const int64_t *map, int32_t *nonfinite = nullptr,
                 const pn::StateRangeFlags *rf = nullptr) {
    if (n == 0) return;
    if (const void *dv = device_view(host)) {
      pn::ck(pn::launch_state_store(precision, (const double *)dv, (int64_t)n, map, dst, stream, nonfinite, rf),
             "put_field kernel");
      return;
    }
    double *st = stage();
    pn::ck(cudaMemcpyAsync(st, host, n * 8, cudaMemcpyHostToDevice, stream), "put_field copy");
    pn::ck(pn::launch_state_store(precision, st, (int64_t)n, map, dst, stream, nonfinite, rf), "put_field kernel");
  }
  // src[map[i]] (or src[i]) in the storage type -> host FP64 field[n]
  void get_field(double *host, const void *src, size_t n, const int64_t *map) {
    if (n == 0 || !host) return;
    if (void *dv = device_view(host)) {
      pn::ck(pn::launch_state_load(precision, src, (int64_t)n, map, (double *)dv, stream), "get_field kernel");
      return;
    }
    double *st = stage();
    pn::ck(pn::launch_state_load(precision, src, (int64_t)n, map, st, stream), "get_field kernel");
    pn::ck(cudaMemcpyAsync(host, st, n * 8, cudaMemcpyDeviceToHost, stream), "get_field copy");
  }

  void clear_marks() {
    for (auto &m : marks) {
      cudaEventDestroy(m.a);
      cudaEventDestroy(m.b);
    }
    marks.clear();
  }

  ~pn_solver() {
    clear_marks();
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
  }
};

namespace pn {

// shared by both forms (pn_capi.cpp)
// (may_alloc false: refill the resident table in place, never grow it)
void ensure_signal_rows(pn_solver *s, int64_t nsteps, bool may_alloc = true);
int64_t sig_row(const pn_solver *s, int64_t step_in_call);  // row of this step

// table form (pn_table.cpp)
int64_t table_footprint(const MeshTables &m, const MaterialTables &mt, int precision);
void table_create(pn_solver *s);
void table_sources(pn_solver *s);
void table_sensors(pn_solver *s, const std::vector<std::pair<int32_t, int32_t>> &sorted);
void table_run(pn_solver *s, int32_t nsteps);
void table_put_state(pn_solver *s, const double *const *V, const double *const *S);
void table_get_state(pn_solver *s, double *const *V, double *const *S);

// grid form (pn_grid.cpp)
// whether the grid form serves this mesh (why: the reason when not)
bool grid_eligible(const MeshTables &m, const MaterialTables &mt, int precision, const GridMap &g,
                   std::string *why = nullptr);
// per tile: 1 + the highest solid cell layer in the columns of its cell box
// with the apron, i.e. the cell layers the tensor-copy kernel marches
std::vector<int32_t> grid_tile_tops(const GridMap &g, int tile_rows = kGridTileRows);
// tile rows a new solver's tensor-copy kernel starts with
int grid_default_tile_rows(int precision, const GridMap &g);
// re-tile a solver's tensor-copy kernel (maps, tile tops, source and sensor
// lists); false when it has no such kernel or tiles of that many rows
bool grid_set_tile_rows(pn_solver *s, int rows);
int64_t grid_footprint(const GridMap &g, const MaterialTables &mt, int precision);
// algorithmic HBM bytes of one grid step over the lattice the kernel marches
int64_t grid_step_bytes(const GridMap &g, int32_t n_mat, int64_t e, int tile_rows = kGridTileRows);
void grid_create(pn_solver *s);
void grid_sources(pn_solver *s);
void grid_sensors(pn_solver *s, const std::vector<std::pair<int32_t, int32_t>> &sorted);
void grid_run(pn_solver *s, int32_t nsteps);
// writes the idle half of the double buffer and swaps to it unless a value
// is NaN or infinite: returns 0, or bit 1 (velocity) / bit 2 (stress) with the
// state left as it was
int grid_put_state(pn_solver *s, const double *const *V, const double *const *S);
void grid_split_upload(pn_solver *s);  // the fix-up tables of split sites
void grid_get_state(pn_solver *s, double *const *V, double *const *S);

// FP64 form: every tile back on the FP64 path for the next step (state or
// tiling changed; pn_grid.cpp)
void grid_reset_range_flags(pn_solver *s);

// algorithmic HBM bytes of one step in the solver's form
int64_t step_bytes(const pn_solver *s);

// argument blocks of one solver (pointers, tables, constants; the per-step
// fields -- signal row, record, buffers -- are the caller's to set)
template <typename T> void table_args(pn_solver *s, VelArgs<T> &va, StressArgs<T> &sa);
template <typename T> void grid_args(pn_solver *s, GridArgs<T> &a);
// tensor maps of input buffer `in` (0/1) for the tensor-copy kernel, or null
const void *grid_maps_for(const pn_solver *s, int in);

// rebuild the source lists after sources changed (pn_capi.cpp)
void refresh_sources(pn_solver *s);

// the calling thread's message for pn_last_error(); returns code (pn_capi.cpp)
int set_last_error(int code, const std::string &msg);

// FP64 kinetic and strain energy of the current state (pn_energy.cpp)
void energy(pn_solver *s, double &kinetic, double &strain);

// PN_ERR_DEVICE_CHECK (and the word cleared) when a kernel recorded an error
// in the solver's device error word; the stream must be synchronised
int device_check(pn_solver *s);

// issue rates of the arithmetic pipes on the current device (rsg_pipes.cu):
// FP64 FMA, FP64 add, FP32 FMA, double->float, float->double, integer pair
cudaError_t measure_pipe_rates(double *rates, int n);

}  // namespace pn
