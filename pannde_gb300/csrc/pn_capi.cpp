// pn_capi.cpp -- the C ABI (include/pannde_gb300.h): solver object, device
// memory, signal tables and the per-step launch sequence.
//
// A step is two kernel launches on the solver's stream, velocity update then
// stress update, followed by time += dt on the host (HostRSGTDUT.hpp:162-169).
// solve() only enqueues; host reads (get_state, get_traces) synchronise.
// Errors never cross the ABI as exceptions: every entry point catches and
// returns a status, with the message kept per thread for pn_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <memory>
#include <type_traits>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pannde_gb300.h"
#include "pn_setup.hpp"
#include "rsg_common.cuh"

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

struct CudaError {
  cudaError_t e;
  const char *what;
};

void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw CudaError{e, what};
}

// Optional artificial HBM budget (bytes) for allocation-failure tests:
// PN_HBM_BUDGET_BYTES caps the device memory one solver may hold.
int64_t hbm_budget() {
  const char *s = std::getenv("PN_HBM_BUDGET_BYTES");
  if (!s || !*s) return -1;
  return std::strtoll(s, nullptr, 10);
}

constexpr int64_t kSigRowsCap = 1 << 16;  // signal rows uploaded at once

}  // namespace

struct pn_solver {
  int device = 0;
  int precision = PN_PREC_F64;
  cudaStream_t stream = nullptr;
  double dt = 0., time = 0.;
  int64_t step = 0;
  size_t esz = 8;  // bytes per state value

  pn::MeshTables mesh;
  pn::MaterialTables mat;

  std::vector<void *> allocs;
  int64_t dev_bytes = 0;

  void *V[3] = {nullptr, nullptr, nullptr};
  void *S[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int4 *d_hex = nullptr, *d_ncc = nullptr;
  void *d_coef = nullptr, *d_ctab = nullptr, *d_gnode = nullptr, *d_gcell = nullptr;
  int32_t *d_mat = nullptr;

  // sources
  std::vector<pn_window_source> src;
  std::vector<std::vector<double>> src_t, src_v;  // owned copies of signal arrays
  std::vector<pn::Series> series;
  bool src_dirty = false;
  int32_t n_force = 0, n_moment = 0, n_src_nodes = 0, n_src_cells = 0;
  int2 *d_ftile = nullptr, *d_mtile = nullptr;
  int32_t *d_felem = nullptr, *d_fcode = nullptr, *d_melem = nullptr, *d_mcode = nullptr;
  void *d_fw = nullptr, *d_mw = nullptr;
  bool has_moments = false;
  // signal table: rows [sig_step0, sig_step0 + sig_rows) of [n_sig] values;
  // sig_hold: the last row holds for every later step
  void *d_sig = nullptr;
  int64_t sig_step0 = 0, sig_rows = 0, sig_alloc_rows = 0;
  bool sig_hold = false, sig_valid = false;

  // sensors
  int32_t n_sens = 0;
  int2 *d_stile = nullptr;
  int32_t *d_snode = nullptr, *d_sidx = nullptr;
  double *d_traces = nullptr;
  int64_t rec_cap = 0, rec_count = 0;

  // optional per-kernel event timing: (start, end, kernel 0=velocity 1=stress)
  bool timing = false;
  struct Mark { cudaEvent_t a, b; int kind; };
  std::vector<Mark> marks;

  template <typename P>
  P *alloc(size_t bytes) {
    if (bytes == 0) bytes = 16;
    const int64_t budget = hbm_budget();
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

  void release(void *&p) {
    if (!p) return;
    auto it = std::find(allocs.begin(), allocs.end(), p);
    if (it != allocs.end()) allocs.erase(it);
    cudaFree(p);
    p = nullptr;
  }

  bool is_df64() const { return precision == PN_PREC_DF64; }

  // upload a double host array in the storage type (double, float, or the
  // (hi, lo) float pair of the double-float form)
  void upload_real(void *dst, const double *src_, size_t n) {
    if (n == 0) return;
    if (is_df64()) {
      std::vector<float> tmp(2 * n);
      for (size_t i = 0; i < n; i++) pn::split_df(src_[i], tmp[2 * i], tmp[2 * i + 1]);
      ck(cudaMemcpyAsync(dst, tmp.data(), n * 8, cudaMemcpyHostToDevice, stream), "upload");
      ck(cudaStreamSynchronize(stream), "upload sync");
    } else if (esz == 8) {
      ck(cudaMemcpyAsync(dst, src_, n * 8, cudaMemcpyHostToDevice, stream), "upload");
    } else {
      std::vector<float> tmp(n);
      for (size_t i = 0; i < n; i++) tmp[i] = (float)src_[i];
      ck(cudaMemcpyAsync(dst, tmp.data(), n * 4, cudaMemcpyHostToDevice, stream), "upload");
      ck(cudaStreamSynchronize(stream), "upload sync");
    }
  }

  // download n values of the storage type into doubles
  void download_real(double *dst, const void *src_, size_t n) {
    if (n == 0 || !dst) return;
    if (is_df64()) {
      std::vector<float> tmp(2 * n);
      ck(cudaMemcpy(tmp.data(), src_, n * 8, cudaMemcpyDeviceToHost), "download");
      for (size_t i = 0; i < n; i++) dst[i] = (double)tmp[2 * i] + (double)tmp[2 * i + 1];
    } else if (esz == 8) {
      ck(cudaMemcpy(dst, src_, n * 8, cudaMemcpyDeviceToHost), "download");
    } else {
      std::vector<float> tmp(n);
      ck(cudaMemcpy(tmp.data(), src_, n * 4, cudaMemcpyDeviceToHost), "download");
      for (size_t i = 0; i < n; i++) dst[i] = (double)tmp[i];
    }
  }
  void upload_raw(void *dst, const void *src_, size_t bytes) {
    if (bytes == 0) return;
    ck(cudaMemcpyAsync(dst, src_, bytes, cudaMemcpyHostToDevice, stream), "upload");
  }

  void clear_marks() {
    for (auto &m : marks) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
    marks.clear();
  }

  ~pn_solver() {
    clear_marks();
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
  }
};

namespace {

int64_t algorithmic_bytes(const pn_solver *s) {
  // per cell: S read in the velocity step, S read+write in the stress step,
  // material id, cell->node table; per node: V read+write in the velocity
  // step, V read in the stress step, dt/rho, node->cell slots
  const int64_t e = (int64_t)s->esz;
  return (int64_t)s->mesh.n_cells * (6 * e + 12 * e + 4 + 32) +
         (int64_t)s->mesh.n_nodes * (6 * e + 3 * e + e + 32);
}

// device bytes of the fixed tables and state (sources, sensors and signal
// rows come on top and are small)
int64_t footprint(const pn::MeshTables &m, const pn::MaterialTables &mt, int precision) {
  const int64_t nn = m.n_nodes, nc = m.n_cells;
  const int64_t e = precision == PN_PREC_F32 ? 4 : 8;
  const bool per_elem = precision == PN_PREC_F64_EXACT || !m.uniform;
  int64_t need = nn * 3 * e + nc * 6 * e + nc * 32 + nn * 32 + nn * e + nc * 4 +
                 (int64_t)mt.n_mat * 36 * e;
  if (per_elem) need += nn * 3 * e + nc * 3 * e;
  return need;
}

void create_device(pn_solver *s) {
  const int32_t nn = s->mesh.n_nodes, nc = s->mesh.n_cells;
  const size_t e = s->esz;
  const bool exact = s->precision == PN_PREC_F64_EXACT;
  const bool per_elem = exact || !s->mesh.uniform;
  // size everything first so that a budget failure allocates nothing
  const int64_t need = footprint(s->mesh, s->mat, s->precision);
  const int64_t budget = hbm_budget();
  if (budget >= 0 && need > budget)
    throw pn::SetupError{PN_ERR_ALLOC, "solver needs " + std::to_string(need) +
                                           " device bytes, PN_HBM_BUDGET_BYTES is " + std::to_string(budget)};
  ck(cudaGetDevice(&s->device), "cudaGetDevice");
  for (int k = 0; k < 3; k++) s->V[k] = s->alloc<void>((size_t)nn * e);
  for (int k = 0; k < 6; k++) s->S[k] = s->alloc<void>((size_t)nc * e);
  s->d_hex = s->alloc<int4>((size_t)nc * 32);
  s->d_ncc = s->alloc<int4>((size_t)nn * 32);
  s->d_coef = s->alloc<void>((size_t)nn * e);
  s->d_mat = s->alloc<int32_t>((size_t)nc * 4);
  s->d_ctab = s->alloc<void>((size_t)s->mat.n_mat * 36 * e);
  for (int k = 0; k < 3; k++) ck(cudaMemsetAsync(s->V[k], 0, (size_t)nn * e, s->stream), "memset");
  for (int k = 0; k < 6; k++) ck(cudaMemsetAsync(s->S[k], 0, (size_t)nc * e, s->stream), "memset");
  s->upload_raw(s->d_hex, s->mesh.hex.data(), (size_t)nc * 32);
  s->upload_raw(s->d_ncc, s->mesh.ncc.data(), (size_t)nn * 32);
  s->upload_real(s->d_coef, s->mat.coef.data(), nn);
  s->upload_raw(s->d_mat, s->mat.cell_mat.data(), (size_t)nc * 4);
  std::vector<double> ct(s->mat.c36);
  if (!exact)
    for (double &v : ct) v *= s->dt;  // fast forms fold dt into C
  s->upload_real(s->d_ctab, ct.data(), ct.size());
  if (per_elem) {
    std::vector<double> g((size_t)nn * 3), h((size_t)nc * 3);
    const std::vector<double> *dn[3] = {&s->mesh.dxn, &s->mesh.dyn, &s->mesh.dzn};
    const std::vector<double> *dc[3] = {&s->mesh.dxc, &s->mesh.dyc, &s->mesh.dzc};
    for (int a = 0; a < 3; a++) {
      for (int32_t n = 0; n < nn; n++) g[(size_t)a * nn + n] = exact ? (*dn[a])[n] : 0.25 / (*dn[a])[n];
      for (int32_t c = 0; c < nc; c++) h[(size_t)a * nc + c] = exact ? (*dc[a])[c] : 0.25 / (*dc[a])[c];
    }
    s->d_gnode = s->alloc<void>(g.size() * e);
    s->d_gcell = s->alloc<void>(h.size() * e);
    s->upload_real(s->d_gnode, g.data(), g.size());
    s->upload_real(s->d_gcell, h.data(), h.size());
  }
  ck(cudaStreamSynchronize(s->stream), "create sync");
}

// a host double in the storage type T
template <typename T> T to_store(double v);
template <> double to_store<double>(double v) { return v; }
template <> float to_store<float>(double v) { return (float)v; }
template <> float2 to_store<float2>(double v) {
  float2 r;
  pn::split_df(v, r.x, r.y);
  return r;
}

template <typename T>
void fill_launch_args(pn_solver *s, pn::VelArgs<T> &va, pn::StressArgs<T> &sa) {
  std::memset(&va, 0, sizeof(va));
  std::memset(&sa, 0, sizeof(sa));
  const bool exact = s->precision == PN_PREC_F64_EXACT;
  va.n_nodes = s->mesh.n_nodes;
  va.ncc = s->d_ncc;
  va.V0 = (T *)s->V[0]; va.V1 = (T *)s->V[1]; va.V2 = (T *)s->V[2];
  va.S0 = (const T *)s->S[0]; va.S1 = (const T *)s->S[1]; va.S2 = (const T *)s->S[2];
  va.S3 = (const T *)s->S[3]; va.S4 = (const T *)s->S[4]; va.S5 = (const T *)s->S[5];
  va.coef = (const T *)s->d_coef;
  va.gx = to_store<T>(0.25 / s->mesh.hx);
  va.gy = to_store<T>(0.25 / s->mesh.hy);
  va.gz = to_store<T>(0.25 / s->mesh.hz);
  va.gnode = (const T *)s->d_gnode;
  if (s->n_force > 0) {
    va.tile_src = s->d_ftile; va.src_elem = s->d_felem; va.src_code = s->d_fcode;
    va.src_w = (const T *)s->d_fw;
  }
  va.n_sig = (int32_t)s->src.size();
  if (s->n_sens > 0) {
    va.tile_sens = s->d_stile; va.sens_node = s->d_snode; va.sens_idx = s->d_sidx;
    va.traces = s->d_traces; va.n_sens = s->n_sens; va.rec_cap = s->rec_cap;
  }
  sa.n_cells = s->mesh.n_cells;
  sa.hex = s->d_hex;
  sa.V0 = (const T *)s->V[0]; sa.V1 = (const T *)s->V[1]; sa.V2 = (const T *)s->V[2];
  sa.S0 = (T *)s->S[0]; sa.S1 = (T *)s->S[1]; sa.S2 = (T *)s->S[2];
  sa.S3 = (T *)s->S[3]; sa.S4 = (T *)s->S[4]; sa.S5 = (T *)s->S[5];
  sa.mat = s->d_mat;
  sa.ctab = (const T *)s->d_ctab;
  sa.gx = va.gx; sa.gy = va.gy; sa.gz = va.gz;
  sa.gcell = (const T *)s->d_gcell;
  sa.dt = to_store<T>(s->dt);
  if (s->n_moment > 0) {
    sa.tile_src = s->d_mtile; sa.src_elem = s->d_melem; sa.src_code = s->d_mcode;
    sa.src_w = (const T *)s->d_mw;
  }
  sa.n_sig = va.n_sig;
  sa.has_moments = s->has_moments ? 1 : 0;
  (void)exact;
}

// rebuild the sparse source lists on the device
void rebuild_sources(pn_solver *s) {
  const bool exact = s->precision == PN_PREC_F64_EXACT;
  std::vector<pn::SourceEntry> fe, me;
  pn::build_source_entries(s->mesh, s->src, exact, fe, me);
  ck(cudaStreamSynchronize(s->stream), "sources sync");
  void **olds[] = {(void **)&s->d_ftile, (void **)&s->d_felem, (void **)&s->d_fcode, &s->d_fw,
                   (void **)&s->d_mtile, (void **)&s->d_melem, (void **)&s->d_mcode, &s->d_mw};
  for (void **p : olds) s->release(*p);
  s->n_force = (int32_t)fe.size();
  s->n_moment = (int32_t)me.size();
  bool mom = false;
  for (auto &w : s->src) mom = mom || (w.kind == PN_SOURCE_MOMENT);
  s->has_moments = mom;
  auto upload_list = [&](const std::vector<pn::SourceEntry> &L, int32_t n_elem, int shift, bool fold_dt,
                         int2 *&tile, int32_t *&elem, int32_t *&code, void *&w, int32_t &n_touched) {
    n_touched = 0;
    if (L.empty()) return;
    std::vector<int32_t> el(L.size()), cd(L.size()), rg;
    std::vector<double> wt(L.size());
    for (size_t i = 0; i < L.size(); i++) {
      el[i] = L[i].elem;
      cd[i] = L[i].comp | (L[i].sig << shift);
      wt[i] = (fold_dt && !exact) ? s->dt * L[i].w : L[i].w;
      if (i == 0 || L[i].elem != L[i - 1].elem) n_touched++;
    }
    pn::tile_ranges(el, n_elem, pn::kTile, rg);
    tile = s->alloc<int2>(rg.size() * 4);
    elem = s->alloc<int32_t>(el.size() * 4);
    code = s->alloc<int32_t>(cd.size() * 4);
    w = s->alloc<void>(wt.size() * s->esz);
    s->upload_raw(tile, rg.data(), rg.size() * 4);
    s->upload_raw(elem, el.data(), el.size() * 4);
    s->upload_raw(code, cd.data(), cd.size() * 4);
    s->upload_real(w, wt.data(), wt.size());
  };
  upload_list(fe, s->mesh.n_nodes, 2, false, s->d_ftile, s->d_felem, s->d_fcode, s->d_fw, s->n_src_nodes);
  upload_list(me, s->mesh.n_cells, 3, true, s->d_mtile, s->d_melem, s->d_mcode, s->d_mw, s->n_src_cells);
  ck(cudaStreamSynchronize(s->stream), "sources upload");
  s->src_dirty = false;
  s->sig_valid = false;
}

// make the signal table cover global steps [s->step, s->step + nsteps)
void ensure_signal_rows(pn_solver *s, int64_t nsteps) {
  const int64_t nsig = (int64_t)s->src.size();
  if (nsig == 0) return;
  const int64_t first = s->step, last = s->step + nsteps - 1;
  if (s->sig_valid && first >= s->sig_step0 &&
      (s->sig_hold || last < s->sig_step0 + s->sig_rows))
    return;
  double tmax = -1e300;
  for (auto &sr : s->series) tmax = std::max(tmax, sr.last_time());
  // rows for at least this call (capped), fewer once every signal holds
  const int64_t want = std::min<int64_t>(std::max<int64_t>(nsteps, 1024), kSigRowsCap);
  std::vector<double> rows;
  rows.reserve((size_t)want * nsig);
  double t = s->time;
  int64_t r = 0;
  bool hold = false;
  for (;;) {
    for (int64_t k = 0; k < nsig; k++) rows.push_back(s->series[k].eval(t));
    r++;
    if (t >= tmax && s->dt > 0) { hold = true; break; }  // every signal past its last sample
    if (r >= want) break;
    t += s->dt;  // the same accumulation as solve(): time += dt
  }
  ck(cudaStreamSynchronize(s->stream), "signal sync");
  if (r > s->sig_alloc_rows) {
    s->release(s->d_sig);
    s->d_sig = s->alloc<void>((size_t)r * nsig * s->esz);
    s->sig_alloc_rows = r;
  }
  s->upload_real(s->d_sig, rows.data(), rows.size());
  ck(cudaStreamSynchronize(s->stream), "signal upload");
  s->sig_step0 = s->step;
  s->sig_rows = r;
  s->sig_hold = hold;
  s->sig_valid = true;
}

template <typename T>
void run_steps(pn_solver *s, int32_t nsteps) {
  pn::VelArgs<T> va;
  pn::StressArgs<T> sa;
  fill_launch_args<T>(s, va, sa);
  const int64_t nsig = (int64_t)s->src.size();
  int32_t done = 0;
  while (done < nsteps) {
    int32_t chunk = nsteps - done;
    ensure_signal_rows(s, chunk);
    if (nsig > 0 && !s->sig_hold)
      chunk = (int32_t)std::min<int64_t>(chunk, s->sig_step0 + s->sig_rows - s->step);
    va.rec_base = s->rec_count;
    for (int32_t k = 0; k < chunk; k++) {
      if (nsig > 0) {
        const int64_t row = std::min<int64_t>(s->step + k - s->sig_step0, s->sig_rows - 1);
        va.sigval = (const T *)s->d_sig + row * nsig;
        sa.sigval = va.sigval;
      }
      cudaError_t e1, e2;
      pn_solver::Mark mv{}, ms{};
      if (s->timing) {
        for (auto *m : {&mv, &ms}) {
          ck(cudaEventCreate(&m->a), "event");
          ck(cudaEventCreate(&m->b), "event");
        }
        mv.kind = 0;
        ms.kind = 1;
        ck(cudaEventRecord(mv.a, s->stream), "event");
      }
      auto between = [&]() {
        if (!s->timing) return;
        ck(cudaEventRecord(mv.b, s->stream), "event");
        ck(cudaEventRecord(ms.a, s->stream), "event");
      };
      if constexpr (std::is_same<T, float2>::value) {
        e1 = pn::launch_velocity_df64(va, k, s->mesh.uniform, s->stream);
        between();
        e2 = pn::launch_stress_df64(sa, k, s->mesh.uniform, s->stream);
      } else if constexpr (std::is_same<T, double>::value) {
        if (s->precision == PN_PREC_F64_EXACT) {
          e1 = pn::launch_velocity_exact(va, k, s->stream);
          between();
          e2 = pn::launch_stress_exact(sa, k, s->stream);
        } else {
          e1 = pn::launch_velocity_f64(va, k, s->mesh.uniform, s->stream);
          between();
          e2 = pn::launch_stress_f64(sa, k, s->mesh.uniform, s->stream);
        }
      } else {
        e1 = pn::launch_velocity_f32(va, k, s->mesh.uniform, s->stream);
        between();
        e2 = pn::launch_stress_f32(sa, k, s->mesh.uniform, s->stream);
      }
      if (s->timing) {
        ck(cudaEventRecord(ms.b, s->stream), "event");
        s->marks.push_back(mv);
        s->marks.push_back(ms);
      }
      ck(e1, "velocity launch");
      ck(e2, "stress launch");
      s->time += s->dt;  // HostRSGTDUT.hpp:166
    }
    s->step += chunk;
    s->rec_count += chunk;
    done += chunk;
  }
}

template <typename F>
int guarded(F &&f) {
  g_err.clear();
  try {
    return f();
  } catch (const pn::SetupError &e) {
    return set_err(e.code, e.msg);
  } catch (const CudaError &e) {
    (void)cudaGetLastError();
    return set_err(PN_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::bad_alloc &) {
    return set_err(PN_ERR_ALLOC, "host allocation failed");
  } catch (const std::exception &e) {
    return set_err(PN_ERR_RUNTIME, e.what());
  }
}

int create_common(const pn_mesh *mesh, double dt, int32_t precision, pn_solver **out,
                  const pn_material *fields, const pn_material_table *table) {
  return guarded([&]() -> int {
    if (!out) return set_err(PN_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!mesh) return set_err(PN_ERR_INVALID, "null mesh");
    if (precision < PN_PREC_F64_EXACT || precision > PN_PREC_DF64)
      return set_err(PN_ERR_INVALID, "unknown precision");
    if (!std::isfinite(dt)) return set_err(PN_ERR_NOT_FINITE, "non-finite dt");
    std::unique_ptr<pn_solver> s(new pn_solver());
    s->precision = precision;
    s->esz = precision == PN_PREC_F32 ? 4 : 8;
    s->dt = dt;
    pn::build_mesh_tables(*mesh, s->mesh);
    if (fields) pn::build_material_from_fields(*fields, s->mesh, dt, s->mat);
    else pn::build_material_from_table(*table, s->mesh, dt, s->mat);
    create_device(s.get());
    *out = s.release();
    return PN_OK;
  });
}

}  // namespace

extern "C" {

int pn_abi_version(void) { return PN_ABI_VERSION; }

const char *pn_last_error(void) { return g_err.c_str(); }

int pn_plan_solver(const pn_mesh *mesh, const pn_material *material, const pn_material_table *table,
                   double dt, int32_t precision, pn_plan *out) {
  return guarded([&]() -> int {
    if (!mesh || !out || (!material && !table) || (material && table))
      return set_err(PN_ERR_INVALID, "plan arguments");
    if (precision < PN_PREC_F64_EXACT || precision > PN_PREC_DF64)
      return set_err(PN_ERR_INVALID, "unknown precision");
    if (!std::isfinite(dt)) return set_err(PN_ERR_NOT_FINITE, "non-finite dt");
    pn::MeshTables m;
    pn::MaterialTables mt;
    pn::build_mesh_tables(*mesh, m);
    if (material) pn::build_material_from_fields(*material, m, dt, mt);
    else pn::build_material_from_table(*table, m, dt, mt);
    std::memset(out, 0, sizeof(*out));
    out->n_nodes = m.n_nodes;
    out->n_cells = m.n_cells;
    out->n_materials = mt.n_mat;
    out->uniform_spacing = m.uniform ? 1 : 0;
    out->hx = m.hx;
    out->hy = m.hy;
    out->hz = m.hz;
    out->device_bytes = footprint(m, mt, precision);
    const int64_t e = precision == PN_PREC_F32 ? 4 : 8;
    out->algorithmic_bytes_per_step =
        (int64_t)m.n_cells * (18 * e + 36) + (int64_t)m.n_nodes * (10 * e + 32);
    return PN_OK;
  });
}

int pn_plan_sources(const pn_mesh *mesh, const pn_window_source *src, int32_t n, double *node_force_w,
                    double *cell_moment_w, int32_t *n_source_nodes, int32_t *n_source_cells) {
  return guarded([&]() -> int {
    if (!mesh || n < 0 || (n > 0 && !src)) return set_err(PN_ERR_INVALID, "plan arguments");
    pn::MeshTables m;
    pn::build_mesh_tables(*mesh, m);
    std::vector<pn_window_source> all(src, src + n);
    std::vector<pn::SourceEntry> fe, me;
    pn::build_source_entries(m, all, false, fe, me);
    if (node_force_w)
      std::fill(node_force_w, node_force_w + (size_t)m.n_nodes * 3, 0.0);
    if (cell_moment_w)
      std::fill(cell_moment_w, cell_moment_w + (size_t)m.n_cells * 6, 0.0);
    int32_t nn = 0, nc = 0;
    for (size_t i = 0; i < fe.size(); i++) {
      if (node_force_w) node_force_w[(size_t)fe[i].elem * 3 + fe[i].comp] += fe[i].w;
      if (i == 0 || fe[i].elem != fe[i - 1].elem) nn++;
    }
    for (size_t i = 0; i < me.size(); i++) {
      if (cell_moment_w) cell_moment_w[(size_t)me[i].elem * 6 + me[i].comp] += me[i].w;
      if (i == 0 || me[i].elem != me[i - 1].elem) nc++;
    }
    if (n_source_nodes) *n_source_nodes = nn;
    if (n_source_cells) *n_source_cells = nc;
    return PN_OK;
  });
}

int pn_signal_eval(const pn_signal *signal, const double *t, int32_t n, double *out) {
  return guarded([&]() -> int {
    if (!signal || n < 0 || (n > 0 && (!t || !out))) return set_err(PN_ERR_INVALID, "signal arguments");
    pn::Series s;
    s.build(*signal);
    for (int32_t i = 0; i < n; i++) out[i] = s.eval(t[i]);
    return PN_OK;
  });
}

int pn_solver_create(const pn_mesh *mesh, const pn_material *material, double dt,
                     int32_t precision, pn_solver **out) {
  if (!material) return set_err(PN_ERR_INVALID, "null material");
  return create_common(mesh, dt, precision, out, material, nullptr);
}

int pn_solver_create_indexed(const pn_mesh *mesh, const pn_material_table *material, double dt,
                             int32_t precision, pn_solver **out) {
  if (!material) return set_err(PN_ERR_INVALID, "null material table");
  return create_common(mesh, dt, precision, out, nullptr, material);
}

int pn_solver_set_stream(pn_solver *s, void *cuda_stream) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    ck(cudaStreamSynchronize(s->stream), "stream switch");
    s->stream = (cudaStream_t)cuda_stream;
    return PN_OK;
  });
}

int pn_solver_set_state(pn_solver *s, const double *const *V, const double *const *S) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    const int32_t nn = s->mesh.n_nodes, nc = s->mesh.n_cells;
    for (int k = 0; k < 3; k++)
      if (V && V[k] && !pn::all_finite(V[k], nn)) return set_err(PN_ERR_NOT_FINITE, "non-finite velocity");
    for (int k = 0; k < 6; k++)
      if (S && S[k] && !pn::all_finite(S[k], nc)) return set_err(PN_ERR_NOT_FINITE, "non-finite stress");
    ck(cudaStreamSynchronize(s->stream), "set_state sync");
    for (int k = 0; k < 3; k++) {
      if (V && V[k]) s->upload_real(s->V[k], V[k], nn);
      else ck(cudaMemsetAsync(s->V[k], 0, (size_t)nn * s->esz, s->stream), "memset");
    }
    for (int k = 0; k < 6; k++) {
      if (S && S[k]) s->upload_real(s->S[k], S[k], nc);
      else ck(cudaMemsetAsync(s->S[k], 0, (size_t)nc * s->esz, s->stream), "memset");
    }
    ck(cudaStreamSynchronize(s->stream), "set_state");
    return PN_OK;
  });
}

int pn_solver_add_sources(pn_solver *s, const pn_window_source *src, int32_t n) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (n < 0 || (n > 0 && !src)) return set_err(PN_ERR_INVALID, "source list");
    std::vector<pn_window_source> all(s->src);
    std::vector<std::vector<double>> ts(s->src_t), vs(s->src_v);
    std::vector<pn::Series> ser(s->series);
    for (int32_t i = 0; i < n; i++) {
      pn::Series sr;
      sr.build(src[i].signal);
      pn_window_source w = src[i];
      ts.emplace_back(src[i].signal.t, src[i].signal.t + src[i].signal.n);
      vs.emplace_back(src[i].signal.v, src[i].signal.v + src[i].signal.n);
      all.push_back(w);
      ser.push_back(sr);
    }
    for (size_t i = 0; i < all.size(); i++) {  // re-point at the owned copies
      all[i].signal.t = ts[i].data();
      all[i].signal.v = vs[i].data();
    }
    // validate the whole set before committing (group/slot conflicts)
    std::vector<pn::SourceEntry> fe, me;
    {
      pn::MeshTables empty;
      pn::build_source_entries(empty, all, true, fe, me);
    }
    if (all.size() > (size_t)(1 << 27)) return set_err(PN_ERR_INVALID, "too many sources");
    s->src.swap(all);
    s->src_t.swap(ts);
    s->src_v.swap(vs);
    s->series.swap(ser);
    s->src_dirty = true;
    s->sig_valid = false;
    return PN_OK;
  });
}

int pn_solver_set_sensors(pn_solver *s, const int32_t *nodes, int32_t n, int32_t capacity_steps) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (n < 0 || capacity_steps < 0 || (n > 0 && !nodes)) return set_err(PN_ERR_INVALID, "sensor list");
    for (int32_t i = 0; i < n; i++)
      if (nodes[i] < 0 || nodes[i] >= s->mesh.n_nodes) return set_err(PN_ERR_RANGE, "sensor node out of range");
    ck(cudaStreamSynchronize(s->stream), "sensors sync");
    void **olds[] = {(void **)&s->d_stile, (void **)&s->d_snode, (void **)&s->d_sidx, (void **)&s->d_traces};
    for (void **p : olds) s->release(*p);
    s->n_sens = 0;
    s->rec_cap = 0;
    s->rec_count = 0;
    if (n == 0) return PN_OK;
    std::vector<std::pair<int32_t, int32_t>> pr((size_t)n);
    for (int32_t i = 0; i < n; i++) pr[i] = {nodes[i], i};
    std::sort(pr.begin(), pr.end());
    std::vector<int32_t> nd(n), ix(n), rg;
    for (int32_t i = 0; i < n; i++) { nd[i] = pr[i].first; ix[i] = pr[i].second; }
    pn::tile_ranges(nd, s->mesh.n_nodes, pn::kTile, rg);
    s->d_stile = s->alloc<int2>(rg.size() * 4);
    s->d_snode = s->alloc<int32_t>((size_t)n * 4);
    s->d_sidx = s->alloc<int32_t>((size_t)n * 4);
    s->d_traces = s->alloc<double>((size_t)std::max(capacity_steps, 1) * n * 3 * 8);
    s->upload_raw(s->d_stile, rg.data(), rg.size() * 4);
    s->upload_raw(s->d_snode, nd.data(), nd.size() * 4);
    s->upload_raw(s->d_sidx, ix.data(), ix.size() * 4);
    ck(cudaStreamSynchronize(s->stream), "sensors upload");
    s->n_sens = n;
    s->rec_cap = capacity_steps;
    return PN_OK;
  });
}

int pn_solver_solve(pn_solver *s, int32_t nsteps, double *time_out) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (nsteps < 0) return set_err(PN_ERR_INVALID, "negative step count");
    if (s->src_dirty) rebuild_sources(s);
    if (s->is_df64()) run_steps<float2>(s, nsteps);
    else if (s->esz == 8) run_steps<double>(s, nsteps);
    else run_steps<float>(s, nsteps);
    if (time_out) *time_out = s->time;
    return PN_OK;
  });
}

int pn_solver_get_state(pn_solver *s, double *const *V, double *const *S) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    ck(cudaStreamSynchronize(s->stream), "get_state sync");
    for (int k = 0; k < 3; k++) if (V) s->download_real(V[k], s->V[k], (size_t)s->mesh.n_nodes);
    for (int k = 0; k < 6; k++) if (S) s->download_real(S[k], s->S[k], (size_t)s->mesh.n_cells);
    return PN_OK;
  });
}

int pn_solver_get_traces(pn_solver *s, double *out, int64_t max_records, int64_t *n_records) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (max_records < 0 || (max_records > 0 && !out)) return set_err(PN_ERR_INVALID, "trace buffer");
    ck(cudaStreamSynchronize(s->stream), "get_traces sync");
    const int64_t have = std::min(s->rec_count, s->rec_cap);
    const int64_t n = std::min(have, max_records);
    if (n > 0 && s->n_sens > 0)
      ck(cudaMemcpy(out, s->d_traces, (size_t)n * s->n_sens * 3 * 8, cudaMemcpyDeviceToHost), "traces");
    if (n_records) *n_records = have;
    return PN_OK;
  });
}

int pn_solver_clear_traces(pn_solver *s) {
  if (!s) return set_err(PN_ERR_INVALID, "null solver");
  s->rec_count = 0;
  return PN_OK;
}

int pn_solver_get_time(pn_solver *s, double *time_out) {
  if (!s || !time_out) return set_err(PN_ERR_INVALID, "null argument");
  *time_out = s->time;
  return PN_OK;
}

int pn_solver_get_info(pn_solver *s, pn_solver_info *info) {
  if (!s || !info) return set_err(PN_ERR_INVALID, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->n_nodes = s->mesh.n_nodes;
  info->n_cells = s->mesh.n_cells;
  info->precision = s->precision;
  info->n_materials = s->mat.n_mat;
  info->uniform_spacing = s->mesh.uniform ? 1 : 0;
  info->n_source_nodes = s->n_src_nodes;
  info->n_source_cells = s->n_src_cells;
  info->n_sensors = s->n_sens;
  info->algorithmic_bytes_per_step = algorithmic_bytes(s);
  info->device_bytes = s->dev_bytes;
  info->dt = s->dt;
  info->time = s->time;
  return PN_OK;
}

int pn_solver_device_state(pn_solver *s, void **V, void **S) {
  if (!s || !V || !S) return set_err(PN_ERR_INVALID, "null argument");
  for (int k = 0; k < 3; k++) V[k] = s->V[k];
  for (int k = 0; k < 6; k++) S[k] = s->S[k];
  return PN_OK;
}

int pn_solver_synchronize(pn_solver *s) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    ck(cudaStreamSynchronize(s->stream), "synchronize");
    ck(cudaGetLastError(), "device error");
    return PN_OK;
  });
}

int pn_solver_enable_kernel_timing(pn_solver *s, int32_t enable) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    ck(cudaStreamSynchronize(s->stream), "timing sync");
    s->clear_marks();
    s->timing = enable != 0;
    return PN_OK;
  });
}

int pn_solver_kernel_times(pn_solver *s, double *ms, int64_t *launches) {
  return guarded([&]() -> int {
    if (!s || !ms || !launches) return set_err(PN_ERR_INVALID, "null argument");
    ck(cudaStreamSynchronize(s->stream), "timing sync");
    ms[0] = ms[1] = 0.;
    launches[0] = launches[1] = 0;
    for (auto &m : s->marks) {
      float t = 0.f;
      ck(cudaEventElapsedTime(&t, m.a, m.b), "elapsed");
      ms[m.kind] += t;
      launches[m.kind] += 1;
    }
    s->clear_marks();
    return PN_OK;
  });
}

int pn_solver_destroy(pn_solver *s) {
  if (!s) return PN_OK;
  cudaStreamSynchronize(s->stream);
  delete s;
  return PN_OK;
}

}  // extern "C"
