// pn_capi.cpp -- the C ABI (include/pannde_gb300.h): validation, the choice
// of device form, signal tables, and dispatch to the table form
// (pn_table.cpp) or the grid form (pn_grid.cpp).
//
// A step advances the velocity and then the stress of every element and adds
// dt to the time on the host (HostRSGTDUT.hpp:162-169).  solve() only
// enqueues; host reads (get_state, get_traces) synchronise.  Errors never
// cross the ABI as exceptions: every entry point catches and returns a
// status, with the message kept per thread for pn_last_error().
#include <cmath>
#include <cstring>
#include <memory>

#include "pn_solver.hpp"

namespace pn {

void ensure_signal_rows(pn_solver *s, int64_t nsteps, bool may_alloc) {
  const int64_t nsig = (int64_t)s->src.size();
  if (nsig == 0 || s->caller_signals) return;  // caller rows cover the whole call
  const int64_t first = s->step, last = s->step + nsteps - 1;
  if (s->sig_valid && first >= s->sig_step0 && (s->sig_hold || last < s->sig_step0 + s->sig_rows))
    return;
  double tmax = -1e300;
  for (auto &sr : s->series) tmax = std::max(tmax, sr.last_time());
  // rows for at least this call (capped), fewer once every signal holds;
  // without allocation, at most the rows the table already has
  int64_t want = std::min<int64_t>(std::max<int64_t>(nsteps, 1024), kSigRowsCap);
  if (!may_alloc) {
    if (s->sig_alloc_rows <= 0) throw SetupError{PN_ERR_INVALID, "signal table not resident"};
    want = std::min<int64_t>(want, s->sig_alloc_rows);
  }
  std::vector<double> rows;
  rows.reserve((size_t)want * nsig);
  double t = s->time;
  int64_t r = 0;
  bool hold = false;
  for (;;) {
    for (int64_t k = 0; k < nsig; k++) rows.push_back(s->series[k].eval(t));
    r++;
    if (t >= tmax && s->dt > 0) {  // every signal past its last sample
      hold = true;
      break;
    }
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

int64_t sig_row(const pn_solver *s, int64_t k) {
  return std::min<int64_t>(s->step + k - s->sig_step0, s->sig_rows - 1);
}

int64_t step_bytes(const pn_solver *s) {
  const int64_t e = (int64_t)s->esz;
  if (s->form == PN_FORM_GRID) {
    // S read + write, material byte per marched lattice cell; V read + write,
    // dt/rho per marched node (fixed at creation)
    if (s->step_bytes_cached == 0) s->step_bytes_cached = grid_step_bytes(s->grid, s->mat.n_mat, e, s->tile_rows);
    return s->step_bytes_cached;
  }
  // per cell: S read in the velocity step, S read+write in the stress step,
  // material id, cell->node table; per node: V read+write in the velocity
  // step, V read in the stress step, dt/rho, node->cell slots
  return (int64_t)s->mesh.n_cells * (18 * e + 36) + (int64_t)s->mesh.n_nodes * (10 * e + 32);
}

}  // namespace pn

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

template <typename F>
int guarded(F &&f) {
  g_err.clear();
  try {
    return f();
  } catch (const pn::SetupError &e) {
    return set_err(e.code, e.msg);
  } catch (const pn::CudaError &e) {
    (void)cudaGetLastError();
    return set_err(PN_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::bad_alloc &) {
    return set_err(PN_ERR_ALLOC, "host allocation failed");
  } catch (const std::exception &e) {
    return set_err(PN_ERR_RUNTIME, e.what());
  }
}

// precision and form from the combined argument
bool split_mode(int32_t mode, int &precision, int &form) {
  precision = mode & 0xff;
  form = mode & PN_FORM_MASK;
  if ((mode & ~(0xff | PN_FORM_MASK)) != 0) return false;
  if (precision < PN_PREC_F64_EXACT || precision > PN_PREC_DF64) return false;
  return form == PN_FORM_AUTO || form == PN_FORM_TABLE || form == PN_FORM_GRID;
}

// the form a mesh gets; throws when PN_FORM_GRID is asked of a non-grid mesh
int choose_form(const pn::MeshTables &m, const pn::MaterialTables &mt, int precision, int form,
                pn::GridMap &g) {
  auto table = [&]() {
    if (m.n_nodes > pn::kTableMaxElems || m.n_cells > pn::kTableMaxElems)
      throw pn::SetupError{PN_ERR_INVALID, "mesh too large for the connectivity-table form (at most " +
                                               std::to_string(pn::kTableMaxElems) + " nodes and cells)"};
    return PN_FORM_TABLE;
  };
  if (form == PN_FORM_TABLE) return table();
  pn::detect_grid(m, g);
  std::string why;
  if (pn::grid_eligible(m, mt, precision, g, &why)) return PN_FORM_GRID;
  if (form == PN_FORM_GRID) throw pn::SetupError{PN_ERR_INVALID, "grid form unavailable: " + why};
  return table();
}

int create_common(const pn_mesh *mesh, double dt, int32_t mode, pn_solver **out,
                  const pn_material *fields, const pn_material_table *table) {
  return guarded([&]() -> int {
    if (!out) return set_err(PN_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!mesh) return set_err(PN_ERR_INVALID, "null mesh");
    int precision, form;
    if (!split_mode(mode, precision, form)) return set_err(PN_ERR_INVALID, "unknown precision or form");
    if (!std::isfinite(dt)) return set_err(PN_ERR_NOT_FINITE, "non-finite dt");
    std::unique_ptr<pn_solver> s(new pn_solver());
    s->precision = precision;
    s->esz = precision == PN_PREC_F32 ? 4 : 8;
    s->dt = dt;
    pn::build_mesh_tables(*mesh, s->mesh);
    if (fields) pn::build_material_from_fields(*fields, s->mesh, dt, s->mat);
    else pn::build_material_from_table(*table, s->mesh, dt, s->mat);
    s->form = choose_form(s->mesh, s->mat, precision, form, s->grid);
    // size everything first so that a budget failure allocates nothing
    const int64_t need = s->form == PN_FORM_GRID ? pn::grid_footprint(s->grid, s->mat, precision)
                                                 : pn::table_footprint(s->mesh, s->mat, precision);
    const int64_t budget = pn::hbm_budget();
    if (budget >= 0 && need > budget)
      return set_err(PN_ERR_ALLOC, "solver needs " + std::to_string(need) +
                                       " device bytes, PN_HBM_BUDGET_BYTES is " + std::to_string(budget));
    pn::ck(cudaGetDevice(&s->device), "cudaGetDevice");
    if (s->form == PN_FORM_GRID) pn::grid_create(s.get());
    else pn::table_create(s.get());
    *out = s.release();
    return PN_OK;
  });
}

}  // namespace

extern "C" {

int pn_abi_version(void) { return PN_ABI_VERSION; }

const char *pn_last_error(void) { return g_err.c_str(); }

int pn_plan_solver(const pn_mesh *mesh, const pn_material *material, const pn_material_table *table,
                   double dt, int32_t mode, pn_plan *out) {
  return guarded([&]() -> int {
    if (!mesh || !out || (!material && !table) || (material && table))
      return set_err(PN_ERR_INVALID, "plan arguments");
    int precision, form;
    if (!split_mode(mode, precision, form)) return set_err(PN_ERR_INVALID, "unknown precision or form");
    if (!std::isfinite(dt)) return set_err(PN_ERR_NOT_FINITE, "non-finite dt");
    pn::MeshTables m;
    pn::MaterialTables mt;
    pn::build_mesh_tables(*mesh, m);
    if (material) pn::build_material_from_fields(*material, m, dt, mt);
    else pn::build_material_from_table(*table, m, dt, mt);
    pn::GridMap g;
    const int f = choose_form(m, mt, precision, form, g);
    std::memset(out, 0, sizeof(*out));
    out->n_nodes = m.n_nodes;
    out->n_cells = m.n_cells;
    out->n_materials = mt.n_mat;
    out->uniform_spacing = m.uniform ? 1 : 0;
    out->hx = m.hx;
    out->hy = m.hy;
    out->hz = m.hz;
    out->form = f;
    const int64_t e = precision == PN_PREC_F32 ? 4 : 8;
    if (f == PN_FORM_GRID) {
      out->device_bytes = pn::grid_footprint(g, mt, precision);
      out->algorithmic_bytes_per_step = pn::grid_step_bytes(g, mt.n_mat, e);
      out->grid[0] = g.nx;
      out->grid[1] = g.ny;
      out->grid[2] = g.nz;
    } else {
      out->device_bytes = pn::table_footprint(m, mt, precision);
      out->algorithmic_bytes_per_step = (int64_t)m.n_cells * (18 * e + 36) + (int64_t)m.n_nodes * (10 * e + 32);
    }
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
    if (node_force_w) std::fill(node_force_w, node_force_w + (size_t)m.n_nodes * 3, 0.0);
    if (cell_moment_w) std::fill(cell_moment_w, cell_moment_w + (size_t)m.n_cells * 6, 0.0);
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

int pn_solver_create(const pn_mesh *mesh, const pn_material *material, double dt, int32_t precision,
                     pn_solver **out) {
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
    pn::ck(cudaStreamSynchronize(s->stream), "stream switch");
    s->stream = (cudaStream_t)cuda_stream;
    return PN_OK;
  });
}

int pn_solver_set_state(pn_solver *s, const double *const *V, const double *const *S) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    const int32_t nn = s->mesh.n_nodes, nc = s->mesh.n_cells;
    pn::ck(cudaStreamSynchronize(s->stream), "set_state sync");
    if (s->form == PN_FORM_GRID) {  // checked on the device while it is written to the idle buffer half
      const int bad = pn::grid_put_state(s, V, S);
      if (bad & 1) return set_err(PN_ERR_NOT_FINITE, "non-finite velocity");
      if (bad & 2) return set_err(PN_ERR_NOT_FINITE, "non-finite stress");
      return PN_OK;
    }
    for (int k = 0; k < 3; k++)
      if (V && V[k] && !pn::all_finite(V[k], nn)) return set_err(PN_ERR_NOT_FINITE, "non-finite velocity");
    for (int k = 0; k < 6; k++)
      if (S && S[k] && !pn::all_finite(S[k], nc)) return set_err(PN_ERR_NOT_FINITE, "non-finite stress");
    pn::table_put_state(s, V, S);
    pn::ck(cudaStreamSynchronize(s->stream), "set_state");
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
      ts.emplace_back(src[i].signal.t, src[i].signal.t + src[i].signal.n);
      vs.emplace_back(src[i].signal.v, src[i].signal.v + src[i].signal.n);
      all.push_back(src[i]);
      ser.push_back(sr);
    }
    if (all.size() > (size_t)(1 << 20)) return set_err(PN_ERR_INVALID, "too many sources");
    for (size_t i = 0; i < all.size(); i++) {  // point at the owned copies
      all[i].signal.t = ts[i].data();
      all[i].signal.v = vs[i].data();
    }
    {  // validate the whole set (kinds, groups, slots) before committing
      std::vector<pn::SourceEntry> fe, me;
      pn::MeshTables empty;
      pn::build_source_entries(empty, all, true, fe, me);
    }
    s->src.swap(all);
    s->src_t.swap(ts);
    s->src_v.swap(vs);
    s->series.swap(ser);
    s->src_mask.resize(s->src.size());  // geometry sources carry no mask
    bool mom = false;
    for (auto &w : s->src) mom = mom || (w.kind == PN_SOURCE_MOMENT);
    s->has_moments = mom;
    s->src_dirty = true;
    s->sig_valid = false;
    return PN_OK;
  });
}

int pn_solver_add_window_masks(pn_solver *s, const pn_window_mask *masks, int32_t n) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (n < 0 || (n > 0 && !masks)) return set_err(PN_ERR_INVALID, "mask list");
    std::vector<pn_window_source> all(s->src);
    for (int32_t i = 0; i < n; i++) {
      if (!masks[i].inside) return set_err(PN_ERR_INVALID, "null window mask");
      pn_window_source w;
      std::memset(&w, 0, sizeof(w));
      w.kind = masks[i].kind;
      w.group = masks[i].group;
      w.component = masks[i].component;
      all.push_back(w);
    }
    {  // validate kinds, groups and slots with the existing sources
      std::vector<pn::SourceEntry> fe, me;
      pn::MeshTables empty;
      pn::build_source_entries(empty, all, true, fe, me);
    }
    for (int32_t i = 0; i < n; i++) {
      const size_t len = masks[i].kind == PN_SOURCE_FORCE ? (size_t)s->mesh.n_cells : (size_t)s->mesh.n_nodes;
      std::vector<uint8_t> m(masks[i].inside, masks[i].inside + len);
      if (len == 0) m.push_back(0);  // keep the entry non-empty: marks a mask source
      s->src.push_back(all[s->src.size()]);
      s->src_t.emplace_back();
      s->src_v.emplace_back();
      s->series.emplace_back();
      s->src_mask.push_back(std::move(m));
      s->has_moments = s->has_moments || masks[i].kind == PN_SOURCE_MOMENT;
    }
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
    pn::ck(cudaStreamSynchronize(s->stream), "sensors sync");
    s->release(s->d_stile); s->release(s->d_snode); s->release(s->d_sidx);
    s->release(s->d_srng); s->release(s->d_skey); s->release(s->d_traces);
    s->n_sens = 0;
    s->rec_cap = 0;
    s->rec_count = 0;
    if (n == 0) return PN_OK;
    std::vector<std::pair<int32_t, int32_t>> pr((size_t)n);
    for (int32_t i = 0; i < n; i++) pr[i] = {nodes[i], i};
    std::sort(pr.begin(), pr.end());
    if (s->form == PN_FORM_GRID) pn::grid_sensors(s, pr);
    else pn::table_sensors(s, pr);
    s->d_traces = s->alloc<double>((size_t)std::max(capacity_steps, 1) * n * 3 * 8);
    pn::ck(cudaStreamSynchronize(s->stream), "sensors upload");
    s->n_sens = n;
    s->rec_cap = capacity_steps;
    return PN_OK;
  });
}

}  // extern "C"

namespace pn {
int set_last_error(int code, const std::string &msg) { return set_err(code, msg); }

int device_check(pn_solver *s) {
  if (!s->d_err) return PN_OK;
  int32_t v = 0;
  ck(cudaMemcpy(&v, s->d_err, sizeof(v), cudaMemcpyDeviceToHost), "error word");
  if (v == 0) return PN_OK;
  ck(cudaMemset(s->d_err, 0, sizeof(v)), "error word");
  return set_err(PN_ERR_DEVICE_CHECK,
                 "grid step: a wait for staged tiles gave up after 1 s; the state of this solver is invalid");
}

void refresh_sources(pn_solver *s) {
  if (!s->src_dirty) return;
  if (s->form == PN_FORM_GRID) grid_sources(s);
  else table_sources(s);
  s->src_dirty = false;
  s->sig_valid = false;
}
}  // namespace pn

namespace {
using pn::refresh_sources;

void run_any(pn_solver *s, int32_t nsteps) {
  if (s->form == PN_FORM_GRID) pn::grid_run(s, nsteps);
  else pn::table_run(s, nsteps);
}
}  // namespace

extern "C" {

int pn_solver_solve(pn_solver *s, int32_t nsteps, double *time_out) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (nsteps < 0) return set_err(PN_ERR_INVALID, "negative step count");
    if (s->has_mask_sources())
      return set_err(PN_ERR_INVALID, "window-mask sources need pn_solver_solve_signals");
    refresh_sources(s);
    run_any(s, nsteps);
    if (time_out) *time_out = s->time;
    return PN_OK;
  });
}

int pn_solver_solve_signals(pn_solver *s, int32_t nsteps, const double *values, double *time_out) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (nsteps < 0) return set_err(PN_ERR_INVALID, "negative step count");
    const int64_t nsig = (int64_t)s->src.size();
    if (nsig > 0 && nsteps > 0 && !values) return set_err(PN_ERR_INVALID, "null signal values");
    if (nsig > 0 && !pn::all_finite(values, (int64_t)nsteps * nsig))
      return set_err(PN_ERR_NOT_FINITE, "non-finite signal value");
    refresh_sources(s);
    if (nsig > 0 && nsteps > 0) {
      pn::ck(cudaStreamSynchronize(s->stream), "signal sync");
      if (nsteps > s->sig_alloc_rows) {
        s->release(s->d_sig);
        s->d_sig = s->alloc<void>((size_t)nsteps * nsig * s->esz);
        s->sig_alloc_rows = nsteps;
      }
      s->upload_real(s->d_sig, values, (size_t)nsteps * nsig);
      pn::ck(cudaStreamSynchronize(s->stream), "signal upload");
      s->sig_step0 = s->step;
      s->sig_rows = nsteps;
      s->sig_hold = false;
      s->sig_valid = true;
    }
    s->caller_signals = true;
    try {
      run_any(s, nsteps);
    } catch (...) {
      s->caller_signals = false;
      s->sig_valid = false;
      throw;
    }
    s->caller_signals = false;
    s->sig_valid = false;  // the next plain solve evaluates the sources' own signals
    if (time_out) *time_out = s->time;
    return PN_OK;
  });
}

int pn_solver_get_state(pn_solver *s, double *const *V, double *const *S) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    pn::ck(cudaStreamSynchronize(s->stream), "get_state sync");
    if (const int rc = pn::device_check(s)) return rc;
    if (s->form == PN_FORM_GRID) pn::grid_get_state(s, V, S);
    else pn::table_get_state(s, V, S);
    return PN_OK;
  });
}

int pn_solver_get_traces(pn_solver *s, double *out, int64_t max_records, int64_t *n_records) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    if (max_records < 0 || (max_records > 0 && !out)) return set_err(PN_ERR_INVALID, "trace buffer");
    pn::ck(cudaStreamSynchronize(s->stream), "get_traces sync");
    if (const int rc = pn::device_check(s)) return rc;
    const int64_t have = std::min(s->rec_count, s->rec_cap);
    const int64_t n = std::min(have, max_records);
    if (n > 0 && s->n_sens > 0)
      pn::ck(cudaMemcpy(out, s->d_traces, (size_t)n * s->n_sens * 3 * 8, cudaMemcpyDeviceToHost), "traces");
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
  info->algorithmic_bytes_per_step = pn::step_bytes(s);
  info->device_bytes = s->dev_bytes;
  info->dt = s->dt;
  info->time = s->time;
  info->form = s->form;
  if (s->form == PN_FORM_GRID) {
    info->grid[0] = s->grid.nx;
    info->grid[1] = s->grid.ny;
    info->grid[2] = s->grid.nz;
    info->grid_kernel = !s->d_tmaps ? 1 : (s->d_rflags && pn::grid_tma_f64_launches() == 2) ? 3 : 2;
  }
  return PN_OK;
}

int pn_solver_device_state(pn_solver *s, void **V, void **S) {
  return guarded([&]() -> int {
    if (!s || !V || !S) return set_err(PN_ERR_INVALID, "null argument");
    for (int k = 0; k < 3; k++) V[k] = s->V[s->cur][k];
    for (int k = 0; k < 6; k++) S[k] = s->S[s->cur][k];
    if (s->form == PN_FORM_GRID) pn::grid_reset_range_flags(s);  // the caller may write through them
    return PN_OK;
  });
}

int pn_solver_energy(pn_solver *s, double *kinetic, double *strain) {
  return guarded([&]() -> int {
    if (!s || !kinetic || !strain) return set_err(PN_ERR_INVALID, "null argument");
    pn::ck(cudaStreamSynchronize(s->stream), "energy sync");
    if (const int rc = pn::device_check(s)) return rc;
    pn::energy(s, *kinetic, *strain);
    return PN_OK;
  });
}

int pn_solver_path_counts(pn_solver *s, int64_t *fp64_blocks, int64_t *df64_blocks) {
  return guarded([&]() -> int {
    if (!s || !fp64_blocks || !df64_blocks) return set_err(PN_ERR_INVALID, "null argument");
    unsigned long long c[2] = {0ull, 0ull};
    if (s->d_pathcnt) {
      pn::ck(cudaMemcpyAsync(c, s->d_pathcnt, sizeof(c), cudaMemcpyDeviceToHost, s->stream), "path counts");
      pn::ck(cudaStreamSynchronize(s->stream), "path counts");
    }
    *fp64_blocks = (int64_t)c[0];
    *df64_blocks = (int64_t)c[1];
    return PN_OK;
  });
}

int pn_measure_pipe_rates(double *rates, int32_t n) {
  return guarded([&]() -> int {
    if (!rates || n < 0) return set_err(PN_ERR_INVALID, "null rates or negative count");
    pn::ck(pn::measure_pipe_rates(rates, n), "pipe-rate kernels");
    return PN_OK;
  });
}

int pn_solver_synchronize(pn_solver *s) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    pn::ck(cudaStreamSynchronize(s->stream), "synchronize");
    pn::ck(cudaGetLastError(), "device error");
    return pn::device_check(s);
  });
}

int pn_solver_enable_kernel_timing(pn_solver *s, int32_t enable) {
  return guarded([&]() -> int {
    if (!s) return set_err(PN_ERR_INVALID, "null solver");
    pn::ck(cudaStreamSynchronize(s->stream), "timing sync");
    s->clear_marks();
    s->timing = enable != 0;
    return PN_OK;
  });
}

int pn_solver_kernel_times(pn_solver *s, double *ms, int64_t *launches) {
  return guarded([&]() -> int {
    if (!s || !ms || !launches) return set_err(PN_ERR_INVALID, "null argument");
    pn::ck(cudaStreamSynchronize(s->stream), "timing sync");
    for (int k = 0; k < 3; k++) {
      ms[k] = 0.;
      launches[k] = 0;
    }
    for (auto &m : s->marks) {
      float t = 0.f;
      pn::ck(cudaEventElapsedTime(&t, m.a, m.b), "elapsed");
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
