// pn_table.cpp -- table form of the solver: any hex mesh, connectivity tables
// on the device, two kernels per step (velocity then stress).
#include <cstring>
#include <type_traits>

#include "pn_solver.hpp"

namespace pn {

int64_t table_footprint(const MeshTables &m, const MaterialTables &mt, int precision) {
  const int64_t nn = m.n_nodes, nc = m.n_cells;
  const int64_t e = precision == PN_PREC_F32 ? 4 : 8;
  const bool per_elem = precision == PN_PREC_F64_EXACT || !m.uniform;
  int64_t need = nn * 3 * e + nc * 6 * e + nc * 32 + nn * 32 + nn * e + nc * 4 +
                 (int64_t)mt.n_mat * 36 * e;
  if (per_elem) need += nn * 3 * e + nc * 3 * e;
  return need;
}

void table_create(pn_solver *s) {
  const int32_t nn = s->mesh.n_nodes, nc = s->mesh.n_cells;
  const size_t e = s->esz;
  const bool exact = s->precision == PN_PREC_F64_EXACT;
  const bool per_elem = exact || !s->mesh.uniform;
  for (int k = 0; k < 3; k++) s->V[0][k] = s->alloc<void>((size_t)nn * e);
  for (int k = 0; k < 6; k++) s->S[0][k] = s->alloc<void>((size_t)nc * e);
  s->d_hex = s->alloc<int4>((size_t)nc * 32);
  s->d_ncc = s->alloc<int4>((size_t)nn * 32);
  s->d_coef = s->alloc<void>((size_t)nn * e);
  s->d_mat = s->alloc<int32_t>((size_t)nc * 4);
  s->d_ctab = s->alloc<void>((size_t)s->mat.n_mat * 36 * e);
  for (int k = 0; k < 3; k++) ck(cudaMemsetAsync(s->V[0][k], 0, (size_t)nn * e, s->stream), "memset");
  for (int k = 0; k < 6; k++) ck(cudaMemsetAsync(s->S[0][k], 0, (size_t)nc * e, s->stream), "memset");
  s->upload_raw(s->d_hex, s->mesh.hex.data(), (size_t)nc * 32);
  s->upload_raw(s->d_ncc, s->mesh.ncc.data(), (size_t)nn * 32);
  s->upload_real(s->d_coef, s->mat.coef.data(), nn);
  s->upload_raw(s->d_mat, s->mat.cell_mat.data(), (size_t)nc * 4);
  std::vector<double> ct(s->mat.c36);
  if (!exact)
    for (double &v : ct) v *= s->dt;  // fast forms fold dt into C
  s->upload_real(s->d_ctab, ct.data(), ct.size());
  if (per_elem) {
    hvec<double> g((size_t)nn * 3), h((size_t)nc * 3);
    const double *dn[3] = {s->mesh.dxn.data(), s->mesh.dyn.data(), s->mesh.dzn.data()};
    const double *dc[3] = {s->mesh.dxc.data(), s->mesh.dyc.data(), s->mesh.dzc.data()};
    for (int a = 0; a < 3; a++) {
#pragma omp parallel for schedule(static)
      for (int32_t n = 0; n < nn; n++) g[(size_t)a * nn + n] = exact ? dn[a][n] : 0.25 / dn[a][n];
#pragma omp parallel for schedule(static)
      for (int32_t c = 0; c < nc; c++) h[(size_t)a * nc + c] = exact ? dc[a][c] : 0.25 / dc[a][c];
    }
    s->d_gnode = s->alloc<void>(g.size() * e);
    s->d_gcell = s->alloc<void>(h.size() * e);
    s->upload_real(s->d_gnode, g.data(), g.size());
    s->upload_real(s->d_gcell, h.data(), h.size());
  }
  ck(cudaStreamSynchronize(s->stream), "create sync");
}

void table_put_state(pn_solver *s, const double *const *V, const double *const *S) {
  // FP64 storage takes the caller's array as is; FP32 and double-float
  // storage convert on the device (rsg_state.cu)
  const int32_t nn = s->mesh.n_nodes, nc = s->mesh.n_cells;
  const bool raw = s->esz == 8 && !s->is_df64();
  auto put = [&](void *dst, const double *src, int32_t n) {
    if (!src) ck(cudaMemsetAsync(dst, 0, (size_t)n * s->esz, s->stream), "memset");
    else if (raw) s->upload_raw(dst, src, (size_t)n * 8);
    else s->put_field(dst, src, (size_t)n, nullptr);
  };
  for (int k = 0; k < 3; k++) put(s->V[0][k], V ? V[k] : nullptr, nn);
  for (int k = 0; k < 6; k++) put(s->S[0][k], S ? S[k] : nullptr, nc);
}

void table_get_state(pn_solver *s, double *const *V, double *const *S) {
  const bool raw = s->esz == 8 && !s->is_df64();
  auto get = [&](double *dst, const void *src, int32_t n) {
    if (!dst || n == 0) return;
    if (raw) ck(cudaMemcpyAsync(dst, src, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream), "download");
    else s->get_field(dst, src, (size_t)n, nullptr);
  };
  for (int k = 0; k < 3; k++) get(V ? V[k] : nullptr, s->V[0][k], s->mesh.n_nodes);
  for (int k = 0; k < 6; k++) get(S ? S[k] : nullptr, s->S[0][k], s->mesh.n_cells);
  ck(cudaStreamSynchronize(s->stream), "get_state");
}

void table_sources(pn_solver *s) {
  const bool exact = s->precision == PN_PREC_F64_EXACT;
  std::vector<SourceEntry> fe, me;
  const std::vector<const uint8_t *> masks = s->mask_ptrs();
  build_source_entries(s->mesh, s->src, exact, fe, me, &masks);
  ck(cudaStreamSynchronize(s->stream), "sources sync");
  s->release(s->d_ftile); s->release(s->d_felem); s->release(s->d_fcode); s->release(s->d_fw);
  s->release(s->d_mtile); s->release(s->d_melem); s->release(s->d_mcode); s->release(s->d_mw);
  s->n_force = (int32_t)fe.size();
  s->n_moment = (int32_t)me.size();
  auto upload_list = [&](const std::vector<SourceEntry> &L, int32_t n_elem, int shift, bool fold_dt,
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
    tile_ranges(el, n_elem, kTile, rg);
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
}

void table_sensors(pn_solver *s, const std::vector<std::pair<int32_t, int32_t>> &pr) {
  const int32_t n = (int32_t)pr.size();
  std::vector<int32_t> nd(n), ix(n), rg;
  for (int32_t i = 0; i < n; i++) {
    nd[i] = pr[i].first;
    ix[i] = pr[i].second;
  }
  tile_ranges(nd, s->mesh.n_nodes, kTile, rg);
  s->d_stile = s->alloc<int2>(rg.size() * 4);
  s->d_snode = s->alloc<int32_t>((size_t)n * 4);
  s->d_sidx = s->alloc<int32_t>((size_t)n * 4);
  s->upload_raw(s->d_stile, rg.data(), rg.size() * 4);
  s->upload_raw(s->d_snode, nd.data(), nd.size() * 4);
  s->upload_raw(s->d_sidx, ix.data(), ix.size() * 4);
}

template <typename T>
void table_args(pn_solver *s, VelArgs<T> &va, StressArgs<T> &sa) {
  std::memset(&va, 0, sizeof(va));
  std::memset(&sa, 0, sizeof(sa));
  va.n_nodes = s->mesh.n_nodes;
  va.ncc = s->d_ncc;
  T *const *V = (T *const *)s->V[0];
  T *const *S = (T *const *)s->S[0];
  va.V0 = V[0]; va.V1 = V[1]; va.V2 = V[2];
  va.S0 = S[0]; va.S1 = S[1]; va.S2 = S[2]; va.S3 = S[3]; va.S4 = S[4]; va.S5 = S[5];
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
  va.sig_stride = 0;  // single launches point sigval at the step's row
  va.sig_rows = 1;
  if (s->n_sens > 0) {
    va.tile_sens = s->d_stile; va.sens_node = s->d_snode; va.sens_idx = s->d_sidx;
    va.traces = s->d_traces; va.n_sens = s->n_sens; va.rec_cap = s->rec_cap;
  }
  sa.n_cells = s->mesh.n_cells;
  sa.hex = s->d_hex;
  sa.V0 = V[0]; sa.V1 = V[1]; sa.V2 = V[2];
  sa.S0 = S[0]; sa.S1 = S[1]; sa.S2 = S[2]; sa.S3 = S[3]; sa.S4 = S[4]; sa.S5 = S[5];
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
  sa.sig_stride = 0;
  sa.sig_rows = 1;
  sa.has_moments = s->has_moments ? 1 : 0;
}
template void table_args<double>(pn_solver *, VelArgs<double> &, StressArgs<double> &);
template void table_args<float>(pn_solver *, VelArgs<float> &, StressArgs<float> &);
template void table_args<float2>(pn_solver *, VelArgs<float2> &, StressArgs<float2> &);

namespace {

template <typename T>
void run(pn_solver *s, int32_t nsteps) {
  VelArgs<T> va;
  StressArgs<T> sa;
  table_args<T>(s, va, sa);
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
        va.sigval = (const T *)s->d_sig + sig_row(s, k) * nsig;
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
        e1 = launch_velocity_df64(va, k, s->mesh.uniform, s->stream);
        between();
        e2 = launch_stress_df64(sa, k, s->mesh.uniform, s->stream);
      } else if constexpr (std::is_same<T, double>::value) {
        if (s->precision == PN_PREC_F64_EXACT) {
          e1 = launch_velocity_exact(va, k, s->stream);
          between();
          e2 = launch_stress_exact(sa, k, s->stream);
        } else {
          e1 = launch_velocity_f64(va, k, s->mesh.uniform, s->stream);
          between();
          e2 = launch_stress_f64(sa, k, s->mesh.uniform, s->stream);
        }
      } else {
        e1 = launch_velocity_f32(va, k, s->mesh.uniform, s->stream);
        between();
        e2 = launch_stress_f32(sa, k, s->mesh.uniform, s->stream);
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

}  // namespace

void table_run(pn_solver *s, int32_t nsteps) {
  if (s->is_df64()) run<float2>(s, nsteps);
  else if (s->esz == 8) run<double>(s, nsteps);
  else run<float>(s, nsteps);
}

}  // namespace pn
