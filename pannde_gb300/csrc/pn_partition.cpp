// pn_partition.cpp -- one mesh solved as several partitions on one device,
// with the reference's decomposition and its single exchange per step.
//
// The reference shards the path across MPI ranks (MetisHexPartitioner.hpp,
// HostUTModel.hpp:316-326, MPIHaloExchanger.hpp): every node has one home
// partition; a partition's local mesh is every cell touching one of its
// nodes plus those cells' nodes; a step updates the velocity of home nodes,
// exchanges velocity home -> halo copies, then updates the stress of every
// local cell (halo cells recomputed redundantly, no stress exchange).
// Here:
//   * nodes are split by recursive coordinate bisection (longest axis,
//     count-proportional median), standing in for METIS's node partition;
//   * each partition is an ordinary table-form solver over its local mesh
//     with node_owner / partition_id, so only home nodes are updated, exactly
//     as updateVsAtNode's ownership test (HostRSGTDUT.hpp:339);
//   * a step is the velocity half of every partition (one batch launch), a
//     device halo-exchange kernel (rsg_state.cu: each halo node copies its
//     home partition's new velocity), then the stress half of every
//     partition.  On several GPUs the exchange would be peer copies or NCCL
//     send/receive of the same lists.
// Arithmetic per node and cell is the single-partition arithmetic, so the
// result equals the single-partition solve bit for bit.
#include <algorithm>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>

#include "pn_solver.hpp"

struct pn_partitioned {
  int P = 0;
  int precision = PN_PREC_F64;
  double dt = 0.0;
  cudaStream_t stream = nullptr;
  int32_t g_nodes = 0, g_cells = 0;
  std::vector<pn_solver *> parts;
  std::vector<std::vector<int32_t>> gnode, gcell;  // local -> global, per part
  std::vector<int32_t> owner, owner_local;         // global node -> home part, index there
  std::vector<int32_t> cell_part, cell_local;      // global cell -> a part holding it, index there
  int64_t n_halo = 0;
  int4 *d_ex = nullptr;
  void **d_vptr = nullptr;
  void *d_args[2] = {nullptr, nullptr};
  int *d_start[2] = {nullptr, nullptr};
  // sensors: global sensor k is recorded by part sens_part[k] as its sens_slot[k]-th
  int32_t n_sens = 0;
  std::vector<int32_t> sens_part, sens_slot, sens_count;

  ~pn_partitioned() {
    for (void *p : {(void *)d_ex, (void *)d_vptr, d_args[0], d_args[1], (void *)d_start[0], (void *)d_start[1]})
      if (p) cudaFree(p);
    for (pn_solver *s : parts) pn_solver_destroy(s);
  }
};

namespace {

int perr(int code, const std::string &m) { return pn::set_last_error(code, m); }

template <typename F>
int pguard(F &&f) {
  pn::set_last_error(PN_OK, "");
  try {
    return f();
  } catch (const pn::SetupError &e) {
    return perr(e.code, e.msg);
  } catch (const pn::CudaError &e) {
    (void)cudaGetLastError();
    return perr(PN_ERR_CUDA, std::string(e.what) + ": " + cudaGetErrorString(e.e));
  } catch (const std::exception &e) {
    return perr(PN_ERR_RUNTIME, e.what());
  }
}

// recursive coordinate bisection of idx[lo, hi) into np parts from p0
void rcb(const pn::MeshTables &t, std::vector<int32_t> &idx, int64_t lo, int64_t hi, int p0, int np,
         std::vector<int32_t> &part) {
  if (np == 1 || hi - lo <= 1) {
    for (int64_t i = lo; i < hi; i++) part[(size_t)idx[(size_t)i]] = p0;
    return;
  }
  double mn[3] = {1e308, 1e308, 1e308}, mx[3] = {-1e308, -1e308, -1e308};
  const pn::hvec<double> *xyz[3] = {&t.x, &t.y, &t.z};
  for (int64_t i = lo; i < hi; i++)
    for (int d = 0; d < 3; d++) {
      const double v = (*xyz[d])[(size_t)idx[(size_t)i]];
      mn[d] = std::min(mn[d], v);
      mx[d] = std::max(mx[d], v);
    }
  int ax = 0;
  for (int d = 1; d < 3; d++)
    if (mx[d] - mn[d] > mx[ax] - mn[ax]) ax = d;
  const pn::hvec<double> &c = *xyz[ax];
  const int nl = np / 2;
  const int64_t cut = lo + (hi - lo) * nl / np;
  std::nth_element(idx.begin() + lo, idx.begin() + cut, idx.begin() + hi, [&](int32_t a, int32_t b) {
    return c[(size_t)a] < c[(size_t)b] || (c[(size_t)a] == c[(size_t)b] && a < b);
  });
  rcb(t, idx, lo, cut, p0, nl, part);
  rcb(t, idx, cut, hi, p0 + nl, np - nl, part);
}

// argument blocks of every part for one chunk, staged, with the tile prefixes
template <typename T>
void stage(pn_partitioned *q, pn::BatchLaunch &L) {
  const int n = q->P;
  std::vector<pn::VelArgs<T>> va((size_t)n);
  std::vector<pn::StressArgs<T>> sa((size_t)n);
  std::vector<int> vs((size_t)n + 1, 0), ss((size_t)n + 1, 0);
  for (int m = 0; m < n; m++) {
    pn_solver *s = q->parts[(size_t)m];
    pn::table_args<T>(s, va[(size_t)m], sa[(size_t)m]);
    const int64_t nsig = (int64_t)s->src.size();
    if (nsig > 0) {
      const int64_t row0 = pn::sig_row(s, 0);
      va[(size_t)m].sigval = (const T *)s->d_sig + row0 * nsig;
      va[(size_t)m].sig_stride = (int32_t)nsig;
      va[(size_t)m].sig_rows = (int32_t)(s->sig_rows - row0);
      sa[(size_t)m].sigval = va[(size_t)m].sigval;
      sa[(size_t)m].sig_stride = va[(size_t)m].sig_stride;
      sa[(size_t)m].sig_rows = va[(size_t)m].sig_rows;
    }
    va[(size_t)m].rec_base = s->rec_count;
    vs[(size_t)m + 1] = vs[(size_t)m] + (s->mesh.n_nodes + pn::kTile - 1) / pn::kTile;
    ss[(size_t)m + 1] = ss[(size_t)m] + (s->mesh.n_cells + pn::kTile - 1) / pn::kTile;
  }
  pn::ck(cudaMemcpyAsync(q->d_args[0], va.data(), sizeof(pn::VelArgs<T>) * n, cudaMemcpyHostToDevice, q->stream),
         "partition args");
  pn::ck(cudaMemcpyAsync(q->d_args[1], sa.data(), sizeof(pn::StressArgs<T>) * n, cudaMemcpyHostToDevice,
                         q->stream), "partition args");
  pn::ck(cudaMemcpyAsync(q->d_start[0], vs.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, q->stream),
         "partition tiles");
  pn::ck(cudaMemcpyAsync(q->d_start[1], ss.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, q->stream),
         "partition tiles");
  int dev = 0, sms = 1;
  pn::ck(cudaGetDevice(&dev), "device");
  pn::ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
  L.n_members = n;
  L.vel_args = q->d_args[0];
  L.str_args = q->d_args[1];
  L.vel_start = q->d_start[0];
  L.str_start = q->d_start[1];
  L.vel_tiles = vs[(size_t)n];
  L.str_tiles = ss[(size_t)n];
  L.blocks_vel = std::min(vs[(size_t)n], sms * 8);
  L.blocks_str = std::min(ss[(size_t)n], sms * 8);
  // the arguments are staged from host vectors that go out of scope
  pn::ck(cudaStreamSynchronize(q->stream), "partition staging");
}

template <typename T>
void solve_parts(pn_partitioned *q, int32_t nsteps) {
  int32_t done = 0;
  while (done < nsteps) {
    int32_t chunk = nsteps - done;
    for (pn_solver *s : q->parts) {
      pn::ensure_signal_rows(s, chunk);
      if (!s->src.empty() && !s->sig_hold)
        chunk = (int32_t)std::min<int64_t>(chunk, s->sig_step0 + s->sig_rows - s->step);
    }
    chunk = std::max<int32_t>(chunk, 1);
    pn::BatchLaunch L;
    stage<T>(q, L);
    for (int32_t k = 0; k < chunk; k++) {
      pn::ck(pn::launch_table_batch_halves(L, q->precision, k, 1, q->stream), "velocity half");
      pn::ck(pn::launch_halo_exchange(q->precision, q->d_ex, q->n_halo, q->d_vptr, q->stream), "halo exchange");
      pn::ck(pn::launch_table_batch_halves(L, q->precision, k, 2, q->stream), "stress half");
    }
    pn::ck(cudaStreamSynchronize(q->stream), "partition chunk");
    for (pn_solver *s : q->parts) {
      for (int32_t k = 0; k < chunk; k++) s->time += s->dt;  // HostRSGTDUT.hpp:166
      s->step += chunk;
      s->rec_count += chunk;
    }
    done += chunk;
  }
}

}  // namespace

extern "C" {

int pn_partitioned_create(const pn_mesh *mesh, const pn_material_table *materials, double dt, int32_t precision,
                          int32_t n_parts, pn_partitioned **out) {
  return pguard([&]() -> int {
    if (!out) return perr(PN_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!mesh || !materials) return perr(PN_ERR_INVALID, "null mesh or materials");
    if (precision != PN_PREC_F64 && precision != PN_PREC_F32 && precision != PN_PREC_DF64)
      return perr(PN_ERR_INVALID, "partitioned solves run the fast FP64, FP32 and double-float forms");
    if (n_parts < 1) return perr(PN_ERR_INVALID, "at least one partition");
    if (mesh->node_owner) return perr(PN_ERR_INVALID, "the partitioned solve assigns node owners itself");
    pn::MeshTables t;
    pn::build_mesh_tables(*mesh, t);  // validates like a single solver
    const int32_t nn = t.n_nodes, nc = t.n_cells;
    if (n_parts > std::max(nn, 1)) return perr(PN_ERR_INVALID, "more partitions than nodes");
    std::unique_ptr<pn_partitioned> q(new pn_partitioned());
    q->P = n_parts;
    q->precision = precision;
    q->dt = dt;
    q->g_nodes = nn;
    q->g_cells = nc;
    q->owner.assign((size_t)nn, 0);
    std::vector<int32_t> idx((size_t)nn);
    std::iota(idx.begin(), idx.end(), 0);
    rcb(t, idx, 0, nn, 0, n_parts, q->owner);
    q->owner_local.assign((size_t)nn, -1);
    q->cell_part.assign((size_t)nc, -1);
    q->cell_local.assign((size_t)nc, -1);
    q->gnode.resize((size_t)n_parts);
    q->gcell.resize((size_t)n_parts);
    std::vector<int32_t> lnode((size_t)nn, -1);
    for (int p = 0; p < n_parts; p++) {
      // local mesh: cells touching a home node, and those cells' nodes
      std::vector<uint8_t> cin((size_t)nc, 0), nin((size_t)nn, 0);
      for (int32_t n = 0; n < nn; n++)
        if (q->owner[(size_t)n] == p)
          for (int k = 0; k < 8; k++) {
            const int32_t c = t.ncc[(size_t)n * 8 + k];
            if (c >= 0) cin[(size_t)c] = 1;
          }
      std::vector<int32_t> &gc = q->gcell[(size_t)p];
      std::vector<int32_t> &gn = q->gnode[(size_t)p];
      for (int32_t c = 0; c < nc; c++)
        if (cin[(size_t)c]) {
          gc.push_back(c);
          for (int k = 0; k < 8; k++) nin[(size_t)t.hex[(size_t)c * 8 + k]] = 1;
        }
      for (int32_t n = 0; n < nn; n++)
        if (nin[(size_t)n] || q->owner[(size_t)n] == p) gn.push_back(n);  // a cell-less home node too
      for (size_t l = 0; l < gn.size(); l++) lnode[(size_t)gn[l]] = (int32_t)l;
      std::vector<double> x(gn.size()), y(gn.size()), z(gn.size());
      std::vector<int32_t> own(gn.size()), hex(gc.size() * 8), cm(gc.size());
      for (size_t l = 0; l < gn.size(); l++) {
        x[l] = t.x[(size_t)gn[l]];
        y[l] = t.y[(size_t)gn[l]];
        z[l] = t.z[(size_t)gn[l]];
        own[l] = q->owner[(size_t)gn[l]];
        if (own[l] == p) q->owner_local[(size_t)gn[l]] = (int32_t)l;
      }
      for (size_t l = 0; l < gc.size(); l++) {
        for (int k = 0; k < 8; k++) hex[l * 8 + k] = lnode[(size_t)t.hex[(size_t)gc[l] * 8 + k]];
        cm[l] = materials->cell_material[gc[l]];
        if (q->cell_part[(size_t)gc[l]] < 0) {
          q->cell_part[(size_t)gc[l]] = p;
          q->cell_local[(size_t)gc[l]] = (int32_t)l;
        }
      }
      pn_mesh lm{(int32_t)gn.size(), (int32_t)gc.size(), x.data(), y.data(), z.data(), hex.data(), own.data(), p};
      pn_material_table lt{materials->n_materials, materials->density, materials->cij, cm.data()};
      pn_solver *s = nullptr;
      const int rc = pn_solver_create_indexed(&lm, &lt, dt, precision | PN_FORM_TABLE, &s);
      if (rc != PN_OK) return rc;  // message already set
      q->parts.push_back(s);
      // one lattice spacing for every partition: a local mesh's own first cell
      // can round its corner difference differently from the global mesh's
      if (t.uniform && s->mesh.uniform) {
        s->mesh.hx = t.hx;
        s->mesh.hy = t.hy;
        s->mesh.hz = t.hz;
      }
      for (size_t l = 0; l < gn.size(); l++) lnode[(size_t)gn[l]] = -1;
    }
    // halo entries: every local copy of a node that is not home takes the home value
    std::vector<int4> ex;
    for (int p = 0; p < n_parts; p++) {
      const std::vector<int32_t> &gn = q->gnode[(size_t)p];
      for (size_t l = 0; l < gn.size(); l++) {
        const int32_t g = gn[l], home = q->owner[(size_t)g];
        if (home != p) ex.push_back(make_int4(p, (int)l, home, q->owner_local[(size_t)g]));
      }
    }
    q->n_halo = (int64_t)ex.size();
    pn::ck(cudaMalloc(&q->d_ex, std::max<size_t>(ex.size(), 1) * sizeof(int4)), "halo list");
    if (!ex.empty())
      pn::ck(cudaMemcpy(q->d_ex, ex.data(), ex.size() * sizeof(int4), cudaMemcpyHostToDevice), "halo list");
    std::vector<void *> vp((size_t)n_parts * 3);
    for (int p = 0; p < n_parts; p++)
      for (int c = 0; c < 3; c++) vp[(size_t)p * 3 + c] = q->parts[(size_t)p]->V[0][c];
    pn::ck(cudaMalloc((void **)&q->d_vptr, vp.size() * sizeof(void *)), "halo pointers");
    pn::ck(cudaMemcpy(q->d_vptr, vp.data(), vp.size() * sizeof(void *), cudaMemcpyHostToDevice), "halo pointers");
    const size_t abytes = std::max(sizeof(pn::VelArgs<double>), sizeof(pn::StressArgs<double>)) * n_parts;
    for (int k = 0; k < 2; k++) {
      pn::ck(cudaMalloc(&q->d_args[k], abytes), "partition args");
      pn::ck(cudaMalloc((void **)&q->d_start[k], sizeof(int) * (n_parts + 1)), "partition tiles");
    }
    *out = q.release();
    return PN_OK;
  });
}

int pn_partitioned_add_sources(pn_partitioned *q, const pn_window_source *src, int32_t n) {
  if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
  for (pn_solver *s : q->parts) {
    const int rc = pn_solver_add_sources(s, src, n);
    if (rc != PN_OK) return rc;
  }
  return PN_OK;
}

int pn_partitioned_set_sensors(pn_partitioned *q, const int32_t *nodes, int32_t n, int32_t capacity_steps) {
  return pguard([&]() -> int {
    if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
    if (n < 0 || (n > 0 && !nodes)) return perr(PN_ERR_INVALID, "sensor list");
    std::vector<std::vector<int32_t>> loc((size_t)q->P);
    q->sens_part.assign((size_t)n, 0);
    q->sens_slot.assign((size_t)n, 0);
    for (int32_t k = 0; k < n; k++) {
      const int32_t g = nodes[k];
      if (g < 0 || g >= q->g_nodes) return perr(PN_ERR_RANGE, "sensor node out of range");
      const int p = q->owner[(size_t)g];
      q->sens_part[(size_t)k] = p;
      q->sens_slot[(size_t)k] = (int32_t)loc[(size_t)p].size();
      loc[(size_t)p].push_back(q->owner_local[(size_t)g]);
    }
    q->sens_count.assign((size_t)q->P, 0);
    for (int p = 0; p < q->P; p++) {
      q->sens_count[(size_t)p] = (int32_t)loc[(size_t)p].size();
      const int rc = pn_solver_set_sensors(q->parts[(size_t)p], loc[(size_t)p].data(),
                                           (int32_t)loc[(size_t)p].size(), capacity_steps);
      if (rc != PN_OK) return rc;
    }
    q->n_sens = n;
    return PN_OK;
  });
}

int pn_partitioned_set_state(pn_partitioned *q, const double *const *V, const double *const *S) {
  return pguard([&]() -> int {
    if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
    for (int p = 0; p < q->P; p++) {
      const std::vector<int32_t> &gn = q->gnode[(size_t)p], &gc = q->gcell[(size_t)p];
      std::vector<std::vector<double>> lv(3), ls(6);
      const double *vp[3] = {nullptr, nullptr, nullptr}, *sp[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
      for (int c = 0; c < 3; c++)
        if (V && V[c]) {
          lv[c].resize(gn.size());
          for (size_t l = 0; l < gn.size(); l++) lv[c][l] = V[c][gn[l]];
          vp[c] = lv[c].data();
        }
      for (int c = 0; c < 6; c++)
        if (S && S[c]) {
          ls[c].resize(gc.size());
          for (size_t l = 0; l < gc.size(); l++) ls[c][l] = S[c][gc[l]];
          sp[c] = ls[c].data();
        }
      const int rc = pn_solver_set_state(q->parts[(size_t)p], vp, sp);
      if (rc != PN_OK) return rc;
    }
    return PN_OK;
  });
}

int pn_partitioned_solve(pn_partitioned *q, int32_t nsteps, double *time_out) {
  return pguard([&]() -> int {
    if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
    if (nsteps < 0) return perr(PN_ERR_INVALID, "negative step count");
    for (pn_solver *s : q->parts) {
      pn::ck(cudaStreamSynchronize(s->stream), "part sync");
      pn::refresh_sources(s);
    }
    if (nsteps > 0) {
      if (q->precision == PN_PREC_DF64) solve_parts<float2>(q, nsteps);
      else if (q->precision == PN_PREC_F32) solve_parts<float>(q, nsteps);
      else solve_parts<double>(q, nsteps);
    }
    if (time_out) *time_out = q->parts.front()->time;
    return PN_OK;
  });
}

int pn_partitioned_get_state(pn_partitioned *q, double *const *V, double *const *S) {
  return pguard([&]() -> int {
    if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
    std::vector<std::vector<double>> lv((size_t)q->P * 3), ls((size_t)q->P * 6);
    for (int p = 0; p < q->P; p++) {
      double *vp[3], *sp[6];
      for (int c = 0; c < 3; c++) {
        lv[(size_t)p * 3 + c].resize(q->gnode[(size_t)p].size());
        vp[c] = lv[(size_t)p * 3 + c].data();
      }
      for (int c = 0; c < 6; c++) {
        ls[(size_t)p * 6 + c].resize(q->gcell[(size_t)p].size());
        sp[c] = ls[(size_t)p * 6 + c].data();
      }
      const int rc = pn_solver_get_state(q->parts[(size_t)p], vp, sp);
      if (rc != PN_OK) return rc;
    }
    for (int c = 0; c < 3; c++)
      if (V && V[c])
        for (int32_t g = 0; g < q->g_nodes; g++)
          V[c][g] = lv[(size_t)q->owner[(size_t)g] * 3 + c][(size_t)q->owner_local[(size_t)g]];
    for (int c = 0; c < 6; c++)
      if (S && S[c])
        for (int32_t g = 0; g < q->g_cells; g++)
          S[c][g] = ls[(size_t)q->cell_part[(size_t)g] * 6 + c][(size_t)q->cell_local[(size_t)g]];
    return PN_OK;
  });
}

int pn_partitioned_get_traces(pn_partitioned *q, double *out, int64_t max_records, int64_t *n_records) {
  return pguard([&]() -> int {
    if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
    if (max_records < 0 || (max_records > 0 && !out)) return perr(PN_ERR_INVALID, "trace buffer");
    int64_t have = -1;
    std::vector<std::vector<double>> tr((size_t)q->P);
    for (int p = 0; p < q->P; p++) {
      if (q->sens_count.empty() || q->sens_count[(size_t)p] == 0) continue;  // records nothing
      int64_t n = 0;
      int rc = pn_solver_get_traces(q->parts[(size_t)p], nullptr, 0, &n);
      if (rc != PN_OK) return rc;
      have = have < 0 ? n : std::min(have, n);
    }
    if (have < 0) have = 0;
    const int64_t m = std::min(have, max_records);
    if (n_records) *n_records = have;
    if (m == 0) return PN_OK;
    for (int p = 0; p < q->P; p++) {
      const int32_t ns = q->sens_count.empty() ? 0 : q->sens_count[(size_t)p];
      if (ns == 0) continue;
      tr[(size_t)p].resize((size_t)m * ns * 3);
      int64_t n = 0;
      const int rc = pn_solver_get_traces(q->parts[(size_t)p], tr[(size_t)p].data(), m, &n);
      if (rc != PN_OK) return rc;
    }
    for (int64_t r = 0; r < m; r++)
      for (int32_t k = 0; k < q->n_sens; k++) {
        const int p = q->sens_part[(size_t)k];
        const int32_t ns = q->sens_count[(size_t)p], slot = q->sens_slot[(size_t)k];
        for (int c = 0; c < 3; c++)
          out[((size_t)r * q->n_sens + k) * 3 + c] = tr[(size_t)p][((size_t)r * ns + slot) * 3 + c];
      }
    return PN_OK;
  });
}

int pn_partitioned_info(pn_partitioned *q, int32_t *n_parts, int64_t *halo_nodes, int64_t *local_cells) {
  if (!q) return perr(PN_ERR_INVALID, "null partitioned solve");
  if (n_parts) *n_parts = q->P;
  if (halo_nodes) *halo_nodes = q->n_halo;
  if (local_cells) {
    int64_t t = 0;
    for (auto &g : q->gcell) t += (int64_t)g.size();
    *local_cells = t;
  }
  return PN_OK;
}

int pn_partitioned_destroy(pn_partitioned *q) {
  delete q;
  return PN_OK;
}

}  // extern "C"
