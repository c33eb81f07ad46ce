// pn_setup.cpp -- host-side table construction (see pn_setup.hpp).
// Compiled with -ffp-contract=off: window predicates, cell centres and
// spacings must round as the reference's C++ does.
#include "pn_setup.hpp"

#include <omp.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <unordered_map>

namespace pn {

namespace {
[[noreturn]] void fail(int code, const std::string &msg) { throw SetupError{code, msg}; }

bool near_equal(double a, double b) { return std::fabs(a - b) <= 1e-12 * std::fabs(b); }

// *p = max(*p, v) / min(*p, v) when several threads update the same entry
inline void atomic_max(int32_t *p, int32_t v) {
  int32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
}
inline void atomic_min(int32_t *p, int32_t v) {
  int32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (cur > v && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
}

template <typename T>
void fill_par(hvec<T> &v, size_t n, T value) {
  v.resize(n);
  T *p = v.data();
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) p[i] = value;
}
}  // namespace

void pinv_sym6(const double *a, double *out) {
  double m[6][6], v[6][6];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      m[i][j] = 0.5 * (a[i * 6 + j] + a[j * 6 + i]);
      v[i][j] = i == j ? 1.0 : 0.0;
    }
  // cyclic Jacobi: rotate away each off-diagonal entry in turn until they vanish
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < 6; i++) {
      diag += m[i][i] * m[i][i];
      for (int j = i + 1; j < 6; j++) off += m[i][j] * m[i][j];
    }
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < 6; p++)
      for (int q = p + 1; q < 6; q++) {
        if (m[p][q] == 0.0) continue;
        const double theta = (m[q][q] - m[p][p]) / (2.0 * m[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 6; k++) {  // columns p, q
          const double mkp = m[k][p], mkq = m[k][q];
          m[k][p] = c * mkp - sn * mkq;
          m[k][q] = sn * mkp + c * mkq;
        }
        for (int k = 0; k < 6; k++) {  // rows p, q
          const double mpk = m[p][k], mqk = m[q][k];
          m[p][k] = c * mpk - sn * mqk;
          m[q][k] = sn * mpk + c * mqk;
        }
        for (int k = 0; k < 6; k++) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - sn * vkq;
          v[k][q] = sn * vkp + c * vkq;
        }
      }
  }
  double lmax = 0.0;
  for (int i = 0; i < 6; i++) lmax = std::max(lmax, std::fabs(m[i][i]));
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      double s = 0.0;
      for (int k = 0; k < 6; k++)
        if (std::fabs(m[k][k]) > 1e-12 * lmax) s += v[i][k] * v[j][k] / m[k][k];
      out[i * 6 + j] = s;
    }
}

bool all_finite(const double *p, int64_t n) {
  bool ok = true;
#pragma omp parallel for reduction(&& : ok) schedule(static)
  for (int64_t i = 0; i < n; i++) ok = ok && std::isfinite(p[i]);
  return ok;
}

void build_mesh_tables(const pn_mesh &m, MeshTables &t) {
  if (m.n_nodes < 0 || m.n_cells < 0) fail(PN_ERR_INVALID, "negative node or cell count");
  if (m.n_nodes > 0 && (!m.x || !m.y || !m.z)) fail(PN_ERR_INVALID, "null node coordinates");
  if (m.n_cells > 0 && !m.hexes) fail(PN_ERR_INVALID, "null cell connectivity");
  const int32_t nn = m.n_nodes, nc = m.n_cells;
  t.n_nodes = nn;
  t.n_cells = nc;
  // copies, checks and tables are filled by parallel loops over nodes / cells
  t.x.resize(nn);
  t.y.resize(nn);
  t.z.resize(nn);
  t.owned.resize(nn);
  bool finite = true;
#pragma omp parallel for reduction(&& : finite) schedule(static)
  for (int32_t n = 0; n < nn; n++) {
    t.x[n] = m.x[n];
    t.y[n] = m.y[n];
    t.z[n] = m.z[n];
    finite = finite && std::isfinite(m.x[n]) && std::isfinite(m.y[n]) && std::isfinite(m.z[n]);
    t.owned[n] = m.node_owner ? (m.node_owner[n] == m.partition_id) : 1;
  }
  if (!finite) fail(PN_ERR_NOT_FINITE, "non-finite node coordinate");
  // HexMesh::setCell throws std::out_of_range for an invalid node id (the
  // first one in cell order is reported)
  {
    const int64_t nh = (int64_t)nc * 8;
    t.hex.resize((size_t)nh);
    int64_t bad = nh;
#pragma omp parallel for reduction(min : bad) schedule(static)
    for (int64_t k = 0; k < nh; k++) {
      const int32_t q = m.hexes[k];
      t.hex[(size_t)k] = q;
      if (q < 0 || q >= nn) bad = std::min(bad, k);
    }
    if (bad < nh)
      fail(PN_ERR_RANGE, "invalid node id: Node count: " + std::to_string(nn) +
                             ", provided index: " + std::to_string(t.hex[(size_t)bad]));
  }

  // buildLinks: corner k of cell c -> slot k^6 of that node; later cells win,
  // i.e. every slot holds the highest cell index that names it
  fill_par(t.ncc, (size_t)nn * 8, int32_t(-1));
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < nc; c++)
    for (int k = 0; k < 8; k++) atomic_max(&t.ncc[(size_t)t.hex[(size_t)c * 8 + k] * 8 + (k ^ 6)], c);

  // nodePrep (RightHex.hpp:272-309): per axis, the extent of every corner of
  // every incident cell around the node.  Min / max are exact, so taking them
  // per cell first (the cell's corner box) and then over the node's cells
  // gives the same numbers with 8 reads per node instead of 64.  Nodes are
  // independent; the first node (in order) with a non-positive spacing
  // decides the error, as in the reference's loop.
  hvec<double> box((size_t)nc * 6);
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < nc; c++) {
    double lo[3] = {1e308, 1e308, 1e308}, hi[3] = {-1e308, -1e308, -1e308};
    for (int kbb = 0; kbb < 8; kbb++) {
      const int32_t q = t.hex[(size_t)c * 8 + kbb];
      const double pt[3] = {t.x[q], t.y[q], t.z[q]};
      for (int kd = 0; kd < 3; kd++) {
        lo[kd] = std::min(lo[kd], pt[kd]);
        hi[kd] = std::max(hi[kd], pt[kd]);
      }
    }
    for (int kd = 0; kd < 3; kd++) {
      box[(size_t)c * 6 + kd] = lo[kd];
      box[(size_t)c * 6 + 3 + kd] = hi[kd];
    }
  }
  t.dxn.resize(nn);
  t.dyn.resize(nn);
  t.dzn.resize(nn);
  int64_t bad_node = nn;
#pragma omp parallel for reduction(min : bad_node) schedule(static)
  for (int32_t n = 0; n < nn; n++) {
    const double node[3] = {t.x[n], t.y[n], t.z[n]};
    double lo[3] = {node[0], node[1], node[2]};
    double hi[3] = {node[0], node[1], node[2]};
    for (int kb = 0; kb < 8; kb++) {
      const int32_t c = t.ncc[(size_t)n * 8 + kb];
      if (c == -1) continue;
      for (int kd = 0; kd < 3; kd++) {
        lo[kd] = std::min(lo[kd], box[(size_t)c * 6 + kd]);
        hi[kd] = std::max(hi[kd], box[(size_t)c * 6 + 3 + kd]);
      }
    }
    for (int kd = 0; kd < 3; kd++) {
      if (lo[kd] == node[kd]) lo[kd] = 2. * node[kd] - hi[kd];
      if (hi[kd] == node[kd]) hi[kd] = 2. * node[kd] - lo[kd];
    }
    t.dxn[n] = 0.5 * (hi[0] - lo[0]);
    t.dyn[n] = 0.5 * (hi[1] - lo[1]);
    t.dzn[n] = 0.5 * (hi[2] - lo[2]);
    if (0 >= t.dxn[n] || 0 >= t.dyn[n] || 0 >= t.dzn[n]) bad_node = std::min<int64_t>(bad_node, n);
  }
  if (bad_node < nn) {
    const size_t n = (size_t)bad_node;
    fail(PN_ERR_SPACING, 0 >= t.dxn[n] ? "DX" : 0 >= t.dyn[n] ? "DY" : "DZ");
  }
  // cellPrep (RightHex.hpp:253-264)
  t.dxc.resize(nc);
  t.dyc.resize(nc);
  t.dzc.resize(nc);
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < nc; c++) {
    const int32_t a = t.hex[(size_t)c * 8], b = t.hex[(size_t)c * 8 + 6];
    t.dxc[c] = t.x[b] - t.x[a];
    t.dyc[c] = t.y[b] - t.y[a];
    t.dzc[c] = t.z[b] - t.z[a];
  }
  // one (hx,hy,hz) within 1e-12 relative for every cell and node?
  t.uniform = nc > 0;
  if (t.uniform) {
    t.hx = t.dxc[0];
    t.hy = t.dyc[0];
    t.hz = t.dzc[0];
    bool u = true;
#pragma omp parallel for reduction(&& : u) schedule(static)
    for (int32_t c = 0; c < nc; c++)
      u = u && near_equal(t.dxc[c], t.hx) && near_equal(t.dyc[c], t.hy) && near_equal(t.dzc[c], t.hz);
#pragma omp parallel for reduction(&& : u) schedule(static)
    for (int32_t n = 0; n < nn; n++)
      u = u && near_equal(t.dxn[n], t.hx) && near_equal(t.dyn[n], t.hy) && near_equal(t.dzn[n], t.hz);
    t.uniform = u;
  }
}

namespace {

void check_field(const pn_field &f, const MeshTables &t, const char *what) {
  if (f.type < PN_FIELD_NODE || f.type > PN_FIELD_CONSTANT)
    fail(PN_ERR_INVALID, std::string("unknown field type for ") + what);
  if (!f.data) fail(PN_ERR_INVALID, std::string("null data for ") + what);
  const int64_t n = f.type == PN_FIELD_NODE ? t.n_nodes : f.type == PN_FIELD_CELL ? t.n_cells : 1;
  if (!all_finite(f.data, n)) fail(PN_ERR_NOT_FINITE, std::string("non-finite value in ") + what);
}

// HostField::atCell (HostField.hpp:121-133)
double at_cell(const pn_field &f, const MeshTables &t, int32_t c) {
  if (f.type == PN_FIELD_NODE) {
    double v = 0.0;
    for (int k = 0; k < 8; k++) v += f.data[t.hex[(size_t)c * 8 + k]];
    return v / 8.0;
  }
  return f.type == PN_FIELD_CONSTANT ? f.data[0] : f.data[c];
}

// HostField::atNode (HostField.hpp:142-153): a CELL or CONSTANT field sums the
// existing incident cells and divides by 8 (the lumped nodal density)
double at_node(const pn_field &f, const MeshTables &t, int32_t n) {
  if (f.type == PN_FIELD_NODE) return f.data[n];
  double v = 0.0;
  for (int k = 0; k < 8; k++) {
    const int32_t c = t.ncc[(size_t)n * 8 + k];
    v += (c == -1) ? 0. : (f.type == PN_FIELD_CONSTANT ? f.data[0] : f.data[c]);
  }
  return v / 8.0;
}

using Row = std::array<uint64_t, 21>;  // bit patterns of a cell's 21 stiffness values

struct RowHash {
  size_t operator()(const Row &r) const {
    uint64_t h = 1469598103934665603ull;
    for (uint64_t w : r) { h ^= w; h *= 1099511628211ull; }
    return (size_t)h;
  }
};

void expand36(const double *c21, double *c36) {
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) c36[i * 6 + j] = c21[cij_index(i, j)];
}

}  // namespace

void build_material_from_fields(const pn_material &mat, const MeshTables &t, double dt,
                                MaterialTables &out) {
  check_field(mat.density, t, "density");
  for (int k = 0; k < 21; k++) check_field(mat.cij[k], t, "stiffness");
  out.coef.resize(t.n_nodes);
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < t.n_nodes; n++)
    out.coef[n] = t.owned[n] ? dt / at_node(mat.density, t, n) : 0.;
  // De-duplicate the per-cell stiffness rows (bit patterns) into a table,
  // numbered in order of first appearance.  Each thread numbers the rows of
  // its contiguous run of cells in their order of first appearance there;
  // merging the runs in cell order then numbers every row as one pass over
  // all cells would.
  const int32_t nc = t.n_cells;
  out.cell_mat.resize(nc);
  std::vector<std::vector<Row>> seen((size_t)omp_get_max_threads());  // [run] rows, first appearance order
  int team = 1;  // runs = threads the region actually got
  bool out_of_memory = false;
#pragma omp parallel num_threads((int)seen.size()) reduction(|| : out_of_memory)
  try {
    const int nt = omp_get_num_threads(), r = omp_get_thread_num();
    if (r == 0) team = nt;
    const int32_t c0 = (int32_t)((int64_t)nc * r / nt), c1 = (int32_t)((int64_t)nc * (r + 1) / nt);
    std::unordered_map<Row, int32_t, RowHash> ids;
    std::vector<Row> &rows = seen[(size_t)r];
    Row key{}, last{};
    int32_t last_id = -1;
    for (int32_t c = c0; c < c1; c++) {
      for (int k = 0; k < 21; k++) {
        const double v = at_cell(mat.cij[k], t, c);
        std::memcpy(&key[k], &v, 8);
      }
      if (last_id < 0 || key != last) {  // neighbouring cells mostly share a row
        auto it = ids.find(key);
        if (it == ids.end()) {
          last_id = (int32_t)rows.size();
          ids.emplace(key, last_id);
          rows.push_back(key);
        } else {
          last_id = it->second;
        }
        last = key;
      }
      out.cell_mat[c] = last_id;  // numbered within the run for now
    }
  } catch (const std::bad_alloc &) {  // no exception may leave a parallel region
    out_of_memory = true;
  }
  if (out_of_memory) throw std::bad_alloc();
  seen.resize((size_t)team);
  std::unordered_map<Row, int32_t, RowHash> ids;
  std::vector<std::vector<int32_t>> remap(seen.size());
  out.c36.clear();
  for (size_t r = 0; r < seen.size(); r++)
    for (const Row &key : seen[r]) {
      auto it = ids.find(key);
      int32_t id;
      if (it == ids.end()) {
        id = (int32_t)ids.size();
        ids.emplace(key, id);
        double row[21];
        std::memcpy(row, key.data(), sizeof(row));
        out.c36.resize(out.c36.size() + 36);
        expand36(row, &out.c36[(size_t)id * 36]);
      } else {
        id = it->second;
      }
      remap[r].push_back(id);
    }
  const int nt = (int)seen.size();
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nt; r++) {
    const int32_t c0 = (int32_t)((int64_t)nc * r / nt), c1 = (int32_t)((int64_t)nc * (r + 1) / nt);
    for (int32_t c = c0; c < c1; c++) out.cell_mat[c] = remap[(size_t)r][(size_t)out.cell_mat[c]];
  }
  out.n_mat = (int32_t)ids.size();
}

void build_material_from_table(const pn_material_table &mat, const MeshTables &t, double dt,
                               MaterialTables &out) {
  if (mat.n_materials <= 0 || !mat.density || !mat.cij || (t.n_cells > 0 && !mat.cell_material))
    fail(PN_ERR_INVALID, "material table");
  if (!all_finite(mat.density, mat.n_materials) || !all_finite(mat.cij, (int64_t)mat.n_materials * 21))
    fail(PN_ERR_NOT_FINITE, "non-finite value in material table");
  out.cell_mat.resize(t.n_cells);
  bool in_range = true;
#pragma omp parallel for reduction(&& : in_range) schedule(static)
  for (int32_t c = 0; c < t.n_cells; c++) {
    const int32_t id = mat.cell_material[c];
    out.cell_mat[c] = id;
    in_range = in_range && id >= 0 && id < mat.n_materials;
  }
  if (!in_range) fail(PN_ERR_RANGE, "cell material id out of range");
  out.n_mat = mat.n_materials;
  out.c36.resize((size_t)out.n_mat * 36);
  for (int32_t i = 0; i < out.n_mat; i++) expand36(mat.cij + (size_t)i * 21, &out.c36[(size_t)i * 36]);
  out.coef.resize(t.n_nodes);
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < t.n_nodes; n++) {
    double v = 0.0;
    for (int k = 0; k < 8; k++) {
      const int32_t c = t.ncc[(size_t)n * 8 + k];
      v += (c == -1) ? 0. : mat.density[mat.cell_material[c]];
    }
    out.coef[n] = t.owned[n] ? dt / (v / 8.0) : 0.;
  }
}

void Series::build(const pn_signal &s) {
  if (s.n <= 0 || !s.t || !s.v) fail(PN_ERR_RUNTIME, "empty or null signal arrays");
  if (!all_finite(s.t, s.n) || !all_finite(s.v, s.n)) fail(PN_ERR_NOT_FINITE, "non-finite signal sample");
  std::map<double, double> m;  // std::map::emplace keeps the first value per time
  for (int32_t k = 0; k < s.n; k++) m.emplace(s.t[k], s.v[k]);
  t.clear();
  v.clear();
  for (auto &kv : m) { t.push_back(kv.first); v.push_back(kv.second); }
}

double Series::eval(double time) const {
  if (time < t.back()) {
    // first sample with time < t[k]; before the first sample the reference
    // steps before begin() (undefined), here the first value is held
    const size_t k = std::upper_bound(t.begin(), t.end(), time) - t.begin();
    if (k == 0) return v[0];
    const double Dt = t[k] - t[k - 1];
    const double Dv = v[k] - v[k - 1];
    return (Dv / Dt) * (time - t[k - 1]) + v[k - 1];
  }
  return v.back();
}

namespace {

bool window_at(const pn_window_source &w, const double p[3]) {
  double res = 0.0;
  for (int k = 0; k < 3; k++) {
    const double d = p[k] - w.center[k];
    res += d * d;
  }
  const double dist = std::sqrt(res);
  const double distz = std::fabs(p[2] - w.center[2]);
  return (distz <= 0.75 * w.ds) && (dist < w.radius) && (dist >= 0.);
}

// xducers[g][3] / moment_excitation[g][6]: slot -> source index or -1
std::vector<int32_t> group_slots(const std::vector<pn_window_source> &src, int kind, int ncomp,
                                 int32_t &ngroups) {
  int32_t maxg = -1;
  for (auto &s : src) {
    if (s.kind != kind) continue;
    if (s.group < 0) fail(PN_ERR_INVALID, "negative source group");
    if (s.component < 0 || s.component >= ncomp) fail(PN_ERR_INVALID, "source component out of range");
    maxg = std::max(maxg, s.group);
  }
  ngroups = maxg + 1;
  std::vector<int32_t> slot((size_t)std::max(ngroups, 0) * ncomp, -1);
  for (size_t i = 0; i < src.size(); i++) {
    if (src[i].kind != kind) continue;
    int32_t &s = slot[(size_t)src[i].group * ncomp + src[i].component];
    if (s != -1) fail(PN_ERR_INVALID, "two sources in one group slot");
    s = (int32_t)i;
  }
  return slot;
}

void push_entry(std::vector<SourceEntry> &out, bool exact, int32_t elem, int32_t comp, int32_t sig) {
  if (!exact) {
    // merge with an earlier entry of the same element, component and source
    for (size_t i = out.size(); i-- > 0;) {
      if (out[i].elem != elem) break;
      if (out[i].comp == comp && out[i].sig == sig) { out[i].w += 0.125; return; }
    }
  }
  out.push_back(SourceEntry{elem, comp, sig, 0.125});
}

// Runs body(e, list) for the elements e in [0, n) in contiguous runs on the
// threads, each run appending to a list of its own, and concatenates the lists
// in run order: the entries come out in element order, as from one serial
// loop (push_entry only merges entries of the same element, which never
// straddle two runs).
template <typename F>
void entries_by_runs(int32_t n, std::vector<SourceEntry> &out, F body) {
  const int runs = std::max(1, std::min(omp_get_max_threads() * 4, n / 4096 + 1));
  std::vector<std::vector<SourceEntry>> part((size_t)runs);
  bool out_of_memory = false;
#pragma omp parallel for schedule(dynamic, 1) reduction(|| : out_of_memory)
  for (int r = 0; r < runs; r++) {
    const int32_t e0 = (int32_t)((int64_t)n * r / runs), e1 = (int32_t)((int64_t)n * (r + 1) / runs);
    try {
      for (int32_t e = e0; e < e1; e++) body(e, part[(size_t)r]);
    } catch (const std::bad_alloc &) {  // no exception may leave a parallel region
      out_of_memory = true;
    }
  }
  if (out_of_memory) throw std::bad_alloc();
  size_t total = out.size();
  for (auto &p : part) total += p.size();
  out.reserve(total);
  for (auto &p : part) out.insert(out.end(), p.begin(), p.end());
}

}  // namespace

void build_source_entries(const MeshTables &t, const std::vector<pn_window_source> &src, bool exact,
                          std::vector<SourceEntry> &force, std::vector<SourceEntry> &moment,
                          const std::vector<const uint8_t *> *masks) {
  force.clear();
  moment.clear();
  auto mask_of = [&](size_t i) -> const uint8_t * { return masks ? (*masks)[i] : nullptr; };
  for (size_t i = 0; i < src.size(); i++) {
    const pn_window_source &s = src[i];
    if (s.kind != PN_SOURCE_FORCE && s.kind != PN_SOURCE_MOMENT) fail(PN_ERR_INVALID, "unknown source kind");
    if (mask_of(i)) continue;
    const double g[5] = {s.center[0], s.center[1], s.center[2], s.radius, s.ds};
    if (!all_finite(g, 5)) fail(PN_ERR_NOT_FINITE, "non-finite source geometry");
  }
  int32_t ngf = 0, ngm = 0;
  const std::vector<int32_t> fslot = group_slots(src, PN_SOURCE_FORCE, 3, ngf);
  const std::vector<int32_t> mslot = group_slots(src, PN_SOURCE_MOMENT, 6, ngm);

  if (ngf > 0) {
    // cell centres, HostRSGTDUT::cellcenter order (corner order, += 0.125*pt)
    hvec<double> cc((size_t)t.n_cells * 3);
#pragma omp parallel for schedule(static)
    for (int32_t c = 0; c < t.n_cells; c++) {
      double p[3] = {0., 0., 0.};
      for (int kb = 0; kb < 8; kb++) {
        const int32_t q = t.hex[(size_t)c * 8 + kb];
        p[0] += 0.125 * t.x[q];
        p[1] += 0.125 * t.y[q];
        p[2] += 0.125 * t.z[q];
      }
      cc[(size_t)c * 3] = p[0];
      cc[(size_t)c * 3 + 1] = p[1];
      cc[(size_t)c * 3 + 2] = p[2];
    }
    // in-window flag per (cell, force source) -- evaluated once per cell
    std::vector<int32_t> fsrc, flocal(src.size(), -1);
    for (size_t i = 0; i < src.size(); i++)
      if (src[i].kind == PN_SOURCE_FORCE) {
        flocal[i] = (int32_t)fsrc.size();
        fsrc.push_back((int32_t)i);
      }
    const size_t nf = fsrc.size();
    hvec<uint8_t> hit((size_t)t.n_cells * nf);
    hvec<uint8_t> any_cell(t.n_cells);
#pragma omp parallel for schedule(static)
    for (int32_t c = 0; c < t.n_cells; c++) {
      uint8_t any = 0;
      for (size_t l = 0; l < nf; l++) {
        const int32_t i = fsrc[l];
        const uint8_t *mk = mask_of(i);
        const uint8_t in = (mk ? mk[c] != 0 : window_at(src[i], &cc[(size_t)c * 3])) ? 1 : 0;
        hit[(size_t)c * nf + l] = in;
        any |= in;
      }
      any_cell[c] = any;
    }
    // evalXds loop order per node: dir, then slot kb, then transducer g
    entries_by_runs(t.n_nodes, force, [&](int32_t n, std::vector<SourceEntry> &list) {
      if (!t.owned[n]) return;
      bool any = false;
      for (int kb = 0; kb < 8 && !any; kb++) {
        const int32_t c = t.ncc[(size_t)n * 8 + kb];
        any = (c != -1) && any_cell[c];
      }
      if (!any) return;
      for (int dir = 0; dir < 3; dir++)
        for (int kb = 0; kb < 8; kb++) {
          const int32_t c = t.ncc[(size_t)n * 8 + kb];
          if (c == -1 || !any_cell[c]) continue;
          for (int32_t gi = 0; gi < ngf; gi++) {
            const int32_t si = fslot[(size_t)gi * 3 + dir];
            if (si >= 0 && hit[(size_t)c * nf + flocal[si]]) push_entry(list, exact, n, dir, si);
          }
        }
    });
  }
  if (ngm > 0) {
    std::vector<int32_t> msrc, mlocal(src.size(), -1);
    for (size_t i = 0; i < src.size(); i++)
      if (src[i].kind == PN_SOURCE_MOMENT) {
        mlocal[i] = (int32_t)msrc.size();
        msrc.push_back((int32_t)i);
      }
    const size_t nm = msrc.size();
    hvec<uint8_t> hit((size_t)t.n_nodes * nm);
    hvec<uint8_t> any_node(t.n_nodes);
#pragma omp parallel for schedule(static)
    for (int32_t n = 0; n < t.n_nodes; n++) {
      const double r[3] = {t.x[n], t.y[n], t.z[n]};
      uint8_t any = 0;
      for (size_t l = 0; l < nm; l++) {
        const int32_t i = msrc[l];
        const uint8_t *mk = mask_of(i);
        const uint8_t in = (mk ? mk[n] != 0 : window_at(src[i], r)) ? 1 : 0;
        hit[(size_t)n * nm + l] = in;
        any |= in;
      }
      any_node[n] = any;
    }
    // evalMoments loop order per cell: component, then corner kb, then tensor g
    entries_by_runs(t.n_cells, moment, [&](int32_t c, std::vector<SourceEntry> &list) {
      bool any = false;
      for (int kb = 0; kb < 8 && !any; kb++) any = any_node[t.hex[(size_t)c * 8 + kb]];
      if (!any) return;
      for (int comp = 0; comp < 6; comp++)
        for (int kb = 0; kb < 8; kb++) {
          const int32_t q = t.hex[(size_t)c * 8 + kb];
          if (!any_node[q]) continue;
          for (int32_t gi = 0; gi < ngm; gi++) {
            const int32_t si = mslot[(size_t)gi * 6 + comp];
            if (si >= 0 && hit[(size_t)q * nm + mlocal[si]]) push_entry(list, exact, c, comp, si);
          }
        }
    });
  }
  if ((int64_t)force.size() > kMaxSourceEntries || (int64_t)moment.size() > kMaxSourceEntries)
    fail(PN_ERR_INVALID, "too many source entries (" + std::to_string(force.size()) + " force, " +
                             std::to_string(moment.size()) + " moment; at most " +
                             std::to_string(kMaxSourceEntries) + " each)");
}

void detect_grid(const MeshTables &t, GridMap &g, double max_void_fraction) {
  g = GridMap();
  if (!t.uniform || t.n_cells == 0) {
    g.why = t.n_cells == 0 ? "no cells" : "spacing not uniform";
    return;
  }
  double x0 = t.x[0], y0 = t.y[0], z0 = t.z[0];
#pragma omp parallel for reduction(min : x0, y0, z0) schedule(static)
  for (int32_t n = 0; n < t.n_nodes; n++) {
    x0 = std::min(x0, t.x[n]);
    y0 = std::min(y0, t.y[n]);
    z0 = std::min(z0, t.z[n]);
  }
  hvec<int32_t> gi(t.n_nodes), gj(t.n_nodes), gk(t.n_nodes);  // lattice coordinates, < 2^20
  int64_t mi = 0, mj = 0, mk = 0;
  auto lattice = [](double v, double o, double h, int32_t &out) {
    const double f = (v - o) / h;
    const int64_t q = (int64_t)std::llround(f);
    out = (int32_t)q;
    return std::fabs(f - (double)q) <= 1e-6 && q >= 0 && q < (1 << 20);
  };
  bool on = true;
#pragma omp parallel for reduction(max : mi, mj, mk) reduction(&& : on) schedule(static)
  for (int32_t n = 0; n < t.n_nodes; n++) {
    const bool ok = lattice(t.x[n], x0, t.hx, gi[n]) && lattice(t.y[n], y0, t.hy, gj[n]) &&
                    lattice(t.z[n], z0, t.hz, gk[n]);
    on = on && ok;
    if (!ok) continue;
    mi = std::max<int64_t>(mi, gi[n]);
    mj = std::max<int64_t>(mj, gj[n]);
    mk = std::max<int64_t>(mk, gk[n]);
  }
  if (!on) {
    g.why = "node off the lattice";
    return;
  }
  if (mi < 1 || mj < 1 || mk < 1) {
    g.why = "degenerate lattice";
    return;
  }
  const int64_t nx = mi, ny = mj, nz = mk;
  const int64_t gcells = nx * ny * nz;
  const int64_t pnx = GridMap::node_pitch(nx), pcx = GridMap::cell_pitch(nx);
  if (pnx * (ny + 1) * (nz + 1) >= (int64_t(1) << 31) - 1) {
    g.why = "lattice too large for 32-bit indices";
    return;
  }
  if ((double)(gcells - t.n_cells) > max_void_fraction * (double)gcells) {
    g.why = "lattice box mostly void";
    return;
  }
  g.nx = (int32_t)nx;
  g.ny = (int32_t)ny;
  g.nz = (int32_t)nz;
  g.pnx = (int32_t)pnx;
  g.pcx = (int32_t)pcx;
  g.node_grid.resize(t.n_nodes);
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < t.n_nodes; n++) g.node_grid[n] = g.node_at(gi[n], gj[n], gk[n]);
  // The first node (in node order) on a site keeps it; later ones get tail
  // slots, numbered in node order (split sites).  Parallel: the lowest node
  // per site, then per contiguous run of nodes the count of later ones, a
  // prefix sum over the runs, and the numbering within each run.
  hvec<int32_t> first;
  fill_par(first, (size_t)g.node_sites(), INT32_MAX);
  hvec<uint8_t> split;
  fill_par(split, (size_t)g.node_sites(), uint8_t(0));
  const int32_t nn = t.n_nodes;
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < nn; n++) atomic_min(&first[(size_t)g.node_grid[n]], n);
  const int runs = std::max(1, std::min(omp_get_max_threads() * 4, nn / 4096 + 1));
  std::vector<int64_t> later((size_t)runs + 1, 0);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < runs; r++) {
    const int32_t n0 = (int32_t)((int64_t)nn * r / runs), n1 = (int32_t)((int64_t)nn * (r + 1) / runs);
    int64_t cnt = 0;
    for (int32_t n = n0; n < n1; n++) cnt += first[(size_t)g.node_grid[n]] != n;
    later[(size_t)r + 1] = cnt;
  }
  for (int r = 0; r < runs; r++) later[(size_t)r + 1] += later[(size_t)r];
  g.n_extra = later[(size_t)runs];
  if (g.node_len() >= (int64_t(1) << 31) - 1) {
    g.why = "lattice too large for 32-bit indices";
    return;
  }
  if (g.n_extra > 0) {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < runs; r++) {
      const int32_t n0 = (int32_t)((int64_t)nn * r / runs), n1 = (int32_t)((int64_t)nn * (r + 1) / runs);
      int64_t e = later[(size_t)r];
      for (int32_t n = n0; n < n1; n++) {
        const int64_t site = g.node_grid[n];
        if (first[(size_t)site] == n) continue;
        __atomic_store_n(&split[(size_t)site], (uint8_t)1, __ATOMIC_RELAXED);
        g.node_grid[n] = g.node_sites() + e++;
      }
    }
  }
  if (g.n_extra > t.n_nodes / 8) {
    g.why = "too many nodes sharing lattice sites";
    return;
  }
  static const int bx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, by[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                   bz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  g.cell_grid.resize(t.n_cells);
  bool boxes = true;
#pragma omp parallel for reduction(&& : boxes) schedule(static)
  for (int32_t c = 0; c < t.n_cells; c++) {
    const int32_t *h = &t.hex[(size_t)c * 8];
    const int64_t i0 = gi[h[0]], j0 = gj[h[0]], k0 = gk[h[0]];
    bool box = true;
    for (int kb = 0; kb < 8; kb++)
      box = box && gi[h[kb]] == i0 + bx[kb] && gj[h[kb]] == j0 + by[kb] && gk[h[kb]] == k0 + bz[kb];
    boxes = boxes && box;
    g.cell_grid[c] = box ? g.cell_at(i0, j0, k0) : 0;
  }
  if (!boxes) {
    g.why = "cell is not a lattice box in corner order";
    return;
  }
  hvec<uint8_t> ctaken;
  fill_par(ctaken, (size_t)g.cell_sites(), uint8_t(0));
  bool twice = false;
#pragma omp parallel for reduction(|| : twice) schedule(static)
  for (int32_t c = 0; c < t.n_cells; c++)
    twice = __atomic_exchange_n(&ctaken[(size_t)g.cell_grid[c]], (uint8_t)1, __ATOMIC_RELAXED) || twice;
  if (twice) {
    g.why = "two cells on one lattice site";
    return;
  }
  if (g.n_extra > 0) {  // copies and fix cells
    g.copy_of_node.assign((size_t)t.n_nodes, -1);
    for (int32_t n = 0; n < t.n_nodes; n++)
      if (split[(size_t)g.node_at(gi[n], gj[n], gk[n])]) {
        g.copy_of_node[n] = (int32_t)g.copy_node.size();
        g.copy_node.push_back(n);
        g.copy_site.push_back(g.node_at(gi[n], gj[n], gk[n]));
      }
    g.copy_mask.assign(g.copy_node.size(), 0);
    g.fix_of_cell.assign((size_t)t.n_cells, -1);
    for (int32_t c = 0; c < t.n_cells; c++) {
      const int32_t *h = &t.hex[(size_t)c * 8];
      bool fix = false;
      for (int kb = 0; kb < 8; kb++) {
        const int32_t cp = g.copy_of_node[h[kb]];
        if (cp < 0) continue;
        fix = true;
        // the cell sits at (1-bx, 1-by, 1-bz) among the eight around its corner kb
        g.copy_mask[(size_t)cp] |= (uint8_t)(1u << ((1 - bx[kb]) + 2 * (1 - by[kb]) + 4 * (1 - bz[kb])));
      }
      if (fix) {
        g.fix_of_cell[c] = (int32_t)g.fix_cell.size();
        g.fix_cell.push_back(c);
      }
    }
  }
  g.col_top.assign((size_t)nx * ny, 0);
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < t.n_cells; c++) {
    const int64_t q = g.cell_grid[c], i = q % pcx, j = (q / pcx) % ny, k = q / (pcx * ny);
    atomic_max(&g.col_top[(size_t)(j * nx + i)], (int32_t)k + 1);
  }
  g.ok = true;
}

void tile_ranges(const std::vector<int32_t> &elems, int32_t n_elems, int tile,
                 std::vector<int32_t> &ranges) {
  const int64_t n_tiles = ((int64_t)n_elems + tile - 1) / tile;
  ranges.assign((size_t)n_tiles * 2, 0);
  size_t i = 0;
  for (int64_t b = 0; b < n_tiles; b++) {
    const int64_t lo = b * tile, hi = lo + tile;
    while (i < elems.size() && elems[i] < lo) i++;
    ranges[(size_t)b * 2] = (int32_t)i;
    size_t j = i;
    while (j < elems.size() && elems[j] < hi) j++;
    ranges[(size_t)b * 2 + 1] = (int32_t)j;
    i = j;
  }
}

}  // namespace pn
