// pn_grid.cpp -- grid form of the solver: voxel-grid meshes, implicit
// indices, one fused plane-marching kernel per step (rsg_grid.cu) with
// double-buffered state.  Host arrays stay in the caller's numbering; the
// device holds the lattice numbering (x fastest) and this file maps between.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <type_traits>

#include "pn_solver.hpp"

namespace pn {

namespace {

struct Tiles {
  int tx, ty, bx_count, by_count;
  int32_t nx, ny, nz;
  // owning block and local index of lattice column (i, j)
  void locate(int64_t i, int64_t j, int32_t &blk, int32_t &t) const {
    const int64_t bx = i / (tx - 1), by = j / (ty - 1);
    blk = (int32_t)(by * bx_count + bx);
    t = (int32_t)((i - bx * (tx - 1)) + tx * (j - by * (ty - 1)));
  }
  int64_t blocks() const { return (int64_t)bx_count * by_count; }
  // blocks whose node tile [b*(t-1), b*(t-1)+t) holds column (i, j), with the
  // local index there: the owner and, on a tile seam, the neighbour whose
  // apron the column is
  template <typename F>
  void each_block_computing(int64_t i, int64_t j, F &&f) const {
    int64_t bxs[2], bys[2];
    int nbx = 0, nby = 0;
    bxs[nbx++] = i / (tx - 1);
    if (i % (tx - 1) == 0 && i > 0) bxs[nbx++] = i / (tx - 1) - 1;
    bys[nby++] = j / (ty - 1);
    if (j % (ty - 1) == 0 && j > 0) bys[nby++] = j / (ty - 1) - 1;
    for (int a = 0; a < nbx; a++)
      for (int b = 0; b < nby; b++) {
        const int64_t bx = bxs[a], by = bys[b];
        if (bx >= bx_count || by >= by_count) continue;
        f((int32_t)(by * bx_count + bx), (int32_t)((i - bx * (tx - 1)) + tx * (j - by * (ty - 1))));
      }
  }
};

Tiles tiles_of(const GridMap &g, int tile_rows) {
  Tiles T;
  T.tx = kGridTileX;
  T.ty = tile_rows;
  T.nx = g.nx;
  T.ny = g.ny;
  T.nz = g.nz;
  T.bx_count = g.nx / (T.tx - 1) + 1;
  T.by_count = g.ny / (T.ty - 1) + 1;
  return T;
}

void node_ijk(const GridMap &g, int64_t q, int64_t &i, int64_t &j, int64_t &k) {
  const int64_t w = g.pnx, h = g.ny + 1;
  i = q % w;
  j = (q / w) % h;
  k = q / (w * h);
}

void cell_ijk(const GridMap &g, int64_t q, int64_t &i, int64_t &j, int64_t &k) {
  i = q % g.pcx;
  j = (q / g.pcx) % g.ny;
  k = q / ((int64_t)g.pcx * g.ny);
}

// 2: only the C11..C33 block and the shear diagonal; 1: monoclinic about z;
// 0: general (see c_used in rsg_grid.cu)
int symmetry_class(const MaterialTables &mt) {
  bool ortho = true, mono = true;
  for (int32_t m = 0; m < mt.n_mat; m++) {
    const double *c = &mt.c36[(size_t)m * 36];
    for (int k = 0; k < 6; k++)
      for (int j = 0; j < 6; j++) {
        const double v = c[k * 6 + j];
        if (v == 0.0) continue;
        const bool in_ortho = (k < 3 && j < 3) || k == j;
        const bool in_mono = in_ortho || (k == 5 && j < 3) || (j == 5 && k < 3) || (k == 3 && j == 4) ||
                             (k == 4 && j == 3);
        ortho = ortho && in_ortho;
        mono = mono && in_mono;
      }
  }
  return ortho ? 2 : mono ? 1 : 0;
}

// (block, layer, local, payload) rows sorted by (block, layer) with the
// per (block, layer) ranges
struct Keyed {
  int64_t slot;  // block * layers + layer
  int32_t key, sig, idx;
  double w;
};

// entries sorted by (slot, local index), stably: a thread finds its own
// entries of a slot by a binary search (first_local), and one node's entries
// keep their order (the order their terms are added in)
void ranges_of(std::vector<Keyed> &L, int64_t n_slots, std::vector<int32_t> &rng) {
  std::stable_sort(L.begin(), L.end(), [](const Keyed &a, const Keyed &b) {
    return a.slot != b.slot ? a.slot < b.slot : (a.key & 0xffff) < (b.key & 0xffff);
  });
  rng.assign((size_t)n_slots * 2, 0);
  size_t e = 0;
  for (int64_t sl = 0; sl < n_slots; sl++) {
    rng[(size_t)sl * 2] = (int32_t)e;
    while (e < L.size() && L[e].slot == sl) e++;
    rng[(size_t)sl * 2 + 1] = (int32_t)e;
  }
}

}  // namespace

std::vector<int32_t> grid_tile_tops(const GridMap &g, int tile_rows) {
  const Tiles T = tiles_of(g, tile_rows);
  std::vector<int32_t> top((size_t)T.blocks(), 0);
  for (int by = 0; by < T.by_count; by++)
    for (int bx = 0; bx < T.bx_count; bx++) {
      const int64_t i0 = (int64_t)bx * (T.tx - 1), j0 = (int64_t)by * (T.ty - 1);
      int32_t t = 0;
      for (int64_t j = std::max<int64_t>(0, j0 - 1); j < std::min<int64_t>(g.ny, j0 + T.ty); j++)
        for (int64_t i = std::max<int64_t>(0, i0 - 1); i < std::min<int64_t>(g.nx, i0 + T.tx); i++)
          t = std::max(t, g.col_top[(size_t)(j * g.nx + i)]);
      top[(size_t)by * T.bx_count + bx] = t;
    }
  return top;
}

// The tensor-copy kernel (rsg_grid_tma.cu) runs when the stiffness table fits
// its shared-memory rows and every buffer meets the copy rules; otherwise the
// classic kernel (rsg_grid.cu).  PN_GRID_KERNEL=classic selects the classic
// kernel for comparisons.
static bool want_tma(int32_t n_mat) {
  const char *v = std::getenv("PN_GRID_KERNEL");
  if (v && std::strcmp(v, "classic") == 0) return false;
  return n_mat + 1 <= kGridTmaRowsMax;
}

// The grid form moves about 2.3x fewer bytes per cell-step than the tables;
// it serves a mesh whose lattice box it marches in at most twice the mesh's
// own cells.  The tensor-copy kernel stops each tile column at its top solid
// layer (grid_tile_tops); the classic kernel marches the whole box.
bool grid_eligible(const MeshTables &m, const MaterialTables &mt, int precision, const GridMap &g,
                   std::string *why) {
  auto no = [&](const std::string &r) {
    if (why) *why = r;
    return false;
  };
  if (!g.ok) return no(g.why);
  if (precision == PN_PREC_F64_EXACT) return no("the exact FP64 form has no grid kernel");
  if (mt.n_mat >= 255) return no("more than 254 materials");
  int64_t marched = 0;
  if (want_tma(mt.n_mat)) {
    const Tiles T = tiles_of(g, kGridTileRows);
    const std::vector<int32_t> top = grid_tile_tops(g, kGridTileRows);
    for (int by = 0; by < T.by_count; by++)
      for (int bx = 0; bx < T.bx_count; bx++) {
        const int64_t cols = std::min<int64_t>(T.tx - 1, g.nx - (int64_t)bx * (T.tx - 1)) *
                             std::min<int64_t>(T.ty - 1, g.ny - (int64_t)by * (T.ty - 1));
        marched += std::max<int64_t>(cols, 0) * top[(size_t)by * T.bx_count + bx];
      }
  } else {
    marched = g.grid_cells();
  }
  if (marched > 2 * (int64_t)m.n_cells) return no("lattice box mostly void");
  return true;
}

// Algorithmic HBM bytes of one grid step, e bytes per value: S read + write
// and the material byte per marched lattice cell, V read + write and dt/rho
// per marched lattice node.  The tensor-copy kernel marches each tile's owned
// columns up to its top solid layer (node layers 0..top; nothing when top is
// 0), the classic kernel the whole box.
int64_t grid_step_bytes(const GridMap &g, int32_t n_mat, int64_t e, int tile_rows) {
  if (!want_tma(n_mat)) return g.grid_cells() * (12 * e + 1) + g.grid_nodes() * 7 * e;
  const Tiles T = tiles_of(g, tile_rows);
  const std::vector<int32_t> top = grid_tile_tops(g, tile_rows);
  int64_t cells = 0, nodes = 0;
  for (int by = 0; by < T.by_count; by++)
    for (int bx = 0; bx < T.bx_count; bx++) {
      const int64_t i0 = (int64_t)bx * (T.tx - 1), j0 = (int64_t)by * (T.ty - 1);
      const int64_t ccols = std::max<int64_t>(0, std::min<int64_t>(T.tx - 1, g.nx - i0)) *
                            std::max<int64_t>(0, std::min<int64_t>(T.ty - 1, g.ny - j0));
      const int64_t ncols = std::max<int64_t>(0, std::min<int64_t>(T.tx - 1, g.nx + 1 - i0)) *
                            std::max<int64_t>(0, std::min<int64_t>(T.ty - 1, g.ny + 1 - j0));
      const int64_t t = top[(size_t)by * T.bx_count + bx];
      cells += ccols * t;
      nodes += t > 0 ? ncols * (t + 1) : 0;
    }
  return cells * (12 * e + 1) + nodes * 7 * e;
}

int64_t grid_footprint(const GridMap &g, const MaterialTables &mt, int precision) {
  const int64_t e = precision == PN_PREC_F32 ? 4 : 8;
  const int64_t gn = g.node_len(), gc = g.cell_sites();
  // (the default 32 x 8 tiles: more tiles than any other shape)
  const int64_t tiles = (int64_t)(g.nx / (kGridTileX - 1) + 1) * (g.ny / (kGridTileRows - 1) + 1);
  // state (two halves), dt/rho, material bytes, stiffness rows, tensor maps,
  // per-tile top layers, error word and finiteness flags, split-site tables
  // (the copies' and fix cells' source and sensor entries come with those)
  return 2 * (3 * gn + 6 * gc) * e + gn * e + gc + (int64_t)(mt.n_mat + 1) * 36 * e +
         2 * (int64_t)grid_tma_maps_bytes() + tiles * 4 + 64 + 8 +
         (int64_t)g.copy_node.size() * (int64_t)sizeof(SplitCopy) +
         (int64_t)g.fix_cell.size() * (int64_t)sizeof(FixCell) + 16;
}


namespace {

// The FP64 form's double-float range as biased double exponents [e_lo, e_hi]:
// every value the double-float path takes is 0 or lies in
// [2^-100 / min(1, cmin), 2^100 / max(1, cmax)], so that its products with
// the step's coefficients (nonzero magnitudes cmin..cmax) stay within
// 2^-100..2^100, where a double-float keeps its 48-bit significand (the low
// word stays a normal float) and nothing overflows.
void range_bounds(double cmin, double cmax, int32_t &e_lo, int32_t &e_hi) {
  const double lo = std::ldexp(1.0, -100) / std::min(1.0, cmin);
  const double hi = std::ldexp(1.0, 100) / std::max(1.0, cmax);
  const int elo = (int)std::ceil(std::log2(lo)) + 1023;       // 2^(e-1023) >= lo
  const int ehi = (int)std::floor(std::log2(hi)) - 1 + 1023;  // 2^(e-1023+1) <= hi
  e_lo = std::min(2046, std::max(1, elo));
  e_hi = std::min(2046, std::max(0, ehi));
}

// tensor maps of both input parities for tiles of `rows` rows (false: a
// buffer or pitch the copies cannot take, or rows the storage has no kernel for)
bool encode_maps(pn_solver *s, int rows, unsigned char *out) {
  const GridMap &g = s->grid;
  const size_t mb = grid_tma_maps_bytes();
  bool ok = true;
  for (int p = 0; p < 2 && ok; p++) {
    const void *V[3] = {s->V[p][0], s->V[p][1], s->V[p][2]};
    const void *S[6] = {s->S[p][0], s->S[p][1], s->S[p][2], s->S[p][3], s->S[p][4], s->S[p][5]};
    ok = grid_tma_encode(s->precision, rows, g.nx, g.ny, g.nz, g.pnx, g.pcx, V, S, s->d_coef, s->d_gmat,
                         out + p * mb);
  }
  return ok;
}

}  // namespace

// Tile rows of a new solver's tensor-copy kernel (the batch tuner may change
// them): 32 x 8 unless PN_GRID_TILE_ROWS names another shape the storage has.
int grid_default_tile_rows(int precision, const GridMap &g) {
  (void)g;
  if (const char *v = std::getenv("PN_GRID_TILE_ROWS")) {
    const int r = std::atoi(v);
    if (grid_tma_rows_supported(precision, r)) return r;
  }
  return kGridTileRows;
}

// Re-tile a grid-form solver with the tensor-copy kernel: tensor maps, tile
// tops, and the per-(tile, layer) source and sensor lists for `rows` rows.
// Results do not depend on the tiling.  False (nothing changed) when the
// solver has no tensor-copy kernel or its storage no such tiles.
bool grid_set_tile_rows(pn_solver *s, int rows) {
  if (s->form != PN_FORM_GRID || !s->d_tmaps) return rows == s->tile_rows;
  if (rows == s->tile_rows) return true;
  if (!grid_tma_rows_supported(s->precision, rows)) return false;
  const size_t mb = grid_tma_maps_bytes();
  std::vector<unsigned char> maps(2 * mb);
  if (!encode_maps(s, rows, maps.data())) return false;
  ck(cudaStreamSynchronize(s->stream), "retile sync");  // work in flight reads the old tables
  s->tile_rows = rows;
  s->upload_raw(s->d_tmaps, maps.data(), 2 * mb);
  const std::vector<int32_t> top = grid_tile_tops(s->grid, rows);
  s->release(s->d_ktop);
  s->d_ktop = s->alloc<int32_t>(top.size() * sizeof(int32_t));
  s->upload_raw(s->d_ktop, top.data(), top.size() * sizeof(int32_t));
  s->step_bytes_cached = 0;
  if (!s->src.empty() && !s->src_dirty) grid_sources(s);
  if (s->n_sens > 0) {
    s->release(s->d_srng); s->release(s->d_skey); s->release(s->d_sidx);
    grid_sensors(s, s->sensor_pairs);
  }
  ck(cudaStreamSynchronize(s->stream), "retile upload");
  return true;
}

void grid_create(pn_solver *s) {
  const GridMap &g = s->grid;
  const int64_t gn = g.node_len(), gc = g.cell_sites();
  const size_t e = s->esz;
  for (int b = 0; b < 2; b++) {
    for (int k = 0; k < 3; k++) {
      s->V[b][k] = s->alloc<void>((size_t)gn * e);
      ck(cudaMemsetAsync(s->V[b][k], 0, (size_t)gn * e, s->stream), "memset");
    }
    for (int k = 0; k < 6; k++) {
      s->S[b][k] = s->alloc<void>((size_t)gc * e);
      ck(cudaMemsetAsync(s->S[b][k], 0, (size_t)gc * e, s->stream), "memset");
    }
  }
  // every mesh node / cell has its own site: the scatters are race-free
  const int32_t nn = s->mesh.n_nodes, nc = s->mesh.n_cells;
  hvec<double> coef((size_t)gn);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < gn; q++) coef[q] = 0.0;
#pragma omp parallel for schedule(static)
  for (int32_t u = 0; u < nn; u++) coef[g.node_grid[u]] = s->mat.coef[u];
  s->d_coef = s->alloc<void>((size_t)gn * e);
  s->upload_real(s->d_coef, coef.data(), coef.size());
  hvec<uint8_t> gm((size_t)gc);
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < gc; q++) gm[q] = (uint8_t)s->mat.n_mat;  // void row
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < nc; c++) gm[g.cell_grid[c]] = (uint8_t)s->mat.cell_mat[c];
  s->d_gmat = s->alloc<uint8_t>((size_t)gc);
  s->upload_raw(s->d_gmat, gm.data(), gm.size());
  std::vector<double> ct((size_t)(s->mat.n_mat + 1) * 36, 0.0);
  for (size_t q = 0; q < s->mat.c36.size(); q++) ct[q] = s->dt * s->mat.c36[q];
  s->d_ctab = s->alloc<void>(ct.size() * e);
  s->upload_real(s->d_ctab, ct.data(), ct.size());
  s->sym = symmetry_class(s->mat);
  s->cur = 0;
  s->d_err = s->alloc<int32_t>(16);
  ck(cudaMemsetAsync(s->d_err, 0, 16, s->stream), "memset");
  s->tile_rows = kGridTileRows;
  if (want_tma(s->mat.n_mat)) {
    const int rows = grid_default_tile_rows(s->precision, g);
    const size_t mb = grid_tma_maps_bytes();
    std::vector<unsigned char> maps(2 * mb);
    const bool ok = encode_maps(s, rows, maps.data());
    if (ok) {
      s->tile_rows = rows;
      s->d_tmaps = s->alloc<void>(2 * mb);
      s->upload_raw(s->d_tmaps, maps.data(), 2 * mb);
      const std::vector<int32_t> top = grid_tile_tops(g, rows);
      s->d_ktop = s->alloc<int32_t>(top.size() * sizeof(int32_t));
      s->upload_raw(s->d_ktop, top.data(), top.size() * sizeof(int32_t));
      // a cubic lattice: every difference is scaled by the same 0.25/h, which
      // then goes into the coefficients instead of the step (fewer FP64 ops)
      const double h = s->mesh.hx;
      auto near = [](double a, double b) { return std::fabs(a - b) <= 1e-12 * std::fabs(b); };
      if (near(s->mesh.hy, h) && near(s->mesh.hz, h)) {
        const double g = 0.25 / h;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < gn; q++) coef[q] *= g;
        for (double &v : ct) v *= g;
        s->upload_real(s->d_coef, coef.data(), coef.size());
        s->upload_real(s->d_ctab, ct.data(), ct.size());
        s->gfold = g;
      }
    }
  }
  // the FP64 form: each block of a step takes the double-float path unless
  // its tile's neighbourhood holds values outside that path's range
  // (PN_F64_PATH=fp64 keeps every block on the FP64 path, for comparisons)
  const char *path = std::getenv("PN_F64_PATH");
  if (s->precision == PN_PREC_F64 && s->d_tmaps && !(path && std::strcmp(path, "fp64") == 0)) {
    double vmin = 1.0, vmax = 1.0, smin = 1.0, smax = 1.0;
    auto see = [](double v, double &lo, double &hi) {
      v = std::fabs(v);
      if (v == 0.0) return;
      lo = std::min(lo, v);
      hi = std::max(hi, v);
    };
    for (double v : ct) see(v, vmin, vmax);                            // velocities x dt*C*g
    for (int64_t q = 0; q < gn; q++) see(coef[q], smin, smax);          // stresses x dt/rho*g
    if (s->gfold == 1.0)
      for (double h : {s->mesh.hx, s->mesh.hy, s->mesh.hz}) {
        see(0.25 / h, vmin, vmax);
        see(0.25 / h, smin, smax);
      }
    s->r_cmin = vmin;
    s->r_cmax = vmax;
    s->r_cmin_s = smin;
    s->r_cmax_s = smax;
    range_bounds(vmin, vmax, s->r_elo, s->r_ehi);
    range_bounds(smin, smax, s->r_elo_s, s->r_ehi_s);
  }
  // coefficients themselves outside the split's exact range: IEEE double only
  const bool extreme = std::min(s->r_cmin, s->r_cmin_s) < std::ldexp(1.0, -90) ||
                       std::max(s->r_cmax, s->r_cmax_s) > std::ldexp(1.0, 90);
  if (s->precision == PN_PREC_F64 && s->d_tmaps && s->r_elo <= s->r_ehi && s->r_elo_s <= s->r_ehi_s && !extreme) {
    const int64_t tiles = (int64_t)(g.nx / (kGridTileX - 1) + 1) * (g.ny / (kGridTileRows - 1) + 1);
    s->d_rflags = s->alloc<uint32_t>((size_t)(3 * tiles) * sizeof(uint32_t));
    s->d_pathcnt = s->alloc<unsigned long long>(2 * sizeof(unsigned long long));
    ck(cudaMemsetAsync(s->d_pathcnt, 0, 2 * sizeof(unsigned long long), s->stream), "memset");
    grid_reset_range_flags(s);
  }
  grid_split_upload(s);
  ck(cudaStreamSynchronize(s->stream), "create sync");
}

void grid_reset_range_flags(pn_solver *s) {
  if (!s->d_rflags) return;
  const GridMap &g = s->grid;
  const int64_t tiles = (int64_t)(g.nx / (kGridTileX - 1) + 1) * (g.ny / (kGridTileRows - 1) + 1);
  ck(cudaMemsetAsync(s->d_rflags, 0, (size_t)(3 * tiles) * sizeof(uint32_t), s->stream), "memset");
  ck(cudaMemsetAsync(s->d_rflags + (s->step % 3) * tiles, 0xff, (size_t)tiles * sizeof(uint32_t), s->stream),
     "memset");  // every bit: every tile on the FP64 path
}

void grid_split_upload(pn_solver *s) {
  const GridMap &g = s->grid;
  s->release(s->d_copies); s->release(s->d_fix);
  s->release(s->d_cf_dir); s->release(s->d_cf_sig); s->release(s->d_cf_w); s->release(s->d_cs_idx);
  s->release(s->d_cm_comp); s->release(s->d_cm_sig); s->release(s->d_cm_w);
  if (g.copy_node.empty()) return;
  auto &F = s->split_forces;
  auto &Sn = s->split_sensors;
  auto &M = s->fix_moments;
  std::stable_sort(F.begin(), F.end(), [](const auto &a, const auto &b) { return a.copy < b.copy; });
  std::stable_sort(Sn.begin(), Sn.end(), [](const auto &a, const auto &b) { return a.copy < b.copy; });
  std::stable_sort(M.begin(), M.end(), [](const auto &a, const auto &b) { return a.fix < b.fix; });
  std::vector<SplitCopy> cp(g.copy_node.size());
  size_t f = 0, e = 0;
  for (size_t q = 0; q < cp.size(); q++) {
    int64_t i, j, k;
    node_ijk(g, g.copy_site[q], i, j, k);
    SplitCopy &c = cp[q];
    c.i = (int32_t)i;
    c.j = (int32_t)j;
    c.k = (int32_t)k;
    c.mask = g.copy_mask[q];
    c.v = g.node_grid[(size_t)g.copy_node[q]];
    c.f0 = (int32_t)f;
    while (f < F.size() && F[f].copy == (int32_t)q) f++;
    c.f1 = (int32_t)f;
    c.s0 = (int32_t)e;
    while (e < Sn.size() && Sn[e].copy == (int32_t)q) e++;
    c.s1 = (int32_t)e;
  }
  std::vector<FixCell> fx(g.fix_cell.size());
  size_t m = 0;
  for (size_t q = 0; q < fx.size(); q++) {
    const int32_t c = g.fix_cell[q];
    fx[q].cell = g.cell_grid[(size_t)c];
    for (int kb = 0; kb < 8; kb++) fx[q].v[kb] = g.node_grid[(size_t)s->mesh.hex[(size_t)c * 8 + kb]];
    fx[q].m0 = (int32_t)m;
    while (m < M.size() && M[m].fix == (int32_t)q) m++;
    fx[q].m1 = (int32_t)m;
  }
  s->d_copies = s->alloc<SplitCopy>(cp.size() * sizeof(SplitCopy));
  s->upload_raw(s->d_copies, cp.data(), cp.size() * sizeof(SplitCopy));
  s->d_fix = s->alloc<FixCell>(fx.size() * sizeof(FixCell));
  s->upload_raw(s->d_fix, fx.data(), fx.size() * sizeof(FixCell));
  std::vector<int32_t> dir(F.size()), sig(F.size()), idx(Sn.size()), comp(M.size()), msig(M.size());
  std::vector<double> w(F.size()), mw(M.size());
  for (size_t q = 0; q < F.size(); q++) {
    dir[q] = F[q].dir;
    sig[q] = F[q].sig;
    w[q] = F[q].w;
  }
  for (size_t q = 0; q < Sn.size(); q++) idx[q] = Sn[q].idx;
  for (size_t q = 0; q < M.size(); q++) {
    comp[q] = M[q].comp;
    msig[q] = M[q].sig;
    mw[q] = M[q].w;
  }
  s->d_cf_dir = s->alloc<int32_t>(dir.size() * 4);
  s->d_cf_sig = s->alloc<int32_t>(sig.size() * 4);
  s->d_cf_w = s->alloc<void>(w.size() * s->esz);
  s->d_cs_idx = s->alloc<int32_t>(idx.size() * 4);
  s->d_cm_comp = s->alloc<int32_t>(comp.size() * 4);
  s->d_cm_sig = s->alloc<int32_t>(msig.size() * 4);
  s->d_cm_w = s->alloc<void>(mw.size() * s->esz);
  s->upload_raw(s->d_cf_dir, dir.data(), dir.size() * 4);
  s->upload_raw(s->d_cf_sig, sig.data(), sig.size() * 4);
  s->upload_real(s->d_cf_w, w.data(), w.size());
  s->upload_raw(s->d_cs_idx, idx.data(), idx.size() * 4);
  s->upload_raw(s->d_cm_comp, comp.data(), comp.size() * 4);
  s->upload_raw(s->d_cm_sig, msig.data(), msig.size() * 4);
  s->upload_real(s->d_cm_w, mw.data(), mw.size());
}

// node / cell -> lattice position maps on the device (first transfer)
static void ensure_grid_maps(pn_solver *s) {
  const GridMap &g = s->grid;
  if (!s->d_nmap) {
    s->d_nmap = s->alloc<int64_t>(g.node_grid.size() * sizeof(int64_t));
    s->upload_raw(s->d_nmap, g.node_grid.data(), g.node_grid.size() * sizeof(int64_t));
  }
  if (!s->d_cmap) {
    s->d_cmap = s->alloc<int64_t>(g.cell_grid.size() * sizeof(int64_t));
    s->upload_raw(s->d_cmap, g.cell_grid.data(), g.cell_grid.size() * sizeof(int64_t));
  }
}

// The idle half of the double buffer is cleared (void sites stay zero) and
// the caller's fields scattered to their lattice positions on the device
// (rsg_state.cu), which also checks them for NaN and infinity; the solver
// switches to that half only when every value is finite.
int grid_put_state(pn_solver *s, const double *const *V, const double *const *S) {
  const GridMap &g = s->grid;
  const int64_t gn = g.node_len(), gc = g.cell_sites();
  const int b = s->cur ^ 1;
  ensure_grid_maps(s);
  if (!s->d_nonfinite) s->d_nonfinite = s->alloc<int32_t>(4 * sizeof(int32_t));
  ck(cudaMemsetAsync(s->d_nonfinite, 0, 4 * sizeof(int32_t), s->stream), "memset");
  // the FP64 form: the conversion kernels flag the tiles of out-of-range
  // values for the next step directly (word 2: a split-site copy was out of
  // range, which puts every tile on the FP64 path for one step instead)
  const int64_t tiles = (int64_t)(g.nx / (kGridTileX - 1) + 1) * (g.ny / (kGridTileRows - 1) + 1);
  StateRangeFlags rv{}, rs{};
  if (s->d_rflags) {  // staged: a refused state leaves the solver's flags as they were
    if (!s->d_rflags_stage) s->d_rflags_stage = s->alloc<uint32_t>((size_t)tiles * sizeof(uint32_t));
    ck(cudaMemsetAsync(s->d_rflags_stage, 0, (size_t)tiles * sizeof(uint32_t), s->stream), "memset");
    rv.flags = s->d_rflags_stage;
    rv.unplaced = s->d_nonfinite + 2;
    rv.gxc = g.nx / (kGridTileX - 1) + 1;
    rv.ty_own = kGridTileRows - 1;
    rs = rv;
    rv.lattice_len = (int64_t)g.pnx * (g.ny + 1) * (g.nz + 1);
    rv.pitch = g.pnx;
    rv.rows = g.ny + 1;
    rv.e_lo = (uint32_t)s->r_elo;
    rv.e_hi = (uint32_t)s->r_ehi;
    rs.lattice_len = (int64_t)g.pcx * g.ny * g.nz;
    rs.pitch = g.pcx;
    rs.rows = g.ny;
    rs.e_lo = (uint32_t)s->r_elo_s;
    rs.e_hi = (uint32_t)s->r_ehi_s;
    rs.cell = 1;
  }
  for (int k = 0; k < 3; k++) {
    ck(cudaMemsetAsync(s->V[b][k], 0, (size_t)gn * s->esz, s->stream), "memset");
    if (V && V[k])
      s->put_field(s->V[b][k], V[k], (size_t)s->mesh.n_nodes, s->d_nmap, s->d_nonfinite, s->d_rflags ? &rv : nullptr);
  }
  for (int k = 0; k < 6; k++) {
    ck(cudaMemsetAsync(s->S[b][k], 0, (size_t)gc * s->esz, s->stream), "memset");
    if (S && S[k])
      s->put_field(s->S[b][k], S[k], (size_t)s->mesh.n_cells, s->d_cmap, s->d_nonfinite + 1,
                   s->d_rflags ? &rs : nullptr);
  }
  int32_t bad[3] = {0, 0, 0};
  ck(cudaMemcpyAsync(bad, s->d_nonfinite, sizeof(bad), cudaMemcpyDeviceToHost, s->stream), "finite check");
  ck(cudaStreamSynchronize(s->stream), "set_state");
  if (bad[0] || bad[1]) return (bad[0] ? 1 : 0) | (bad[1] ? 2 : 0);
  s->cur = b;
  if (s->d_rflags) {
    if (bad[2]) {
      grid_reset_range_flags(s);  // a split-site copy out of range: FP64 for one step
    } else {
      ck(cudaMemsetAsync(s->d_rflags, 0, (size_t)(3 * tiles) * sizeof(uint32_t), s->stream), "memset");
      ck(cudaMemcpyAsync(s->d_rflags + (s->step % 3) * tiles, s->d_rflags_stage, (size_t)tiles * sizeof(uint32_t),
                         cudaMemcpyDeviceToDevice, s->stream),
         "range flags");
    }
  }
  return 0;
}

void grid_get_state(pn_solver *s, double *const *V, double *const *S) {
  ensure_grid_maps(s);
  for (int k = 0; k < 3; k++)
    if (V && V[k]) s->get_field(V[k], s->V[s->cur][k], (size_t)s->mesh.n_nodes, s->d_nmap);
  for (int k = 0; k < 6; k++)
    if (S && S[k]) s->get_field(S[k], s->S[s->cur][k], (size_t)s->mesh.n_cells, s->d_cmap);
  ck(cudaStreamSynchronize(s->stream), "get_state");
}

void grid_sources(pn_solver *s) {
  std::vector<SourceEntry> fe, me;
  const std::vector<const uint8_t *> masks = s->mask_ptrs();
  build_source_entries(s->mesh, s->src, false, fe, me, &masks);
  ck(cudaStreamSynchronize(s->stream), "sources sync");
  s->release(s->d_frng); s->release(s->d_fkey); s->release(s->d_fsig); s->release(s->d_fw);
  s->release(s->d_mrng); s->release(s->d_mkey); s->release(s->d_msig); s->release(s->d_mw);
  const GridMap &g = s->grid;
  const Tiles T = tiles_of(g, s->tile_rows);
  s->n_force = (int32_t)fe.size();
  s->n_moment = (int32_t)me.size();
  s->n_src_nodes = s->n_src_cells = 0;
  auto upload = [&](std::vector<Keyed> &L, int64_t layers, int2 *&rng, int32_t *&key, int32_t *&sig,
                    void *&w) {
    if (L.empty()) return;
    std::vector<int32_t> r;
    ranges_of(L, T.blocks() * layers, r);
    std::vector<int32_t> k(L.size()), sg(L.size());
    std::vector<double> wt(L.size());
    for (size_t q = 0; q < L.size(); q++) {
      k[q] = L[q].key;
      sg[q] = L[q].sig;
      wt[q] = L[q].w;
    }
    rng = s->alloc<int2>(r.size() * 4);
    key = s->alloc<int32_t>(k.size() * 4);
    sig = s->alloc<int32_t>(sg.size() * 4);
    w = s->alloc<void>(wt.size() * s->esz);
    s->upload_raw(rng, r.data(), r.size() * 4);
    s->upload_raw(key, k.data(), k.size() * 4);
    s->upload_raw(sig, sg.data(), sg.size() * 4);
    s->upload_real(w, wt.data(), wt.size());
  };
  std::vector<Keyed> F, M;
  s->split_forces.clear();
  s->fix_moments.clear();
  for (size_t q = 0; q < fe.size(); q++) {
    if (q == 0 || fe[q].elem != fe[q - 1].elem) s->n_src_nodes++;
    const int32_t cp = g.copy_of_node.empty() ? -1 : g.copy_of_node[(size_t)fe[q].elem];
    if (cp >= 0) {  // a node of a split site: the fix-up applies it
      s->split_forces.push_back({cp, fe[q].comp, fe[q].sig, fe[q].w / s->gfold});
      continue;
    }
    int64_t i, j, k;
    node_ijk(g, g.node_grid[fe[q].elem], i, j, k);
    // every block that computes this node's velocity gets the entry: the
    // owner, and the -x / -y neighbours whose apron column / row it is (they
    // need it for the stress of their own cells)
    T.each_block_computing(i, j, [&](int32_t blk, int32_t t) {
      F.push_back(Keyed{(int64_t)blk * (g.nz + 1) + k, t | (fe[q].comp << 16), fe[q].sig, 0, fe[q].w / s->gfold});
    });
  }
  for (size_t q = 0; q < me.size(); q++) {
    int64_t i, j, k;
    cell_ijk(g, g.cell_grid[me[q].elem], i, j, k);
    int32_t blk, t;
    T.locate(i, j, blk, t);
    M.push_back(Keyed{(int64_t)blk * g.nz + k, t | (me[q].comp << 16), me[q].sig, 0, s->dt * me[q].w});
    if (q == 0 || me[q].elem != me[q - 1].elem) s->n_src_cells++;
    const int32_t fx = g.fix_of_cell.empty() ? -1 : g.fix_of_cell[(size_t)me[q].elem];
    if (fx >= 0) s->fix_moments.push_back({fx, me[q].comp, me[q].sig, s->dt * me[q].w});
  }
  upload(F, g.nz + 1, s->d_frng, s->d_fkey, s->d_fsig, s->d_fw);
  upload(M, g.nz, s->d_mrng, s->d_mkey, s->d_msig, s->d_mw);
  if (s->d_rflags) {  // the stresses' double-float range also covers the source weights
    double cmin = s->r_cmin_s, cmax = s->r_cmax_s;
    for (const std::vector<Keyed> *L : {&F, &M})
      for (const Keyed &k : *L) {
        const double v = std::fabs(k.w);
        if (v == 0.0) continue;
        cmin = std::min(cmin, v);
        cmax = std::max(cmax, v);
      }
    for (auto &f : s->split_forces) if (f.w != 0.0) { cmin = std::min(cmin, std::fabs(f.w)); cmax = std::max(cmax, std::fabs(f.w)); }
    for (auto &m : s->fix_moments) if (m.w != 0.0) { cmin = std::min(cmin, std::fabs(m.w)); cmax = std::max(cmax, std::fabs(m.w)); }
    range_bounds(cmin, cmax, s->r_elo_s, s->r_ehi_s);
    grid_reset_range_flags(s);  // tiles judged under the old bounds: FP64 for one step
  }
  grid_split_upload(s);
  ck(cudaStreamSynchronize(s->stream), "sources upload");
}

void grid_sensors(pn_solver *s, const std::vector<std::pair<int32_t, int32_t>> &pr) {
  const GridMap &g = s->grid;
  const Tiles T = tiles_of(g, s->tile_rows);
  if (&pr != &s->sensor_pairs) s->sensor_pairs = pr;  // kept for re-tiling
  std::vector<Keyed> L;
  s->split_sensors.clear();
  for (auto &p : pr) {
    const int32_t cp = g.copy_of_node.empty() ? -1 : g.copy_of_node[(size_t)p.first];
    if (cp >= 0) {  // a node of a split site: the fix-up records it
      s->split_sensors.push_back({cp, p.second});
      continue;
    }
    int64_t i, j, k;
    node_ijk(g, g.node_grid[p.first], i, j, k);
    int32_t blk, t;
    T.locate(i, j, blk, t);
    L.push_back(Keyed{(int64_t)blk * (g.nz + 1) + k, t, 0, p.second, 0.0});
  }
  std::vector<int32_t> r;
  ranges_of(L, T.blocks() * (g.nz + 1), r);
  std::vector<int32_t> key(L.size()), idx(L.size());
  for (size_t q = 0; q < L.size(); q++) {
    key[q] = L[q].key;
    idx[q] = L[q].idx;
  }
  s->d_srng = s->alloc<int2>(r.size() * 4);
  s->d_skey = s->alloc<int32_t>(key.size() * 4);
  s->d_sidx = s->alloc<int32_t>(idx.size() * 4);
  s->upload_raw(s->d_srng, r.data(), r.size() * 4);
  s->upload_raw(s->d_skey, key.data(), key.size() * 4);
  s->upload_raw(s->d_sidx, idx.data(), idx.size() * 4);
  grid_split_upload(s);
}

template <typename T>
void grid_args(pn_solver *s, GridArgs<T> &a) {
  const GridMap &g = s->grid;
  std::memset(&a, 0, sizeof(a));
  a.nx = g.nx;
  a.ny = g.ny;
  a.nz = g.nz;
  a.pnx = g.pnx;
  a.pcx = g.pcx;
  a.coef = (const T *)s->d_coef;
  a.mat = s->d_gmat;
  a.ctab = (const T *)s->d_ctab;
  const bool folded = s->gfold != 1.0;  // 0.25/h lives in the coefficients
  a.g[0] = to_store<T>(folded ? 1.0 : 0.25 / s->mesh.hx);
  a.g[1] = to_store<T>(folded ? 1.0 : 0.25 / s->mesh.hy);
  a.g[2] = to_store<T>(folded ? 1.0 : 0.25 / s->mesh.hz);
  if (s->n_force > 0) {
    a.f_rng = s->d_frng; a.f_key = s->d_fkey; a.f_sig = s->d_fsig; a.f_w = (const T *)s->d_fw;
  }
  if (s->n_moment > 0) {
    a.m_rng = s->d_mrng; a.m_key = s->d_mkey; a.m_sig = s->d_msig; a.m_w = (const T *)s->d_mw;
  }
  a.n_sens = s->n_sens;
  a.traces = s->d_traces;
  a.rec_cap = s->rec_cap;
  a.s_rng = s->n_sens > 0 ? s->d_srng : nullptr;
  a.s_key = s->d_skey;
  a.s_idx = s->d_sidx;
  a.sig_stride = 0;
  a.sig_rows = 1;
  a.err = s->d_err;
  a.ktop = s->d_ktop;
  a.n_rows = s->mat.n_mat + 1;
  a.ortho_rows = 0;
  for (int32_t r = 0; r <= s->mat.n_mat && r < 32; r++) {  // the last row: void (zero)
    bool ortho = true;
    for (int k = 0; k < 6 && ortho && r < s->mat.n_mat; k++)
      for (int j = 0; j < 6; j++)
        if (!((k < 3 && j < 3) || k == j) && s->mat.c36[(size_t)r * 36 + k * 6 + j] != 0.0) ortho = false;
    if (ortho) a.ortho_rows |= 1u << r;
  }
  a.n_copies = (int32_t)g.copy_node.size();
  a.n_fix = (int32_t)g.fix_cell.size();
  a.copies = s->d_copies;
  a.cf_dir = s->d_cf_dir;
  a.cf_sig = s->d_cf_sig;
  a.cf_w = (const T *)s->d_cf_w;
  a.cs_idx = s->d_cs_idx;
  a.fix = s->d_fix;
  a.cm_comp = s->d_cm_comp;
  a.cm_sig = s->d_cm_sig;
  a.cm_w = (const T *)s->d_cm_w;
  // failure-path test hook: PN_TEST_GRID_SKIP_COPY=<layer> leaves that layer's
  // tile copies unissued, so the tensor-copy kernel's bounded wait runs out
  const char *skip = std::getenv("PN_TEST_GRID_SKIP_COPY");
  a.test_skip_layer = skip && *skip ? std::atoi(skip) : kNoLayer;
  a.tile_rows = s->tile_rows;
  a.rflags = s->d_rflags;
  a.flag_phase = (int32_t)(s->step % 3);
  a.r_elo = s->r_elo;
  a.r_ehi = s->r_ehi;
  a.r_elo_s = s->r_elo_s;
  a.r_ehi_s = s->r_ehi_s;
  a.path_count = s->d_pathcnt;
}

const void *grid_maps_for(const pn_solver *s, int in) {
  return s->d_tmaps ? (const void *)((const unsigned char *)s->d_tmaps + (size_t)in * grid_tma_maps_bytes())
                    : nullptr;
}
template void grid_args<double>(pn_solver *, GridArgs<double> &);
template void grid_args<float>(pn_solver *, GridArgs<float> &);
template void grid_args<float2>(pn_solver *, GridArgs<float2> &);

namespace {

template <typename T>
void run(pn_solver *s, int32_t nsteps) {
  GridArgs<T> a;
  grid_args<T>(s, a);
  const int64_t nsig = (int64_t)s->src.size();
  int32_t done = 0;
  while (done < nsteps) {
    int32_t chunk = nsteps - done;
    ensure_signal_rows(s, chunk);
    if (nsig > 0 && !s->sig_hold)
      chunk = (int32_t)std::min<int64_t>(chunk, s->sig_step0 + s->sig_rows - s->step);
    for (int32_t k = 0; k < chunk; k++) {
      const int in = s->cur, out = s->cur ^ 1;
      for (int c = 0; c < 3; c++) {
        a.V_in[c] = (const T *)s->V[in][c];
        a.V_out[c] = (T *)s->V[out][c];
      }
      for (int c = 0; c < 6; c++) {
        a.S_in[c] = (const T *)s->S[in][c];
        a.S_out[c] = (T *)s->S[out][c];
      }
      a.tmaps = grid_maps_for(s, in);
      a.flag_phase = (int32_t)((s->step + k) % 3);
      a.sigval = nsig > 0 ? (const T *)s->d_sig + sig_row(s, k) * nsig : nullptr;
      a.rec = s->rec_count + k;  // sigval points at this step's row (stride 0)
      pn_solver::Mark m{};
      if (s->timing) {
        ck(cudaEventCreate(&m.a), "event");
        ck(cudaEventCreate(&m.b), "event");
        m.kind = 2;
        ck(cudaEventRecord(m.a, s->stream), "event");
      }
      cudaError_t e;
      if (a.tmaps) e = launch_grid_tma(&a, s->precision, s->sym, s->stream);
      else if constexpr (std::is_same<T, float2>::value) e = launch_grid_df64(a, s->sym, s->stream);
      else if constexpr (std::is_same<T, double>::value) e = launch_grid_f64(a, s->sym, s->stream);
      else e = launch_grid_f32(a, s->sym, s->stream);
      if (e == cudaSuccess && (a.n_copies > 0 || a.n_fix > 0)) e = launch_grid_split(&a, s->precision, s->stream);
      if (s->timing) {
        ck(cudaEventRecord(m.b, s->stream), "event");
        s->marks.push_back(m);
      }
      ck(e, "grid step launch");
      s->cur ^= 1;
      s->time += s->dt;  // HostRSGTDUT.hpp:166
    }
    s->step += chunk;
    s->rec_count += chunk;
    done += chunk;
  }
}

}  // namespace

void grid_run(pn_solver *s, int32_t nsteps) {
  if (s->is_df64()) run<float2>(s, nsteps);
  else if (s->esz == 8) run<double>(s, nsteps);
  else run<float>(s, nsteps);
}

}  // namespace pn
