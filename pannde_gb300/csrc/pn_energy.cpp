// pn_energy.cpp -- host side of the FP64 energy audit (pn_solver_energy).
//
// Tables are built on the first call and kept: the lumped nodal masses
// m_n = rho_n * dxn*dyn*dzn (rho_n = dt / coef_n, the reference's lumped nodal
// density, HostField.hpp:142-153; nodes of other partitions have coef 0 and
// no mass), the cell volumes dxc*dyc*dzc (RightHex.hpp:288-309 spacings), and
// one pseudo-inverse stiffness row per material.  The grid form lays masses
// out on its lattice node sites (void and padding sites: no mass) and uses one
// volume for every cell (void sites have the zero compliance row).
#include "pn_solver.hpp"
#include "rsg_energy.cuh"

namespace pn {

static void energy_tables(pn_solver *s) {
  const MeshTables &m = s->mesh;
  const int32_t nn = m.n_nodes, nc = m.n_cells;
  std::vector<double> mass((size_t)nn, 0.0);
  for (int32_t u = 0; u < nn; u++) {
    const double cf = s->mat.coef[u];
    if (cf != 0.0) mass[u] = s->dt / cf * m.dxn[u] * m.dyn[u] * m.dzn[u];
  }
  const int32_t rows = s->mat.n_mat + 1;  // the last row: void (zero)
  std::vector<double> comp((size_t)rows * 36, 0.0);
  for (int32_t r = 0; r < s->mat.n_mat; r++) pinv_sym6(&s->mat.c36[(size_t)r * 36], &comp[(size_t)r * 36]);
  s->d_ecomp = s->alloc<double>(comp.size() * sizeof(double));
  s->upload_raw(s->d_ecomp, comp.data(), comp.size() * sizeof(double));
  if (s->form == PN_FORM_GRID) {
    const GridMap &g = s->grid;
    std::vector<double> site((size_t)g.node_len(), 0.0);
    for (int32_t u = 0; u < nn; u++) site[(size_t)g.node_grid[u]] = mass[u];
    s->d_emass = s->alloc<double>(site.size() * sizeof(double));
    s->upload_raw(s->d_emass, site.data(), site.size() * sizeof(double));
    s->e_nodes = g.node_len();
    s->e_cells = g.cell_sites();
  } else {
    std::vector<double> vol((size_t)nc);
    for (int32_t c = 0; c < nc; c++) vol[c] = m.dxc[c] * m.dyc[c] * m.dzc[c];
    s->d_emass = s->alloc<double>(mass.size() * sizeof(double));
    s->upload_raw(s->d_emass, mass.data(), mass.size() * sizeof(double));
    s->d_evol = s->alloc<double>(vol.size() * sizeof(double));
    s->upload_raw(s->d_evol, vol.data(), vol.size() * sizeof(double));
    s->e_nodes = nn;
    s->e_cells = nc;
  }
  const int nb = std::max(energy_blocks(s->e_nodes), energy_blocks(s->e_cells));
  s->d_epart = s->alloc<double>((size_t)2 * nb * sizeof(double));
  ck(cudaStreamSynchronize(s->stream), "energy tables");
}

void energy(pn_solver *s, double &kinetic, double &strain) {
  if (!s->d_epart) energy_tables(s);
  const int nbn = energy_blocks(s->e_nodes), nbc = energy_blocks(s->e_cells);
  const int b = s->form == PN_FORM_GRID ? s->cur : 0;
  const void *V[3] = {s->V[b][0], s->V[b][1], s->V[b][2]};
  const void *S[6] = {s->S[b][0], s->S[b][1], s->S[b][2], s->S[b][3], s->S[b][4], s->S[b][5]};
  const int nbmax = std::max(nbn, nbc);
  ck(launch_energy_nodes(s->precision, V, s->d_emass, s->e_nodes, s->d_epart, nbn, s->stream), "energy nodes");
  const bool grid = s->form == PN_FORM_GRID;
  const double vol = grid ? s->mesh.hx * s->mesh.hy * s->mesh.hz : 0.0;
  ck(launch_energy_cells(s->precision, S, grid ? (const void *)s->d_gmat : (const void *)s->d_mat, grid,
                         s->d_ecomp, grid ? nullptr : s->d_evol, vol, s->e_cells, s->d_epart + nbmax, nbc,
                         s->stream),
     "energy cells");
  std::vector<double> part((size_t)2 * nbmax);
  ck(cudaMemcpyAsync(part.data(), s->d_epart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream),
     "energy partials");
  ck(cudaStreamSynchronize(s->stream), "energy");
  kinetic = 0.0;
  strain = 0.0;
  for (int k = 0; k < nbn; k++) kinetic += part[(size_t)k];
  for (int k = 0; k < nbc; k++) strain += part[(size_t)nbmax + k];
}

}  // namespace pn
