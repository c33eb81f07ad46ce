/* The C example of the integration notes (section 3), made runnable: a
   4 x 3 x 2 voxel plate, one transducer, two sensors, ten steps.  Exit 0 after
   a solve; 3 when no CUDA device can be used (the message printed). */
#include <stdio.h>

#include "pannde_gb300.h"

int main(void) {
  enum { NX = 4, NY = 3, NZ = 2 };
  static double x[(NX + 1) * (NY + 1) * (NZ + 1)], y[(NX + 1) * (NY + 1) * (NZ + 1)],
      z[(NX + 1) * (NY + 1) * (NZ + 1)];
  static int32_t hexes[NX * NY * NZ * 8], cell_material[NX * NY * NZ];
  const double h = 1e-4;
  int32_t n_nodes = 0, n_cells = 0;
  for (int k = 0; k <= NZ; k++)
    for (int j = 0; j <= NY; j++)
      for (int i = 0; i <= NX; i++, n_nodes++) {
        x[n_nodes] = i * h;
        y[n_nodes] = j * h;
        z[n_nodes] = k * h;
      }
#define NODE(i, j, k) (((k) * (NY + 1) + (j)) * (NX + 1) + (i))
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++, n_cells++) {
        const int32_t box[8] = {NODE(i, j, k),         NODE(i + 1, j, k),     NODE(i + 1, j + 1, k),
                                NODE(i, j + 1, k),     NODE(i, j, k + 1),     NODE(i + 1, j, k + 1),
                                NODE(i + 1, j + 1, k + 1), NODE(i, j + 1, k + 1)};
        for (int q = 0; q < 8; q++) hexes[n_cells * 8 + q] = box[q];
        cell_material[n_cells] = 0;
      }
  /* isotropic aluminium: lambda 51.08 GPa, mu 26.32 GPa, in the 21-entry order */
  const double l = 51.08e9, m = 26.32e9;
  const double cij21[21] = {l + 2 * m, l, l, 0, 0, 0, l + 2 * m, l, 0, 0, 0, l + 2 * m, 0, 0, 0, m, 0, 0, m, 0, m};
  const double density[1] = {2700.0};
  const double times[3] = {0.0, 1e-8, 1e-6}, values[3] = {0.0, 1.0, 0.0};
  const int32_t sensor_nodes[2] = {NODE(2, 1, 2), NODE(0, 0, 2)};
  double V0[3][(NX + 1) * (NY + 1) * (NZ + 1)], S0[6][NX * NY * NZ];
  double *V[3] = {V0[0], V0[1], V0[2]}, *S[6] = {S0[0], S0[1], S0[2], S0[3], S0[4], S0[5]};
  static double traces[10 * 2 * 3];

  pn_mesh mesh = {n_nodes, n_cells, x, y, z, hexes, NULL, 0};
  pn_material_table mat = {1, density, cij21, cell_material};
  pn_solver *s = NULL;
  if (pn_solver_create_indexed(&mesh, &mat, 5e-9, PN_PREC_DF64, &s) != PN_OK) {
    printf("create: %s\n", pn_last_error());
    return 3;
  }
  pn_window_source xd = {PN_SOURCE_FORCE, 0, 2, {2 * h, 1.5 * h, 2 * h}, 2 * h, h, {3, times, values}};
  double t = 0.0;
  int64_t nrec = 0;
  int rc = pn_solver_add_sources(s, &xd, 1);
  if (rc == PN_OK) rc = pn_solver_set_sensors(s, sensor_nodes, 2, 10);
  if (rc == PN_OK) rc = pn_solver_solve(s, 10, &t); /* enqueue */
  if (rc == PN_OK) rc = pn_solver_get_state(s, V, S);
  if (rc == PN_OK) rc = pn_solver_get_traces(s, traces, 10, &nrec);
  if (rc != PN_OK) printf("error %d: %s\n", rc, pn_last_error());
  else printf("t = %.6e s, %lld records, Vz at sensor 0 = %.6e\n", t, (long long)nrec, traces[9 * 6 + 2]);
  pn_solver_destroy(s);
  return rc == PN_OK ? 0 : 1;
}
