/*
 * pn_oracle.c -- CPU oracle for the RSG elastodynamic leapfrog.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (nasa/PanNDE HostSolver), used to check the CUDA path and as the
 * timed CPU baseline.  The product never links or calls it.
 *
 * It follows the reference's operation order exactly and must be compiled
 * with -ffp-contract=off (no FMA contraction), so its results are
 * bit-identical to the reference HostRSGTDUT / HostUTModel on the same
 * inputs.  That claim is pinned by tests/golden (fixtures produced by the
 * reference itself compiled from its own headers, see oracle/ref_driver.cpp).
 *
 * Reference map (paths inside the PanNDE project):
 *   solve loop ................ HostSolver/include/HostRSGTDUT.hpp:162-169,
 *                               HostUTModel.hpp:186-193
 *   updateVsAtNode ............ HostRSGTDUT.hpp:338-362, HostUTModel.hpp:356-379
 *   evalXds / cellcenter ...... HostRSGTDUT.hpp:387-428
 *   updateTsAtCell ............ HostRSGTDUT.hpp:278-293, HostUTModel.hpp:270-286
 *   evalMoments ............... HostUTModel.hpp:296-311
 *   DD*_cc / DD*_nc ........... HostSolver/include/internal/RightHex.hpp:100-192,225-247
 *   nodePrep / cellPrep ....... RightHex.hpp:253-309
 *   Field::atNode / atCell .... HostData/include/HostField.hpp:110-153
 *   buildLinks ................ HostData/include/HexMesh.hpp:300-313
 *   HostNormalXDZ::evalAt ..... Stubs/include/HostNormalXDZ.hpp:117-123,174-177
 *   HostUnivariate::evalAt .... HostData/include/HostUnivariate.hpp:109-142
 *
 * The node and cell loops, the spacing and coefficient setup and the source
 * hit lists are independent per element, so they run under OpenMP when
 * compiled with -fopenmp; the hit lists are built in two passes (count,
 * prefix sum, fill) and the spacing check reports the first bad node in node
 * order, so results and errors do not depend on the thread count.
 * buildLinks' "a later cell overwrites an earlier one's link" is kept as an
 * atomic maximum of the cell index per slot.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pannde_gb300.h"

#define OR_MAXMSG 256
static char or_msg[OR_MAXMSG];

const char *pn_oracle_last_error(void) { return or_msg; }

static int or_fail(int code, const char *msg) {
  snprintf(or_msg, OR_MAXMSG, "%s", msg);
  return code;
}

/* ---- mesh links: HexMesh::buildLinks (HexMesh.hpp:300-313) ------------- */
/* Later cells win: every slot ends up holding the highest cell index that
   names it, which lets the cells be linked in parallel (an atomic maximum). */
static int build_links(const pn_mesh *m, int32_t *ncc) {
  const int64_t nh = (int64_t)m->n_cells * 8;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int64_t k = 0; k < nh; k++) bad |= m->hexes[k] < 0 || m->hexes[k] >= m->n_nodes;
  if (bad) return or_fail(PN_ERR_RANGE, "invalid node id");
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)m->n_nodes * 8; k++) ncc[k] = -1;
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < m->n_cells; c++) {
    for (int k = 0; k < 8; k++) {
      int32_t *slot = &ncc[(int64_t)m->hexes[(int64_t)c * 8 + k] * 8 + (k ^ 6)];
      int32_t cur = __atomic_load_n(slot, __ATOMIC_RELAXED);
      while (cur < c && !__atomic_compare_exchange_n(slot, &cur, c, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
      }
    }
  }
  return PN_OK;
}

/* ---- RightHex::cellPrep (RightHex.hpp:253-264) ---------------------------*/
static void cell_prep(const pn_mesh *m, double *dxc, double *dyc, double *dzc) {
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < m->n_cells; c++) {
    int32_t a = m->hexes[(int64_t)c * 8 + 0], b = m->hexes[(int64_t)c * 8 + 6];
    dxc[c] = m->x[b] - m->x[a];
    dyc[c] = m->y[b] - m->y[a];
    dzc[c] = m->z[b] - m->z[a];
  }
}

/* ---- RightHex::nodePrep (RightHex.hpp:272-309) ---------------------------*/
static int node_prep(const pn_mesh *m, const int32_t *ncc, double *dxn, double *dyn,
                     double *dzn) {
  /* every node independently; the reference throws at the first node (in
     node order) whose spacing is not positive, checking DX, DY, DZ in turn */
  int32_t first_bad = m->n_nodes;
#pragma omp parallel for schedule(static) reduction(min : first_bad)
  for (int32_t n = 0; n < m->n_nodes; n++) {
    double node[3] = {m->x[n], m->y[n], m->z[n]};
    double lo[3] = {node[0], node[1], node[2]};
    double hi[3] = {node[0], node[1], node[2]};
    for (int kb = 0; kb < 8; kb++) {
      int32_t c = ncc[(int64_t)n * 8 + kb];
      if (c == -1) continue;
      for (int kbb = 0; kbb < 8; kbb++) {
        int32_t q = m->hexes[(int64_t)c * 8 + kbb];
        double pt[3] = {m->x[q], m->y[q], m->z[q]};
        for (int kd = 0; kd < 3; kd++) {
          lo[kd] = (pt[kd] < lo[kd]) ? pt[kd] : lo[kd]; /* std::min(lo,pt) */
          hi[kd] = (hi[kd] < pt[kd]) ? pt[kd] : hi[kd]; /* std::max(hi,pt) */
        }
      }
    }
    for (int kd = 0; kd < 3; kd++) {
      if (lo[kd] == node[kd]) lo[kd] = 2. * node[kd] - hi[kd];
      if (hi[kd] == node[kd]) hi[kd] = 2. * node[kd] - lo[kd];
    }
    dxn[n] = 0.5 * (hi[0] - lo[0]);
    dyn[n] = 0.5 * (hi[1] - lo[1]);
    dzn[n] = 0.5 * (hi[2] - lo[2]);
    if ((0 >= dxn[n] || 0 >= dyn[n] || 0 >= dzn[n]) && n < first_bad) first_bad = n;
  }
  if (first_bad < m->n_nodes) {
    const int32_t n = first_bad;
    if (0 >= dxn[n]) return or_fail(PN_ERR_SPACING, "DX");
    if (0 >= dyn[n]) return or_fail(PN_ERR_SPACING, "DY");
    return or_fail(PN_ERR_SPACING, "DZ");
  }
  return PN_OK;
}

/* ---- HostField::atCell / atNode (HostField.hpp:121-153) ------------------*/
static double field_at_cell(const pn_mesh *m, const pn_field *f, int32_t c) {
  if (f->type == PN_FIELD_NODE) {
    double v = 0.0;
    for (int k = 0; k < 8; k++) v += f->data[m->hexes[(int64_t)c * 8 + k]];
    return v / 8.0;
  }
  return (f->type == PN_FIELD_CONSTANT) ? f->data[0] : f->data[c];
}

static double field_at_node(const pn_field *f, const int32_t *ncc, int32_t n) {
  if (f->type == PN_FIELD_NODE) return f->data[n];
  double v = 0.0;
  for (int k = 0; k < 8; k++) {
    int32_t c = ncc[(int64_t)n * 8 + k];
    v += (c == -1) ? 0. : ((f->type == PN_FIELD_CONSTANT) ? f->data[0] : f->data[c]);
  }
  return v / 8.0;
}

/* Voigt (i,j) -> index into the 21 unique entries (upper triangle, row order). */
static int cij_index(int i, int j) {
  if (i > j) { int t = i; i = j; j = t; }
  return i * 6 - i * (i - 1) / 2 + (j - i);
}

/* ---- HostUnivariate (HostUnivariate.hpp:75-142) --------------------------*/
typedef struct { int32_t n; double *t, *v; } or_series;

static int series_build(const pn_signal *sig, or_series *s) {
  s->n = 0; s->t = s->v = NULL;
  if (sig->n <= 0) return or_fail(PN_ERR_RUNTIME, "empty signal");
  s->t = (double *)malloc(sizeof(double) * sig->n);
  s->v = (double *)malloc(sizeof(double) * sig->n);
  if (!s->t || !s->v) return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  /* std::map<double,double>::emplace: sorted by time, first value kept on
     duplicate times.  Insertion sort keeps it simple (signals are short). */
  for (int32_t k = 0; k < sig->n; k++) {
    double tk = sig->t[k], vk = sig->v[k];
    int32_t pos = 0;
    while (pos < s->n && s->t[pos] < tk) pos++;
    if (pos < s->n && s->t[pos] == tk) continue;
    memmove(s->t + pos + 1, s->t + pos, sizeof(double) * (s->n - pos));
    memmove(s->v + pos + 1, s->v + pos, sizeof(double) * (s->n - pos));
    s->t[pos] = tk; s->v[pos] = vk; s->n++;
  }
  return PN_OK;
}

static double series_eval(const or_series *s, double t) {
  if (t < s->t[s->n - 1]) {
    for (int32_t k = 0; k < s->n; k++) {
      if (t < s->t[k]) {
        /* the reference takes std::prev(begin) when t precedes the first
           sample (undefined); the oracle holds the first value there */
        if (k == 0) return s->v[0];
        double Dt = s->t[k] - s->t[k - 1];
        double Dv = s->v[k] - s->v[k - 1];
        return (Dv / Dt) * (t - s->t[k - 1]) + s->v[k - 1];
      }
    }
    return 0.;
  }
  return s->v[s->n - 1];
}

/* ---- HostNormalXDZ window (HostNormalXDZ.hpp:117-123,174-177) ------------*/
static int window_at(const pn_window_source *w, const double p[3]) {
  double res = 0.0;
  for (int k = 0; k < 3; k++) {
    double d = p[k] - w->center[k];
    res += d * d;
  }
  double dist = sqrt(res);
  double distz = fabs(p[2] - w->center[2]);
  return (distz <= 0.75 * w->ds) && (dist < w->radius) && (dist >= 0.);
}

/* ---- HostRSGTDUT::cellcenter (HostRSGTDUT.hpp:419-428) -------------------*/
static void cell_center(const pn_mesh *m, int32_t c, double cc[3]) {
  cc[0] = cc[1] = cc[2] = 0.;
  for (int kb = 0; kb < 8; kb++) {
    int32_t q = m->hexes[(int64_t)c * 8 + kb];
    cc[0] += 0.125 * m->x[q];
    cc[1] += 0.125 * m->y[q];
    cc[2] += 0.125 * m->z[q];
  }
}

/* Sparse list of static window hits.  The window does not depend on time and
   evalAt = signal(t) * window with window in {0,1}, so a source term equals
   the in-order sum of 0.125*signal(t) over the (incident element, source)
   pairs inside the window; pairs outside add 0.0, which changes no sum. */
typedef struct {
  int64_t *start;   /* [n_elems*ncomp + 1] offsets into sig */
  int32_t *sig;     /* source index per hit, in reference order */
} or_hits;

static void hits_free(or_hits *h) { free(h->start); free(h->sig); h->start = NULL; h->sig = NULL; }

/* Sources grouped the way the reference stores them: xducers[g][3] and
   moment_excitation[g][6], each slot holding at most one source. */
typedef struct {
  int32_t ngroups;
  int32_t *slot;  /* [ngroups*ncomp] source index or -1 */
} or_groups;

static int group_sources(const pn_window_source *src, int32_t nsrc, int kind, int ncomp,
                         or_groups *g) {
  int32_t maxg = -1;
  for (int32_t i = 0; i < nsrc; i++) {
    if (src[i].kind != kind) continue;
    if (src[i].group < 0) return or_fail(PN_ERR_INVALID, "negative source group");
    if (src[i].component < 0 || src[i].component >= ncomp)
      return or_fail(PN_ERR_INVALID, "source component out of range");
    if (src[i].group > maxg) maxg = src[i].group;
  }
  g->ngroups = maxg + 1;
  g->slot = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->ngroups > 0 ? g->ngroups : 1) * ncomp);
  if (!g->slot) return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  for (int32_t k = 0; k < g->ngroups * ncomp; k++) g->slot[k] = -1;
  for (int32_t i = 0; i < nsrc; i++) {
    if (src[i].kind != kind) continue;
    int32_t *s = &g->slot[src[i].group * ncomp + src[i].component];
    if (*s != -1) return or_fail(PN_ERR_INVALID, "two sources in one group slot");
    *s = i;
  }
  return PN_OK;
}

/* the hits of node n, direction dir, in the loop order of evalXds (kb, then
   xd); written to out when given; returns their number */
static int32_t force_hits_at(const pn_mesh *m, const int32_t *ncc, const pn_window_source *src,
                             const or_groups *g, int32_t n, int dir, int32_t *out) {
  int32_t cnt = 0;
  for (int kb = 0; kb < 8; kb++) {
    int32_t c = ncc[(int64_t)n * 8 + kb];
    if (c == -1) continue;
    double cc[3];
    cell_center(m, c, cc);
    for (int32_t gi = 0; gi < g->ngroups; gi++) {
      int32_t si = g->slot[gi * 3 + dir];
      if (si < 0 || !window_at(&src[si], cc)) continue;
      if (out) out[cnt] = si;
      cnt++;
    }
  }
  return cnt;
}

/* the hits of cell c, Voigt component comp, in the loop order of evalMoments */
static int32_t moment_hits_at(const pn_mesh *m, const pn_window_source *src, const or_groups *g,
                              int32_t c, int comp, int32_t *out) {
  int32_t cnt = 0;
  for (int kb = 0; kb < 8; kb++) {
    int32_t q = m->hexes[(int64_t)c * 8 + kb];
    double r[3] = {m->x[q], m->y[q], m->z[q]};
    for (int32_t gi = 0; gi < g->ngroups; gi++) {
      int32_t si = g->slot[gi * 6 + comp];
      if (si < 0 || !window_at(&src[si], r)) continue;
      if (out) out[cnt] = si;
      cnt++;
    }
  }
  return cnt;
}

/* Hit lists per element and component, built in two passes over the
   elements in parallel (count, prefix sum, fill): every element's hits keep
   the reference's order, and the list is the same as a serial build's. */
static int build_hits(const pn_mesh *m, const int32_t *ncc, const pn_window_source *src,
                      const or_groups *g, int forces, or_hits *h) {
  const int ncomp = forces ? 3 : 6;
  const int32_t nel = forces ? m->n_nodes : m->n_cells;
  const int64_t ne = (int64_t)nel * ncomp;
  h->start = (int64_t *)calloc((size_t)ne + 1, sizeof(int64_t));
  if (!h->start) return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  if (g->ngroups > 0) {
#pragma omp parallel for schedule(static)
    for (int32_t e = 0; e < nel; e++)
      for (int k = 0; k < ncomp; k++)
        h->start[(int64_t)e * ncomp + k + 1] =
            forces ? force_hits_at(m, ncc, src, g, e, k, NULL) : moment_hits_at(m, src, g, e, k, NULL);
    for (int64_t q = 0; q < ne; q++) h->start[q + 1] += h->start[q];
  }
  h->sig = (int32_t *)malloc(sizeof(int32_t) * (size_t)(h->start[ne] > 0 ? h->start[ne] : 1));
  if (!h->sig) return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  if (g->ngroups > 0 && h->start[ne] > 0) {
#pragma omp parallel for schedule(static)
    for (int32_t e = 0; e < nel; e++)
      for (int k = 0; k < ncomp; k++) {
        int32_t *out = h->sig + h->start[(int64_t)e * ncomp + k];
        if (forces) force_hits_at(m, ncc, src, g, e, k, out);
        else moment_hits_at(m, src, g, e, k, out);
      }
  }
  return PN_OK;
}

/* force hits per node and direction: loop order of evalXds (kb, then xd). */
static int force_hits(const pn_mesh *m, const int32_t *ncc, const pn_window_source *src,
                      const or_groups *g, or_hits *h) {
  return build_hits(m, ncc, src, g, 1, h);
}

/* moment hits per cell and Voigt component: loop order of evalMoments. */
static int moment_hits(const pn_mesh *m, const pn_window_source *src, const or_groups *g,
                       or_hits *h) {
  return build_hits(m, NULL, src, g, 0, h);
}

/* ---- operators (RightHex.hpp:100-192, 225-247) ---------------------------*/
/* fwd/bwd corner (or slot) sets per axis */
static const int FWD[3][4] = {{1, 2, 5, 6}, {2, 3, 6, 7}, {4, 5, 6, 7}};
static const int BWD[3][4] = {{0, 3, 4, 7}, {0, 1, 4, 5}, {0, 1, 2, 3}};

static inline double dd_cc(const int32_t *box, const double *f, int axis, double d) {
  double value = 0.0;
  for (int k = 0; k < 4; k++) value += (f[box[FWD[axis][k]]] - f[box[BWD[axis][k]]]);
  return (value * 0.25 / d);
}

static inline double dd_nc(const int32_t *box, const double *f, int axis, double d) {
  double value = 0.0;
  for (int k = 0; k < 4; k++) {
    int32_t a = box[FWD[axis][k]], b = box[BWD[axis][k]];
    value += (((-1 == a) ? 0. : f[a]) - ((-1 == b) ? 0. : f[b]));
  }
  return (value * 0.25 / d);
}

/* ---- the solver ----------------------------------------------------------*/
typedef struct {
  const pn_mesh *m;
  int32_t *ncc;
  double *dxc, *dyc, *dzc, *dxn, *dyn, *dzn;
  double *coef;       /* dt / density->atNode(n) */
  double *cij;        /* [n_cells][21] atCell values */
  int32_t nsrc;
  or_series *series;  /* per source */
  double *sigval;     /* per source, value at the current time */
  or_hits fh, mh;
  int has_moments;
} or_model;

static void model_free(or_model *M) {
  free(M->ncc); free(M->dxc); free(M->dyc); free(M->dzc);
  free(M->dxn); free(M->dyn); free(M->dzn); free(M->coef); free(M->cij);
  if (M->series) {
    for (int32_t i = 0; i < M->nsrc; i++) { free(M->series[i].t); free(M->series[i].v); }
  }
  free(M->series); free(M->sigval);
  hits_free(&M->fh); hits_free(&M->mh);
}

static int check_field(const pn_field *f, const char *what) {
  if (!f->data) return or_fail(PN_ERR_INVALID, what);
  if (f->type < 0 || f->type > 2) return or_fail(PN_ERR_INVALID, what);
  return PN_OK;
}

static int model_setup(or_model *M, const pn_mesh *m, const pn_material *mat, double dt,
                       const pn_window_source *src, int32_t nsrc) {
  memset(M, 0, sizeof(*M));
  M->m = m;
  if (!m || !mat || m->n_nodes < 0 || m->n_cells < 0) return or_fail(PN_ERR_INVALID, "mesh");
  if ((m->n_nodes > 0 && (!m->x || !m->y || !m->z)) || (m->n_cells > 0 && !m->hexes))
    return or_fail(PN_ERR_INVALID, "mesh arrays");
  int rc = check_field(&mat->density, "density field");
  for (int k = 0; k < 21 && rc == PN_OK; k++) rc = check_field(&mat->cij[k], "stiffness field");
  if (rc) return rc;
  size_t nn = (size_t)m->n_nodes, nc = (size_t)m->n_cells;
  M->ncc = (int32_t *)malloc(sizeof(int32_t) * (nn * 8 + 1));
  M->dxc = (double *)malloc(sizeof(double) * (nc + 1));
  M->dyc = (double *)malloc(sizeof(double) * (nc + 1));
  M->dzc = (double *)malloc(sizeof(double) * (nc + 1));
  M->dxn = (double *)malloc(sizeof(double) * (nn + 1));
  M->dyn = (double *)malloc(sizeof(double) * (nn + 1));
  M->dzn = (double *)malloc(sizeof(double) * (nn + 1));
  M->coef = (double *)malloc(sizeof(double) * (nn + 1));
  M->cij = (double *)malloc(sizeof(double) * (nc * 21 + 1));
  if (!M->ncc || !M->dxc || !M->dyc || !M->dzc || !M->dxn || !M->dyn || !M->dzn || !M->coef ||
      !M->cij)
    return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  if ((rc = build_links(m, M->ncc))) return rc;
  /* the reference constructor order: setupProperties, setupSolution,
     setupComms, then RightHex (nodePrep before cellPrep) */
  if ((rc = node_prep(m, M->ncc, M->dxn, M->dyn, M->dzn))) return rc;
  cell_prep(m, M->dxc, M->dyc, M->dzc);
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < m->n_nodes; n++) M->coef[n] = dt / field_at_node(&mat->density, M->ncc, n);
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < m->n_cells; c++)
    for (int k = 0; k < 21; k++) M->cij[(size_t)c * 21 + k] = field_at_cell(m, &mat->cij[k], c);

  M->nsrc = nsrc;
  M->series = (or_series *)calloc((size_t)(nsrc > 0 ? nsrc : 1), sizeof(or_series));
  M->sigval = (double *)calloc((size_t)(nsrc > 0 ? nsrc : 1), sizeof(double));
  if (!M->series || !M->sigval) return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  for (int32_t i = 0; i < nsrc; i++) {
    if (src[i].kind != PN_SOURCE_FORCE && src[i].kind != PN_SOURCE_MOMENT)
      return or_fail(PN_ERR_INVALID, "unknown source kind");
    if (!src[i].signal.t || !src[i].signal.v) return or_fail(PN_ERR_INVALID, "signal arrays");
    if ((rc = series_build(&src[i].signal, &M->series[i]))) return rc;
  }
  or_groups gf = {0, NULL}, gm = {0, NULL};
  if ((rc = group_sources(src, nsrc, PN_SOURCE_FORCE, 3, &gf))) { free(gf.slot); return rc; }
  if ((rc = group_sources(src, nsrc, PN_SOURCE_MOMENT, 6, &gm))) { free(gf.slot); free(gm.slot); return rc; }
  M->has_moments = gm.ngroups > 0;
  rc = force_hits(m, M->ncc, src, &gf, &M->fh);
  if (!rc) rc = moment_hits(m, src, &gm, &M->mh);
  free(gf.slot); free(gm.slot);
  return rc;
}

static void update_vs(or_model *M, double *const *V, double *const *S) {
  const pn_mesh *m = M->m;
  int32_t own = m->partition_id;
#pragma omp parallel for schedule(static)
  for (int32_t n = 0; n < m->n_nodes; n++) {
    if (m->node_owner && m->node_owner[n] != own) continue;
    const int32_t *box = &M->ncc[(int64_t)n * 8];
    double xd[3];
    for (int dir = 0; dir < 3; dir++) {
      double r = 0.;
      for (int64_t h = M->fh.start[(int64_t)n * 3 + dir]; h < M->fh.start[(int64_t)n * 3 + dir + 1]; h++)
        r += 0.125 * M->sigval[M->fh.sig[h]];
      xd[dir] = r;
    }
    double c = M->coef[n];
    /* HostRSGTDUT.hpp:343-360: x uses S0,S5,S4; y S5,S1,S3; z S4,S3,S2 */
    V[0][n] += c * (dd_nc(box, S[0], 0, M->dxn[n]) + dd_nc(box, S[5], 1, M->dyn[n]) +
                    dd_nc(box, S[4], 2, M->dzn[n]) + xd[0]);
    V[1][n] += c * (dd_nc(box, S[5], 0, M->dxn[n]) + dd_nc(box, S[1], 1, M->dyn[n]) +
                    dd_nc(box, S[3], 2, M->dzn[n]) + xd[1]);
    V[2][n] += c * (dd_nc(box, S[4], 0, M->dxn[n]) + dd_nc(box, S[3], 1, M->dyn[n]) +
                    dd_nc(box, S[2], 2, M->dzn[n]) + xd[2]);
  }
}

static void update_ts(or_model *M, double *const *V, double *const *S, double dt) {
  const pn_mesh *m = M->m;
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < m->n_cells; c++) {
    const int32_t *box = &m->hexes[(int64_t)c * 8];
    double d[3][3];
    for (int k1 = 0; k1 < 3; k1++) {
      d[0][k1] = dd_cc(box, V[k1], 0, M->dxc[c]);
      d[1][k1] = dd_cc(box, V[k1], 1, M->dyc[c]);
      d[2][k1] = dd_cc(box, V[k1], 2, M->dzc[c]);
    }
    const double *C = &M->cij[(size_t)c * 21];
    for (int ks = 0; ks < 6; ks++) {
      double acc = C[cij_index(ks, 0)] * d[0][0] + C[cij_index(ks, 1)] * d[1][1] +
                   C[cij_index(ks, 2)] * d[2][2] + C[cij_index(ks, 3)] * (d[1][2] + d[2][1]) +
                   C[cij_index(ks, 4)] * (d[0][2] + d[2][0]) +
                   C[cij_index(ks, 5)] * (d[0][1] + d[1][0]);
      if (M->has_moments) {
        double r = 0.;
        int64_t e = (int64_t)c * 6 + ks;
        for (int64_t h = M->mh.start[e]; h < M->mh.start[e + 1]; h++)
          r += 0.125 * M->sigval[M->mh.sig[h]];
        acc = acc + r;
      }
      S[ks][c] += dt * acc;
    }
  }
}

/* Run nsteps of the leapfrog from state (V0,S0) (NULL = zero) and return the
   final state, the time and per-step sensor traces [nsteps][nsens][3].
   has_moment_term selects HostUTModel's stress update (which always adds the
   moment sum) over HostRSGTDUT's; both agree whenever no moment source is
   given. */
int pn_oracle_run(const pn_mesh *m, const pn_material *mat, double dt, const double *const *V0,
                  const double *const *S0, const pn_window_source *src, int32_t nsrc,
                  int32_t nsteps, const int32_t *sensors, int32_t nsens, double *traces,
                  double *const *Vout, double *const *Sout, double *time_out) {
  or_msg[0] = 0;
  if (nsteps < 0 || nsrc < 0 || nsens < 0 || (nsrc > 0 && !src) || (nsens > 0 && (!sensors || !traces)))
    return or_fail(PN_ERR_INVALID, "arguments");
  if (!Vout || !Sout) return or_fail(PN_ERR_INVALID, "output arrays");
  for (int k = 0; k < 3; k++) if (!Vout[k]) return or_fail(PN_ERR_INVALID, "output arrays");
  for (int k = 0; k < 6; k++) if (!Sout[k]) return or_fail(PN_ERR_INVALID, "output arrays");
  or_model M;
  int rc = model_setup(&M, m, mat, dt, src, nsrc);
  if (rc) { model_free(&M); return rc; }
  for (int32_t i = 0; i < nsens; i++)
    if (sensors[i] < 0 || sensors[i] >= m->n_nodes) { model_free(&M); return or_fail(PN_ERR_RANGE, "sensor node"); }
  for (int k = 0; k < 3; k++) {
    if (V0 && V0[k]) memcpy(Vout[k], V0[k], sizeof(double) * (size_t)m->n_nodes);
    else memset(Vout[k], 0, sizeof(double) * (size_t)m->n_nodes);
  }
  for (int k = 0; k < 6; k++) {
    if (S0 && S0[k]) memcpy(Sout[k], S0[k], sizeof(double) * (size_t)m->n_cells);
    else memset(Sout[k], 0, sizeof(double) * (size_t)m->n_cells);
  }
  double time = 0.;
  for (int32_t step = 0; step < nsteps; step++) {
    for (int32_t i = 0; i < nsrc; i++) M.sigval[i] = series_eval(&M.series[i], time);
    update_vs(&M, Vout, Sout);
    update_ts(&M, Vout, Sout, dt);
    time += dt;
    for (int32_t i = 0; i < nsens; i++)
      for (int d = 0; d < 3; d++)
        traces[((int64_t)step * nsens + i) * 3 + d] = Vout[d][sensors[i]];
  }
  if (time_out) *time_out = time;
  model_free(&M);
  return PN_OK;
}

/* ---- operator-level entry points for the RightHex known-answer tests ----*/

/* DD{x,y,z}_cc of a node field at one cell (RightHex.hpp:100-141). */
int pn_oracle_dd_cc(const pn_mesh *m, const double *node_field, int32_t cell, int32_t axis,
                    double *out) {
  if (!m || cell < 0 || cell >= m->n_cells || axis < 0 || axis > 2 || !out)
    return or_fail(PN_ERR_INVALID, "arguments");
  const int32_t *box = &m->hexes[(int64_t)cell * 8];
  int32_t a = box[0], b = box[6];
  double d = axis == 0 ? m->x[b] - m->x[a] : axis == 1 ? m->y[b] - m->y[a] : m->z[b] - m->z[a];
  *out = dd_cc(box, node_field, axis, d);
  return PN_OK;
}

/* DD{x,y,z}_nc of a cell field at one node (RightHex.hpp:151-192) and the
   node spacings getNodeD{x,y,z} (RightHex.hpp:199-215). */
int pn_oracle_dd_nc(const pn_mesh *m, const double *cell_field, int32_t node, int32_t axis,
                    double *out, double *spacing_out) {
  if (!m || node < 0 || node >= m->n_nodes || axis < 0 || axis > 2 || !out)
    return or_fail(PN_ERR_INVALID, "arguments");
  size_t nn = (size_t)m->n_nodes;
  int32_t *ncc = (int32_t *)malloc(sizeof(int32_t) * nn * 8);
  double *d3 = (double *)malloc(sizeof(double) * nn * 3);
  if (!ncc || !d3) { free(ncc); free(d3); return or_fail(PN_ERR_ALLOC, "oracle: out of memory"); }
  int rc = build_links(m, ncc);
  if (!rc) rc = node_prep(m, ncc, d3, d3 + nn, d3 + 2 * nn);
  if (!rc) {
    double d = d3[axis * nn + node];
    *out = dd_nc(&ncc[(int64_t)node * 8], cell_field, axis, d);
    if (spacing_out) *spacing_out = d;
  }
  free(ncc); free(d3);
  return rc;
}

/* The nodal force weights the reference applies: for node n and direction
   dir, the number of (incident cell, source) pairs in the window times
   0.125, summed over sources of that direction.  Used to check the device
   setup's window tables. */
int pn_oracle_force_weights(const pn_mesh *m, const pn_window_source *src, int32_t nsrc,
                            double *w /* [n_nodes][3] */) {
  int32_t *ncc = (int32_t *)malloc(sizeof(int32_t) * ((size_t)m->n_nodes * 8 + 1));
  if (!ncc) return or_fail(PN_ERR_ALLOC, "oracle: out of memory");
  int rc = build_links(m, ncc);
  or_groups g = {0, NULL};
  or_hits h = {NULL, NULL};
  if (!rc) rc = group_sources(src, nsrc, PN_SOURCE_FORCE, 3, &g);
  if (!rc) rc = force_hits(m, ncc, src, &g, &h);
  if (!rc) {
    for (int64_t e = 0; e < (int64_t)m->n_nodes * 3; e++)
      w[e] = 0.125 * (double)(h.start[e + 1] - h.start[e]);
  }
  hits_free(&h); free(g.slot); free(ncc);
  return rc;
}

/* HostUnivariate::evalAt at n times (HostUnivariateTests known answers). */
int pn_oracle_signal_eval(const pn_signal *sig, const double *t, int32_t n, double *out) {
  or_series s;
  int rc = series_build(sig, &s);
  if (!rc)
    for (int32_t i = 0; i < n; i++) out[i] = series_eval(&s, t[i]);
  free(s.t);
  free(s.v);
  return rc;
}

/* HostNormalXDZ::evalAt(x,y,z,t) = signal(t) * window (HostNormalXDZTests). */
int pn_oracle_window_eval(const pn_window_source *w, const double *args4, double *out) {
  or_series s;
  int rc = series_build(&w->signal, &s);
  if (!rc) *out = series_eval(&s, args4[3]) * (double)window_at(w, args4);
  free(s.t);
  free(s.v);
  return rc;
}
