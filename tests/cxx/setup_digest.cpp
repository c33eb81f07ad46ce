// setup_digest.cpp -- builds every host table of pn_setup.cpp (links,
// spacings, material tables, voxel-grid map with split sites, source
// entries) for one mesh and returns a 64-bit FNV-1a digest of each array, so
// that a test can check the tables bit for bit across thread counts.  Compiled by
// tests/test_setup_threads_cpu.py together with pn_setup.cpp.
#include <cstdio>

#include "pn_setup.hpp"

namespace {
uint64_t fnv(const void *p, size_t n, uint64_t h = 1469598103934665603ull) {
  const unsigned char *b = (const unsigned char *)p;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}
template <class V>
uint64_t digest_of(const V &v) {
  return fnv(v.data(), v.size() * sizeof(v[0]), 1469598103934665603ull ^ v.size());
}
}  // namespace

// Returns the number of digests written to out (at most 40), or -1 with the
// error code and message in msg when setup rejects the input.
extern "C" int setup_digest(const pn_mesh *m, const pn_material *mat, const pn_material_table *tab,
                            double dt, uint64_t *out, char *msg, int msg_len) {
  int i = 0;
  msg[0] = 0;
  try {
    pn::MeshTables t;
    pn::MaterialTables mt;
    pn::GridMap g;
    pn::build_mesh_tables(*m, t);
    if (mat) pn::build_material_from_fields(*mat, t, dt, mt);
    else pn::build_material_from_table(*tab, t, dt, mt);
    pn::detect_grid(t, g, 0.95);
    for (const auto *v : {&t.x, &t.y, &t.z, &t.dxc, &t.dyc, &t.dzc, &t.dxn, &t.dyn, &t.dzn, &mt.coef})
      out[i++] = digest_of(*v);
    out[i++] = digest_of(t.hex);
    out[i++] = digest_of(t.ncc);
    out[i++] = digest_of(t.owned);
    out[i++] = (uint64_t)t.uniform;
    out[i++] = fnv(&t.hx, 8) ^ fnv(&t.hy, 8) ^ fnv(&t.hz, 8);
    out[i++] = (uint64_t)mt.n_mat;
    out[i++] = digest_of(mt.c36);
    out[i++] = digest_of(mt.cell_mat);
    out[i++] = (uint64_t)g.ok;
    out[i++] = fnv(g.why.data(), g.why.size());
    out[i++] = ((uint64_t)g.nx << 40) ^ ((uint64_t)g.ny << 20) ^ (uint64_t)g.nz;
    if (g.ok) {
      out[i++] = digest_of(g.node_grid);
      out[i++] = digest_of(g.cell_grid);
      out[i++] = digest_of(g.col_top);
      out[i++] = (uint64_t)g.n_extra;
      out[i++] = digest_of(g.copy_node);
      out[i++] = digest_of(g.copy_site);
      out[i++] = digest_of(g.copy_mask);
      out[i++] = digest_of(g.copy_of_node);
      out[i++] = digest_of(g.fix_cell);
      out[i++] = digest_of(g.fix_of_cell);
    }
    return i;
  } catch (const pn::SetupError &e) {
    snprintf(msg, (size_t)msg_len, "%d %s", e.code, e.msg.c_str());
    return -1;
  }
}

// Source entries (build_source_entries) of n window sources: the force and
// moment entry counts and a digest of each list (element, component, source,
// weight); -1 with the error in msg when setup rejects the input.
extern "C" int setup_digest_sources(const pn_mesh *m, const pn_window_source *src, int n, int exact,
                                    uint64_t *out, char *msg, int msg_len) {
  msg[0] = 0;
  try {
    pn::MeshTables t;
    pn::build_mesh_tables(*m, t);
    std::vector<pn_window_source> all(src, src + n);
    std::vector<pn::SourceEntry> fe, me;
    pn::build_source_entries(t, all, exact != 0, fe, me);
    auto digest_entries = [](const std::vector<pn::SourceEntry> &v) {
      uint64_t h = 1469598103934665603ull;
      for (const pn::SourceEntry &e : v) {
        h = fnv(&e.elem, 4, h);
        h = fnv(&e.comp, 4, h);
        h = fnv(&e.sig, 4, h);
        h = fnv(&e.w, 8, h);
      }
      return h;
    };
    out[0] = fe.size();
    out[1] = me.size();
    out[2] = digest_entries(fe);
    out[3] = digest_entries(me);
    return 4;
  } catch (const pn::SetupError &e) {
    snprintf(msg, (size_t)msg_len, "%d %s", e.code, e.msg.c_str());
    return -1;
  }
}
