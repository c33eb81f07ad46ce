// pn_setup.hpp -- host-side preparation of the device tables from a
// reference-style mesh / domain description.  Pure C++ (no CUDA calls), so
// every validation and error path here runs without a GPU.
//
// Each step restates the reference semantics it replaces:
//   links      HexMesh::buildLinks            HexMesh.hpp:300-313
//   spacings   RightHex::nodePrep / cellPrep  RightHex.hpp:253-309
//   density    HostField::atNode              HostField.hpp:142-153
//   stiffness  HostField::atCell              HostField.hpp:121-133
//   windows    HostNormalXDZ::evalAt          HostNormalXDZ.hpp:117-123,174-177
//   centres    HostRSGTDUT::cellcenter        HostRSGTDUT.hpp:419-428
//   signals    HostUnivariate::evalAt         HostUnivariate.hpp:109-142
// This file must be compiled with -ffp-contract=off so that the window
// predicates and spacings round exactly as the reference's C++ does.
// The loops over nodes and cells run under OpenMP; every table, and every
// error reported, is the same with any number of threads.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/pannde_gb300.h"

namespace pn {

struct SetupError {
  int code;
  std::string msg;
};

// Allocator that leaves elements default-initialised (for numbers: not
// written) when a vector is sized, so that the parallel loop filling a large
// table is also the first to touch its pages: the page faults of a
// multi-gigabyte table are then spread over the threads instead of taken by
// one zero-filling thread.
template <typename T>
struct UninitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() noexcept = default;
  template <typename U>
  UninitAlloc(const UninitAlloc<U> &) noexcept {}
  template <typename U>
  void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value) {
    ::new ((void *)p) U;
  }
  template <typename U, typename... A>
  void construct(U *p, A &&...a) {
    ::new ((void *)p) U(std::forward<A>(a)...);
  }
};
template <typename T>
using hvec = std::vector<T, UninitAlloc<T>>;

// Largest node or cell count of the connectivity-table form: its kernels
// address the spacing rows of a non-uniform mesh as a*n + i (a < 3) and the
// two int4 halves of a connectivity row as 2*i + h in 32-bit arithmetic.
constexpr int32_t kTableMaxElems = 715827882;  // (2^31 - 1) / 3
// Largest number of force or moment entries of one solver: 32-bit offsets,
// and the grid form hands an entry to up to four blocks.
constexpr int64_t kMaxSourceEntries = (int64_t(1) << 29) - 1;

// Voigt (i,j) -> index into the 21 unique entries.
inline int cij_index(int i, int j) {
  if (i > j) { int t = i; i = j; j = t; }
  return i * 6 - i * (i - 1) / 2 + (j - i);
}

struct MeshTables {
  int32_t n_nodes = 0, n_cells = 0;
  hvec<double> x, y, z;
  hvec<int32_t> hex;       // [n_cells*8]
  hvec<int32_t> ncc;       // [n_nodes*8], -1 = none
  hvec<uint8_t> owned;     // [n_nodes]
  hvec<double> dxc, dyc, dzc, dxn, dyn, dzn;
  bool uniform = false;
  double hx = 0, hy = 0, hz = 0;
};

// Validates and builds links + spacings.  Throws SetupError.
void build_mesh_tables(const pn_mesh &m, MeshTables &t);

struct MaterialTables {
  int32_t n_mat = 0;
  std::vector<double> c36;        // [n_mat][36] raw stiffness (C[i][j])
  hvec<int32_t> cell_mat;         // [n_cells]
  hvec<double> coef;              // [n_nodes] dt / rho_node, 0 = not owned
};

// From reference-style fields (density + 21 Cij, NODE/CELL/CONSTANT).
void build_material_from_fields(const pn_material &mat, const MeshTables &t, double dt,
                                MaterialTables &out);
// From an indexed table (density[n_mat], cij[n_mat][21], cell_material[n_cells]),
// equivalent to CELL fields density[c] = density[mat[c]] etc.
void build_material_from_table(const pn_material_table &mat, const MeshTables &t, double dt,
                               MaterialTables &out);

// Piecewise-linear signal with HostUnivariate semantics.
struct Series {
  std::vector<double> t, v;
  void build(const pn_signal &s);  // throws SetupError
  double eval(double time) const;
  double last_time() const { return t.back(); }
};

// One sparse source entry: element (node or cell), component, source index,
// weight.  Entries are sorted by element; within an element they keep the
// reference's accumulation order.
struct SourceEntry {
  int32_t elem;
  int32_t comp;
  int32_t sig;
  double w;
};

// Builds force entries (per node, per direction) and moment entries (per
// cell, per Voigt component).  exact=true keeps one 0.125-weight entry per
// in-window (element, source) pair in reference order; exact=false merges
// equal (element, component, source) entries into one weight.
// masks (optional, parallel to src): a non-null entry replaces source i's
// geometric window by the caller's per-cell (force) or per-node (moment)
// in-window flags (pn_window_mask).
void build_source_entries(const MeshTables &t, const std::vector<pn_window_source> &src,
                          bool exact, std::vector<SourceEntry> &force,
                          std::vector<SourceEntry> &moment,
                          const std::vector<const uint8_t *> *masks = nullptr);

// Voxel-grid view of a mesh: every node on the lattice x0 + i*hx (etc.),
// every cell the axis-aligned box (i..i+1, j..j+1, k..k+1) with its corners
// in the reference's corner order, no two cells on one lattice site.
// Lattice sites without a mesh node / cell are "void": their velocity and
// stress stay zero, which is what a missing (-1) slot contributes in the
// reference (RightHex.hpp:225-231).  Internal numbering is x fastest with
// padded rows, so that every row starts on a 16-byte boundary (a tensor-copy
// requirement on row strides):
//   grid node (i,j,k) -> (k*(ny+1) + j)*pnx + i,  pnx = (nx+1) rounded up to 4
//   grid cell (i,j,k) -> (k*ny + j)*pcx + i,      pcx = nx rounded up to 16
// Padding sites are void.
// Several mesh nodes may share a lattice site: a crack modelled as
// disconnected faces gives the cells on either side nodes of their own there.
// Such a site is "split"; its first node lives in the lattice buffers, the
// others ("extra copies") in a tail after the lattice sites, and every node of
// a split site is a "copy" with the mask of the site's eight cells it joins
// (bit a + 2b + 4c for cell (i-1+a, j-1+b, k-1+c)).  Cells with a corner on a
// split site are "fix cells": the grid step's fix-up recomputes them.
struct GridMap {
  bool ok = false;
  std::string why;               // reason when not a grid
  int32_t nx = 0, ny = 0, nz = 0;  // cells per axis
  int32_t pnx = 0, pcx = 0;        // row pitch (sites) of node / cell buffers
  hvec<int64_t> node_grid;         // mesh node -> grid node
  hvec<int64_t> cell_grid;         // mesh cell -> grid cell
  std::vector<int32_t> col_top;    // [ny][nx] 1 + the highest solid cell layer of column (i, j), 0 if none
  int64_t n_extra = 0;                // extra copies (tail slots node_sites() + e)
  std::vector<int32_t> copy_node;     // mesh node of every copy (nodes of split sites), ascending
  std::vector<int64_t> copy_site;     // [copies] lattice node index of the copy's site
  std::vector<uint8_t> copy_mask;     // [copies] cells of the site the copy joins
  std::vector<int32_t> copy_of_node;  // mesh node -> copy, or -1 (empty when no site is split)
  std::vector<int32_t> fix_cell;      // mesh cells with a corner on a split site, ascending
  std::vector<int32_t> fix_of_cell;   // mesh cell -> fix cell, or -1 (empty when no site is split)
  // lattice sites (the box, without padding)
  int64_t grid_nodes() const { return (int64_t)(nx + 1) * (ny + 1) * (nz + 1); }
  int64_t grid_cells() const { return (int64_t)nx * ny * nz; }
  // buffer lengths (with padding)
  int64_t node_sites() const { return (int64_t)pnx * (ny + 1) * (nz + 1); }
  int64_t cell_sites() const { return (int64_t)pcx * ny * nz; }
  int64_t node_len() const { return node_sites() + n_extra; }  // node buffers: lattice + tail
  int64_t node_at(int64_t i, int64_t j, int64_t k) const { return (k * (ny + 1) + j) * pnx + i; }
  int64_t cell_at(int64_t i, int64_t j, int64_t k) const { return (k * ny + j) * pcx + i; }
  static int32_t node_pitch(int64_t nx) { return (int32_t)((nx + 1 + 3) / 4 * 4); }
  static int32_t cell_pitch(int64_t nx) { return (int32_t)((nx + 15) / 16 * 16); }
};

// Detects the voxel-grid structure of a uniformly spaced mesh; gives up
// (ok=false) when the lattice box holds more than max_void_fraction void cells.
// Whether the grid form pays on a sparse box is decided later by the work of
// its kernel (grid_eligible).
void detect_grid(const MeshTables &t, GridMap &g, double max_void_fraction = 0.95);

// Per-tile [begin,end) ranges of a list sorted by element.
void tile_ranges(const std::vector<int32_t> &elems, int32_t n_elems, int tile,
                 std::vector<int32_t> &ranges /* [n_tiles*2] */);

// NaN / Inf scan.
bool all_finite(const double *p, int64_t n);

// Moore-Penrose pseudo-inverse of a symmetric 6x6 matrix (row-major), by the
// cyclic Jacobi eigenvalue method; eigenvalues below 1e-12 of the largest are
// treated as zero (a fluid's stiffness has no shear part).
void pinv_sym6(const double *a, double *out);

// Split a double into the (hi, lo) float pair of the double-float form:
// hi = the nearest float, lo = the nearest float to the remainder.
inline void split_df(double d, float &hi, float &lo) {
  hi = (float)d;
  lo = (float)(d - (double)hi);
}

}  // namespace pn
