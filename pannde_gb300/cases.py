"""Meshes, materials, signals and the benchmark cases of the RSG solver.

Restates, in numpy, the geometry and material logic of the reference's
builders so that the device path and the oracle read the same inputs:

* ``plate_builder``: Stubs::PlateBuilder (modules/Stubs/include/PlateBuilder.hpp:
  setGridSpacingAndDimensions, makeNodes, makeCells) -- node index
  kz + Nz*(ky + Ny*kx), corner order 0=(0,0,0) 1=(1,0,0) 2=(1,1,0) 3=(0,1,0),
  4..7 the same at +z.
* ``voxel_mesh``: the voxel-to-hex loop of the case makers
  (py_utils/Case_Makers/*_Case_Maker.py, e.g. Small_Plate_wHoles...py:191-213):
  points exist where any adjacent voxel is solid, x slowest and z fastest,
  cells in the same order, coordinates i*h.
* ``isotropic`` / ``rotate_about_z``: the Voigt stiffness of the case makers
  (Small_Plate...py:163-174) and the Bond rotation about z of
  Stubs::TransverseIsoPlate::rotateCij (MaterialStubs.hpp:197-267) /
  Composite_Laminate...py:rotateStiffnessMatrix.
* ``tone_burst``: the windowed sine of the case makers (Small_Plate...py:255-265).

The benchmark cases are synthetic stand-ins with the shapes, sizes and
parameters of the published workload descriptions (plate 64x64x8 Al,
laminate 400x400x40, plate 1024x1024x24 with holes); all randomness comes
from explicit seeds.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native as N

# ---- meshes -----------------------------------------------------------------


@dataclass
class HexMesh:
    """A hex mesh in the reference's layout (HexMesh.hpp:324-342)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    hexes: np.ndarray                  # [n_cells, 8] int32
    node_owner: Optional[np.ndarray] = None
    partition_id: int = 0
    node_ijk: Optional[np.ndarray] = None   # [n_nodes, 3] grid indices (voxel meshes)
    cell_ijk: Optional[np.ndarray] = None   # [n_cells, 3]

    @property
    def n_nodes(self) -> int:
        return int(self.x.shape[0])

    @property
    def n_cells(self) -> int:
        return int(self.hexes.shape[0])

    def as_struct(self):
        """(PnMesh, keepalive) for the C ABI."""
        keep = [N.f64(self.x), N.f64(self.y), N.f64(self.z), N.i32(self.hexes.reshape(-1))]
        own = N.i32(self.node_owner) if self.node_owner is not None else None
        keep.append(own)
        m = N.PnMesh(self.n_nodes, self.n_cells, N.dptr(keep[0]), N.dptr(keep[1]),
                     N.dptr(keep[2]), N.iptr(keep[3]), N.iptr(own), int(self.partition_id))
        return m, keep

    def cell_centers(self) -> np.ndarray:
        """Cell centres summed as the reference does (0.125*pt in corner order)."""
        cc = np.zeros((self.n_cells, 3))
        for kb in range(8):
            q = self.hexes[:, kb]
            cc[:, 0] += 0.125 * self.x[q]
            cc[:, 1] += 0.125 * self.y[q]
            cc[:, 2] += 0.125 * self.z[q]
        return cc


def plate_builder(length=50.8e-3, width=50.8e-3, thickness=3.175e-3, n_length=128,
                  n_thickness=16) -> HexMesh:
    """Stubs::PlateBuilder::makeMesh restated (PlateBuilder.hpp:75-235)."""
    dz = thickness / float(n_thickness)
    ds = length / float(n_length)
    n0 = int(math.ceil(length / ds)) + 1
    if n0 != n_length + 1:
        raise RuntimeError(f"bad math: {n0} vs {n_length}")
    n1 = int(math.ceil(width / ds)) + 1
    n2 = n_thickness + 1
    kx, ky, kz = np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij")
    x = (kx.reshape(-1) * ds).astype(np.float64)
    y = (ky.reshape(-1) * ds).astype(np.float64)
    z = (kz.reshape(-1) * dz).astype(np.float64)
    cx, cy, cz = np.meshgrid(np.arange(n0 - 1), np.arange(n1 - 1), np.arange(n2 - 1), indexing="ij")
    idx = (cz + n2 * (cy + n1 * cx)).reshape(-1)
    xs, ys = n2 * n1, n2
    hexes = np.stack([idx, idx + xs, idx + xs + ys, idx + ys,
                      idx + 1, idx + 1 + xs, idx + 1 + xs + ys, idx + 1 + ys], axis=1).astype(np.int32)
    node_ijk = np.stack([kx.reshape(-1), ky.reshape(-1), kz.reshape(-1)], axis=1)
    cell_ijk = np.stack([cx.reshape(-1), cy.reshape(-1), cz.reshape(-1)], axis=1)
    return HexMesh(x, y, z, hexes, node_ijk=node_ijk, cell_ijk=cell_ijk)


def voxel_mesh(solid: np.ndarray, h, origin=(0.0, 0.0, 0.0)) -> HexMesh:
    """Hex mesh of the solid voxels of ``solid`` [nx, ny, nz] (bool).

    Points exist where any adjacent voxel is solid; nodes and cells are
    numbered with x slowest and z fastest; coordinates origin + i*h.
    """
    solid = np.asarray(solid, dtype=bool)
    nx, ny, nz = solid.shape
    hx, hy, hz = (h, h, h) if np.isscalar(h) else h
    pad = np.zeros((nx + 2, ny + 2, nz + 2), dtype=bool)
    pad[1:-1, 1:-1, 1:-1] = solid
    used = np.zeros((nx + 1, ny + 1, nz + 1), dtype=bool)
    for di in (0, 1):
        for dj in (0, 1):
            for dk in (0, 1):
                used |= pad[di:di + nx + 1, dj:dj + ny + 1, dk:dk + nz + 1]
    flat = np.flatnonzero(used.reshape(-1))
    nid = np.full(used.size, -1, dtype=np.int32)  # lattice point (flat) -> node id
    nid[flat] = np.arange(flat.size, dtype=np.int32)
    ii, jj, kk = np.unravel_index(flat, used.shape)
    x = origin[0] + ii * hx
    y = origin[1] + jj * hy
    z = origin[2] + kk * hz
    cells = np.flatnonzero(solid.reshape(-1))  # C order: x slowest, z fastest
    ci, cj, ck = np.unravel_index(cells, solid.shape)
    # flat lattice point of each cell's corner 0, then the corners' offsets
    sj, si = nz + 1, (ny + 1) * (nz + 1)
    base = ci * si + cj * sj + ck
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    hexes = np.empty((cells.size, 8), dtype=np.int32)
    for q, (a, b, c) in enumerate(corners):
        hexes[:, q] = nid[base + (a * si + b * sj + c)]
    node_ijk = np.empty((flat.size, 3), dtype=np.int64)
    node_ijk[:, 0], node_ijk[:, 1], node_ijk[:, 2] = ii, jj, kk
    cell_ijk = np.empty((cells.size, 3), dtype=np.int64)
    cell_ijk[:, 0], cell_ijk[:, 1], cell_ijk[:, 2] = ci, cj, ck
    return HexMesh(x.astype(np.float64), y.astype(np.float64), z.astype(np.float64), hexes,
                   node_ijk=node_ijk, cell_ijk=cell_ijk)


# ---- materials --------------------------------------------------------------

VOIGT = ((0, 5, 4), (5, 1, 3), (4, 3, 2))  # ijtable, MaterialStubs.hpp:279-281
UPPER = [(i, j) for i in range(6) for j in range(i, 6)]  # the 21-entry order


def c21_from_6x6(c: np.ndarray) -> np.ndarray:
    return np.array([c[i, j] for i, j in UPPER], dtype=np.float64)


def c6x6_from_21(c21) -> np.ndarray:
    c = np.zeros((6, 6))
    for k, (i, j) in enumerate(UPPER):
        c[i, j] = c[j, i] = c21[k]
    return c


def isotropic(E: float, nu: float) -> np.ndarray:
    """6x6 Voigt stiffness of an isotropic solid (lambda+2mu, lambda, mu)."""
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    c = np.zeros((6, 6))
    c[:3, :3] = lam
    for i in range(3):
        c[i, i] = lam + 2 * mu
        c[i + 3, i + 3] = mu
    return c


def rotate_about_z(c: np.ndarray, angle_deg: float) -> np.ndarray:
    """Rotate a 6x6 Voigt stiffness about z: C'_ijkl = R_ia R_jb R_kc R_ld C_abcd."""
    cijkl = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    cijkl[i, j, k, l] = c[VOIGT[i][j], VOIGT[k][l]]
    a = angle_deg * np.pi / 180.0
    R = np.eye(3)
    R[0, 0] = np.cos(a)
    R[0, 1] = -np.sin(a)
    R[1, 0] = np.sin(a)
    R[1, 1] = np.cos(a)
    rot = np.einsum("ia,jb,kc,ld,abcd->ijkl", R, R, R, R, cijkl)
    out = np.zeros((6, 6))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    out[VOIGT[i][j], VOIGT[k][l]] = rot[i, j, k, l]
    return out


def orthotropic_ply(C11, C22, C33, C12, C13, C23, C44, C55, C66) -> np.ndarray:
    c = np.zeros((6, 6))
    c[0, 0], c[1, 1], c[2, 2] = C11, C22, C33
    c[0, 1] = c[1, 0] = C12
    c[0, 2] = c[2, 0] = C13
    c[1, 2] = c[2, 1] = C23
    c[3, 3], c[4, 4], c[5, 5] = C44, C55, C66
    return c


def max_wave_speed(c6: np.ndarray, rho: float) -> float:
    return float(np.sqrt(max(c6[0, 0], c6[1, 1], c6[2, 2]) / rho))


def cfl_dt(h: float, c_max: float, fraction: float = 0.5) -> float:
    """dt = fraction * h / (c_max * sqrt(3)), the 3-D explicit-scheme bound."""
    return fraction * h / (c_max * math.sqrt(3.0))


# ---- signals ----------------------------------------------------------------


def hann(m: int) -> np.ndarray:
    """Symmetric Hann window of length m (0.5 - 0.5 cos(2 pi n / (m-1)))."""
    if m == 1:
        return np.ones(1)
    n = np.arange(m)
    return 0.5 - 0.5 * np.cos(2.0 * np.pi * n / (m - 1))


def tone_burst(freq: float, n_cycles: float, dt: float, amp: float = 1.0):
    """Hann-windowed sine burst sampled at dt, normalised to max 1."""
    steps = int(np.ceil((n_cycles / freq) / dt))
    t = np.arange(steps) * dt
    wf = amp * np.sin(t * freq * 2 * np.pi) * hann(steps)
    wf = wf / wf.max()
    return t.astype(np.float64), wf.astype(np.float64)


# ---- sources / cases --------------------------------------------------------


@dataclass
class WindowSource:
    """A Stubs::HostNormalXDZ window with a HostUnivariate signal."""
    kind: int
    group: int
    component: int
    center: tuple
    radius: float
    ds: float
    times: np.ndarray
    values: np.ndarray


def sources_struct(sources):
    """(PnWindowSource[n], keepalive) for the C ABI."""
    arr = (N.PnWindowSource * max(len(sources), 1))()
    keep = []
    for i, s in enumerate(sources):
        t, v = N.f64(s.times), N.f64(s.values)
        keep += [t, v]
        w = arr[i]
        w.kind, w.group, w.component = int(s.kind), int(s.group), int(s.component)
        for k in range(3):
            w.center[k] = float(s.center[k])
        w.radius, w.ds = float(s.radius), float(s.ds)
        w.signal = N.PnSignal(int(t.shape[0]), N.dptr(t), N.dptr(v))
    return arr, keep


@dataclass
class Case:
    name: str
    mesh: HexMesh
    density: np.ndarray          # [n_mat]
    cij: np.ndarray              # [n_mat, 21]
    cell_material: np.ndarray    # [n_cells] int32
    dt: float
    sources: list = field(default_factory=list)
    sensors: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    nsteps: int = 1
    meta: dict = field(default_factory=dict)

    def material_table(self):
        keep = [N.f64(self.density), N.f64(self.cij.reshape(-1)), N.i32(self.cell_material)]
        t = N.PnMaterialTable(int(self.density.shape[0]), N.dptr(keep[0]), N.dptr(keep[1]),
                              N.iptr(keep[2]))
        return t, keep

    def material_fields(self):
        """CELL fields (density, 21 Cij) as the reference's domain bundle holds them."""
        rho = N.f64(self.density[self.cell_material])
        cs = [N.f64(self.cij[self.cell_material, k]) for k in range(21)]
        m = N.PnMaterial()
        m.density = N.PnField(N.PN_FIELD_CELL, N.dptr(rho))
        for k in range(21):
            m.cij[k] = N.PnField(N.PN_FIELD_CELL, N.dptr(cs[k]))
        return m, [rho] + cs


def top_face_nodes(mesh: HexMesh) -> np.ndarray:
    return np.flatnonzero(mesh.z == mesh.z.max()).astype(np.int32)


def seeded_sensors(mesh: HexMesh, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    top = top_face_nodes(mesh)
    return np.sort(rng.choice(top, size=min(n, top.size), replace=False)).astype(np.int32)


def transducer_z(center, radius, h_z, times, values, group=0) -> WindowSource:
    """A z-force transducer as TransducerModel builds it ({null,null,XD})."""
    return WindowSource(N.PN_SOURCE_FORCE, group, 2, tuple(center), radius, h_z, times, values)


ALUMINIUM = dict(rho=2700.0, E=70e9, nu=0.33)


def al_plate_case(nx=64, ny=64, nz=8, h=0.1e-3, nsteps=2000, freq=1e6, radius=2e-3,
                  n_sensors=16, seed=0, holes=None, name="al-plate") -> Case:
    """Aluminium plate, z-force tone burst on a circular patch centred on the top face."""
    solid = np.ones((nx, ny, nz), dtype=bool)
    if holes:
        ii, jj = np.meshgrid((np.arange(nx) + 0.5) * h, (np.arange(ny) + 0.5) * h, indexing="ij")
        for (cx, cy, r) in holes:
            solid[(ii - cx) ** 2 + (jj - cy) ** 2 < r * r, :] = False
    mesh = voxel_mesh(solid, h)
    c6 = isotropic(ALUMINIUM["E"], ALUMINIUM["nu"])
    rho = ALUMINIUM["rho"]
    dt = cfl_dt(h, max_wave_speed(c6, rho))
    t, v = tone_burst(freq, 5, dt)
    center = (nx * h / 2, ny * h / 2, nz * h)
    src = [transducer_z(center, radius, h, t, v)]
    return Case(name, mesh, np.array([rho]), c21_from_6x6(c6)[None, :],
                np.zeros(mesh.n_cells, np.int32), dt, src, seeded_sensors(mesh, n_sensors, seed),
                nsteps, dict(nx=nx, ny=ny, nz=nz, h=h, freq=freq))


LAYUP = (0.0, 90.0, 45.0, -45.0, -45.0, 45.0, 90.0, 0.0)  # [0/90/+45/-45]s


def laminate_case(nx=400, ny=400, nz=40, h=0.05e-3, nsteps=5000, freq=500e3, radius=2e-3,
                  n_sensors=64, seed=1, layup=LAYUP, name="laminate") -> Case:
    """Composite laminate, plies of nz/len(layup) cells, orthotropic ply rotated about z."""
    ply = orthotropic_ply(140e9, 10e9, 10e9, 6e9, 6e9, 4e9, 3e9, 5e9, 5e9)
    rho = 1600.0
    mats = [rotate_about_z(ply, a) for a in layup]
    cells_per_ply = nz // len(layup)
    kply = np.minimum(np.arange(nz) // cells_per_ply, len(layup) - 1)
    mesh = voxel_mesh(np.ones((nx, ny, nz), dtype=bool), h)
    cell_material = kply[mesh.cell_ijk[:, 2]].astype(np.int32)
    cmax = max(max_wave_speed(m, rho) for m in mats)
    dt = cfl_dt(h, cmax)
    t, v = tone_burst(freq, 5, dt)
    center = (nx * h / 2, ny * h / 2, nz * h)
    src = [transducer_z(center, radius, h, t, v)]
    return Case(name, mesh, np.full(len(layup), rho), np.stack([c21_from_6x6(m) for m in mats]),
                cell_material, dt, src, seeded_sensors(mesh, n_sensors, seed), nsteps,
                dict(nx=nx, ny=ny, nz=nz, h=h, freq=freq, layup=list(layup)))


def holed_plate_case(nx=1024, ny=1024, nz=24, h=0.1e-3, nsteps=4000, n_holes=12, seed=3,
                     n_sensors=128, name="al-plate-holes") -> Case:
    """Aluminium plate with seeded through-thickness holes (radii 1-4 mm)."""
    rng = np.random.default_rng(seed)
    L, W = nx * h, ny * h
    holes = []
    for _ in range(n_holes):
        r = rng.uniform(1e-3, 4e-3)
        holes.append((rng.uniform(r, L - r), rng.uniform(r, W - r), r))
    case = al_plate_case(nx, ny, nz, h, nsteps, 1e6, 2e-3, n_sensors, seed, holes, name)
    case.meta["holes"] = holes
    return case


# ---- angle brackets (L-sections) --------------------------------------------

WATER = dict(rho=1000.0, c=1480.0)


def fluid_stiffness(rho: float, c: float) -> np.ndarray:
    """Acoustic fluid through the 21 Cij: C11=C22=C33=C12=C13=C23=rho c^2, no shear."""
    k = rho * c * c
    out = np.zeros((6, 6))
    out[:3, :3] = k
    return out


def disconnect_face(mesh: HexMesh, cells_above: np.ndarray, node_mask: np.ndarray) -> HexMesh:
    """Split the mesh along a face: the nodes in node_mask get a duplicate that
    the cells in cells_above use instead, so the two sides share no node there
    (a zero-thickness crack; the reference then sees a missing incident cell on
    each side, RightHex.hpp:225-231)."""
    dup = np.flatnonzero(node_mask)
    new_id = np.full(mesh.n_nodes, -1, dtype=np.int64)
    new_id[dup] = mesh.n_nodes + np.arange(dup.size)
    hexes = mesh.hexes.copy()
    sub = hexes[cells_above]
    repl = new_id[sub]
    sub[repl >= 0] = repl[repl >= 0]
    hexes[cells_above] = sub
    x = np.concatenate([mesh.x, mesh.x[dup]])
    y = np.concatenate([mesh.y, mesh.y[dup]])
    z = np.concatenate([mesh.z, mesh.z[dup]])
    ijk = np.concatenate([mesh.node_ijk, mesh.node_ijk[dup]]) if mesh.node_ijk is not None else None
    return HexMesh(x, y, z, hexes.astype(np.int32), node_ijk=ijk, cell_ijk=mesh.cell_ijk)


def bracket_case(seed: int, h=0.1e-3, nsteps=3000, water_column=False, n_sensors=8,
                 scale=1.0, name="bracket", crack="faces") -> Case:
    """Aluminium L-section angle bracket with a seeded planar crack at the inner fillet.

    Cross-section in (y, z): a vertical leg (y < t) and a horizontal leg (z < t),
    extruded along x (the voxel construction of AL_Angle_Bracket_Water_Column_Case_Maker.py:
    geometry[:, :t, :] = geometry[:, :, :t] = 1).  Leg lengths 60-220 cells, thickness
    12-30 cells, depth 40-160 cells, drawn from the seed (scale shrinks them for tests).
    The crack lies in the plane z = t under the vertical leg, opening at the inner
    face y = t, 1-6 mm long along x: crack="faces" makes it disconnected faces
    (duplicated nodes), crack="slab" removes a 150 um slab of cells there instead
    (the construction of Bracket_Crack...py:52-66; the mesh stays a voxel
    lattice).  With water_column, a
    cylinder of fluid cells (rho 1000, c 1480 m/s) stands on the horizontal leg's top
    face and the excitation is a pressure (xx, yy, zz moment) window at its top;
    otherwise a z-force transducer acts on the horizontal leg's outer face."""
    rng = np.random.default_rng(seed)
    ly = max(4, int(round(rng.integers(60, 221) * scale)))
    lz = max(4, int(round(rng.integers(60, 221) * scale)))
    t = max(2, int(round(rng.integers(12, 31) * scale)))
    d = max(4, int(round(rng.integers(40, 161) * scale)))
    ly, lz = max(ly, t + 2), max(lz, t + 2)
    col_r = max(1, int(round(rng.integers(5, 16) * scale)))
    col_h = max(1, int(round(rng.integers(10, 31) * scale)))
    nz_box = max(lz, t + col_h) if water_column else lz
    solid = np.zeros((d, ly, nz_box), dtype=bool)
    solid[:, :t, :lz] = True
    solid[:, :, :t] = True
    fluid = np.zeros_like(solid)
    yc = (t + ly) / 2.0
    if water_column:
        ii, jj = np.meshgrid(np.arange(d) + 0.5, np.arange(ly) + 0.5, indexing="ij")
        disk = ((ii - d / 2.0) ** 2 + (jj - yc) ** 2 < col_r ** 2) & (jj >= t)
        for k in range(t, t + col_h):
            fluid[:, :, k] |= disk
        fluid &= ~solid
        solid |= fluid
    # crack: plane z = t, x in (x0, x0 + c), y in (t - cw, t], under the vertical leg
    c_len = max(2, int(round(rng.uniform(1e-3, 6e-3) / h * min(1.0, scale * 2))))
    c_len = min(c_len, d - 2)
    cw = max(1, min(t - 1, int(round(rng.uniform(0.2, 0.6) * t))))
    x0 = int(rng.integers(1, max(2, d - c_len)))
    if crack == "slab":
        slab = max(1, int(round(150e-6 / h)))
        solid[x0:x0 + c_len, t - cw:t, t:min(t + slab, lz)] = False
    mesh = voxel_mesh(solid, h)
    ci, cj, ck = mesh.cell_ijk[:, 0], mesh.cell_ijk[:, 1], mesh.cell_ijk[:, 2]
    cell_material = fluid[ci, cj, ck].astype(np.int32)
    if crack == "faces":
        ni, nj, nk = mesh.node_ijk[:, 0], mesh.node_ijk[:, 1], mesh.node_ijk[:, 2]
        on_face = (nk == t) & (ni > x0) & (ni < x0 + c_len) & (nj > t - cw) & (nj <= t)
        above = np.flatnonzero((ck >= t) & (cj < t) & (cell_material == 0))
        mesh = disconnect_face(mesh, above, on_face)
    elif crack != "slab":
        raise ValueError(f"crack must be 'faces' or 'slab', not {crack!r}")
    c_al = isotropic(ALUMINIUM["E"], ALUMINIUM["nu"])
    rho_al = ALUMINIUM["rho"]
    c_w = fluid_stiffness(WATER["rho"], WATER["c"])
    dt = cfl_dt(h, max_wave_speed(c_al, rho_al))
    freq = float(rng.uniform(0.5e6, 2e6))
    tt, vv = tone_burst(freq, 5, dt)
    if water_column:
        ztop = (t + col_h) * h
        src = [WindowSource(N.PN_SOURCE_MOMENT, 0, comp, (d * h / 2, yc * h, ztop), col_r * h * 0.9, h, tt, -vv)
               for comp in (0, 1, 2)]
    else:
        src = [transducer_z((d * h / 2, yc * h, 0.0), max(2, col_r) * h, h, tt, vv)]
    outer = np.flatnonzero((mesh.z == 0.0) | (mesh.y == 0.0))
    sens = np.sort(rng.choice(outer, size=min(n_sensors, outer.size), replace=False)).astype(np.int32)
    return Case(f"{name}-{seed}", mesh, np.array([rho_al, WATER["rho"]]),
                np.stack([c21_from_6x6(c_al), c21_from_6x6(c_w)]), cell_material, dt, src, sens, nsteps,
                dict(ly=ly, lz=lz, t=t, d=d, crack=(x0, c_len, cw), crack_kind=crack,
                     water_column=water_column, h=h, freq=freq))
