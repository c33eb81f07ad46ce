"""Parity of the grid form (voxel meshes: implicit lattice indices, one fused
kernel per step, double-buffered state) against the CPU oracle, through the
C ABI.  Tolerances (relative L2 over every field and every trace): FP64 and
double-float 1e-10, FP32 1e-4.
"""
import numpy as np
import pytest

import oracle
from pannde_gb300 import _native as N
from pannde_gb300 import cases
from pannde_gb300.solver import Solver
from tests.test_parity_gpu import compare, random_state, water_column_sources

pytestmark = pytest.mark.gpu

PRECS = ["f64", "df64", "f32"]


def run_grid(mesh, material, dt, sources, nsteps, sensors=None, prec="f64", V0=None, S0=None,
             chunks=None):
    with Solver(mesh, material, dt, prec, "grid") as s:
        assert s.info()["form_name"] == "grid"
        if V0 is not None or S0 is not None:
            s.set_state(V0, S0)
        if sources:
            s.add_sources(sources)
        if sensors is not None and len(sensors):
            s.set_sensors(sensors, nsteps)
        t = 0.0
        for n in (chunks or [nsteps]):
            t = s.solve(n)
        V, S = s.get_state()
        tr = s.traces() if sensors is not None and len(sensors) else None
        return (V, S, tr), t


@pytest.mark.parametrize("prec", PRECS)
def test_grid_transducer_plate(cuda_device, prec):
    c = cases.al_plate_case(nx=40, ny=19, nz=5, nsteps=60, radius=0.6e-3, n_sensors=9)
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, c.nsteps, c.sensors)
    dev, t = run_grid(c.mesh, c, c.dt, c.sources, c.nsteps, c.sensors, prec)
    assert t == ref["time"]
    compare(prec, dev, ref)
    assert np.abs(ref["traces"]).max() > 0


@pytest.mark.parametrize("prec", PRECS)
def test_grid_holes_random_state(cuda_device, prec):
    """Void lattice sites (holes, a notch) behave as the reference's missing cells."""
    solid = np.ones((45, 17, 6), dtype=bool)
    solid[10:14, 5:9, :] = False
    solid[30:, 0:4, 3:] = False
    solid[:, 12:, 5] = False
    m = cases.voxel_mesh(solid, (1e-4, 1.5e-4, 0.8e-4))
    c = cases.Case("g", m, np.array([2700.0]),
                   cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None], np.zeros(m.n_cells, np.int32), 4e-9)
    V0, S0 = random_state(m, 3)
    sens = np.array([0, 17, m.n_nodes // 2, m.n_nodes - 1], np.int32)
    ref = oracle.run(m, c.material_fields(), c.dt, [], 30, sens, V0=V0, S0=S0)
    dev, _ = run_grid(m, c, c.dt, [], 30, sens, prec, V0=V0, S0=S0)
    compare(prec, dev, ref)


def stepped_solid():
    """Columns of many heights: a staircase along y for x < 29, short columns
    (4 layers) for x >= 29 so that the second tile column stops early, a void
    shaft, and an overhang (void below solid)."""
    solid = np.zeros((50, 20, 24), dtype=bool)
    for j in range(20):
        solid[:29, j, :3 + (5 * j) % 21] = True
    solid[29:, :, :4] = True
    solid[12:17, 6:9, :] = False
    solid[3:8, 14:18, 2:5] = False
    return solid


@pytest.mark.parametrize("kchunk", [None, "3"])
@pytest.mark.parametrize("prec", PRECS)
def test_grid_stepped_columns(cuda_device, prec, kchunk, monkeypatch):
    """The tensor-copy kernel stops each tile's march at the tile's top solid
    layer; columns of every height, with and without z chunks, against the
    oracle from a random state with a force and a moment source."""
    if kchunk:
        monkeypatch.setenv("PN_GRID_KCHUNK", kchunk)
    m = cases.voxel_mesh(stepped_solid(), 1e-4)
    c = cases.Case("steps", m, np.array([2700.0]),
                   cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None], np.zeros(m.n_cells, np.int32), 4e-9)
    t = np.linspace(0.0, 2e-7, 60)
    v = np.sin(2e7 * t)
    src = [cases.WindowSource(N.PN_SOURCE_FORCE, 0, 2, (1.0e-3, 1.5e-3, 0.4e-3), 0.3e-3, 1e-4, t, v),
           cases.WindowSource(N.PN_SOURCE_MOMENT, 1, 0, (4.0e-3, 1.0e-3, 0.2e-3), 0.3e-3, 1e-4, t, v)]
    V0, S0 = random_state(m, 21)
    sens = np.array([0, 101, m.n_nodes // 3, m.n_nodes - 1], np.int32)
    ref = oracle.run(m, c.material_fields(), c.dt, src, 30, sens, V0=V0, S0=S0)
    with Solver(m, c, c.dt, prec, "grid") as s:
        assert s.info()["kernel_name"] == "tma"
    dev, _ = run_grid(m, c, c.dt, src, 30, sens, prec, V0=V0, S0=S0, chunks=[11, 19])
    compare(prec, dev, ref)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_grid_slab_cracked_brackets(cuda_device, prec):
    """L-brackets (crack as a removed cell slab) take the grid form: their
    lattice box is mostly void, but the march per tile ends at the tile's top
    solid layer."""
    for seed, wc in ((1003, False), (1006, True)):
        c = cases.bracket_case(seed, nsteps=40, water_column=wc, crack="slab", scale=0.35)
        ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, c.nsteps, c.sensors)
        dev, t = run_grid(c.mesh, c, c.dt, c.sources, c.nsteps, c.sensors, prec)
        assert t == ref["time"]
        compare(prec, dev, ref)


def cracked_block(h=1e-4, axis=2):
    """A 24 x 14 x 10 voxel block (two materials) with a crack as
    disconnected faces in a lattice plane normal to `axis` (z = 5, x in
    (5, 15), y in (3, 9); x = 12 or y = 7 likewise): the cells on its upper
    side get nodes of their own there (split lattice sites)."""
    solid = np.ones((24, 14, 10), dtype=bool)
    m = cases.voxel_mesh(solid, h)
    ni, nj, nk = m.node_ijk[:, 0], m.node_ijk[:, 1], m.node_ijk[:, 2]
    if axis == 2:
        on_face = (nk == 5) & (ni > 5) & (ni < 15) & (nj > 3) & (nj < 9)
    elif axis == 0:
        on_face = (ni == 12) & (nj > 3) & (nj < 9) & (nk > 2) & (nk < 8)
    else:
        on_face = (nj == 7) & (ni > 5) & (ni < 15) & (nk > 2) & (nk < 8)
    above = np.flatnonzero(m.cell_ijk[:, axis] >= (12, 7, 5)[axis])
    n0 = m.n_nodes
    m = cases.disconnect_face(m, above, on_face)
    assert m.n_nodes == n0 + int(on_face.sum())
    mat = (m.cell_ijk[:, 0] >= 12).astype(np.int32)
    cij = np.stack([cases.c21_from_6x6(cases.isotropic(70e9, 0.33)),
                    cases.c21_from_6x6(cases.isotropic(200e9, 0.29))])
    c = cases.Case("crack", m, np.array([2700.0, 7800.0]), cij, mat, 4e-9)
    return c, np.flatnonzero(on_face), np.arange(n0, m.n_nodes)


@pytest.mark.parametrize("h,axis", [(1e-4, 2), ((1e-4, 1.2e-4, 0.8e-4), 2), (1e-4, 0), (1e-4, 1)],
                         ids=["z-cubic", "z-graded", "x-cubic", "y-cubic"])
@pytest.mark.parametrize("prec", PRECS)
def test_grid_crack_as_disconnected_faces(cuda_device, prec, h, axis):
    """Split lattice sites: force windows on the crack plane (both faces'
    nodes), a moment window beside it, sensors on both copies of crack nodes,
    from a random state; cubic voxels (0.25/h folded into the coefficients)
    and unequal spacings."""
    c, lower, upper = cracked_block(h, axis)
    m = c.mesh
    hx, hy, hz = (h, h, h) if np.isscalar(h) else h
    t = np.linspace(0.0, 2e-7, 60)
    v = np.sin(2e7 * t)
    src = [cases.WindowSource(N.PN_SOURCE_FORCE, 0, 2, (10 * hx, 6 * hy, 5 * hz), 2.5 * hx, hz, t, v),
           cases.WindowSource(N.PN_SOURCE_FORCE, 1, 0, (8 * hx, 5 * hy, 5 * hz), 2.0 * hx, hz, t, -v),
           cases.WindowSource(N.PN_SOURCE_MOMENT, 2, 1, (14 * hx, 7 * hy, 4.5 * hz), 2.0 * hx, hz, t, v)]
    V0, S0 = random_state(m, 31)
    sens = np.sort(np.concatenate([lower[::7], upper[::5], [0, m.n_nodes // 2]])).astype(np.int32)
    ref = oracle.run(m, c.material_fields(), c.dt, src, 25, sens, V0=V0, S0=S0)
    with Solver(m, c, c.dt, prec, "grid") as s:
        assert s.info()["form_name"] == "grid"
    dev, t_end = run_grid(m, c, c.dt, src, 25, sens, prec, V0=V0, S0=S0, chunks=[9, 16])
    assert t_end == ref["time"]
    compare(prec, dev, ref)


@pytest.mark.parametrize("prec", PRECS)
def test_grid_cracked_brackets(cuda_device, prec):
    """L-brackets with the crack as disconnected faces (with and without a
    water column) take the grid form and match the oracle."""
    for seed, wc in ((1003, False), (1006, True)):
        c = cases.bracket_case(seed, nsteps=40, water_column=wc, scale=0.35)
        with Solver.from_case(c, precision=prec) as s:
            assert s.info()["form_name"] == "grid"
        ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, c.nsteps, c.sensors)
        dev, t = run_grid(c.mesh, c, c.dt, c.sources, c.nsteps, c.sensors, prec)
        assert t == ref["time"]
        compare(prec, dev, ref)


@pytest.mark.parametrize("prec", PRECS)
def test_grid_laminate_moments_and_forces(cuda_device, prec):
    c = cases.laminate_case(nx=33, ny=29, nz=8, nsteps=40, radius=0.5e-3, n_sensors=6)
    h = c.meta["h"]
    t, v = c.sources[0].times, c.sources[0].values
    src = list(c.sources)
    src += water_column_sources((0.6e-3, 0.5e-3, 0.4e-3), 0.3e-3, h, t, v)
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 1, 0, (1.1e-3, 0.9e-3, 0.4e-3), 0.3e-3, h, t, -v))
    V0, S0 = random_state(c.mesh, 9)
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, src, c.nsteps, c.sensors, V0=V0, S0=S0)
    dev, _ = run_grid(c.mesh, c, c.dt, src, c.nsteps, c.sensors, prec, V0=V0, S0=S0)
    compare(prec, dev, ref)


def test_grid_general_anisotropy(cuda_device):
    """A stiffness with every entry non-zero takes the general (36-entry) path."""
    m = cases.voxel_mesh(np.ones((20, 11, 4), dtype=bool), 1e-4)
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, (6, 6))
    c6 = cases.isotropic(70e9, 0.3) + 5e9 * (a + a.T)
    c = cases.Case("g", m, np.array([2000.0]), cases.c21_from_6x6(c6)[None],
                   np.zeros(m.n_cells, np.int32), 1e-9)
    V0, S0 = random_state(m, 5)
    ref = oracle.run(m, c.material_fields(), c.dt, [], 12, None, V0=V0, S0=S0)
    for prec in PRECS:
        dev, _ = run_grid(m, c, c.dt, [], 12, None, prec, V0=V0, S0=S0)
        compare(prec, dev, ref)


def test_grid_partition_ownership(cuda_device):
    c = cases.al_plate_case(nx=35, ny=10, nz=3, nsteps=10, radius=0.3e-3, n_sensors=4)
    m = c.mesh
    m.node_owner = (m.node_ijk[:, 0] >= 20).astype(np.int32)
    V0, S0 = random_state(m, 5)
    sens = np.array([0, m.n_nodes - 1], np.int32)  # one owned, one not
    ref = oracle.run(m, c.material_fields(), c.dt, c.sources, 10, sens, V0=V0, S0=S0)
    dev, _ = run_grid(m, c, c.dt, c.sources, 10, sens, "f64", V0=V0, S0=S0)
    compare("f64", dev, ref)
    off = m.node_owner == 1
    assert np.array_equal(dev[0][0][off], V0[0][off])
    m.node_owner = None


def test_grid_chunked_solve_is_deterministic(cuda_device):
    c = cases.al_plate_case(nx=40, ny=19, nz=5, nsteps=40, radius=0.6e-3, n_sensors=9)
    a, ta = run_grid(c.mesh, c, c.dt, c.sources, 40, c.sensors, "df64")
    b, tb = run_grid(c.mesh, c, c.dt, c.sources, 40, c.sensors, "df64", chunks=[1] * 5 + [3, 32])
    assert ta == tb
    for k in range(3):
        assert np.array_equal(a[0][k], b[0][k])
    for k in range(6):
        assert np.array_equal(a[1][k], b[1][k])
    assert np.array_equal(a[2], b[2])


@pytest.mark.parametrize("dims", [(1, 1, 1), (31, 7, 2), (32, 8, 3), (62, 14, 1), (5, 40, 3), (12, 9, 70)])
def test_grid_tile_edges(cuda_device, dims):
    """Lattices at, below and above the 31 x 7 owned-cell tile sizes."""
    m = cases.voxel_mesh(np.ones(dims, dtype=bool), 1e-4)
    c = cases.Case("g", m, np.array([2700.0]),
                   cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None], np.zeros(m.n_cells, np.int32), 5e-9)
    V0, S0 = random_state(m, 1)
    ref = oracle.run(m, c.material_fields(), c.dt, [], 7, None, V0=V0, S0=S0)
    dev, _ = run_grid(m, c, c.dt, [], 7, None, "f64", V0=V0, S0=S0)
    compare("f64", dev, ref)


def test_grid_and_table_forms_agree(cuda_device):
    c = cases.laminate_case(nx=24, ny=20, nz=8, nsteps=30, radius=0.4e-3, n_sensors=5)
    out = {}
    for form in ("grid", "table"):
        with Solver.from_case(c, precision="f64", form=form) as s:
            s.solve(c.nsteps)
            out[form] = (s.get_state(), s.traces())
    (Vg, Sg), tg = out["grid"]
    (Vt, St), tt = out["table"]
    for k in range(3):
        np.testing.assert_allclose(Vg[k], Vt[k], rtol=0, atol=1e-12 * np.abs(Vt[k]).max())
    np.testing.assert_allclose(tg, tt, rtol=0, atol=1e-12 * np.abs(tt).max())


@pytest.mark.parametrize("prec", PRECS)
def test_grid_kernels_agree(cuda_device, prec, monkeypatch):
    """The tensor-copy (TMA) staged kernel and the classic register-prefetch
    kernel compute the same step: same sums in the same order, so FP64 and
    double-float agree to rounding noise and FP32 to 1e-5."""
    c = cases.laminate_case(nx=70, ny=23, nz=9, nsteps=25, radius=0.5e-3, n_sensors=6)
    V0, S0 = random_state(c.mesh, 2)
    out = {}
    for kern in ("tma", "classic"):
        if kern == "classic":
            monkeypatch.setenv("PN_GRID_KERNEL", "classic")
        with Solver.from_case(c, precision=prec, form="grid") as s:
            assert s.info()["kernel_name"] == kern
            s.set_state(V0, S0)
            s.solve(c.nsteps)
            out[kern] = (s.get_state(), s.traces())
        monkeypatch.delenv("PN_GRID_KERNEL", raising=False)
    tol = 1e-5 if prec == "f32" else 1e-12
    (Va, Sa), ta = out["tma"]
    (Vb, Sb), tb = out["classic"]
    for x, y in list(zip(Va, Vb)) + list(zip(Sa, Sb)) + [(ta, tb)]:
        d = np.linalg.norm(y)
        assert np.linalg.norm(x - y) <= tol * (d if d > 0 else 1.0)


def test_grid_many_materials_use_classic_kernel(cuda_device):
    """More stiffness rows than the staged table holds: the classic kernel."""
    m = cases.voxel_mesh(np.ones((20, 9, 40), dtype=bool), 1e-4)
    base = cases.c21_from_6x6(cases.isotropic(70e9, 0.33))
    mats = np.stack([base * (1.0 + 0.01 * q) for q in range(40)])
    cm = (m.cell_ijk[:, 2] % 40).astype(np.int32)
    c = cases.Case("g", m, np.full(40, 2700.0), mats, cm, 5e-9)
    V0, S0 = random_state(m, 6)
    ref = oracle.run(m, c.material_fields(), c.dt, [], 9, None, V0=V0, S0=S0)
    with Solver(m, c, c.dt, "df64", "grid") as s:
        assert s.info()["kernel_name"] == "classic"
    dev, _ = run_grid(m, c, c.dt, [], 9, None, "df64", V0=V0, S0=S0)
    compare("df64", dev, ref)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_grid_crack_on_the_classic_kernel(cuda_device, prec):
    """Split sites with more materials than the tensor-copy kernel stages: the
    classic kernel marches the whole box and the same fix-up follows it."""
    c0, lower, upper = cracked_block()
    m = c0.mesh
    base = cases.c21_from_6x6(cases.isotropic(70e9, 0.33))
    mats = np.stack([base * (1.0 + 0.01 * q) for q in range(40)])
    cm = ((m.cell_ijk[:, 0] + 3 * m.cell_ijk[:, 2]) % 40).astype(np.int32)
    c = cases.Case("crack40", m, np.full(40, 2700.0), mats, cm, 4e-9)
    V0, S0 = random_state(m, 8)
    sens = np.sort(np.concatenate([lower[::6], upper[::4]])).astype(np.int32)
    ref = oracle.run(m, c.material_fields(), c.dt, [], 12, sens, V0=V0, S0=S0)
    with Solver(m, c, c.dt, prec, "grid") as s:
        assert s.info()["kernel_name"] == "classic"
    dev, _ = run_grid(m, c, c.dt, [], 12, sens, prec, V0=V0, S0=S0)
    compare(prec, dev, ref)


def test_grid_split_sites_state_roundtrip_and_energy(cuda_device):
    """Nodes of split sites live in tail slots of the node buffers: a state
    set and read back at zero steps is the same bits, and the FP64 energy
    audit (each copy with its own lumped mass) matches numpy after steps."""
    from tests.test_energy_gpu import numpy_energy
    c, lower, upper = cracked_block()
    V0, S0 = random_state(c.mesh, 41)
    for prec in PRECS:
        with Solver(c.mesh, c, c.dt, prec, "grid") as s:
            s.set_state(V0, S0)
            assert s.solve(0) == 0.0
            V, S = s.get_state()
            if prec == "f64":
                for x, y in zip(V + S, V0 + S0):
                    assert np.array_equal(x, y)
            s.solve(9)
            V, S = s.get_state()
            k, e = s.energy()
        kn, en = numpy_energy(c, V, S)
        assert abs(k - kn) <= 1e-12 * kn and abs(e - en) <= 1e-12 * en
