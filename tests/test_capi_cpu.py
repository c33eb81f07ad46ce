"""The C-ABI library without a GPU: it loads, exports every entry point the
header declares, and its host-side logic (validation, spacings, material
de-duplication, source windows, signals, footprint, error codes) agrees with
the oracle.  No compute call is made here."""
import ctypes
import os
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from pannde_gb300 import _native as N
from pannde_gb300 import cases

HEADERS = sorted((Path(__file__).resolve().parent.parent / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(pn_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = N.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared but not exported"
        assert n in N.SIGNATURES, f"{n} has no ctypes prototype"
    assert set(N.SIGNATURES) <= names
    assert lib.pn_abi_version() == N.ABI_VERSION == 3


def plan(mesh, material=None, table=None, dt=1e-9, precision=N.PN_PREC_F64):
    lib = N.load()
    m, keep = mesh.as_struct()
    out = N.PnPlan()
    mat = ctypes.byref(material[0]) if material else None
    tab = ctypes.byref(table[0]) if table else None
    rc = lib.pn_plan_solver(ctypes.byref(m), mat, tab, dt, precision, ctypes.byref(out))
    return rc, out, lib.pn_last_error().decode()


def test_plan_plate():
    c = cases.al_plate_case(nx=10, ny=8, nz=3)
    table = N.PN_FORM_TABLE
    rc, p, _ = plan(c.mesh, table=c.material_table(), precision=N.PN_PREC_F64 | table)
    assert rc == 0 and p.form == table
    assert (p.n_nodes, p.n_cells, p.n_materials, p.uniform_spacing) == (11 * 9 * 4, 240, 1, 1)
    assert abs(p.hx - 1e-4) < 1e-18 and abs(p.hz - 1e-4) < 1e-18
    assert p.algorithmic_bytes_per_step == 240 * 180 + 396 * 112
    rc32, p32, _ = plan(c.mesh, table=c.material_table(), precision=N.PN_PREC_F32 | table)
    assert p32.algorithmic_bytes_per_step == 240 * 108 + 396 * 72
    assert p32.device_bytes < p.device_bytes


def test_form_selection():
    """Voxel meshes get the grid form (no connectivity tables: S r/w + 1 material
    byte per lattice cell, V r/w + dt/rho per lattice node); the exact FP64
    form and non-lattice meshes get the table form."""
    c = cases.al_plate_case(nx=10, ny=8, nz=3)
    rc, p, _ = plan(c.mesh, table=c.material_table(), precision=N.PN_PREC_F64)
    assert rc == 0 and p.form == N.PN_FORM_GRID and list(p.grid) == [10, 8, 3]
    assert p.algorithmic_bytes_per_step == 240 * (96 + 1) + 396 * 56
    rc, p, _ = plan(c.mesh, table=c.material_table(), precision=N.PN_PREC_F32)
    assert p.algorithmic_bytes_per_step == 240 * (48 + 1) + 396 * 28
    rc, p, _ = plan(c.mesh, table=c.material_table(), precision=N.PN_PREC_F64_EXACT)
    assert rc == 0 and p.form == N.PN_FORM_TABLE
    h = cases.holed_plate_case(nx=120, ny=100, nz=3, n_holes=2)
    rc, p, _ = plan(h.mesh, table=h.material_table(), precision=N.PN_PREC_DF64)
    assert rc == 0 and p.form == N.PN_FORM_GRID and p.n_cells < 120 * 100 * 3
    g = cases.plate_builder(1.0, 1.0, 0.25, 3, 2)
    g.x = g.x * (1 + 0.1 * g.x)
    gc = cases.Case("g", g, np.array([1.0]), np.ones((1, 21)), np.zeros(g.n_cells, np.int32), 1.0)
    rc, p, _ = plan(g, table=gc.material_table(), precision=N.PN_PREC_F64)
    assert rc == 0 and p.form == N.PN_FORM_TABLE
    rc, p, msg = plan(g, table=gc.material_table(), precision=N.PN_PREC_F64 | N.PN_FORM_GRID)
    assert rc == N.PN_ERR_INVALID and "grid form unavailable" in msg
    rc, p, msg = plan(c.mesh, table=c.material_table(), precision=N.PN_PREC_F64_EXACT | N.PN_FORM_GRID)
    assert rc == N.PN_ERR_INVALID


def test_form_selection_sparse_boxes_and_split_sites():
    """The grid form takes a lattice box it marches in at most twice the mesh's
    cells (each tile column stops at its top solid layer) and lattice sites
    that several nodes share (a crack as disconnected faces), within limits."""
    for crack in ("faces", "slab"):  # L-brackets: about a quarter of the box solid
        b = cases.bracket_case(1003, nsteps=10, crack=crack, scale=0.35)
        rc, p, _ = plan(b.mesh, table=b.material_table(), precision=N.PN_PREC_F32)
        assert rc == 0 and p.form == N.PN_FORM_GRID, crack
    # solid only along the box's diagonal: the tiles' columns are mostly void
    solid = np.zeros((60, 60, 6), dtype=bool)
    for q in range(60):
        solid[q, q, :] = True
    d = cases.voxel_mesh(solid, 1e-4)
    dc = cases.Case("diag", d, np.array([2700.0]), cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None],
                    np.zeros(d.n_cells, np.int32), 1e-9)
    rc, p, _ = plan(d, table=dc.material_table(), precision=N.PN_PREC_F32)
    assert rc == 0 and p.form == N.PN_FORM_TABLE
    rc, p, msg = plan(d, table=dc.material_table(), precision=N.PN_PREC_F32 | N.PN_FORM_GRID)
    assert rc == N.PN_ERR_INVALID and "mostly void" in msg
    # four cracked planes: more than an eighth of the nodes share a lattice site
    m = cases.voxel_mesh(np.ones((10, 10, 10), dtype=bool), 1e-4)
    for z in (2, 4, 6, 8):
        ni, nj, nk = m.node_ijk[:, 0], m.node_ijk[:, 1], m.node_ijk[:, 2]
        face = (nk == z) & (ni > 0) & (ni < 10) & (nj > 0) & (nj < 10)
        m = cases.disconnect_face(m, np.flatnonzero(m.cell_ijk[:, 2] >= z), face)
    mc = cases.Case("planes", m, np.array([2700.0]), cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None],
                    np.zeros(m.n_cells, np.int32), 1e-9)
    rc, p, msg = plan(m, table=mc.material_table(), precision=N.PN_PREC_F32 | N.PN_FORM_GRID)
    assert rc == N.PN_ERR_INVALID and "sharing lattice sites" in msg
    rc, p, _ = plan(m, table=mc.material_table(), precision=N.PN_PREC_F32)
    assert rc == 0 and p.form == N.PN_FORM_TABLE


def test_plan_dedups_field_materials():
    c = cases.laminate_case(nx=6, ny=5, nz=8, nsteps=1, n_sensors=2)
    rc, p, _ = plan(c.mesh, material=c.material_fields())
    # [0/90/+45/-45]s has 4 distinct plies: per-cell fields de-duplicate to 4 rows
    assert rc == 0 and p.n_materials == 4
    rc, p2, _ = plan(c.mesh, table=c.material_table())
    assert p2.n_materials == 8  # a table is taken as given
    assert p2.device_bytes - p.device_bytes == 4 * 36 * 8


def test_plan_graded_mesh_is_not_uniform():
    m = cases.plate_builder(1.0, 1.0, 0.25, 3, 2)
    m.x = m.x * (1 + 0.1 * m.x)
    c = cases.Case("g", m, np.array([1.0]), np.ones((1, 21)), np.zeros(m.n_cells, np.int32), 1.0)
    rc, p, _ = plan(m, table=c.material_table())
    assert rc == 0 and p.uniform_spacing == 0


def isolated_node_mesh():
    m = cases.plate_builder(1.0, 1.0, 0.25, 1, 1)
    m.x, m.y, m.z = (np.append(a, 5.0) for a in (m.x, m.y, m.z))
    return m


@pytest.mark.parametrize("impl", ["device_host", "oracle"])
def test_spacing_error_dx(impl):
    m = isolated_node_mesh()
    c = cases.Case("x", m, np.array([1.0]), np.ones((1, 21)), np.zeros(1, np.int32), 1.0)
    if impl == "oracle":
        with pytest.raises(oracle.OracleError) as e:
            oracle.run(m, c.material_fields(), 1.0, [], 1)
        assert (e.value.code, e.value.msg) == (N.PN_ERR_SPACING, "DX")
    else:
        rc, _, msg = plan(m, table=c.material_table())
        assert (rc, msg) == (N.PN_ERR_SPACING, "DX")


def test_invalid_node_id_and_non_finite():
    m = cases.plate_builder(1.0, 1.0, 0.25, 1, 1)
    c = cases.Case("x", m, np.array([1.0]), np.ones((1, 21)), np.zeros(1, np.int32), 1.0)
    bad = cases.HexMesh(m.x, m.y, m.z, m.hexes.copy())
    bad.hexes[0, 5] = 8
    rc, _, msg = plan(bad, table=c.material_table())
    assert rc == N.PN_ERR_RANGE and "invalid node id" in msg
    nan = cases.HexMesh(m.x.copy(), m.y, m.z, m.hexes)
    nan.x[2] = np.nan
    rc, _, _ = plan(nan, table=c.material_table())
    assert rc == N.PN_ERR_NOT_FINITE
    c2 = cases.Case("x", m, np.array([np.inf]), np.ones((1, 21)), np.zeros(1, np.int32), 1.0)
    rc, _, _ = plan(m, table=c2.material_table())
    assert rc == N.PN_ERR_NOT_FINITE
    rc, _, _ = plan(m, table=c.material_table(), precision=7)
    assert rc == N.PN_ERR_INVALID
    c3 = cases.Case("x", m, np.array([1.0]), np.ones((1, 21)), np.array([3], np.int32), 1.0)
    rc, _, _ = plan(m, table=c3.material_table())
    assert rc == N.PN_ERR_RANGE


def plan_sources(mesh, sources):
    lib = N.load()
    m, keep = mesh.as_struct()
    arr, keep_s = cases.sources_struct(sources)
    fw = np.zeros((mesh.n_nodes, 3))
    mw = np.zeros((mesh.n_cells, 6))
    nn, nc = ctypes.c_int32(0), ctypes.c_int32(0)
    rc = lib.pn_plan_sources(ctypes.byref(m), arr, len(sources), N.dptr(fw), N.dptr(mw),
                             ctypes.byref(nn), ctypes.byref(nc))
    return rc, fw, mw, nn.value, nc.value


def test_force_windows_match_oracle():
    c = cases.al_plate_case(nx=20, ny=18, nz=4, radius=0.6e-3)
    rc, fw, mw, nn, nc = plan_sources(c.mesh, c.sources)
    assert rc == 0 and nc == 0
    ref = oracle.force_weights(c.mesh, c.sources)
    assert np.array_equal(fw, ref)
    assert nn == int((ref.sum(axis=1) > 0).sum()) > 0
    # top layer of cells only: nodes of the two top node layers get weights
    zs = np.unique(c.mesh.z[fw[:, 2] > 0])
    assert len(zs) == 2


def test_moment_windows_count_corners():
    c = cases.al_plate_case(nx=10, ny=10, nz=3)
    t, v = np.array([0.0, 1.0]), np.array([0.0, 1.0])
    src = [cases.WindowSource(N.PN_SOURCE_MOMENT, 0, k, (0.5e-3, 0.5e-3, 0.3e-3), 0.25e-3, 1e-4, t, v)
           for k in (0, 1, 2)]
    rc, fw, mw, nn, nc = plan_sources(c.mesh, src)
    assert rc == 0 and nn == 0 and nc > 0
    # the window takes nodes with |z - 0.3mm| <= 0.075mm and |p - c| < r
    m = c.mesh
    d = np.sqrt((m.x - 0.5e-3) ** 2 + (m.y - 0.5e-3) ** 2 + (m.z - 0.3e-3) ** 2)
    inw = (np.abs(m.z - 0.3e-3) <= 0.75 * 1e-4) & (d < 0.25e-3)
    expect = 0.125 * inw[m.hexes].sum(axis=1)
    for k in range(3):
        assert np.array_equal(mw[:, k], expect)
    assert np.all(mw[:, 3:] == 0)


def test_source_slot_conflict_is_invalid():
    c = cases.al_plate_case(nx=4, ny=4, nz=2)
    s = c.sources[0]
    rc, *_ = plan_sources(c.mesh, [s, s])
    assert rc == N.PN_ERR_INVALID


def signal_eval(t, v, q):
    lib = N.load()
    t, v, q = N.f64(t), N.f64(v), N.f64(q)
    out = np.zeros(len(q))
    sig = N.PnSignal(len(t), N.dptr(t), N.dptr(v))
    rc = lib.pn_signal_eval(ctypes.byref(sig), N.dptr(q), len(q), N.dptr(out))
    return rc, out


def test_signal_known_answers():
    k = np.arange(101)
    rc, out = signal_eval(0.01 * k, -10. * k, [0.01, 0.001, 0.0001, 0.015, 1., 1.1, 11.])
    assert rc == 0
    np.testing.assert_allclose(out, [-10., -1., -0.1, -15., -1000., -1000., -1000.], rtol=1.2e-7)
    rc, out = signal_eval([2., 0., 1., 1.], [20., 0., 10., 99.], [0.5, 1.0, 1.5, 3.0])
    assert list(out) == [5., 10., 15., 20.]
    rc, out = signal_eval([], [], [0.0])
    assert rc == N.PN_ERR_RUNTIME


def test_signal_matches_oracle_on_tone_burst():
    t, v = cases.tone_burst(1e6, 5, 4.6e-9)
    q = np.arange(0, len(t) + 50) * 4.6e-9 * 1.0000001
    rc, out = signal_eval(t, v, q)
    from tests.test_oracle_golden import signal_eval as oracle_eval
    assert rc == 0 and np.array_equal(out, oracle_eval(t, v, q))


def test_hbm_budget_refuses_before_any_device_call(monkeypatch):
    """An artificial HBM budget makes create fail with PN_ERR_ALLOC before any
    allocation (fault injection on the host)."""
    monkeypatch.setenv("PN_HBM_BUDGET_BYTES", "1000")
    c = cases.al_plate_case(nx=6, ny=6, nz=2)
    lib = N.load()
    m, keep = c.mesh.as_struct()
    tab, keep_t = c.material_table()
    h = ctypes.c_void_p()
    rc = lib.pn_solver_create_indexed(ctypes.byref(m), ctypes.byref(tab), c.dt, N.PN_PREC_F64,
                                      ctypes.byref(h))
    assert rc == N.PN_ERR_ALLOC and not h.value
    assert "PN_HBM_BUDGET_BYTES" in lib.pn_last_error().decode()


def test_null_arguments():
    lib = N.load()
    h = ctypes.c_void_p()
    assert lib.pn_solver_create(None, None, 1.0, 1, ctypes.byref(h)) == N.PN_ERR_INVALID
    assert lib.pn_solver_solve(None, 1, None) == N.PN_ERR_INVALID
    assert lib.pn_solver_destroy(None) == N.PN_OK


def test_integration_c_example_builds(tmp_path):
    """The C example of the integration notes compiles as C99 against the
    header and links against the library; it runs a solve on a GPU and
    reports that no CUDA device is usable elsewhere."""
    import shutil
    import subprocess
    from pathlib import Path
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    root = Path(__file__).resolve().parent.parent
    lib = root / "pannde_gb300" / "_build"
    exe = tmp_path / "capi_example"
    r = subprocess.run(["gcc", "-std=c99", "-O1", "-Wall", "-Werror", "-I", str(root / "include"),
                        str(root / "tests" / "cxx" / "capi_example.c"), "-L", str(lib), "-lpannde_gb300",
                        f"-Wl,-rpath,{lib}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode in (0, 3), run.stdout + run.stderr
    if run.returncode == 0:
        assert "10 records" in run.stdout
    else:
        assert "create:" in run.stdout


def test_plan_counts_split_site_storage():
    """A crack's extra node copies (tail slots of the state and dt/rho
    buffers) and the fix-up tables are in the grid form's footprint."""
    solid = np.ones((16, 10, 8), dtype=bool)
    m0 = cases.voxel_mesh(solid, 1e-4)
    ni, nj, nk = m0.node_ijk[:, 0], m0.node_ijk[:, 1], m0.node_ijk[:, 2]
    face = (nk == 4) & (ni > 3) & (ni < 12) & (nj > 2) & (nj < 8)
    m1 = cases.disconnect_face(m0, np.flatnonzero(m0.cell_ijk[:, 2] >= 4), face)
    tab = cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None]
    sizes = []
    for m in (m0, m1):
        c = cases.Case("b", m, np.array([2700.0]), tab, np.zeros(m.n_cells, np.int32), 1e-9)
        rc, p, _ = plan(m, table=c.material_table(), precision=N.PN_PREC_F64)
        assert rc == 0 and p.form == N.PN_FORM_GRID
        sizes.append(p.device_bytes)
    extra = int(face.sum())
    copies = 2 * extra                  # both copies of every split site
    state = extra * (2 * 3 + 1) * 8     # V in both halves and dt/rho, FP64
    assert sizes[1] - sizes[0] >= state + copies * 40
