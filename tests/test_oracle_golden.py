"""The CPU oracle pinned to the reference (no GPU).

* golden fixtures produced by the reference HostSolver compiled from its own
  sources (tests/golden/make_golden.py): the C oracle must reproduce every
  field, trace and the time bit for bit;
* the known answers of the reference's own unit tests:
  RightHexTests (HostSolver/testing/include/HostRSGTDUTTests.hpp:121-257),
  HostUnivariateTests (HostData/testing/include/HostUnivariateTests.hpp:52-72),
  HostNormalXDZTests (Stubs/testing/include/HostNormalXDZTests.hpp:58-79),
  with EXPECT_DOUBLE_EQ's 4-ULP tolerance where the reference uses it.
"""
import ctypes
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
from pannde_gb300 import _native as N
from pannde_gb300 import cases
from tests.golden.make_golden import load

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(p for p in GOLDEN.glob("*.npz") if p.name != "righthex_ops.npz")


def ulps_equal(a, b, ulps=4):
    """gtest EXPECT_DOUBLE_EQ: within 4 units in the last place."""
    if a == b:
        return True
    ia = np.array([a], np.float64).view(np.int64)[0]
    ib = np.array([b], np.float64).view(np.int64)[0]
    if (ia < 0) != (ib < 0):
        return abs(a - b) == 0.0
    return abs(int(ia) - int(ib)) <= ulps


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.stem)
def test_oracle_matches_reference_fixture(path):
    g = load(path)
    r = oracle.run(g["mesh"], g["material"], g["dt"], g["sources"], g["nsteps"], g["sensors"],
                   V0=g["V0"], S0=g["S0"], impl="port")
    assert r["time"] == g["time"]
    for k in range(3):
        assert np.array_equal(r["V"][k], g["V"][k]), f"V{k}"
    for k in range(6):
        assert np.array_equal(r["S"][k], g["S"][k]), f"S{k}"
    assert np.array_equal(r["traces"], g["traces"])
    assert np.abs(g["V"]).max() > 0


def test_fixture_inputs_are_regenerable():
    """The stored plate fixture equals what the generators build today."""
    g = load(GOLDEN / "rsgtdut_plate.npz")
    c = cases.al_plate_case(nx=12, ny=10, nz=4, nsteps=40, radius=0.45e-3, n_sensors=6, seed=5)
    assert np.array_equal(g["mesh"].hexes, c.mesh.hexes)
    assert np.array_equal(g["mesh"].z, c.mesh.z)
    assert g["dt"] == c.dt
    assert np.array_equal(g["sensors"], c.sensors)
    assert np.array_equal(g["sources"][0].values, c.sources[0].values)


# ---- RightHexTests ------------------------------------------------------------

def unit_cell():
    return cases.plate_builder(1.0, 1.0, 0.25, 1, 1)   # HostRSGTDUTTests.hpp:121-126


def eight_pack():
    return cases.plate_builder(1.0, 1.0, 0.25, 2, 2)   # HostRSGTDUTTests.hpp:127-132


def test_unit_cell_mesh():
    m = unit_cell()
    assert (m.n_cells, m.n_nodes) == (1, 8)
    expect = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
              (0, 0, .25), (1, 0, .25), (1, 1, .25), (0, 1, .25)]
    for kb, e in enumerate(expect):
        q = m.hexes[0, kb]
        assert (m.x[q], m.y[q], m.z[q]) == e


@pytest.mark.parametrize("impl", ["port", "reference"])
def test_derivatives_of_coordinates(impl):
    if impl == "reference" and oracle.reference() is None:
        pytest.skip("reference sources not present")
    m = unit_cell()
    for fi, f in enumerate((m.x, m.y, m.z)):
        for axis in range(3):
            v, _ = oracle.dd(m, f, 0, axis, True, impl=impl)
            assert ulps_equal(v, float(fi == axis))


def test_derivatives_of_distance():
    m = unit_cell()
    f = np.sqrt(m.x ** 2 + m.y ** 2 + m.z ** 2)
    ddx = 0.25 * (math.sqrt(2.) + (math.sqrt(33.) / 4.) - (1. / 4.)) / 1.
    ddz = 0.25 * ((math.sqrt(17.) / 2. + math.sqrt(33.) / 4. + 1. / 4.) - (2. + math.sqrt(2.))) / 0.25
    for axis, e in enumerate((ddx, ddx, ddz)):
        v, _ = oracle.dd(m, f, 0, axis, True)
        assert ulps_equal(v, e), (axis, v, e)


def test_derivatives_of_node_index():
    m = unit_cell()
    f = np.arange(m.n_nodes, dtype=np.float64)
    ddx = 0.25 * ((4. + 5. + 6. + 7.) - (0. + 1. + 2. + 3.)) / 1.
    ddy = 0.25 * ((2. + 3. + 6. + 7.) - (0. + 1. + 4. + 5.)) / 1.
    ddz = 0.25 * ((1. + 3. + 5. + 7.) - (0. + 2. + 4. + 6.)) / 0.25
    for axis, e in enumerate((ddx, ddy, ddz)):
        v, _ = oracle.dd(m, f, 0, axis, True)
        assert ulps_equal(v, e)


def test_eight_pack_and_cell_coordinate_derivatives():
    m = eight_pack()
    assert (m.n_cells, m.n_nodes) == (8, 27)
    assert (m.x[13], m.y[13], m.z[13]) == (0.5, 0.5, 0.125)
    cc = np.zeros((8, 3))
    for kc in range(8):
        for kb in range(8):
            q = m.hexes[kc, kb]
            cc[kc] += np.array([m.x[q], m.y[q], m.z[q]]) / 8.
    for idx in range(3):
        for axis, sp_expect in enumerate((0.5, 0.5, 0.125)):
            v, sp = oracle.dd(m, cc[:, idx], 13, axis, False)
            assert ulps_equal(sp, sp_expect)
            assert ulps_equal(v, float(idx == axis)), (idx, axis, v)


def test_righthex_fixture_matches_port():
    ops = np.load(GOLDEN / "righthex_ops.npz")["ops"]
    unit, pack = unit_cell(), eight_pack()
    fields_u = [unit.x, unit.y, unit.z, np.sqrt(unit.x ** 2 + unit.y ** 2 + unit.z ** 2),
                np.arange(unit.n_nodes, dtype=np.float64)]
    cc = pack.cell_centers()
    for mesh_id, fi, axis, value, spacing in ops:
        if mesh_id == 0:
            v, _ = oracle.dd(unit, fields_u[int(fi)], 0, int(axis), True)
            assert v == value
        else:
            v, sp = oracle.dd(pack, cc[:, int(fi)], 13, int(axis), False)
            assert v == value and sp == spacing


# ---- HostUnivariateTests / HostNormalXDZTests -----------------------------------

def signal_eval(times, values, ts):
    lib = oracle.port()
    lib.pn_oracle_signal_eval.restype = ctypes.c_int
    lib.pn_oracle_signal_eval.argtypes = [ctypes.POINTER(N.PnSignal), N.P_double, ctypes.c_int32,
                                          N.P_double]
    t, v, q = N.f64(times), N.f64(values), N.f64(ts)
    out = np.zeros(len(ts))
    sig = N.PnSignal(len(t), N.dptr(t), N.dptr(v))
    assert lib.pn_oracle_signal_eval(ctypes.byref(sig), N.dptr(q), len(q), N.dptr(out)) == 0
    return out


def test_univariate_linear_and_hold():
    k = np.arange(101)
    t, v = 0.01 * k, -10. * k          # HostUnivariateTests.hpp:20-25
    q = [0.01, 0.001, 0.0001, 0.015, 1., 1.1, 11.]
    e = [-10., -1., -0.1, -15., -1000., -1000., -1000.]
    out = signal_eval(t, v, q)
    np.testing.assert_allclose(out, e, rtol=1.2e-7, atol=0)   # EXPECT_FLOAT_EQ


def test_univariate_unsorted_and_duplicate_times():
    """std::map::emplace: sorted by time, the first value kept for a repeated time."""
    out = signal_eval([2., 0., 1., 1.], [20., 0., 10., 99.], [0.5, 1.0, 1.5, 3.0])
    assert list(out) == [5., 10., 15., 20.]


def window_eval(args4):
    lib = oracle.port()
    lib.pn_oracle_window_eval.restype = ctypes.c_int
    lib.pn_oracle_window_eval.argtypes = [ctypes.POINTER(N.PnWindowSource), N.P_double, N.P_double]
    nt = 1001
    k = np.arange(nt)
    t = N.f64(k * 0.001)                # HostNormalXDZTests.hpp:24-33
    v = N.f64(0.5 * (1. - np.cos(2. * np.pi * k / (nt - 1))) * np.sin(2. * np.pi * 5. * k / (nt - 1)))
    w = N.PnWindowSource()
    w.kind, w.group, w.component = 0, 0, 2
    for i, c in enumerate((1.0, -1.0, 0.5)):
        w.center[i] = c
    w.radius, w.ds = 0.5, 0.01
    w.signal = N.PnSignal(nt, N.dptr(t), N.dptr(v))
    a = N.f64(args4)
    out = ctypes.c_double(0.)
    assert lib.pn_oracle_window_eval(ctypes.byref(w), N.dptr(a), ctypes.byref(out)) == 0
    return out.value


def test_normal_xdz_window():
    assert window_eval([1., -1., 0.5, 1.]) == 0.0       # signal zero at t = 1
    assert window_eval([1., -1., 0.5, 10.]) == 0.0      # held last value (0)
    assert window_eval([1.5, -1., 0.5, 0.25]) == 0.0    # |p - c| = radius: outside
    assert window_eval([1., -1., 0.5, 0.25]) > 0.0


# ---- oracle error paths -----------------------------------------------------------

def test_isolated_node_raises_dx():
    """RightHex::nodePrep throws logic_error("DX") for a node without cells."""
    m = cases.plate_builder(1.0, 1.0, 0.25, 1, 1)
    m.x = np.append(m.x, 5.0)
    m.y = np.append(m.y, 5.0)
    m.z = np.append(m.z, 5.0)
    c = cases.Case("x", m, np.array([1.0]), cases.c21_from_6x6(np.eye(6))[None], np.zeros(1, np.int32), 1.0)
    with pytest.raises(oracle.OracleError) as e:
        oracle.run(m, c.material_fields(), 1.0, [], 1)
    assert e.value.code == N.PN_ERR_SPACING and e.value.msg == "DX"


def test_bad_node_id_raises_range():
    m = cases.plate_builder(1.0, 1.0, 0.25, 1, 1)
    m.hexes = m.hexes.copy()
    m.hexes[0, 3] = 99
    c = cases.Case("x", m, np.array([1.0]), cases.c21_from_6x6(np.eye(6))[None], np.zeros(1, np.int32), 1.0)
    with pytest.raises(oracle.OracleError) as e:
        oracle.run(m, c.material_fields(), 1.0, [], 1)
    assert e.value.code == N.PN_ERR_RANGE


def test_empty_mesh_and_zero_steps():
    m = cases.HexMesh(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros((0, 8), np.int32))
    c = cases.Case("e", m, np.array([1.0]), np.ones((1, 21)), np.zeros(0, np.int32), 1.0)
    r = oracle.run(m, c.material_fields(), 1.0, [], 5)
    assert r["time"] == 5.0
    p = cases.al_plate_case(nx=4, ny=4, nz=2, nsteps=0, n_sensors=2)
    r = oracle.run(p.mesh, p.material_fields(), p.dt, p.sources, 0, p.sensors)
    assert r["time"] == 0.0 and all(np.all(v == 0) for v in r["V"])


def _random_cases():
    """Seeded small cases the fixtures do not cover together."""
    from tests.test_grid_gpu import cracked_block
    rng = np.random.default_rng(2024)
    out = []
    # holes, two materials, a transducer, a random state (HostRSGTDUT)
    solid = np.ones((14, 10, 5), dtype=bool)
    solid[4:7, 3:6, :] = False
    solid[10:, :3, 3:] = False
    m = cases.voxel_mesh(solid, 1e-4)
    mat = (m.cell_ijk[:, 0] >= 7).astype(np.int32)
    cij = np.stack([cases.c21_from_6x6(cases.isotropic(70e9, 0.33)),
                    cases.c21_from_6x6(cases.rotate_about_z(
                        cases.orthotropic_ply(140e9, 10e9, 10e9, 6e9, 6e9, 4e9, 3e9, 5e9, 5e9), 30.0))])
    c = cases.Case("holes", m, np.array([2700.0, 1600.0]), cij, mat, 4e-9)
    t = np.linspace(0.0, 2e-7, 40)
    v = np.sin(3e7 * t)
    src = [cases.transducer_z((0.7e-3, 0.5e-3, 0.5e-3), 0.3e-3, 1e-4, t, v)]
    out.append((c, src, 0))
    # water-column moments and a transducer (HostUTModel)
    src2 = [cases.WindowSource(N.PN_SOURCE_MOMENT, 0, k, (0.3e-3, 0.3e-3, 0.5e-3), 0.25e-3, 1e-4, t, v * s)
            for k, s in ((0, 1.0), (1, 0.5), (2, -0.8))] + src
    out.append((c, src2, 1))
    # a crack as disconnected faces
    cb, _, _ = cracked_block()
    out.append((cb, [cases.transducer_z((1.0e-3, 0.6e-3, 0.5e-3), 0.25e-3, 1e-4, t, v)], 0))
    # graded spacing along x
    g = cases.plate_builder(1.2e-3, 0.8e-3, 0.3e-3, 6, 3)
    g.x = g.x * (1 + 80.0 * g.x)
    gc = cases.Case("graded", g, np.array([2700.0]), cij[:1], np.zeros(g.n_cells, np.int32), 2e-9)
    out.append((gc, [], 0))
    # duplicated cells of the other material: a node's slot keeps the later
    # cell (HexMesh::buildLinks), which then sets its density and differences
    dup = rng.choice(m.n_cells, size=12, replace=False)
    md = cases.HexMesh(m.x, m.y, m.z, np.concatenate([m.hexes, m.hexes[dup]]).astype(np.int32))
    dc = cases.Case("duplicated", md, c.density, cij, np.concatenate([mat, 1 - mat[dup]]).astype(np.int32), 4e-9)
    out.append((dc, src, 0))
    return [(c, s, k, rng.integers(1 << 30)) for c, s, k in out]


@pytest.mark.parametrize("idx", range(5), ids=["holes", "moments", "crack", "graded", "duplicated"])
def test_port_matches_compiled_reference(idx):
    """The C restatement against the reference HostSolver compiled from its own
    sources, on seeded cases from a random state: every field, trace and the
    time bit for bit."""
    if oracle.reference() is None:
        pytest.skip("reference sources not present")
    c, src, kind, seed = _random_cases()[idx]
    r = np.random.default_rng(int(seed))
    V0 = [r.uniform(-1e-3, 1e-3, c.mesh.n_nodes) for _ in range(3)]
    S0 = [r.uniform(-1e5, 1e5, c.mesh.n_cells) for _ in range(6)]
    sens = np.sort(r.choice(c.mesh.n_nodes, size=6, replace=False)).astype(np.int32)
    args = (c.mesh, c.material_fields(), c.dt, src, 15, sens)
    port = oracle.run(*args, V0=V0, S0=S0, impl="port")
    ref = oracle.run(*args, V0=V0, S0=S0, impl="reference", model_kind=kind)
    assert port["time"] == ref["time"]
    for a, b in zip(port["V"] + port["S"] + [port["traces"]], ref["V"] + ref["S"] + [ref["traces"]]):
        assert np.array_equal(a, b)
