"""Parity of the CUDA RSG leapfrog against the CPU oracle (through the C ABI),
table form (connectivity tables, any hex mesh).  tests/test_grid_gpu.py covers
the grid form.

Tolerances (relative L2 over every field and every trace):
  f64_exact  bit-identical (np.array_equal)
  f64        1e-10
  df64       1e-10  (double-float: 48-bit significand on the FP32 pipes)
  f32        1e-4   (FP32 state; traces are recorded in FP64)
df64 and f32 have FP32's exponent range.  A sensor the wave has not reached
holds only the stencil's leakage ahead of the wave front, values of 1e-160
and the like in FP64, which these forms hold as zero or as subnormals (FP32
below 1.2e-38; a double-float below about 2e-31, whose low word is then
subnormal) with few significand bits.  For these two forms each trace's
error is therefore taken relative to at least 1e-6 of the largest trace's
norm (TRACE_FLOOR) and at least 1e-30 per value in root-mean-square
(RANGE_FLOOR).  A field component can be pure round-off (the shear stresses
of a solid driven only by a pressure source: 1e-43 beside normal stresses of
1e-10), which no form that reorders the arithmetic reproduces; outside exact
mode each component's error is taken relative to at least 1e-6 of the
largest norm among the components of its vector / tensor (FIELD_FLOOR).
"""
import numpy as np
import pytest

import oracle
from pannde_gb300 import _native as N
from pannde_gb300 import cases
from pannde_gb300.solver import Solver

pytestmark = pytest.mark.gpu

TOL = {"f64_exact": 0.0, "f64": 1e-10, "df64": 1e-10, "f32": 1e-4}
TRACE_FLOOR = {"df64": 1e-6, "f32": 1e-6}  # of the largest trace norm
FIELD_FLOOR = 1e-6  # of the largest component norm of V (S)
RANGE_FLOOR = {"df64": 1e-30, "f32": 1e-30}  # root-mean-square per value


def rel_l2(a, b, floor=0.0):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    d = max(np.linalg.norm(b), floor)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def compare(prec, dev, ref):
    V, S, tr = dev
    if prec == "f64_exact":
        for k in range(3):
            assert np.array_equal(V[k], ref["V"][k]), f"V{k}"
        for k in range(6):
            assert np.array_equal(S[k], ref["S"][k]), f"S{k}"
        if tr is not None:
            assert np.array_equal(tr, ref["traces"])
        return 0.0
    tiny = RANGE_FLOOR.get(prec, 0.0)
    fv = max(FIELD_FLOOR * max(np.linalg.norm(x) for x in ref["V"]), tiny * np.sqrt(ref["V"][0].size))
    fs = max(FIELD_FLOOR * max(np.linalg.norm(x) for x in ref["S"]), tiny * np.sqrt(ref["S"][0].size))
    errs = [rel_l2(V[k], ref["V"][k], fv) for k in range(3)] + \
           [rel_l2(S[k], ref["S"][k], fs) for k in range(6)]
    if tr is not None and ref["traces"].size:
        rt = ref["traces"]
        floor = max(TRACE_FLOOR.get(prec, 0.0) * max(np.linalg.norm(rt[:, i]) for i in range(rt.shape[1])),
                    tiny * np.sqrt(rt[:, 0].size))
        for i in range(tr.shape[1]):  # every trace on its own
            errs.append(rel_l2(tr[:, i], rt[:, i], floor))
    worst = max(errs)
    assert worst <= TOL[prec], f"{prec}: worst rel L2 {worst:.3e}"
    return worst


def run_dev(mesh, material, dt, sources, nsteps, sensors=None, prec="f64", V0=None, S0=None,
            chunks=None, form="table"):
    with Solver(mesh, material, dt, prec, form) as s:
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


@pytest.fixture(scope="module")
def plate():
    return cases.al_plate_case(nx=16, ny=16, nz=4, nsteps=60, radius=0.5e-3, n_sensors=8)


@pytest.mark.parametrize("prec", ["f64_exact", "f64", "df64", "f32"])
def test_transducer_plate(cuda_device, plate, prec):
    c = plate
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, c.nsteps, c.sensors)
    dev, t = run_dev(c.mesh, c, c.dt, c.sources, c.nsteps, c.sensors, prec)
    assert t == ref["time"]
    compare(prec, dev, ref)
    assert np.abs(ref["traces"]).max() > 0


@pytest.mark.parametrize("prec", ["f64_exact", "f64"])
def test_field_material_matches_indexed(cuda_device, plate, prec):
    """pn_solver_create (fields) and pn_solver_create_indexed give one result."""
    c = plate
    a, _ = run_dev(c.mesh, c, c.dt, c.sources, 20, c.sensors, prec)
    b, _ = run_dev(c.mesh, c.material_fields(), c.dt, c.sources, 20, c.sensors, prec)
    for k in range(3):
        assert np.array_equal(a[0][k], b[0][k])
    for k in range(6):
        assert np.array_equal(a[1][k], b[1][k])


def random_state(mesh, seed):
    rng = np.random.default_rng(seed)
    V0 = [rng.uniform(-1e-3, 1e-3, mesh.n_nodes) for _ in range(3)]
    S0 = [rng.uniform(-1e5, 1e5, mesh.n_cells) for _ in range(6)]
    return V0, S0


def holed_warped_mesh():
    """Voxel block with a hole and a notch (missing cells) on graded coordinates."""
    solid = np.ones((9, 7, 5), dtype=bool)
    solid[3:5, 2:4, :] = False       # through hole
    solid[7:, 0:2, 3:] = False       # corner notch
    m = cases.voxel_mesh(solid, 1e-3)
    i, j, k = m.node_ijk[:, 0], m.node_ijk[:, 1], m.node_ijk[:, 2]
    m.x = 1e-3 * (i + 0.15 * np.sin(1.3 * i))
    m.y = 1e-3 * (j + 0.1 * np.cos(0.7 * j))
    m.z = 0.5e-3 * (k + 0.2 * k * k / 5.0)
    return m


def laminate_material(mesh):
    ply = cases.orthotropic_ply(140e9, 10e9, 10e9, 6e9, 6e9, 4e9, 3e9, 5e9, 5e9)
    mats = [cases.rotate_about_z(ply, a) for a in (0, 45, -45, 90)]
    cm = (mesh.cell_ijk[:, 2] % 4).astype(np.int32)
    return cases.Case("lam", mesh, np.array([1600.0, 1500.0, 1700.0, 1650.0]),
                      np.stack([cases.c21_from_6x6(x) for x in mats]), cm, 1e-9)


@pytest.mark.parametrize("prec", ["f64_exact", "f64", "df64", "f32"])
def test_holes_graded_anisotropic_random_state(cuda_device, prec):
    m = holed_warped_mesh()
    c = laminate_material(m)
    V0, S0 = random_state(m, 7)
    sens = np.array([0, 5, m.n_nodes - 1, m.n_nodes // 2], np.int32)
    ref = oracle.run(m, c.material_fields(), 2e-9, [], 25, sens, V0=V0, S0=S0)
    dev, t = run_dev(m, c, 2e-9, [], 25, sens, prec, V0=V0, S0=S0)
    assert t == ref["time"]
    compare(prec, dev, ref)


def node_and_constant_fields(mesh, seed=3):
    """density as a NODE field, C as CONSTANT fields except C11 on NODES."""
    rng = np.random.default_rng(seed)
    rho = N.f64(rng.uniform(2000, 3000, mesh.n_nodes))
    c6 = cases.isotropic(70e9, 0.33)
    c21 = cases.c21_from_6x6(c6)
    arrays = [rho]
    mat = N.PnMaterial()
    mat.density = N.PnField(N.PN_FIELD_NODE, N.dptr(rho))
    for k in range(21):
        if k == 0:
            a = N.f64(c21[0] * rng.uniform(0.9, 1.1, mesh.n_nodes))
            mat.cij[k] = N.PnField(N.PN_FIELD_NODE, N.dptr(a))
        else:
            a = N.f64([c21[k]])
            mat.cij[k] = N.PnField(N.PN_FIELD_CONSTANT, N.dptr(a))
        arrays.append(a)
    return mat, arrays


@pytest.mark.parametrize("prec", ["f64_exact", "f64"])
def test_node_and_constant_fields(cuda_device, prec):
    m = holed_warped_mesh()
    mat = node_and_constant_fields(m)
    V0, S0 = random_state(m, 11)
    ref = oracle.run(m, mat, 1e-9, [], 15, None, V0=V0, S0=S0)
    dev, _ = run_dev(m, mat, 1e-9, [], 15, None, prec, V0=V0, S0=S0)
    compare(prec, dev, ref)


def water_column_sources(center, radius, ds, t, v):
    """RoundWaterExcitationManager: XX, YY, ZZ moment windows (Boss.hpp:586-627)."""
    out = []
    for comp, scale in ((0, 1.0), (1, 0.5), (2, -0.8)):
        out.append(cases.WindowSource(N.PN_SOURCE_MOMENT, 0, comp, center, radius, ds, t, v * scale))
    return out


@pytest.mark.parametrize("prec", ["f64_exact", "f64", "df64", "f32"])
def test_moment_and_force_sources(cuda_device, prec):
    """HostUTModel: a water column (moments) plus two transducers."""
    c = cases.al_plate_case(nx=14, ny=12, nz=4, nsteps=50, radius=0.4e-3, n_sensors=6)
    h = c.meta["h"]
    t, v = c.sources[0].times, c.sources[0].values
    src = water_column_sources((0.7e-3, 0.6e-3, 0.4e-3), 0.35e-3, h, t, v)
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 0, 2, (0.5e-3, 0.5e-3, 0.4e-3), 0.3e-3, h, t, v))
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 1, 0, (0.9e-3, 0.6e-3, 0.4e-3), 0.3e-3, h, t, -v))
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 1, 2, (0.9e-3, 0.6e-3, 0.4e-3), 0.3e-3, h, t, v))
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, src, c.nsteps, c.sensors)
    dev, _ = run_dev(c.mesh, c, c.dt, src, c.nsteps, c.sensors, prec)
    compare(prec, dev, ref)
    assert np.abs(ref["S"][0]).max() > 0


@pytest.mark.parametrize("prec", ["f64_exact", "f64"])
def test_chunked_solve_equals_single(cuda_device, plate, prec):
    c = plate
    a, ta = run_dev(c.mesh, c, c.dt, c.sources, 40, c.sensors, prec)
    b, tb = run_dev(c.mesh, c, c.dt, c.sources, 40, c.sensors, prec, chunks=[1] * 7 + [13, 20])
    assert ta == tb
    for k in range(3):
        assert np.array_equal(a[0][k], b[0][k])
    assert np.array_equal(a[2], b[2])


def test_partition_ownership(cuda_device):
    """Nodes homed on another partition are never updated (HostRSGTDUT.hpp:339)."""
    c = cases.al_plate_case(nx=10, ny=8, nz=3, nsteps=10, radius=0.3e-3, n_sensors=4)
    m = c.mesh
    m.node_owner = (m.node_ijk[:, 0] >= 7).astype(np.int32)  # x >= 7 on partition 1
    m.partition_id = 0
    V0, S0 = random_state(m, 5)
    ref = oracle.run(m, c.material_fields(), c.dt, c.sources, 10, c.sensors, V0=V0, S0=S0)
    dev, _ = run_dev(m, c, c.dt, c.sources, 10, c.sensors, "f64_exact", V0=V0, S0=S0)
    compare("f64_exact", dev, ref)
    off = m.node_owner == 1
    assert np.array_equal(dev[0][0][off], V0[0][off])
    m.node_owner = None


def test_zero_steps_and_state_roundtrip(cuda_device, plate):
    c = plate
    V0, S0 = random_state(c.mesh, 2)
    with Solver(c.mesh, c, c.dt, "f64") as s:
        s.set_state(V0, S0)
        assert s.solve(0) == 0.0
        V, S = s.get_state()
    for k in range(3):
        assert np.array_equal(V[k], V0[k])
    for k in range(6):
        assert np.array_equal(S[k], S0[k])


def test_info_bytes(cuda_device, plate):
    c = plate
    with Solver(c.mesh, c, c.dt, "f64", "table") as s:
        inf = s.info()
    assert inf["uniform_spacing"] == 1 and inf["form_name"] == "table"
    assert inf["algorithmic_bytes_per_step"] == c.mesh.n_cells * 180 + c.mesh.n_nodes * 112
    with Solver(c.mesh, c, c.dt, "f32", "table") as s:
        assert s.info()["algorithmic_bytes_per_step"] == c.mesh.n_cells * 108 + c.mesh.n_nodes * 72
    with Solver(c.mesh, c, c.dt, "f64") as s:  # a voxel plate gets the grid form
        inf = s.info()
    assert inf["form_name"] == "grid" and inf["grid"] == (16, 16, 4)
    assert inf["algorithmic_bytes_per_step"] == c.mesh.n_cells * 97 + c.mesh.n_nodes * 56


@pytest.mark.parametrize("form", ["grid", "table"])
@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_state_transfer_pinned_and_pageable_agree(cuda_device, plate, prec, form):
    """set_state / get_state read and write page-locked caller buffers
    directly (aligned or not) and stage any other memory: all give the same
    bits."""
    import torch
    c = plate
    V0, S0 = random_state(c.mesh, 5)

    def buf(n, pin, shift):
        # page-locked or not; shift 1: starts 8 bytes past a 16-byte boundary
        return torch.empty(n + shift, dtype=torch.float64, pin_memory=pin).numpy()[shift:]

    def copy_of(a, pin, shift):
        t = buf(a.size, pin, shift)
        t[:] = a
        return t

    out = []
    for pin, shift in ((False, 0), (True, 0), (True, 1)):
        Vi = [copy_of(a, pin, shift) for a in V0]
        Si = [copy_of(a, pin, shift) for a in S0]
        with Solver(c.mesh, c, c.dt, prec, form) as s:
            s.set_state(Vi, Si)
            s.solve(3)
            Vo = [buf(c.mesh.n_nodes, pin, shift) for _ in range(3)]
            So = [buf(c.mesh.n_cells, pin, shift) for _ in range(6)]
            s.get_state_into(Vo, So)
        out.append([x.copy() for x in Vo + So])
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("form", ["grid", "table"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_non_finite_state_is_refused_and_changes_nothing(cuda_device, plate, prec, form):
    """set_state refuses NaN and infinity (PN_ERR_NOT_FINITE, naming the
    field) and leaves the solver's state as it was: the solve goes on with
    the same bits as a solver that never saw the call."""
    c = plate
    V0, S0 = random_state(c.mesh, 6)
    results = []
    for poison in (False, True):
        with Solver(c.mesh, c, c.dt, prec, form) as s:
            s.set_state(V0, S0)
            s.solve(2)
            if poison:
                badV = [v.copy() for v in V0]
                badV[1][7] = np.nan
                with pytest.raises(N.PnError) as e:
                    s.set_state(badV, S0)
                assert e.value.code == N.PN_ERR_NOT_FINITE and "velocity" in e.value.msg
                badS = [x.copy() for x in S0]
                badS[3][-1] = np.inf
                with pytest.raises(N.PnError) as e:
                    s.set_state(V0, badS)
                assert e.value.code == N.PN_ERR_NOT_FINITE and "stress" in e.value.msg
            s.solve(3)
            results.append(s.get_state())
    for a, b in zip(results[0][0] + results[0][1], results[1][0] + results[1][1]):
        assert np.array_equal(a, b)
