"""Sources given by the caller's own window predicate and per-step signal
values (pn_solver_add_window_masks + pn_solver_solve_signals, the path the C++
adapter uses for the reference's MultiVariate objects) reproduce the geometry
sources exactly: the window is HostNormalXDZ::checkAt restated in numpy at the
reference's cell centres / nodes, and the signal HostUnivariate::evalAt at the
accumulated step times."""
import numpy as np
import pytest

import oracle
from pannde_gb300 import _native as N
from pannde_gb300 import cases
from pannde_gb300.solver import Solver
from tests.test_parity_gpu import compare, water_column_sources

pytestmark = pytest.mark.gpu


def check_at(src, pts):
    """Stubs::HostNormalXDZ::checkAt (HostNormalXDZ.hpp:140-145, 174-177)."""
    d2 = (pts[:, 0] - src.center[0]) ** 2
    d2 = d2 + (pts[:, 1] - src.center[1]) ** 2
    d2 = d2 + (pts[:, 2] - src.center[2]) ** 2
    dist = np.sqrt(d2)
    distz = np.abs(pts[:, 2] - src.center[2])
    return ((distz <= 0.75 * src.ds) & (dist < src.radius) & (dist >= 0.)).astype(np.uint8)


def signal_values(srcs, dt, nsteps):
    from tests.test_capi_cpu import signal_eval
    t = np.zeros(nsteps)
    acc = 0.0
    for k in range(nsteps):  # time += dt in FP64, as solve() accumulates it
        t[k] = acc
        acc += dt
    cols = []
    for s in srcs:
        rc, v = signal_eval(s.times, s.values, t)
        assert rc == 0
        cols.append(v)
    return np.stack(cols, axis=1)


@pytest.mark.parametrize("prec,form", [("f64_exact", "table"), ("f64", "grid"), ("df64", "grid")])
def test_masks_reproduce_geometry_sources(cuda_device, prec, form):
    c = cases.al_plate_case(nx=37, ny=15, nz=4, nsteps=45, radius=0.5e-3, n_sensors=7)
    h = c.meta["h"]
    t, v = c.sources[0].times, c.sources[0].values
    src = list(c.sources) + water_column_sources((1.5e-3, 0.7e-3, 0.4e-3), 0.4e-3, h, t, v)
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, src, c.nsteps, c.sensors)
    centres = c.mesh.cell_centers()
    nodes = np.stack([c.mesh.x, c.mesh.y, c.mesh.z], axis=1)
    masks = [(s.kind, s.group, s.component,
              check_at(s, centres if s.kind == N.PN_SOURCE_FORCE else nodes)) for s in src]
    values = signal_values(src, c.dt, c.nsteps)
    with Solver(c.mesh, c, c.dt, prec, form) as s:
        s.add_window_masks(masks)
        s.set_sensors(c.sensors, c.nsteps)
        with pytest.raises(N.PnError):
            s.solve(1)  # mask sources need caller signal values
        tt = 0.0
        for a, b in ((0, 1), (1, 20), (20, c.nsteps)):
            tt = s.solve_signals(values[a:b])
        V, S = s.get_state()
        tr = s.traces()
    assert tt == ref["time"]
    compare(prec, (V, S, tr), ref)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_masks_on_split_sites(cuda_device, prec):
    """The same on a grid-form mesh whose crack (disconnected faces) splits
    lattice sites: mask forces on both faces' nodes and a mask moment on cells
    at the crack take the fix-up's lists."""
    from tests.test_grid_gpu import cracked_block
    c, lower, upper = cracked_block()
    m = c.mesh
    t = np.linspace(0.0, 2e-7, 60)
    v = np.sin(2e7 * t)
    src = [cases.WindowSource(N.PN_SOURCE_FORCE, 0, 2, (1.0e-3, 0.6e-3, 0.5e-3), 0.25e-3, 1e-4, t, v),
           cases.WindowSource(N.PN_SOURCE_MOMENT, 1, 1, (1.2e-3, 0.6e-3, 0.5e-3), 0.2e-3, 1e-4, t, v)]
    nsteps = 30
    sens = np.sort(np.concatenate([lower[::7], upper[::5]])).astype(np.int32)
    ref = oracle.run(m, c.material_fields(), c.dt, src, nsteps, sens)
    centres = m.cell_centers()
    nodes = np.stack([m.x, m.y, m.z], axis=1)
    masks = [(s.kind, s.group, s.component,
              check_at(s, centres if s.kind == N.PN_SOURCE_FORCE else nodes)) for s in src]
    values = signal_values(src, c.dt, nsteps)
    with Solver(m, c, c.dt, prec, "grid") as s:
        assert s.info()["form_name"] == "grid"
        s.add_window_masks(masks)
        s.set_sensors(sens, nsteps)
        tt = 0.0
        for a, b in ((0, 11), (11, nsteps)):
            tt = s.solve_signals(values[a:b])
        V, S = s.get_state()
        tr = s.traces()
    assert tt == ref["time"]
    compare(prec, (V, S, tr), ref)
