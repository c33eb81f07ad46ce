"""The FP64 form's two paths (grid form, tensor-copy kernel): each block of a
step computes in double-float (48-bit significand on the FP32 pipes, double
storage) unless its tile or a neighbouring one stored a value outside the
double-float range in the previous step, or a source term of its layers lies
outside it, and then in IEEE double.  Every case is held to the FP64
contract with no floor: <= 1e-10 relative L2 per field component and per
trace against the oracle -- including traces made only of values far below
float's range (1e-200), which only the FP64 path keeps -- and the path
counters show which paths ran."""
import numpy as np
import pytest

import oracle
from pannde_gb300 import cases
from pannde_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def run(case, V0, S0, steps, sensors, monkeypatch=None, fp64_only=False):
    if fp64_only:
        monkeypatch.setenv("PN_F64_PATH", "fp64")
    with Solver(case.mesh, case, case.dt, "f64", "grid") as s:
        if monkeypatch is not None and fp64_only:
            monkeypatch.delenv("PN_F64_PATH")
        s.set_state(V0, S0)
        if case.sources:
            s.add_sources(case.sources)
        s.set_sensors(sensors, steps)
        s.solve(steps // 3)
        s.solve(steps - steps // 3)
        V, S = s.get_state()
        return V, S, s.traces(), s.path_counts()


def check(case, V0, S0, steps, sensors):
    ref = oracle.run(case.mesh, case.material_fields(), case.dt, case.sources, steps, sensors, V0=V0, S0=S0)
    V, S, tr, counts = run(case, V0, S0, steps, sensors)
    errs = [rel(V[k], ref["V"][k]) for k in range(3)] + [rel(S[k], ref["S"][k]) for k in range(6)]
    errs += [rel(tr[:, i], ref["traces"][:, i]) for i in range(tr.shape[1])]
    assert max(errs) <= 1e-10, max(errs)
    return counts, ref, (V, S, tr)


def plate():
    return cases.al_plate_case(nx=96, ny=40, nz=6, nsteps=30, radius=0.8e-3, n_sensors=4)


def test_developed_state_takes_double_float(cuda_device):
    """A random state of ordinary magnitudes: set_state flags no tile (every
    value is inside the double-float range), so the blocks take the
    double-float path from the first step."""
    c = plate()
    rng = np.random.default_rng(3)
    V0 = [rng.uniform(-1e-3, 1e-3, c.mesh.n_nodes) for _ in range(3)]
    S0 = [rng.uniform(-1e5, 1e5, c.mesh.n_cells) for _ in range(6)]
    counts, _, _ = check(c, V0, S0, 30, c.sensors)
    fp64, df = counts
    assert df > 0 and df > 5 * fp64, counts


def test_values_far_below_float_range_stay_exact(cuda_device):
    """Half the plate holds values near 1e-200 (far outside double-float's
    range), the other half ordinary ones; sensors sit in both halves and
    every trace, tiny or not, meets the FP64 contract without a floor."""
    c = plate()
    rng = np.random.default_rng(5)
    x = c.mesh.x
    xn = x / x.max()
    xc = c.mesh.x[c.mesh.hexes].mean(axis=1) / x.max()
    scale_n = np.where(xn < 0.5, 1e-3, 1e-200)
    scale_c = np.where(xc < 0.5, 1e5, 1e-195)
    V0 = [rng.uniform(-1, 1, c.mesh.n_nodes) * scale_n for _ in range(3)]
    S0 = [rng.uniform(-1, 1, c.mesh.n_cells) * scale_c for _ in range(6)]
    top = np.flatnonzero(c.mesh.z == c.mesh.z.max())
    far = top[c.mesh.x[top] > 0.9 * x.max()][:3]
    near = top[c.mesh.x[top] < 0.1 * x.max()][:3]
    sens = np.concatenate([far, near]).astype(np.int32)
    case = cases.Case(c.name, c.mesh, c.density, c.cij, c.cell_material, c.dt, [], sens, 20)
    counts, ref, _ = check(case, V0, S0, 20, sens)
    assert np.abs(ref["traces"][:, :3]).max() < 1e-150  # the far traces are tiny throughout
    fp64, df = counts
    assert fp64 > 0 and df > 0, counts


def test_tone_burst_front_matches_fp64_path(cuda_device, monkeypatch):
    """From rest with a tone burst: the stencil's leakage ahead of the wave
    (values down to the double's subnormals) on the FP64 path, the wave on the
    double-float path; fields and traces within 1e-10 of the oracle and of the
    FP64-only kernel."""
    c = cases.al_plate_case(nx=64, ny=64, nz=8, nsteps=60, radius=1.0e-3, n_sensors=12, seed=11)
    zero_v = [np.zeros(c.mesh.n_nodes) for _ in range(3)]
    zero_s = [np.zeros(c.mesh.n_cells) for _ in range(6)]
    counts, ref, (V, S, tr) = check(c, zero_v, zero_s, 60, c.sensors)
    V2, S2, tr2, c2 = run(c, zero_v, zero_s, 60, c.sensors, monkeypatch, fp64_only=True)
    assert c2 == (0, 0)  # no path choice in the FP64-only kernel
    for k in range(3):
        assert rel(V[k], V2[k]) <= 1e-10
    for i in range(tr.shape[1]):
        assert rel(tr[:, i], tr2[:, i]) <= 1e-10
    assert counts[1] > 0, counts


def test_set_state_flags_only_the_tiles_it_must(cuda_device):
    """set_state flags the tiles of its out-of-range values for the first
    step (and the neighbours that read their edges): the rest start on the
    double-float path at once.  96 x 40 x 6 cells = 4 x 6 tile columns, one
    block each; values near 1e-200 in the last four node columns (the tiles
    of bx = 3, whose first column the tiles of bx = 2 read)."""
    c = plate()
    V0 = [np.zeros(c.mesh.n_nodes) for _ in range(3)]
    S0 = [np.zeros(c.mesh.n_cells) for _ in range(6)]
    rng = np.random.default_rng(9)
    far = np.flatnonzero(c.mesh.x > c.mesh.x.max() - 3.5 * 0.1e-3)
    V0[2][far] = rng.uniform(-1, 1, far.size) * 1e-200
    with Solver(c.mesh, c, c.dt, "f64", "grid") as s:
        s.set_state(V0, S0)
        s.solve(1)
        fp64, df = s.path_counts()
    assert fp64 + df == 24, (fp64, df)
    assert fp64 == 12 and df == 12, (fp64, df)
