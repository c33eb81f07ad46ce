"""Block-tile shapes of the tensor-copy grid kernel: 32 x 16 tiles (FP32
storage) give bit-identical fields, traces and times to 32 x 8 tiles, for a
single solver (tile rows chosen at creation, PN_GRID_TILE_ROWS) and for
batches whose launch-shape tuner re-tiles the members while it tries
(rows, z-chunk) candidates; the tuner's choice is reported by
pn_batch_plan_stats.  Sources on tile seams, moments, sensors and cracks as
split lattice sites are covered."""
import numpy as np
import pytest

from pannde_gb300 import cases
from pannde_gb300.solver import Batch, Solver
from tests.test_batch_gpu import same

pytestmark = pytest.mark.gpu


def run_alone(case, rows, steps, monkeypatch, prec="f32"):
    monkeypatch.setenv("PN_GRID_TILE_ROWS", str(rows))
    with Solver.from_case(case, precision=prec, form="grid", capacity=steps) as s:
        s.solve(steps // 2)
        s.solve(steps - steps // 2)
        out = s.get_state(), s.traces(), s.time
    monkeypatch.delenv("PN_GRID_TILE_ROWS")
    return out


@pytest.mark.parametrize("case", [
    lambda: cases.laminate_case(nx=70, ny=45, nz=16, nsteps=30, radius=0.6e-3, n_sensors=9),
    lambda: cases.al_plate_case(nx=33, ny=31, nz=5, nsteps=30, radius=0.5e-3, n_sensors=7),
    lambda: cases.bracket_case(1002, nsteps=30, water_column=True, scale=0.3),
], ids=["laminate", "plate", "bracket_crack_water"])
def test_sixteen_rows_equal_eight(cuda_device, monkeypatch, case):
    c = case()
    same(run_alone(c, 16, 30, monkeypatch), run_alone(c, 8, 30, monkeypatch))


def test_eight_byte_storage_keeps_eight_rows(cuda_device, monkeypatch):
    """Double-float storage has no 32 x 16 kernel: the request is ignored."""
    c = cases.al_plate_case(nx=20, ny=20, nz=4, nsteps=10, radius=0.5e-3, n_sensors=3)
    same(run_alone(c, 16, 10, monkeypatch, prec="df64"), run_alone(c, 8, 10, monkeypatch, prec="df64"))


def test_batch_tuner_retiles_members(cuda_device, monkeypatch):
    """A chunk long enough for tuning tries 8- and 16-row tiles (members
    re-tiled in between); every member still equals its run alone, and the
    shape in use is reported."""
    cs = [cases.laminate_case(nx=70, ny=45, nz=16, nsteps=80, radius=0.6e-3, n_sensors=5),
          cases.bracket_case(1003, nsteps=80, water_column=False, scale=0.3),
          cases.al_plate_case(nx=64, ny=40, nz=6, nsteps=80, radius=0.5e-3, n_sensors=4, seed=4)]
    ref = [run_alone(c, 8, 80, monkeypatch) for c in cs]
    sv = [Solver.from_case(c, precision="f32", form="grid", capacity=80) for c in cs]
    with Batch() as b:
        for s in sv:
            b.add(s)
        b.solve(30)  # 2 rounds x 6 shapes x 2 steps + 1: tuned in this chunk
        st = b.plan_stats()
        assert st["tuned_classes"] >= 1
        assert st["tile_rows"] in (8, 16) and st["shape"] in (0, 1, 2)
        b.solve(25)
        b.solve(25)
    for s, r in zip(sv, ref):
        same((s.get_state(), s.traces(), s.time), r)
        s.close()


def test_noalloc_keeps_the_tuned_tiling(cuda_device, monkeypatch):
    """After a tuned pn_batch_solve the allocation-free call runs with the
    members' tiling as it is (no re-tiling, which would allocate)."""
    cs = [cases.laminate_case(nx=70, ny=45, nz=16, nsteps=60, radius=0.6e-3, n_sensors=5),
          cases.al_plate_case(nx=64, ny=40, nz=6, nsteps=60, radius=0.5e-3, n_sensors=4, seed=4)]
    ref = [run_alone(c, 8, 60, monkeypatch) for c in cs]
    sv = [Solver.from_case(c, precision="f32", form="grid", capacity=60) for c in cs]
    with Batch() as b:
        for s in sv:
            b.add(s)
        b.solve(30)
        rows = b.plan_stats()["tile_rows"]
        b.solve_noalloc(30)
        assert b.plan_stats()["tile_rows"] == rows
    for s, r in zip(sv, ref):
        same((s.get_state(), s.traces(), s.time), r)
        s.close()
