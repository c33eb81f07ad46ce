"""Tail split of the tensor-copy grid kernel: when a one-chunk launch has a
last, partial wave of tile columns, those columns are cut into shorter
z-chunks (a 1D grid: whole columns first, then the tail's chunks).  Results
are bit-identical with the split off (PN_GRID_TAIL_CHUNKS=1), with the
launcher's choice and with forced cuts, down to one-layer chunks, in every
storage form -- the FP64 form's per-tile path choice included -- and on a
holed plate whose tile columns stop at different heights."""
import numpy as np
import pytest

from pannde_gb300 import cases
from pannde_gb300.solver import Solver
from tests.test_batch_gpu import same

pytestmark = pytest.mark.gpu


def run(case, prec, steps, monkeypatch, cuts):
    if cuts is None:
        monkeypatch.delenv("PN_GRID_TAIL_CHUNKS", raising=False)
    else:
        monkeypatch.setenv("PN_GRID_TAIL_CHUNKS", str(cuts))
    with Solver.from_case(case, precision=prec, form="grid", capacity=steps) as s:
        s.solve(steps // 2)
        s.solve(steps - steps // 2)
        out = s.get_state(), s.traces(), s.time
    monkeypatch.delenv("PN_GRID_TAIL_CHUNKS", raising=False)
    return out


# 400 x 350 cells: 13 x 51 = 663 tile columns, more than one wave of resident
# blocks for every storage form (4 x 152 FP32, 3 x 152 with 8-byte storage)
def laminate():
    return cases.laminate_case(nx=400, ny=350, nz=8, nsteps=12, radius=0.8e-3, n_sensors=12)


@pytest.mark.parametrize("prec", ["f32", "df64", "f64"])
def test_split_equals_whole_columns(cuda_device, monkeypatch, prec):
    c = laminate()
    ref = run(c, prec, 12, monkeypatch, 1)
    same(run(c, prec, 12, monkeypatch, None), ref)
    same(run(c, prec, 12, monkeypatch, 8), ref)  # one-layer chunks


def test_split_holed_plate(cuda_device, monkeypatch):
    c = cases.holed_plate_case(nx=420, ny=360, nz=6, nsteps=10, n_holes=5, seed=11, n_sensors=16)
    ref = run(c, "f32", 10, monkeypatch, 1)
    same(run(c, "f32", 10, monkeypatch, 3), ref)
    same(run(c, "f32", 10, monkeypatch, None), ref)


def test_fp64_form_paths_with_split(cuda_device, monkeypatch):
    """From rest the FP64 form runs tiles near the source on the FP64 path;
    the tail's chunks of one column decide alike, and the step count per path
    sums to the blocks launched."""
    c = laminate()
    monkeypatch.setenv("PN_GRID_TAIL_CHUNKS", "4")
    with Solver.from_case(c, precision="f64", form="grid", capacity=12) as s:
        s.solve(12)
        fp64, dfl = s.path_counts()
        out = s.get_state(), s.traces(), s.time
    monkeypatch.delenv("PN_GRID_TAIL_CHUNKS")
    # every block counted once per step; the tail's columns in 4 chunks each
    assert (fp64 + dfl) % 12 == 0 and (fp64 + dfl) // 12 > 13 * 51
    assert fp64 > 0 and dfl > 0
    same(out, run(c, "f64", 12, monkeypatch, 1))
