"""pn_batch_solve_noalloc: the batch solve staged in the library's fixed
device scratch instead of buffers grown with cudaMalloc.  Two calls in a row
give bit-identical fields, traces and times to pn_batch_solve on twin
batches; batches too large for the scratch and members whose tables are not
built yet are refused with PN_ERR_INVALID.  Collected last (file name), and
independent of what ran before it."""
import numpy as np
import pytest

from pannde_gb300 import _native as N
from pannde_gb300 import cases
from pannde_gb300.solver import Batch, Solver

pytestmark = pytest.mark.gpu


def members():
    return [cases.al_plate_case(nx=40, ny=19, nz=5, nsteps=30, radius=0.6e-3, n_sensors=5),
            cases.laminate_case(nx=33, ny=29, nz=8, nsteps=30, radius=0.5e-3, n_sensors=4),
            cases.al_plate_case(nx=12, ny=70, nz=3, nsteps=30, radius=0.3e-3, n_sensors=3, seed=9)]


def snapshot(s):
    return s.get_state(), s.traces(), s.time


def same(a, b):
    (Va, Sa), ta, tta = a
    (Vb, Sb), tb, ttb = b
    assert tta == ttb
    for k in range(3):
        assert np.array_equal(Va[k], Vb[k]), f"V{k}"
    for k in range(6):
        assert np.array_equal(Sa[k], Sb[k]), f"S{k}"
    assert np.array_equal(ta, tb)


@pytest.mark.parametrize("form,prec", [("grid", "f32"), ("grid", "df64"), ("table", "f32"), ("table", "f64")])
def test_two_calls_match_batch_solve(cuda_device, form, prec):
    cs = members()
    grown = [Solver.from_case(c, precision=prec, form=form, capacity=30) for c in cs]
    fixed = [Solver.from_case(c, precision=prec, form=form, capacity=30) for c in cs]
    with Batch() as a, Batch() as b:
        for s in grown:
            a.add(s)
        for s in fixed:
            b.add(s)
        # one ordinary step builds the members' source and signal tables
        a.solve(1)
        b.solve(1)
        a.solve(7)
        a.solve(12)
        b.solve_noalloc(7)
        b.solve_noalloc(12)
    for x, y in zip(grown, fixed):
        same(snapshot(x), snapshot(y))
        assert abs(y.time - 20 * y.info()["dt"]) < 1e-20 + 1e-12 * y.time
        x.close()
        y.close()


def test_members_with_split_sites(cuda_device):
    """Grid-form members whose cracks split lattice sites (the staging then
    also holds the prefixes of their copies and fix cells) beside one
    without: two calls match pn_batch_solve."""
    cs = [cases.bracket_case(1000 + i, nsteps=30, water_column=(i == 0), scale=0.3) for i in range(2)]
    cs.append(members()[0])
    grown = [Solver.from_case(c, precision="f32", form="grid", capacity=30) for c in cs]
    fixed = [Solver.from_case(c, precision="f32", form="grid", capacity=30) for c in cs]
    with Batch() as a, Batch() as b:
        for s in grown:
            a.add(s)
        for s in fixed:
            b.add(s)
        a.solve(1)
        b.solve(1)
        a.solve(9)
        a.solve(10)
        b.solve_noalloc(9)
        b.solve_noalloc(10)
    for x, y in zip(grown, fixed):
        same(snapshot(x), snapshot(y))
        x.close()
        y.close()


def test_second_call_takes_no_device_memory(cuda_device):
    """After one warm call (which may load kernels lazily), a further call
    leaves the device's free memory where it was: nothing is allocated."""
    import torch
    cs = members()
    sv = [Solver.from_case(c, precision="f32", form="grid", capacity=40) for c in cs]
    try:
        with Batch() as b:
            for s in sv:
                b.add(s)
            b.solve(1)
            b.solve_noalloc(5)
            torch.cuda.synchronize()
            free0, _ = torch.cuda.mem_get_info()
            b.solve_noalloc(9)
            torch.cuda.synchronize()
            free1, _ = torch.cuda.mem_get_info()
        assert free1 >= free0, (free0, free1)
    finally:
        for s in sv:
            s.close()


def test_members_without_tables_are_refused(cuda_device):
    c = members()[0]
    with Solver.from_case(c, precision="f32", capacity=10) as s, Batch() as b:
        b.add(s)
        with pytest.raises(N.PnError) as e:
            b.solve_noalloc(3)
        assert e.value.code == N.PN_ERR_INVALID and "not built" in e.value.msg
        b.solve(1)  # builds them
        b.solve_noalloc(3)
        assert s.info()["time"] > 0


def test_batch_larger_than_scratch_is_refused(cuda_device):
    m = cases.voxel_mesh(np.ones((2, 2, 2), dtype=bool), 1e-4)
    c = cases.Case("tiny", m, np.array([2700.0]), cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None],
                   np.zeros(m.n_cells, np.int32), 1e-9)
    sv = []
    try:
        with Batch() as b:
            refused = False
            for k in range(400):
                s = Solver(m, c, c.dt, "f32", "grid")
                sv.append(s)
                b.add(s)
                try:
                    b.solve_noalloc(1)
                except N.PnError as e:
                    assert e.code == N.PN_ERR_INVALID and "more than the fixed 262144 bytes" in e.msg
                    refused = True
                    break
            assert refused and 200 < len(sv) < 400
            b.solve(1)  # the allocating solve takes any size
    finally:
        for s in sv:
            s.close()
