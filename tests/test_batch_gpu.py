"""Batches (pn_batch_*): every member's fields, traces and time are
bit-identical whether it runs alone or in a batch, for both device forms and
the three fast precisions, including members that join and leave mid-way."""
import numpy as np
import pytest

from pannde_gb300 import cases
from pannde_gb300.solver import Batch, Solver

pytestmark = pytest.mark.gpu


def members():
    return [cases.al_plate_case(nx=40, ny=19, nz=5, nsteps=30, radius=0.6e-3, n_sensors=5),
            cases.laminate_case(nx=33, ny=29, nz=8, nsteps=30, radius=0.5e-3, n_sensors=4),
            cases.al_plate_case(nx=12, ny=70, nz=3, nsteps=30, radius=0.3e-3, n_sensors=3, seed=9)]


def alone(case, prec, form, steps):
    with Solver.from_case(case, precision=prec, form=form, capacity=steps) as s:
        for n in steps_list(steps):
            s.solve(n)
        return s.get_state(), s.traces(), s.time


def steps_list(total):
    return [total]


def same(a, b):
    (Va, Sa), ta, tta = a
    (Vb, Sb), tb, ttb = b
    assert tta == ttb
    for k in range(3):
        assert np.array_equal(Va[k], Vb[k]), f"V{k}"
    for k in range(6):
        assert np.array_equal(Sa[k], Sb[k]), f"S{k}"
    assert np.array_equal(ta, tb)


@pytest.mark.parametrize("form", ["grid", "table"])
@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_batch_equals_alone(cuda_device, prec, form):
    cs = members()
    ref = [alone(c, prec, form, 30) for c in cs]
    sv = [Solver.from_case(c, precision=prec, form=form, capacity=30) for c in cs]
    with Batch() as b:
        for s in sv:
            b.add(s)
        b.solve(11)
        b.solve(19)
    for s, r in zip(sv, ref):
        same((s.get_state(), s.traces(), s.time), r)
        s.close()


def test_batch_join_and_leave(cuda_device):
    """A member joins after 10 steps and another leaves after 20; each one's
    own step count decides its result."""
    cs = members()
    sv = [Solver.from_case(c, precision="df64", capacity=40) for c in cs]
    with Batch() as b:
        b.add(sv[0])
        b.add(sv[1])
        b.solve(10)
        b.add(sv[2])
        b.solve(10)
        b.remove(sv[0])
        b.solve(7)
    steps = [20, 27, 17]
    for s, c, n in zip(sv, cs, steps):
        same((s.get_state(), s.traces(), s.time), alone(c, "df64", "auto", n))
        s.close()


def test_batch_rejects_mixed_members(cuda_device):
    from pannde_gb300 import _native as N
    cs = members()
    a = Solver.from_case(cs[0], precision="f64")
    b32 = Solver.from_case(cs[1], precision="f32")
    ex = Solver.from_case(cs[2], precision="f64_exact")
    with Batch() as b:
        b.add(a)
        with pytest.raises(N.PnError):
            b.add(b32)
        with pytest.raises(N.PnError):
            b.add(ex)
    for s in (a, b32, ex):
        s.close()


@pytest.mark.parametrize("form", ["grid", "table"])
def test_tuned_shapes_and_graph_replay_keep_results(cuda_device, form):
    """On a created stream, equal chunks are captured once as a CUDA graph and
    replayed; the first chunk tunes the launch shape on real steps.  Results
    stay bit-identical to the members run alone."""
    import torch
    cs = members()
    ref = [alone(c, "f32", form, 100) for c in cs]
    sv = [Solver.from_case(c, precision="f32", form=form, capacity=100) for c in cs]
    stream = torch.cuda.Stream()
    with Batch() as b:
        b.set_stream(stream)
        for s in sv:
            b.add(s)
        for _ in range(4):
            b.solve(25)  # the first chunk tunes: 2 rounds x up to 6 shapes x 2 steps + 1
        st = b.plan_stats()
    assert st["tuned_classes"] == 1
    assert st["graph_captures"] == 1 and st["graph_launches"] >= 2
    for s, r in zip(sv, ref):
        same((s.get_state(), s.traces(), s.time), r)
        s.close()


@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_batch_cracked_brackets_grid(cuda_device, prec):
    """Grid-form members with split lattice sites (cracks as disconnected
    faces, one with a water column) beside a member without any: the batch's
    fix-up of split sites gives every member the same bits as alone."""
    cs = [cases.bracket_case(1000 + i, nsteps=30, water_column=(i == 0), scale=0.3) for i in range(3)]
    cs.append(members()[0])
    ref = [alone(c, prec, "grid", 30) for c in cs]
    sv = [Solver.from_case(c, precision=prec, form="grid", capacity=30) for c in cs]
    with Batch() as b:
        for s in sv:
            b.add(s)
        b.solve(11)
        b.solve(19)
    for s, r in zip(sv, ref):
        same((s.get_state(), s.traces(), s.time), r)
        s.close()
