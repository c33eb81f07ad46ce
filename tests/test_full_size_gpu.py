"""Parity at the full sizes of the benchmarked workloads, through the C ABI.

Workloads:
  laminate      400 x 400 x 40 cells (6.4 M cells, 6.59 M nodes), plies
                [0/90/+45/-45]s, 500 kHz tone burst, 64 sensors: the headline
  holed plate   aluminium 1024 x 1024 x 24 cells with 12 through-holes
                (24.4 M cells, 25.5 M nodes), 1 MHz tone burst, 128 sensors

Checks:
* a short run from a random state (every cell and node carries a value) with
  the tone burst on, against the C oracle on the same inputs:
  bit-identical in f64_exact, relative L2 <= 1e-10 in f64 / df64, <= 1e-4 in
  f32, per field and per trace;
* 200 steps of the laminate's tone burst from rest against the oracle (the
  wave crosses about 60 cells);
* properties that hold at any run length: a repeated run gives the same bits
  (no races between blocks), and power-of-two homogeneity -- the signals and
  the initial state doubled give every output doubled.  Scaling by 2 is exact
  in binary floating point except where a value passes through the subnormal
  range (the wave's leading edge), so the doubled run must agree with twice
  the plain one to relative L2 <= 1e-15 (all forms).  A kernel that mixed
  values of different steps or blocks would fail it;
* the FP64 energy audit of the holed plate without sources: bounded, and the
  FP32 form's energy follows the FP64 form's within 1e-4;
* the batched workload: 96 seeded L-brackets (51 M cells in all, cracks as
  disconnected faces, every sixth with a water column), FP32, in one batch:
  every member bit-identical to its run alone, two members against the oracle
  (and bit-identical to it in exact mode).
"""
import dataclasses

import numpy as np
import pytest

import oracle
from pannde_gb300 import cases
from pannde_gb300.solver import Batch, Solver
from tests.test_energy_gpu import pulse_state
from tests.test_parity_gpu import compare, random_state, rel_l2, run_dev

pytestmark = pytest.mark.gpu

FORMS = [("f64_exact", "table"), ("f64", "grid"), ("df64", "grid"), ("f32", "grid"),
         ("f64", "table"), ("f32", "table")]


@pytest.fixture(scope="module")
def laminate():
    return cases.laminate_case()


@pytest.fixture(scope="module")
def laminate_random(laminate):
    c = laminate
    V0, S0 = random_state(c.mesh, 11)
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, 12, c.sensors, V0=V0, S0=S0)
    return V0, S0, ref


@pytest.fixture(scope="module")
def laminate_burst(laminate):
    c = laminate
    return oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, 200, c.sensors)


@pytest.mark.parametrize("prec,form", FORMS)
def test_laminate_random_state_matches_oracle(cuda_device, laminate, laminate_random, prec, form):
    c = laminate
    V0, S0, ref = laminate_random
    dev, t = run_dev(c.mesh, c, c.dt, c.sources, 12, c.sensors, prec, V0=V0, S0=S0, form=form)
    assert t == ref["time"]
    compare(prec, dev, ref)


@pytest.mark.parametrize("prec", ["f64_exact", "f64", "df64", "f32"])
def test_laminate_tone_burst_matches_oracle(cuda_device, laminate, laminate_burst, prec):
    c = laminate
    ref = laminate_burst
    dev, t = run_dev(c.mesh, c, c.dt, c.sources, 200, c.sensors, prec, chunks=[64, 64, 72],
                     form="table" if prec == "f64_exact" else "grid")
    assert t == ref["time"]
    compare(prec, dev, ref)
    assert np.abs(ref["traces"]).max() > 0  # the burst reached sensors


def doubled(sources):
    return [dataclasses.replace(s, values=2.0 * np.asarray(s.values, np.float64)) for s in sources]


@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_laminate_repeatable_and_homogeneous(cuda_device, laminate, prec):
    """1000 steps (1/5 of the benchmark's 5000) from a random state with the
    burst on: two plain runs give identical bits; the doubled run gives twice
    the plain one."""
    c = laminate
    V0, S0 = random_state(c.mesh, 12)
    runs = []
    for scale in (1.0, 1.0, 2.0):
        src = c.sources if scale == 1.0 else doubled(c.sources)
        (V, S, tr), _ = run_dev(c.mesh, c, c.dt, src, 1000, c.sensors, prec,
                                V0=[scale * v for v in V0], S0=[scale * s for s in S0], form="grid")
        runs.append((V, S, tr))
    a, b, d = runs
    for x, y in zip(a[0] + a[1] + [a[2]], b[0] + b[1] + [b[2]]):
        assert np.array_equal(x, y)
    errs = [rel_l2(y, 2.0 * x) for x, y in zip(a[0] + a[1] + [a[2]], d[0] + d[1] + [d[2]])]
    assert max(errs) <= 1e-15, max(errs)


@pytest.fixture(scope="module")
def holed():
    return cases.holed_plate_case()


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_holed_plate_random_state_matches_oracle(cuda_device, holed, prec):
    c = holed
    V0, S0 = random_state(c.mesh, 13)
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, 6, c.sensors, V0=V0, S0=S0)
    with Solver.from_case(c, precision=prec, form="grid") as s:
        assert s.info()["form_name"] == "grid"
        s.set_state(V0, S0)
        t = s.solve(6)
        dev = (*s.get_state(), s.traces())
    assert t == ref["time"]
    compare(prec, dev, ref)


def test_holed_plate_energy_audit(cuda_device, holed):
    """No sources, a smooth pulse: the FP64 audit stays within 2% over 600
    steps, and the FP32 form's energy follows the FP64 form's within 1e-4."""
    c = holed
    V0, S0 = pulse_state(c.mesh, width=6.0)
    tot = {}
    for prec in ("f64", "f32"):
        with Solver(c.mesh, c, c.dt, prec, "grid") as s:
            s.set_state(V0, S0)
            seq = [sum(s.energy())]
            for _ in range(6):
                s.solve(100)
                seq.append(sum(s.energy()))
            tot[prec] = np.array(seq)
    e64 = tot["f64"]
    assert e64[0] > 0
    assert np.all(np.abs(e64 - e64[0]) <= 0.02 * e64[0])
    assert np.max(np.abs(tot["f32"] - e64) / e64) <= 1e-4


def test_bracket_batch_full_size(cuda_device):
    steps = 40
    cs = [cases.bracket_case(1000 + i, nsteps=steps, water_column=(i % 6 == 0)) for i in range(96)]
    assert sum(c.mesh.n_cells for c in cs) > 50_000_000
    alone = []
    for c in cs:
        with Solver.from_case(c, precision="f32", capacity=steps) as s:
            s.solve(steps)
            alone.append((s.get_state(), s.traces(), s.time))
    sv = [Solver.from_case(c, precision="f32", capacity=steps) for c in cs]
    try:
        with Batch() as b:
            for s in sv:
                b.add(s)
            b.solve(17)
            b.solve(steps - 17)
        for s, ((V, S), tr, t) in zip(sv, alone):
            assert s.time == t
            Vb, Sb = s.get_state()
            for x, y in zip(V + S, Vb + Sb):
                assert np.array_equal(x, y)
            assert np.array_equal(s.traces(), tr)
    finally:
        for s in sv:
            s.close()
    for i in (0, 7):  # member 0 carries a water column
        c = cs[i]
        ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, steps, c.sensors)
        (V, S), tr, t = alone[i]
        assert t == ref["time"]
        compare("f32", (V, S, tr), ref)
        dev, t = run_dev(c.mesh, c, c.dt, c.sources, steps, c.sensors, "f64_exact")
        assert t == ref["time"]
        compare("f64_exact", dev, ref)
