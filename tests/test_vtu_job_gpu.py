"""The device solver on the runners' own inputs.  A job file (.vtu, laid out
as the reference's case makers write it) is read back the way TransducerModel
and WaterColumnModel build their problem (pannde_gb300.vtu.read_*_job:
per-cell density and C11..C66, dt, excitation windows with the thickness of
cell 0), then solved through the C ABI and by the oracle on that same read
problem.  The oracle gives the same bits on the read problem as on the
problem that was written, so the file carries the solve exactly.
Tolerances as tests/test_parity_gpu.py: f64_exact bit-identical, f64 and
df64 1e-10, f32 1e-4 (relative L2 per field and per trace)."""
import numpy as np
import pytest

import oracle
from pannde_gb300 import cases, vtu
from tests.test_parity_gpu import compare, run_dev

pytestmark = pytest.mark.gpu


def check_job(c, read, path, write, prec_forms):
    write(path, c, [10 * c.dt, c.nsteps * c.dt], encoding="appended", compress=True)
    r = read(path, sensors=c.sensors, nsteps=c.nsteps)
    ref = oracle.run(r.mesh, r.material_fields(), r.dt, r.sources, r.nsteps, r.sensors)
    ref0 = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, c.nsteps, c.sensors)
    for a, b in zip(ref["V"] + ref["S"] + [ref["traces"]], ref0["V"] + ref0["S"] + [ref0["traces"]]):
        assert np.array_equal(a, b)
    assert np.abs(ref["traces"]).max() > 0
    for prec, form in prec_forms:
        dev, t = run_dev(r.mesh, r, r.dt, r.sources, r.nsteps, r.sensors, prec, form=form)
        assert t == ref["time"]
        compare(prec, dev, ref)


def test_transducer_job(cuda_device, tmp_path):
    c = cases.laminate_case(nx=40, ny=36, nz=8, nsteps=80, radius=0.6e-3, n_sensors=8)
    check_job(c, vtu.read_transducer_job, tmp_path / "laminate.vtu", vtu.write_transducer_job,
              [("f64_exact", "table"), ("f64", "auto"), ("df64", "auto"), ("f32", "auto"), ("f64", "table")])


def test_water_column_job(cuda_device, tmp_path):
    """An L-bracket with a water column and a crack as disconnected faces."""
    c = cases.bracket_case(7, water_column=True, scale=0.2, nsteps=200, n_sensors=8)
    check_job(c, vtu.read_water_column_job, tmp_path / "bracket.vtu", vtu.write_water_column_job,
              [("f64_exact", "table"), ("f64", "auto"), ("df64", "auto"), ("f32", "auto")])
