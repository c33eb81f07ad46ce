"""Long runs against the CPU oracle: every recorded trace and the final
fields, relative L2.

* the plate workload in full: aluminium 64x64x8 cells (0.1 mm), 1 MHz
  5-cycle tone burst on a 2 mm radius patch, dt = 0.5 x CFL, 2000 steps,
  16 seeded top-face sensors;
* a laminate proxy: [0/90/+45/-45]s plies, 48x48x40 cells, 500 kHz burst,
  1500 steps, 16 sensors.

Bounds: FP64 and double-float forms 1e-10 on every trace and field (the
FP64 drop-in contract); FP32 1e-4.
"""
import numpy as np
import pytest

import oracle
from pannde_gb300 import cases
from pannde_gb300.solver import Solver

pytestmark = pytest.mark.gpu

BOUND = {"f64": 1e-10, "df64": 1e-10, "f32": 1e-4}


def rel_l2(a, b):
    d = np.linalg.norm(b)
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / (d if d > 0 else 1.0))


def run_both(case):
    ref = oracle.run(case.mesh, case.material_fields(), case.dt, case.sources, case.nsteps,
                     case.sensors)
    out = {}
    for prec in BOUND:
        with Solver.from_case(case, precision=prec) as s:
            s.solve(case.nsteps)
            V, S = s.get_state()
            tr = s.traces()
        trace_err = [rel_l2(tr[:, i], ref["traces"][:, i]) for i in range(tr.shape[1])]
        field_err = [rel_l2(V[k], ref["V"][k]) for k in range(3)] + \
                    [rel_l2(S[k], ref["S"][k]) for k in range(6)]
        out[prec] = (max(trace_err), max(field_err))
    return out


@pytest.fixture(scope="module")
def plate_errors():
    return run_both(cases.al_plate_case())


@pytest.fixture(scope="module")
def laminate_errors():
    return run_both(cases.laminate_case(nx=48, ny=48, nz=40, nsteps=1500, n_sensors=16))


@pytest.mark.parametrize("prec", list(BOUND))
def test_plate_2000_steps(cuda_device, plate_errors, prec):
    tr, fld = plate_errors[prec]
    print(f"plate {prec}: worst trace rel L2 {tr:.3e}, worst field {fld:.3e}")
    assert tr <= BOUND[prec] and fld <= BOUND[prec]


@pytest.mark.parametrize("prec", list(BOUND))
def test_laminate_1500_steps(cuda_device, laminate_errors, prec):
    tr, fld = laminate_errors[prec]
    print(f"laminate {prec}: worst trace rel L2 {tr:.3e}, worst field {fld:.3e}")
    assert tr <= BOUND[prec] and fld <= BOUND[prec]
