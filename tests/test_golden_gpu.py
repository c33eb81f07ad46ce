"""The device path against the reference's own outputs, directly.

tests/golden/*.npz hold inputs and outputs of the reference HostSolver
(HostRSGTDUT::solve, HostRSGTDUT.hpp:162-169, and HostUTModel::solve,
HostUTModel.hpp:186-193) compiled from its own headers and run on small
seeded cases (tests/golden/make_golden.py):
  rsgtdut_plate          TransducerModel's path: plate, z-force transducer, sensors
  utmodel_holes_moments  WaterColumnModel's path: holed, graded, anisotropic block,
                         water-column moments and two transducers, random state
  fields_ownership       NODE/CONSTANT material fields and partition ownership
Each runs through the C ABI in every arithmetic form, in the table form and,
where the mesh is a uniform lattice, in the grid form, and is compared with
the fixture itself (not with the oracle):
  f64_exact  bit-identical fields, traces and time
  f64, df64  <= 1e-10 relative L2 per field component and per trace
  f32        <= 1e-4
with the floors of tests/test_parity_gpu.py (double-float and FP32 hold
FP32's exponent range; pure round-off components).
"""
from pathlib import Path

import numpy as np
import pytest

from pannde_gb300 import _native as N
from pannde_gb300.solver import Solver
from tests.golden.make_golden import load
from tests.test_parity_gpu import compare

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = ["rsgtdut_plate", "utmodel_holes_moments", "fields_ownership"]
PRECS = ["f64_exact", "f64", "df64", "f32"]


@pytest.fixture(scope="module", params=FIXTURES)
def golden(request):
    return load(GOLDEN / f"{request.param}.npz")


def run_fixture(g, prec, form):
    with Solver(g["mesh"], g["material"], g["dt"], prec, form) as s:
        if g["V0"] is not None:
            s.set_state(g["V0"], g["S0"])
        if g["sources"]:
            s.add_sources(g["sources"])
        sens = np.asarray(g["sensors"], np.int32)
        if sens.size:
            s.set_sensors(sens, g["nsteps"])
        t = s.solve(g["nsteps"])
        V, S = s.get_state()
        tr = s.traces() if sens.size else None
        used = s.info()["form_name"]
    return (V, S, tr), t, used


@pytest.mark.parametrize("prec", PRECS)
def test_table_form_matches_reference(cuda_device, golden, prec):
    dev, t, used = run_fixture(golden, prec, "table")
    assert used == "table"
    assert t == golden["time"]
    compare(prec, dev, golden)
    assert np.abs(golden["V"]).max() > 0


@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_grid_form_matches_reference(cuda_device, golden, prec):
    try:
        dev, t, used = run_fixture(golden, prec, "grid")
    except N.PnError as e:  # graded spacing or a non-lattice mesh: the table form's case
        assert e.code == N.PN_ERR_INVALID
        pytest.skip(f"not a uniform lattice: {e.msg}")
    assert used == "grid"
    assert t == golden["time"]
    compare(prec, dev, golden)


def test_some_fixture_takes_the_grid_form(cuda_device):
    """At least the plate (TransducerModel's path) runs in the grid form."""
    g = load(GOLDEN / "rsgtdut_plate.npz")
    _, _, used = run_fixture(g, "f64", "auto")
    assert used == "grid"
