"""Failure detection without a GPU fault: the tensor-copy grid kernel bounds
every wait for its staged tiles (about one second).  A test hook leaves one
layer's copies unissued, so that wait runs out: the kernel records the
solver's device error word, drains its own copies in flight and returns; the
host reports PN_ERR_DEVICE_CHECK at the next synchronising call, and the
context stays usable for the next solver."""
import numpy as np
import pytest

import oracle
from pannde_gb300 import _native as N
from pannde_gb300 import cases
from pannde_gb300.solver import Solver
from tests.test_parity_gpu import compare

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_is_reported_and_context_survives(cuda_device, monkeypatch):
    c = cases.al_plate_case(nx=20, ny=6, nz=3, nsteps=5, radius=0.4e-3, n_sensors=2)
    monkeypatch.setenv("PN_TEST_GRID_SKIP_COPY", "1")
    with Solver.from_case(c, precision="f32", form="grid") as s:
        assert s.info()["kernel_name"] == "tma"
        s.solve(1)  # enqueued; the wait for layer 1 gives up on the device
        with pytest.raises(N.PnError) as e:
            s.synchronize()
        assert e.value.code == N.PN_ERR_DEVICE_CHECK and "gave up" in e.value.msg
        s.synchronize()  # the word was cleared
    monkeypatch.delenv("PN_TEST_GRID_SKIP_COPY")
    ref = oracle.run(c.mesh, c.material_fields(), c.dt, c.sources, c.nsteps, c.sensors)
    with Solver.from_case(c, precision="f32", form="grid") as s:
        s.solve(c.nsteps)
        V, S = s.get_state()
        compare("f32", (V, S, s.traces()), ref)
