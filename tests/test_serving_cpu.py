"""The serving loop's host logic on CPU (pannde_gb300.serving.Server), with
stand-ins for the device solver, the batch and the footprint planner:
requests are admitted in arrival order only while their footprints fit the
HBM budget, requests that arrive while others run join the running batch,
quanta end exactly when the next admitted request finishes, every request
runs exactly its own step count, and its memory is released at the end."""
import threading
import time

import numpy as np
import pytest

from pannde_gb300 import cases, serving


class FakeSolver:
    live = 0
    lock = threading.Lock()

    def __init__(self, case, nsteps):
        self.case, self.nsteps, self.steps, self.time = case, nsteps, 0, 0.0
        with FakeSolver.lock:
            FakeSolver.live += 1

    @classmethod
    def from_case(cls, case, precision="f32", capacity=None, **kw):
        return cls(case, capacity)

    def traces(self):
        return np.full((self.steps, 1, 3), float(self.steps))

    def close(self):
        with FakeSolver.lock:
            FakeSolver.live -= 1


class FakeBatch:
    log = []

    def __init__(self):
        self.members = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def set_stream(self, stream):
        pass

    def add(self, s):
        self.members.append(s)

    def remove(self, s):
        self.members.remove(s)

    def solve(self, n):
        assert n > 0 and self.members
        FakeBatch.log.append((n, len(self.members)))
        time.sleep(n * 1e-4)  # 0.1 ms per step, so later arrivals find requests running
        for s in self.members:
            s.steps += n
            s.time += n * s.case.dt
            assert s.steps <= s.nsteps  # a quantum never runs a request past its end


FOOT = 100  # bytes per request in the stand-in planner


@pytest.fixture
def fake(monkeypatch):
    FakeSolver.live = 0
    FakeBatch.log = []
    used = {"now": 0, "peak": 0}
    monkeypatch.setattr(serving, "Solver", FakeSolver)
    monkeypatch.setattr(serving, "Batch", FakeBatch)
    monkeypatch.setattr(serving, "plan_bytes", lambda case, precision, form="auto": FOOT)
    monkeypatch.setattr(serving, "_new_stream", lambda: None)
    monkeypatch.setattr(serving, "_current_device", lambda: None)
    return used


def request(rid, arrival, nsteps):
    c = cases.al_plate_case(nx=4, ny=3, nz=2, nsteps=nsteps, n_sensors=1)
    return serving.Request(rid, arrival, c, nsteps)


def test_requests_overlap_and_run_their_own_steps(fake):
    reqs = [request(0, 0.0, 700), request(1, 0.01, 300), request(2, 0.02, 1000), request(3, 0.5, 200)]
    srv = serving.Server(hbm_budget_bytes=10 * FOOT, precision="f32", quantum=250, prepare_ahead=4)
    res, st = srv.run(reqs)
    assert [r.rid for r in res] == [0, 1, 2, 3]
    for r, q in zip(res, reqs):
        assert r.nsteps == q.nsteps and r.traces.shape[0] == q.nsteps
        assert r.finished >= r.admitted >= r.arrival - 1e-9
    assert st["max_active"] >= 2  # requests that arrived while others ran joined the batch
    assert max(n for n, _ in FakeBatch.log) <= 250
    assert FakeSolver.live == 0  # every solver closed


def test_budget_limits_admission(fake):
    """With room for one request's footprint the requests run one at a time."""
    reqs = [request(k, 0.0, 120) for k in range(3)]
    srv = serving.Server(hbm_budget_bytes=FOOT, precision="f32", quantum=50, prepare_ahead=2)
    res, st = srv.run(reqs)
    assert st["max_active"] == 1 and all(m == 1 for _, m in FakeBatch.log)
    assert sorted(r.rid for r in res) == [0, 1, 2] and FakeSolver.live == 0


def test_request_larger_than_the_budget_is_refused(fake):
    srv = serving.Server(hbm_budget_bytes=FOOT - 1, precision="f32")
    with pytest.raises(ValueError, match="more than the budget"):
        srv.run([request(0, 0.0, 10)])
