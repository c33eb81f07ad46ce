"""Serving loop (continuous batching): requests that arrive while others run
join the batch; admission respects the HBM budget; every request's traces
equal the same request solved alone (bit for bit), and the FP32 serving
result stays within 1e-4 relative L2 of a double-float spot-check solve."""
import numpy as np
import pytest

from pannde_gb300 import serving
from pannde_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def small_requests(n=6, seed=3, gap=0.005, steps=(500, 900)):
    """Small plates arriving almost together: each runs for many quanta, so the
    later ones are prepared and admitted while the first ones are on the GPU."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        reqs.append(serving.mapod_request(i, gap * i, rng, cells_range=(2e4, 1.5e5), steps_range=steps))
    return reqs


def rel_l2(a, b):
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def test_results_same_alone_and_in_the_mix(cuda_device):
    reqs = small_requests()
    srv = serving.Server(hbm_budget_bytes=8 << 30, precision="f32", quantum=40, prepare_ahead=6)
    results, stats = srv.run(reqs)
    assert stats["requests"] == len(reqs) and stats["max_active"] >= 2
    for r, q in zip(results, sorted(reqs, key=lambda q: q.rid)):
        with Solver.from_case(q.case, precision="f32", capacity=q.nsteps) as s:
            s.solve(q.nsteps)
            tr = s.traces()
            assert s.time == r.final_time
        assert np.array_equal(tr, r.traces), f"request {q.rid}"
        assert r.latency >= 0


def test_admission_by_footprint(cuda_device):
    reqs = small_requests(5, seed=8)
    need = sorted(serving.plan_bytes(q.case, "f32") for q in reqs)
    budget = need[-1] + need[-2] - 1  # never the two largest together
    seen = []
    srv = serving.Server(hbm_budget_bytes=budget, precision="f32", quantum=30)
    results, stats = srv.run(reqs, on_admit=lambda r, now: seen.append(r.rid))
    assert stats["requests"] == len(reqs) and sorted(seen) == list(range(len(reqs)))


def test_fp32_spot_check_against_double_float(cuda_device):
    q = small_requests(1, seed=11)[0]
    out = {}
    for prec in ("f32", "df64"):
        with Solver.from_case(q.case, precision=prec, capacity=q.nsteps) as s:
            s.solve(q.nsteps)
            out[prec] = s.traces()
    errs = [rel_l2(out["f32"][:, i], out["df64"][:, i]) for i in range(out["f32"].shape[1])
            if np.abs(out["df64"][:, i]).max() > 0]
    assert errs and max(errs) <= 1e-4
