"""Serving loop for parametric (MAPOD-style) solves with continuous batching.

Requests arrive over time; each is a plate solve with its own mesh size,
material, transducer and step count.  The loop

* prepares an arrived request (its solver: host tables, device upload) on a
  background thread when its device footprint (pn_plan_solver, no
  allocation) fits in the free part of the HBM budget;
* admits prepared requests into the running batch while the GPU is not
  saturated, and advances every admitted request together (pn_batch_solve:
  one launch per step covers all of them), in quanta that end exactly when
  the next request finishes, so requests that arrive while others run join
  the batch at the next quantum;
* retires finished requests (downloads their sensor traces, frees their
  memory) and records their latency from arrival to completion.

A request's result does not depend on which other requests shared its
batches: members of a batch are computed independently.
"""
from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _native as N
from . import cases
from .solver import Batch, Solver, _precision


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    case: cases.Case
    nsteps: int
    meta: dict = field(default_factory=dict)


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    finished: float
    nsteps: int
    cells: int
    traces: np.ndarray
    final_time: float

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def plan_bytes(case: cases.Case, precision: str, form: str = "auto") -> int:
    """Device bytes pn_solver_create would allocate for this case (no GPU call)."""
    lib = N.load()
    m, keep = case.mesh.as_struct()
    tab, keep_t = case.material_table()
    out = N.PnPlan()
    N.check(lib.pn_plan_solver(ctypes.byref(m), None, ctypes.byref(tab), case.dt,
                               _precision(precision, form), ctypes.byref(out)))
    sensors = 3 * 8 * max(case.sensors.size, 1) * case.nsteps
    return int(out.device_bytes) + sensors + (1 << 20)


class Server:
    """Continuous-batching request loop on the current CUDA device.

    * ``prepare_threads`` preparation threads build the solvers of arrived
      requests (host tables, device upload, sources, sensors) while the GPU
      works on the admitted ones, each as soon as its footprint fits in the
      free HBM budget (taken in arrival order); at most ``prepare_ahead``
      prepared solvers wait for admission.
    * The GPU loop admits prepared solvers while the admitted set holds fewer
      than ``saturation_cells`` cells (one step launch over that many cells
      keeps the GPU busy; sharing it further only delays everyone), then
      advances the batch in quanta that end when the next request finishes.
    * A finished request's traces are read back, its memory freed, and its
      latency (arrival to traces) recorded.
    """

    def __init__(self, hbm_budget_bytes: int, precision: str = "f32", quantum: int = 250,
                 saturation_cells: int = 8_000_000, prepare_ahead: int = 2, prepare_threads: int = 2,
                 clock: Callable[[], float] = time.perf_counter):
        self.budget = int(hbm_budget_bytes)
        self.precision = precision
        self.quantum = int(quantum)
        self.saturation = int(saturation_cells)
        self.ahead = int(prepare_ahead)
        self.threads = max(1, int(prepare_threads))
        self.clock = clock

    def run(self, requests: list[Request], on_admit=None) -> tuple[list[Result], dict]:
        import queue
        import threading

        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        ready: "queue.Queue" = queue.Queue()
        lock = threading.Condition()
        state = dict(used=0, prepared=0, error=None, next=0)
        device = _current_device()
        t0 = self.clock()

        def prepare():
            try:
                _set_device(device)  # solvers live on the caller's current device
                while True:
                    with lock:  # the next request, in arrival order
                        if state["next"] >= len(pending) or state["error"] is not None:
                            return
                        r = pending[state["next"]]
                        state["next"] += 1
                    with lock:
                        while self.clock() - t0 < r.arrival:
                            lock.wait(timeout=min(0.05, max(0.001, r.arrival - (self.clock() - t0))))
                    need = plan_bytes(r.case, self.precision)
                    if need > self.budget:
                        raise ValueError(f"request {r.rid} needs {need} bytes, more than the budget")
                    with lock:
                        while (self.clock() - t0 < r.arrival or state["used"] + need > self.budget
                               or state["prepared"] >= self.ahead):
                            lock.wait(timeout=max(0.0, min(0.05, r.arrival - (self.clock() - t0))) or 0.01)
                        state["used"] += need
                        state["prepared"] += 1
                    s = Solver.from_case(r.case, precision=self.precision, capacity=r.nsteps)
                    ready.put((r, s, need))
            except BaseException as e:  # surfaced by the GPU loop
                state["error"] = e
                ready.put(None)

        workers = [threading.Thread(target=prepare, daemon=True) for _ in range(self.threads)]
        for th in workers:
            th.start()
        results: list[Result] = []
        active: dict[int, dict] = {}
        cell_steps = 0
        max_active = 0
        done = 0
        admitted = 0
        arrivals = [r.arrival for r in pending]
        queue_log: list[tuple[float, int]] = []  # (time, requests arrived and not yet admitted)

        def log_queue():
            now = self.clock() - t0
            arrived = int(np.searchsorted(arrivals, now, side="right"))
            queue_log.append((now, arrived - admitted))

        with Batch() as batch:
            stream = _new_stream()
            if stream is not None:  # a created stream: repeated quanta replay as CUDA graphs
                batch.set_stream(stream)
            while done < len(pending):
                # admit prepared solvers while the GPU is not saturated
                while True:
                    cells = sum(a["req"].case.mesh.n_cells for a in active.values())
                    if active and cells >= self.saturation:
                        break
                    try:
                        item = ready.get(timeout=0.05) if not active else ready.get_nowait()
                    except queue.Empty:
                        break
                    if item is None:
                        raise state["error"]
                    r, s, need = item
                    batch.add(s)
                    admitted += 1
                    now = self.clock() - t0
                    active[r.rid] = dict(req=r, solver=s, left=r.nsteps, need=need, admitted=now)
                    with lock:
                        state["prepared"] -= 1
                        lock.notify_all()
                    if on_admit:
                        on_admit(r, now)
                log_queue()
                if not active:
                    continue
                max_active = max(max_active, len(active))
                q = min(self.quantum, min(a["left"] for a in active.values()))
                batch.solve(q)
                cell_steps += q * sum(a["req"].case.mesh.n_cells for a in active.values())
                for rid in list(active):
                    a = active[rid]
                    a["left"] -= q
                    if a["left"] == 0:
                        s = a["solver"]
                        batch.remove(s)
                        tr = s.traces()
                        results.append(Result(rid, a["req"].arrival, a["admitted"], self.clock() - t0,
                                              a["req"].nsteps, a["req"].case.mesh.n_cells, tr, s.time))
                        s.close()
                        del active[rid]
                        done += 1
                        with lock:
                            state["used"] -= a["need"]
                            lock.notify_all()
        for th in workers:
            th.join(timeout=5.0)
        elapsed = self.clock() - t0
        lat = np.array([r.latency for r in results]) if results else np.zeros(1)
        stats = dict(requests=len(results), elapsed_s=elapsed,
                     sims_per_hour=len(results) / elapsed * 3600.0 if elapsed > 0 else 0.0,
                     p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                     gcell_steps_per_s=cell_steps / elapsed / 1e9 if elapsed > 0 else 0.0,
                     max_active=max_active, queue=queue_stats(queue_log, elapsed))
        return sorted(results, key=lambda r: r.rid), stats


def queue_stats(log: list[tuple[float, int]], elapsed: float) -> dict:
    """Admission queue depth (requests arrived and not yet admitted) from
    (time, depth) samples taken at every pass of the GPU loop, each held until
    the next sample: time-weighted mean, the share of the run with a
    non-empty queue, and the largest depth."""
    if not log or elapsed <= 0:
        return dict(mean_depth=0.0, nonempty_frac=0.0, max_depth=0, samples=0)
    t = np.array([x[0] for x in log] + [elapsed])
    d = np.array([x[1] for x in log], dtype=np.float64)
    w = np.clip(np.diff(t), 0.0, None)
    span = max(float(w.sum()), 1e-12)
    return dict(mean_depth=float((w * d).sum() / span), nonempty_frac=float(w[d > 0].sum() / span),
                max_depth=int(d.max()), samples=len(log))


def _current_device():
    try:
        import torch
        return torch.cuda.current_device() if torch.cuda.is_available() else None
    except ImportError:
        return None


def _new_stream():
    try:
        import torch
        return torch.cuda.Stream() if torch.cuda.is_available() else None
    except ImportError:
        return None


def _set_device(device):
    if device is not None:
        import torch
        torch.cuda.set_device(device)


def run_sequential(requests: list[Request], precision: str = "f64") -> tuple[list[Result], dict]:
    """Each request alone, one after another, in arrival order (the baseline)."""
    t0 = time.perf_counter()
    out = []
    for r in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        start = time.perf_counter() - t0
        with Solver.from_case(r.case, precision=precision, capacity=r.nsteps) as s:
            s.solve(r.nsteps)
            tr = s.traces()
            out.append(Result(r.rid, r.arrival, start, time.perf_counter() - t0, r.nsteps,
                              r.case.mesh.n_cells, tr, s.time))
    elapsed = time.perf_counter() - t0
    lat = np.array([r.latency for r in out])
    return out, dict(requests=len(out), elapsed_s=elapsed, sims_per_hour=len(out) / elapsed * 3600.0,
                     p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)))


# ---- MAPOD-style request generator -------------------------------------------------

def perturbed(c6: np.ndarray, rng, spread=0.05) -> np.ndarray:
    """Stiffness with each of the 21 unique entries scaled by 1 +- spread, kept
    positive definite (the perturbation is halved until it is)."""
    for _ in range(10):
        f = 1.0 + rng.uniform(-spread, spread, (6, 6))
        f = np.triu(f) + np.triu(f, 1).T
        c = c6 * f
        if np.linalg.eigvalsh(c).min() > 0:
            return c
        spread *= 0.5
    return c6.copy()


def mapod_request(rid: int, arrival: float, rng, cells_range=(0.2e6, 20e6), steps_range=(1000, 8000),
                  freq_range=(0.25e6, 2e6)) -> Request:
    """An aluminium or laminate plate: cell count log-uniform in cells_range,
    transducer position, frequency and +-5% stiffness perturbation drawn from rng."""
    cells = float(np.exp(rng.uniform(np.log(cells_range[0]), np.log(cells_range[1]))))
    nsteps = int(rng.integers(steps_range[0], steps_range[1] + 1))
    freq = float(rng.uniform(*freq_range))
    laminate = bool(rng.integers(0, 2))
    if laminate:
        nz, h, rho = 40, 0.05e-3, 1600.0
        ply = cases.orthotropic_ply(140e9, 10e9, 10e9, 6e9, 6e9, 4e9, 3e9, 5e9, 5e9)
        base = [cases.rotate_about_z(ply, a) for a in cases.LAYUP]
    else:
        nz, h, rho = 8, 0.1e-3, cases.ALUMINIUM["rho"]
        base = [cases.isotropic(cases.ALUMINIUM["E"], cases.ALUMINIUM["nu"])]
    side = max(8, int(round(math.sqrt(cells / nz))))
    mats = [perturbed(c, rng) for c in base]
    mesh = cases.voxel_mesh(np.ones((side, side, nz), dtype=bool), h)
    if laminate:
        cm = np.minimum(np.arange(nz) // (nz // len(base)), len(base) - 1)[mesh.cell_ijk[:, 2]]
    else:
        cm = np.zeros(mesh.n_cells)
    cmax = max(cases.max_wave_speed(c, rho) for c in mats)
    dt = cases.cfl_dt(h, cmax)
    t, v = cases.tone_burst(freq, 5, dt)
    L = side * h
    cx, cy = rng.uniform(0.25 * L, 0.75 * L, 2)
    radius = min(2e-3, 0.2 * L)
    src = [cases.transducer_z((cx, cy, nz * h), radius, h, t, v)]
    sens = cases.seeded_sensors(mesh, 16, int(rng.integers(0, 1 << 30)))
    case = cases.Case(f"req{rid}", mesh, np.full(len(mats), rho), np.stack([cases.c21_from_6x6(c) for c in mats]),
                      cm.astype(np.int32), dt, src, sens, nsteps,
                      dict(laminate=laminate, freq=freq, side=side, nz=nz))
    return Request(rid, arrival, case, nsteps, dict(laminate=laminate, freq=freq, cells=mesh.n_cells))


def poisson_requests(n: int, rate_per_s: float, seed: int, **kw) -> list[Request]:
    """n requests with exponential inter-arrival times (rate from the seed's stream)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate_per_s))
        out.append(mapod_request(i, t, rng, **kw))
    return out
