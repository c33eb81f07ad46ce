"""Benchmark of the RSG elastodynamic leapfrog on one GB300 (or N replicas).

Workload (default): composite laminate 400x400x40 cells (6.4 M cells,
6.59 M nodes), 0.05 mm voxels, [0/90/+45/-45]s plies of the orthotropic ply
(C11=140, C22=C33=10, C12=C13=6, C23=4, C44=3, C55=C66=5 GPa, rho=1600)
rotated about z, a 5-cycle 500 kHz Hann tone burst (z force) on a 2 mm
radius patch centred on the top face, 64 seeded top-face sensors recorded
every step.  Synthetic inputs with the published workload's shapes.

A step is one leapfrog step over the whole mesh: the node velocity update
then the cell stress update (one fused launch on voxel meshes, two on the
connectivity-table form).  Every step moves more than the 129 MB L2 (about
1 GB in FP64), so no L2 flush is needed.

value  = cells x steps / device time of the timed region (CUDA events on the
         solver's stream), FP64 drop-in form, summed over ranks.
e2e    = the same metric through the C ABI from host buffers: upload of the
         initial state from pinned host memory, the steps (one pn_solver_solve
         call per step, as the reference runners call Model::solve), download of
         the traces and the final state, timed on the host.
--impl reference times the CPU implementation of the path (the compiled
reference HostSolver when it exists on this machine, else the C restatement
of its algorithm) on the same workload with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-steps/s & % HBM roofline"
DTYPES = {"f64": "f64", "f64_exact": "f64", "f32": "f32", "df64": "f32x2 (double-float)"}
FORMS = {"f64": "FP64 drop-in form", "f64_exact": "FP64 reference-order form",
         "f32": "FP32 form", "df64": "double-float FP64-class form"}
UNIT = "Gcell-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--case", default="laminate", choices=["laminate", "plate", "holes"])
    p.add_argument("--nx", type=int, default=None, help="laminate / holed-plate size override (profiling)")
    p.add_argument("--ny", type=int, default=None)
    p.add_argument("--nz", type=int, default=None)
    p.add_argument("--precisions", default="f64,df64,f32",
                   help="forms to time; the first is the headline value")
    p.add_argument("--form", default="auto", choices=["auto", "table", "grid"],
                   help="device form: voxel-grid kernels or connectivity tables")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-fp32", action="store_true")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-batch", action="store_true", help="skip the batched-brackets leg")
    p.add_argument("--batch-members", type=int, default=96)
    p.add_argument("--batch-sample-steps", type=int, default=300)
    p.add_argument("--batch-form", default="auto", choices=["auto", "table", "grid"],
                   help="device form of the batch members (auto: grid, the brackets are lattices)")
    p.add_argument("--batch-kind", default="brackets", choices=["brackets", "plates"],
                   help="batch members: the seeded L-brackets (config 4), or full-box aluminium plates of "
                        "150-178 x 140-170 x 24 cells (a traffic comparison)")
    p.add_argument("--no-serving", action="store_true", help="skip the serving leg")
    p.add_argument("--no-pipes", action="store_true", help="skip the arithmetic pipe-rate leg")
    p.add_argument("--no-holes", action="store_true",
                   help="skip the FP32 holed-plate (1024x1024x24, 12 holes) bandwidth leg")
    p.add_argument("--serving-requests", type=int, default=32)
    p.add_argument("--serving-rate", type=float, default=4.0, help="Poisson arrivals per second")
    p.add_argument("--serving-fp64-subset", type=int, default=8,
                   help="requests of the serving run also solved in sequential FP64")
    return p.parse_args()


def make_case(name, nx=None, ny=None, nz=None):
    from pannde_gb300 import cases
    if name == "laminate":
        nx, ny, nz = nx or 400, ny or 400, nz or 40
        c = cases.laminate_case(nx=nx, ny=ny, nz=nz)
        desc = (f"laminate {nx}x{ny}x{nz} cells (0.05 mm), [0/90/+45/-45]s orthotropic plies, "
                "500 kHz 5-cycle tone burst, 64 sensors")
    elif name == "plate":
        c = cases.al_plate_case()
        desc = "aluminium plate 64x64x8 cells (0.1 mm), 1 MHz tone burst, 16 sensors"
    else:
        nx, ny, nz = nx or 1024, ny or 1024, nz or 24
        c = cases.holed_plate_case(nx=nx, ny=ny, nz=nz)
        desc = f"aluminium plate {nx}x{ny}x{nz} cells (0.1 mm), 12 holes, 1 MHz tone burst, 128 sensors"
    return c, desc


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_figures(case, form, prec, what="traffic"):
    """Per-kernel figures from the committed ncu summaries (profiles/*.txt),
    lines '<what> <case>.<form>.<precision>.<kernel> = <value>': 'traffic'
    (DRAM bytes per launch), 'fp64pipe' (FP64 pipe busy fraction), 'dpops'
    (FP64 operations per cell-step)."""
    out = {}
    prefix = f"{case}.{form}.{prec}."
    for f in sorted((ROOT / "profiles").glob("*.txt")):
        for line in f.read_text().splitlines():
            if line.startswith(what + " ") and "=" in line:
                key, val = line[len(what) + 1:].split("=", 1)
                key = key.strip()
                if key.startswith(prefix):
                    out[key[len(prefix):]] = float(val.split()[0])
    return out


def profile_traffic(case, form, prec):
    return profile_figures(case, form, prec, "traffic")


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


FORM = "auto"


def reduce_max(value, dist, torch):
    """The largest value over all ranks (every rank calls it: the max-over-ranks
    time of a step range); the value itself in a single process."""
    if not dist:
        return value
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, seconds, ws):
    """Whole-job throughput: each of ws ranks processed units_per_rank, the
    slowest in `seconds` (weak scaling: independent replicas)."""
    return ws * units_per_rank / seconds


def time_device(case, prec, steps, warmup, torch, dist, energy=False, state=None):
    """Device throughput of the hot path with inputs resident in HBM (from
    rest, or from `state` = (V, S))."""
    from pannde_gb300.solver import Solver
    s = Solver.from_case(case, precision=prec, capacity=warmup + steps, form=FORM)
    stream = torch.cuda.Stream()
    s.set_stream(stream)
    if state is not None:
        s.set_state(*state)
    s.solve(warmup)
    s.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    s.enable_kernel_timing(True)
    p0 = s.path_counts()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.solve(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = reduce_max(e0.elapsed_time(e1), dist, torch)
    kt = s.kernel_times()
    info = s.info()
    p1 = s.path_counts()
    info["path_counts"] = (p1[0] - p0[0], p1[1] - p0[1])
    if energy:  # FP64 energy audit of the final state
        info["energy"] = s.energy()
    s.close()
    return ms, kt, info


def roofline(case, info, kt, prec, peak, peak_kind):
    """HBM roofline of the dominant kernel from its CUDA-event average.

    Algorithmic bytes per launch:
      table form  velocity: S read (6e/cell), V read+write, dt/rho, node slots (7e+32 /node)
                  stress:   S read+write, material id, corner table (12e+36 /cell), V read (3e /node)
      grid form   fused step: S read+write + material byte (12e+1 /lattice cell),
                  V read+write + dt/rho (7e /lattice node) -- pn_solver_info
    with e the bytes per value (4 FP32, 8 FP64 and double-float)."""
    e = 4 if prec == "f32" else 8
    nc, nn = info["n_cells"], info["n_nodes"]
    avg = {k: kt[k][0] / max(kt[k][1], 1) for k in kt if kt[k][1] > 0}
    if info.get("form_name") == "grid":
        alg = {"grid_step": info["algorithmic_bytes_per_step"]}
    else:
        alg = {"velocity": nc * 6 * e + nn * (7 * e + 32),
               "stress": nc * (12 * e + 36) + nn * 3 * e}
    dom = max(avg, key=lambda k: avg[k])
    achieved = alg[dom] / (avg[dom] * 1e-3) / 1e9
    form = info.get("form_name", "table")
    traffic = profile_traffic(case, form, prec).get(dom)
    step_ms = sum(avg.values())
    out = {"bound": "hbm", "kernel": dom, "form": form, "achieved": round(achieved, 1),
           "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
           "traffic": traffic, "algorithmic_bytes": alg[dom],
           "avg_ms": {k: round(v, 4) for k, v in avg.items()},
           "step_bytes_frac": round(sum(alg.values()) / (step_ms * 1e-3) / 1e9 / peak, 4)}
    if prec == "f64" and sum(info.get("path_counts", (0, 0))) > 0:
        fp64, df = info["path_counts"]
        out["f64_paths"] = {"fp64_blocks": fp64, "double_float_blocks": df,
                            "double_float_share": round(df / (fp64 + df), 4),
                            "note": "blocks of the timed steps by arithmetic path (pn_solver_path_counts)"}
    if prec == "f64":
        # pipe use of the FP64 form's step from the committed ncu summary
        # (profiles/*.txt lines 'fp64pipe' / 'fmapipe' / 'issue' for this key)
        fig = {w: profile_figures(case, form, prec, w).get(dom) for w in ("fp64pipe", "fmapipe", "issue")}
        if any(v is not None for v in fig.values()):
            out["pipes_ncu"] = {"fp64_pipe_busy": fig["fp64pipe"], "fma_pipe_busy": fig["fmapipe"],
                                "issue_active": fig["issue"],
                                "note": "FP64 form: double-float blocks on the FP32/integer pipes beside IEEE-double "
                                        "blocks on the FP64 pipe, one launch"}
    return out


def e2e_run(case, prec, steps, torch, dist=None):
    """Through the C ABI with host buffers (pinned), copies inside the timed
    region; every rank runs it, started together, and the slowest rank's time
    counts."""
    from pannde_gb300.solver import Solver
    s = Solver.from_case(case, precision=prec, capacity=steps, form=FORM)
    nn, nc = case.mesh.n_nodes, case.mesh.n_cells

    def pinned(n):
        return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()

    V0 = [pinned(nn) for _ in range(3)]
    S0 = [pinned(nc) for _ in range(6)]
    for a in V0 + S0:
        a[:] = 0.0
    V = [pinned(nn) for _ in range(3)]
    S = [pinned(nc) for _ in range(6)]
    s.solve(2)  # first-call setup (source tables) outside the timed region
    s.get_state_into(V, S)  # first-transfer setup (the grid form's index maps), likewise
    s.synchronize()
    s.clear_traces()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    s.set_state(V0, S0)
    ta = time.perf_counter()
    for _ in range(steps):
        s.solve(1)
    tb = time.perf_counter()
    tr = s.traces()
    tc = time.perf_counter()
    s.get_state_into(V, S)
    t1 = time.perf_counter()
    sig_rows = min(steps, 1 << 16)
    h2d = (3 * nn + 6 * nc) * 8 + sig_rows * len(case.sources) * 8
    d2h = (3 * nn + 6 * nc) * 8 + tr.size * 8
    s.close()
    # host wall-clock parts: the state upload (returns when done), the solve
    # calls (they enqueue), the traces (wait for the steps), the state download
    parts = {"set_state_ms": round((ta - t0) * 1e3, 3), "solve_calls_ms": round((tb - ta) * 1e3, 3),
             "traces_ms": round((tc - tb) * 1e3, 3), "get_state_ms": round((t1 - tc) * 1e3, 3)}
    return reduce_max(t1 - t0, dist, torch), h2d, d2h, parts


def state_transfer_leg(case, prec, torch, reps=3):
    """pn_solver_set_state / pn_solver_get_state of the whole state between
    page-locked host buffers and the device, two ways: the conversion kernels
    reading and writing the mapped host buffers directly over the CPU-GPU
    link, and (PN_STATE_COPY=dma) a copy-engine transfer to a device staging
    buffer with the conversion kernel on device memory.  Best of `reps`,
    wall clock around each call (each waits for its transfers)."""
    from pannde_gb300.solver import Solver
    nn, nc = case.mesh.n_nodes, case.mesh.n_cells
    nbytes = (3 * nn + 6 * nc) * 8

    def pinned(n):
        return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()

    V = [pinned(nn) for _ in range(3)]
    S = [pinned(nc) for _ in range(6)]
    rng = np.random.default_rng(1)
    for a in V + S:
        a[:] = rng.uniform(-1.0, 1.0, a.size)
    out = {}
    with Solver.from_case(case, precision=prec, capacity=1, form=FORM) as s:
        for mode in ("kernel", "dma"):
            if mode == "dma":
                os.environ["PN_STATE_COPY"] = "dma"
            try:
                put, get = [], []
                for _ in range(reps):
                    t0 = time.perf_counter()
                    s.set_state(V, S)
                    t1 = time.perf_counter()
                    s.get_state_into(V, S)
                    t2 = time.perf_counter()
                    put.append(t1 - t0)
                    get.append(t2 - t1)
            finally:
                os.environ.pop("PN_STATE_COPY", None)
            out[mode] = {"set_state_GBps": round(nbytes / min(put) / 1e9, 1),
                         "get_state_GBps": round(nbytes / min(get) / 1e9, 1),
                         "set_state_ms": round(min(put) * 1e3, 3), "get_state_ms": round(min(get) * 1e3, 3)}
    out["bytes_each_way"] = nbytes
    out["how"] = ("kernel: conversion kernels on mapped page-locked buffers; dma: cudaMemcpyAsync to a device "
                  "staging buffer + conversion kernel (PN_STATE_COPY=dma); best of %d" % reps)
    return out


def batch_leg(n_members, sample_steps, torch, steps_total=3000, form="auto", peak=None, peak_kind=None,
              kind="brackets"):
    """Batched sims/hour: n_members seeded L-brackets (legs 60-220 cells, 12-30
    thick, 40-160 deep, 0.1 mm voxels, a 1-6 mm crack at the inner fillet as
    disconnected faces; every sixth with an acoustic-fluid column and a
    pressure source, the others a z-force transducer), FP32, 3000 steps each,
    advanced together by pn_batch_solve calls of 25 steps (equal calls replay
    a captured CUDA graph, as a serving loop's quanta do).  The brackets are voxel lattices
    whose cracks split lattice sites, so they take the grid form: one fused
    launch per step for all members plus the two small fix-up launches of the
    split sites (form="table": the connectivity-table kernels, two launches
    per step).  A sample of the steps is timed with CUDA events on the
    batch's stream; the per-step cost does not change along the run.
    kind="plates": full-box aluminium plates instead, for comparing the
    kernel's DRAM traffic on members without the brackets' geometry."""
    from pannde_gb300 import cases
    from pannde_gb300.solver import Batch, Solver
    warm = 25  # long enough for the launch-shape tuning (2 rounds x up to 6 shapes x 2 steps + 1) to run untimed
    quantum = 25  # steps per pn_batch_solve call: equal calls replay a captured CUDA graph
    sample_steps = max(quantum, sample_steps // quantum * quantum)
    t0 = time.perf_counter()
    if kind == "plates":
        cs = [cases.al_plate_case(nx=150 + 7 * (i % 5), ny=140 + 5 * (i % 7), nz=24, nsteps=steps_total,
                                  radius=1e-3, n_sensors=8, seed=i) for i in range(n_members)]
    else:
        cs = [cases.bracket_case(1000 + i, nsteps=steps_total, water_column=(i % 6 == 0))
              for i in range(n_members)]
    solvers = [Solver.from_case(c, precision="f32", capacity=warm + 2 * quantum + sample_steps, form=form)
               for c in cs]
    setup_s = time.perf_counter() - t0
    cells = sum(c.mesh.n_cells for c in cs)
    forms = sorted({s.info()["form_name"] for s in solvers})
    alg = sum(s.info()["algorithmic_bytes_per_step"] for s in solvers)
    with Batch() as b:
        for s in solvers:
            b.add(s)
        stream = torch.cuda.Stream()
        b.set_stream(stream)
        b.solve(warm)
        b.solve(quantum)
        b.solve(quantum)  # the second equal call is captured as a CUDA graph
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(sample_steps // quantum):
            b.solve(quantum)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        plan = b.plan_stats()
    for s in solvers:
        s.close()
    per_step_s = ms * 1e-3 / sample_steps
    roof = None
    if peak:
        achieved = alg / per_step_s / 1e9
        traffic = profile_figures("%s%d" % (kind, n_members), forms[0], "f32", "traffic").get("batch_step")
        roof = {"bound": "hbm", "kernel": "batch step (fused step launch + split-site fix-up)",
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": peak_kind, "traffic": traffic, "algorithmic_bytes": alg,
                "note": "algorithmic bytes: every member's marched lattice (12e+1 per cell, 7e per node, e=4)"}
    return {"sims_per_hour": round(n_members / (per_step_s * steps_total) * 3600.0, 1),
            "gcell_steps_per_s": round(cells / per_step_s / 1e9, 4),
            "members": n_members, "cells_total": cells, "steps_per_sim": steps_total,
            "timed_steps": sample_steps, "ms_per_batch_step": round(ms / sample_steps, 4),
            "steps_per_call": quantum, "graph_launches": plan["graph_launches"],
            "tuned_shape": {"tile": f"32x{plan['tile_rows']}", "z_chunks_per_column": plan["shape"] or "launcher"},
            "dtype": "f32", "form": ",".join(forms), "setup_s": round(setup_s, 1), "roofline": roof,
            "workload": (f"{n_members} full-box aluminium plates (150-178 x 140-170 x 24 cells), FP32, one "
                         "pn_batch_solve over all members" if kind == "plates" else
                         f"{n_members} seeded L-brackets with a disconnected-face crack, every sixth with a "
                         "water column (pressure source), FP32, one pn_batch_solve over all members")}


def serving_leg(n_requests, rate, torch, seed=7, subset=8):
    """Serving: Poisson arrivals (rate per second, seeded); each request an
    aluminium or laminate plate, cells log-uniform 0.2 M - 20 M, transducer
    position, 0.25-2 MHz, +-5% stiffness, 1000-8000 steps.  Continuous
    batching in FP32 (pannde_gb300.serving.Server) with the admission queue
    depth sampled along the run.  The baseline is the same requests solved
    one after another in plain FP64 on the same GPU: `subset` of them, drawn
    by the seed, are solved (set-up included) and their seconds per cell-step
    extrapolate the sequential run of all requests; the same FP64 solves are
    the spot check of those requests' FP32 traces (relative L2 per request)."""
    from pannde_gb300 import serving
    t0 = time.perf_counter()
    reqs = serving.poisson_requests(n_requests, rate, seed)
    gen_s = time.perf_counter() - t0
    free, _ = torch.cuda.mem_get_info()
    srv = serving.Server(hbm_budget_bytes=int(0.7 * free), precision="f32", quantum=250)
    res, st = srv.run(reqs)
    rng = np.random.default_rng(seed + 1)
    pick = sorted(rng.choice(len(reqs), size=min(subset, len(reqs)), replace=False).tolist())
    sub = [serving.Request(reqs[i].rid, 0.0, reqs[i].case, reqs[i].nsteps, reqs[i].meta) for i in pick]
    seq, sst = serving.run_sequential(sub, precision="f64")
    by_rid = {r.rid: r for r in res}
    errs = []
    for q in seq:
        d = np.linalg.norm(q.traces)
        errs.append(float(np.linalg.norm(by_rid[q.rid].traces - q.traces) / (d if d > 0 else 1.0)))
    cs = {r.rid: r.case.mesh.n_cells * r.nsteps for r in reqs}
    s_per_cs = sst["elapsed_s"] / sum(cs[i] for i in (reqs[k].rid for k in pick))
    seq_est_s = s_per_cs * sum(cs.values())
    seq_sph = len(reqs) / seq_est_s * 3600.0
    return {"sims_per_hour": round(st["sims_per_hour"], 1), "p50_s": round(st["p50_s"], 3),
            "p99_s": round(st["p99_s"], 3), "gcell_steps_per_s": round(st["gcell_steps_per_s"], 3),
            "max_in_flight": st["max_active"], "requests": st["requests"], "rate_per_s": rate,
            "elapsed_s": round(st["elapsed_s"], 2),
            "queue": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in st["queue"].items()},
            "sequential_fp64": {"sims_per_hour": round(seq_sph, 1), "measured_requests": len(pick),
                                "measured_s": round(sst["elapsed_s"], 2),
                                "s_per_gcell_step": round(s_per_cs * 1e9, 4),
                                "how": "FP64 solves (set-up included) of a seeded subset, one after another; "
                                       "their seconds per cell-step times all requests' cell-steps"},
            "sims_per_hour_vs_sequential_fp64": round(st["sims_per_hour"] / max(seq_sph, 1e-9), 2),
            "fp32_trace_rel_l2_vs_fp64_max": max(errs) if errs else None,
            "fp64_spot_checked_requests": len(errs),
            "request_generation_s": round(gen_s, 1),
            "workload": "Poisson arrivals; Al or laminate plates 0.2-20 M cells (log-uniform), "
                        "1000-8000 steps, 0.25-2 MHz; FP32 continuous batching vs sequential plain FP64; "
                        "latency = arrival to traces"}


def holes_leg(steps, warmup, torch, peak, peak_kind):
    """The FP32 large-mesh bandwidth workload: aluminium plate 1024x1024x24
    cells (0.1 mm voxels) with 12 seeded through-thickness holes of 1-4 mm
    radius (24.4 M cells left), a 2 mm radius 1 MHz transducer on the top
    face, 128 seeded sensors recorded every step; FP32 state and material
    rows.  Device throughput over `steps` steps after `warmup` (each step moves
    far more than the L2), the tensor-copy kernel's HBM roofline over the
    lattice it marches (each tile to its top solid layer), and the FP64
    energy audit of the final state."""
    case, desc = make_case("holes")
    t0 = time.perf_counter()
    ms, kt, info = time_device(case, "f32", steps, warmup, torch, None, energy=True)
    cells = info["n_cells"]
    kin, strain = info["energy"]
    return {"workload": desc + " (FP32 form)", "cells": cells, "nodes": info["n_nodes"],
            "lattice": info["grid"], "value": round(cells * steps / (ms * 1e-3) / 1e9, 4), "unit": UNIT,
            "ms_per_step": round(ms / steps, 4), "steps": steps, "warmup": warmup, "dtype": "f32",
            "algorithmic_bytes_per_step": info["algorithmic_bytes_per_step"],
            "roofline": roofline("holes", info, kt, "f32", peak, peak_kind),
            "energy_audit_fp64": {"after_steps": warmup + steps, "kinetic_J": kin, "strain_J": strain},
            "setup_and_run_s": round(time.perf_counter() - t0, 1)}


def cpu_reference(case, budget_s):
    """The CPU implementation on a bounded sample of the workload (all threads)."""
    import oracle
    lib_kind = "reference" if oracle.reference() is not None else "port"
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    mat = case.material_fields()

    def run(n):
        t0 = time.perf_counter()
        oracle.run(case.mesh, mat, case.dt, case.sources, n, case.sensors, impl=lib_kind)
        return time.perf_counter() - t0

    t1 = run(1)
    t3 = run(3)
    per_step = max((t3 - t1) / 2.0, 1e-9)
    n = int(max(2, min(50, budget_s / per_step)))
    tn = run(1 + n)
    per_step = max((tn - t1) / n, 1e-9)
    value = case.mesh.n_cells / per_step / 1e9
    threads_used = threads if lib_kind == "port" else 1
    return {"value": value, "unit": UNIT, "cores": threads_used,
            "kind": "reference" if lib_kind == "reference" else "port",
            "sample": f"{n} steps on the full {case.mesh.n_cells}-cell mesh "
                      f"(setup cancelled by differencing a 1-step run), {case.name}"}


def main():
    args = parse()
    global FORM
    FORM = args.form
    ws, rank, local = dist_setup()
    if args.impl == "reference" and rank != 0:
        return 0  # the CPU reference arm runs on rank 0 alone
    assert args.warmup >= 3 or args.impl == "reference", "at least 3 warm-up steps"
    case, desc = make_case(args.case, args.nx, args.ny, args.nz)
    precs = [p for p in args.precisions.split(",") if p]
    if args.no_fp32:
        precs = [p for p in precs if p != "f32"]

    if args.impl == "reference":
        cb = cpu_reference(case, args.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": case.mesh.n_cells / (cb["value"] * 1e9) * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": {"workload": desc, "cells": case.mesh.n_cells,
                                                "nodes": case.mesh.n_nodes},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    dist = None
    if ws > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist
    else:
        torch.cuda.set_device(0)
    from pannde_gb300 import _native
    _native.load()

    peak, peak_kind = peaks()
    head = precs[0]
    with Clocks(local) as clk:
        ms, kt, info = time_device(case, head, args.steps, args.warmup, torch, dist)
    clocks = clk.summary()
    cells = info["n_cells"]
    value = whole_job_rate(cells * args.steps, ms * 1e-3, ws) / 1e9
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES[head], "data": "synthetic",
            "config": {"workload": desc + f" ({FORMS[head]})", "cells": cells,
                       "nodes": info["n_nodes"], "materials": info["n_materials"],
                       "algorithmic_bytes_per_step": info["algorithmic_bytes_per_step"],
                       "l2": "no flush: each step moves far more than the 129 MB L2",
                       "parallelism": f"{ws} independent replica(s), one per GPU"},
            "roofline": roofline(args.case, info, kt, head, peak, peak_kind),
            "gpu_launches": int(kt["grid_step"][1] * info["launches_per_step"] + kt["velocity"][1] + kt["stress"][1]),
            "clocks": clocks}
    if head == "f64" and line["roofline"].get("f64_paths"):
        # the same step from a developed state (every value inside the
        # double-float range), beside the window from rest above
        rng = np.random.default_rng(11)
        state = ([rng.uniform(-1e-3, 1e-3, case.mesh.n_nodes) for _ in range(3)],
                 [rng.uniform(-1e5, 1e5, case.mesh.n_cells) for _ in range(6)])
        msd, ktd, infod = time_device(case, head, args.steps, args.warmup, torch, dist, state=state)
        rd = roofline(args.case, infod, ktd, head, peak, peak_kind)
        line["roofline"]["f64_developed_state"] = {
            "value": round(whole_job_rate(cells * args.steps, msd * 1e-3, ws) / 1e9, 4), "unit": UNIT,
            "ms_per_step": round(msd / args.steps, 4), "frac": rd["frac"],
            "double_float_share": rd.get("f64_paths", {}).get("double_float_share"),
            "state": "seeded uniform random velocities (+-1e-3 m/s) and stresses (+-1e5 Pa): a step well "
                     "into a run, every value inside the double-float range"}
        del state
    forms = {}
    for prec in precs[1:]:
        msp, ktp, infop = time_device(case, prec, args.steps, args.warmup, torch, dist)
        vp = whole_job_rate(cells * args.steps, msp * 1e-3, ws) / 1e9
        forms[prec] = {"value": round(vp, 4), "unit": UNIT, "dtype": DTYPES[prec],
                       "ms_per_step": round(msp / args.steps, 4),
                       "roofline": roofline(args.case, infop, ktp, prec, peak, peak_kind)}
    if forms:
        line["other_forms"] = forms
    if not args.no_e2e:  # every rank: the slowest rank's wall time counts
        # three runs, the median reported (the host side shares its machine)
        runs = [e2e_run(case, head, args.steps, torch, dist) for _ in range(3)]
        runs.sort(key=lambda r: r[0])
        secs, h2d, d2h, parts = runs[1]
        parts = dict(parts, runs_ms=[round(r[0] * 1e3, 3) for r in runs])
        line["e2e"] = {"value": round(whole_job_rate(cells * args.steps, secs, ws) / 1e9, 4), "unit": UNIT,
                       "h2d_bytes_per_step": int(ws * h2d / args.steps),
                       "d2h_bytes_per_step": int(ws * d2h / args.steps),
                       "how": "pn_solver_set_state from pinned host, one pn_solver_solve per step, "
                              "pn_solver_get_traces + pn_solver_get_state to pinned host; wall clock, "
                              "max over ranks, the median of three runs; bytes summed over ranks",
                       "parts": parts}
        if rank == 0 and ws == 1:
            line["e2e"]["state_transfer"] = state_transfer_leg(case, head, torch)
    if rank == 0:
        if ws == 1 and not args.no_holes:
            line["configs"] = {"holes": holes_leg(args.steps, args.warmup, torch, peak, peak_kind)}
        if ws == 1 and not args.no_batch:
            line["batch"] = batch_leg(args.batch_members, args.batch_sample_steps, torch, form=args.batch_form,
                                      peak=peak, peak_kind=peak_kind, kind=args.batch_kind)
        if ws == 1 and not args.no_serving:
            line["serving"] = serving_leg(args.serving_requests, args.serving_rate, torch,
                                         subset=args.serving_fp64_subset)
        if ws == 1 and not args.no_pipes:
            from pannde_gb300.solver import measure_pipe_rates
            line["pipes"] = {"ops_per_s": {k: float(f"{v:.4g}") for k, v in measure_pipe_rates().items()},
                             "how": "pn_measure_pipe_rates: 8 independent chains per thread, full grid of "
                                    "resident blocks, CUDA events, best of 3; thread-level operations/s"}
        if ws == 1 and not args.no_cpu:
            line["cpu_baseline"] = cpu_reference(case, args.cpu_seconds)
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
