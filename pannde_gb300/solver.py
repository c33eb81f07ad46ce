"""Thin object wrapper over the C ABI solver handle (pn_solver_*).

Every call goes to the CUDA library; nothing here computes the physics.
"""
from __future__ import annotations

import ctypes
from ctypes import c_double, c_int64, c_void_p

import numpy as np

from . import _native as N
from .cases import Case, HexMesh, sources_struct

PRECISIONS = {"f64_exact": N.PN_PREC_F64_EXACT, "f64": N.PN_PREC_F64, "f32": N.PN_PREC_F32,
              "df64": N.PN_PREC_DF64}


FORMS = {"auto": N.PN_FORM_AUTO, "table": N.PN_FORM_TABLE, "grid": N.PN_FORM_GRID}


def _precision(p, form="auto") -> int:
    prec = PRECISIONS[p] if isinstance(p, str) else int(p)
    return prec | (FORMS[form] if isinstance(form, str) else int(form))


class Solver:
    """One RSG leapfrog instance resident on the current CUDA device.

    ``material`` is either a Case (indexed material table) or a
    (PnMaterial, keepalive) pair of reference-style fields.
    """

    def __init__(self, mesh: HexMesh, material, dt: float, precision="f64", form="auto"):
        self._lib = N.load()
        self.mesh = mesh
        self.precision = _precision(precision, form)
        m, keep = mesh.as_struct()
        h = c_void_p()
        if isinstance(material, Case):
            tab, keep_t = material.material_table()
            rc = self._lib.pn_solver_create_indexed(ctypes.byref(m), ctypes.byref(tab), float(dt),
                                                    self.precision, ctypes.byref(h))
        else:
            mat, keep_t = material
            rc = self._lib.pn_solver_create(ctypes.byref(m), ctypes.byref(mat), float(dt),
                                            self.precision, ctypes.byref(h))
        N.check(rc)
        self._h = h
        self.n_sensors = 0
        del keep, keep_t

    @classmethod
    def from_case(cls, case: Case, precision="f64", sensors=True, capacity=None, form="auto"):
        s = cls(case.mesh, case, case.dt, precision, form)
        if case.sources:
            s.add_sources(case.sources)
        if sensors and case.sensors.size:
            s.set_sensors(case.sensors, capacity if capacity is not None else case.nsteps)
        return s

    # -- lifecycle --
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pn_solver_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- calls --
    def set_stream(self, stream):
        """stream: a torch.cuda.Stream, a raw cudaStream_t int, or None."""
        handle = getattr(stream, "cuda_stream", stream)
        N.check(self._lib.pn_solver_set_stream(self._h, c_void_p(handle or 0)))

    def set_state(self, V=None, S=None):
        v = [N.f64(a) if a is not None else None for a in (V or [None] * 3)]
        s = [N.f64(a) if a is not None else None for a in (S or [None] * 6)]
        N.check(self._lib.pn_solver_set_state(self._h, N.ptr_array(v), N.ptr_array(s)))

    def add_sources(self, sources):
        arr, keep = sources_struct(sources)
        N.check(self._lib.pn_solver_add_sources(self._h, arr, len(sources)))
        del keep

    def add_window_masks(self, masks):
        """masks: list of (kind, group, component, inside[uint8]) -- inside over
        cells (force) or nodes (moment), the caller's own window predicate."""
        arr = (N.PnWindowMask * max(len(masks), 1))()
        keep = []
        for i, (kind, group, comp, inside) in enumerate(masks):
            a = np.ascontiguousarray(inside, dtype=np.uint8)
            keep.append(a)
            arr[i] = N.PnWindowMask(int(kind), int(group), int(comp),
                                    a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        N.check(self._lib.pn_solver_add_window_masks(self._h, arr, len(masks)))
        del keep

    def solve_signals(self, values) -> float:
        """Advance len(values) steps with the signal of every source given per
        step: values[k][i] for source i (addition order) at step k."""
        v = N.f64(values)
        nsteps = int(v.shape[0]) if v.ndim else 0
        t = c_double(0.0)
        N.check(self._lib.pn_solver_solve_signals(self._h, nsteps, N.dptr(v.reshape(-1)), ctypes.byref(t)))
        return t.value

    def set_sensors(self, nodes, capacity_steps):
        nd = N.i32(nodes)
        N.check(self._lib.pn_solver_set_sensors(self._h, N.iptr(nd), int(nd.shape[0]),
                                                int(capacity_steps)))
        self.n_sensors = int(nd.shape[0])

    def solve(self, nsteps=1) -> float:
        t = c_double(0.0)
        N.check(self._lib.pn_solver_solve(self._h, int(nsteps), ctypes.byref(t)))
        return t.value

    def get_state(self):
        V = [np.empty(self.mesh.n_nodes) for _ in range(3)]
        S = [np.empty(self.mesh.n_cells) for _ in range(6)]
        N.check(self._lib.pn_solver_get_state(self._h, N.ptr_array(V), N.ptr_array(S)))
        return V, S

    def get_state_into(self, V, S):
        """Download into caller-owned float64 arrays (None entries skipped)."""
        N.check(self._lib.pn_solver_get_state(self._h, N.ptr_array(V), N.ptr_array(S)))

    def traces(self, max_records=None) -> np.ndarray:
        n = c_int64(0)
        N.check(self._lib.pn_solver_get_traces(self._h, N.P_double(), 0, ctypes.byref(n)))
        rec = n.value if max_records is None else min(n.value, max_records)
        out = np.zeros((max(rec, 1), max(self.n_sensors, 1), 3))
        N.check(self._lib.pn_solver_get_traces(self._h, N.dptr(out), rec, ctypes.byref(n)))
        return out[:rec, :self.n_sensors]

    def clear_traces(self):
        N.check(self._lib.pn_solver_clear_traces(self._h))

    @property
    def time(self) -> float:
        t = c_double(0.0)
        N.check(self._lib.pn_solver_get_time(self._h, ctypes.byref(t)))
        return t.value

    def info(self) -> dict:
        inf = N.PnSolverInfo()
        N.check(self._lib.pn_solver_get_info(self._h, ctypes.byref(inf)))
        d = {k: getattr(inf, k) for k, _ in N.PnSolverInfo._fields_}
        d["grid"] = tuple(d["grid"])
        d["form_name"] = {N.PN_FORM_GRID: "grid", N.PN_FORM_TABLE: "table"}.get(d["form"], "?")
        d["kernel_name"] = {1: "classic", 2: "tma", 3: "tma-f64-two-launch"}.get(d["grid_kernel"], "table")
        d["launches_per_step"] = 2 if d["grid_kernel"] == 3 else (1 if d["form"] == N.PN_FORM_GRID else 2)
        return d

    def device_state(self):
        V = (c_void_p * 3)()
        S = (c_void_p * 6)()
        N.check(self._lib.pn_solver_device_state(self._h, V, S))
        return [v for v in V], [s for s in S]

    def enable_kernel_timing(self, on=True):
        N.check(self._lib.pn_solver_enable_kernel_timing(self._h, 1 if on else 0))

    def kernel_times(self):
        """{"velocity" | "stress" | "grid_step": (ms_total, launches)} since enabled"""
        ms = (c_double * 3)()
        n = (c_int64 * 3)()
        N.check(self._lib.pn_solver_kernel_times(self._h, ms, n))
        return {"velocity": (ms[0], n[0]), "stress": (ms[1], n[1]), "grid_step": (ms[2], n[2])}

    def energy(self):
        """(kinetic, strain) energy of the current state, in FP64 (pn_solver_energy)."""
        k, e = c_double(0.0), c_double(0.0)
        N.check(self._lib.pn_solver_energy(self._h, ctypes.byref(k), ctypes.byref(e)))
        return k.value, e.value

    def synchronize(self):
        N.check(self._lib.pn_solver_synchronize(self._h))

    def path_counts(self) -> tuple[int, int]:
        """(FP64-path blocks, double-float-path blocks) of the FP64 grid
        form's steps so far (pn_solver_path_counts)."""
        a, b = c_int64(0), c_int64(0)
        N.check(self._lib.pn_solver_path_counts(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


class Batch:
    """Solvers advanced together by shared launches (pn_batch_*).

    Members keep their own state, sources, sensors and time; a member's
    results are the same alone and in the batch.  The batch does not own its
    members."""

    def __init__(self):
        self._lib = N.load()
        h = c_void_p()
        N.check(self._lib.pn_batch_create(ctypes.byref(h)))
        self._h = h
        self.members = []

    def add(self, solver: Solver):
        N.check(self._lib.pn_batch_add(self._h, solver._h))
        self.members.append(solver)

    def remove(self, solver: Solver):
        N.check(self._lib.pn_batch_remove(self._h, solver._h))
        self.members.remove(solver)

    def set_stream(self, stream):
        handle = getattr(stream, "cuda_stream", stream)
        N.check(self._lib.pn_batch_set_stream(self._h, c_void_p(handle or 0)))

    def solve(self, nsteps: int):
        N.check(self._lib.pn_batch_solve(self._h, int(nsteps)))

    def solve_noalloc(self, nsteps: int):
        """pn_batch_solve_noalloc: the same steps staged in the library's fixed
        device scratch, with no device allocation."""
        N.check(self._lib.pn_batch_solve_noalloc(self._h, int(nsteps)))

    def plan_stats(self) -> dict:
        """{"graph_launches", "graph_captures", "tuned_classes", "tile_rows", "shape"}
        (pn_batch_plan_stats; tile_rows and shape of the last chunk run)"""
        gl, gc, tc = c_int64(0), c_int64(0), ctypes.c_int32(0)
        tr, sh = ctypes.c_int32(0), ctypes.c_int32(0)
        N.check(self._lib.pn_batch_plan_stats(self._h, ctypes.byref(gl), ctypes.byref(gc), ctypes.byref(tc),
                                              ctypes.byref(tr), ctypes.byref(sh)))
        return {"graph_launches": gl.value, "graph_captures": gc.value, "tuned_classes": tc.value,
                "tile_rows": tr.value, "shape": sh.value}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pn_batch_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Partitioned:
    """One mesh as several partitions on the current device with a halo
    exchange per step (pn_partitioned_*); results equal a single Solver."""

    def __init__(self, case: Case, n_parts: int, precision="f64"):
        self._lib = N.load()
        self.mesh = case.mesh
        m, keep = case.mesh.as_struct()
        tab, keep_t = case.material_table()
        h = c_void_p()
        N.check(self._lib.pn_partitioned_create(ctypes.byref(m), ctypes.byref(tab), float(case.dt),
                                                PRECISIONS[precision], int(n_parts), ctypes.byref(h)))
        self._h = h
        self.n_sensors = 0
        del keep, keep_t

    def add_sources(self, sources):
        arr, keep = sources_struct(sources)
        N.check(self._lib.pn_partitioned_add_sources(self._h, arr, len(sources)))
        del keep

    def set_sensors(self, nodes, capacity_steps):
        nd = N.i32(nodes)
        N.check(self._lib.pn_partitioned_set_sensors(self._h, N.iptr(nd), int(nd.shape[0]), int(capacity_steps)))
        self.n_sensors = int(nd.shape[0])

    def set_state(self, V=None, S=None):
        v = [N.f64(a) if a is not None else None for a in (V or [None] * 3)]
        s = [N.f64(a) if a is not None else None for a in (S or [None] * 6)]
        N.check(self._lib.pn_partitioned_set_state(self._h, N.ptr_array(v), N.ptr_array(s)))

    def solve(self, nsteps=1) -> float:
        t = c_double(0.0)
        N.check(self._lib.pn_partitioned_solve(self._h, int(nsteps), ctypes.byref(t)))
        return t.value

    def get_state(self):
        V = [np.empty(self.mesh.n_nodes) for _ in range(3)]
        S = [np.empty(self.mesh.n_cells) for _ in range(6)]
        N.check(self._lib.pn_partitioned_get_state(self._h, N.ptr_array(V), N.ptr_array(S)))
        return V, S

    def traces(self) -> np.ndarray:
        n = c_int64(0)
        N.check(self._lib.pn_partitioned_get_traces(self._h, N.P_double(), 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), max(self.n_sensors, 1), 3))
        N.check(self._lib.pn_partitioned_get_traces(self._h, N.dptr(out), n.value, ctypes.byref(n)))
        return out[:n.value, :self.n_sensors]

    def info(self) -> dict:
        p, hn, lc = ctypes.c_int32(0), c_int64(0), c_int64(0)
        N.check(self._lib.pn_partitioned_info(self._h, ctypes.byref(p), ctypes.byref(hn), ctypes.byref(lc)))
        return {"n_parts": p.value, "halo_nodes": hn.value, "local_cells": lc.value}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.pn_partitioned_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


PIPE_RATE_NAMES = ("fp64_fma", "fp64_add", "fp32_fma", "cvt_f64_to_f32", "cvt_f32_to_f64", "int_xor_add")


def measure_pipe_rates() -> dict:
    """Thread-level operations per second of the arithmetic pipes on the
    current device (pn_measure_pipe_rates), keyed by PIPE_RATE_NAMES."""
    lib = N.load()
    out = np.zeros(len(PIPE_RATE_NAMES), np.float64)
    N.check(lib.pn_measure_pipe_rates(out.ctypes.data_as(N.P_double), len(PIPE_RATE_NAMES)))
    return dict(zip(PIPE_RATE_NAMES, out.tolist()))
