"""CPU oracle for the RSG leapfrog -- TEST INFRASTRUCTURE ONLY.

Two CPU implementations with one calling convention:

* ``port``: oracle/pn_oracle.c, a plain-C restatement of the reference
  HostSolver algorithm (bit-identical by construction; pinned by the golden
  fixtures in tests/golden).  Built by ``make -C oracle`` into
  oracle/_build/libpn_oracle.so; travels everywhere.
* ``reference``: oracle/_ref/libpannde_ref.so, the reference's own
  header-only HostRSGTDUT / HostUTModel compiled from its sources by
  ``make -C oracle ref`` (only where the reference sources are present).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, and only as the checker / the timed CPU baseline.  The product
(pannde_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32
from pathlib import Path

import numpy as np

from pannde_gb300 import _native as N

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libpn_oracle.so"
REF_LIB = HERE / "_ref" / "libpannde_ref.so"
# the PanNDE sources: $PANNDE_REFERENCE, else a "reference" directory beside
# this repository's root
REF_SRC = Path(os.environ.get("PANNDE_REFERENCE") or (HERE.parent.parent / "reference"))

_RUN_ARGS = [POINTER(N.PnMesh), POINTER(N.PnMaterial), c_double, POINTER(N.P_double),
             POINTER(N.P_double), POINTER(N.PnWindowSource), c_int32, c_int32, N.P_int32, c_int32,
             N.P_double, POINTER(N.P_double), POINTER(N.P_double), N.P_double]

_libs: dict = {}


def build(reference: bool | None = None) -> None:
    """Compile the C port; also the reference driver when its sources exist."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if reference is None:
        reference = (REF_SRC / "modules" / "HostSolver" / "include" / "HostRSGTDUT.hpp").exists()
    if reference:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_SRC}"], check=True)


def port():
    """The C restatement (builds it if missing)."""
    if "port" not in _libs:
        if not PORT_LIB.exists():
            build(reference=False)
        lib = ctypes.CDLL(str(PORT_LIB))
        lib.pn_oracle_run.restype = c_int
        lib.pn_oracle_run.argtypes = _RUN_ARGS
        lib.pn_oracle_last_error.restype = c_char_p
        lib.pn_oracle_dd_cc.restype = c_int
        lib.pn_oracle_dd_cc.argtypes = [POINTER(N.PnMesh), N.P_double, c_int32, c_int32, N.P_double]
        lib.pn_oracle_dd_nc.restype = c_int
        lib.pn_oracle_dd_nc.argtypes = [POINTER(N.PnMesh), N.P_double, c_int32, c_int32,
                                        N.P_double, N.P_double]
        lib.pn_oracle_force_weights.restype = c_int
        lib.pn_oracle_force_weights.argtypes = [POINTER(N.PnMesh), POINTER(N.PnWindowSource),
                                                c_int32, N.P_double]
        _libs["port"] = lib
    return _libs["port"]


def reference():
    """The reference HostSolver compiled from its sources, or None if absent."""
    if "ref" not in _libs:
        if not REF_LIB.exists():
            return None
        lib = ctypes.CDLL(str(REF_LIB))
        lib.pnref_run.restype = c_int
        lib.pnref_run.argtypes = [c_int32] + _RUN_ARGS
        lib.pnref_last_error.restype = c_char_p
        lib.pnref_dd.restype = c_int
        lib.pnref_dd.argtypes = [POINTER(N.PnMesh), N.P_double, c_int32, c_int32, c_int32,
                                 N.P_double, N.P_double]
        _libs["ref"] = lib
    return _libs["ref"]


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


def run(mesh, material, dt, sources, nsteps, sensors=None, V0=None, S0=None, impl="port",
        model_kind=None):
    """Run nsteps of the leapfrog on the CPU.

    mesh: cases.HexMesh; material: (PnMaterial, keepalive) from
    Case.material_fields(); sources: list of cases.WindowSource.
    impl "port" (C restatement) or "reference" (compiled HostSolver);
    model_kind 0 = HostRSGTDUT, 1 = HostUTModel (default: 1 if any moment source).
    Returns dict(V=[3 arrays], S=[6 arrays], traces=[nsteps, nsens, 3], time).
    """
    from pannde_gb300.cases import sources_struct
    m, keep_m = mesh.as_struct()
    mat, keep_mat = material
    src, keep_s = sources_struct(sources)
    sens = N.i32(sensors if sensors is not None else np.zeros(0, np.int32))
    nsens = int(sens.shape[0])
    traces = np.zeros((max(nsteps, 1), max(nsens, 1), 3))
    V = [np.zeros(mesh.n_nodes) for _ in range(3)]
    S = [np.zeros(mesh.n_cells) for _ in range(6)]
    v0 = [N.f64(a) if a is not None else None for a in (V0 or [None] * 3)]
    s0 = [N.f64(a) if a is not None else None for a in (S0 or [None] * 6)]
    t = c_double(0.0)
    args = [ctypes.byref(m), ctypes.byref(mat), float(dt), N.ptr_array(v0), N.ptr_array(s0),
            src, len(sources), int(nsteps), N.iptr(sens), nsens, N.dptr(traces),
            N.ptr_array(V), N.ptr_array(S), ctypes.byref(t)]
    if impl == "port":
        lib = port()
        rc = lib.pn_oracle_run(*args)
        err = lib.pn_oracle_last_error
    else:
        lib = reference()
        if lib is None:
            raise FileNotFoundError(f"{REF_LIB} not built (reference sources absent)")
        if model_kind is None:
            model_kind = 1 if any(s.kind == N.PN_SOURCE_MOMENT for s in sources) else 0
        rc = lib.pnref_run(int(model_kind), *args)
        err = lib.pnref_last_error
    if rc != 0:
        msg = err()
        raise OracleError(rc, msg.decode() if msg else "")
    del keep_m, keep_mat, keep_s
    return dict(V=V, S=S, traces=traces[:nsteps, :nsens], time=t.value)


def dd(mesh, field, idx, axis, on_nodes, impl="port"):
    """RightHex DD*_cc (field on nodes, idx = cell) or DD*_nc (field on cells,
    idx = node).  Returns (value, node spacing or None)."""
    m, keep = mesh.as_struct()
    f = N.f64(field)
    out, sp = c_double(0.0), c_double(0.0)
    if impl == "port":
        lib = port()
        if on_nodes:
            rc = lib.pn_oracle_dd_cc(ctypes.byref(m), N.dptr(f), idx, axis, ctypes.byref(out))
        else:
            rc = lib.pn_oracle_dd_nc(ctypes.byref(m), N.dptr(f), idx, axis, ctypes.byref(out),
                                     ctypes.byref(sp))
        err = lib.pn_oracle_last_error
    else:
        lib = reference()
        rc = lib.pnref_dd(ctypes.byref(m), N.dptr(f), 1 if on_nodes else 0, idx, axis,
                          ctypes.byref(out), ctypes.byref(sp))
        err = lib.pnref_last_error
    if rc != 0:
        raise OracleError(rc, err().decode())
    del keep
    return out.value, (None if on_nodes else sp.value)


def force_weights(mesh, sources):
    from pannde_gb300.cases import sources_struct
    m, keep = mesh.as_struct()
    src, keep_s = sources_struct(sources)
    w = np.zeros((mesh.n_nodes, 3))
    rc = port().pn_oracle_force_weights(ctypes.byref(m), src, len(sources), N.dptr(w))
    if rc != 0:
        raise OracleError(rc, port().pn_oracle_last_error().decode())
    return w
