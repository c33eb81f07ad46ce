"""ctypes view of the C ABI declared in include/pannde_gb300.h.

The library is the in-tree build ``pannde_gb300/_build/libpannde_gb300.so``.
There is no fallback: if it is missing, loading raises ``ExtensionMissing``.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libpannde_gb300.so"
ABI_VERSION = 3  # PN_ABI_VERSION of include/pannde_gb300.h these declarations follow

# status codes (enum pn_status)
PN_OK = 0
PN_ERR_INVALID = 1
PN_ERR_SPACING = 2
PN_ERR_RANGE = 3
PN_ERR_RUNTIME = 4
PN_ERR_CUDA = 5
PN_ERR_ALLOC = 6
PN_ERR_NOT_FINITE = 7
PN_ERR_DEVICE_CHECK = 8

# precision (enum pn_precision)
PN_PREC_F64_EXACT = 0
PN_PREC_F64 = 1
PN_PREC_F32 = 2
PN_PREC_DF64 = 3

# device forms (OR into the precision argument)
PN_FORM_AUTO = 0
PN_FORM_TABLE = 0x100
PN_FORM_GRID = 0x200

# field types (enum pn_field_type) == PanNDE::Field::FieldType
PN_FIELD_NODE = 0
PN_FIELD_CELL = 1
PN_FIELD_CONSTANT = 2

# source kinds
PN_SOURCE_FORCE = 0
PN_SOURCE_MOMENT = 1

P_double = POINTER(c_double)
P_int32 = POINTER(c_int32)


class PnMesh(ctypes.Structure):
    _fields_ = [("n_nodes", c_int32), ("n_cells", c_int32),
                ("x", P_double), ("y", P_double), ("z", P_double),
                ("hexes", P_int32), ("node_owner", P_int32), ("partition_id", c_int32)]


class PnField(ctypes.Structure):
    _fields_ = [("type", c_int32), ("data", P_double)]


class PnMaterial(ctypes.Structure):
    _fields_ = [("density", PnField), ("cij", PnField * 21)]


class PnMaterialTable(ctypes.Structure):
    _fields_ = [("n_materials", c_int32), ("density", P_double), ("cij", P_double),
                ("cell_material", P_int32)]


class PnSignal(ctypes.Structure):
    _fields_ = [("n", c_int32), ("t", P_double), ("v", P_double)]


class PnWindowSource(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("group", c_int32), ("component", c_int32),
                ("center", c_double * 3), ("radius", c_double), ("ds", c_double),
                ("signal", PnSignal)]


class PnWindowMask(ctypes.Structure):
    _fields_ = [("kind", c_int32), ("group", c_int32), ("component", c_int32),
                ("inside", POINTER(ctypes.c_uint8))]


class PnSolverInfo(ctypes.Structure):
    _fields_ = [("n_nodes", c_int32), ("n_cells", c_int32), ("precision", c_int32),
                ("n_materials", c_int32), ("uniform_spacing", c_int32),
                ("n_source_nodes", c_int32), ("n_source_cells", c_int32), ("n_sensors", c_int32),
                ("algorithmic_bytes_per_step", c_int64), ("device_bytes", c_int64),
                ("dt", c_double), ("time", c_double), ("form", c_int32), ("grid", c_int32 * 3),
                ("grid_kernel", c_int32)]


class PnPlan(ctypes.Structure):
    _fields_ = [("n_nodes", c_int32), ("n_cells", c_int32), ("n_materials", c_int32),
                ("uniform_spacing", c_int32), ("hx", c_double), ("hy", c_double), ("hz", c_double),
                ("device_bytes", c_int64), ("algorithmic_bytes_per_step", c_int64),
                ("form", c_int32), ("grid", c_int32 * 3)]


# every entry point the header declares: name -> (restype, argtypes)
SIGNATURES = {
    "pn_abi_version": (c_int, []),
    "pn_last_error": (c_char_p, []),
    "pn_plan_solver": (c_int, [POINTER(PnMesh), POINTER(PnMaterial), POINTER(PnMaterialTable),
                               c_double, c_int32, POINTER(PnPlan)]),
    "pn_plan_sources": (c_int, [POINTER(PnMesh), POINTER(PnWindowSource), c_int32, P_double,
                                P_double, P_int32, P_int32]),
    "pn_signal_eval": (c_int, [POINTER(PnSignal), P_double, c_int32, P_double]),
    "pn_solver_create": (c_int, [POINTER(PnMesh), POINTER(PnMaterial), c_double, c_int32,
                                 POINTER(c_void_p)]),
    "pn_solver_create_indexed": (c_int, [POINTER(PnMesh), POINTER(PnMaterialTable), c_double,
                                         c_int32, POINTER(c_void_p)]),
    "pn_solver_set_stream": (c_int, [c_void_p, c_void_p]),
    "pn_solver_set_state": (c_int, [c_void_p, POINTER(P_double), POINTER(P_double)]),
    "pn_solver_add_sources": (c_int, [c_void_p, POINTER(PnWindowSource), c_int32]),
    "pn_solver_add_window_masks": (c_int, [c_void_p, POINTER(PnWindowMask), c_int32]),
    "pn_solver_set_sensors": (c_int, [c_void_p, P_int32, c_int32, c_int32]),
    "pn_solver_solve": (c_int, [c_void_p, c_int32, P_double]),
    "pn_solver_solve_signals": (c_int, [c_void_p, c_int32, P_double, P_double]),
    "pn_solver_get_state": (c_int, [c_void_p, POINTER(P_double), POINTER(P_double)]),
    "pn_solver_get_traces": (c_int, [c_void_p, P_double, c_int64, POINTER(c_int64)]),
    "pn_solver_clear_traces": (c_int, [c_void_p]),
    "pn_solver_get_time": (c_int, [c_void_p, P_double]),
    "pn_solver_get_info": (c_int, [c_void_p, POINTER(PnSolverInfo)]),
    "pn_solver_device_state": (c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p)]),
    "pn_solver_energy": (c_int, [c_void_p, P_double, P_double]),
    "pn_solver_synchronize": (c_int, [c_void_p]),
    "pn_solver_enable_kernel_timing": (c_int, [c_void_p, c_int32]),
    "pn_solver_kernel_times": (c_int, [c_void_p, P_double, POINTER(c_int64)]),
    "pn_solver_destroy": (c_int, [c_void_p]),
    "pn_batch_create": (c_int, [POINTER(c_void_p)]),
    "pn_batch_add": (c_int, [c_void_p, c_void_p]),
    "pn_batch_remove": (c_int, [c_void_p, c_void_p]),
    "pn_batch_size": (c_int, [c_void_p, P_int32]),
    "pn_batch_set_stream": (c_int, [c_void_p, c_void_p]),
    "pn_batch_solve": (c_int, [c_void_p, c_int32]),
    "pn_batch_solve_noalloc": (c_int, [c_void_p, c_int32]),
    "pn_batch_plan_stats": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64), P_int32, P_int32, P_int32]),
    "pn_batch_synchronize": (c_int, [c_void_p]),
    "pn_batch_destroy": (c_int, [c_void_p]),
    "pn_partitioned_create": (c_int, [POINTER(PnMesh), POINTER(PnMaterialTable), c_double, c_int32, c_int32,
                                      POINTER(c_void_p)]),
    "pn_partitioned_add_sources": (c_int, [c_void_p, POINTER(PnWindowSource), c_int32]),
    "pn_partitioned_set_sensors": (c_int, [c_void_p, P_int32, c_int32, c_int32]),
    "pn_partitioned_set_state": (c_int, [c_void_p, POINTER(P_double), POINTER(P_double)]),
    "pn_partitioned_solve": (c_int, [c_void_p, c_int32, P_double]),
    "pn_partitioned_get_state": (c_int, [c_void_p, POINTER(P_double), POINTER(P_double)]),
    "pn_partitioned_get_traces": (c_int, [c_void_p, P_double, c_int64, POINTER(c_int64)]),
    "pn_partitioned_info": (c_int, [c_void_p, P_int32, POINTER(c_int64), POINTER(c_int64)]),
    "pn_partitioned_destroy": (c_int, [c_void_p]),
    "pn_measure_pipe_rates": (c_int, [P_double, c_int32]),
    "pn_solver_path_counts": (c_int, [c_void_p, POINTER(c_int64), POINTER(c_int64)]),
}


class ExtensionMissing(RuntimeError):
    """The CUDA extension library has not been built."""


class PnError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


_lib = None


def load(path: Path | None = None):
    """Load the extension library (once) and declare its prototypes."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ExtensionMissing(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.pn_abi_version() != ABI_VERSION:
        raise ExtensionMissing(f"{p} has ABI {lib.pn_abi_version()}, expected {ABI_VERSION}: rebuild it")
    if path is None:
        _lib = lib
    return lib


def check(code: int) -> None:
    if code != PN_OK:
        msg = load().pn_last_error()
        raise PnError(code, msg.decode() if msg else "")


# ---- helpers to pass numpy arrays -------------------------------------------

def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def dptr(a: np.ndarray | None):
    return a.ctypes.data_as(P_double) if a is not None else P_double()


def iptr(a: np.ndarray | None):
    return a.ctypes.data_as(P_int32) if a is not None else P_int32()


def ptr_array(arrays):
    """double*[k] from a list of float64 arrays (None -> NULL)."""
    arr = (P_double * len(arrays))()
    for k, a in enumerate(arrays):
        arr[k] = dptr(a) if a is not None else P_double()
    return arr
