"""Build the GB300 extension library ``libpannde_gb300.so`` in-tree.

Sources (``pannde_gb300/csrc``):
  rsg_fast.cu   fast FP64 / FP32 kernels      nvcc, sm_103a
  rsg_exact.cu  reference-order FP64 kernels  nvcc, sm_103a, -fmad=false
  rsg_grid.cu   fused voxel-grid step kernel  nvcc, sm_103a
  rsg_grid_tma.cu  grid step, tensor-copy staging (32 x 8 tiles)  nvcc, sm_103a
  rsg_grid_tma16.cu  the same with 32 x 16 tiles (FP32 storage)  nvcc, sm_103a
  rsg_grid_tma_f64.cu  the FP64 form's step (double-float / FP64 path per block)  nvcc, sm_103a
  rsg_state.cu  state convert / permute       nvcc, sm_103a
  rsg_split.cu  grid form: fix-up of split lattice sites (cracks)  nvcc, sm_103a
  pn_noalloc.cu fixed scratch of the allocation-free batch solve   nvcc
  rsg_energy.cu FP64 energy audit             nvcc, sm_103a
  rsg_pipes.cu  pipe issue-rate measurement   nvcc, sm_103a
  pn_energy.cpp energy audit tables           g++
  pn_partition.cpp partitioned solve (halo exchange on one device)  g++
  pn_setup.cpp  host table construction       g++, -ffp-contract=off, OpenMP loops
  pn_table.cpp  table form (any hex mesh)     g++
  pn_grid.cpp   grid form (voxel meshes)      g++
  pn_capi.cpp   C ABI                         g++
  pn_batch.cpp  batches of solvers            g++
Translation units compile in parallel; the link uses nvcc (static cudart).
Output: ``pannde_gb300/_build/libpannde_gb300.so``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libpannde_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _jobs() -> list[tuple[list[str], Path]]:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    inc = ["-I", str(CSRC), "-I", str(HERE.parent / "include")]
    # PN_BUILD_DEFINES: extra -D switches for the CUDA units (tuning sweeps)
    defs = [f"-D{d}" for d in os.environ.get("PN_BUILD_DEFINES", "").split()]
    common_cu = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", *defs, *inc]
    cxx = os.environ.get("CXX", "g++")
    common_cc = [cxx, "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                 "-I", str(cuda / "include"), *inc]
    jobs = [
        (common_cu + ["-c", str(CSRC / "rsg_fast.cu")], OUT / "rsg_fast.o"),
        (common_cu + ["-fmad=false", "-c", str(CSRC / "rsg_exact.cu")], OUT / "rsg_exact.o"),
        (common_cu + ["-c", str(CSRC / "rsg_grid.cu")], OUT / "rsg_grid.o"),
        (common_cu + ["-c", str(CSRC / "rsg_grid_tma.cu")], OUT / "rsg_grid_tma.o"),
        (common_cu + ["-c", str(CSRC / "rsg_grid_tma16.cu")], OUT / "rsg_grid_tma16.o"),
        (common_cu + ["-c", str(CSRC / "rsg_grid_tma_f64.cu")], OUT / "rsg_grid_tma_f64.o"),
        (common_cu + ["-c", str(CSRC / "rsg_state.cu")], OUT / "rsg_state.o"),
        (common_cu + ["-c", str(CSRC / "rsg_split.cu")], OUT / "rsg_split.o"),
        (common_cu + ["-c", str(CSRC / "pn_noalloc.cu")], OUT / "pn_noalloc.o"),
        (common_cu + ["-c", str(CSRC / "rsg_energy.cu")], OUT / "rsg_energy.o"),
        (common_cu + ["-c", str(CSRC / "rsg_pipes.cu")], OUT / "rsg_pipes.o"),
        (common_cc + ["-c", str(CSRC / "pn_energy.cpp")], OUT / "pn_energy.o"),
        (common_cc + ["-c", str(CSRC / "pn_partition.cpp")], OUT / "pn_partition.o"),
        (common_cc + ["-c", str(CSRC / "pn_setup.cpp")], OUT / "pn_setup.o"),
        (common_cc + ["-c", str(CSRC / "pn_table.cpp")], OUT / "pn_table.o"),
        (common_cc + ["-c", str(CSRC / "pn_grid.cpp")], OUT / "pn_grid.o"),
        (common_cc + ["-c", str(CSRC / "pn_capi.cpp")], OUT / "pn_capi.o"),
        (common_cc + ["-c", str(CSRC / "pn_batch.cpp")], OUT / "pn_batch.o"),
    ]
    return [(cmd + ["-o", str(obj)], obj) for cmd, obj in jobs]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    OUT.mkdir(parents=True, exist_ok=True)
    jobs = _jobs()
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(lambda j: _run(j[0]), jobs))
    nvcc = str(_cuda_home() / "bin" / "nvcc")
    link = [nvcc, "-shared", *ARCH, "-Xcompiler", "-fopenmp", "-o", str(LIB)] + [str(o) for _, o in jobs]
    _run(link)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
