"""The reference's own runners, TransducerModel.cpp and WaterColumnModel.cpp,
compile and link unchanged against the device solver when include/standin
precedes the reference's headers (single-rank NetMPI::MPICommunicator,
pass-through NetMPI::MetisPartitioner, VTK-free VTKIO::VTKGateway, and
HostSolver::HostRSGTDUT / HostUTModel mapped to the device classes).  Run on
a job that pannde_gb300.vtu wrote, each reads its mesh, material fields,
excitations and timing through the stand-in gateway and reaches model
construction; with a GPU it runs and writes <out>_<k>.vtu and
velocities_<k>.vtt, without one model construction reports that no CUDA
device is usable.  Skipped where the reference sources are absent."""
import shutil
import subprocess
from pathlib import Path

import pytest

import oracle

from pannde_gb300 import cases, vtu

ROOT = Path(__file__).resolve().parent.parent
REF = oracle.REF_SRC
LIB = ROOT / "pannde_gb300" / "_build"
RUNNERS = REF / "applications" / "source" / "CaseRunners"


def build(tmp_path, name):
    if not (RUNNERS / f"{name}.cpp").exists():
        pytest.skip("reference runner sources not present")
    inc = ["-I", str(ROOT / "include" / "standin"), "-I", str(ROOT / "include")]
    for m in ("PanNDE", "Controller", "HostData", "HostSolver", "Stubs"):
        inc += ["-I", str(REF / "modules" / m / "include")]
    inc += ["-I", str(REF / "applications" / "include")]
    exe = tmp_path / name
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-ffp-contract=off", "-w", *inc, str(RUNNERS / f"{name}.cpp"), "-L", str(LIB),
                        "-lpannde_gb300", f"-Wl,-rpath,{LIB}", "-lz", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def run(exe, job, cwd):
    cmd = [str(exe), "-f", str(job), "-o", str(cwd / "out")]
    if shutil.which("stdbuf"):
        cmd = ["stdbuf", "-oL"] + cmd
    return subprocess.run(cmd, capture_output=True, text=True, cwd=cwd, timeout=600)


def check(r, cwd, loaded):
    for line in loaded:
        assert line in r.stdout, r.stdout + r.stderr
    if r.returncode == 0:  # a GPU: the run completed and wrote its outputs
        assert (cwd / "out_0.vtu").exists()
    else:
        assert "CUDA" in r.stderr or "cuda" in r.stderr, r.stdout + r.stderr


def test_transducer_model_runs_unchanged(tmp_path):
    exe = build(tmp_path, "TransducerModel")
    c = cases.al_plate_case(nx=16, ny=16, nz=4, nsteps=30, radius=0.5e-3)
    job = tmp_path / "plate.vtu"
    vtu.write_transducer_job(job, c, [10 * c.dt, 20 * c.dt])
    r = run(exe, job, tmp_path)
    check(r, tmp_path, ["load fields", "Loading 1 transducers", "dt=4.657685e-09", "build model"])
    if r.returncode == 0:
        tab = vtu.read_vtt(tmp_path / "velocities_1.vtt")
        assert set(tab["columns"]) == {"Vx", "Vy", "Vz"}


def test_water_column_model_runs_unchanged(tmp_path):
    exe = build(tmp_path, "WaterColumnModel")
    c = cases.bracket_case(5, water_column=True, scale=0.12, nsteps=20)
    job = tmp_path / "bracket.vtu"
    vtu.write_water_column_job(job, c, [5 * c.dt])
    r = run(exe, job, tmp_path)
    check(r, tmp_path, ["load timing data", "commence model creation"])
