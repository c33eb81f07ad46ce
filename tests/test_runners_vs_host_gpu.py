"""The reference's own runners, unchanged, over the device solver against the
same runners over the reference HostSolver, on one GB300.

TransducerModel.cpp (HostRSGTDUT) and WaterColumnModel.cpp (HostUTModel) are
compiled three times from the reference's sources:
  host        the reference HostSolver headers, with the single-rank
              NetMPI::MPICommunicator, pass-through MetisPartitioner and
              VTK-free VTKGateway stand-ins (no MPI, METIS or VTK here)
  f64_exact   include/standin ahead of HostSolver: HostRSGTDUT / HostUTModel
              are DeviceSolver::DeviceRSGTDUT / DeviceUTModel, built with
              PN_DEFAULT_PRECISION=PN_PREC_F64_EXACT
  f64         the same with the default drop-in precision PN_PREC_F64
Each binary runs the same job file (pannde_gb300.vtu writers) through the
runner's own loop -- while(time < write_time) time = model->solve();
getStates(); writeSolution; writeTable("velocities")
(TransducerModel.cpp:63-83, WaterColumnModel.cpp:99-110) -- and every array
of every output file (<out>_<k>.vtu point and cell data, velocities_<k>.vtt
columns) is compared with the host run's: bit-identical for f64_exact,
<= 1e-10 relative L2 per array for f64 (each array's error taken relative
to at least 1e-6 of the largest norm among its file's arrays of the same
kind: a component that is pure round-off has no FP64-reorder-stable value).
Needs the reference sources ($PANNDE_REFERENCE) and a GPU; skipped otherwise.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from pannde_gb300 import cases, vtu

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
REF = oracle.REF_SRC
LIB = ROOT / "pannde_gb300" / "_build"
RUNNERS = REF / "applications" / "source" / "CaseRunners"
STANDIN = ROOT / "include" / "standin"
# the stand-ins a host build takes: everything but the solver aliases
HOST_STANDINS = ("MPICommunicator.hpp", "MetisPartitioner.hpp", "VTKGateway.hpp")


def build(tmp_path, name, variant):
    if not (RUNNERS / f"{name}.cpp").exists():
        pytest.skip("reference runner sources not present")
    out = tmp_path / f"{name}_{variant}"
    if variant == "host":
        inc_dir = tmp_path / "host_standin"
        inc_dir.mkdir(exist_ok=True)
        for h in HOST_STANDINS:
            shutil.copy(STANDIN / h, inc_dir / h)
        inc = ["-I", str(inc_dir), "-I", str(ROOT / "include")]
        defs = []
    else:
        inc = ["-I", str(STANDIN), "-I", str(ROOT / "include")]
        defs = ["-DPN_DEFAULT_PRECISION=PN_PREC_F64_EXACT"] if variant == "f64_exact" else []
    for m in ("PanNDE", "Controller", "HostData", "HostSolver", "Stubs"):
        inc += ["-I", str(REF / "modules" / m / "include")]
    inc += ["-I", str(REF / "applications" / "include")]
    # -ffp-contract=off: every product and sum rounded on its own, as written
    # (g++ fuses a*b+c into one FMA on aarch64 at -O2 otherwise, which is not
    # the reference's source-level arithmetic; the oracle builds the same way)
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-w", *defs, *inc, str(RUNNERS / f"{name}.cpp"),
           "-L", str(LIB),
           "-lpannde_gb300", f"-Wl,-rpath,{LIB}", "-lz", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def run(exe, job, cwd):
    cwd.mkdir(exist_ok=True)
    r = subprocess.run([str(exe), "-f", str(job), "-o", str(cwd / "out")], capture_output=True, text=True,
                       cwd=cwd, timeout=900)
    assert r.returncode == 0, (r.stdout + r.stderr)[-3000:]
    return sorted(p.name for p in cwd.iterdir() if p.suffix in (".vtu", ".vtt"))


def arrays(path):
    if path.suffix == ".vtt":
        return {"row": vtu.read_vtt(path)["columns"]}
    d = vtu.read_vtu(path)
    return {"point": d["point_data"], "cell": d["cell_data"]}


def compare_dirs(host_dir, dev_dir, files, exact):
    """Worst relative L2 over every array of every output file (exact: every
    array bit-identical, the differing ones listed)."""
    worst = 0.0
    bad = []
    for f in files:
        a, b = arrays(dev_dir / f), arrays(host_dir / f)
        assert a.keys() == b.keys()
        for kind in b:
            assert set(a[kind]) == set(b[kind]), (f, kind)
            norms = [np.linalg.norm(np.asarray(v, np.float64)) for v in b[kind].values()]
            floor = 1e-6 * max(norms) if norms else 0.0
            for name, hb in b[kind].items():
                hb = np.asarray(hb, np.float64)
                ha = np.asarray(a[kind][name], np.float64)
                assert ha.shape == hb.shape, (f, name)
                if exact:
                    if not np.array_equal(ha, hb):
                        bad.append((f, name, int((ha != hb).sum()), float(np.abs(ha - hb).max())))
                    continue
                d = max(np.linalg.norm(hb), floor)
                if d > 0:
                    worst = max(worst, float(np.linalg.norm(ha - hb) / d))
    assert not bad, f"arrays that differ (file, array, values, max abs): {bad[:12]}"
    return worst


def run_three(tmp_path, name, job):
    exes = {v: build(tmp_path, name, v) for v in ("host", "f64_exact", "f64")}
    files = {}
    for v, exe in exes.items():
        files[v] = run(exe, job, tmp_path / v)
    assert files["f64_exact"] == files["host"] == files["f64"]
    exact = compare_dirs(tmp_path / "host", tmp_path / "f64_exact", files["host"], exact=True)
    fast = compare_dirs(tmp_path / "host", tmp_path / "f64", files["host"], exact=False)
    print(f"{name}: files {files['host']}; f64_exact identical (max-rel {exact}); f64 max-rel {fast:.3e}")
    assert fast <= 1e-10
    return files["host"]


def test_transducer_model_device_equals_host(cuda_device, tmp_path):
    c = cases.al_plate_case(nx=24, ny=20, nz=4, nsteps=60, radius=0.6e-3)
    job = tmp_path / "plate.vtu"
    vtu.write_transducer_job(job, c, [20 * c.dt, 40 * c.dt, 60 * c.dt])
    files = run_three(tmp_path, "TransducerModel", job)
    for k in range(3):
        assert f"out_{k}.vtu" in files and f"velocities_{k}.vtt" in files


def test_water_column_model_device_equals_host(cuda_device, tmp_path):
    c = cases.bracket_case(5, water_column=True, scale=0.12, nsteps=30)
    job = tmp_path / "bracket.vtu"
    vtu.write_water_column_job(job, c, [10 * c.dt, 30 * c.dt])
    files = run_three(tmp_path, "WaterColumnModel", job)
    assert "out_0.vtu" in files and "out_1.vtu" in files
