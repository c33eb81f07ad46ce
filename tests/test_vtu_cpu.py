"""VTK XML I/O without the VTK library: the Python writer/reader
(pannde_gb300/vtu.py) and the C++ reader/writer (include/pn_vtu.hpp) agree on
every encoding the reader accepts (ascii, inline base64 binary, appended raw,
zlib-compressed), and a TransducerModel job written for a case carries
PanNDE's StandardNames keys."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from pannde_gb300 import cases, vtu

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def reader(tmp_path_factory):
    exe = tmp_path_factory.mktemp("vtu") / "vtu_check"
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-Wall", "-I", str(ROOT / "include"),
                        str(ROOT / "tests" / "cxx" / "vtu_check.cpp"), "-lz", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def summary(exe, path, out=None):
    args = [str(exe), str(path)] + ([str(out)] if out else [])
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = {}
    for line in r.stdout.splitlines():
        sec, name, n, s, q = line.split()
        rows[(sec, name)] = (int(n), float(s), float(q))
    return rows


def sample():
    c = cases.al_plate_case(nx=7, ny=5, nz=3, nsteps=4)
    m = c.mesh
    rng = np.random.default_rng(2)
    pts = np.stack([m.x, m.y, m.z], axis=1)
    pdata = {"Vx": rng.normal(size=m.n_nodes), "Vz": rng.normal(size=m.n_nodes)}
    cdata = {"density": np.full(m.n_cells, 2700.0), "C11": rng.uniform(1e9, 1e11, m.n_cells)}
    fdata = {"dt": np.array([4.6e-9]), "write_times": np.linspace(1e-7, 1e-6, 5)}
    return pts, m.hexes, pdata, cdata, fdata


@pytest.mark.parametrize("encoding,compress", [("binary", False), ("ascii", False), ("appended", False),
                                               ("appended", True), ("binary", True)])
def test_cpp_reads_python_files(reader, tmp_path, encoding, compress):
    pts, hexes, pdata, cdata, fdata = sample()
    f = tmp_path / "job.vtu"
    vtu.write_vtu(f, pts, hexes, pdata, cdata, fdata, encoding=encoding, compress=compress)
    rows = summary(reader, f)
    def check(key, a):
        n, s, q = rows[key]
        a = np.asarray(a, dtype=np.float64).reshape(-1)
        assert n == a.size
        np.testing.assert_allclose([s, q], [a.sum(), (a * a).sum()], rtol=1e-12, atol=1e-300)
    check(("Points", "points"), pts)
    check(("Cells", "connectivity"), hexes)
    for k, v in pdata.items():
        check(("PointData", k), v)
    for k, v in cdata.items():
        check(("CellData", k), v)
    for k, v in fdata.items():
        check(("FieldData", k), v)


def test_python_reads_cpp_files(reader, tmp_path):
    pts, hexes, pdata, cdata, fdata = sample()
    f, g = tmp_path / "a.vtu", tmp_path / "b.vtu"
    vtu.write_vtu(f, pts, hexes, pdata, cdata, fdata)
    summary(reader, f, g)
    back = vtu.read_vtu(g)
    assert np.array_equal(back["points"], pts) and np.array_equal(back["hexes"], hexes)
    for k, v in pdata.items():
        assert np.array_equal(back["point_data"][k], v)
    for k, v in cdata.items():
        assert np.array_equal(back["cell_data"][k], v)
    for k, v in fdata.items():
        assert np.array_equal(back["field_data"][k], v)


def test_transducer_job_keys(tmp_path):
    c = cases.al_plate_case(nx=10, ny=8, nz=3, nsteps=20)
    f = tmp_path / "plate.vtu"
    vtu.write_transducer_job(f, c, [1e-7, 2e-7])
    d = vtu.read_vtu(f)
    assert set(vtu.CIJ_NAMES) | {"density"} <= set(d["cell_data"])
    fd = d["field_data"]
    assert fd["dt"][0] == c.dt and fd["NTransducers"][0] == 1
    for key in ("XD0/XCenter", "XD0/YCenter", "XD0/ZCenter", "XD0/Radius", "XD0/SignalTimes", "XD0/SignalValues"):
        assert key in fd
    assert np.array_equal(fd["XD0/SignalValues"], c.sources[0].values)


def test_standin_gateway_reads_and_writes(tmp_path):
    """include/standin/VTKGateway.hpp over the reference's HostData factories."""
    ref = oracle.REF_SRC
    if not (ref / "modules" / "HostData" / "include" / "HostField.hpp").exists():
        pytest.skip("reference headers not present")
    inc = ["-I", str(ROOT / "include" / "standin"), "-I", str(ROOT / "include")]
    for m in ("PanNDE", "Controller", "HostData"):
        inc += ["-I", str(ref / "modules" / m / "include")]
    exe = tmp_path / "gateway_check"
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-w", *inc, str(ROOT / "tests" / "cxx" / "gateway_check.cpp"),
                        "-lz", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    pts, hexes, pdata, cdata, fdata = sample()
    job = tmp_path / "job.vtu"
    vtu.write_vtu(job, pts, hexes, pdata, cdata, fdata, encoding="appended", compress=True)
    r = subprocess.run([str(exe), str(job), str(tmp_path / "sol")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    nn, nc, trho, tvx, rsum, vsum, dt, nwt = r.stdout.split()
    assert int(nn) == len(pts) and int(nc) == len(hexes)
    assert int(trho) == 1 and int(tvx) == 0  # CELL, NODE
    assert float(rsum) == pytest.approx(cdata["density"].sum(), rel=1e-15)
    assert float(vsum) == pytest.approx(pdata["Vx"].sum(), rel=1e-12)
    assert float(dt) == fdata["dt"][0] and int(nwt) == fdata["write_times"].size
    sol = vtu.read_vtu(tmp_path / "sol_3.vtu")
    assert np.array_equal(sol["points"], pts) and np.array_equal(sol["hexes"], hexes)
    assert np.array_equal(sol["cell_data"]["density"], cdata["density"])
    assert np.array_equal(sol["point_data"]["Vx"], pdata["Vx"])
    assert sol["field_data"]["time"][0] == 1.5e-6
    tab = vtu.read_vtt(tmp_path / "sol_table_3.vtt")
    assert np.array_equal(tab["columns"]["write_times"], fdata["write_times"])


def same_problem(a, b):
    """Two cases describe the same solve: mesh, every cell's density and
    stiffness, dt and the excitation windows with their signals."""
    assert np.array_equal(a.mesh.x, b.mesh.x) and np.array_equal(a.mesh.y, b.mesh.y)
    assert np.array_equal(a.mesh.z, b.mesh.z) and np.array_equal(a.mesh.hexes, b.mesh.hexes)
    assert np.array_equal(a.density[a.cell_material], b.density[b.cell_material])
    assert np.array_equal(a.cij[a.cell_material], b.cij[b.cell_material])
    assert a.dt == b.dt and len(a.sources) == len(b.sources)
    key = lambda s: (s.kind, s.group, s.component)
    for s, t in zip(sorted(a.sources, key=key), sorted(b.sources, key=key)):
        assert (s.kind, s.component, tuple(s.center), s.radius, s.ds) == \
               (t.kind, t.component, tuple(t.center), t.radius, t.ds)
        assert np.array_equal(s.times, t.times) and np.array_equal(s.values, t.values)


@pytest.mark.parametrize("encoding,compress", [("binary", False), ("appended", True)])
def test_transducer_job_reads_back_the_problem(tmp_path, encoding, compress):
    c = cases.laminate_case(nx=12, ny=10, nz=8, nsteps=20, radius=0.2e-3, n_sensors=4)
    f = tmp_path / "lam.vtu"
    vtu.write_transducer_job(f, c, [5 * c.dt, 10 * c.dt], encoding=encoding, compress=compress)
    r = vtu.read_transducer_job(f, sensors=c.sensors, nsteps=c.nsteps)
    same_problem(c, r)
    assert np.array_equal(r.meta["write_times"], [5 * c.dt, 10 * c.dt])


@pytest.mark.parametrize("encoding,compress", [("binary", False), ("appended", True)])
def test_water_column_job_reads_back_the_problem(tmp_path, encoding, compress):
    c = cases.bracket_case(5, water_column=True, scale=0.12, nsteps=20)
    f = tmp_path / "wc.vtu"
    vtu.write_water_column_job(f, c, [5 * c.dt], encoding=encoding, compress=compress)
    same_problem(c, vtu.read_water_column_job(f, sensors=c.sensors, nsteps=c.nsteps))
