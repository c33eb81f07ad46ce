"""The host tables do not depend on the number of threads that build them.

pn_setup.cpp builds the links (HexMesh::buildLinks, "later cells win"), the
spacings (RightHex nodePrep / cellPrep, first bad node reported), the
de-duplicated material table (rows numbered in order of first appearance)
the voxel-grid map (split sites numbered in node order) and the source
entries (concatenated per run of elements, in element order) with OpenMP
loops.  tests/cxx/setup_digest.cpp digests every table; the digests and the
error messages must be identical with 1 thread and with several, on voxel
meshes with cracks as disconnected faces, fluid columns, removed slabs,
shuffled numbering, partition ownership, duplicated cells and per-cell
materials, and on rejected inputs.
"""
import json
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "pannde_gb300" / "csrc"

SCRIPT = r'''
import ctypes, json, sys
import numpy as np
sys.path.insert(0, sys.argv[2])
from pannde_gb300 import cases
lib = ctypes.CDLL(sys.argv[1])

def digest(c, fields, mesh=None):
    m, k1 = (mesh or c.mesh).as_struct()
    if fields:
        mat, k2 = c.material_fields(); tab = None
    else:
        tab, k2 = c.material_table(); mat = None
    out = (ctypes.c_uint64 * 40)(); msg = ctypes.create_string_buffer(256)
    n = lib.setup_digest(ctypes.byref(m), ctypes.byref(mat) if mat else None,
                         ctypes.byref(tab) if tab else None, ctypes.c_double(c.dt), out, msg, 256)
    return [n, [str(v) for v in out[:max(n, 0)]], msg.value.decode()]

def plan(c, mode):
    """pn_plan_solver of the library itself (host-only): form, footprint, lattice."""
    from pannde_gb300 import _native as N
    m, k1 = c.mesh.as_struct()
    tab, k2 = c.material_table()
    out = N.PnPlan()
    rc = N.load().pn_plan_solver(ctypes.byref(m), None, ctypes.byref(tab), c.dt, mode, ctypes.byref(out))
    return [rc, out.n_materials, out.form, out.device_bytes, out.algorithmic_bytes_per_step, list(out.grid)]

def digest_sources(mesh, srcs, exact):
    m, k1 = mesh.as_struct()
    st, k2 = cases.sources_struct(srcs)
    out = (ctypes.c_uint64 * 4)(); msg = ctypes.create_string_buffer(256)
    n = lib.setup_digest_sources(ctypes.byref(m), st, len(srcs), exact, out, msg, 256)
    return [n, [str(v) for v in out[:max(n, 0)]], msg.value.decode()]

res = {}
small = cases.al_plate_case(nx=24, ny=20, nz=6, nsteps=4)
m = small.mesh
rng = np.random.default_rng(5)
pc, pn_ = rng.permutation(m.n_cells), rng.permutation(m.n_nodes)
inv = np.argsort(pn_)
shuffled = cases.Case("s", cases.HexMesh(m.x[pn_], m.y[pn_], m.z[pn_], inv[m.hexes[pc]].astype(np.int32)),
                      small.density, small.cij, small.cell_material[pc], small.dt)
nm = 40
many = cases.Case("m", m, small.density[[0] * nm] * rng.uniform(0.9, 1.1, nm),
                  small.cij[[0] * nm] * rng.uniform(0.9, 1.1, (nm, 1)),
                  rng.integers(0, nm, m.n_cells).astype(np.int32), small.dt)
dup = cases.Case("d", cases.HexMesh(m.x, m.y, m.z, np.concatenate([m.hexes, m.hexes[5:9]])),
                 small.density, small.cij, np.concatenate([small.cell_material, small.cell_material[5:9]]), small.dt)
owners = cases.HexMesh(m.x, m.y, m.z, m.hexes, node_owner=(np.arange(m.n_nodes) % 3).astype(np.int32),
                       partition_id=1)
iso = cases.HexMesh(np.append(m.x, 1.0), np.append(m.y, 1.0), np.append(m.z, 1.0), m.hexes)
bad_id = m.hexes.copy(); bad_id[40, 3] = m.n_nodes + 2; bad_id[50, 1] = -1
for fields in (0, 1):
    for seed in range(3):
        for wc in (False, True):
            for crack in ("faces", "slab"):
                c = cases.bracket_case(100 + seed, nsteps=4, water_column=wc, scale=0.3, crack=crack)
                res[f"bracket{seed}-{wc}-{crack}-{fields}"] = digest(c, fields)
                if fields:
                    for mode in (1, 2, 3):  # f64, f32, df64; form chosen automatically
                        res[f"plan-bracket{seed}-{wc}-{crack}-{mode}"] = plan(c, mode)
    res[f"shuffled-{fields}"] = digest(shuffled, fields)
    res[f"materials-{fields}"] = digest(many, fields)
    res[f"duplicated-{fields}"] = digest(dup, fields)
    res[f"owners-{fields}"] = digest(small, fields, owners)
    res[f"isolated-{fields}"] = digest(small, fields, iso)
    res[f"bad-id-{fields}"] = digest(small, fields, cases.HexMesh(m.x, m.y, m.z, bad_id))
F, M = cases.N.PN_SOURCE_FORCE, cases.N.PN_SOURCE_MOMENT
zt, h, s0 = m.z.max(), 0.1e-3, small.sources[0]
mixed = [cases.WindowSource(F, g, d, (1e-3 + g * 0.8e-3, 1e-3, zt), 0.9e-3, h, s0.times, s0.values)
         for g in range(2) for d in range(3)]
mixed += [cases.WindowSource(M, 0, k, (1.2e-3, 1e-3, zt), 0.7e-3, h, s0.times, s0.values) for k in range(6)]
for exact in (0, 1):
    res[f"sources-mixed-{exact}"] = digest_sources(m, mixed, exact)
    res[f"sources-owners-{exact}"] = digest_sources(owners, mixed, exact)
    for wc in (False, True):
        c = cases.bracket_case(200, nsteps=4, water_column=wc, scale=0.4)
        res[f"sources-bracket-{wc}-{exact}"] = digest_sources(c.mesh, c.sources, exact)
print(json.dumps(res))
'''


@pytest.fixture(scope="module")
def digest_lib(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = tmp_path_factory.mktemp("setup") / "libsetup_digest.so"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-I", str(CSRC), "-I", str(ROOT / "include"), "-shared", "-o", str(out),
           str(ROOT / "tests" / "cxx" / "setup_digest.cpp"), str(CSRC / "pn_setup.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run_with_threads(lib, threads, **extra):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), **extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(lib), str(ROOT)], capture_output=True,
                       text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def test_host_tables_independent_of_thread_count(digest_lib):
    one = run_with_threads(digest_lib, 1)
    # the inputs exercise what they are meant to: split sites, rejections, materials
    assert any(int(v[1][-7]) > 0 for k, v in one.items() if "faces" in k and v[0] > 30)
    assert one["isolated-0"][2].startswith("2 DX") and one["bad-id-1"][2].startswith("3 invalid node id")
    assert one["duplicated-0"][0] > 0 and one["materials-1"][0] > 0
    assert all(v[0] == 0 for k, v in one.items() if k.startswith("plan-"))
    assert all(int(v[1][0]) > 0 and int(v[1][1]) > 0 for k, v in one.items() if k.startswith("sources-mixed"))
    for threads in (3, 8):
        assert run_with_threads(digest_lib, threads) == one
    # teams smaller than asked for (a thread limit below the thread count)
    assert run_with_threads(digest_lib, 8, OMP_THREAD_LIMIT="3") == one
