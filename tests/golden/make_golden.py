"""Generate the golden fixtures of the RSG leapfrog from the reference itself.

Runs the reference HostSolver (HostRSGTDUT / HostUTModel, RightHex),
compiled from its own headers by ``make -C oracle ref`` into
oracle/_ref/libpannde_ref.so, on small seeded inputs and stores inputs and
outputs as .npz files beside this script.  The fixtures pin the C oracle
(tests/test_oracle_golden.py) and the device path (tests/test_golden_gpu.py)
to the reference bit for bit.

    python tests/golden/make_golden.py        # needs the reference sources
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from pannde_gb300 import _native as N  # noqa: E402
from pannde_gb300 import cases  # noqa: E402


def pack_sources(src):
    if not src:
        return dict(src_meta=np.zeros((0, 8)), src_off=np.zeros(1, np.int64),
                    src_t=np.zeros(0), src_v=np.zeros(0))
    meta = np.array([[s.kind, s.group, s.component, *s.center, s.radius, s.ds] for s in src])
    off = np.cumsum([0] + [len(s.times) for s in src]).astype(np.int64)
    return dict(src_meta=meta, src_off=off, src_t=np.concatenate([s.times for s in src]),
                src_v=np.concatenate([s.values for s in src]))


def unpack_sources(d):
    out = []
    for i, m in enumerate(d["src_meta"]):
        a, b = d["src_off"][i], d["src_off"][i + 1]
        out.append(cases.WindowSource(int(m[0]), int(m[1]), int(m[2]), tuple(m[3:6]), float(m[6]),
                                      float(m[7]), d["src_t"][a:b].copy(), d["src_v"][a:b].copy()))
    return out


def field_material(types, arrays):
    """(PnMaterial, keepalive) from 22 field types and arrays (density first)."""
    arrs = [N.f64(a) for a in arrays]
    m = N.PnMaterial()
    m.density = N.PnField(int(types[0]), N.dptr(arrs[0]))
    for k in range(21):
        m.cij[k] = N.PnField(int(types[k + 1]), N.dptr(arrs[k + 1]))
    return m, arrs


def fields_from_case(c):
    types = [N.PN_FIELD_CELL] * 22
    arrays = [c.density[c.cell_material]] + [c.cij[c.cell_material, k] for k in range(21)]
    return types, arrays


def save(name, mesh, types, arrays, dt, src, nsteps, sensors, model_kind, V0=None, S0=None):
    mat = field_material(types, arrays)
    r = oracle.run(mesh, mat, dt, src, nsteps, sensors, V0=V0, S0=S0, impl="reference",
                   model_kind=model_kind)
    d = dict(x=mesh.x, y=mesh.y, z=mesh.z, hexes=mesh.hexes,
             node_owner=mesh.node_owner if mesh.node_owner is not None else np.zeros(0, np.int32),
             partition_id=np.int32(mesh.partition_id),
             field_types=np.array(types, np.int32), dt=np.float64(dt), nsteps=np.int32(nsteps),
             sensors=np.asarray(sensors, np.int32), model_kind=np.int32(model_kind),
             V=np.stack(r["V"]), S=np.stack(r["S"]), traces=r["traces"], time=np.float64(r["time"]))
    for k, a in enumerate(arrays):
        d[f"field{k}"] = np.asarray(a, np.float64)
    if V0 is not None:
        d["V0"] = np.stack(V0)
        d["S0"] = np.stack(S0)
    d.update(pack_sources(src))
    np.savez_compressed(HERE / f"{name}.npz", **d)
    print(f"{name}: {mesh.n_cells} cells, {mesh.n_nodes} nodes, {nsteps} steps, "
          f"|V|max {np.abs(d['V']).max():.3e}")


def load(path):
    """Fixture -> dict(mesh, material (PnMaterial, keep), dt, sources, nsteps, sensors, ...)"""
    d = dict(np.load(path))
    owner = d["node_owner"] if d["node_owner"].size else None
    mesh = cases.HexMesh(d["x"], d["y"], d["z"], d["hexes"], owner, int(d["partition_id"]))
    arrays = [d[f"field{k}"] for k in range(22)]
    return dict(mesh=mesh, types=d["field_types"], arrays=arrays,
                material=field_material(d["field_types"], arrays), dt=float(d["dt"]),
                sources=unpack_sources(d), nsteps=int(d["nsteps"]), sensors=d["sensors"],
                model_kind=int(d["model_kind"]), V0=list(d["V0"]) if "V0" in d else None,
                S0=list(d["S0"]) if "S0" in d else None, V=d["V"], S=d["S"], traces=d["traces"],
                time=float(d["time"]))


def warped_block():
    solid = np.ones((9, 7, 5), dtype=bool)
    solid[3:5, 2:4, :] = False
    solid[7:, 0:2, 3:] = False
    m = cases.voxel_mesh(solid, 1e-3)
    i, j, k = m.node_ijk[:, 0], m.node_ijk[:, 1], m.node_ijk[:, 2]
    m.x = 1e-3 * (i + 0.15 * np.sin(1.3 * i))
    m.y = 1e-3 * (j + 0.1 * np.cos(0.7 * j))
    m.z = 0.5e-3 * (k + 0.2 * k * k / 5.0)
    return m


def main():
    if oracle.reference() is None:
        oracle.build(reference=True)
    # 1. TransducerModel's path: HostRSGTDUT, one z-force transducer, sensors
    c = cases.al_plate_case(nx=12, ny=10, nz=4, nsteps=40, radius=0.45e-3, n_sensors=6, seed=5)
    t, a = fields_from_case(c)
    save("rsgtdut_plate", c.mesh, t, a, c.dt, c.sources, c.nsteps, c.sensors, 0)

    # 2. WaterColumnModel's path: HostUTModel with a water column (XX,YY,ZZ
    #    moments) and two transducers on a holed, graded, anisotropic block,
    #    from a random state
    m = warped_block()
    ply = cases.orthotropic_ply(140e9, 10e9, 10e9, 6e9, 6e9, 4e9, 3e9, 5e9, 5e9)
    mats = [cases.rotate_about_z(ply, ang) for ang in (0, 45, -45, 90)]
    cm = (m.cell_ijk[:, 2] % 4).astype(np.int32)
    rho = np.array([1600.0, 1500.0, 1700.0, 1650.0])
    c21 = np.stack([cases.c21_from_6x6(x) for x in mats])
    types = [N.PN_FIELD_CELL] * 22
    arrays = [rho[cm]] + [c21[cm, k] for k in range(21)]
    rng = np.random.default_rng(17)
    V0 = [rng.uniform(-1e-3, 1e-3, m.n_nodes) for _ in range(3)]
    S0 = [rng.uniform(-1e5, 1e5, m.n_cells) for _ in range(6)]
    dt = 2e-9
    tt = np.arange(30) * dt * 0.7
    sig = np.sin(2e7 * tt)
    src = [cases.WindowSource(N.PN_SOURCE_MOMENT, 0, comp, (4.2e-3, 3.1e-3, 2.4e-3), 2.0e-3, 0.6e-3,
                              tt, sig * sc) for comp, sc in ((0, 1.0), (1, 0.5), (2, -0.8))]
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 0, 2, (2.0e-3, 2.0e-3, 2.4e-3), 1.5e-3, 0.6e-3, tt, sig))
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 1, 0, (6.0e-3, 4.0e-3, 2.4e-3), 1.5e-3, 0.6e-3, tt, -sig))
    src.append(cases.WindowSource(N.PN_SOURCE_FORCE, 1, 2, (6.0e-3, 4.0e-3, 2.4e-3), 1.5e-3, 0.6e-3, tt, sig))
    sens = np.array([0, 7, m.n_nodes // 3, m.n_nodes - 1], np.int32)
    save("utmodel_holes_moments", m, types, arrays, dt, src, 25, sens, 1, V0, S0)

    # 3. NODE and CONSTANT fields (HostField::atNode / atCell semantics) and
    #    node ownership on the same block
    m = warped_block()
    m.node_owner = (m.node_ijk[:, 0] >= 6).astype(np.int32)
    rng = np.random.default_rng(23)
    c21 = cases.c21_from_6x6(cases.isotropic(70e9, 0.33))
    types = [N.PN_FIELD_NODE, N.PN_FIELD_NODE] + [N.PN_FIELD_CONSTANT] * 20
    arrays = [rng.uniform(2000, 3000, m.n_nodes), c21[0] * rng.uniform(0.9, 1.1, m.n_nodes)]
    arrays += [np.array([c21[k]]) for k in range(1, 21)]
    V0 = [rng.uniform(-1e-3, 1e-3, m.n_nodes) for _ in range(3)]
    S0 = [rng.uniform(-1e5, 1e5, m.n_cells) for _ in range(6)]
    save("fields_ownership", m, types, arrays, 1e-9, [], 15, np.array([1, 50], np.int32), 0, V0, S0)

    # 4. RightHexTests meshes (HostRSGTDUTTests.hpp:121-257): operator values
    ops = []
    unit = cases.plate_builder(1.0, 1.0, 0.25, 1, 1)
    pack = cases.plate_builder(1.0, 1.0, 0.25, 2, 2)
    fields_u = {"x": unit.x, "y": unit.y, "z": unit.z,
                "dist": np.sqrt(unit.x ** 2 + unit.y ** 2 + unit.z ** 2),
                "index": np.arange(unit.n_nodes, dtype=np.float64)}
    for fi, (name, f) in enumerate(fields_u.items()):
        for axis in range(3):
            v, _ = oracle.dd(unit, f, 0, axis, True, impl="reference")
            ops.append((0, fi, axis, v, 0.0))
    cc = pack.cell_centers()
    for fi in range(3):
        for axis in range(3):
            v, sp = oracle.dd(pack, cc[:, fi], 13, axis, False, impl="reference")
            ops.append((1, fi, axis, v, sp))
    np.savez_compressed(HERE / "righthex_ops.npz", ops=np.array(ops))
    print(f"righthex_ops: {len(ops)} operator values")


if __name__ == "__main__":
    main()
