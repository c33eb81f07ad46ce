"""Partitioned solve on one device (pn_partitioned_*): the reference's domain
decomposition -- home nodes by coordinate bisection, local meshes of the
cells touching home nodes, one velocity halo exchange per step, halo cells
recomputed -- gives the single-partition result bit for bit, for any number
of partitions, with sources, sensors, holes and a random state."""
import numpy as np
import pytest

from pannde_gb300 import _native as N
from pannde_gb300 import cases
from pannde_gb300.solver import Partitioned, Solver
from tests.test_parity_gpu import random_state


def run_single(c, prec, steps, V0=None, S0=None):
    with Solver.from_case(c, precision=prec, form="table", capacity=steps) as s:
        if V0 is not None:
            s.set_state(V0, S0)
        s.solve(steps)
        return s.get_state(), s.traces(), s.time


def run_parts(c, prec, steps, parts, V0=None, S0=None):
    with Partitioned(c, parts, prec) as p:
        if c.sources:
            p.add_sources(c.sources)
        p.set_sensors(c.sensors, steps)
        if V0 is not None:
            p.set_state(V0, S0)
        t = p.solve(steps)
        info = p.info()
        return (p.get_state(), p.traces(), t), info


def same(a, b):
    (Va, Sa), ta, tta = a
    (Vb, Sb), tb, ttb = b
    assert tta == ttb
    for k in range(3):
        assert np.array_equal(Va[k], Vb[k]), f"V{k}"
    for k in range(6):
        assert np.array_equal(Sa[k], Sb[k]), f"S{k}"
    assert np.array_equal(ta, tb)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32", "df64"])
@pytest.mark.parametrize("parts", [1, 2, 3, 5])
def test_partitioned_equals_single(cuda_device, prec, parts):
    c = cases.laminate_case(nx=30, ny=22, nz=8, nsteps=25, radius=0.5e-3, n_sensors=7)
    ref = run_single(c, prec, 25)
    got, info = run_parts(c, prec, 25, parts)
    assert info["n_parts"] == parts and (parts == 1) == (info["halo_nodes"] == 0)
    same(got, ref)


@pytest.mark.gpu
def test_partitioned_holes_random_state(cuda_device):
    solid = np.ones((26, 14, 6), dtype=bool)
    solid[8:12, 4:9, :] = False
    solid[18:, 0:3, 3:] = False
    m = cases.voxel_mesh(solid, 1e-4)
    c = cases.Case("h", m, np.array([2700.0]), cases.c21_from_6x6(cases.isotropic(70e9, 0.33))[None],
                   np.zeros(m.n_cells, np.int32), 4e-9, [], cases.seeded_sensors(m, 5, 3), 20)
    V0, S0 = random_state(m, 11)
    ref = run_single(c, "f64", 20, V0, S0)
    got, info = run_parts(c, "f64", 20, 4, V0, S0)
    assert info["halo_nodes"] > 0
    same(got, ref)


def test_partitioned_refuses_exact_form_and_given_owners():
    c = cases.al_plate_case(nx=6, ny=5, nz=2, nsteps=2)
    with pytest.raises(N.PnError) as e:
        Partitioned(c, 2, "f64_exact")
    assert e.value.code == N.PN_ERR_INVALID
    c.mesh.node_owner = np.zeros(c.mesh.n_nodes, np.int32)
    with pytest.raises(N.PnError) as e:
        Partitioned(c, 2, "f64")
    assert e.value.code == N.PN_ERR_INVALID
    c.mesh.node_owner = None
