"""FP64 energy audit (pn_solver_energy).

The device sums are checked against a numpy restatement of the same
definitions on the state the device holds (the lumped nodal mass
rho_n * h^3 with rho_n = sum of the incident cells' density / 8, and
1/2 vol S . pinv(C) S per cell), for both forms and every precision; an
unforced leapfrog keeps the total bounded; and the FP32 form's energy
follows the FP64 form's within 1e-4.
"""
import numpy as np
import pytest

from pannde_gb300 import cases
from pannde_gb300.solver import Solver
from tests.test_parity_gpu import random_state

pytestmark = pytest.mark.gpu


def numpy_energy(case, V, S):
    m = case.mesh
    h3 = float(np.diff(np.unique(m.x))[0] * np.diff(np.unique(m.y))[0] * np.diff(np.unique(m.z))[0])
    rho_c = case.density[case.cell_material]
    rho_n = np.zeros(m.n_nodes)
    np.add.at(rho_n, m.hexes.reshape(-1), np.repeat(rho_c, 8) / 8.0)
    kin = 0.5 * np.sum(rho_n * h3 * (V[0] ** 2 + V[1] ** 2 + V[2] ** 2))
    comp = np.stack([np.linalg.pinv(cases.c6x6_from_21(c), rcond=1e-12) for c in case.cij])
    s = np.stack(S, axis=1)  # [cells, 6]
    q = np.einsum("ci,cij,cj->c", s, comp[case.cell_material], s)
    return kin, 0.5 * h3 * np.sum(q)


def pulse_state(mesh, width=3.0):
    """A smooth Gaussian velocity pulse at the centre of the mesh."""
    c = np.array([mesh.x.mean(), mesh.y.mean(), mesh.z.mean()])
    h = np.diff(np.sort(np.unique(mesh.x)))[0]
    r2 = ((mesh.x - c[0]) ** 2 + (mesh.y - c[1]) ** 2 + (mesh.z - c[2]) ** 2) / (width * h) ** 2
    g = np.exp(-r2)
    return [g, 0.5 * g, -0.25 * g], [np.zeros(mesh.n_cells) for _ in range(6)]


@pytest.mark.parametrize("form", ["grid", "table"])
@pytest.mark.parametrize("prec", ["f64", "df64", "f32"])
def test_energy_matches_numpy_on_device_state(cuda_device, form, prec):
    c = cases.laminate_case(nx=30, ny=21, nz=8, nsteps=20, radius=0.5e-3, n_sensors=3)
    V0, S0 = random_state(c.mesh, 4)
    with Solver.from_case(c, precision=prec, form=form) as s:
        s.set_state(V0, S0)
        s.solve(7)
        V, S = s.get_state()
        k, e = s.energy()
    kn, en = numpy_energy(c, V, S)
    assert k > 0 and e > 0
    assert abs(k - kn) <= 1e-12 * kn and abs(e - en) <= 1e-12 * en


def test_energy_bounded_without_sources_and_fp32_follows_fp64(cuda_device):
    c = cases.al_plate_case(nx=40, ny=40, nz=12, nsteps=400, radius=0.5e-3, n_sensors=3)
    V0, S0 = pulse_state(c.mesh)
    tot = {}
    for prec in ("f64", "f32"):
        with Solver(c.mesh, c, c.dt, prec) as s:
            s.set_state(V0, S0)
            seq = []
            for _ in range(8):
                s.solve(50)
                seq.append(sum(s.energy()))
            tot[prec] = np.array(seq)
    e64 = tot["f64"]
    assert np.all(np.abs(e64 - e64[0]) <= 0.02 * e64[0])  # leapfrog: bounded, no growth
    assert np.max(np.abs(tot["f32"] - e64) / e64) <= 1e-4
