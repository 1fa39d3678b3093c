"""The divergence-free perturbation of the 3D adjoint configuration (cases.FourierPotential).

Face velocities are face fluxes of curl A by Stokes' theorem from exact edge integrals, so the
discrete divergence of every cell vanishes to rounding, the normal velocity on the domain walls
is zero (A vanishes there), and grad() is the exact transpose of the linear map.
"""
import numpy as np
import pytest

from ns_multiphase_gb300.cases import FourierPotential
from ns_multiphase_gb300.mesh import Mesh


@pytest.fixture(scope="module")
def setup():
    m = Mesh(Nx=12, Ny=10, Nz=9, Lx=1.0, Ly=0.8, Lz=0.9)
    return m, FourierPotential(m, 8)


def test_discretely_divergence_free(setup):
    m, F = setup
    C = 0.02 * np.random.default_rng(1).standard_normal((3, 8, 8, 8))
    uf, vf, wf = F.faces(C)
    div = ((uf[1:, :-1, :-1] - uf[:-1, :-1, :-1]) * (m.dy * m.dz) + (vf[:-1, 1:, :-1] - vf[:-1, :-1, :-1]) * (m.dx * m.dz)
           + (wf[:-1, :-1, 1:] - wf[:-1, :-1, :-1]) * (m.dx * m.dy))
    assert np.max(np.abs(div)) <= 1e-15 * max(1.0, np.max(np.abs(uf)))


def test_no_flow_through_the_walls(setup):
    m, F = setup
    C = np.random.default_rng(2).standard_normal((3, 8, 8, 8))
    uf, vf, wf = F.faces(C)
    g = m.nghost
    for f, ax, N in ((uf, 0, m.Nx), (vf, 1, m.Ny), (wf, 2, m.Nz)):
        for face in (g, g + N):
            sl = [slice(g, -g)] * 3
            sl[ax] = face
            assert np.max(np.abs(f[tuple(sl)])) <= 1e-13


def test_grad_is_the_transpose(setup):
    m, F = setup
    rng = np.random.default_rng(3)
    C = rng.standard_normal((3, 8, 8, 8))
    G = [rng.standard_normal(m.cell_shape) for _ in range(3)]
    lhs = sum(float(np.sum(a * b)) for a, b in zip(F.faces(C), G))
    rhs = float(np.sum(C * F.grad(*G)))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
