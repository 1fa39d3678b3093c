"""The CPU restatement of divg_cell / divergence! (src/Velocity.jl:59-122) and A!
(src/Pressure.jl:83-115), checked by invariants (the reference's tests hold no fixtures for
them): a uniform flow has no divergence; a linear flow u = a (x - x0) has divergence a, exactly
for the finite-difference scheme and to O(a^2 dt) for the semi-Lagrangian cells (their
pre-image volume is the cell's volume times exp(-a dt) up to the RK4 error); A! with zero
pressure is the divergence of the face velocities, and a pressure linear in x changes the
finite-difference divergence only through the density's variation."""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle


def state(N=10, tess="5_tets", xper=False):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess, xper=xper)
    o = Oracle(m)
    VF = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
    band = o.init_state(VF)[0]
    return m, o, band


def linear_faces(m, a):
    """uf = a (x - 0.5) at the faces, vf = wf = 0."""
    uf = m.cell_array()
    x = np.asarray(m.x)[:m.cell_shape[0]]  # x[i] of cells imino_..imaxo_
    uf[...] = (a * (x - 0.5))[:, None, None]
    return uf, m.cell_array(), m.cell_array()


@pytest.mark.parametrize("tess", ["5_tets", "6_tets", "24_tets"])
def test_uniform_flow_has_no_divergence(tess):
    m, o, band = state(tess=tess)
    uf, vf, wf = m.cell_array(), m.cell_array(), m.cell_array()
    uf[...] = 0.7
    vf[...] = -0.3
    wf[...] = 0.2
    dt = 0.5 * m.dx
    for scheme in (0, 1):  # semi-lagrangian, finite-difference
        divg = o.divergence(dt, uf, vf, wf, band, scheme)
        assert np.max(np.abs(m.interior(divg))) <= 1e-10, scheme
    assert np.count_nonzero(np.abs(m.interior(band)) <= m.nband) > 100


@pytest.mark.parametrize("tess", ["5_tets", "24_tets"])
def test_linear_flow_divergence(tess):
    m, o, band = state(tess=tess)
    a = 0.8
    uf, vf, wf = linear_faces(m, a)
    dt = 0.5 * m.dx
    fd = m.interior(o.divergence(dt, uf, vf, wf, band, 1))
    assert np.max(np.abs(fd - a)) <= 1e-12
    sl = m.interior(o.divergence(dt, uf, vf, wf, band, 0))
    inband = np.abs(m.interior(band)) <= m.nband
    assert inband.sum() > 100
    # the projected cell's volume is exp(-a dt) of the cell's, up to RK4's (a dt)^5/120
    exact = (1.0 - np.exp(-a * dt)) / dt
    assert np.max(np.abs(sl[inband] - exact)) <= 5e-8
    # cells outside the band: finite-difference fluxes (exact), SLfluxVol through a face next to
    # the band (the swept volume differs from the flux by O(a^2 dt x) per unit area)
    b = np.abs(band) <= m.nband
    near = np.zeros_like(b)
    for ax in range(3):
        near |= np.roll(b, 1, axis=ax) | np.roll(b, -1, axis=ax)
    near = m.interior(near)
    far = ~inband & ~near
    assert far.sum() > 100
    assert np.max(np.abs(sl[far] - a)) <= 1e-12
    assert np.max(np.abs(sl[~inband & near] - a)) <= 0.5 * a * a * dt / m.dx


def test_A_with_zero_pressure_is_the_divergence():
    m, o, band = state()
    uf, vf, wf = cases.deformation3d_faces(m, 0.3, 3.0)
    dt = 0.5 * m.dx / 2.0
    P = m.cell_array()
    ones = np.ones(m.cell_shape, order="F")
    for scheme in (0, 1):
        LHS = o.A(dt, P, uf, vf, wf, ones, ones, ones, band, scheme)[0]
        divg = o.divergence(dt, uf, vf, wf, band, scheme)
        # the corrected velocities equal uf only on A!'s index ranges; the interior's
        # stencils stay inside them
        assert np.array_equal(m.interior(LHS), m.interior(divg)), scheme


def test_A_pressure_gradient_terms():
    m, o, band = state()
    uf, vf, wf = m.cell_array(), m.cell_array(), m.cell_array()
    dt = 0.01
    P = m.cell_array()
    P[...] = (np.arange(m.cell_shape[0]) * 0.5)[:, None, None]   # dP/dx = 0.5 / dx per cell
    rho = np.ones(m.cell_shape, order="F")
    LHS, gx, gy, gz = o.A(dt, P, uf, vf, wf, rho, rho, rho, band, 1)
    # Neumann! copies P[1] to P[0] and P[N] to P[N+1], so the end faces see no gradient; the
    # others -dt*0.5/dx
    g = m.nghost
    assert np.all(gx[g, g:-g, g:-g] == 0.0) and np.all(gx[g + m.Nx, g:-g, g:-g] == 0.0)
    assert np.allclose(gx[g + 1:g + m.Nx, g:-g, g:-g], -dt * 0.5 / m.dx, rtol=1e-12)
    # ... which leaves divergence only in the first and last cell layers
    inner = m.interior(LHS)
    assert np.max(np.abs(inner[1:-1])) <= 1e-9
    assert np.allclose(inner[0], -dt * 0.5 / m.dx / m.dx, rtol=1e-9)
    assert np.allclose(inner[-1], dt * 0.5 / m.dx / m.dx, rtol=1e-9)
