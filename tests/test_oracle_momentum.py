"""transport!'s momentum in the CPU restatement (src/Transport.jl:34-166, src/VFgeom.jl:428-509).

No reference fixture holds momentum values, so these are analytic checks: a uniform velocity
field is a steady solution of the convective update, for band cells (us = vrhoU/vrho over the
clipped pre-image, whatever the densities) and for the other cells, whose face fluxes mix
the finite-difference form and, at band edges, the semi-Lagrangian flux volume; and the flux
volume of a face in uniform flow is the swept prism, dt * (u . n) * face area.
"""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle


def state(tess, rho_liq=1000.0, rho_gas=1.2):
    m = Mesh(Nx=12, Ny=10, Nz=8, Lx=1.2, Ly=1.0, Lz=0.8, CFL=0.5, tesselation=tess, rho_liq=rho_liq,
             rho_gas=rho_gas)
    o = Oracle(m)
    VF = cases.vf_spheres(m, np.array([[0.55, 0.5, 0.4]]), np.array([0.27]), nF=8)
    band, nx, ny, nz, D = o.init_state(VF)
    return m, o, VF, band, nx, ny, nz, D


@pytest.mark.parametrize("tess", ["5_tets", "6_tets", "24_tets"])
def test_uniform_flow_keeps_uniform_momentum(tess):
    m, o, VF, band, nx, ny, nz, D = state(tess)
    U = (0.31, -0.22, 0.17)
    uf, vf, wf = cases.uniform_faces(m, *U)
    u, v, w = (np.full(m.cell_shape, x, order="F") for x in U)
    dt = 0.5 * m.dx / 0.31
    flags, us, vs, ws = o.transport_mom(dt, VF, uf, vf, wf, nx, ny, nz, D, band, u, v, w)
    assert flags == 0
    for got, x in zip((us, vs, ws), U):
        assert np.max(np.abs(m.interior(got) - x)) <= 1e-12, np.max(np.abs(m.interior(got) - x))
    # both kinds of cells are present
    inner = np.abs(m.interior(band).astype(int))
    assert (inner <= m.nband).any() and (inner > m.nband).any()


@pytest.mark.parametrize("tess", ["5_tets", "24_tets"])
def test_flux_volume_of_uniform_flow_is_the_swept_prism(tess):
    m, o = state(tess)[:2]
    U = (0.31, -0.22, 0.17)
    uf, vf, wf = cases.uniform_faces(m, *U)
    dt = 0.4 * m.dx / 0.31
    area = (m.dy * m.dz, m.dx * m.dz, m.dx * m.dy)
    for direction in range(3):
        for (i, j, k) in [(3, 4, 2), (4, 4, 2), (7, 2, 5)]:
            vol = o.sl_flux_vol(direction, i, j, k, uf, vf, wf, dt)
            assert abs(vol - dt * U[direction] * area[direction]) <= 1e-15, (direction, i, j, k, vol)
