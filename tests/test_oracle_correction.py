"""The restatement of the flux-correction tets (add_correction_tets, src/VFgeom.jl:514-664;
pressure_scheme "finite-difference", src/Transport.jl:121-124), checked by what they are for:
with them, a band cell's transported volume is the cell volume minus dt times the
finite-difference flux balance, i.e. (v2 - vol)/v2/dt is the finite-difference divergence of
the face velocities (src/Velocity.jl:71-122), for any velocity field; without them it is the
projected cell's volume.  The reference's tests hold no fixture for them."""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle


def setup(scheme, seed=5):
    m = Mesh(Nx=12, Ny=12, Nz=12, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, pressure_scheme=scheme)
    o = Oracle(m)
    VF = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
    band, nx, ny, nz, D = o.init_state(VF)
    uf, vf, wf = cases.deformation3d_faces(m, 0.3, 3.0)
    rng = np.random.default_rng(seed)
    for f in (uf, vf, wf):
        f += 0.1 * rng.standard_normal(f.shape)   # not divergence-free
    dt = 0.5 * m.dx / 2.0
    return m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt


def band_cells(m, band, count=20):
    idx = [(i, j, k) for k in range(2, m.Nz) for j in range(2, m.Ny) for i in range(2, m.Nx)
           if abs(int(band[m.cidx(i, j, k)])) <= m.nband]
    rng = np.random.default_rng(1)
    return [idx[q] for q in rng.choice(len(idx), size=min(count, len(idx)), replace=False)]


def test_corrected_volume_matches_finite_difference_divergence():
    m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt = setup("finite-difference")
    fd = o.divergence(dt, uf, vf, wf, band, 1)
    sl = o.divergence(dt, uf, vf, wf, band, 0)
    v2 = m.dx * m.dy * m.dz
    cells = band_cells(m, band)
    assert len(cells) >= 10
    worst_fd, worst_sl = 0.0, 0.0
    for c in cells:
        r, vol, flags = o.sl_cell(dt, *c, uf, vf, wf, nx, ny, nz, D)
        assert flags == 0 and 0.0 <= r <= 1.0 + 1e-12
        d = (v2 - vol) / v2 / dt
        worst_fd = max(worst_fd, abs(d - fd[m.cidx(*c)]))
        worst_sl = max(worst_sl, abs(d - sl[m.cidx(*c)]))
    assert worst_fd <= 1e-9 * max(1.0, np.max(np.abs(fd)))
    assert worst_sl > 1e-6   # the correction changes the volume


def test_semi_lagrangian_scheme_has_no_correction():
    m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt = setup("semi-lagrangian")
    sl = o.divergence(dt, uf, vf, wf, band, 0)
    v2 = m.dx * m.dy * m.dz
    for c in band_cells(m, band, 10):
        r, vol, flags = o.sl_cell(dt, *c, uf, vf, wf, nx, ny, nz, D)
        assert abs((v2 - vol) / v2 / dt - sl[m.cidx(*c)]) <= 1e-9
