"""Edge cases of the step on the GPU against the CPU restatement: an empty and a full domain
(nothing to transport, the band is empty), cells with three different spacings, an interface
that reaches the wall of a bounded domain (pre-images at the clamped index range), and grids
only a few cells wide.  FP64 bit for bit; the mixed path within its tolerance."""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()


def run_both(m, VF0, steps, t0=0.2, T=3.0, precision="fp64"):
    from ns_multiphase_gb300.slvof import SLVOF
    dt = 0.5 * min(m.dx, m.dy, m.dz) / 2.0
    o = Oracle(m)
    VFo = VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VFo)
    g = SLVOF(m, precision)
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    g.init_state()
    for n in range(steps):
        uf, vf, wf = cases.deformation3d_faces(m, t0 + (n + 0.5) * dt, T)
        g.upload_velocity(uf, vf, wf)
        mass = g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
    VFg = g.download_vf()
    counters = g.counters()
    g.close()
    return VFg, VFo, mass, o.mass(VFo), counters


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("fill", [0.0, 1.0])
def test_empty_and_full_domain(precision, fill):
    m = Mesh(Nx=12, Ny=10, Nz=8, Lx=1.2, Ly=1.0, Lz=0.8, CFL=0.5)
    VF0 = m.vf_array()
    m.interior(VF0)[...] = fill
    VFg, VFo, mass, mo, counters = run_both(m, VF0, 3, precision=precision)
    assert np.array_equal(m.interior(VFg), m.interior(VF0))
    assert counters["band_cells"] == 0 and counters["interface_cells"] == 0
    assert mass == mo == fill * m.Lx * m.Ly * m.Lz or abs(mass - mo) <= 1e-15


def test_three_different_spacings():
    m = Mesh(Nx=16, Ny=12, Nz=10, Lx=1.6, Ly=0.9, Lz=1.2, CFL=0.5)
    VF0 = cases.vf_spheres(m, np.array([[0.7, 0.45, 0.6]]), np.array([0.3]), nF=8)
    VFg, VFo, mass, mo, _ = run_both(m, VF0, 4)
    assert np.array_equal(VFg, VFo)
    assert abs(mass - mo) <= 1e-13 * mo
    VFm, _, mass_m, _, _ = run_both(m, VF0, 4, precision="mixed")
    assert np.max(np.abs(m.interior(VFm) - m.interior(VFo))) <= 5e-3
    # FP32 geometry: ~1e-7 per interface cell, relative to this small grid's few hundred cells
    assert abs(mass_m - mo) <= 2e-8 * mo


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_interface_at_the_wall(precision):
    """A sphere cut by the x = 0 and y = 0 walls of a bounded domain."""
    m = Mesh(Nx=16, Ny=16, Nz=16, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    VF0 = cases.vf_spheres(m, np.array([[0.04, 0.06, 0.5]]), np.array([0.3]), nF=8)
    VFg, VFo, mass, mo, _ = run_both(m, VF0, 5, precision=precision)
    if precision == "fp64":
        assert np.array_equal(VFg, VFo)
        assert abs(mass - mo) <= 1e-13 * mo
    else:
        assert np.max(np.abs(m.interior(VFg) - m.interior(VFo))) <= 5e-3
        assert abs(mass - mo) <= 2e-8 * mo


@pytest.mark.parametrize("N", [3, 5])
def test_few_cells(N):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, xper=True, yper=True, zper=True)
    VF0 = cases.vf_spheres(m, np.array([[0.5, 0.5, 0.5]]), np.array([0.3]), nF=8)
    VFg, VFo, mass, mo, _ = run_both(m, VF0, 3)
    assert np.array_equal(VFg, VFo)
    assert abs(mass - mo) <= 1e-13 * mo
