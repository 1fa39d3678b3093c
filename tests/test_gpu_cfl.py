"""The step at CFL numbers above the benchmark's 0.5: pre-images that reach one to three cells
away, so donors lie beyond the 3x3x3 neighbourhood the mixed clip caches and index boxes are
wider than 2, and the reference widens the band (nband = ceil(CFL), src/Parameters.jl:70) and
from CFL > 2 the ghost layers (nghost = 3 + ceil(CFL) - 2, src/Mesh.jl:66).  FP64 bit for
bit against the CPU restatement; the mixed path within its tolerance."""
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


def run(m, VF0, steps, precision):
    from ns_multiphase_gb300.slvof import SLVOF
    dt = m.CFL * m.dx / 2.0  # Deformation3D: max |u| = 2
    o = Oracle(m)
    VFo = VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VFo)
    g = SLVOF(m, precision)
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    g.init_state()
    for n in range(steps):
        uf, vf, wf = cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
        g.upload_velocity(uf, vf, wf)
        mass = g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
    VFg = g.download_vf()
    g.close()
    return VFg, VFo, mass, o.mass(VFo)


@pytest.mark.parametrize("scheme", ["semi-lagrangian", "finite-difference"])
@pytest.mark.parametrize("cfl", [1.0, 2.0, 3.0])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_at_larger_cfl(cfl, precision, scheme):
    """With pressure_scheme "finite-difference" the correction tets' apexes also reach past the
    traced corners, into the wider index boxes of larger CFL numbers."""
    m = Mesh(Nx=24, Ny=20, Nz=22, Lx=1.0, Ly=1.0, Lz=1.0, CFL=cfl, pressure_scheme=scheme)
    assert m.nband == int(np.ceil(cfl)) and m.nghost == 3 + max(0, int(np.ceil(cfl)) - 2)
    VF0 = cases.vf_spheres(m, np.array([[0.45, 0.5, 0.5], [0.72, 0.3, 0.62]]), np.array([0.24, 0.12]), nF=6)
    VFg, VFo, mass, mo = run(m, VF0, 3, precision)
    if precision == "fp64":
        assert np.array_equal(VFg, VFo)
        assert abs(mass - mo) <= 1e-13 * mo
    else:
        d = np.abs(m.interior(VFg) - m.interior(VFo))
        assert d.max() <= 5e-3
        assert np.quantile(d[d > 0], 0.99) <= 1e-4 if (d > 0).any() else True
        assert abs(mass - mo) <= 2e-8 * mo
