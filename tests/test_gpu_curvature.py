"""compute_curvature! (src/ELVIRA.jl:141-184) and compute_props! (src/Tools.jl:1186-1210) on
the GPU against the CPU restatement, bit for bit; the resident curvature from the context's own
normals (FP64 context: the same normals as the restatement's)."""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return True


def shapes():
    m3 = Mesh(Nx=16, Ny=16, Nz=16, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, xper=True)
    V3 = cases.vf_spheres(m3, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
    m2 = Mesh(Nx=32, Ny=32, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 32, CFL=0.5, zper=True)
    V2 = cases.vf_spheres(m2, np.array([[0.5, 0.6, 0.0]]), np.array([0.2]), nF=8, dims=2)
    return [(m3, V3), (m2, V2)]


@pytest.mark.parametrize("which", [0, 1])
def test_curvature_bit_identical(built, which):
    import torch
    from ns_multiphase_gb300.slvof import SLVOF
    m, VF0 = shapes()[which]
    o = Oracle(m)
    VF = VF0.copy(order="F")
    _, nx, ny, nz, _ = o.init_state(VF)
    ref = o.curvature(VF, nx, ny, nz)
    assert np.count_nonzero(ref) > 20
    for prec in ("fp64", "mixed"):
        g = SLVOF(m, prec)
        assert np.array_equal(g.computeCurvature(VF, nx, ny, nz), ref), prec
        g.close()
    # resident: the FP64 context's normals of the same VF
    g = SLVOF(m, "fp64")
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    g.prepare()
    d = torch.zeros(tuple(reversed(m.cell_shape)), dtype=torch.float64, device="cuda")
    g.compute_curvature_device(d.data_ptr())
    assert np.array_equal(d.cpu().numpy().T, ref)
    g.close()


def test_props_bit_identical(built):
    from ns_multiphase_gb300.slvof import SLVOF
    m = Mesh(Nx=12, Ny=10, Nz=8, Lx=1.2, Ly=1.0, Lz=0.8, CFL=0.5)
    VF = np.asfortranarray(np.random.default_rng(5).uniform(-0.1, 1.1, m.vf_shape))
    o = Oracle(m)
    g = SLVOF(m, "fp64")
    for mu in ((1e-3, 1.8e-5), (None, None)):
        got = g.computeProps(VF, 1000.0, 1.2, *mu)
        ref = o.props(VF, 1000.0, 1.2, *mu)
        assert len(got) == len(ref)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    g.close()
