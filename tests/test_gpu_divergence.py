"""divg_cell / divergence! (src/Velocity.jl:59-122) and A! (src/Pressure.jl:83-115) on the GPU
against the CPU restatement, bit for bit: both schemes, the three tessellations, periodic and
bounded domains, 2D, and the device-pointer entry points against the host ones."""
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


def setup(tess="5_tets", per=False, two_d=False, projection="RK4", seed=3):
    if two_d:
        m = Mesh(Nx=24, Ny=24, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 24, CFL=0.5, zper=True, tesselation=tess,
                 projection=projection)
        VF = cases.vf_spheres(m, np.array([[0.5, 0.6, 0.0]]), np.array([0.2]), nF=8, dims=2)
        uf, vf, wf = cases.deformation2d_faces(m, 0.4, 8.0)
    else:
        m = Mesh(Nx=12, Ny=12, Nz=12, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess, xper=per, yper=per,
                 zper=per, projection=projection)
        VF = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
        uf, vf, wf = cases.deformation3d_faces(m, 0.3, 3.0)
    rng = np.random.default_rng(seed)
    for f in (uf, vf, wf) if not two_d else (uf, vf):
        f += 0.05 * rng.standard_normal(f.shape)
    o = Oracle(m)
    band = o.init_state(VF)[0]
    dt = 0.5 * m.dx / 2.0
    return m, o, band, uf, vf, wf, dt


CASES = [("5_tets", False, False), ("6_tets", False, False), ("24_tets", False, False), ("5_tets", True, False),
         ("5_tets", False, True)]


@pytest.mark.parametrize("tess,per,two_d", CASES)
@pytest.mark.parametrize("scheme", ["semi-lagrangian", "finite-difference"])
def test_divergence_bit_identical(built, tess, per, two_d, scheme):
    from ns_multiphase_gb300.slvof import SLVOF
    m, o, band, uf, vf, wf, dt = setup(tess, per, two_d)
    g = SLVOF(m, "fp64")
    got = g.divergence(dt, uf, vf, wf, band, scheme)
    g.close()
    ref = o.divergence(dt, uf, vf, wf, band, SLVOF.SCHEME[scheme])
    assert np.array_equal(got, ref)
    assert np.count_nonzero(np.abs(m.interior(band)) <= m.nband) > 20


@pytest.mark.parametrize("tess,per,two_d", CASES)
def test_A_bit_identical(built, tess, per, two_d):
    from ns_multiphase_gb300.slvof import SLVOF
    m, o, band, uf, vf, wf, dt = setup(tess, per, two_d)
    rng = np.random.default_rng(11)
    P = np.asfortranarray(rng.standard_normal(m.cell_shape))
    den = [np.asfortranarray(1.0 + rng.uniform(0.0, 999.0, m.cell_shape)) for _ in range(3)]
    for scheme in ("semi-lagrangian", "finite-difference"):
        g = SLVOF(m, "mixed")  # the operators run in FP64 in either precision
        Pg = P.copy(order="F")
        got = g.A(dt, Pg, uf, vf, wf, *den, band, scheme)
        g.close()
        Po = P.copy(order="F")
        ref = o.A(dt, Po, uf, vf, wf, *den, band, SLVOF.SCHEME[scheme])[0]
        assert np.array_equal(got, ref), scheme
        assert np.array_equal(Pg, Po), scheme


def test_zalesak_rotation_divergence(built):
    """The Zalesak rotation is rigid: the projected cells keep their volume."""
    from ns_multiphase_gb300.slvof import SLVOF
    m, o, band, uf, vf, wf, dt = setup(two_d=True, projection="Zalesak")
    g = SLVOF(m, "fp64")
    got = g.divergence(dt, uf, vf, wf, band)
    g.close()
    assert np.array_equal(got, o.divergence(dt, uf, vf, wf, band, 0))
    inband = np.abs(m.interior(band)) <= m.nband
    assert np.max(np.abs(m.interior(got)[inband])) <= 1e-9


def test_device_entry_points(built):
    import torch
    from ns_multiphase_gb300.slvof import SLVOF
    m, o, band, uf, vf, wf, dt = setup()
    rng = np.random.default_rng(4)
    P = np.asfortranarray(rng.standard_normal(m.cell_shape))
    den = [np.asfortranarray(1.0 + rng.uniform(0.0, 9.0, m.cell_shape)) for _ in range(3)]
    g = SLVOF(m, "fp64")
    host_div = g.divergence(dt, uf, vf, wf, band)
    Ph = P.copy(order="F")
    host_A = g.A(dt, Ph, uf, vf, wf, *den, band)

    def dev(a):  # a Fortran-ordered host array as a device buffer with the same memory layout
        return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    d_u, d_v, d_w, d_P = dev(uf), dev(vf), dev(wf), dev(P)
    d_den = [dev(x) for x in den]
    d_band = dev(band)
    d_out = torch.zeros_like(d_u)
    g.divergence_device(dt, d_out.data_ptr(), d_u.data_ptr(), d_v.data_ptr(), d_w.data_ptr(), d_band.data_ptr())
    assert np.array_equal(d_out.cpu().numpy().T, host_div)
    g.A_device(dt, d_out.data_ptr(), d_P.data_ptr(), d_u.data_ptr(), d_v.data_ptr(), d_w.data_ptr(),
               *[x.data_ptr() for x in d_den], d_band.data_ptr())
    assert np.array_equal(d_out.cpu().numpy().T, host_A)
    assert np.array_equal(d_P.cpu().numpy().T, Ph)
    g.close()
