"""slvof_step_host, the per-step drop-in with host buffers: each call uploads the face
velocities, steps, and returns the new VF and mass.  VF goes to the host on a second stream
while the new state's normals, PLIC, band and mass are built, so the test checks that the
returned array is the device state after the call, and that the call gives what the
device-resident path gives on the same inputs (FP64: bit for bit, and against the CPU
restatement; mixed: within its tolerance)."""
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


def _state(m, precision):
    from ns_multiphase_gb300.slvof import SLVOF
    VF0 = cases.vf_spheres(m, np.array([[0.35, 0.4, 0.45], [0.7, 0.6, 0.55]]), np.array([0.17, 0.12]), nF=6)
    g = SLVOF(m, precision)
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    g.init_state()
    return g, VF0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_host_returns_the_state_the_device_path_reaches(precision):
    m = Mesh(Nx=40, Ny=36, Nz=32, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    dt = 0.5 * m.dx / 2.0
    g, VF0 = _state(m, precision)
    r, _ = _state(m, precision)
    o = Oracle(m) if precision == "fp64" else None
    if o is not None:
        VFo = VF0.copy(order="F")
        band, nx, ny, nz, D = o.init_state(VFo)
    VFh = m.vf_array()
    for n in range(5):
        uf, vf, wf = cases.deformation3d_faces(m, (n + 0.5) * dt, 3.0)
        VFh[...] = np.nan
        mass_h = g.step_host(dt, uf, vf, wf, VFh)
        # the copy overlapped the geometry stages: it must hold the final state of the call
        assert np.array_equal(VFh, g.download_vf())
        r.upload_velocity(uf, vf, wf)
        mass_r = r.step(dt)
        VFr = r.download_vf()
        if precision == "fp64":
            assert np.array_equal(VFh, VFr)
            assert mass_h == mass_r
            assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
            assert np.array_equal(m.interior(VFh), m.interior(VFo))
        else:
            # batches of the clip differ between runs, so the last bits of VF may differ
            assert np.max(np.abs(m.interior(VFh) - m.interior(VFr))) < 1e-5
            assert abs(mass_h - mass_r) <= 1e-12 * abs(mass_r)
    g.close()
    r.close()


def test_step_host_refuses_null_outputs_before_any_work():
    import ctypes
    from ns_multiphase_gb300.slvof import SLVOF
    m = Mesh(Nx=8, Ny=8, Nz=8, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    g, _ = _state(m, "fp64")
    before = g.download_vf()
    uf = np.zeros(m.cell_shape, order="F")
    L = g.L
    P = ctypes.c_void_p
    mass = ctypes.c_double()
    up = uf.ctypes.data_as(P)
    # VF null
    assert L.slvof_step_host(g.h, ctypes.c_double(1e-3), 3, up, up, up, None, ctypes.byref(mass)) == -1
    # mass requested, null
    VFh = m.vf_array()
    assert L.slvof_step_host(g.h, ctypes.c_double(1e-3), 2, up, up, up, VFh.ctypes.data_as(P), None) == -1
    assert np.array_equal(g.download_vf(), before)
    g.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_deferred_state_gives_the_same_steps(precision):
    """SLVOF_STEP_DEFER builds each state's normals, PLIC and band at the start of the next call,
    beside its upload: the same VF and mass every step as without the flag (FP64: bit for bit),
    and every other entry point sees the complete state (here the downloads and a device-resident
    step after deferring calls, and a step without the flag between deferring ones)."""
    m = Mesh(Nx=40, Ny=36, Nz=32, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    dt = 0.5 * m.dx / 2.0
    g, _ = _state(m, precision)
    r, _ = _state(m, precision)
    VFh, VFr = m.vf_array(), m.vf_array()
    for n in range(6):
        uf, vf, wf = cases.deformation3d_faces(m, (n + 0.5) * dt, 3.0)
        mass_h = g.step_host(dt, uf, vf, wf, VFh, defer=(n != 3))
        mass_r = r.step_host(dt, uf, vf, wf, VFr)
        if precision == "fp64":
            assert np.array_equal(VFh, VFr) and mass_h == mass_r
        else:
            assert np.max(np.abs(m.interior(VFh) - m.interior(VFr))) < 1e-5
            assert abs(mass_h - mass_r) <= 1e-12 * abs(mass_r)
    # the last call deferred: the downloads build its state first
    for a, b in zip(g.download_normals(), r.download_normals()):
        if precision == "fp64":
            assert np.array_equal(a, b)
        else:
            # VF differs in its last bits between runs, which can move an ELVIRA near-tie
            assert np.isfinite(a).all() and np.mean(np.abs(a - b) > 1e-6) < 1e-3
    if precision == "fp64":
        assert np.array_equal(g.download_plic(), r.download_plic())
        assert np.array_equal(g.download_band(), r.download_band())
    # a deferring call, then the device-resident step
    uf, vf, wf = cases.deformation3d_faces(m, 6.5 * dt, 3.0)
    g.step_host(dt, uf, vf, wf, VFh, defer=True)
    r.step_host(dt, uf, vf, wf, VFr)
    uf, vf, wf = cases.deformation3d_faces(m, 7.5 * dt, 3.0)
    for x in (g, r):
        x.upload_velocity(uf, vf, wf)
    mg, mr = g.step(dt), r.step(dt)
    if precision == "fp64":
        assert np.array_equal(g.download_vf(), r.download_vf()) and mg == mr
        assert np.array_equal(g.download_band(), r.download_band())
    else:
        assert np.max(np.abs(m.interior(g.download_vf()) - m.interior(r.download_vf()))) < 1e-5
    g.close()
    r.close()
