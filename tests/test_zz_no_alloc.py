"""slvof_mass_noalloc: the mass sum for callers that cannot allocate device memory.

Such a caller (a framework that owns every device allocation, or code running after the
solver reserved all device memory) hands in a VF array already on the device and a device
double for the result; the entry point keeps its scratch in a fixed static device array of
the library.  Its result must match the context-based slvof_mass within the 1e-13 relative
tolerance the other mass checks use, on two calls in a row (the second call reuses the same
scratch array with different data).  The device buffers here are the test's own, made with
torch; the entry point itself allocates nothing.  Kept in a file that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    from ns_multiphase_gb300.slvof import load_library
    return load_library()


def device_copy(torch, a):
    """The VF parent as a flat device buffer in its Fortran (column-major) order."""
    return torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()


def test_mass_noalloc_matches_context_mass_on_two_calls(lib):
    import torch
    from ns_multiphase_gb300.slvof import SLVOF
    m = Mesh(Nx=28, Ny=24, Nz=20, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    c, r = cases.config_spheres(8, seed=3)
    g = SLVOF(m, "fp64")
    g.case_vf_spheres(c, 2.0 * r, nF=8)
    g.init_state()
    d_mass = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    desc = m.desc()
    dt = 0.5 * m.dx / 2.0
    for call in range(2):
        if call == 1:  # new data for the second call: one transport step
            g.upload_velocity(*cases.deformation3d_faces(m, 0.5 * dt, 3.0))
            g.step(dt)
        VF = g.download_vf()
        expected = g.mass()
        d_VF = device_copy(torch, VF)
        st = lib.slvof_mass_noalloc(ctypes.byref(desc), ctypes.c_void_p(d_VF.data_ptr()),
                                    ctypes.c_void_p(d_mass.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == 0
        torch.cuda.synchronize()
        got = float(d_mass.item())
        assert abs(got - expected) <= TOL * abs(expected), (call, got, expected)
    g.close()


def test_mass_noalloc_rejects_grids_beyond_its_scratch(lib):
    import torch
    m = Mesh(Nx=2, Ny=2, Nz=8193, Lx=1.0, Ly=1.0, Lz=1.0)
    d = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = lib.slvof_mass_noalloc(ctypes.byref(m.desc()), ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                None)
    assert st == -5  # SLVOF_E_TOO_LARGE, before any device work
