"""slvof_mass_noalloc: the mass sum for callers that cannot allocate device memory.

Such a caller (a framework that owns every device allocation, or code running after the
solver reserved all device memory) hands in a VF array already on the device and a device
double for the result; the entry point keeps its scratch in a fixed static device array of
the library.  Its result must match the context-based slvof_mass within the 1e-13 relative
tolerance the other mass checks use, on two calls in a row (the second call reuses the same
scratch array with different data): once with CFL 0.5 (three ghost layers) on torch's current
stream, once with CFL 2.5 (four ghost layers, so other VF strides and offsets) on a stream of
the test's own, where the device's free memory must also stay the same across the calls.  The
first call in a process loads the library's device code and its static scratch array, which
the driver places in device memory; the free-memory check therefore starts after one call.
The device buffers here are the test's own, made with torch; the entry point itself allocates
nothing.  Kept in a file that pytest collects last.
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


def noalloc(lib, desc, d_VF, d_mass, stream_handle):
    return lib.slvof_mass_noalloc(ctypes.byref(desc), ctypes.c_void_p(d_VF.data_ptr()),
                                  ctypes.c_void_p(d_mass.data_ptr()), ctypes.c_void_p(stream_handle))


def two_calls(lib, torch, m, dt, stream, check_memory):
    from ns_multiphase_gb300.slvof import SLVOF
    c, r = cases.config_spheres(8, seed=3)
    g = SLVOF(m, "fp64")
    g.case_vf_spheres(c, 2.0 * r, nF=8)
    g.init_state()
    desc = m.desc()
    with torch.cuda.stream(stream):
        d_mass = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        if call == 1:  # new data for the second call: one transport step
            g.upload_velocity(*cases.deformation3d_faces(m, 0.5 * dt, 3.0))
            g.step(dt)
        VF = g.download_vf()
        expected = g.mass()
        with torch.cuda.stream(stream):
            d_VF = device_copy(torch, VF)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        assert noalloc(lib, desc, d_VF, d_mass, stream.cuda_stream) == 0
        stream.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        got = float(d_mass.item())
        assert abs(got - expected) <= TOL * abs(expected), (call, got, expected)
        if check_memory and call == 1:
            assert free1 == free0, (free0, free1)
    g.close()


def test_mass_noalloc_matches_context_mass_on_two_calls(lib):
    import torch
    m = Mesh(Nx=28, Ny=24, Nz=20, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    two_calls(lib, torch, m, 0.5 * m.dx / 2.0, torch.cuda.current_stream(), False)


def test_mass_noalloc_four_ghost_layers_on_own_stream_allocates_nothing(lib):
    import torch
    m = Mesh(Nx=20, Ny=26, Nz=18, Lx=1.0, Ly=1.0, Lz=1.0, CFL=2.5)
    assert m.nghost == 4
    two_calls(lib, torch, m, 2.5 * m.dx / 2.0, torch.cuda.Stream(), True)


def test_mass_noalloc_rejects_grids_beyond_its_scratch(lib):
    import torch
    from ns_multiphase_gb300 import slvof
    m = Mesh(Nx=2, Ny=2, Nz=8193, Lx=1.0, Ly=1.0, Lz=1.0)
    d = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = lib.slvof_mass_noalloc(ctypes.byref(m.desc()), ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                None)
    assert st == slvof.E_TOO_LARGE  # before any device work
