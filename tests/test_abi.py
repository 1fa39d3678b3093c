"""The C-ABI library loads and exports every entry point include/slvof.h declares (CPU only:
no compute calls), and the host-side layout helpers match the reference's extents."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from ns_multiphase_gb300 import build as nb
from ns_multiphase_gb300 import slvof
from ns_multiphase_gb300.mesh import Mesh, MeshDesc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "slvof.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(slvof_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    nb.build()
    return ctypes.CDLL(nb.LIB)


def test_library_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    # the Python binding declares exactly the header's entry points
    assert sorted(n for n, _, _ in slvof.SYMBOLS) == syms


def test_descriptor_layout_matches_header(tmp_path):
    """ctypes' MeshDesc against the C compiler's layout of slvof_mesh (include/slvof.h)."""
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "slvof.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu\\n", sizeof(slvof_mesh), offsetof(slvof_mesh, Lx), '
                   'offsetof(slvof_mesh, x), offsetof(slvof_mesh, zm), offsetof(slvof_mesh, tesselation)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    size, lx, x, zm, tess = (int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                                              check=True).stdout.split())
    assert ctypes.sizeof(MeshDesc) == size
    assert (MeshDesc.Lx.offset, MeshDesc.x.offset, MeshDesc.zm.offset, MeshDesc.tesselation.offset) == (lx, x, zm, tess)


def test_extents_follow_initArrays():
    m = Mesh(Nx=7, Ny=5, Nz=3, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    assert m.nghost == 3
    assert m.cell_shape == (13, 11, 9)
    assert m.vf_shape == (19, 17, 15)
    m2 = Mesh(Nx=7, Ny=5, Nz=3, Lx=1.0, Ly=1.0, Lz=1.0, CFL=3.5)  # nghost = 3 + ceil(3.5) - 2
    assert m2.nghost == 5 and m2.nband == 4
    VF = m.vf_array()
    assert VF.flags.f_contiguous
    assert m.interior(VF).shape == (7, 5, 3)


def test_create_rejects_bad_descriptor_without_gpu(lib):
    # argument validation happens before any CUDA call
    h = ctypes.c_void_p()
    lib.slvof_create.restype = ctypes.c_int
    assert lib.slvof_create(None, 0, ctypes.byref(h)) == -1
    m = Mesh(Nx=4, Ny=4, Nz=4, Lx=1.0, Ly=1.0, Lz=1.0)
    assert lib.slvof_create(ctypes.byref(m.desc()), 7, ctypes.byref(h)) == -1


@pytest.mark.parametrize("field,value,code", [
    ("Nx", 0, -1), ("nghost", 2, -1), ("projection", 4, -1), ("nband", -1, -1), ("tesselation", 7, -1),
    ("pressure_scheme", 2, -1), ("x", None, -1),
    # thresholds are compared as bit patterns: positive finite only
    ("VFlo", 0.0, -3), ("VFlo", -1e-10, -3), ("VFhi", float("nan"), -3), ("VFhi", float("inf"), -3),
])
def test_create_rejects_each_bad_field_without_gpu(lib, field, value, code):
    m = Mesh(Nx=4, Ny=4, Nz=4, Lx=1.0, Ly=1.0, Lz=1.0)
    d = m.desc()
    setattr(d, field, value)
    h = ctypes.c_void_p()
    lib.slvof_create.restype = ctypes.c_int
    for precision in (0, 1):
        assert lib.slvof_create(ctypes.byref(d), precision, ctypes.byref(h)) == code
        assert h.value is None


@pytest.mark.parametrize("precision,tess,code", [(0, 6, -3), (1, 6, -3), (0, 24, -3), (1, 24, -3)])
def test_create_refuses_finite_difference_outside_5_tets(lib, precision, tess, code):
    m = Mesh(Nx=4, Ny=4, Nz=4, Lx=1.0, Ly=1.0, Lz=1.0, tesselation=f"{tess}_tets",
             pressure_scheme="finite-difference")
    h = ctypes.c_void_p()
    lib.slvof_create.restype = ctypes.c_int
    assert lib.slvof_create(ctypes.byref(m.desc()), precision, ctypes.byref(h)) == code


@pytest.mark.parametrize("shape", [(1300, 1300, 1300), (40000, 4, 4), (4, 40000, 4), (4, 4, 40000)])
def test_create_refuses_grids_past_32_bit_cell_indices(lib, shape):
    # cell lists hold 32-bit linear indices of the (N + 2 nghost)^3 cell arrays
    m = Mesh(Nx=shape[0], Ny=shape[1], Nz=shape[2], Lx=1.0, Ly=1.0, Lz=1.0)
    h = ctypes.c_void_p()
    lib.slvof_create.restype = ctypes.c_int
    assert lib.slvof_create(ctypes.byref(m.desc()), 1, ctypes.byref(h)) == -3


def test_python_mirror_constants_match_the_header():
    """The precision, step-flag and status constants of the Python mirror are the header's."""
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "slvof.h")).read()
    defs = {k: int(v) for k, v in re.findall(r"#define SLVOF_(\w+) \(?(-?\d+)\)?", hdr)}
    for name in ("FP64", "MIXED", "STEP_BAND", "STEP_MASS", "STEP_DEFER", "OK", "E_ARG", "E_CUDA",
                 "E_UNSUPPORTED", "E_NOMEM", "E_TOO_LARGE", "DEV_INDEX", "DEV_DEPTH", "DEV_NAN", "DEV_VOLUME",
                 "DEV_WAIT"):
        assert getattr(slvof, name) == defs[name], name
