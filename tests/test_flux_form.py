"""The flux form of the SL update, checked on the CPU against the restatement's cell form.

The mixed path computes VFnew = (VF |C| + sum of its faces' signed swept liquid) / (|C| + sum
of their signed swept volumes) instead of clipping the whole pre-image of each cell
(src/Transport.jl:111-148); the prism geometry lives in ns_multiphase_gb300/csrc/flux.cuh.
tests/flux_harness.cpp builds that geometry on the host in FP64 with the FP64 cutTet of
adj64.cuh.  In exact arithmetic both forms give the same VFnew, so in FP64 they must agree to
rounding: 1e-12 per cell, for the three tessellations, the RK4/Euler/Midpoint projections and
CFL 0.5 and 2.5, in 3D and in 2D (z periodic).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TOL = 1e-12


@pytest.fixture(scope="module")
def flib():
    src = os.path.join(HERE, "flux_harness.cpp")
    out = os.path.join(HERE, "_build", "libfluxh.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    deps = [src] + [os.path.join(ROOT, "ns_multiphase_gb300", "csrc", f) for f in ("adj64.cuh", "flux.cuh", "mesh_view.h")]
    if not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out) for d in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                        "-I", ROOT, src, "-o", out + ".tmp"], check=True)
        os.replace(out + ".tmp", out)
    L = ctypes.CDLL(out)
    d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.fluxh_sl_cell.restype = d
    L.fluxh_sl_cell.argtypes = [p, d, i, i, i] + [p] * 8 + [p]
    L.fluxh_face_correction.restype = i
    L.fluxh_face_correction.argtypes = [p, d, i, i, i, i, p, p, p, p]
    return L


def ptr(a):
    return a.ctypes.data


def state(tess, projection, cfl, dims, scheme="semi-lagrangian"):
    if dims == 2:
        m = Mesh(Nx=14, Ny=14, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 14, CFL=cfl, zper=True, tesselation=tess,
                 projection=projection, pressure_scheme=scheme)
        VF = cases.vf_spheres(m, np.array([[0.45, 0.55, 0.0]]), np.array([0.27]), nF=8, dims=2)
        uf, vf, wf = cases.deformation2d_faces(m, 0.7, 8.0)
        vmax = 1.0
    else:
        m = Mesh(Nx=10, Ny=10, Nz=10, Lx=1.0, Ly=1.0, Lz=1.0, CFL=cfl, tesselation=tess, projection=projection,
                 pressure_scheme=scheme)
        VF = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
        uf, vf, wf = cases.deformation3d_faces(m, 0.4, 3.0)
        vmax = 2.0
    o = Oracle(m)
    band, nx, ny, nz, D = o.init_state(VF)
    rng = np.random.default_rng(7)
    for f in (uf, vf, wf) if dims == 3 else (uf, vf):
        f += 0.02 * rng.standard_normal(f.shape)
    dt = cfl * m.dx / vmax
    return m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt


CASES = [("5_tets", "RK4", 0.5, 3), ("6_tets", "RK4", 0.5, 3), ("24_tets", "RK4", 0.5, 3),
         ("5_tets", "Euler", 0.5, 3), ("5_tets", "Midpoint", 0.5, 3), ("5_tets", "RK4", 2.5, 3),
         ("5_tets", "RK4", 0.5, 2), ("24_tets", "RK4", 0.5, 2)]


@pytest.mark.parametrize("tess,projection,cfl,dims,scheme",
                         [c + ("semi-lagrangian",) for c in CASES] +
                         [("5_tets", "RK4", 0.5, 3, "finite-difference"), ("5_tets", "RK4", 2.5, 3, "finite-difference"),
                          ("5_tets", "RK4", 0.5, 2, "finite-difference")])
def test_flux_form_equals_cell_form_in_fp64(flib, tess, projection, cfl, dims, scheme):
    """With pressure_scheme "finite-difference" each band cell also adds its faces' correction
    tets (src/Transport.jl:121-124) with its parity sign; a face's tets depend on the face alone
    and its two cells' parities differ, so they join the face's flux like its prism."""
    m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state(tess, projection, cfl, dims, scheme)
    desc = m.desc()
    err = ctypes.c_int()
    worst, n = 0.0, 0
    ks = range(1, m.Nz + 1)
    for k in ks:
        for j in range(1, m.Ny + 1):
            for i in range(1, m.Nx + 1):
                if abs(int(band[m.cidx(i, j, k)])) > m.nband:
                    continue
                r, vol, flags = o.sl_cell(dt, i, j, k, uf, vf, wf, nx, ny, nz, D)
                q = flib.fluxh_sl_cell(ctypes.byref(desc), dt, i, j, k, ptr(VF), ptr(uf), ptr(vf), ptr(wf), ptr(nx),
                                       ptr(ny), ptr(nz), ptr(D), ctypes.addressof(err))
                assert err.value == 0 and flags == 0
                worst = max(worst, abs(q - r))
                n += 1
    assert n > 50
    assert worst <= TOL, worst


def test_face_correction_in_cell_units_matches_the_fp64_reverse(flib):
    """The mixed path's correction apex and volume (flux::face_correction, cell units on the
    traced corners) against the FP64 reverse's own construction (adj::corr_face, physical
    units), face by face over the band of a deforming sphere, both in FP64: the same
    construction in different units, so they agree to rounding."""
    m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state("5_tets", "RK4", 0.5, 3, "finite-difference")
    desc = m.desc()
    out = (ctypes.c_double * 8)()
    worst_e, worst_v, n = 0.0, 0.0, 0
    scale = m.dx * m.dy * m.dz
    for k in range(2, m.Nz + 1):
        for j in range(2, m.Ny + 1):
            for i in range(2, m.Nx + 1):
                if abs(int(band[m.cidx(i, j, k)])) > m.nband:
                    continue
                for d in range(3):
                    assert flib.fluxh_face_correction(ctypes.byref(desc), dt, d, i, j, k, ptr(uf), ptr(vf), ptr(wf),
                                                      out) == 0
                    worst_e = max(worst_e, max(abs(out[q] - out[4 + q]) for q in range(3)) / m.dx)
                    worst_v = max(worst_v, abs(out[3] - out[7]) / scale)
                    n += 1
    assert n > 100
    assert worst_e <= 1e-12 and worst_v <= 1e-13, (worst_e, worst_v)
