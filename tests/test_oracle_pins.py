"""Pins of the CPU restatement (oracle/) before it is trusted as the checker.

* The reference's own fixtures for this path: the PLIC-distance known answers of
  test/test_PLIC_dist.jl:41-51 and the 1000-case computeDist -> computePLIC2VF round trip of
  test/runtests.jl:32-45 (mesh of test/test_PLIC_dist_cutting.jl:1-49: 10x10x1 cells on
  3x1x1, so non-cubic cells), both at the reference's 1e-12 tolerance.  The reference's
  round trip draws unseeded normals; here they are seeded.
* Analytic invariants for the parts the reference's tests leave unpinned: the PLIC->VF clip
  against an exact plane/box volume, ELVIRA's exact reconstruction of planar interfaces,
  and exact transport of a plane by a uniform velocity (pre-image = translated cell).
"""
import math

import numpy as np
import pytest

from ns_multiphase_gb300.mesh import Mesh
from ns_multiphase_gb300 import cases
from oracle.oracle import Oracle

from planevol import box_fraction

TOL = 1e-12  # tests/runtests.jl testValue tolerance


def plic_test_mesh():
    # test/test_PLIC_dist_cutting.jl:3-33
    return Mesh(Nx=10, Ny=10, Nz=1, Lx=3.0, Ly=1.0, Lz=1.0, CFL=0.1)


def test_mesh_matches_create_mesh():
    m = plic_test_mesh()
    assert m.nghost == 3
    assert m.dx == 0.3 - 0.0 and m.dy == 0.1 and m.dz == 1.0
    g = m.nghost
    assert m.x[g] == 0.0 and m.x[g + 10] == 3.0
    assert m.x[g - 1] == -m.dx and m.x[g + 11] == 3.0 + m.dx
    assert np.all(m.xm == 0.5 * (m.x[:-1] + m.x[1:]))


@pytest.mark.parametrize("VF", [1e-9, 0.01, 0.25, 0.5, 0.7, 0.999, 1 - 1e-9] + list(np.random.default_rng(1).random(40)))
def test_plic_dist_known_answers(VF):
    # test/test_PLIC_dist.jl:91-99
    m = plic_test_mesh()
    o = Oracle(m)
    i = j = k = 1
    d = o.computeDist(i, j, k, 1.0, 0.0, 0.0, VF)
    assert abs(d - (m.x[m.nghost] + VF * m.dx)) <= TOL
    d = o.computeDist(i, j, k, 0.0, 1.0, 0.0, VF)
    assert abs(d - (m.y[m.nghost] + VF * m.dy)) <= TOL


def random_cases(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx, ny, nz = rng.random(3) * 2.0 - 1.0  # test/runtests.jl:36
        VF = rng.random()
        norm = math.sqrt(nx * nx + ny * ny + nz * nz)
        out.append((nx / norm, ny / norm, nz / norm, VF))
    return out


@pytest.mark.parametrize("tess", ["5_tets", "6_tets", "24_tets"])
def test_plic_round_trip_1000(tess):
    # test/runtests.jl:32-45 -> test/test_PLIC_dist_cutting.jl:141-149 (the reference runs it
    # with its default tessellation; computeDist does not depend on it, computePLIC2VF does)
    m = Mesh(Nx=10, Ny=10, Nz=1, Lx=3.0, Ly=1.0, Lz=1.0, CFL=0.1, tesselation=tess)
    o = Oracle(m)
    worst = 0.0
    for nx, ny, nz, VF in random_cases(1000, 20261203):
        d = o.computeDist(1, 1, 1, nx, ny, nz, VF)
        v = o.computePLIC2VF(1, 1, 1, nx, ny, nz, d)
        worst = max(worst, abs(v - VF))
    assert worst <= TOL, worst


def test_plic2vf_against_exact_plane_volume():
    """computePLIC2VF (5-tet clip, cut tables) vs an independent exact plane/box volume."""
    m = Mesh(Nx=6, Ny=5, Nz=4, Lx=1.3, Ly=0.7, Lz=0.9)
    o = Oracle(m)
    rng = np.random.default_rng(7)
    g = m.nghost
    worst = 0.0
    for t in range(300):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        i, j, k = (int(rng.integers(0, 8)) for _ in range(3))  # includes ghost and odd cells
        lo = (m.x[i - 1 + g], m.y[j - 1 + g], m.z[k - 1 + g])
        hi = (m.x[i + g], m.y[j + g], m.z[k + g])
        centre = [0.5 * (a + b) for a, b in zip(lo, hi)]
        c = float(np.dot(n, centre) + rng.uniform(-0.6, 0.6) * 0.5)
        v = o.computePLIC2VF(i, j, k, n[0], n[1], n[2], c)
        worst = max(worst, abs(v - box_fraction(n, c, lo, hi)))
    assert worst <= TOL, worst


def test_compute_alpha_branches():
    """All four branches of the Scardovelli-Zaleski inverse against the exact volume."""
    o = Oracle(plic_test_mesh())
    rng = np.random.default_rng(3)
    for _ in range(400):
        mvec = np.abs(rng.normal(size=3))
        mvec /= mvec.sum()
        VF = rng.uniform(0.0, 0.5)
        a = o.computeAlpha(mvec, VF)
        # exact fraction of the unit cube below m.s = a
        f = box_fraction(mvec, a, (0, 0, 0), (1, 1, 1))
        assert abs(f - VF) <= 1e-12


def test_detmath_against_libm():
    from oracle.oracle import lib
    L = lib()
    rng = np.random.default_rng(11)

    def ulps(a, b):
        if a == b:
            return 0
        return abs(a - b) / math.ulp(max(abs(a), abs(b), 1e-300))

    xs = np.concatenate([rng.uniform(0, 8, 3000), 10.0 ** rng.uniform(-12, 3, 3000), [0.0, 1.0, 8.0, 27.0, 1e-300]])
    assert max(ulps(L.orc_detm_cbrt(float(x)), np.cbrt(x)) for x in xs) <= 1
    assert L.orc_detm_cbrt(-8.0) == -2.0
    xs = np.concatenate([rng.uniform(-1, 1, 5000), [-1.0, -0.5, 0.0, 0.5, 1.0, 0.49999999, 0.50000001]])
    assert max(ulps(L.orc_detm_acos(float(x)), math.acos(x)) for x in xs) <= 2
    xs = np.concatenate([rng.uniform(0, math.pi / 3, 5000), rng.uniform(-2.3, 2.3, 2000)])
    assert max(ulps(L.orc_detm_sin(float(x)), math.sin(x)) for x in xs if abs(math.sin(x)) > 1e-3) <= 2
    assert max(ulps(L.orc_detm_cos(float(x)), math.cos(x)) for x in xs if abs(math.cos(x)) > 1e-3) <= 2


def plane_vf(m, n, c):
    """Exact VF of the plane n.x < c on every cell of imino_:imaxo_ (extra layers 0)."""
    VF = m.vf_array()
    g = m.nghost
    nxo, nyo, nzo = m.cell_shape
    for kp in range(nzo):
        for jp in range(nyo):
            for ip in range(nxo):
                lo = (m.x[ip], m.y[jp], m.z[kp])
                hi = (m.x[ip + 1], m.y[jp + 1], m.z[kp + 1])
                VF[ip + 3, jp + 3, kp + 3] = box_fraction(n, c, lo, hi)
    return VF


def test_elvira_reconstructs_planes_exactly():
    """ELVIRA recovers a planar interface whose height columns are resolved in the block."""
    m = Mesh(Nx=8, Ny=8, Nz=8, Lx=1.0, Ly=1.0, Lz=1.0)
    o = Oracle(m)
    n0 = np.array([0.3, -0.2, 1.0])
    n0 /= np.linalg.norm(n0)
    c = float(np.dot(n0, [0.5, 0.5, 0.52]))
    VF = plane_vf(m, n0, c)
    o.vf_ghost_fill(VF)
    nx, ny, nz, flags = o.ELVIRA(VF)
    assert flags == 0
    checked = 0
    for k in range(2, 8):
        for j in range(2, 8):
            for i in range(2, 8):
                v = VF[m.vidx(i, j, k)]
                if not (1e-10 <= v <= 1 - 1e-10):
                    continue
                # all nine 3-cell z-columns must hold the interface (full below, empty above)
                ok = all(VF[m.vidx(i + a, j + b, k - 2)] > 1 - 1e-10 and VF[m.vidx(i + a, j + b, k + 2)] < 1e-10
                         for a in (-1, 0, 1) for b in (-1, 0, 1))
                if not ok:
                    continue
                got = np.array([nx[m.cidx(i, j, k)], ny[m.cidx(i, j, k)], nz[m.cidx(i, j, k)]])
                assert np.max(np.abs(got - n0)) <= 1e-12, (i, j, k, got, n0)
                checked += 1
    assert checked >= 10


@pytest.mark.parametrize("tess", ["5_tets", "6_tets", "24_tets"])
def test_full_cell_volume_of_every_tessellation(tess):
    """The tets of each tessellation tile the cell with positive orientation: a plane that
    leaves the whole cell liquid gives VF = 1, on odd and even cells."""
    m = Mesh(Nx=4, Ny=4, Nz=4, Lx=1.0, Ly=0.7, Lz=1.3, tesselation=tess)
    o = Oracle(m)
    for (i, j, k) in [(1, 1, 1), (2, 1, 1), (3, 4, 2), (4, 4, 4)]:
        v = o.computePLIC2VF(i, j, k, 0.3, -0.5, 0.8, 10.0)
        assert abs(v - 1.0) <= 1e-14, (tess, i, j, k, v)
        assert o.computePLIC2VF(i, j, k, 0.3, -0.5, 0.8, -10.0) == 0.0


@pytest.mark.parametrize("tess", ["5_tets", "6_tets", "24_tets"])
def test_uniform_translation_of_plane_is_exact(tess):
    """A uniform velocity carries a plane exactly: the pre-image is the translated cell, and
    every donor's PLIC plane is the exact plane, so VFnew is the exact shifted fraction."""
    m = Mesh(Nx=10, Ny=10, Nz=10, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess)
    o = Oracle(m)
    n0 = np.array([0.25, 0.1, 1.0])
    n0 /= np.linalg.norm(n0)
    c = float(np.dot(n0, [0.5, 0.5, 0.48]))
    VF = plane_vf(m, n0, c)
    band, nx, ny, nz, D = o.init_state(VF)
    band[...] = 0
    u = (0.31, -0.27, 0.43)
    uf, vf, wf = cases.uniform_faces(m, *u)
    dt = 0.5 * m.dx / 0.43
    VF0 = VF.copy()
    flags, VFnew = o.transport(dt, VF, uf, vf, wf, nx, ny, nz, D, band)
    assert flags == 0
    shift = dt * float(np.dot(n0, u))
    checked = 0
    for k in range(3, 9):
        for j in range(3, 9):
            for i in range(3, 9):
                lo = (m.x[m.cidx(i, j, k)[0]], m.y[m.cidx(i, j, k)[1]], m.z[m.cidx(i, j, k)[2]])
                hi = (m.x[m.cidx(i, j, k)[0] + 1], m.y[m.cidx(i, j, k)[1] + 1], m.z[m.cidx(i, j, k)[2] + 1])
                # donors near the plane must carry the exact normal
                exact = box_fraction(n0, c + shift, lo, hi)
                if 1e-10 < VF0[m.vidx(i, j, k)] < 1 - 1e-10 or 1e-10 < exact < 1 - 1e-10:
                    assert abs(VF[m.vidx(i, j, k)] - exact) <= 1e-12, (i, j, k)
                    checked += 1
    assert checked > 20


@pytest.mark.parametrize("tess", ["5_tets", "6_tets", "24_tets"])
def test_pre_image_volume_uniform_flow(tess):
    m = Mesh(Nx=6, Ny=6, Nz=6, Lx=1.0, Ly=1.0, Lz=1.0, tesselation=tess)
    o = Oracle(m)
    uf, vf, wf = cases.uniform_faces(m, 0.2, -0.1, 0.3)
    VF = m.vf_array()
    VF[...] = 1.0
    nx, ny, nz = m.cell_array(), m.cell_array(), m.cell_array()
    D = m.cell_array()
    D[...] = 3.0
    cv = m.dx * m.dy * m.dz
    for (i, j, k) in [(1, 1, 1), (3, 4, 2), (6, 6, 6), (2, 5, 3)]:
        r, vol, flags = o.sl_cell(0.05, i, j, k, uf, vf, wf, nx, ny, nz, D)
        assert flags == 0
        assert abs(vol - cv) <= 1e-14 * cv * 10
        assert r == 1.0
