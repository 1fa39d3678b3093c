"""The CPU restatement of compute_curvature! (src/ELVIRA.jl:141-184) and compute_props!
(src/Tools.jl:1186-1210), checked by invariants (no reference fixtures): a plane has zero
curvature, a circle 1/R and a sphere 2/R to the height function's accuracy, and the face
properties are the clamped face average's linear blend."""
import ctypes

import numpy as np

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle


def curvature_of(m, VF):
    o = Oracle(m)
    VF = VF.copy(order="F")
    _, nx, ny, nz, _ = o.init_state(VF)
    return o.curvature(VF, nx, ny, nz), VF, (nx, ny, nz)


def test_plane_has_no_curvature():
    """Exact cut-cell fractions of a tilted plane (computePLIC2VF): linear heights."""
    m = Mesh(Nx=16, Ny=16, Nz=16, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    o = Oracle(m)
    n = np.array([0.3, 0.2, 1.0])
    n /= np.linalg.norm(n)
    VF = m.vf_array()
    desc = m.desc()
    g = m.nghost + 3
    for k in range(1, m.Nz + 1):
        for j in range(1, m.Ny + 1):
            for i in range(1, m.Nx + 1):
                VF[g + i - 1, g + j - 1, g + k - 1] = o.L.orc_compute_plic2vf(ctypes.byref(desc), i, j, k, *n, 0.55)
    o.vf_ghost_fill(VF)
    C, VF, _ = curvature_of(m, VF)
    inner = m.interior(C)
    v = m.interior(VF)
    sel = (v > 0.01) & (v < 0.99)
    sel[:3] = sel[-3:] = False
    sel[:, :3] = sel[:, -3:] = False
    sel[:, :, :3] = sel[:, :, -3:] = False
    assert sel.sum() > 20
    assert np.max(np.abs(inner[sel])) <= 1e-9


def test_circle_and_sphere():
    m2 = Mesh(Nx=48, Ny=48, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 48, CFL=0.5, zper=True)
    R2 = 0.3
    VF2 = cases.vf_spheres(m2, np.array([[0.5, 0.5, 0.0]]), np.array([R2]), nF=16, dims=2)
    C2, VF2, _ = curvature_of(m2, VF2)
    m3 = Mesh(Nx=32, Ny=32, Nz=32, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    R3 = 0.3
    VF3 = cases.vf_spheres(m3, np.array([[0.5, 0.5, 0.5]]), np.array([R3]), nF=10)
    C3, VF3, _ = curvature_of(m3, VF3)
    for m, C, VF, expect in ((m2, C2, VF2, 1 / R2), (m3, C3, VF3, 2 / R3)):
        v = m.interior(VF)
        iface = (v > 0.2) & (v < 0.8)
        k = np.abs(m.interior(C)[iface])
        assert iface.sum() > 20
        # the height function's error: a few per cent on resolved cells, more where the
        # 7-cell column leaves the interface (the steep side of the dominant direction)
        assert abs(np.median(k) - expect) <= 0.05 * expect, (np.median(k), expect)


def test_props_blend():
    m = Mesh(Nx=8, Ny=8, Nz=8, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    rng = np.random.default_rng(2)
    VF = np.asfortranarray(rng.uniform(-0.1, 1.1, m.vf_shape))
    o = Oracle(m)
    denx, deny, denz, vx, vy, vz = o.props(VF, 1000.0, 1.2, 1e-3, 1.8e-5)
    g = m.nghost + 3
    lo = 3  # cell arrays start 3 VF layers in
    n = m.cell_shape
    for d, (den, visc) in enumerate(((denx, vx), (deny, vy), (denz, vz))):
        sl = tuple(slice(lo, lo + n[q]) for q in range(3))
        sm = tuple(slice(lo - (q == d), lo - (q == d) + n[q]) for q in range(3))
        f = np.minimum(1.0, np.maximum(0.0, (VF[sl] + VF[sm]) / 2))
        assert np.array_equal(den, 1000.0 * f + 1.2 * (1 - f))
        assert np.array_equal(visc, f * 1e-3 + (1 - f) * 1.8e-5)
    assert len(o.props(VF, 1000.0, 1.2)) == 3
