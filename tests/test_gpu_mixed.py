"""GPU tests of the mixed-precision path (FP32 geometry and candidate errors, FP64 PLIC root,
volume sums and mass) against the FP64 path and against exact planar transport.

Tolerances: a plane carried by a uniform velocity must come out within 2e-6 of the exact
fraction (FP32 geometry in cell units).  ELVIRA's FP32 candidate errors are arbitrated in FP64
wherever two candidates are within rounding of each other, so the chosen normals must equal
the FP64 path's in at least 99.5% of interface cells.  Over short deformation runs every cell
must stay within 5e-3 of the FP64 path, and 99% of the interface cells within 1e-5 except for
the sphere centred at (0.35,0.35,0.35): on a uniform grid its three mirror planes hold exact
FP64 ties between mirror candidates, which the ~1e-7 VF differences of the FP32 transport can
break the other way.  The total volume must agree within a relative bound per case, a few
times the measured difference (2e-10 to 1e-8 over 10 steps on these small grids), and on the
benchmark's own 200-sphere state at 128^3 within the metric's 1e-10 after 64 steps.
"""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()


def make(mesh, VF, precision):
    from ns_multiphase_gb300.slvof import SLVOF
    g = SLVOF(mesh, precision)
    g.upload_vf(VF)
    g.vf_ghost_fill()
    g.init_state()
    return g


def test_mixed_uniform_translation_of_plane():
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from planevol import box_fraction
    from test_oracle_pins import plane_vf
    m = Mesh(Nx=10, Ny=10, Nz=10, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    n0 = np.array([0.25, 0.1, 1.0])
    n0 /= np.linalg.norm(n0)
    c = float(np.dot(n0, [0.5, 0.5, 0.48]))
    VF = plane_vf(m, n0, c)
    g = make(m, VF, "mixed")
    band = m.cell_array(np.int16)
    g.upload_band(band)
    u = (0.31, -0.27, 0.43)
    g.upload_velocity(*cases.uniform_faces(m, *u))
    dt = 0.5 * m.dx / 0.43
    g.transport(dt)
    out = g.download_vf()
    shift = dt * float(np.dot(n0, u))
    worst = 0.0
    for k in range(3, 9):
        for j in range(3, 9):
            for i in range(3, 9):
                ip, jp, kp = m.cidx(i, j, k)
                exact = box_fraction(n0, c + shift, (m.x[ip], m.y[jp], m.z[kp]), (m.x[ip + 1], m.y[jp + 1], m.z[kp + 1]))
                worst = max(worst, abs(out[m.vidx(i, j, k)] - exact))
    assert worst <= 2e-6, worst


def case(shape):
    if shape == "vortex2d":
        m = Mesh(Nx=48, Ny=48, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 48, CFL=0.5, zper=True)
        VF = cases.vf_spheres(m, [[0.5, 0.75, 0.0]], [0.15], nF=10, dims=2)
        vel = lambda t: cases.deformation2d_faces(m, t, 8.0)
        dt = 0.5 * m.dx
    else:
        m = Mesh(Nx=32, Ny=32, Nz=32, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
        if shape == "sphere3d":
            VF = cases.vf_spheres(m, [[0.35, 0.35, 0.35]], [0.15], nF=20)
        else:
            c, r = cases.config_spheres(12, seed=4)
            VF = cases.vf_spheres(m, c, 2.5 * r, nF=8)
        vel = lambda t: cases.deformation3d_faces(m, t, 3.0)
        dt = 0.5 * m.dx / 2.0
    return m, VF, vel, dt


@pytest.mark.parametrize("shape", ["sphere3d", "spheres3d", "vortex2d"])
def test_mixed_normals_match_fp64(shape):
    m, VF, vel, dt = case(shape)
    g64, g32 = make(m, VF, "fp64"), make(m, VF, "mixed")
    a, b = g64.download_normals(), g32.download_normals()
    V = m.interior(g64.download_vf())
    iface = (V >= 1e-10) & (V <= 1 - 1e-10)
    same = np.ones(iface.shape, bool)
    for p, q in zip(a, b):
        same &= m.interior(p) == m.interior(q)
    frac = same[iface].mean()
    assert frac >= 0.995, frac


@pytest.mark.parametrize("shape", ["sphere3d", "spheres3d", "vortex2d"])
def test_mixed_tracks_fp64(shape):
    m, VF, vel, dt = case(shape)
    g64, g32 = make(m, VF, "fp64"), make(m, VF, "mixed")
    t = 0.0
    n_if = 0
    steps = 10
    for s in range(steps):
        uf, vf, wf = vel(t + 0.5 * dt)
        g64.upload_velocity(uf, vf, wf)
        g32.upload_velocity(uf, vf, wf)
        M64 = g64.step(dt)
        M32 = g32.step(dt)
        t += dt
        V = m.interior(g64.download_vf())
        n_if += int(((V >= 1e-10) & (V <= 1 - 1e-10)).sum())
    V64, V32 = m.interior(g64.download_vf()), m.interior(g32.download_vf())
    cv = m.dx * m.dy * m.dz
    d = np.abs(V64 - V32)
    iface = (V64 >= 1e-10) & (V64 <= 1 - 1e-10)
    print(f"{shape}: mass rel diff {abs(M32 - M64) / M64:.3e}, p99 {np.percentile(d[iface], 99):.3e}, "
          f"max {d.max():.3e}")
    # measured 4.5e-10 (one sphere of radius 4.8 cells), 2.8e-11 (twelve spheres), 2.3e-9 (2D,
    # 48^2): small grids hold few interface cells per unit of mass, so their relative drift is
    # larger than the 256^3 benchmark's 1e-11 level
    bound = {"sphere3d": 2e-9, "spheres3d": 2e-10, "vortex2d": 1e-8}[shape]
    assert abs(M32 - M64) <= bound * M64, (M32, M64, abs(M32 - M64) / M64)
    if shape != "sphere3d":
        assert float(np.percentile(d[iface], 99)) <= 1e-5, float(np.percentile(d[iface], 99))
    assert float(d.max()) <= 5e-3, float(d.max())
    assert V32.min() >= -1e-6 and V32.max() <= 1 + 1e-6


@pytest.mark.parametrize("tess", ["6_tets", "24_tets"])
def test_mixed_other_tessellations_track_fp64(tess):
    """6_tets and 24_tets in the mixed path (tets seeded from the tessellation, 24_tets with
    FP32 mean points): a plane carried by a uniform velocity comes out exact to 2e-6, and a
    deforming sphere stays with the FP64 path of the same tessellation."""
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from planevol import box_fraction
    from test_oracle_pins import plane_vf
    m = Mesh(Nx=10, Ny=10, Nz=10, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess)
    n0 = np.array([0.25, 0.1, 1.0])
    n0 /= np.linalg.norm(n0)
    c = float(np.dot(n0, [0.5, 0.5, 0.48]))
    g = make(m, plane_vf(m, n0, c), "mixed")
    g.upload_band(m.cell_array(np.int16))
    u = (0.31, -0.27, 0.43)
    g.upload_velocity(*cases.uniform_faces(m, *u))
    dt = 0.5 * m.dx / 0.43
    g.transport(dt)
    out = g.download_vf()
    shift = dt * float(np.dot(n0, u))
    worst = 0.0
    for k in range(3, 9):
        for j in range(3, 9):
            for i in range(3, 9):
                ci = m.cidx(i, j, k)
                lo = (m.x[ci[0]], m.y[ci[1]], m.z[ci[2]])
                hi = (m.x[ci[0] + 1], m.y[ci[1] + 1], m.z[ci[2] + 1])
                worst = max(worst, abs(out[m.vidx(i, j, k)] - box_fraction(n0, c + shift, lo, hi)))
    assert worst <= 2e-6, worst

    m = Mesh(Nx=20, Ny=20, Nz=20, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess)
    VF = cases.vf_spheres(m, [[0.42, 0.47, 0.4]], [0.21], nF=10)
    g64, g32 = make(m, VF, "fp64"), make(m, VF, "mixed")
    dt = 0.5 * m.dx / 2.0
    for s in range(6):
        uf, vf, wf = cases.deformation3d_faces(m, 0.2 + (s + 0.5) * dt, 3.0)
        g64.upload_velocity(uf, vf, wf)
        g32.upload_velocity(uf, vf, wf)
        M64, M32 = g64.step(dt), g32.step(dt)
    V64, V32 = m.interior(g64.download_vf()), m.interior(g32.download_vf())
    iface = (V64 >= 1e-10) & (V64 <= 1 - 1e-10)
    d = np.abs(V64 - V32)
    assert float(np.percentile(d[iface], 99)) <= 1e-5
    assert float(d.max()) <= 5e-3
    assert abs(M32 - M64) <= 1e-6 * m.dx * m.dy * m.dz * np.sqrt(6 * iface.sum())


def test_mixed_zalesak_rotation_tracks_fp64():
    m = Mesh(Nx=40, Ny=40, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 40, CFL=0.5, zper=True, projection="Zalesak")
    VF = cases.vf_spheres(m, [[0.5, 0.75, 0.0]], [0.15], nF=10, dims=2)
    g64, g32 = make(m, VF, "fp64"), make(m, VF, "mixed")
    zero = m.cell_array()
    for g in (g64, g32):
        g.upload_velocity(zero, zero, zero)
    dt = 0.5 * m.dx / (2 * np.pi * 0.5)
    for s in range(8):
        M64, M32 = g64.step(dt), g32.step(dt)
    V64, V32 = m.interior(g64.download_vf()), m.interior(g32.download_vf())
    iface = (V64 >= 1e-10) & (V64 <= 1 - 1e-10)
    d = np.abs(V64 - V32)
    assert float(np.percentile(d[iface], 99)) <= 1e-5
    assert float(d.max()) <= 5e-3
    assert abs(M32 - M64) <= 1e-6 * m.dx * m.dy * m.dz * np.sqrt(8 * iface.sum())


@pytest.mark.parametrize("scheme", ["semi-lagrangian", "finite-difference"])
def test_mixed_mass_drift_over_64_steps(scheme):
    """The metric's bar on the benchmark's own initial state at 128^3 (200 spheres, seed
    20261203, radii U[0.02, 0.08], the time-varying Deformation3D field with T = 3, CFL 0.5):
    after 64 steps the mixed path's total volume is within 1e-10 (relative) of the FP64 path's,
    in each of two runs (the mixed path's work lists are filled by atomics, so its last bits
    may differ between runs); 99% of the interface cells within 1e-6 of the FP64 path's VF and
    every cell within 5e-3.  Both pressure schemes: "finite-difference" adds the flux-correction
    tets to every band cell (measured 2.2e-11 after 64 steps; 1.4e-11 without them)."""
    from ns_multiphase_gb300.slvof import SLVOF
    n, steps = 128, 64
    m = Mesh(Nx=n, Ny=n, Nz=n, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, pressure_scheme=scheme)
    centres, radii = cases.config_spheres(200, 20261203)
    dt = 0.5 * m.dx / 2.0
    ctx = {}
    for name, precision in (("fp64", "fp64"), ("mixed_a", "mixed"), ("mixed_b", "mixed")):
        g = SLVOF(m, precision)
        g.case_vf_spheres(centres, radii, nF=20, dims=3)
        g.init_state()
        ctx[name] = g
    M = {}
    for s in range(steps):
        for name, g in ctx.items():
            g.case_deformation3d((s + 0.5) * dt, 3.0)
            M[name] = g.step(dt)
    V64 = m.interior(ctx["fp64"].download_vf())
    iface = (V64 >= m.VFlo) & (V64 <= m.VFhi)
    rel = {}
    for name in ("mixed_a", "mixed_b"):
        V32 = m.interior(ctx[name].download_vf())
        d = np.abs(V64 - V32)
        rel[name] = abs(M[name] - M["fp64"]) / M["fp64"]
        print(f"{name}: mass rel diff {rel[name]:.3e}, p99 {np.percentile(d[iface], 99):.3e}, max {d.max():.3e}")
        assert rel[name] <= 1e-10, rel
        assert float(np.percentile(d[iface], 99)) <= 1e-6
        assert float(d.max()) <= 5e-3
    for g in ctx.values():
        g.close()
