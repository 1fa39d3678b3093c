"""GPU parity: the FP64 CUDA path against the CPU restatement, bit for bit.

Every call goes through the C ABI (ns_multiphase_gb300.slvof -> libslvof.so).  The FP64
kernels keep the reference's expression order without FMA and share the deterministic
elementary functions with the restatement, so normals, PLIC distances, band and VF are
compared with array_equal; the total volume is compared at 1e-13 relative.
"""
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


def ctx(mesh, precision="fp64"):
    from ns_multiphase_gb300.slvof import SLVOF
    return SLVOF(mesh, precision)


def assert_same(a, b, what):
    if not np.array_equal(a, b):
        d = np.abs(a.astype(np.float64) - b.astype(np.float64))
        idx = np.unravel_index(np.argmax(d), d.shape)
        raise AssertionError(f"{what}: {int((d > 0).sum())} cells differ, max {d.max():.3e} at parent {idx}")


def spheres_mesh(N=16, seed=5, n=4):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.25, 0.75, size=(n, 3))
    r = rng.uniform(0.12, 0.22, size=n)
    return m, cases.vf_spheres(m, c, r, nF=8)


def init_both(m, VF, precision="fp64"):
    o = Oracle(m)
    VFo = VF.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VFo)
    g = ctx(m, precision)
    g.upload_vf(VF)
    g.vf_ghost_fill()
    g.init_state()
    return o, g, VFo, band, nx, ny, nz, D


def test_vf_ghost_fill_normals_plic_band():
    m, VF = spheres_mesh()
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    assert_same(g.download_vf(), VFo, "VF ghost fill")
    gx, gy, gz = g.download_normals()
    assert_same(gx, nx, "nx")
    assert_same(gy, ny, "ny")
    assert_same(gz, nz, "nz")
    assert_same(g.download_plic(), D, "D")
    assert_same(g.download_band(), band, "band")


def test_one_transport_step():
    m, VF = spheres_mesh(N=20, seed=9)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    dt = 0.5 * m.dx / 2.0
    uf, vf, wf = cases.deformation3d_faces(m, 0.3, 3.0)
    g.upload_velocity(uf, vf, wf)
    g.transport(dt)
    flags, _ = o.transport(dt, VFo, uf, vf, wf, nx, ny, nz, D, band)
    assert flags == 0
    assert_same(g.download_vf(), VFo, "VF after SL update")


@pytest.mark.parametrize("projection", ["RK4", "Euler", "Midpoint"])
def test_multistep_sphere_deformation(projection):
    """Config-1 shape (sphere r=0.15 at 0.35^3, Deformation3D T=3) at 24^3, 6 steps."""
    m = Mesh(Nx=24, Ny=24, Nz=24, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, projection=projection)
    VF = cases.vf_spheres(m, [[0.35, 0.35, 0.35]], [0.15], nF=20)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    dt = 0.5 * m.dx / 2.0
    t = 0.0
    for s in range(6):
        uf, vf, wf = cases.deformation3d_faces(m, t + 0.5 * dt, 3.0)
        g.upload_velocity(uf, vf, wf)
        mass = g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
        t += dt
    assert_same(g.download_vf(), VFo, "VF")
    gx, gy, gz = g.download_normals()
    assert_same(gx, nx, "nx")
    assert_same(gy, ny, "ny")
    assert_same(gz, nz, "nz")
    assert_same(g.download_plic(), D, "D")
    assert_same(g.download_band(), band, "band")
    mo = o.mass(VFo)
    assert abs(mass - mo) <= 1e-13 * abs(mo)


def test_multistep_2d_vortex_periodic_z():
    """Config-0 shape: 2D single vortex (T=8), circle r=0.15 at (0.5,0.75), z periodic."""
    m = Mesh(Nx=32, Ny=32, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 32, CFL=0.5, zper=True)
    VF = cases.vf_spheres(m, [[0.5, 0.75, 0.0]], [0.15], nF=10, dims=2)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    dt = 0.5 * m.dx
    t = 0.0
    for s in range(12):
        uf, vf, wf = cases.deformation2d_faces(m, t + 0.5 * dt, 8.0)
        g.upload_velocity(uf, vf, wf)
        g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
        t += dt
    assert_same(g.download_vf(), VFo, "VF")
    gx, gy, gz = g.download_normals()
    assert_same(gx, nx, "nx")
    assert_same(gy, ny, "ny")
    assert_same(g.download_plic(), D, "D")
    assert_same(g.download_band(), band, "band")


def test_all_cells_semi_lagrangian_like_the_test_scripts():
    """test/test_deformation.jl:144 forces band = 0 so every cell takes the SL update."""
    m, VF = spheres_mesh(N=14, seed=2, n=3)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    band[...] = 0
    g.upload_band(band)
    dt = 0.5 * m.dx / 2.0
    uf, vf, wf = cases.deformation3d_faces(m, 0.7, 3.0)
    g.upload_velocity(uf, vf, wf)
    g.transport(dt)
    o.transport(dt, VFo, uf, vf, wf, nx, ny, nz, D, band)
    assert_same(g.download_vf(), VFo, "VF, every cell SL")


def test_host_dropins_match_the_restatement():
    m, VF = spheres_mesh(N=12, seed=3, n=3)
    o = Oracle(m)
    o.vf_ghost_fill(VF)
    g = ctx(m)
    nx, ny, nz = m.cell_array(), m.cell_array(), m.cell_array()
    g.computeNormal(nx, ny, nz, VF)
    ox, oy, oz, _ = o.ELVIRA(VF)
    assert_same(nx, ox, "computeNormal nx")
    assert_same(nz, oz, "computeNormal nz")
    D = m.cell_array()
    g.computePLIC(D, nx, ny, nz, VF)
    assert_same(D, o.computePLIC(ox, oy, oz, VF), "computePLIC")
    band = m.cell_array(np.int16)
    g.computeBand(band, VF)
    assert_same(band, o.computeBand(VF), "computeBand")
    dt = 0.01
    uf, vf, wf = cases.deformation3d_faces(m, 0.2, 3.0)
    VFg = VF.copy(order="F")
    g.transportSL(dt, VFg, uf, vf, wf, nx, ny, nz, D, band)
    VFo = VF.copy(order="F")
    o.transport(dt, VFo, uf, vf, wf, ox, oy, oz, D, band)
    assert_same(VFg, VFo, "transportSL")


def test_case_generator_matches_numpy():
    m = Mesh(Nx=20, Ny=18, Nz=16, Lx=1.0, Ly=1.0, Lz=1.0)
    c, r = cases.config_spheres(12, seed=11)
    ref = cases.vf_spheres(m, c, r, nF=6)
    Oracle(m).vf_ghost_fill(ref)
    g = ctx(m)
    g.case_vf_spheres(c, r, nF=6)
    assert_same(g.download_vf(), ref, "VF spheres")


@pytest.mark.parametrize("tess", ["6_tets", "24_tets"])
def test_multistep_other_tessellations(tess):
    """6_tets and 24_tets (src/VFgeom.jl:257-330): ELVIRA's PLIC2VF and the SL clip over the
    tessellation's tets (24_tets with the mean points of the projected vertices), bit for bit
    against the restatement; 3D sphere deformation, 4 steps."""
    m = Mesh(Nx=20, Ny=20, Nz=20, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess)
    VF = cases.vf_spheres(m, [[0.4, 0.45, 0.4]], [0.2], nF=10)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    gx, gy, gz = g.download_normals()
    assert_same(gx, nx, "nx at start")
    dt = 0.5 * m.dx / 2.0
    t = 0.0
    for s in range(4):
        uf, vf, wf = cases.deformation3d_faces(m, t + 0.5 * dt, 3.0)
        g.upload_velocity(uf, vf, wf)
        mass = g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
        t += dt
    assert_same(g.download_vf(), VFo, "VF")
    gx, gy, gz = g.download_normals()
    assert_same(gx, nx, "nx")
    assert_same(gy, ny, "ny")
    assert_same(gz, nz, "nz")
    assert_same(g.download_plic(), D, "D")
    mo = o.mass(VFo)
    assert abs(mass - mo) <= 1e-13 * abs(mo)


@pytest.mark.parametrize("tess", ["6_tets", "24_tets"])
def test_2d_vortex_other_tessellations(tess):
    m = Mesh(Nx=24, Ny=24, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 24, CFL=0.5, zper=True, tesselation=tess)
    VF = cases.vf_spheres(m, [[0.5, 0.7, 0.0]], [0.18], nF=10, dims=2)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    dt = 0.5 * m.dx
    for s in range(6):
        uf, vf, wf = cases.deformation2d_faces(m, (s + 0.5) * dt, 8.0)
        g.upload_velocity(uf, vf, wf)
        g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
    assert_same(g.download_vf(), VFo, "VF")


def test_zalesak_rotation_projection():
    """test_case "Zalesak" (src/Tools.jl:396-399): the pre-image is the exact rotation about
    (0.5, 0.5), no velocity interpolation; FP64 path bit for bit against the restatement."""
    m = Mesh(Nx=40, Ny=40, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 40, CFL=0.5, zper=True, projection="Zalesak")
    VF = cases.vf_spheres(m, [[0.5, 0.75, 0.0]], [0.15], nF=10, dims=2)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    dt = 0.5 * m.dx / (2 * np.pi * 0.5)
    zero = m.cell_array()
    g.upload_velocity(zero, zero, zero)
    for s in range(8):
        g.step(dt)
        assert o.step(dt, VFo, zero, zero, zero, nx, ny, nz, D, band) == 0
    assert_same(g.download_vf(), VFo, "VF")
    gx, gy, gz = g.download_normals()
    assert_same(gx, nx, "nx")
    assert_same(g.download_plic(), D, "D")


def momentum_state(tess):
    m = Mesh(Nx=18, Ny=16, Nz=14, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess, rho_liq=1000.0, rho_gas=1.2)
    VF = cases.vf_spheres(m, [[0.45, 0.5, 0.48]], [0.23], nF=8)
    o = Oracle(m)
    VFo = VF.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VFo)
    uf, vf, wf = cases.deformation3d_faces(m, 0.25, 3.0)
    # cell-centred velocities: face averages plus a smooth perturbation
    u = np.asfortranarray(0.5 * (uf + np.roll(uf, -1, axis=0)) + 0.1 * np.sin(3 * m.xm)[:, None, None])
    v = np.asfortranarray(0.5 * (vf + np.roll(vf, -1, axis=1)) - 0.07 * np.cos(2 * m.ym)[None, :, None])
    w = np.asfortranarray(0.5 * (wf + np.roll(wf, -1, axis=2)) + 0.05)
    dt = 0.5 * m.dx / 2.0
    return m, o, VFo, band, nx, ny, nz, D, uf, vf, wf, u, v, w, dt


@pytest.mark.parametrize("tess", ["5_tets", "24_tets"])
def test_transport_momentum_matches_restatement(tess):
    """transport!'s momentum (src/Transport.jl:34-166): us, vs, ws of every interior cell, band
    cells from the clip with rho_liq/rho_gas, the others from FD fluxes and SL flux volumes at
    the band edges; bit for bit against the restatement, host drop-in and resident call."""
    m, o, VFo, band, nx, ny, nz, D, uf, vf, wf, u, v, w, dt = momentum_state(tess)
    g = ctx(m)
    VFg = VFo.copy(order="F")
    us, vs, ws = g.transportSL_momentum(dt, VFg, uf, vf, wf, nx, ny, nz, D, band, u, v, w)
    flags, uso, vso, wso = o.transport_mom(dt, VFo, uf, vf, wf, nx, ny, nz, D, band, u, v, w)
    assert flags == 0
    assert_same(VFg, VFo, "VF")
    for a, b, name in ((us, uso, "us"), (vs, vso, "vs"), (ws, wso, "ws")):
        assert_same(m.interior(a), m.interior(b), name)
    inner = np.abs(m.interior(band).astype(int))
    assert (inner <= m.nband).any() and (inner > m.nband).any()
    # resident: state, velocities and the momentum call
    m2, o2, VF2, band2, nx2, ny2, nz2, D2, uf2, vf2, wf2, u2, v2, w2, dt2 = momentum_state(tess)
    g2 = ctx(m2)
    g2.upload_vf(VF2)
    g2.vf_ghost_fill()
    g2.init_state()
    g2.upload_velocity(uf2, vf2, wf2)
    g2.upload_cell_velocity(u2, v2, w2)
    g2.transport_momentum(dt2)
    r = g2.download_momentum()
    for a, b, name in zip(r, (uso, vso, wso), ("us", "vs", "ws")):
        assert_same(m2.interior(a), m2.interior(b), "resident " + name)


def test_host_transport_refreshes_phase_codes_of_uploaded_planes():
    """A drop-in call on a context that last held another state: the pure-donor codes come
    from the uploaded planes, not from the previous state."""
    m, VF = spheres_mesh(N=16, seed=3)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    m2, VFb = spheres_mesh(N=16, seed=11)
    o2 = Oracle(m2)
    VFb = VFb.copy(order="F")
    band_b, nxb, nyb, nzb, Db = o2.init_state(VFb)
    uf, vf, wf = cases.deformation3d_faces(m2, 0.4, 3.0)
    dt = 0.5 * m2.dx / 2.0
    VFg = VFb.copy(order="F")
    g.transportSL(dt, VFg, uf, vf, wf, nxb, nyb, nzb, Db, band_b)
    flags, _ = o2.transport(dt, VFb, uf, vf, wf, nxb, nyb, nzb, Db, band_b)
    assert flags == 0
    assert_same(VFg, VFb, "VF")


def test_finite_difference_scheme_correction_tets():
    """pressure_scheme "finite-difference": band cells add the flux-correction tets
    (add_correction_tets, src/VFgeom.jl:514-664) and band-edge momentum fluxes are finite
    differences; VF over several steps and the momentum, bit for bit against the restatement."""
    m = Mesh(Nx=20, Ny=20, Nz=20, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, pressure_scheme="finite-difference")
    VF = cases.vf_spheres(m, [[0.45, 0.52, 0.5]], [0.22], nF=10)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF)
    dt = 0.5 * m.dx / 2.0
    rng = np.random.default_rng(8)
    noise = [0.05 * rng.standard_normal(m.cell_shape) for _ in range(3)]
    for s in range(4):
        uf, vf, wf = (a + e for a, e in zip(cases.deformation3d_faces(m, 0.2 + (s + 0.5) * dt, 3.0), noise))
        uf, vf, wf = (np.asfortranarray(x) for x in (uf, vf, wf))
        g.upload_velocity(uf, vf, wf)
        mass = g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
    assert_same(g.download_vf(), VFo, "VF")
    mo = o.mass(VFo)
    assert abs(mass - mo) <= 1e-13 * abs(mo)
    g.close()
    # momentum with the finite-difference scheme's fluxes
    mm = Mesh(Nx=18, Ny=16, Nz=14, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, rho_liq=1000.0, rho_gas=1.2,
              pressure_scheme="finite-difference")
    _, _, VF2, band2, nx2, ny2, nz2, D2, uf2, vf2, wf2, u2, v2, w2, dt2 = momentum_state("5_tets")
    o2 = Oracle(mm)
    g2 = ctx(mm)
    VFg = VF2.copy(order="F")
    r = g2.transportSL_momentum(dt2, VFg, uf2, vf2, wf2, nx2, ny2, nz2, D2, band2, u2, v2, w2)
    flags, *ro = o2.transport_mom(dt2, VF2, uf2, vf2, wf2, nx2, ny2, nz2, D2, band2, u2, v2, w2)
    assert flags == 0
    assert_same(VFg, VF2, "VF (momentum call)")
    for a, b, name in zip(r, ro, ("us", "vs", "ws")):
        assert_same(mm.interior(a), mm.interior(b), name)
    g2.close()


def test_finite_difference_scheme_in_2d():
    """pressure_scheme "finite-difference" in 2D (Nz = 1, z periodic, w = 0; the z faces carry
    flat prisms and degenerate correction tets): the FP64 context bit for bit against the
    restatement over 8 steps of the single vortex, and the mixed context's flux form with the
    correction tets within its tolerance (measured: max |dVF| 6.5e-8, mass 3.8e-10 relative on
    this 40^2 grid, whose small mass per interface cell makes the relative figure larger than
    in 3D)."""
    m = Mesh(Nx=40, Ny=40, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 40, CFL=0.5, zper=True,
             pressure_scheme="finite-difference")
    VF = cases.vf_spheres(m, [[0.5, 0.75, 0.0]], [0.15], nF=10, dims=2)
    dt = 0.5 * m.dx
    for prec in ("fp64", "mixed"):
        o, g, VFo, band, nx, ny, nz, D = init_both(m, VF, prec)
        for s in range(8):
            uf, vf, wf = cases.deformation2d_faces(m, (s + 0.5) * dt, 8.0)
            g.upload_velocity(uf, vf, wf)
            mass = g.step(dt)
            assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
        VFg = g.download_vf()
        g.close()
        mo = o.mass(VFo)
        if prec == "fp64":
            assert_same(VFg, VFo, "VF")
            assert abs(mass - mo) <= 1e-13 * abs(mo)
        else:
            d = np.abs(m.interior(VFg) - m.interior(VFo))
            assert d.max() <= 1e-5 and np.quantile(d, 0.99) <= 1e-6, (d.max(), np.quantile(d, 0.99))
            assert abs(mass - mo) <= 4e-9 * abs(mo), abs(mass - mo) / abs(mo)


def test_finite_difference_scheme_in_a_mixed_context():
    """A mixed context with the finite-difference scheme: mixed normals and plane constants, and
    the update in flux form with each face's correction tets (apex and volume in FP64, their
    liquid from the FP32 clip; near-pure cells by the cell form with the cell's twelve
    correction tets).  VF within the mixed path's tolerance of the restatement over several
    steps, and the momentum call (FP64 clip in either precision) like an FP64 context's on the
    same inputs."""
    m = Mesh(Nx=20, Ny=20, Nz=20, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, pressure_scheme="finite-difference")
    VF = cases.vf_spheres(m, [[0.45, 0.52, 0.5]], [0.22], nF=10)
    o, g, VFo, band, nx, ny, nz, D = init_both(m, VF, "mixed")
    dt = 0.5 * m.dx / 2.0
    rng = np.random.default_rng(8)
    noise = [0.05 * rng.standard_normal(m.cell_shape) for _ in range(3)]
    for s in range(4):
        uf, vf, wf = (a + e for a, e in zip(cases.deformation3d_faces(m, 0.2 + (s + 0.5) * dt, 3.0), noise))
        uf, vf, wf = (np.asfortranarray(x) for x in (uf, vf, wf))
        g.upload_velocity(uf, vf, wf)
        mass = g.step(dt)
        assert o.step(dt, VFo, uf, vf, wf, nx, ny, nz, D, band) == 0
    # the plane constants differ from the FP64 ones in their last bits, so VF does too
    d = np.abs(m.interior(g.download_vf()) - m.interior(VFo))
    assert d.max() <= 5e-3 and np.quantile(d, 0.99) <= 1e-6, (d.max(), np.quantile(d, 0.99))
    mo = o.mass(VFo)
    assert abs(mass - mo) <= 1e-10 * abs(mo)
    g.close()
    mm = Mesh(Nx=18, Ny=16, Nz=14, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, rho_liq=1000.0, rho_gas=1.2,
              pressure_scheme="finite-difference")
    _, _, VF2, band2, nx2, ny2, nz2, D2, uf2, vf2, wf2, u2, v2, w2, dt2 = momentum_state("5_tets")
    out = []
    for prec in ("fp64", "mixed"):
        g2 = ctx(mm, prec)
        VFg = VF2.copy(order="F")
        r = g2.transportSL_momentum(dt2, VFg, uf2, vf2, wf2, nx2, ny2, nz2, D2, band2, u2, v2, w2)
        out.append((VFg, *r))
        g2.close()
    for a, b, name in zip(out[0], out[1], ("VF", "us", "vs", "ws")):
        assert_same(a, b, name)


@pytest.mark.parametrize("precision,tess", [("mixed", "24_tets"), ("fp64", "24_tets"), ("mixed", "6_tets")])
def test_finite_difference_scheme_unsupported_combinations(precision, tess):
    """The correction tets are defined for 5_tets (the reference keeps the first five tets);
    other tessellations are refused at creation."""
    from ns_multiphase_gb300.slvof import SLVOF
    m = Mesh(Nx=8, Ny=8, Nz=8, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess, pressure_scheme="finite-difference")
    with pytest.raises(RuntimeError):
        SLVOF(m, precision)


def test_momentum_in_a_mixed_context_runs_the_fp64_path():
    """A mixed-precision context's momentum call runs the FP64 clip: the same VF and us, vs, ws
    as an FP64 context on the same inputs."""
    m, o, VFo, band, nx, ny, nz, D, uf, vf, wf, u, v, w, dt = momentum_state("5_tets")
    out = []
    for prec in ("fp64", "mixed"):
        g = ctx(m, prec)
        VFg = VFo.copy(order="F")
        r = g.transportSL_momentum(dt, VFg, uf, vf, wf, nx, ny, nz, D, band, u, v, w)
        out.append((VFg, *r))
        g.close()
    for a, b, name in zip(out[0], out[1], ("VF", "us", "vs", "ws")):
        assert_same(a, b, name)
