"""The adjoint on the GPU against central finite differences of the CPU restatement.

Loss L = sum_c w_c VF_c over the interior after the rollout, seeded weights w.  The GPU
reverse pass (slvof_adjoint_step through ns_multiphase_gb300.adjoint.Rollout) gives dL/d(face
velocities) and dL/d(initial VF); each sampled entry is compared with (L(x+h) - L(x-h))/2h,
h = 1e-6, of the restatement's FP64 step (the reference's CPU path restated).  Velocities
carry seeded noise on every face, as the adjoint configurations do.  Tolerance: 1e-6 relative
to the largest sampled derivative.
"""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

H = 1e-6
RTOL = 1e-6


@pytest.fixture(scope="module")
def built():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return True


def oracle_rollout(m, VF0, vel, dt, steps, w):
    """L after `steps` FP64 steps of the restatement from VF0 (ghosts filled here)."""
    o = Oracle(m)
    VF = VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VF)
    for n in range(steps):
        uf, vf, wf = vel(n)
        f = o.step(dt, VF, uf, vf, wf, nx, ny, nz, D, band, True)
        assert f == 0
    return float(np.sum(m.interior(VF) * w))


def gpu_gradients(m, VF0, vel, dt, steps, w, every, precision="fp64"):
    from ns_multiphase_gb300.adjoint import Rollout
    from ns_multiphase_gb300.slvof import SLVOF
    g = SLVOF(m, precision)
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    R = Rollout(g, dt, steps, vel, every=every)
    VFT = R.forward()
    gT = m.vf_array()
    m.interior(gT)[...] = w
    gVF0, (gu, gv, gw) = R.backward(gT)
    L = float(np.sum(m.interior(VFT) * w))
    g.close()
    return L, gVF0, gu, gv, gw


def noisy(m, base, sigma, seed):
    rng = np.random.default_rng(seed)
    noise = [sigma * rng.standard_normal(m.cell_shape) for _ in range(3)]
    if m.Nz == 1:
        noise[2][...] = 0.0

    def vel(n):
        uf, vf, wf = base(n)
        return tuple(np.asfortranarray(a + e) for a, e in zip((uf, vf, wf), noise))
    return vel, noise


def sample_faces(grads, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for q, g in enumerate(grads):
        idx = np.argwhere(np.abs(g) > 0)
        if len(idx) == 0:
            continue
        order = np.argsort(-np.abs(g[tuple(idx.T)]))
        for p in list(order[:count // 2]) + list(rng.choice(len(idx), size=min(count // 2, len(idx)), replace=False)):
            out.append((q, tuple(idx[p])))
    return out


def fd_velocity(m, VF0, noise, base, dt, steps, w, q, idx):
    vals = []
    for sgn in (1.0, -1.0):
        pert = [a.copy(order="F") for a in noise]
        pert[q][idx] += sgn * H

        def vel(n):
            uf, vf, wf = base(n)
            return tuple(np.asfortranarray(a + e) for a, e in zip((uf, vf, wf), pert))
        vals.append(oracle_rollout(m, VF0, vel, dt, steps, w))
    return (vals[0] - vals[1]) / (2 * H)


def check_velocity(m, VF0, base, noise, dt, steps, w, grads, count=12):
    worst, scale, n = 0.0, 0.0, 0
    picks = sample_faces(grads, count, 7)
    fds = []
    for q, idx in picks:
        fds.append(fd_velocity(m, VF0, noise, base, dt, steps, w, q, idx))
    scale = max(abs(f) for f in fds)
    for (q, idx), fd in zip(picks, fds):
        worst = max(worst, abs(fd - grads[q][idx]) / scale)
        n += 1
    return worst, n


def sphere3d(N=12, scheme="semi-lagrangian"):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, pressure_scheme=scheme)
    VF0 = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
    return m, VF0


def test_single_step_3d_velocity_gradient(built):
    m, VF0 = sphere3d()
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, noise = noisy(m, base, 0.05, 31)
    w = np.random.default_rng(2).standard_normal((m.Nx, m.Ny, m.Nz))
    L_gpu, gVF0, gu, gv, gw = gpu_gradients(m, VF0, vel, dt, 1, w, every=1)
    L_cpu = oracle_rollout(m, VF0, vel, dt, 1, w)
    assert abs(L_gpu - L_cpu) <= 1e-12 * max(1.0, abs(L_cpu))
    worst, n = check_velocity(m, VF0, base, noise, dt, 1, w, (gu, gv, gw))
    assert n >= 12
    assert worst <= RTOL, worst


def test_single_step_3d_initial_vf_gradient(built):
    m, VF0 = sphere3d()
    # The sub-sampled sphere holds VF in multiples of 1/512, so neighbours often tie exactly:
    # ELVIRA's +-1 components compare neighbours and its candidate errors then tie, discrete
    # choices that a step of h flips.  Seeded jitter on the interface cells removes the ties.
    inner = m.interior(VF0)
    mixed = (inner > 0.02) & (inner < 0.98)
    inner[mixed] += np.random.default_rng(8).uniform(-0.01, 0.01, size=int(mixed.sum()))
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, noise = noisy(m, base, 0.05, 31)
    w = np.random.default_rng(2).standard_normal((m.Nx, m.Ny, m.Nz))
    _, gVF0, _, _, _ = gpu_gradients(m, VF0, vel, dt, 1, w, every=1)
    # interface cells only: a pure cell moved by h becomes an interface cell (band and ELVIRA
    # switch), where the step is not differentiable
    inner = m.interior(VF0)
    cand = np.argwhere((inner > 1e-3) & (inner < 1 - 1e-3))
    rng = np.random.default_rng(4)
    picks = cand[rng.choice(len(cand), size=10, replace=False)]
    fds, adj = [], []
    for (a, b, c) in picks:
        idx = m.vidx(a + 1, b + 1, c + 1)
        vals = []
        for sgn in (1.0, -1.0):
            V = VF0.copy(order="F")
            V[idx] += sgn * H
            vals.append(oracle_rollout(m, V, vel, dt, 1, w))
        fds.append((vals[0] - vals[1]) / (2 * H))
        adj.append(gVF0[idx])
    fds, adj = np.array(fds), np.array(adj)
    assert np.max(np.abs(fds - adj)) <= RTOL * np.max(np.abs(fds)), (fds, adj)


def test_rollout_2d_vortex_with_checkpoints(built):
    """The 2D single-vortex adjoint configuration at reduced size: 32x32, circle r = 0.15 at
    (0.5, 0.75), noise 0.05 on every face, 6 steps, VF checkpoint every 3 steps."""
    N = 32
    m = Mesh(Nx=N, Ny=N, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / N, CFL=0.5, zper=True)
    VF0 = cases.vf_spheres(m, np.array([[0.5, 0.75, 0.0]]), np.array([0.15]), nF=10, dims=2)
    dt = 0.5 * m.dx
    base = lambda n: cases.deformation2d_faces(m, (n + 0.5) * dt, 8.0)
    vel, noise = noisy(m, base, 0.05, 17)
    steps = 6
    w = np.random.default_rng(9).standard_normal((m.Nx, m.Ny, m.Nz))
    L_gpu, gVF0, gu, gv, gw = gpu_gradients(m, VF0, vel, dt, steps, w, every=3)
    L_cpu = oracle_rollout(m, VF0, vel, dt, steps, w)
    assert abs(L_gpu - L_cpu) <= 1e-12 * max(1.0, abs(L_cpu))
    worst, n = check_velocity(m, VF0, base, noise, dt, steps, w, (gu, gv, gw), count=16)
    assert n >= 16
    assert worst <= RTOL, worst


def test_checkpoint_interval_does_not_change_the_gradient(built):
    N = 24
    m = Mesh(Nx=N, Ny=N, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / N, CFL=0.5, zper=True)
    VF0 = cases.vf_spheres(m, np.array([[0.5, 0.6, 0.0]]), np.array([0.2]), nF=10, dims=2)
    dt = 0.5 * m.dx
    base = lambda n: cases.deformation2d_faces(m, (n + 0.5) * dt, 8.0)
    vel, _ = noisy(m, base, 0.05, 5)
    w = np.random.default_rng(1).standard_normal((m.Nx, m.Ny, m.Nz))
    a = gpu_gradients(m, VF0, vel, dt, 5, w, every=5)
    b = gpu_gradients(m, VF0, vel, dt, 5, w, every=2)
    for x, y in zip(a[1:], b[1:]):
        assert np.allclose(x, y, rtol=1e-12, atol=1e-12 * np.max(np.abs(x)))


def test_mixed_reverse_against_finite_differences(built):
    """A mixed-precision context's reverse (boundary form, FP32 cell-local geometry, FP64
    accumulation) around its own states, against central differences of the FP64 restatement,
    and against the FP64 context's reverse (relative L2 over all face derivatives)."""
    m, VF0 = sphere3d(16)
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, noise = noisy(m, base, 0.05, 3)
    w = np.random.default_rng(6).standard_normal((m.Nx, m.Ny, m.Nz))
    a = gpu_gradients(m, VF0, vel, dt, 2, w, every=1, precision="fp64")
    b = gpu_gradients(m, VF0, vel, dt, 2, w, every=1, precision="mixed")
    ga = np.concatenate([x.ravel() for x in a[2:]])
    gb = np.concatenate([x.ravel() for x in b[2:]])
    assert np.linalg.norm(ga - gb) <= 5e-6 * np.linalg.norm(ga)
    assert np.linalg.norm(a[1] - b[1]) <= 5e-6 * np.linalg.norm(a[1])
    worst, n = check_velocity(m, VF0, base, noise, dt, 2, w, b[2:])
    assert n >= 12
    assert worst <= RTOL, worst


@pytest.mark.parametrize("case", ["6_tets", "24_tets", "2d"])
def test_mixed_reverse_other_tessellations_and_2d(built, case):
    """The mixed reverse over 6_tets and 24_tets (3D, one step) and a 2D vortex rollout (32^2,
    6 steps, checkpoint every 3) against the FP64 context's reverse."""
    if case == "2d":
        m = Mesh(Nx=32, Ny=32, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 32, CFL=0.5, zper=True)
        VF0 = cases.vf_spheres(m, np.array([[0.5, 0.75, 0.0]]), np.array([0.15]), nF=10, dims=2)
        dt = 0.5 * m.dx
        base = lambda n: cases.deformation2d_faces(m, (n + 0.5) * dt, 8.0)
        steps, every = 6, 3
    else:
        m = Mesh(Nx=12, Ny=12, Nz=12, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=case)
        VF0 = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
        dt = 0.5 * m.dx / 2.0
        base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
        steps, every = 1, 1
    vel, _ = noisy(m, base, 0.05, 31)
    w = np.random.default_rng(2).standard_normal((m.Nx, m.Ny, m.Nz))
    a = gpu_gradients(m, VF0, vel, dt, steps, w, every=every, precision="fp64")
    b = gpu_gradients(m, VF0, vel, dt, steps, w, every=every, precision="mixed")
    ga = np.concatenate([x.ravel() for x in a[2:]])
    gb = np.concatenate([x.ravel() for x in b[2:]])
    assert np.linalg.norm(ga - gb) <= 5e-6 * np.linalg.norm(ga)
    assert np.linalg.norm(a[1] - b[1]) <= 5e-6 * np.linalg.norm(a[1])


def test_mixed_reverse_with_the_step_result_given(built):
    """slvof_adjoint_step_next with the step's result (the rollout's stored states) gives the
    derivatives that slvof_adjoint_step computes after recomputing the clipped volumes.  The
    reverse accumulates with FP64 atomics, whose order varies from run to run; where such a
    last-bit difference reaches a cell's FP32 seed it can move it by one FP32 rounding, so two
    runs of the same rollout agree to about 1e-8 of the largest entry, not bit for bit."""
    from ns_multiphase_gb300.adjoint import Rollout
    from ns_multiphase_gb300.slvof import SLVOF
    m, VF0 = sphere3d(16)
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, _ = noisy(m, base, 0.05, 9)
    w = np.random.default_rng(3).standard_normal((m.Nx, m.Ny, m.Nz))
    out = []
    for give in (True, False):
        g = SLVOF(m, "mixed")
        g.upload_vf(VF0)
        g.vf_ghost_fill()
        R = Rollout(g, dt, 4, vel, every=2, give_next=give)
        R.forward()
        gT = m.vf_array()
        m.interior(gT)[...] = w
        gVF0, grads = R.backward(gT)
        out.append([gVF0, *grads])
        g.close()
    for x, y in zip(*out):
        assert np.allclose(x, y, rtol=0.0, atol=1e-7 * np.max(np.abs(x)))


@pytest.mark.parametrize("which", ["2d", "3d"])
def test_adjoint_configurations_at_reduced_size(built, which):
    """The two adjoint configurations (tests/adjoint_configs.py) at reduced size,
    checked against central differences of the CPU restatement on random entries of the
    derivative's support: 2D 32^2 vortex + noise on every face (8 steps, checkpoint every 3),
    3D 16^3 deformation + curl of the 3 x 512-coefficient potential (4 steps, every 2)."""
    import adjoint_configs as A
    if which == "2d":
        cfg = A.config2d(N=32, steps=8, every=3)
        out = A.check(cfg, 12, "cpu")
    else:
        cfg = A.config3d(N=16, steps=4, every=2)
        out = A.check(cfg, 8, "cpu")
    assert out["checked"] >= 8
    assert out["max_abs_err_over_max_fd"] <= RTOL, out


@pytest.mark.parametrize("tess", ["6_tets", "24_tets"])
def test_single_step_other_tessellations(built, tess):
    """The reverse pass over 6_tets and 24_tets (mean points' derivatives shared out to the
    vertices they average) against central differences of the restatement."""
    m = Mesh(Nx=12, Ny=12, Nz=12, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess)
    VF0 = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, noise = noisy(m, base, 0.05, 31)
    w = np.random.default_rng(2).standard_normal((m.Nx, m.Ny, m.Nz))
    L_gpu, gVF0, gu, gv, gw = gpu_gradients(m, VF0, vel, dt, 1, w, every=1)
    L_cpu = oracle_rollout(m, VF0, vel, dt, 1, w)
    assert abs(L_gpu - L_cpu) <= 1e-12 * max(1.0, abs(L_cpu))
    worst, n = check_velocity(m, VF0, base, noise, dt, 1, w, (gu, gv, gw))
    assert n >= 12
    assert worst <= RTOL, worst


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 2e-6)])
def test_against_forward_mode_on_a_small_grid(built, precision, tol):
    """One step on 12^3: the GPU reverse pass's dL/d(face velocities) against forward-mode
    derivatives of the FP64 restatement (Dual numbers through the CPU path, the analogue of a
    ForwardDiff.jl gradient), on every face the reverse pass reaches.  The FP64 reverse agrees to
    rounding; the mixed one (FP32 geometry around its own states) to FP32 accuracy."""
    forward_mode_check(sphere3d(12), precision, tol)


@pytest.mark.parametrize("projection", ["Euler", "Midpoint"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 2e-6)])
def test_other_projections_against_forward_mode(built, projection, precision, tol):
    """The reverse of project!'s Euler and Midpoint stages (src/Tools.jl:392-418), as the RK4
    case above."""
    m = Mesh(Nx=12, Ny=12, Nz=12, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, projection=projection)
    VF0 = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=8)
    forward_mode_check((m, VF0), precision, tol)


def forward_mode_check(mesh_vf, precision, tol):
    import sys
    import os
    sys.path.insert(0, os.path.dirname(__file__))
    from test_adjoint_host import forward_mode_grads
    m, VF0 = mesh_vf
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, noise = noisy(m, base, 0.05, 17)
    w = np.random.default_rng(5).standard_normal((m.Nx, m.Ny, m.Nz))
    L, gVF0, gu, gv, gw = gpu_gradients(m, VF0, vel, dt, 1, w, every=1, precision=precision)
    o = Oracle(m)
    VF = VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VF)
    uf, vf, wf = vel(0)
    cells = [(i, j, k) for k in range(1, m.Nz + 1) for j in range(1, m.Ny + 1) for i in range(1, m.Nx + 1)
             if abs(int(band[m.cidx(i, j, k)])) <= m.nband]
    weights = np.array([w[i - 1, j - 1, k - 1] for i, j, k in cells])
    grads = (gu, gv, gw)
    entries = [(a, tuple(int(x) for x in idx)) for a in range(3) for idx in np.argwhere(grads[a] != 0.0)]
    assert len(entries) > 100
    st = (m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt)
    fwd = forward_mode_grads(o, st, cells, weights, entries)
    rev = np.array([grads[a][idx] for a, idx in entries])
    assert np.max(np.abs(fwd - rev)) <= tol * np.max(np.abs(fwd))


@pytest.mark.parametrize("scheme", ["semi-lagrangian", "finite-difference"])
def test_rollout_against_forward_mode(built, scheme):
    """The FP64 reverse of a 3-step rollout (checkpoint every step) against forward-mode
    derivatives of the restatement's whole rollout (Dual numbers through the initial state and
    every step's SL update, normals, PLIC and band: the analogue of a ForwardDiff.jl gradient of
    the transport loop), on 12^3 with the velocities frozen over the rollout.  The entries are
    the 32 largest face-velocity derivatives and 16 interface entries of VF0, whose derivatives
    run back through every step's ELVIRA and plane-constant solve to the initial state's.  The
    FP64 path is the restatement bit for bit, so both take the same branches and agree to
    rounding.  With pressure_scheme "finite-difference" every band cell also clips its twelve
    flux-correction tets (add_correction_tets, src/VFgeom.jl:514-664), whose reverse runs
    through their apex solve, the faces' flux volumes and the face velocities."""
    m, VF0 = sphere3d(12, scheme)
    dt = 0.5 * m.dx / 2.0
    steps = 3
    base = lambda n: cases.deformation3d_faces(m, 0.3 + 0.5 * dt, 3.0)
    vel, _ = noisy(m, base, 0.05, 23)
    w = np.random.default_rng(8).standard_normal((m.Nx, m.Ny, m.Nz))
    L, gVF0, gu, gv, gw = gpu_gradients(m, VF0, vel, dt, steps, w, every=1, precision="fp64")
    o = Oracle(m)
    uf, vf, wf = vel(0)
    grads = (gu, gv, gw)
    entries = [(a, tuple(int(x) for x in idx)) for a in range(3) for idx in np.argwhere(grads[a] != 0.0)]
    entries.sort(key=lambda e: -abs(grads[e[0]][e[1]]))
    faces = entries[:32]
    g3 = m.nghost + 3
    vfi = m.interior(VF0)
    iface = np.argwhere((vfi > 0.02) & (vfi < 0.98))
    cells = [tuple(int(x) for x in iface[q]) for q in np.linspace(0, len(iface) - 1, 16).astype(int)]
    K = o.ndual()
    fwd, rev = [], []
    for c0 in range(0, len(faces), K):
        batch = faces[c0:c0 + K]
        Lo, dL = o.rollout_forward(dt, steps, VF0, uf, vf, wf, batch, [], w)
        fwd += list(dL)
        rev += [grads[a][idx] for a, idx in batch]
    assert abs(L - Lo) <= 1e-12 * max(1.0, abs(Lo))
    parents = [tuple(q + g3 for q in c) for c in cells]
    Lo, dL = o.rollout_forward(dt, steps, VF0, uf, vf, wf, [], parents, w)
    fwd += list(dL)
    rev += [gVF0[p] for p in parents]  # the derivative comes back in VF layout
    fwd, rev = np.array(fwd), np.array(rev)
    assert np.max(np.abs(fwd[32:])) > 0
    assert np.max(np.abs(fwd - rev)) <= 1e-9 * np.max(np.abs(fwd)), np.max(np.abs(fwd - rev)) / np.max(np.abs(fwd))


def test_finite_difference_reverse_in_a_mixed_context(built):
    """A mixed context's finite-difference step runs the flux form with the correction tets, on
    its FP64 winner normals and plane constants, and its reverse is the FP64 one (k_adj_sl_fd):
    against the FP64 context's reverse on the same rollout (relative L2 over all face and
    initial-VF derivatives)."""
    m, VF0 = sphere3d(12, "finite-difference")
    dt = 0.5 * m.dx / 2.0
    base = lambda n: cases.deformation3d_faces(m, 0.3 + (n + 0.5) * dt, 3.0)
    vel, _ = noisy(m, base, 0.05, 29)
    w = np.random.default_rng(9).standard_normal((m.Nx, m.Ny, m.Nz))
    a = gpu_gradients(m, VF0, vel, dt, 2, w, every=1, precision="fp64")
    b = gpu_gradients(m, VF0, vel, dt, 2, w, every=1, precision="mixed")
    ga = np.concatenate([x.ravel() for x in a[2:]])
    gb = np.concatenate([x.ravel() for x in b[2:]])
    assert np.linalg.norm(ga) > 0
    assert np.linalg.norm(ga - gb) <= 1e-6 * np.linalg.norm(ga), np.linalg.norm(ga - gb) / np.linalg.norm(ga)
    assert np.linalg.norm(a[1] - b[1]) <= 1e-6 * np.linalg.norm(a[1]), np.linalg.norm(a[1] - b[1]) / np.linalg.norm(a[1])
