"""Forward-mode derivatives of a whole rollout through the restatement (Dual numbers through the
initial state and every step's SL update, normals, PLIC and band: the CPU analogue of a
ForwardDiff.jl gradient of the transport loop).  Its value is the plain restatement's, and its
derivatives agree with central differences where the rollout is smooth."""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle


def setup(N=10, steps=2):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    VF0 = cases.vf_spheres(m, np.array([[0.45, 0.52, 0.55]]), np.array([0.27]), nF=6)
    dt = 0.5 * m.dx / 2.0
    rng = np.random.default_rng(3)
    uf, vf, wf = cases.deformation3d_faces(m, 0.3 + 0.5 * dt, 3.0)
    uf, vf, wf = (np.asfortranarray(a + 0.05 * rng.standard_normal(a.shape)) for a in (uf, vf, wf))
    w = rng.standard_normal((m.Nx, m.Ny, m.Nz))
    return m, VF0, dt, steps, (uf, vf, wf), w


def plain_rollout(o, m, VF0, dt, steps, vel, w):
    VF = VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VF)
    for _ in range(steps):
        assert o.step(dt, VF, *vel, nx, ny, nz, D, band) == 0
    return float(np.sum(m.interior(VF) * w))


def interface_cells(m, VF0, count):
    g = m.nghost + 3
    vfi = m.interior(VF0)
    idx = np.argwhere((vfi > 0.05) & (vfi < 0.95))
    return [tuple(int(x) + g for x in idx[q]) for q in np.linspace(0, len(idx) - 1, count).astype(int)]


def test_rollout_value_is_the_restatements():
    m, VF0, dt, steps, vel, w = setup()
    o = Oracle(m)
    L, _ = o.rollout_forward(dt, steps, VF0, *vel, [], [], w)
    assert L == pytest.approx(plain_rollout(o, m, VF0, dt, steps, vel, w), rel=1e-13, abs=1e-13)


def test_rollout_derivatives_against_central_differences():
    m, VF0, dt, steps, vel, w = setup()
    o = Oracle(m)
    # face entries of the velocity next to interface cells, and interface entries of VF0
    faces = [(a, (i - 3, j - 3, k - 3)) for a, (i, j, k) in zip([0, 1, 2, 0, 1, 2], interface_cells(m, VF0, 6))]
    cells = interface_cells(m, VF0, 4)
    L, dL = o.rollout_forward(dt, steps, VF0, *vel, faces, cells, w)
    def central(h):
        out = []
        for a, idx in faces:
            vp = [x.copy(order="F") for x in vel]
            vm = [x.copy(order="F") for x in vel]
            vp[a][idx] += h
            vm[a][idx] -= h
            out.append((plain_rollout(o, m, VF0, dt, steps, vp, w) - plain_rollout(o, m, VF0, dt, steps, vm, w)) / (2 * h))
        for idx in cells:
            Vp, Vm = VF0.copy(order="F"), VF0.copy(order="F")
            Vp[idx] += h
            Vm[idx] -= h
            out.append((plain_rollout(o, m, Vp, dt, steps, vel, w) - plain_rollout(o, m, Vm, dt, steps, vel, w)) / (2 * h))
        return np.array(out)
    fd, fd8 = central(1e-6), central(1e-6 / 8)
    # an entry is smooth where the two step sizes agree; a perturbation that flips an ELVIRA
    # near-tie (this sphere is nearly symmetric) makes the rollout jump, and there forward mode
    # gives the derivative of the branch taken while the differences see the jump
    scale = np.max(np.abs(dL))
    smooth = np.abs(fd - fd8) <= 1e-6 * scale
    assert smooth.sum() >= 8 and smooth[:len(faces)].all(), (fd, fd8, dL)
    assert np.max(np.abs(fd - dL)[smooth]) <= 1e-6 * scale, (fd, dL)
