"""Synthetic inputs for the SL-VOF path: deformation velocity fields and sphere/circle VF.

These are input generators, not part of the transport path.  They restate the reference's
own generators with the period made a parameter:

* face velocities are sampled pointwise at the face centres, ghosts included, exactly as
  ``defineVelocity!`` does (src/Tools.jl:648-693; ``uf[i,j,k] = u(x[i], ym[j], zm[k])``);
  the reference hard-codes the period T=2, the workloads here use T=8 (2D) and T=3 (3D);
* VF of a sphere (or of a union of spheres) uses ``VFsphere``'s sub-sampling rule
  (src/Tools.jl:907-922): nF points per direction at ``xmin + i/(nF+1)*dx``, i = 1..nF,
  each point inside adding 1/nF^3 in sequence; the 2D circle uses the same rule in x-y.
  IC! fills every cell of ``imino_:imaxo_`` and leaves VF's three extra layers at zero
  (examples/example5_deformation3D.jl:65, src/Tools.jl:144).

The numpy versions here serve small grids; the CUDA library has the same generators for
the 256^3 workload (``slvof_case_*``).
"""
from __future__ import annotations

import math

import numpy as np

from .mesh import Mesh

PI = math.pi


def seq_sum_table(c: float, n: int) -> np.ndarray:
    """table[m] = ((0 + c) + c) + ... (m times): the reference's running ``VF += VFsubcell``."""
    t = np.empty(n + 1)
    s = 0.0
    t[0] = 0.0
    for m in range(1, n + 1):
        s = s + c
        t[m] = s
    return t


def deformation2d_faces(mesh: Mesh, t: float, T: float = 8.0):
    """Single-vortex field u = -2 sin^2(pi x) sin(pi y) cos(pi y) cos(pi t/T),
    v = 2 sin^2(pi y) sin(pi x) cos(pi x) cos(pi t/T), w = 0 (src/Tools.jl:656-658)."""
    ct = math.cos(PI * t / T)
    x, y, xm, ym = mesh.x[:-1], mesh.y[:-1], mesh.xm, mesh.ym
    nz = mesh.cell_shape[2]
    # u at (x[i], ym[j]); v at (xm[i], y[j])
    sx = np.sin(PI * x)[:, None]
    uf2 = ((-2.0 * sx ** 2) * np.sin(PI * ym)[None, :]) * np.cos(PI * ym)[None, :] * ct
    sy = np.sin(PI * y)[None, :]
    vf2 = ((2.0 * sy ** 2) * np.sin(PI * xm)[:, None]) * np.cos(PI * xm)[:, None] * ct
    uf = np.asfortranarray(np.repeat(uf2[:, :, None], nz, axis=2))
    vf = np.asfortranarray(np.repeat(vf2[:, :, None], nz, axis=2))
    wf = mesh.cell_array()
    return uf, vf, wf


def deformation3d_faces(mesh: Mesh, t: float, T: float = 3.0):
    """u = 2 sin^2(pi x) sin(2 pi y) sin(2 pi z) cos(pi t/T), v = -sin^2(pi y) sin(2 pi x)
    sin(2 pi z) cos(pi t/T), w = -sin^2(pi z) sin(2 pi x) sin(2 pi y) cos(pi t/T)
    (src/Tools.jl:660-662 with the period as a parameter)."""
    ct = math.cos(PI * t / T)
    x, y, z = mesh.x[:-1], mesh.y[:-1], mesh.z[:-1]
    xm, ym, zm = mesh.xm, mesh.ym, mesh.zm

    def s2(a):
        return np.sin(PI * a) ** 2

    def s2pi(a):
        return np.sin(2 * PI * a)

    uf = ((2.0 * s2(x)[:, None, None]) * s2pi(ym)[None, :, None]) * s2pi(zm)[None, None, :] * ct
    vf = ((-s2(y)[None, :, None]) * s2pi(xm)[:, None, None]) * s2pi(zm)[None, None, :] * ct
    wf = ((-s2(z)[None, None, :]) * s2pi(xm)[:, None, None]) * s2pi(ym)[None, :, None] * ct
    return (np.asfortranarray(uf), np.asfortranarray(vf), np.asfortranarray(wf))


class Deformation3DFaces:
    """deformation3d_faces with the time-independent products formed once: faces(t, T) returns
    the same arrays bit for bit (each component is (space product) * cos(pi t/T), multiplied in
    the same order), for runs that need the field at many times."""

    def __init__(self, mesh: Mesh):
        x, y, z = mesh.x[:-1], mesh.y[:-1], mesh.z[:-1]
        xm, ym, zm = mesh.xm, mesh.ym, mesh.zm
        s2 = lambda a: np.sin(PI * a) ** 2
        s2pi = lambda a: np.sin(2 * PI * a)
        self.p = (np.asfortranarray((2.0 * s2(x)[:, None, None]) * s2pi(ym)[None, :, None] * s2pi(zm)[None, None, :]),
                  np.asfortranarray((-s2(y)[None, :, None]) * s2pi(xm)[:, None, None] * s2pi(zm)[None, None, :]),
                  np.asfortranarray((-s2(z)[None, None, :]) * s2pi(xm)[:, None, None] * s2pi(ym)[None, :, None]))

    def faces(self, t: float, T: float = 3.0):
        ct = math.cos(PI * t / T)
        return tuple(np.asfortranarray(a * ct) for a in self.p)


def uniform_faces(mesh: Mesh, u: float, v: float, w: float):
    uf, vf, wf = mesh.cell_array(), mesh.cell_array(), mesh.cell_array()
    uf[...] = u
    vf[...] = v
    wf[...] = w
    return uf, vf, wf


def vf_spheres(mesh: Mesh, centres, radii, nF: int = 20, dims: int = 3) -> np.ndarray:
    """VF over ``imino_:imaxo_`` of the union of spheres (dims=3) or circles in x-y (dims=2).

    Cells whose box lies inside a sphere take the full sequential sum, cells away from every
    sphere take 0, the rest are sub-sampled point by point.
    """
    centres = np.asarray(centres, dtype=np.float64).reshape(-1, 3)
    radii = np.asarray(radii, dtype=np.float64).reshape(-1)
    npts = nF ** dims
    table = seq_sum_table(1.0 / npts, npts)
    g = mesh.nghost
    shape = mesh.cell_shape
    x, y, z = mesh.x, mesh.y, mesh.z
    count = np.zeros(shape, dtype=np.int64)
    full = np.zeros(shape, dtype=bool)
    frac = np.arange(1, nF + 1) / (nF + 1)
    # candidate cells per sphere (index boxes), then exact sub-sampling
    cand = np.zeros(shape, dtype=bool)
    for c, r in zip(centres, radii):
        lo = [np.searchsorted(a, c[d] - r, side="right") - 1 for d, a in enumerate((x, y, z))]
        hi = [np.searchsorted(a, c[d] + r, side="left") for d, a in enumerate((x, y, z))]
        if dims == 2:
            lo[2], hi[2] = 0, shape[2]
        sl = tuple(slice(max(l, 0), min(h, n)) for l, h, n in zip(lo, hi, shape))
        cand[sl] = True
    idx = np.argwhere(cand)
    if len(idx):
        ci, cj, ck = idx[:, 0], idx[:, 1], idx[:, 2]
        x0, x1 = x[ci], x[ci + 1]
        y0, y1 = y[cj], y[cj + 1]
        z0, z1 = z[ck], z[ck + 1]
        # whole cell inside one sphere?  (all 8 corners strictly inside)
        for c, r in zip(centres, radii):
            if dims == 3:
                far = (np.maximum(np.abs(x0 - c[0]), np.abs(x1 - c[0])) ** 2 +
                       np.maximum(np.abs(y0 - c[1]), np.abs(y1 - c[1])) ** 2 +
                       np.maximum(np.abs(z0 - c[2]), np.abs(z1 - c[2])) ** 2)
            else:
                far = (np.maximum(np.abs(x0 - c[0]), np.abs(x1 - c[0])) ** 2 +
                       np.maximum(np.abs(y0 - c[1]), np.abs(y1 - c[1])) ** 2)
            inside = far < r * r * (1 - 1e-12)
            full[ci[inside], cj[inside], ck[inside]] = True
        todo = ~full[ci, cj, ck]
        ci, cj, ck = ci[todo], cj[todo], ck[todo]
        x0, x1, y0, y1, z0, z1 = x0[todo], x1[todo], y0[todo], y1[todo], z0[todo], z1[todo]
        chunk = max(1, 2_000_000 // npts)
        for s in range(0, len(ci), chunk):
            e = s + chunk
            xh = x0[s:e, None] + frac[None, :] * (x1[s:e] - x0[s:e])[:, None]
            yh = y0[s:e, None] + frac[None, :] * (y1[s:e] - y0[s:e])[:, None]
            zh = z0[s:e, None] + frac[None, :] * (z1[s:e] - z0[s:e])[:, None]
            hit = np.zeros((len(xh), nF, nF, nF if dims == 3 else 1), dtype=bool)
            for c, r in zip(centres, radii):
                dxs = (xh - c[0]) ** 2
                dys = (yh - c[1]) ** 2
                if dims == 3:
                    dzs = (zh - c[2]) ** 2
                    G = r ** 2 - ((dxs[:, :, None, None] + dys[:, None, :, None]) + dzs[:, None, None, :])
                else:
                    G = (r ** 2 - (dxs[:, :, None] + dys[:, None, :]))[:, :, :, None]
                hit |= G > 0.0
            count[ci[s:e], cj[s:e], ck[s:e]] = hit.reshape(len(xh), -1).sum(axis=1)
    count[full] = npts
    vf = mesh.vf_array()
    vf[3:-3, 3:-3, 3:-3] = table[count]
    return vf


def config_spheres(n_spheres: int = 200, seed: int = 20261203):
    """Centres U[0.1,0.9]^3 and radii U[0.02,0.08] from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.1, 0.9, size=(n_spheres, 3))
    radii = rng.uniform(0.02, 0.08, size=n_spheres)
    return centres, radii


class FourierPotential:
    """Divergence-free face velocities from the curl of a vector potential.

    A_q(x, y, z) = sum_{a,b,c < M} C[q, a, b, c] / |k_abc| sin(pi (a+1) x/Lx) sin(pi (b+1) y/Ly)
    sin(pi (c+1) z/Lz), q = x, y, z (M = 8: 3 x 512 coefficients), |k_abc| = pi sqrt((a+1)^2 +
    (b+1)^2 + (c+1)^2): each mode scaled so that a unit coefficient gives a velocity of order
    one (curl multiplies a mode by its wavenumber).  A vanishes on the domain
    boundary, so curl A has no normal component there.  Each face's velocity is its flux of
    curl A, i.e. by Stokes the circulation of A around the face's four edges (line integrals
    of the sines, exact), over the face area: the face fluxes of every cell then sum to zero
    exactly (each edge enters two faces with opposite signs), a discretely divergence-free
    field.  Faces in the ghost layers use the same formula at their coordinates.

    The map C -> (uf, vf, wf) is linear and separable; ``grad`` is its transpose, taking
    dL/d(face velocities) to dL/dC.
    """

    def __init__(self, mesh: Mesh, modes: int = 8):
        self.m = mesh
        self.M = modes
        L = (mesh.Lx, mesh.Ly, mesh.Lz)
        faces = (mesh.x, mesh.y, mesh.z)
        k = PI * np.arange(1, modes + 1)
        # node values S[d][a, i] = sin(k_a p_i / L) at faces p_i (cell-array index i), and the
        # edge integrals I[d][a, i] = int_{p_i}^{p_{i+1}} sin(k_a p / L) dp
        self.S, self.I = [], []
        for d in range(3):
            p = np.asarray(faces[d])
            ka = k[:, None] / L[d]
            self.S.append(np.sin(ka * p[None, :-1]))
            self.I.append((np.cos(ka * p[None, :-1]) - np.cos(ka * p[None, 1:])) / ka)
        self.area = (mesh.dy * mesh.dz, mesh.dx * mesh.dz, mesh.dx * mesh.dy)
        n = np.arange(1, modes + 1, dtype=np.float64)
        self.W = 1.0 / (PI * np.sqrt(n[:, None, None] ** 2 + n[None, :, None] ** 2 + n[None, None, :] ** 2))

    def _edge(self, C, q):
        """Line integrals of A_q along the q-directed edges: E[i, j, k] over the cell-array
        index ranges (the edge from node (i, j, k) one cell along q)."""
        f = [self.I[d] if d == q else self.S[d] for d in range(3)]
        return np.einsum("abc,ai,bj,ck->ijk", C[q] * self.W, f[0], f[1], f[2], optimize=True)

    def faces(self, C):
        """(uf, vf, wf) cell arrays (Fortran order) of curl A."""
        Ex, Ey, Ez = (self._edge(C, q) for q in range(3))
        sh = self.m.cell_shape
        uf, vf, wf = np.zeros(sh), np.zeros(sh), np.zeros(sh)
        # x-face (i, j, k): +Ey(k) - Ey(k+1) + Ez(j+1) - Ez(j)
        uf[:, :-1, :-1] = (Ey[:, :-1, :-1] - Ey[:, :-1, 1:]) + (Ez[:, 1:, :-1] - Ez[:, :-1, :-1])
        # y-face (i, j, k): +Ez(i) - Ez(i+1) + Ex(k+1) - Ex(k)
        vf[:-1, :, :-1] = (Ez[:-1, :, :-1] - Ez[1:, :, :-1]) + (Ex[:-1, :, 1:] - Ex[:-1, :, :-1])
        # z-face (i, j, k): +Ex(j) - Ex(j+1) + Ey(i+1) - Ey(i)
        wf[:-1, :-1, :] = (Ex[:-1, :-1, :] - Ex[:-1, 1:, :]) + (Ey[1:, :-1, :] - Ey[:-1, :-1, :])
        return tuple(np.asfortranarray(a / ar) for a, ar in zip((uf, vf, wf), self.area))

    def grad(self, gu, gv, gw):
        """dL/dC (3, M, M, M) from dL/d(uf, vf, wf): the transpose of faces()."""
        gu, gv, gw = gu / self.area[0], gv / self.area[1], gw / self.area[2]
        sh = self.m.cell_shape
        gEx, gEy, gEz = np.zeros(sh), np.zeros(sh), np.zeros(sh)
        a = gu[:, :-1, :-1]
        gEy[:, :-1, :-1] += a; gEy[:, :-1, 1:] -= a; gEz[:, 1:, :-1] += a; gEz[:, :-1, :-1] -= a
        b = gv[:-1, :, :-1]
        gEz[:-1, :, :-1] += b; gEz[1:, :, :-1] -= b; gEx[:-1, :, 1:] += b; gEx[:-1, :, :-1] -= b
        c = gw[:-1, :-1, :]
        gEx[:-1, :-1, :] += c; gEx[:-1, 1:, :] -= c; gEy[1:, :-1, :] += c; gEy[:-1, :-1, :] -= c
        out = np.zeros((3, self.M, self.M, self.M))
        for q, gE in enumerate((gEx, gEy, gEz)):
            f = [self.I[d] if d == q else self.S[d] for d in range(3)]
            out[q] = np.einsum("ijk,ai,bj,ck->abc", gE, f[0], f[1], f[2], optimize=True) * self.W
        return out
