"""The algorithmic operation count of the step: the restatement's ELVIRA, plane-constant and
SL paths instantiated with a counting scalar.  The counted instantiation must compute the
same values as the double restatement bit for bit (so the count is of the restatement's own
arithmetic), and the counts must be deterministic and additive over cells."""
import numpy as np
import pytest

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh
from oracle.oracle import Oracle


@pytest.fixture(scope="module")
def state():
    m = Mesh(Nx=18, Ny=16, Nz=14, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    VF = cases.vf_spheres(m, np.array([[0.4, 0.45, 0.5], [0.7, 0.6, 0.4]]), np.array([0.22, 0.13]), nF=6)
    o = Oracle(m)
    band, nx, ny, nz, D = o.init_state(VF)
    dt = 0.5 * m.dx / 2.0
    uf, vf, wf = cases.deformation3d_faces(m, 0.5 * dt, 3.0)
    inner = (slice(m.nghost, m.nghost + m.Nx), slice(m.nghost, m.nghost + m.Ny), slice(m.nghost, m.nghost + m.Nz))
    vfi = m.interior(VF)
    iface = np.flatnonzero(((vfi >= m.VFlo) & (vfi <= m.VFhi)).ravel(order="F"))
    bnd = np.flatnonzero((np.abs(band[inner]) <= m.nband).ravel(order="F"))
    assert len(iface) > 50 and len(bnd) > len(iface)
    return m, o, VF, uf, vf, wf, nx, ny, nz, D, band, dt, iface, bnd


def _ijk(m, L):
    return 1 + L % m.Nx, 1 + (L // m.Nx) % m.Ny, 1 + L // (m.Nx * m.Ny)


def test_counted_paths_compute_the_restatements_values(state):
    m, o, VF, uf, vf, wf, nx, ny, nz, D, band, dt, iface, bnd = state
    counts, normals, dist, vfnew = o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, iface, bnd, values=True)
    for q, L in enumerate(iface):
        i, j, k = _ijk(m, L)
        c = (i - 1 + m.nghost, j - 1 + m.nghost, k - 1 + m.nghost)
        assert (normals[q] == np.array([nx[c], ny[c], nz[c]])).all()
        assert dist[q] == D[c]
    for q, L in enumerate(bnd[::7]):
        i, j, k = _ijk(m, L)
        r, _, flags = o.sl_cell(dt, i, j, k, uf, vf, wf, nx, ny, nz, D)
        assert flags == 0
        assert vfnew[7 * q] == r


def test_counts_are_deterministic_and_additive(state):
    m, o, VF, uf, vf, wf, nx, ny, nz, D, band, dt, iface, bnd = state
    a = o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, iface, bnd)
    assert a == o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, iface, bnd)
    h1, h2 = len(iface) // 2, len(bnd) // 2
    p = o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, iface[:h1], bnd[:h2])
    q = o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, iface[h1:], bnd[h2:])
    assert {k: p[k] + q[k] for k in a} == a
    assert o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, [], []) == {"elvira": 0, "plic": 0, "sl": 0}


def test_count_sizes(state):
    """Lower bounds from the structure of the paths: ELVIRA scores 27 candidates on 27
    neighbours, each neighbour's computePLIC2VF evaluating 4 plane distances (3 products, 2
    sums, 1 difference) and at least one tet volume (24 operations) in each of 5 tets; the SL
    update projects 8 vertices by RK4 (4 velocity samples of 3 staggered trilinear blends)."""
    m, o, VF, uf, vf, wf, nx, ny, nz, D, band, dt, iface, bnd = state
    a = o.count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, iface, bnd)
    per_if = a["elvira"] / len(iface)
    assert per_if >= 27 * 27 * 5 * (4 * 6 + 24)
    assert a["plic"] / len(iface) >= 20
    assert a["sl"] / len(bnd) >= 8 * 4 * 3 * 20
