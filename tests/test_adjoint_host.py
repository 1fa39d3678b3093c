"""The adjoint's per-cell derivatives, checked on the CPU against central finite differences.

tests/adj_harness.cpp compiles the adjoint routines the GPU kernels run (adj64.cuh) for the
host.  Each derivative here is compared with central differences (h = 1e-6) of the CPU
restatement of the reference function it differentiates: the SL update of one cell
(src/Transport.jl:111-148) with respect to face velocities and donor planes, computeDist
(src/VF.jl:109-156) with respect to the normal and VF, and the ELVIRA candidate normal
(src/ELVIRA.jl:62-115) with respect to the VF block.  Tolerance: 1e-6 relative to the largest
derivative of the set, the bar the adjoint has to meet against finite differences.
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
H = 1e-6
RTOL = 1e-6


@pytest.fixture(scope="module")
def hlib():
    src = os.path.join(HERE, "adj_harness.cpp")
    out = os.path.join(HERE, "_build", "libadjh.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    deps = [src] + [os.path.join(ROOT, "ns_multiphase_gb300", "csrc", f) for f in ("adj64.cuh", "adj32.cuh", "mesh_view.h")]
    if not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out) for d in deps):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                        "-I", ROOT, src, "-o", out + ".tmp"], check=True)
        os.replace(out + ".tmp", out)
    L = ctypes.CDLL(out)
    d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.adjh_sl_cell.restype = d
    L.adjh_sl_cell.argtypes = [p, d, i, i, i] + [p] * 7 + [d] + [p] * 8
    L.adjh_dist_partials.restype = i
    L.adjh_dist_partials.argtypes = [p, i, i, i, d, d, d, d, p]
    L.adjh_candidate.restype = None
    L.adjh_candidate.argtypes = [p, p, i, i, i, i, p]
    L.adjh_elvira_reverse.restype = None
    L.adjh_elvira_reverse.argtypes = [p, p, p, i, i, i, i, p]
    L.adjh_preimage.restype = i
    L.adjh_preimage.argtypes = [i, i, i, i, i, i, i, p]
    L.adjh_preimage_vertices.restype = None
    L.adjh_preimage_vertices.argtypes = [p, d, i, i, i, p, p, p, p]
    L.adjh_sl_vertices_pl.restype = d
    L.adjh_sl_vertices_pl.argtypes = [p, i, i, i, p, p, p, p, p, d, p, p, p]
    L.adjh_sd_vertices.restype = None
    L.adjh_sd_vertices.argtypes = [p, i, i, i, i, p, p, p, p, p, d, d, p, p]
    L.adjh_sd_dist.restype = i
    L.adjh_sd_dist.argtypes = [p, i, i, i, i, d, d, d, d, p]
    return L


def ptr(a):
    return a.ctypes.data


def sphere_state(N=10, centre=(0.45, 0.52, 0.55), r=0.27, t=0.4, tess="5_tets", scheme="semi-lagrangian"):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, tesselation=tess, pressure_scheme=scheme)
    o = Oracle(m)
    VF = cases.vf_spheres(m, np.array([centre]), np.array([r]), nF=8)
    band, nx, ny, nz, D = o.init_state(VF)
    uf, vf, wf = cases.deformation3d_faces(m, t, 3.0)
    # seeded face noise, as the adjoint configurations use: the deformation field alone has
    # grid nodes that do not move, whose pre-image vertices sit exactly on mesh planes, where
    # the clipped volume is only once differentiable and central differences lose accuracy
    rng = np.random.default_rng(20261203)
    for f in (uf, vf, wf):
        f += 0.02 * rng.standard_normal(f.shape)
    dt = 0.5 * m.dx / 2.0
    return m, o, VF, band, nx, ny, nz, D, uf, vf, wf, dt


@pytest.fixture(scope="module", params=["5_tets", "6_tets", "24_tets"])
def state(request):
    return sphere_state(tess=request.param)


def interface_preimage_cells(m, o, st, count):
    """Band cells whose SL update gives a fraction strictly inside (0, 1)."""
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = st
    out = []
    for k in range(2, m.Nz):
        for j in range(2, m.Ny):
            for i in range(2, m.Nx):
                if abs(int(band[m.cidx(i, j, k)])) > m.nband:
                    continue
                r, vol, flags = o.sl_cell(dt, i, j, k, uf, vf, wf, nx, ny, nz, D)
                if 1e-3 < r < 1 - 1e-3:
                    out.append((i, j, k))
    rng = np.random.default_rng(5)
    sel = rng.choice(len(out), size=min(count, len(out)), replace=False)
    return [out[s] for s in sorted(sel)]


def harness_grads(hlib, m, st, cell, g=1.0):
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = st
    grads = [m.cell_array() for _ in range(7)]
    err = ctypes.c_int()
    desc = m.desc()
    r = hlib.adjh_sl_cell(ctypes.byref(desc), dt, *cell, ptr(uf), ptr(vf), ptr(wf), ptr(nx), ptr(ny), ptr(nz),
                          ptr(D), g, *[ptr(a) for a in grads], ctypes.addressof(err))
    return r, grads, err.value


def test_sl_cell_forward_matches_restatement(hlib, state):
    """Same pre-image and clip tree as the restatement; one-sided sub-trees are single leaves
    in the reverse pass, so the value agrees to rounding."""
    m, o = state[0], state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state
    cells = interface_preimage_cells(m, o, state, 12)
    assert len(cells) >= 8
    for c in cells:
        r, _, err = harness_grads(hlib, m, state, c)
        ref, _, flags = o.sl_cell(dt, *c, uf, vf, wf, nx, ny, nz, D)
        assert err == 0 and flags == 0
        assert abs(r - ref) <= 1e-14, (c, r, ref)


def fd_sl(o, st, cell, arr, idx):
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = st
    x0 = arr[idx]
    arr[idx] = x0 + H
    rp = o.sl_cell(dt, *cell, uf, vf, wf, nx, ny, nz, D)[0]
    arr[idx] = x0 - H
    rm = o.sl_cell(dt, *cell, uf, vf, wf, nx, ny, nz, D)[0]
    arr[idx] = x0
    return (rp - rm) / (2 * H)


def check_entries(o, st, cell, pairs):
    """pairs: (array, gradient array); compare the largest entries and a random sample."""
    rng = np.random.default_rng(11)
    worst = 0.0
    scale = max(float(np.max(np.abs(g))) for _, g in pairs)
    assert scale > 0.0
    n = 0
    for arr, g in pairs:
        nz_idx = np.argwhere(np.abs(g) > 0)
        if len(nz_idx) == 0:
            continue
        order = np.argsort(-np.abs(g[tuple(nz_idx.T)]))
        pick = list(order[:4]) + list(rng.choice(len(nz_idx), size=min(3, len(nz_idx)), replace=False))
        for p in pick:
            idx = tuple(nz_idx[p])
            fd = fd_sl(o, st, cell, arr, idx)
            worst = max(worst, abs(fd - g[idx]) / scale)
            n += 1
    return worst, n


def test_sl_cell_velocity_gradient_matches_finite_differences(hlib, state):
    m, o = state[0], state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state
    cells = interface_preimage_cells(m, o, state, 6)
    for c in cells:
        _, grads, err = harness_grads(hlib, m, state, c)
        assert err == 0
        worst, n = check_entries(o, state, c, [(uf, grads[0]), (vf, grads[1]), (wf, grads[2])])
        assert n >= 9
        assert worst <= RTOL, (c, worst)


def test_sl_cell_plane_gradient_matches_finite_differences(hlib, state):
    m, o = state[0], state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state
    cells = interface_preimage_cells(m, o, state, 6)
    for c in cells:
        _, grads, err = harness_grads(hlib, m, state, c)
        assert err == 0
        worst, n = check_entries(o, state, c, [(nx, grads[3]), (ny, grads[4]), (nz, grads[5]), (D, grads[6])])
        assert n >= 4
        assert worst <= RTOL, (c, worst)


@pytest.fixture(scope="module")
def fd_state():
    return sphere_state(scheme="finite-difference")


def test_sl_cell_with_correction_tets_forward_matches_restatement(hlib, fd_state):
    """pressure_scheme "finite-difference": the cell's tets and its twelve flux-correction tets
    (add_correction_tets, src/VFgeom.jl:514-664) give the restatement's VFnew to rounding."""
    m, o = fd_state[0], fd_state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = fd_state
    cells = interface_preimage_cells(m, o, fd_state, 12)
    assert len(cells) >= 8
    for c in cells:
        r, _, err = harness_grads(hlib, m, fd_state, c)
        ref, _, flags = o.sl_cell(dt, *c, uf, vf, wf, nx, ny, nz, D)
        assert err == 0 and flags == 0
        assert abs(r - ref) <= 1e-14, (c, r, ref)


def test_sl_cell_with_correction_tets_gradients_match_finite_differences(hlib, fd_state):
    """The reverse through the correction tets' apex solve, the flux volume and the face
    velocity of the target volume, against central differences of the restatement."""
    m, o = fd_state[0], fd_state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = fd_state
    cells = interface_preimage_cells(m, o, fd_state, 6)
    for c in cells:
        _, grads, err = harness_grads(hlib, m, fd_state, c)
        assert err == 0
        worst, n = check_entries(o, fd_state, c, [(uf, grads[0]), (vf, grads[1]), (wf, grads[2])])
        assert n >= 9
        assert worst <= RTOL, (c, worst)
        worst, n = check_entries(o, fd_state, c, [(nx, grads[3]), (ny, grads[4]), (nz, grads[5]), (D, grads[6])])
        assert n >= 4
        assert worst <= RTOL, (c, worst)


def test_sl_cell_gradient_is_linear_in_the_seed(hlib, state):
    m, o = state[0], state[1]
    c = interface_preimage_cells(m, o, state, 1)[0]
    _, g1, _ = harness_grads(hlib, m, state, c, 1.0)
    _, g3, _ = harness_grads(hlib, m, state, c, -3.0)
    for a, b in zip(g1, g3):
        assert np.allclose(-3.0 * a, b, rtol=1e-13, atol=1e-300)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_dist_partials_match_finite_differences(hlib, seed):
    # non-cubic cells, as in the reference's round-trip test (test/runtests.jl:32-45)
    m = Mesh(Nx=10, Ny=10, Nz=1, Lx=3.0, Ly=1.0, Lz=1.0)
    o = Oracle(m)
    rng = np.random.default_rng(seed)
    desc = m.desc()
    checked = 0
    for _ in range(40):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        VFv = rng.uniform(0.02, 0.98)
        i, j = int(rng.integers(1, 11)), int(rng.integers(1, 11))
        D = o.computeDist(i, j, 1, *n, VFv)
        out = np.zeros(4)
        ok = hlib.adjh_dist_partials(ctypes.byref(desc), i, j, 1, *n, D, ptr(out))
        assert ok == 1
        fd = []
        for q in range(3):
            e = np.zeros(3)
            e[q] = H
            fd.append((o.computeDist(i, j, 1, *(n + e), VFv) - o.computeDist(i, j, 1, *(n - e), VFv)) / (2 * H))
        fd.append((o.computeDist(i, j, 1, *n, VFv + H) - o.computeDist(i, j, 1, *n, VFv - H)) / (2 * H))
        fd = np.array(fd)
        scale = np.max(np.abs(fd))
        assert np.max(np.abs(fd - out)) <= 1e-6 * scale, (n, VFv, fd, out)
        checked += 1
    assert checked == 40


def test_elvira_candidates_reproduce_the_chosen_normal(hlib, state):
    """Every interface normal of the restatement is one of the harness's candidates, normalised
    as check_normal! does, bit for bit."""
    m, o = state[0], state[1]
    VF, nx, ny, nz = state[2], state[4], state[5], state[6]
    desc = m.desc()
    found = 0
    for k in range(1, m.Nz + 1):
        for j in range(1, m.Ny + 1):
            for i in range(1, m.Nx + 1):
                v = VF[m.vidx(i, j, k)]
                if not (m.VFlo <= v <= m.VFhi):
                    continue
                target = np.array([nx[m.cidx(i, j, k)], ny[m.cidx(i, j, k)], nz[m.cidx(i, j, k)]])
                hit = False
                for lane in range(27):
                    c = np.zeros(3)
                    hlib.adjh_candidate(ctypes.byref(desc), ptr(VF), i, j, k, lane, ptr(c))
                    norm = np.sqrt((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2])
                    if np.array_equal(c / norm, target):
                        hit = True
                        break
                assert hit, (i, j, k)
                found += 1
    assert found > 50


def test_elvira_reverse_matches_finite_differences(hlib, state):
    m = state[0]
    VF = state[2].copy(order="F")
    desc = m.desc()
    rng = np.random.default_rng(3)

    def normal(lane, i, j, k):
        c = np.zeros(3)
        hlib.adjh_candidate(ctypes.byref(desc), ptr(VF), i, j, k, lane, ptr(c))
        return c / np.sqrt((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2])

    checked = 0
    for _ in range(30):
        i, j, k = (int(x) for x in rng.integers(2, m.Nx, size=3))
        lane = int(rng.integers(0, 27))
        gn = rng.normal(size=3)
        gVF = m.vf_array()
        hlib.adjh_elvira_reverse(ctypes.byref(desc), ptr(VF), ptr(gVF), i, j, k, lane, ptr(gn))
        # the family's normal direction: its +-1 component compares the two neighbours along it,
        # a discrete choice that a step of h flips when they are equal (both 0 or both 1)
        fams = [f for f, on in enumerate((m.Nz > 1, m.Ny > 1, m.Nx > 1)) if on]
        tn = (2, 1, 0)[fams[lane // 9]]
        for dk in (-1, 0, 1):
            for dj in (-1, 0, 1):
                for di in (-1, 0, 1):
                    off = (di, dj, dk)
                    if sum(abs(x) for x in off) == 1 and off[tn] != 0:
                        up = [0, 0, 0]
                        up[tn] = 1
                        if VF[m.vidx(i + up[0], j + up[1], k + up[2])] == VF[m.vidx(i - up[0], j - up[1], k - up[2])]:
                            continue
                    idx = m.vidx(i + di, j + dj, k + dk)
                    x0 = VF[idx]
                    VF[idx] = x0 + H
                    fp = normal(lane, i, j, k)
                    VF[idx] = x0 - H
                    fm = normal(lane, i, j, k)
                    VF[idx] = x0
                    fd = float(np.dot(gn, (fp - fm) / (2 * H)))
                    assert abs(fd - gVF[idx]) <= 1e-6 * max(1.0, abs(fd)), (i, j, k, lane, di, dj, dk)
                    checked += 1
    assert checked >= 30 * 25


@pytest.mark.parametrize("per,neu", [(1, 1), (0, 1), (1, 0), (0, 0)])
def test_ghost_preimage_inverts_the_source_map(hlib, per, neu):
    N, g = 7, 3
    lo, hi = 1 - g - 3, N + g + 3
    src_of = {}
    for p in range(lo, hi + 1):
        q = p
        if per and 1 - g <= q <= 0:
            q += N
        if per and N + 1 <= q <= N + g:
            q -= N
        if neu and q == N + 1:
            q = N
        if neu and q == 0:
            q = 1
        src_of[p] = q
    buf = np.zeros(64, dtype=np.int32)
    for q in range(lo, hi + 1):
        n = hlib.adjh_preimage(q, N, g, per, neu, lo, hi, ptr(buf))
        got = sorted(buf[:n].tolist())
        want = sorted(p for p in range(lo, hi + 1) if src_of[p] == q)
        assert got == want, (q, got, want)


@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 1e-5)])
def test_boundary_form_matches_clip_tree_reverse(hlib, state, prec, tol):
    """The mixed path's reverse takes the clipped volume's derivatives from the pre-image's
    boundary (adj32.cuh): liquid moments of its boundary triangles for the vertices, the PLIC
    polygons inside each tet and donor cell for the planes.  Against the FP64 reverse of the
    cutTet tree on the same pre-images: to rounding in double, to FP32 rounding in float."""
    m, o = state[0], state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state
    desc = m.desc()
    nc = int(np.prod(m.cell_shape))
    cells = interface_preimage_cells(m, o, state, 12)
    assert len(cells) >= 8
    for c in cells:
        vt = np.zeros(24)
        hlib.adjh_preimage_vertices(ctypes.byref(desc), dt, *c, ptr(uf), ptr(vf), ptr(wf), ptr(vt))
        g0, p0 = np.zeros(24), np.zeros(4 * nc)
        err = ctypes.c_int()
        r = hlib.adjh_sl_vertices_pl(ctypes.byref(desc), *c, ptr(vt), ptr(nx), ptr(ny), ptr(nz), ptr(D), 1.0,
                                     ptr(g0), ptr(p0), ctypes.addressof(err))
        assert err.value == 0
        g1, p1 = np.zeros(24), np.zeros(4 * nc)
        hlib.adjh_sd_vertices(ctypes.byref(desc), prec, *c, ptr(vt), ptr(nx), ptr(ny), ptr(nz), ptr(D), r, 1.0,
                              ptr(g1), ptr(p1))
        assert np.max(np.abs(g1 - g0)) <= tol * np.max(np.abs(g0)), c
        assert np.max(np.abs(p1 - p0)) <= tol * np.max(np.abs(p0)), c


@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 1e-5)])
def test_plane_polygon_gives_computeDist_partials(hlib, state, prec, tol):
    """computeDist's derivatives from the plane's polygon in the cell (dD/dVF = |grad d| / A,
    dD/dn = centroid) against the implicit derivative of the five-tet cut-cell fraction."""
    m, o = state[0], state[1]
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = state
    desc = m.desc()
    n = 0
    for k in range(1, m.Nz + 1):
        for j in range(1, m.Ny + 1):
            for i in range(1, m.Nx + 1):
                t = m.cidx(i, j, k)
                v = VF[m.vidx(i, j, k)]
                if not (m.VFlo <= v <= m.VFhi) or v < 1e-3 or v > 1 - 1e-3:
                    continue
                a, b = np.zeros(4), np.zeros(4)
                if not hlib.adjh_dist_partials(ctypes.byref(desc), i, j, k, nx[t], ny[t], nz[t], D[t], ptr(a)):
                    continue
                assert hlib.adjh_sd_dist(ctypes.byref(desc), prec, i, j, k, nx[t], ny[t], nz[t], D[t], ptr(b))
                assert np.all(np.abs(b - a) <= tol * np.maximum(np.abs(a), 1.0)), ((i, j, k), a, b)
                n += 1
    assert n >= 20


def forward_mode_grads(o, st, cells, weights, entries):
    """dL/d(face value) for L = sum_c w_c VFnew_c, by forward-mode Dual numbers through the
    restatement, entries (array 0/1/2, parent index) in chunks of ndual()."""
    _, _, VF, band, nx, ny, nz, D, uf, vf, wf, dt = st
    K = o.ndual()
    out = np.zeros(len(entries))
    for c0 in range(0, len(entries), K):
        chunk = entries[c0:c0 + K]
        _, g = o.sl_forward(dt, cells, uf, vf, wf, chunk, nx, ny, nz, D)
        out[c0:c0 + len(chunk)] = weights @ g
    return out


def test_forward_mode_matches_reverse_pass(hlib, state):
    """The hand-written reverse of one cell's SL update against forward-mode derivatives of the
    restatement (Dual numbers, the CPU analogue of a ForwardDiff.jl gradient): every face value
    the cell's update reads, to rounding."""
    m, o = state[0], state[1]
    cells = interface_preimage_cells(m, o, state, 8)
    assert len(cells) >= 6
    worst = 0.0
    for c in cells:
        _, grads, err = harness_grads(hlib, m, state, c)
        assert err == 0
        entries = [(a, tuple(int(x) for x in idx)) for a in range(3) for idx in np.argwhere(grads[a] != 0.0)]
        assert len(entries) > 10
        fwd = forward_mode_grads(o, state, [c], np.ones(1), entries)
        rev = np.array([grads[a][idx] for a, idx in entries])
        worst = max(worst, float(np.max(np.abs(fwd - rev)) / np.max(np.abs(rev))))
    assert worst <= 1e-11, worst
