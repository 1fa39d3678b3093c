"""ctypes binding of the CPU restatement (slvof_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, as the checker.  The product library never loads this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "slvof_oracle.cpp")
INC = os.path.join(os.path.dirname(HERE), "ns_multiphase_gb300", "csrc")
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the restatement with gcc: -O2, OpenMP, and no FMA contraction so that every
    expression rounds as the reference's Julia code (and as the FP64 CUDA path) does."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    deps = [SRC, os.path.join(INC, "detmath.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", "-I", INC, SRC, "-o", LIB + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        for name in ("orc_detm_cbrt", "orc_detm_acos", "orc_detm_sin", "orc_detm_cos"):
            getattr(L, name).restype = d
            getattr(L, name).argtypes = [d]
        L.orc_compute_alpha.restype = d
        L.orc_compute_alpha.argtypes = [p, d]
        L.orc_compute_dist.restype = d
        L.orc_compute_dist.argtypes = [p, i, i, i, d, d, d, d]
        L.orc_compute_plic2vf.restype = d
        L.orc_compute_plic2vf.argtypes = [p, i, i, i, d, d, d, d]
        L.orc_tet_vol.restype = d
        L.orc_tet_vol.argtypes = [p]
        L.orc_elvira.restype = i
        L.orc_elvira.argtypes = [p, p, p, p, p, i, i]
        L.orc_transport_mom.restype = i
        L.orc_transport_mom.argtypes = [p, d] + [p] * 16
        L.orc_sl_flux_vol.restype = d
        L.orc_sl_flux_vol.argtypes = [p, i, i, i, i, p, p, p, d]
        L.orc_divergence.restype = i
        L.orc_divergence.argtypes = [p, d, i, p, p, p, p, p]
        L.orc_ndual.restype = i
        L.orc_ndual.argtypes = []
        L.orc_sl_forward.restype = i
        L.orc_sl_forward.argtypes = [p, d, i, p, p, p, p, p, p, p, p, p, p, p, p, p]
        L.orc_rollout_forward.restype = i
        L.orc_rollout_forward.argtypes = [p, d, i, i, p, p, p, p, p, p, p, p, p, p, p]
        L.orc_count_ops.restype = i
        L.orc_count_ops.argtypes = [p, d, p, p, p, p, p, p, p, p, i, p, i, p, p, p]
        L.orc_curvature.restype = i
        L.orc_curvature.argtypes = [p, p, p, p, p, p]
        L.orc_props.restype = i
        L.orc_props.argtypes = [p, p, d, d, d, d, p, p, p, p, p, p]
        L.orc_A.restype = i
        L.orc_A.argtypes = [p, d, i, p, p, p, p, p, p, p, p, p, p, p, p]
        L.orc_compute_plic.restype = i
        L.orc_compute_plic.argtypes = [p, p, p, p, p, p]
        L.orc_compute_band.restype = i
        L.orc_compute_band.argtypes = [p, p, p]
        L.orc_vf_ghost_fill.restype = i
        L.orc_vf_ghost_fill.argtypes = [p, p]
        L.orc_compute_plic_slab.restype = i
        L.orc_compute_plic_slab.argtypes = [p, p, p, p, p, p, i, i]
        L.orc_compute_band_slab.restype = i
        L.orc_compute_band_slab.argtypes = [p, p, p, i, i]
        L.orc_vf_spheres.restype = i
        L.orc_vf_spheres.argtypes = [p, p, p, i, i, i, p]
        L.orc_transport.restype = i
        L.orc_transport.argtypes = [p, d, p, p, p, p, p, p, p, p, p, p, i, i]
        L.orc_sl_cell.restype = d
        L.orc_sl_cell.argtypes = [p, d, i, i, i, p, p, p, p, p, p, p, p, p]
        L.orc_project.restype = i
        L.orc_project.argtypes = [p, p, i, i, i, p, p, p, d]
        L.orc_mass.restype = d
        L.orc_mass.argtypes = [p, p]
        L.orc_step.restype = i
        L.orc_step.argtypes = [p, d, p, p, p, p, p, p, p, p, p, p, i]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.flags.f_contiguous or a.ndim <= 1, "arrays must be Fortran-ordered parents"
    return a.ctypes.data


def _m(mesh):
    return ctypes.byref(mesh.desc())


class Oracle:
    """Reference-named wrappers over one Mesh (see ns_multiphase_gb300.mesh)."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.L = lib()

    def computeDist(self, i, j, k, nx, ny, nz, VF):
        return self.L.orc_compute_dist(_m(self.mesh), i, j, k, nx, ny, nz, VF)

    def computePLIC2VF(self, i, j, k, nx, ny, nz, dist):
        return self.L.orc_compute_plic2vf(_m(self.mesh), i, j, k, nx, ny, nz, dist)

    def computeAlpha(self, m, VF):
        m = np.ascontiguousarray(m, dtype=np.float64)
        return self.L.orc_compute_alpha(m.ctypes.data, VF)

    def vf_ghost_fill(self, VF):
        self.L.orc_vf_ghost_fill(_m(self.mesh), _p(VF))

    def vf_spheres(self, centres, radii, nF=20, dims=3):
        """VF of a union of spheres by VFsphere's rule (src/Tools.jl:907-922), ghosts filled:
        the CPU baseline's copy of the workload the GPU library generates on the device."""
        c = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(radii, dtype=np.float64).reshape(-1)
        VF = self.mesh.vf_array()
        self.L.orc_vf_spheres(_m(self.mesh), c.ctypes.data, r.ctypes.data, len(r), nF, dims, _p(VF))
        self.vf_ghost_fill(VF)
        return VF

    def computePLIC_slab(self, nx, ny, nz, VF, D, klo, khi):
        """computePLIC!'s per-cell work on the cells k in [klo, khi] (CPU baseline sample)."""
        self.L.orc_compute_plic_slab(_m(self.mesh), _p(D), _p(nx), _p(ny), _p(nz), _p(VF), klo, khi)
        return D

    def computeBand_slab(self, VF, band, klo, khi):
        """computeBand!'s per-cell passes on the cells k in [klo, khi] (CPU baseline sample)."""
        self.L.orc_compute_band_slab(_m(self.mesh), _p(band), _p(VF), klo, khi)
        return band

    def ELVIRA(self, VF, nx=None, ny=None, nz=None, klo=1, khi=0):
        m = self.mesh
        nx = m.cell_array() if nx is None else nx
        ny = m.cell_array() if ny is None else ny
        nz = m.cell_array() if nz is None else nz
        flags = self.L.orc_elvira(_m(m), _p(VF), _p(nx), _p(ny), _p(nz), klo, khi)
        return nx, ny, nz, flags

    def computePLIC(self, nx, ny, nz, VF, D=None):
        D = self.mesh.cell_array() if D is None else D
        self.L.orc_compute_plic(_m(self.mesh), _p(D), _p(nx), _p(ny), _p(nz), _p(VF))
        return D

    def computeBand(self, VF, band=None):
        band = self.mesh.cell_array(np.int16) if band is None else band
        self.L.orc_compute_band(_m(self.mesh), _p(band), _p(VF))
        return band

    def transport(self, dt, VF, uf, vf, wf, nx, ny, nz, D, band, klo=1, khi=0, VFnew=None):
        """SL cell loop + VF copy + ghost fill; VF updated in place (sample mode when
        klo <= khi: only VFnew is written)."""
        VFnew = self.mesh.vf_array() if VFnew is None else VFnew
        flags = self.L.orc_transport(_m(self.mesh), dt, _p(VF), _p(VFnew), _p(uf), _p(vf), _p(wf),
                                     _p(nx), _p(ny), _p(nz), _p(D), _p(band), klo, khi)
        return flags, VFnew

    def transport_mom(self, dt, VF, uf, vf, wf, nx, ny, nz, D, band, u, v, w):
        """transport!'s SL loop with its momentum (pressure_scheme "semi-lagrangian"): VF is
        updated in place; returns (flags, us, vs, ws)."""
        m = self.mesh
        VFnew = m.vf_array()
        us, vs, ws = m.cell_array(), m.cell_array(), m.cell_array()
        flags = self.L.orc_transport_mom(_m(m), dt, _p(VF), _p(VFnew), _p(uf), _p(vf), _p(wf), _p(nx), _p(ny),
                                         _p(nz), _p(D), _p(band), _p(u), _p(v), _p(w), _p(us), _p(vs), _p(ws))
        return flags, us, vs, ws

    def divergence(self, dt, uf, vf, wf, band, scheme=0):
        """divergence! (src/Velocity.jl:59-68) with divg_cell; scheme 0 "semi-lagrangian",
        1 "finite-difference".  Returns divg (cell array, 0 outside the interior)."""
        m = self.mesh
        divg = m.cell_array()
        self.L.orc_divergence(_m(m), dt, scheme, _p(divg), _p(uf), _p(vf), _p(wf), _p(band))
        return divg

    def A(self, dt, P, uf, vf, wf, denx, deny, denz, band, scheme=0):
        """A! (src/Pressure.jl:83-115): P's ghosts are filled in place; returns (LHS, gradx,
        grady, gradz)."""
        m = self.mesh
        LHS, gx, gy, gz = m.cell_array(), m.cell_array(), m.cell_array(), m.cell_array()
        self.L.orc_A(_m(m), dt, scheme, _p(LHS), _p(P), _p(uf), _p(vf), _p(wf), _p(denx), _p(deny), _p(denz),
                     _p(band), _p(gx), _p(gy), _p(gz))
        return LHS, gx, gy, gz

    def sl_forward(self, dt, cells, uf, vf, wf, seeds, nx, ny, nz, D):
        """Forward-mode derivatives of the SL update (Dual numbers through the restatement):
        cells is a list of (i, j, k); seeds a list of up to ndual() (array 0/1/2, parent index)
        face entries.  Returns (VFnew per cell, d VFnew / d seed, shape (cells, seeds))."""
        m = self.mesh
        K = self.L.orc_ndual()
        assert len(seeds) <= K
        slots = [np.full(m.cell_shape, -1, dtype=np.int32, order="F") for _ in range(3)]
        for s, (a, idx) in enumerate(seeds):
            slots[a][idx] = s
        cl = np.ascontiguousarray(np.asarray(cells, dtype=np.int32).reshape(-1, 3))
        out = np.zeros(len(cl))
        grad = np.zeros((len(cl), K))
        f = self.L.orc_sl_forward(_m(m), dt, len(cl), cl.ctypes.data, _p(uf), _p(vf), _p(wf), *[_p(x) for x in slots],
                                  _p(nx), _p(ny), _p(nz), _p(D), out.ctypes.data, grad.ctypes.data)
        if f:
            raise RuntimeError(f"restatement flags {f}")
        return out, grad[:, :len(seeds)]

    def ndual(self):
        return self.L.orc_ndual()

    def rollout_forward(self, dt, steps, VF0, uf, vf, wf, face_seeds, vf_seeds, w):
        """Forward-mode derivatives of L = sum(w * VF_T) over a `steps`-step rollout from VF0
        (initial state and every step's normals, PLIC and band included).  uf, vf, wf: arrays
        (frozen velocities) or lists of per-step arrays.  face_seeds: (array 0/1/2, parent index)
        face entries, the same entry of every step's velocities; vf_seeds: parent indices of VF0
        entries; at most ndual() together.  Returns (L, dL per seed)."""
        m = self.mesh
        per_step = isinstance(uf, (list, tuple))
        nv = len(uf) if per_step else 1
        pack = lambda a: np.concatenate([np.asfortranarray(x).ravel(order="F") for x in a]) if per_step else a
        uf, vf, wf = pack(uf), pack(vf), pack(wf)
        K = self.L.orc_ndual()
        assert len(face_seeds) + len(vf_seeds) <= K
        slots = [np.full(m.cell_shape, -1, dtype=np.int32, order="F") for _ in range(3)]
        for s, (a, idx) in enumerate(face_seeds):
            slots[a][idx] = s
        svf = np.full(m.vf_shape, -1, dtype=np.int32, order="F")
        for s, idx in enumerate(vf_seeds):
            svf[idx] = len(face_seeds) + s
        wv = np.ascontiguousarray(np.asarray(w, dtype=np.float64).ravel(order="F"))
        Lv = ctypes.c_double()
        dL = np.zeros(K)
        f = self.L.orc_rollout_forward(_m(m), dt, steps, nv, _p(VF0), _p(uf), _p(vf), _p(wf),
                                       *[_p(x) for x in slots], _p(svf), wv.ctypes.data, ctypes.byref(Lv),
                                       dL.ctypes.data)
        if f:
            raise RuntimeError(f"restatement flags {f}")
        return Lv.value, dL[:len(face_seeds) + len(vf_seeds)]

    def count_ops(self, dt, VF, uf, vf, wf, nx, ny, nz, D, if_cells, band_cells, values=False):
        """Algorithmic operation counts of a step's per-cell parts (each +, -, *, / and each
        sqrt, cbrt, acos, sin, cos of the restatement), summed over the given interior cells
        (linear indices (i-1) + Nx*((j-1) + Ny*(k-1))), on one thread.  Returns
        {"elvira": .., "plic": .., "sl": ..} (interface cells, interface cells, band cells),
        and with values=True also the values the counted paths computed (normals (n, 3), D,
        VFnew), which equal the double paths' bit for bit."""
        m = self.mesh
        ic = np.ascontiguousarray(np.asarray(if_cells, dtype=np.int32).ravel())
        bc = np.ascontiguousarray(np.asarray(band_cells, dtype=np.int32).ravel())
        out = (ctypes.c_ulonglong * 3)()
        vals = np.zeros(4 * len(ic) + len(bc)) if values else None
        f = self.L.orc_count_ops(_m(m), dt, _p(VF), _p(nx), _p(ny), _p(nz), _p(D), _p(uf), _p(vf), _p(wf), len(ic),
                                 ic.ctypes.data, len(bc), bc.ctypes.data, out,
                                 vals.ctypes.data if values else None)
        if f:
            raise RuntimeError(f"restatement flags {f}")
        counts = {"elvira": int(out[0]), "plic": int(out[1]), "sl": int(out[2])}
        if not values:
            return counts
        n = len(ic)
        return counts, vals[:3 * n].reshape(n, 3), vals[3 * n:4 * n], vals[4 * n:]

    def curvature(self, VF, nx, ny, nz):
        """transport!'s curvature section (src/Transport.jl:187-191, compute_curvature!)."""
        Curve = self.mesh.cell_array()
        self.L.orc_curvature(_m(self.mesh), _p(Curve), _p(VF), _p(nx), _p(ny), _p(nz))
        return Curve

    def props(self, VF, rho_liq, rho_gas, mu_liq=None, mu_gas=None):
        """compute_props! (or compute_dens! without viscosities): (denx, deny, denz[, viscx,
        viscy, viscz])."""
        m = self.mesh
        den = [m.cell_array() for _ in range(3)]
        visc = [m.cell_array() for _ in range(3)] if mu_liq is not None else [None] * 3
        self.L.orc_props(_m(m), _p(VF), rho_liq, rho_gas, mu_liq or 0.0, mu_gas or 0.0,
                         *[_p(a) for a in den], *[_p(a) if a is not None else None for a in visc])
        return tuple(den) + (tuple(visc) if mu_liq is not None else ())

    def sl_flux_vol(self, direction, i, j, k, uf, vf, wf, dt):
        """SLfluxVol (src/VFgeom.jl:428-509); direction 0, 1, 2 for x, y, z."""
        return self.L.orc_sl_flux_vol(_m(self.mesh), direction, i, j, k, _p(uf), _p(vf), _p(wf), dt)

    def sl_cell(self, dt, i, j, k, uf, vf, wf, nx, ny, nz, D):
        vol = ctypes.c_double()
        flags = ctypes.c_int()
        r = self.L.orc_sl_cell(_m(self.mesh), dt, i, j, k, _p(uf), _p(vf), _p(wf), _p(nx), _p(ny),
                               _p(nz), _p(D), ctypes.addressof(vol), ctypes.addressof(flags))
        return r, vol.value, flags.value

    def project(self, pt, i, j, k, uf, vf, wf, dt):
        p = np.ascontiguousarray(pt, dtype=np.float64).copy()
        self.L.orc_project(_m(self.mesh), p.ctypes.data, i, j, k, _p(uf), _p(vf), _p(wf), dt)
        return p

    def mass(self, VF):
        return self.L.orc_mass(_m(self.mesh), _p(VF))

    def step(self, dt, VF, uf, vf, wf, nx, ny, nz, D, band, do_band=True):
        VFnew = self.mesh.vf_array()
        return self.L.orc_step(_m(self.mesh), dt, _p(VF), _p(VFnew), _p(uf), _p(vf), _p(wf),
                               _p(nx), _p(ny), _p(nz), _p(D), _p(band), int(do_band))

    def init_state(self, VF, do_band=True):
        """run_solver's start (src/NavierStokes_Parallel.jl:73-98): Neumann!+VF borders,
        computeBand!, computeNormal!, computePLIC!.  VF is modified in place."""
        self.vf_ghost_fill(VF)
        band = self.computeBand(VF) if do_band else self.mesh.cell_array(np.int16)
        nx, ny, nz, flags = self.ELVIRA(VF)
        D = self.computePLIC(nx, ny, nz, VF)
        return band, nx, ny, nz, D
