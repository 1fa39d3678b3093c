"""Python binding of the sm_103a SL-VOF library (C ABI in include/slvof.h).

This is the host-side mirror of the reference's operator interface for the path:
``computeNormal!`` (src/VF.jl:79), ``computePLIC!`` (src/VF.jl:94), ``computeBand!``
(src/VF.jl:16) and the SL section of ``transport!`` (src/Transport.jl:108-151,179-181), with
the same array arguments (OffsetArray parents, Fortran order).  Like the reference, a failed
operation raises.  There is no CPU fallback: if the CUDA library is missing or no GPU is
present, calls fail loudly.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .mesh import Mesh

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libslvof.so")

FP64 = 0
MIXED = 1
STEP_BAND = 1
STEP_MASS = 2
STEP_DEFER = 4
# status codes (SLVOF_OK, SLVOF_E_*)
OK = 0
E_ARG = -1
E_CUDA = -2
E_UNSUPPORTED = -3
E_NOMEM = -4
E_TOO_LARGE = -5
# device error bits (SLVOF_DEV_*), OR-ed into a positive status
DEV_INDEX = 1
DEV_DEPTH = 2
DEV_NAN = 4
DEV_VOLUME = 8
DEV_WAIT = 16

# (name, restype, argtypes) of every symbol declared in include/slvof.h
_P, _I, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
SYMBOLS = [
    ("slvof_create", _I, [_P, _I, _P]),
    ("slvof_destroy", _I, [_P]),
    ("slvof_last_error", _I, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    ("slvof_last_kernel_ms", _I, [_P, _P]),
    ("slvof_stage_ms", _I, [_P, _P, _I]),
    ("slvof_set_stream", _I, [_P, _P]),
    ("slvof_counters", _I, [_P, _P, _I]),
    ("slvof_upload_vf", _I, [_P, _P]),
    ("slvof_upload_velocity", _I, [_P, _P, _P, _P]),
    ("slvof_upload_band", _I, [_P, _P]),
    ("slvof_upload_plic", _I, [_P, _P, _P, _P, _P]),
    ("slvof_download_vf", _I, [_P, _P]),
    ("slvof_download_normals", _I, [_P, _P, _P, _P]),
    ("slvof_download_plic", _I, [_P, _P]),
    ("slvof_download_band", _I, [_P, _P]),
    ("slvof_vf_ghost_fill", _I, [_P]),
    ("slvof_compute_normal", _I, [_P]),
    ("slvof_compute_plic", _I, [_P]),
    ("slvof_compute_band", _I, [_P]),
    ("slvof_transport", _I, [_P, _D]),
    ("slvof_step", _I, [_P, _D, _I, _P]),
    ("slvof_mass", _I, [_P, _P]),
    ("slvof_computeNormal", _I, [_P, _P, _P, _P, _P]),
    ("slvof_computePLIC", _I, [_P, _P, _P, _P, _P, _P]),
    ("slvof_computeBand", _I, [_P, _P, _P]),
    ("slvof_transportSL", _I, [_P, _D, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("slvof_step_host", _I, [_P, _D, _I, _P, _P, _P, _P, _P]),
    ("slvof_case_vf_spheres", _I, [_P, _P, _P, _I, _I, _I]),
    ("slvof_case_deformation3d", _I, [_P, _D, _D]),
    ("slvof_mass_noalloc", _I, [_P, _P, _P, _P]),
    ("slvof_upload_cell_velocity", _I, [_P, _P, _P, _P]),
    ("slvof_download_momentum", _I, [_P, _P, _P, _P]),
    ("slvof_transport_momentum", _I, [_P, _D]),
    ("slvof_transportSL_momentum", _I, [_P, _D] + [_P] * 15),
    ("slvof_prepare", _I, [_P]),
    ("slvof_copy_vf_device", _I, [_P, _P]),
    ("slvof_load_vf_device", _I, [_P, _P]),
    ("slvof_adjoint_set_vf", _I, [_P, _P]),
    ("slvof_adjoint_get", _I, [_P, _P, _P, _P, _P]),
    ("slvof_adjoint_zero_velocity", _I, [_P]),
    ("slvof_divergence", _I, [_P, _D, _I, _P, _P, _P, _P, _P]),
    ("slvof_divergence_device", _I, [_P, _D, _I, _P, _P, _P, _P, _P]),
    ("slvof_A", _I, [_P, _D, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("slvof_A_device", _I, [_P, _D, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("slvof_computeCurvature", _I, [_P, _P, _P, _P, _P, _P]),
    ("slvof_compute_curvature_device", _I, [_P, _P]),
    ("slvof_computeProps", _I, [_P, _D, _D, _D, _D, _P, _P, _P, _P, _P, _P, _P]),
    ("slvof_adjoint_step", _I, [_P, _D]),
    ("slvof_adjoint_step_next", _I, [_P, _D, _P]),
    ("slvof_adjoint_fold", _I, [_P]),
]

_lib = None


def load_library(path: str = LIB_PATH):
    """Load the in-tree library and declare its C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"SL-VOF CUDA library not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    for name, res, args in SYMBOLS:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class DeviceError(RuntimeError):
    """A kernel raised SLVOF_DEV_* bits (index range, clip depth, NaN distance, volume, bounded
    wait)."""

    def __init__(self, bits: int, msg: str):
        super().__init__(msg)
        self.bits = bits


def _ptr(a: np.ndarray, dtype, shape=None):
    if a.dtype != dtype:
        raise TypeError(f"expected {np.dtype(dtype)}, got {a.dtype}")
    if not a.flags.f_contiguous:
        raise TypeError("arrays must be Fortran-ordered OffsetArray parents")
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a.ctypes.data


class SLVOF:
    """A device context for one mesh (slvof_create).  precision: "fp64" or "mixed"."""

    def __init__(self, mesh: Mesh, precision: str = "fp64"):
        self.L = load_library()
        self.mesh = mesh
        self.precision = {"fp64": FP64, "mixed": MIXED}[precision]
        self._desc = mesh.desc()
        h = ctypes.c_void_p()
        st = self.L.slvof_create(ctypes.byref(self._desc), self.precision, ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"slvof_create failed with status {st}")
        self.h = h

    # ---- housekeeping --------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.slvof_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(512)
        self.L.slvof_last_error(self.h, buf, 512)
        return buf.value.decode()

    def last_kernel_ms(self) -> float:
        v = ctypes.c_double()
        self.L.slvof_last_kernel_ms(self.h, ctypes.byref(v))
        return v.value

    STAGES = ("sl_classify", "sl_update", "vf_ghost", "elvira_pure", "elvira_candidates", "normal_ghost", "plic",
              "band", "mass")

    def stage_ms(self) -> dict:
        a = np.zeros(len(self.STAGES))
        self.L.slvof_stage_ms(self.h, a.ctypes.data, len(a))
        return dict(zip(self.STAGES, a.tolist()))

    COUNTERS = ("band_cells", "interface_cells", "clipped_cells", "plic_solves", "fp64_arbitrations",
                "traced_nodes", "swept_faces", "clipped_faces")

    def counters(self) -> dict:
        a = np.zeros(len(self.COUNTERS), dtype=np.int32)
        self._check(self.L.slvof_counters(self.h, a.ctypes.data, len(a)), "counters")
        return dict(zip(self.COUNTERS, a.tolist()))

    def set_stream(self, stream_handle: int | None):
        """Run on a caller-owned cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self.L.slvof_set_stream(self.h, stream_handle or None), "set_stream")

    def _check(self, st: int, what: str):
        if st < 0:
            raise RuntimeError(f"{what}: status {st}: {self.last_error()}")
        if st > 0:
            raise DeviceError(st, f"{what}: {self.last_error()}")
        return st

    # ---- transfers --------------------------------------------------------------------
    def upload_vf(self, VF):
        self._check(self.L.slvof_upload_vf(self.h, _ptr(VF, np.float64, self.mesh.vf_shape)), "upload_vf")

    def upload_velocity(self, uf, vf, wf):
        s = self.mesh.cell_shape
        self._check(self.L.slvof_upload_velocity(self.h, _ptr(uf, np.float64, s), _ptr(vf, np.float64, s),
                                                 _ptr(wf, np.float64, s)), "upload_velocity")

    def upload_band(self, band):
        self._check(self.L.slvof_upload_band(self.h, _ptr(band, np.int16, self.mesh.cell_shape)), "upload_band")

    def upload_plic(self, nx, ny, nz, D):
        s = self.mesh.cell_shape
        self._check(self.L.slvof_upload_plic(self.h, _ptr(nx, np.float64, s), _ptr(ny, np.float64, s),
                                             _ptr(nz, np.float64, s), _ptr(D, np.float64, s)), "upload_plic")

    def download_vf(self, out=None):
        out = self.mesh.vf_array() if out is None else out
        self._check(self.L.slvof_download_vf(self.h, _ptr(out, np.float64, self.mesh.vf_shape)), "download_vf")
        return out

    def download_normals(self):
        m = self.mesh
        nx, ny, nz = m.cell_array(), m.cell_array(), m.cell_array()
        self._check(self.L.slvof_download_normals(self.h, nx.ctypes.data, ny.ctypes.data, nz.ctypes.data),
                    "download_normals")
        return nx, ny, nz

    def download_plic(self):
        D = self.mesh.cell_array()
        self._check(self.L.slvof_download_plic(self.h, D.ctypes.data), "download_plic")
        return D

    def download_band(self):
        b = self.mesh.cell_array(np.int16)
        self._check(self.L.slvof_download_band(self.h, b.ctypes.data), "download_band")
        return b

    # ---- resident operations ------------------------------------------------------------
    def vf_ghost_fill(self):
        self._check(self.L.slvof_vf_ghost_fill(self.h), "vf_ghost_fill")

    def compute_normal(self):
        self._check(self.L.slvof_compute_normal(self.h), "compute_normal")

    def compute_plic(self):
        self._check(self.L.slvof_compute_plic(self.h), "compute_plic")

    def compute_band(self):
        self._check(self.L.slvof_compute_band(self.h), "compute_band")

    def transport(self, dt: float):
        self._check(self.L.slvof_transport(self.h, dt), "transport")

    def step(self, dt: float, band: bool = True, mass: bool = True):
        flags = (STEP_BAND if band else 0) | (STEP_MASS if mass else 0)
        m = ctypes.c_double(np.nan)
        self._check(self.L.slvof_step(self.h, dt, flags, ctypes.byref(m)), "step")
        return m.value if mass else None

    def mass(self) -> float:
        m = ctypes.c_double()
        self._check(self.L.slvof_mass(self.h, ctypes.byref(m)), "mass")
        return m.value

    def init_state(self, band: bool = True):
        """run_solver's start after IC! (src/NavierStokes_Parallel.jl:73-98) on device VF:
        band, normals, PLIC."""
        if band:
            self.compute_band()
        self.compute_normal()
        self.compute_plic()

    # ---- momentum of transport! -----------------------------------------------------------
    def upload_cell_velocity(self, u, v, w):
        s = self.mesh.cell_shape
        self._check(self.L.slvof_upload_cell_velocity(self.h, _ptr(u, np.float64, s), _ptr(v, np.float64, s),
                                                      _ptr(w, np.float64, s)), "upload_cell_velocity")

    def download_momentum(self):
        m = self.mesh
        us, vs, ws = m.cell_array(), m.cell_array(), m.cell_array()
        self._check(self.L.slvof_download_momentum(self.h, us.ctypes.data, vs.ctypes.data, ws.ctypes.data),
                    "download_momentum")
        return us, vs, ws

    def transport_momentum(self, dt: float):
        self._check(self.L.slvof_transport_momentum(self.h, dt), "transport_momentum")

    def transportSL_momentum(self, dt, VF, uf, vf, wf, nx, ny, nz, D, band, u, v, w):
        """SL + momentum sections of transport! (src/Transport.jl:34-181); returns us, vs, ws."""
        m, s = self.mesh, self.mesh.cell_shape
        us, vs, ws = m.cell_array(), m.cell_array(), m.cell_array()
        args = [_ptr(VF, np.float64, m.vf_shape)] + [_ptr(a, np.float64, s) for a in (uf, vf, wf, nx, ny, nz, D)]
        args += [_ptr(band, np.int16, s)] + [_ptr(a, np.float64, s) for a in (u, v, w)]
        args += [us.ctypes.data, vs.ctypes.data, ws.ctypes.data]
        self._check(self.L.slvof_transportSL_momentum(self.h, dt, *args), "transportSL_momentum")
        return us, vs, ws

    def prepare(self):
        """Ghost fill, normals, PLIC and band of the current VF: the state a step starts from."""
        self._check(self.L.slvof_prepare(self.h), "prepare")

    def copy_vf_device(self, d_ptr: int):
        """Copy the current VF to a caller's device buffer (VF-array sized, float64)."""
        self._check(self.L.slvof_copy_vf_device(self.h, d_ptr), "copy_vf_device")

    def load_vf_device(self, d_ptr: int):
        """Make a caller's device buffer the current VF (then prepare() before stepping)."""
        self._check(self.L.slvof_load_vf_device(self.h, d_ptr), "load_vf_device")

    # ---- divergence and the pressure operator (FP64, either precision) -------------------
    SCHEME = {"semi-lagrangian": 0, "finite-difference": 1}

    def divergence(self, dt, uf, vf, wf, band, scheme="semi-lagrangian"):
        """divergence! with divg_cell (src/Velocity.jl:59-122) of host face velocities."""
        s = self.mesh.cell_shape
        divg = self.mesh.cell_array()
        self._check(self.L.slvof_divergence(self.h, dt, self.SCHEME[scheme], divg.ctypes.data,
                                            _ptr(uf, np.float64, s), _ptr(vf, np.float64, s),
                                            _ptr(wf, np.float64, s), _ptr(band, np.int16, s)), "divergence")
        return divg

    def divergence_device(self, dt, d_divg, d_uf, d_vf, d_wf, d_band, scheme="semi-lagrangian"):
        self._check(self.L.slvof_divergence_device(self.h, dt, self.SCHEME[scheme], d_divg, d_uf, d_vf, d_wf,
                                                   d_band), "divergence_device")

    def A(self, dt, P, uf, vf, wf, denx, deny, denz, band, scheme="semi-lagrangian"):
        """A! (src/Pressure.jl:83-115): returns LHS; P's ghosts are filled in place."""
        s = self.mesh.cell_shape
        LHS = self.mesh.cell_array()
        self._check(self.L.slvof_A(self.h, dt, self.SCHEME[scheme], LHS.ctypes.data, _ptr(P, np.float64, s),
                                   _ptr(uf, np.float64, s), _ptr(vf, np.float64, s), _ptr(wf, np.float64, s),
                                   _ptr(denx, np.float64, s), _ptr(deny, np.float64, s),
                                   _ptr(denz, np.float64, s), _ptr(band, np.int16, s)), "A")
        return LHS

    def A_device(self, dt, d_LHS, d_P, d_uf, d_vf, d_wf, d_denx, d_deny, d_denz, d_band,
                 scheme="semi-lagrangian"):
        self._check(self.L.slvof_A_device(self.h, dt, self.SCHEME[scheme], d_LHS, d_P, d_uf, d_vf, d_wf, d_denx,
                                          d_deny, d_denz, d_band), "A_device")

    # ---- curvature and face properties (FP64, either precision) --------------------------
    def computeCurvature(self, VF, nx, ny, nz):
        """transport!'s curvature section (compute_curvature!, src/ELVIRA.jl:141-184)."""
        s = self.mesh.cell_shape
        Curve = self.mesh.cell_array()
        self._check(self.L.slvof_computeCurvature(self.h, Curve.ctypes.data, _ptr(VF, np.float64, self.mesh.vf_shape),
                                                  _ptr(nx, np.float64, s), _ptr(ny, np.float64, s),
                                                  _ptr(nz, np.float64, s)), "computeCurvature")
        return Curve

    def compute_curvature_device(self, d_curve: int):
        self._check(self.L.slvof_compute_curvature_device(self.h, d_curve), "compute_curvature_device")

    def computeProps(self, VF, rho_liq, rho_gas, mu_liq=None, mu_gas=None):
        """compute_props! (compute_dens! without viscosities): (denx, deny, denz[, viscx, viscy, viscz])."""
        m = self.mesh
        den = [m.cell_array() for _ in range(3)]
        visc = [m.cell_array() for _ in range(3)] if mu_liq is not None else None
        ptrs = [a.ctypes.data for a in den] + ([a.ctypes.data for a in visc] if visc else [None, None, None])
        self._check(self.L.slvof_computeProps(self.h, rho_liq, rho_gas, mu_liq or 0.0, mu_gas or 0.0, *ptrs,
                                              _ptr(VF, np.float64, m.vf_shape)), "computeProps")
        return tuple(den) + (tuple(visc) if visc else ())

    # ---- reverse pass ----------------------------------------------------------------------
    def adjoint_set_vf(self, gVF=None):
        """dL/dVF of the current result (VF-array shaped); None sets zero."""
        p = None if gVF is None else _ptr(gVF, np.float64, self.mesh.vf_shape)
        self._check(self.L.slvof_adjoint_set_vf(self.h, p), "adjoint_set_vf")

    def adjoint_get(self):
        """(dL/dVF, dL/duf, dL/dvf, dL/dwf) held by the context."""
        m = self.mesh
        g = m.vf_array()
        gu, gv, gw = m.cell_array(), m.cell_array(), m.cell_array()
        self._check(self.L.slvof_adjoint_get(self.h, g.ctypes.data, gu.ctypes.data, gv.ctypes.data, gw.ctypes.data),
                    "adjoint_get")
        return g, gu, gv, gw

    def adjoint_zero_velocity(self):
        self._check(self.L.slvof_adjoint_zero_velocity(self.h), "adjoint_zero_velocity")

    def adjoint_step(self, dt: float, vf_next_ptr: int | None = None):
        """Reverse of one step(dt, band=True) from the current (prepared) state.  vf_next_ptr
        may give the step's result (a device VF buffer, as copy_vf_device writes it), which a
        mixed-precision context then does not recompute."""
        if vf_next_ptr is None:
            self._check(self.L.slvof_adjoint_step(self.h, dt), "adjoint_step")
        else:
            self._check(self.L.slvof_adjoint_step_next(self.h, dt, vf_next_ptr), "adjoint_step")

    def adjoint_fold(self):
        """Fold ghost derivatives onto the interior cells they copy."""
        self._check(self.L.slvof_adjoint_fold(self.h), "adjoint_fold")

    # ---- host-buffer drop-ins (reference signatures) -------------------------------------
    def computeNormal(self, nx, ny, nz, VF):
        s = self.mesh.cell_shape
        self._check(self.L.slvof_computeNormal(self.h, _ptr(nx, np.float64, s), _ptr(ny, np.float64, s),
                                               _ptr(nz, np.float64, s), _ptr(VF, np.float64, self.mesh.vf_shape)),
                    "computeNormal")

    def computePLIC(self, D, nx, ny, nz, VF):
        s = self.mesh.cell_shape
        self._check(self.L.slvof_computePLIC(self.h, _ptr(D, np.float64, s), _ptr(nx, np.float64, s),
                                             _ptr(ny, np.float64, s), _ptr(nz, np.float64, s),
                                             _ptr(VF, np.float64, self.mesh.vf_shape)), "computePLIC")

    def computeBand(self, band, VF):
        self._check(self.L.slvof_computeBand(self.h, _ptr(band, np.int16, self.mesh.cell_shape),
                                             _ptr(VF, np.float64, self.mesh.vf_shape)), "computeBand")

    def transportSL(self, dt, VF, uf, vf, wf, nx, ny, nz, D, band):
        s = self.mesh.cell_shape
        self._check(self.L.slvof_transportSL(self.h, dt, _ptr(VF, np.float64, self.mesh.vf_shape),
                                             _ptr(uf, np.float64, s), _ptr(vf, np.float64, s),
                                             _ptr(wf, np.float64, s), _ptr(nx, np.float64, s),
                                             _ptr(ny, np.float64, s), _ptr(nz, np.float64, s),
                                             _ptr(D, np.float64, s), _ptr(band, np.int16, s)), "transportSL")

    def step_host(self, dt, uf, vf, wf, VF_out, band=True, mass=True, defer=False):
        s = self.mesh.cell_shape
        flags = (STEP_BAND if band else 0) | (STEP_MASS if mass else 0) | (STEP_DEFER if defer else 0)
        m = ctypes.c_double(np.nan)
        self._check(self.L.slvof_step_host(self.h, dt, flags, _ptr(uf, np.float64, s), _ptr(vf, np.float64, s),
                                           _ptr(wf, np.float64, s), _ptr(VF_out, np.float64, self.mesh.vf_shape),
                                           ctypes.byref(m)), "step_host")
        return m.value if mass else None

    # ---- synthetic inputs ----------------------------------------------------------------
    def case_vf_spheres(self, centres, radii, nF=20, dims=3):
        c = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(radii, dtype=np.float64).reshape(-1)
        self._check(self.L.slvof_case_vf_spheres(self.h, c.ctypes.data, r.ctypes.data, len(r), nF, dims),
                    "case_vf_spheres")

    def case_deformation3d(self, t, T=3.0):
        self._check(self.L.slvof_case_deformation3d(self.h, t, T), "case_deformation3d")
