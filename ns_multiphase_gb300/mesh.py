"""Single-rank mesh and array layout of Mist.jl, restated for the C-ABI.

`create_mesh` follows src/Mesh.jl:55-108 (one MPI rank, so the local block is the whole
domain) and `init_arrays` follows the OffsetArray extents of src/Tools.jl:136-191:

* cell, face, normal, PLIC-distance and band arrays span ``imino_:imaxo_`` = N + 2*nghost
  cells per direction;
* VF spans three more ghost layers on every side (src/Tools.jl:144), N + 2*nghost + 6.

Arrays are numpy arrays in Fortran order (i fastest) holding the OffsetArray *parents*, so a
pointer to ``A.ctypes.data`` is exactly what a Julia caller passes for ``parent(A)``.
Index helpers convert the reference's Julia indices (interior 1..N) to parent indices.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from fractions import Fraction

import numpy as np

PROJECTION = {"Euler": 0, "Midpoint": 1, "RK4": 2, "Zalesak": 3}  # Zalesak: test_case, src/Tools.jl:396-399


def _axis(N: int, L: float, g: int):
    """Face coordinates x[imino_ .. imaxo_+1] and centres xm[imino_ .. imaxo_].

    ``range(0, stop=L, length=N+1)`` in Julia yields the correctly rounded values of the
    rational k*L/N (src/Mesh.jl:83); ghosts are extrapolated with the first cell width
    (src/Mesh.jl:88-100) and centres are face midpoints (src/Mesh.jl:106-108).
    """
    Lr = Fraction(repr(float(L)))
    interior = [float(Fraction(k) * Lr / N) for k in range(N + 1)]
    d = interior[1] - interior[0]
    x = np.empty(N + 2 * g + 1)
    x[g:g + N + 1] = interior
    for n in range(1, g + 1):
        x[g - n] = interior[0] - n * d
        x[g + N + n] = interior[N] + n * d
    xm = 0.5 * (x[:-1] + x[1:])
    return x, xm, d


class MeshDesc(ctypes.Structure):
    """C layout shared by ``slvof_mesh`` (include/slvof.h) and the oracle's descriptor."""

    _fields_ = [
        ("Nx", ctypes.c_int32), ("Ny", ctypes.c_int32), ("Nz", ctypes.c_int32),
        ("nghost", ctypes.c_int32), ("nband", ctypes.c_int32), ("projection", ctypes.c_int32),
        ("xper", ctypes.c_int32), ("yper", ctypes.c_int32), ("zper", ctypes.c_int32),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("Lz", ctypes.c_double),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("VFlo", ctypes.c_double), ("VFhi", ctypes.c_double),
        ("rho_liq", ctypes.c_double), ("rho_gas", ctypes.c_double),
        ("x", ctypes.POINTER(ctypes.c_double)), ("y", ctypes.POINTER(ctypes.c_double)),
        ("z", ctypes.POINTER(ctypes.c_double)), ("xm", ctypes.POINTER(ctypes.c_double)),
        ("ym", ctypes.POINTER(ctypes.c_double)), ("zm", ctypes.POINTER(ctypes.c_double)),
        ("tesselation", ctypes.c_int32), ("pressure_scheme", ctypes.c_int32),
    ]


TESSELATION = {"5_tets": 5, "6_tets": 6, "24_tets": 24}
PRESSURE_SCHEME = {"semi-lagrangian": 0, "finite-difference": 1}  # src/Parameters.jl:60


@dataclass
class Mesh:
    """The fields of ``mesh_struct`` (src/Mesh.jl:1-53) that the SL-VOF path reads, plus the
    ``parameters`` knobs it uses (src/Parameters.jl:68-77)."""

    Nx: int
    Ny: int
    Nz: int
    Lx: float
    Ly: float
    Lz: float
    CFL: float = 0.5
    xper: bool = False
    yper: bool = False
    zper: bool = False
    VFlo: float = 1e-10
    VFhi: float | None = None
    nband: int | None = None
    projection: str = "RK4"
    tesselation: str = "5_tets"
    pressure_scheme: str = "semi-lagrangian"
    rho_liq: float = 1.0
    rho_gas: float = 1.0
    nghost: int = field(init=False)
    x: np.ndarray = field(init=False, repr=False)
    y: np.ndarray = field(init=False, repr=False)
    z: np.ndarray = field(init=False, repr=False)
    xm: np.ndarray = field(init=False, repr=False)
    ym: np.ndarray = field(init=False, repr=False)
    zm: np.ndarray = field(init=False, repr=False)
    dx: float = field(init=False)
    dy: float = field(init=False)
    dz: float = field(init=False)

    def __post_init__(self):
        if self.VFhi is None:
            self.VFhi = 1.0 - self.VFlo  # src/Parameters.jl:69
        if self.nband is None:
            self.nband = int(math.ceil(self.CFL))  # src/Parameters.jl:70
        self.nghost = 3 + max(0, int(math.ceil(self.CFL) - 2))  # src/Mesh.jl:66
        g = self.nghost
        self.x, self.xm, self.dx = _axis(self.Nx, self.Lx, g)
        self.y, self.ym, self.dy = _axis(self.Ny, self.Ly, g)
        self.z, self.zm, self.dz = _axis(self.Nz, self.Lz, g)
        self._desc = None

    # ---- extents -------------------------------------------------------------------
    @property
    def N(self):
        return (self.Nx, self.Ny, self.Nz)

    @property
    def cell_shape(self):
        g = self.nghost
        return (self.Nx + 2 * g, self.Ny + 2 * g, self.Nz + 2 * g)

    @property
    def vf_shape(self):
        g = self.nghost
        return (self.Nx + 2 * g + 6, self.Ny + 2 * g + 6, self.Nz + 2 * g + 6)

    def cidx(self, i, j, k):
        """Parent index of Julia cell index (i, j, k) in a cell-extent array."""
        g = self.nghost
        return (i - 1 + g, j - 1 + g, k - 1 + g)

    def vidx(self, i, j, k):
        """Parent index of Julia cell index (i, j, k) in the VF array."""
        g = self.nghost + 3
        return (i - 1 + g, j - 1 + g, k - 1 + g)

    def interior(self, A):
        """View of the interior cells 1..N of a cell-extent or VF-extent array."""
        g = self.nghost if A.shape == self.cell_shape else self.nghost + 3
        return A[g:g + self.Nx, g:g + self.Ny, g:g + self.Nz]

    # ---- arrays (src/Tools.jl:136-191) ---------------------------------------------
    def cell_array(self, dtype=np.float64):
        return np.zeros(self.cell_shape, dtype=dtype, order="F")

    def vf_array(self):
        return np.zeros(self.vf_shape, dtype=np.float64, order="F")

    # ---- descriptor ------------------------------------------------------------------
    def desc(self) -> MeshDesc:
        """ctypes descriptor; the coordinate arrays stay owned by this Mesh."""
        if self._desc is None:
            def p(a):
                return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            self._desc = MeshDesc(
                self.Nx, self.Ny, self.Nz, self.nghost, int(self.nband),
                PROJECTION[self.projection], int(self.xper), int(self.yper), int(self.zper),
                self.Lx, self.Ly, self.Lz, self.dx, self.dy, self.dz,
                self.VFlo, self.VFhi, self.rho_liq, self.rho_gas,
                p(self.x), p(self.y), p(self.z), p(self.xm), p(self.ym), p(self.zm),
                TESSELATION[self.tesselation], PRESSURE_SCHEME[self.pressure_scheme])
        return self._desc
