"""Reverse step of the finite-difference scheme (flux-correction tets, FP64) on one GPU: the
workload for the profile of its reverse kernel.

    python -m ns_multiphase_gb300.profile_fd_adjoint

A 64^3 grid with pressure_scheme "finite-difference", 12 spheres (seed 11, nF = 6), the
Deformation3D field at t = 0.3 (T = 3), CFL 0.5; the reverse of one step seeded with normal
weights (seed 1) on every interior cell, run twice, with each call's wall time printed.
"""
import time

import numpy as np

from . import cases
from .mesh import Mesh
from .slvof import SLVOF


def main():
    m = Mesh(Nx=64, Ny=64, Nz=64, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5, pressure_scheme="finite-difference")
    c, r = cases.config_spheres(12, seed=11)
    g = SLVOF(m, "fp64")
    g.case_vf_spheres(c, r, nF=6)
    g.init_state()
    dt = 0.5 * m.dx / 2.0
    g.case_deformation3d(0.3, 3.0)
    gv = m.vf_array()
    m.interior(gv)[...] = np.random.default_rng(1).standard_normal((m.Nx, m.Ny, m.Nz))
    for _ in range(2):
        g.adjoint_set_vf(gv)
        g.adjoint_zero_velocity()
        t0 = time.perf_counter()
        g.adjoint_step(dt)
        print("adjoint step (fd, fp64, 64^3)", 1e3 * (time.perf_counter() - t0), "ms", flush=True)
    g.close()


if __name__ == "__main__":
    main()
