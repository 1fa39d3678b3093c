"""The two FP64 transport configurations at their own sizes, on the GPU path and on the CPU
restatement, with the reference's shape-error measure.

    python tests/config_runs.py 2d [--steps 1024]   # 64^2 single vortex to t = T
    python tests/config_runs.py 3d [--steps 8]      # 128^3 sphere deformation
    python tests/config_runs.py drift [--steps 64]  # 256^3 mass: FP64, FP64 on FP32 velocities, mixed

2d: [0,1]^2, 64x64x1 (z periodic), circle r = 0.15 at (0.5, 0.75) by 10x10 sub-sampling,
    single-vortex face velocities sampled at the faces (period T = 8) at t_n + dt/2,
    dt = 0.5 dx (max |u| = 1): 1024 steps reach t = T, where the exact solution is the initial
    circle again.
3d: 128^3 unit cube, sphere r = 0.15 at (0.35, 0.35, 0.35) by 20^3 sub-sampling,
    Deformation3D (T = 3) at t_n + dt/2, dt = 0.5 dx / 2.

Each run reports the largest per-cell difference between the GPU's and the restatement's VF
(the FP64 path's bar is 1e-12), the relative difference of their total volumes (1e-13), the
relative volume change over the run, and the shape error sum|VF_T - VF_0| / N_cells
(test/deformation_error.jl:22).
"""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import argparse
import json
import time

import numpy as np

from ns_multiphase_gb300 import cases
from ns_multiphase_gb300.mesh import Mesh


def config2d():
    m = Mesh(Nx=64, Ny=64, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / 64, CFL=0.5, zper=True)
    VF0 = cases.vf_spheres(m, np.array([[0.5, 0.75, 0.0]]), np.array([0.15]), nF=10, dims=2)
    dt = 0.5 * m.dx
    vel = lambda n: cases.deformation2d_faces(m, (n + 0.5) * dt, 8.0)
    return m, VF0, dt, vel, 1024


def config3d():
    m = Mesh(Nx=128, Ny=128, Nz=128, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    VF0 = cases.vf_spheres(m, np.array([[0.35, 0.35, 0.35]]), np.array([0.15]), nF=20)
    dt = 0.5 * m.dx / 2.0
    vel = lambda n: cases.deformation3d_faces(m, (n + 0.5) * dt, 3.0)
    return m, VF0, dt, vel, 1536


def run(which: str, steps: int | None = None, precision: str = "fp64", cpu: bool = True):
    from ns_multiphase_gb300.slvof import SLVOF
    m, VF0, dt, vel, full = config2d() if which == "2d" else config3d()
    steps = full if steps is None else steps
    g = SLVOF(m, precision)
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    g.init_state()
    M0 = g.mass()
    t0 = time.perf_counter()
    for n in range(steps):
        g.upload_velocity(*vel(n))
        mass = g.step(dt)
    gpu_s = time.perf_counter() - t0
    VFg = g.download_vf()
    g.close()
    out = {"config": which, "grid": list(m.N), "steps": steps, "t": steps * dt, "precision": precision,
           "mass_rel_change": abs(mass - M0) / M0,
           "shape_error": float(np.sum(np.abs(m.interior(VFg) - m.interior(VF0))) / (m.Nx * m.Ny * m.Nz)),
           "gpu_seconds": gpu_s}
    if cpu:
        from oracle.oracle import Oracle
        o = Oracle(m)
        VFo = VF0.copy(order="F")
        band, nx, ny, nz, D = o.init_state(VFo)
        t0 = time.perf_counter()
        for n in range(steps):
            f = o.step(dt, VFo, *vel(n), nx, ny, nz, D, band, True)
            if f:
                raise RuntimeError(f"restatement step {n}: flags {f}")
        out["cpu_seconds"] = time.perf_counter() - t0
        mo = o.mass(VFo)
        out["max_abs_dVF_vs_restatement"] = float(np.max(np.abs(m.interior(VFg) - m.interior(VFo))))
        out["mass_rel_diff_vs_restatement"] = abs(mass - mo) / abs(mo)
        out["bit_identical"] = bool(np.array_equal(VFg, VFo))
    return out


def drift(steps: int = 64):
    """Mass after `steps` steps of the 256^3 benchmark workload (200 spheres, seed 20261203,
    Deformation3D at t = dt/2, frozen, CFL 0.5) in three runs: the FP64 path, the FP64 path fed
    the face velocities rounded to FP32 (the mixed path's input precision), and the mixed path.
    Separates the effect of the FP32 velocity input from that of the FP32 geometry."""
    from ns_multiphase_gb300.slvof import SLVOF
    m = Mesh(Nx=256, Ny=256, Nz=256, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    centres, radii = cases.config_spheres(200, 20261203)
    dt = 0.5 * m.dx / 2.0
    vel = cases.deformation3d_faces(m, 0.5 * dt, 3.0)
    vel32 = tuple(a.astype(np.float32).astype(np.float64) for a in vel)
    out = {"workload": "256^3, 200 spheres seed 20261203, Deformation3D T=3 at t=dt/2, CFL 0.5", "steps": steps}
    for name, precision, v in (("fp64", "fp64", vel), ("fp64_on_fp32_velocities", "fp64", vel32),
                               ("mixed", "mixed", vel)):
        g = SLVOF(m, precision)
        g.case_vf_spheres(centres, radii, nF=20, dims=3)
        g.init_state()
        g.upload_velocity(*v)
        M0 = g.mass()
        for _ in range(steps):
            M = g.step(dt)
        g.close()
        out[name] = {"mass0": M0, "mass": M, "rel_change": abs(M - M0) / M0}
    ref = out["fp64"]["mass"]
    for name in ("fp64_on_fp32_velocities", "mixed"):
        out[name]["rel_diff_vs_fp64"] = abs(out[name]["mass"] - ref) / abs(ref)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=["2d", "3d", "drift"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--no-cpu", action="store_true")
    a = ap.parse_args()
    if a.config == "drift":
        print(json.dumps(drift(a.steps or 64)))
        return
    print(json.dumps(run(a.config, a.steps, a.precision, not a.no_cpu)))


if __name__ == "__main__":
    main()
