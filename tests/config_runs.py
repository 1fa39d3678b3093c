"""The two FP64 transport configurations at their own sizes, on the GPU path and on the CPU
restatement, with the reference's shape-error measure.

    python tests/config_runs.py 2d [--steps 1024]   # 64^2 single vortex to t = T
    python tests/config_runs.py 3d [--steps 8]      # 128^3 sphere deformation
    python tests/config_runs.py drift [--steps 64] [--n 256] [--frozen]
        # benchmark workload's mass: FP64, FP64 on FP32 velocities, mixed

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
    field = cases.Deformation3DFaces(m)
    vel = lambda n: field.faces((n + 0.5) * dt, 3.0)
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


def drift(steps: int = 64, n: int = 256, frozen: bool = False, marks=(8, 64, 256, 1024, 3072)):
    """Mixed-vs-FP64 mass difference over `steps` steps of the benchmark workload at n^3 (200
    spheres, seed 20261203, Deformation3D with T = 3, CFL 0.5, dt = 0.25 dx), in three runs: the
    FP64 path, the FP64 path fed the face velocities rounded to FP32 (the mixed path's input
    precision), and the mixed path.  The face velocities follow the field in time, evaluated at
    t_n + dt/2 for step n (frozen=True keeps the field of step 0).  Reports, at each step in
    `marks` (and the last), each run's mass, the relative mass difference against the FP64 run,
    and for the mixed run the largest and the 99th-percentile per-cell |dVF| over interface
    cells."""
    from ns_multiphase_gb300.slvof import SLVOF
    m = Mesh(Nx=n, Ny=n, Nz=n, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    centres, radii = cases.config_spheres(200, 20261203)
    dt = 0.5 * m.dx / 2.0
    marks = sorted({s for s in marks if s <= steps} | {steps})
    out = {"workload": f"{n}^3, 200 spheres seed 20261203, Deformation3D T=3 "
                       f"({'frozen at t=dt/2' if frozen else 'at t_n + dt/2'}), CFL 0.5", "steps": steps,
           "marks": marks}
    runs = (("fp64", "fp64", False), ("fp64_on_fp32_velocities", "fp64", True), ("mixed", "mixed", False))
    ctx = {}
    for name, precision, round32 in runs:
        g = SLVOF(m, precision)
        g.case_vf_spheres(centres, radii, nF=20, dims=3)
        g.init_state()
        ctx[name] = (g, round32)
        out[name] = {"mass0": g.mass(), "mass": {}}
    vel_cache = None
    t0 = time.perf_counter()
    for s in range(steps):
        t = 0.5 * dt if frozen else (s + 0.5) * dt
        for name, (g, round32) in ctx.items():
            if round32:
                if vel_cache is None or not frozen:
                    vel_cache = tuple(a.astype(np.float32).astype(np.float64)
                                      for a in cases.deformation3d_faces(m, t, 3.0))
                if s == 0 or not frozen:
                    g.upload_velocity(*vel_cache)
            elif s == 0 or not frozen:
                g.case_deformation3d(t, 3.0)
            M = g.step(dt)
            if s + 1 in marks:
                out[name]["mass"][s + 1] = M
        if s + 1 in marks:
            V64 = m.interior(ctx["fp64"][0].download_vf())
            V32 = m.interior(ctx["mixed"][0].download_vf())
            iface = (V64 >= m.VFlo) & (V64 <= m.VFhi)
            d = np.abs(V32 - V64)
            out["mixed"].setdefault("max_abs_dVF", {})[s + 1] = float(d.max())
            out["mixed"].setdefault("p99_abs_dVF_interface", {})[s + 1] = float(np.percentile(d[iface], 99))
            print(json.dumps({"step": s + 1, "seconds": round(time.perf_counter() - t0, 1),
                              "mixed_rel_diff": abs(out["mixed"]["mass"][s + 1] - out["fp64"]["mass"][s + 1])
                              / abs(out["fp64"]["mass"][s + 1])}), file=sys.stderr, flush=True)
    for g, _ in ctx.values():
        g.close()
    ref = out["fp64"]["mass"]
    for name in ("fp64_on_fp32_velocities", "mixed"):
        out[name]["rel_diff_vs_fp64"] = {s: abs(out[name]["mass"][s] - ref[s]) / abs(ref[s]) for s in marks}
    out["fp64"]["rel_change"] = {s: abs(ref[s] - out["fp64"]["mass0"]) / out["fp64"]["mass0"] for s in marks}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=["2d", "3d", "drift"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=256, help="drift: grid size")
    ap.add_argument("--frozen", action="store_true", help="drift: keep the field of step 0")
    a = ap.parse_args()
    if a.config == "drift":
        print(json.dumps(drift(a.steps or 64, a.n, a.frozen)))
        return
    print(json.dumps(run(a.config, a.steps, a.precision, not a.no_cpu)))


if __name__ == "__main__":
    main()
