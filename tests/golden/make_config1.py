"""Golden checksums of the 3D deformation configuration run to t = T by the CPU restatement.

    python tests/golden/make_config1.py [--steps 1536] [--out tests/golden/config1.json]

128^3 unit cube, sphere r = 0.15 at (0.35, 0.35, 0.35) by VFsphere's rule with 20^3 sub-samples
(examples/example5_deformation3D.jl:61-66), Deformation3D face velocities with period T = 3
sampled at the faces at t_n + dt/2 (src/Tools.jl:660-662), CFL 0.5 (dt = 0.25 dx), 1536
steps to t = T, band and plane constants every step (tests/config_runs.py config3d).  The
restatement (oracle/slvof_oracle.cpp, OpenMP) records the mass sum(VF) dx dy dz
(src/WriteData.jl:33) every 64 steps and the SHA-256 of the interior VF (float64, Fortran
order) at steps 64, 512 and 1536.  The FP64 GPU path must reproduce every mass to 1e-13 and
every hash exactly (tests/test_gpu_golden.py).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np

HASH_STEPS = (64, 512, 1536)
MASS_EVERY = 64


def vf_hash(m, VF) -> str:
    inner = np.asfortranarray(m.interior(VF))
    return hashlib.sha256(inner.tobytes(order="F")).hexdigest()


def main():
    from config_runs import config3d
    from oracle.oracle import Oracle, build
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1536)
    ap.add_argument("--out", default=os.path.join(HERE, "config1.json"))
    a = ap.parse_args()
    build()
    m, VF0, dt, vel, full = config3d()
    o = Oracle(m)
    VF = VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VF)
    out = {"config": "3D deformation 128^3, sphere r=0.15 at (0.35,0.35,0.35), nF=20, Deformation3D T=3 at "
                     "t_n + dt/2, CFL 0.5 (dt = 0.25 dx), nband 1, RK4, 5 tets",
           "made_by": "python tests/golden/make_config1.py (CPU restatement, oracle/slvof_oracle.cpp)",
           "dt": dt, "steps": a.steps, "mass0": o.mass(VF), "mass": {}, "sha256_interior_vf": {}}
    t0 = time.time()
    for n in range(a.steps):
        f = o.step(dt, VF, *vel(n), nx, ny, nz, D, band, True)
        if f:
            raise RuntimeError(f"restatement step {n}: flags {f}")
        s = n + 1
        if s % MASS_EVERY == 0 or s == a.steps:
            out["mass"][str(s)] = o.mass(VF)
            print(s, f"{time.time() - t0:.0f}s", out["mass"][str(s)], flush=True)
        if s in HASH_STEPS:
            out["sha256_interior_vf"][str(s)] = vf_hash(m, VF)
    with open(a.out, "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
