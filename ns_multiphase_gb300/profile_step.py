"""Per-stage timing of the SL-VOF step on one GPU: the driver used for stage profiles.

    python -m ns_multiphase_gb300.profile_step [N] [fp64|mixed] [steps]

Builds the N^3 workload the benchmark uses (200 spheres, seed 20261203, Deformation3D with
T = 3, CFL 0.5) on cuda:0 and runs `steps` steps, printing after each step the CUDA-event
time of every stage (ms) and the work-list sizes.  It is small enough to run under a kernel
profiler with a kernel filter.
"""
import sys

import numpy as np

from . import cases
from .mesh import Mesh
from .slvof import SLVOF

SEED = 20261203


def main(argv):
    N = int(argv[0]) if len(argv) > 0 else 256
    prec = argv[1] if len(argv) > 1 else "mixed"
    steps = int(argv[2]) if len(argv) > 2 else 3
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    c, r = cases.config_spheres(200, SEED)
    dt = 0.5 * m.dx / 2.0
    g = SLVOF(m, prec)
    g.case_vf_spheres(c, r, nF=20, dims=3)
    g.init_state()
    g.case_deformation3d(0.5 * dt, 3.0)
    for s in range(steps):
        g.step(dt)
        print(s, {k: round(v, 3) for k, v in g.stage_ms().items()}, g.counters(), flush=True)
    VF = g.download_vf()
    band = g.download_band()
    inner = m.interior(VF)
    print("interface cells", int(((inner >= m.VFlo) & (inner <= m.VFhi)).sum()),
          "band cells", int((np.abs(m.interior(band)) <= m.nband).sum()))
    g.close()


if __name__ == "__main__":
    main(sys.argv[1:])
