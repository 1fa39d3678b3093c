"""Per-stage timing of the SL-VOF step on one GPU: the driver used for stage profiles.

    python -m ns_multiphase_gb300.profile_step [N] [fp64|mixed] [steps] [adjoint]

Builds the N^3 workload the benchmark uses (200 spheres, seed 20261203, Deformation3D with
T = 3, CFL 0.5) on cuda:0 and runs `steps` steps, printing after each step the CUDA-event
time of every stage (ms) and the work-list sizes.  With `adjoint`, it then runs `steps`
reverse steps from the last state (the step's result given, as a rollout holds it), seeded
with normal weights on the interior, and prints their times.  It is small enough to run under
a kernel profiler with a kernel filter.
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
    if len(argv) > 3 and argv[3] == "adjoint":
        import torch
        nvf = int(np.prod(m.vf_shape))
        s0 = torch.empty(nvf, dtype=torch.float64, device="cuda")
        s1 = torch.empty_like(s0)
        g.copy_vf_device(s0.data_ptr())
        g.step(dt, band=True, mass=False)
        g.copy_vf_device(s1.data_ptr())
        g.load_vf_device(s0.data_ptr())
        g.prepare()
        gT = m.vf_array()
        m.interior(gT)[...] = np.random.default_rng(SEED).standard_normal((N, N, N))
        g.adjoint_set_vf(gT)
        g.adjoint_zero_velocity()
        for s in range(steps):
            g.adjoint_step(dt, s1.data_ptr())
            print("adjoint", s, round(g.last_kernel_ms(), 3), flush=True)
    VF = g.download_vf()
    band = g.download_band()
    inner = m.interior(VF)
    print("interface cells", int(((inner >= m.VFlo) & (inner <= m.VFhi)).sum()),
          "band cells", int((np.abs(m.interior(band)) <= m.nband).sum()))
    g.close()


if __name__ == "__main__":
    main(sys.argv[1:])
