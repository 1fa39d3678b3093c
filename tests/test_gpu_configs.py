"""The FP64 path at the transport configurations' own sizes against the CPU restatement, bit
for bit: the 2D single vortex on 64^2 run to t = T (1024 steps) and the 3D sphere deformation on
128^3 for 6 steps (tests/config_runs.py)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.mark.parametrize("which,steps", [("2d", None), ("3d", 6)])
def test_configuration_bit_identical(built, which, steps):
    from config_runs import run
    out = run(which, steps)
    assert out["bit_identical"], out
    assert out["max_abs_dVF_vs_restatement"] <= 1e-12
    assert out["mass_rel_diff_vs_restatement"] <= 1e-13
    if which == "2d":
        # the vortex returns the circle at t = T; the reference's measure of how well it does
        # (8.1e-3 with these face samples) stays that of a converged interface, not a smeared one
        assert out["shape_error"] < 2e-2, out


def test_benchmark_state_generated_alike_on_gpu_and_cpu(built):
    """The benchmark's initial VF (union of spheres by VFsphere's rule) generated by the GPU
    library and by the restatement (the reference arm's state) is the same to the bit."""
    import numpy as np
    from ns_multiphase_gb300 import cases
    from ns_multiphase_gb300.mesh import Mesh
    from ns_multiphase_gb300.slvof import SLVOF
    from oracle.oracle import Oracle
    m = Mesh(Nx=48, Ny=40, Nz=44, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    c, r = cases.config_spheres(200, 20261203)
    with SLVOF(m, "fp64") as g:
        g.case_vf_spheres(c, 2.0 * r, nF=20, dims=3)
        Vg = g.download_vf()
    Vo = Oracle(m).vf_spheres(c, 2.0 * r, nF=20, dims=3)
    assert np.array_equal(Vg, Vo), float(np.max(np.abs(Vg - Vo)))
