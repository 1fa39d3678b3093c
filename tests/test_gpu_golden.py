"""The FP64 GPU path against golden checksums of the CPU restatement over the whole 3D
deformation run: 128^3, sphere r = 0.15 at (0.35, 0.35, 0.35), Deformation3D with T = 3, all
1536 steps to t = T (examples/example5_deformation3D.jl:61-66, test/test_deformation3D.jl).
tests/golden/config1.json (made by tests/golden/make_config1.py on the CPU) holds the mass every
64 steps and the SHA-256 of the interior VF at steps 64, 512 and 1536.  Every mass must agree
to 1e-13 relative (the GPU sums exactly, the restatement with compensation) and every hash
exactly: the FP64 path is the restatement's arithmetic, bit for bit, over the whole run."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def built():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return True


def test_config1_full_run_matches_golden_checksums(built):
    from config_runs import config3d
    from ns_multiphase_gb300.slvof import SLVOF
    gold = json.load(open(os.path.join(HERE, "golden", "config1.json")))
    m, VF0, dt, vel, full = config3d()
    assert gold["steps"] == full and gold["dt"] == dt
    g = SLVOF(m, "fp64")
    g.upload_vf(VF0)
    g.vf_ghost_fill()
    g.init_state()
    assert abs(g.mass() - gold["mass0"]) <= 1e-13 * gold["mass0"]
    bad = []
    for n in range(full):
        g.upload_velocity(*vel(n))
        M = g.step(dt)
        s = str(n + 1)
        if s in gold["mass"] and abs(M - gold["mass"][s]) > 1e-13 * abs(gold["mass"][s]):
            bad.append(("mass", s, M, gold["mass"][s]))
        if s in gold["sha256_interior_vf"]:
            inner = np.asfortranarray(m.interior(g.download_vf()))
            h = hashlib.sha256(inner.tobytes(order="F")).hexdigest()
            if h != gold["sha256_interior_vf"][s]:
                bad.append(("hash", s))
        assert not bad, bad[:3]
    g.close()
