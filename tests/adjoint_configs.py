"""The two adjoint configurations of the SL-VOF path, with their finite-difference checks.

    python tests/adjoint_configs.py 2d [--fd 64]      # 256^2, 40 steps
    python tests/adjoint_configs.py 3d [--fd 16] [--precision mixed]
    python tests/adjoint_configs.py 2d --save-gradient g.npz   # the reverse pass (GPU)
    python tests/adjoint_configs.py 2d --forward-mode g.npz    # against forward mode (CPU)
    python tests/adjoint_configs.py 3d --h-sweep --also mixed --out tests/golden/adjoint_3d.json
        # per-entry deviations at h = 1e-5, 1e-6, 1e-7 (check_sweep)

2d: single-vortex deformation on 256x256 (Nz = 1, z periodic), circle r = 0.15 at
    (0.5, 0.75) by 10x10 sub-sampling, stream-function face velocities (period T = 8) at
    t_n + dt/2 plus seeded N(0, 0.05^2) noise on every face (the same noise every step), FP64,
    40 steps with a VF checkpoint every 10.  Loss 1/2 ||VF_40 - VF_target||^2, the target from
    the noise-free field.  The gradient is with respect to every face velocity (the noise).
3d: Deformation3D (T = 3) on 128^3, sphere r = 0.15 at (0.35, 0.35, 0.35), plus the curl of a
    vector potential with 8x8x8 sine modes per component (3 x 512 coefficients, N(0, 0.02^2),
    seeded; ``cases.FourierPotential``), 30 steps with a checkpoint every 10.  Loss as above,
    gradient with respect to the 3 x 512 coefficients (FP64 accumulation; the forward runs in
    FP64 or mixed precision).

The gradient comes from the library's reverse pass (``adjoint.Rollout``).  Finite
differences are central, h = 1e-6, of the FP64 forward: the CPU restatement, or the FP64 GPU
path, whose results are bit-identical to it.  The check reports the largest deviation relative
to the largest finite difference of the checked entries.  Entries are drawn at random among
those with a nonzero derivative (the rest are exactly zero on both sides).
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

SEED = 20261203
H = 1e-6


class Config:
    """A rollout with parameters p: vel(n, p) -> face velocities of step n."""

    def __init__(self, name, mesh, VF0, dt, steps, every, base, perturb, p0, grad_of_faces):
        self.name, self.mesh, self.VF0, self.dt = name, mesh, VF0, dt
        self.steps, self.every = steps, every
        self.base, self.perturb, self.p0, self.grad_of_faces = base, perturb, p0, grad_of_faces
        self.target = None

    def vel(self, n, p):
        d = self.perturb(p)
        return tuple(np.asfortranarray(a + e) for a, e in zip(self.base(n), d))


def config2d(N=256, steps=40, every=10, sigma=0.05, seed=SEED):
    m = Mesh(Nx=N, Ny=N, Nz=1, Lx=1.0, Ly=1.0, Lz=1.0 / N, CFL=0.5, zper=True)
    VF0 = cases.vf_spheres(m, np.array([[0.5, 0.75, 0.0]]), np.array([0.15]), nF=10, dims=2)
    dt = 0.5 * m.dx  # CFL 0.5 on the vortex field (max |u| = 1)
    base = lambda n: cases.deformation2d_faces(m, (n + 0.5) * dt, 8.0)
    rng = np.random.default_rng(seed)
    noise = np.stack([sigma * rng.standard_normal(m.cell_shape), sigma * rng.standard_normal(m.cell_shape),
                      np.zeros(m.cell_shape)])

    def perturb(p):
        return p[0], p[1], p[2]
    return Config("2d", m, VF0, dt, steps, every, base, perturb, noise, lambda gu, gv, gw: np.stack([gu, gv, gw]))


def config3d(N=128, steps=30, every=10, sigma=0.02, modes=8, seed=SEED):
    m = Mesh(Nx=N, Ny=N, Nz=N, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    VF0 = cases.vf_spheres(m, np.array([[0.35, 0.35, 0.35]]), np.array([0.15]), nF=20)
    F = cases.FourierPotential(m, modes)
    C = sigma * np.random.default_rng(seed).standard_normal((3, modes, modes, modes))
    pert = F.faces(C)
    umax = max(np.max(np.abs(a + b)) for a, b in zip(cases.deformation3d_faces(m, 0.0, 3.0), pert))
    dt = 0.5 * m.dx / umax  # CFL 0.5 on the perturbed field
    base = lambda n: cases.deformation3d_faces(m, (n + 0.5) * dt, 3.0)
    return Config("3d", m, VF0, dt, steps, every, base, F.faces, C, F.grad)


# ---- forward evaluations -----------------------------------------------------------------
def rollout_cpu(cfg, p):
    """VF after the rollout by the CPU restatement (FP64)."""
    from oracle.oracle import Oracle
    o = Oracle(cfg.mesh)
    VF = cfg.VF0.copy(order="F")
    band, nx, ny, nz, D = o.init_state(VF)
    for n in range(cfg.steps):
        f = o.step(cfg.dt, VF, *cfg.vel(n, p), nx, ny, nz, D, band, True)
        if f:
            raise RuntimeError(f"restatement step {n}: error bits {f}")
    return VF


def rollout_gpu(cfg, p, precision="fp64"):
    from ns_multiphase_gb300.slvof import SLVOF
    g = SLVOF(cfg.mesh, precision)
    g.upload_vf(cfg.VF0)
    g.vf_ghost_fill()
    g.prepare()
    for n in range(cfg.steps):
        g.upload_velocity(*cfg.vel(n, p))
        g.step(cfg.dt, band=True, mass=False)
    VF = g.download_vf()
    g.close()
    return VF


def loss(cfg, VF):
    r = cfg.mesh.interior(VF) - cfg.mesh.interior(cfg.target)
    return 0.5 * float(np.sum(r * r))


def gradient(cfg, precision="fp64"):
    """(loss, dL/dp, timings) by the library's reverse pass."""
    from ns_multiphase_gb300.adjoint import Rollout
    from ns_multiphase_gb300.slvof import SLVOF
    m = cfg.mesh
    g = SLVOF(m, precision)
    g.upload_vf(cfg.VF0)
    g.vf_ghost_fill()
    R = Rollout(g, cfg.dt, cfg.steps, lambda n: cfg.vel(n, cfg.p0), every=cfg.every)
    VFT = R.forward()
    gT = m.vf_array()
    m.interior(gT)[...] = m.interior(VFT) - m.interior(cfg.target)
    _, (gu, gv, gw) = R.backward(gT)
    g.close()
    times = {"forward_ms": R.fwd_ms, "backward_ms": R.bwd_ms,
             "fwd_step_ms": float(np.mean(R.fwd_step_ms)), "adj_step_ms": float(np.mean(R.adj_step_ms))}
    return loss(cfg, VFT), cfg.grad_of_faces(gu, gv, gw), times


def check(cfg, count, fd_backend="cpu", precision="fp64", seed=7, also=(), sweep_all=False):
    """Gradient by the reverse pass against central differences on `count` entries.  `also`
    lists further forward precisions whose gradients are compared on the same entries."""
    evaluate = rollout_cpu if fd_backend == "cpu" else rollout_gpu
    cfg.target = evaluate(cfg, np.zeros_like(cfg.p0))
    L, G, times = gradient(cfg, precision)
    others = {pr: gradient(cfg, pr) for pr in also}
    rng = np.random.default_rng(seed)
    support = np.argwhere(np.abs(G) > 0)
    picks = [tuple(support[k]) for k in rng.choice(len(support), size=min(count, len(support)), replace=False)]
    def fd_at(idx, h):
        vals = []
        for sgn in (1.0, -1.0):
            p = cfg.p0.copy()
            p[idx] += sgn * h
            vals.append(loss(cfg, evaluate(cfg, p)))
        return (vals[0] - vals[1]) / (2 * h)

    rows = []
    t0 = time.perf_counter()
    for idx in picks:
        rows.append((float(G[idx]), fd_at(idx, H)))
    adj = np.array([r[0] for r in rows])
    fd = np.array([r[1] for r in rows])
    scale = float(np.max(np.abs(fd)))
    # Entries off by more than 1e-6 of the scale: central differences again with h/8.  Where the
    # two differ by more than the tolerance themselves, the loss is not smooth within +-h of the
    # input (a discrete choice of the step switches there) and neither estimate is a derivative.
    sweep = {}
    for q, idx in enumerate(picks):
        if sweep_all or (scale > 0 and abs(adj[q] - fd[q]) > 1e-6 * scale):
            sweep[q] = fd_at(idx, H / 8)
    fd_s = time.perf_counter() - t0
    smooth = [q for q in range(len(picks)) if q not in sweep or abs(sweep[q] - fd[q]) <= 1e-6 * scale]
    rough = [q for q in range(len(picks)) if q not in smooth]
    extra = {}
    for pr, (Lp, Gp, tp) in others.items():
        ap = np.array([float(Gp[idx]) for idx in picks])
        extra[pr] = {"loss": Lp, "max_abs_err_over_max_fd": float(np.max(np.abs(ap - fd)) / scale) if scale > 0 else None,
                     "rel_l2_vs_" + precision: float(np.linalg.norm(Gp - G) / np.linalg.norm(G)), "timings": tp}
    return {"config": cfg.name, "also": extra, "grid": list(cfg.mesh.cell_shape), "steps": cfg.steps, "checkpoint_every": cfg.every,
            "precision_forward": precision, "fd_backend": fd_backend, "h": H, "loss": L,
            "params": int(cfg.p0.size), "support": int(len(support)), "checked": len(rows),
            "max_abs_err_over_max_fd": float(np.max(np.abs(adj - fd)) / scale) if scale > 0 else None,
            "smooth_entries": len(smooth),
            "max_abs_err_over_max_fd_smooth": float(np.max(np.abs(adj[smooth] - fd[smooth])) / scale)
            if scale > 0 and smooth else None,
            "not_smooth": [{"index": [int(x) for x in picks[q]], "adjoint": float(adj[q]), "fd_h": float(fd[q]),
                            "fd_h_over_8": float(sweep[q])} for q in rough],
            "max_abs_err_over_max_fd_h_over_8": float(max(abs(adj[q] - sweep[q]) for q in sweep) / scale)
            if sweep and scale > 0 else None,
            "max_fd": scale, "fd_seconds": fd_s, "timings": times,
            "entries": [{"index": [int(x) for x in idx], "adjoint": a, "fd": f, "fd_h_over_8": sweep.get(q)}
                        for q, (idx, (a, f)) in enumerate(zip(picks, rows))]}


H_SWEEP = (1e-5, 1e-6, 1e-7)


def sweep_entry(a, fds, others=None):
    """One entry of a step sweep: the reverse pass's derivative `a` against central differences
    `fds` (h -> value).  Its relative deviation at every h (the absolute one where the difference
    is exactly zero), its best h, and whether the loss is smooth on the check's scale: the
    differences at h = 1e-6 and 1e-7 agree to 1e-6 of |FD|.  Where they do not, a discrete
    choice of the step (an ELVIRA candidate, a d2case sign, a band bit) switches within +-1e-6
    of the input, and neither difference there is a derivative, or the differences at the
    smaller steps are dominated by the loss's rounding (which grows as 1/h).  That rounding is
    estimated for h = 1e-5 from the spread between h = 1e-6 and 1e-7, and the entry is also
    judged against 1e-6 of |FD| plus that estimate.  `others` maps further precisions to their
    reverse-pass derivatives."""
    rel = {h: (abs(a - f) / abs(f) if f != 0 else None) for h, f in fds.items()}
    cands = [h for h in H_SWEEP if rel[h] is not None]
    best = min(cands, key=lambda h: rel[h]) if cands else None
    f5, f6, f7 = fds[1e-5], fds[1e-6], fds[1e-7]
    smooth = abs(f6 - f7) <= 1e-6 * max(abs(f6), abs(f7)) if (f6 != 0 or f7 != 0) else True
    # rounding of the loss enters a central difference as 1/h: the spread between h = 1e-6 and
    # 1e-7 (dominated by the smaller step's) scaled to h = 1e-5 estimates that difference's noise
    noise5 = abs(f7 - f6) * 1e-2
    e = {"adjoint": a, "fd": {str(h): f for h, f in fds.items()},
         "rel_err": {str(h): r for h, r in rel.items()}, "abs_err": {str(h): abs(a - f) for h, f in fds.items()},
         "best_h": best, "rel_err_best": rel[best] if best is not None else None,
         "fd_zero": best is None, "smooth": bool(smooth),
         "fd_noise_rel_h_1e-5": noise5 / abs(f5) if f5 != 0 else None,
         "within_1e-6_plus_fd_noise_at_h_1e-5": bool(f5 != 0 and abs(a - f5) <= 1e-6 * abs(f5) + noise5)}
    for pr, ap in (others or {}).items():
        e["adjoint_" + pr] = ap
        e["rel_err_best_" + pr] = abs(ap - fds[best]) / abs(fds[best]) if best is not None else None
    return e


def sweep_summary(entries, precisions=()):
    """Counts over a sweep's entries: smooth ones, their worst relative deviation at their best
    h, how many are within 1e-6, the not-smooth and zero-difference ones, and for each further
    precision its worst deviation over the smooth entries.  The scale for zero differences is
    the largest |FD| at h = 1e-6 of the check."""
    scale = max(abs(e["fd"][str(1e-6)]) for e in entries)
    sm = [e for e in entries if e["smooth"] and not e["fd_zero"]]
    nz = [e for e in entries if not e["fd_zero"]]
    out = {"checked": len(entries),
           "within_1e-6_at_best_h": sum(1 for e in nz if e["rel_err_best"] <= 1e-6),
           "within_1e-6_plus_fd_noise_at_h_1e-5": sum(1 for e in nz if e["within_1e-6_plus_fd_noise_at_h_1e-5"]),
           "neither": [{"index": e["index"], "rel_err": e["rel_err"], "fd_noise_rel_h_1e-5": e["fd_noise_rel_h_1e-5"]}
                       for e in nz if e["rel_err_best"] > 1e-6 and not e["within_1e-6_plus_fd_noise_at_h_1e-5"]],
           "smooth_entries": len(sm),
           "max_rel_err_best_smooth": max((e["rel_err_best"] for e in sm), default=None),
           "smooth_entries_within_1e-6": sum(1 for e in sm if e["rel_err_best"] <= 1e-6),
           "not_smooth": [{"index": e["index"], "rel_err_best": e["rel_err_best"], "best_h": e["best_h"]}
                          for e in entries if not e["smooth"]],
           "fd_zero": [{"index": e["index"], "adjoint": e["adjoint"],
                        "abs_adjoint_over_max_fd": abs(e["adjoint"]) / scale if scale > 0 else None}
                       for e in entries if e["fd_zero"]],
           "max_fd_h_1e-6": scale}
    for pr in precisions:
        out["max_rel_err_best_smooth_" + pr] = max((e["rel_err_best_" + pr] for e in sm
                                                    if e.get("rel_err_best_" + pr) is not None), default=None)
    return out


def check_sweep(cfg, count, fd_backend="gpu", precision="fp64", seed=7, also=()):
    """Per-entry check with a step sweep: central differences at h = 1e-5, 1e-6 and 1e-7 for
    every entry (sweep_entry), summarised by sweep_summary.  `also` lists further forward
    precisions whose reverse-pass gradients are reported on the same entries."""
    evaluate = rollout_cpu if fd_backend == "cpu" else rollout_gpu
    cfg.target = evaluate(cfg, np.zeros_like(cfg.p0))
    L, G, times = gradient(cfg, precision)
    others = {pr: gradient(cfg, pr) for pr in also}
    rng = np.random.default_rng(seed)
    support = np.argwhere(np.abs(G) > 0)
    picks = [tuple(support[k]) for k in rng.choice(len(support), size=min(count, len(support)), replace=False)]

    def fd_at(idx, h):
        vals = []
        for sgn in (1.0, -1.0):
            p = cfg.p0.copy()
            p[idx] += sgn * h
            vals.append(loss(cfg, evaluate(cfg, p)))
        return (vals[0] - vals[1]) / (2 * h)

    t0 = time.perf_counter()
    entries = []
    for idx in picks:
        e = sweep_entry(float(G[idx]), {h: fd_at(idx, h) for h in H_SWEEP},
                        {pr: float(Gp[idx]) for pr, (Lp, Gp, tp) in others.items()})
        entries.append({"index": [int(x) for x in idx], **e})
    out = {"config": cfg.name, "grid": list(cfg.mesh.cell_shape), "steps": cfg.steps,
           "checkpoint_every": cfg.every, "precision_forward": precision, "fd_backend": fd_backend,
           "h_sweep": list(H_SWEEP), "loss": L, "params": int(cfg.p0.size), "support": int(len(support)),
           **sweep_summary(entries, tuple(others)),
           "fd_seconds": time.perf_counter() - t0, "timings": times,
           "also": {pr: {"loss": Lp, "rel_l2_vs_" + precision: float(np.linalg.norm(Gp - G) / np.linalg.norm(G)),
                         "timings": tp} for pr, (Lp, Gp, tp) in others.items()},
           "entries": entries}
    return out


def resummarize(path):
    """A saved sweep's entries re-evaluated by sweep_entry and sweep_summary (the differences
    and derivatives themselves are kept)."""
    d = json.load(open(path))
    prs = tuple(d.get("also", {}))
    entries = []
    for e in d["entries"]:
        fds = {h: e["fd"][str(h)] for h in H_SWEEP}
        entries.append({"index": e["index"], **sweep_entry(e["adjoint"], fds,
                                                           {pr: e["adjoint_" + pr] for pr in prs})})
    for k in ("checked", "smooth_entries", "max_rel_err_best_smooth", "smooth_entries_within_1e-6", "not_smooth",
              "fd_zero", "max_fd_h_1e-6", "within_1e-6_at_best_h", "within_1e-6_plus_fd_noise_at_h_1e-5", "neither"):
        d.pop(k, None)
    for pr in prs:
        d.pop("max_rel_err_best_smooth_" + pr, None)
        d.get("also", {}).get(pr, {}).pop("max_rel_err_best_smooth", None)
    ent = d.pop("entries")
    d.update(sweep_summary(entries, prs))
    d["entries"] = entries
    return d


def save_gradient(cfg, path, precision="fp64"):
    """The reverse pass's gradient of the configuration (GPU), with its loss, saved for
    forward_mode_check (which needs no GPU)."""
    cfg.target = rollout_gpu(cfg, np.zeros_like(cfg.p0))
    L, G, times = gradient(cfg, precision)
    np.savez(path, loss=L, grad=G, precision=precision, steps=cfg.steps, every=cfg.every)
    return {"config": cfg.name, "saved": path, "loss": L, "timings": times}


def forward_mode_check(cfg, path, count, seed=7):
    """The saved reverse-pass gradient against forward-mode derivatives of the restatement's
    whole rollout (Dual numbers through the initial state and every step's SL update, normals,
    PLIC and band; the analogue of a ForwardDiff.jl gradient), on `count` entries drawn as check
    draws them.  For L = 1/2 ||VF_T - target||^2, dL = sum((VF_T - target) * dVF_T).  Face
    parameters only (the 2D configuration's per-face noise): each seed perturbs one face of
    every step's velocities."""
    from oracle.oracle import Oracle
    saved = np.load(path)
    G = saved["grad"]
    m = cfg.mesh
    cfg.target = rollout_cpu(cfg, np.zeros_like(cfg.p0))
    VFT = rollout_cpu(cfg, cfg.p0)
    w = m.interior(VFT) - m.interior(cfg.target)
    rng = np.random.default_rng(seed)
    support = np.argwhere(np.abs(G) > 0)
    picks = [tuple(int(x) for x in support[k]) for k in rng.choice(len(support), size=min(count, len(support)),
                                                                  replace=False)]
    o = Oracle(m)
    vel = [cfg.vel(n, cfg.p0) for n in range(cfg.steps)]
    us, vs, ws = [v[0] for v in vel], [v[1] for v in vel], [v[2] for v in vel]
    K = o.ndual()
    fwd = []
    t0 = time.perf_counter()
    for c0 in range(0, len(picks), K):
        batch = [(idx[0], idx[1:]) for idx in picks[c0:c0 + K]]
        Lf, dL = o.rollout_forward(cfg.dt, cfg.steps, cfg.VF0, us, vs, ws, batch, [], w)
        fwd += list(dL)
    secs = time.perf_counter() - t0
    fwd = np.array(fwd)
    adj = np.array([float(G[idx]) for idx in picks])
    scale = float(np.max(np.abs(fwd)))
    return {"config": cfg.name, "grid": list(m.cell_shape), "steps": cfg.steps, "checkpoint_every": cfg.every,
            "reverse_precision": str(saved["precision"]), "reverse_loss": float(saved["loss"]),
            "loss_restatement": loss(cfg, VFT), "checked": len(picks),
            "max_abs_err_over_max_forward_mode": float(np.max(np.abs(adj - fwd)) / scale) if scale > 0 else None,
            "max_forward_mode": scale, "forward_mode_seconds": secs,
            "entries": [{"index": list(idx), "adjoint": float(a), "forward_mode": float(f)}
                        for idx, a, f in zip(picks, adj, fwd)]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=["2d", "3d"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--fd", type=int, default=None)
    ap.add_argument("--fd-backend", choices=["cpu", "gpu"], default=None)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--also", choices=["fp64", "mixed"], nargs="*", default=[])
    ap.add_argument("--sweep-all", action="store_true", help="central differences with h/8 for every entry")
    ap.add_argument("--h-sweep", action="store_true",
                    help="per-entry relative deviations at h = 1e-5, 1e-6, 1e-7 (check_sweep)")
    ap.add_argument("--out", metavar="FILE", help="also write the JSON result to FILE")
    ap.add_argument("--resummarize", metavar="FILE",
                    help="re-evaluate a saved --h-sweep result's per-entry verdicts and summary (no GPU)")
    ap.add_argument("--save-gradient", metavar="FILE", help="save the reverse pass's gradient (GPU) and stop")
    ap.add_argument("--forward-mode", metavar="FILE",
                    help="check a saved gradient against forward-mode derivatives of the restatement (2d, CPU)")
    a = ap.parse_args()
    if a.resummarize:
        out = resummarize(a.resummarize)
        with open(a.out or a.resummarize, "w") as fh:
            json.dump(out, fh, indent=1)
            fh.write("\n")
        print(json.dumps({k: v for k, v in out.items() if k not in ("entries", "timings")}))
        return
    if a.save_gradient or a.forward_mode:
        cfg = config2d(N=a.n or 256, steps=a.steps or 40, every=a.every) if a.config == "2d" else \
            config3d(N=a.n or 128, steps=a.steps or 30, every=a.every)
        if a.save_gradient:
            print(json.dumps(save_gradient(cfg, a.save_gradient, a.precision)))
        else:
            assert a.config == "2d", "forward mode seeds face parameters: the 2d configuration"
            print(json.dumps(forward_mode_check(cfg, a.forward_mode, a.fd or 64)))
        return
    if a.config == "2d":
        cfg = config2d(N=a.n or 256, steps=a.steps or 40, every=a.every)
        count, backend = a.fd or 64, a.fd_backend or "cpu"
    else:
        cfg = config3d(N=a.n or 128, steps=a.steps or 30, every=a.every)
        count, backend = a.fd or 16, a.fd_backend or "gpu"
    if a.h_sweep:
        out = check_sweep(cfg, count, backend, a.precision, also=a.also)
    else:
        out = check(cfg, count, backend, a.precision, also=a.also, sweep_all=a.sweep_all)
    print(json.dumps(out))
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(out, fh, indent=1)
            fh.write("\n")


if __name__ == "__main__":
    main()
