#!/usr/bin/env python
"""SL-VOF transport step benchmark (one JSON line on rank 0).

Workload (the reference path's 256^3 configuration): 256^3 unit cube, VF = union of 200
spheres (radii U[0.02,0.08], centres U[0.1,0.9]^3, numpy default_rng(20261203)) sampled by
VFsphere's rule with nF=20, Deformation3D face velocities with period T=3, CFL 0.5
(dt = 0.5*dx/max|u| = 0.25/256), band recomputed every step (nband = 1) and the mass summed
every step.  A step is one resident call of slvof_step: SL update of the band cells, VF ghost
fill, ELVIRA, PLIC distances, band, mass.  1 cell-update = 1 interior cell advanced one step
(all 256^3 cells count).  The face velocities are the field at t0 + dt/2 and stay resident
over the timed window; every field is larger than L2 (129 MB), so no flush is needed.

Arms:
  value      mixed precision (the SL update in flux form: FP64 node traces and face volumes,
             FP32 clip; FP32 ELVIRA errors with FP64 arbitration; FP64 PLIC root, volume sums,
             mass), device-resident, CUDA events on the launching stream;
  fp64       the plain FP64 path (bit-identical to the CPU restatement) on the same state;
  e2e        slvof_step_host: H2D of the step's face velocities from pinned memory, the
             step, D2H of VF and the mass; with SLVOF_STEP_DEFER, which builds each state's
             normals, PLIC and band beside the next call's upload ("without_defer": the same
             calls with everything built inside the call that made the state);
  cpu_baseline / --impl reference: the CPU restatement of the reference (C++, OpenMP on
             all host cores) on a bounded z-slab of the same state.

Rooflines: "roofline" is the HBM roofline of the dominant stage (algorithmic bytes over its
CUDA-event time, against the measured copy bandwidth); "roofline.compute" counts the
reference algorithm's operations on a sample of the state (the restatement run with a
counting scalar, in the CPU leg: absent with --no-cpu) and sets them against the CUDA
cores' nominal FP32 rate (mixed) and FP64 rate (the FP64 arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SL-VOF cell-updates/s at 256³: mixed vs FP64 at ≤1e-10 mass err; adj/fwd time"
SEED = 20261203


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=256)
    p.add_argument("--fp64-steps", type=int, default=3)
    p.add_argument("--drift-steps", type=int, default=256,
                   help="steps of the mixed-vs-FP64 mass comparison (time-varying field); the FP64 masses come "
                        "from tests/golden/drift_fp64_<n>.json when it covers them (checked live over the first "
                        "8 steps), else from a live FP64 run")
    p.add_argument("--drift-record", action="store_true",
                   help="run the FP64 path for --drift-steps steps and write tests/golden/drift_fp64_<n>.json")
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--adj-steps", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--count-sample", type=int, default=1500,
                   help="interface cells sampled for the operation count of the CPU leg (twice as many band "
                        "cells); 0 skips it")
    p.add_argument("--stage-run", choices=["step", "adjoint", "fd-adjoint"], default=None,
                   help="workload for kernel profilers only (no JSON line): 'step' runs --steps resident steps "
                        "of the --n^3 workload in --precision and prints each step's stage times; 'adjoint' "
                        "then runs --steps reverse steps from the last state (the step's result given); "
                        "'fd-adjoint' runs two reverse steps of the finite-difference scheme at 64^3 (FP64)")
    p.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_rate(ms, cells, steps, ws, device):
    """Whole-job throughput of ws replicas, each advancing `cells` cells `steps` steps: every
    rank's cells over the slowest rank's time (all-reduce MAX of the per-rank milliseconds on
    `device`: "cuda" under NCCL, "cpu" under gloo).  Returns (cell-updates/s, ms)."""
    if ws > 1:
        import torch
        import torch.distributed as tdist
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms = float(t.item())
    return ws * cells * steps / (ms / 1e3), ms


def workload(n):
    from ns_multiphase_gb300 import cases
    from ns_multiphase_gb300.mesh import Mesh
    m = Mesh(Nx=n, Ny=n, Nz=n, Lx=1.0, Ly=1.0, Lz=1.0, CFL=0.5)
    centres, radii = cases.config_spheres(200, SEED)
    dt = 0.5 * m.dx / 2.0
    return m, centres, radii, dt


DRIFT_MARKS = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 3072)


def drift_record_path(n):
    return os.path.join(ROOT, "tests", "golden", f"drift_fp64_{n}.json")


def drift_run(m, centres, radii, dt, steps, precision, VF0, marks):
    """The workload advanced `steps` steps with the face velocities of Deformation3D at
    t_n + dt/2 for step n (the field follows time, as the 3D deformation run does); returns the
    context and the masses at the marks."""
    g = make_ctx(m, centres, radii, precision, 0.5 * dt, VF0)
    masses = {}
    for s in range(steps):
        g.case_deformation3d((s + 0.5) * dt, 3.0)
        M = g.step(dt)
        if s + 1 in marks:
            masses[s + 1] = M
    return g, masses


def drift_record(args):
    """--drift-record: the FP64 path's masses over the drift run, as a fixture for the bench."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)
    m, centres, radii, dt = workload(args.n)
    marks = [k for k in DRIFT_MARKS if k <= args.drift_steps]
    t0 = time.time()
    g, masses = drift_run(m, centres, radii, dt, args.drift_steps, "fp64", None, set(marks))
    g.close()
    rec = {"workload": workload_config(args.n)["workload"], "field": "Deformation3D T=3 at t_n + dt/2",
           "dt": dt, "made_by": f"python bench.py --drift-record --n {args.n} --drift-steps {args.drift_steps} "
                                f"(the FP64 path, deterministic: bit-identical to the CPU restatement)",
           "mass": {str(k): v for k, v in masses.items()}}
    with open(drift_record_path(args.n), "w") as fh:
        json.dump(rec, fh, indent=1)
        fh.write("\n")
    print(json.dumps({"recorded": drift_record_path(args.n), "seconds": time.time() - t0}), flush=True)


def drift_leg(m, centres, radii, dt, steps, VF0):
    """Mixed-vs-FP64 mass difference over `steps` steps at the marks, the FP64 masses from the
    recorded run when it covers them (its first mark is reproduced live: the FP64 path is
    deterministic), and the per-cell |dVF| of the two paths after the first mark."""
    marks = sorted(k for k in DRIFT_MARKS if k <= steps)
    rec = None
    try:
        rec = json.load(open(drift_record_path(m.Nx)))
        if not all(str(k) in rec["mass"] for k in marks) or rec["dt"] != dt:
            rec = None
    except (OSError, ValueError, KeyError):
        rec = None
    first = marks[0]
    g64, m64 = drift_run(m, centres, radii, dt, first if rec else steps, "fp64", VF0, set(marks))
    g32, m32 = drift_run(m, centres, radii, dt, first, "mixed", VF0, set(marks))
    V64, V32 = m.interior(g64.download_vf()), m.interior(g32.download_vf())
    iface = (V64 >= m.VFlo) & (V64 <= m.VFhi)
    d = np.abs(V64 - V32)
    cell = {"step": first, "max_abs_dVF": float(d.max()), "p99_abs_dVF_interface": float(np.percentile(d[iface], 99))}
    g64.close()
    for s in range(first, steps):
        g32.case_deformation3d((s + 0.5) * dt, 3.0)
        M = g32.step(dt)
        if s + 1 in marks:
            m32[s + 1] = M
    g32.close()
    # a second mixed run: its work lists are filled by atomics, so the last bits may differ
    g32b, m32b = drift_run(m, centres, radii, dt, steps, "mixed", VF0, set(marks))
    g32b.close()
    source = "live FP64 run"
    if rec:
        ref = {k: rec["mass"][str(k)] for k in marks}
        source = ("tests/golden/drift_fp64_%d.json (made by %s); its step-%d mass reproduced live: %s"
                  % (m.Nx, rec["made_by"], first, "bit-identical" if ref[first] == m64[first] else
                     "DIFFERENT (%r live)" % m64[first]))
    else:
        ref = m64
    curve = {str(k): abs(m32[k] - ref[k]) / abs(ref[k]) for k in marks}
    curve_b = {str(k): abs(m32b[k] - ref[k]) / abs(ref[k]) for k in marks}
    spread = max(abs(m32[k] - m32b[k]) / abs(ref[k]) for k in marks)
    return {"steps": steps, "field": "Deformation3D T=3 at t_n + dt/2 (time-varying)",
            "mass_rel_diff_mixed_vs_fp64": curve, "mass_rel_diff_mixed_vs_fp64_second_run": curve_b,
            "mixed_run_to_run_mass_spread": spread, "fp64_masses": source, "per_cell": cell}


def make_ctx(m, centres, radii, precision, t, VF0=None):
    """Context holding the workload's state: the sphere union generated on the device, or a
    copy of an already generated VF0 (host array)."""
    from ns_multiphase_gb300.slvof import SLVOF
    g = SLVOF(m, precision)
    if VF0 is None:
        g.case_vf_spheres(centres, radii, nF=20, dims=3)
    else:
        g.upload_vf(VF0)
        g.vf_ghost_fill()
    g.init_state(band=True)
    g.case_deformation3d(t, 3.0)
    return g


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": num(rows[0][2]),
                "reasons": reasons, "samples": len(rows)}


def timed_steps(g, dt, steps, torch):
    """K resident steps bracketed by synchronize + CUDA events on the library's stream."""
    stream = torch.cuda.current_stream()
    g.set_stream(stream.cuda_stream)
    stage = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        g.step(dt, band=True, mass=True)
        for k, v in g.stage_ms().items():
            stage[k] = stage.get(k, 0.0) + v
    e1.record(stream)
    torch.cuda.synchronize()
    g.set_stream(None)
    return e0.elapsed_time(e1), {k: v / steps for k, v in stage.items()}


def adjoint_timing(g, m, dt, steps, torch, next_ptr=None):
    """Mean time of the reverse of one step (slvof_adjoint_step, or slvof_adjoint_step_next with
    the step's result on the device) from the context's current state, seeded with dL/dVF =
    seeded normal weights on the interior; CUDA events on the launching stream, one untimed
    call first."""
    gT = m.vf_array()
    m.interior(gT)[...] = np.random.default_rng(SEED).standard_normal((m.Nx, m.Ny, m.Nz))
    g.adjoint_set_vf(gT)
    g.adjoint_zero_velocity()
    g.adjoint_step(dt, next_ptr)
    stream = torch.cuda.current_stream()
    g.set_stream(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        g.adjoint_step(dt, next_ptr)
    e1.record(stream)
    torch.cuda.synchronize()
    g.set_stream(None)
    return e0.elapsed_time(e1) / steps


def adjoint_mixed(g, m, dt, steps, torch):
    """The mixed context's reverse of one step from its current state, given the step's result
    (as a rollout's reverse pass has it) and recomputing it."""
    nvf = int(np.prod(m.vf_shape))
    s0 = torch.empty(nvf, dtype=torch.float64, device="cuda")
    s1 = torch.empty_like(s0)
    g.copy_vf_device(s0.data_ptr())
    g.step(dt, band=True, mass=False)
    g.copy_vf_device(s1.data_ptr())
    g.load_vf_device(s0.data_ptr())
    g.prepare()
    given = adjoint_timing(g, m, dt, steps, torch, s1.data_ptr())
    recompute = adjoint_timing(g, m, dt, steps, torch, None)
    return given, recompute


class CpuSample:
    """The CPU restatement of one step on a centred z-slab of the state, all host threads:
    the SL update of the slab's band cells (src/Transport.jl:108-151), the VF ghost fill
    (:179-181), ELVIRA (src/ELVIRA.jl:6-55), computePLIC! (src/VF.jl:94-103) and computeBand!
    (src/VF.jl:16-74) of the slab's cells; the ghost fill runs on the whole grid.  The slab's
    layer count is set once so that a sample takes about budget_s / 4."""

    def __init__(self, m, VF, uf, vf, wf, nx, ny, nz, D, band, dt):
        from oracle.oracle import Oracle
        self.o = Oracle(m)
        self.m, self.dt = m, dt
        self.state = (VF, uf, vf, wf, nx, ny, nz, D, band)
        self.VFn = m.vf_array()
        self.out = (m.cell_array(), m.cell_array(), m.cell_array(), m.cell_array(), band.copy(order="F"))
        self.nk = 2

    def run(self):
        VF, uf, vf, wf, nx, ny, nz, D, band = self.state
        o, N, nk = self.o, self.m.Nz, self.nk
        klo = N // 2 - nk // 2 + 1
        khi = klo + nk - 1
        np.copyto(self.VFn, VF)  # cells outside the slab keep their VF, as non-band cells do
        nx2, ny2, nz2, D2, band2 = self.out
        t0 = time.perf_counter()
        f, _ = o.transport(self.dt, VF, uf, vf, wf, nx, ny, nz, D, band, klo=klo, khi=khi, VFnew=self.VFn)
        o.vf_ghost_fill(self.VFn)
        o.ELVIRA(self.VFn, nx2, ny2, nz2, klo=klo, khi=khi)
        o.computePLIC_slab(nx2, ny2, nz2, self.VFn, D2, klo, khi)
        o.computeBand_slab(self.VFn, band2, klo, khi)
        sec = time.perf_counter() - t0
        if f:
            raise RuntimeError(f"restatement flags {f}")
        return self.m.Nx * self.m.Ny * nk / sec, sec

    def calibrate(self, budget_s):
        N = self.m.Nz
        while True:
            _, sec = self.run()
            if sec >= budget_s / 4 or self.nk >= N:
                return
            self.nk = min(N, max(self.nk * 2, int(self.nk * budget_s / 4 / max(sec, 1e-3))))

    def describe(self, sec):
        return (f"SL update + VF ghost fill + ELVIRA + computePLIC! + computeBand! of {self.nk} centred z-layers "
                f"of the {self.m.Nx}^3 state ({sec:.1f} s), C++ restatement, OpenMP on all host cores")


def cpu_sample(m, VF, uf, vf, wf, nx, ny, nz, D, band, dt, budget_s):
    """One calibrated CpuSample: (cell-updates/s, description)."""
    cs = CpuSample(m, VF, uf, vf, wf, nx, ny, nz, D, band, dt)
    cs.calibrate(budget_s)
    v, sec = cs.run()
    return v, cs.describe(sec)


def op_counts(m, VF, uf, vf, wf, nx, ny, nz, D, band, dt, counters, n_if):
    """Algorithmic operations of one step: the restatement's ELVIRA, plane-constant and SL
    paths run with a counting scalar (each +, -, *, / and each sqrt, cbrt, acos, sin, cos) on a
    seeded sample of this state's interface cells and band cells, scaled to the step by its own
    work-list sizes.  Pure cells do no arithmetic (axis normals, constant plane distances)."""
    from oracle.oracle import Oracle, build
    build()
    g = m.nghost
    vfi = m.interior(VF)
    iface = np.flatnonzero(((vfi >= m.VFlo) & (vfi <= m.VFhi)).ravel(order="F"))
    bnd = np.flatnonzero((np.abs(band[g:g + m.Nx, g:g + m.Ny, g:g + m.Nz]) <= m.nband).ravel(order="F"))
    rng = np.random.default_rng(SEED)
    si = np.sort(rng.choice(iface, min(n_if, len(iface)), replace=False))
    sb = np.sort(rng.choice(bnd, min(2 * n_if, len(bnd)), replace=False))
    t0 = time.perf_counter()
    c = Oracle(m).count_ops(dt, VF, uf, vf, wf, nx, ny, nz, D, si, sb)
    sec = time.perf_counter() - t0
    per = {"elvira_per_interface_cell": c["elvira"] / len(si), "plic_per_interface_cell": c["plic"] / len(si),
           "sl_per_band_cell": c["sl"] / len(sb)}
    n_if_step, n_band_step = counters["interface_cells"], counters["band_cells"]
    parts = {"elvira": per["elvira_per_interface_cell"] * n_if_step,
             "plic": per["plic_per_interface_cell"] * n_if_step,
             "sl": per["sl_per_band_cell"] * n_band_step}
    return {"ops_per_step": sum(parts.values()), "parts": parts, "per_cell": per,
            "sample": f"{len(si)} interface and {len(sb)} band cells of the FP64 state after the accuracy steps "
                      f"(seed {SEED}), counted on one host thread in {sec:.1f} s; scaled by this step's "
                      f"{n_if_step} interface and {n_band_step} band cells"}


def workload_config(n):
    """config of both arms' JSON lines: the workload and the L2 note, nothing else."""
    return {"workload": f"SL-VOF transport step, {n}^3, 200 spheres seed {SEED}, Deformation3D T=3, CFL 0.5, "
                        f"nband 1, RK4, 5 tets",
            "l2": "every field > L2 (no flush needed)"}


def reference_arm(args, rank):
    """--impl reference: the CPU restatement of the reference (the Julia reference cannot run
    here) on the host cores, for the same workload.  Nothing here loads the GPU library: the
    state is generated on the CPU (VFsphere's rule, then computeBand!, ELVIRA and computePLIC!
    of the whole grid by the restatement), and each step is a bounded sample of the step's
    stages on a centred z-slab (CpuSample)."""
    from oracle.oracle import Oracle, build
    from ns_multiphase_gb300 import cases
    build()
    if rank != 0:
        return
    m, centres, radii, dt = workload(args.n)
    o = Oracle(m)
    VF = o.vf_spheres(centres, radii, nF=20, dims=3)
    band, nx, ny, nz, D = o.init_state(VF)
    uf, vf, wf = cases.deformation3d_faces(m, 0.5 * dt, 3.0)
    cs = CpuSample(m, VF, uf, vf, wf, nx, ny, nz, D, band, dt)
    cs.calibrate(min(args.cpu_seconds, 120.0 / max(1, args.steps)))
    for _ in range(args.warmup):
        cs.run()
    vals, secs = [], []
    for _ in range(max(1, args.steps)):
        v, sec = cs.run()
        vals.append(v)
        secs.append(sec)
    value = statistics.median(vals)
    cores = os.cpu_count()
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * m.Nx * m.Ny * m.Nz / value,
            "higher_is_better": True, "scaling": "weak", "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.n),
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                             "sample": cs.describe(statistics.median(secs)) + " (the Julia reference is not "
                                       "installed: no julia on this machine or the GPU box)"},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "vs_baseline": None}
    print(json.dumps(line), flush=True)


def stage_run(args):
    """Small workloads for kernel-profiler captures: no timing legs and no JSON line."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from ns_multiphase_gb300 import cases
    from ns_multiphase_gb300.mesh import Mesh
    torch.cuda.set_device(0)
    if args.stage_run == "fd-adjoint":
        # 64^3, pressure_scheme "finite-difference", 12 spheres (seed 11, nF 6), Deformation3D
        # at t = 0.3 (T = 3), CFL 0.5; reverse of one step seeded with normal weights (seed 1)
        from ns_multiphase_gb300.slvof import SLVOF
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
            print("adjoint step (fd, fp64, 64^3)", round(1e3 * (time.perf_counter() - t0), 3), "ms", flush=True)
        g.close()
        return
    m, centres, radii, dt = workload(args.n)
    g = make_ctx(m, centres, radii, args.precision, 0.5 * dt)
    for s in range(args.steps):
        g.step(dt)
        print(s, {k: round(v, 3) for k, v in g.stage_ms().items()}, g.counters(), flush=True)
    if args.stage_run == "adjoint":
        nvf = int(np.prod(m.vf_shape))
        s0 = torch.empty(nvf, dtype=torch.float64, device="cuda")
        s1 = torch.empty_like(s0)
        g.copy_vf_device(s0.data_ptr())
        g.step(dt, band=True, mass=False)
        g.copy_vf_device(s1.data_ptr())
        g.load_vf_device(s0.data_ptr())
        g.prepare()
        gT = m.vf_array()
        m.interior(gT)[...] = np.random.default_rng(SEED).standard_normal((m.Nx, m.Ny, m.Nz))
        g.adjoint_set_vf(gT)
        g.adjoint_zero_velocity()
        for s in range(args.steps):
            g.adjoint_step(dt, s1.data_ptr())
            print("adjoint", s, round(g.last_kernel_ms(), 3), flush=True)
    g.close()


def main():
    args = parse()
    if args.stage_run:
        stage_run(args)
        return
    if args.drift_record:
        drift_record(args)
        return
    ws, rank, local = dist_env()
    if args.impl == "reference":
        # the CPU restatement on the host cores: rank 0 alone, no GPU and no process group
        if rank == 0:
            reference_arm(args, rank)
        return
    import torch
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__
    __graft_entry__.build()
    from ns_multiphase_gb300.slvof import SLVOF
    torch.cuda.set_device(local)
    m, centres, radii, dt = workload(args.n)
    cells = m.Nx * m.Ny * m.Nz

    # ---- mixed precision, resident (value) -----------------------------------------------
    g = make_ctx(m, centres, radii, "mixed", 0.5 * dt)
    VF0 = g.download_vf() if rank == 0 else None
    for _ in range(args.warmup):
        g.step(dt, band=True, mass=True)
    if ws > 1:
        tdist.barrier()
    with Clocks(local) as ck:
        ms, stage = timed_steps(g, dt, args.steps, torch)
    clocks = ck.summary()
    counters = g.counters()
    value, ms = aggregate_rate(ms, cells, args.steps, ws, "cuda")
    ms_step = ms / args.steps
    g.close()

    out = None
    if rank == 0:
        # ---- mixed-vs-FP64 mass over the drift run ------------------------------------------
        accuracy = drift_leg(m, centres, radii, dt, args.drift_steps, VF0)
        # ---- FP64 arm on the benchmark state, and the reverse passes ---------------------------
        g64 = make_ctx(m, centres, radii, "fp64", 0.5 * dt, VF0)
        g32 = make_ctx(m, centres, radii, "mixed", 0.5 * dt, VF0)
        for s in range(3):
            g64.step(dt)
            g32.step(dt)
        ms64, stage64 = timed_steps(g64, dt, args.fp64_steps, torch)
        value64 = cells * args.fp64_steps / (ms64 / 1e3)
        adj32, adj32_re = adjoint_mixed(g32, m, dt, args.adj_steps, torch)
        g32.close()
        adj64 = adjoint_timing(g64, m, dt, args.adj_steps, torch)
        adjoint = {"workload": f"{m.Nx}^3 benchmark state after 3 steps, reverse of one step seeded with "
                               "normal weights on every interior cell",
                   "adj_ms_per_step": adj32, "fwd_mixed_ms_per_step": ms_step, "adj_over_fwd_mixed": adj32 / ms_step,
                   "mixed": "boundary-form reverse (FP32 cell-local geometry, FP64 accumulation), the step's "
                            "result given as a rollout holds it (slvof_adjoint_step_next)",
                   "adj_recompute_ms_per_step": adj32_re,
                   "adj_recompute_over_fwd_mixed": adj32_re / ms_step,
                   "adj_fp64_ms_per_step": adj64, "fwd_fp64_ms_per_step": ms64 / args.fp64_steps,
                   "adj_over_fwd_fp64": adj64 / (ms64 / args.fp64_steps),
                   "fp64": "clip trees run backwards in FP64 (recorded candidate lanes, recomputed pre-images)",
                   "fd_check": "tests/test_gpu_adjoint.py: central differences (h=1e-6) of the CPU restatement, "
                               "1e-6 relative to the largest sampled derivative, FP64 and mixed contexts"}
        VF = g64.download_vf()
        nx, ny, nz = g64.download_normals()
        D = g64.download_plic()
        band = g64.download_band()
        g64.close()

        # ---- e2e through the host-buffer drop-in -------------------------------------------
        from ns_multiphase_gb300 import cases
        uf, vf, wf = cases.deformation3d_faces(m, 0.5 * dt, 3.0)
        shp = tuple(reversed(m.cell_shape))

        def pinned(a, shape):
            t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
            h = t.numpy().T
            if a is not None:
                h[...] = a
            return t, h
        tu, huf = pinned(uf, shp)
        tv, hvf = pinned(vf, shp)
        tw, hwf = pinned(wf, shp)
        tV, hVF = pinned(None, tuple(reversed(m.vf_shape)))
        def e2e_run(defer):
            ge = make_ctx(m, centres, radii, "mixed", 0.5 * dt, VF0)
            for _ in range(max(5, args.warmup)):  # warm: first touches of the pinned buffers
                ge.step_host(dt, huf, hvf, hwf, hVF, defer=defer)
            torch.cuda.synchronize()
            per_step = []
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                t1 = time.perf_counter()
                ge.step_host(dt, huf, hvf, hwf, hVF, defer=defer)  # synchronous: returns with VF on the host
                per_step.append(time.perf_counter() - t1)
            e2e_s = time.perf_counter() - t0
            ge.close()
            return {"value": cells * args.e2e_steps / e2e_s, "unit": "cell-updates/s",
                    "ms_per_step": {"mean": 1e3 * e2e_s / args.e2e_steps, "min": 1e3 * min(per_step),
                                    "median": 1e3 * statistics.median(per_step), "max": 1e3 * max(per_step),
                                    "each": [round(1e3 * t, 3) for t in per_step]}}

        # each call uploads its velocities while the previous state's normals, PLIC and band
        # are built (SLVOF_STEP_DEFER): in the steady state every step still does all the work
        e2e = e2e_run(True)
        e2e.update({"h2d_bytes_per_step": int(3 * huf.nbytes), "d2h_bytes_per_step": int(hVF.nbytes + 8),
                    "api": "slvof_step_host with SLVOF_STEP_DEFER (pinned host face velocities in, VF + mass "
                           "out; the normals, PLIC and band of each state built beside the next upload)",
                    "without_defer": e2e_run(False)})

        # ---- CPU restatement on a bounded slab ---------------------------------------------
        cpu = None
        ops = None
        if not args.no_cpu:
            # the CPU leg also counts the reference algorithm's operations on a sample
            if args.count_sample > 0:
                ops = op_counts(m, VF, uf, vf, wf, nx, ny, nz, D, band, dt, counters, args.count_sample)
            from oracle.oracle import build
            build()
            v, desc = cpu_sample(m, VF, uf, vf, wf, nx, ny, nz, D, band, dt, args.cpu_seconds)
            cpu = {"value": v, "unit": "cell-updates/s", "cores": os.cpu_count(), "kind": "port", "sample": desc}

        # ---- roofline of the dominant kernel -----------------------------------------------
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except OSError:
            pass
        hbm = peaks.get("hbm_gbs", 6800.0)
        dom = max(stage, key=stage.get)
        alg = algorithmic_bytes(m, dom, counters)
        achieved = alg / (stage[dom] / 1e3) / 1e9 if stage[dom] > 0 else 0.0
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": profiled_traffic(dom),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
                "algorithmic_bytes": alg, "kernel_ms": stage[dom],
                "note": "sl_update = k_flux_lists + k_flux_nodes + k_flux_faces + k_flux_clip + k_flux_cells + "
                        "k_sl32_clipw (the flux form); issue-, latency- and FP64-bound, not HBM-bound "
                        "(profiles/sl_update_256_mixed_dram.txt, profiles/k_flux_clip_128_mixed_ncu.txt); the HBM "
                        "fraction is reported per the contract",
                "step": {"algorithmic_bytes": 28 * cells, "achieved_gbs": 28 * cells / (ms_step / 1e3) / 1e9,
                         "frac": 28 * cells / (ms_step / 1e3) / 1e9 / hbm}}
        if ops is not None:
            # CUDA-core peaks from the SM count and the measured maximum SM clock: 128 FP32 lanes
            # per SM, an FMA counting two operations; GB300's FP64 rate is 1/64 of that
            sms = torch.cuda.get_device_properties(0).multi_processor_count
            mhz = peaks.get("sm_max_mhz", 2070.0)
            fp32 = sms * 128 * 2 * mhz * 1e6 / 1e12
            fp64 = fp32 / 64
            ms64_step = ms64 / args.fp64_steps

            def rate(n, ms_):
                return n / (ms_ / 1e3) / 1e12
            roof["compute"] = {
                "unit": "TFLOP/s", "ops_per_step": ops["ops_per_step"], "per_cell": ops["per_cell"],
                "sample": ops["sample"],
                "peak_fp32": fp32, "peak_fp64": fp64,
                "peak_source": f"nominal: {sms} SMs x 128 lanes x 2 x {mhz:.0f} MHz (FP32), FP64 at 1/64",
                "kernel": {"stage": dom, "ops": ops["parts"]["sl"], "achieved": rate(ops["parts"]["sl"], stage[dom]),
                           "frac_fp32": rate(ops["parts"]["sl"], stage[dom]) / fp32},
                "step_mixed": {"achieved": rate(ops["ops_per_step"], ms_step),
                               "frac_fp32": rate(ops["ops_per_step"], ms_step) / fp32},
                "step_fp64": {"achieved": rate(ops["ops_per_step"], ms64_step),
                              "frac_fp64": rate(ops["ops_per_step"], ms64_step) / fp64},
                "note": "operations of the reference's algorithm (the restatement with a counting scalar); the "
                        "mixed ELVIRA scores candidates with a closed-form plane/cube volume instead of five tet "
                        "clips, so its share of the mixed step's rate is an effective rate"}
        out = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
               "config": workload_config(args.n), "precision": "mixed",
               "parallelism": "replicas" if ws > 1 else "1 GPU",
               "fp64": {"value": value64, "ms_per_step": ms64 / args.fp64_steps, "speedup_mixed": value / ws / value64,
                        "stages_ms": stage64},
               "accuracy": accuracy,
               "adjoint": adjoint,
               "stages_ms": stage,
               "stages_note": "CUDA events per stage on the stream each stage runs on; the band runs on a second "
                              "stream beside elvira_candidates and plic, so its span overlaps theirs and the "
                              "stages sum to more than ms_per_step",
               "work_lists": counters, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
               "gpu_launches": launches_per_step(m) * args.steps}
        print(json.dumps(out), flush=True)
    if ws > 1:
        tdist.barrier()
        tdist.destroy_process_group()


def algorithmic_bytes(m, stage, ctr):
    """Minimum unique HBM bytes of one launch of a stage (mixed-precision storage), from the
    work-list sizes of the step: each band cell of the SL update reads its FP32 face velocities
    (12 B) and donor plane (16 B) and writes VF (8 B); each ELVIRA interface cell reads VF and
    writes three normals (32 B)."""
    interior = m.Nx * m.Ny * m.Nz
    ncell = int(np.prod(m.cell_shape))
    table = {
        "sl_classify": interior * (2 + 8 + 8),
        "sl_update": ctr.get("band_cells", interior) * (12 + 16 + 8),
        "vf_ghost": (int(np.prod(m.vf_shape)) - interior) * 16,
        "elvira_pure": interior * (8 + 24),
        "elvira_candidates": ctr.get("interface_cells", interior) * (8 + 24),
        "normal_ghost": (ncell - interior) * 24,
        "plic": ncell * (8 * 4 + 8 + 16 + 1),
        "band": interior * (8 + 2 * 2 * 2),
        "mass": 8 * 1024,
    }
    return table.get(stage, interior * 28)


def profiled_traffic(stage):
    """dram read+write bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "sl_update_256_mixed_dram.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == "traffic_bytes" and parts[1] == stage:
                return float(parts[2])
    except OSError:
        pass
    return None


def launches_per_step(m):
    # mixed step: classify; SL update (flux lists, nodes, faces, clip, cells, near-pure cells);
    # VF ghost; ELVIRA pure; ELVIRA candidates (FP32 scoring, FP64 arbitration, FP64 winner);
    # normal ghost; PLIC (pure, Newton); band (first + ghost + nband*(sweep + ghost)); mass final
    return 1 + 6 + 1 + 1 + 3 + 1 + 2 + 2 + 2 * int(m.nband) + 1


if __name__ == "__main__":
    main()
