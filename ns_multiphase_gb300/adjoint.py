"""Reverse-mode rollouts of the SL-VOF step with VF checkpoints.

A rollout is ``steps`` calls of the step, each with its own face velocities.  The forward
pass keeps VF on the device every ``every`` steps (the checkpoints); the reverse pass walks
the segments backwards, recomputes each segment's states from its checkpoint (pre-images,
normals, PLIC planes and band are recomputed, not stored), and runs the step's reverse
(``slvof_adjoint_step_next``, given the step's result from the stored states) from the last
state to the first.  This is the pullback a Julia
caller would register as a ChainRules ``rrule`` around its loop over ``transport!``; here it
is the Python analogue of a ``torch.autograd.Function`` over the whole rollout.

Device memory for checkpoints comes from torch (plumbing only: the kernels are the
library's).  The velocity derivatives are accumulated over all steps when
``per_step=False`` (the derivative with respect to a perturbation added to every step's
velocity), or returned step by step.
"""
from __future__ import annotations

import time
from typing import Callable, Optional

import numpy as np

from .slvof import SLVOF


class Rollout:
    """Forward steps with device checkpoints and their reverse pass on one SLVOF context.

    velocity(n) returns the host face velocities (uf, vf, wf) of step n (Fortran-ordered
    cell arrays).  The context must hold the initial VF (ghosts filled) when forward() is
    called; forward() prepares it.
    """

    def __init__(self, solver: SLVOF, dt: float, steps: int, velocity: Callable[[int], tuple], every: int = 10,
                 give_next: bool = True):
        import torch

        if steps < 1 or every < 1:
            raise ValueError("steps and every must be positive")
        self.s = solver
        self.dt = float(dt)
        self.steps = int(steps)
        self.every = int(every)
        self.velocity = velocity
        self.give_next = bool(give_next)  # hand each reverse step its step's result
        self.final = None
        self.torch = torch
        self.nvf = int(np.prod(solver.mesh.vf_shape))
        self.ckpt: dict[int, object] = {}
        self.fwd_ms = 0.0
        self.bwd_ms = 0.0
        self.adj_step_ms: list[float] = []
        self.fwd_step_ms: list[float] = []

    def _buf(self):
        return self.torch.empty(self.nvf, dtype=self.torch.float64, device="cuda")

    def _save(self):
        b = self._buf()
        self.s.copy_vf_device(b.data_ptr())
        return b

    def _load(self, b):
        self.s.load_vf_device(b.data_ptr())
        self.s.prepare()

    def forward(self):
        """Run the rollout; returns the final VF (host)."""
        t0 = time.perf_counter()
        self.s.prepare()
        self.ckpt = {}
        for n in range(self.steps):
            if n % self.every == 0:
                self.ckpt[n] = self._save()
            self.s.upload_velocity(*self.velocity(n))
            self.s.step(self.dt, band=True, mass=False)
            self.fwd_step_ms.append(self.s.last_kernel_ms())
        self.final = self._save()
        out = self.s.download_vf()
        self.fwd_ms = (time.perf_counter() - t0) * 1e3
        return out

    def backward(self, gVF_final: np.ndarray, per_step: bool = False):
        """dL/d(initial VF interior) and dL/d(face velocities) for dL/d(final VF) = gVF_final.

        Returns (gVF0, (guf, gvf, gwf)) with the velocity derivatives summed over the steps,
        or (gVF0, [(guf, gvf, gwf) per step]) when per_step is set.
        """
        t0 = time.perf_counter()
        s = self.s
        s.adjoint_set_vf(gVF_final)
        s.adjoint_zero_velocity()
        per: list[Optional[tuple]] = [None] * self.steps
        starts = sorted(self.ckpt)
        for k0 in reversed(starts):
            k1 = min(k0 + self.every, self.steps)
            # recompute the segment's states from its checkpoint
            states = {k0: self.ckpt[k0]}
            if k1 - k0 > 1:
                self._load(self.ckpt[k0])
                for n in range(k0, k1 - 1):
                    s.upload_velocity(*self.velocity(n))
                    s.step(self.dt, band=True, mass=False)
                    states[n + 1] = self._save()
            for n in range(k1 - 1, k0 - 1, -1):
                self._load(states[n])
                s.upload_velocity(*self.velocity(n))
                nxt = states.get(n + 1, self.ckpt.get(n + 1, self.final if n + 1 == self.steps else None))
                s.adjoint_step(self.dt, nxt.data_ptr() if (self.give_next and nxt is not None) else None)
                self.adj_step_ms.append(s.last_kernel_ms())
                if per_step:
                    _, gu, gv, gw = s.adjoint_get()
                    per[n] = (gu, gv, gw)
                    s.adjoint_zero_velocity()
        s.adjoint_fold()
        gVF0, gu, gv, gw = s.adjoint_get()
        self.bwd_ms = (time.perf_counter() - t0) * 1e3
        m = s.mesh
        interior = np.zeros_like(gVF0)
        m.interior(interior)[...] = m.interior(gVF0)
        return interior, (per if per_step else (gu, gv, gw))
