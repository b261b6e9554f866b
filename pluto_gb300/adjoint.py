"""Differentiable multi-step rollout over the C ABI.

``Rollout`` advances a PLUTO domain through a fixed (frozen) sequence of time
steps on the GPU.  ``rollout(runner, vc, *faces)`` is a
``torch.autograd.Function``: its forward runs the steps and stores a
device-resident checkpoint every ``every`` steps (``pg_checkpoint_save``);
its backward walks the segments from last to first, recomputes the states
inside a segment from its checkpoint, and applies the hand-written adjoint of
each step (``pg_adjoint_step``) in reverse order.  The dt sequence is frozen:
the derivative is that of the state map for the given dts, which is what
PLUTO's own step computes for a given g_dt (Src/Time_Stepping/rk_step.c:27).

``tangent_linear`` runs the FP64 tangent-linear model (precision
"fp64_tangent") for the same dts: the directional derivative of the final
state along a direction of the initial state.

Tensors are CPU float64, as the C ABI takes host arrays (interior layout:
cells [8][nz][ny][nx], face d one longer along axis d).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib as L
from .solver import Solver


class Rollout:
    """One FP64 solver and a frozen dt sequence."""

    def __init__(self, spec: dict, dts, every: int = 16):
        self.spec = dict(spec)
        self.dts = [float(x) for x in dts]
        self.every = int(every)
        nseg = -(-len(self.dts) // self.every)
        if nseg + self.every > L.PG_MAX_CHECKPOINTS:
            raise ValueError("too many checkpoint slots for this many steps")
        self.solver = Solver(spec, "fp64")
        self.dims = self.solver.dims
        self.ct = self.solver.ct

    @property
    def nsteps(self) -> int:
        return len(self.dts)

    def face_list(self, faces):
        return [faces[d] if (self.ct and d < self.dims) else None for d in range(3)]

    def run(self, vc, faces, checkpoint: bool = False):
        s = self.solver
        s.upload(vc, self.face_list(faces))
        for q, dt in enumerate(self.dts):
            if checkpoint and q % self.every == 0:
                s.checkpoint_save(q // self.every)
            s.advance(dt)
        return s.download()

    def gradient(self, lvc, lfaces, slots: bool = True):
        """Adjoint of the whole rollout (after ``run(..., checkpoint=True)``).

        Per segment, from its checkpoint: with ``slots`` (and room on the
        device for one segment's steps) each step is recomputed once,
        saving its stage outputs (adjoint_forward), and the steps are then
        reversed from them (adjoint_reverse); otherwise the step states are
        rebuilt first and every adjoint_step recomputes its own step again.
        Both give the same gradient to round-off (the reversal's scatter adds
        are FP64 atomics, so no two runs agree to the last bit)."""
        s = self.solver
        s.adjoint_set(lvc, self.face_list(lfaces))
        n, e = self.nsteps, self.every
        nseg = -(-n // e)
        use_slots = slots and s.adjoint_slots(min(n, e))
        base = nseg  # checkpoint slots of the states inside one segment
        for seg in range(nseg - 1, -1, -1):
            q0, q1 = seg * e, min(n, seg * e + e)
            s.checkpoint_load(seg)
            if use_slots:
                for q in range(q0, q1):
                    s.adjoint_forward(self.dts[q], q - q0)
                for q in range(q1 - 1, q0 - 1, -1):
                    s.adjoint_reverse(self.dts[q], q - q0)
                continue
            for q in range(q0, q1 - 1):  # states q0+1 .. q1-1 from the checkpoint
                s.checkpoint_save(base + q - q0)
                s.advance(self.dts[q])
            s.checkpoint_save(base + q1 - 1 - q0)
            for q in range(q1 - 1, q0 - 1, -1):
                s.checkpoint_load(base + q - q0)
                s.adjoint_step(self.dts[q])
        if use_slots:
            s.adjoint_slots(0)
        return s.adjoint_get()


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, runner: Rollout, vc: torch.Tensor, *faces: torch.Tensor):
        ctx.runner = runner
        fin = [f.detach().numpy() if f is not None else None for f in faces]
        vT, fT = runner.run(vc.detach().numpy(), fin + [None] * (3 - len(fin)), checkpoint=True)
        outs = [torch.from_numpy(vT)]
        for d in range(len(faces)):
            outs.append(torch.from_numpy(fT[d]) if fT[d] is not None else None)
        ctx.nfaces = len(faces)
        return tuple(outs)

    @staticmethod
    def backward(ctx, gvc, *gfaces):
        runner = ctx.runner
        lvc = gvc.detach().numpy() if gvc is not None else np.zeros((8,) + tuple(reversed(runner.solver.nx)))
        lf = []
        for d in range(ctx.nfaces):
            g = gfaces[d] if d < len(gfaces) else None
            lf.append(g.detach().numpy() if g is not None else
                      (np.zeros(runner.solver.face_shape(d)) if (runner.ct and d < runner.dims) else None))
        gv, gf = runner.gradient(lvc, lf + [None] * (3 - len(lf)))
        grads = [torch.from_numpy(gv)]
        for d in range(ctx.nfaces):
            grads.append(torch.from_numpy(gf[d]) if gf[d] is not None else None)
        return (None, *grads)


def rollout(runner: Rollout, vc: torch.Tensor, *faces: torch.Tensor):
    """Differentiable rollout: returns (vc_T, *faces_T)."""
    return _RolloutFn.apply(runner, vc, *faces)


def tangent_linear(spec: dict, dts, vc, faces, dvc, dfaces, kink: bool = False):
    """FP64 tangent-linear model: (final state, its derivative along (dvc,
    dfaces)); with kink=True also the kink margin of the run (the smallest
    perturbation along the direction at which, to first order, some branch of
    some step switches; see Solver.tangent_kink)."""
    s = Solver(spec, "fp64_tangent")
    try:
        fl = [faces[d] if (s.ct and d < s.dims) else None for d in range(3)]
        dl = [dfaces[d] if (s.ct and d < s.dims) else None for d in range(3)]
        s.upload(vc, fl)
        s.tangent_upload(dvc, dl)
        if kink:
            s.tangent_kink(True)
        for dt in dts:
            s.advance(float(dt))
        margin = s.tangent_kink(False) if kink else None
        state = s.download()
        tangent = s.tangent_download()
    finally:
        s.close()
    return (state, tangent, margin) if kink else (state, tangent)


def _two_sum(a, b):
    """a + b as an unevaluated pair (sum, error), exactly (Knuth's TwoSum)."""
    t = a + b
    bb = t - a
    return t, (a - (t - bb)) + (b - bb)


def dd_perturbed_run(spec: dict, dts, vc, faces, dvc, dfaces, h: float):
    """The step in double-double arithmetic (precision "fp64_dd") over the
    frozen dt sequence from x + h*delta, the start formed exactly as a pair
    of doubles; returns the final cell state as (high parts, low parts).  For
    central differences with h far below FP64 resolution."""
    hv, lv = _two_sum(np.asarray(vc, dtype=np.float64), h * np.asarray(dvc, dtype=np.float64))
    hf, lf = [None] * 3, [None] * 3
    for d in range(3):
        if faces[d] is not None:
            hf[d], lf[d] = _two_sum(faces[d], h * dfaces[d])
    s = Solver(spec, "fp64_dd")
    try:
        fl = [hf[d] if (s.ct and d < s.dims) else None for d in range(3)]
        dl = [lf[d] if (s.ct and d < s.dims) else None for d in range(3)]
        s.upload(hv, fl)
        s.tangent_upload(lv, dl)
        for dt in dts:
            s.advance(float(dt))
        (h1, _), (l1, _) = s.download(), s.tangent_download()
    finally:
        s.close()
    return h1, l1


def cfl_dt_sequence(spec: dict, vc, faces, nsteps: int, first_dt: float, cfl: float,
                    cfl_max_var: float = 1.1):
    """The dt sequence PLUTO's main loop takes from this state (NextTimeStep,
    Src/main.c:459-532), recorded with single FP64 steps; returned frozen."""
    s = Solver(spec, "fp64")
    try:
        s.upload(vc, [faces[d] if (s.ct and d < s.dims) else None for d in range(3)])
        dts, dt = [], float(first_dt)
        for _ in range(nsteps):
            dts.append(dt)
            inv, _, _ = s.advance(dt)  # invDt_hyp, already divided by DIMENSIONS
            dt = min(cfl / inv, cfl_max_var * dt)
    finally:
        s.close()
    return dts
