"""torch.autograd wrapper of the reverse-mode C ABI, for analysis scripts.

``ProjectionSteps.apply(solver, t0, nsteps, every, u0, v0, w0, p0, alpha)``
runs ``nsteps`` projection steps (src/Timestep.cpp:97-141, the loop of
src/main.cpp:149-156) on a ``mifgpu.Solver`` from the given initial velocity
and pressure (float64 CPU tensors in the reference layout, shape (Ez, Ey, Ex))
and Taylor-Green forcing amplitude ``alpha`` (0-d tensor), and returns the
final (u, v, w, p). Its backward pass calls ``mifgpu_backward``: the
checkpointed discrete adjoint on the device. The solver's other fields are
scratch. The reference has no differentiation; this is an extension and is
not on the time-step path.
"""
from __future__ import annotations

import numpy as np
import torch

import mifgpu

_NAMES = ("u", "v", "w", "p")


def _np(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().cpu().numpy(), dtype=np.float64)


class ProjectionSteps(torch.autograd.Function):
    @staticmethod
    def forward(ctx, solver, t0, nsteps, every, u0, v0, w0, p0, alpha):
        solver.set_forcing_amplitude(float(alpha))
        for n, a in zip(_NAMES, (u0, v0, w0, p0)):
            solver.upload(n, _np(a))
        solver.run(float(t0), int(nsteps))
        outs = tuple(torch.from_numpy(solver.download(n)) for n in _NAMES)
        ctx.solver = solver
        ctx.args = (float(t0), int(nsteps), int(every), float(alpha))
        ctx.save_for_backward(u0, v0, w0, p0)
        return outs

    @staticmethod
    def backward(ctx, gu, gv, gw, gp):
        solver = ctx.solver
        t0, nsteps, every, alpha = ctx.args
        solver.set_forcing_amplitude(alpha)
        for n, a in zip(_NAMES, ctx.saved_tensors):
            solver.upload(n, _np(a))
        seeds = {n: (None if g is None else _np(g)) for n, g in zip(_NAMES, (gu, gv, gw, gp))}
        res = solver.backward(t0, nsteps, every, seeds)
        grads = [torch.from_numpy(solver.adjoint(n)) for n in _NAMES]
        dalpha = torch.tensor(res["dloss_dalpha"], dtype=torch.float64)
        return (None, None, None, None, *grads, dalpha)
