"""A thin torch.autograd.Function over the tape (quids_gpu_forward /
quids_gpu_simulate_backward_observable): the expected value of a built-in
observable after a run of rule ops, as a differentiable function of the
rule angles.  Used by the gradient tests."""
from __future__ import annotations

import numpy as np
import torch

import quids_gb300 as quids


def expected_value(initial_packed, build_ops, observable: int, max_num_object: int = quids.U64_MAX,
                   checkpoint_every: int = 1, ctx: quids.Context | None = None):
    """Returns f(angles) -> loss.  build_ops(angles as a numpy array) gives
    (ops, slots): the rules/modifiers of the run and, per angle use, (op
    index, component 0..2 = theta/phi/xi, angle index)."""

    class _Expected(torch.autograd.Function):
        @staticmethod
        def forward(fctx, angles):
            a = angles.detach().cpu().to(torch.float64).numpy()
            ops, slots = build_ops(a)
            tape = quids.Tape(ctx)
            final, _ = tape.forward(quids.it_t(tape.ctx, initial_packed), ops, max_num_object, checkpoint_every)
            fctx.tape, fctx.slots, fctx.n = tape, slots, len(a)
            return angles.new_tensor(quids.average_value(final, observable))

        @staticmethod
        def backward(fctx, gout):
            _, g = fctx.tape.backward_observable(observable)
            grad = np.zeros(fctx.n)
            for oi, comp, ai in fctx.slots:
                grad[ai] += g[oi, comp]
            return gout * torch.from_numpy(grad).to(gout.dtype)

    return _Expected.apply
