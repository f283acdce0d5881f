"""torch.autograd bindings over the tape sweeps.

``tape_apply(tape, *inputs)`` evaluates a registered tape on device tensors (forward = the
value sweep) and differentiates through it with the adjoint sweep (backward), like a CasADi
Function called inside an autograd graph. Inputs and outputs are float64 CUDA tensors of
shape ``(nnz, n)`` (instance-minor); the backward returns gradients of the same shapes.

Checkpointing: a long rollout written as a chain of segment tapes keeps only each segment's
inputs for the backward pass; the backward of a segment re-runs its value sweep (recording
partials) and its adjoint sweep. ``checkpointed_rollout`` builds the cart-pole rollout that
way: ``steps`` RK4 steps in segments of ``every`` steps.

This is the only module of the package that needs PyTorch's autograd; the sweeps themselves
are the CUDA library behind the C ABI.
"""
import torch

from . import runtime as R
from . import workloads as W


class _TapeFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, tape, *inputs):
        n = next(x.shape[-1] for x in inputs if x is not None)
        args = [None if x is None else x.contiguous() for x in inputs]
        res = tape.eval(args, n=n)
        ctx.tape = tape
        ctx.n = n
        ctx.save_for_backward(*[x if x is not None else torch.empty(0) for x in args])
        ctx.none = [x is None for x in args]
        return tuple(res)

    @staticmethod
    def backward(ctx, *grads):
        tape, n = ctx.tape, ctx.n
        saved = ctx.saved_tensors
        args = [None if ctx.none[j] else saved[j] for j in range(len(saved))]
        # adjoint seeds: one direction; outputs without a gradient are unseeded (null)
        aseeds = [None if g is None else g.contiguous().reshape(1, *g.shape) for g in grads]
        if all(s is None for s in aseeds):
            return (None,) + tuple(None for _ in args)
        _, asens = tape.reverse(args, aseeds, n=n)
        out = []
        for j, a in enumerate(asens):
            need = ctx.needs_input_grad[j + 1]
            out.append(a[0] if need else None)
        return (None,) + tuple(out)


def tape_apply(tape, *inputs):
    """Evaluate ``tape`` (a :class:`runtime.CudaTape`) on ``inputs``; differentiable."""
    return _TapeFn.apply(tape, *inputs)


class CheckpointedRollout:
    """Cart-pole rollout of ``steps`` RK4 steps as ``steps // every`` segment tapes of ``every``
    steps each: ``cost(x0, U) = sum_k ||x_k||^2 + 0.01 u_k^2``. Only segment boundaries are
    stored for the backward pass."""

    def __init__(self, steps=100, every=10):
        if steps % every:
            raise ValueError("steps must be a multiple of the checkpoint interval")
        self.steps, self.every = steps, every
        self.segment = R.CudaTape(W.cartpole_rollout(every))

    def __call__(self, x0, U):
        """x0: (4, n), U: (steps, n) float64 CUDA tensors -> (xN (4, n), cost (1, n))."""
        x = x0
        cost = None
        for s in range(self.steps // self.every):
            xn, c = tape_apply(self.segment, x, U[s * self.every:(s + 1) * self.every])
            cost = c if cost is None else cost + c
            x = xn
        return x, cost


def full_rollout_tape(steps=100):
    """The same rollout as one tape (no checkpoints), for comparison."""
    return W.cartpole_rollout(steps)
