"""torch.autograd binding: a 100-step cart-pole rollout built from ten checkpointed 10-step
segment tapes, differentiated by the adjoint sweeps, against the oracle's adjoint of the
single 100-step tape and against central finite differences."""
import os

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import workloads as W

from helpers import assert_adjoint_close, assert_close, magnitudes, value_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
NTHREADS = os.cpu_count() or 1


def test_checkpointed_rollout_gradient(gpu_lib):
    from casadi_gb300.autograd import CheckpointedRollout
    n = 2048
    x0, U = W.cartpole_inputs(n, steps=100, seed=4)
    U = U * 0.1  # keep the 100-step trajectories bounded
    tx = torch.from_numpy(x0).cuda().requires_grad_(True)
    tu = torch.from_numpy(U).cuda().requires_grad_(True)
    roll = CheckpointedRollout(steps=100, every=10)
    xN, cost = roll(tx, tu)
    cost.sum().backward()
    gx, gu = tx.grad.cpu().numpy(), tu.grad.cpu().numpy()
    F = W.cartpole_rollout(100)
    wres = O.eval(F.tape, [x0, U], n, NTHREADS)
    vb = value_bounds(F.tape, [x0, U], n)
    assert_close(xN.detach().cpu().numpy(), wres[0], "xN", bound=vb[0])
    assert_close(cost.detach().cpu().numpy(), wres[1], "cost", bound=vb[1])
    seeds = [np.zeros((1, 4, n)), np.ones((1, 1, n))]
    _, was = O.reverse(F.tape, [x0, U], seeds, n, NTHREADS)
    _, mag = magnitudes(O.reverse, F.tape, [x0, U], seeds, n, NTHREADS)
    # a 1-ulp change of one sin/cos result moves this gradient by up to ~6e-12 of itself (100
    # RK4 steps): element-wise within 1e-13 of the magnitude of the chain-rule terms plus 4 ulps
    # of every libm result propagated through the adjoint Function f.reverse(1)
    assert_adjoint_close([gx, gu], [was[0][0], was[1][0]], [mag[0][0], mag[1][0]], F, [x0, U],
                         [s[0] for s in seeds], "d cost / d (x0, U)")
    # central differences on a few instances and coordinates
    h = 1e-6
    m = 4
    for blk, row in ((0, 2), (1, 0), (1, 57)):
        p = [x0[:, :m].copy(), U[:, :m].copy()]
        q = [x0[:, :m].copy(), U[:, :m].copy()]
        p[blk][row] += h
        q[blk][row] -= h
        fd = (O.eval(F.tape, p, m)[1][0] - O.eval(F.tape, q, m)[1][0]) / (2 * h)
        g = (gx if blk == 0 else gu)[row, :m]
        assert np.max(np.abs(fd - g) / np.maximum(np.abs(g), 1.0)) < 1e-4


def test_tape_apply_gradcheck(gpu_lib):
    from casadi_gb300 import runtime as R
    from casadi_gb300.autograd import tape_apply
    tape = R.CudaTape(W.cartpole_step())
    x0, u = W.cartpole_inputs(3, steps=1, seed=1)
    tx = torch.from_numpy(x0).cuda().requires_grad_(True)
    tu = torch.from_numpy(u).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda a, b: tape_apply(tape, a, b)[0], (tx, tu),
                                    eps=1e-6, atol=1e-7, rtol=1e-6)
