"""Tapes with OP_CALL instructions (nested Functions): a 3-step cart-pole rollout written as
three calls of the one-step tape, inlined by the library. Its values equal three chained
evaluations of the step tape bit for bit, and its values and adjoint match the oracle's
evaluation of the same rollout built without calls."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import runtime as R
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W

from helpers import RTOL, assert_bitexact, assert_close, call_rollout, magnitudes, value_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_call_rollout_matches_chained_steps_and_oracle(gpu_lib):
    steps, n = 3, 2049
    step = R.CudaTape(W.cartpole_step())
    tape, calls = call_rollout(steps)
    ct = R.CudaTape(tape, calls=[(step, d, r) for d, r in calls])
    x0, U = W.cartpole_inputs(n, steps=steps, seed=13)
    args = [torch.from_numpy(x0).cuda(), torch.from_numpy(U).cuda()]
    xN = ct.eval(args)[0]
    # three chained evaluations of the step tape
    x = args[0]
    for k in range(steps):
        x = step.eval([x, args[1][k:k + 1].contiguous()])[0]
    assert_bitexact(xN.cpu().numpy(), x.cpu().numpy(), "inlined calls vs chained steps")
    # the same rollout built without calls, on the oracle
    F = W.cartpole_rollout(steps)
    want = O.eval(F.tape, [x0, U], n)[0]
    assert_close(xN.cpu().numpy(), want, "values vs oracle",
                 bound=value_bounds(F.tape, [x0, U], n)[0])
    seeds = np.random.default_rng(3).standard_normal((1, 4, n))
    _, asens = ct.reverse(args, [torch.from_numpy(seeds).cuda()])
    oseeds = [seeds, np.zeros((1, 1, n))]
    _, was = O.reverse(F.tape, [x0, U], oseeds, n)
    _, mag = magnitudes(O.reverse, F.tape, [x0, U], oseeds, n)
    for g, w, m in zip(asens, was, mag):
        assert_close(g.cpu().numpy(), w, "adjoint vs oracle", bound=RTOL * m)
    ct.sync()


def test_bad_call_tables_are_refused(gpu_lib):
    step = R.CudaTape(W.cartpole_step())
    tape, calls = call_rollout(1)
    with pytest.raises(R.CasadiGpuError):
        R.CudaTape(tape, calls=[(step, [0, 1, 2, 3, 99], calls[0][1])])  # dep slot out of range
