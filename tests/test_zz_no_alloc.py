"""The allocation-free adjoint entry point (casadi_gb300_reverse_noalloc).

Callers that cannot allocate device memory when they need derivatives (a solver inside a CUDA
graph capture, a real-time loop that forbids allocation after start-up, a plugin whose host
framework owns the allocator) use this entry point: its scratch is a fixed 64 MiB device array
inside the library. These tests call it through the C ABI and check it against the regular
adjoint entry point, on two calls in a row (the shared array keeps the previous call's
contents), and check that a call needing more than the fixed scratch is refused.

This file is collected last so that a run stopping at its first failure has already run
every other test.
"""
import ctypes as ct

import numpy as np
import pytest

from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import RTOL, assert_close

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _ptrs(ts):
    return R._ptr_array(ts)


def _noalloc(ct_tape, args, aseeds, n, nadj):
    res = [torch.full((k, n), np.nan, dtype=torch.float64, device="cuda")
           for k in ct_tape.nnz_out]
    asens = [torch.full((nadj, k, n), np.nan, dtype=torch.float64, device="cuda")
             for k in ct_tape.nnz_in]
    st = R.load().casadi_gb300_reverse_noalloc(
        ct_tape.id, n, n, nadj, _ptrs(args), _ptrs(res), _ptrs(aseeds), _ptrs(asens),
        ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    R.check(st)
    ct_tape.sync()
    return [r.cpu().numpy() for r in res], [a.cpu().numpy() for a in asens]


@pytest.mark.parametrize("steps,n,nadj", [(20, 1024, 1), (4, 3001, 2)])
def test_noalloc_matches_reverse_twice(gpu_lib, steps, n, nadj):
    F = W.cartpole_rollout(steps)
    tape = R.CudaTape(F)
    rng = np.random.default_rng(steps)
    args = [torch.from_numpy(a).cuda() for a in W.cartpole_inputs(n, steps=steps, seed=7)]
    aseeds = [torch.from_numpy(rng.standard_normal((nadj, k, n))).cuda() for k in F.tape.nnz_out]
    res_ref, asens_ref = tape.reverse(args, aseeds)
    res_ref = [r.cpu().numpy() for r in res_ref]
    asens_ref = [a.cpu().numpy() for a in asens_ref]
    for call in range(2):
        res, asens = _noalloc(tape, args, aseeds, n, nadj)
        for g, w in zip(res, res_ref):
            assert_close(g, w, "values, call %d" % call, rtol=RTOL)
        for g, w in zip(asens, asens_ref):
            assert_close(g, w, "adjoint, call %d" % call, rtol=RTOL)


def test_noalloc_refuses_oversized_call(gpu_lib):
    F = W.cartpole_rollout(20)
    tape = R.CudaTape(F)
    n = (64 << 20) // (8 * tape.n_partials) + 64  # one wave more than the fixed scratch holds
    st = R.load().casadi_gb300_reverse_noalloc(tape.id, n, n, 1, None, None, None, None, None)
    assert st == -5
    msg = R.load().casadi_gb300_last_error().decode()
    assert "allocation-free adjoint" in msg and str(64 << 20) in msg
