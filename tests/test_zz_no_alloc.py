"""The allocation-free adjoint entry point (casadi_gb300_reverse_noalloc).

Callers that cannot allocate device memory when they need derivatives (a real-time loop that
forbids allocation after start-up, a plugin whose host framework owns the device allocator)
use this entry point: its scratch is a fixed 64 MiB device array inside the library. These
tests call it through the C ABI on two calls in a row (the shared array keeps the previous
call's contents) and check it against the regular adjoint entry point and against the oracle:
values bit for bit, adjoints element-wise within 1e-13 of the magnitude of their chain-rule
terms (oracle.magnitude). They also check the value-only call (no adjoint directions), that a
call needing more than the fixed scratch is refused, and that a tape whose work vector does
not fit in shared memory -- where this entry point keeps it -- is refused with a clear error.

This file is collected last so that a run stopping at its first failure has already run
every other test.
"""
import ctypes as ct

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W

from helpers import assert_bitexact, same_bits

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

AD_RTOL = 1e-13


def _ptrs(ts):
    return R._ptr_array(ts)


def _noalloc(ct_tape, args, aseeds, n, nadj):
    res = [torch.full((k, n), np.nan, dtype=torch.float64, device="cuda")
           for k in ct_tape.nnz_out]
    asens = [torch.full((nadj, k, n), np.nan, dtype=torch.float64, device="cuda")
             for k in ct_tape.nnz_in]
    st = R.load().casadi_gb300_reverse_noalloc(
        ct_tape.id, n, n, nadj, _ptrs(args), _ptrs(res), _ptrs(aseeds) if nadj else None,
        _ptrs(asens) if nadj else None, ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    R.check(st)
    ct_tape.sync()
    return [r.cpu().numpy() for r in res], [a.cpu().numpy() for a in asens]


def _within(got, ref, mag, what):
    d = np.abs(got - ref)
    bad = ~(same_bits(got, ref) | (d <= AD_RTOL * mag))
    assert not bad.any(), "%s: %d of %d beyond %.0e x magnitude" % (what, int(bad.sum()),
                                                                     bad.size, AD_RTOL)


@pytest.mark.parametrize("steps,n,nadj", [(20, 1024, 1), (4, 3001, 2)])
def test_noalloc_matches_reverse_and_oracle_twice(gpu_lib, steps, n, nadj):
    F = W.cartpole_rollout(steps)
    tape = R.CudaTape(F)
    rng = np.random.default_rng(steps)
    hargs = W.cartpole_inputs(n, steps=steps, seed=7)
    hseeds = [rng.standard_normal((nadj, k, n)) for k in F.tape.nnz_out]
    args = [torch.from_numpy(a).cuda() for a in hargs]
    aseeds = [torch.from_numpy(s).cuda() for s in hseeds]
    res_ref, asens_ref = tape.reverse(args, aseeds)
    res_ref = [r.cpu().numpy() for r in res_ref]
    asens_ref = [a.cpu().numpy() for a in asens_ref]
    ores, oasens = O.reverse(F.tape, hargs, hseeds, n)
    with O.magnitude():
        _, mag = O.reverse(F.tape, hargs, hseeds, n)
    bound = O.libm_bound(F.tape, hargs, n)
    for call in range(2):
        res, asens = _noalloc(tape, args, aseeds, n, nadj)
        for g, w in zip(res, res_ref):
            assert_bitexact(g, w, "values vs casadi_gb300_reverse, call %d" % call)
        for g, w, m in zip(asens, asens_ref, mag):
            _within(g, w, m, "adjoint vs casadi_gb300_reverse, call %d" % call)
        for g, w, m in zip(asens, oasens, mag):
            _within(g, w, m, "adjoint vs oracle, call %d" % call)
        for g, w, b in zip(res, ores, bound):
            # relative 1e-13, or within 4 ulps of every sin/cos result propagated to the value
            d = np.abs(g - w)
            assert np.all((d <= 1e-13 * np.abs(w)) | (d <= 4 * 2.0**-52 * b)), call


def test_noalloc_values_only(gpu_lib):
    F = W.cartpole_step()
    tape = R.CudaTape(F)
    n = 777
    args = [torch.from_numpy(a).cuda() for a in W.cartpole_inputs(n, steps=1, seed=9)]
    want = [r.cpu().numpy() for r in tape.eval(args)]
    for call in range(2):
        res, _ = _noalloc(tape, args, None, n, 0)
        for g, w in zip(res, want):
            assert_bitexact(g, w, "values, call %d" % call)


def test_noalloc_refuses_oversized_call(gpu_lib):
    F = W.cartpole_rollout(20)
    tape = R.CudaTape(F)
    n = (64 << 20) // (8 * tape.n_partials) + 64  # one wave more than the fixed scratch holds
    st = R.load().casadi_gb300_reverse_noalloc(tape.id, n, n, 1, None, None, None, None, None)
    assert st == -5
    msg = R.load().casadi_gb300_last_error().decode()
    assert "allocation-free adjoint" in msg and str(64 << 20) in msg


def test_noalloc_refuses_a_work_vector_beyond_shared_memory(gpu_lib):
    """1500 values that all stay live until the second chain uses them in reverse order:
    sz_w 1502, 384 KB per tile; casadi_gb300_reverse runs it from global memory."""
    x = S.sym("x", 1)
    ys = [S.sin(x[0] + 0.001 * k) for k in range(1500)]
    z1 = ys[0]
    for y in ys[1:]:
        z1 = z1 + y
    z2 = ys[-1]
    for y in reversed(ys[:-1]):
        z2 = z2 - y
    tape = R.CudaTape(S.Function("wide", [x], [[z1 * z2]]))
    n = 64
    args = [torch.linspace(0, 1, n, dtype=torch.float64, device="cuda")[None, :].contiguous()]
    seeds = [torch.ones((1, 1, n), dtype=torch.float64, device="cuda")]
    res = [torch.empty((1, n), dtype=torch.float64, device="cuda")]
    asens = [torch.empty((1, 1, n), dtype=torch.float64, device="cuda")]
    st = R.load().casadi_gb300_reverse_noalloc(
        tape.id, n, n, 1, _ptrs(args), _ptrs(res), _ptrs(seeds), _ptrs(asens),
        ct.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == -6
    assert "shared memory" in R.load().casadi_gb300_last_error().decode()
    _, a = tape.reverse(args, seeds)  # the regular entry point handles it
    assert torch.isfinite(a[0]).all()
    tape.sync()
