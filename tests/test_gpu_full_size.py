"""Parity at the benchmark's own sizes, through the same entry points the benchmark times.

* Cart-pole 20-step rollout, N = 262144 (the headline step, ``jacobian_reverse``: forward
  Jacobian by 24 unit directions + adjoint of the cost): instance windows at the start, the
  middle and the ragged end, launched alone, give the full launch's bits at those instances (a
  size-independent property: each instance's arithmetic does not depend on how many others
  share the launch), and a strided sample of 2048 instances matches the oracle element-wise.
* Random DAG 64 in / 10000 nodes / 16 out, N = 16384 (values, adjoint of the sum of outputs,
  sp_forward and sp_reverse): every instance against the oracle; the sparsity words bit for
  bit.
"""
import os

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import workloads as W
from casadi_gb300.runtime import CudaTape

from helpers import (RTOL, assert_adjoint_close, assert_bitexact, assert_close, magnitudes,
                     value_bounds)

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
NTHREADS = os.cpu_count() or 1


def _host(ts):
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in ts]


def test_rollout_at_the_benchmark_size(gpu_lib):
    F = W.cartpole_rollout(20)
    n = 262144
    args = W.cartpole_inputs(n, steps=20, seed=0)
    seeds = [np.zeros((1, 4, n)), np.ones((1, 1, n))]
    dargs = [torch.from_numpy(a).cuda() for a in args]
    dseeds = [torch.from_numpy(s).cuda() for s in seeds]
    ct = CudaTape(F)
    res, jac, asens = [_host(x) for x in ct.jacobian_reverse(dargs, dseeds)]
    # windows launched alone give the same bits
    m = 997
    for lo in (0, n // 2 + 13, n - m):
        sub = [a[:, lo:lo + m].contiguous() for a in dargs]
        sseeds = [s[:, :, lo:lo + m].contiguous() for s in dseeds]
        r2, j2, a2 = [_host(x) for x in ct.jacobian_reverse(sub, sseeds)]
        for full, part in ((res, r2), (asens, a2)):
            for f, p in zip(full, part):
                assert_bitexact(f[..., lo:lo + m], p, "window at %d" % lo)
        for f, p in zip(jac, j2):
            assert_bitexact(f[..., lo:lo + m], p, "Jacobian window at %d" % lo)
    # a strided sample against the oracle
    idx = np.arange(0, n, 128)
    k = idx.size
    sargs = [np.ascontiguousarray(a[:, idx]) for a in args]
    sseeds = [np.ascontiguousarray(s[:, :, idx]) for s in seeds]
    wres, wjac = O.jacobian(F.tape, sargs, k, NTHREADS)
    _, jmag = magnitudes(O.jacobian, F.tape, sargs, k, NTHREADS)
    vb = value_bounds(F.tape, sargs, k)
    for j in range(2):
        assert_close(res[j][:, idx], wres[j], "value %d" % j, bound=vb[j])
        assert_close(jac[j][..., idx], wjac[j], "Jacobian block %d" % j, bound=RTOL * jmag[j])
    _, was = O.reverse(F.tape, sargs, sseeds, k, NTHREADS)
    _, amag = magnitudes(O.reverse, F.tape, sargs, sseeds, k, NTHREADS)
    assert_adjoint_close([a[0][:, idx] for a in asens], [w[0] for w in was],
                         [mg[0] for mg in amag], F, sargs, [s[0] for s in sseeds],
                         "adjoint of the cost")
    ct.sync()


def test_dag_at_the_benchmark_size(gpu_lib):
    G = W.random_dag()
    t = G.tape
    n = 16384
    args = W.dag_inputs(n)
    ct = CudaTape(G)
    dargs = [torch.from_numpy(a).cuda() for a in args]
    got = _host(ct.eval(dargs))[0]
    assert_close(got, O.eval(t, args, n, NTHREADS)[0], "values",
                 bound=value_bounds(t, args, n)[0])
    seeds = [np.ones((1, 16, n))]
    _, asens = ct.reverse(dargs, [torch.from_numpy(seeds[0]).cuda()])
    _, was = O.reverse(t, args, seeds, n, NTHREADS)
    _, amag = magnitudes(O.reverse, t, args, seeds, n, NTHREADS)
    assert_adjoint_close([_host(asens)[0][0]], [was[0][0]], [amag[0][0]], G, args,
                         [seeds[0][0]], "adjoint of the sum of outputs")
    rng = np.random.default_rng(8)
    bits = rng.integers(0, 2**63, size=(64, n), dtype=np.int64)
    res = _host(ct.sp_forward([torch.from_numpy(bits).cuda()]))[0]
    want = O.sp_forward(t, [bits.view(np.uint64)], n)[0]
    assert np.array_equal(res.view(np.uint64), want)
    arg0 = np.zeros((64, n), np.int64)
    rseed = rng.integers(0, 2**63, size=(16, n), dtype=np.int64)
    da, dr = [torch.from_numpy(arg0).cuda()], [torch.from_numpy(rseed).cuda()]
    ct.sp_reverse(da, dr)
    wa, wr = [arg0.view(np.uint64).copy()], [rseed.view(np.uint64).copy()]
    O.sp_reverse(t, wa, wr, n)
    assert np.array_equal(_host(da)[0].view(np.uint64), wa[0])
    assert not _host(dr)[0].any()
    ct.sync()
