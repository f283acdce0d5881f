"""Global-memory work vectors: the same sweeps with the work vector in per-CTA blocks of
global memory instead of shared memory. Forced on a small tape, every result must equal the
shared-memory path bit for bit; on a tape whose scheduled work vector does not fit shared
memory (the quadcopter NLP's Lagrangian with both outputs, 1447 slots) the path is taken
automatically and checked against the oracle."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import RTOL, assert_bitexact, assert_close

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(arrs):
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _host(ts):
    return [t.cpu().numpy() for t in ts]


def test_forced_global_equals_shared(gpu_lib):
    F = W.cartpole_rollout(6)
    n = 3001
    args = _dev(W.cartpole_inputs(n, steps=6, seed=41))
    rng = np.random.default_rng(41)
    fseeds = _dev([rng.standard_normal((3, k, n)) for k in F.tape.nnz_in])
    aseeds = _dev([rng.standard_normal((2, k, n)) for k in F.tape.nnz_out])
    bits = [torch.randint(0, 1 << 62, (k, n), dtype=torch.int64, device="cuda")
            for k in F.tape.nnz_in]

    def run(ct):
        out = [_host(ct.eval(args))]
        out.append(_host(ct.forward(args, fseeds)[1]))
        out.append(_host(ct.jacobian(args)[1]))
        out.append(_host(ct.reverse(args, aseeds)[1]))
        out.append(_host(ct.sp_forward(bits)))
        sens = [torch.zeros((k, n), dtype=torch.int64, device="cuda") for k in F.tape.nnz_in]
        seeds = [torch.randint(0, 1 << 62, (k, n), dtype=torch.int64, device="cuda",
                               generator=torch.Generator(device="cuda").manual_seed(5))
                 for k in F.tape.nnz_out]
        ct.sp_reverse(sens, seeds)
        out.append(_host(sens))
        ct.sync()
        return out

    sh = R.CudaTape(F)
    sh.set_residence(2)
    shared = run(sh)
    g = R.CudaTape(F)
    g.set_residence(1)
    glob = run(g)
    for a, b in zip(shared, glob):
        for x, y in zip(a, b):
            if x.dtype == np.int64:
                assert np.array_equal(x, y)
            else:
                assert_bitexact(x, y, "global work vector")


def test_tape_larger_than_shared_memory(gpu_lib):
    F = W.quad_ms_lagrangian(100)
    ct = R.CudaTape(F)
    assert ct.sz_w > 900  # does not fit the shared-memory sweeps
    n = 300
    args = W.quad_ms_inputs(n, intervals=100, seed=7)
    res = _host(ct.eval(_dev(args)))
    want = O.eval(F.tape, args, n)
    for g, w in zip(res, want):
        assert_close(g, w, "values", rtol=RTOL)
    seeds = [np.zeros((1, k, n)) for k in F.tape.nnz_out]
    seeds[1][:] = 1.0
    _, asens = ct.reverse(_dev(args), _dev(seeds))
    _, was = O.reverse(F.tape, args, seeds, n)
    for g, w in zip(_host(asens), was):
        assert_close(g, w, "adjoint of the Lagrangian", rtol=RTOL)
    ct.sync()
