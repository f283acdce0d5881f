"""The adjoint with segment checkpointing (casadi_gb300_reverse_checkpointed) through the C ABI:
values equal the value sweep's bit for bit, sensitivities match the oracle element-wise (and the
unsegmented adjoint within 1e-13 of their magnitude), across segment counts, several adjoint
directions, instance waves, a tape whose work vector lives in global memory, and a values-only
call. The scratch it needs shrinks with the segment count."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import RTOL, assert_adjoint_close, assert_bitexact, assert_close, magnitudes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _host(ts):
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in ts]


def _check(f, args, seeds, n, segments, scratch_limit=None):
    ct = R.CudaTape(f)
    res, asens = ct.reverse_checkpointed(_dev(args), _dev(seeds), segments,
                                         scratch_limit=scratch_limit)
    res, asens = _host(res), _host(asens)
    for g, w in zip(res, _host(ct.eval(_dev(args)))):
        assert_bitexact(g, w, "values, %d segments" % segments)
    _, plain = ct.reverse(_dev(args), _dev(seeds))
    plain = _host(plain)
    _, was = O.reverse(f.tape, args, seeds, n)
    _, mag = magnitudes(O.reverse, f.tape, args, seeds, n)
    for g, p, m in zip(asens, plain, mag):
        assert_close(g, p, "against the unsegmented adjoint", bound=RTOL * m)
    for d in range(seeds[0].shape[0]):
        assert_adjoint_close([a[d] for a in asens], [w[d] for w in was], [m[d] for m in mag], f,
                             args, [s[d] for s in seeds], "direction %d" % d)
    ct.sync()
    return res, asens


@pytest.mark.parametrize("segments", [1, 3, 8])
def test_rollout_checkpointed_adjoint(gpu_lib, segments):
    f = W.cartpole_rollout(20)
    n = 5000
    args = list(W.cartpole_inputs(n, steps=20, seed=6))
    rng = np.random.default_rng(segments)
    seeds = [rng.standard_normal((2, 4, n)), rng.standard_normal((2, 1, n))]
    _check(f, args, seeds, n, segments)


def test_dag_checkpointed_adjoint(gpu_lib):
    f = W.random_dag()
    n = 3000
    args = list(W.dag_inputs(n))
    _check(f, args, [np.ones((1, 16, n))], n, 4)


def test_global_memory_work_vector_and_waves(gpu_lib):
    """The quadcopter Lagrangian (work vector beyond shared memory), 4 segments, with the
    scratch at its minimum (one warp of instances per wave) and in one wave: same bits."""
    f = W.quad_ms_lagrangian(20)
    n = 200
    args = list(W.quad_ms_inputs(n, intervals=20, seed=5))
    seeds = [np.zeros((1, k, n)) for k in f.tape.nnz_out]
    seeds[1][:] = 1.0
    one = _check(f, args, seeds, n, 4)
    ct = R.CudaTape(f)
    few = ct.reverse_checkpointed(_dev(args), _dev(seeds), 4, scratch_limit=1)
    for a, b in zip(one[1], _host(few[1])):
        assert_bitexact(a, b, "one wave vs waves of 32 instances")
    ct.sync()


def test_scratch_shrinks_with_segments(gpu_lib):
    f = W.cartpole_rollout(100)
    ct = R.CudaTape(f)
    n = 1 << 16
    plain = ct.scratch_bytes(n)
    sc, k = ct.checkpoint_scratch(10, 1, n)
    assert k == 10
    assert sc.numel() < plain / 6
    del sc


def test_values_only_and_bad_calls(gpu_lib):
    f = W.cartpole_rollout(4)
    n = 300
    args = list(W.cartpole_inputs(n, steps=4, seed=2))
    ct = R.CudaTape(f)
    res, _ = ct.reverse_checkpointed(_dev(args), [], 3)
    for g, w in zip(_host(res), _host(ct.eval(_dev(args)))):
        assert_bitexact(g, w, "values only")
    with pytest.raises(R.CasadiGpuError):
        ct.reverse_checkpointed(_dev(args), _dev([np.ones((1, 4, n)), np.ones((1, 1, n))]), 0)
    st = R.load().casadi_gb300_reverse_checkpointed(ct.id, n, n, 1, 3, None, None, None, None,
                                                    None, 0, None)
    assert st == -5
    ct.sync()
