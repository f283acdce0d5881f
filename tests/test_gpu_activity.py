"""GPU activity analysis (SXFunction::eval_activity, casadi/core/sx_function.cpp:1684-1718)
through the C ABI: bit-exact against the golden fixtures that the reference's own zero checkers
produced, against the oracle on larger seeded cases, in both work-vector residences, and the
bool-mask interface of Function::activity (casadi/core/function.cpp:1269-1294)."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import workloads as W
from casadi_gb300.runtime import CudaTape

from helpers import golden_list, golden_tape, load_npz

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(arrs):
    return [torch.from_numpy(np.ascontiguousarray(a, np.uint64).view(np.int64)).cuda()
            for a in arrs]


def _host(ts):
    torch.cuda.synchronize()
    return [t.cpu().numpy().view(np.uint64) for t in ts]


def _tape(name):
    if name == "ops":
        return golden_tape(load_npz("activity.npz"), "ops")
    return golden_tape(load_npz("tapes.npz"), name)


@pytest.mark.parametrize("name", ["ops", "cartpole", "rollout", "dag"])
@pytest.mark.parametrize("residence", [1, 2])
def test_activity_golden(gpu_lib, name, residence):
    z = load_npz("activity.npz")
    t = _tape(name)
    args = golden_list(z, name, "act_arg", len(t.nnz_in))
    want = golden_list(z, name, "act_res", len(t.nnz_out))
    ct = CudaTape(t)
    ct.set_residence(residence)
    got = _host(ct.eval_activity(_dev(args)))
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    ct.sync()


def test_activity_dag_full_grid_vs_oracle(gpu_lib):
    """The 10000-node random DAG over enough instances to fill the GPU several times (the
    residence autotuner runs), with half the inputs inactive per instance."""
    t = W.random_dag().tape
    n = 80000
    rng = np.random.default_rng(21)
    args = [np.where(rng.random((64, n)) < 0.5, np.uint64(0), np.uint64(2**64 - 1))]
    args[0][:, :5] = 0  # instances with every input inactive
    ct = CudaTape(t)
    got = _host(ct.eval_activity(_dev(args)))
    want = O.activity(t, args, n, nthreads=8)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    ct.sync()


def test_activity_bool_masks_and_null_inputs(gpu_lib):
    f = W.cartpole_rollout(20)
    ct = CudaTape(f.tape)
    n = 97
    rng = np.random.default_rng(4)
    masks = rng.random((24, n)) < 0.7
    masks[:, 0] = False
    masks[:, 1] = True
    got = ct.activity(masks)
    words = [np.where(masks[:4], np.uint64(2**64 - 1), np.uint64(0)),
             np.where(masks[4:], np.uint64(2**64 - 1), np.uint64(0))]
    want = O.activity(f.tape, words, n)
    assert np.array_equal(got, np.concatenate(want) != 0)
    # a null input reads as inactive
    res = _host(ct.eval_activity([None, _dev([words[1]])[0]], n=n))
    want0 = O.activity(f.tape, [np.zeros_like(words[0]), words[1]], n)
    for g, w in zip(res, want0):
        assert np.array_equal(g, w)
    with pytest.raises(ValueError):
        ct.activity(masks[:5])
    ct.sync()
