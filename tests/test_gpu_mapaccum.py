"""Mapaccum on the GPU (Function::mapaccum, casadi/core/function.cpp:668-747) through the C ABI:
N chained calls of one step tape with the accumulator fed back in place. Values, forward and
reverse modes are checked against chaining the step tape's own sweeps call by call (the same
device arithmetic: bit for bit for values and tangents), against the unrolled rollout tape
and the oracle (tolerance), and by a dot-product test between the two modes."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W
from casadi_gb300.runtime import CasadiGpuError, CudaMapaccum, CudaTape

from helpers import RTOL, assert_bitexact, assert_close, magnitudes, rounding_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
N = 20


def dev(arrs):
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def host(ts):
    torch.cuda.synchronize()
    return [None if t is None else t.cpu().numpy() for t in ts]


def step_with_cost():
    """f(x[4], u) -> (x_next[4], stage cost ||x||^2 + 0.01 u^2)."""
    x = S.sym("x", 4)
    u = S.sym("u")
    c = (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3]) + 0.01 * u * u
    return S.Function("fc", [x, [u]], [W.rk4_step(x, u), [c]])


def _inputs(n, seed):
    x0, U = W.cartpole_inputs(n, steps=N, seed=seed)
    return [x0, U * 0.3]


def test_values_chain_the_step_tape_bit_for_bit(gpu_lib):
    f = step_with_cost()
    n = 1000
    x0, U = _inputs(n, 1)
    acc = CudaMapaccum(f, N)
    xs, cs = host(acc.eval(dev([x0, U])))
    assert xs.shape == (4 * N, n) and cs.shape == (N, n)
    ct = CudaTape(f)
    x = x0
    for k in range(N):
        xn, c = host(ct.eval(dev([x, U[k:k + 1]])))
        assert_bitexact(xs[4 * k:4 * k + 4], xn, "x_%d" % (k + 1))
        assert_bitexact(cs[k:k + 1], c, "cost %d" % k)
        x = xn
    # the unrolled rollout tape on the oracle: xN and the summed cost
    F = W.cartpole_rollout(N)
    xN, cost = O.eval(F.tape, [x0, U], n)
    # the chain and the unrolled tape may round any instruction differently (and numpy sums
    # the stage costs in its own order): 4 ulps of every rounded result, propagated
    rb = rounding_bounds(F.tape, [x0, U], n)
    assert_close(xs[-4:], xN, "xN vs unrolled", bound=rb[0])
    assert_close(np.sum(cs, axis=0), cost[0], "cost vs unrolled", bound=rb[1][0])
    # an accumulator output that is not kept lives in the scratch
    _, cs2 = host(acc.eval(dev([x0, U]), keep=[False, True]))
    assert_bitexact(cs2, cs, "costs without keeping x")
    ct.sync()


def test_forward_mode(gpu_lib):
    f = step_with_cost()
    n = 513
    x0, U = _inputs(n, 2)
    rng = np.random.default_rng(2)
    fx = rng.standard_normal((3, 4, n))
    fu = rng.standard_normal((3, N, n))
    acc = CudaMapaccum(f, N)
    (xs, cs), (dxs, dcs) = [host(r) for r in acc.forward(dev([x0, U]), dev([fx, fu]))]
    # chaining the step tape's forward mode call by call
    ct = CudaTape(f)
    x, dx = x0, fx
    for k in range(N):
        (xn, c), (dxn, dc) = [host(r) for r in ct.forward(dev([x, U[k:k + 1]]),
                                                         dev([dx, fu[:, k:k + 1]]))]
        assert_bitexact(xs[4 * k:4 * k + 4], xn, "x_%d" % (k + 1))
        assert_bitexact(dxs[:, 4 * k:4 * k + 4], dxn, "dx_%d" % (k + 1))
        assert_bitexact(dcs[:, k:k + 1], dc, "dcost %d" % k)
        x, dx = xn, dxn
    # the unrolled rollout's forward mode on the oracle (xN block)
    F = W.cartpole_rollout(N)
    _, (dxN, _) = O.forward(F.tape, [x0, U], [fx, fu], n)
    _, (mag, _) = magnitudes(O.forward, F.tape, [x0, U], [fx, fu], n)
    assert_close(dxs[:, -4:], dxN, "dxN vs unrolled", bound=RTOL * mag)
    ct.sync()


@pytest.mark.parametrize("keep_x", [True, False])
def test_reverse_mode(gpu_lib, keep_x):
    f = step_with_cost()
    n = 700
    x0, U = _inputs(n, 3)
    acc = CudaMapaccum(f, N)
    # seed: x_N and every stage cost -> the gradient of the unrolled rollout's (xN, cost)
    rng = np.random.default_rng(3)
    sx = np.zeros((2, 4 * N, n))
    sx[:, -4:] = rng.standard_normal((2, 4, n))
    sc = np.zeros((2, N, n))
    sc[:] = rng.standard_normal((2, 1, n))
    keep = None if keep_x else [False, True]
    res, (ax0, aU) = acc.reverse(dev([x0, U]), dev([sx, sc]), keep=keep)
    ax0, aU = host([ax0, aU])
    F = W.cartpole_rollout(N)
    seeds = [sx[:, -4:], sc[:, :1]]
    _, (wx0, wU) = O.reverse(F.tape, [x0, U], seeds, n)
    _, (mx0, mU) = magnitudes(O.reverse, F.tape, [x0, U], seeds, n)
    assert_close(ax0, wx0, "d/dx0", bound=RTOL * mx0)
    assert_close(aU, wU, "d/dU", bound=RTOL * mU)
    # dot-product test with the forward mode on random seeds of every block
    ax, au = rng.standard_normal((1, 4, n)), rng.standard_normal((1, N, n))
    _, (dxs, dcs) = [host(r) for r in acc.forward(dev([x0, U]), dev([ax, au]))]
    lhs = np.sum(sx[:1] * dxs, axis=(0, 1)) + np.sum(sc[:1] * dcs, axis=(0, 1))
    rhs = np.sum(ax0[:1] * ax, axis=(0, 1)) + np.sum(aU[:1] * au, axis=(0, 1))
    assert np.all(np.abs(lhs - rhs) <= 1e-9 * np.maximum(1.0, np.abs(lhs)))
    acc.tape.sync()


def test_keep_flags_give_the_same_bits_and_bad_arguments(gpu_lib):
    f = step_with_cost()
    n = 64
    x0, U = _inputs(n, 4)
    acc = CudaMapaccum(f, N)
    seeds = dev([np.ones((1, 4 * N, n)), np.ones((1, N, n))])
    _, a1 = acc.reverse(dev([x0, U]), seeds)
    _, a2 = acc.reverse(dev([x0, U]), seeds, keep=[False, False])
    for x, y in zip(host(a1), host(a2)):
        assert_bitexact(x, y, "reverse without kept outputs")
    with pytest.raises(CasadiGpuError):
        CudaMapaccum(f, 0).eval(dev([x0, U]))
    with pytest.raises(CasadiGpuError):
        CudaMapaccum(f, N, n_accum=3).eval(dev([x0, U]))  # more accumulators than inputs
    acc.tape.sync()


def test_reverse_recorded_forward_gives_the_checkpointed_bits(gpu_lib):
    """With room for every call's partials the reverse records them on the way forward and
    runs adjoint sweeps only on the way back: the same bits as the checkpointed form."""
    f = step_with_cost()
    n = 1500
    x0, U = _inputs(n, 6)
    rng = np.random.default_rng(6)
    seeds = dev([rng.standard_normal((2, 4 * N, n)), rng.standard_normal((2, N, n))])
    res_c, sens_c = CudaMapaccum(f, N).reverse(dev([x0, U]), seeds)
    acc = CudaMapaccum(f, N)
    res_r, sens_r = acc.reverse(dev([x0, U]), seeds, record_all=True)
    for a, b in zip(host(res_c) + host(sens_c), host(res_r) + host(sens_r)):
        assert_bitexact(a, b, "recorded forward vs checkpointed")
    acc.tape.sync()
