"""MapSum on the GPU (casadi/core/mapsum.cpp) through the C ABI: shared inputs, outputs summed
over the instances, its forward and reverse modes (shared seeds / summed sensitivities) and
its sparsity sweeps.

Bars: the instance-order sums are the reference's own order, so they equal the oracle bit for
bit on +,-,*,/,sqrt tapes and equal the in-order sum of the GPU's own per-instance values on
any tape; the tree order equals its restatement (``tree_sum`` below) over the same values bit
for bit; against the oracle with transcendentals the per-instance tolerance (1e-13) applies to
the sum of magnitudes. Sparsity is bit-exact."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W
from casadi_gb300.runtime import CasadiGpuError, CudaMapSum, CudaTape

from helpers import RTOL

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
EPS = np.finfo(float).eps


def tree_sum(rows):
    """The blocked tree of order 1: per level 256-instance blocks, lane l of a warp adds
    x[b*256 + m*32 + l] for m = 0..7 from +0, then a butterfly over the 32 lanes (xor 16, 8,
    4, 2, 1); block sums form the next level until one value remains."""
    x = np.asarray(rows, dtype=np.float64)
    lead = x.shape[:-1]
    x = x.reshape(-1, x.shape[-1])
    lanes = np.arange(32)
    while True:
        m = x.shape[1]
        nb = max(1, -(-m // 256))
        p = np.zeros((x.shape[0], nb * 256))
        p[:, :m] = x
        p = p.reshape(x.shape[0], nb, 8, 32)
        acc = np.zeros((x.shape[0], nb, 32))
        for k in range(8):
            acc = acc + p[:, :, k, :]
        for s in (16, 8, 4, 2, 1):
            acc = acc + acc[:, :, lanes ^ s]
        x = acc[:, :, 0]
        if nb == 1:
            return x[:, 0].reshape(lead)


def dev(arrs):
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def host(ts):
    torch.cuda.synchronize()
    return [None if t is None else t.cpu().numpy() for t in ts]


def mapsum2_fun():
    """The function of the reference's test_mapsum2 (test/python/function.py:807-860):
    f(x, y[2], z[2x2], v[upper 3x3]) = (z@y + x, sin(y*x)^T, v/x)."""
    x = S.sym("x")
    y = S.sym("y", 2)
    z = S.sym("z", 4)  # column-major 2x2
    v = S.sym("v", 6)  # upper triangle of 3x3, column-major nonzeros
    a = [z[i] * y[0] + z[i + 2] * y[1] + x for i in range(2)]
    b = [S.sin(y[k] * x) for k in range(2)]
    c = [v[k] / x for k in range(6)]
    return S.Function("f", [[x], y, z, v], [a, b, c])


def _materialise(args, reduce_in, n):
    return [np.repeat(np.asarray(a)[:, None], n, axis=1) if r else a
            for a, r in zip(args, reduce_in)]


def _inputs(n, seed=0):
    rng = np.random.default_rng(seed)
    return [rng.random((1, n)) + 0.5, rng.random((2, n)), rng.random(4), rng.random(6)]


RIN = [False, False, True, True]
ROUT = [True, False, False]


@pytest.mark.parametrize("n", [2, 255, 256, 257, 5000, 70001])
@pytest.mark.parametrize("order", [0, 1])
def test_mapsum2_eval(gpu_lib, n, order):
    f = mapsum2_fun()
    args = _inputs(n, n)
    F = CudaMapSum(f, n, RIN, ROUT, order=order)
    got = host(F(dev(args)))
    # per-instance values of the same GPU, summed on the host in the same order
    per = host(F.tape.eval(dev(_materialise(args, RIN, n))))
    want0 = O.ordered_sum(per[0]) if order == 0 else tree_sum(per[0])
    assert np.array_equal(got[0], want0)
    assert np.array_equal(got[1], per[1]) and np.array_equal(got[2], per[2])
    # against the oracle's MapSum (instance order, host libm)
    ref = O.mapsum_eval(f.tape, args, n, RIN, ROUT)
    scale = O.ordered_sum(np.abs(per[0]))
    assert np.all(np.abs(got[0] - ref[0]) <= (RTOL + n * EPS) * scale)
    np.testing.assert_allclose(got[1], ref[1], rtol=RTOL, atol=0)
    assert np.array_equal(got[2], ref[2])  # v/x: one division, exact
    F.tape.sync()


def _arith_fun(n_in=6, n_nodes=400, seed=3):
    rng = np.random.default_rng(seed)
    xs = S.sym("x", n_in)
    p = S.sym("p", 3)
    nodes = list(xs) + list(p)
    for k in range(len(nodes), n_nodes):
        a = nodes[int(rng.integers(max(0, k - 40), k))]
        b = nodes[int(rng.integers(max(0, k - 40), k))]
        r = rng.random()
        e = a + b if r < 0.3 else a - b if r < 0.5 else a * b * 0.5 if r < 0.8 else \
            a / (b * b + 1.0) if r < 0.9 else S.sqrt(a * a + 1.0)
        nodes.append(e)
    return S.Function("g", [xs, p], [nodes[-4:], nodes[-7:-4]])


@pytest.mark.parametrize("n", [1, 300, 4096])
def test_exact_tape_bits_equal_the_oracle(gpu_lib, n):
    """+,-,*,/,sqrt: the per-instance values are the oracle's bits, so the instance-order
    sums, forward and adjoint included, are too."""
    g = _arith_fun()
    rng = np.random.default_rng(n)
    args = [rng.uniform(-1, 1, (6, n)), rng.uniform(-1, 1, 3)]
    rin, rout = [False, True], [True, False]
    F = CudaMapSum(g, n, rin, rout, order=0)
    got = host(F(dev(args)))
    want = O.mapsum_eval(g.tape, args, n, rin, rout)
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    fseeds = [rng.standard_normal((2, 6, n)), rng.standard_normal((2, 3))]
    res, fs = F.forward(dev(args), dev(fseeds))
    wres, wfs = O.mapsum_forward(g.tape, args, fseeds, n, rin, rout)
    for a, b in zip(host(res) + host(fs), wres + wfs):
        assert np.array_equal(a, b)
    aseeds = [rng.standard_normal((3, 4)), rng.standard_normal((3, 3, n))]
    res, asn = F.reverse(dev(args), dev(aseeds))
    wres, was = O.mapsum_reverse(g.tape, args, aseeds, n, rin, rout)
    for a, b in zip(host(res) + host(asn), wres + was):
        assert np.array_equal(a, b)
    F.tape.sync()


@pytest.mark.parametrize("order", [0, 1])
def test_rollout_gradient_of_a_summed_cost(gpu_lib, order):
    """Controls shared by every instance, cost summed: the adjoint of the summed cost w.r.t.
    the shared controls is the sum of the per-instance gradients (MapSum::get_reverse);
    dot-product test against the forward mode."""
    f = W.cartpole_rollout(20)
    n = 20000
    x0, U = W.cartpole_inputs(n, steps=20, seed=5)
    args = [x0, np.ascontiguousarray(U[:, 0])]
    rin, rout = [False, True], [False, True]
    F = CudaMapSum(f, n, rin, rout, order=order)
    aseeds = [np.zeros((1, 4, n)), np.ones((1, 1))]
    res, asens = F.reverse(dev(args), dev(aseeds))
    gU = host(asens)[1][0]  # (20,)
    # the same GPU's per-instance adjoints, summed on the host in the same order
    tape = F.tape
    full = _materialise(args, rin, n)
    _, per = tape.reverse(dev(full), dev([np.zeros((1, 4, n)), np.ones((1, 1, n))]))
    per = host(per)[1][0]  # (20, n)
    want = O.ordered_sum(per) if order == 0 else tree_sum(per)
    assert np.array_equal(gU, want)
    # oracle (host libm), tolerance on the sum of magnitudes
    _, was = O.mapsum_reverse(f.tape, args, [np.zeros((1, 4, n)), np.ones((1, 1))], n, rin, rout)
    scale = O.ordered_sum(np.abs(per))
    assert np.all(np.abs(gU - was[1][0]) <= (1e-12 + n * EPS) * scale)
    # dot-product test: <dU, d cost/dU> == forward sensitivity of the summed cost
    rng = np.random.default_rng(1)
    dU = rng.standard_normal((1, 20))
    _, fs = F.forward(dev(args), dev([np.zeros((1, 4, n)), dU]))
    lhs = float(dU[0] @ gU)
    rhs = float(host(fs)[1][0, 0])
    assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(lhs))
    tape.sync()


def test_sparsity_sweeps_bit_exact(gpu_lib):
    g = W.random_dag(n_in=16, n_nodes=900, n_out=6, seed=4)
    # two inputs: split the 16 into a per-instance block and a shared block
    t = g.tape
    n = 1000
    rng = np.random.default_rng(2)
    rin, rout = [True], [True]
    F = CudaMapSum(g, n, rin, rout)
    bits = rng.integers(0, 2**63, size=16, dtype=np.int64).view(np.uint64)
    got = host(F.sp_forward(dev([bits.view(np.int64)])))[0].view(np.uint64)
    want = O.mapsum_sp_forward(t, [bits], n, rin, rout)[0]
    assert np.array_equal(got, want)
    # per-instance inputs, summed outputs
    F2 = CudaMapSum(g, n, [False], [True])
    bits2 = rng.integers(0, 2**63, size=(16, n), dtype=np.int64).view(np.uint64)
    got2 = host(F2.sp_forward(dev([bits2.view(np.int64)])))[0].view(np.uint64)
    want2 = O.mapsum_sp_forward(t, [bits2], n, [False], [True])[0]
    assert np.array_equal(got2, want2)
    # reverse: shared input accumulates the OR of all instances; summed seeds cleared
    arg0 = rng.integers(0, 256, size=16, dtype=np.int64).view(np.uint64)
    seed = rng.integers(0, 2**63, size=6, dtype=np.int64).view(np.uint64)
    a_dev, r_dev = dev([arg0.view(np.int64)]), dev([seed.view(np.int64)])
    F.sp_reverse(a_dev, r_dev)
    ga, gr = host(a_dev)[0].view(np.uint64), host(r_dev)[0].view(np.uint64)
    wa, wr = [arg0.copy()], [seed.copy()]
    O.mapsum_sp_reverse(t, wa, wr, n, rin, rout)
    assert np.array_equal(ga, wa[0]) and np.array_equal(gr, wr[0])
    assert (gr == 0).all()
    F.tape.sync()


def test_edges_zero_instances_signed_zero_and_errors(gpu_lib):
    x = S.sym("x", 2)
    f = S.Function("h", [x], [[x[0] * x[1]], [x[0] - x[1]]])
    # n = 0: a summed output is zero (MapSum clears it and adds nothing)
    F0 = CudaMapSum(f, 0, [False], [True, True])
    got = host(F0([torch.zeros((2, 0), dtype=torch.float64, device="cuda")]))
    assert np.array_equal(got[0], [0.0]) and np.array_equal(got[1], [0.0])
    # every per-instance value -0: the sum starts from +0, so it is +0 in both orders
    n = 300
    args = [np.vstack([np.full(n, -0.0), np.full(n, 1.0)])]
    for order in (0, 1):
        F = CudaMapSum(f, n, [False], [True, False], order=order)
        got = host(F(dev(args)))
        assert got[0][0] == 0.0 and not np.signbit(got[0][0])
    # a null summed output is skipped; a bad order is an error
    F = CudaMapSum(f, n, [False], [True, True])
    res = F.eval(dev(args), res=[None, torch.empty(1, dtype=torch.float64, device="cuda")])
    assert host([res[1]])[0][0] == O.ordered_sum(np.full(n, -1.0))
    with pytest.raises(CasadiGpuError):
        CudaMapSum(f, n, [False], [True, True], order=2)(dev(args))
    F.tape.sync()
