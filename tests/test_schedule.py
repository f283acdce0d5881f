"""Register-pressure scheduling (casadi_gb300_tape_schedule, host code of the C ABI): the GPU
runs each tape in an order with fewer live values. These checks need no GPU: the oracle runs
the original tape and the scheduled one and every value, forward and adjoint sensitivity and
sparsity pattern must agree bit for bit, while the work vector gets shorter."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import golden_list, golden_tape, load_npz, same_bits

CASES = [
    ("cartpole", lambda: W.cartpole_step(), lambda n: W.cartpole_inputs(n, steps=1, seed=1)),
    ("rollout20", lambda: W.cartpole_rollout(20), lambda n: W.cartpole_inputs(n, steps=20, seed=2)),
    ("dag", lambda: W.random_dag(n_in=16, n_nodes=1500, n_out=6, seed=3),
     lambda n: W.dag_inputs(n, n_in=16, seed=3)),
    ("dag_bounded", lambda: W.random_dag(n_in=16, n_nodes=3000, n_out=4, seed=4, window=64,
                                         bounded=True),
     lambda n: W.dag_inputs(n, n_in=16, seed=4)),
]


def _all_bits_equal(a, b, what):
    for x, y in zip(a, b):
        assert same_bits(x, y).all(), what


@pytest.mark.parametrize("name,make,inputs", CASES, ids=[c[0] for c in CASES])
def test_schedule_keeps_every_result_bit_for_bit(name, make, inputs):
    t = make().tape
    s = R.schedule(t)
    assert s.n_instr == t.n_instr
    assert sorted(s.op.tolist()) == sorted(t.op.tolist())
    assert s.sz_w <= t.sz_w
    n = 37
    args = inputs(n)
    _all_bits_equal(O.eval(s, args, n), O.eval(t, args, n), "values")
    rng = np.random.default_rng(5)
    fseeds = [rng.standard_normal((3, k, n)) for k in t.nnz_in]
    _all_bits_equal(O.forward(s, args, fseeds, n)[1], O.forward(t, args, fseeds, n)[1],
                    "forward")
    aseeds = [rng.standard_normal((2, k, n)) for k in t.nnz_out]
    _all_bits_equal(O.reverse(s, args, aseeds, n)[1], O.reverse(t, args, aseeds, n)[1],
                    "adjoint")
    _all_bits_equal(O.jacobian(s, args, n)[1], O.jacobian(t, args, n)[1], "jacobian")
    bits = [np.full((k, n), np.uint64(0), np.uint64) for k in t.nnz_in]
    for j, b in enumerate(bits):
        for k in range(b.shape[0]):
            b[k, :] = np.uint64(1) << np.uint64((j * 7 + k) % 64)
    _all_bits_equal(O.sp_forward(s, bits, n), O.sp_forward(t, bits, n), "sp_forward")


def test_schedule_shortens_the_rollout_work_vector():
    t = W.cartpole_rollout(20).tape
    s = R.schedule(t)
    assert t.sz_w == 122 and s.sz_w <= 70


def test_schedule_golden_tapes():
    z = load_npz("tapes.npz")
    for name in ("cartpole", "rollout", "dag"):
        t = golden_tape(z, name)
        s = R.schedule(t)
        args = golden_list(z, name, "arg", len(t.nnz_in))
        n = args[0].shape[-1]
        _all_bits_equal(O.eval(s, args, n), O.eval(t, args, n), name)
        aseeds = golden_list(z, name, "aseed", len(t.nnz_out))
        _all_bits_equal(O.reverse(s, args, aseeds, n)[1], O.reverse(t, args, aseeds, n)[1], name)


def test_schedule_rejects_read_before_write():
    t = W.cartpole_step().tape
    k = int(np.argmax(t.op == C.OP_MUL))
    t.i1[k] = t.sz_w - 1
    # make sure that slot has not been written before k
    written = set(int(t.i0[j]) for j in range(k) if t.op[j] != C.OP_OUTPUT)
    if t.sz_w - 1 in written:
        pytest.skip("slot already written in this tape")
    with pytest.raises(R.CasadiGpuError, match="before it is written"):
        R.schedule(t)


def test_schedule_is_idempotent_on_its_output():
    t = W.cartpole_rollout(5).tape
    s1 = R.schedule(t)
    s2 = R.schedule(s1)
    assert s2.sz_w <= s1.sz_w
