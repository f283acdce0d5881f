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


# ---- level schedule of the cooperative sweeps (casadi_gb300_tape_levels) -------------------
def _reads_writes(op, i0, i1, i2):
    """Slots an instruction reads and the slot it writes (None for OUTPUT)."""
    if op == C.OP_OUTPUT:
        return {int(i1)}, None
    if op in (C.OP_CONST, C.OP_INPUT):
        return set(), int(i0)
    return ({int(i1), int(i2)} if op in C.BINARY_OPS else {int(i1)}), int(i0)


LEVEL_CASES = CASES + [
    ("quad_constraints", lambda: W.quad_ms_constraints(6),
     lambda n: W.quad_ms_inputs(n, intervals=6, seed=2)),
]


@pytest.mark.parametrize("name,make,inputs", LEVEL_CASES, ids=[c[0] for c in LEVEL_CASES])
@pytest.mark.parametrize("width,cap", [(8, 16), (64, 400)])
def test_levels_are_independent_and_keep_every_bit(name, make, inputs, width, cap):
    t = make().tape
    s = R.schedule(t)
    lt, src, begin = R.levels(t, width=width, slot_cap=cap)
    # every instruction of the scheduled tape exactly once, with its own operation
    assert sorted(src.tolist()) == list(range(s.n_instr))
    assert np.array_equal(lt.op, s.op[src])
    assert np.all(np.diff(begin) >= 1) and np.all(np.diff(begin) <= width)
    assert begin[0] == 0 and begin[-1] == lt.n_instr
    # members of a level are independent: nobody reads or writes what another member writes
    for l in range(len(begin) - 1):
        writes, reads = [], []
        for k in range(begin[l], begin[l + 1]):
            r, w = _reads_writes(lt.op[k], lt.i0[k], lt.i1[k], lt.i2[k])
            reads.append(r)
            writes.append(w)
        ws = [w for w in writes if w is not None]
        assert len(ws) == len(set(ws)), "two writes of one slot in level %d" % l
        for a, w in enumerate(writes):
            if w is None:
                continue
            for b, r in enumerate(reads):
                assert a == b or w not in r, "level %d reads a slot it writes" % l
    # executed in order, the leveled tape gives the same bits
    n = 23
    args = inputs(n)
    _all_bits_equal(O.eval(lt, args, n), O.eval(t, args, n), "values")
    bits = [np.full((k, n), np.uint64(0), np.uint64) for k in t.nnz_in]
    for j, b in enumerate(bits):
        for k in range(b.shape[0]):
            b[k, :] = np.uint64(1) << np.uint64((j * 5 + k) % 64)
    _all_bits_equal(O.sp_forward(lt, bits, n), O.sp_forward(t, bits, n), "sp_forward")


def test_levels_expose_parallel_work():
    """The 10000-node random DAG runs in a few hundred levels, the quadcopter multiple-shooting
    constraints in far fewer levels than instructions, with a bounded work vector."""
    dag = W.random_dag().tape
    _, _, begin = R.levels(dag, width=64, slot_cap=400)
    assert len(begin) - 1 < dag.n_instr / 25
    q = W.quad_ms_constraints(100).tape
    lt, _, begin = R.levels(q, width=64, slot_cap=400)
    assert len(begin) - 1 < q.n_instr / 30
    assert lt.sz_w <= 400 + 64


@pytest.mark.parametrize("name,make,inputs", LEVEL_CASES, ids=[c[0] for c in LEVEL_CASES])
def test_reverse_levels_keep_the_users_of_each_value_in_order(name, make, inputs):
    """The cooperative reverse sweep's schedule (negative width): besides independence, no
    two users of a non-constant value share a level and the users of each value follow the
    scheduled tape's order, so adjoints sum their contributions in the sequential order."""
    t = make().tape
    lt, src, begin = R.levels(t, width=-64, slot_cap=400)
    definer = {}  # slot -> (defining op, value id)
    users = {}    # value id -> source indices of its users in level order
    for l in range(len(begin) - 1):
        level_reads = {}
        for k in range(begin[l], begin[l + 1]):
            r, _ = _reads_writes(lt.op[k], lt.i0[k], lt.i1[k], lt.i2[k])
            for slot in r:
                op, vid = definer[slot]
                if op != C.OP_CONST:
                    assert slot not in level_reads, "two users of one value in level %d" % l
                    level_reads[slot] = k
                    users.setdefault(vid, []).append(int(src[k]))
        for k in range(begin[l], begin[l + 1]):
            _, w = _reads_writes(lt.op[k], lt.i0[k], lt.i1[k], lt.i2[k])
            if w is not None:
                definer[w] = (int(lt.op[k]), k)
    for vid, u in users.items():
        assert u == sorted(u), "users of value %d out of order" % vid
    n = 19
    args = inputs(n)
    _all_bits_equal(O.eval(lt, args, n), O.eval(t, args, n), "values")
    rng = np.random.default_rng(3)
    aseeds = [rng.standard_normal((1, k, n)) for k in t.nnz_out]
    _all_bits_equal(O.reverse(lt, args, aseeds, n)[1], O.reverse(R.schedule(t), args, aseeds,
                                                                  n)[1], "adjoint")


# ---- randomized tapes (hypothesis; skipped where it is not installed) ------------------------
def _random_tape(seed, n_in, n_nodes, n_out, window):
    """A random SX DAG over +,-,*,/,sqrt,sin and constants (bounded values)."""
    from casadi_gb300 import sx as S
    rng = np.random.default_rng(seed)
    xs = S.sym("x", n_in)
    nodes = list(xs)
    for k in range(n_nodes):
        a = nodes[int(rng.integers(max(0, len(nodes) - window), len(nodes)))]
        b = nodes[int(rng.integers(max(0, len(nodes) - window), len(nodes)))]
        r = rng.random()
        if r < 0.25:
            e = a + b
        elif r < 0.4:
            e = a - b
        elif r < 0.6:
            e = a * b * 0.5
        elif r < 0.7:
            e = a / (b * b + 1.0)
        elif r < 0.8:
            e = S.sqrt(a * a + 1.0)
        elif r < 0.9:
            e = S.sin(a) + 0.25
        else:
            e = a * float(rng.integers(1, 4))
        nodes.append(e)
    return S.Function("r", [xs], [nodes[-n_out:]]).tape


def test_levels_hold_on_random_tapes():
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=25, deadline=None)
    @hyp.given(seed=st.integers(0, 10**6), n_in=st.integers(1, 6), n_nodes=st.integers(1, 120),
               n_out=st.integers(1, 5), window=st.integers(1, 40),
               width=st.integers(1, 40), cap=st.integers(1, 60),
               ordered=st.booleans())
    def check(seed, n_in, n_nodes, n_out, window, width, cap, ordered):
        t = _random_tape(seed, n_in, n_nodes, min(n_out, n_nodes + n_in), window)
        s = R.schedule(t)
        lt, src, begin = R.levels(t, width=-width if ordered else width, slot_cap=cap)
        assert sorted(src.tolist()) == list(range(s.n_instr))
        assert np.all(np.diff(begin) >= 1) and np.all(np.diff(begin) <= width)
        for l in range(len(begin) - 1):
            ws, rs = [], []
            for k in range(begin[l], begin[l + 1]):
                r_, w_ = _reads_writes(lt.op[k], lt.i0[k], lt.i1[k], lt.i2[k])
                rs.append(r_)
                ws.append(w_)
            real = [w_ for w_ in ws if w_ is not None]
            assert len(real) == len(set(real))
            for a_, w_ in enumerate(ws):
                if w_ is not None:
                    assert all(a_ == b_ or w_ not in r_ for b_, r_ in enumerate(rs))
        n = 5
        args = [np.random.default_rng(seed).uniform(-1, 1, (t.nnz_in[0], n))]
        _all_bits_equal(O.eval(lt, args, n), O.eval(t, args, n), "values")
        if ordered:
            aseeds = [np.ones((1, t.nnz_out[0], n))]
            _all_bits_equal(O.reverse(lt, args, aseeds, n)[1], O.reverse(s, args, aseeds, n)[1],
                            "adjoint")

    check()
