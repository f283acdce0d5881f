"""Tape builder: CasADi's SX simplification rules and SXFunction::init, checked against the
tapes the reference's own libcasadi builds for the same functions (tests/golden/casadi.npz,
written by tests/golden/make_casadi_golden.py; more cases in test_casadi_parity.py)."""
import numpy as np
import pytest

from casadi_gb300 import calculus as C
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W

from helpers import golden_tape, load_npz, tape_sha256




@pytest.mark.parametrize("name,make", [
    ("cartpole", W.cartpole_step),
    ("rollout", lambda: W.cartpole_rollout(20)),
])
def test_tape_matches_casadi(name, make):
    z = load_npz("casadi.npz")
    t = make().tape
    assert t.n_instr == int(z[name + "/n_instr"]) and t.sz_w == int(z[name + "/sz_w"])
    ops = z[name + "/op"]
    assert t.histogram() == {C.OP_NAMES[int(o)]: int((ops == o).sum()) for o in np.unique(ops)}
    assert tape_sha256(t) == str(z[name + "/tape_sha256"])


@pytest.mark.parametrize("name,casadi_name,make", [
    ("cartpole", "cartpole", W.cartpole_step),
    ("rollout", "rollout", lambda: W.cartpole_rollout(20)),
    ("dag", "dag_small", lambda: W.random_dag(n_in=16, n_nodes=800, n_out=6, seed=3)),
])
def test_builder_reproduces_golden_tapes(name, casadi_name, make):
    """tapes.npz holds the builder's tapes of these functions; they are CasADi's."""
    z = load_npz("tapes.npz")
    g = golden_tape(z, name)
    t = make().tape
    for f in ("op", "i0", "i1", "i2"):
        np.testing.assert_array_equal(getattr(t, f), getattr(g, f), err_msg=f)
    np.testing.assert_array_equal(t.d.view(np.uint64), g.d.view(np.uint64))
    assert t.sz_w == g.sz_w and t.nnz_in == g.nnz_in and t.nnz_out == g.nnz_out
    assert tape_sha256(g) == str(load_npz("casadi.npz")[casadi_name + "/tape_sha256"])


def _check_tape_wellformed(t):
    """Every slot is written before it is read, slots < sz_w, unary ops carry i2 == i1."""
    written = set()
    for k in range(t.n_instr):
        op, i0, i1, i2 = int(t.op[k]), int(t.i0[k]), int(t.i1[k]), int(t.i2[k])
        if op == C.OP_OUTPUT:
            assert i1 in written
        elif op in (C.OP_CONST, C.OP_INPUT):
            assert 0 <= i0 < t.sz_w
            written.add(i0)
        else:
            assert i1 in written and i2 in written
            if C.ndeps(op) == 1:
                assert i1 == i2
            written.add(i0)


def test_tapes_wellformed():
    for f in (W.cartpole_step(), W.cartpole_rollout(5), W.random_dag(n_in=8, n_nodes=300,
                                                                      n_out=4, seed=1)):
        _check_tape_wellformed(f.tape)


def test_on_the_fly_simplification():
    x, y = S.sym("x"), S.sym("y")
    assert (x * x).is_op(C.OP_SQ)
    assert (2 * x).is_op(C.OP_TWICE) and (x * 2).is_op(C.OP_TWICE)
    assert (x + 0) is x and (0 + x) is x and (x * 1) is x and (x - 0) is x
    assert (x - x).is_zero() and (x / x).is_one()
    assert (-(-x)) is x
    assert (x + (-y)).is_op(C.OP_SUB)
    assert (x + x).is_op(C.OP_TWICE)
    assert S.sq(S.sqrt(x)) is x
    assert S.const(2.0) is S.const(2)               # constants are cached by value
    assert (S.const(3.0) * 4.0).is_constant() and float(S.const(3.0) * 4.0) == 12.0
    assert S.power(x, 3).is_op(C.OP_MUL)            # x*pow(x,2) = x*sq(x)
    assert S.power(x, 0.5).is_op(C.OP_SQRT)
    assert S.if_else_zero(S.const(0.0), x).is_zero()


def test_live_variables_reuse_slots():
    x = S.sym("x", 2)
    e = S.sin(x[0]) + S.cos(x[1])
    f = S.Function("f", [x], [[e, e * x[0]]])
    f_nolive = S.Function("f", [x], [[e, e * x[0]]], live_variables=False)
    assert f.sz_w() < f_nolive.sz_w()
    assert f.n_instructions() == f_nolive.n_instructions()


def test_instruction_accessors():
    f = W.cartpole_step()
    for k in range(f.n_instructions()):
        op = f.instruction_id(k)
        if op == C.OP_INPUT:
            assert len(f.instruction_input(k)) == 2
        if op == C.OP_OUTPUT:
            assert len(f.instruction_output(k)) == 2
        if op == C.OP_CONST:
            assert f.instruction_input(k) == []
            assert f.instruction_constant(k) == f.tape.d[k]


def test_free_variable_rejected():
    x, p = S.sym("x"), S.sym("p")
    with pytest.raises(ValueError):
        S.Function("f", [[x]], [[x * p]])


def test_atomic_array_layout():
    t = W.cartpole_step().tape
    a = t.atomic_array()
    assert a.itemsize == 16
    k = int(np.argmax(t.op == C.OP_CONST))
    assert a["u"][k] == t.d[k:k + 1].view(np.uint64)[0]
    k = int(np.argmax(t.op == C.OP_ADD))
    assert a["u"][k] == (int(t.i1[k]) | (int(t.i2[k]) << 32))
