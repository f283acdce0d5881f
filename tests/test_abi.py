"""The C ABI library: it loads, exports every entry point include/casadi_gb300.h declares, and
its host-side tape validation rejects malformed tapes before any device work (these run
without a GPU)."""
import ctypes as ct

import numpy as np
import pytest

from casadi_gb300 import calculus as C
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W


@pytest.fixture(scope="module")
def lib():
    return R.load()


def test_header_declares_entry_points():
    syms = R.declared_symbols()
    for s in ("casadi_gb300_tape_create", "casadi_gb300_eval", "casadi_gb300_forward",
              "casadi_gb300_reverse", "casadi_gb300_sp_forward", "casadi_gb300_sp_reverse",
              "casadi_gb300_map_eval", "casadi_gb300_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in R.declared_symbols():
        assert hasattr(lib, s), s


def test_version(lib):
    assert R.version().count(".") == 2


def _create(lib, tape, op=None, i0=None, i1=None, i2=None, sz_w=None):
    atoms = tape.atomic_array()
    if op is not None:
        atoms["op"] = op
    nnz_in = np.asarray(tape.nnz_in, np.int32)
    nnz_out = np.asarray(tape.nnz_out, np.int32)
    st = lib.casadi_gb300_tape_create(atoms.ctypes.data, tape.n_instr, len(tape.nnz_in),
                                      nnz_in.ctypes.data, len(tape.nnz_out),
                                      nnz_out.ctypes.data,
                                      tape.sz_w if sz_w is None else sz_w)
    return st, lib.casadi_gb300_last_error().decode()


def _mutate(tape, k, field, value):
    t = W.cartpole_step().tape
    getattr(t, field)[k] = value
    return t


def test_rejects_slot_out_of_range(lib):
    t = W.cartpole_step().tape
    k = int(np.argmax(t.op == C.OP_MUL))
    t.i1[k] = t.sz_w
    st, msg = _create(lib, t)
    assert st == -2 and "slot out of range" in msg


def test_rejects_bad_input_reference(lib):
    t = W.cartpole_step().tape
    k = int(np.argmax(t.op == C.OP_INPUT))
    t.i2[k] = 99
    st, msg = _create(lib, t)
    assert st == -2 and "input reference" in msg


def test_rejects_unknown_op_and_call(lib):
    t = W.cartpole_step().tape
    k = int(np.argmax(t.op == C.OP_ADD))
    t.op[k] = 77
    st, msg = _create(lib, t)
    assert st == -6 and "unknown op" in msg
    t = W.cartpole_step().tape
    t.op[k] = C.OP_CALL
    st, msg = _create(lib, t)
    assert st == -6 and "OP_CALL" in msg


def test_rejects_unwritten_output(lib):
    t = W.cartpole_step().tape
    keep = np.ones(t.n_instr, bool)
    keep[np.flatnonzero(t.op == C.OP_OUTPUT)[-1]] = False
    from casadi_gb300.sx import Tape
    t2 = Tape(t.op[keep], t.i0[keep], t.i1[keep], t.i2[keep], t.d[keep], t.nnz_in, t.nnz_out,
              t.sz_w)
    st, msg = _create(lib, t2)
    assert st == -2 and "never written" in msg


def test_rejects_bad_ids(lib):
    assert lib.casadi_gb300_tape_free(12345) == -1
    assert lib.casadi_gb300_eval(12345, 1, 1, None, None, None) == -1
    assert "no tape" in lib.casadi_gb300_last_error().decode()


def test_package_map_and_mapaccum_pick_the_reference_shapes():
    """casadi_gb300.map / mapaccum mirror Function::map / mapaccum: n == 1 returns f, reduce
    flags give a MapSum, other parallelizations are refused (no device needed to check)."""
    import casadi_gb300 as cg
    f = W.cartpole_step()
    assert cg.map(f, 1) is f
    with pytest.raises(ValueError):
        cg.map(f, 4, "openmp")
