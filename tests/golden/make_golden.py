"""Generate the golden fixtures of this directory from the reference's own op semantics.

Run where the reference source tree is available (it builds oracle/_ref from the reference's
casadi/core sources):

    CASADI_REFERENCE=<reference tree> python tests/golden/make_golden.py \
        [ops] [enum] [tapes] [activity] [serial]  # default: all

Fixtures:
  ops.npz        value and partials of every scalar op over a grid of special and ordinary
                 arguments: casadi_math<double>::fun/der (calculus.hpp:1299-1439) as compiled
                 from the reference header.
  enum.npz       the numeric ids of enum Operation (calculus.hpp:60-218).
  activity.npz   the zero checkers of every op (operation_checker<F0XChecker/FX0Checker/
                 F00Checker>, calculus.hpp:485-540, :1128-1131, as compiled) and the
                 activity words of SXFunction::eval_activity's loop (sx_function.cpp:
                 1684-1718) driving those checkers, on a tape that applies every op to every
                 pair of active/inactive operands and on the tapes of tapes.npz, for seeded
                 input activity words (zero, all ones and partial bit patterns).
  tapes.npz      the cart-pole step, the 20-step rollout and a small random DAG as tapes, with
                 seeded inputs, forward seeds and adjoint seeds, and the reference harness's
                 outputs: values (SXFunction::eval's loop over CASADI_MATH_FUN_BUILTIN),
                 forward sensitivities, adjoint sensitivities and the unit-seed Jacobian
                 (numeric sweeps with partials from CASADI_MATH_DER_BUILTIN and the
                 structural-zero rules of the reference's derivative expressions).
  serialized_issue3074.txt
                 the one serialized Function the reference's tests hold (test/python/
                 function.py, test_issue_3074: the text passed to StringDeserializer), copied
                 verbatim: an MXFunction written by an earlier CasADi in the saved form (type
                 byte, shared Function), with ProtoFunction body version 1 and FunctionInternal
                 body version 2.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from casadi_gb300 import calculus as C  # noqa: E402
from casadi_gb300 import sx as S  # noqa: E402
from casadi_gb300 import workloads as W  # noqa: E402

SPECIAL = [0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, -2.0, 3.7, -3.7, 1e-300, -1e-300, 5e-324,
           1e300, -1e300, math.inf, -math.inf, math.nan, 0.999999, -0.999999, 1.000001,
           0.7, -0.7, 100.0, -100.0, 710.0, -745.0, 1e-8]


def op_grid():
    rng = np.random.default_rng(1234)
    xs, ys, ops = [], [], []
    for op in sorted(C.ARITH_OPS - {C.OP_PRINTME}):
        ordinary = list(rng.uniform(-4, 4, 24)) + list(rng.uniform(-0.99, 0.99, 8)) + \
            list(np.exp(rng.uniform(-20, 20, 8)))
        vals = SPECIAL + ordinary
        if op in C.BINARY_OPS:
            sub = SPECIAL[:18] + ordinary[:10]
            for x in sub:
                for y in sub:
                    xs.append(x); ys.append(y); ops.append(op)
        else:
            for x in vals:
                xs.append(x); ys.append(x); ops.append(op)
    ops = np.array(ops, np.int32)
    xs = np.array(xs)
    ys = np.array(ys)
    f = np.array([O.ref_fun(int(o), x, y) for o, x, y in zip(ops, xs, ys)])
    d = np.array([O.ref_der(int(o), x, y, fi) for o, x, y, fi in zip(ops, xs, ys, f)])
    return dict(op=ops, x=xs, y=ys, f=f, d0=d[:, 0], d1=d[:, 1])


def tape_case(name, fun, args, nfwd_seed_dirs=None, nadj=1, seed=7):
    t = fun.tape
    n = args[0].shape[-1]
    rng = np.random.default_rng(seed)
    res = O.ref_eval(t, args, n)
    fseeds = [rng.standard_normal((nfwd_seed_dirs, k, n)) for k in t.nnz_in]
    fsens = O.ref_forward(t, args, fseeds, n)
    aseeds = [rng.standard_normal((nadj, k, n)) for k in t.nnz_out]
    asens = O.ref_reverse(t, args, aseeds, n)
    jac = O.ref_jacobian(t, args, n)
    out = {name + "/op": t.op, name + "/i0": t.i0, name + "/i1": t.i1, name + "/i2": t.i2,
           name + "/d": t.d, name + "/nnz_in": np.array(t.nnz_in), name + "/nnz_out":
           np.array(t.nnz_out), name + "/sz_w": np.array(t.sz_w)}
    for j, a in enumerate(args):
        out["%s/arg%d" % (name, j)] = a
    for j, r in enumerate(res):
        out["%s/res%d" % (name, j)] = r
    for j, s in enumerate(fseeds):
        out["%s/fseed%d" % (name, j)] = s
    for j, s in enumerate(fsens):
        out["%s/fsens%d" % (name, j)] = s
    for j, s in enumerate(aseeds):
        out["%s/aseed%d" % (name, j)] = s
    for j, s in enumerate(asens):
        out["%s/asens%d" % (name, j)] = s
    for j, s in enumerate(jac):
        out["%s/jac%d" % (name, j)] = s
    return out


def activity_ops_tape(seed=5, layer2=400):
    """Every arithmetic op applied to every pair drawn from two inputs and the constants 0,
    1.5, -0 and NaN, then ``layer2`` random ops over those results; every result is an
    output nonzero, and the two inputs pass straight to a second output."""
    rng = np.random.default_rng(seed)
    ops, i0, i1, i2, d = [], [], [], [], []

    def emit(op, a, b=0, c=0, v=0.0):
        ops.append(op); i0.append(a); i1.append(b); i2.append(c); d.append(v)

    emit(C.OP_INPUT, 0, 0, 0)
    emit(C.OP_INPUT, 1, 0, 1)
    for slot, v in ((2, 0.0), (3, 1.5), (4, -0.0), (5, math.nan)):
        emit(C.OP_CONST, slot, v=v)
    pool = list(range(6))
    results = []
    slot = 6
    for op in sorted(C.ARITH_OPS):
        pairs = [(a, b) for a in pool for b in pool] if op in C.BINARY_OPS else \
            [(a, a) for a in pool]
        for a, b in pairs:
            emit(op, slot, a, b)
            results.append(slot)
            slot += 1
    arith = sorted(C.ARITH_OPS)
    for _ in range(layer2):
        op = int(arith[rng.integers(len(arith))])
        a = int(results[rng.integers(len(results))])
        b = int(results[rng.integers(len(results))]) if op in C.BINARY_OPS else a
        emit(op, slot, a, b)
        results.append(slot)
        slot += 1
    for k, r in enumerate(results):
        emit(C.OP_OUTPUT, 0, r, k)
    emit(C.OP_OUTPUT, 1, 0, 0)
    emit(C.OP_OUTPUT, 1, 1, 1)
    return S.Tape(ops, i0, i1, i2, d, [2], [len(results), 2], slot)


def activity_words(nnz, n, rng):
    """Seeded activity words: zero, all ones, single bits and random partial patterns."""
    kinds = rng.integers(0, 5, size=(nnz, n))
    rand = rng.integers(0, 2**63, size=(nnz, n), dtype=np.int64).view(np.uint64)
    out = np.zeros((nnz, n), np.uint64)
    out[kinds == 1] = np.uint64(0xFFFFFFFFFFFFFFFF)
    out[kinds == 2] = np.uint64(1)
    out[kinds == 3] = np.uint64(1) << np.uint64(63)
    out[kinds == 4] = rand[kinds == 4] | np.uint64(4)
    return out


def activity_case():
    out = {}
    ops = sorted(C.ARITH_OPS)
    out["checker/op"] = np.array(ops, np.int32)
    for w, name in enumerate(("zero_first", "zero_second", "zero_both")):
        out["checker/" + name] = np.array([O.ref_zero_checker(w, op) for op in ops], bool)
    rng = np.random.default_rng(77)
    t = activity_ops_tape()
    out.update({"ops/op": t.op, "ops/i0": t.i0, "ops/i1": t.i1, "ops/i2": t.i2, "ops/d": t.d,
                "ops/nnz_in": np.array(t.nnz_in), "ops/nnz_out": np.array(t.nnz_out),
                "ops/sz_w": np.array(t.sz_w)})
    cases = [("ops", t, 300)]
    z = np.load(os.path.join(HERE, "tapes.npz"))
    for name in ("cartpole", "rollout", "dag"):
        tt = S.Tape(z[name + "/op"], z[name + "/i0"], z[name + "/i1"], z[name + "/i2"],
                    z[name + "/d"], z[name + "/nnz_in"].tolist(), z[name + "/nnz_out"].tolist(),
                    int(z[name + "/sz_w"]))
        cases.append((name, tt, 64))
    for name, tt, n in cases:
        args = [activity_words(k, n, rng) for k in tt.nnz_in]
        # some instances with every input inactive
        for a in args:
            a[:, :3] = 0
        res = O.ref_activity(tt, args, n)
        for j, a in enumerate(args):
            out["%s/act_arg%d" % (name, j)] = a
        for j, r in enumerate(res):
            out["%s/act_res%d" % (name, j)] = r
    return out


REFERENCE = os.environ.get("CASADI_REFERENCE")


def serialized_fixture():
    """The serialized text of test_issue_3074 in the reference's test/python/function.py."""
    if not REFERENCE:
        raise SystemExit("set CASADI_REFERENCE to the reference source tree")
    path = os.path.join(REFERENCE, "test", "python", "function.py")
    lines = open(path).read().splitlines()
    start = next(i for i, l in enumerate(lines) if "def test_issue_3074" in l)
    for line in lines[start:]:
        stripped = line.strip()
        if stripped.startswith("data = \""):
            return stripped.split("\"")[1]
    raise SystemExit("no serialized text in test_issue_3074")


def main(which=None):
    which = set(which or ("ops", "enum", "tapes", "activity", "serial"))
    written = []
    if "serial" in which:
        with open(os.path.join(HERE, "serialized_issue3074.txt"), "w") as fh:
            fh.write(serialized_fixture() + "\n")
        written.append("serialized_issue3074.txt")
    if which - {"serial"}:
        O.build(ref=True, tree=REFERENCE)
        if not O.ref_available():
            raise SystemExit("the reference harness could not be built")
    if "ops" in which:
        np.savez_compressed(os.path.join(HERE, "ops.npz"), **op_grid())
        written.append("ops.npz")
    if "enum" in which:
        names = sorted(C.OP_NAMES.values())
        ids = np.array([O.ref().ref_op_id(("OP_" + s).encode()) for s in names], np.int32)
        np.savez_compressed(os.path.join(HERE, "enum.npz"), names=np.array(names), ids=ids)
        written.append("enum.npz")
    if "tapes" in which:
        write_tapes()
        written.append("tapes.npz")
    if "activity" in which:
        np.savez_compressed(os.path.join(HERE, "activity.npz"), **activity_case())
        written.append("activity.npz")
    for f in written:
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


def write_tapes():
    tapes = {}
    tapes.update(tape_case("cartpole", W.cartpole_step(), W.cartpole_inputs(96, steps=1, seed=0),
                           nfwd_seed_dirs=3))
    tapes.update(tape_case("rollout", W.cartpole_rollout(20), W.cartpole_inputs(40, steps=20,
                                                                                seed=1),
                           nfwd_seed_dirs=2, nadj=2))
    tapes.update(tape_case("dag", W.random_dag(n_in=16, n_nodes=800, n_out=6, seed=3),
                           W.dag_inputs(40, n_in=16, seed=2), nfwd_seed_dirs=2))
    np.savez_compressed(os.path.join(HERE, "tapes.npz"), **tapes)


if __name__ == "__main__":
    main(sys.argv[1:])
