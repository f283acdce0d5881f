"""Generate the golden fixtures of this directory from the reference's own op semantics.

Run where the reference source tree is available (it builds oracle/_ref from the reference's
casadi/core/calculus.hpp):

    python tests/golden/make_golden.py

Fixtures:
  ops.npz        value and partials of every scalar op over a grid of special and ordinary
                 arguments: casadi_math<double>::fun/der (calculus.hpp:1299-1439) as compiled
                 from the reference header.
  enum.npz       the numeric ids of enum Operation (calculus.hpp:60-218).
  tapes.npz      the cart-pole step, the 20-step rollout and a small random DAG as tapes, with
                 seeded inputs, forward seeds and adjoint seeds, and the reference harness's
                 outputs: values (SXFunction::eval's loop over CASADI_MATH_FUN_BUILTIN),
                 forward sensitivities, adjoint sensitivities and the unit-seed Jacobian
                 (numeric sweeps with partials from CASADI_MATH_DER_BUILTIN and the
                 structural-zero rules of the reference's derivative expressions).
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


def main():
    O.build(ref=True)
    if not O.ref_available():
        raise SystemExit("the reference harness could not be built")
    np.savez_compressed(os.path.join(HERE, "ops.npz"), **op_grid())
    names = sorted(C.OP_NAMES.values())
    ids = np.array([O.ref().ref_op_id(("OP_" + s).encode()) for s in names], np.int32)
    np.savez_compressed(os.path.join(HERE, "enum.npz"), names=np.array(names), ids=ids)
    tapes = {}
    tapes.update(tape_case("cartpole", W.cartpole_step(), W.cartpole_inputs(96, steps=1, seed=0),
                           nfwd_seed_dirs=3))
    tapes.update(tape_case("rollout", W.cartpole_rollout(20), W.cartpole_inputs(40, steps=20,
                                                                                seed=1),
                           nfwd_seed_dirs=2, nadj=2))
    tapes.update(tape_case("dag", W.random_dag(n_in=16, n_nodes=800, n_out=6, seed=3),
                           W.dag_inputs(40, n_in=16, seed=2), nfwd_seed_dirs=2))
    np.savez_compressed(os.path.join(HERE, "tapes.npz"), **tapes)
    for f in ("ops.npz", "enum.npz", "tapes.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
