"""Generate ``casadi.npz`` and the ``serialized_casadi_*.txt`` fixtures from CasADi itself.

Everything here comes out of the reference's own libcasadi, compiled from its casadi/core
sources by ``oracle/Makefile`` (``make casadi``) and driven through ``oracle/casadi_bridge.cpp``:
the tapes its SX builds, the outputs of its Function calls (plain evaluation, ``jacobian()``,
``reverse(1)``, ``forward(2)``), its bvec_t sparsity sweeps, Jacobian sparsity, the seed
colourings of ``get_partition`` and ``Sparsity::uni_coloring`` / ``star_coloring``, the SX
``hessian()`` / ``jacobian()`` Functions of the scenario-MPC Lagrangian, the call records of a
rollout written as never-inlined calls, and ``Function::serialize()`` texts.

Run where the reference source tree is available:

    CASADI_REFERENCE=<reference tree> python tests/golden/make_casadi_golden.py

Inputs are drawn by this repository's seeded generators (casadi_gb300.workloads) and stored
beside the outputs, so a test needs only the fixture. Large tapes are stored as the SHA-256 of
their canonical bytes (tests/helpers.py: canonical_tape_bytes) with their sizes; small ones in
full. Layout: instance-minor ``(nnz, n)`` per input/output; forward seeds/sensitivities
``(ndir, nnz, n)``; adjoint ones ``(nadj, nnz, n)``.
"""
import hashlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from casadi_gb300 import workloads as W  # noqa: E402
from oracle import casadi_ref as R  # noqa: E402
from helpers import canonical_tape_bytes  # noqa: E402

FULL_TAPE_MAX = 10000


def build_casadi():
    ref = os.environ.get("CASADI_REFERENCE")
    if not ref:
        raise SystemExit("set CASADI_REFERENCE to the reference source tree")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "casadi",
                           "REF=" + ref])


def put_tape(out, name, f):
    op, i0, i1, i2, d = f.tape()
    out[name + "/n_instr"] = np.array(f.n_instr)
    out[name + "/sz_w"] = np.array(f.sz_w)
    out[name + "/nnz_in"] = np.array(f.nnz_in, np.int32)
    out[name + "/nnz_out"] = np.array(f.nnz_out, np.int32)
    out[name + "/tape_sha256"] = np.array(
        hashlib.sha256(canonical_tape_bytes(op, i0, i1, i2, d)).hexdigest())
    if f.n_instr <= FULL_TAPE_MAX:
        for k, v in zip(("op", "i0", "i1", "i2", "d"), (op, i0, i1, i2, d)):
            out["%s/%s" % (name, k)] = v


def put_reverse_tape(out, name, f):
    """The sizes and hash of f.reverse(1)'s tape (sx.reverse_function rebuilds it)."""
    r = f.reverse(1)
    out[name + "/rev1_n_instr"] = np.array(r.n_instr)
    out[name + "/rev1_sz_w"] = np.array(r.sz_w)
    out[name + "/rev1_tape_sha256"] = np.array(
        hashlib.sha256(canonical_tape_bytes(*r.tape())).hexdigest())


def put_list(out, name, key, arrs):
    for j, a in enumerate(arrs):
        out["%s/%s%d" % (name, key, j)] = np.asarray(a)


def put_pattern(out, key, p):
    out[key + "_shape"] = np.array([p.nrow, p.ncol], np.int32)
    out[key + "_colind"] = p.colind.astype(np.int32)
    out[key + "_row"] = p.row.astype(np.int32)


def eval_case(out, name, f, args, n, rng, nfwd=2, jac=True):
    """Values, jacobian() blocks, reverse(1) and forward(nfwd) with seeded seeds."""
    put_list(out, name, "arg", args)
    put_list(out, name, "res", f.eval(args, n))
    n_in, n_out = f.n_in, f.n_out
    if jac:
        J = f.jacobian()
        blocks = J.eval(list(args) + [None] * n_out, n)
        k = 0
        for o in range(n_out):
            for i in range(n_in):
                put_pattern(out, "%s/jac_%d_%d" % (name, o, i), J.sparsity_out(k))
                out["%s/jac_%d_%d" % (name, o, i)] = blocks[k]
                k += 1
    # reverse(1): inputs (args, outputs (no nonzeros needed), adjoint seeds)
    aseeds = [rng.standard_normal((1, m, n)) for m in f.nnz_out]
    B = f.reverse(1)
    asens = B.eval(list(args) + [None] * n_out + [a[0] for a in aseeds], n)
    put_list(out, name, "aseed", aseeds)
    put_list(out, name, "asens", [a[None] for a in asens])
    # forward(nfwd): seed of input i is its (nnz_i x nfwd) matrix, nonzero d*nnz_i + k
    fseeds = [rng.standard_normal((nfwd, m, n)) for m in f.nnz_in]
    Fw = f.forward(nfwd)
    fs = Fw.eval(list(args) + [None] * n_out + [s.reshape(nfwd * s.shape[1], n)
                                                  for s in fseeds], n)
    put_list(out, name, "fseed", fseeds)
    put_list(out, name, "fsens", [s.reshape(nfwd, m, n) for s, m in zip(fs, f.nnz_out)])


def sp_case(out, name, f, trials, rng):
    """bvec_t sweeps: ``trials`` independent calls with random 64-bit words, stored as
    (nnz, trials) like instances."""
    def words(m):
        return rng.integers(0, 2**63, size=(m, trials), dtype=np.int64).view(np.uint64) ^ \
            (rng.integers(0, 2, size=(m, trials), dtype=np.int64).view(np.uint64) << 63)
    seeds_f = [words(m) for m in f.nnz_in]
    res_f = [np.zeros((m, trials), np.uint64) for m in f.nnz_out]
    seeds_r = [words(m) for m in f.nnz_out]
    res_r = [np.zeros((m, trials), np.uint64) for m in f.nnz_in]
    for t in range(trials):
        r = f.sp_forward([s[:, t] for s in seeds_f])
        for j, v in enumerate(r):
            res_f[j][:, t] = v
        a, consumed = f.sp_reverse([s[:, t] for s in seeds_r])
        for j, v in enumerate(a):
            res_r[j][:, t] = v
        assert all((c == 0).all() for c in consumed)
    put_list(out, name, "spf_seed", seeds_f)
    put_list(out, name, "spf_res", res_f)
    put_list(out, name, "spr_seed", seeds_r)
    put_list(out, name, "spr_res", res_r)
    for o in range(f.n_out):
        for i in range(f.n_in):
            put_pattern(out, "%s/jacsp_%d_%d" % (name, o, i), f.jac_sparsity(o, i))


EXACT_MAP = np.array([0, 1, 3, 3, 8, 3, 8, 1, 8, 0], np.int32)


def exact_dag_nodes(n_in, n_nodes, seed):
    """A node list of the random-DAG generator whose ops are all IEEE-exact: add, sub,
    a/(b^2+1), sqrt(a^2+1) (mul -> div, sin/exp/sqrt -> sqrt, cos -> div, log -> sub,
    tanh -> add), so every value stays finite and of moderate size."""
    op, a, b = W.dag_nodes(n_in, n_nodes, seed, 256)
    return EXACT_MAP[op], a, b


def main():
    build_casadi()
    out = {"casadi_version": np.array(R.version(), np.int32)}
    rng = np.random.default_rng(2024)

    f = R.build("cartpole")
    put_tape(out, "cartpole", f)
    put_reverse_tape(out, "cartpole", f)
    eval_case(out, "cartpole", f, W.cartpole_inputs(128, steps=1, seed=21), 128, rng, nfwd=3)

    f = R.build("rollout", 20)
    put_tape(out, "rollout", f)
    put_reverse_tape(out, "rollout", f)
    eval_case(out, "rollout", f, W.cartpole_inputs(32, steps=20, seed=22), 32, rng)

    f = R.build("rollout", 100)
    put_tape(out, "rollout100", f)
    args = W.cartpole_inputs(8, steps=100, seed=23)
    put_list(out, "rollout100", "arg", args)
    put_list(out, "rollout100", "res", f.eval(args, 8))
    seed = [np.zeros((4, 8)), np.ones((1, 8))]
    put_list(out, "rollout100", "asens",
             [a[None] for a in f.reverse(1).eval(list(args) + [None, None] + seed, 8)])

    op, a, b = W.dag_nodes(64, 10000, 0, 256)
    f = R.build_dag(64, 16, op, a, b)
    put_tape(out, "dag", f)
    put_reverse_tape(out, "dag", f)
    args = W.dag_inputs(32, n_in=64, seed=24)
    put_list(out, "dag", "arg", args)
    put_list(out, "dag", "res", f.eval(args, 32))
    ones = [np.ones((16, 32))]
    put_list(out, "dag", "asens_sum", f.reverse(1).eval(list(args) + [None] + ones, 32))
    sp_case(out, "dag", f, 16, rng)

    op, a, b = exact_dag_nodes(64, 3000, 5)
    out["dag_exact/nodes"] = np.stack([op, a, b])
    f = R.build_dag(64, 16, op, a, b)
    put_tape(out, "dag_exact", f)
    put_reverse_tape(out, "dag_exact", f)
    eval_case(out, "dag_exact", f, W.dag_inputs(16, n_in=64, seed=25), 16, rng)

    put_tape(out, "dag_small", R.build_dag(16, 6, *W.dag_nodes(16, 800, 3, 256)))

    f = R.build("rollout_calls", 20)
    put_tape(out, "rollout_calls", f)
    calls = []
    for e in range(R.lib().cb_n_calls(f.h)):
        import ctypes as ct
        dep = np.zeros(5, np.int32)
        res = np.zeros(4, np.int32)
        callee = ct.c_int()
        R._check(R.lib().cb_call_info(f.h, e, ct.byref(callee), R._ptr(dep), R._ptr(res)))
        calls.append(np.concatenate([dep, res]))
    out["rollout_calls/calls"] = np.array(calls, np.int32)
    args = W.cartpole_inputs(16, steps=20, seed=26)
    put_list(out, "rollout_calls", "arg", args)
    put_list(out, "rollout_calls", "res", f.eval(args, 16))

    # scenario MPC: the Lagrangian, its gradient, the SX hessian() and jacobian() Functions,
    # and the seed colourings jacobian/hessian would use
    K = 100
    L = R.build("quad_lagrangian", K)
    put_tape(out, "quad_lagrangian", L)
    G = R.build("quad_gradient", K)
    put_tape(out, "quad_gradient", G)
    n = 1
    args = W.quad_ms_inputs(n, intervals=K, seed=27)
    put_list(out, "quad", "arg", args)
    put_list(out, "quad", "res", L.eval(args, n))
    put_list(out, "quad", "grad", G.eval(args, n))
    H = R.build("quad_hessian", K)
    put_pattern(out, "quad/hess", H.sparsity_out(0))
    out["quad/hess"] = H.eval(args, n)[0]
    Jg = R.build("quad_jac_g", K)
    put_pattern(out, "quad/jac_g", Jg.sparsity_out(0))
    out["quad/jac_g"] = Jg.eval(args, n)[0]
    gh = R.build("quad_grad_helper", K)
    star, _ = gh.partition(0, 0, symmetric=True)
    out["quad/partition_hess_star"] = star
    hp = gh.jac_sparsity(0, 0)
    put_pattern(out, "quad/hess_jacsp", hp)
    gj = R.build("quad_g_helper", K)
    fwd, adj = gj.partition(0, 0, symmetric=False)
    out["quad/partition_jac_fwd"] = fwd if fwd is not None else np.zeros(0, np.int32)
    out["quad/partition_jac_adj"] = adj if adj is not None else np.zeros(0, np.int32)
    jp = gj.jac_sparsity(0, 0)
    put_pattern(out, "quad/jac_jacsp", jp)
    out["quad/uni_coloring_jac"] = R.coloring("uni", jp)[0]
    out["quad/star_coloring_hess"] = R.coloring("star", hp, 1)[0]

    # the 20-step rollout's jacobian() tape in full: the CPU reference legs of the benchmark
    # evaluate CasADi's own derivative tapes (this one and reverse(1), which
    # sx.reverse_function rebuilds) on the oracle's restatement of SXFunction::eval
    J = R.build("rollout", 20).jacobian()
    jt = {}
    put_tape(jt, "jacobian", J)
    op, i0, i1, i2, d = J.tape()
    jt.update({"jacobian/op": op, "jacobian/i0": i0, "jacobian/i1": i1, "jacobian/i2": i2,
               "jacobian/d": d})
    for k in range(J.n_out):
        put_pattern(jt, "jacobian/out%d" % k, J.sparsity_out(k))
    # CasADi's own Jacobian of xN alone (the rollout with xN as its only output): the CPU legs
    # of the benchmark's step (forward Jacobian of xN + adjoint of the cost) run this tape;
    # its values on the rollout's golden inputs pin it
    Jx = R.build("rollout_xn", 20).jacobian()
    put_tape(jt, "jacobian_xn", Jx)
    op, i0, i1, i2, d = Jx.tape()
    jt.update({"jacobian_xn/op": op, "jacobian_xn/i0": i0, "jacobian_xn/i1": i1,
               "jacobian_xn/i2": i2, "jacobian_xn/d": d})
    for k in range(Jx.n_out):
        put_pattern(jt, "jacobian_xn/out%d" % k, Jx.sparsity_out(k))
    ra = W.cartpole_inputs(32, steps=20, seed=22)  # the "rollout" case's inputs
    for k, r in enumerate(Jx.eval(list(ra) + [None], ra[0].shape[1])):
        jt["jacobian_xn/res%d" % k] = r
    jpath = os.path.join(HERE, "casadi_rollout20_jacobian.npz")
    np.savez_compressed(jpath, **jt)
    print("casadi_rollout20_jacobian.npz", os.path.getsize(jpath), "bytes")

    path = os.path.join(HERE, "casadi.npz")
    np.savez_compressed(path, **out)
    print("casadi.npz", os.path.getsize(path), "bytes")

    for name, fn in (("cartpole", R.build("cartpole")),
                     ("rollout_calls", R.build("rollout_calls", 20)),
                     ("dag", R.build_dag(16, 6, *W.dag_nodes(16, 800, 3, 256)))):
        L_ = R.lib()
        m = L_.cb_serialize(fn.h, None, 0)
        buf = (np.zeros(m + 1, np.uint8))
        R._check(L_.cb_serialize(fn.h, R._ptr(buf), m))
        p = os.path.join(HERE, "serialized_casadi_%s.txt" % name)
        with open(p, "wb") as fh:
            fh.write(buf[:m].tobytes() + b"\n")
        print(os.path.basename(p), os.path.getsize(p), "bytes")


if __name__ == "__main__":
    main()
