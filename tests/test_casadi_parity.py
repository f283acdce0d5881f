"""Parity with CasADi itself, on the CPU: the builder's tapes, the oracle's sweeps, the
colourings and the serialized-Function decoder against what the reference's own libcasadi
produced (tests/golden/casadi.npz and serialized_casadi_*.txt, written by
tests/golden/make_casadi_golden.py through oracle/casadi_bridge.cpp).

Bars:
  * tapes: identical instruction for instruction (canonical bytes, SHA-256);
  * evaluation: bit-exact on tapes of IEEE-exact ops; elsewhere relative error <= 1e-13 per
    element (bit-exact on the host that generated the fixtures, whose libm CasADi used);
  * sparsity sweeps, Jacobian patterns and colourings: identical;
  * numeric AD (the oracle's sweeps, like the GPU's) against CasADi's symbolic derivative
    Functions: |a - b| <= 1e-13 x magnitude per element, the magnitude being the same sweep
    over |partials| and |seeds| (oracle.magnitude). The two cannot share bits: CasADi's
    symbolic partials simplify, e.g. inv(y)*seed to seed/y (one rounding instead of two,
    casadi/core/calculus.hpp simplifications), so even +,-,*,/ tapes round differently;
  * CasADi's own derivative Function (f.reverse(1), rebuilt by sx.reverse_function) evaluated
    by a value sweep: the reference's results operation for operation, bit-exact on exact
    tapes.
"""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import coloring as K
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W
from oracle import casadi_ref as CR

from helpers import (EXACT_OPS, assert_bitexact, casadi_tape, golden_list, load_npz,
                     rel_err, same_bits, tape_sha256)

AD_RTOL = 1e-13
EXACT_MAP = np.array([0, 1, 3, 3, 8, 3, 8, 1, 8, 0], np.int32)


@pytest.fixture(scope="module")
def z():
    return load_npz("casadi.npz")


def builders():
    op, a, b = W.dag_nodes(64, 3000, 5, 256)
    return {
        "cartpole": W.cartpole_step,
        "rollout": lambda: W.cartpole_rollout(20),
        "rollout100": lambda: W.cartpole_rollout(100),
        "dag": lambda: W.random_dag(64, 10000, 16, seed=0),
        "dag_exact": lambda: W.dag_from_nodes(64, 16, EXACT_MAP[op], a, b),
        "dag_small": lambda: W.random_dag(16, 800, 6, seed=3),
        "quad_lagrangian": lambda: W.quad_ms_lagrangian(100),
    }


_cache = {}


def built(name):
    if name not in _cache:
        _cache[name] = builders()[name]()
    return _cache[name]


def quad_gradient_function():
    if "quad_gradient" not in _cache:
        L = built("quad_lagrangian")
        _cache["quad_gradient"] = S.Function("grad_L", L.inputs, [S.gradient(L, 1, 0)])
    return _cache["quad_gradient"]


def assert_within_magnitude(got, ref, mag, what, rtol=AD_RTOL):
    got, ref, mag = (np.asarray(v, np.float64) for v in (got, ref, mag))
    d = np.abs(got - ref)
    bad = ~(same_bits(got, ref) | (d <= rtol * mag))
    if bad.any():
        i = tuple(np.argwhere(bad)[0])
        raise AssertionError("%s: %d of %d beyond %.0e x magnitude, e.g. %s: %r vs %r (mag %r)"
                             % (what, int(bad.sum()), bad.size, rtol, i, got[i], ref[i], mag[i]))
    return float(np.max(np.where(mag > 0, d / np.where(mag > 0, mag, 1), 0.0), initial=0.0))


def is_exact(t):
    return all(int(o) in EXACT_OPS or int(o) in (C.OP_CONST, C.OP_INPUT, C.OP_OUTPUT)
               for o in np.unique(t.op))


def test_fixtures_come_from_casadi_3_7_2(z):
    assert z["casadi_version"].tolist() == [3, 7, 2]


# ---- tapes --------------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["cartpole", "rollout", "rollout100", "dag", "dag_exact",
                                  "dag_small", "quad_lagrangian"])
def test_builder_tapes_are_casadis(z, name):
    t = built(name).tape
    assert t.n_instr == int(z[name + "/n_instr"])
    assert t.sz_w == int(z[name + "/sz_w"])
    assert t.nnz_in == z[name + "/nnz_in"].tolist()
    assert t.nnz_out == z[name + "/nnz_out"].tolist()
    assert tape_sha256(t) == str(z[name + "/tape_sha256"])


def test_builder_gradient_tape_is_casadis(z):
    """gradient(lag, w) of the MPC Lagrangian: the Hessian's input tape."""
    t = quad_gradient_function().tape
    assert (t.n_instr, t.sz_w) == (int(z["quad_gradient/n_instr"]), int(z["quad_gradient/sz_w"]))
    assert tape_sha256(t) == str(z["quad_gradient/tape_sha256"])


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag", "dag_exact"])
def test_builder_reverse_functions_are_casadis(z, name):
    """f.reverse(1) as CasADi builds it (symbolic ad_reverse): the same tape."""
    t = S.reverse_function(built(name)).tape
    assert t.n_instr == int(z[name + "/rev1_n_instr"])
    assert t.sz_w == int(z[name + "/rev1_sz_w"])
    assert tape_sha256(t) == str(z[name + "/rev1_tape_sha256"])


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag", "dag_exact"])
def test_stored_tapes_equal_builders(z, name):
    """The fixture's full tapes (what the GPU tests run) are the builder's tapes."""
    t = casadi_tape(z, name)
    assert tape_sha256(t) == str(z[name + "/tape_sha256"]) == tape_sha256(built(name).tape)


# ---- evaluation ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag", "dag_exact", "rollout100"])
def test_oracle_eval_matches_casadi(z, name):
    t = built(name).tape
    args = golden_list(z, name, "arg", len(t.nnz_in))
    res = O.eval(t, args, args[0].shape[1])
    for j, r in enumerate(golden_list(z, name, "res", len(t.nnz_out))):
        if is_exact(t):
            assert_bitexact(res[j], r, "%s res%d" % (name, j))
        else:
            assert rel_err(res[j], r) <= 1e-13, name


def test_oracle_eval_matches_casadi_on_the_mpc(z):
    t = built("quad_lagrangian").tape
    args = golden_list(z, "quad", "arg", 3)
    res = O.eval(t, args, 1)
    for j, r in enumerate(golden_list(z, "quad", "res", 2)):
        assert rel_err(res[j], r) <= 1e-13


# ---- numeric AD against CasADi's derivative Functions ----------------------------------------
def _pattern(z, key):
    nr, nc = z[key + "_shape"]
    return K.Pattern(nr, nc, z[key + "_colind"], z[key + "_row"])


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag_exact"])
def test_oracle_jacobian_matches_casadi_jacobian(z, name):
    t = built(name).tape
    args = golden_list(z, name, "arg", len(t.nnz_in))
    n = args[0].shape[1]
    _, jac = O.jacobian(t, args, n)
    with O.magnitude():
        _, mag = O.jacobian(t, args, n)
    off = np.cumsum([0] + t.nnz_in)
    for o in range(len(t.nnz_out)):
        for i in range(len(t.nnz_in)):
            key = "%s/jac_%d_%d" % (name, o, i)
            p = _pattern(z, key)
            rows, cols = p.row, p.col()
            assert_within_magnitude(jac[o][off[i] + cols, rows], z[key],
                                    mag[o][off[i] + cols, rows], key)
            # entries outside CasADi's pattern are structurally zero here too
            full = np.zeros((p.nrow, p.ncol), bool)
            full[rows, cols] = True
            outside = jac[o][off[i]:off[i + 1]].transpose(1, 0, 2)[~full]
            assert (outside == 0).all(), key


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag_exact"])
def test_oracle_reverse_and_forward_match_casadi(z, name):
    t = built(name).tape
    nin, nout = len(t.nnz_in), len(t.nnz_out)
    args = golden_list(z, name, "arg", nin)
    n = args[0].shape[1]
    aseeds = golden_list(z, name, "aseed", nout)
    _, asens = O.reverse(t, args, aseeds, n)
    with O.magnitude():
        _, amag = O.reverse(t, args, aseeds, n)
    for j, r in enumerate(golden_list(z, name, "asens", nin)):
        assert_within_magnitude(asens[j], r, amag[j], "%s asens%d" % (name, j))
    fseeds = golden_list(z, name, "fseed", nin)
    _, fsens = O.forward(t, args, fseeds, n)
    with O.magnitude():
        _, fmag = O.forward(t, args, fseeds, n)
    for j, r in enumerate(golden_list(z, name, "fsens", nout)):
        assert_within_magnitude(fsens[j], r, fmag[j], "%s fsens%d" % (name, j))


def test_oracle_adjoints_of_long_tapes_match_casadi(z):
    """The DAG's adjoint of the sum of its outputs, the 100-step rollout's cost gradient."""
    t = built("dag").tape
    args = golden_list(z, "dag", "arg", 1)
    seed = [np.ones((1, 16, args[0].shape[1]))]
    _, a = O.reverse(t, args, seed, args[0].shape[1])
    with O.magnitude():
        _, m = O.reverse(t, args, seed, args[0].shape[1])
    assert_within_magnitude(a[0][0], z["dag/asens_sum0"], m[0][0], "dag adjoint")
    t = built("rollout100").tape
    args = golden_list(z, "rollout100", "arg", 2)
    n = args[0].shape[1]
    seed = [np.zeros((1, 4, n)), np.ones((1, 1, n))]
    _, a = O.reverse(t, args, seed, n)
    with O.magnitude():
        _, m = O.reverse(t, args, seed, n)
    for j in range(2):
        assert_within_magnitude(a[j], z["rollout100/asens%d" % j], m[j], "rollout100 %d" % j)


def test_oracle_mpc_gradient_matches_casadi(z):
    t = built("quad_lagrangian").tape
    args = golden_list(z, "quad", "arg", 3)
    seed = [np.zeros((1, t.nnz_out[0], 1)), np.ones((1, 1, 1))]
    _, a = O.reverse(t, args, seed, 1)
    with O.magnitude():
        _, m = O.reverse(t, args, seed, 1)
    assert_within_magnitude(a[0][0], z["quad/grad0"], m[0][0], "MPC gradient")


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag_exact"])
def test_casadi_reverse_function_evaluated_gives_casadis_bits(z, name):
    """The reference's way: f.reverse(1) is an SXFunction whose tape a value sweep evaluates
    (this is what a mapped derivative runs through the value kernel); on the generating host
    that reproduces CasADi's adjoint bit for bit."""
    f = built(name)
    B = S.reverse_function(f)
    nin, nout = len(f.tape.nnz_in), len(f.tape.nnz_out)
    args = golden_list(z, name, "arg", nin)
    seeds = [s[0] for s in golden_list(z, name, "aseed", nout)]
    res = O.eval(B.tape, args + [None] * nout + seeds, args[0].shape[1])
    for j, r in enumerate(golden_list(z, name, "asens", nin)):
        if is_exact(f.tape):
            assert_bitexact(res[j], r[0], "%s reverse(1) %d" % (name, j))
        else:
            assert rel_err(res[j], r[0]) <= 1e-13


# ---- sparsity -----------------------------------------------------------------------------
def test_oracle_sparsity_sweeps_match_casadi(z):
    t = built("dag").tape
    seeds = golden_list(z, "dag", "spf_seed", 1)
    n = seeds[0].shape[1]
    res = O.sp_forward(t, seeds, n)
    assert (res[0] == z["dag/spf_res0"]).all()
    out_seeds = [np.array(s) for s in golden_list(z, "dag", "spr_seed", 1)]
    args = [np.zeros_like(seeds[0])]
    O.sp_reverse(t, args, out_seeds, n)
    assert (args[0] == z["dag/spr_res0"]).all()
    assert (out_seeds[0] == 0).all()


def _pattern_by_forward_sweeps(t, n_in):
    """Jacobian pattern of output 0 w.r.t. input 0 from bvec forward sweeps, 64 columns per
    sweep: instance s seeds column 64*s + bit."""
    n = (n_in + 63) // 64
    seeds = np.zeros((n_in, n), np.uint64)
    for c in range(n_in):
        seeds[c, c // 64] = np.uint64(1) << np.uint64(c % 64)
    args = [seeds] + [np.zeros((k, n), np.uint64) for k in t.nnz_in[1:]]
    r = O.sp_forward(t, args, n)[0]
    mask = np.zeros((t.nnz_out[0], n_in), bool)
    for c in range(n_in):
        mask[:, c] = (r[:, c // 64] >> np.uint64(c % 64)) & np.uint64(1) == 1
    return mask


def test_jacobian_patterns_match_casadi(z):
    t = built("dag").tape
    p = _pattern(z, "dag/jacsp_0_0")
    assert (_pattern_by_forward_sweeps(t, 64) == p.dense()).all()


def test_mpc_patterns_match_casadi(z):
    """The MPC's constraint-Jacobian pattern and the (symmetric) Hessian pattern from the
    gradient tape, as the coloured sweeps derive them, equal CasADi's."""
    L = built("quad_lagrangian")
    g = S.Function("g", L.inputs, [L.outputs[0]])
    jac = _pattern_by_forward_sweeps(g.tape, 1612)
    assert (jac == _pattern(z, "quad/jac_jacsp").dense()).all()
    assert (jac == _pattern(z, "quad/jac_g").dense()).all()
    h = _pattern_by_forward_sweeps(quad_gradient_function().tape, 1612)
    assert ((h | h.T) == _pattern(z, "quad/hess_jacsp").dense()).all()
    assert ((h | h.T) == _pattern(z, "quad/hess").dense()).all()


@pytest.fixture(scope="module")
def lib():
    from casadi_gb300 import runtime as R
    try:
        return R.load()
    except Exception as e:  # built by __graft_entry__.build()
        pytest.skip("library not built: %s" % e)


def test_colorings_match_casadi(z, lib):
    jp = _pattern(z, "quad/jac_jacsp")
    assert (K.uni_coloring(jp) == z["quad/uni_coloring_jac"]).all()
    hp = _pattern(z, "quad/hess_jacsp")
    star = K.star_coloring(hp)
    assert (star == z["quad/star_coloring_hess"]).all()
    # get_partition's seeds for hessian(): the same star colouring
    assert (star == z["quad/partition_hess_star"]).all()
    assert star.max() + 1 == 10 and K.uni_coloring(jp).max() + 1 == 14
    # for jacobian(g, w) get_partition weighs forward against adjoint colourings; the one it
    # keeps is recorded (forward mode here, the uni colouring of the columns)
    fwd, adj = z["quad/partition_jac_fwd"], z["quad/partition_jac_adj"]
    assert fwd.size == 1612 and adj.size == 0
    assert (fwd == z["quad/uni_coloring_jac"]).all()


# ---- serialized Functions written by CasADi ----------------------------------------------------
@pytest.mark.parametrize("name,key", [("cartpole", "cartpole"), ("dag", "dag_small")])
def test_decoder_reads_casadis_serialize_output(z, lib, name, key):
    from casadi_gb300 import runtime as R
    from helpers import GOLDEN
    import os
    text = open(os.path.join(GOLDEN, "serialized_casadi_%s.txt" % name)).read()
    t = R.decode_serialized(text)
    assert tape_sha256(t) == str(z[key + "/tape_sha256"])


def test_decoder_reads_casadis_call_records(z, lib):
    from casadi_gb300 import runtime as R
    from helpers import GOLDEN
    import os
    text = open(os.path.join(GOLDEN, "serialized_casadi_rollout_calls.txt")).read()
    d = R.describe_serialized(text)
    top = d["functions"][d["tops"][0]]
    assert top["class"] == "SXFunction" and top["n_instr"] == int(z["rollout_calls/n_instr"])
    assert top["calls"] == [0] * 20
    assert d["functions"][0]["n_instr"] == int(z["cartpole/n_instr"])


# ---- live comparisons where the reference's library is built -------------------------------------
live = pytest.mark.skipif(not CR.available(), reason="libcasadi not built here")


@live
@pytest.mark.parametrize("seed,n_in,n_nodes,n_out,bounded", [
    (11, 8, 300, 3, False), (12, 32, 2000, 8, True), (13, 64, 5000, 16, False),
    (14, 4, 50, 1, False), (15, 128, 4000, 32, True)])
def test_live_random_dags(seed, n_in, n_nodes, n_out, bounded):
    op, a, b = W.dag_nodes(n_in, n_nodes, seed, 256)
    ref = CR.build_dag(n_in, n_out, op, a, b, bounded)
    mine = W.dag_from_nodes(n_in, n_out, op, a, b, bounded)
    import hashlib
    from helpers import canonical_tape_bytes
    assert tape_sha256(mine.tape) == hashlib.sha256(canonical_tape_bytes(*ref.tape())).hexdigest()
    n = 16
    args = W.dag_inputs(n, n_in=n_in, seed=seed)
    for got, want in zip(O.eval(mine.tape, args, n), ref.eval(args, n)):
        assert_bitexact(got, want, "live DAG %d" % seed)


def _jacobian_tape():
    j = load_npz("casadi_rollout20_jacobian.npz")
    return casadi_tape(j, "jacobian"), j


def test_casadi_jacobian_of_xn_fixture_gives_casadis_values(z):
    """CasADi's Jacobian of the rollout's xN alone (the benchmark's CPU legs run it for the
    step's forward Jacobian of xN): the stored tape is pinned by its SHA-256, and the oracle's
    restatement of SXFunction::eval gives CasADi's values of it bit for bit, and they are the
    full jacobian()'s xN blocks at their structural positions, bit for bit."""
    j = load_npz("casadi_rollout20_jacobian.npz")
    t = casadi_tape(j, "jacobian_xn")
    assert tape_sha256(t) == str(j["jacobian_xn/tape_sha256"]) and t.n_instr == 15467
    args = golden_list(z, "rollout", "arg", 2)
    n = args[0].shape[1]
    res = O.eval(t, list(args) + [None], n)
    for k in range(2):
        assert_bitexact(res[k], j["jacobian_xn/res%d" % k], "jac xN block %d" % k)
        p = _pattern(j, "jacobian_xn/out%d" % k)
        full = _pattern(z, "rollout/jac_0_%d" % k)
        dense = np.zeros((full.nrow, full.ncol, n))
        dense[full.row, full.col()] = z["rollout/jac_0_%d" % k]
        assert_bitexact(res[k], dense[p.row, p.col()], "against jacobian()'s xN block")


def test_casadi_jacobian_tape_fixture_gives_casadis_jacobian(z):
    """The rollout's jacobian() tape, as CasADi built it, on the oracle's restatement of
    SXFunction::eval gives CasADi's Jacobian bit for bit (the CPU reference legs of the
    benchmark run exactly this)."""
    t, j = _jacobian_tape()
    assert tape_sha256(t) == str(j["jacobian/tape_sha256"]) and t.n_instr == 19964
    args = golden_list(z, "rollout", "arg", 2)
    n = args[0].shape[1]
    res = O.eval(t, list(args) + [None, None], n)
    for k, key in enumerate(("jac_0_0", "jac_0_1", "jac_1_0", "jac_1_1")):
        assert_bitexact(res[k], z["rollout/" + key], key)
