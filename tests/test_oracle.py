"""The oracle (plain-C restatement of the SX VM) checked against the golden fixtures that the
reference's own op semantics produced, and, where the reference harness is built, directly
against it. These pin the oracle before it is trusted as the GPU parity checker."""
import math

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import sx as S

from helpers import (EXACT_OPS, RTOL, assert_bitexact, assert_close, golden_list, golden_tape,
                     load_npz, same_bits)


def test_enum_ids_match_reference():
    z = load_npz("enum.npz")
    by_name = {v: k for k, v in C.OP_NAMES.items()}
    for name, rid in zip(z["names"], z["ids"]):
        assert by_name[str(name)] == int(rid), name


def _grid_eval(fun, der):
    z = load_npz("ops.npz")
    f = np.array([fun(int(o), x, y) for o, x, y in zip(z["op"], z["x"], z["y"])])
    d = np.array([der(int(o), x, y, fr) for o, x, y, fr in zip(z["op"], z["x"], z["y"], z["f"])])
    return z, f, d


def test_oracle_ops_vs_golden():
    z, f, d = _grid_eval(O.fun, O.der)
    exact = np.isin(z["op"], list(EXACT_OPS))
    assert_bitexact(f[exact], z["f"][exact], "exact-op values")
    assert_bitexact(d[exact, 0], z["d0"][exact], "exact-op d0")
    assert_bitexact(d[exact, 1], z["d1"][exact], "exact-op d1")
    # transcendentals: the oracle calls the host libm; allow a few ulp between libm builds
    for op in sorted(set(z["op"].tolist()) - EXACT_OPS):
        m = z["op"] == op
        for got, ref, what in ((f[m], z["f"][m], "f"), (d[m, 0], z["d0"][m], "d0"),
                               (d[m, 1], z["d1"][m], "d1")):
            assert_close(got, ref, "%s %s" % (C.OP_NAMES[op], what), rtol=4e-16 * 8,
                         floor=1e-300)


def test_python_folding_vs_golden():
    z = load_npz("ops.npz")
    f = np.array([C.fun(int(o), x, y) for o, x, y in zip(z["op"], z["x"], z["y"])])
    exact = np.isin(z["op"], list(EXACT_OPS))
    assert_bitexact(f[exact], z["f"][exact], "folding exact ops")
    for op in sorted(set(z["op"].tolist()) - EXACT_OPS):
        m = z["op"] == op
        assert_close(f[m], z["f"][m], C.OP_NAMES[op], rtol=4e-16 * 8, floor=1e-300)


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag"])
def test_oracle_tapes_vs_golden(name):
    z = load_npz("tapes.npz")
    t = golden_tape(z, name)
    args = golden_list(z, name, "arg", len(t.nnz_in))
    n = args[0].shape[-1]
    res = O.eval(t, args, n)
    for j, r in enumerate(golden_list(z, name, "res", len(t.nnz_out))):
        assert_close(res[j], r, "%s res%d" % (name, j))
    # the harness's numeric sweeps add d0*x + d1*y unfused; the oracle fuses them (as the
    # GPU): derivatives agree within 1e-13 of the magnitude of their chain-rule terms
    fseeds = golden_list(z, name, "fseed", len(t.nnz_in))
    _, fsens = O.forward(t, args, fseeds, n)
    with O.magnitude():
        _, fmag = O.forward(t, args, fseeds, n)
    for j, r in enumerate(golden_list(z, name, "fsens", len(t.nnz_out))):
        assert_close(fsens[j], r, "%s fsens%d" % (name, j), bound=RTOL * fmag[j])
    aseeds = golden_list(z, name, "aseed", len(t.nnz_out))
    _, asens = O.reverse(t, args, aseeds, n)
    with O.magnitude():
        _, amag = O.reverse(t, args, aseeds, n)
    for j, r in enumerate(golden_list(z, name, "asens", len(t.nnz_in))):
        assert_close(asens[j], r, "%s asens%d" % (name, j), bound=RTOL * amag[j])
    _, jac = O.jacobian(t, args, n)
    with O.magnitude():
        _, jmag = O.jacobian(t, args, n)
    for j, r in enumerate(golden_list(z, name, "jac", len(t.nnz_out))):
        assert_close(jac[j], r, "%s jac%d" % (name, j), bound=RTOL * jmag[j])


def test_jacobian_equals_forward_with_unit_seeds():
    z = load_npz("tapes.npz")
    t = golden_tape(z, "rollout")
    args = golden_list(z, "rollout", "arg", 2)
    n = args[0].shape[-1]
    nz = sum(t.nnz_in)
    eye = np.eye(nz)
    fseeds = [np.repeat(eye[:, :4, None], n, axis=2), np.repeat(eye[:, 4:, None], n, axis=2)]
    _, fs = O.forward(t, args, fseeds, n)
    _, jac = O.jacobian(t, args, n)
    for a, b in zip(fs, jac):
        # unit seeds only add exact zeros: same numbers up to the sign of zero
        assert np.array_equal(a, b)


def test_oracle_threads_agree():
    z = load_npz("tapes.npz")
    t = golden_tape(z, "rollout")
    args = golden_list(z, "rollout", "arg", 2)
    a = O.eval(t, args, args[0].shape[-1], nthreads=1)
    b = O.eval(t, args, args[0].shape[-1], nthreads=4)
    for x, y in zip(a, b):
        assert same_bits(x, y).all()


def test_oracle_sparsity_matches_structure():
    """sp_forward with one bit per input gives exactly the dependency pattern, and
    sp_reverse with one bit per output gives its transpose (SXFunction::sp_forward/
    sp_reverse semantics)."""
    from casadi_gb300 import workloads as W
    f = W.random_dag(n_in=16, n_nodes=600, n_out=8, seed=5)
    t = f.tape
    n = 3
    bits = np.zeros((16, n), np.uint64)
    for k in range(16):
        bits[k, :] = np.uint64(1) << np.uint64(k)
    fwd = O.sp_forward(t, [bits], n)[0]
    seeds = np.zeros((8, n), np.uint64)
    for k in range(8):
        seeds[k, :] = np.uint64(1) << np.uint64(k)
    sens = np.zeros((16, n), np.uint64)
    O.sp_reverse(t, [sens], [seeds], n)
    assert (seeds == 0).all()  # seeds are consumed
    for o in range(8):
        for i in range(16):
            dep_f = bool(int(fwd[o, 0]) >> i & 1)
            dep_r = bool(int(sens[i, 0]) >> o & 1)
            assert dep_f == dep_r


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built on this host")
def test_oracle_matches_reference_harness_exactly():
    """On the host where the reference harness is built, the oracle's libm is the reference's
    libm: every op value and partial must agree bit for bit."""
    z, f, d = _grid_eval(O.fun, O.der)
    _, rf, rd = _grid_eval(O.ref_fun, O.ref_der)
    assert_bitexact(f, rf, "values")
    assert_bitexact(d, rd, "partials")


def test_rtol_is_the_documented_tolerance():
    assert RTOL == 1e-13 and math.isfinite(RTOL)


# ---- activity analysis (SXFunction::eval_activity) ------------------------------------------
ACTIVITY_CASES = ("ops", "cartpole", "rollout", "dag")


def _activity_tape(name):
    if name == "ops":
        return golden_tape(load_npz("activity.npz"), "ops")
    return golden_tape(load_npz("tapes.npz"), name)


def test_oracle_zero_checkers_vs_golden():
    """The oracle's F0X/FX0/F00 tables equal the reference's operation_checker templates."""
    z = load_npz("activity.npz")
    for w, name in enumerate(("zero_first", "zero_second", "zero_both")):
        for op, want in zip(z["checker/op"], z["checker/" + name]):
            assert O.zero_checker(w, int(op)) == bool(want), (name, C.OP_NAMES[int(op)])


@pytest.mark.parametrize("name", ACTIVITY_CASES)
def test_oracle_activity_vs_golden(name):
    z = load_npz("activity.npz")
    t = _activity_tape(name)
    args = golden_list(z, name, "act_arg", len(t.nnz_in))
    want = golden_list(z, name, "act_res", len(t.nnz_out))
    n = args[0].shape[1]
    got = O.activity(t, args, n, nthreads=2)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_activity_fixture_is_not_trivial():
    """The op tape's golden outputs hold inactive and active results, and the pass-through
    output keeps partial bit patterns (words other than 0 and all ones)."""
    z = load_npz("activity.npz")
    r0, r1 = z["ops/act_res0"], z["ops/act_res1"]
    assert (r0 == 0).mean() > 0.1 and (r0 != 0).mean() > 0.5
    full = np.uint64(0xFFFFFFFFFFFFFFFF)
    assert ((r1 != 0) & (r1 != full)).any()
    assert set(np.unique(r0).tolist()) <= {0, int(full)}


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built on this host")
def test_oracle_activity_matches_reference_harness():
    from casadi_gb300 import workloads as W
    t = W.random_dag(n_in=16, n_nodes=700, n_out=6, seed=9).tape
    rng = np.random.default_rng(3)
    n = 50
    args = [np.where(rng.random((16, n)) < 0.5, np.uint64(0), np.uint64(2**64 - 1))]
    got = O.activity(t, args, n)
    want = O.ref_activity(t, args, n)
    assert np.array_equal(got[0], want[0])


# ---- MapSum restatement ----------------------------------------------------------------------
def test_oracle_mapsum_matches_unrolled_instances():
    """The oracle's MapSum equals an explicit loop over instances: shared inputs repeated,
    summed outputs accumulated from zero in instance order (mapsum.cpp:153-181)."""
    from casadi_gb300 import workloads as W
    f = W.cartpole_rollout(3)
    n = 7
    x0, U = W.cartpole_inputs(n, steps=3, seed=2)
    shared_u = np.ascontiguousarray(U[:, 0])
    res = O.mapsum_eval(f.tape, [x0, shared_u], n, [False, True], [True, False])
    acc = np.zeros(4)
    xs = []
    for i in range(n):
        r = O.eval(f.tape, [x0[:, i:i + 1].copy(), shared_u[:, None].copy()], 1)
        acc = acc + r[0][:, 0]
        xs.append(r[1][:, 0])
    assert np.array_equal(res[0], acc)
    assert np.array_equal(res[1], np.array(xs).T)
    # sparsity: a shared input's reverse bits are the OR over the instances
    t = W.random_dag(n_in=8, n_nodes=200, n_out=3, seed=1).tape
    arg = [np.zeros(8, np.uint64)]
    seed = [np.array([1, 2, 4], np.uint64)]
    O.mapsum_sp_reverse(t, arg, seed, 5, [True], [True])
    one = [np.zeros((8, 1), np.uint64)]
    O.sp_reverse(t, one, [np.array([[1], [2], [4]], np.uint64)], 1)
    assert np.array_equal(arg[0], one[0][:, 0]) and not seed[0].any()


def test_libm_bound_on_hand_checked_tapes():
    """sum over libm results of |d out / d w_k| * |w_k|: 3 sin(x) - x gives 3|sin x|;
    exp(sin x) gives exp(sin x) (the exp) + exp(sin x)|sin x| (the sin through exp)."""
    x = S.sym("x", 1)
    f = S.Function("f", [x], [[S.sin(x[0]) * 3.0 - x[0], S.exp(S.sin(x[0]))]])
    xs = np.array([0.5, -1e-3, 2.0, 0.0])
    b = O.libm_bound(f.tape, [xs[None, :]], xs.size)[0]
    np.testing.assert_allclose(b[0], 3 * np.abs(np.sin(xs)), rtol=1e-15)
    e = np.exp(np.sin(xs))
    np.testing.assert_allclose(b[1], e + e * np.abs(np.sin(xs)), rtol=1e-15)
    # exact tapes have no libm term
    g = S.Function("g", [x], [[x[0] * x[0] / (x[0] + 3.0)]])
    assert (O.libm_bound(g.tape, [xs[None, :]], xs.size)[0] == 0).all()


def test_rounding_bound_counts_every_rounded_result():
    """x*x / (x+3): each of the three rounded results w_k contributes |d out/d w_k| |w_k| =
    |out|, so the bound is 3|out|; 3 sin(x) - x: 3|sin x| (the sin and the product, each) plus
    |3 sin x - x| (the difference)."""
    x = S.sym("x", 1)
    xs = np.array([0.5, -1e-3, 2.0, 0.0, -2.5])
    g = S.Function("g", [x], [[x[0] * x[0] / (x[0] + 3.0)]])
    b = O.rounding_bound(g.tape, [xs[None, :]], xs.size)[0][0]
    np.testing.assert_allclose(b, 3 * np.abs(xs * xs / (xs + 3.0)), rtol=1e-15)
    f = S.Function("f", [x], [[S.sin(x[0]) * 3.0 - x[0]]])
    b = O.rounding_bound(f.tape, [xs[None, :]], xs.size)[0][0]
    s = np.abs(np.sin(xs))
    np.testing.assert_allclose(b, 6 * s + np.abs(3 * np.sin(xs) - xs), rtol=1e-15)


def test_magnitude_mode_is_the_sweep_over_absolute_values():
    """In magnitude mode the adjoint of a * b - c * d at (2, -3, 5, 7) with seed -1 is
    (|b|, |a|, |d|, |c|) = (3, 2, 7, 5); outside it the signed adjoint returns."""
    v = S.sym("v", 4)
    f = S.Function("f", [v], [[v[0] * v[1] - v[2] * v[3]]])
    args = [np.array([[2.0], [-3.0], [5.0], [7.0]])]
    seed = [-np.ones((1, 1, 1))]
    with O.magnitude():
        _, m = O.reverse(f.tape, args, seed, 1)
    np.testing.assert_array_equal(m[0][0][:, 0], [3, 2, 7, 5])
    _, a = O.reverse(f.tape, args, seed, 1)
    np.testing.assert_array_equal(a[0][0][:, 0], [3, -2, 7, 5])


def test_adjoint_bound_helper_takes_rounding_and_rejects_a_planted_error():
    """assert_adjoint_close passes the oracle's own adjoint moved within 1e-13 of the
    magnitude, and on one element by a little over that but within the adjoint-Function bound;
    an error planted at 1e-9 relative on one element fails it."""
    from casadi_gb300 import workloads as W
    from helpers import adjoint_bounds, assert_adjoint_close
    F = W.cartpole_rollout(10)
    n = 48
    args = list(W.cartpole_inputs(n, steps=10, seed=2))
    seeds = [np.zeros((1, 4, n)), np.ones((1, 1, n))]
    _, was = O.reverse(F.tape, args, seeds, n)
    with O.magnitude():
        _, mag = O.reverse(F.tape, args, seeds, n)
    want = [w[0] for w in was]
    mags = [m[0] for m in mag]
    aseed = [s[0] for s in seeds]
    got = [w + 0.5 * RTOL * m for w, m in zip(want, mags)]
    assert_adjoint_close(got, want, mags, F, args, aseed, "rounding")
    ab = adjoint_bounds(F, args, aseed, n)
    got[1][3, 7] = want[1][3, 7] + RTOL * mags[1][3, 7] + 0.5 * ab[1][3, 7]
    assert_adjoint_close(got, want, mags, F, args, aseed, "within the adjoint bound")
    got[1][3, 7] = want[1][3, 7] * (1 + 1e-9) + 1e-9
    with pytest.raises(AssertionError):
        assert_adjoint_close(got, want, mags, F, args, aseed, "planted")
