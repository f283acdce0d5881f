"""GPU parity against CasADi itself: the CUDA sweeps, called through the C ABI, on the tapes
the reference's libcasadi built, against the outputs of its own Function calls
(tests/golden/casadi.npz; written by tests/golden/make_casadi_golden.py).

Bars (the fixtures were computed with the generating host's glibc; the GPU uses CUDA's libm):
  * sparsity sweeps and Jacobian patterns: identical;
  * values of tapes of IEEE-exact ops (+,-,*,/,sqrt and exact sign/compare/select ops, no FMA
    contraction): bit-exact;
  * values where libm transcendentals are involved: relative error <= 1e-13 per element, or,
    where an output cancels (or a long trajectory amplifies), within 4 ulp-sized relative
    perturbations of every libm result propagated to that output (oracle.libm_bound: the sum
    over libm instructions of |d out / d w_k| * |w_k|);
  * the numeric AD sweeps against CasADi's symbolic derivative Functions: |a - b| <= 1e-13 x
    the magnitude of the derivative's chain-rule terms per element (oracle.magnitude on the
    same inputs); the two round differently by construction (CasADi simplifies inv(y)*seed to
    seed/y, and so on), so no bit parity is possible there;
  * CasADi's derivative Function f.reverse(1) evaluated by the value sweep (what a mapped
    derivative runs): bit-exact on exact tapes, the value bars above elsewhere.
"""
import os

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W
from casadi_gb300.runtime import CudaTape

from helpers import (EXACT_OPS, GOLDEN, assert_bitexact, casadi_tape, golden_list, load_npz,
                     same_bits, tape_sha256)

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

AD_RTOL = 1e-13
VALUE_RTOL = 1e-13
LIBM_ULPS = 4
EXACT_MAP = np.array([0, 1, 3, 3, 8, 3, 8, 1, 8, 0], np.int32)


@pytest.fixture(scope="module")
def z():
    return load_npz("casadi.npz")


def dev(arrs):
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
            for a in arrs]


def host(ts):
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in ts]


def is_exact(t):
    return all(int(o) in EXACT_OPS or int(o) in (C.OP_CONST, C.OP_INPUT, C.OP_OUTPUT)
               for o in np.unique(t.op))


def assert_within_magnitude(got, ref, mag, what, rtol=AD_RTOL):
    got, ref, mag = (np.asarray(v, np.float64) for v in (got, ref, mag))
    d = np.abs(got - ref)
    bad = ~(same_bits(got, ref) | (d <= rtol * mag))
    if bad.any():
        i = tuple(np.argwhere(bad)[0])
        raise AssertionError("%s: %d of %d beyond %.0e x magnitude, e.g. %s: %r vs %r (mag %r)"
                             % (what, int(bad.sum()), bad.size, rtol, i, got[i], ref[i], mag[i]))


def assert_values(got, ref, exact, what, bound=None):
    """Bit-exact on exact tapes; else relative error <= 1e-13 or, given the libm bound of the
    output, a difference within LIBM_ULPS ulps of every libm result propagated to it."""
    if exact:
        assert_bitexact(got, ref, what)
        return
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    d = np.abs(got - ref)
    ok = same_bits(got, ref) | (d <= VALUE_RTOL * np.abs(ref))
    if bound is not None:
        ok |= d <= LIBM_ULPS * 2.0**-52 * np.asarray(bound)
    if not ok.all():
        i = tuple(np.argwhere(~ok)[0])
        raise AssertionError("%s: %d of %d beyond the bar, e.g. %s: %r vs %r%s" % (
            what, int((~ok).sum()), ok.size, i, got[i], ref[i],
            "" if bound is None else " (libm bound %r)" % np.asarray(bound)[i]))


def tape_of(z, name):
    if name + "/op" in z:
        return casadi_tape(z, name)
    t = W.cartpole_rollout(100).tape if name == "rollout100" else None
    assert tape_sha256(t) == str(z[name + "/tape_sha256"])
    return t


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag", "dag_exact", "rollout100"])
def test_eval_matches_casadi(gpu_lib, z, name):
    t = tape_of(z, name)
    ct = CudaTape(t)
    args = golden_list(z, name, "arg", len(t.nnz_in))
    res = host(ct.eval(dev(args)))
    bound = None if is_exact(t) else O.libm_bound(t, args, args[0].shape[1])
    for j, r in enumerate(golden_list(z, name, "res", len(t.nnz_out))):
        assert_values(res[j], r, is_exact(t), "%s res%d" % (name, j),
                      None if bound is None else bound[j])
    ct.sync()


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag_exact"])
def test_jacobian_matches_casadi_jacobian(gpu_lib, z, name):
    t = tape_of(z, name)
    ct = CudaTape(t)
    args = golden_list(z, name, "arg", len(t.nnz_in))
    n = args[0].shape[1]
    _, jac = ct.jacobian(dev(args))
    jac = host(jac)
    with O.magnitude():
        _, mag = O.jacobian(t, args, n)
    off = np.cumsum([0] + t.nnz_in)
    for o in range(len(t.nnz_out)):
        for i in range(len(t.nnz_in)):
            key = "%s/jac_%d_%d" % (name, o, i)
            nc = int(z[key + "_shape"][1])
            cols = np.repeat(np.arange(nc), np.diff(z[key + "_colind"]))
            rows = z[key + "_row"]
            assert_within_magnitude(jac[o][off[i] + cols, rows], z[key],
                                    mag[o][off[i] + cols, rows], key)
    ct.sync()


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag_exact"])
def test_reverse_and_forward_match_casadi(gpu_lib, z, name):
    t = tape_of(z, name)
    ct = CudaTape(t)
    nin, nout = len(t.nnz_in), len(t.nnz_out)
    args = golden_list(z, name, "arg", nin)
    n = args[0].shape[1]
    aseeds = golden_list(z, name, "aseed", nout)
    _, asens = ct.reverse(dev(args), dev(aseeds))
    asens = host(asens)
    with O.magnitude():
        _, amag = O.reverse(t, args, aseeds, n)
    for j, r in enumerate(golden_list(z, name, "asens", nin)):
        assert_within_magnitude(asens[j], r, amag[j], "%s asens%d" % (name, j))
    fseeds = golden_list(z, name, "fseed", nin)
    _, fsens = ct.forward(dev(args), dev(fseeds))
    fsens = host(fsens)
    with O.magnitude():
        _, fmag = O.forward(t, args, fseeds, n)
    for j, r in enumerate(golden_list(z, name, "fsens", nout)):
        assert_within_magnitude(fsens[j], r, fmag[j], "%s fsens%d" % (name, j))
    ct.sync()


def test_dag_adjoint_and_sparsity_match_casadi(gpu_lib, z):
    t = tape_of(z, "dag")
    ct = CudaTape(t)
    args = golden_list(z, "dag", "arg", 1)
    n = args[0].shape[1]
    seed = [np.ones((1, 16, n))]
    _, a = ct.reverse(dev(args), dev(seed))
    a = host(a)
    with O.magnitude():
        _, m = O.reverse(t, args, seed, n)
    assert_within_magnitude(a[0][0], z["dag/asens_sum0"], m[0][0], "DAG adjoint of the sum")
    # bvec_t sweeps: 64 directions per word, bit-exact
    seeds = golden_list(z, "dag", "spf_seed", 1)
    m = seeds[0].shape[1]
    i64 = [torch.from_numpy(s.view(np.int64)).cuda() for s in seeds]
    res = host(ct.sp_forward(i64))
    assert (res[0].view(np.uint64) == z["dag/spf_res0"]).all()
    out = [torch.from_numpy(np.array(s).view(np.int64)).cuda()
           for s in golden_list(z, "dag", "spr_seed", 1)]
    arg = [torch.zeros((64, m), dtype=torch.int64, device="cuda")]
    ct.sp_reverse(arg, out)
    assert (host(arg)[0].view(np.uint64) == z["dag/spr_res0"]).all()
    assert (host(out)[0] == 0).all()
    from casadi_gb300.sparse_ad import jacobian_pattern
    p = jacobian_pattern(ct, 0, 0)
    assert (p.colind == z["dag/jacsp_0_0_colind"]).all() and (p.row == z["dag/jacsp_0_0_row"]).all()
    ct.sync()


@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag_exact"])
def test_casadi_reverse_function_on_the_value_sweep(gpu_lib, z, name):
    """CasADi's f.reverse(1) (rebuilt by sx.reverse_function, the same tape) evaluated by
    the GPU value sweep: the reference's adjoint operation for operation."""
    f = {"cartpole": W.cartpole_step, "rollout": lambda: W.cartpole_rollout(20),
         "dag_exact": lambda: W.dag_from_nodes(64, 16, *z["dag_exact/nodes"])}[name]()
    assert tape_sha256(f.tape) == str(z[name + "/tape_sha256"])
    B = S.reverse_function(f)
    assert tape_sha256(B.tape) == str(z[name + "/rev1_tape_sha256"])
    nin, nout = len(f.tape.nnz_in), len(f.tape.nnz_out)
    args = golden_list(z, name, "arg", nin)
    seeds = [s[0] for s in golden_list(z, name, "aseed", nout)]
    ct = CudaTape(B.tape)
    bargs = args + [None] * nout + seeds
    res = host(ct.eval(dev(bargs)))
    bound = None if is_exact(f.tape) else O.libm_bound(B.tape, bargs, args[0].shape[1])
    for j, r in enumerate(golden_list(z, name, "asens", nin)):
        assert_values(res[j], r[0], is_exact(f.tape), "%s reverse(1) %d" % (name, j),
                      None if bound is None else bound[j])
    ct.sync()


def test_rollout100_gradient_through_autograd_matches_casadi(gpu_lib, z):
    from casadi_gb300.autograd import CheckpointedRollout
    x0, U = golden_list(z, "rollout100", "arg", 2)
    n = x0.shape[1]
    tx = torch.from_numpy(x0).cuda().requires_grad_(True)
    tu = torch.from_numpy(U).cuda().requires_grad_(True)
    xN, cost = CheckpointedRollout(steps=100, every=10)(tx, tu)
    cost.sum().backward()
    t = W.cartpole_rollout(100).tape
    with O.magnitude():
        _, m = O.reverse(t, [x0, U], [np.zeros((1, 4, n)), np.ones((1, 1, n))], n)
    for j, g in enumerate((tx.grad, tu.grad)):
        ref = z["rollout100/asens%d" % j][0]
        got = g.cpu().numpy()
        assert_within_magnitude(got, ref, m[j][0], "rollout100 gradient %d" % j)


def test_mpc_sparse_jacobian_and_hessian_match_casadi(gpu_lib, z):
    from casadi_gb300.sparse_ad import ColoredHessian, ColoredJacobian
    L = W.quad_ms_lagrangian(100)
    assert tape_sha256(L.tape) == str(z["quad_lagrangian/tape_sha256"])
    args = golden_list(z, "quad", "arg", 3)
    d = dev(args)
    g = S.Function("g", L.inputs, [L.outputs[0]])
    J = ColoredJacobian(g, out=0, wrt=0)
    assert J.n_colors == 14
    assert (J.pattern.colind == z["quad/jac_g_colind"]).all()
    assert (J.pattern.row == z["quad/jac_g_row"]).all()
    jv = J(d).cpu().numpy()[:, 0]
    with O.magnitude():
        _, jm = O.jacobian(g.tape, args, 1)
    rows, cols = J.pattern.row, J.pattern.col()
    assert_within_magnitude(jv, z["quad/jac_g"][:, 0], jm[0][cols, rows, 0], "MPC jac_g")
    H = ColoredHessian(L, out=1, wrt=0)
    assert tape_sha256(H.gradient_function.tape) == str(z["quad_gradient/tape_sha256"])
    assert H.n_colors == 10
    hv = H(d).cpu().numpy()[:, 0]  # lower triangle, CCS order of the lower part
    hp_shape = z["quad/hess_shape"]
    hcols = np.repeat(np.arange(hp_shape[1]), np.diff(z["quad/hess_colind"]))
    full = {(int(r), int(c)): v for r, c, v in zip(z["quad/hess_row"], hcols, z["quad/hess"][:, 0])}
    ref = np.array([full[(int(r), int(c))] for r, c in zip(H.rows, H.cols)])
    with O.magnitude():
        _, hm = O.jacobian(H.gradient_function.tape, args, 1)
    mag = hm[0][H.cols, H.rows, 0]
    assert_within_magnitude(hv, ref, mag, "MPC Hessian")


def test_casadi_call_records_on_the_gpu(gpu_lib, z):
    """The rollout as 20 never-inlined calls (CasADi's OP_CALL tape and ExtendedAlgEl
    records), inlined by the library, against CasADi's evaluation of it."""
    step = CudaTape(casadi_tape(z, "cartpole"))
    t = casadi_tape(z, "rollout_calls")
    calls = z["rollout_calls/calls"]
    ct = CudaTape(t, calls=[(step, c[:5].tolist(), c[5:].tolist()) for c in calls])
    args = golden_list(z, "rollout_calls", "arg", 2)
    res = host(ct.eval(dev(args)))
    bound = O.libm_bound(W.cartpole_rollout(20).tape, args, args[0].shape[1])
    assert_values(res[0], z["rollout_calls/res0"], False, "rollout calls", bound[0])
    ct.sync()


def test_casadi_serialized_text_on_the_gpu(gpu_lib, z):
    text = open(os.path.join(GOLDEN, "serialized_casadi_cartpole.txt")).read()
    ct = CudaTape.deserialize(text)
    args = golden_list(z, "cartpole", "arg", 2)
    res = host(ct.eval(dev(args)))
    ref = host(CudaTape(casadi_tape(z, "cartpole")).eval(dev(args)))
    assert_bitexact(res[0], ref[0], "deserialized vs in-memory")
    bound = O.libm_bound(casadi_tape(z, "cartpole"), args, args[0].shape[1])
    assert_values(res[0], z["cartpole/res0"], False, "deserialized cartpole", bound[0])
    ct.sync()


def test_map_sparsity_sweeps_with_host_buffers_match_casadi(gpu_lib, z):
    """Map::sp_forward / sp_reverse through the host-buffer entry points (instance-major bvec
    words, casadi_gb300_map_sp_forward/_reverse) against CasADi's own sweeps, bit for bit."""
    from casadi_gb300.runtime import CudaMap
    t = tape_of(z, "dag")
    seeds = golden_list(z, "dag", "spf_seed", 1)
    n = seeds[0].shape[1]
    M = CudaMap(CudaTape(t), n)
    res = M.sp_forward([np.ascontiguousarray(seeds[0].T)])
    assert (res[0].T == z["dag/spf_res0"]).all()
    out = [np.ascontiguousarray(np.array(s).T) for s in golden_list(z, "dag", "spr_seed", 1)]
    arg = [np.zeros((n, 64), np.uint64)]
    M.sp_reverse(arg, out)
    assert (arg[0].T == z["dag/spr_res0"]).all()
    assert (out[0] == 0).all()


def test_casadi_jacobian_function_on_the_value_sweep(gpu_lib, z):
    """CasADi's F.jacobian() tape of the rollout (the drop-in's F.jacobian().map(N, "cuda"))
    evaluated by the GPU value sweep against CasADi's Jacobian: element-wise within 1e-13
    relative or the libm-propagation bound of each entry."""
    j = load_npz("casadi_rollout20_jacobian.npz")
    t = casadi_tape(j, "jacobian")
    assert tape_sha256(t) == str(j["jacobian/tape_sha256"])
    args = golden_list(z, "rollout", "arg", 2)
    n = args[0].shape[1]
    ct = CudaTape(t)
    res = host(ct.eval(dev(list(args) + [None, None])))
    bound = O.libm_bound(t, list(args) + [None, None], n)
    for k, key in enumerate(("jac_0_0", "jac_0_1", "jac_1_0", "jac_1_1")):
        assert_values(res[k], z["rollout/" + key], False, key, bound[k])
    ct.sync()
