"""GPU parity of the tape sweeps, through the C ABI, against the golden fixtures (reference op
semantics) and the oracle on the same seeded inputs.

Bars: bit-exact for sparsity and for tapes of +,-,*,/,sqrt. Where libm transcendentals are
involved, element by element: a value within 1e-13 of itself or within 4 ulps of every libm
result propagated to it (helpers.value_bounds); a derivative within 1e-13 of itself or of the
magnitude of its chain-rule terms (helpers.magnitudes)."""
import os

import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W
from casadi_gb300.runtime import CudaMap, CudaTape, CasadiGpuError

from helpers import (EXACT_OPS, RTOL, assert_bitexact, assert_close, golden_list, golden_tape,
                     load_npz, magnitudes, value_bounds)

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
NTHREADS = os.cpu_count() or 1


def dev(arrs, dtype=None):
    out = []
    for a in arrs:
        if a is None:
            out.append(None)
        else:
            t = torch.from_numpy(np.ascontiguousarray(a))
            out.append(t.cuda() if dtype is None else t.to(dtype).cuda())
    return out


def host(ts):
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in ts]


def u64_to_i64(a):
    return np.ascontiguousarray(a, np.uint64).view(np.int64)


# ---- golden fixtures (reference op semantics) ------------------------------------------------
@pytest.mark.parametrize("name", ["cartpole", "rollout", "dag"])
def test_golden_eval_forward_reverse(gpu_lib, name):
    z = load_npz("tapes.npz")
    t = golden_tape(z, name)
    ct = CudaTape(t)
    args = golden_list(z, name, "arg", len(t.nnz_in))
    n = args[0].shape[-1]
    res = host(ct.eval(dev(args)))
    ct.sync()
    vb = value_bounds(t, args, n)
    for j, r in enumerate(golden_list(z, name, "res", len(t.nnz_out))):
        assert_close(res[j], r, "%s eval res%d" % (name, j), bound=vb[j])
    fseeds = golden_list(z, name, "fseed", len(t.nnz_in))
    res2, fsens = ct.forward(dev(args), dev(fseeds))
    res2, fsens = host(res2), host(fsens)
    _, fmag = magnitudes(O.forward, t, args, fseeds, n)
    for j, r in enumerate(golden_list(z, name, "fsens", len(t.nnz_out))):
        assert_close(fsens[j], r, "%s fsens%d" % (name, j), bound=RTOL * fmag[j])
    aseeds = golden_list(z, name, "aseed", len(t.nnz_out))
    res3, asens = ct.reverse(dev(args), dev(aseeds))
    res3, asens = host(res3), host(asens)
    _, amag = magnitudes(O.reverse, t, args, aseeds, n)
    for j, r in enumerate(golden_list(z, name, "asens", len(t.nnz_in))):
        assert_close(asens[j], r, "%s asens%d" % (name, j), bound=RTOL * amag[j])
    res4, jac = ct.jacobian(dev(args))
    res4, jac = host(res4), host(jac)
    _, jmag = magnitudes(O.jacobian, t, args, n)
    for j, r in enumerate(golden_list(z, name, "jac", len(t.nnz_out))):
        assert_close(jac[j], r, "%s jac%d" % (name, j), bound=RTOL * jmag[j])
    # the value outputs of all sweeps are the same numbers
    for a, b, c, d in zip(res, res2, res3, res4):
        assert_bitexact(a, b, "eval vs forward values")
        assert_bitexact(a, c, "eval vs reverse values")
        assert_bitexact(a, d, "eval vs jacobian values")
    ct.sync()


# ---- every op, value and both partials, over the golden grid ---------------------------------
def _single_op_tape(op):
    binary = op in C.BINARY_OPS
    ops = [C.OP_INPUT, C.OP_INPUT, op, C.OP_OUTPUT]
    i0 = [0, 1, 2, 0]
    i1 = [0, 1, 0, 2]
    i2 = [0, 0, 1 if binary else 0, 0]
    return S.Tape(ops, i0, i1, i2, [0.0] * 4, [1, 1], [1], 3)


def test_ops_grid_values_and_partials(gpu_lib):
    z = load_npz("ops.npz")
    for op in sorted(set(z["op"].tolist())):
        m = z["op"] == op
        x, y = z["x"][m][None, :], z["y"][m][None, :]
        ct = CudaTape(_single_op_tape(op))
        f = host(ct.eval(dev([x, y])))[0][0]
        name = C.OP_NAMES[op]
        # erfinv follows the reference's own algorithm (Newton polish through erf and exp);
        # near |x| -> 1 it amplifies a 1-ulp difference of erf by 1/(2/sqrt(pi) exp(-y^2)),
        # ~1e5 at |x| = 0.999999, so its tolerance there is scaled by that condition number
        # (its partial (sqrt(pi)/2)*exp(f^2) multiplies that by another 2*f^2 ~ 25)
        tol = {C.OP_ERFINV: 1e-9}.get(op, None)
        if op in EXACT_OPS:
            assert_bitexact(f, z["f"][m], name + " value")
        else:
            assert_close(f, z["f"][m], name + " value", floor=1e-300,
                         **({} if tol is None else {"rtol": tol}))
        # adjoint seed 1 on the output gives d0 on x and d1 on y: a first contribution is
        # assigned (the reference's 0 + x -> x), so it is d*1 bit for bit
        n = x.shape[1]
        _, asens = ct.reverse(dev([x, y]), dev([np.ones((1, 1, n))]))
        ax, ay = host(asens)
        d1 = z["d1"][m]
        if op == C.OP_IF_ELSE_ZERO:
            # the adjoint rule is if_else_zero(d1, seed), not d1*seed (sx_function.cpp:1470-1474)
            d1 = np.where(d1 == 0, 0.0, 1.0)
        for got, ref, what in ((ax[0, 0], z["d0"][m], "d0"), (ay[0, 0], d1, "d1")):
            if op in EXACT_OPS:
                assert_bitexact(got, ref, "%s %s" % (name, what))
            else:
                assert_close(got, ref, "%s %s" % (name, what), floor=1e-300,
                             **({} if tol is None else {"rtol": tol}))
        ct.sync()


def _twice_op_tape(op):
    """op(x, y) and op(y, x) (op(x) and op(y) when unary) as two outputs: each operand slot
    receives two adjoint contributions (assigned, then accumulated), and seeds on x and y
    activate one or both operands of each instruction."""
    binary = op in C.BINARY_OPS
    ops = [C.OP_INPUT, C.OP_INPUT, op, op, C.OP_OUTPUT, C.OP_OUTPUT]
    i0 = [0, 1, 2, 3, 0, 1]
    i1 = [0, 1, 0, 1, 2, 3]
    i2 = [0, 0, 1 if binary else 0, 0 if binary else 1, 0, 0]
    return S.Tape(ops, i0, i1, i2, [0.0] * 6, [1, 1], [1, 1], 4)


def test_ops_grid_tangents_and_accumulated_adjoints(gpu_lib):
    """Every op's tangent forms (one operand or both carrying a derivative) and adjoint
    contributions (first and later ones) against the oracle, over the golden grid."""
    z = load_npz("ops.npz")
    rng = np.random.default_rng(3)
    for op in sorted(set(z["op"].tolist())):
        m = z["op"] == op
        x, y = z["x"][m][None, :], z["y"][m][None, :]
        n = x.shape[1]
        t = _twice_op_tape(op)
        ct = CudaTape(t)
        name = C.OP_NAMES[op]
        tol = {C.OP_ERFINV: 1e-9}.get(op, None)

        def check(got, want, mag, what):
            # exact ops: bit for bit; libm ops: within 1e-13 (erfinv: 1e-9, see above) of the
            # magnitude of the chain-rule terms, since the partials of the two libms differ by
            # an ulp and two contributions can cancel
            if op in EXACT_OPS:
                assert_bitexact(got, want, "%s %s" % (name, what))
            else:
                assert_close(got, want, "%s %s" % (name, what),
                             bound=(RTOL if tol is None else tol) * np.asarray(mag))

        # directions: x only, y only, both (general seeds)
        fseeds = [np.array([1.0, 0.0, 0.7])[:, None, None] * np.ones((3, 1, n)),
                  np.array([0.0, 1.0, -1.3])[:, None, None] * np.ones((3, 1, n))]
        _, fs = ct.forward(dev([x, y]), dev(fseeds))
        _, wfs = O.forward(t, [x, y], fseeds, n, NTHREADS)
        _, mfs = magnitudes(O.forward, t, [x, y], fseeds, n, NTHREADS)
        for k, (g, w, mg) in enumerate(zip(host(fs), wfs, mfs)):
            check(g, w, mg, "tangent of output %d" % k)
        aseeds = [rng.standard_normal((2, 1, n)), rng.standard_normal((2, 1, n))]
        _, asn = ct.reverse(dev([x, y]), dev(aseeds))
        _, was = O.reverse(t, [x, y], aseeds, n, NTHREADS)
        _, mas = magnitudes(O.reverse, t, [x, y], aseeds, n, NTHREADS)
        for k, (g, w, mg) in enumerate(zip(host(asn), was, mas)):
            check(g, w, mg, "adjoint of input %d" % k)
        ct.sync()


# ---- bit-exact on +,-,*,/,sqrt tapes -----------------------------------------------------------
def _arith_dag(n_in=24, n_nodes=3000, n_out=8, seed=11):
    rng = np.random.default_rng(seed)
    xs = S.sym("x", n_in)
    nodes = list(xs)
    for k in range(n_in, n_nodes):
        a = nodes[int(rng.integers(max(0, k - 128), k))]
        b = nodes[int(rng.integers(max(0, k - 128), k))]
        r = rng.random()
        if r < 0.3:
            e = a + b
        elif r < 0.5:
            e = a - b
        elif r < 0.8:
            e = a * b * 0.5
        elif r < 0.9:
            e = a / (b * b + 1.0)
        else:
            e = S.sqrt(a * a + 1.0)
        nodes.append(e)
    return S.Function("A", [xs], [nodes[-n_out:]])


def test_arithmetic_tape_bitexact(gpu_lib):
    f = _arith_dag()
    t = f.tape
    assert set(C.OP_NAMES[o] for o in np.unique(t.op)) <= {
        "ADD", "SUB", "MUL", "DIV", "SQRT", "SQ", "TWICE", "CONST", "INPUT", "OUTPUT", "NEG"}
    n = 3001
    rng = np.random.default_rng(0)
    args = [rng.uniform(-1, 1, (24, n))]
    ct = CudaTape(t)
    got = host(ct.eval(dev(args)))
    want = O.eval(t, args, n, NTHREADS)
    assert_bitexact(got[0], want[0], "eval")
    fseeds = [rng.standard_normal((3, 24, n))]
    _, fs = ct.forward(dev(args), dev(fseeds))
    _, wfs = O.forward(t, args, fseeds, n, NTHREADS)
    assert_bitexact(host(fs)[0], wfs[0], "forward")
    aseeds = [rng.standard_normal((2, 8, n))]
    _, asn = ct.reverse(dev(args), dev(aseeds))
    _, was = O.reverse(t, args, aseeds, n, NTHREADS)
    assert_bitexact(host(asn)[0], was[0], "reverse")
    ct.sync()


# ---- the benchmark workloads against the oracle --------------------------------------------
def test_cartpole_full_size(gpu_lib):
    f = W.cartpole_step()
    n = 65536
    args = W.cartpole_inputs(n, steps=1, seed=0)
    ct = CudaTape(f)
    got = host(ct.eval(dev(args)))
    want = O.eval(f.tape, args, n, NTHREADS)
    assert_close(got[0], want[0], "cartpole eval N=65536", bound=value_bounds(f.tape, args, n)[0])
    ct.sync()


def test_rollout_jacobian_and_adjoint(gpu_lib):
    F = W.cartpole_rollout(20)
    n = 8192
    args = W.cartpole_inputs(n, steps=20, seed=3)
    ct = CudaTape(F)
    # forward Jacobian of xN: 24 unit seed directions over (x0, U), generated on the device
    res, fsens = ct.jacobian(dev(args))
    res, fsens = host(res), host(fsens)
    wres, wfsens = O.jacobian(F.tape, args, n, NTHREADS)
    vb = value_bounds(F.tape, args, n)
    _, jmag = magnitudes(O.jacobian, F.tape, args, n, NTHREADS)
    assert_close(res[0], wres[0], "xN", bound=vb[0])
    assert_close(fsens[0], wfsens[0], "d xN / d (x0,U)", bound=RTOL * jmag[0])
    # the same Jacobian from explicit unit seeds through the general forward sweep
    eye = np.eye(24)
    m = 512
    fseeds = [np.repeat(eye[:, :4, None], m, axis=2), np.repeat(eye[:, 4:, None], m, axis=2)]
    sub = [a[:, :m].copy() for a in args]
    _, fs2 = ct.forward(dev(sub), dev(fseeds))
    fs2 = host(fs2)
    for a, b in zip(fs2, fsens):
        assert np.array_equal(a, b[:, :, :m])
    # adjoint of cost
    aseeds = [np.zeros((1, 4, n)), np.ones((1, 1, n))]
    _, asens = ct.reverse(dev(args), dev(aseeds))
    asens = host(asens)
    _, wasens = O.reverse(F.tape, args, aseeds, n, NTHREADS)
    _, amag = magnitudes(O.reverse, F.tape, args, aseeds, n, NTHREADS)
    # CUDA's and the host libm's sin/cos differ by an ulp here and there; twenty RK4 steps
    # carry that into the adjoint, within 1e-13 of the magnitude of its chain-rule terms
    assert_close(asens[0], wasens[0], "d cost / d x0", bound=RTOL * amag[0])
    assert_close(asens[1], wasens[1], "d cost / d U", bound=RTOL * amag[1])
    # the adjoint agrees with the forward Jacobian of the cost output row
    jac_cost = fsens[1][:, 0, :]  # (24, n)
    adj = np.concatenate([asens[0][0], asens[1][0]], axis=0)  # (24, n)
    assert_close(adj, jac_cost, "adjoint vs forward", bound=RTOL * jmag[1][:, 0, :])
    # and central finite differences (h = 1e-6) on a few instances
    h = 1e-6
    m = 16
    sub = [a[:, :m].copy() for a in args]
    fd = np.zeros((24, m))
    for k in range(24):
        p = [a.copy() for a in sub]
        q = [a.copy() for a in sub]
        blk, row = (0, k) if k < 4 else (1, k - 4)
        p[blk][row] += h
        q[blk][row] -= h
        fd[k] = (O.eval(F.tape, p, m)[1][0] - O.eval(F.tape, q, m)[1][0]) / (2 * h)
    assert np.max(np.abs(fd - adj[:, :m]) / np.maximum(np.abs(adj[:, :m]), 1.0)) < 1e-5
    ct.sync()


def test_dag_full_size_eval_and_adjoint(gpu_lib):
    G = W.random_dag()
    n = 2048
    args = W.dag_inputs(n)
    ct = CudaTape(G)
    got = host(ct.eval(dev(args)))
    want = O.eval(G.tape, args, n, NTHREADS)
    assert_close(got[0], want[0], "dag eval", bound=value_bounds(G.tape, args, n)[0])
    aseeds = [np.ones((1, 16, n))]
    _, asens = ct.reverse(dev(args), dev(aseeds))
    _, wasens = O.reverse(G.tape, args, aseeds, n, NTHREADS)
    _, amag = magnitudes(O.reverse, G.tape, args, aseeds, n, NTHREADS)
    assert_close(host(asens)[0], wasens[0], "dag adjoint of sum of outputs",
                 bound=RTOL * amag[0])
    ct.sync()


# ---- sparsity (bit-exact) -----------------------------------------------------------------------
def test_sparsity_sweeps_bitexact(gpu_lib):
    G = W.random_dag()
    t = G.tape
    n = 777
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 2**63, size=(64, n), dtype=np.int64).view(np.uint64)
    bits &= rng.integers(0, 2**63, size=(64, n), dtype=np.int64).view(np.uint64)
    ct = CudaTape(t)
    got = host(ct.sp_forward(dev([u64_to_i64(bits)])))[0].view(np.uint64)
    want = O.sp_forward(t, [bits], n)[0]
    assert np.array_equal(got, want)
    arg0 = rng.integers(0, 2**63, size=(64, n), dtype=np.int64).view(np.uint64) & np.uint64(0xff)
    seeds = rng.integers(0, 2**63, size=(16, n), dtype=np.int64).view(np.uint64)
    a_dev, r_dev = dev([u64_to_i64(arg0)]), dev([u64_to_i64(seeds)])
    ct.sp_reverse(a_dev, r_dev)
    ga, gr = host(a_dev)[0].view(np.uint64), host(r_dev)[0].view(np.uint64)
    wa, wr = [arg0.copy()], [seeds.copy()]
    O.sp_reverse(t, wa, wr, n)
    assert np.array_equal(ga, wa[0]) and np.array_equal(gr, wr[0])
    assert (gr == 0).all()
    ct.sync()


# ---- edge cases ----------------------------------------------------------------------------------
def test_edge_sizes_null_io_and_waves(gpu_lib):
    F = W.cartpole_rollout(4)
    t = F.tape
    ct = CudaTape(F)
    for n in (1, 2, 31, 33, 1000):
        args = W.cartpole_inputs(n, steps=4, seed=n)
        got = host(ct.eval(dev(args)))
        want = O.eval(t, args, n)
        for g, w, b in zip(got, want, value_bounds(t, args, n)):
            assert_close(g, w, "n=%d" % n, bound=b)
    # n = 0 is a no-op
    e = torch.empty((4, 0), dtype=torch.float64, device="cuda")
    ct.eval([e, torch.empty((4, 0), dtype=torch.float64, device="cuda")], n=0)
    # null input reads zeros, null output is skipped
    n = 50
    args = W.cartpole_inputs(n, steps=4, seed=1)
    res = ct.eval(dev([args[0], None]), n=n, res=[torch.zeros((4, n), dtype=torch.float64,
                                                             device="cuda"), None])
    want = O.eval(t, [args[0], None], n)
    assert_close(host([res[0]])[0], want[0], "null input",
                 bound=value_bounds(t, [args[0], None], n)[0])
    # adjoint in several waves (scratch limited to ~3 warps of instances) == one wave
    n = 1000
    args = W.cartpole_inputs(n, steps=4, seed=2)
    aseeds = [np.random.default_rng(0).standard_normal((3, 4, n)), np.ones((3, 1, n))]
    _, one = ct.reverse(dev(args), dev(aseeds))
    one = host(one)
    ct2 = CudaTape(F)
    _, many = ct2.reverse(dev(args), dev(aseeds), scratch_limit=8 * ct2.n_partials * 96)
    many = host(many)
    for a, b in zip(one, many):
        assert_bitexact(a, b, "waves")
    # forward with a direction count that is not a multiple of the CTA direction width
    fseeds = [np.random.default_rng(1).standard_normal((5, 4, n)),
              np.random.default_rng(2).standard_normal((5, 4, n))]
    _, fs = ct.forward(dev(args), dev(fseeds))
    _, wfs = O.forward(t, args, fseeds, n)
    _, fmag = magnitudes(O.forward, t, args, fseeds, n)
    for g, w, m in zip(host(fs), wfs, fmag):
        assert_close(g, w, "nfwd=5", bound=RTOL * m)
    ct.sync()
    ct2.sync()


def test_tangent_work_queue_gives_the_static_split_bits(gpu_lib):
    """The tangent sweep claims its items from a counter kept past the partials in the
    scratch; a scratch without those bytes runs the static split. Both, and a queued sweep in
    several waves, give the same bits (15000 (tile, direction) items: more than the grid)."""
    F = W.cartpole_rollout(20)
    n = 20000
    args = dev(W.cartpole_inputs(n, steps=20, seed=5))
    ct = CudaTape(F)
    _, queued = ct.jacobian(args)
    exact = 8 * ct.n_partials * ((n + 31) // 32 * 32)
    ct_static = CudaTape(F)
    _, static = ct_static.jacobian(args, scratch_limit=exact)
    ct_waves = CudaTape(F)
    _, waves = ct_waves.jacobian(args, scratch_limit=8 * ct.n_partials * 6720 + 256)
    for q, s, w in zip(host(queued), host(static), host(waves)):
        assert_bitexact(q, s, "queued vs static split")
        assert_bitexact(q, w, "queued in waves")
    for c in (ct, ct_static, ct_waves):
        c.sync()


def test_scratch_too_small_is_an_error(gpu_lib):
    F = W.cartpole_rollout(2)
    ct = CudaTape(F)
    args = dev(W.cartpole_inputs(64, steps=2))
    sc = torch.empty(16, dtype=torch.uint8, device="cuda")
    import ctypes as ct_
    from casadi_gb300 import runtime as R
    aseeds = dev([np.ones((1, 4, 64)), np.ones((1, 1, 64))])
    asens = [torch.empty((1, k, 64), dtype=torch.float64, device="cuda") for k in (4, 2)]
    st = R.load().casadi_gb300_reverse(ct.id, 64, 64, 1, R._ptr_array(args), R._ptr_array(
        [torch.empty((k, 64), dtype=torch.float64, device="cuda") for k in (4, 1)]),
        R._ptr_array(aseeds), R._ptr_array(asens), ct_.c_void_p(sc.data_ptr()), 16, None)
    assert st == -5
    assert "scratch" in R.load().casadi_gb300_last_error().decode()


# ---- host-buffer Map path --------------------------------------------------------------------------
def test_map_eval_and_reverse_host_buffers(gpu_lib):
    f = W.cartpole_step()
    n = 4099
    x, u = W.cartpole_inputs(n, steps=1, seed=9)
    F = CudaMap(f, n)
    out = F(x.T.copy(), u.T.copy())[0]          # instance-major (n, 4)
    want = O.eval(f.tape, [x, u], n)[0]          # instance-minor (4, n)
    assert_close(out.T, want, "map eval", bound=value_bounds(f.tape, [x, u], n)[0])
    aseed = np.random.default_rng(3).standard_normal((n, 2, 4))
    res, asens = F.reverse([x.T.copy(), u.T.copy()], [aseed])
    oseed = [np.transpose(aseed, (1, 2, 0))]
    _, wasens = O.reverse(f.tape, [x, u], oseed, n)
    _, amag = magnitudes(O.reverse, f.tape, [x, u], oseed, n)
    assert_close(np.transpose(asens[0], (1, 2, 0)), wasens[0], "map reverse x",
                 bound=RTOL * amag[0])
    assert_close(np.transpose(asens[1], (1, 2, 0)), wasens[1], "map reverse u",
                 bound=RTOL * amag[1])
    # forward mode: seeds (n, nfwd, nnz) instance-major, the Map's forward(nfwd) layout
    rng = np.random.default_rng(4)
    fx, fu = rng.standard_normal((n, 3, 4)), rng.standard_normal((n, 3, 1))
    _, fsens = F.forward([x.T.copy(), u.T.copy()], [fx, fu])
    oseed = [np.transpose(fx, (1, 2, 0)), np.transpose(fu, (1, 2, 0))]
    _, wfs = O.forward(f.tape, [x, u], oseed, n)
    _, fmag = magnitudes(O.forward, f.tape, [x, u], oseed, n)
    assert_close(np.transpose(fsens[0], (1, 2, 0)), wfs[0], "map forward", bound=RTOL * fmag[0])


def test_host_buffer_calls_in_pipelined_chunks(gpu_lib):
    """Host-buffer calls large enough to run in pipelined chunks (copies of one chunk
    overlapping the sweeps of another) give the device entry points' bits."""
    f = W.cartpole_rollout(3)
    n = 2 * 131072 + 77
    x, u = W.cartpole_inputs(n, steps=3, seed=12)
    F = CudaMap(f, n)
    res, jac = F.jacobian(x.T.copy(), u.T.copy())
    ct = CudaTape(f)
    dres, djac = ct.jacobian(dev([x, u]))
    assert_bitexact(res[0].T, host(dres)[0], "values")
    assert_bitexact(np.transpose(jac[0], (1, 2, 0)), host(djac)[0], "jacobian")


@pytest.mark.parametrize("n", [1000, 2 * 131072 + 77])
def test_map_derivatives_in_the_maps_own_order(gpu_lib, n):
    """Seeds and sensitivities in the order of Map::get_forward/get_reverse (direction-major,
    (d*n + i)*nnz; casadi/core/map.cpp:233-264) give the bits of the inner order
    ((i*ndir + d)*nnz), at a size run in one chunk and at one run in pipelined chunks."""
    f = W.cartpole_rollout(2)
    x, u = W.cartpole_inputs(n, steps=2, seed=31)
    args = [x.T.copy(), u.T.copy()]
    F = CudaMap(f, n)
    rng = np.random.default_rng(31)
    fo = [rng.standard_normal((3, n, 4)), rng.standard_normal((3, n, 2))]
    r_o, s_o = F.forward(args, fo, outer=True)
    r_i, s_i = F.forward(args, [np.ascontiguousarray(np.transpose(a, (1, 0, 2))) for a in fo])
    for a, b in zip(r_o, r_i):
        assert_bitexact(a, b, "forward values")
    for a, b in zip(s_o, s_i):
        assert_bitexact(a, np.transpose(b, (1, 0, 2)), "forward, Map order")
    ao = [rng.standard_normal((2, n, 4)), rng.standard_normal((2, n, 1))]
    r_o, a_o = F.reverse(args, ao, outer=True)
    r_i, a_i = F.reverse(args, [np.ascontiguousarray(np.transpose(a, (1, 0, 2))) for a in ao])
    for a, b in zip(a_o, a_i):
        assert_bitexact(a, np.transpose(b, (1, 0, 2)), "reverse, Map order")


# ---- derivative-sweep variants and the autotuner ------------------------------------------------
def test_every_variant_gives_the_same_bits(gpu_lib):
    """The variants differ in prefetch depth and register cap only: forward, Jacobian and
    adjoint results must be identical bit for bit across all of them."""
    from casadi_gb300 import runtime as R
    F = W.cartpole_rollout(6)
    n = 2500
    args = dev(W.cartpole_inputs(n, steps=6, seed=21))
    rng = np.random.default_rng(21)
    fseeds = dev([rng.standard_normal((5, k, n)) for k in F.tape.nnz_in])  # 5: ragged groups
    aseeds = dev([rng.standard_normal((2, k, n)) for k in F.tape.nnz_out])
    ct = CudaTape(F)
    base = None
    for v in range(max(R.N_TAN_VARIANTS, R.N_ADJ_VARIANTS)):
        ct.set_variant(0, min(v, R.N_TAN_VARIANTS - 1))
        ct.set_variant(1, min(v, R.N_TAN_VARIANTS - 1))
        ct.set_variant(2, min(v, R.N_ADJ_VARIANTS - 1))
        got = [host(ct.forward(args, fseeds)[1]), host(ct.jacobian(args)[1]),
               host(ct.reverse(args, aseeds)[1])]
        if base is None:
            base = got
            continue
        for g, b in zip(got, base):
            for x, y in zip(g, b):
                assert_bitexact(x, y, "variant %d" % v)
    ct.sync()


def test_linear_tape_with_a_constant_output_every_variant(gpu_lib):
    """A tape with no recorded partials (ADD, SUB, NEG, TWICE), a constant output (no tangent
    entries; its adjoint seed lands on a constant's slot) and an unused input: forward,
    Jacobian and adjoint of every variant against the oracle, bit for bit."""
    from casadi_gb300 import runtime as R
    x, u = S.sym("x", 3), S.sym("u", 2)
    f = S.Function("L", [x, u], [[x[0] + x[1], x[0] - (x[2] + x[2]), -x[1]],
                                 [S.const(3.0), x[1] - x[0] - x[0]]])
    t = f.tape
    assert C.OP_CONST in t.op.tolist() and C.OP_TWICE in t.op.tolist()
    n = 777
    rng = np.random.default_rng(5)
    args = [rng.standard_normal((3, n)), rng.standard_normal((2, n))]
    fseeds = [rng.standard_normal((3, 3, n)), rng.standard_normal((3, 2, n))]
    aseeds = [rng.standard_normal((2, 3, n)), rng.standard_normal((2, 2, n))]
    _, wfs = O.forward(t, args, fseeds, n, NTHREADS)
    _, was = O.reverse(t, args, aseeds, n, NTHREADS)
    _, wj = O.jacobian(t, args, n, NTHREADS)
    ct = CudaTape(t)
    assert ct.n_partials == 0
    for v in range(max(R.N_TAN_VARIANTS, R.N_ADJ_VARIANTS)):
        ct.set_variant(0, min(v, R.N_TAN_VARIANTS - 1))
        ct.set_variant(1, min(v, R.N_TAN_VARIANTS - 1))
        ct.set_variant(2, min(v, R.N_ADJ_VARIANTS - 1))
        for g, w in zip(host(ct.forward(dev(args), dev(fseeds))[1]), wfs):
            assert_bitexact(g, w, "forward, variant %d" % v)
        for g, w in zip(host(ct.jacobian(dev(args))[1]), wj):
            assert_bitexact(g, w, "jacobian, variant %d" % v)
        for g, w in zip(host(ct.reverse(dev(args), dev(aseeds))[1]), was):
            assert_bitexact(g, w, "reverse, variant %d" % v)
    ct.sync()


def _every_op_dag(n_in=6, n_nodes=400, window=20, seed=17):
    """A random tape over every differentiable op kind (and a few with zero derivatives),
    operands drawn from the previous ``window`` nodes, inputs kept in well-defined ranges."""
    rng = np.random.default_rng(seed)
    xs = S.sym("x", n_in)
    nodes = list(xs)
    pos = lambda e: S.sq(e) + 1.0  # noqa: E731 (a positive operand)
    unary = [S.sin, S.cos, S.atan, S.tanh, S.erf, S.sq, S.twice, lambda e: -e, S.fabs,
             lambda e: S.sqrt(pos(e)), lambda e: S.log1p(S.sq(e)), lambda e: S.expm1(S.tanh(e)),
             lambda e: S.exp(S.tanh(e)), S.floor, S.sign, lambda e: S.asinh(e)]
    binary = [lambda a, b: a + b, lambda a, b: a - b, lambda a, b: a * b,
              lambda a, b: a / pos(b), S.fmin, S.fmax, S.atan2, S.hypot,
              lambda a, b: S.fmod(a, pos(b)), lambda a, b: S.remainder(a, pos(b)),
              S.copysign, lambda a, b: S.if_else_zero(S.lt(a, b), a * b)]
    for k in range(n_in, n_nodes):
        a = nodes[int(rng.integers(max(0, k - window), k))]
        b = nodes[int(rng.integers(max(0, k - window), k))]
        if rng.random() < 0.4:
            e = unary[int(rng.integers(len(unary)))](a)
        else:
            e = binary[int(rng.integers(len(binary)))](a, b)
        nodes.append(e)
    return S.Function("E", [xs], [nodes[-6:], [S.const(2.5)]])


def test_every_op_tape_every_variant(gpu_lib):
    """Union-stream (K > 1) and single-direction variants on a tape of every op kind: the
    Jacobian (unit seeds, so K-direction groups hold mixed entries) and two adjoint directions
    agree bit for bit across all variants and with the oracle within 1e-13 of the chain-rule
    magnitude."""
    from casadi_gb300 import runtime as R
    f = _every_op_dag()
    t = f.tape
    n = 1000
    rng = np.random.default_rng(8)
    args = [rng.standard_normal((6, n))]
    aseeds = [rng.standard_normal((2, 6, n)), rng.standard_normal((2, 1, n))]
    _, wj = O.jacobian(t, args, n, NTHREADS)
    _, mj = magnitudes(O.jacobian, t, args, n, NTHREADS)
    _, wa = O.reverse(t, args, aseeds, n, NTHREADS)
    _, ma = magnitudes(O.reverse, t, args, aseeds, n, NTHREADS)
    ct = CudaTape(t)
    base = None
    for v in range(max(R.N_TAN_VARIANTS, R.N_ADJ_VARIANTS) - 1):
        ct.set_variant(1, min(v, R.N_TAN_VARIANTS - 2))
        ct.set_variant(2, min(v, R.N_ADJ_VARIANTS - 2))
        got = [host(ct.jacobian(dev(args))[1]), host(ct.reverse(dev(args), dev(aseeds))[1])]
        if base is None:
            base = got
            for g, w, m in zip(got[0], wj, mj):
                assert_close(g, w, "jacobian", bound=RTOL * m)
            for g, w, m in zip(got[1], wa, ma):
                assert_close(g, w, "adjoint", bound=RTOL * m)
            continue
        for gs, bs in zip(got, base):
            for g, b in zip(gs, bs):
                assert_bitexact(g, b, "variant %d" % v)
    ct.sync()


def test_sin_cos_pairs_share_one_sincos(gpu_lib):
    """The record sweeps compute a SIN/COS pair of one operand value once (the second takes the
    first's sincos): adjacent pairs, pairs broken by another SIN/COS in between, repeats and
    large arguments give the value sweep's bits, and derivatives agree with the oracle."""
    import bench
    x, y = S.sym("x"), S.sym("y")
    u = x * y
    outs = [S.sin(x), S.cos(x), S.sin(y), S.cos(x) + S.sin(x), S.sin(u), S.cos(y), S.cos(u),
            S.sin(u) * S.cos(u), S.sin(x + 1.0), S.cos(y * 2.0), S.sin(y * 2.0)]
    f = S.Function("P", [[x, y]], [outs])
    t = f.tape
    assert sum(bench.sincos_reuse(t).values()) > 0
    n = 997
    rng = np.random.default_rng(12)
    args = [np.vstack([rng.uniform(-4, 4, n), 10.0 ** rng.uniform(-3, 6, n)])]
    aseeds = [rng.standard_normal((2, len(outs), n))]
    ct = CudaTape(t)
    vals = host(ct.eval(dev(args)))
    res_r, asens = ct.reverse(dev(args), dev(aseeds))
    res_j, jac = ct.jacobian(dev(args))
    for a, b, c in zip(vals, host(res_r), host(res_j)):
        assert_bitexact(a, b, "eval vs record values")
        assert_bitexact(a, c, "eval vs jacobian record values")
    _, wa = O.reverse(t, args, aseeds, n, NTHREADS)
    _, ma = magnitudes(O.reverse, t, args, aseeds, n, NTHREADS)
    for g, w, m in zip(host(asens), wa, ma):
        assert_close(g, w, "adjoint", bound=RTOL * m)
    _, wj = O.jacobian(t, args, n, NTHREADS)
    _, mj = magnitudes(O.jacobian, t, args, n, NTHREADS)
    for g, w, m in zip(host(jac), wj, mj):
        assert_close(g, w, "jacobian", bound=RTOL * m)
    ct.sync()


def test_autotuner_keeps_a_variant_and_results(gpu_lib):
    from casadi_gb300 import runtime as R
    F = W.cartpole_rollout(4)
    n = 400000  # a wave that fills the GPU several times over
    args = dev(W.cartpole_inputs(n, steps=4, seed=22))
    aseeds = dev([np.ones((1, 4, n)), np.ones((1, 1, n))])
    ct = CudaTape(F)
    ct.set_variant(2, 0)
    _, want = ct.reverse(args, aseeds)
    ct.set_variant(2, -1)
    R.autotune(True)
    _, got = ct.reverse(args, aseeds)
    assert 0 <= ct.tuned_variant(2) < R.N_ADJ_VARIANTS
    for x, y in zip(host(got), host(want)):
        assert_bitexact(x, y, "autotuned adjoint")
    ct.sync()


@pytest.mark.parametrize("n", [3001, 2 * 131072 + 77])
def test_jacobian_reverse_equals_the_two_calls(gpu_lib, n):
    """One record sweep feeding both derivative sweeps gives the same bits as calling
    jacobian and reverse one after the other, on device buffers and on host buffers (where
    the Jacobian's download overlaps the adjoint sweep)."""
    F = W.cartpole_rollout(5)
    args_h = W.cartpole_inputs(n, steps=5, seed=31)
    rng = np.random.default_rng(31)
    aseeds_h = [rng.standard_normal((2, k, n)) for k in F.tape.nnz_out]
    ct = CudaTape(F)
    args, aseeds = dev(args_h), dev(aseeds_h)
    r1, jac1 = ct.jacobian(args)
    _, as1 = ct.reverse(args, aseeds)
    r2, jac2, as2 = ct.jacobian_reverse(args, aseeds)
    for a, b in zip(host(r1) + host(jac1) + host(as1), host(r2) + host(jac2) + host(as2)):
        assert_bitexact(a, b, "fused jacobian+reverse")
    m = CudaMap(F, n)
    hargs = [a.T.copy() for a in args_h]
    hseeds = [np.transpose(s, (2, 0, 1)).copy() for s in aseeds_h]
    _, hj1 = m.jacobian(*hargs)
    _, ha1 = m.reverse(hargs, hseeds)
    _, hj2, ha2 = m.jacobian_reverse(hargs, hseeds)
    for a, b in zip(hj1 + ha1, hj2 + ha2):
        assert_bitexact(a, b, "host-buffer fused jacobian+reverse")
    # host layout agrees with the device layout
    assert_bitexact(np.transpose(hj2[0], (1, 2, 0)), host(jac2)[0], "layouts")
    ct.sync()


def test_jacobian_of_some_outputs_prunes_and_keeps_their_bits(gpu_lib):
    """A Jacobian requested for xN only (the cost's sensitivities null): the tangent plan
    drops the instructions only the cost needs, and xN's rows are the full Jacobian's bit for
    bit, with the device entry points and with host buffers; the cost adjoint is unchanged."""
    F = W.cartpole_rollout(20)
    n = 4099
    args_h = W.cartpole_inputs(n, steps=20, seed=41)
    aseeds_h = [np.zeros((1, 4, n)), np.ones((1, 1, n))]
    ct = CudaTape(F)
    args, aseeds = dev(args_h), dev(aseeds_h)
    _, full = ct.jacobian(args)
    part = [torch.empty((24, 4, n), dtype=torch.float64, device="cuda"), None]
    ct.jacobian(args, jac=part)
    assert_bitexact(host([part[0]])[0], host(full)[0], "jacobian of xN")
    r1, j1, a1 = ct.jacobian_reverse(args, aseeds)
    j2 = [torch.empty((24, 4, n), dtype=torch.float64, device="cuda"), None]
    r2, _, a2 = ct.jacobian_reverse(args, aseeds, jac=j2)
    for x, y in zip(host(r1) + [host(j1)[0]] + host(a1), host(r2) + host([j2[0]]) + host(a2)):
        assert_bitexact(x, y, "jacobian_reverse with the cost's Jacobian left out")
    m = CudaMap(F, n)
    hargs = [a.T.copy() for a in args_h]
    hseeds = [np.transpose(s, (2, 0, 1)).copy() for s in aseeds_h]
    _, hj, ha = m.jacobian_reverse(hargs, hseeds, jac=[np.empty((n, 24, 4)), None])
    assert_bitexact(np.transpose(hj[0], (1, 2, 0)), host(j1)[0], "host buffers")
    ct.sync()


def test_sweeps_replay_from_a_cuda_graph(gpu_lib):
    """After one warm-up call (plans built, variants tuned), the derivative entry points can
    be captured into a CUDA graph and replayed: the replays read the inputs' current contents
    and give the same bits as direct calls."""
    F = W.cartpole_rollout(4)
    n = 4096
    ct = CudaTape(F)
    args = dev(W.cartpole_inputs(n, steps=4, seed=51))
    aseeds = dev([np.zeros((1, 4, n)), np.ones((1, 1, n))])
    res, jac, asens = ct.jacobian_reverse(args, aseeds)  # warm-up
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ct.jacobian_reverse(args, aseeds, res=res, jac=jac, asens=asens, stream=s)
    for seed in (52, 53):
        for a, v in zip(args, dev(W.cartpole_inputs(n, steps=4, seed=seed))):
            a.copy_(v)
        g.replay()
        torch.cuda.synchronize()
        want_r, want_j, want_a = ct.jacobian_reverse(args, aseeds)
        for x, y in zip(host(res) + host(jac) + host(asens),
                        host(want_r) + host(want_j) + host(want_a)):
            assert_bitexact(x, y, "graph replay")
    ct.sync()


@pytest.mark.parametrize("case", ["rollout_general", "rollout_jacobian", "dag_jacobian"])
def test_windowed_tangent_gives_the_warp_sweep_bits(gpu_lib, case):
    """The windowed tangent sweep (a tile's directions co-scheduled on one SM, partials and
    entries staged into shared memory) does k_tangent's arithmetic entry for entry: forward
    sensitivities and Jacobians are identical bit for bit, with ragged instance counts,
    general seeds, and more directions than one CTA holds (several direction groups)."""
    from casadi_gb300 import runtime as R
    if case == "dag_jacobian":
        F = W.random_dag(n_in=40, n_nodes=1500, n_out=6, seed=8, bounded=True)
        n = 1000
        args = dev(W.dag_inputs(n, n_in=40, seed=8))
    else:
        F = W.cartpole_rollout(8)
        n = 2003
        args = dev(W.cartpole_inputs(n, steps=8, seed=23))
    ct = CudaTape(F)
    kind = 0 if case == "rollout_general" else 1

    def run():
        if kind == 0:
            rng = np.random.default_rng(23)
            fseeds = dev([rng.standard_normal((6, k, n)) for k in F.tape.nnz_in])
            return host(ct.forward(args, fseeds)[1])
        return host(ct.jacobian(args)[1])

    ct.set_variant(kind, 0)
    want = run()
    ct.set_variant(kind, R.TAN_WINDOWED)
    got = run()
    assert ct.tuned_variant(kind) == R.TAN_WINDOWED
    for x, y in zip(got, want):
        assert_bitexact(x, y, "windowed tangent, " + case)
    ct.sync()
