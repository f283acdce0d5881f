"""Colour-compressed sparse Jacobians and Hessians (coloured forward sweeps + device
gather) on the multiple-shooting quadcopter NLP: the constraint Jacobian against the dense
unit-seed Jacobian of the same tape (same bits) and the oracle, the Lagrangian Hessian
against the oracle's dense Jacobian of the same symbolic gradient, against central
differences of the oracle's adjoint, and its symmetry."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import workloads as W

from helpers import RTOL, assert_close, magnitudes, same_bits

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

INTERVALS = 3


def _inputs(n, seed=0):
    return W.quad_ms_inputs(n, intervals=INTERVALS, seed=seed)


def test_colored_constraint_jacobian(gpu_lib):
    from casadi_gb300.sparse_ad import ColoredJacobian
    F = W.quad_ms_constraints(INTERVALS)
    n = 333
    args = _inputs(n, 1)
    J = ColoredJacobian(F, out=0, wrt=0)
    nw = F.tape.nnz_in[0]
    assert J.n_colors < nw / 4  # the coloring compresses the 12+4 per interval band
    vals = J([torch.from_numpy(a).cuda() for a in args]).cpu().numpy()
    rows, cols = J.pattern.row, J.pattern.col()
    # dense unit-seed Jacobian of the same tape: jac[0] has shape (nnz_in_total, nnz_g, n)
    _, jac = J.tape.jacobian([torch.from_numpy(a).cuda() for a in args])
    dense = jac[0].cpu().numpy()[:nw]  # rows: w nonzeros
    assert same_bits(vals, dense[cols, rows]).all()
    # and every entry outside the pattern is zero
    mask = np.ones((nw, dense.shape[1]), bool)
    mask[cols, rows] = False
    assert not np.any(dense[mask])
    _, wjac = O.jacobian(F.tape, args, n)
    _, jmag = magnitudes(O.jacobian, F.tape, args, n)
    assert_close(vals, wjac[0][cols, rows], "colored constraint Jacobian",
                 bound=RTOL * jmag[0][cols, rows])


def test_colored_lagrangian_hessian(gpu_lib):
    from casadi_gb300.sparse_ad import ColoredHessian
    F = W.quad_ms_lagrangian(INTERVALS)
    n = 257
    args = _inputs(n, 2)
    H = ColoredHessian(F, out=1, wrt=0)
    nw = F.tape.nnz_in[0]
    assert H.n_colors < nw / 3
    vals = H([torch.from_numpy(a).cuda() for a in args]).cpu().numpy()
    # oracle: dense Jacobian of the same gradient tape
    G = H.gradient_function
    _, gj = O.jacobian(G.tape, args, n)
    _, gm = magnitudes(O.jacobian, G.tape, args, n)
    dense = gj[0][:nw]  # [w nonzero j][gradient entry i][instance] = H[i, j]
    mag = gm[0][:nw]
    assert_close(vals, dense[H.cols, H.rows], "colored Hessian vs oracle",
                 bound=RTOL * mag[H.cols, H.rows])
    # symmetric: H[i, j] == H[j, i] in the oracle's dense Hessian, up to the rounding of the
    # two different chain-rule sums that give them
    assert_close(dense[H.rows, H.cols], dense[H.cols, H.rows], "symmetry",
                 bound=RTOL * (mag[H.rows, H.cols] + mag[H.cols, H.rows]))
    # central differences of the oracle's adjoint (gradient of the Lagrangian) on 3 instances
    m, h = 3, 1e-6
    Hd = np.zeros((nw, nw, m))
    Hd[H.rows, H.cols] = vals[:, :m]
    Hd[H.cols, H.rows] = vals[:, :m]
    sub = [a[:, :m].copy() for a in args]
    seeds = [np.zeros((1, k, m)) for k in F.tape.nnz_out]
    seeds[1][:] = 1.0
    for j in (0, 5, 12, 20, nw - 13):
        p = [a.copy() for a in sub]
        q = [a.copy() for a in sub]
        p[0][j] += h
        q[0][j] -= h
        gp = O.reverse(F.tape, p, seeds, m)[1][0][0]
        gq = O.reverse(F.tape, q, seeds, m)[1][0][0]
        col = (gp - gq) / (2 * h)  # column j of H, (nw, m)
        assert np.max(np.abs(Hd[:, j] - col) / np.maximum(np.abs(col), 1.0)) < 1e-5


def test_colored_sweeps_in_one_batch_launch(gpu_lib):
    """The constraint Jacobian and the Lagrangian Hessian as two items of one persistent
    batch (replayed from a CUDA graph): the same bits as the separate coloured calls."""
    from casadi_gb300 import runtime as R
    from casadi_gb300.sparse_ad import ColoredHessian, ColoredJacobian
    L = W.quad_ms_lagrangian(INTERVALS)
    J = ColoredJacobian(W.quad_ms_constraints(INTERVALS), out=0, wrt=0)
    H = ColoredHessian(L, out=1, wrt=0)
    n = 1000
    args = [torch.from_numpy(a).cuda() for a in _inputs(n, 3)]
    want_j, want_h = J(args).cpu().numpy(), H(args).cpu().numpy()
    b = R.Batch()
    cj = J.add_to_batch(b, args)
    ch = H.add_to_batch(b, args)
    for _ in range(2):
        b.run(graph=True)
        b.status()
        got_j = J.gather(cj, n).cpu().numpy()
        got_h = H.gather(ch, n).cpu().numpy()
        assert same_bits(got_j, want_j).all()
        assert same_bits(got_h, want_h).all()


@pytest.mark.parametrize("variant", [0, 6, 7])
def test_colored_sweeps_same_bits_in_every_tangent_variant(gpu_lib, variant):
    """Coloured seeding (identity directions through a colour map) with the sequential
    tangent sweep (variants 0 and 6) and the cooperative level sweep (variant 7): the same bits as
    the autotuned call."""
    from casadi_gb300.sparse_ad import ColoredHessian, ColoredJacobian
    L = W.quad_ms_lagrangian(INTERVALS)
    J = ColoredJacobian(W.quad_ms_constraints(INTERVALS), out=0, wrt=0)
    H = ColoredHessian(L, out=1, wrt=0)
    n = 777
    args = [torch.from_numpy(a).cuda() for a in _inputs(n, 4)]
    want_j, want_h = J(args).cpu().numpy(), H(args).cpu().numpy()
    J.tape.set_variant(1, variant)
    H.tape.set_variant(1, variant)
    got_j, got_h = J(args).cpu().numpy(), H(args).cpu().numpy()
    assert same_bits(got_j, want_j).all()
    assert same_bits(got_h, want_h).all()
    J.tape.sync()


def test_jacobian_pattern_forward_equals_reverse(gpu_lib):
    """The Jacobian sparsity from forward bit sweeps (one bit per input nonzero) and from
    reverse bit sweeps (one bit per output nonzero) are the same pattern."""
    from casadi_gb300 import runtime as R
    from casadi_gb300.sparse_ad import jacobian_pattern
    for f, out in ((W.quad_ms_constraints(INTERVALS), 0), (W.random_dag(n_in=70, n_nodes=900,
                                                                        n_out=130, seed=8), 0)):
        ct = R.CudaTape(f)
        pf = jacobian_pattern(ct, out, 0, mode="forward")
        pr = jacobian_pattern(ct, out, 0, mode="reverse")
        assert np.array_equal(pf.dense(), pr.dense())
        pa = jacobian_pattern(ct, out, 0)
        assert np.array_equal(pa.dense(), pf.dense())
        ph = jacobian_pattern(ct, out, 0, mode="hierarchical")
        assert np.array_equal(ph.dense(), pf.dense())
        ct.sync()


def test_hierarchical_pattern_on_the_device_is_casadis(gpu_lib):
    """The MPC constraint Jacobian (1212 x 1612, hierarchical in the reference as here) from
    the device's refinement sweeps equals CasADi's get_jac_sparsity_hierarchical pattern, in
    two levels of one word each."""
    from casadi_gb300 import runtime as R
    from casadi_gb300 import sx as S
    from casadi_gb300.sparse_ad import jacobian_pattern_hierarchical
    from helpers import load_npz
    L = W.quad_ms_lagrangian(100)
    g = S.Function("g", L.inputs, [L.outputs[0]])
    ct = R.CudaTape(g)
    stats = {}
    p = jacobian_pattern_hierarchical(ct, 0, 0, stats=stats)
    z = load_npz("casadi.npz")
    nr, nc = z["quad/jac_jacsp_shape"]
    assert (p.nrow, p.ncol) == (nr, nc)
    assert np.array_equal(p.colind, z["quad/jac_jacsp_colind"])
    assert np.array_equal(p.row, z["quad/jac_jacsp_row"])
    assert stats == {"levels": 2, "words": 2}
    ct.sync()


def test_kkt_function_of_the_nlp(gpu_lib):
    """Nlpsol::kkt(): the constraint Jacobian and the full symmetric Lagrangian Hessian (upper
    triangle mirrored on the device) of the multiple-shooting NLP, against the oracle's dense
    derivatives; the batched graph gives the same bits as the separate calls."""
    from casadi_gb300.sparse_ad import KKT
    w, x0bar, obj, g = W.quad_ms_nlp(INTERVALS)
    kkt = KKT(w, x0bar, obj, g)
    n = 129
    rng = np.random.default_rng(6)
    ww, _, xb = _inputs(n, 6)
    lam_f = rng.uniform(0.5, 2.0, (1, n))
    lam_g = rng.standard_normal((len(g), n))
    args_h = [ww, xb, lam_f, lam_g]
    args = [torch.from_numpy(a).cuda() for a in args_h]
    jac, hess = [t.cpu().numpy() for t in kkt(args)]
    nw = len(w)
    # Jacobian of g against the oracle's dense Jacobian
    _, gj = O.jacobian(kkt.g_function.tape, args_h, n)
    _, gm = magnitudes(O.jacobian, kkt.g_function.tape, args_h, n)
    rows, cols = kkt.jac_pattern.row, kkt.jac_pattern.col()
    assert_close(jac, gj[0][cols, rows], "jac:g:x", bound=RTOL * gm[0][cols, rows])
    # Hessian: symmetric bit for bit, and the oracle's Jacobian of the symbolic gradient
    hp = kkt.hess_pattern
    hr, hc = hp.row, hp.col()
    full = {(int(i), int(j)): k for k, (i, j) in enumerate(zip(hr, hc))}
    for k, (i, j) in enumerate(zip(hr, hc)):
        assert same_bits(hess[k], hess[full[(int(j), int(i))]]).all()
    _, hj = O.jacobian(kkt.hess.gradient_function.tape, args_h, n)
    _, hm = magnitudes(O.jacobian, kkt.hess.gradient_function.tape, args_h, n)
    assert_close(hess, hj[0][:nw][hc, hr], "hess:gamma:x:x", bound=RTOL * hm[0][:nw][hc, hr])
    # the batched graph
    run = kkt.batched(args)
    for _ in range(2):
        bj, bh = run()
        run.batch.status()
        assert same_bits(bj.cpu().numpy(), jac).all() and same_bits(bh.cpu().numpy(), hess).all()
