"""Hierarchical Jacobian sparsity (sparse_ad.jacobian_pattern_hierarchical), checked on the CPU
with the oracle's bvec sweeps as the sweeper: the MPC constraint Jacobian (1212 x 1612) and the
Hessian pattern of the Lagrangian's gradient equal the patterns CasADi's own
get_jac_sparsity_hierarchical produced (both sides exceed 3 x 64 nonzeros, so the reference took
that path), random DAGs equal one bit per nonzero, and the refinement sweeps fewer words than
one bit per nonzero does on sparse Jacobians."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import coloring as K
from casadi_gb300 import sparse_ad as SA
from casadi_gb300 import sx as S
from casadi_gb300 import workloads as W

from helpers import load_npz


def oracle_sweeper(tape, out, wrt):
    def sweep(forward, seeds):
        n = seeds.shape[1]
        if forward:
            args = [np.zeros((k, n), np.uint64) for k in tape.nnz_in]
            args[wrt] = seeds
            return O.sp_forward(tape, args, n)[out]
        args = [np.zeros((k, n), np.uint64) for k in tape.nnz_in]
        res = [np.zeros((k, n), np.uint64) for k in tape.nnz_out]
        res[out] = seeds.copy()
        O.sp_reverse(tape, args, res, n)
        return args[wrt]
    return sweep


def one_bit_per_nonzero(tape, out, wrt):
    n_in = tape.nnz_in[wrt]
    n = (n_in + 63) // 64
    seeds = np.zeros((n_in, n), np.uint64)
    for c in range(n_in):
        seeds[c, c // 64] = np.uint64(1) << np.uint64(c % 64)
    r = oracle_sweeper(tape, out, wrt)(True, seeds)
    mask = np.zeros((tape.nnz_out[out], n_in), bool)
    for c in range(n_in):
        mask[:, c] = (r[:, c // 64] >> np.uint64(c % 64)) & np.uint64(1) == 1
    return mask, n


def _pattern(z, key):
    nr, nc = z[key + "_shape"]
    return K.Pattern(nr, nc, z[key + "_colind"], z[key + "_row"])


@pytest.fixture(scope="module")
def lagrangian():
    return W.quad_ms_lagrangian(100)


def test_mpc_constraint_jacobian_is_casadis(lagrangian):
    g = S.Function("g", lagrangian.inputs, [lagrangian.outputs[0]])
    stats = {}
    p = SA.jacobian_pattern_hierarchical(g.tape, 0, 0, sweep=oracle_sweeper(g.tape, 0, 0),
                                         stats=stats)
    want = _pattern(load_npz("casadi.npz"), "quad/jac_jacsp")
    assert (p.nrow, p.ncol) == (want.nrow, want.ncol) == (1212, 1612)
    assert np.array_equal(p.colind, want.colind) and np.array_equal(p.row, want.row)
    _, plain_words = one_bit_per_nonzero(g.tape, 0, 0)
    assert stats["levels"] == 2 and stats["words"] < plain_words


def test_mpc_hessian_pattern_is_casadis(lagrangian):
    G = S.Function("grad_L", lagrangian.inputs, [S.gradient(lagrangian, 1, 0)])
    p = SA.jacobian_pattern_hierarchical(G.tape, 0, 0, sweep=oracle_sweeper(G.tape, 0, 0))
    want = _pattern(load_npz("casadi.npz"), "quad/hess_jacsp")
    assert np.array_equal(p.dense() | p.dense().T, want.dense())


@pytest.mark.parametrize("n_in,n_nodes,n_out,seed", [(300, 2500, 250, 1), (200, 900, 400, 2),
                                                     (70, 400, 9, 3), (5, 40, 3, 4)])
def test_random_dags_equal_one_bit_per_nonzero(n_in, n_nodes, n_out, seed):
    f = W.random_dag(n_in=n_in, n_nodes=n_nodes, n_out=n_out, seed=seed)
    p = SA.jacobian_pattern_hierarchical(f.tape, 0, 0, sweep=oracle_sweeper(f.tape, 0, 0))
    mask, _ = one_bit_per_nonzero(f.tape, 0, 0)
    assert np.array_equal(p.dense(), mask)


def test_mode_weight_and_other_inputs():
    """Reverse-leaning weights give the same pattern; a second input stays unseeded."""
    x, y = S.sym("x", 300), S.sym("y", 2)
    outs = [x[(k * 7) % 300] * x[(k * 13 + 1) % 300] + y[k % 2] for k in range(260)]
    f = S.Function("f", [x, y], [outs])
    fwd = SA.jacobian_pattern_hierarchical(f.tape, 0, 0, sweep=oracle_sweeper(f.tape, 0, 0))
    rev = SA.jacobian_pattern_hierarchical(f.tape, 0, 0, sweep=oracle_sweeper(f.tape, 0, 0),
                                           weight=0.99)
    mask, _ = one_bit_per_nonzero(f.tape, 0, 0)
    assert np.array_equal(fwd.dense(), mask) and np.array_equal(rev.dense(), mask)
    assert fwd.nnz == 2 * 260 - sum(1 for k in range(260) if (k * 7) % 300 == (k * 13 + 1) % 300)
