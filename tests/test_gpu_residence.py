"""Global-memory work vectors: the same sweeps with the work vector in per-CTA blocks of
global memory instead of shared memory. Forced on a small tape, every result must equal the
shared-memory path bit for bit; on a tape whose scheduled work vector does not fit shared
memory (the quadcopter NLP's Lagrangian with both outputs, 1447 slots) the path is taken
automatically and checked against the oracle. The cooperative level sweep (residence 3: several
warps share a tile and run the tape level by level) must give the same bits as well."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import assert_adjoint_close, assert_bitexact, assert_close, magnitudes, value_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(arrs):
    return [None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def _host(ts):
    return [t.cpu().numpy() for t in ts]


@pytest.mark.parametrize("mode", [1, 3])
def test_forced_residence_equals_shared(gpu_lib, mode):
    F = W.cartpole_rollout(6)
    n = 3001
    args = _dev(W.cartpole_inputs(n, steps=6, seed=41))
    rng = np.random.default_rng(41)
    fseeds = _dev([rng.standard_normal((3, k, n)) for k in F.tape.nnz_in])
    aseeds = _dev([rng.standard_normal((2, k, n)) for k in F.tape.nnz_out])
    bits = [torch.randint(0, 1 << 62, (k, n), dtype=torch.int64, device="cuda")
            for k in F.tape.nnz_in]

    def run(ct):
        out = [_host(ct.eval(args))]
        out.append(_host(ct.forward(args, fseeds)[1]))
        out.append(_host(ct.jacobian(args)[1]))
        out.append(_host(ct.reverse(args, aseeds)[1]))
        out.append(_host(ct.sp_forward(bits)))
        sens = [torch.zeros((k, n), dtype=torch.int64, device="cuda") for k in F.tape.nnz_in]
        seeds = [torch.randint(0, 1 << 62, (k, n), dtype=torch.int64, device="cuda",
                               generator=torch.Generator(device="cuda").manual_seed(5))
                 for k in F.tape.nnz_out]
        ct.sp_reverse(sens, seeds)
        out.append(_host(sens))
        ct.sync()
        return out

    sh = R.CudaTape(F)
    sh.set_residence(2)
    shared = run(sh)
    g = R.CudaTape(F)
    g.set_residence(mode)
    glob = run(g)
    for a, b in zip(shared, glob):
        for x, y in zip(a, b):
            if x.dtype == np.int64:
                assert np.array_equal(x, y)
            else:
                assert_bitexact(x, y, "residence %d" % mode)


def test_tape_larger_than_shared_memory(gpu_lib):
    F = W.quad_ms_lagrangian(100)
    ct = R.CudaTape(F)
    assert ct.sz_w > 900  # does not fit the shared-memory sweeps
    n = 300
    args = W.quad_ms_inputs(n, intervals=100, seed=7)
    res = _host(ct.eval(_dev(args)))
    want = O.eval(F.tape, args, n)
    for g, w, b in zip(res, want, value_bounds(F.tape, args, n)):
        assert_close(g, w, "values", bound=b)
    seeds = [np.zeros((1, k, n)) for k in F.tape.nnz_out]
    seeds[1][:] = 1.0
    _, asens = ct.reverse(_dev(args), _dev(seeds))
    _, was = O.reverse(F.tape, args, seeds, n)
    _, mag = magnitudes(O.reverse, F.tape, args, seeds, n)
    # a handful of sensitivities cancel so far that the sin/cos ulps of the primal values,
    # carried through the partials, exceed 1e-13 of their magnitude: the adjoint-Function bound
    assert_adjoint_close([a[0] for a in _host(asens)], [w[0] for w in was], [m[0] for m in mag],
                         F, args, [s[0] for s in seeds], "adjoint of the Lagrangian")
    ct.sync()


@pytest.mark.parametrize("n", [1, 31, 4096, 100000])
def test_cooperative_sweeps_on_wide_tapes(gpu_lib, n):
    """The quadcopter multiple-shooting constraints (34156 instructions, wide levels) and the
    random DAG: values, the unit-seed Jacobian and the adjoint with the cooperative value,
    record, tangent and adjoint sweeps equal the sequential sweeps bit for bit (and the oracle
    within tolerance);
    100000 instances is past the launch size where the autotuner considers the cooperative
    sweep, so there it runs only because it is forced."""
    cases = [(W.random_dag(), W.dag_inputs(n, seed=3))]
    if n <= 4096:
        cases.append((W.quad_ms_constraints(100), W.quad_ms_inputs(n, intervals=100, seed=3)))
    for F, args_h in cases:
        args = _dev(args_h)
        rng = np.random.default_rng(n)
        aseeds = _dev([rng.standard_normal((1, k, n)) for k in F.tape.nnz_out])
        out = {}
        for mode in (2, 1, 3):
            ct = R.CudaTape(F)
            ct.set_residence(mode)
            if mode == 3:
                # the cooperative tangent and adjoint sweeps too
                ct.set_variant(1, R.N_TAN_VARIANTS - 1)
                ct.set_variant(2, R.N_ADJ_VARIANTS - 1)
            r = [_host(ct.eval(args))]
            r.append(_host(ct.reverse(args, aseeds)[1]))
            if F.tape.n_instr < 20000:
                r.append(_host(ct.jacobian(args)[1]))
            ct.sync()
            out[mode] = r
        for mode in (1, 3):
            for a, b in zip(out[2], out[mode]):
                for x, y in zip(a, b):
                    assert_bitexact(x, y, "residence %d" % mode)
        if n <= 4096:
            m = min(n, 64)
            sub = [a[:, :m].copy() for a in args_h]
            want = O.eval(F.tape, sub, m)
            for g, w, b in zip(out[3][0], want, value_bounds(F.tape, sub, m)):
                assert_close(g[:, :m], w, "values", bound=b)
