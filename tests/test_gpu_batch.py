"""Persistent multi-tape batches (casadi_gb300_batch_*): several tapes over their own
instance ranges in one launch must give the same numbers as evaluating each tape on its own
(the per-tape value sweep and the per-tape adjoint sweep run the same device arithmetic, so
the comparison is bit for bit), and the oracle's within the documented tolerance."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import RTOL, assert_close, magnitudes, same_bits, value_bounds

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _items():
    """(Function, n, nadj, inputs) covering eval-only and adjoint items, ragged tiles, a
    one-instance item, two tapes of very different length, and split items (two or more
    directions) recorded cooperatively before the launch (few tiles) or by record units."""
    out = []
    f = W.cartpole_rollout(4)
    out.append((f, 1000, 1, W.cartpole_inputs(1000, steps=4, seed=1)))
    out.append((f, 33, 2, W.cartpole_inputs(33, steps=4, seed=2)))
    # two directions over more tiles than the cooperative pre-record takes: per-tile record
    # units inside the persistent launch
    out.append((f, 20000, 2, W.cartpole_inputs(20000, steps=4, seed=7)))
    g = W.random_dag(n_in=16, n_nodes=3000, n_out=4, seed=3, window=64, bounded=True)
    out.append((g, 5000, 1, W.dag_inputs(5000, n_in=16, seed=3)))
    out.append((g, 1, 0, W.dag_inputs(1, n_in=16, seed=4)))
    h = W.random_dag(n_in=16, n_nodes=300, n_out=4, seed=5, window=32, bounded=True)
    out.append((h, 777, 0, W.dag_inputs(777, n_in=16, seed=5)))
    out.append((h, 64, 3, W.dag_inputs(64, n_in=16, seed=6)))
    return out


def _seeds(f, n, nadj, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((nadj, k, n)) for k in f.tape.nnz_out]


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_per_tape_sweeps(gpu_lib, graph):
    items = _items()
    tapes = {}
    b = R.Batch()
    queued = []
    for k, (f, n, nadj, args) in enumerate(items):
        t = tapes.setdefault(id(f), R.CudaTape(f))
        dargs = [_cuda(a) for a in args]
        dseeds = [_cuda(s) for s in _seeds(f, n, nadj, k)] if nadj else None
        res, asens = b.add(t, dargs, dseeds)
        queued.append((t, dargs, dseeds, res, asens))
    b.run(graph=graph)
    if graph:
        b.run(graph=True)  # replay
    b.status()
    for t, dargs, dseeds, res, asens in queued:
        t.sync()
        if dseeds is None:
            want = t.eval(dargs)
            for g, w in zip(res, want):
                assert same_bits(g.cpu().numpy(), w.cpu().numpy()).all()
        else:
            want_r, want_s = t.reverse(dargs, dseeds)
            for g, w in zip(res, want_r):
                assert same_bits(g.cpu().numpy(), w.cpu().numpy()).all()
            for g, w in zip(asens, want_s):
                assert same_bits(g.cpu().numpy(), w.cpu().numpy()).all()


def test_batch_matches_oracle(gpu_lib):
    items = _items()
    b = R.Batch()
    queued = []
    for k, (f, n, nadj, args) in enumerate(items):
        t = R.CudaTape(f)
        seeds = _seeds(f, n, nadj, k) if nadj else None
        res, asens = b.add(t, [_cuda(a) for a in args],
                           [_cuda(s) for s in seeds] if seeds else None)
        queued.append((f, n, args, seeds, res, asens, t))
    b.run()
    b.status()
    for k, (f, n, args, seeds, res, asens, t) in enumerate(queued):
        t.sync()
        # thousands of sin/cos/exp/tanh nodes carry the <= 1-ulp differences between CUDA's and
        # the host libm into values and adjoints: element-wise bounds from the oracle
        want = O.eval(f.tape, args, n)
        vb = value_bounds(f.tape, args, n)
        for j, (g, w) in enumerate(zip(res, want)):
            assert_close(g.cpu().numpy(), w, "item %d value %d" % (k, j), bound=vb[j])
        if seeds:
            for d in range(seeds[0].shape[0]):
                sd = [s[d:d + 1] for s in seeds]
                _, ws = O.reverse(f.tape, args, sd, n)
                _, ms = magnitudes(O.reverse, f.tape, args, sd, n)
                for j, (w, m) in enumerate(zip(ws, ms)):
                    assert_close(asens[j][d].cpu().numpy(), w[0],
                                 "item %d adjoint %d/%d" % (k, d, j), bound=RTOL * m[0])


def test_batch_graph_replay_sees_new_inputs(gpu_lib):
    """A replayed graph reads the inputs' current contents (same pointers, new values)."""
    f = W.cartpole_rollout(4)
    t = R.CudaTape(f)
    n = 300
    args = [_cuda(a) for a in W.cartpole_inputs(n, steps=4, seed=11)]
    seeds = [_cuda(s) for s in _seeds(f, n, 1, 11)]
    b = R.Batch()
    res, asens = b.add(t, args, seeds)
    b.run(graph=True)
    new = W.cartpole_inputs(n, steps=4, seed=12)
    for a, v in zip(args, new):
        a.copy_(_cuda(v))
    b.run(graph=True)
    want_r, want_s = t.reverse(args, seeds)
    for g, w in zip(res + asens, want_r + want_s):
        assert same_bits(g.cpu().numpy(), w.cpu().numpy()).all()


def test_batch_rejects_small_scratch_and_bad_ids(gpu_lib):
    import ctypes as ct
    lib = R.load()
    assert lib.casadi_gb300_batch_run(12345, None, 0, 0, None) == -1
    f = W.cartpole_rollout(2)
    t = R.CudaTape(f)
    b = R.Batch()
    args = [_cuda(a) for a in W.cartpole_inputs(64, steps=2, seed=1)]
    b.add(t, args, [_cuda(s) for s in _seeds(f, 64, 1, 1)])
    assert b.scratch_bytes() > 0
    st = lib.casadi_gb300_batch_run(b.id, None, 0, 0, ct.c_void_p(0))
    assert st == -5
    assert lib.casadi_gb300_batch_add(b.id, 999999, 1, 1, 0, None, None, None, None) == -1


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_residence_gives_the_same_bits(gpu_lib, mode):
    """The batch with its work vectors forced into global (1) or shared (2) memory."""
    items = _items()
    tapes = {}
    b = R.Batch()
    b.set_residence(mode)
    queued = []
    for k, (f, n, nadj, args) in enumerate(items):
        t = tapes.setdefault(id(f), R.CudaTape(f))
        dargs = [_cuda(a) for a in args]
        dseeds = [_cuda(s) for s in _seeds(f, n, nadj, k)] if nadj else None
        res, asens = b.add(t, dargs, dseeds)
        queued.append((t, dargs, dseeds, res, asens))
    b.run(graph=True)
    b.status()
    for t, dargs, dseeds, res, asens in queued:
        if dseeds is None:
            for g, w in zip(res, t.eval(dargs)):
                assert same_bits(g.cpu().numpy(), w.cpu().numpy()).all()
        else:
            want_r, want_s = t.reverse(dargs, dseeds)
            for g, w in zip(res + asens, want_r + want_s):
                assert same_bits(g.cpu().numpy(), w.cpu().numpy()).all()
