"""The segment plan of the checkpointed adjoint (casadi_gb300_tape_segments, host only),
checked on the CPU: the segment tapes, chained through the oracle -- forward in order keeping
the live slots at every cut, backward in reverse seeding each segment with the next one's
live-in adjoints -- give the oracle's values and adjoints of the whole scheduled tape bit for
bit (each adjoint sum associates across a cut as in the whole sweep), and the cuts land where
few slots are live."""
import numpy as np
import pytest

import oracle as O
from casadi_gb300 import calculus as C
from casadi_gb300 import runtime as R
from casadi_gb300 import workloads as W

from helpers import assert_bitexact


def _written(t, out_idx):
    """Nonzeros of output ``out_idx`` that tape t writes."""
    m = (np.asarray(t.op) == C.OP_OUTPUT) & (np.asarray(t.i0) == out_idx)
    return np.asarray(t.i2)[m]


def _read(t, in_idx):
    """Nonzeros of input ``in_idx`` that tape t reads."""
    m = (np.asarray(t.op) == C.OP_INPUT) & (np.asarray(t.i1) == in_idx)
    return np.asarray(t.i2)[m]


def _chain(tape, segs, args, aseeds, n):
    n_in, n_out = len(tape.nnz_in), len(tape.nnz_out)
    res = [np.zeros((k, n)) for k in tape.nnz_out]
    nadj = aseeds[0].shape[0]
    asens = [np.zeros((nadj, k, n)) for k in tape.nnz_in]
    ckpt = [np.zeros((0, n))]
    for s, g in enumerate(segs):
        r = O.eval(g, list(args) + [ckpt[s]], n)
        for j in range(n_out):
            nz = _written(g, j)
            res[j][nz] = r[j][nz]
        ckpt.append(r[n_out])
    adj = np.zeros((nadj, 0, n))
    for s in range(len(segs) - 1, -1, -1):
        g = segs[s]
        _, a = O.reverse(g, list(args) + [ckpt[s]], list(aseeds) + [adj], n)
        for j in range(n_in):
            nz = _read(g, j)
            asens[j][:, nz] = a[j][:, nz]
        adj = a[n_in]
    return res, asens


@pytest.mark.parametrize("name,k", [("rollout", 1), ("rollout", 2), ("rollout", 5),
                                    ("rollout", 13), ("dag", 3), ("dag", 8), ("quad", 4)])
def test_chained_segments_give_the_whole_tapes_bits(name, k):
    if name == "rollout":
        f = W.cartpole_rollout(20)
        n = 37
        args = list(W.cartpole_inputs(n, steps=20, seed=1))
    elif name == "dag":
        f = W.random_dag(n_in=16, n_nodes=1500, n_out=6, seed=4)
        n = 29
        args = list(W.dag_inputs(n, n_in=16, seed=2))
    else:
        f = W.quad_ms_lagrangian(4)
        n = 11
        args = list(W.quad_ms_inputs(n, intervals=4, seed=3))
    sched = R.schedule(f.tape)
    cut, live, segs = R.segments(f.tape, k)
    assert len(segs) == k and cut[0] == 0 and cut[-1] == sched.n_instr
    assert all(a < b for a, b in zip(cut, cut[1:]))
    assert live[0] == 0 and live[-1] == 0
    rng = np.random.default_rng(k)
    aseeds = [rng.standard_normal((2, m, n)) for m in f.tape.nnz_out]
    res, asens = _chain(sched, segs, args, aseeds, n)
    wres, wasens = O.reverse(sched, args, aseeds, n)
    for g, w in zip(res, wres):
        assert_bitexact(g, w, "%s k=%d values" % (name, k))
    for g, w in zip(asens, wasens):
        assert_bitexact(g, w, "%s k=%d adjoints" % (name, k))


def test_cuts_prefer_few_live_slots():
    """On the 20-step rollout a cut lands between steps, where the state and the running
    cost are live with a few temporaries (14 slots), half the scheduled work vector (28)."""
    f = W.cartpole_rollout(20)
    sched = R.schedule(f.tape)
    cut, live, segs = R.segments(f.tape, 10)
    assert max(live) <= 16 and 2 * max(live) <= sched.sz_w
    # partial counts of the segments are within a factor two of an equal share
    parts = [sum(1 for o in g.op if o not in (C.OP_CONST, C.OP_INPUT, C.OP_OUTPUT))
             for g in segs]
    assert max(parts) < 2 * sum(parts) / len(parts)


def test_segment_counts_beyond_the_tape_and_bad_ones():
    f = W.cartpole_step()
    sched = R.schedule(f.tape)
    cut, live, segs = R.segments(f.tape, 10 * sched.n_instr)
    assert len(segs) == sched.n_instr and all(b - a == 1 for a, b in zip(cut, cut[1:]))
    with pytest.raises(R.CasadiGpuError):
        R.segments(f.tape, 0)
