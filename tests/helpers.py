"""Shared test helpers: fixture loading and the comparison rules used by the parity tests.

Tolerances:
  * EXACT_OPS and tapes built only from them (+,-,*,/,sqrt and the sign/compare/select ops):
    bit-exact (NaN == NaN, -0 and +0 distinguished only where the op defines the sign).
  * anything that calls a libm transcendental: element-wise |a-b| <= RTOL * |b| with
    RTOL = 1e-13, or within a stated per-element bound (assert_close): for a value, the
    libm and rounding perturbations propagated to it (value_bounds); for a derivative, 1e-13
    of the magnitude of its chain-rule terms (magnitudes), plus, on long chains, the libm
    propagation through the derivative Function (adjoint_bounds).
"""
import math
import os

import numpy as np

from casadi_gb300 import calculus as C
from casadi_gb300 import sx as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL = 1e-13

EXACT_OPS = frozenset([
    C.OP_ASSIGN, C.OP_ADD, C.OP_SUB, C.OP_MUL, C.OP_DIV, C.OP_NEG, C.OP_SQRT, C.OP_SQ,
    C.OP_TWICE, C.OP_LT, C.OP_LE, C.OP_EQ, C.OP_NE, C.OP_NOT, C.OP_AND, C.OP_OR, C.OP_FLOOR,
    C.OP_CEIL, C.OP_FMOD, C.OP_REMAINDER, C.OP_FABS, C.OP_SIGN, C.OP_COPYSIGN,
    C.OP_IF_ELSE_ZERO, C.OP_FMIN, C.OP_FMAX, C.OP_INV, C.OP_LIFT])


def load_npz(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_tape(z, name):
    t = S.Tape(z[name + "/op"], z[name + "/i0"], z[name + "/i1"], z[name + "/i2"],
               z[name + "/d"], z[name + "/nnz_in"].tolist(), z[name + "/nnz_out"].tolist(),
               int(z[name + "/sz_w"]))
    return t


def canonical_tape_bytes(op, i0, i1, i2, d):
    """The bytes two tapes are compared by. The reference's ScalarAtomic overlays the constant
    ``d`` on ``{i1, i2}`` (casadi/core/sx_function.hpp:37-44), so an OP_CONST is compared by its
    ``d`` and every other instruction by ``i1, i2``: int32 op, i0, i1, i2 (zero for constants)
    followed by the float64 bits of d (zero for non-constants)."""
    op = np.asarray(op, np.int32)
    c = op == C.OP_CONST
    i1 = np.where(c, 0, np.asarray(i1)).astype(np.int32)
    i2 = np.where(c, 0, np.asarray(i2)).astype(np.int32)
    d = np.where(c, np.asarray(d, np.float64), 0.0)
    return b"".join(np.ascontiguousarray(a).tobytes()
                    for a in (op, np.asarray(i0, np.int32), i1, i2, d))


def tape_sha256(t):
    """SHA-256 of a Tape's canonical bytes."""
    import hashlib
    return hashlib.sha256(canonical_tape_bytes(t.op, t.i0, t.i1, t.i2, t.d)).hexdigest()


def casadi_tape(z, name):
    """A tape the reference's libcasadi built, from casadi.npz (stored in full), with the
    union of d and {i1, i2} resolved: constants carry d, other instructions i1, i2."""
    op = z[name + "/op"]
    c = op == C.OP_CONST
    return S.Tape(op, z[name + "/i0"], np.where(c, 0, z[name + "/i1"]),
                  np.where(c, 0, z[name + "/i2"]), np.where(c, z[name + "/d"], 0.0),
                  z[name + "/nnz_in"].tolist(), z[name + "/nnz_out"].tolist(),
                  int(z[name + "/sz_w"]))


def golden_list(z, name, key, count):
    return [z["%s/%s%d" % (name, key, j)] for j in range(count)]


def same_bits(a, b):
    """Elementwise: identical doubles, or both NaN."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))


def assert_bitexact(a, b, what=""):
    ok = same_bits(a, b)
    if not ok.all():
        idx = np.argwhere(~ok)[:5]
        raise AssertionError("%s: %d of %d differ, e.g. %s" % (
            what, int((~ok).sum()), ok.size,
            [(tuple(int(v) for v in i), float(np.asarray(a)[tuple(i)]),
              float(np.asarray(b)[tuple(i)])) for i in idx]))


def rel_err(a, b, floor=1e-300):
    """Max of |a-b| / max(|b|, floor) over finite entries; NaN/inf must match exactly."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    fin = np.isfinite(b)
    if not np.array_equal(np.isnan(a), np.isnan(b)):
        return math.inf
    if not np.array_equal(a[np.isinf(b)], b[np.isinf(b)]):
        return math.inf
    if not fin.any():
        return 0.0
    d = np.abs(a[fin] - b[fin]) / np.maximum(np.abs(b[fin]), floor)
    return float(d.max())


def assert_close(a, b, what="", rtol=RTOL, floor=None, bound=None):
    """Element-wise: |a - b| <= rtol * max(|b|, floor) for every element (floor defaults to
    1e-300, i.e. none: each element is held to the relative bar), or, where a per-element
    ``bound`` is given, |a - b| <= bound -- the scale a difference of rounding is limited to
    for that element: 4 ulps of every libm result propagated to a value
    (``libm_ulps(oracle.libm_bound(...))``), or rtol times the magnitude of a derivative's
    chain-rule terms (``rtol * mag`` with mag from ``oracle.magnitude``). NaN and inf must
    match exactly. Returns the largest relative error."""
    a = np.asarray(a, np.float64)
    b_arr = np.asarray(b, np.float64)
    floor = 1e-300 if floor is None else floor
    if not np.array_equal(np.isnan(a), np.isnan(b_arr)):
        raise AssertionError("%s: NaN positions differ" % what)
    inf = np.isinf(b_arr)
    if not np.array_equal(a[inf], b_arr[inf]):
        raise AssertionError("%s: inf entries differ" % what)
    fin = np.isfinite(b_arr)
    with np.errstate(invalid="ignore"):  # inf - inf at matching infinities
        d = np.abs(a - b_arr)
    ok = ~fin | (d <= rtol * np.maximum(np.abs(b_arr), floor))
    if bound is not None:
        ok |= d <= np.asarray(bound, np.float64)
    if not ok.all():
        i = tuple(np.argwhere(~ok)[0])
        raise AssertionError("%s: %d of %d elements beyond the bar (rtol %.1e, floor %.1e%s), "
                             "e.g. %s: %r vs %r" % (what, int((~ok).sum()), ok.size, rtol,
                                                   floor, ", bounded" if bound is not None
                                                   else "", i, a[i], b_arr[i]))
    e = rel_err(a, b_arr, floor)
    return e


def libm_ulps(bound, ulps=4):
    """Per-element allowance for values: ``ulps`` relative perturbations of every libm result
    propagated to each value (bound from oracle.libm_bound)."""
    return ulps * 2.0**-52 * np.asarray(bound, np.float64)


def value_bounds(tape, args, n, nthreads=None):
    """Per output, the element-wise allowance of a value against the oracle's evaluation of the
    same tape: 4 ulps of every libm result (CUDA's and the host's libm each err by up to about
    2 ulps) and 1 ulp of every rounded result (an input that moved by a few ulps can flip the
    rounding of any instruction downstream), each propagated to the value to first order:
    2**-52 * (4 * libm_bound + rounding_bound)."""
    import oracle as O
    nt = nthreads or os.cpu_count() or 1
    lb = O.libm_bound(tape, args, n, nt)
    rb = O.rounding_bound(tape, args, n, nt)
    return [2.0**-52 * (4.0 * a + b) for a, b in zip(lb, rb)]


def rounding_bounds(tape, args, n):
    """Per output, the element-wise allowance of a value against the same function evaluated
    by a tape that rounds any instruction differently (another association of its sums, a
    chain of calls instead of one unrolled tape): 4 ulps of every rounded result propagated
    to it."""
    import oracle as O
    return [libm_ulps(b) for b in O.rounding_bound(tape, args, n)]


def adjoint_bounds(f, args, aseed, n):
    """Per input, the allowance of one adjoint direction (seeds ``aseed``, one (nnz_out, n)
    array per output) against the oracle's: 4 ulps of every libm result of the reference's
    adjoint Function f.reverse(1) (sx.reverse_function) at the same point, propagated to each
    sensitivity -- the sin/cos differences of the primal values carried through the partials.
    On long chains (a 100-step rollout) this exceeds 1e-13 of the magnitude of the chain-rule
    terms; the rounding of the adjoint sums themselves is what that magnitude term covers."""
    import oracle as O
    B = S.reverse_function(f)
    bargs = list(args) + [None] * len(f.tape.nnz_out) + list(aseed)
    return [libm_ulps(b) for b in O.libm_bound(B.tape, bargs, n, os.cpu_count() or 1)]


def magnitudes(fn, *args, **kw):
    """``fn`` (oracle.forward / reverse / jacobian) run in the oracle's magnitude mode: its
    derivative outputs are then the sums over chain-rule paths of |partials| x |seeds|."""
    import oracle as O
    with O.magnitude():
        return fn(*args, **kw)


def assert_adjoint_close(got, want, mag, f, args, aseed, what=""):
    """One adjoint direction of ``f`` (sensitivities ``got`` against the oracle's ``want``, one
    (nnz_in, n) array per input; ``mag`` their magnitudes; ``aseed`` one (nnz_out, n) seed per
    output) element-wise within 1e-13 of the magnitude, or, on the instances where that is
    exceeded, within that plus :func:`adjoint_bounds` (computed on those instances only)."""
    got = [np.asarray(g, np.float64) for g in got]
    want = [np.asarray(w, np.float64) for w in want]
    over = set()
    for g, w, m in zip(got, want, mag):
        bad = ~(same_bits(g, w) | (np.abs(g - w) <= RTOL * m))
        over.update(np.nonzero(bad.any(axis=0))[0].tolist())
    cols = np.array(sorted(over), dtype=np.int64)
    ab = None
    if cols.size:
        sub = [None if a is None else np.ascontiguousarray(a[:, cols]) for a in args]
        ab = adjoint_bounds(f, sub, [np.ascontiguousarray(s[:, cols]) for s in aseed], cols.size)
    for j, (g, w, m) in enumerate(zip(got, want, mag)):
        bound = RTOL * np.asarray(m, np.float64)
        if ab is not None:
            bound = bound.copy()
            bound[:, cols] += ab[j]
        assert_close(g, w, "%s (input %d)" % (what, j), bound=bound)


def call_rollout(steps):
    """Caller tape of a `steps`-step cart-pole rollout written as OP_CALL instructions of the
    one-step function (call index in i1): x0 (4 slots), U (steps slots), one call per step,
    xN out. Returns the tape and each call's (dep slots, res slots)."""
    op, i0, i1, i2 = [], [], [], []

    def emit(o, a, b, c):
        op.append(o), i0.append(a), i1.append(b), i2.append(c)

    for k in range(4):
        emit(C.OP_INPUT, k, 0, k)
    for k in range(steps):
        emit(C.OP_INPUT, 4 + k, 1, k)
    x = [0, 1, 2, 3]
    nxt = 4 + steps
    calls = []
    for k in range(steps):
        res = list(range(nxt, nxt + 4))
        calls.append((x + [4 + k], res))
        emit(C.OP_CALL, 0, k, 0)
        x, nxt = res, nxt + 4
    for k in range(4):
        emit(C.OP_OUTPUT, 0, x[k], k)
    tape = S.Tape(op, i0, i1, i2, np.zeros(len(op)), [4, steps], [4], nxt)
    return tape, calls


def call_rollout_serializable(steps):
    """The caller of :func:`call_rollout` with its expression graph (CallSX/OutputSX nodes of
    the step function) as the writer of oracle.serialize takes it, and the step function."""
    from oracle import serialize as SZ
    from casadi_gb300 import workloads as W
    step = W.cartpole_step()
    step_s = SZ.from_function(step)
    tape, calls = call_rollout(steps)
    x0, U = S.sym("x0", 4), S.sym("U", steps)
    x = list(x0)
    for k in range(steps):
        c = SZ.CallNode(step_s, x + [U[k]])
        x = [SZ.OutputNode(c, j) for j in range(4)]
    caller = SZ.Serializable("rollout_calls", tape, [x0, U], [x],
                             calls=[(step_s, d, r) for d, r in calls],
                             name_in=["x0", "U"], name_out=["xN"])
    return caller, step, calls
