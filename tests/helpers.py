"""Shared test helpers: fixture loading and the comparison rules used by the parity tests.

Tolerances:
  * EXACT_OPS and tapes built only from them (+,-,*,/,sqrt and the sign/compare/select ops):
    bit-exact (NaN == NaN, -0 and +0 distinguished only where the op defines the sign).
  * anything that calls a libm transcendental: |a-b| <= RTOL * max(|b|, floor) with
    RTOL = 1e-13, the tolerance the evaluator is held to against the CPU reference.
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


def assert_close(a, b, what="", rtol=RTOL, floor=None):
    """Relative check; `floor` (default: 1e-3 of the largest magnitude in b, at least 1e-300)
    keeps values that cancel to near zero from dominating."""
    b_arr = np.asarray(b, np.float64)
    if floor is None:
        fin = b_arr[np.isfinite(b_arr)]
        floor = max(1e-300, 1e-3 * float(np.abs(fin).max())) if fin.size else 1e-300
    e = rel_err(a, b, floor)
    assert e <= rtol, "%s: relative error %.3e > %.1e (floor %.3e)" % (what, e, rtol, floor)
    return e
