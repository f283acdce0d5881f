"""A scalar expression graph that produces CasADi SX virtual-machine tapes.

Tapes evaluated by this package normally come from CasADi itself (``SXFunction::algorithm_``
handed over by the ``"cuda"`` Map plugin). For tests, benchmarks and Python users without
libcasadi, this module rebuilds the same tapes:

* node creation with CasADi's on-the-fly simplification: ``SXElem::binary``/``unary``
  (casadi/core/sx_elem.cpp:189-262), ``common_simp_binary``/``common_simp_unary``
  (casadi/core/calculus.hpp:1812-2139), unary minus (sx_elem.cpp:150-161), constant folding
  (casadi/core/binary_sx.hpp:55-67, casadi/core/unary_sx.hpp:55-66) and value-cached
  constants (sx_elem.cpp:71-92, casadi/core/constant_sx.hpp:138-152);
* tape construction as ``SXFunction::init`` does it: depth-first topological sort
  (casadi/core/x_function.hpp:411-438), instruction emission (sx_function.cpp:522-687),
  LIFO live-variable slot reuse (sx_function.cpp:689-751) and input marking
  (sx_function.cpp:784-825).

The tape accessors of :class:`Function` mirror ``Function::n_instructions``,
``instruction_id``, ``instruction_input``, ``instruction_output`` and
``instruction_constant`` (casadi/core/function.hpp:1109-1151, sx_function.hpp:185-231).
"""
import math
import numpy as np

from . import calculus as C

EQ_DEPTH = 1  # SXNode::eq_depth_ (casadi/core/sx_node.cpp:232)


class SXElem:
    """One scalar node. ``op`` is an ``OP_*`` id; constants use OP_CONST and symbols
    OP_PARAMETER, as the reference's node classes report them."""
    __slots__ = ("op", "dep0", "dep1", "val", "name", "_kind", "__weakref__")

    # kinds: 'c' constant, 's' symbolic, 'u' unary, 'b' binary

    def __init__(self, kind, op, dep0=None, dep1=None, val=0.0, name=""):
        self._kind = kind
        self.op = op
        self.dep0 = dep0
        self.dep1 = dep1
        self.val = val
        self.name = name

    # ---- classification --------------------------------------------------------------
    def is_constant(self):
        return self._kind == "c"

    def is_symbolic(self):
        return self._kind == "s"

    def is_op(self, op):
        return self._kind in "ub" and self.op == op

    def n_dep(self):
        return {"c": 0, "s": 0, "u": 1, "b": 2}[self._kind]

    def dep(self, i=0):
        if self._kind == "u":
            return self.dep0
        return self.dep0 if i == 0 else self.dep1

    def is_zero(self):
        return self._kind == "c" and self.val == 0

    def is_one(self):
        return self._kind == "c" and self.val == 1

    def is_minus_one(self):
        return self._kind == "c" and self.val == -1

    def is_half(self):
        return self._kind == "c" and self.val == 0.5

    def is_inf(self):
        return self._kind == "c" and self.val == math.inf

    def is_minus_inf(self):
        return self._kind == "c" and self.val == -math.inf

    def is_integer(self):
        # IntegerSX and the 0/1/2/-1 singletons are integers, RealtypeSX is not
        return self._kind == "c" and math.isfinite(self.val) and self.val == int(self.val) \
            and -2**31 <= self.val < 2**31

    def to_int(self):
        return int(self.val)

    def is_nonnegative(self):
        # SXElem::is_nonnegative (sx_elem.cpp:318-326)
        if self._kind == "c":
            return self.val >= 0
        if self._kind == "u":
            return self.op in C.NONNEGATIVE_OPS
        return False

    def is_doubled(self):
        # SXElem::is_doubled (sx_elem.cpp:168-171)
        return (self.is_op(C.OP_ADD) and is_equal(self.dep0, self.dep1, EQ_DEPTH)) or \
            self.is_op(C.OP_TWICE)

    def __float__(self):
        if self._kind != "c":
            raise TypeError("symbolic SXElem has no numeric value")
        return self.val

    def __repr__(self):
        if self._kind == "c":
            return repr(self.val)
        if self._kind == "s":
            return self.name
        if self._kind == "u":
            return "%s(%r)" % (C.OP_NAMES[self.op].lower(), self.dep0)
        return "%s(%r, %r)" % (C.OP_NAMES[self.op].lower(), self.dep0, self.dep1)

    def __hash__(self):
        return id(self)

    # ---- operators (sx_elem.hpp / generic_expression.hpp) --------------------------------
    def __add__(self, o):
        return binary(C.OP_ADD, self, o)

    def __radd__(self, o):
        return binary(C.OP_ADD, o, self)

    def __sub__(self, o):
        return binary(C.OP_SUB, self, o)

    def __rsub__(self, o):
        return binary(C.OP_SUB, o, self)

    def __mul__(self, o):
        return binary(C.OP_MUL, self, o)

    def __rmul__(self, o):
        return binary(C.OP_MUL, o, self)

    def __truediv__(self, o):
        return binary(C.OP_DIV, self, o)

    def __rtruediv__(self, o):
        return binary(C.OP_DIV, o, self)

    def __pow__(self, o):
        return binary(C.OP_POW, self, o)

    def __rpow__(self, o):
        return binary(C.OP_POW, o, self)

    def __neg__(self):
        # SXElem::operator- (sx_elem.cpp:150-161)
        if self.is_op(C.OP_NEG):
            return self.dep0
        if self.is_zero():
            return const(0.0)
        if self.is_minus_one():
            return const(1.0)
        if self.is_one():
            return const(-1.0)
        return unary(C.OP_NEG, self)

    def __pos__(self):
        return self

    def __lt__(self, o):
        return binary(C.OP_LT, self, o)

    def __le__(self, o):
        return binary(C.OP_LE, self, o)

    def __gt__(self, o):
        return binary(C.OP_LT, o, self)

    def __ge__(self, o):
        return binary(C.OP_LE, o, self)

    def inv(self):
        return unary(C.OP_INV, self)


# ---- constants: cached by value (sx_elem.cpp:71-92, constant_sx.hpp:138-152) ----------------
_CONSTANTS = {}
_NAN = SXElem("c", C.OP_CONST, val=math.nan)


def const(v):
    v = float(v)
    if math.isnan(v):
        return _NAN
    if v == 0:
        v = 0.0  # IntegerSX(0): the zero singleton has a positive sign
    node = _CONSTANTS.get(v)
    if node is None:
        node = SXElem("c", C.OP_CONST, val=v)
        _CONSTANTS[v] = node
    return node


def _sx(x):
    return x if isinstance(x, SXElem) else const(x)


def sym(name, n=None):
    """A symbolic scalar (``n is None``) or a list of ``n`` symbolic scalars."""
    if n is None:
        return SXElem("s", C.OP_PARAMETER, name=name)
    return [SXElem("s", C.OP_PARAMETER, name="%s_%d" % (name, i)) for i in range(n)]


def is_equal(x, y, depth=0):
    """SXElem::is_equal (sx_elem.cpp:303-312) with the node overrides of
    binary_sx.hpp:90-100, unary_sx.hpp:85-88 and constant_sx.hpp:84-87."""
    x, y = _sx(x), _sx(y)
    if x is y:
        return True
    if depth <= 0:
        return False
    if x._kind == "c":
        return y._kind == "c" and y.val == x.val
    if x._kind == "u":
        return y._kind == "u" and y.op == x.op and is_equal(y.dep0, x.dep0, depth - 1)
    if x._kind == "b":
        if y._kind != "b" or y.op != x.op:
            return False
        if is_equal(y.dep0, x.dep0, depth - 1) and is_equal(y.dep1, x.dep1, depth - 1):
            return True
        return x.op in C.COMMUTATIVE_OPS and is_equal(y.dep1, x.dep0, depth - 1) \
            and is_equal(y.dep0, x.dep1, depth - 1)
    return False


def _create_binary(op, x, y):
    # BinarySX::create (binary_sx.hpp:55-67): fold constants
    if x.is_constant() and y.is_constant():
        return const(C.fun(op, x.val, y.val))
    return SXElem("b", op, x, y)


def _create_unary(op, x):
    # UnarySX::create (unary_sx.hpp:55-66)
    if x.is_constant():
        return const(C.fun(op, x.val, x.val))
    return SXElem("u", op, x)


def binary(op, x, y):
    """SXElem::binary (sx_elem.cpp:189-232)."""
    x, y = _sx(x), _sx(y)
    if y.is_op(C.OP_IF_ELSE_ZERO):
        if op == C.OP_MUL:
            return if_else_zero(y.dep0, x * y.dep1)
        if op == C.OP_ADD and x.is_op(C.OP_IF_ELSE_ZERO) and is_equal(x.dep0, y.dep0):
            return if_else_zero(y.dep0, x.dep1 + y.dep1)
    elif x.is_op(C.OP_IF_ELSE_ZERO) and op == C.OP_MUL:
        return if_else_zero(x.dep0, x.dep1 * y)
    hit, ret = _common_simp_binary(op, x, y, EQ_DEPTH)
    if hit:
        return _sx(ret)
    if op == C.OP_MUL:
        if x.is_constant() and y.is_op(C.OP_TWICE):
            return (x * 2) * y.dep0
        if y.is_constant() and x.is_op(C.OP_TWICE):
            return (2 * y) * x.dep0
    return _create_binary(op, x, y)


def unary(op, x):
    """SXElem::unary (sx_elem.cpp:239-262)."""
    x = _sx(x)
    if op == C.OP_NOT:
        if x.is_op(C.OP_NOT):
            return x.dep0
    elif op == C.OP_TWICE:
        if x.is_op(C.OP_MUL) and x.dep0.is_constant():
            return (2 * x.dep0) * x.dep1
        if x.is_op(C.OP_MUL) and x.dep1.is_constant():
            return (2 * x.dep1) * x.dep0
        if x.is_op(C.OP_TWICE):
            return 4 * x.dep0
    hit, ret = _common_simp_unary(op, x)
    if hit:
        return _sx(ret)
    return _create_unary(op, x)


def _common_simp_unary(op, x):
    """common_simp_unary (calculus.hpp:1812-1869)."""
    if op == C.OP_TWICE:
        if x.is_op(C.OP_MUL) and x.dep0.is_constant() and x.dep0.is_half():
            return True, x.dep1
        if x.is_op(C.OP_MUL) and x.dep1.is_constant() and x.dep1.is_half():
            return True, x.dep0
    elif op == C.OP_SQ:
        if x.is_op(C.OP_SQRT):
            return True, x.dep0
        if x.is_op(C.OP_NEG) or x.is_op(C.OP_FABS):
            return True, sq(x.dep0)
    elif op == C.OP_FABS:
        if x.is_nonnegative():
            return True, x
        if x.is_op(C.OP_NEG):
            return True, fabs(x.dep0)
    elif op == C.OP_LOG:
        if x.is_op(C.OP_EXP):
            return True, x.dep0
    elif op == C.OP_INV:
        if x.is_op(C.OP_INV):
            return True, x.dep0
    elif op == C.OP_SQRT:
        if x.is_op(C.OP_SQ):
            return True, fabs(x.dep0)
    elif op == C.OP_COS:
        if x.is_op(C.OP_NEG) or x.is_op(C.OP_FABS):
            return True, cos(x.dep0)
    elif op == C.OP_NEG:
        if x.is_op(C.OP_NEG):
            return True, x.dep0
    return False, None


def _common_simp_binary(op, x, y, depth):
    """common_simp_binary (calculus.hpp:1872-2139), with unique_x = unique_y = false."""
    eq = lambda a, b: is_equal(a, b, depth)  # noqa: E731
    if op == C.OP_ADD:
        if x.is_zero():
            return True, y
        if y.is_zero():
            return True, x
        if y.is_op(C.OP_NEG):
            return True, x - (-y)
        if x.is_op(C.OP_NEG):
            return True, y - x.dep0
        if eq(x, y):
            return True, 2 * x
        if x.is_op(C.OP_MUL) and y.is_op(C.OP_MUL) and x.dep0.is_constant() and \
                x.dep0.val == 0.5 and y.dep0.is_constant() and y.dep0.val == 0.5 and \
                eq(y.dep1, x.dep1):
            return True, x.dep1
        if x.is_op(C.OP_DIV) and y.is_op(C.OP_DIV) and x.dep1.is_constant() and \
                x.dep1.val == 2 and y.dep1.is_constant() and y.dep1.val == 2 and \
                eq(y.dep0, x.dep0):
            return True, x.dep0
        if x.is_op(C.OP_MUL) and y.is_op(C.OP_MUL) and x.dep0.is_constant() and \
                y.dep0.is_constant() and x.dep0.val + y.dep0.val == 1 and eq(y.dep1, x.dep1):
            return True, x.dep1
        if x.is_op(C.OP_SUB) and eq(x.dep1, y):
            return True, x.dep0
        if y.is_op(C.OP_SUB) and eq(x, y.dep1):
            return True, y.dep0
        if x.is_op(C.OP_SQ) and y.is_op(C.OP_SQ) and \
                ((x.dep0.is_op(C.OP_SIN) and y.dep0.is_op(C.OP_COS)) or
                 (x.dep0.is_op(C.OP_COS) and y.dep0.is_op(C.OP_SIN))) and \
                eq(x.dep0.dep0, y.dep0.dep0):
            return True, 1.0
        if x.is_doubled() and eq(x.dep0, y):
            return True, 3 * x.dep0
        if y.is_doubled() and eq(y.dep0, x):
            return True, 3 * y.dep0
        if x.is_op(C.OP_MUL) and y.is_op(C.OP_MUL) and eq(x.dep0, y.dep0) and \
                (x.dep1 + y.dep1).is_one():
            return True, x.dep0
    elif op == C.OP_SUB:
        if y.is_zero():
            return True, x
        if x.is_zero():
            return True, -y
        if eq(x, y):
            return True, 0.0
        if y.is_op(C.OP_NEG):
            return True, x + y.dep0
        if x.is_op(C.OP_ADD) and eq(x.dep1, y):
            return True, x.dep0
        if x.is_op(C.OP_ADD) and eq(x.dep0, y):
            return True, x.dep1
        if y.is_op(C.OP_ADD) and eq(x, y.dep1):
            return True, -y.dep0
        if y.is_op(C.OP_ADD) and eq(x, y.dep0):
            return True, -y.dep1
        if x.is_op(C.OP_NEG):
            return True, -(x.dep0 + y)
        if x.is_op(C.OP_MUL) and y.is_op(C.OP_MUL) and x.dep0.is_constant() and \
                y.dep0.is_constant() and x.dep0.val - y.dep0.val == 1 and eq(y.dep1, x.dep1):
            return True, x.dep1
        if x.is_doubled() and eq(x.dep0, y):
            return True, y
        if y.is_doubled() and eq(y.dep0, x):
            return True, -x
    elif op == C.OP_MUL:
        if eq(y, x):
            return True, sq(x)
        if not x.is_constant() and y.is_constant():
            return True, y * x
        if x.is_zero() or y.is_zero():
            return True, 0.0
        if x.is_one():
            return True, y
        if y.is_one():
            return True, x
        if y.is_minus_one():
            return True, -x
        if x.is_minus_one():
            return True, -y
        if y.is_op(C.OP_INV):
            return True, x / y.inv()
        if x.is_op(C.OP_INV):
            return True, y / x.inv()
        if x.is_constant() and y.is_op(C.OP_MUL) and y.dep0.is_constant() and \
                x.val * y.dep0.val == 1:
            return True, y.dep1
        if x.is_constant() and y.is_doubled() and x.val * 2 == 1:
            return True, y.dep0
        if x.is_constant() and y.is_op(C.OP_DIV) and y.dep1.is_constant() and \
                x.val == y.dep1.val:
            return True, y.dep0
        if x.is_constant() and x.val == 2:
            return True, unary(C.OP_TWICE, y)
        if y.is_constant() and y.val == 2:
            return True, unary(C.OP_TWICE, x)
        if x.is_op(C.OP_DIV) and eq(x.dep1, y):
            return True, x.dep0
        if y.is_op(C.OP_DIV) and eq(y.dep1, x):
            return True, y.dep0
        if x.is_op(C.OP_NEG):
            return True, -(x.dep0 * y)
        if y.is_op(C.OP_NEG):
            return True, -(x * y.dep0)
        # the (a +- b/c)*c rewrites need unique_x/unique_y, which are false here
        if x.is_constant() and y.is_op(C.OP_MUL) and y.dep0.is_constant():
            return True, x * y.dep0 * y.dep1
        if y.is_constant() and x.is_op(C.OP_MUL) and x.dep0.is_constant():
            return True, y * x.dep0 * x.dep1
    elif op == C.OP_DIV:
        if y.is_zero():
            return True, math.inf
        if x.is_zero():
            return True, 0.0
        if y.is_one():
            return True, x
        if y.is_minus_one():
            return True, -x
        if y.is_half():
            return True, 2 * x
        if eq(x, y):
            return True, 1.0
        if x.is_doubled() and y.is_constant() and y.val == 2:
            return True, x.dep0
        if x.is_doubled() and eq(y, x.dep0):
            return True, 2.0
        if x.is_op(C.OP_MUL) and eq(y, x.dep0):
            return True, x.dep1
        if x.is_op(C.OP_MUL) and eq(y, x.dep1):
            return True, x.dep0
        if x.is_one():
            return True, y.inv()
        if y.is_op(C.OP_INV):
            return True, x * y.inv()
        if x.is_doubled() and y.is_doubled():
            return True, x.dep0 / y.dep0
        if y.is_constant() and x.is_op(C.OP_DIV) and x.dep1.is_constant() and \
                y.val * x.dep1.val == 1:
            return True, x.dep0
        if y.is_op(C.OP_MUL) and eq(y.dep1, x):
            return True, 1 / y.dep0
        if y.is_doubled() and eq(y.dep0, x):
            return True, 0.5
        if x.is_op(C.OP_NEG) and eq(x.dep0, y):
            return True, -1.0
        if y.is_op(C.OP_NEG) and eq(y.dep0, x):
            return True, -1.0
        if y.is_op(C.OP_NEG) and x.is_op(C.OP_NEG) and eq(x.dep0, y.dep0):
            return True, 1.0
        if x.is_op(C.OP_DIV) and eq(y, x.dep0):
            return True, x.dep1.inv()
        if x.is_op(C.OP_NEG):
            return True, -(x.dep0 / y)
        if y.is_op(C.OP_NEG):
            return True, -(x / y.dep0)
    elif op == C.OP_POW:
        if y.is_constant():
            if y.is_integer():
                nn = y.to_int()
                if nn == 0:
                    return True, 1.0
                if nn > 100 or nn < -100:
                    return True, _create_binary(C.OP_CONSTPOW, x, const(nn))
                if nn < 0:
                    return True, 1 / power(x, -nn)
                if nn % 2 == 1:
                    return True, x * power(x, nn - 1)
                rt = power(x, nn // 2)
                return True, rt * rt
            if y.val == 0.5:
                return True, sqrt(x)
            return True, binary(C.OP_CONSTPOW, x, y)
    elif op == C.OP_LE:
        if (y - x).is_nonnegative():
            return True, 1.0
    elif op == C.OP_FMIN:
        if x.is_inf():
            return True, y
        if y.is_inf():
            return True, x
        if x.is_minus_inf() or y.is_minus_inf():
            return True, -math.inf
        if eq(x, y):
            return True, x
    elif op == C.OP_FMAX:
        if x.is_minus_inf():
            return True, y
        if y.is_minus_inf():
            return True, x
        if x.is_inf() or y.is_inf():
            return True, math.inf
        if eq(x, y):
            return True, x
    elif op == C.OP_LT:
        if (x - y).is_nonnegative():
            return True, 0.0
    elif op == C.OP_EQ:
        if eq(x, y):
            return True, 1.0
    elif op == C.OP_NE:
        if eq(x, y):
            return True, 0.0
    elif op == C.OP_IF_ELSE_ZERO:
        if y.is_zero():
            return True, y
        if x.is_constant():
            return True, (y if x.val != 0 else 0.0)
    return False, None


# ---- elementary functions ------------------------------------------------------------------
def _u(op):
    return lambda x: unary(op, x)


sqrt, exp, log, sq, twice = (_u(C.OP_SQRT), _u(C.OP_EXP), _u(C.OP_LOG), _u(C.OP_SQ),
                             _u(C.OP_TWICE))
sin, cos, tan, asin, acos, atan = (_u(C.OP_SIN), _u(C.OP_COS), _u(C.OP_TAN),
                                   _u(C.OP_ASIN), _u(C.OP_ACOS), _u(C.OP_ATAN))
sinh, cosh, tanh, asinh, acosh, atanh = (_u(C.OP_SINH), _u(C.OP_COSH), _u(C.OP_TANH),
                                         _u(C.OP_ASINH), _u(C.OP_ACOSH), _u(C.OP_ATANH))
floor, ceil, fabs, sign, erf, erfinv = (_u(C.OP_FLOOR), _u(C.OP_CEIL), _u(C.OP_FABS),
                                        _u(C.OP_SIGN), _u(C.OP_ERF), _u(C.OP_ERFINV))
log1p, expm1, logic_not = _u(C.OP_LOG1P), _u(C.OP_EXPM1), _u(C.OP_NOT)


def _b(op):
    return lambda x, y: binary(op, x, y)


fmin, fmax, atan2, hypot = _b(C.OP_FMIN), _b(C.OP_FMAX), _b(C.OP_ATAN2), _b(C.OP_HYPOT)
fmod, remainder, copysign = _b(C.OP_FMOD), _b(C.OP_REMAINDER), _b(C.OP_COPYSIGN)
if_else_zero, logic_and, logic_or = _b(C.OP_IF_ELSE_ZERO), _b(C.OP_AND), _b(C.OP_OR)
eq, ne, lt, le = _b(C.OP_EQ), _b(C.OP_NE), _b(C.OP_LT), _b(C.OP_LE)
constpow = _b(C.OP_CONSTPOW)


def power(x, n):
    return binary(C.OP_POW, x, n)


# ---- tape construction (SXFunction::init, sx_function.cpp:476-841) ------------------------
class Tape:
    """A flat SX tape: the fields of ``ScalarAtomic`` (sx_function.hpp:37-44) as arrays.

    For OP_CONST ``d`` holds the constant and ``i1``/``i2`` are unused (zero); for every
    other op ``d`` is zero. Unary ops carry ``i2 == i1`` (sx_function.cpp:746-750)."""

    def __init__(self, op, i0, i1, i2, d, nnz_in, nnz_out, sz_w):
        self.op = np.asarray(op, dtype=np.int32)
        self.i0 = np.asarray(i0, dtype=np.int32)
        self.i1 = np.asarray(i1, dtype=np.int32)
        self.i2 = np.asarray(i2, dtype=np.int32)
        self.d = np.asarray(d, dtype=np.float64)
        self.nnz_in = [int(v) for v in nnz_in]
        self.nnz_out = [int(v) for v in nnz_out]
        self.sz_w = int(sz_w)

    @property
    def n_instr(self):
        return int(self.op.size)

    def atomic_array(self):
        """The tape as a contiguous array with ScalarAtomic's 16-byte layout."""
        dt = np.dtype([("op", "<i4"), ("i0", "<i4"), ("u", "<u8")])
        a = np.zeros(self.n_instr, dtype=dt)
        a["op"] = self.op
        a["i0"] = self.i0
        ints = (self.i1.astype(np.uint32).astype(np.uint64)
                | (self.i2.astype(np.uint32).astype(np.uint64) << np.uint64(32)))
        dbits = self.d.view(np.uint64)
        a["u"] = np.where(self.op == C.OP_CONST, dbits, ints)
        return a

    @staticmethod
    def from_atomic_array(a, nnz_in, nnz_out, sz_w):
        """Inverse of :meth:`atomic_array`."""
        op = np.asarray(a["op"], np.int32)
        u = np.asarray(a["u"], np.uint64)
        is_c = op == C.OP_CONST
        i1 = np.where(is_c, 0, (u & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.int32))
        i2 = np.where(is_c, 0, (u >> np.uint64(32)).astype(np.uint32).view(np.int32))
        d = np.where(is_c, u.view(np.float64), 0.0)
        return Tape(op, np.asarray(a["i0"], np.int32), i1, i2, d, nnz_in, nnz_out, sz_w)

    def histogram(self):
        ops, counts = np.unique(self.op, return_counts=True)
        return {C.OP_NAMES.get(int(o), str(int(o))): int(c) for o, c in zip(ops, counts)}

    def save(self, path):
        np.savez_compressed(path, op=self.op, i0=self.i0, i1=self.i1, i2=self.i2, d=self.d,
                            nnz_in=np.asarray(self.nnz_in, np.int64),
                            nnz_out=np.asarray(self.nnz_out, np.int64),
                            sz_w=np.int64(self.sz_w))

    @staticmethod
    def load(path):
        z = np.load(path)
        return Tape(z["op"], z["i0"], z["i1"], z["i2"], z["d"], z["nnz_in"].tolist(),
                    z["nnz_out"].tolist(), int(z["sz_w"]))


class Function:
    """An SX function of vector inputs and outputs, compiled to a tape.

    ``inputs`` and ``outputs`` are lists of lists of scalars (each inner list is one
    dense column vector, i.e. the nonzeros of one input/output)."""

    def __init__(self, name, inputs, outputs, live_variables=True):
        self.name = name
        self.inputs = [list(v) for v in inputs]
        self.outputs = [[_sx(e) for e in v] for v in outputs]
        for v in self.inputs:
            for e in v:
                if not (isinstance(e, SXElem) and e.is_symbolic()):
                    raise ValueError("Function inputs must be purely symbolic")
        self.tape = _build_tape(self.inputs, self.outputs, live_variables)

    # mirrors of the reference's Function accessors
    def n_in(self):
        return len(self.inputs)

    def n_out(self):
        return len(self.outputs)

    def nnz_in(self, i=None):
        return sum(self.tape.nnz_in) if i is None else self.tape.nnz_in[i]

    def nnz_out(self, i=None):
        return sum(self.tape.nnz_out) if i is None else self.tape.nnz_out[i]

    def sz_w(self):
        return self.tape.sz_w

    def n_instructions(self):
        return self.tape.n_instr

    def instruction_id(self, k):
        return int(self.tape.op[k])

    def instruction_input(self, k):
        t, op = self.tape, int(self.tape.op[k])
        if C.ndeps(op) == 2 or op == C.OP_INPUT:
            return [int(t.i1[k]), int(t.i2[k])]
        if C.ndeps(op) == 1:
            return [int(t.i1[k])]
        return []

    def instruction_output(self, k):
        t = self.tape
        if int(t.op[k]) == C.OP_OUTPUT:
            return [int(t.i0[k]), int(t.i2[k])]
        return [int(t.i0[k])]

    def instruction_constant(self, k):
        return float(self.tape.d[k])


def _sorted_nodes(outputs):
    """Depth-first topological order of the nodes that the outputs depend on, with a None
    marker after each output nonzero (sort_depth_first, x_function.hpp:411-438)."""
    temp = {}  # node -> SXNode::temp during the sort
    nodes = []
    for vec in outputs:
        for e in vec:
            s = [e]
            while s:
                t = s[-1]
                tt = temp.get(t, 0)
                if tt >= 0:
                    temp[t] = tt + 1
                    if tt < t.n_dep():
                        s.append(t.dep(tt))
                    else:
                        nodes.append(t)
                        temp[t] = -1
                        s.pop()
                else:
                    s.pop()
            nodes.append(None)
    return nodes


def _build_tape(inputs, outputs, live_variables=True):
    temp = {}  # node -> SXNode::temp during the sort

    nodes = []
    for vec in outputs:
        for e in vec:
            # sort_depth_first (x_function.hpp:411-438)
            s = [e]
            while s:
                t = s[-1]
                tt = temp.get(t, 0)
                if tt >= 0:
                    temp[t] = tt + 1
                    if tt < t.n_dep():
                        s.append(t.dep(tt))
                    else:
                        nodes.append(t)
                        temp[t] = -1
                        s.pop()
                else:
                    s.pop()
            nodes.append(None)
    index = {}
    for i, n in enumerate(nodes):
        if n is not None:
            index[n] = i

    # instruction emission (sx_function.cpp:586-687)
    alg = []  # [op, i0, i1, i2, d]
    symb_loc = []
    refcount = [0] * len(nodes)
    out_pos = [(oi, nz) for oi, vec in enumerate(outputs) for nz in range(len(vec))]
    out_iter = iter(out_pos)
    for n in nodes:
        if n is None:
            oi, nz = next(out_iter)
            ae = [C.OP_OUTPUT, oi, index[outputs[oi][nz]], nz, 0.0]
            deps = [2]
        elif n.is_constant():
            ae = [C.OP_CONST, index[n], 0, 0, n.val]
            deps = []
        elif n.is_symbolic():
            symb_loc.append((len(alg), n))
            ae = [C.OP_PARAMETER, index[n], 0, 0, 0.0]
            deps = []
        elif n._kind == "u":
            ae = [n.op, index[n], index[n.dep0], index[n.dep0], 0.0]
            deps = [2]
        else:
            ae = [n.op, index[n], index[n.dep0], index[n.dep1], 0.0]
            deps = [2, 3]
        for c in deps:
            refcount[ae[c]] += 1
        alg.append(ae)

    # live-variable slot allocation (sx_function.cpp:689-751)
    place = [0] * len(nodes)
    unused = []
    worksize = 0
    for a in alg:
        op = a[0]
        nd = C.ndeps(op)
        dep_fields = [2, 3][:nd]
        for c in reversed(dep_fields):
            ch = a[c]
            refcount[ch] -= 1
            if refcount[ch] == 0:
                unused.append(place[ch])
        if op != C.OP_OUTPUT:
            r = a[1]
            if live_variables and unused:
                place[r] = unused.pop()
            else:
                place[r] = worksize
                worksize += 1
            a[1] = place[r]
        for c in dep_fields:
            a[c] = place[a[c]]
        if nd == 1 and op != C.OP_OUTPUT:
            a[3] = a[2]

    # input marking (sx_function.cpp:784-825)
    mark = {n: k + 1 for k, n in symb_loc}
    for ind, vec in enumerate(inputs):
        for nz, e in enumerate(vec):
            k = mark.get(e, 0) - 1
            if k >= 0:
                alg[k][0] = C.OP_INPUT
                alg[k][2] = ind
                alg[k][3] = nz
                mark[e] = 0
    free = [n.name for k, n in symb_loc if mark.get(n, 0) != 0]
    if free:
        raise ValueError("Initialization failed since variables %s are free" % free)

    arr = np.array([a[:4] for a in alg], dtype=np.int64).reshape(-1, 4)
    d = np.array([a[4] for a in alg], dtype=np.float64)
    return Tape(arr[:, 0], arr[:, 1], arr[:, 2], arr[:, 3], d,
                [len(v) for v in inputs], [len(v) for v in outputs], worksize)


# ---- symbolic reverse mode (SXFunction::ad_reverse, sx_function.cpp:1368-1569) ----------------
def _der_sx(op, x, y, f):
    """Symbolic partials (d0, d1) of op at operands x, y with result f, as
    BinaryOperation<OP>::der / UnaryOperation<OP>::der write them (calculus.hpp:598-1018)."""
    one, zero = const(1.0), const(0.0)
    if op in (C.OP_ASSIGN, C.OP_PRINTME, C.OP_LIFT):
        return one, zero
    if op == C.OP_ADD:
        return one, one
    if op == C.OP_SUB:
        return one, const(-1.0)
    if op == C.OP_MUL:
        return y, x
    if op == C.OP_DIV:
        return one / y, -f / y
    if op == C.OP_NEG:
        return const(-1.0), zero
    if op == C.OP_EXP:
        return f, zero
    if op == C.OP_LOG:
        return one / x, zero
    if op == C.OP_POW:
        return y * power(x, y - one), log(x) * f
    if op == C.OP_CONSTPOW:
        return y * power(x, y - one), zero
    if op == C.OP_SQRT:
        return one / twice(f), zero
    if op == C.OP_SQ:
        return twice(x), zero
    if op == C.OP_TWICE:
        return const(2.0), zero
    if op == C.OP_SIN:
        return cos(x), zero
    if op == C.OP_COS:
        return -sin(x), zero
    if op == C.OP_TAN:
        return one / sq(cos(x)), zero
    if op == C.OP_ASIN:
        return one / sqrt(one - x * x), zero
    if op == C.OP_ACOS:
        return const(-1.0) / sqrt(one - x * x), zero
    if op == C.OP_ATAN:
        return one / (one + x * x), zero
    if op in (C.OP_LT, C.OP_LE, C.OP_EQ, C.OP_NE, C.OP_AND, C.OP_OR):
        return zero, zero
    if op in (C.OP_FLOOR, C.OP_CEIL, C.OP_NOT, C.OP_SIGN):
        return zero, zero
    if op in (C.OP_FMOD, C.OP_REMAINDER):
        return one, (f - x) / y
    if op == C.OP_ERF:
        return const(2.0 / math.sqrt(math.pi)) * exp(-x * x), zero
    if op == C.OP_FABS:
        return sign(x), zero
    if op == C.OP_COPYSIGN:
        return copysign(one, y), zero
    if op == C.OP_FMIN:
        a, b = x <= y, y <= x
        c = a + b
        return a / c, b / c
    if op == C.OP_FMAX:
        a, b = y <= x, x <= y
        c = a + b
        return a / c, b / c
    if op == C.OP_INV:
        return (-f) * f, zero
    if op == C.OP_SINH:
        return cosh(x), zero
    if op == C.OP_COSH:
        return sinh(x), zero
    if op == C.OP_TANH:
        return one - f * f, zero
    if op == C.OP_ASINH:
        return one / sqrt(one + x * x), zero
    if op == C.OP_ACOSH:
        return one / sqrt(x - one) / sqrt(x + one), zero
    if op == C.OP_ATANH:
        return one / (one - x * x), zero
    if op == C.OP_ERFINV:
        return const(math.sqrt(math.pi) / 2) * exp(f * f), zero
    if op == C.OP_LOG1P:
        return one / (one + x), zero
    if op == C.OP_EXPM1:
        return exp(x), zero
    if op == C.OP_ATAN2:
        t = x * x + y * y
        return y / t, -x / t
    if op == C.OP_IF_ELSE_ZERO:
        return zero, x
    if op == C.OP_HYPOT:
        return x / f, y / f
    raise ValueError("no symbolic derivative for op %s" % C.OP_NAMES.get(op, op))


def reverse(f, aseed):
    """Adjoint sensitivity expressions of Function ``f`` for one adjoint direction:
    ``aseed[j]`` gives the seed of every nonzero of output j (numbers or SXElem; None for
    an unseeded output). Returns one list of SXElem per input. Follows SXFunction::ad_reverse:
    symbolic partials of every operation in tape order, then a reverse sweep in which each
    operation passes d0*seed and d1*seed to its operands (if_else_zero(d1, seed) for
    IF_ELSE_ZERO) and the simplification rules drop structural zeros."""
    outputs = f.outputs
    nodes = _sorted_nodes(outputs)
    der = {}
    for n in nodes:
        if n is None or n.is_constant() or n.is_symbolic():
            continue
        if n not in der:
            der[n] = _der_sx(n.op, n.dep0, n.dep1 if n._kind == "b" else n.dep0, n)
    zero = const(0.0)
    w = {}
    out_pos = [(oi, nz) for oi, vec in enumerate(outputs) for nz in range(len(vec))]
    k_out = len(out_pos)
    sens_of = {}
    for n in reversed(nodes):
        if n is None:
            k_out -= 1
            oi, nz = out_pos[k_out]
            s = aseed[oi]
            if s is None:
                continue
            node = outputs[oi][nz]
            w[node] = w.get(node, zero) + _sx(s[nz])
            continue
        if n.is_constant():
            w.pop(n, None)
            continue
        if n.is_symbolic():
            sens_of[n] = w.pop(n, zero)
            continue
        seed = w.pop(n, zero)
        d0, d1 = der[n]
        if n.op == C.OP_IF_ELSE_ZERO:
            w[n.dep1] = w.get(n.dep1, zero) + if_else_zero(d1, seed)
        elif n._kind == "b":
            w[n.dep0] = w.get(n.dep0, zero) + d0 * seed
            w[n.dep1] = w.get(n.dep1, zero) + d1 * seed
        else:
            w[n.dep0] = w.get(n.dep0, zero) + d0 * seed
    return [[sens_of.get(e, zero) for e in vec] for vec in f.inputs]


class _Helper:
    """Inputs and outputs of a temporary Function whose other symbols stay free (the
    reference's ``allow_free`` helper Functions)."""

    def __init__(self, inputs, outputs):
        self.inputs = [list(v) for v in inputs]
        self.outputs = [[_sx(e) for e in v] for v in outputs]


def gradient_expr(ex, arg):
    """Gradient expressions of the scalar ``ex`` with respect to the symbols ``arg``, built as
    the reference builds ``gradient(ex, arg)``: ``jtimes(ex, arg, 1, true)``
    (casadi/core/generic_matrix.hpp:1695-1704), i.e. one symbolic adjoint sweep of a
    temporary Function ``arg -> ex`` with free variables allowed (``SX::reverse``,
    casadi/core/sx_instantiator.cpp:1208-1230). The sweep's order, and with it the order of
    every adjoint sum, follows that temporary Function's tape."""
    return reverse(_Helper([list(arg)], [[ex]]), [[1.0]])[0]


def gradient(f, out, wrt):
    """Gradient expressions of the scalar output ``out`` of ``f`` with respect to input
    ``wrt``, as the reference's ``gradient(f_out, f_wrt)`` (:func:`gradient_expr`)."""
    if len(f.outputs[out]) != 1:
        raise ValueError("the gradient needs a scalar output")
    return gradient_expr(f.outputs[out][0], f.inputs[wrt])


def reverse_function(f):
    """The Function ``f.reverse(1)`` as the reference builds it (XFunction::get_reverse with
    SXFunction::ad_reverse, casadi/core/sx_function.cpp:1368-1569): inputs are f's inputs,
    one placeholder per output with no nonzeros (``out_*``), then one adjoint seed per output
    (``adj_*``); outputs are the adjoint sensitivities of f's inputs. Evaluating its tape
    with the value sweep gives the reference's adjoint results operation for operation."""
    adj = [sym("adj_o%d" % j, len(v)) for j, v in enumerate(f.outputs)]
    sens = reverse(f, adj)
    return Function("adj1_" + f.name, f.inputs + [[] for _ in f.outputs] + adj, sens)
