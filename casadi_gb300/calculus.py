"""Scalar operation table of CasADi's SX virtual machine.

The operation ids are CasADi's ``enum Operation`` (casadi/core/calculus.hpp:60-218);
a tape produced by CasADi's ``SXFunction`` (``algorithm_``, casadi/core/sx_function.hpp:245)
carries these ids, so they are an interface and must keep the reference numbering.

``fun`` restates ``casadi_math<double>::fun`` (calculus.hpp:1299-1360) on Python floats.
It is used only for constant folding while building tapes
(``BinarySX::create``/``UnarySX::create``, casadi/core/binary_sx.hpp:55-67,
casadi/core/unary_sx.hpp:55-66); Python's ``math`` module calls the platform libm,
as ``std::`` does in the reference (calculus.hpp:229-263).
"""
import math

import numpy as np

# --- enum Operation (calculus.hpp:60-218), numbering is the interface ---------------------
OP_ASSIGN = 0
OP_ADD, OP_SUB, OP_MUL, OP_DIV = 1, 2, 3, 4
OP_NEG, OP_EXP, OP_LOG, OP_POW, OP_CONSTPOW = 5, 6, 7, 8, 9
OP_SQRT, OP_SQ, OP_TWICE = 10, 11, 12
OP_SIN, OP_COS, OP_TAN = 13, 14, 15
OP_ASIN, OP_ACOS, OP_ATAN = 16, 17, 18
OP_LT, OP_LE, OP_EQ, OP_NE, OP_NOT, OP_AND, OP_OR = 19, 20, 21, 22, 23, 24, 25
OP_FLOOR, OP_CEIL, OP_FMOD, OP_FABS, OP_SIGN, OP_COPYSIGN, OP_IF_ELSE_ZERO = (
    26, 27, 28, 29, 30, 31, 32)
OP_ERF, OP_FMIN, OP_FMAX = 33, 34, 35
OP_INV = 36
OP_SINH, OP_COSH, OP_TANH = 37, 38, 39
OP_ASINH, OP_ACOSH, OP_ATANH = 40, 41, 42
OP_ATAN2 = 43
OP_CONST = 44
OP_INPUT, OP_OUTPUT = 45, 46
OP_PARAMETER = 47
OP_CALL = 48
OP_ERFINV = 86
OP_PRINTME = 87
OP_LIFT = 88
OP_LOG1P = 93
OP_EXPM1 = 94
OP_HYPOT = 95
OP_REMAINDER = 97

OP_NAMES = {
    OP_ASSIGN: "ASSIGN", OP_ADD: "ADD", OP_SUB: "SUB", OP_MUL: "MUL", OP_DIV: "DIV",
    OP_NEG: "NEG", OP_EXP: "EXP", OP_LOG: "LOG", OP_POW: "POW", OP_CONSTPOW: "CONSTPOW",
    OP_SQRT: "SQRT", OP_SQ: "SQ", OP_TWICE: "TWICE", OP_SIN: "SIN", OP_COS: "COS",
    OP_TAN: "TAN", OP_ASIN: "ASIN", OP_ACOS: "ACOS", OP_ATAN: "ATAN", OP_LT: "LT",
    OP_LE: "LE", OP_EQ: "EQ", OP_NE: "NE", OP_NOT: "NOT", OP_AND: "AND", OP_OR: "OR",
    OP_FLOOR: "FLOOR", OP_CEIL: "CEIL", OP_FMOD: "FMOD", OP_FABS: "FABS", OP_SIGN: "SIGN",
    OP_COPYSIGN: "COPYSIGN", OP_IF_ELSE_ZERO: "IF_ELSE_ZERO", OP_ERF: "ERF",
    OP_FMIN: "FMIN", OP_FMAX: "FMAX", OP_INV: "INV", OP_SINH: "SINH", OP_COSH: "COSH",
    OP_TANH: "TANH", OP_ASINH: "ASINH", OP_ACOSH: "ACOSH", OP_ATANH: "ATANH",
    OP_ATAN2: "ATAN2", OP_CONST: "CONST", OP_INPUT: "INPUT", OP_OUTPUT: "OUTPUT",
    OP_PARAMETER: "PARAMETER", OP_CALL: "CALL", OP_ERFINV: "ERFINV",
    OP_PRINTME: "PRINTME", OP_LIFT: "LIFT", OP_LOG1P: "LOG1P", OP_EXPM1: "EXPM1",
    OP_HYPOT: "HYPOT", OP_REMAINDER: "REMAINDER",
}

# CASADI_MATH_BINARY_BUILTIN + OP_IF_ELSE_ZERO (calculus.hpp:1507-1528, 1612-1620)
BINARY_OPS = frozenset([
    OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW, OP_CONSTPOW, OP_LT, OP_LE, OP_EQ, OP_NE,
    OP_AND, OP_OR, OP_COPYSIGN, OP_FMOD, OP_REMAINDER, OP_FMIN, OP_FMAX, OP_ATAN2,
    OP_PRINTME, OP_LIFT, OP_HYPOT, OP_IF_ELSE_ZERO])

# CASADI_MATH_UNARY_BUILTIN (calculus.hpp:1530-1559)
UNARY_OPS = frozenset([
    OP_ASSIGN, OP_NEG, OP_EXP, OP_LOG, OP_SQRT, OP_SQ, OP_TWICE, OP_SIN, OP_COS, OP_TAN,
    OP_ASIN, OP_ACOS, OP_ATAN, OP_FLOOR, OP_CEIL, OP_NOT, OP_ERF, OP_FABS, OP_SIGN,
    OP_INV, OP_SINH, OP_COSH, OP_TANH, OP_ASINH, OP_ACOSH, OP_ATANH, OP_ERFINV,
    OP_LOG1P, OP_EXPM1])

# Every scalar op the numeric VM evaluates (CASADI_MATH_FUN_BUILTIN, calculus.hpp:1302-1353)
ARITH_OPS = BINARY_OPS | UNARY_OPS

# CommChecker (calculus.hpp:548-557)
COMMUTATIVE_OPS = frozenset([OP_ADD, OP_MUL, OP_EQ, OP_NE, OP_AND, OP_OR, OP_HYPOT])

# NonnegativeChecker (calculus.hpp:560-575), consulted only for unary ops and constants
NONNEGATIVE_OPS = frozenset([OP_SQRT, OP_SQ, OP_EXP, OP_LT, OP_LE, OP_EQ, OP_NE, OP_NOT,
                             OP_AND, OP_OR, OP_HYPOT, OP_FABS])


def ndeps(op):
    """casadi_math<T>::ndeps (calculus.hpp:1632-1647)."""
    if op in (OP_CONST, OP_PARAMETER, OP_INPUT):
        return 0
    if op in BINARY_OPS:
        return 2
    if op == OP_CALL:
        return -1
    return 1


def _sign(x):
    # calculus.hpp:270: x<0 ? -1 : x>0 ? 1 : x  (sign(nan) == nan)
    return -1.0 if x < 0 else (1.0 if x > 0 else x)


def _truth(x):
    # C++ conversion of a double to bool: nonzero (NaN included) is true
    return x != 0 or math.isnan(x)


def _erfinv(x):
    """The reference's own erfinv approximation (calculus.hpp:297-328): a rational
    start value followed by two Newton polishing steps. Used when the C library has
    no ``erfinv`` (glibc has none)."""
    if x >= 1:
        return math.inf if x == 1 else math.nan
    if x <= -1:
        return -math.inf if x == -1 else math.nan
    if x < -0.7:
        z = math.sqrt(-math.log((1.0 + x) / 2.0))
        return -(((1.641345311 * z + 3.429567803) * z - 1.624906493) * z - 1.970840454) / \
            ((1.637067800 * z + 3.543889200) * z + 1.0)
    if x < 0.7:
        z = x * x
        y = x * (((-0.140543331 * z + 0.914624893) * z - 1.645349621) * z + 0.886226899) / \
            ((((-0.329097515 * z + 0.012229801) * z + 1.442710462) * z - 2.118377725) * z + 1.0)
    else:
        z = math.sqrt(-math.log((1.0 - x) / 2.0))
        y = (((1.641345311 * z + 3.429567803) * z - 1.624906493) * z - 1.970840454) / \
            ((1.637067800 * z + 3.543889200) * z + 1.0)
    two_over_sqrt_pi = 2.0 / math.sqrt(math.pi)
    y = y - (math.erf(y) - x) / (two_over_sqrt_pi * math.exp(-y * y))
    y = y - (math.erf(y) - x) / (two_over_sqrt_pi * math.exp(-y * y))
    return y


def _safe(f):
    def g(*a):
        try:
            return f(*a)
        except (ValueError, ZeroDivisionError):
            return math.nan
        except OverflowError:
            return math.inf
    return g


def _div(x, y):
    if y == 0:
        if x == 0 or math.isnan(x):
            return math.nan
        return math.copysign(math.inf, x) * math.copysign(1.0, y)
    return x / y


def _pow(x, y):
    if x == 0 and y < 0:
        # C pow: +-inf for odd integer y (sign of x), +inf otherwise
        odd = float(y).is_integer() and abs(y) < 2**53 and int(y) % 2 == 1
        return math.copysign(math.inf, x) if odd else math.inf
    try:
        return math.pow(x, y)
    except ValueError:
        return math.nan
    except OverflowError:
        return math.inf if x > 0 or float(y).is_integer() and int(y) % 2 == 0 else -math.inf
    except ZeroDivisionError:
        return math.inf


def _fmin(x, y):
    if math.isnan(x):
        return y
    if math.isnan(y):
        return x
    return x if x <= y else y


def _fmax(x, y):
    if math.isnan(x):
        return y
    if math.isnan(y):
        return x
    return x if x >= y else y


_FUN = {
    OP_ASSIGN: lambda x, y: x,
    OP_ADD: lambda x, y: x + y,
    OP_SUB: lambda x, y: x - y,
    OP_MUL: lambda x, y: x * y,
    OP_DIV: _div,
    OP_NEG: lambda x, y: -x,
    OP_EXP: _safe(lambda x, y=None: math.exp(x)),
    OP_LOG: lambda x, y: (-math.inf if x == 0 else _safe(math.log)(x)),
    OP_POW: _pow,
    OP_CONSTPOW: _pow,
    OP_SQRT: _safe(lambda x, y=None: math.sqrt(x)),
    OP_SQ: lambda x, y: x * x,
    OP_TWICE: lambda x, y: 2.0 * x,
    OP_SIN: _safe(lambda x, y=None: math.sin(x)),
    OP_COS: _safe(lambda x, y=None: math.cos(x)),
    OP_TAN: _safe(lambda x, y=None: math.tan(x)),
    OP_ASIN: _safe(lambda x, y=None: math.asin(x)),
    OP_ACOS: _safe(lambda x, y=None: math.acos(x)),
    OP_ATAN: lambda x, y: math.atan(x),
    OP_LT: lambda x, y: float(x < y),
    OP_LE: lambda x, y: float(x <= y),
    OP_EQ: lambda x, y: float(x == y),
    OP_NE: lambda x, y: float(x != y),
    OP_NOT: lambda x, y: float(not _truth(x)),
    OP_AND: lambda x, y: float(_truth(x) and _truth(y)),
    OP_OR: lambda x, y: float(_truth(x) or _truth(y)),
    OP_FLOOR: lambda x, y: float(np.floor(np.float64(x))),
    OP_CEIL: lambda x, y: float(np.ceil(np.float64(x))),
    OP_FMOD: _safe(math.fmod),
    OP_REMAINDER: _safe(math.remainder),
    OP_FABS: lambda x, y: math.fabs(x),
    OP_SIGN: lambda x, y: _sign(x),
    OP_COPYSIGN: lambda x, y: math.copysign(x, y),
    OP_IF_ELSE_ZERO: lambda x, y: (0.0 if x == 0 else y),
    OP_ERF: lambda x, y: math.erf(x),
    OP_FMIN: _fmin,
    OP_FMAX: _fmax,
    OP_INV: lambda x, y: _div(1.0, x),
    OP_SINH: lambda x, y: (math.copysign(math.inf, x) if abs(x) > 710.5
                           else math.sinh(x)),
    OP_COSH: _safe(lambda x, y=None: math.cosh(x)),
    OP_TANH: lambda x, y: math.tanh(x),
    OP_ASINH: lambda x, y: math.asinh(x),
    OP_ACOSH: _safe(lambda x, y=None: math.acosh(x)),
    OP_ATANH: lambda x, y: (math.copysign(math.inf, x) if abs(x) == 1
                            else _safe(lambda v: math.atanh(v))(x)),
    OP_ATAN2: lambda x, y: math.atan2(x, y),
    OP_ERFINV: lambda x, y: _erfinv(x),
    OP_PRINTME: lambda x, y: x,
    OP_LIFT: lambda x, y: x,
    OP_LOG1P: _safe(lambda x, y=None: (-math.inf if x == -1 else math.log1p(x))),
    OP_EXPM1: _safe(lambda x, y=None: math.expm1(x)),
    OP_HYPOT: lambda x, y: math.hypot(x, y),
}


def fun(op, x, y):
    """Evaluate one scalar op on doubles (constant folding only)."""
    return float(_FUN[op](float(x), float(y)))
