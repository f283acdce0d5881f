// Scalar op semantics of CasADi's SX virtual machine on sm_103a, in FP64.
//
// Values follow casadi_math<double>::fun (casadi/core/calculus.hpp:598-1018 and the dispatch
// macro :1302-1355); partial derivatives follow BinaryOperation<OP>::der with the same
// operation order (calculus.hpp:598-1018, dispatch :1388-1439). Every arithmetic step is an
// explicitly rounded intrinsic (__dadd_rn, __dmul_rn, ...): nothing is contracted into an
// FMA, so +,-,*,/,sqrt tapes reproduce the CPU reference bit for bit. Transcendentals call
// CUDA's own double-precision functions.
//
// NEG, FABS, SIGN and COPYSIGN act on the sign bit with integer instructions: bit-identical
// to the FP64 forms and they keep the FP64 pipe (the scarce unit on GB300) free.
#pragma once
#include <cstdint>
#include <math_constants.h>

namespace cgb {

typedef unsigned long long u64;

// Device opcodes: CasADi's enum Operation ids 0..46 unchanged (ASSIGN..OUTPUT), the
// scalar ops numbered above OP_CALL remapped into 47..53 so an opcode fits in 6 bits.
enum DevOp : unsigned {
  D_ASSIGN = 0, D_ADD, D_SUB, D_MUL, D_DIV, D_NEG, D_EXP, D_LOG, D_POW, D_CONSTPOW,
  D_SQRT, D_SQ, D_TWICE, D_SIN, D_COS, D_TAN, D_ASIN, D_ACOS, D_ATAN, D_LT, D_LE, D_EQ,
  D_NE, D_NOT, D_AND, D_OR, D_FLOOR, D_CEIL, D_FMOD, D_FABS, D_SIGN, D_COPYSIGN,
  D_IF_ELSE_ZERO, D_ERF, D_FMIN, D_FMAX, D_INV, D_SINH, D_COSH, D_TANH, D_ASINH, D_ACOSH,
  D_ATANH, D_ATAN2, D_CONST, D_INPUT, D_OUTPUT,
  D_ERFINV = 47, D_PRINTME, D_LIFT, D_LOG1P, D_EXPM1, D_HYPOT, D_REMAINDER,
  D_NOP = 63
};

// 64-bit instruction word: op in bits 0-5, three 18-bit fields a (bits 6-23), b (24-41),
// c (42-59), then the op's recorded-partial mask (bits 60-61, see partial_mask) and a
// binary-op flag (bit 62), so the AD sweeps read both without a lookup.
//   arithmetic: a = result slot, b, c = operand slots (c == b for unary ops)
//   CONST:      a = slot, b = index into the constant pool
//   INPUT:      a = slot, b = input index, c = nonzero
//   OUTPUT:     a = output index, b = slot, c = nonzero
constexpr unsigned kFieldBits = 18;
constexpr unsigned kFieldMax = (1u << kFieldBits) - 1;

__host__ __device__ __forceinline__ unsigned dec_op(u64 w) { return (unsigned)(w & 63u); }
__host__ __device__ __forceinline__ unsigned dec_a(u64 w) { return (unsigned)(w >> 6) & kFieldMax; }
__host__ __device__ __forceinline__ unsigned dec_b(u64 w) { return (unsigned)(w >> 24) & kFieldMax; }
__host__ __device__ __forceinline__ unsigned dec_c(u64 w) { return (unsigned)(w >> 42) & kFieldMax; }
__host__ __device__ __forceinline__ unsigned dec_pmask(u64 w) { return (unsigned)(w >> 60) & 3u; }
__host__ __device__ __forceinline__ bool dec_binary(u64 w) { return (w >> 62) & 1u; }
// Bit 63: a SIN or COS whose sin/cos pair the previous SIN/COS of the same operand value
// computed (the sweeps take it again); bit 62 on a SIN or COS (unary ops leave it clear): the
// first of such a pair, which the value sweeps then compute as one sincos (see
// mark_sincos_pairs).
constexpr u64 kSincosReuse = 1ull << 63;
constexpr u64 kSincosFirst = 1ull << 62;

// Partials an instruction records for the AD sweeps: bit 0 = d0, bit 1 = d1.
// Ops whose partials are constants (ADD, SUB, NEG, TWICE, ASSIGN, comparisons, ...) record
// nothing; kConstD0/kConstD1 give their values.
__host__ __device__ __forceinline__ unsigned partial_mask(unsigned op) {
  switch (op) {
    case D_MUL: case D_DIV: case D_POW: case D_ATAN2: case D_HYPOT: case D_FMIN: case D_FMAX:
      return 3u;
    case D_FMOD: case D_REMAINDER: case D_IF_ELSE_ZERO:
      return 2u;
    case D_CONSTPOW: case D_COPYSIGN:
    case D_EXP: case D_LOG: case D_SQRT: case D_SQ: case D_SIN: case D_COS: case D_TAN:
    case D_ASIN: case D_ACOS: case D_ATAN: case D_FABS: case D_ERF: case D_INV: case D_SINH:
    case D_COSH: case D_TANH: case D_ASINH: case D_ACOSH: case D_ATANH: case D_ERFINV:
    case D_LOG1P: case D_EXPM1:
      return 1u;
    default:
      return 0u;
  }
}

__host__ __device__ __forceinline__ bool is_binary(unsigned op) {
  switch (op) {
    case D_ADD: case D_SUB: case D_MUL: case D_DIV: case D_POW: case D_CONSTPOW: case D_LT:
    case D_LE: case D_EQ: case D_NE: case D_AND: case D_OR: case D_COPYSIGN: case D_FMOD:
    case D_REMAINDER: case D_FMIN: case D_FMAX: case D_ATAN2: case D_PRINTME: case D_LIFT:
    case D_HYPOT: case D_IF_ELSE_ZERO:
      return true;
    default:
      return false;
  }
}

// Constant partials of the ops that record none (calculus.hpp:640-1018).
__host__ __device__ __forceinline__ double const_d0(unsigned op) {
  switch (op) {
    case D_ASSIGN: case D_ADD: case D_SUB: case D_PRINTME: case D_LIFT: case D_FMOD:
    case D_REMAINDER:
      return 1.0;
    case D_NEG: return -1.0;
    case D_TWICE: return 2.0;
    default: return 0.0;
  }
}
__host__ __device__ __forceinline__ double const_d1(unsigned op) {
  switch (op) {
    case D_ADD: return 1.0;
    case D_SUB: return -1.0;
    default: return 0.0;
  }
}

__host__ __device__ __forceinline__ u64 enc(unsigned op, unsigned a, unsigned b, unsigned c) {
  return (u64)op | ((u64)a << 6) | ((u64)b << 24) | ((u64)c << 42) |
         ((u64)partial_mask(op) << 60) | ((u64)(is_binary(op) ? 1u : 0u) << 62);
}

// Whether an operand's partial is not the constant zero (it can carry a derivative).
__host__ __device__ __forceinline__ bool carries_d0(unsigned op) {
  return (partial_mask(op) & 1u) || const_d0(op) != 0.0;
}
__host__ __device__ __forceinline__ bool carries_d1(unsigned op) {
  return is_binary(op) && ((partial_mask(op) & 2u) || const_d1(op) != 0.0);
}

// Activity analysis (SXFunction::eval_activity, casadi/core/sx_function.cpp:1684-1718): a
// result is inactive (0) only when the op is known to give zero for its zero operands, else
// active (all bits set). One bit per device opcode, from the reference's zero checkers
// (calculus.hpp:485-540):
//   kZeroFirst   f(0, y) == 0 for every y (F0XChecker)
//   kZeroSecond  f(x, 0) == 0 for every x (FX0Checker)
//   kZeroBoth    f(0, 0) == 0 (F00Checker: either of the above, or ADD SUB FMIN FMAX AND OR
//                COPYSIGN LT HYPOT)
constexpr u64 op_bit(unsigned op) { return 1ull << op; }
constexpr u64 kZeroFirst =
    op_bit(D_ASSIGN) | op_bit(D_MUL) | op_bit(D_DIV) | op_bit(D_NEG) | op_bit(D_SQRT) |
    op_bit(D_SQ) | op_bit(D_TWICE) | op_bit(D_SIN) | op_bit(D_TAN) | op_bit(D_ATAN) |
    op_bit(D_ASIN) | op_bit(D_FLOOR) | op_bit(D_CEIL) | op_bit(D_FMOD) | op_bit(D_REMAINDER) |
    op_bit(D_FABS) | op_bit(D_SIGN) | op_bit(D_COPYSIGN) | op_bit(D_ERF) | op_bit(D_SINH) |
    op_bit(D_TANH) | op_bit(D_ASINH) | op_bit(D_ATANH) | op_bit(D_ERFINV) | op_bit(D_AND) |
    op_bit(D_IF_ELSE_ZERO) | op_bit(D_LOG1P) | op_bit(D_EXPM1);
constexpr u64 kZeroSecond = op_bit(D_MUL) | op_bit(D_AND) | op_bit(D_IF_ELSE_ZERO);
constexpr u64 kZeroBoth = kZeroFirst | kZeroSecond | op_bit(D_ADD) | op_bit(D_SUB) |
                          op_bit(D_FMIN) | op_bit(D_FMAX) | op_bit(D_OR) | op_bit(D_COPYSIGN) |
                          op_bit(D_LT) | op_bit(D_HYPOT);

// Activity of an arithmetic result from its operands' activity words x (first) and y (second;
// ignored for unary ops).
__host__ __device__ __forceinline__ u64 activity_of(unsigned op, bool binary, u64 x, u64 y) {
  u64 zero_if;
  if (!binary) {
    if (x) return ~0ull;
    zero_if = kZeroFirst;
  } else if (x && y) {
    return ~0ull;
  } else {
    zero_if = x ? kZeroSecond : y ? kZeroFirst : kZeroBoth;
  }
  return ((zero_if >> op) & 1ull) ? 0ull : ~0ull;
}

#ifdef __CUDACC__
constexpr unsigned long long kSignBit = 0x8000000000000000ull;

__device__ __forceinline__ double d_neg(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)kSignBit);
}
// 2*x: for a normal x whose double stays finite (exponent field 1..2045) the exponent field
// is incremented with an integer add, which is exactly 2*x; zeros, subnormals, the largest
// binade, inf and NaN go through the FP64 add. Identical to __dadd_rn(x, x) in every case;
// keeps the FP64 pipe free for the common case.
__device__ __forceinline__ double d_twice(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned e = static_cast<unsigned>((b >> 52) & 0x7ff);
  if (e - 1u < 2045u) return __longlong_as_double(b + (1ll << 52));
  return __dadd_rn(x, x);
}
__device__ __forceinline__ double d_fabs(double x) {
  return __longlong_as_double(__double_as_longlong(x) & (long long)~kSignBit);
}
// x == 0.0 (either sign) on the bit pattern, without an FP64 comparison
__device__ __forceinline__ bool d_iszero(double x) {
  return (__double_as_longlong(x) & (long long)~kSignBit) == 0;
}
__device__ __forceinline__ bool d_isnan(double x) {
  return (__double_as_longlong(x) & (long long)~kSignBit) > 0x7ff0000000000000ll;
}
// sign(x) = x<0 ? -1 : x>0 ? 1 : x (calculus.hpp:270), on the bit pattern
__device__ __forceinline__ double d_sign(double x) {
  long long b = __double_as_longlong(x);
  long long m = b & (long long)~kSignBit;
  if (m == 0 || m > 0x7ff0000000000000ll) return x;  // +-0 and NaN
  return b < 0 ? -1.0 : 1.0;
}
__device__ __forceinline__ double d_copysign(double x, double y) {
  long long bx = __double_as_longlong(x) & (long long)~kSignBit;
  long long sy = __double_as_longlong(y) & (long long)kSignBit;
  return __longlong_as_double(bx | sy);
}
// fmin/fmax: NaN operand yields the other; ties (+0/-0 included) yield the first operand,
// as the x86-64 reference build resolves std::fmin/fmax.
__device__ __forceinline__ double d_fmin(double x, double y) {
  if (d_isnan(x)) return y;
  if (d_isnan(y)) return x;
  return y < x ? y : x;
}
__device__ __forceinline__ double d_fmax(double x, double y) {
  if (d_isnan(x)) return y;
  if (d_isnan(y)) return x;
  return y > x ? y : x;
}

// The reference's erfinv (calculus.hpp:297-328; glibc provides none): rational start value,
// then two Newton steps. Same constants and operation order, no contraction.
static __device__ __noinline__ double d_erfinv(double x) {
  if (x >= 1) return x == 1 ? CUDART_INF : CUDART_NAN;
  if (x <= -1) return x == -1 ? -CUDART_INF : CUDART_NAN;
  if (x < -0.7) {
    double z = __dsqrt_rn(d_neg(log(__ddiv_rn(__dadd_rn(1.0, x), 2.0))));
    double num = __dsub_rn(__dmul_rn(__dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(1.641345311, z),
                 3.429567803), z), 1.624906493), z), 1.970840454);
    double den = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(1.637067800, z), 3.543889200), z), 1.0);
    return d_neg(__ddiv_rn(num, den));
  }
  double y;
  if (x < 0.7) {
    double z = __dmul_rn(x, x);
    double num = __dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(-0.140543331, z),
                 0.914624893), z), 1.645349621), z), 0.886226899);
    double den = __dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(__dadd_rn(
                 __dmul_rn(-0.329097515, z), 0.012229801), z), 1.442710462), z), 2.118377725),
                 z), 1.0);
    y = __ddiv_rn(__dmul_rn(x, num), den);
  } else {
    double z = __dsqrt_rn(d_neg(log(__ddiv_rn(__dsub_rn(1.0, x), 2.0))));
    double num = __dsub_rn(__dmul_rn(__dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(1.641345311, z),
                 3.429567803), z), 1.624906493), z), 1.970840454);
    double den = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(1.637067800, z), 3.543889200), z), 1.0);
    y = __ddiv_rn(num, den);
  }
  const double k = __ddiv_rn(2.0, __dsqrt_rn(CUDART_PI));
  y = __dsub_rn(y, __ddiv_rn(__dsub_rn(erf(y), x), __dmul_rn(k, exp(d_neg(__dmul_rn(y, y))))));
  y = __dsub_rn(y, __ddiv_rn(__dsub_rn(erf(y), x), __dmul_rn(k, exp(d_neg(__dmul_rn(y, y))))));
  return y;
}

// Value of an arithmetic op (CASADI_MATH_FUN_BUILTIN).
__device__ __forceinline__ double dev_fun(unsigned op, double x, double y) {
  switch (op) {
    case D_ASSIGN: return x;
    case D_ADD: return __dadd_rn(x, y);
    case D_SUB: return __dsub_rn(x, y);
    case D_MUL: return __dmul_rn(x, y);
    case D_DIV: return __ddiv_rn(x, y);
    case D_NEG: return d_neg(x);
    case D_EXP: return exp(x);
    case D_LOG: return log(x);
    case D_POW: case D_CONSTPOW: return pow(x, y);
    case D_SQRT: return __dsqrt_rn(x);
    case D_SQ: return __dmul_rn(x, x);
    case D_TWICE: return d_twice(x);  // == 2.*x exactly
    case D_SIN: return sin(x);
    case D_COS: return cos(x);
    case D_TAN: return tan(x);
    case D_ASIN: return asin(x);
    case D_ACOS: return acos(x);
    case D_ATAN: return atan(x);
    case D_LT: return x < y ? 1.0 : 0.0;
    case D_LE: return x <= y ? 1.0 : 0.0;
    case D_EQ: return x == y ? 1.0 : 0.0;
    case D_NE: return x != y ? 1.0 : 0.0;
    case D_NOT: return x == 0.0 ? 1.0 : 0.0;
    case D_AND: return (x != 0.0 && y != 0.0) ? 1.0 : 0.0;
    case D_OR: return (x != 0.0 || y != 0.0) ? 1.0 : 0.0;
    case D_FLOOR: return floor(x);
    case D_CEIL: return ceil(x);
    case D_FMOD: return fmod(x, y);
    case D_REMAINDER: return remainder(x, y);
    case D_FABS: return d_fabs(x);
    case D_SIGN: return d_sign(x);
    case D_COPYSIGN: return d_copysign(x, y);
    case D_IF_ELSE_ZERO: return x == 0.0 ? 0.0 : y;
    case D_ERF: return erf(x);
    case D_FMIN: return d_fmin(x, y);
    case D_FMAX: return d_fmax(x, y);
    case D_INV: return __drcp_rn(x);
    case D_SINH: return sinh(x);
    case D_COSH: return cosh(x);
    case D_TANH: return tanh(x);
    case D_ASINH: return asinh(x);
    case D_ACOSH: return acosh(x);
    case D_ATANH: return atanh(x);
    case D_ATAN2: return atan2(x, y);
    case D_ERFINV: return d_erfinv(x);
    case D_PRINTME: return x;  // the reference also prints the value; the GPU does not
    case D_LIFT: return x;
    case D_LOG1P: return log1p(x);
    case D_EXPM1: return expm1(x);
    case D_HYPOT: return hypot(x, y);
    default: return CUDART_NAN;
  }
}

// Value and recorded partials (BinaryOperation<OP>::der). Only the partials selected by
// partial_mask(op) are meaningful; the others are given by const_d0/const_d1.
__device__ __forceinline__ double dev_fun_der(unsigned op, double x, double y, double& d0,
                                              double& d1) {
  double f;
  switch (op) {
    case D_MUL: f = __dmul_rn(x, y); d0 = y; d1 = x; return f;
    case D_DIV:
      f = __ddiv_rn(x, y); d0 = __drcp_rn(y); d1 = __ddiv_rn(d_neg(f), y); return f;
    case D_EXP: f = exp(x); d0 = f; return f;
    case D_LOG: f = log(x); d0 = __drcp_rn(x); return f;
    case D_POW:
      f = pow(x, y); d0 = __dmul_rn(y, pow(x, __dsub_rn(y, 1.0))); d1 = __dmul_rn(log(x), f);
      return f;
    case D_CONSTPOW: f = pow(x, y); d0 = __dmul_rn(y, pow(x, __dsub_rn(y, 1.0))); return f;
    case D_SQRT: f = __dsqrt_rn(x); d0 = __drcp_rn(__dadd_rn(f, f)); return f;
    case D_SQ: f = __dmul_rn(x, x); d0 = d_twice(x); return f;
    case D_SIN: { double s, c; sincos(x, &s, &c); d0 = c; return s; }
    case D_COS: { double s, c; sincos(x, &s, &c); d0 = d_neg(s); return c; }
    case D_TAN: { f = tan(x); double c = cos(x); d0 = __drcp_rn(__dmul_rn(c, c)); return f; }
    case D_ASIN:
      f = asin(x); d0 = __drcp_rn(__dsqrt_rn(__dsub_rn(1.0, __dmul_rn(x, x)))); return f;
    case D_ACOS:
      f = acos(x); d0 = d_neg(__drcp_rn(__dsqrt_rn(__dsub_rn(1.0, __dmul_rn(x, x))))); return f;
    case D_ATAN: f = atan(x); d0 = __drcp_rn(__dadd_rn(1.0, __dmul_rn(x, x))); return f;
    case D_FMOD: f = fmod(x, y); d1 = __ddiv_rn(__dsub_rn(f, x), y); return f;
    case D_REMAINDER: f = remainder(x, y); d1 = __ddiv_rn(__dsub_rn(f, x), y); return f;
    case D_FABS: f = d_fabs(x); d0 = d_sign(x); return f;
    case D_COPYSIGN: f = d_copysign(x, y); d0 = d_copysign(1.0, y); return f;
    case D_IF_ELSE_ZERO: f = x == 0.0 ? 0.0 : y; d1 = x; return f;
    case D_ERF:
      f = erf(x);
      d0 = __dmul_rn(__ddiv_rn(2.0, __dsqrt_rn(CUDART_PI)), exp(d_neg(__dmul_rn(x, x))));
      return f;
    case D_FMIN: case D_FMAX: {
      f = op == D_FMIN ? d_fmin(x, y) : d_fmax(x, y);
      bool le = x <= y, ge = y <= x;
      bool a = op == D_FMIN ? le : ge, b = op == D_FMIN ? ge : le;
      if (a && b) { d0 = 0.5; d1 = 0.5; }
      else if (a || b) { d0 = a ? 1.0 : 0.0; d1 = b ? 1.0 : 0.0; }
      else { d0 = CUDART_NAN; d1 = CUDART_NAN; }  // 0/0 in the reference formula
      return f;
    }
    case D_INV: f = __drcp_rn(x); d0 = d_neg(__dmul_rn(f, f)); return f;
    case D_SINH: f = sinh(x); d0 = cosh(x); return f;
    case D_COSH: f = cosh(x); d0 = sinh(x); return f;
    case D_TANH: f = tanh(x); d0 = __dsub_rn(1.0, __dmul_rn(f, f)); return f;
    case D_ASINH:
      f = asinh(x); d0 = __drcp_rn(__dsqrt_rn(__dadd_rn(1.0, __dmul_rn(x, x)))); return f;
    case D_ACOSH:
      f = acosh(x);
      d0 = __ddiv_rn(__drcp_rn(__dsqrt_rn(__dsub_rn(x, 1.0))), __dsqrt_rn(__dadd_rn(x, 1.0)));
      return f;
    case D_ATANH: f = atanh(x); d0 = __drcp_rn(__dsub_rn(1.0, __dmul_rn(x, x))); return f;
    case D_ATAN2: {
      f = atan2(x, y);
      double t = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
      d0 = __ddiv_rn(y, t); d1 = __ddiv_rn(d_neg(x), t);
      return f;
    }
    case D_ERFINV:
      f = d_erfinv(x); d0 = __dmul_rn(__dmul_rn(__dsqrt_rn(CUDART_PI), 0.5), exp(__dmul_rn(f, f)));
      return f;
    case D_LOG1P: f = log1p(x); d0 = __drcp_rn(__dadd_rn(1.0, x)); return f;
    case D_EXPM1: f = expm1(x); d0 = exp(x); return f;
    case D_HYPOT: f = hypot(x, y); d0 = __ddiv_rn(x, f); d1 = __ddiv_rn(y, f); return f;
    default:
      return dev_fun(op, x, y);
  }
}

// dev_fun_der with the record sweeps' sin/cos pair (s, c): a SIN or COS computes the pair and
// keeps it, or, marked kSincosReuse, takes the kept pair of the same operand value; the bits
// are dev_fun_der's either way.
__device__ __forceinline__ double dev_fun_der_pair(unsigned op, double x, double y, double& d0,
                                                   double& d1, u64 ins, double& s, double& c) {
  if (op == D_SIN || op == D_COS) {
    if (!(ins & kSincosReuse)) sincos(x, &s, &c);
    d0 = op == D_SIN ? c : d_neg(s);
    return op == D_SIN ? s : c;
  }
  return dev_fun_der(op, x, y, d0, d1);
}

// dev_fun with the value sweeps' sin/cos pair: the first of a marked pair computes both as one
// sincos and keeps them, the second takes the kept one; unpaired SIN/COS call sin or cos. Same
// bits as dev_fun (sincos gives sin's and cos's results).
__device__ __forceinline__ double dev_fun_pair(unsigned op, double x, double y, u64 ins,
                                               double& s, double& c) {
  if ((op == D_SIN || op == D_COS) && (ins & (kSincosReuse | kSincosFirst))) {
    if (!(ins & kSincosReuse)) sincos(x, &s, &c);
    return op == D_SIN ? s : c;
  }
  return dev_fun(op, x, y);
}
#endif  // __CUDACC__

}  // namespace cgb
