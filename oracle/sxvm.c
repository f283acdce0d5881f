/*
 * ORACLE — test infrastructure only. Nothing in the product links or calls this file;
 * only tests/, the smoke check and the CPU-baseline leg of bench.py load it, as the
 * checker of the CUDA sweeps and as the timed CPU port.
 *
 * A plain-C restatement of CasADi's SX virtual machine over many instances:
 *   sxo_fun / sxo_der   casadi_math<double>::fun / der   (casadi/core/calculus.hpp:598-1018,
 *                        dispatch macros :1302-1355 and :1388-1439, sign :270,
 *                        if_else_zero :295, erfinv :297-328)
 *   sxo_eval            SXFunction::eval                 (casadi/core/sx_function.cpp:110-124)
 *   sxo_forward         numeric analogue of SXFunction::ad_forward (sx_function.cpp:1248-1364)
 *   sxo_jacobian        forward mode with unit seeds, the numeric analogue of the Jacobian
 *                       that XFunction::jac builds (casadi/core/x_function.hpp:441-840)
 *   sxo_reverse         numeric analogue of SXFunction::ad_reverse (sx_function.cpp:1418-1560)
 *   sxo_sp_forward      SXFunction::sp_forward           (sx_function.cpp:1657-1682)
 *   sxo_sp_reverse      SXFunction::sp_reverse           (sx_function.cpp:1742-1782)
 *   sxo_activity        SXFunction::eval_activity        (sx_function.cpp:1684-1718) with
 *                       the zero checkers of calculus.hpp:485-540 (sxo_zero_checker)
 *
 * Data layout (the layout the CUDA sweeps use): instance-minor. Input j of instance i,
 * nonzero k lives at arg[j][k*n + i]; outputs likewise. A null arg[j] reads zeros, a null
 * res[j] is skipped, as in SXFunction::eval.
 *
 * Forward seeds: fseed[j][(d*nnz_in[j] + k)*n + i] for direction d; sensitivities likewise.
 * Adjoint seeds aseed[j] (outputs) and sensitivities asens[j] (inputs) use the same
 * direction-major layout.
 *
 * Built with -ffp-contract=off: every operation rounds to double as the reference does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sxvm.h"

static double sxo_sign(double x) { return x < 0 ? -1 : x > 0 ? 1 : x; }

/* std::fmin/fmax as the reference build resolves them on x86-64: a NaN operand yields the
 * other operand and a tie (+0 vs -0 included) yields the first operand. C leaves the sign
 * of a zero tie unspecified; this fixes it so results compare bit for bit. */
static double sxo_fmin(double x, double y) {
  if (isnan(x)) return y;
  if (isnan(y)) return x;
  return y < x ? y : x;
}
static double sxo_fmax(double x, double y) {
  if (isnan(x)) return y;
  if (isnan(y)) return x;
  return y > x ? y : x;
}

/* calculus.hpp:297-328, used because the C library provides no erfinv */
static double sxo_erfinv(double x) {
  if (x >= 1) {
    return x == 1 ? INFINITY : NAN;
  } else if (x <= -1) {
    return x == -1 ? -INFINITY : NAN;
  } else if (x < -0.7) {
    double z = sqrt(-log((1.0 + x) / 2.0));
    return -(((1.641345311 * z + 3.429567803) * z - 1.624906493) * z - 1.970840454) /
           ((1.637067800 * z + 3.543889200) * z + 1.0);
  } else {
    double y;
    if (x < 0.7) {
      double z = x * x;
      y = x * (((-0.140543331 * z + 0.914624893) * z - 1.645349621) * z + 0.886226899) /
          ((((-0.329097515 * z + 0.012229801) * z + 1.442710462) * z - 2.118377725) * z + 1.0);
    } else {
      double z = sqrt(-log((1.0 - x) / 2.0));
      y = (((1.641345311 * z + 3.429567803) * z - 1.624906493) * z - 1.970840454) /
          ((1.637067800 * z + 3.543889200) * z + 1.0);
    }
    y = y - (erf(y) - x) / (2.0 / sqrt(M_PI) * exp(-y * y));
    y = y - (erf(y) - x) / (2.0 / sqrt(M_PI) * exp(-y * y));
    return y;
  }
}

static inline double fun_op(int op, double x, double y) {
  switch (op) {
    case SXO_ASSIGN: return x;
    case SXO_ADD: return x + y;
    case SXO_SUB: return x - y;
    case SXO_MUL: return x * y;
    case SXO_DIV: return x / y;
    case SXO_NEG: return -x;
    case SXO_EXP: return exp(x);
    case SXO_LOG: return log(x);
    case SXO_POW: return pow(x, y);
    case SXO_CONSTPOW: return pow(x, y);
    case SXO_SQRT: return sqrt(x);
    case SXO_SQ: return x * x;
    case SXO_TWICE: return 2. * x;
    case SXO_SIN: return sin(x);
    case SXO_COS: return cos(x);
    case SXO_TAN: return tan(x);
    case SXO_ASIN: return asin(x);
    case SXO_ACOS: return acos(x);
    case SXO_ATAN: return atan(x);
    case SXO_LT: return x < y;
    case SXO_LE: return x <= y;
    case SXO_EQ: return x == y;
    case SXO_NE: return x != y;
    case SXO_NOT: return !x;
    case SXO_AND: return x && y;
    case SXO_OR: return x || y;
    case SXO_FLOOR: return floor(x);
    case SXO_CEIL: return ceil(x);
    case SXO_FMOD: return fmod(x, y);
    case SXO_REMAINDER: return remainder(x, y);
    case SXO_FABS: return fabs(x);
    case SXO_SIGN: return sxo_sign(x);
    case SXO_COPYSIGN: return copysign(x, y);
    case SXO_IF_ELSE_ZERO: return x == 0 ? 0 : y;
    case SXO_ERF: return erf(x);
    case SXO_FMIN: return sxo_fmin(x, y);
    case SXO_FMAX: return sxo_fmax(x, y);
    case SXO_INV: return 1. / x;
    case SXO_SINH: return sinh(x);
    case SXO_COSH: return cosh(x);
    case SXO_TANH: return tanh(x);
    case SXO_ASINH: return asinh(x);
    case SXO_ACOSH: return acosh(x);
    case SXO_ATANH: return atanh(x);
    case SXO_ATAN2: return atan2(x, y);
    case SXO_ERFINV: return sxo_erfinv(x);
    case SXO_PRINTME: return x; /* the reference also prints; the oracle does not */
    case SXO_LIFT: return x;
    case SXO_LOG1P: return log1p(x);
    case SXO_EXPM1: return expm1(x);
    case SXO_HYPOT: return hypot(x, y);
    default: return NAN;
  }
}

/* BinaryOperation<OP>::der (calculus.hpp:598-1018); unary ops set d[1] = 0 (:384-387) */
static inline void der_op(int op, double x, double y, double f, double* d) {
  d[1] = 0;
  switch (op) {
    case SXO_ASSIGN: d[0] = 1; break;
    case SXO_ADD: d[0] = d[1] = 1; break;
    case SXO_SUB: d[0] = 1; d[1] = -1; break;
    case SXO_MUL: d[0] = y; d[1] = x; break;
    case SXO_DIV: d[0] = 1 / y; d[1] = -f / y; break;
    case SXO_NEG: d[0] = -1; break;
    case SXO_EXP: d[0] = f; break;
    case SXO_LOG: d[0] = 1 / x; break;
    case SXO_POW: d[0] = y * pow(x, y - 1); d[1] = log(x) * f; break;
    case SXO_CONSTPOW: d[0] = y * pow(x, y - 1); d[1] = 0; break;
    case SXO_SQRT: d[0] = 1 / (f + f); break;
    case SXO_SQ: d[0] = x + x; break;
    case SXO_TWICE: d[0] = 2; break;
    case SXO_SIN: d[0] = cos(x); break;
    case SXO_COS: d[0] = -sin(x); break;
    case SXO_TAN: { double c = cos(x); d[0] = 1 / (c * c); } break;
    case SXO_ASIN: d[0] = 1 / sqrt(1 - x * x); break;
    case SXO_ACOS: d[0] = -1 / sqrt(1 - x * x); break;
    case SXO_ATAN: d[0] = 1 / (1 + x * x); break;
    case SXO_LT: case SXO_LE: case SXO_EQ: case SXO_NE: case SXO_AND: case SXO_OR:
      d[0] = d[1] = 0; break;
    case SXO_NOT: case SXO_FLOOR: case SXO_CEIL: case SXO_SIGN: d[0] = 0; break;
    case SXO_FMOD: case SXO_REMAINDER: d[0] = 1; d[1] = (f - x) / y; break;
    case SXO_FABS: d[0] = sxo_sign(x); break;
    case SXO_COPYSIGN: d[0] = copysign(1.0, y); d[1] = 0; break;
    case SXO_IF_ELSE_ZERO: d[0] = 0; d[1] = x; break;
    case SXO_ERF: d[0] = (2 / sqrt(M_PI)) * exp(-x * x); break;
    case SXO_FMIN: {
      double a = x <= y, b = y <= x, c = a + b;
      d[0] = a / c; d[1] = b / c;
    } break;
    case SXO_FMAX: {
      double a = y <= x, b = x <= y, c = a + b;
      d[0] = a / c; d[1] = b / c;
    } break;
    case SXO_INV: d[0] = -f * f; break;
    case SXO_SINH: d[0] = cosh(x); break;
    case SXO_COSH: d[0] = sinh(x); break;
    case SXO_TANH: d[0] = 1 - f * f; break;
    case SXO_ASINH: d[0] = 1 / sqrt(1 + x * x); break;
    case SXO_ACOSH: d[0] = 1 / sqrt(x - 1) / sqrt(x + 1); break;
    case SXO_ATANH: d[0] = 1 / (1 - x * x); break;
    case SXO_ATAN2: { double t = x * x + y * y; d[0] = y / t; d[1] = -x / t; } break;
    case SXO_ERFINV: d[0] = (sqrt(M_PI) / 2) * exp(f * f); break;
    case SXO_PRINTME: case SXO_LIFT: d[0] = 1; d[1] = 0; break;
    case SXO_LOG1P: d[0] = 1 / (1 + x); break;
    case SXO_EXPM1: d[0] = exp(x); break;
    case SXO_HYPOT: d[0] = x / f; d[1] = y / f; break;
    default: d[0] = d[1] = NAN;
  }
}

/* the exported forms of the two (the sweeps below use the inlined ones) */
double sxo_fun(int op, double x, double y) { return fun_op(op, x, y); }
void sxo_der(int op, double x, double y, double f, double* d) { der_op(op, x, y, f, d); }

int sxo_ndeps(int op) {
  switch (op) {
    case SXO_CONST: case SXO_PARAMETER: case SXO_INPUT: return 0;
    case SXO_ADD: case SXO_SUB: case SXO_MUL: case SXO_DIV: case SXO_POW: case SXO_CONSTPOW:
    case SXO_LT: case SXO_LE: case SXO_EQ: case SXO_NE: case SXO_AND: case SXO_OR:
    case SXO_COPYSIGN: case SXO_FMOD: case SXO_REMAINDER: case SXO_FMIN: case SXO_FMAX:
    case SXO_ATAN2: case SXO_PRINTME: case SXO_LIFT: case SXO_HYPOT: case SXO_IF_ELSE_ZERO:
      return 2;
    default: return 1;
  }
}

/* ---------------------------------------------------------------------------------------- */
/* one instance                                                                              */
/* ---------------------------------------------------------------------------------------- */

/* One instruction as SXFunction::eval walks it: an AlgEl-like record (op, i0, i1, i2, d). */
typedef struct {
  int op, i0, i1, i2;
  double d;
} sxo_ins;

static void eval_one(const sxo_ins* alg, int n_instr, long n, long i, const double* const* arg,
                     double* const* res, double* w) {
  for (const sxo_ins* e = alg; e != alg + n_instr; ++e) {
    switch (e->op) {
      case SXO_CONST: w[e->i0] = e->d; break;
      case SXO_INPUT: w[e->i0] = arg[e->i1] ? arg[e->i1][(long)e->i2 * n + i] : 0; break;
      case SXO_OUTPUT: if (res[e->i0]) res[e->i0][(long)e->i2 * n + i] = w[e->i1]; break;
      default: w[e->i0] = fun_op(e->op, w[e->i1], w[e->i2]);
    }
  }
}

/* Magnitude mode (set by sxo_set_magnitude): the AD sweeps run on |partials| and |seeds|,
 * so each derivative result is the sum over its chain-rule paths of |product of partials| x
 * |seed| -- the scale that the rounding error of any evaluation order of that derivative is
 * bounded by (each path's product and the sum over paths round with relative error of order
 * path length x eps). The tests use it to compare two AD results that round differently
 * (this numeric sweep, the reference's symbolic one) element by element. */
static int g_magnitude = 0;

void sxo_set_magnitude(int on) { g_magnitude = on != 0; }

/* values plus the partials of every arithmetic instruction, in tape order */
static void eval_partials(const sxo_tape* t, long n, long i, const double* const* arg,
                          double* const* res, double* w, double* dp) {
  for (int k = 0; k < t->n_instr; ++k) {
    int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
    switch (op) {
      case SXO_CONST: w[i0] = t->d[k]; break;
      case SXO_INPUT: w[i0] = arg[i1] ? arg[i1][(long)i2 * n + i] : 0; break;
      case SXO_OUTPUT: if (res && res[i0]) res[i0][(long)i2 * n + i] = w[i1]; break;
      default: {
        double x = w[i1], y = w[i2];
        double f = fun_op(op, x, y);
        der_op(op, x, y, f, dp + 2 * (long)k);
        if (g_magnitude) {
          dp[2 * (long)k] = fabs(dp[2 * (long)k]);
          dp[2 * (long)k + 1] = fabs(dp[2 * (long)k + 1]);
        }
        w[i0] = f;
      }
    }
  }
}

int sxo_eval(const sxo_tape* t, long n, const double* const* arg, double* const* res,
             int nthreads) {
  int err = 0;
  /* the tape as one array of records, walked once per instance */
  sxo_ins* alg = (sxo_ins*)malloc(sizeof(sxo_ins) * (t->n_instr > 0 ? t->n_instr : 1));
  if (!alg) return 1;
  for (int k = 0; k < t->n_instr; ++k) {
    alg[k].op = t->op[k];
    alg[k].i0 = t->i0[k];
    alg[k].i1 = t->i1[k];
    alg[k].i2 = t->i2[k];
    alg[k].d = t->d[k];
  }
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    double* w = (double*)malloc(sizeof(double) * (t->sz_w > 0 ? t->sz_w : 1));
    if (!w) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) eval_one(alg, t->n_instr, n, i, arg, res, w);
    }
    free(w);
  }
  free(alg);
  return err;
}

/* Structural activity (both AD sweeps): a slot is active when its derivative is not
 * structurally zero. The reference builds derivatives symbolically, where constants and
 * unseeded inputs are the zero expression and 0*x -> 0, x+0 -> x, 0-x -> -x simplify away
 * (casadi/core/calculus.hpp:1872-1990); the numeric sweeps below apply the same rules, so an
 * operand contributes only when it is active and its partial is not the constant zero. */
static int nonzero_d0(int op) {
  switch (op) {
    case SXO_LT: case SXO_LE: case SXO_EQ: case SXO_NE: case SXO_AND: case SXO_OR:
    case SXO_NOT: case SXO_FLOOR: case SXO_CEIL: case SXO_SIGN: case SXO_IF_ELSE_ZERO:
      return 0;
    default: return 1;
  }
}
static int nonzero_d1(int op) {
  switch (op) {
    case SXO_ADD: case SXO_SUB: case SXO_MUL: case SXO_DIV: case SXO_POW: case SXO_FMOD:
    case SXO_REMAINDER: case SXO_FMIN: case SXO_FMAX: case SXO_ATAN2: case SXO_HYPOT:
    case SXO_IF_ELSE_ZERO:
      return 1;
    default: return 0;
  }
}

/* Ops whose partials are exactly +-1 or 2 (their products with a seed are exact). */
static int exact_partials(int op) {
  return op == SXO_ADD || op == SXO_SUB || op == SXO_NEG || op == SXO_TWICE ||
         op == SXO_ASSIGN;
}

/* one forward direction over one instance; seed(j, k) gives the seed (NAN-free) of input
 * nonzero k of input j, active(j, k) whether it is seeded */
static void tangent_one(const sxo_tape* t, const double* dp, double* wd, char* act,
                        const int* in_off, int unit_dir, long n, long i, int dir,
                        const double* const* fseed, double* const* fsens) {
  for (int k = 0; k < t->n_instr; ++k) {
    int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
    const double* d = dp + 2 * (long)k;
    switch (op) {
      case SXO_INPUT:
        if (unit_dir >= 0) {
          act[i0] = in_off[i1] + i2 == unit_dir;
          if (act[i0]) wd[i0] = 1.0;
        } else {
          const double* s = fseed[i1];
          act[i0] = s != 0;
          if (s) wd[i0] = s[((long)dir * t->nnz_in[i1] + i2) * n + i];
          if (s && g_magnitude) wd[i0] = fabs(wd[i0]);
        }
        break;
      case SXO_OUTPUT: {
        double* s = fsens[i0];
        if (s) s[((long)dir * t->nnz_out[i0] + i2) * n + i] = act[i1] ? wd[i1] : 0;
      } break;
      case SXO_CONST: case SXO_PARAMETER: act[i0] = 0; break;
      default: {
        int bin = sxo_ndeps(op) == 2;
        int cb = act[i1] && nonzero_d0(op);
        int cc = bin && act[i2] && nonzero_d1(op);
        if (cb || cc) {
          double xb = cb ? wd[i1] : 0, xc = cc ? wd[i2] : 0, r;
          if (op == SXO_IF_ELSE_ZERO) r = d[1] == 0 ? 0 : xc;
          /* both operands: one fused multiply-add, d0*xb + (d1*xc) rounded once */
          else if (cb && cc) r = fma(d[0], xb, d[1] * xc);
          else if (cb) r = d[0] * xb;
          else r = d[1] * xc;
          wd[i0] = r;
        }
        act[i0] = cb || cc;
      }
    }
  }
}

static int forward_impl(const sxo_tape* t, long n, int nfwd, int unit, const double* const* arg,
                        double* const* res, const double* const* fseed, double* const* fsens,
                        int nthreads) {
  int err = 0;
  int in_off[256];
  if (t->n_in > 256) return 1;
  for (int j = 0, o = 0; j < t->n_in; o += t->nnz_in[j], ++j) in_off[j] = o;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    int sz = t->sz_w > 0 ? t->sz_w : 1;
    double* w = (double*)malloc(sizeof(double) * sz);
    double* wd = (double*)malloc(sizeof(double) * sz);
    char* act = (char*)malloc(sz);
    double* dp = (double*)malloc(sizeof(double) * 2 * (t->n_instr > 0 ? t->n_instr : 1));
    if (!w || !wd || !act || !dp) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) {
        eval_partials(t, n, i, arg, res, w, dp);
        for (int dir = 0; dir < nfwd; ++dir)
          tangent_one(t, dp, wd, act, in_off, unit ? dir : -1, n, i, dir, fseed, fsens);
      }
    }
    free(w); free(wd); free(act); free(dp);
  }
  return err;
}

int sxo_forward(const sxo_tape* t, long n, int nfwd, const double* const* arg,
                double* const* res, const double* const* fseed, double* const* fsens,
                int nthreads) {
  return forward_impl(t, n, nfwd, 0, arg, res, fseed, fsens, nthreads);
}

/* Jacobian by forward mode with unit seeds: direction d is input nonzero d (input order);
 * jac[j][(d*nnz_out[j] + k)*n + i]. */
int sxo_jacobian(const sxo_tape* t, long n, const double* const* arg, double* const* res,
                 double* const* jac, int nthreads) {
  int nz = 0;
  for (int j = 0; j < t->n_in; ++j) nz += t->nnz_in[j];
  return forward_impl(t, n, nz, 1, arg, res, 0, jac, nthreads);
}

/* nadj adjoint directions over one instance from its recorded partials dp */
static void adjoint_one(const sxo_tape* t, const double* dp, double* wb, char* act, long n,
                        long i, int nadj, const double* const* aseed, double* const* asens) {
  for (int dir = 0; dir < nadj; ++dir) {
    for (int s = 0; s < t->sz_w; ++s) { wb[s] = 0; act[s] = 0; }
    /* asens starts at zero for every input nonzero (sx_function.cpp:1413-1422) */
    for (int j = 0; j < t->n_in; ++j) {
      if (!asens[j]) continue;
      for (int k = 0; k < t->nnz_in[j]; ++k)
        asens[j][((long)dir * t->nnz_in[j] + k) * n + i] = 0;
    }
    for (int k = t->n_instr - 1; k >= 0; --k) {
      int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
      const double* d = dp + 2 * (long)k;
      switch (op) {
        case SXO_INPUT: {
          double* s = asens[i1];
          if (s) s[((long)dir * t->nnz_in[i1] + i2) * n + i] = act[i0] ? wb[i0] : 0;
          wb[i0] = 0; act[i0] = 0;
        } break;
        case SXO_OUTPUT: {
          const double* s = aseed[i0];
          if (s) {
            double v = s[((long)dir * t->nnz_out[i0] + i2) * n + i];
            if (g_magnitude) v = fabs(v);
            wb[i1] = act[i1] ? wb[i1] + v : v;
            act[i1] = 1;
          }
        } break;
        case SXO_CONST: case SXO_PARAMETER: wb[i0] = 0; act[i0] = 0; break;
        default: {
          if (!act[i0]) break;
          double seed = wb[i0], c;
          wb[i0] = 0; act[i0] = 0;
          /* a later contribution d*seed of a general op is added with one fused
           * multiply-add; the partials of ADD, SUB, NEG, TWICE and ASSIGN are exact
           * (+-1, 2), so their products are exact and added with one rounding */
          if (nonzero_d0(op)) {
            c = d[0] * seed;
            wb[i1] = !act[i1] ? c : exact_partials(op) ? wb[i1] + c
                                                       : fma(d[0], seed, wb[i1]);
            act[i1] = 1;
          }
          if (sxo_ndeps(op) == 2 && nonzero_d1(op)) {
            if (op == SXO_IF_ELSE_ZERO) {
              c = d[1] == 0 ? 0 : seed;
              wb[i2] = act[i2] ? wb[i2] + c : c;
            } else {
              c = d[1] * seed;
              wb[i2] = !act[i2] ? c : exact_partials(op) ? wb[i2] + c
                                                         : fma(d[1], seed, wb[i2]);
            }
            act[i2] = 1;
          }
        }
      }
    }
  }
}

/* Values, tangents of the unit directions (jac, as sxo_jacobian) when jac is given, and
 * nadj adjoint directions (asens, as sxo_reverse) when nadj > 0, all from one record of the
 * partials per instance. */
static int derivs_impl(const sxo_tape* t, long n, const double* const* arg, double* const* res,
                       double* const* jac, int nadj, const double* const* aseed,
                       double* const* asens, int nthreads) {
  int err = 0;
  int in_off[256];
  if (t->n_in > 256) return 1;
  int nz = 0;
  for (int j = 0; j < t->n_in; nz += t->nnz_in[j], ++j) in_off[j] = nz;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    int sz = t->sz_w > 0 ? t->sz_w : 1;
    double* w = (double*)malloc(sizeof(double) * sz);
    double* wb = (double*)malloc(sizeof(double) * sz);
    char* act = (char*)malloc(sz);
    double* dp = (double*)malloc(sizeof(double) * 2 * (t->n_instr > 0 ? t->n_instr : 1));
    if (!w || !wb || !act || !dp) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) {
        eval_partials(t, n, i, arg, res, w, dp);
        if (jac)
          for (int dir = 0; dir < nz; ++dir)
            tangent_one(t, dp, wb, act, in_off, dir, n, i, dir, 0, jac);
        if (nadj > 0) adjoint_one(t, dp, wb, act, n, i, nadj, aseed, asens);
      }
    }
    free(w); free(wb); free(act); free(dp);
  }
  return err;
}

int sxo_reverse(const sxo_tape* t, long n, int nadj, const double* const* arg,
                double* const* res, const double* const* aseed, double* const* asens,
                int nthreads) {
  return derivs_impl(t, n, arg, res, 0, nadj, aseed, asens, nthreads);
}

int sxo_jacobian_reverse(const sxo_tape* t, long n, const double* const* arg,
                         double* const* res, double* const* jac, int nadj,
                         const double* const* aseed, double* const* asens, int nthreads) {
  return derivs_impl(t, n, arg, res, jac, nadj, aseed, asens, nthreads);
}

/* Ops whose results are libm calls (not correctly rounded in general, so two libms may
 * return different last bits): everything but the IEEE-exact arithmetic, comparisons and
 * selections. */
static int is_libm(int op) {
  switch (op) {
    case SXO_EXP: case SXO_LOG: case SXO_POW: case SXO_CONSTPOW: case SXO_SIN: case SXO_COS:
    case SXO_TAN: case SXO_ASIN: case SXO_ACOS: case SXO_ATAN: case SXO_ERF: case SXO_SINH:
    case SXO_COSH: case SXO_TANH: case SXO_ASINH: case SXO_ACOSH: case SXO_ATANH:
    case SXO_ATAN2: case SXO_ERFINV: case SXO_LOG1P: case SXO_EXPM1: case SXO_HYPOT:
      return 1;
    default: return 0;
  }
}

/* First-order sensitivity of every output to relative perturbations of the libm results:
 * bound[j][nz] = sum over libm instructions k of |d out(j,nz) / d w_k| * |w_k|, the
 * derivative taken through |partials| (one magnitude adjoint sweep per output nonzero).
 * If two evaluations differ only in that each libm result may be off by up to c ulps, their
 * outputs differ by at most about c * 2^-52 * bound (to first order). */
static int bound_impl(const sxo_tape* t, long n, const double* const* arg, double* const* bound,
                      int nthreads, int every_op) {
  int err = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    int sz = t->sz_w > 0 ? t->sz_w : 1;
    long ni = t->n_instr > 0 ? t->n_instr : 1;
    double* w = (double*)malloc(sizeof(double) * sz);
    double* wb = (double*)malloc(sizeof(double) * sz);
    double* dp = (double*)malloc(sizeof(double) * 2 * ni);
    double* fv = (double*)malloc(sizeof(double) * ni);
    if (!w || !wb || !dp || !fv) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) {
        /* values, partials and every instruction's own result */
        for (int k = 0; k < t->n_instr; ++k) {
          int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
          fv[k] = 0;
          switch (op) {
            case SXO_CONST: w[i0] = t->d[k]; break;
            case SXO_INPUT: w[i0] = arg[i1] ? arg[i1][(long)i2 * n + i] : 0; break;
            case SXO_OUTPUT: break;
            default: {
              double x = w[i1], y = w[i2];
              double f = fun_op(op, x, y);
              der_op(op, x, y, f, dp + 2 * (long)k);
              w[i0] = fv[k] = f;
            }
          }
        }
        for (int ko = 0; ko < t->n_instr; ++ko) {
          if (t->op[ko] != SXO_OUTPUT || !bound[t->i0[ko]]) continue;
          for (int s = 0; s < t->sz_w; ++s) wb[s] = 0;
          double acc = 0;
          wb[t->i1[ko]] = 1;
          for (int k = ko - 1; k >= 0; --k) {
            int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
            if (op == SXO_OUTPUT) continue;
            double seed = wb[i0];
            wb[i0] = 0;
            if (op == SXO_CONST || op == SXO_INPUT || op == SXO_PARAMETER || seed == 0) continue;
            if (every_op || is_libm(op)) acc += seed * fabs(fv[k]);
            const double* d = dp + 2 * (long)k;
            wb[i1] += fabs(d[0]) * seed;
            if (sxo_ndeps(op) == 2) wb[i2] += fabs(d[1]) * seed;
          }
          bound[t->i0[ko]][(long)t->i2[ko] * n + i] = acc;
        }
      }
    }
    free(w); free(wb); free(dp); free(fv);
  }
  return err;
}

int sxo_libm_bound(const sxo_tape* t, long n, const double* const* arg, double* const* bound,
                   int nthreads) {
  return bound_impl(t, n, arg, bound, nthreads, 0);
}

int sxo_rounding_bound(const sxo_tape* t, long n, const double* const* arg,
                       double* const* bound, int nthreads) {
  return bound_impl(t, n, arg, bound, nthreads, 1);
}

int sxo_sp_forward(const sxo_tape* t, long n, const uint64_t* const* arg,
                   uint64_t* const* res, int nthreads) {
  int err = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    uint64_t* w = (uint64_t*)malloc(sizeof(uint64_t) * (t->sz_w > 0 ? t->sz_w : 1));
    if (!w) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) {
        for (int k = 0; k < t->n_instr; ++k) {
          int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
          switch (op) {
            case SXO_CONST: case SXO_PARAMETER: w[i0] = 0; break;
            case SXO_INPUT: w[i0] = arg[i1] ? arg[i1][(long)i2 * n + i] : 0; break;
            case SXO_OUTPUT: if (res[i0]) res[i0][(long)i2 * n + i] = w[i1]; break;
            default: w[i0] = w[i1] | w[i2];
          }
        }
      }
    }
    free(w);
  }
  return err;
}

int sxo_sp_reverse(const sxo_tape* t, long n, uint64_t* const* arg, uint64_t* const* res,
                   int nthreads) {
  int err = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    uint64_t* w = (uint64_t*)malloc(sizeof(uint64_t) * (t->sz_w > 0 ? t->sz_w : 1));
    if (!w) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) {
        for (int s = 0; s < t->sz_w; ++s) w[s] = 0;
        for (int k = t->n_instr - 1; k >= 0; --k) {
          int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
          uint64_t seed;
          switch (op) {
            case SXO_CONST: case SXO_PARAMETER: w[i0] = 0; break;
            case SXO_INPUT:
              if (arg[i1]) arg[i1][(long)i2 * n + i] |= w[i0];
              w[i0] = 0;
              break;
            case SXO_OUTPUT:
              if (res[i0]) {
                w[i1] |= res[i0][(long)i2 * n + i];
                res[i0][(long)i2 * n + i] = 0;
              }
              break;
            default:
              seed = w[i0]; w[i0] = 0;
              w[i1] |= seed;
              w[i2] |= seed;
          }
        }
      }
    }
    free(w);
  }
  return err;
}

/* The reference's zero checkers (calculus.hpp:485-540). which = 0: f(0, y) == 0 for every y
 * (F0XChecker); 1: f(x, 0) == 0 for every x (FX0Checker); 2: f(0, 0) == 0 (F00Checker). */
int sxo_zero_checker(int which, int op) {
  int first = 0, second = 0, both = 0;
  switch (op) {
    case SXO_ASSIGN: case SXO_DIV: case SXO_NEG: case SXO_SQRT: case SXO_SQ: case SXO_TWICE:
    case SXO_SIN: case SXO_TAN: case SXO_ATAN: case SXO_ASIN: case SXO_FLOOR: case SXO_CEIL:
    case SXO_FMOD: case SXO_REMAINDER: case SXO_FABS: case SXO_SIGN: case SXO_ERF:
    case SXO_SINH: case SXO_TANH: case SXO_ASINH: case SXO_ATANH: case SXO_ERFINV:
    case SXO_LOG1P: case SXO_EXPM1:
      first = 1;
      break;
    case SXO_COPYSIGN:
      first = both = 1;
      break;
    case SXO_MUL: case SXO_IF_ELSE_ZERO:
      first = second = 1;
      break;
    case SXO_AND:
      first = second = both = 1;
      break;
    case SXO_ADD: case SXO_SUB: case SXO_FMIN: case SXO_FMAX: case SXO_OR: case SXO_LT:
    case SXO_HYPOT:
      both = 1;
      break;
    default:
      break;
  }
  if (which == 0) return first;
  if (which == 1) return second;
  return both || first || second;
}

int sxo_activity(const sxo_tape* t, long n, const uint64_t* const* arg, uint64_t* const* res,
                 int nthreads) {
  const uint64_t all = ~(uint64_t)0;
  int err = 0;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
  {
    uint64_t* w = (uint64_t*)malloc(sizeof(uint64_t) * (t->sz_w > 0 ? t->sz_w : 1));
    if (!w) {
#pragma omp atomic write
      err = 1;
    } else {
#pragma omp for schedule(static)
      for (long i = 0; i < n; ++i) {
        for (int k = 0; k < t->n_instr; ++k) {
          int op = t->op[k], i0 = t->i0[k], i1 = t->i1[k], i2 = t->i2[k];
          switch (op) {
            case SXO_CONST: w[i0] = t->d[k] != 0 ? all : 0; break;
            case SXO_PARAMETER: w[i0] = all; break;
            case SXO_INPUT: w[i0] = arg[i1] ? arg[i1][(long)i2 * n + i] : 0; break;
            case SXO_OUTPUT: if (res[i0]) res[i0][(long)i2 * n + i] = w[i1]; break;
            default:
              if (sxo_ndeps(op) == 1) {
                w[i0] = w[i1] ? all : (sxo_zero_checker(0, op) ? 0 : all);
              } else {
                int a = w[i1] != 0, b = w[i2] != 0;
                int zero = a && b ? 0 : a ? sxo_zero_checker(1, op)
                                          : b ? sxo_zero_checker(0, op) : sxo_zero_checker(2, op);
                w[i0] = zero ? 0 : all;
              }
          }
        }
      }
    }
    free(w);
  }
  return err;
}
