// ORACLE PIN — test infrastructure only, built into oracle/_ref/ from the reference's own
// sources where they lie (the reference tree is needed at build time; it is not copied).
//
// The reference's scalar-op semantics are header-only templates in casadi/core/calculus.hpp.
// This harness compiles that header as is and exposes, over a C ABI:
//   ref_fun / ref_der   casadi_math<double>::fun / der (calculus.hpp:1299-1439)
//   ref_ndeps           casadi_math<double>::ndeps (calculus.hpp:1632-1647)
//   ref_op_id           the numeric value of enum Operation members (calculus.hpp:60-218)
//   ref_zero_checker    operation_checker<F0XChecker / FX0Checker / F00Checker>
//                       (calculus.hpp:485-540, :1128-1131)
//   ref_activity        SXFunction::eval_activity's instruction loop (sx_function.cpp:
//                       1684-1718) driving the reference's own checkers
//   ref_eval            SXFunction::eval's instruction loop (casadi/core/sx_function.cpp:110-124)
//                       driving the reference's own CASADI_MATH_FUN_BUILTIN dispatch macro
//   ref_forward / ref_jacobian / ref_reverse
//                       the numeric forward/adjoint sweeps that mirror the structure of
//                       SXFunction::ad_forward/ad_reverse (sx_function.cpp:1248-1364,
//                       :1418-1560) with partials from CASADI_MATH_DER_BUILTIN and the
//                       structural-zero rules of the reference's derivative expressions
// The rest of libcasadi needs CMake-generated headers and is not built.
#include <iomanip>
#include <cstdint>
#include <cstring>
#include <vector>
#include "casadi/core/exception.hpp"
#include "casadi/core/calculus.hpp"

namespace casadi {
// calculus.hpp's printme() writes to uout(); libcasadi defines it in casadi_logger.cpp.
std::ostream& uout() { return std::cout; }
}  // namespace casadi

using namespace casadi;

extern "C" {

double ref_fun(int op, double x, double y) {
  double f;
  casadi_math<double>::fun(static_cast<unsigned char>(op), x, y, f);
  return f;
}

void ref_der(int op, double x, double y, double f, double* d) {
  casadi_math<double>::der(static_cast<unsigned char>(op), x, y, f, d);
}

int ref_ndeps(int op) { return static_cast<int>(casadi_math<double>::ndeps(op)); }

int ref_op_id(const char* name) {
#define ID(X) if (!std::strcmp(name, #X)) return X;
  ID(OP_ASSIGN) ID(OP_ADD) ID(OP_SUB) ID(OP_MUL) ID(OP_DIV) ID(OP_NEG) ID(OP_EXP) ID(OP_LOG)
  ID(OP_POW) ID(OP_CONSTPOW) ID(OP_SQRT) ID(OP_SQ) ID(OP_TWICE) ID(OP_SIN) ID(OP_COS)
  ID(OP_TAN) ID(OP_ASIN) ID(OP_ACOS) ID(OP_ATAN) ID(OP_LT) ID(OP_LE) ID(OP_EQ) ID(OP_NE)
  ID(OP_NOT) ID(OP_AND) ID(OP_OR) ID(OP_FLOOR) ID(OP_CEIL) ID(OP_FMOD) ID(OP_FABS)
  ID(OP_SIGN) ID(OP_COPYSIGN) ID(OP_IF_ELSE_ZERO) ID(OP_ERF) ID(OP_FMIN) ID(OP_FMAX)
  ID(OP_INV) ID(OP_SINH) ID(OP_COSH) ID(OP_TANH) ID(OP_ASINH) ID(OP_ACOSH) ID(OP_ATANH)
  ID(OP_ATAN2) ID(OP_CONST) ID(OP_INPUT) ID(OP_OUTPUT) ID(OP_PARAMETER) ID(OP_CALL)
  ID(OP_ERFINV) ID(OP_PRINTME) ID(OP_LIFT) ID(OP_LOG1P) ID(OP_EXPM1) ID(OP_HYPOT)
  ID(OP_REMAINDER)
#undef ID
  return -1;
}

int ref_zero_checker(int which, int op) {
  if (which == 0) return operation_checker<F0XChecker>(op) ? 1 : 0;
  if (which == 1) return operation_checker<FX0Checker>(op) ? 1 : 0;
  return operation_checker<F00Checker>(op) ? 1 : 0;
}

// Instance-minor layout as ref_eval.
int ref_activity(int n_instr, const int* op, const int* i0, const int* i1, const int* i2,
                 const double* d, int sz_w, long n, const uint64_t* const* arg,
                 uint64_t* const* res) {
  const uint64_t nz = ~static_cast<uint64_t>(0);
  std::vector<uint64_t> w(sz_w > 0 ? sz_w : 1);
  for (long i = 0; i < n; ++i) {
    for (int k = 0; k < n_instr; ++k) {
      switch (op[k]) {
        case OP_CONST: w[i0[k]] = d[k] != 0 ? nz : 0; break;
        case OP_PARAMETER: w[i0[k]] = nz; break;
        case OP_INPUT: w[i0[k]] = arg[i1[k]] != nullptr ? arg[i1[k]][i2[k] * n + i] : 0; break;
        case OP_OUTPUT: if (res[i0[k]] != nullptr) res[i0[k]][i2[k] * n + i] = w[i1[k]]; break;
        default:
          if (casadi_math<double>::ndeps(op[k]) == 1) {
            w[i0[k]] = w[i1[k]] ? nz : (operation_checker<F0XChecker>(op[k]) ? 0 : nz);
          } else {
            const bool z0 = w[i1[k]] != 0, z1 = w[i2[k]] != 0;
            if (!z0 && !z1) w[i0[k]] = operation_checker<F00Checker>(op[k]) ? 0 : nz;
            else if (!z0) w[i0[k]] = operation_checker<F0XChecker>(op[k]) ? 0 : nz;
            else if (!z1) w[i0[k]] = operation_checker<FX0Checker>(op[k]) ? 0 : nz;
            else w[i0[k]] = nz;
          }
      }
    }
  }
  return 0;
}

// Instance-minor layout: arg[j][k*n + i]; see oracle/sxvm.c.
int ref_eval(int n_instr, const int* op, const int* i0, const int* i1, const int* i2,
             const double* d, int sz_w, long n, const double* const* arg,
             double* const* res) {
  std::vector<double> w(sz_w > 0 ? sz_w : 1);
  for (long i = 0; i < n; ++i) {
    for (int k = 0; k < n_instr; ++k) {
      switch (op[k]) {
        CASADI_MATH_FUN_BUILTIN(w[i1[k]], w[i2[k]], w[i0[k]])
        case OP_CONST: w[i0[k]] = d[k]; break;
        case OP_INPUT: w[i0[k]] = arg[i1[k]] == nullptr ? 0 : arg[i1[k]][i2[k] * n + i]; break;
        case OP_OUTPUT: if (res[i0[k]] != nullptr) res[i0[k]][i2[k] * n + i] = w[i1[k]]; break;
        default: return 1;
      }
    }
  }
  return 0;
}

static void partials(int n_instr, const int* op, const int* i0, const int* i1, const int* i2,
                     const double* d, long n, long i, const double* const* arg,
                     std::vector<double>& w, std::vector<double>& dp) {
  for (int k = 0; k < n_instr; ++k) {
    switch (op[k]) {
      case OP_CONST: w[i0[k]] = d[k]; break;
      case OP_INPUT: w[i0[k]] = arg[i1[k]] == nullptr ? 0 : arg[i1[k]][i2[k] * n + i]; break;
      case OP_OUTPUT: break;
      default: {
        double x = w[i1[k]], y = w[i2[k]], f;
        casadi_math<double>::fun(static_cast<unsigned char>(op[k]), x, y, f);
        casadi_math<double>::der(static_cast<unsigned char>(op[k]), x, y, f, &dp[2 * k]);
        w[i0[k]] = f;
      }
    }
  }
}

// Structural activity: an operand contributes when its derivative is not structurally zero
// and its partial is not the constant zero -- the simplifications 0*x -> 0, x+0 -> x,
// 0-x -> -x that the reference applies while building derivative expressions
// (calculus.hpp:1872-1990). The partials come from CASADI_MATH_DER_BUILTIN; an operand's
// partial is a constant zero exactly when the reference's der() writes a literal 0 for it.
static bool const_zero_partial(int op, int which) {
  // evaluate der() at points on both sides of x == y; a literal zero is zero at all of them
  const double pts[3][2] = {{0.3, 0.7}, {2.3, 0.7}, {-1.9, 2.3}};
  for (const auto& q : pts) {
    double f, d[2];
    casadi_math<double>::fun(static_cast<unsigned char>(op), q[0], q[1], f);
    casadi_math<double>::der(static_cast<unsigned char>(op), q[0], q[1], f, d);
    if (!(d[which] == 0)) return false;
  }
  return true;
}

static int forward_impl(int n_instr, const int* op, const int* i0, const int* i1,
                        const int* i2, const double* d, int sz_w, int n_in, const int* nnz_in,
                        const int* nnz_out, long n, int nfwd, bool unit,
                        const double* const* arg, const double* const* fseed,
                        double* const* fsens) {
  std::vector<double> w(sz_w > 0 ? sz_w : 1), wd(sz_w > 0 ? sz_w : 1), dp(2 * n_instr + 2);
  std::vector<char> act(sz_w > 0 ? sz_w : 1);
  std::vector<int> off(n_in + 1, 0);
  for (int j = 0; j < n_in; ++j) off[j + 1] = off[j] + nnz_in[j];
  for (long i = 0; i < n; ++i) {
    partials(n_instr, op, i0, i1, i2, d, n, i, arg, w, dp);
    for (int dir = 0; dir < nfwd; ++dir) {
      for (int k = 0; k < n_instr; ++k) {
        const double* p = &dp[2 * k];
        switch (op[k]) {
          case OP_INPUT:
            if (unit) {
              act[i0[k]] = off[i1[k]] + i2[k] == dir;
              if (act[i0[k]]) wd[i0[k]] = 1.0;
            } else {
              act[i0[k]] = fseed[i1[k]] != nullptr;
              if (fseed[i1[k]]) wd[i0[k]] = fseed[i1[k]][(dir * nnz_in[i1[k]] + i2[k]) * n + i];
            }
            break;
          case OP_OUTPUT:
            if (fsens[i0[k]])
              fsens[i0[k]][(dir * nnz_out[i0[k]] + i2[k]) * n + i] = act[i1[k]] ? wd[i1[k]] : 0;
            break;
          case OP_CONST: case OP_PARAMETER: act[i0[k]] = 0; break;
          default: {
            bool bin = casadi_math<double>::ndeps(op[k]) == 2;
            bool cb = act[i1[k]] && !const_zero_partial(op[k], 0);
            bool cc = bin && act[i2[k]] && !const_zero_partial(op[k], 1);
            if (cb || cc) {
              double xb = cb ? wd[i1[k]] : 0, xc = cc ? wd[i2[k]] : 0, r;
              if (op[k] == OP_IF_ELSE_ZERO) r = if_else_zero(p[1], xc);
              else if (cb && cc) r = p[0] * xb + p[1] * xc;
              else if (cb) r = p[0] * xb;
              else r = p[1] * xc;
              wd[i0[k]] = r;
            }
            act[i0[k]] = cb || cc;
          }
        }
      }
    }
  }
  return 0;
}

int ref_forward(int n_instr, const int* op, const int* i0, const int* i1, const int* i2,
                const double* d, int sz_w, int n_in, const int* nnz_in, const int* nnz_out,
                long n, int nfwd, const double* const* arg, const double* const* fseed,
                double* const* fsens) {
  return forward_impl(n_instr, op, i0, i1, i2, d, sz_w, n_in, nnz_in, nnz_out, n, nfwd, false,
                      arg, fseed, fsens);
}

int ref_jacobian(int n_instr, const int* op, const int* i0, const int* i1, const int* i2,
                 const double* d, int sz_w, int n_in, const int* nnz_in, const int* nnz_out,
                 long n, const double* const* arg, double* const* jac) {
  int nz = 0;
  for (int j = 0; j < n_in; ++j) nz += nnz_in[j];
  return forward_impl(n_instr, op, i0, i1, i2, d, sz_w, n_in, nnz_in, nnz_out, n, nz, true, arg,
                      nullptr, jac);
}

int ref_reverse(int n_instr, const int* op, const int* i0, const int* i1, const int* i2,
                const double* d, int sz_w, int n_in, const int* nnz_in, const int* nnz_out,
                long n, int nadj, const double* const* arg, const double* const* aseed,
                double* const* asens) {
  std::vector<double> w(sz_w > 0 ? sz_w : 1), wb(sz_w > 0 ? sz_w : 1), dp(2 * n_instr + 2);
  std::vector<char> act(sz_w > 0 ? sz_w : 1);
  for (long i = 0; i < n; ++i) {
    partials(n_instr, op, i0, i1, i2, d, n, i, arg, w, dp);
    for (int dir = 0; dir < nadj; ++dir) {
      std::fill(wb.begin(), wb.end(), 0.0);
      std::fill(act.begin(), act.end(), 0);
      for (int j = 0; j < n_in; ++j) {
        if (!asens[j]) continue;
        for (int k = 0; k < nnz_in[j]; ++k) asens[j][(dir * nnz_in[j] + k) * n + i] = 0;
      }
      for (int k = n_instr - 1; k >= 0; --k) {
        const double* p = &dp[2 * k];
        switch (op[k]) {
          case OP_INPUT:
            if (asens[i1[k]])
              asens[i1[k]][(dir * nnz_in[i1[k]] + i2[k]) * n + i] = act[i0[k]] ? wb[i0[k]] : 0;
            wb[i0[k]] = 0;
            act[i0[k]] = 0;
            break;
          case OP_OUTPUT:
            if (aseed[i0[k]]) {
              double v = aseed[i0[k]][(dir * nnz_out[i0[k]] + i2[k]) * n + i];
              wb[i1[k]] = act[i1[k]] ? wb[i1[k]] + v : v;
              act[i1[k]] = 1;
            }
            break;
          case OP_CONST: case OP_PARAMETER: wb[i0[k]] = 0; act[i0[k]] = 0; break;
          default: {
            if (!act[i0[k]]) break;
            double seed = wb[i0[k]], c;
            wb[i0[k]] = 0;
            act[i0[k]] = 0;
            if (!const_zero_partial(op[k], 0)) {
              c = p[0] * seed;
              wb[i1[k]] = act[i1[k]] ? wb[i1[k]] + c : c;
              act[i1[k]] = 1;
            }
            if (casadi_math<double>::ndeps(op[k]) == 2 && !const_zero_partial(op[k], 1)) {
              c = op[k] == OP_IF_ELSE_ZERO ? if_else_zero(p[1], seed) : p[1] * seed;
              wb[i2[k]] = act[i2[k]] ? wb[i2[k]] + c : c;
              act[i2[k]] = 1;
            }
          }
        }
      }
    }
  }
  return 0;
}

}  // extern "C"
