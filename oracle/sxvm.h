/*
 * ORACLE — test infrastructure only (see sxvm.c). Operation ids are CasADi's
 * enum Operation (casadi/core/calculus.hpp:60-218).
 */
#ifndef SXVM_ORACLE_H
#define SXVM_ORACLE_H
#include <stdint.h>

enum {
  SXO_ASSIGN = 0, SXO_ADD, SXO_SUB, SXO_MUL, SXO_DIV, SXO_NEG, SXO_EXP, SXO_LOG, SXO_POW,
  SXO_CONSTPOW, SXO_SQRT, SXO_SQ, SXO_TWICE, SXO_SIN, SXO_COS, SXO_TAN, SXO_ASIN, SXO_ACOS,
  SXO_ATAN, SXO_LT, SXO_LE, SXO_EQ, SXO_NE, SXO_NOT, SXO_AND, SXO_OR, SXO_FLOOR, SXO_CEIL,
  SXO_FMOD, SXO_FABS, SXO_SIGN, SXO_COPYSIGN, SXO_IF_ELSE_ZERO, SXO_ERF, SXO_FMIN, SXO_FMAX,
  SXO_INV, SXO_SINH, SXO_COSH, SXO_TANH, SXO_ASINH, SXO_ACOSH, SXO_ATANH, SXO_ATAN2,
  SXO_CONST, SXO_INPUT, SXO_OUTPUT, SXO_PARAMETER, SXO_CALL,
  SXO_ERFINV = 86, SXO_PRINTME = 87, SXO_LIFT = 88, SXO_LOG1P = 93, SXO_EXPM1 = 94,
  SXO_HYPOT = 95, SXO_REMAINDER = 97
};

typedef struct {
  int n_instr;
  const int* op;
  const int* i0;
  const int* i1;
  const int* i2;
  const double* d;
  int n_in;
  const int* nnz_in;
  int n_out;
  const int* nnz_out;
  int sz_w;
} sxo_tape;

double sxo_fun(int op, double x, double y);
void sxo_der(int op, double x, double y, double f, double* d);
int sxo_ndeps(int op);
int sxo_eval(const sxo_tape* t, long n, const double* const* arg, double* const* res,
             int nthreads);
int sxo_forward(const sxo_tape* t, long n, int nfwd, const double* const* arg,
                double* const* res, const double* const* fseed, double* const* fsens,
                int nthreads);
int sxo_jacobian(const sxo_tape* t, long n, const double* const* arg, double* const* res,
                 double* const* jac, int nthreads);
int sxo_reverse(const sxo_tape* t, long n, int nadj, const double* const* arg,
                double* const* res, const double* const* aseed, double* const* asens,
                int nthreads);
int sxo_jacobian_reverse(const sxo_tape* t, long n, const double* const* arg,
                         double* const* res, double* const* jac, int nadj,
                         const double* const* aseed, double* const* asens, int nthreads);
int sxo_sp_forward(const sxo_tape* t, long n, const uint64_t* const* arg, uint64_t* const* res,
                   int nthreads);
int sxo_sp_reverse(const sxo_tape* t, long n, uint64_t* const* arg, uint64_t* const* res,
                   int nthreads);
int sxo_zero_checker(int which, int op);
void sxo_set_magnitude(int on);
int sxo_libm_bound(const sxo_tape* t, long n, const double* const* arg, double* const* bound,
                   int nthreads);
/* As sxo_libm_bound over every computing instruction: the first-order sensitivity of each
 * output to a relative perturbation of every rounded result, which bounds (times a few ulps)
 * the difference between two evaluations that round any instruction differently. */
int sxo_rounding_bound(const sxo_tape* t, long n, const double* const* arg,
                       double* const* bound, int nthreads);
int sxo_activity(const sxo_tape* t, long n, const uint64_t* const* arg, uint64_t* const* res,
                 int nthreads);
#endif
