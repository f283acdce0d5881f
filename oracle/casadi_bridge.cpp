/* ORACLE — test infrastructure only.
 *
 * A ctypes bridge to the reference's own libcasadi (compiled from the reference's
 * casadi/core sources by oracle/Makefile into oracle/_ref/). The golden-fixture generator
 * (tests/golden/make_golden.py), the CPU tests that run where the library is built, and the
 * dev-host CasADi timing use it; the product never does.
 *
 * What it gives access to, all through CasADi's own code:
 *   - the workload Functions built with CasADi's SX (cart-pole RK4 step, n-step rollout,
 *     random DAG from a node list, quadcopter multiple-shooting Lagrangian), written with the
 *     same operation order as casadi_gb300/workloads.py so the two builders can be compared
 *     instruction for instruction;
 *   - the raw algorithm tape of an SXFunction (SXFunction::algorithm_,
 *     casadi/core/sx_function.hpp:258; ScalarAtomic layout :37-44);
 *   - derived Functions: jacobian() (function.cpp / function_internal.cpp:2403-2442),
 *     forward(n), reverse(n) (function_internal.cpp:2285-2340), SX gradient / hessian /
 *     jacobian Functions (matrix_impl.hpp:2831-2850);
 *   - numeric evaluation through the raw operator()(const double**, double**, casadi_int*,
 *     double*, int) (function.hpp), one instance per call, instance-major buffers;
 *   - bvec_t sparsity sweeps through operator()(const bvec_t**, ...) and rev(...)
 *     (function.cpp:1243-1258), Jacobian sparsity jac_sparsity(), get_partition's seed
 *     colourings (function_internal.cpp:2068-2160), Sparsity::uni_coloring / star_coloring;
 *   - timing of Map "openmp" / "serial" through the raw operator() (map.cpp:340-386).
 *
 * Status convention as casadi_c.cpp:320-332: 0 ok, -1 bad id, -2 std::exception (text from
 * cb_last_error), -3 unknown exception.
 */
#include <casadi/casadi.hpp>
#include <casadi/core/function_internal.hpp>
#include <casadi/core/sx_function.hpp>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

using namespace casadi;

namespace {

std::vector<Function> g_funs;
std::string g_err;

#define CB_TRY try {
#define CB_CATCH                                      \
  }                                                   \
  catch (std::exception & e) {                        \
    g_err = e.what();                                 \
    return -2;                                        \
  }                                                   \
  catch (...) {                                       \
    g_err = "unknown exception";                      \
    return -3;                                        \
  }

int put(const Function& f) {
  g_funs.push_back(f);
  return static_cast<int>(g_funs.size()) - 1;
}

const Function* get(int h) {
  if (h < 0 || h >= static_cast<int>(g_funs.size())) return nullptr;
  return &g_funs[h];
}

// ---- workload builders (operation order as casadi_gb300/workloads.py) -------------------

struct Cartpole { double mc = 1.0, mp = 0.1, l = 0.5, g = 9.81, dt = 0.02; };

std::vector<SXElem> cartpole_ode(const std::vector<SXElem>& x, const SXElem& u) {
  const Cartpole p;
  SXElem th = x[2], om = x[3];
  SXElem s = sin(th);
  SXElem c = cos(th);
  SXElem den = p.mc + p.mp * s * s;
  SXElem acc = (u + p.mp * s * (p.l * om * om + p.g * c)) / den;
  SXElem alpha = (-u * c - p.mp * p.l * om * om * c * s - (p.mc + p.mp) * p.g * s) / (p.l * den);
  return {x[1], acc, om, alpha};
}

struct Quad { double m = 1.0, Ixx = 0.01, Iyy = 0.01, Izz = 0.02, g = 9.81, dt = 0.05; };

std::vector<SXElem> quad_ode(const std::vector<SXElem>& x, const std::vector<SXElem>& u) {
  const Quad p;
  SXElem phi = x[6], th = x[7], psi = x[8];
  SXElem pr = x[9], qr = x[10], rr = x[11];
  SXElem T = u[0];
  SXElem cphi = cos(phi), sphi = sin(phi);
  SXElem cth = cos(th), sth = sin(th);
  SXElem cpsi = cos(psi), spsi = sin(psi);
  SXElem ax = T / p.m * (cphi * sth * cpsi + sphi * spsi);
  SXElem ay = T / p.m * (cphi * sth * spsi - sphi * cpsi);
  SXElem az = T / p.m * (cphi * cth) - p.g;
  SXElem tth = sth / cth;
  SXElem dphi = pr + (qr * sphi + rr * cphi) * tth;
  SXElem dth = qr * cphi - rr * sphi;
  SXElem dpsi = (qr * sphi + rr * cphi) / cth;
  SXElem dp = (u[1] + (p.Iyy - p.Izz) * qr * rr) / p.Ixx;
  SXElem dq = (u[2] + (p.Izz - p.Ixx) * pr * rr) / p.Iyy;
  SXElem dr = (u[3] + (p.Ixx - p.Iyy) * pr * qr) / p.Izz;
  return {x[3], x[4], x[5], ax, ay, az, dphi, dth, dpsi, dp, dq, dr};
}

template <class Ode>
std::vector<SXElem> rk4_step(const std::vector<SXElem>& x, Ode ode, double dt) {
  auto axpy = [&](const std::vector<SXElem>& k, double h) {
    std::vector<SXElem> r(x.size());
    for (size_t i = 0; i < x.size(); ++i) r[i] = x[i] + h * k[i];
    return r;
  };
  std::vector<SXElem> k1 = ode(x);
  std::vector<SXElem> k2 = ode(axpy(k1, dt / 2));
  std::vector<SXElem> k3 = ode(axpy(k2, dt / 2));
  std::vector<SXElem> k4 = ode(axpy(k3, dt));
  std::vector<SXElem> r(x.size());
  for (size_t i = 0; i < x.size(); ++i)
    r[i] = x[i] + dt / 6 * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
  return r;
}

std::vector<SXElem> elems(const SX& v) { return v.nonzeros(); }

Function build_cartpole_step() {
  SX x = SX::sym("x", 4), u = SX::sym("u");
  SXElem ue = u.nonzeros()[0];
  std::vector<SXElem> xn = rk4_step(elems(x), [&](const std::vector<SXElem>& s) {
    return cartpole_ode(s, ue); }, Cartpole().dt);
  return Function("f", {x, u}, {SX(xn)});
}

Function build_rollout(int steps) {
  SX x0 = SX::sym("x0", 4), U = SX::sym("U", steps);
  std::vector<SXElem> x = elems(x0), u = elems(U);
  SXElem cost = 0;
  for (int k = 0; k < steps; ++k) {
    cost = cost + (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3]) + 0.01 * u[k] * u[k];
    SXElem uk = u[k];
    x = rk4_step(x, [&](const std::vector<SXElem>& s) { return cartpole_ode(s, uk); },
                 Cartpole().dt);
  }
  return Function("F", {x0, U}, {SX(x), SX(cost)});
}

// The rollout's final state alone, F(x0, U) -> xN (the same operations as build_rollout
// without the cost): its jacobian() is CasADi's own Jacobian of xN.
Function build_rollout_xn(int steps) {
  SX x0 = SX::sym("x0", 4), U = SX::sym("U", steps);
  std::vector<SXElem> x = elems(x0), u = elems(U);
  for (int k = 0; k < steps; ++k) {
    SXElem uk = u[k];
    x = rk4_step(x, [&](const std::vector<SXElem>& s) { return cartpole_ode(s, uk); },
                 Cartpole().dt);
  }
  return Function("FxN", {x0, U}, {SX(x)});
}

// The rollout as never-inlined calls of the step Function: one OP_CALL per step
// (Function::call(..., never_inline=true), sx_function.cpp:630-661 for the tape records).
Function build_rollout_calls(int steps) {
  Function f = build_cartpole_step();
  SX x0 = SX::sym("x0", 4), U = SX::sym("U", steps);
  SX x = x0;
  for (int k = 0; k < steps; ++k) {
    std::vector<SX> res;
    f.call(std::vector<SX>{x, U(k)}, res, false, true);
    x = res.at(0);
  }
  return Function("F_calls", {x0, U}, {x});
}

// op codes of the node list: index into add, sub, mul, div, sin, cos, exp, log, sqrt, tanh
Function build_dag(int n_in, int n_nodes, int n_out, const int* op, const int* a,
                   const int* b, int bounded) {
  SX xs = SX::sym("x", n_in);
  std::vector<SXElem> nodes = elems(xs);
  for (int k = n_in; k < n_nodes; ++k) {
    const SXElem& A = nodes.at(a[k - n_in]);
    const SXElem& B = nodes.at(b[k - n_in]);
    SXElem e;
    switch (op[k - n_in]) {
      case 0: e = bounded ? 0.5 * (A + B) : A + B; break;
      case 1: e = bounded ? 0.5 * (A - B) : A - B; break;
      case 2: e = bounded ? A * tanh(B) : A * B; break;
      case 3: e = A / (sq(B) + 1.0); break;
      case 4: e = sin(A); break;
      case 5: e = cos(A); break;
      case 6: { double c = bounded ? 1.0 : 5.0; e = exp(fmin(fmax(A, -c), c)); break; }
      case 7: e = log(fabs(A) + 1.0); break;
      case 8: e = sqrt(sq(A) + 1.0); break;
      case 9: e = tanh(A); break;
      default: throw CasadiException("dag: bad op code");
    }
    nodes.push_back(e);
  }
  std::vector<SXElem> outs(nodes.end() - n_out, nodes.end());
  return Function("G", {xs}, {SX(outs)});
}

struct QuadNlp { SX w, lam, x0bar, g, lag; };

QuadNlp quad_nlp(int K) {
  const int nx = 12, nu = 4;
  QuadNlp r;
  r.w = SX::sym("w", K * (nx + nu) + nx);
  r.x0bar = SX::sym("x0", nx);
  std::vector<SXElem> w = elems(r.w), xb = elems(r.x0bar);
  auto xs = [&](int k) { return std::vector<SXElem>(w.begin() + k * (nx + nu),
                                                    w.begin() + k * (nx + nu) + nx); };
  auto us = [&](int k) { return std::vector<SXElem>(w.begin() + k * (nx + nu) + nx,
                                                    w.begin() + k * (nx + nu) + nx + nu); };
  std::vector<SXElem> g;
  std::vector<SXElem> x0 = xs(0);
  for (int i = 0; i < nx; ++i) g.push_back(x0[i] - xb[i]);
  SXElem obj = 0;
  for (int k = 0; k < K; ++k) {
    std::vector<SXElem> xk = xs(k), uk = us(k), xk1 = xs(k + 1);
    std::vector<SXElem> xn = rk4_step(xk, [&](const std::vector<SXElem>& s) {
      return quad_ode(s, uk); }, Quad().dt);
    for (int i = 0; i < nx; ++i) g.push_back(xn[i] - xk1[i]);
    SXElem sx = 0, su = 0;
    for (const SXElem& xi : xk) sx = sx + xi * xi;
    for (const SXElem& ui : uk) su = su + ui * ui;
    obj = obj + sx + 0.1 * su;
  }
  r.lam = SX::sym("lam", static_cast<casadi_int>(g.size()));
  std::vector<SXElem> lam = elems(r.lam);
  SXElem lag = obj;
  for (size_t i = 0; i < g.size(); ++i) lag = lag + lam[i] * g[i];
  r.g = SX(g);
  r.lag = SX(lag);
  return r;
}

// Copies the pattern of a Sparsity into caller buffers (two-call protocol on nnz).
void put_sparsity(const Sparsity& sp, int* nrow, int* ncol, int* nnz, int* colind, int* row,
                  int cap) {
  *nrow = static_cast<int>(sp.size1());
  *ncol = static_cast<int>(sp.size2());
  *nnz = static_cast<int>(sp.nnz());
  if (colind && row && cap >= sp.nnz()) {
    const casadi_int* ci = sp.colind();
    const casadi_int* r = sp.row();
    for (casadi_int j = 0; j <= sp.size2(); ++j) colind[j] = static_cast<int>(ci[j]);
    for (casadi_int k = 0; k < sp.nnz(); ++k) row[k] = static_cast<int>(r[k]);
  }
}

Sparsity make_sparsity(int nrow, int ncol, const int* colind, const int* row) {
  std::vector<casadi_int> ci(colind, colind + ncol + 1);
  std::vector<casadi_int> r(row, row + colind[ncol]);
  return Sparsity(nrow, ncol, ci, r);
}

// The colour of every column from a seed-matrix Sparsity (column j of colour c is the
// nonzero at row j of column c, the form both colourings return).
int colors_of(const Sparsity& D, int* color) {
  const casadi_int* ci = D.colind();
  const casadi_int* r = D.row();
  for (casadi_int c = 0; c < D.size2(); ++c)
    for (casadi_int k = ci[c]; k < ci[c + 1]; ++k) color[r[k]] = static_cast<int>(c);
  return static_cast<int>(D.size2());
}

}  // namespace

extern "C" {

const char* cb_last_error() { return g_err.c_str(); }

int cb_version(int* major, int* minor, int* patch) {
  *major = CASADI_MAJOR_VERSION; *minor = CASADI_MINOR_VERSION; *patch = CASADI_PATCH_VERSION;
  return 0;
}

int cb_build(const char* name, int param) {
  CB_TRY
  std::string n(name);
  if (n == "cartpole") return put(build_cartpole_step());
  if (n == "rollout") return put(build_rollout(param));
  QuadNlp q;
  if (n.rfind("quad_", 0) == 0) q = quad_nlp(param);
  if (n == "quad_lagrangian") return put(Function("L", {q.w, q.lam, q.x0bar}, {q.g, q.lag}));
  if (n == "quad_gradient")
    return put(Function("grad_L", {q.w, q.lam, q.x0bar}, {gradient(q.lag, q.w)}));
  if (n == "quad_hessian")
    return put(Function("hess_L", {q.w, q.lam, q.x0bar}, {hessian(q.lag, q.w)}));
  if (n == "quad_jac_g")
    return put(Function("jac_g", {q.w, q.lam, q.x0bar}, {jacobian(q.g, q.w)}));
  // the temporary Functions SX::jacobian / SX::hessian colour (sx_instantiator.cpp)
  Dict free{{"allow_free", true}};
  if (n == "quad_g_helper") return put(Function("jac_helper", {q.w}, {q.g}, free));
  if (n == "quad_grad_helper")
    return put(Function("jac_helper", {q.w}, {gradient(q.lag, q.w)}, free));
  if (n == "rollout_calls") return put(build_rollout_calls(param));
  if (n == "rollout_xn") return put(build_rollout_xn(param));
  g_err = "unknown workload " + n;
  return -2;
  CB_CATCH
}

int cb_build_dag(int n_in, int n_nodes, int n_out, const int* op, const int* a, const int* b,
                 int bounded) {
  CB_TRY
  return put(build_dag(n_in, n_nodes, n_out, op, a, b, bounded));
  CB_CATCH
}

/* kind: "jacobian" -> f.jacobian(); "forward" -> f.forward(k); "reverse" -> f.reverse(k). */
int cb_derive(int h, const char* kind, int k) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  std::string s(kind);
  if (s == "jacobian") return put(f->jacobian());
  if (s == "forward") return put(f->forward(k));
  if (s == "reverse") return put(f->reverse(k));
  g_err = "unknown derivative kind " + s;
  return -2;
  CB_CATCH
}

int cb_io(int h, int* n_in, int* n_out, int* nnz_in, int* nnz_out, int* sz_w, int* n_instr) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  *n_in = static_cast<int>(f->n_in());
  *n_out = static_cast<int>(f->n_out());
  if (nnz_in) for (casadi_int j = 0; j < f->n_in(); ++j) nnz_in[j] = f->nnz_in(j);
  if (nnz_out) for (casadi_int j = 0; j < f->n_out(); ++j) nnz_out[j] = f->nnz_out(j);
  *sz_w = static_cast<int>(f->sz_w());
  *n_instr = f->is_a("SXFunction") ? static_cast<int>(f->n_instructions()) : -1;
  return 0;
  CB_CATCH
}

/* The pattern of input j (in) or output j (out). */
int cb_io_sparsity(int h, int out, int j, int* nrow, int* ncol, int* nnz, int* colind,
                   int* row, int cap) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  put_sparsity(out ? f->sparsity_out(j) : f->sparsity_in(j), nrow, ncol, nnz, colind, row, cap);
  return 0;
  CB_CATCH
}

/* The raw algorithm: SXFunction::algorithm_ element by element. */
int cb_tape(int h, int* op, int* i0, int* i1, int* i2, double* d) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  const SXFunction* s = dynamic_cast<const SXFunction*>(f->get());
  if (!s) { g_err = "not an SXFunction"; return -2; }
  for (size_t k = 0; k < s->algorithm_.size(); ++k) {
    const auto& e = s->algorithm_[k];
    op[k] = e.op; i0[k] = e.i0; i1[k] = e.i1; i2[k] = e.i2; d[k] = e.d;
  }
  return 0;
  CB_CATCH
}

/* Call records of an SXFunction with OP_CALL instructions (SXFunction::call_.el): the
 * count, then per record the callee (registered, its handle returned) and the work-vector
 * slots of its argument and result nonzeros (dep: sum of callee nnz_in, res: of nnz_out;
 * -1 for a result that is not used). */
int cb_n_calls(int h) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  const SXFunction* s = dynamic_cast<const SXFunction*>(f->get());
  if (!s) { g_err = "not an SXFunction"; return -2; }
  return static_cast<int>(s->call_.el.size());
  CB_CATCH
}

int cb_call_info(int h, int e, int* callee, int* dep, int* res) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  const SXFunction* s = dynamic_cast<const SXFunction*>(f->get());
  if (!s || e < 0 || e >= static_cast<int>(s->call_.el.size())) return -1;
  const auto& m = s->call_.el[e];
  *callee = put(m.f);
  for (size_t k = 0; k < m.dep.size(); ++k) dep[k] = m.dep[k];
  for (size_t k = 0; k < m.res.size(); ++k) res[k] = m.res[k];
  return 0;
  CB_CATCH
}

/* Function::serialize() text; returns its length, writes it when cap allows. */
int cb_serialize(int h, char* buf, int cap) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  std::string t = f->serialize();
  if (buf && cap >= static_cast<int>(t.size())) std::memcpy(buf, t.data(), t.size());
  return static_cast<int>(t.size());
  CB_CATCH
}

/* n instances, one raw call each. arg[j]: n x nnz_in(j) doubles, instance-major (null:
 * zeros); res[j]: n x nnz_out(j) (null: skipped). */
int cb_eval(int h, int n, const double* const* arg, double* const* res) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  casadi_int n_in = f->n_in(), n_out = f->n_out();
  std::vector<const double*> a(f->sz_arg());
  std::vector<double*> r(f->sz_res());
  std::vector<casadi_int> iw(f->sz_iw());
  std::vector<double> w(f->sz_w());
  for (int i = 0; i < n; ++i) {
    for (casadi_int j = 0; j < n_in; ++j)
      a[j] = arg[j] ? arg[j] + static_cast<size_t>(i) * f->nnz_in(j) : nullptr;
    for (casadi_int j = 0; j < n_out; ++j)
      r[j] = res[j] ? res[j] + static_cast<size_t>(i) * f->nnz_out(j) : nullptr;
    if ((*f)(a.data(), r.data(), iw.data(), w.data(), 0)) {
      g_err = "evaluation failed";
      return -2;
    }
  }
  return 0;
  CB_CATCH
}

/* One bvec_t sweep (64 directions). fwd: operator()(const bvec_t**, bvec_t**, ...) with
 * arg = seeds, res = results. Reverse: rev(bvec_t** arg, bvec_t** res, ...) with res = seeds
 * (consumed) and arg |= results. */
int cb_sp(int h, int fwd, uint64_t* const* arg, uint64_t* const* res) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  static_assert(sizeof(bvec_t) == sizeof(uint64_t), "bvec_t is 64 bits");
  std::vector<bvec_t*> a(f->sz_arg()), r(f->sz_res());
  for (casadi_int j = 0; j < f->n_in(); ++j) a[j] = reinterpret_cast<bvec_t*>(arg[j]);
  for (casadi_int j = 0; j < f->n_out(); ++j) r[j] = reinterpret_cast<bvec_t*>(res[j]);
  std::vector<casadi_int> iw(f->sz_iw());
  std::vector<bvec_t> w(f->sz_w());
  int flag;
  if (fwd) {
    std::vector<const bvec_t*> ac(a.begin(), a.end());
    flag = (*f)(ac.data(), r.data(), iw.data(), w.data(), 0);
  } else {
    flag = f->rev(a.data(), r.data(), iw.data(), w.data(), 0);
  }
  if (flag) { g_err = "sparsity sweep failed"; return -2; }
  return 0;
  CB_CATCH
}

int cb_jac_sparsity(int h, int oind, int iind, int* nrow, int* ncol, int* nnz, int* colind,
                    int* row, int cap) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  put_sparsity(f->jac_sparsity(oind, iind), nrow, ncol, nnz, colind, row, cap);
  return 0;
  CB_CATCH
}

/* get_partition as jacobian() calls it: fills color1 (forward seeds, -1 when none) or color2
 * (adjoint seeds) with one colour per column of the input (forward) / row of the output
 * (adjoint); returns the counts in n1/n2 (0 when that mode is not chosen). */
int cb_partition(int h, int iind, int oind, int symmetric, int* n1, int* color1, int* n2,
                 int* color2) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  Sparsity D1, D2;
  (*f)->get_partition(iind, oind, D1, D2, true, symmetric != 0, true, true);
  *n1 = D1.is_null() ? 0 : colors_of(D1, color1);
  *n2 = D2.is_null() ? 0 : colors_of(D2, color2);
  return 0;
  CB_CATCH
}

/* Sparsity::uni_coloring (kind 0) or star_coloring(ordering) (kind 1, ordering = param) or
 * star_coloring2 (kind 2) of a pattern; writes one colour per column, returns the count. */
int cb_coloring(int kind, int param, int nrow, int ncol, const int* colind, const int* row,
                int* color, int* n_colors) {
  CB_TRY
  Sparsity A = make_sparsity(nrow, ncol, colind, row);
  Sparsity D;
  if (kind == 0) D = A.uni_coloring(A.T());
  else if (kind == 1) D = A.star_coloring(param);
  else D = A.star_coloring2(param);
  *n_colors = colors_of(D, color);
  return 0;
  CB_CATCH
}

/* f.map(n, parallelization) timed through the raw operator(): one checkout, one warm-up
 * call, then reps timed calls; writes each call's seconds. */
int cb_time_map(int h, int n, const char* parallelization, int reps,
                const double* const* arg, double* const* res, double* seconds) {
  CB_TRY
  const Function* f = get(h);
  if (!f) return -1;
  Function m = f->map(n, parallelization);
  std::vector<const double*> a(m.sz_arg());
  std::vector<double*> r(m.sz_res());
  for (casadi_int j = 0; j < m.n_in(); ++j) a[j] = arg[j];
  for (casadi_int j = 0; j < m.n_out(); ++j) r[j] = res[j];
  std::vector<casadi_int> iw(m.sz_iw());
  std::vector<double> w(m.sz_w());
  int mem = m.checkout();
  int flag = m(a.data(), r.data(), iw.data(), w.data(), mem);
  for (int k = 0; k < reps && !flag; ++k) {
    auto t0 = std::chrono::steady_clock::now();
    flag = m(a.data(), r.data(), iw.data(), w.data(), mem);
    auto t1 = std::chrono::steady_clock::now();
    seconds[k] = std::chrono::duration<double>(t1 - t0).count();
  }
  m.release(mem);
  if (flag) { g_err = "map evaluation failed"; return -2; }
  return 0;
  CB_CATCH
}

}  // extern "C"
