"""Synthetic SX workloads: the tapes and seeded inputs the tests and the benchmark run.

* cart-pole RK4 step ``f(x[4], u) -> x_next[4]`` (mc=1.0, mp=0.1, l=0.5, g=9.81, dt=0.02);
* a ``steps``-step cart-pole rollout ``F(x0[4], U[steps]) -> (xN[4], cost)`` with
  cost = sum_k ||x_k||^2 + 0.01 u_k^2;
* a seeded random DAG (64 inputs, 10 000 nodes, 16 outputs; op mix add .25, sub .15,
  mul .25, div .05, sin .06, cos .06, exp(clip(x,-5,5)) .06, log(|x|+1) .04,
  sqrt(x^2+1) .04, tanh .04; operands drawn from the previous 256 nodes);
* a quadcopter multiple-shooting NLP (12 states, 4 inputs, RK4, 100 intervals, dt=0.05).

Inputs are drawn from seeded generators with the distributions stated for each workload.
"""
import math
import numpy as np

from . import sx as S

CARTPOLE = dict(mc=1.0, mp=0.1, l=0.5, g=9.81, dt=0.02)
X_LO = np.array([-2.0, -3.0, -math.pi, -5.0])
X_HI = np.array([2.0, 3.0, math.pi, 5.0])
U_LO, U_HI = -10.0, 10.0


def cartpole_ode(x, u, p=CARTPOLE):
    """Cart-pole dynamics; x = (position, velocity, angle, angular velocity)."""
    mc, mp, l, g = p["mc"], p["mp"], p["l"], p["g"]
    th, om = x[2], x[3]
    s = S.sin(th)
    c = S.cos(th)
    den = mc + mp * s * s
    acc = (u + mp * s * (l * om * om + g * c)) / den
    alpha = (-u * c - mp * l * om * om * c * s - (mc + mp) * g * s) / (l * den)
    return [x[1], acc, om, alpha]


def rk4_step(x, u, dt=CARTPOLE["dt"], ode=cartpole_ode):
    k1 = ode(x, u)
    k2 = ode([xi + dt / 2 * ki for xi, ki in zip(x, k1)], u)
    k3 = ode([xi + dt / 2 * ki for xi, ki in zip(x, k2)], u)
    k4 = ode([xi + dt * ki for xi, ki in zip(x, k3)], u)
    return [xi + dt / 6 * (a + 2 * b + 2 * c + d)
            for xi, a, b, c, d in zip(x, k1, k2, k3, k4)]


def cartpole_step():
    """``f(x[4], u[1]) -> x_next[4]``: one RK4 step."""
    x = S.sym("x", 4)
    u = S.sym("u")
    return S.Function("f", [x, [u]], [rk4_step(x, u)])


def cartpole_rollout(steps=20):
    """``F(x0[4], U[steps]) -> (xN[4], cost)`` with cost = sum ||x_k||^2 + 0.01 u_k^2
    over k = 0..steps-1 (x_k the state before control u_k)."""
    x0 = S.sym("x0", 4)
    U = S.sym("U", steps)
    x = list(x0)
    cost = S.const(0.0)
    for k in range(steps):
        cost = cost + (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3]) \
            + 0.01 * U[k] * U[k]
        x = rk4_step(x, U[k])
    return S.Function("F", [x0, U], [x, [cost]])


def cartpole_inputs(n, steps=1, seed=0):
    """x ~ U([-2,2]x[-3,3]x[-pi,pi]x[-5,5]), u ~ U(-10,10); instance-minor (nnz, n)."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(X_LO[:, None], X_HI[:, None], size=(4, n))
    u = rng.uniform(U_LO, U_HI, size=(steps, n))
    return [x, u]


# ---- random DAG ------------------------------------------------------------------------------
DAG_OPS = ["add", "sub", "mul", "div", "sin", "cos", "exp", "log", "sqrt", "tanh"]
DAG_P = [0.25, 0.15, 0.25, 0.05, 0.06, 0.06, 0.06, 0.04, 0.04, 0.04]


def dag_nodes(n_in=64, n_nodes=10000, seed=0, window=256):
    """The node list of the seeded random DAG: for every node k >= n_in, the index of its op
    in ``DAG_OPS`` and two operand indices drawn uniformly from the previous ``window`` nodes
    (unary ops ignore the second). Returns int32 arrays ``(op, a, b)`` of n_nodes - n_in."""
    rng = np.random.default_rng(seed)
    cum = np.cumsum(DAG_P)
    m = n_nodes - n_in
    op = np.empty(m, np.int32)
    a = np.empty(m, np.int32)
    b = np.empty(m, np.int32)
    for k in range(n_in, n_nodes):
        r = rng.random()
        op[k - n_in] = int(np.searchsorted(cum, r * cum[-1], side="right"))
        lo = max(0, k - window)
        a[k - n_in] = int(rng.integers(lo, k))
        b[k - n_in] = int(rng.integers(lo, k))
    return op, a, b


def dag_from_nodes(n_in, n_out, op, a, b, bounded=False):
    """Build the DAG of a node list (see :func:`dag_nodes`); the outputs are the last
    ``n_out`` nodes. Unary ops are guarded: exp(clip(x,-5,5)), log(|x|+1), sqrt(x^2+1). With
    ``bounded`` the sums are averaged (0.5*(a+b)), products take one tanh-squashed factor
    (a*tanh(b)) and exp is clipped to [-1, 1], which keeps every node of a deep, narrow DAG
    finite and of order one."""
    xs = S.sym("x", n_in)
    nodes = list(xs)
    for code, ia, ib in zip(op.tolist(), a.tolist(), b.tolist()):
        name = DAG_OPS[code]
        x, y = nodes[ia], nodes[ib]
        if name == "add":
            e = 0.5 * (x + y) if bounded else x + y
        elif name == "sub":
            e = 0.5 * (x - y) if bounded else x - y
        elif name == "mul":
            e = x * S.tanh(y) if bounded else x * y
        elif name == "div":
            e = x / (S.sq(y) + 1.0)
        elif name == "sin":
            e = S.sin(x)
        elif name == "cos":
            e = S.cos(x)
        elif name == "exp":
            c = 1.0 if bounded else 5.0
            e = S.exp(S.fmin(S.fmax(x, -c), c))
        elif name == "log":
            e = S.log(S.fabs(x) + 1.0)
        elif name == "sqrt":
            e = S.sqrt(S.sq(x) + 1.0)
        else:
            e = S.tanh(x)
        nodes.append(e)
    outs = nodes[-n_out:]
    return S.Function("G", [xs], [outs])


def random_dag(n_in=64, n_nodes=10000, n_out=16, seed=0, window=256, bounded=False):
    """A seeded random expression DAG: node k (k >= n_in) applies an op drawn from the mix
    above to operands drawn uniformly from the previous ``window`` nodes; the outputs are the
    last ``n_out`` nodes (:func:`dag_nodes`, :func:`dag_from_nodes`)."""
    op, a, b = dag_nodes(n_in, n_nodes, seed, window)
    return dag_from_nodes(n_in, n_out, op, a, b, bounded)


def dag_inputs(n, n_in=64, seed=0):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((n_in, n))]


def mixed_batch(n_tapes=8, total=1 << 20, seed=0, median=4096, sigma=1.5, bounded=False):
    """The mixed-size multi-tape workload: ``n_tapes`` random DAGs from the generator above
    (64 inputs, 16 outputs, operands from the previous 256 nodes) whose node counts are
    spread log-uniformly over 200..20000, and work items (tape, instance count) with counts
    drawn log-normal (median ``median``, log-sigma ``sigma``) on tapes drawn uniformly, until
    ``total`` instances. Returns ``(functions, items)`` with items ``[(tape index, n, seed)]``.
    With ``bounded`` the DAGs use the bounded op variants (finite values at any depth)."""
    rng = np.random.default_rng(seed)
    nodes = np.exp(np.linspace(np.log(200), np.log(20000), n_tapes)).astype(int)
    funs = [random_dag(n_in=64, n_nodes=int(nodes[k]), n_out=16, seed=seed * 100 + k,
                       window=256, bounded=bounded) for k in range(n_tapes)]
    items = []
    left = total
    while left > 0:
        n = int(min(left, max(1, round(rng.lognormal(np.log(median), sigma)))))
        items.append((int(rng.integers(n_tapes)), n, seed * 100000 + len(items)))
        left -= n
    return funs, items


# ---- quadcopter multiple shooting -----------------------------------------------------------
QUAD = dict(m=1.0, Ixx=0.01, Iyy=0.01, Izz=0.02, g=9.81, dt=0.05)


def quad_ode(x, u, p=QUAD):
    """Quadcopter with thrust/torque inputs u = (T, tau_x, tau_y, tau_z);
    x = (px, py, pz, vx, vy, vz, phi, theta, psi, p, q, r)."""
    m, Ixx, Iyy, Izz, g = p["m"], p["Ixx"], p["Iyy"], p["Izz"], p["g"]
    phi, th, psi = x[6], x[7], x[8]
    pr, qr, rr = x[9], x[10], x[11]
    T = u[0]
    cphi, sphi = S.cos(phi), S.sin(phi)
    cth, sth = S.cos(th), S.sin(th)
    cpsi, spsi = S.cos(psi), S.sin(psi)
    ax = T / m * (cphi * sth * cpsi + sphi * spsi)
    ay = T / m * (cphi * sth * spsi - sphi * cpsi)
    az = T / m * (cphi * cth) - g
    tth = sth / cth
    dphi = pr + (qr * sphi + rr * cphi) * tth
    dth = qr * cphi - rr * sphi
    dpsi = (qr * sphi + rr * cphi) / cth
    dp = (u[1] + (Iyy - Izz) * qr * rr) / Ixx
    dq = (u[2] + (Izz - Ixx) * pr * rr) / Iyy
    dr = (u[3] + (Ixx - Iyy) * pr * qr) / Izz
    return [x[3], x[4], x[5], ax, ay, az, dphi, dth, dpsi, dp, dq, dr]


def quad_ms_constraints(intervals=100):
    """The constraints of :func:`quad_ms_lagrangian` alone: ``g(w, lam, x0bar)`` (``lam`` is
    unused; same inputs so the same scenario arrays serve both)."""
    L = quad_ms_lagrangian(intervals)
    return S.Function("g", L.inputs, [L.outputs[0]])


def quad_ms_nlp(intervals=100):
    """The multiple-shooting NLP as SX expressions: decision vector w = (x_0, u_0, ...,
    x_{K-1}, u_{K-1}, x_K) with 12 + 4 variables per interval, parameter x0bar (initial
    state), constraints g_k = F(x_k, u_k) - x_{k+1} (and x_0 - x0bar), objective
    sum ||x_k||^2 + 0.1 ||u_k||^2. Returns ``(w, x0bar, objective, g)``."""
    nx, nu = 12, 4
    K = intervals
    w = S.sym("w", K * (nx + nu) + nx)
    x0bar = S.sym("x0", nx)
    xs = [w[k * (nx + nu): k * (nx + nu) + nx] for k in range(K + 1)]
    us = [w[k * (nx + nu) + nx: k * (nx + nu) + nx + nu] for k in range(K)]
    g = [xs[0][i] - x0bar[i] for i in range(nx)]
    obj = S.const(0.0)
    for k in range(K):
        xn = rk4_step(xs[k], us[k], dt=QUAD["dt"], ode=lambda x, u: quad_ode(x, u))
        g += [xn[i] - xs[k + 1][i] for i in range(nx)]
        obj = obj + sum((xi * xi for xi in xs[k]), S.const(0.0)) + \
            0.1 * sum((ui * ui for ui in us[k]), S.const(0.0))
    return w, x0bar, obj, g


def quad_ms_lagrangian(intervals=100):
    """The Lagrangian of :func:`quad_ms_nlp` with multipliers lam (one per constraint):
    Function ``L(w, lam, x0bar) -> (g, objective + lam'g)``."""
    w, x0bar, obj, g = quad_ms_nlp(intervals)
    lam = S.sym("lam", len(g))
    lag = obj
    for i, gi in enumerate(g):
        lag = lag + lam[i] * gi
    return S.Function("L", [w, lam, x0bar], [g, [lag]])


def quad_ms_inputs(n, intervals=100, seed=0):
    """Scenario inputs of :func:`quad_ms_lagrangian` for n instances (instance-minor):
    initial states with positions ~ U(-1, 1) m and angles ~ U(-0.5, 0.5) rad (velocities and
    rates zero); the decision vector perturbs that state along the horizon (positions
    U(-1, 1), velocities U(-0.5, 0.5), angles U(-0.5, 0.5), rates U(-0.5, 0.5); thrust
    m*g + U(-1, 1), torques U(-0.05, 0.05)); multipliers ~ N(0, 1)."""
    rng = np.random.default_rng(seed)
    nx, nu, K = 12, 4, intervals
    lo_x = np.array([-1, -1, -1, -.5, -.5, -.5, -.5, -.5, -.5, -.5, -.5, -.5])
    hi_x = -lo_x
    x0 = np.zeros((nx, n))
    x0[0:3] = rng.uniform(-1, 1, (3, n))
    x0[6:9] = rng.uniform(-0.5, 0.5, (3, n))
    w = np.empty((K * (nx + nu) + nx, n))
    hover = QUAD["m"] * QUAD["g"]
    for k in range(K + 1):
        o = k * (nx + nu)
        w[o:o + nx] = rng.uniform(lo_x[:, None], hi_x[:, None], (nx, n))
        if k < K:
            w[o + nx] = hover + rng.uniform(-1, 1, n)
            w[o + nx + 1:o + nx + nu] = rng.uniform(-0.05, 0.05, (nu - 1, n))
    lam = rng.standard_normal(((K + 1) * nx, n))
    return [w, lam, x0]

