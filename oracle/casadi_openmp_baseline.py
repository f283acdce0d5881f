"""ORACLE -- test infrastructure only: CasADi's own Map "openmp" against the oracle port.

Times, on this host's cores, the reference's libcasadi (built from the reference sources by
oracle/Makefile, with the OpenMP map and without the per-call memory mutex) through the raw
operator() of f.map(N, "openmp") (casadi/core/map.cpp:340-386, one checkout, one warm-up call,
the median of the timed calls), next to the oracle's restatement of the same step on the same
threads. The step of each workload is the benchmark's:

  cartpole: the RK4 step, values only;
  rollout:  the Jacobian of xN (jacobian() of the rollout with xN as its only output) +
            F.reverse(1) (seed on the cost); the oracle twice: CasADi's algorithm restated
            (those two derivative tapes, as CasADi built them, on the oracle's restatement of
            SXFunction::eval) and the GPU's algorithm (one record, unit-seed Jacobian by 24
            forward directions, adjoint);
  dag:      values + F.reverse(1) (seed on every output).

Usage: python -m oracle.casadi_openmp_baseline [instances_scale]   (prints JSON)
The GPU benchmark cannot run this (the reference library exists only where its sources are);
the figures calibrate the oracle port that the benchmark's CPU legs time there.
"""
import json
import os
import statistics
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from casadi_gb300 import workloads as W  # noqa: E402
from oracle import casadi_ref as R  # noqa: E402


def _median_port(fn, reps):
    fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def main(scale=1.0, reps=5, rounds=7):
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    out = {"threads": threads, "host_cpus": os.cpu_count(), "casadi_version": R.version(),
           "workloads": {}}

    n = int(65536 * scale)
    f = R.build("cartpole")
    args = W.cartpole_inputs(n, steps=1, seed=0)
    sec, _ = f.time_map(args, n, "openmp", reps)
    tape = W.cartpole_step().tape
    port = _median_port(lambda: O.eval(tape, args, n, threads), reps)
    out["workloads"]["cartpole"] = {"instances": n, "casadi_openmp_evals_per_s": n / np.median(sec),
                                    "port_evals_per_s": n / port}

    n = int(16384 * scale)
    F = R.build("rollout", 20)
    args = W.cartpole_inputs(n, steps=20, seed=0)
    J, B = R.build("rollout_xn", 20).jacobian(), F.reverse(1)
    seeds = [np.zeros((4, n)), np.ones((1, n))]
    tape = W.cartpole_rollout(20).tape
    port = _median_port(lambda: O.jacobian_reverse(
        tape, args, [np.zeros((1, 4, n)), np.ones((1, 1, n))], n, threads), reps)
    from casadi_gb300 import calculus as C
    from casadi_gb300 import sx as S
    op, i0, i1, i2, d = J.tape()
    c = op == C.OP_CONST
    jt = S.Tape(op, i0, np.where(c, 0, i1), np.where(c, 0, i2), np.where(c, d, 0.0), J.nnz_in,
                J.nnz_out, J.sz_w)
    bt = S.reverse_function(W.cartpole_rollout(20)).tape
    # CasADi and the restatement alternate in rounds (the host is shared: its speed drifts);
    # the factor between them is the median of the rounds' ratios
    sj, sb, rest, ratios = [], [], [], []
    for _ in range(rounds):
        tj, _ = J.time_map(list(args) + [None], n, "openmp", reps)
        tb, _ = B.time_map(list(args) + [None, None] + seeds, n, "openmp", reps)
        tr = _median_port(lambda: (O.eval(jt, list(args) + [None], n, threads),
                                   O.eval(bt, list(args) + [None, None] + seeds, n,
                                          threads)), reps)
        sj.append(np.median(tj))
        sb.append(np.median(tb))
        rest.append(tr)
        ratios.append(tr / (sj[-1] + sb[-1]))
    restated = float(np.median(rest))
    out["workloads"]["rollout"] = {
        "instances": n, "casadi_openmp_evals_per_s": n / (np.median(sj) + np.median(sb)),
        "casadi_jacobian_s": float(np.median(sj)), "casadi_reverse_s": float(np.median(sb)),
        "casadi_algorithm_restated_evals_per_s": n / restated,
        "casadi_over_restated_rounds": [float(r) for r in ratios],
        "port_evals_per_s": n / port}

    n = int(4096 * scale)
    op, a, b = W.dag_nodes(64, 10000, 0, 256)
    G = R.build_dag(64, 16, op, a, b)
    args = W.dag_inputs(n, n_in=64, seed=0)
    GB = G.reverse(1)
    sb, _ = GB.time_map(list(args) + [None, np.ones((16, n))], n, "openmp", reps)
    tape = W.random_dag().tape
    port = _median_port(lambda: O.reverse(tape, args, [np.ones((1, 16, n))], n, threads), reps)
    out["workloads"]["dag"] = {"instances": n, "casadi_openmp_evals_per_s": n / np.median(sb),
                               "port_evals_per_s": n / port}
    for w in out["workloads"].values():
        w["port_over_casadi"] = w["port_evals_per_s"] / w["casadi_openmp_evals_per_s"]
        if "casadi_over_restated_rounds" in w:
            w["casadi_over_restated"] = float(np.median(w["casadi_over_restated_rounds"]))
    return out


if __name__ == "__main__":
    if not R.available():
        raise SystemExit("libcasadi not built (oracle/Makefile: make casadi REF=<tree>)")
    print(json.dumps(main(float(sys.argv[1]) if len(sys.argv) > 1 else 1.0), indent=1))
