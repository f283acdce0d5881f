"""Benchmark: SX tape sweeps over many instances on one GB300.

Workload (default): the cart-pole 20-step RK4 rollout F(x0[4], U[20]) -> (xN[4], cost),
N = 262144 instances, FP64. One step = the forward-mode Jacobian of all outputs w.r.t. the
24 inputs (values + 24 unit directions) plus the adjoint of the cost (values + 1 adjoint
direction), over all N instances. `value` is instances per second for that step with inputs
resident in HBM; `e2e` is the same step through the C ABI's host-buffer Map entry points
(casadi_gb300_map_jacobian + casadi_gb300_map_reverse) with pinned host buffers, host<->device
copies inside the timed region.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
                       [--workload rollout20|cartpole|dag|mixed|mpc]
For N > 1 (torchrun) every rank runs an independent replica on its own instances (the path
has no exchange step); rank 0 prints the max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SX tape evals/s & adjoint evals/s per GB300 vs plain kernel; % FP64/HBM roof"
UNIT = "evals/s"
L2_FLUSH_BYTES = 256 << 20


# ---- workloads -------------------------------------------------------------------------------
def make_workload(name, instances=None):
    from casadi_gb300 import workloads as W
    if name == "rollout20":
        F = W.cartpole_rollout(20)
        n = instances or 262144
        args = W.cartpole_inputs(n, steps=20, seed=0)
        desc = "cart-pole 20-step RK4 rollout F(x0[4],U[20])->(xN[4],cost), N=%d: " \
               "forward Jacobian of xN (24 unit directions) + adjoint of cost" % n
        return F, n, args, [np.zeros((1, 4, n)), np.ones((1, 1, n))], desc
    if name == "cartpole":
        F = W.cartpole_step()
        n = instances or 65536
        args = W.cartpole_inputs(n, steps=1, seed=0)
        return F, n, args, [np.ones((1, 4, n))], "cart-pole RK4 step, N=%d" % n
    if name == "dag":
        F = W.random_dag()
        n = instances or 16384
        args = W.dag_inputs(n)
        return F, n, args, [np.ones((1, 16, n))], \
            "random DAG 64in/10000 nodes/16out, N=%d: eval + adjoint of the sum of outputs + " \
            "sp_forward + sp_reverse" % n
    raise SystemExit("unknown workload " + name)


# ---- algorithmic work per instance --------------------------------------------------------------
# Counted in FP64-pipe instructions (DADD, DMUL and DFMA each count one; a libm call counts its
# measured DFMA-instruction equivalents from op_weights.json), split by kind: on GB300 the pipe
# issues a DFMA chain at a higher rate than DADD or DMUL (casadi_gb300_fp64_rate, measured in the
# same run), so each kernel's ceiling is the rate of its own instruction mix.
def _carries(op):
    from casadi_gb300 import calculus as C
    zero_d0 = {C.OP_LT, C.OP_LE, C.OP_EQ, C.OP_NE, C.OP_NOT, C.OP_AND, C.OP_OR, C.OP_FLOOR,
               C.OP_CEIL, C.OP_SIGN, C.OP_IF_ELSE_ZERO}
    d1 = {C.OP_ADD, C.OP_SUB, C.OP_MUL, C.OP_DIV, C.OP_POW, C.OP_FMOD, C.OP_REMAINDER,
          C.OP_FMIN, C.OP_FMAX, C.OP_ATAN2, C.OP_HYPOT, C.OP_IF_ELSE_ZERO}
    return op not in zero_d0, op in d1


def _mix():
    return {"dadd": 0, "dmul": 0, "dfma": 0}


def _needed(tape, wanted_out):
    """Per instruction: does its result reach an output in ``wanted_out`` (None: all)? The
    tangent plans prune the others (one backward pass over the slots read later)."""
    from casadi_gb300 import calculus as C
    ops, i0, i1, i2 = (tape.op.tolist(), tape.i0.tolist(), tape.i1.tolist(), tape.i2.tolist())
    if wanted_out is None or all(wanted_out):
        return [True] * len(ops)
    need = [False] * len(ops)
    live = [False] * max(1, tape.sz_w)
    for k in range(len(ops) - 1, -1, -1):
        op = ops[k]
        if op == C.OP_OUTPUT:
            need[k] = bool(wanted_out[i0[k]])
            if need[k]:
                live[i1[k]] = True
            continue
        if not live[i0[k]]:
            continue
        need[k] = True
        live[i0[k]] = False
        if op in (C.OP_CONST, C.OP_INPUT):
            continue
        live[i1[k]] = True
        if op in C.BINARY_OPS:
            live[i2[k]] = True
    return need


def structural_tangent_ops(tape, unit_dirs=True, ndir=None, wanted_out=None):
    """FP64 instructions of the forward sweep with unit seeds, summed over all directions and
    split by kind, following the structural rules the sweeps apply (the tangent kernel's
    cases): ADD/SUB of two carried operands one DADD; a general op one DMUL per carried
    operand, two carried: DMUL + DFMA; TWICE, NEG, ASSIGN, IF_ELSE_ZERO none (integer
    exponent/sign operations, selections). Instructions that reach no output of
    ``wanted_out`` (the outputs whose sensitivities are requested) count nothing."""
    from casadi_gb300 import calculus as C
    nz = sum(tape.nnz_in)
    offs = np.cumsum([0] + list(tape.nnz_in))
    ops, i0, i1, i2 = (tape.op.tolist(), tape.i0.tolist(), tape.i1.tolist(), tape.i2.tolist())
    carry = {op: _carries(op) for op in set(ops)}
    need = _needed(tape, wanted_out)
    mix = _mix()
    for d in range(nz if unit_dirs else 1):
        act = [False] * max(1, tape.sz_w)
        for k, op in enumerate(ops):
            if op == C.OP_INPUT:
                act[i0[k]] = (offs[i1[k]] + i2[k] == d) if unit_dirs else True
                continue
            if op == C.OP_CONST:
                act[i0[k]] = False
                continue
            if op == C.OP_OUTPUT:
                continue
            c0, c1 = carry[op]
            cb = act[i1[k]] and c0
            cc = op in C.BINARY_OPS and act[i2[k]] and c1
            act[i0[k]] = cb or cc
            if not (cb or cc) or not need[k]:
                continue
            if op in (C.OP_ADD, C.OP_SUB):
                mix["dadd"] += 1 if (cb and cc) else 0
            elif op in (C.OP_TWICE, C.OP_NEG, C.OP_ASSIGN, C.OP_IF_ELSE_ZERO):
                pass
            else:
                mix["dmul"] += 1
                mix["dfma"] += 1 if (cb and cc) else 0
    scale = 1 if unit_dirs else (ndir or 1)
    return {k: v * scale for k, v in mix.items()}


def structural_adjoint_ops(tape, seeded_out):
    """FP64 instructions of one adjoint direction by kind (the adjoint kernel's cases): a
    seeded output or an ADD/SUB/ASSIGN/NEG/TWICE/IF_ELSE_ZERO contribution that is not the
    slot's first one DADD; a general op's contribution DMUL when first, else one DFMA into the
    running adjoint."""
    from casadi_gb300 import calculus as C
    ops, i0, i1, i2 = (tape.op.tolist(), tape.i0.tolist(), tape.i1.tolist(), tape.i2.tolist())
    act = [False] * max(1, tape.sz_w)
    mix = _mix()
    for k in range(len(ops) - 1, -1, -1):
        op = ops[k]
        if op == C.OP_OUTPUT:
            if seeded_out[i0[k]]:
                mix["dadd"] += 1 if act[i1[k]] else 0
                act[i1[k]] = True
            continue
        if op in (C.OP_INPUT, C.OP_CONST):
            act[i0[k]] = False
            continue
        if not act[i0[k]]:
            continue
        act[i0[k]] = False
        c0, c1 = _carries(op)
        for slot, carries in ((i1[k], c0), (i2[k], c1 and op in C.BINARY_OPS)):
            if not carries:
                continue
            first = not act[slot]
            if op in (C.OP_ADD, C.OP_SUB, C.OP_ASSIGN, C.OP_NEG, C.OP_IF_ELSE_ZERO, C.OP_TWICE):
                mix["dadd"] += 0 if first else 1
            else:
                mix["dmul" if first else "dfma"] += 1
            act[slot] = True
    return mix


SIMPLE_OPS = ("ADD", "SUB", "MUL", "SQ", "IF_ELSE_ZERO", "LT", "LE", "EQ", "NE", "FMIN", "FMAX")


def sincos_pairs(tape):
    """SIN/COS pairs of one operand value (the library's rule, on the scheduled tape): per op,
    the instructions that take the previous SIN/COS's sin/cos again ("reuse") and those whose
    sincos a later one takes ("first")."""
    from casadi_gb300 import calculus as C
    from casadi_gb300 import runtime as R
    t = R.schedule(tape)
    ver, cache, owner = {}, None, None
    reuse, first = {C.OP_SIN: 0, C.OP_COS: 0}, set()
    for k in range(t.n_instr):
        o = int(t.op[k])
        if o in (C.OP_SIN, C.OP_COS):
            key = (int(t.i1[k]), ver.get(int(t.i1[k])))
            if key == cache:
                reuse[o] += 1
                first.add(owner)
            else:
                cache, owner = key, k
        if o != C.OP_OUTPUT:
            ver[int(t.i0[k])] = k
    firsts = {C.OP_SIN: 0, C.OP_COS: 0}
    for k in first:
        firsts[int(t.op[k])] += 1
    return {"reuse": reuse, "first": firsts}


def sincos_reuse(tape):
    """SIN/COS instructions that take the previous SIN/COS's sin/cos pair: op -> count."""
    return sincos_pairs(tape)["reuse"]


def algorithmic_flops(tape, weights, rates, seeded_out=None, unit_dirs=True, wanted_out=None):
    """Per instance and kernel family: FP64-pipe instructions ("instr") and their time at the
    measured rates expressed in DFMA-chain instructions ("dfma_time"); the family's ceiling
    is rate_dfma * instr / dfma_time. Value and record sweeps: simple ops (one DADD or DMUL
    each, weight 1) at the DADD/DMUL rate, libm calls at their measured DFMA equivalents
    (op_weights.json); TWICE, the sign-bit ops and selections cost no FP64 instruction. A SIN or
    COS that takes the previous one's sin/cos pair costs none; a record of SIN or COS is one
    sincos (the value and the partial), and so is the value of the first of a pair
    (sincos_pairs)."""
    from casadi_gb300 import calculus as C
    slow = rates["dfma"] / min(rates["dadd"], rates["dmul"])
    out = {"eval": {"instr": 0.0, "dfma_time": 0.0}, "record": {"instr": 0.0, "dfma_time": 0.0}}
    pairs = sincos_pairs(tape)
    reuse, first = pairs["reuse"], pairs["first"]
    for op, cnt in zip(*np.unique(tape.op, return_counts=True)):
        op = int(op)
        if op in (C.OP_CONST, C.OP_INPUT, C.OP_OUTPUT):
            continue
        name = C.OP_NAMES[op]
        w = 0.0 if name == "TWICE" else float(weights.get(name, 1.0))
        t = w * (slow if name in SIMPLE_OPS else 1.0)
        wp = float(weights.get(name + "_partial", 0.0))
        ec, fc = cnt - reuse.get(op, 0) - first.get(op, 0), first.get(op, 0)
        out["eval"]["instr"] += ec * w + fc * (w + wp)
        out["eval"]["dfma_time"] += ec * t + fc * (t + wp)
        rc = cnt - reuse.get(op, 0)
        out["record"]["instr"] += rc * (w + wp)
        out["record"]["dfma_time"] += rc * (t + wp)
    seeded_out = seeded_out or [True] * len(tape.nnz_out)
    for fam, mix in (("tangent", structural_tangent_ops(tape, unit_dirs, wanted_out=wanted_out)),
                     ("adjoint", structural_adjoint_ops(tape, seeded_out))):
        out[fam] = {"instr": float(sum(mix.values())), "mix": mix,
                    "dfma_time": mix["dfma"] + (mix["dadd"] + mix["dmul"]) * slow}
    for v in out.values():
        v["peak"] = rates["dfma"] * v["instr"] / v["dfma_time"] if v["dfma_time"] else None
    return out


def load_weights():
    p = os.path.join(ROOT, "casadi_gb300", "op_weights.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)["weights"]
    return {}


# ---- clocks ------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---- FP64 peak, measured live ------------------------------------------------------------------
def fp64_pipe_rates(R):
    """The FP64 pipe's measured instruction rates (T thread-instructions/s) from the library's
    chain probe: DFMA (the roofline denominator: every sweep instruction counts one), DADD,
    DMUL."""
    return {k: R.fp64_rate(k, reps=5) / 1e12
            for k in ("dfma", "dadd", "dmul", "dmul_as_dfma", "dadd_as_dfma")}


def fp64_peak_tflops(torch):
    """cuBLAS FP64 GEMM throughput (4096^3, best of 5) — the measured FP64 ceiling, in the
    spirit of the driver's cuBLAS bf16 figure."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


# ---- CPU baseline (the reference's algorithm restated, all host threads) -----------------------
_CASADI_TAPES = {}


def casadi_rollout_tapes():
    """CasADi's own derivative Functions for the 20-step rollout's step: the jacobian() tape
    of xN (the rollout with xN as its only output, as the reference built it:
    tests/golden/casadi_rollout20_jacobian.npz, pinned by its SHA-256) and F.reverse(1),
    which sx.reverse_function rebuilds instruction for instruction."""
    if not _CASADI_TAPES:
        from casadi_gb300 import calculus as C
        from casadi_gb300 import sx as S
        from casadi_gb300 import workloads as W
        z = np.load(os.path.join(ROOT, "tests", "golden", "casadi_rollout20_jacobian.npz"))
        key = "jacobian_xn"
        op = z[key + "/op"]
        c = op == C.OP_CONST
        _CASADI_TAPES["jacobian"] = S.Tape(
            op, z[key + "/i0"], np.where(c, 0, z[key + "/i1"]),
            np.where(c, 0, z[key + "/i2"]), np.where(c, z[key + "/d"], 0.0),
            z[key + "/nnz_in"].tolist(), z[key + "/nnz_out"].tolist(), int(z[key + "/sz_w"]))
        _CASADI_TAPES["reverse"] = S.reverse_function(W.cartpole_rollout(20)).tape
    return _CASADI_TAPES["jacobian"], _CASADI_TAPES["reverse"]


def casadi_calibration():
    """CasADi's compiled library against the oracle's restatement of its algorithm, both on
    the dev host's cores (profiles/cpu_casadi_openmp_devhost.json; the reference library cannot
    be built where its sources are absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "cpu_casadi_openmp_devhost.json")) as f:
            return json.load(f)["workloads"]
    except (OSError, ValueError, KeyError):
        return {}


def cpu_step(tape, args, aseeds, n, threads, workload):
    import oracle as O
    if workload == "rollout20":
        # the reference's algorithm: CasADi's Jacobian of xN and F.reverse(1) are SXFunctions
        # of their own (symbolic derivative tapes) that its VM evaluates; here those very
        # tapes run on the oracle's restatement of SXFunction::eval
        jt, bt = casadi_rollout_tapes()
        t0 = time.perf_counter()
        O.eval(jt, list(args) + [None] * (len(jt.nnz_in) - 2), n, threads)
        O.eval(bt, list(args) + [None, None] + [s[0] for s in aseeds], n, threads)
        return time.perf_counter() - t0
    t0 = time.perf_counter()
    if workload == "dag":
        O.reverse(tape, args, aseeds, n, threads)
        bits = [np.repeat((np.uint64(1) << np.arange(64, dtype=np.uint64))[:, None], n, axis=1)]
        O.sp_forward(tape, bits, n, threads)
        seeds = [np.repeat((np.uint64(1) << np.arange(16, dtype=np.uint64))[:, None], n, axis=1)]
        O.sp_reverse(tape, [np.zeros((64, n), np.uint64)], seeds, n, threads)
    else:
        O.eval(tape, args, n, threads)
    return time.perf_counter() - t0


def cpu_baseline(F, args, aseeds, workload, budget_s=12.0):
    threads = os.cpu_count() or 1
    tape = F.tape
    m = 256
    sub = lambda arrs, k: [np.ascontiguousarray(a[..., :k]) for a in arrs]  # noqa: E731
    t = cpu_step(tape, sub(args, m), sub(aseeds, m), m, threads, workload)
    m2 = int(min(args[0].shape[-1], max(m, m * budget_s / max(t, 1e-6) / 2)))
    t2 = cpu_step(tape, sub(args, m2), sub(aseeds, m2), m2, threads, workload)
    out = {"value": m2 / t2, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": "%d of the instances, same step (oracle C restatement, OpenMP, %d threads)"
                     % (m2, threads)}
    if workload == "rollout20":
        out["sample"] = ("%d of the instances per step: CasADi's own jacobian() of xN and "
                         "reverse(1) tapes on the oracle's restatement of SXFunction::eval "
                         "(OpenMP, %d threads)" % (m2, threads))
        cal = casadi_calibration().get("rollout", {})
        if cal.get("casadi_over_restated"):
            out["casadi_compiled_over_restatement_devhost"] = cal["casadi_over_restated"]
            out["casadi_openmp_estimate"] = out["value"] * cal["casadi_over_restated"]
    return out


def headline_parity(F, args_h, aseeds_h, res, jac, asens, m=1024, threads=None):
    """Check of the timed step's own results, part of the CPU-baseline leg: the device's
    values, Jacobian and cost adjoint of the last timed step on the first m instances against
    the oracle's same step; values element-wise (relative), derivatives element-wise against
    the magnitude of their chain-rule terms (oracle.magnitude)."""
    import oracle as O
    threads = threads or os.cpu_count() or 1
    sub = [np.ascontiguousarray(x[..., :m]) for x in args_h]
    seeds = [np.ascontiguousarray(x[..., :m]) for x in aseeds_h]
    r, j, a = O.jacobian_reverse(F.tape, sub, seeds, m, threads)
    with O.magnitude():
        _, jm, am = O.jacobian_reverse(F.tape, sub, seeds, m, threads)
    worst, same, total = 0.0, 0, 0
    for got, want, mag in ([(x[..., :m].cpu().numpy(), y, np.abs(y)) for x, y in zip(res, r)] +
                           [(x[..., :m].cpu().numpy(), y, z) for x, y, z in zip(jac, j, jm)
                            if x is not None] +
                           [(x[..., :m].cpu().numpy(), y, z) for x, y, z in zip(asens, a, am)]):
        d = np.abs(got - want)
        worst = max(worst, float(np.max(np.where(d == 0, 0.0, d / np.maximum(mag, 1e-300)),
                                        initial=0.0)))
        same += int(np.sum(got.view(np.uint64) == want.view(np.uint64)))
        total += got.size
    return {"instances": m, "outputs_checked": total, "bitwise_equal_fraction": same / total,
            "max_error_over_magnitude": worst, "bar": 1e-13, "ok": worst <= 1e-13}


# ---- native arm ----------------------------------------------------------------------------------
def _seed_block(nnz_in, flat_color, n_colors, m):
    """Dense forward seeds of a colouring for the oracle: one (n_colors, nnz, m) array per
    input, direction d = 1 on the nonzeros of colour d."""
    out, off = [], 0
    for k in nnz_in:
        blk = np.zeros((n_colors, k, m))
        for q in range(k):
            c = flat_color[off + q]
            if c >= 0:
                blk[c, q, :] = 1.0
        out.append(blk)
        off += k
    return out


def mixed_component(torch, R, stream, reps=3, total=1 << 20, cpu=False):
    """Mixed-size batch: eight random-DAG tapes (200..20000 nodes, 64 inputs, 16 outputs)
    and work items with log-normal instance counts (median 4096, sigma 1.5) up to 2^20
    instances, each evaluated with the adjoint of the sum of its outputs: one launch pair per
    item (record + adjoint, one item after the other on one stream) against the persistent
    batch (all items in one launch, replayed from a CUDA graph). The per-item launches run
    twice: as the plain one-tape-per-launch kernels (one instance per thread, shared-memory
    work vectors: residence 2) and with everything the per-tape entry points tune for
    (the cooperative level sweep for items with few tiles included)."""
    from casadi_gb300 import workloads as W
    funs, items = W.mixed_batch(n_tapes=8, total=total, seed=0)
    tapes = [R.CudaTape(f) for f in funs]
    b = R.Batch()
    plain = []
    total = 0
    for k, n, sd in items:
        t = tapes[k]
        args = [torch.from_numpy(x).cuda() for x in W.dag_inputs(n, n_in=64, seed=sd)]
        seeds = [torch.ones((1, 16, n), dtype=torch.float64, device="cuda")]
        res, asens = b.add(t, args, seeds)
        plain.append((t, args, seeds, [torch.empty_like(r) for r in res],
                      [torch.empty_like(x) for x in asens]))
        total += n
    limit = max(b.scratch_bytes(), 1 << 30)
    shared = torch.empty(limit, dtype=torch.uint8, device="cuda")
    for t in tapes:
        t._scratch = shared

    def run_plain():
        for t, args, seeds, res, asens in plain:
            t.reverse(args, seeds, res=res, asens=asens, stream=stream, scratch_limit=limit)

    def run_batch():
        b.run(graph=True, stream=stream)

    def timeit(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    for t in tapes:
        t.set_residence(2)
    ms_plain = timeit(run_plain)
    for t in tapes:
        t.set_residence(0)
    ms_tuned = timeit(run_plain)
    ms_batch = timeit(run_batch)
    same = all(bool(torch.equal(x.view(torch.int64), y.view(torch.int64))) for
               (_, _, _, r0, s0), (_, _, r1, _, s1) in zip(plain, b._keep)
               for x, y in zip(r0 + s0, r1 + s1))
    for t in tapes:
        t.sync()
        t._scratch = None
    counts = [n for _, n, _ in items]
    cpu_rate = None
    if cpu:
        # the oracle port on the host cores: every item on 1/64 of its instances
        import oracle as O
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        sampled = 0
        for k, n, sd in items:
            m = max(1, n // 64)
            args = W.dag_inputs(m, n_in=64, seed=sd)
            O.reverse(funs[k].tape, args, [np.ones((1, 16, m))], m, threads)
            sampled += m
        cpu_rate = {"value": sampled / (time.perf_counter() - t0), "unit": UNIT,
                    "cores": threads, "kind": "port",
                    "sample": "1/64 of every item's instances (%d), value + adjoint" % sampled}
    return {"instances": total, "items": len(items), "cpu_port": cpu_rate,
            "tape_instructions": [f.tape.n_instr for f in funs],
            "item_instances_median": int(np.median(counts)), "item_instances_max": max(counts),
            "plain_ms": ms_plain, "per_item_tuned_ms": ms_tuned, "persistent_ms": ms_batch,
            "plain_evals_per_s": total / (ms_plain * 1e-3),
            "persistent_evals_per_s": total / (ms_batch * 1e-3),
            "speedup": ms_plain / ms_batch, "speedup_vs_per_item_tuned": ms_tuned / ms_batch,
            "bitwise_equal": same}


def maps_component(torch, stream, n=1 << 18, steps=20, reps=3):
    """Function::mapaccum and MapSum on the headline's shapes. mapaccum: the 20-step cart-pole
    rollout written as mapaccum(20) of the one-step function with its stage cost, values of
    every step and the reverse sweep of x_20 and all stage costs back to x0 and U (the
    accumulator checkpointed at every call), against the unrolled rollout tape's value and
    adjoint sweeps on the same inputs. MapSum: the unrolled rollout with the control sequence
    U shared by all instances (reduce_in) and the cost summed over instances (reduce_out), in
    instance order (the reference's bits) and in the blocked-tree order: values, and the
    adjoint of the summed cost, which gives the gradient with respect to the shared U summed
    over the instances."""
    from casadi_gb300 import runtime as R
    from casadi_gb300 import sx as S
    from casadi_gb300 import workloads as W
    x, u = S.sym("x", 4), S.sym("u")
    cost = (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3]) + 0.01 * u * u
    f = S.Function("fc", [x, [u]], [W.rk4_step(x, u), [cost]])
    x0, U = W.cartpole_inputs(n, steps=steps, seed=5)
    dx0 = torch.from_numpy(x0).cuda()
    dU = torch.from_numpy(np.ascontiguousarray(U * 0.3)).cuda()

    def ms(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    acc = R.CudaMapaccum(f, steps)
    sx = torch.zeros((1, 4 * steps, n), dtype=torch.float64, device="cuda")
    sx[:, -4:] = 1.0
    sc = torch.ones((1, steps, n), dtype=torch.float64, device="cuda")
    out = {"instances": n, "steps": steps}
    out["mapaccum_eval_ms"] = ms(lambda: acc.eval([dx0, dU], stream=stream))
    out["mapaccum_reverse_ms"] = ms(lambda: acc.reverse([dx0, dU], [sx, sc], stream=stream))
    acc2 = R.CudaMapaccum(f, steps)
    out["mapaccum_reverse_recorded_ms"] = ms(
        lambda: acc2.reverse([dx0, dU], [sx, sc], stream=stream, record_all=True))
    F = W.cartpole_rollout(steps)
    ct = R.CudaTape(F)
    seeds = [torch.ones((1, 4, n), dtype=torch.float64, device="cuda"),
             torch.ones((1, 1, n), dtype=torch.float64, device="cuda")]
    out["unrolled_eval_ms"] = ms(lambda: ct.eval([dx0, dU], stream=stream))
    out["unrolled_reverse_ms"] = ms(lambda: ct.reverse([dx0, dU], seeds, stream=stream))
    dUs = dU[:, 0].contiguous()
    aseeds = [None, torch.ones((1, 1), dtype=torch.float64, device="cuda")]
    # order 0: instance order, one dependent add per instance (the reference's bits);
    # order 1: the blocked tree (deterministic, other bits)
    for order, tag in ((0, "mapsum"), (1, "mapsum_tree")):
        msum = R.CudaMapSum(F, n, reduce_in=[False, True], reduce_out=[False, True],
                            order=order)
        out[tag + "_eval_ms"] = ms(lambda: msum.eval([dx0, dUs], stream=stream))
        out[tag + "_reverse_ms"] = ms(lambda: msum.reverse([dx0, dUs], aseeds, stream=stream))
    for k in ("mapaccum_eval", "mapaccum_reverse", "mapaccum_reverse_recorded",
              "unrolled_eval", "unrolled_reverse",
              "mapsum_eval", "mapsum_reverse", "mapsum_tree_eval", "mapsum_tree_reverse"):
        out[k + "_evals_per_s"] = n / (out[k + "_ms"] * 1e-3)
    acc.tape.sync()
    acc2.tape.sync()
    ct.sync()
    return out


def rollout_autograd_component(torch, stream, n=1 << 20, reps=2):
    """The cart-pole 100-step rollout over 2^20 instances differentiated through
    torch.autograd: ten checkpointed 10-step segment tapes; forward stores only the segment
    inputs, backward re-runs each segment's record sweep and its adjoint sweep. One step =
    forward + backward of sum(cost) with respect to x0 and U[100]."""
    from casadi_gb300 import workloads as W
    from casadi_gb300.autograd import CheckpointedRollout
    x0, U = W.cartpole_inputs(n, steps=100, seed=3)
    tx = torch.from_numpy(x0).cuda().requires_grad_(True)
    tu = torch.from_numpy(U * 0.1).cuda().requires_grad_(True)
    roll = CheckpointedRollout(steps=100, every=10)

    def fb():
        tx.grad = None
        tu.grad = None
        _, cost = roll(tx, tu)
        cost.sum().backward()

    fb()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.current_stream())
    for _ in range(reps):
        fb()
    e1.record(torch.cuda.current_stream())
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    finite = bool(torch.isfinite(tu.grad).all().item())
    return {"instances": n, "steps": 100, "checkpoint_every": 10, "ms": ms,
            "evals_per_s": n / (ms * 1e-3), "grad_finite": finite,
            "peak_device_gb": torch.cuda.max_memory_allocated() / 1e9}


def checkpoint_component(torch, stream, n=1 << 18, steps=100, reps=3):
    """The adjoint of one long tape with segment checkpointing (casadi_gb300_reverse_checkpointed):
    the cart-pole 100-step rollout as a single tape, adjoint of the cost, N = 2^18. The plain
    adjoint records all partials (one wave); the checkpointed one keeps the live slots at each
    cut and re-records one segment at a time. Time and scratch bytes of each."""
    from casadi_gb300 import runtime as R
    from casadi_gb300 import workloads as W
    F = W.cartpole_rollout(steps)
    x0, U = W.cartpole_inputs(n, steps=steps, seed=0)
    args = [torch.from_numpy(x0).cuda(), torch.from_numpy(np.ascontiguousarray(U * 0.1)).cuda()]
    seeds = [torch.zeros((1, 4, n), dtype=torch.float64, device="cuda"),
             torch.ones((1, 1, n), dtype=torch.float64, device="cuda")]
    ct = R.CudaTape(F)
    res, asens = ct.reverse(args, seeds, stream=stream)

    def ms(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    out = {"instances": n, "steps": steps, "tape_instructions": F.tape.n_instr,
           "plain_ms": ms(lambda: ct.reverse(args, seeds, res=res, asens=asens, stream=stream)),
           "plain_scratch_gb": ct.scratch_bytes(n) / 1e9}
    lib = R.load()
    for k in (5, 10, 20):
        sc, made = ct.checkpoint_scratch(k, 1, n)

        def run():
            R.check(lib.casadi_gb300_reverse_checkpointed(
                ct.id, n, n, 1, k, R._ptr_array(args), R._ptr_array(res), R._ptr_array(seeds),
                R._ptr_array(asens), R.ct.c_void_p(sc.data_ptr()), sc.numel(),
                R._stream_handle(stream)))

        out["segments_%d" % made] = {"ms": ms(run), "scratch_gb": sc.numel() / 1e9}
        del sc
    ct.sync(stream)
    return out


def mpc_sparse_component(torch, stream, n=4096, intervals=100, reps=3, cpu=False):
    """Scenario MPC: the quadcopter multiple-shooting NLP (100 intervals, 1612 decision
    variables, 1212 constraints) over 4096 scenarios: the constraint Jacobian by uni-coloured
    forward sweeps and the Lagrangian Hessian by star-coloured forward sweeps over the
    symbolic gradient, nonzeros recovered on the device. One step = both, all scenarios."""
    from casadi_gb300 import workloads as W
    from casadi_gb300.sparse_ad import ColoredHessian, ColoredJacobian
    t0 = time.perf_counter()
    F = W.quad_ms_lagrangian(intervals)
    J = ColoredJacobian(W.quad_ms_constraints(intervals), out=0, wrt=0)
    H = ColoredHessian(F, out=1, wrt=0)
    setup_s = time.perf_counter() - t0
    args = [torch.from_numpy(x).cuda() for x in W.quad_ms_inputs(n, intervals, seed=5)]

    def step():
        J(args, stream=stream)
        H(args, stream=stream)

    # the same work as two items of one persistent batch launch replayed from a CUDA graph,
    # followed by the two device gathers
    from casadi_gb300 import runtime as R
    b = R.Batch()
    cj = J.add_to_batch(b, args)
    ch = H.add_to_batch(b, args)
    vj = torch.empty((J.src_row.numel(), n), dtype=torch.float64, device="cuda")
    vh = torch.empty((H.src_row.numel(), n), dtype=torch.float64, device="cuda")

    def step_batch():
        b.run(graph=True, stream=stream)
        J.gather(cj, n, out=vj, stream=stream)
        H.gather(ch, n, out=vh, stream=stream)

    def timeit(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ms = timeit(step)
    ms_batch = timeit(step_batch)
    rj, rh = J(args, stream=stream), H(args, stream=stream)
    stream.synchronize()  # the separate calls ran on `stream`; compare after they finish
    same = bool(torch.equal(vj.view(torch.int64), rj.view(torch.int64)) and
                torch.equal(vh.view(torch.int64), rh.view(torch.int64)))
    cpu_rate = None
    if cpu:
        # the oracle port on the host cores: the same coloured forward sweeps on 64 scenarios
        import oracle as O
        threads = os.cpu_count() or 1
        m = 64
        sub = [a[:, :m].cpu().numpy() for a in args]
        sj = _seed_block(J.tape.nnz_in, J._flat, J.n_colors, m)
        sh = _seed_block(H.tape.nnz_in, H._flat, H.n_colors, m)
        t0 = time.perf_counter()
        O.forward(J.tape.tape, sub, sj, m, threads)
        O.forward(H.tape.tape, sub, sh, m, threads)
        cpu_rate = {"value": m / (time.perf_counter() - t0), "unit": "scenarios/s",
                    "cores": threads, "kind": "port",
                    "sample": "%d scenarios, same coloured forward sweeps" % m}
    return {"scenarios": n, "intervals": intervals, "decision_variables": F.tape.nnz_in[0],
            "cpu_port": cpu_rate,
            "constraints": F.tape.nnz_out[0], "lagrangian_instructions": F.tape.n_instr,
            "gradient_instructions": H.gradient_function.tape.n_instr,
            "jacobian_nnz": J.pattern.nnz, "jacobian_colors": J.n_colors,
            "hessian_nnz_lower": int(H.rows.size), "hessian_colors": H.n_colors,
            "ms": ms, "scenarios_per_s": n / (ms * 1e-3),
            "persistent_graph_ms": ms_batch, "persistent_scenarios_per_s": n / (ms_batch * 1e-3),
            "bitwise_equal": same, "host_setup_s": setup_s}


def side_workload_component(torch, R, stream, name, rates, weights, cpu=False, reps=10):
    """The other single-tape workloads of the benchmark set, each timed like the headline step
    (L2 flushed between timed steps, CUDA events on the launching stream) with the per-launch
    device time of every kernel family and a roofline entry per family:
      cartpole: the RK4 step f(x[4],u) -> x_next[4] over 65536 instances, values only;
      dag: the random DAG (64 inputs, 10000 nodes, 16 outputs) over 16384 instances: values +
           adjoint of the sum of the outputs, then the bvec_t sp_forward (64 directions, input
           k on bit k) and sp_reverse (output k on bit k) sweeps."""
    F, n, args_h, aseeds_h, desc = make_workload(name)
    ct = R.CudaTape(F)
    dargs = [torch.from_numpy(x).cuda() for x in args_h]
    daseeds = [torch.from_numpy(x).cuda() for x in aseeds_h]
    res = [torch.empty((k, n), dtype=torch.float64, device="cuda") for k in F.tape.nnz_out]
    asens = [torch.empty((1, k, n), dtype=torch.float64, device="cuda") for k in F.tape.nnz_in]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    if name == "dag":
        sp_in = torch.tensor([1 << k if k < 63 else -(1 << 63) for k in range(64)],
                             dtype=torch.int64, device="cuda")[:, None].expand(64, n).contiguous()
        sp_seed0 = torch.tensor([1 << k for k in range(16)], dtype=torch.int64,
                                device="cuda")[:, None].expand(16, n).contiguous()
        sp_seed = torch.empty_like(sp_seed0)
        sp_sens = torch.empty((64, n), dtype=torch.int64, device="cuda")

    def step():
        if name == "dag":
            ct.reverse(dargs, daseeds, res=res, asens=asens, stream=stream)
            ct.sp_forward([sp_in], stream=stream)
            sp_seed.copy_(sp_seed0)
            sp_sens.zero_()
            ct.sp_reverse([sp_sens], [sp_seed], stream=stream)
        else:
            ct.eval(dargs, res=res, stream=stream)

    for _ in range(3):
        step()
    ct.sync()
    R.profile(True)
    R.profile_collect()
    times = []
    torch.cuda.synchronize()
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        times.append((e0, e1))
    torch.cuda.synchronize()
    prof = R.profile_collect()
    R.profile(False)
    ct.sync()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in times) / reps
    work = algorithmic_flops(F.tape, weights, rates)
    sp_bytes = 8 * (sum(F.tape.nnz_in) + sum(F.tape.nnz_out))
    roof = {}
    for fam, (fms, nl) in prof.items():
        if nl == 0:
            continue
        per_launch_ms = fms / nl
        inst_per_launch = n * reps / nl
        if fam in ("eval", "record", "adjoint"):
            w = work[fam]
            ach = w["instr"] * inst_per_launch / (per_launch_ms * 1e-3) / 1e12
            roof[fam] = {"bound": "fp64", "achieved": ach, "peak": w["peak"],
                         "unit": "T FP64 instr/s", "frac": ach / w["peak"],
                         "ms_per_launch": per_launch_ms,
                         "instr_per_instance": w["instr"], "mix": w.get("mix")}
        else:
            ach = sp_bytes * inst_per_launch / (per_launch_ms * 1e-3) / 1e9
            roof[fam] = {"bound": "smem/latency (bvec OR sweep; HBM bytes shown)",
                         "achieved": ach, "unit": "GB/s", "ms_per_launch": per_launch_ms,
                         "algorithmic_bytes_per_instance": sp_bytes}
    out = {"workload": desc, "instances": n, "tape_instructions": F.tape.n_instr,
           "ms_per_step": ms, "evals_per_s": n / (ms * 1e-3),
           "kernel_ms_per_step": {k: v[0] / reps for k, v in prof.items() if v[1]},
           "launches_per_step": {k: v[1] / reps for k, v in prof.items() if v[1]},
           "roofline": roof}
    if cpu:
        out["cpu_baseline"] = cpu_baseline(F, args_h, aseeds_h, name, budget_s=6.0)
    return out


def run_mixed(a):
    """The mixed-size persistent batch alone (profiling captures of k_batch): one line with
    the persistent batch's rate and the one-launch-pair-per-item comparison."""
    import torch
    from casadi_gb300 import runtime as R
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    comp = mixed_component(torch, R, torch.cuda.current_stream(), reps=max(1, a.steps),
                           total=a.instances or (1 << 20))
    print(json.dumps({"metric": METRIC, "value": comp["persistent_evals_per_s"], "unit": UNIT,
                      "n_gpus": 1, "steps": a.steps, "warmup": 1,
                      "ms_per_step": comp["persistent_ms"], "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic",
                      "config": {"workload": "mixed-size batch: 8 random-DAG tapes, "
                                             "log-normal item sizes, value + adjoint"},
                      "components": {"mixed_batch": comp}}), flush=True)


def run_mpc(a):
    """The scenario-MPC component alone (profiling captures of its kernels): the coloured
    constraint Jacobian and Lagrangian Hessian over the scenarios, separate calls and the
    persistent batch graph."""
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    comp = mpc_sparse_component(torch, torch.cuda.current_stream(), n=a.instances or 4096,
                                reps=max(1, a.steps))
    print(json.dumps({"metric": METRIC, "value": comp["persistent_scenarios_per_s"],
                      "unit": "scenarios/s", "n_gpus": 1, "steps": a.steps, "warmup": 1,
                      "ms_per_step": comp["persistent_graph_ms"], "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic",
                      "config": {"workload": "scenario MPC: quadcopter multiple shooting, "
                                             "100 intervals, coloured Jacobian + Hessian"},
                      "components": {"mpc_sparse_hessian": comp}}), flush=True)


def run_native(a):
    import torch
    from casadi_gb300 import runtime as R

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    F, n, args_h, aseeds_h, desc = make_workload(a.workload, a.instances)
    ct = R.CudaTape(F)
    dargs = [torch.from_numpy(x).cuda() for x in args_h]
    daseeds = [torch.from_numpy(x).cuda() for x in aseeds_h]
    nz = sum(F.tape.nnz_in)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    res = [torch.empty((k, n), dtype=torch.float64, device="cuda") for k in F.tape.nnz_out]
    # the step's Jacobian is of xN (output 0); the cost's row comes from its adjoint, and the
    # tangent plan prunes the instructions that only the cost needs
    jac = [torch.empty((nz, F.tape.nnz_out[0], n), dtype=torch.float64, device="cuda"), None] \
        if a.workload == "rollout20" else None
    asens = [torch.empty((1, k, n), dtype=torch.float64, device="cuda") for k in F.tape.nnz_in]
    ct.scratch(n)

    if a.workload == "dag":
        # bvec_t patterns: input nonzero k carries bit k (64 inputs, one forward sweep);
        # output nonzero k seeds bit k of the reverse sweep (16 outputs, one sweep)
        sp_in = torch.tensor([1 << k if k < 63 else -(1 << 63) for k in range(64)],
                             dtype=torch.int64, device="cuda")[:, None].expand(64, n).contiguous()
        sp_seed0 = torch.tensor([1 << k for k in range(16)], dtype=torch.int64,
                                device="cuda")[:, None].expand(16, n).contiguous()
        sp_seed = torch.empty_like(sp_seed0)
        sp_sens = torch.empty((64, n), dtype=torch.int64, device="cuda")

    def step():
        if a.workload == "rollout20":
            # one record sweep feeds the Jacobian of xN (24 unit directions) and the cost adjoint
            ct.jacobian_reverse(dargs, daseeds, res=res, jac=jac, asens=asens, stream=stream)
        elif a.workload == "dag":
            # eval + adjoint of the sum of outputs, then both sparsity sweeps
            ct.reverse(dargs, daseeds, res=res, asens=asens, stream=stream)
            ct.sp_forward([sp_in], stream=stream)
            sp_seed.copy_(sp_seed0)
            sp_sens.zero_()
            ct.sp_reverse([sp_sens], [sp_seed], stream=stream)
        else:
            ct.eval(dargs, res=res, stream=stream)

    for _ in range(a.warmup):
        step()
    ct.sync()
    R.profile(True)
    R.profile_collect()
    times = []
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(a.steps):
            flush.fill_(1.0)  # evict L2 between timed steps (outside the events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            times.append((e0, e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ms = [e0.elapsed_time(e1) for e0, e1 in times]
    prof = R.profile_collect()
    R.profile(False)
    ct.sync()
    ms_step = sum(ms) / len(ms)
    if dist:
        from casadi_gb300 import replicas as RP
        ms_step = RP.max_over_ranks(ms_step, device="cuda")  # the slowest replica's step
    value = world * n / (ms_step * 1e-3)

    # component rates (outside the timed region): eval-only and adjoint-only
    comps = {}

    def rate(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return n / (e0.elapsed_time(e1) / reps * 1e-3)

    comps["eval_evals_per_s"] = rate(lambda: ct.eval(dargs, res=res, stream=stream))
    comps["adjoint_evals_per_s"] = rate(
        lambda: ct.reverse(dargs, daseeds, res=res, asens=asens, stream=stream))
    if a.workload == "rollout20":
        # the Jacobian of every output (xN and the cost) alone
        jac_all = [torch.empty((nz, k, n), dtype=torch.float64, device="cuda")
                   for k in F.tape.nnz_out]
        comps["jacobian24_evals_per_s"] = rate(
            lambda: ct.jacobian(dargs, res=res, jac=jac_all, stream=stream))
        del jac_all
    # derivative-sweep variants the autotuner kept (tangent 8: the windowed sweep)
    comps["tuned_variants"] = {"jacobian": ct.tuned_variant(1), "adjoint": ct.tuned_variant(2)}
    if a.workload == "rollout20":
        # the drop-in's own route for the same results: CasADi's derivative Functions
        # (jacobian(), reverse(1)) mapped with "cuda", i.e. their tapes on the value sweep
        jt, bt = casadi_rollout_tapes()
        cj, cb = R.CudaTape(jt), R.CudaTape(bt)
        jres = [torch.empty((k, n), dtype=torch.float64, device="cuda") for k in jt.nnz_out]
        bres = [torch.empty((k, n), dtype=torch.float64, device="cuda") for k in bt.nnz_out]
        bargs = dargs + [None, None] + [x[0] for x in daseeds]

        def derivative_functions():
            cj.eval(dargs + [None] * (len(jt.nnz_in) - 2), res=jres, stream=stream)
            cb.eval(bargs, res=bres, stream=stream)

        comps["casadi_derivative_functions_evals_per_s"] = rate(derivative_functions)
        comps["casadi_derivative_function_instructions"] = {"jacobian": jt.n_instr,
                                                            "reverse": bt.n_instr}
        cj.sync()
        cb.sync()
    ct.sync()

    weights = load_weights()
    rates = fp64_pipe_rates(R)
    if not a.no_mixed:
        cpu = not a.no_cpu and rank == 0
        if a.workload == "rollout20":
            for side in ("cartpole", "dag"):
                comps[side] = side_workload_component(torch, R, stream, side, rates,
                                                      weights, cpu=cpu)
        comps["mixed_batch"] = mixed_component(torch, R, stream, cpu=cpu)
        comps["rollout100_autograd"] = rollout_autograd_component(torch, stream)
        comps["checkpointed_adjoint"] = checkpoint_component(torch, stream)
        comps["mpc_sparse_hessian"] = mpc_sparse_component(torch, stream, cpu=cpu)
        comps["mapaccum_mapsum"] = maps_component(torch, stream)

    # roofline of the dominant kernel family (device time from the per-launch events)
    work = algorithmic_flops(F.tape, weights, rates,
                             seeded_out=[bool(np.any(x)) for x in aseeds_h],
                             wanted_out=[True, False] if a.workload == "rollout20" else None)
    fam_ms = {k: v for k, v in prof.items() if v[1] > 0}
    dom = max(fam_ms, key=lambda k: fam_ms[k][0])
    dom_ms, dom_launches = fam_ms[dom]
    per_inst = work[dom]["instr"] if dom in work else 0.0
    launches_per_step = dom_launches / a.steps
    flops_per_launch = per_inst * n / launches_per_step
    achieved = flops_per_launch / (dom_ms / dom_launches * 1e-3) / 1e12
    # the FP64 pipe's measured rate for this kernel's instruction mix (DFMA chains issue
    # faster than DADD/DMUL on this part)
    peak = work[dom]["peak"] if dom in work else rates["dfma"]
    dgemm = fp64_peak_tflops(torch)
    fam_roof = {}
    for fam, (fms, nl) in fam_ms.items():
        if fam in work:
            ach_f = work[fam]["instr"] * n / (nl / a.steps) / (fms / nl * 1e-3) / 1e12
            fam_roof[fam] = {"achieved": ach_f, "peak": work[fam]["peak"],
                             "frac": ach_f / work[fam]["peak"], "ms_per_step": fms / a.steps,
                             "instr_per_instance": work[fam]["instr"],
                             "mix": work[fam].get("mix")}
    gpu_launches = sum(v[1] for v in prof.values())
    # DRAM bytes per launch of the dominant kernel from the committed ncu capture, scaled by
    # the instances one launch processes (traffic grows in proportion: the partial reads do)
    traffic = None
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                               "traffic.json")) as f:
            tr = json.load(f).get(dom)
        if tr and a.workload == "rollout20":
            traffic = tr["dram_bytes_per_launch"] * (n / launches_per_step) / tr["instances"]
    except (OSError, ValueError, KeyError):
        traffic = None
    io_bytes = 8 * n * (sum(F.tape.nnz_in) + sum(F.tape.nnz_out))

    # end-to-end through the host-buffer Map entry points (pinned host memory)
    e2e = None
    if rank == 0 or world > 1:
        cm = R.CudaMap(ct, n)

        def pinned(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

        hargs = [pinned((n, x.shape[0])) for x in args_h]
        for h, x in zip(hargs, args_h):
            h[:] = x.T
        hres = [pinned((n, k)) for k in F.tape.nnz_out]
        hseed = [pinned((n, 1, k)) for k in F.tape.nnz_out]
        for h, x in zip(hseed, aseeds_h):
            h[:] = np.transpose(x, (2, 0, 1))
        hasens = [pinned((n, 1, k)) for k in F.tape.nnz_in]
        hjac = [pinned((n, nz, F.tape.nnz_out[0])), None] if a.workload == "rollout20" else None

        def e2e_step():
            if a.workload == "rollout20":
                cm.jacobian_reverse(hargs, hseed, res=hres, jac=hjac, asens=hasens)
            elif a.workload == "dag":
                cm.reverse(hargs, hseed, res=hres, asens=hasens)
            else:
                cm(*hargs, res=hres)

        for _ in range(max(1, a.warmup)):
            e2e_step()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e2e_step()
        t_e2e = (time.perf_counter() - t0) / a.steps
        in_b = 8 * n * sum(F.tape.nnz_in)
        out_b = 8 * n * sum(F.tape.nnz_out)
        if a.workload == "rollout20":
            h2d = in_b + 8 * n * sum(F.tape.nnz_out)
            d2h = out_b + 8 * n * nz * F.tape.nnz_out[0] + in_b
        elif a.workload == "dag":
            h2d = in_b + 8 * n * sum(F.tape.nnz_out)
            d2h = out_b + in_b
        else:
            h2d, d2h = in_b, out_b
        e2e = {"value": world * n / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e * 1e3}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "instances_per_gpu": n, "tape_instructions": F.tape.n_instr,
                   "sz_w": F.tape.sz_w, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between timed steps (256 MiB write)"},
        "components": comps,
        "e2e": e2e,
        "gpu_launches": gpu_launches,
        "kernel_ms": {k: round(v[0], 4) for k, v in prof.items() if v[1]},
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "T FP64 instr/s", "frac": achieved / peak if peak else None,
                     "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu, scaled from the committed capture)",
                     "flop": "one FP64-pipe instruction (DADD, DMUL, DFMA); libm calls weighted by "
                             "casadi_gb300/op_weights.json; derivative sweeps count structural work "
                             "(a two-operand tangent: DMUL + DFMA; a later adjoint contribution: "
                             "one DFMA)",
                     "peak_source": "FP64 chain probes of this run (casadi_gb300_fp64_rate: "
                                    "every thread of a full grid runs 8 independent chains; "
                                    "thread-level instructions per second), weighted by the "
                                    "kernel's DFMA/DADD/DMUL mix",
                     "families": fam_roof,
                     "fp64_pipe_rates_tips": rates,
                     "cublas_dgemm_tflops": dgemm,
                     "io_bytes_per_step": io_bytes,
                     "hbm_gbs_io": io_bytes / (ms_step * 1e-3) / 1e9},
        "clocks": clk.summary(),
    }
    if not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(F, args_h, aseeds_h, a.workload)
        if a.workload == "rollout20":
            line["parity_check"] = headline_parity(F, args_h, aseeds_h, res, jac, asens)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---- reference arm (the reference's algorithm restated, on the host cores) ------------------------
def ref_algo(workload):
    return {"rollout20": "CasADi's own jacobian() of xN and reverse(1) tapes on the oracle's "
                         "restatement of SXFunction::eval",
            "cartpole": "the tape on the oracle's restatement of SXFunction::eval",
            "dag": "the oracle's numeric adjoint and bvec sweeps"}.get(workload, "oracle")


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    F, n, args_h, aseeds_h, desc = make_workload(a.workload, a.instances)
    threads = os.cpu_count() or 1
    # bounded sample per step so that warmup + steps finish within a few minutes
    m = 256
    sub = lambda arrs, k: [np.ascontiguousarray(x[..., :k]) for x in arrs]  # noqa: E731
    t = cpu_step(F.tape, sub(args_h, m), sub(aseeds_h, m), m, threads, a.workload)
    # every instance of the workload when warmup + steps fit in about three minutes, else the
    # largest prefix that does
    per_step = 180.0 / max(1, a.steps + a.warmup)
    m = int(min(n, max(m, m * per_step / max(t, 1e-6) * 0.8)))
    sa, ss = sub(args_h, m), sub(aseeds_h, m)
    for _ in range(a.warmup):
        cpu_step(F.tape, sa, ss, m, threads, a.workload)
    ts = [cpu_step(F.tape, sa, ss, m, threads, a.workload) for _ in range(a.steps)]
    sec = sum(ts) / len(ts)
    v = m / sec
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": desc, "instances_per_step": m, "same_instances": m == n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d of the %d instances per step, the same step by the "
                                       "reference's algorithm (%s; OpenMP, %d threads; the "
                                       "reference library itself needs its sources, absent on "
                                       "this host)" % (m, n, ref_algo(a.workload), threads)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    cal = casadi_calibration().get("rollout", {}) if a.workload == "rollout20" else {}
    if cal.get("casadi_over_restated"):
        line["cpu_baseline"]["casadi_compiled_over_restatement_devhost"] = \
            cal["casadi_over_restated"]
        line["cpu_baseline"]["casadi_openmp_estimate"] = v * cal["casadi_over_restated"]
    print(json.dumps(line), flush=True)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="native", choices=["native", "reference"])
    p.add_argument("--workload", default="rollout20",
                   choices=["rollout20", "cartpole", "dag", "mixed", "mpc"])
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--instances", type=int, default=None,
                   help="override the workload's instance count (profiling captures)")
    p.add_argument("--no-mixed", action="store_true",
                   help="skip the mixed multi-tape component (profiling captures)")
    a = p.parse_args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "mixed":
        run_mixed(a)
    elif a.workload == "mpc":
        run_mpc(a)
    else:
        run_native(a)


if __name__ == "__main__":
    main()
