"""ORACLE — test infrastructure only.

ctypes access to the plain-C restatement (``sxvm.c`` -> ``_build/liboracle.so``) and, where
the reference tree was available at build time, to the reference-op-semantics harness
(``ref_calculus.cpp`` -> ``_ref/libref_calculus.so``). Only tests, the smoke check and the
CPU-baseline leg of the benchmark use this package; the product never does.

Array layout: instance-minor, ``(nnz, n)`` per input/output; forward/adjoint seeds
``(ndir, nnz, n)``.
"""
import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_calculus.so")

_lib = None
_ref = None


def reference_tree():
    """The reference source tree named by the CASADI_REFERENCE environment variable, or None
    (no default: the tree exists only where the fixtures are generated)."""
    tree = os.environ.get("CASADI_REFERENCE")
    if tree and os.path.isdir(os.path.join(tree, "casadi", "core")):
        return tree
    return None


def build(ref=None, tree=None):
    """Compile the oracle; with a reference tree (``tree`` or CASADI_REFERENCE) also the
    reference op-semantics harness and the reference's own libcasadi with its bridge."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    tree = tree or reference_tree()
    if ref is None:
        ref = tree is not None
    if ref:
        if tree is None:
            raise RuntimeError("the reference harness needs CASADI_REFERENCE")
        jobs = str(max(1, min(16, os.cpu_count() or 1)))
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "casadi", "REF=" + tree,
                               "JOBS=" + jobs])


class _Tape(ct.Structure):
    _fields_ = [("n_instr", ct.c_int), ("op", ct.c_void_p), ("i0", ct.c_void_p),
                ("i1", ct.c_void_p), ("i2", ct.c_void_p), ("d", ct.c_void_p),
                ("n_in", ct.c_int), ("nnz_in", ct.c_void_p), ("n_out", ct.c_int),
                ("nnz_out", ct.c_void_p), ("sz_w", ct.c_int)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        _lib = ct.CDLL(LIB_PATH)
        _lib.sxo_fun.restype = ct.c_double
        _lib.sxo_fun.argtypes = [ct.c_int, ct.c_double, ct.c_double]
        _lib.sxo_der.argtypes = [ct.c_int, ct.c_double, ct.c_double, ct.c_double, ct.c_void_p]
        for name in ("sxo_eval", "sxo_forward", "sxo_jacobian", "sxo_reverse",
                     "sxo_sp_forward", "sxo_sp_reverse", "sxo_activity", "sxo_zero_checker"):
            getattr(_lib, name).restype = ct.c_int
    return _lib


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        _ref = ct.CDLL(REF_PATH)
        _ref.ref_fun.restype = ct.c_double
        _ref.ref_fun.argtypes = [ct.c_int, ct.c_double, ct.c_double]
        _ref.ref_der.argtypes = [ct.c_int, ct.c_double, ct.c_double, ct.c_double, ct.c_void_p]
        _ref.ref_op_id.argtypes = [ct.c_char_p]
        _ref.ref_op_id.restype = ct.c_int
        _ref.ref_ndeps.restype = ct.c_int
    return _ref


class TapeArrays:
    """Keeps contiguous int32/float64 copies of a tape alive for the C calls."""

    def __init__(self, tape):
        self.tape = tape
        self.op = np.ascontiguousarray(tape.op, dtype=np.int32)
        self.i0 = np.ascontiguousarray(tape.i0, dtype=np.int32)
        self.i1 = np.ascontiguousarray(tape.i1, dtype=np.int32)
        self.i2 = np.ascontiguousarray(tape.i2, dtype=np.int32)
        self.d = np.ascontiguousarray(tape.d, dtype=np.float64)
        self.nnz_in = np.ascontiguousarray(tape.nnz_in, dtype=np.int32)
        self.nnz_out = np.ascontiguousarray(tape.nnz_out, dtype=np.int32)
        self.struct = _Tape(tape.n_instr, self.op.ctypes.data, self.i0.ctypes.data,
                            self.i1.ctypes.data, self.i2.ctypes.data, self.d.ctypes.data,
                            len(tape.nnz_in), self.nnz_in.ctypes.data, len(tape.nnz_out),
                            self.nnz_out.ctypes.data, tape.sz_w)


def _ptrs(arrays):
    return (ct.c_void_p * max(1, len(arrays)))(
        *[(a.ctypes.data if a is not None else None) for a in arrays])


def _outs(nnz, n, ndir=None, dtype=np.float64):
    if ndir is None:
        return [np.zeros((k, n), dtype=dtype) for k in nnz]
    return [np.zeros((ndir, k, n), dtype=dtype) for k in nnz]


def _prep(args, dtype=np.float64):
    return [None if a is None else np.ascontiguousarray(a, dtype=dtype) for a in args]


def _check(arrays, nnz, n, what, ndir=None):
    """The C sweeps trust the buffer sizes: refuse any array of the wrong shape."""
    if len(arrays) != len(nnz):
        raise ValueError("%s: %d arrays for %d slots" % (what, len(arrays), len(nnz)))
    for a, k in zip(arrays, nnz):
        want = (k, n) if ndir is None else (ndir, k, n)
        if a is not None and a.shape != want:
            raise ValueError("%s: shape %s, expected %s" % (what, a.shape, want))


def eval(tape, args, n, nthreads=1):
    t = TapeArrays(tape)
    args = _prep(args)
    _check(args, tape.nnz_in, n, "arguments")
    res = _outs(tape.nnz_out, n)
    rc = lib().sxo_eval(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(res),
                        ct.c_int(nthreads))
    assert rc == 0
    return res


def forward(tape, args, fseeds, n, nthreads=1):
    """Values and nfwd forward sensitivities; fseeds[j] has shape (nfwd, nnz_in[j], n)."""
    t = TapeArrays(tape)
    args = _prep(args)
    fseeds = _prep(fseeds)
    nfwd = next(s.shape[0] for s in fseeds if s is not None)
    _check(args, tape.nnz_in, n, "arguments")
    _check(fseeds, tape.nnz_in, n, "forward seeds", nfwd)
    res = _outs(tape.nnz_out, n)
    fsens = _outs(tape.nnz_out, n, nfwd)
    rc = lib().sxo_forward(ct.byref(t.struct), ct.c_long(n), ct.c_int(nfwd), _ptrs(args),
                           _ptrs(res), _ptrs(fseeds), _ptrs(fsens), ct.c_int(nthreads))
    assert rc == 0
    return res, fsens


def jacobian(tape, args, n, nthreads=1):
    """Values and the Jacobian by unit forward seeds: jac[j] has shape (nnz_in_total,
    nnz_out[j], n)."""
    t = TapeArrays(tape)
    args = _prep(args)
    _check(args, tape.nnz_in, n, "arguments")
    nz = sum(tape.nnz_in)
    res = _outs(tape.nnz_out, n)
    jac = _outs(tape.nnz_out, n, nz)
    rc = lib().sxo_jacobian(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(res),
                            _ptrs(jac), ct.c_int(nthreads))
    assert rc == 0
    return res, jac


def reverse(tape, args, aseeds, n, nthreads=1):
    """Values and nadj adjoint sensitivities; aseeds[j] has shape (nadj, nnz_out[j], n)."""
    t = TapeArrays(tape)
    args = _prep(args)
    aseeds = _prep(aseeds)
    nadj = next(s.shape[0] for s in aseeds if s is not None)
    _check(args, tape.nnz_in, n, "arguments")
    _check(aseeds, tape.nnz_out, n, "adjoint seeds", nadj)
    res = _outs(tape.nnz_out, n)
    asens = _outs(tape.nnz_in, n, nadj)
    rc = lib().sxo_reverse(ct.byref(t.struct), ct.c_long(n), ct.c_int(nadj), _ptrs(args),
                           _ptrs(res), _ptrs(aseeds), _ptrs(asens), ct.c_int(nthreads))
    assert rc == 0
    return res, asens


def jacobian_reverse(tape, args, aseeds, n, nthreads=1):
    """Values, the unit-seed Jacobian (as :func:`jacobian`) and nadj adjoint directions (as
    :func:`reverse`) from one record of the partials per instance."""
    t = TapeArrays(tape)
    args = _prep(args)
    aseeds = _prep(aseeds)
    nadj = next(s.shape[0] for s in aseeds if s is not None)
    _check(args, tape.nnz_in, n, "arguments")
    _check(aseeds, tape.nnz_out, n, "adjoint seeds", nadj)
    nz = sum(tape.nnz_in)
    res = _outs(tape.nnz_out, n)
    jac = _outs(tape.nnz_out, n, nz)
    asens = _outs(tape.nnz_in, n, nadj)
    rc = lib().sxo_jacobian_reverse(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(res),
                                    _ptrs(jac), ct.c_int(nadj), _ptrs(aseeds), _ptrs(asens),
                                    ct.c_int(nthreads))
    assert rc == 0
    return res, jac, asens


def libm_bound(tape, args, n, nthreads=1):
    """Per output element, the first-order sensitivity to relative perturbations of the
    tape's libm results: sum over libm instructions k of |d out / d w_k| * |w_k| (through
    |partials|). Two evaluations whose libm results differ by at most c ulps give outputs
    within about c * 2**-52 times this bound; shape (nnz_out[j], n) per output."""
    t = TapeArrays(tape)
    args = _prep(args)
    _check(args, tape.nnz_in, n, "arguments")
    out = _outs(tape.nnz_out, n)
    rc = lib().sxo_libm_bound(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(out),
                              ct.c_int(nthreads))
    assert rc == 0
    return out


def rounding_bound(tape, args, n, nthreads=1):
    """As libm_bound over every computing instruction (sum over all of them of
    |d out / d w_k| * |w_k|): two evaluations of the same function whose instructions round
    differently, or that differ in the order of their sums, give outputs within a few times
    2**-52 times this bound."""
    t = TapeArrays(tape)
    args = _prep(args)
    _check(args, tape.nnz_in, n, "arguments")
    out = _outs(tape.nnz_out, n)
    rc = lib().sxo_rounding_bound(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(out),
                                  ct.c_int(nthreads))
    assert rc == 0
    return out


class magnitude:
    """Context in which forward / jacobian / reverse return magnitudes: the same sweeps over
    |partials| and |seeds|, i.e. per derivative entry the sum over its chain-rule paths of
    |product of partials| x |seed|. Two evaluations of one derivative that round differently
    (this sweep, the reference's symbolic derivative Function) differ by at most a modest
    multiple of eps times that magnitude, which is how the tests compare them."""

    def __enter__(self):
        lib().sxo_set_magnitude(1)
        return self

    def __exit__(self, *exc):
        lib().sxo_set_magnitude(0)
        return False


def sp_forward(tape, args, n, nthreads=1):
    t = TapeArrays(tape)
    args = _prep(args, np.uint64)
    res = _outs(tape.nnz_out, n, dtype=np.uint64)
    rc = lib().sxo_sp_forward(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(res),
                              ct.c_int(nthreads))
    assert rc == 0
    return res


def sp_reverse(tape, args, res, n, nthreads=1):
    """In place, like SXFunction::sp_reverse: args |= sensitivities, res seeds cleared."""
    t = TapeArrays(tape)
    rc = lib().sxo_sp_reverse(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(res),
                              ct.c_int(nthreads))
    assert rc == 0
    return args, res


def activity(tape, args, n, nthreads=1):
    """SXFunction::eval_activity over n instances: uint64 activity words (nnz, n)."""
    t = TapeArrays(tape)
    args = _prep(args, np.uint64)
    _check(args, tape.nnz_in, n, "activity words")
    res = _outs(tape.nnz_out, n, dtype=np.uint64)
    rc = lib().sxo_activity(ct.byref(t.struct), ct.c_long(n), _ptrs(args), _ptrs(res),
                            ct.c_int(nthreads))
    assert rc == 0
    return res


# ---- MapSum (casadi/core/mapsum.cpp) -------------------------------------------------------
def _broadcast(a, n, shared, ndir=False):
    """A shared input (nnz,) or seed (ndir, nnz) repeated for every instance."""
    if a is None or not shared:
        return a
    a = np.asarray(a)
    return np.ascontiguousarray(np.repeat(a[..., None], n, axis=-1))


def ordered_sum(rows):
    """Sum over the last (instance) axis in instance order starting from zero: MapSum's
    casadi_clear then one casadi_add per instance (mapsum.cpp:141-146, :160-178)."""
    rows = np.asarray(rows, dtype=np.float64)
    acc = np.zeros(rows.shape[:-1])
    for i in range(rows.shape[-1]):
        acc = acc + rows[..., i]
    return acc


def _or_all(rows):
    rows = np.asarray(rows, dtype=np.uint64)
    return np.bitwise_or.reduce(rows, axis=-1) if rows.shape[-1] else \
        np.zeros(rows.shape[:-1], np.uint64)


def mapsum_eval(tape, args, n, reduce_in, reduce_out, nthreads=1):
    """MapSum::eval_gen (mapsum.cpp:153-181): shared inputs are (nnz,), summed outputs (nnz,)."""
    full = [_broadcast(a, n, r) for a, r in zip(args, reduce_in)]
    res = eval(tape, full, n, nthreads)
    return [ordered_sum(r) if red else r for r, red in zip(res, reduce_out)]


def mapsum_forward(tape, args, fseeds, n, reduce_in, reduce_out, nthreads=1):
    """MapSum::get_forward (mapsum.cpp:255-349): shared seeds (nfwd, nnz), summed
    sensitivities (nfwd, nnz)."""
    full = [_broadcast(a, n, r) for a, r in zip(args, reduce_in)]
    seeds = [_broadcast(a, n, r) for a, r in zip(fseeds, reduce_in)]
    res, fsens = forward(tape, full, seeds, n, nthreads)
    res = [ordered_sum(r) if red else r for r, red in zip(res, reduce_out)]
    fsens = [ordered_sum(r) if red else r for r, red in zip(fsens, reduce_out)]
    return res, fsens


def mapsum_reverse(tape, args, aseeds, n, reduce_in, reduce_out, nthreads=1):
    """MapSum::get_reverse (mapsum.cpp:351-413): the seeds of summed outputs are shared, the
    sensitivities of shared inputs summed."""
    full = [_broadcast(a, n, r) for a, r in zip(args, reduce_in)]
    seeds = [_broadcast(a, n, r) for a, r in zip(aseeds, reduce_out)]
    res, asens = reverse(tape, full, seeds, n, nthreads)
    res = [ordered_sum(r) if red else r for r, red in zip(res, reduce_out)]
    asens = [ordered_sum(r) if red else r for r, red in zip(asens, reduce_in)]
    return res, asens


def mapsum_sp_forward(tape, args, n, reduce_in, reduce_out):
    """MapSum::sp_forward (mapsum.cpp:190-193 with the bvec_t casadi_add, :148-152)."""
    full = [_broadcast(a, n, r) for a, r in zip(args, reduce_in)]
    res = sp_forward(tape, full, n)
    return [_or_all(r) if red else r for r, red in zip(res, reduce_out)]


def mapsum_sp_reverse(tape, args, res, n, reduce_in, reduce_out):
    """MapSum::sp_reverse (mapsum.cpp:196-232), in place: every instance sees the seed of a
    summed output (cleared at the end); a shared input ORs in every instance's bits."""
    if n == 0:
        return args, res
    work_args = [np.zeros((a.shape[0], n), np.uint64) if (a is not None and r) else a
                 for a, r in zip(args, reduce_in)]
    work_res = [_broadcast(s, n, r).astype(np.uint64) if (s is not None and r) else s
                for s, r in zip(res, reduce_out)]
    sp_reverse(tape, work_args, work_res, n)
    for j, r in enumerate(reduce_in):
        if r and args[j] is not None:
            args[j] |= _or_all(work_args[j])
    for j, r in enumerate(reduce_out):
        if r and res[j] is not None:
            res[j][...] = 0
    return args, res


def zero_checker(which, op):
    """0: f(0, y) == 0; 1: f(x, 0) == 0; 2: f(0, 0) == 0 (calculus.hpp:485-540)."""
    return bool(lib().sxo_zero_checker(which, op))


def fun(op, x, y):
    return lib().sxo_fun(op, x, y)


def der(op, x, y, f):
    d = np.zeros(2)
    lib().sxo_der(op, x, y, f, d.ctypes.data)
    return d


# ---- reference harness (only where it was built) --------------------------------------------
def ref_fun(op, x, y):
    return ref().ref_fun(op, x, y)


def ref_der(op, x, y, f):
    d = np.zeros(2)
    ref().ref_der(op, x, y, f, d.ctypes.data)
    return d


def ref_zero_checker(which, op):
    return bool(ref().ref_zero_checker(which, op))


def ref_activity(tape, args, n):
    t = TapeArrays(tape)
    args = _prep(args, np.uint64)
    res = _outs(tape.nnz_out, n, dtype=np.uint64)
    rc = ref().ref_activity(ct.c_int(tape.n_instr), t.op.ctypes.data_as(ct.c_void_p),
                            t.i0.ctypes.data_as(ct.c_void_p), t.i1.ctypes.data_as(ct.c_void_p),
                            t.i2.ctypes.data_as(ct.c_void_p), t.d.ctypes.data_as(ct.c_void_p),
                            ct.c_int(tape.sz_w), ct.c_long(n), _ptrs(args), _ptrs(res))
    assert rc == 0
    return res


def ref_eval(tape, args, n):
    t = TapeArrays(tape)
    args = _prep(args)
    res = _outs(tape.nnz_out, n)
    rc = ref().ref_eval(ct.c_int(tape.n_instr), t.op.ctypes.data_as(ct.c_void_p),
                        t.i0.ctypes.data_as(ct.c_void_p), t.i1.ctypes.data_as(ct.c_void_p),
                        t.i2.ctypes.data_as(ct.c_void_p), t.d.ctypes.data_as(ct.c_void_p),
                        ct.c_int(tape.sz_w), ct.c_long(n), _ptrs(args), _ptrs(res))
    assert rc == 0
    return res


def ref_forward(tape, args, fseeds, n):
    t = TapeArrays(tape)
    args = _prep(args)
    fseeds = _prep(fseeds)
    nfwd = next(s.shape[0] for s in fseeds if s is not None)
    _check(args, tape.nnz_in, n, "arguments")
    _check(fseeds, tape.nnz_in, n, "forward seeds", nfwd)
    fsens = _outs(tape.nnz_out, n, nfwd)
    rc = ref().ref_forward(ct.c_int(tape.n_instr), t.op.ctypes.data_as(ct.c_void_p),
                           t.i0.ctypes.data_as(ct.c_void_p), t.i1.ctypes.data_as(ct.c_void_p),
                           t.i2.ctypes.data_as(ct.c_void_p), t.d.ctypes.data_as(ct.c_void_p),
                           ct.c_int(tape.sz_w), ct.c_int(len(tape.nnz_in)),
                           t.nnz_in.ctypes.data_as(ct.c_void_p),
                           t.nnz_out.ctypes.data_as(ct.c_void_p), ct.c_long(n),
                           ct.c_int(nfwd), _ptrs(args), _ptrs(fseeds), _ptrs(fsens))
    assert rc == 0
    return fsens


def ref_jacobian(tape, args, n):
    t = TapeArrays(tape)
    args = _prep(args)
    nz = sum(tape.nnz_in)
    jac = _outs(tape.nnz_out, n, nz)
    rc = ref().ref_jacobian(ct.c_int(tape.n_instr), t.op.ctypes.data_as(ct.c_void_p),
                            t.i0.ctypes.data_as(ct.c_void_p), t.i1.ctypes.data_as(ct.c_void_p),
                            t.i2.ctypes.data_as(ct.c_void_p), t.d.ctypes.data_as(ct.c_void_p),
                            ct.c_int(tape.sz_w), ct.c_int(len(tape.nnz_in)),
                            t.nnz_in.ctypes.data_as(ct.c_void_p),
                            t.nnz_out.ctypes.data_as(ct.c_void_p), ct.c_long(n), _ptrs(args),
                            _ptrs(jac))
    assert rc == 0
    return jac


def ref_reverse(tape, args, aseeds, n):
    t = TapeArrays(tape)
    args = _prep(args)
    aseeds = _prep(aseeds)
    nadj = next(s.shape[0] for s in aseeds if s is not None)
    _check(args, tape.nnz_in, n, "arguments")
    _check(aseeds, tape.nnz_out, n, "adjoint seeds", nadj)
    asens = _outs(tape.nnz_in, n, nadj)
    rc = ref().ref_reverse(ct.c_int(tape.n_instr), t.op.ctypes.data_as(ct.c_void_p),
                           t.i0.ctypes.data_as(ct.c_void_p), t.i1.ctypes.data_as(ct.c_void_p),
                           t.i2.ctypes.data_as(ct.c_void_p), t.d.ctypes.data_as(ct.c_void_p),
                           ct.c_int(tape.sz_w), ct.c_int(len(tape.nnz_in)),
                           t.nnz_in.ctypes.data_as(ct.c_void_p),
                           t.nnz_out.ctypes.data_as(ct.c_void_p), ct.c_long(n),
                           ct.c_int(nadj), _ptrs(args), _ptrs(aseeds), _ptrs(asens))
    assert rc == 0
    return asens
