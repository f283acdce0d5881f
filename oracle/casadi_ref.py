"""ORACLE — test infrastructure only.

ctypes access to the reference's own libcasadi through ``casadi_bridge.cpp``
(``_ref/libcasadi_bridge.so``, built by ``make casadi REF=<reference tree>`` from the
reference's casadi/core sources). Used by the golden-fixture generator and by CPU tests that
run where the library was built; the product never loads it, and nothing on the GPU machine does
(the reference tree is not there, so neither is the library).

Array conventions: the functions here take and return this repository's instance-minor
layout, ``(nnz, n)`` per input/output, and convert to CasADi's instance-major buffers
(``arg[j] + i*nnz_in(j)``, casadi/core/map.cpp:150) internally.
"""
import ctypes as ct
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BRIDGE_PATH = os.path.join(HERE, "_ref", "libcasadi_bridge.so")

_lib = None


def available():
    return os.path.exists(BRIDGE_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = ct.CDLL(BRIDGE_PATH)
        _lib.cb_last_error.restype = ct.c_char_p
        _lib.cb_build.argtypes = [ct.c_char_p, ct.c_int]
        _lib.cb_derive.argtypes = [ct.c_int, ct.c_char_p, ct.c_int]
    return _lib


def _check(rc):
    if rc < 0:
        raise RuntimeError("libcasadi bridge: %s (status %d)"
                           % (lib().cb_last_error().decode(), rc))
    return rc


def _ptr(a):
    return ct.c_void_p(a.ctypes.data) if a is not None else ct.c_void_p(0)


def _ptrs(arrs):
    return (ct.c_void_p * max(1, len(arrs)))(*[_ptr(a).value for a in arrs])


def version():
    v = [ct.c_int() for _ in range(3)]
    lib().cb_version(*[ct.byref(x) for x in v])
    return tuple(x.value for x in v)


class Pattern:
    """A CCS sparsity pattern as CasADi stores it."""

    def __init__(self, nrow, ncol, colind, row):
        self.nrow, self.ncol = int(nrow), int(ncol)
        self.colind = np.asarray(colind, np.int64)
        self.row = np.asarray(row, np.int64)

    @property
    def nnz(self):
        return int(self.colind[-1])

    def col(self):
        return np.repeat(np.arange(self.ncol), np.diff(self.colind))


def _pattern(call):
    nrow, ncol, nnz = ct.c_int(), ct.c_int(), ct.c_int()
    _check(call(ct.byref(nrow), ct.byref(ncol), ct.byref(nnz), None, None, 0))
    colind = np.zeros(ncol.value + 1, np.int32)
    row = np.zeros(max(1, nnz.value), np.int32)
    _check(call(ct.byref(nrow), ct.byref(ncol), ct.byref(nnz), colind.ctypes.data_as(
        ct.POINTER(ct.c_int)), row.ctypes.data_as(ct.POINTER(ct.c_int)), nnz.value))
    return Pattern(nrow.value, ncol.value, colind, row[:nnz.value])


class Fn:
    """A casadi::Function held by the bridge."""

    def __init__(self, handle):
        self.h = _check(handle)
        n_in, n_out, sz_w, n_instr = ct.c_int(), ct.c_int(), ct.c_int(), ct.c_int()
        _check(lib().cb_io(self.h, ct.byref(n_in), ct.byref(n_out), None, None,
                           ct.byref(sz_w), ct.byref(n_instr)))
        nnz_in = np.zeros(max(1, n_in.value), np.int32)
        nnz_out = np.zeros(max(1, n_out.value), np.int32)
        _check(lib().cb_io(self.h, ct.byref(n_in), ct.byref(n_out), nnz_in.ctypes.data_as(
            ct.POINTER(ct.c_int)), nnz_out.ctypes.data_as(ct.POINTER(ct.c_int)),
            ct.byref(sz_w), ct.byref(n_instr)))
        self.n_in, self.n_out = n_in.value, n_out.value
        self.nnz_in = nnz_in[:self.n_in].tolist()
        self.nnz_out = nnz_out[:self.n_out].tolist()
        self.sz_w = sz_w.value
        self.n_instr = n_instr.value

    # -- structure ----------------------------------------------------------------------
    def tape(self):
        """The raw algorithm (SXFunction::algorithm_): arrays op, i0, i1, i2, d."""
        n = self.n_instr
        op, i0, i1, i2 = (np.zeros(n, np.int32) for _ in range(4))
        d = np.zeros(n, np.float64)
        _check(lib().cb_tape(self.h, *[_ptr(a) for a in (op, i0, i1, i2, d)]))
        return op, i0, i1, i2, d

    def sparsity_in(self, j):
        return _pattern(lambda *a: lib().cb_io_sparsity(self.h, 0, j, *a))

    def sparsity_out(self, j):
        return _pattern(lambda *a: lib().cb_io_sparsity(self.h, 1, j, *a))

    def jac_sparsity(self, oind, iind):
        return _pattern(lambda *a: lib().cb_jac_sparsity(self.h, oind, iind, *a))

    def partition(self, iind=0, oind=0, symmetric=False):
        """get_partition's seed colourings: (forward colours or None, adjoint colours or
        None) -- one colour per input column / output row."""
        n_col = self.sparsity_in(iind).nrow * self.sparsity_in(iind).ncol
        n_row = self.sparsity_out(oind).nrow * self.sparsity_out(oind).ncol
        c1 = np.full(max(1, self.nnz_in[iind], n_col), -1, np.int32)
        c2 = np.full(max(1, self.nnz_out[oind], n_row), -1, np.int32)
        n1, n2 = ct.c_int(), ct.c_int()
        _check(lib().cb_partition(self.h, iind, oind, int(symmetric), ct.byref(n1), _ptr(c1),
                                  ct.byref(n2), _ptr(c2)))
        return ((c1[:self.nnz_in[iind]] if n1.value else None),
                (c2[:self.nnz_out[oind]] if n2.value else None))

    # -- derived Functions --------------------------------------------------------------
    def jacobian(self):
        return Fn(lib().cb_derive(self.h, b"jacobian", 0))

    def forward(self, k):
        return Fn(lib().cb_derive(self.h, b"forward", k))

    def reverse(self, k):
        return Fn(lib().cb_derive(self.h, b"reverse", k))

    # -- numerics -----------------------------------------------------------------------
    def eval(self, args, n):
        """args: list (one per input) of (nnz_in, n) arrays or None; returns the outputs as
        (nnz_out, n) arrays. One raw operator() call per instance."""
        a_im = [None if a is None or self.nnz_in[j] == 0 else
                np.ascontiguousarray(np.asarray(a, np.float64).reshape(self.nnz_in[j], n).T)
                for j, a in enumerate(args)]
        a_im += [None] * (self.n_in - len(a_im))
        r_im = [np.zeros((n, k)) for k in self.nnz_out]
        _check(lib().cb_eval(self.h, n, _ptrs(a_im), _ptrs(r_im)))
        return [r.T.copy() for r in r_im]

    def sp_forward(self, seeds):
        """One bvec_t forward sweep: seeds (one uint64 array per input nonzero list) ->
        dependency words of every output nonzero."""
        a = [np.ascontiguousarray(s, np.uint64) for s in seeds]
        r = [np.zeros(k, np.uint64) for k in self.nnz_out]
        _check(lib().cb_sp(self.h, 1, _ptrs(a), _ptrs(r)))
        return r

    def sp_reverse(self, seeds):
        """One bvec_t reverse sweep: output seeds -> input words (the seeds are consumed, as
        in the reference; copies are passed here)."""
        a = [np.zeros(k, np.uint64) for k in self.nnz_in]
        r = [np.array(s, np.uint64) for s in seeds]
        _check(lib().cb_sp(self.h, 0, _ptrs(a), _ptrs(r)))
        return a, r

    def time_map(self, args, n, parallelization="openmp", reps=5):
        """Seconds of each of ``reps`` calls of f.map(n, parallelization) through the raw
        operator() (one checkout, one warm-up call first). args instance-minor (nnz, n)."""
        a_im = [np.ascontiguousarray(np.asarray(a, np.float64).reshape(self.nnz_in[j], n).T)
                if a is not None and self.nnz_in[j] else None for j, a in enumerate(args)]
        a_im += [None] * (self.n_in - len(a_im))
        r_im = [np.zeros((n, k)) for k in self.nnz_out]
        sec = np.zeros(reps)
        _check(lib().cb_time_map(self.h, n, parallelization.encode(), reps, _ptrs(a_im),
                                 _ptrs(r_im), _ptr(sec)))
        return sec, [r.T.copy() for r in r_im]


def build(name, param=0):
    """A workload Function built with CasADi's SX: "cartpole", "rollout" (param = steps),
    "quad_lagrangian" / "quad_gradient" / "quad_hessian" / "quad_jac_g" (param =
    intervals)."""
    return Fn(lib().cb_build(name.encode(), int(param)))


def build_dag(n_in, n_out, op, a, b, bounded=False):
    """The random DAG of a node list (casadi_gb300.workloads.dag_nodes) built with CasADi's
    SX."""
    op, a, b = (np.ascontiguousarray(v, np.int32) for v in (op, a, b))
    return Fn(lib().cb_build_dag(n_in, n_in + op.size, n_out, _ptr(op), _ptr(a), _ptr(b),
                                 int(bounded)))


def coloring(kind, A, param=1):
    """Colour of every column of pattern A by Sparsity::uni_coloring ("uni"),
    star_coloring(param) ("star") or star_coloring2(param) ("star2")."""
    k = {"uni": 0, "star": 1, "star2": 2}[kind]
    colind = np.ascontiguousarray(A.colind, np.int32)
    row = np.ascontiguousarray(A.row if A.row.size else np.zeros(1), np.int32)
    color = np.zeros(max(1, A.ncol), np.int32)
    nc = ct.c_int()
    _check(lib().cb_coloring(k, int(param), A.nrow, A.ncol, _ptr(colind), _ptr(row),
                             _ptr(color), ct.byref(nc)))
    return color[:A.ncol].astype(np.int64), nc.value
