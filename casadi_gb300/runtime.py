"""Python host side of the GB300 evaluator: ctypes bindings over the C ABI in
``include/casadi_gb300.h`` and a tape object that runs the sweeps on device tensors.

The CUDA library is the only compute path. If it is missing or cannot be loaded this module
raises; there is no CPU fallback.

Device arrays use the instance-minor layout of the C ABI: one tensor per input/output of shape
``(nnz, n)`` (float64, contiguous, on the tape's CUDA device); seeds and sensitivities have
shape ``(ndir, nnz, n)``.
"""
import ctypes as ct
import os
import re

import numpy as np

from . import sx as _sx

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcasadi_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "casadi_gb300.h")

_lib = None


class CasadiGpuError(RuntimeError):
    """A C-ABI call returned a nonzero status."""

    def __init__(self, status, message):
        super().__init__("casadi_gb300 status %d: %s" % (status, message))
        self.status = status


class Atomic(ct.Structure):
    """casadi_gb300_atomic: the 16-byte ScalarAtomic layout."""
    _fields_ = [("op", ct.c_int), ("i0", ct.c_int), ("u", ct.c_uint64)]


def declared_symbols():
    """Entry points declared in include/casadi_gb300.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"CASADI_GB300_API\s+[\w\s\*]+?\b(casadi_gb300_\w+)\s*\(", text)))


def load(path=None):
    """Load libcasadi_gb300.so (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    lib = ct.CDLL(path)
    vp, i64, cint, sz = ct.c_void_p, ct.c_int64, ct.c_int, ct.c_size_t
    sig = {
        "casadi_gb300_last_error": (ct.c_char_p, []),
        "casadi_gb300_version": (ct.c_char_p, []),
        "casadi_gb300_tape_create": (cint, [vp, cint, cint, vp, cint, vp, cint]),
        "casadi_gb300_tape_free": (cint, [cint]),
        "casadi_gb300_tape_create_calls": (cint, [vp, cint, cint, vp, cint, vp, cint, cint, vp, vp,
                                                  vp]),
        "casadi_gb300_tape_deserialize": (cint, [ct.c_char_p, sz]),
        "casadi_gb300_serialized_decode": (cint, [ct.c_char_p, sz, vp, cint, vp, vp, vp, vp, vp,
                                                  vp]),
        "casadi_gb300_serialized_describe": (cint, [ct.c_char_p, sz, vp, sz, vp]),
        "casadi_gb300_push_file": (cint, [ct.c_char_p]),
        "casadi_gb300_pop_file": (cint, []),
        "casadi_gb300_n_loaded": (cint, []),
        "casadi_gb300_loaded_tape": (cint, [ct.c_char_p]),
        "casadi_gb300_loaded_name": (ct.c_char_p, [cint]),
        "casadi_gb300_tape_schedule": (cint, [vp, cint, cint, vp, cint, vp, cint, vp, vp]),
        "casadi_gb300_tape_info": (cint, [cint, vp, vp, vp, vp, vp]),
        "casadi_gb300_tape_levels": (cint, [vp, cint, cint, vp, cint, vp, cint, cint, cint, vp,
                                             vp, vp, vp, vp]),
        "casadi_gb300_scratch_size": (cint, [cint, i64, vp]),
        "casadi_gb300_scratch_min": (cint, [cint, vp]),
        "casadi_gb300_eval": (cint, [cint, i64, i64, vp, vp, vp]),
        "casadi_gb300_forward": (cint, [cint, i64, i64, cint, vp, vp, vp, vp, vp, sz, vp]),
        "casadi_gb300_reverse": (cint, [cint, i64, i64, cint, vp, vp, vp, vp, vp, sz, vp]),
        "casadi_gb300_sp_forward": (cint, [cint, i64, i64, vp, vp, vp]),
        "casadi_gb300_sp_reverse": (cint, [cint, i64, i64, vp, vp, vp]),
        "casadi_gb300_eval_activity": (cint, [cint, i64, i64, vp, vp, vp]),
        "casadi_gb300_mapsum_scratch_size": (cint, [cint, i64, cint, vp, vp]),
        "casadi_gb300_mapaccum_scratch_size": (cint, [cint, cint, cint, i64, cint, vp]),
        "casadi_gb300_mapaccum_reverse_scratch_size": (cint, [cint, cint, cint, i64, cint, vp]),
        "casadi_gb300_mapaccum_eval": (cint, [cint, cint, cint, i64, i64, vp, vp, vp, sz, vp]),
        "casadi_gb300_mapaccum_forward": (cint, [cint, cint, cint, i64, i64, cint, vp, vp, vp,
                                                 vp, vp, sz, vp]),
        "casadi_gb300_mapaccum_reverse": (cint, [cint, cint, cint, i64, i64, cint, vp, vp, vp,
                                                 vp, vp, sz, vp]),
        "casadi_gb300_mapsum_eval": (cint, [cint, i64, i64, vp, vp, vp, vp, sz, vp]),
        "casadi_gb300_mapsum_forward": (cint, [cint, i64, i64, vp, cint, vp, vp, vp, vp, vp, sz,
                                               vp]),
        "casadi_gb300_mapsum_reverse": (cint, [cint, i64, i64, vp, cint, vp, vp, vp, vp, vp, sz,
                                               vp]),
        "casadi_gb300_mapsum_sp_forward": (cint, [cint, i64, i64, vp, vp, vp, vp, sz, vp]),
        "casadi_gb300_mapsum_sp_reverse": (cint, [cint, i64, i64, vp, vp, vp, vp, sz, vp]),
        "casadi_gb300_sync": (cint, [cint, vp]),
        "casadi_gb300_checkout": (cint, []),
        "casadi_gb300_release": (cint, [cint]),
        "casadi_gb300_map_eval": (cint, [cint, cint, i64, vp, vp]),
        "casadi_gb300_map_reverse": (cint, [cint, cint, i64, cint, vp, vp, vp, vp]),
        "casadi_gb300_map_forward": (cint, [cint, cint, i64, cint, vp, vp, vp, vp]),
        "casadi_gb300_map_forward_outer": (cint, [cint, cint, i64, cint, vp, vp, vp, vp]),
        "casadi_gb300_map_sp_forward": (cint, [cint, cint, i64, vp, vp]),
        "casadi_gb300_map_sp_reverse": (cint, [cint, cint, i64, vp, vp]),
        "casadi_gb300_map_reverse_outer": (cint, [cint, cint, i64, cint, vp, vp, vp, vp]),
        "casadi_gb300_jacobian": (cint, [cint, i64, i64, vp, vp, vp, vp, sz, vp]),
        "casadi_gb300_map_jacobian": (cint, [cint, cint, i64, vp, vp, vp]),
        "casadi_gb300_jacobian_reverse": (cint, [cint, i64, i64, vp, vp, vp, cint, vp, vp, vp, sz,
                                                 vp]),
        "casadi_gb300_map_jacobian_reverse": (cint, [cint, cint, i64, vp, vp, vp, cint, vp, vp]),
        "casadi_gb300_reverse_noalloc": (cint, [cint, i64, i64, cint, vp, vp, vp, vp, vp]),
        "casadi_gb300_checkpoint_scratch_size": (cint, [cint, cint, cint, i64, vp, vp]),
        "casadi_gb300_reverse_checkpointed": (cint, [cint, i64, i64, cint, cint, vp, vp, vp, vp,
                                                     vp, sz, vp]),
        "casadi_gb300_tape_segments": (cint, [vp, cint, cint, vp, cint, vp, cint, cint, vp, vp,
                                              vp, vp, cint, vp]),
        "casadi_gb300_profile": (cint, [cint]),
        "casadi_gb300_profile_collect": (cint, [vp, vp, cint]),
        "casadi_gb300_autotune": (cint, [cint]),
        "casadi_gb300_tuned_variant": (cint, [cint, cint, vp]),
        "casadi_gb300_set_variant": (cint, [cint, cint, cint]),
        "casadi_gb300_set_residence": (cint, [cint, cint]),
        "casadi_gb300_uni_coloring": (cint, [cint, cint, vp, vp, vp]),
        "casadi_gb300_jacobian_colored": (cint, [cint, i64, i64, cint, vp, vp, vp, vp, vp, sz,
                                                 vp]),
        "casadi_gb300_gather": (cint, [i64, i64, cint, vp, vp, vp, vp]),
        "casadi_gb300_star_coloring": (cint, [cint, vp, vp, cint, vp]),
        "casadi_gb300_batch_create": (cint, []),
        "casadi_gb300_batch_free": (cint, [cint]),
        "casadi_gb300_batch_add": (cint, [cint, cint, i64, i64, cint, vp, vp, vp, vp]),
        "casadi_gb300_batch_scratch_size": (cint, [cint, vp]),
        "casadi_gb300_batch_status": (cint, [cint]),
        "casadi_gb300_batch_set_residence": (cint, [cint, cint]),
        "casadi_gb300_check_wait_timeout": (cint, [vp]),
        "casadi_gb300_batch_add_jacobian_colored": (cint, [cint, cint, i64, i64, cint, vp, vp, vp,
                                                           vp]),
        "casadi_gb300_batch_run": (cint, [cint, vp, sz, cint, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status < 0:
        msg = load().casadi_gb300_last_error().decode(errors="replace")
        raise CasadiGpuError(status, msg)
    return status


def _ptr_array(tensors):
    arr = (ct.c_void_p * max(1, len(tensors)))()
    for k, t in enumerate(tensors):
        arr[k] = None if t is None else t.data_ptr()
    return arr


def _stream_handle(stream):
    if stream is None:
        import torch
        return ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    return ct.c_void_p(getattr(stream, "cuda_stream", stream))


def schedule(tape):
    """The tape in the order and slots the GPU sweeps run it (host only, no device needed):
    returns a new :class:`sx.Tape` with the same instructions reordered for fewer live values
    and a shorter work vector."""
    if isinstance(tape, _sx.Function):
        tape = tape.tape
    lib = load()
    atoms = tape.atomic_array()
    out = np.zeros_like(atoms)
    nnz_in = np.ascontiguousarray(tape.nnz_in, dtype=np.int32)
    nnz_out = np.ascontiguousarray(tape.nnz_out, dtype=np.int32)
    szw = ct.c_int()
    check(lib.casadi_gb300_tape_schedule(atoms.ctypes.data, tape.n_instr, len(tape.nnz_in),
                                         nnz_in.ctypes.data, len(tape.nnz_out),
                                         nnz_out.ctypes.data, tape.sz_w, out.ctypes.data,
                                         ct.byref(szw)))
    return _sx.Tape.from_atomic_array(out, tape.nnz_in, tape.nnz_out, szw.value)


def segments(tape, count):
    """The segment plan of :meth:`CudaTape.reverse_checkpointed` (host only, no device
    needed): returns (cut positions in :func:`schedule`'s instruction list, live slot count at
    each cut, the segment tapes as :class:`sx.Tape`). Segment s has the tape's inputs plus one
    more (the slots live at cut s) and its outputs plus one more (the slots live at cut s+1);
    it writes only the outputs of its own instructions."""
    if isinstance(tape, _sx.Function):
        tape = tape.tape
    lib = load()
    atoms = tape.atomic_array()
    nnz_in = np.ascontiguousarray(tape.nnz_in, dtype=np.int32)
    nnz_out = np.ascontiguousarray(tape.nnz_out, dtype=np.int32)
    cut = np.zeros(count + 1, dtype=np.int32)
    live = np.zeros(count + 1, dtype=np.int32)
    seg_len = np.zeros(max(1, count), dtype=np.int32)
    cap = tape.n_instr + 2 * tape.sz_w * count
    out = np.zeros(max(1, cap), dtype=atoms.dtype)
    szw = ct.c_int()
    k = check(lib.casadi_gb300_tape_segments(atoms.ctypes.data, tape.n_instr, len(tape.nnz_in),
                                             nnz_in.ctypes.data, len(tape.nnz_out),
                                             nnz_out.ctypes.data, tape.sz_w, count,
                                             cut.ctypes.data, live.ctypes.data,
                                             seg_len.ctypes.data, out.ctypes.data, cap,
                                             ct.byref(szw)))
    tapes, off = [], 0
    for s in range(k):
        a = out[off:off + seg_len[s]]
        off += seg_len[s]
        tapes.append(_sx.Tape.from_atomic_array(a.copy(), list(tape.nnz_in) + [int(live[s])],
                                                list(tape.nnz_out) + [int(live[s + 1])],
                                                szw.value))
    return cut[:k + 1].tolist(), live[:k + 1].tolist(), tapes


def levels(tape, width=32, slot_cap=None):
    """The level schedule of the cooperative sweeps (host only): returns (leveled tape,
    source index of each instruction in :func:`schedule`'s tape, level offsets)."""
    if isinstance(tape, _sx.Function):
        tape = tape.tape
    lib = load()
    atoms = tape.atomic_array()
    nnz_in = np.ascontiguousarray(tape.nnz_in, dtype=np.int32)
    nnz_out = np.ascontiguousarray(tape.nnz_out, dtype=np.int32)
    out = np.zeros_like(atoms)
    src = np.zeros(max(1, tape.n_instr), dtype=np.int32)
    begin = np.zeros(tape.n_instr + 1, dtype=np.int32)
    nl, szw = ct.c_int(), ct.c_int()
    cap = slot_cap if slot_cap is not None else 1 << 30
    check(lib.casadi_gb300_tape_levels(atoms.ctypes.data, tape.n_instr, len(tape.nnz_in),
                                       nnz_in.ctypes.data, len(tape.nnz_out),
                                       nnz_out.ctypes.data, tape.sz_w, width, cap,
                                       out.ctypes.data, src.ctypes.data, begin.ctypes.data,
                                       ct.byref(nl), ct.byref(szw)))
    lt = _sx.Tape.from_atomic_array(out, tape.nnz_in, tape.nnz_out, szw.value)
    return lt, src[:tape.n_instr], begin[:nl.value + 1]


def _serial_text(text):
    """Serialized text as bytes: a str/bytes of CasADi's serialization, or a path to a file
    that Function::save wrote."""
    if isinstance(text, os.PathLike) or (isinstance(text, str) and os.path.exists(text)):
        with open(text, "rb") as fh:
            return fh.read()
    return text.encode() if isinstance(text, str) else bytes(text)


def describe_serialized(text):
    """Summary of a serialized CasADi Function (any class) as a dict: ``functions`` (class,
    name, inputs/outputs with their names and sparsity sizes, and for SXFunctions the
    instruction count, work-vector size and called functions), ``top`` (index of the
    serialized one), ``debug``, ``saved_form``. Host only."""
    import json
    b = _serial_text(text)
    lib = load()
    need = ct.c_size_t()
    check(lib.casadi_gb300_serialized_describe(b, len(b), None, 0, ct.byref(need)))
    buf = ct.create_string_buffer(need.value)
    check(lib.casadi_gb300_serialized_describe(b, len(b), buf, need.value, None))
    return json.loads(buf.value.decode())


def decode_serialized(text):
    """The :class:`sx.Tape` of a serialized SXFunction without calls, decoded on the host (the
    algorithm, nonzero counts and work-vector size CasADi wrote)."""
    b = _serial_text(text)
    lib = load()
    n, nin, nout, szw = ct.c_int(), ct.c_int(), ct.c_int(), ct.c_int()
    check(lib.casadi_gb300_serialized_decode(b, len(b), None, 0, ct.byref(n), ct.byref(nin),
                                             None, ct.byref(nout), None, ct.byref(szw)))
    atoms = np.zeros(n.value, dtype=np.dtype([("op", "<i4"), ("i0", "<i4"), ("u", "<u8")]))
    nnz_in = np.zeros(max(1, nin.value), dtype=np.int32)
    nnz_out = np.zeros(max(1, nout.value), dtype=np.int32)
    check(lib.casadi_gb300_serialized_decode(b, len(b), atoms.ctypes.data, n.value, None, None,
                                             nnz_in.ctypes.data, None, nnz_out.ctypes.data,
                                             None))
    return _sx.Tape.from_atomic_array(atoms, nnz_in[:nin.value].tolist(),
                                      nnz_out[:nout.value].tolist(), szw.value)


def push_file(path):
    """Load every SXFunction of a file Function::save or a FileSerializer wrote (one Function
    or a vector of them) into the library's list of loaded functions, as casadi_c_push_file
    does; returns {name: CudaTape} for the functions of this file. The tapes belong to the
    list (pop_file frees them)."""
    lib = load()
    check(lib.casadi_gb300_push_file(os.fsencode(path)))
    d = describe_serialized(path)
    out = {}
    for k in d["tops"]:
        f = d["functions"][k]
        out[f["name"]] = CudaTape._wrap(check(lib.casadi_gb300_loaded_tape(f["name"].encode())),
                                        f, None, owned=False)
    return out


def pop_file():
    """Free the tapes the last push_file loaded."""
    check(load().casadi_gb300_pop_file())


def loaded_names():
    lib = load()
    return [lib.casadi_gb300_loaded_name(k).decode() for k in range(lib.casadi_gb300_n_loaded())]


class CudaTape:
    """A tape registered with the GPU library (one CUDA device)."""

    @classmethod
    def deserialize(cls, text):
        """The tape of a serialized SXFunction (the text Function::serialize() returns, or a
        file Function::save wrote); SXFunctions it calls are decoded and inlined."""
        b = _serial_text(text)
        lib = load()
        tid = check(lib.casadi_gb300_tape_deserialize(b, len(b)))
        top = describe_serialized(b)
        return cls._wrap(tid, top["functions"][top["top"]], b)

    @classmethod
    def _wrap(cls, tid, f, text, owned=True):
        """A CudaTape object for tape `tid` of the serialized function described by `f`."""
        lib = load()
        self = cls.__new__(cls)
        self.id = tid
        self._owned = owned
        nnz_in = [io["nnz"] for io in f["inputs"]]
        nnz_out = [io["nnz"] for io in f["outputs"]]
        self.name = f["name"]
        self.name_in = [io["name"] for io in f["inputs"]]
        self.name_out = [io["name"] for io in f["outputs"]]
        self.tape = decode_serialized(text) if text is not None and not f["calls"] else \
            _sx.Tape.from_atomic_array(np.zeros(0, dtype=np.dtype([("op", "<i4"), ("i0", "<i4"),
                                                                    ("u", "<u8")])),
                                       nnz_in, nnz_out, f["sz_w"])
        self._nnz_in = np.ascontiguousarray(nnz_in, dtype=np.int32)
        self._nnz_out = np.ascontiguousarray(nnz_out, dtype=np.int32)
        vals = [ct.c_int() for _ in range(5)]
        check(lib.casadi_gb300_tape_info(self.id, *[ct.byref(v) for v in vals]))
        self.n_instr, self.n_in, self.n_out, self.sz_w, self.n_partials = [v.value for v in vals]
        self._scratch = None
        return self

    def __init__(self, tape, calls=None):
        """``tape``: an :class:`sx.Function` or :class:`sx.Tape`. ``calls``: for tapes with
        OP_CALL instructions (call index in ``i1``), a list of ``(callee CudaTape, dep slots,
        res slots)``; the calls are inlined by the library."""
        if isinstance(tape, _sx.Function):
            tape = tape.tape
        self.tape = tape
        lib = load()
        atoms = tape.atomic_array()
        self._nnz_in = np.ascontiguousarray(tape.nnz_in, dtype=np.int32)
        self._nnz_out = np.ascontiguousarray(tape.nnz_out, dtype=np.int32)
        if calls:
            ids = np.ascontiguousarray([c[0].id for c in calls], dtype=np.int32)
            deps = [np.ascontiguousarray(c[1], dtype=np.int32) for c in calls]
            ress = [np.ascontiguousarray(c[2], dtype=np.int32) for c in calls]
            dptr = (ct.c_void_p * len(calls))(*[d.ctypes.data for d in deps])
            rptr = (ct.c_void_p * len(calls))(*[x.ctypes.data for x in ress])
            self._callees = [c[0] for c in calls]  # keep the callee tapes registered
            self.id = check(lib.casadi_gb300_tape_create_calls(
                atoms.ctypes.data, tape.n_instr, len(tape.nnz_in), self._nnz_in.ctypes.data,
                len(tape.nnz_out), self._nnz_out.ctypes.data, tape.sz_w, len(calls),
                ids.ctypes.data, dptr, rptr))
        else:
            self.id = check(lib.casadi_gb300_tape_create(
                atoms.ctypes.data, tape.n_instr, len(tape.nnz_in), self._nnz_in.ctypes.data,
                len(tape.nnz_out), self._nnz_out.ctypes.data, tape.sz_w))
        vals = [ct.c_int() for _ in range(5)]
        check(lib.casadi_gb300_tape_info(self.id, *[ct.byref(v) for v in vals]))
        self.n_instr, self.n_in, self.n_out, self.sz_w, self.n_partials = [v.value for v in vals]
        self._scratch = None

    def __del__(self):
        try:
            if (getattr(self, "id", None) is not None and _lib is not None
                    and getattr(self, "_owned", True)):
                _lib.casadi_gb300_tape_free(self.id)
        except Exception:
            pass

    @property
    def nnz_in(self):
        return list(self.tape.nnz_in)

    @property
    def nnz_out(self):
        return list(self.tape.nnz_out)

    # -- scratch for the AD sweeps (device memory owned by this object) --------------------------
    def scratch_bytes(self, n):
        b = ct.c_size_t()
        check(load().casadi_gb300_scratch_size(self.id, n, ct.byref(b)))
        return b.value

    def scratch(self, n, max_bytes=None):
        import torch
        need = self.scratch_bytes(n)
        if max_bytes is not None:
            mn = ct.c_size_t()
            check(load().casadi_gb300_scratch_min(self.id, ct.byref(mn)))
            need = max(mn.value, min(need, max_bytes))
        if self._scratch is None or self._scratch.numel() < need:
            self._scratch = torch.empty(max(need, 8), dtype=torch.uint8, device="cuda")
        return self._scratch

    # -- sweeps on device tensors ----------------------------------------------------------------
    def _outs(self, nnz, n, ndir=None, dtype=None):
        import torch
        dtype = dtype or torch.float64
        shape = (lambda k: (k, n)) if ndir is None else (lambda k: (ndir, k, n))
        return [torch.empty(shape(k), dtype=dtype, device="cuda") for k in nnz]

    @staticmethod
    def _n(args):
        for a in args:
            if a is not None:
                return a.shape[-1]
        raise ValueError("cannot infer the instance count from all-null inputs")

    def eval(self, args, n=None, res=None, stream=None):
        n = self._n(args) if n is None else n
        res = self._outs(self.nnz_out, n) if res is None else res
        check(load().casadi_gb300_eval(self.id, n, n, _ptr_array(args), _ptr_array(res),
                                       _stream_handle(stream)))
        return res

    def forward(self, args, fseeds, n=None, res=None, fsens=None, stream=None,
                scratch_limit=None):
        n = self._n(args) if n is None else n
        nfwd = next(s.shape[0] for s in fseeds if s is not None)
        res = self._outs(self.nnz_out, n) if res is None else res
        fsens = self._outs(self.nnz_out, n, nfwd) if fsens is None else fsens
        sc = self.scratch(n, scratch_limit)
        check(load().casadi_gb300_forward(
            self.id, n, n, nfwd, _ptr_array(args), _ptr_array(res), _ptr_array(fseeds),
            _ptr_array(fsens), ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream)))
        return res, fsens

    def reverse(self, args, aseeds, n=None, res=None, asens=None, stream=None,
                scratch_limit=None):
        n = self._n(args) if n is None else n
        nadj = next(s.shape[0] for s in aseeds if s is not None)
        res = self._outs(self.nnz_out, n) if res is None else res
        asens = self._outs(self.nnz_in, n, nadj) if asens is None else asens
        sc = self.scratch(n, scratch_limit)
        check(load().casadi_gb300_reverse(
            self.id, n, n, nadj, _ptr_array(args), _ptr_array(res), _ptr_array(aseeds),
            _ptr_array(asens), ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream)))
        return res, asens

    def jacobian(self, args, n=None, res=None, jac=None, stream=None, scratch_limit=None):
        """Values and the Jacobian of every output w.r.t. every input nonzero:
        jac[j] has shape (nnz_in_total, nnz_out[j], n); jac[j][d, k, i] = d out_j[k] / d in[d]."""
        n = self._n(args) if n is None else n
        nz = sum(self.nnz_in)
        res = self._outs(self.nnz_out, n) if res is None else res
        jac = self._outs(self.nnz_out, n, nz) if jac is None else jac
        sc = self.scratch(n, scratch_limit)
        check(load().casadi_gb300_jacobian(
            self.id, n, n, _ptr_array(args), _ptr_array(res), _ptr_array(jac),
            ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream)))
        return res, jac

    def jacobian_reverse(self, args, aseeds, n=None, res=None, jac=None, asens=None,
                         stream=None, scratch_limit=None):
        """Jacobian (as :meth:`jacobian`) and adjoint sensitivities (as :meth:`reverse`) from
        one record sweep."""
        n = self._n(args) if n is None else n
        nz = sum(self.nnz_in)
        nadj = next(s.shape[0] for s in aseeds if s is not None)
        res = self._outs(self.nnz_out, n) if res is None else res
        jac = self._outs(self.nnz_out, n, nz) if jac is None else jac
        asens = self._outs(self.nnz_in, n, nadj) if asens is None else asens
        sc = self.scratch(n, scratch_limit)
        check(load().casadi_gb300_jacobian_reverse(
            self.id, n, n, _ptr_array(args), _ptr_array(res), _ptr_array(jac), nadj,
            _ptr_array(aseeds), _ptr_array(asens), ct.c_void_p(sc.data_ptr()), sc.numel(),
            _stream_handle(stream)))
        return res, jac, asens

    def checkpoint_scratch(self, segments, nadj, n, max_bytes=None):
        """Scratch of :meth:`reverse_checkpointed` (one wave of all n instances, or at most
        max_bytes but not below the minimum); returns (buffer, segments made)."""
        import torch
        full, least = ct.c_size_t(), ct.c_size_t()
        k = check(load().casadi_gb300_checkpoint_scratch_size(self.id, segments, nadj, n,
                                                              ct.byref(full), ct.byref(least)))
        need = full.value if max_bytes is None else max(least.value, min(full.value, max_bytes))
        return torch.empty(max(need, 8), dtype=torch.uint8, device="cuda"), k

    def reverse_checkpointed(self, args, aseeds, segments, n=None, res=None, asens=None,
                             stream=None, scratch_limit=None):
        """As :meth:`reverse`, with segment checkpointing: the tape cut into ``segments``
        runs, the live slots at each cut kept, each run re-recorded in the backward pass."""
        n = self._n(args) if n is None else n
        nadj = next((s.shape[0] for s in aseeds if s is not None), 0) if aseeds else 0
        res = self._outs(self.nnz_out, n) if res is None else res
        asens = self._outs(self.nnz_in, n, nadj) if asens is None else asens
        sc, _ = self.checkpoint_scratch(segments, nadj, n, scratch_limit)
        check(load().casadi_gb300_reverse_checkpointed(
            self.id, n, n, nadj, segments, _ptr_array(args), _ptr_array(res),
            _ptr_array(aseeds) if aseeds else None, _ptr_array(asens) if nadj else None,
            ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream)))
        self._keep = sc  # the sweep may still be running on the stream
        return res, asens

    def sp_forward(self, args, n=None, stream=None):
        """args: int64 tensors holding bvec_t bit patterns, shape (nnz, n)."""
        import torch
        n = self._n(args) if n is None else n
        res = self._outs(self.nnz_out, n, dtype=torch.int64)
        check(load().casadi_gb300_sp_forward(self.id, n, n, _ptr_array(args), _ptr_array(res),
                                             _stream_handle(stream)))
        return res

    def eval_activity(self, args, n=None, stream=None):
        """Activity words of the outputs (SXFunction::eval_activity): args are int64 tensors
        (nnz, n) of input activity words (nonzero: possibly nonzero input)."""
        import torch
        n = self._n(args) if n is None else n
        res = self._outs(self.nnz_out, n, dtype=torch.int64)
        check(load().casadi_gb300_eval_activity(self.id, n, n, _ptr_array(args),
                                                _ptr_array(res), _stream_handle(stream)))
        return res

    def activity(self, masks):
        """Function::activity over instances (casadi/core/function.cpp:1269-1294): ``masks``
        is a bool array (nnz_in_total, n) of possibly-nonzero inputs; returns a bool array
        (nnz_out_total, n) of possibly-nonzero outputs."""
        import torch
        masks = np.asarray(masks, dtype=bool)
        if masks.ndim != 2 or masks.shape[0] != sum(self.nnz_in):
            raise ValueError("activity: expected a mask of %d input nonzeros per instance"
                             % sum(self.nnz_in))
        n = masks.shape[1]
        words = torch.from_numpy(np.where(masks, -1, 0).astype(np.int64)).cuda()
        args, off = [], 0
        for k in self.nnz_in:
            args.append(words[off:off + k])
            off += k
        res = self.eval_activity(args, n=n)
        return np.concatenate([r.cpu().numpy() != 0 for r in res], axis=0) if res else \
            np.zeros((0, n), dtype=bool)

    def sp_reverse(self, args, res, n=None, stream=None):
        """In place: args |= propagated bits, res cleared (SXFunction::sp_reverse)."""
        n = self._n(args + res) if n is None else n
        check(load().casadi_gb300_sp_reverse(self.id, n, n, _ptr_array(args), _ptr_array(res),
                                             _stream_handle(stream)))
        return args, res

    def sync(self, stream=None):
        check(load().casadi_gb300_sync(self.id, _stream_handle(stream)))

    def set_residence(self, mode):
        """Work-vector residence: 0 auto (tuned), 1 global memory, 2 shared memory when it fits,
        3 the cooperative level sweep for value/record/sparsity sweeps."""
        check(load().casadi_gb300_set_residence(self.id, mode))

    def set_variant(self, kind, variant):
        """Fix the derivative-sweep variant of one kind (-1: let the autotuner choose)."""
        check(load().casadi_gb300_set_variant(self.id, kind, variant))

    def tuned_variant(self, kind):
        """Derivative-sweep variant the autotuner kept: kind 0 forward, 1 Jacobian, 2 adjoint."""
        v = ct.c_int()
        check(load().casadi_gb300_tuned_variant(self.id, kind, ct.byref(v)))
        return v.value


class _MapSumSpec(ct.Structure):
    _fields_ = [("reduce_in", ct.c_void_p), ("reduce_out", ct.c_void_p), ("order", ct.c_int)]


class CudaMapSum:
    """``f.map(name, "cuda", n, reduce_in, reduce_out)``: MapSum over n instances
    (casadi/core/mapsum.cpp) on device tensors. A shared input (``reduce_in``) is one column,
    shape (nnz,), used by every instance; a summed output (``reduce_out``) is returned as its
    sum over the instances, shape (nnz,). Other inputs/outputs are (nnz, n) as in
    :class:`CudaTape`. Seeds of shared inputs and sensitivities of summed outputs carry a
    leading direction axis: (ndir, nnz).

    ``order=0`` sums in instance order (MapSum's own order, the reference's bits);
    ``order=1`` uses a fixed blocked tree that does not chain n dependent adds."""

    class_name = "MapSum"
    parallelization = "cuda"

    def __init__(self, f, n, reduce_in=None, reduce_out=None, order=0):
        self.tape = f if isinstance(f, CudaTape) else CudaTape(f)
        self.n = int(n)
        nin, nout = len(self.tape.nnz_in), len(self.tape.nnz_out)
        self.reduce_in = [bool(v) for v in (reduce_in or [False] * nin)]
        self.reduce_out = [bool(v) for v in (reduce_out or [False] * nout)]
        if len(self.reduce_in) != nin or len(self.reduce_out) != nout:
            raise ValueError("reduce_in/reduce_out: one flag per input/output")
        self._rin = np.ascontiguousarray(self.reduce_in, dtype=np.int32)
        self._rout = np.ascontiguousarray(self.reduce_out, dtype=np.int32)
        self._spec = _MapSumSpec(self._rin.ctypes.data, self._rout.ctypes.data, int(order))
        self._scratch = None
        self.name = "mapsum%d_%s" % (self.n, getattr(f, "name", "f"))

    @property
    def order(self):
        return self._spec.order

    def scratch(self, ndir=0):
        import torch
        b = ct.c_size_t()
        check(load().casadi_gb300_mapsum_scratch_size(self.tape.id, self.n, ndir,
                                                      ct.byref(self._spec), ct.byref(b)))
        if self._scratch is None or self._scratch.numel() < b.value:
            self._scratch = torch.empty(max(b.value, 8), dtype=torch.uint8, device="cuda")
        return self._scratch

    def _res(self, nnz, summed, ndir=None, dtype=None):
        import torch
        dtype = dtype or torch.float64
        out = []
        for k, red in zip(nnz, summed):
            shape = (k,) if red else (k, self.n)
            if ndir is not None:
                shape = (ndir,) + shape
            out.append(torch.empty(shape, dtype=dtype, device="cuda"))
        return out

    def _call(self, name, *args):
        check(getattr(load(), name)(self.tape.id, self.n, self.n, ct.byref(self._spec), *args))

    def __call__(self, args, stream=None):
        return self.eval(args, stream=stream)

    def eval(self, args, res=None, stream=None):
        res = self._res(self.tape.nnz_out, self.reduce_out) if res is None else res
        sc = self.scratch(0)
        self._call("casadi_gb300_mapsum_eval", _ptr_array(args), _ptr_array(res),
                   ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream))
        return res

    def forward(self, args, fseeds, res=None, fsens=None, stream=None):
        nfwd = next(s.shape[0] for s in fseeds if s is not None)
        res = self._res(self.tape.nnz_out, self.reduce_out) if res is None else res
        fsens = self._res(self.tape.nnz_out, self.reduce_out, nfwd) if fsens is None else fsens
        sc = self.scratch(nfwd)
        self._call("casadi_gb300_mapsum_forward", nfwd, _ptr_array(args), _ptr_array(res),
                   _ptr_array(fseeds), _ptr_array(fsens), ct.c_void_p(sc.data_ptr()),
                   sc.numel(), _stream_handle(stream))
        return res, fsens

    def reverse(self, args, aseeds, res=None, asens=None, stream=None):
        nadj = next(s.shape[0] for s in aseeds if s is not None)
        res = self._res(self.tape.nnz_out, self.reduce_out) if res is None else res
        asens = self._res(self.tape.nnz_in, self.reduce_in, nadj) if asens is None else asens
        sc = self.scratch(nadj)
        self._call("casadi_gb300_mapsum_reverse", nadj, _ptr_array(args), _ptr_array(res),
                   _ptr_array(aseeds), _ptr_array(asens), ct.c_void_p(sc.data_ptr()),
                   sc.numel(), _stream_handle(stream))
        return res, asens

    def sp_forward(self, args, stream=None):
        import torch
        res = self._res(self.tape.nnz_out, self.reduce_out, dtype=torch.int64)
        sc = self.scratch(0)
        self._call("casadi_gb300_mapsum_sp_forward", _ptr_array(args), _ptr_array(res),
                   ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream))
        return res

    def sp_reverse(self, args, res, stream=None):
        """In place, like MapSum::sp_reverse: args |= propagated bits, res seeds cleared."""
        sc = self.scratch(0)
        self._call("casadi_gb300_mapsum_sp_reverse", _ptr_array(args), _ptr_array(res),
                   ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream))
        return args, res


class CudaMapaccum:
    """``f.mapaccum(N, n_accum)`` (casadi/core/function.cpp:668-747) over n instances on
    device tensors: N chained calls of one tape, the first ``n_accum`` outputs of each call
    feeding the first ``n_accum`` inputs of the next. Accumulator inputs are (nnz, n); other
    inputs and every output stack the N calls: (nnz*N, n), call k's block at rows
    [k*nnz, (k+1)*nnz). Seeds and sensitivities add a leading direction axis."""

    class_name = "Mapaccum"

    def __init__(self, f, N, n_accum=1):
        self.tape = f if isinstance(f, CudaTape) else CudaTape(f)
        self.N, self.n_accum = int(N), int(n_accum)
        self._scratch = None
        self.name = "mapaccum_%s" % getattr(f, "name", "f")

    def _in_rows(self, j):
        k = self.tape.nnz_in[j]
        return k if j < self.n_accum else k * self.N

    def scratch(self, n, ndir=0, record_all=False):
        import torch
        b = ct.c_size_t()
        size = (load().casadi_gb300_mapaccum_reverse_scratch_size if record_all
                else load().casadi_gb300_mapaccum_scratch_size)
        check(size(self.tape.id, self.N, self.n_accum, n,
                                                        ndir, ct.byref(b)))
        if self._scratch is None or self._scratch.numel() < b.value:
            self._scratch = torch.empty(max(b.value, 8), dtype=torch.uint8, device="cuda")
        return self._scratch

    def _outs(self, n, ndir=None, keep=None):
        import torch
        out = []
        for j, k in enumerate(self.tape.nnz_out):
            if keep is not None and not keep[j]:
                out.append(None)
                continue
            shape = (k * self.N, n) if ndir is None else (ndir, k * self.N, n)
            out.append(torch.empty(shape, dtype=torch.float64, device="cuda"))
        return out

    def eval(self, args, n=None, keep=None, stream=None):
        """``keep``: per output, whether to return it (accumulators not kept live in scratch)."""
        n = CudaTape._n(args) if n is None else n
        res = self._outs(n, keep=keep)
        sc = self.scratch(n)
        check(load().casadi_gb300_mapaccum_eval(
            self.tape.id, self.N, self.n_accum, n, n, _ptr_array(args), _ptr_array(res),
            ct.c_void_p(sc.data_ptr()), sc.numel(), _stream_handle(stream)))
        return res

    def forward(self, args, fseeds, n=None, stream=None):
        n = CudaTape._n(args) if n is None else n
        nfwd = next(s.shape[0] for s in fseeds if s is not None)
        res, fsens = self._outs(n), self._outs(n, nfwd)
        sc = self.scratch(n, nfwd)
        check(load().casadi_gb300_mapaccum_forward(
            self.tape.id, self.N, self.n_accum, n, n, nfwd, _ptr_array(args), _ptr_array(res),
            _ptr_array(fseeds), _ptr_array(fsens), ct.c_void_p(sc.data_ptr()), sc.numel(),
            _stream_handle(stream)))
        return res, fsens

    def reverse(self, args, aseeds, n=None, keep=None, stream=None, record_all=False):
        import torch
        n = CudaTape._n(args) if n is None else n
        nadj = next(s.shape[0] for s in aseeds if s is not None)
        res = self._outs(n, keep=keep)
        asens = [torch.empty((nadj, self._in_rows(j), n), dtype=torch.float64, device="cuda")
                 for j in range(len(self.tape.nnz_in))]
        sc = self.scratch(n, nadj, record_all)
        check(load().casadi_gb300_mapaccum_reverse(
            self.tape.id, self.N, self.n_accum, n, n, nadj, _ptr_array(args), _ptr_array(res),
            _ptr_array(aseeds), _ptr_array(asens), ct.c_void_p(sc.data_ptr()), sc.numel(),
            _stream_handle(stream)))
        return res, asens


class MapMemory:
    """A checked-out memory object (stream + staging buffers) for the host-buffer path."""

    def __init__(self):
        self.id = check(load().casadi_gb300_checkout())

    def __del__(self):
        try:
            if _lib is not None:
                _lib.casadi_gb300_release(self.id)
        except Exception:
            pass


def _host_ptrs(arrays):
    arr = (ct.c_void_p * max(1, len(arrays)))()
    for k, a in enumerate(arrays):
        arr[k] = None if a is None else a.ctypes.data
    return arr


class CudaMap:
    """``f.map(n, "cuda")``: evaluate an SX function over n instances with host buffers in
    CasADi's Map layout (instance-major: input j of instance i at ``arg[j][i, :]``), like
    ``Map::eval`` (casadi/core/map.cpp:141-157, :327-386)."""

    parallelization = "cuda"
    class_name = "CudaMap"

    def __init__(self, f, n):
        self.f = f
        self.n = int(n)
        self.tape = f if isinstance(f, CudaTape) else CudaTape(f)
        self.mem = MapMemory()
        self.name = "cudamap%d_%s" % (self.n, getattr(f, "name", "f"))

    def _host_out(self, nnz, ndir=1):
        return [np.empty((self.n, ndir * k) if ndir > 1 else (self.n, k)) for k in nnz]

    def __call__(self, *args, res=None):
        """args: arrays of shape (n, nnz_in[j]) (C-contiguous float64) or None."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in args]
        res = self._host_out(self.tape.nnz_out) if res is None else res
        check(load().casadi_gb300_map_eval(self.tape.id, self.mem.id, self.n, _host_ptrs(args),
                                           _host_ptrs(res)))
        return res

    def sp_forward(self, args, res=None):
        """bvec_t forward sweep with instance-major uint64 host buffers ((n, nnz_in[j]) per
        input); returns the output words (n, nnz_out[j]) (Map::sp_forward)."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.uint64) for a in args]
        res = [np.zeros((self.n, k), np.uint64) for k in self.tape.nnz_out] if res is None else res
        check(load().casadi_gb300_map_sp_forward(self.tape.id, self.mem.id, self.n,
                                                 _host_ptrs(args), _host_ptrs(res)))
        return res

    def sp_reverse(self, args, res):
        """bvec_t reverse sweep in place (Map::sp_reverse): args[j] |= propagated bits,
        res[j] (the seeds) cleared; uint64 arrays of shape (n, nnz)."""
        check(load().casadi_gb300_map_sp_reverse(self.tape.id, self.mem.id, self.n,
                                                 _host_ptrs(args), _host_ptrs(res)))
        return args, res

    def jacobian(self, *args, res=None, jac=None):
        """Jacobian with instance-major host buffers: jac[j] has shape
        (n, nnz_in_total, nnz_out[j])."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in args]
        nz = sum(self.tape.nnz_in)
        res = self._host_out(self.tape.nnz_out) if res is None else res
        jac = [np.empty((self.n, nz, k)) for k in self.tape.nnz_out] if jac is None else jac
        check(load().casadi_gb300_map_jacobian(self.tape.id, self.mem.id, self.n,
                                               _host_ptrs(args), _host_ptrs(res), _host_ptrs(jac)))
        return res, jac

    def jacobian_reverse(self, args, aseeds, res=None, jac=None, asens=None):
        """Host-buffer Jacobian (as :meth:`jacobian`) and adjoint (as :meth:`reverse`) from
        one record sweep."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in args]
        aseeds = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in aseeds]
        nadj = next(a.shape[1] for a in aseeds if a is not None)
        nz = sum(self.tape.nnz_in)
        res = self._host_out(self.tape.nnz_out) if res is None else res
        jac = [np.empty((self.n, nz, k)) for k in self.tape.nnz_out] if jac is None else jac
        asens = [np.empty((self.n, nadj, k)) for k in self.tape.nnz_in] if asens is None else asens
        check(load().casadi_gb300_map_jacobian_reverse(
            self.tape.id, self.mem.id, self.n, _host_ptrs(args), _host_ptrs(res),
            _host_ptrs(jac), nadj, _host_ptrs(aseeds), _host_ptrs(asens)))
        return res, jac, asens

    def forward(self, args, fseeds, res=None, fsens=None, outer=False):
        """Forward sweep with host buffers. Inner order (the mapped f.forward(nfwd)'s):
        fseeds[j] of shape (n, nfwd, nnz_in[j]), fsens[j] (n, nfwd, nnz_out[j]). outer=True:
        the Map's own derivative order (Map::get_forward), fseeds[j] of shape
        (nfwd, n, nnz_in[j]), fsens[j] (nfwd, n, nnz_out[j]). Returns (res, fsens)."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in args]
        fseeds = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in fseeds]
        nfwd = next(a.shape[0 if outer else 1] for a in fseeds if a is not None)
        res = self._host_out(self.tape.nnz_out) if res is None else res
        if fsens is None:
            fsens = [np.empty((nfwd, self.n, k) if outer else (self.n, nfwd, k))
                     for k in self.tape.nnz_out]
        fn = load().casadi_gb300_map_forward_outer if outer else load().casadi_gb300_map_forward
        check(fn(self.tape.id, self.mem.id, self.n, nfwd, _host_ptrs(args), _host_ptrs(res),
                 _host_ptrs(fseeds), _host_ptrs(fsens)))
        return res, fsens

    def reverse(self, args, aseeds, res=None, asens=None, outer=False):
        """Adjoint sweep with host buffers. Inner order: aseeds[j] of shape
        (n, nadj, nnz_out[j]), asens[j] (n, nadj, nnz_in[j]); outer=True: the Map's own
        derivative order (Map::get_reverse), aseeds[j] (nadj, n, nnz_out[j]), asens[j]
        (nadj, n, nnz_in[j]). Returns (res, asens)."""
        args = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in args]
        aseeds = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in aseeds]
        nadj = next(a.shape[0 if outer else 1] for a in aseeds if a is not None)
        res = self._host_out(self.tape.nnz_out) if res is None else res
        if asens is None:
            asens = [np.empty((nadj, self.n, k) if outer else (self.n, nadj, k))
                     for k in self.tape.nnz_in]
        fn = load().casadi_gb300_map_reverse_outer if outer else load().casadi_gb300_map_reverse
        check(fn(self.tape.id, self.mem.id, self.n, nadj, _host_ptrs(args), _host_ptrs(res),
                 _host_ptrs(aseeds), _host_ptrs(asens)))
        return res, asens


class Batch:
    """Several tapes over their own instance ranges, evaluated in ONE persistent launch.

    ``add(tape, args, aseeds=None)`` queues a value sweep (no seeds) or a value + adjoint
    sweep of ``tape`` (a :class:`CudaTape`) on device tensors; it returns ``(res, asens)``
    tensors that ``run()`` fills. ``run(graph=True)`` replays a captured CUDA graph after the
    first call. The tensors passed to or returned by ``add`` are held by the batch so the
    pointers the launch uses stay valid."""

    def __init__(self):
        self.id = check(load().casadi_gb300_batch_create())
        self._keep = []
        self._scratch = None

    def __del__(self):
        try:
            if getattr(self, "id", None) is not None and _lib is not None:
                _lib.casadi_gb300_batch_free(self.id)
        except Exception:
            pass

    def add(self, tape, args, aseeds=None, n=None, res=None, asens=None):
        n = CudaTape._n(args) if n is None else n
        nadj = 0
        if aseeds is not None:
            nadj = next(s.shape[0] for s in aseeds if s is not None)
        res = tape._outs(tape.nnz_out, n) if res is None else res
        if nadj:
            asens = tape._outs(tape.nnz_in, n, nadj) if asens is None else asens
        else:
            aseeds, asens = [], []
        check(load().casadi_gb300_batch_add(self.id, tape.id, n, n, nadj, _ptr_array(args),
                                            _ptr_array(res), _ptr_array(aseeds),
                                            _ptr_array(asens)))
        self._keep.append((tape, list(args), res, list(aseeds), asens))
        return res, asens

    def add_jacobian_colored(self, tape, args, n_colors, color, outputs=None, n=None):
        """Queue colour-compressed forward directions (``color``: int32 array, one colour per
        flat input nonzero, -1 = unseeded). Returns the compressed blocks, one
        (n_colors, nnz_out, n) tensor per output in ``outputs`` (default: all), None for the
        others."""
        import torch
        n = CudaTape._n(args) if n is None else n
        color = np.ascontiguousarray(color, dtype=np.int32)
        comp = [torch.empty((n_colors, k, n), dtype=torch.float64, device="cuda")
                if outputs is None or j in outputs else None
                for j, k in enumerate(tape.nnz_out)]
        res = [None] * len(tape.nnz_out)
        check(load().casadi_gb300_batch_add_jacobian_colored(
            self.id, tape.id, n, n, n_colors, color.ctypes.data, _ptr_array(args),
            _ptr_array(res), _ptr_array(comp)))
        self._keep.append((tape, list(args), comp, color))
        return comp

    def scratch_bytes(self):
        b = ct.c_size_t()
        check(load().casadi_gb300_batch_scratch_size(self.id, ct.byref(b)))
        return b.value

    def set_residence(self, mode):
        """Work vectors: 0 tuned (default), 1 global memory, 2 shared memory."""
        check(load().casadi_gb300_batch_set_residence(self.id, mode))

    def status(self):
        """Wait for the last run and raise if a unit of it failed on the device."""
        check(load().casadi_gb300_batch_status(self.id))

    def run(self, graph=False, stream=None):
        import torch
        need = self.scratch_bytes()
        if self._scratch is None or self._scratch.numel() < need:
            self._scratch = torch.empty(max(need, 8), dtype=torch.uint8, device="cuda")
        check(load().casadi_gb300_batch_run(self.id, ct.c_void_p(self._scratch.data_ptr()),
                                            self._scratch.numel(), 1 if graph else 0,
                                            _stream_handle(stream)))


N_TAN_VARIANTS = 8  # tangent-sweep kernel variants (forward, Jacobian); the last one is the
#                     cooperative level sweep, used only by launches of few tiles
N_ADJ_VARIANTS = 7  # adjoint-sweep kernel variants; the last one is the cooperative level
#                     sweep, used only by launches of few tiles
TAN_WINDOWED = 8    # the windowed tangent sweep (a tile's directions on one SM, partials and
#                     entries staged in shared memory window by window; >= 4 directions)

FAMILIES = ("eval", "record", "tangent", "adjoint", "sp_forward", "sp_reverse", "batch",
            "activity")


def fp64_rate(kind="dfma", reps=5):
    """Measured FP64 pipe rate of the current device (thread-level instructions per second)
    for independent chains of DFMA, DADD, DMUL, or a product / sum issued as a DFMA
    (casadi_gb300_fp64_rate)."""
    k = {"dfma": 0, "dadd": 1, "dmul": 2, "dmul_as_dfma": 3, "dadd_as_dfma": 4}[kind]
    out = ct.c_double()
    check(load().casadi_gb300_fp64_rate(k, reps, ct.byref(out)))
    return out.value


def profile(enable=True):
    """Turn per-launch CUDA-event timing of the sweep kernels on or off."""
    check(load().casadi_gb300_profile(1 if enable else 0))


def profile_collect():
    """{family: (device ms summed, launches)} since the last collect."""
    ms = (ct.c_double * len(FAMILIES))()
    nl = (ct.c_int * len(FAMILIES))()
    check(load().casadi_gb300_profile_collect(ms, nl, len(FAMILIES)))
    return {f: (ms[k], nl[k]) for k, f in enumerate(FAMILIES)}


def autotune(enable=True):
    """Turn the derivative-sweep autotuner on or off (process-wide)."""
    check(load().casadi_gb300_autotune(1 if enable else 0))


def version():
    return load().casadi_gb300_version().decode()
