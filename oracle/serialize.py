"""Writer of CasADi's serialization of SXFunctions -- test infrastructure.

Produces, from this package's SX builder, the text the reference writes for an SXFunction, so
the library's decoder can be checked on SX bodies (the reference's own tests hold no
serialized SXFunction; the one serialized Function they hold is an MXFunction, which pins the
common layers: tests/golden/serialized_issue3074.txt). Nothing in the product imports this.

Restated from the reference's writer side:
  SerializingStream header, primitives, debug tags and descriptors, shared objects
      casadi/core/serializing_stream.cpp:76-118, :157-330; serializing_stream.hpp:263-333
  Function::serialize (null flag) function.cpp:1482-1489; saved form (type byte 5, shared
      Function) serializer.cpp:255-270 (SERIALIZE macro), function.cpp:1541-1549
  ProtoFunction::serialize_body v2, FunctionInternal::serialize_body v8
      function_internal.cpp:4165-4267
  XFunction::serialize_body / delayed members x_function.hpp:322-334
  SXFunction::serialize_body v3 sx_function.cpp:1999-2041
  SX nodes: SXNode::serialize sx_node.cpp:238-241 and the serialize_node methods of
      SymbolicSX, the ConstantSX kinds, UnarySX, BinarySX, CallSX, OutputSX
  Sparsity::serialize (compressed, dense shorthand) sparsity.cpp:1321-1327, :2079-2085
"""
import math
import struct

import numpy as np

from casadi_gb300 import calculus as C

CHECK = 123456789012345
PROTOCOL = 3
SERIALIZED_FUNCTION = 5


class CallNode:
    """A call of a Function inside an expression (CallSX): op OP_CALL, the callee, its
    argument nodes."""

    def __init__(self, fn, deps):
        self.fn, self.deps = fn, list(deps)


class OutputNode:
    """Output `oind` of a CallNode (OutputSX, op -1)."""

    def __init__(self, call, oind):
        self.call, self.oind = call, oind


class Writer:
    def __init__(self, debug=False):
        self.out = bytearray()
        self.debug = False
        self.shared = {}
        self._keep = []  # nodes keyed by id() stay alive while written
        self._raw(struct.pack("<q", CHECK))
        self._raw(struct.pack("<q", PROTOCOL))
        self._raw(bytes([1 if debug else 0]))
        self.debug = debug

    # -- primitives ------------------------------------------------------------------------
    def _raw(self, b):
        self.out += b

    def deco(self, c):
        if self.debug:
            self.out.append(ord(c))

    def descr(self, d):
        if self.debug and d is not None:
            self._str(d)

    def _str(self, s):
        b = s.encode()
        self.deco("s")
        self.deco("i")
        self._raw(struct.pack("<i", len(b)))
        self._raw(b)

    def i64(self, v, d=None):
        self.descr(d)
        self.deco("J")
        self._raw(struct.pack("<q", v))

    def size(self, v, d=None):
        self.descr(d)
        self.deco("K")
        self._raw(struct.pack("<Q", v))

    def i32(self, v, d=None):
        self.descr(d)
        self.deco("i")
        self._raw(struct.pack("<i", v))

    def boolean(self, v, d=None):
        self.descr(d)
        self.deco("b")
        self._raw(bytes([1 if v else 0]))

    def dbl(self, v, d=None):
        self.descr(d)
        self.deco("d")
        self._raw(struct.pack("<d", v))

    def ch(self, c, d=None):
        self.descr(d)
        self._raw(c.encode() if isinstance(c, str) else bytes([c]))

    def string(self, s, d=None):
        self.descr(d)
        self._str(s)

    def vector(self, items, put, d=None):
        self.descr(d)
        self.deco("V")
        self.i64(len(items))
        for x in items:
            put(x)

    def dict(self, dct, d=None):
        self.descr(d)
        self.deco("D")
        self.i64(len(dct))
        for k, v in dct.items():
            self.string(k)
            self.generic(v)

    def version(self, name, v):
        self.i32(v, name + "::serialization::version")

    # -- shared objects --------------------------------------------------------------------
    def _shared(self, key, body):
        if key in self.shared:
            self.ch("r", "Shared::flag")
            self.i64(self.shared[key], "Shared::reference")
            return
        self.ch("d", "Shared::flag")
        body()
        self.shared[key] = len(self.shared)

    def sparsity(self, shape, d=None):
        """A dense nrow x ncol pattern (the only kind SX builder inputs/outputs have)."""
        self.descr(d)
        self.deco("S")
        nrow, ncol = shape
        self._shared(("S", nrow, ncol), lambda: self.vector(
            [nrow, ncol, 1], self.i64, "SparsityInternal::compressed"))

    def generic(self, v, d=None):
        self.descr(d)
        self.deco("G")
        self._keep.append(v)

        def body():
            if isinstance(v, bool):
                self.i32(1, "GenericType::type")
                self.boolean(v, "GenericType::d")
            elif isinstance(v, int):
                self.i32(2, "GenericType::type")
                self.i64(v, "GenericType::d")
            elif isinstance(v, float):
                self.i32(3, "GenericType::type")
                self.dbl(v, "GenericType::d")
            elif isinstance(v, str):
                self.i32(4, "GenericType::type")
                self.string(v, "GenericType::d")
            elif isinstance(v, dict):
                self.i32(11, "GenericType::type")
                self.dict(v, "GenericType::d")
            else:
                raise TypeError(type(v))
        # every GenericType value is its own shared object (GenericType(d) makes a new one)
        self._shared(("G", len(self._keep)), body)

    def _const(self, val):
        if math.isnan(val):
            self.ch("n", "ConstantSX::type")
        elif val == math.inf:
            self.ch("F", "ConstantSX::type")
        elif val == -math.inf:
            self.ch("f", "ConstantSX::type")
        elif val == 0 and math.copysign(1.0, val) > 0:
            self.ch("0", "ConstantSX::type")
        elif val == 1:
            self.ch("1", "ConstantSX::type")
        elif val == -1:
            self.ch("m", "ConstantSX::type")
        elif val == int(val) and abs(val) < 2 ** 31:
            self.ch("i", "ConstantSX::type")
            self.i32(int(val), "ConstantSX::value")
        else:
            self.ch("r", "ConstantSX::type")
            self.dbl(val, "ConstantSX::value")

    def sx(self, root, d=None):
        """One SX node (SXElem), pre-order with an explicit stack: flag, op, then the
        dependencies; the node's shared index is taken once they are written."""
        st = [[root, d, 0]]
        while st:
            fr = st[-1]
            node, dd, stage = fr
            key = ("E", id(node))
            if stage == 0:
                self.descr(dd)
                self.deco("E")
                if key in self.shared:
                    self.ch("r", "Shared::flag")
                    self.i64(self.shared[key], "Shared::reference")
                    st.pop()
                    continue
                self._keep.append(node)
                self.ch("d", "Shared::flag")
                if isinstance(node, CallNode):
                    self.i64(C.OP_CALL, "SXNode::op")
                    self.function(node.fn, "CallSX::f")
                    self.descr("CallSX::dep")
                    self.deco("V")
                    self.i64(len(node.deps))
                    fr[2] = 1
                    for dep in reversed(node.deps):
                        st.append([dep, None, 0])
                    continue
                if isinstance(node, OutputNode):
                    self.i64(-1, "SXNode::op")
                    fr[2] = 1
                    st.append([node.call, "OutputSX::dep", 0])
                    continue
                self.i64(node.op, "SXNode::op")
                kind = node._kind
                if kind == "s":
                    self.string(node.name, "SymbolicSX::name")
                elif kind == "c":
                    self._const(float(node.val))
                elif kind == "u":
                    fr[2] = 1
                    st.append([node.dep0, "UnarySX::dep", 0])
                    continue
                elif kind == "b":
                    fr[2] = 2
                    st.append([node.dep0, "UnarySX::dep0", 0])
                    continue
                self.shared[key] = len(self.shared)
                st.pop()
            elif stage == 2:
                fr[2] = 1
                st.append([node.dep1, "UnarySX::dep1", 0])
            else:
                if isinstance(node, OutputNode):
                    self.i32(node.oind, "OutputSX::oind")
                self.shared[key] = len(self.shared)
                st.pop()

    def sx_matrix(self, nz):
        self.sparsity((len(nz), 1), "Matrix::sparsity")
        self.vector(nz, self.sx, "Matrix::nonzeros")

    # -- Functions -------------------------------------------------------------------------
    def function(self, f, d=None):
        self.descr(d)
        self.deco("F")
        self._keep.append(f)
        self._shared(("F", id(f) if f is not None else None), lambda: self.function_body(f))

    def function_body(self, f):
        self.boolean(f is None, "Function::null")
        if f is None:
            return
        self.string("SXFunction", "FunctionInternal::base_function")
        self.version("ProtoFunction", 2)
        self.string(f.name, "ProtoFunction::name")
        for k in ("verbose", "print_time", "record_time", "regularity_check"):
            self.boolean(False, "ProtoFunction::" + k)
        self.boolean(True, "ProtoFunction::error_on_fail")
        nin, nout = list(f.tape.nnz_in), list(f.tape.nnz_out)
        fi = "FunctionInternal::"
        self.version("FunctionInternal", 8)
        self.vector([True] * len(nin), self.boolean, fi + "is_diff_in")
        self.vector([True] * len(nout), self.boolean, fi + "is_diff_out")
        self.vector([(k, 1) for k in nin], self.sparsity, fi + "sp_in")
        self.vector([(k, 1) for k in nout], self.sparsity, fi + "sp_out")
        self.vector(f.name_in, self.string, fi + "name_in")
        self.vector(f.name_out, self.string, fi + "name_out")
        self.boolean(False, fi + "jit")
        self.boolean(True, fi + "jit_cleanup")
        self.string("source", fi + "jit_serialize")
        self.boolean(True, fi + "jit_temp_suffix")
        self.string("jit_tmp", fi + "jit_base_name")
        self.dict(f.jit_options, fi + "jit_options")
        self.string("clang", fi + "compiler_plugin")
        self.boolean(False, fi + "has_refcount")
        self.dict({}, fi + "cache_init")
        self.function(None, fi + "derivative_of")
        self.dbl(2.0, fi + "jac_penalty")
        for k in ("forward", "reverse", "jacobian", "fd", "forward_op", "reverse_op",
                  "jacobian_op", "fd_op"):
            self.boolean(True, fi + "enable_" + k)
        self.dbl(-1.0, fi + "ad_weight")
        self.dbl(-1.0, fi + "ad_weight_sp")
        self.boolean(False, fi + "always_inline")
        self.boolean(False, fi + "never_inline")
        self.i64(64, fi + "max_num_dir")
        self.boolean(True, fi + "inputs_check")
        self.dbl(1e-8, fi + "fd_step")
        self.string("", fi + "fd_method")
        self.boolean(False, fi + "print_in")
        self.boolean(False, fi + "print_out")
        self.boolean(False, fi + "print_canonical")
        self.i64(10000, fi + "max_io")
        self.boolean(False, fi + "dump_in")
        self.boolean(False, fi + "dump_out")
        self.string(".", fi + "dump_dir")
        self.string("mtx", fi + "dump_format")
        for k in ("forward_options", "reverse_options", "jacobian_options", "der_options"):
            self.dict({}, fi + k)
        self.function(None, fi + "custom_jacobian")
        self.vector([], self.function, fi + "registered_functions")
        for k, v in zip(("arg_per", "res_per", "iw_per", "w_per", "arg_tmp", "res_tmp",
                         "iw_tmp", "w_tmp"),
                        (len(nin), len(nout), 0, f.tape.sz_w, 0, 0, 0, 0)):
            self.size(v, fi + "sz_" + k)
        # XFunction: the symbolic inputs
        self.version("XFunction", 1)
        self.vector(f.inputs, self.sx_matrix, "XFunction::in")
        # SXFunction
        t = f.tape
        sf = "SXFunction::"
        self.version("SXFunction", 3)
        self.size(t.n_instr, sf + "n_instr")
        self.size(t.sz_w, sf + "worksize")
        self.vector(f.free_vars, self.sx, sf + "free_vars")
        self.vector(f.operations, self.sx, sf + "operations")
        self.vector(f.constants, self.sx, sf + "constants")
        self.vector([0.0] * len(nin), self.dbl, sf + "default_in")
        szs = f.call_sizes()
        for k, v in zip(("call_sz_arg", "call_sz_res", "call_sz_iw", "call_sz_w",
                         "call_sz_arg", "call_sz_res"), szs):
            self.size(v, sf + k)
        self.size(len(f.calls), sf + "call_el_size")
        for callee, dep, res in f.calls:
            self.function(callee, sf + "call_el_f")
            self.vector(list(dep), self.i32, sf + "call_el_dep")
            self.vector(list(res), self.i32, sf + "call_el_res")
            self.vector([], self.i32, sf + "call_el_copy_elision_arg")
            self.vector([], self.i32, sf + "call_el_copy_elision_offset")
        self.vector([False] * t.n_instr, self.boolean, sf + "copy_elision")
        u = t.atomic_array()["u"]
        for k in range(t.n_instr):
            self.i32(int(t.op[k]), sf + "ScalarAtomic::op")
            self.i32(int(t.i0[k]), sf + "ScalarAtomic::i0")
            bits = int(u[k])
            self.i32(struct.unpack("<i", struct.pack("<I", bits & 0xFFFFFFFF))[0],
                     sf + "ScalarAtomic::i1")
            self.i32(struct.unpack("<i", struct.pack("<I", bits >> 32))[0],
                     sf + "ScalarAtomic::i2")
        self.boolean(True, sf + "live_variables")
        self.boolean(False, sf + "print_instructions")
        self.vector(f.outputs, self.sx_matrix, "XFunction::out")

    def text(self):
        return "".join(chr(97 + (b & 15)) + chr(97 + (b >> 4)) for b in self.out)


class Serializable:
    """What the writer needs of one SXFunction: name, io names, the tape, the expression
    nodes of its inputs/outputs/operations/constants and its call records."""

    def __init__(self, name, tape, inputs, outputs, operations=(), constants=(), calls=(),
                 name_in=None, name_out=None, jit_options=None, free_vars=()):
        self.name, self.tape = name, tape
        self.free_vars = list(free_vars)
        self.inputs, self.outputs = [list(v) for v in inputs], [list(v) for v in outputs]
        self.operations, self.constants = list(operations), list(constants)
        self.calls = list(calls)
        self.name_in = name_in or ["i%d" % j for j in range(len(tape.nnz_in))]
        self.name_out = name_out or ["o%d" % j for j in range(len(tape.nnz_out))]
        self.jit_options = jit_options or {}

    def call_sizes(self):
        if not self.calls:
            return (0, 0, 0, 0, 0, 0)
        fs = [c[0] for c in self.calls]
        return (max(len(f.tape.nnz_in) for f in fs), max(len(f.tape.nnz_out) for f in fs), 0,
                max(f.tape.sz_w for f in fs), max(sum(f.tape.nnz_in) for f in fs),
                max(sum(f.tape.nnz_out) for f in fs))


def from_function(fn, **kw):
    """Serializable of an sx.Function: its expression graph gives the operation and constant
    nodes (every distinct non-symbolic node reachable from the outputs)."""
    ops, consts, seen = [], [], set()
    stack = [e for v in fn.outputs for e in v]
    while stack:
        e = stack.pop()
        if id(e) in seen:
            continue
        seen.add(id(e))
        if e.is_constant():
            consts.append(e)
        elif not e.is_symbolic():
            ops.append(e)
            stack.extend(x for x in (e.dep0, e.dep1) if x is not None)
    return Serializable(fn.name, fn.tape, fn.inputs, fn.outputs, ops, consts, **kw)


def serialize(f, debug=False, saved_form=False):
    """Text of `f` (a Serializable or sx.Function) as Function::serialize() returns it, or,
    with saved_form, as Function::save writes it."""
    if not isinstance(f, Serializable):
        f = from_function(f)
    w = Writer(debug)
    if saved_form:
        w.ch(SERIALIZED_FUNCTION)
        w.function(f)
    else:
        w.function_body(f)
    return w.text()


def serialize_vector(fs, debug=False):
    """Text of a vector of Functions as a FileSerializer writes it (type byte 15, then the
    vector), the other form casadi_c_push_file reads."""
    fs = [f if isinstance(f, Serializable) else from_function(f) for f in fs]
    w = Writer(debug)
    w.ch(15)
    w.vector(fs, w.function)
    return w.text()


def tape_arrays(t):
    """(op, i0, 16-byte payload, nnz_in, nnz_out, sz_w) of a tape, for exact comparisons."""
    return (np.asarray(t.op), np.asarray(t.i0), np.asarray(t.atomic_array()["u"]),
            list(t.nnz_in), list(t.nnz_out), int(t.sz_w))
