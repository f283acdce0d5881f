"""GB300-native evaluator for CasADi SX virtual-machine tapes.

* :mod:`casadi_gb300.sx`         scalar expression graph -> SXFunction tapes (CasADi's rules)
* :mod:`casadi_gb300.calculus`   operation ids and scalar semantics used for constant folding
* :mod:`casadi_gb300.runtime`    ctypes bindings over the C ABI (include/casadi_gb300.h):
                                 :class:`CudaTape` sweeps on device tensors, :class:`CudaMap`,
                                 :class:`CudaMapSum`, :class:`CudaMapaccum`, :class:`Batch`
* :mod:`casadi_gb300.sparse_ad`  colour-compressed Jacobians, Hessians and the NLP KKT function
* :mod:`casadi_gb300.autograd`   torch.autograd.Function over the value/adjoint sweeps
* :mod:`casadi_gb300.workloads`  synthetic tapes and seeded inputs

:func:`map` and :func:`mapaccum` follow ``Function::map`` / ``Function::mapaccum``
(casadi/core/function.cpp:668-895) for the ``"cuda"`` parallelization; :func:`load` and
:func:`deserialize` follow ``Function::load`` / ``Function::deserialize`` (function.cpp:
1541-1560) for SXFunctions, giving their tapes on the GPU.
"""
__version__ = "0.1.0"


def map(f, n, parallelization="cuda", reduce_in=None, reduce_out=None):
    """``f.map(n, "cuda")`` (casadi/core/function.cpp:861-895): a :class:`runtime.CudaMap`
    (CasADi's instance-major host layout), or, with ``reduce_in``/``reduce_out`` flags, a
    :class:`runtime.CudaMapSum` (function.cpp:787-827; device tensors). ``n == 1`` without
    reductions returns ``f`` itself, as the reference does."""
    from . import runtime as R
    if parallelization != "cuda":
        raise ValueError("only the 'cuda' parallelization is provided here")
    if reduce_in is not None or reduce_out is not None:
        return R.CudaMapSum(f, n, reduce_in, reduce_out)
    if n == 1:
        return f
    return R.CudaMap(f, n)


def mapaccum(f, N, n_accum=1):
    """``f.mapaccum(N, n_accum)`` (casadi/core/function.cpp:668-747): N chained calls, the
    first ``n_accum`` outputs feeding the first ``n_accum`` inputs (:class:`runtime.CudaMapaccum`)."""
    from . import runtime as R
    return R.CudaMapaccum(f, N, n_accum)


def load(path):
    """``Function.load(path)`` (casadi/core/function.cpp:1541-1549) for a file that
    ``Function::save`` wrote holding one SXFunction: its tape as a :class:`runtime.CudaTape`
    (called SXFunctions inlined). Files holding several Functions: :func:`runtime.push_file`."""
    from . import runtime as R
    with open(path, "rb") as fh:
        return R.CudaTape.deserialize(fh.read())


def deserialize(text):
    """``Function.deserialize(text)`` (function.cpp:1556-1560): the tape of the SXFunction
    that ``Function::serialize()`` returned the text of, as a :class:`runtime.CudaTape`."""
    from . import runtime as R
    return R.CudaTape.deserialize(text.encode() if isinstance(text, str) else bytes(text))
