"""GB300-native evaluator for CasADi SX virtual-machine tapes.

* :mod:`casadi_gb300.sx`        scalar expression graph -> SXFunction tapes (CasADi's rules)
* :mod:`casadi_gb300.calculus`  operation ids and scalar semantics used for constant folding
* :mod:`casadi_gb300.runtime`   ctypes bindings over the C ABI (include/casadi_gb300.h),
                                :class:`CudaTape` sweeps on device tensors, :class:`CudaMap`
* :mod:`casadi_gb300.autograd`  torch.autograd.Function over the value/adjoint sweeps
* :mod:`casadi_gb300.workloads` synthetic tapes and seeded inputs
"""
__version__ = "0.1.0"
