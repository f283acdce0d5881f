"""Sparse Jacobians and Hessians over many instances by colour-compressed sweeps.

``ColoredJacobian(f, out, wrt)`` computes the nonzeros of d f_out / d x_wrt for every
instance: the Jacobian's sparsity pattern comes from one bvec_t forward sparsity sweep on
the GPU (64 input nonzeros per instance, one instance per 64 columns), its columns are
coloured (``coloring.uni_coloring``: columns of one colour share no row), one forward sweep
per colour runs on the GPU with direction d seeded on the columns of colour d
(``casadi_gb300_jacobian_colored``), and a device gather picks every nonzero out of the
compressed block (``casadi_gb300_gather``).

``ColoredHessian(f, out, wrt)`` computes the lower-triangle nonzeros of the Hessian of the
scalar output ``out`` with respect to input ``wrt``: the gradient is built symbolically
(``sx.gradient``, the reference's ``SXFunction::ad_reverse``), and its Jacobian — symmetric —
is compressed with a star colouring and recovered with the star recovery
(``coloring.hessian_recovery``). This is how the reference forms Hessians of SX functions
(``FunctionInternal::get_partition`` with ``symmetric``, casadi/core/function_internal.cpp:
2068-2160, over the gradient's Jacobian, casadi/core/x_function.hpp:441-840).

Values are device tensors of shape (nnz, n), nonzeros in compressed-column order (the lower
triangle's, for Hessians).
"""
import ctypes as ct

import numpy as np

from . import coloring as K
from . import runtime as R
from . import sx as S


def _bit_seeds(count):
    """One bit per nonzero: nonzero k is bit k % 64 of chunk k // 64, shape (count, chunks)."""
    import torch
    nchunk = max(1, (count + 63) // 64)
    bits = torch.zeros((max(count, 1), nchunk), dtype=torch.int64)
    for k in range(count):
        b = k % 64
        bits[k, k // 64] = (1 << b) if b < 63 else -(1 << 63)
    return bits, nchunk


def jacobian_pattern(tape, out, wrt, mode="auto"):
    """Sparsity of d output[out] / d input[wrt] of a :class:`runtime.CudaTape` as a
    :class:`coloring.Pattern` (rows: output nonzeros, columns: input nonzeros), from
    bvec_t sparsity sweeps on the device: ``forward`` seeds one bit per input nonzero
    (ceil(ncol/64) instances of one sp_forward launch), ``reverse`` one bit per output
    nonzero (ceil(nrow/64) instances of one sp_reverse launch); ``auto`` takes the one with
    fewer instances, as the reference picks the mode with fewer sweeps
    (FunctionInternal::get_jac_sparsity, casadi/core/function_internal.cpp:1928-1975)."""
    ncol = tape.nnz_in[wrt]
    nrow = tape.nnz_out[out]
    if mode == "auto":
        mode = "forward" if (ncol + 63) // 64 <= (nrow + 63) // 64 else "reverse"
    if mode == "reverse":
        return _jacobian_pattern_reverse(tape, out, wrt)
    if mode != "forward":
        raise ValueError("mode must be 'forward', 'reverse' or 'auto'")
    import torch
    nchunk = max(1, (ncol + 63) // 64)
    bits = torch.zeros((max(ncol, 1), nchunk), dtype=torch.int64)
    for k in range(ncol):
        b = k % 64
        bits[k, k // 64] = (1 << b) if b < 63 else -(1 << 63)
    args = [None] * len(tape.nnz_in)
    args[wrt] = bits.cuda()
    res = tape.sp_forward(args, n=nchunk)
    ob = res[out].cpu().numpy().view(np.uint64)  # (nrow, nchunk)
    mask = np.zeros((nrow, ncol), dtype=bool)
    for c in range(nchunk):
        for b in range(min(64, ncol - 64 * c)):
            mask[:, 64 * c + b] = (ob[:, c] >> np.uint64(b)) & np.uint64(1) != 0
    return K.Pattern.from_dense(mask)


def _jacobian_pattern_reverse(tape, out, wrt):
    import torch
    ncol = tape.nnz_in[wrt]
    nrow = tape.nnz_out[out]
    seeds, nchunk = _bit_seeds(nrow)
    args = [torch.zeros((k, nchunk), dtype=torch.int64, device="cuda") for k in tape.nnz_in]
    res = [None] * len(tape.nnz_out)
    res[out] = seeds.cuda()
    tape.sp_reverse(args, res, n=nchunk)
    ib = args[wrt].cpu().numpy().view(np.uint64)  # (ncol, nchunk)
    mask = np.zeros((nrow, ncol), dtype=bool)
    for c in range(nchunk):
        for b in range(min(64, nrow - 64 * c)):
            mask[64 * c + b, :] = (ib[:, c] >> np.uint64(b)) & np.uint64(1) != 0
    return K.Pattern.from_dense(mask)


class _Compressed:
    """Shared machinery: a tape, a colouring of one input's nonzeros and a recovery map."""

    def _setup(self, tape, out, wrt, color, src_row):
        import torch
        self.tape, self.out, self.wrt = tape, out, wrt
        self.color = np.asarray(color, dtype=np.int64)
        self.n_colors = int(self.color.max()) + 1 if self.color.size else 0
        flat = np.full(sum(tape.nnz_in), -1, dtype=np.int32)
        off = int(np.sum(tape.nnz_in[:wrt]))
        flat[off:off + tape.nnz_in[wrt]] = self.color
        self._flat = flat
        self.src_row = torch.from_numpy(np.asarray(src_row, dtype=np.int64)).cuda()

    def compressed(self, args, n=None, stream=None, scratch_limit=None):
        """The compressed block of the output: (n_colors, nnz_out, n)."""
        import torch
        n = R.CudaTape._n(args) if n is None else n
        comp = [None] * len(self.tape.nnz_out)
        comp[self.out] = torch.empty((self.n_colors, self.tape.nnz_out[self.out], n),
                                     dtype=torch.float64, device="cuda")
        res = [None] * len(self.tape.nnz_out)
        sc = self.tape.scratch(n, scratch_limit)
        R.check(R.load().casadi_gb300_jacobian_colored(
            self.tape.id, n, n, self.n_colors, self._flat.ctypes.data, R._ptr_array(args),
            R._ptr_array(res), R._ptr_array(comp), ct.c_void_p(sc.data_ptr()), sc.numel(),
            R._stream_handle(stream)))
        return comp[self.out]

    def gather(self, comp, n, out=None, stream=None):
        """Nonzeros (nnz, n) picked out of a compressed block (n_colors, nnz_out, n)."""
        import torch
        vals = torch.empty((self.src_row.numel(), n), dtype=torch.float64, device="cuda") \
            if out is None else out
        R.check(R.load().casadi_gb300_gather(
            n, n, self.src_row.numel(), ct.c_void_p(self.src_row.data_ptr()),
            ct.c_void_p(comp.data_ptr()), ct.c_void_p(vals.data_ptr()),
            R._stream_handle(stream)))
        return vals

    def __call__(self, args, n=None, stream=None, scratch_limit=None):
        """Nonzeros of every instance: a (nnz, n) float64 device tensor."""
        n = R.CudaTape._n(args) if n is None else n
        return self.gather(self.compressed(args, n, stream, scratch_limit), n, stream=stream)

    def add_to_batch(self, batch, args, n=None):
        """Queue the compressed sweeps as an item of a :class:`runtime.Batch`; returns the
        compressed block that ``batch.run()`` fills (recover with :meth:`gather`)."""
        return batch.add_jacobian_colored(self.tape, args, self.n_colors, self._flat,
                                          outputs=[self.out], n=n)[self.out]


class ColoredJacobian(_Compressed):
    """Sparse Jacobian of output ``out`` with respect to input ``wrt`` of an SX Function."""

    def __init__(self, f, out=0, wrt=0, tape=None):
        tape = tape or R.CudaTape(f)
        self.pattern = jacobian_pattern(tape, out, wrt)
        color = K.uni_coloring(self.pattern)
        self._setup(tape, out, wrt, color, K.jacobian_recovery(self.pattern, color))


class ColoredHessian(_Compressed):
    """Lower triangle of the Hessian of the scalar output ``out`` of an SX Function with
    respect to input ``wrt``."""

    def __init__(self, f, out=0, wrt=0):
        if len(f.outputs[out]) != 1:
            raise ValueError("the Hessian needs a scalar output")
        self.gradient_function = S.Function(f.name + "_grad", f.inputs,
                                            [S.gradient(f, out, wrt)])
        tape = R.CudaTape(self.gradient_function)
        p = jacobian_pattern(tape, 0, wrt)
        mask = p.dense()
        self.pattern = K.Pattern.from_dense(mask | mask.T)
        color = K.star_coloring(self.pattern)
        self.rows, self.cols, idx = K.hessian_recovery(self.pattern, color)
        self._setup(tape, 0, wrt, color, idx)


class KKT:
    """The KKT Function of an NLP, ``Nlpsol::kkt()`` (casadi/core/nlpsol.cpp:936-954):
    ``(x, p, lam_f, lam_g) -> (jac:g:x, hess:gamma:x:x)`` with the Lagrangian
    ``gamma = lam_f*f + lam_g'g``, evaluated over many scenarios by colour-compressed sweeps
    (:class:`ColoredJacobian` of g, :class:`ColoredHessian` of gamma).

    ``x``, ``p`` are lists of SX symbols, ``f`` an SX scalar, ``g`` a list of SX. Values come
    back as device tensors: the Jacobian's nonzeros (nnz_J, n) in compressed-column order of
    :attr:`jac_pattern` (rows: constraints, columns: x), the Hessian's nonzeros (nnz_H, n) in
    compressed-column order of the full symmetric :attr:`hess_pattern` (both triangles; the
    upper one mirrored from the lower on the device)."""

    def __init__(self, x, p, f, g, name="nlp"):
        import torch
        x, p, g = list(x), list(p), list(g)
        lam_f = S.sym("lam_f")
        lam_g = S.sym("lam_g", len(g))
        gamma = lam_f * f
        for li, gi in zip(lam_g, g):
            gamma = gamma + li * gi
        inputs = [x, p, [lam_f], lam_g]
        self.g_function = S.Function(name + "_g", inputs, [g])
        self.gamma_function = S.Function(name + "_gamma", inputs, [[gamma]])
        self.jac = ColoredJacobian(self.g_function, out=0, wrt=0)
        self.hess = ColoredHessian(self.gamma_function, out=0, wrt=0)
        self.jac_pattern = self.jac.pattern
        h = self.hess
        nx = len(x)
        mask = np.zeros((nx, nx), dtype=bool)
        mask[h.rows, h.cols] = True
        mask[h.cols, h.rows] = True
        self.hess_pattern = K.Pattern.from_dense(mask)
        lower = {(int(i), int(j)): k for k, (i, j) in enumerate(zip(h.rows, h.cols))}
        rows, cols = self.hess_pattern.row, self.hess_pattern.col()
        mirror = [lower[(max(int(i), int(j)), min(int(i), int(j)))] for i, j in zip(rows, cols)]
        self._mirror = torch.tensor(mirror, dtype=torch.int64).cuda()

    def _full(self, lower, n, stream=None):
        import torch
        vals = torch.empty((self._mirror.numel(), n), dtype=torch.float64, device="cuda")
        R.check(R.load().casadi_gb300_gather(
            n, n, self._mirror.numel(), ct.c_void_p(self._mirror.data_ptr()),
            ct.c_void_p(lower.data_ptr()), ct.c_void_p(vals.data_ptr()),
            R._stream_handle(stream)))
        return vals

    def __call__(self, args, n=None, stream=None):
        """args: [x, p, lam_f, lam_g] as (nnz, n) device tensors; returns (jac, hess)."""
        n = R.CudaTape._n(args) if n is None else n
        jac = self.jac(args, n, stream=stream)
        hess = self._full(self.hess(args, n, stream=stream), n, stream)
        return jac, hess

    def batched(self, args, n=None):
        """Both coloured sweeps as items of one persistent batch replayed from a CUDA graph;
        returns a function that runs it and returns (jac, hess)."""
        n = R.CudaTape._n(args) if n is None else n
        b = R.Batch()
        cj = self.jac.add_to_batch(b, args, n)
        ch = self.hess.add_to_batch(b, args, n)

        def run(stream=None):
            b.run(graph=True, stream=stream)
            return self.jac.gather(cj, n, stream=stream), self._full(
                self.hess.gather(ch, n, stream=stream), n, stream)

        run.batch = b
        return run
