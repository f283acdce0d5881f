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
    nonzero (ceil(nrow/64) instances of one sp_reverse launch), ``hierarchical`` refines
    blocks (:func:`jacobian_pattern_hierarchical`). ``auto`` decides as the reference does
    (FunctionInternal::get_jac_sparsity, casadi/core/function_internal.cpp:1928-1975):
    hierarchical when both sides exceed 3 x 64 nonzeros, else forward when 0.49 x its sweeps
    <= 0.51 x the reverse sweeps. All give the same pattern."""
    ncol = tape.nnz_in[wrt]
    nrow = tape.nnz_out[out]
    if mode == "auto":
        if ncol > 192 and nrow > 192:
            mode = "hierarchical"
        else:
            mode = ("forward" if 0.49 * ((ncol + 63) // 64) <= 0.51 * ((nrow + 63) // 64)
                    else "reverse")
    if mode == "hierarchical":
        return jacobian_pattern_hierarchical(tape, out, wrt)
    if mode == "reverse":
        return _jacobian_pattern_reverse(tape, out, wrt)
    if mode != "forward":
        raise ValueError("mode must be 'forward', 'reverse', 'hierarchical' or 'auto'")
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


def _subdivide(part):
    """Each block [part[k], part[k+1]) of a partition cut into at most 64 blocks of
    ceil(size / 64) nonzeros (the last one shorter)."""
    out = [int(part[0])]
    for a, b in zip(part[:-1], part[1:]):
        step = max(1, -(-(int(b) - int(a)) // 64))
        out.extend(range(int(a) + step, int(b), step))
        out.append(int(b))
    return np.asarray(out, dtype=np.int64)


def _pack(widths):
    """First-fit packing of colours (each needing ``widths[c]`` <= 64 bits) into 64-bit words in
    colour order: (word of each colour, bit offset of each colour, number of words)."""
    word = np.zeros(len(widths), np.int64)
    off = np.zeros(len(widths), np.int64)
    cur, pos = 0, 0
    for c, w in enumerate(widths):
        if pos + w > 64:
            cur, pos = cur + 1, 0
        word[c], off[c] = cur, pos
        pos += w
    return word, off, cur + 1


class _BlockLevel:
    """One side's coarse partition refined by :func:`_subdivide`, with the colouring of its
    coarse blocks over a coarse pattern (blocks of one colour reach no common block of the
    other side) and the bit layout of the seeds."""

    def __init__(self, part, pairs_self, pairs_other, n_other_blocks):
        self.part = part
        self.fine = _subdivide(part)
        nb = len(part) - 1
        self.first = np.searchsorted(self.fine, part[:-1])
        self.nfine = np.searchsorted(self.fine, part[1:]) - self.first
        P = K.Pattern.from_triplets(n_other_blocks, nb, pairs_other, pairs_self)
        self.color = K.uni_coloring(P) if nb else np.zeros(0, np.int64)
        ncol = int(self.color.max()) + 1 if nb else 0
        widths = np.zeros(ncol, np.int64)
        np.maximum.at(widths, self.color, self.nfine)
        self.word, self.off, self.n_words = _pack(widths.tolist())
        self.widths = widths

    def seeds(self, n):
        """Seed words (n, n_words): nonzero i of fine block l of coarse block k carries bit
        off[colour(k)] + l of word word[colour(k)]."""
        idx = np.arange(n)
        coarse = np.searchsorted(self.part, idx, side="right") - 1
        fine = np.searchsorted(self.fine, idx, side="right") - 1
        c = self.color[coarse]
        bit = (self.off[c] + fine - self.first[coarse]).astype(np.uint64)
        s = np.zeros((n, self.n_words), np.uint64)
        s[idx, self.word[c]] = np.uint64(1) << bit
        return s


def jacobian_pattern_hierarchical(tape, out, wrt, sweep=None, weight=0.49, stats=None):
    """Sparsity of d output[out] / d input[wrt] (rows: output nonzeros, columns: input
    nonzeros) by the reference's hierarchical refinement
    (FunctionInternal::get_jac_sparsity_hierarchical, casadi/core/function_internal.cpp:
    1613-1911; the reference takes it when both sides exceed 3 x 64 nonzeros, :1944-1950).

    The Jacobian starts as one block. Each level cuts every block of both sides into at most
    64 fine blocks, colours the coarse blocks of the seeded side so that blocks of one colour
    reach no common block of the other side (``coloring.uni_coloring`` over the coarse
    pattern), gives the fine blocks of a coarse block distinct bits within their colour's bit
    range (colours packed first-fit into 64-bit words, all blocks of a colour sharing its
    bits), runs one bvec_t sweep per word, and reads each set bit in a fine block of the other
    side back to the one fine block that set it: the coarse block of that colour whose coarse
    pattern reaches the other side's coarse block. It stops when every block is one nonzero;
    the pattern is exact, equal to one bit per nonzero. Each level seeds the side whose words,
    weighted by ``weight`` (forward) and 1 - ``weight`` (reverse), cost less, as the
    reference's ``ad_weight_sp`` (0.49: forward on ties).

    ``tape``: a :class:`runtime.CudaTape`; its sp_forward / sp_reverse sweeps run all words of a
    level in one launch, one instance per word. ``sweep(forward, seeds)``, if given, replaces
    them: seeds (n_seed_side, words) uint64 -> sensitivities (n_other_side, words) uint64.
    ``stats`` (a dict) receives the levels and the words swept."""
    n_in, n_out = tape.nnz_in[wrt], tape.nnz_out[out]
    if sweep is None:
        sweep = _device_sweeper(tape, out, wrt)
    if stats is not None:
        stats.update(levels=0, words=0)
    if n_in == 0 or n_out == 0:
        return K.Pattern.from_triplets(n_out, n_in, [], [])
    part_in = np.array([0, n_in], np.int64)
    part_out = np.array([0, n_out], np.int64)
    pin = np.zeros(1, np.int64)   # coarse pattern: (input block, output block) pairs
    pout = np.zeros(1, np.int64)
    while True:
        lin = _BlockLevel(part_in, pin, pout, len(part_out) - 1)
        lout = _BlockLevel(part_out, pout, pin, len(part_in) - 1)
        forward = weight * lin.n_words <= (1 - weight) * lout.n_words
        seed_side, sens_side = (lin, lout) if forward else (lout, lin)
        pseed, psens = (pin, pout) if forward else (pout, pin)
        n_seed = n_in if forward else n_out
        sens = np.asarray(sweep(forward, seed_side.seeds(n_seed)), np.uint64)
        # OR over the nonzeros of each fine block of the sensitivity side
        spsens = np.bitwise_or.reduceat(sens, sens_side.fine[:-1], axis=0)
        coarse_of_fine = np.searchsorted(sens_side.part, sens_side.fine[:-1], side="right") - 1
        # owner of every (word, bit): the colour, and its coarse seed block per sensitivity
        # block (unique by the colouring)
        owner = np.full((seed_side.n_words, 64), -1, np.int64)
        for c in range(len(seed_side.widths)):
            owner[seed_side.word[c], seed_side.off[c]:seed_side.off[c] + seed_side.widths[c]] = c
        nsb = len(sens_side.part) - 1
        table = {}
        for a, b in zip(pseed.tolist(), psens.tolist()):
            table[int(seed_side.color[a]) * nsb + b] = a
        got_seed, got_sens = [], []
        for bit in range(64):
            fb, w = np.nonzero((spsens >> np.uint64(bit)) & np.uint64(1))
            if fb.size == 0:
                continue
            c = owner[w, bit]
            keys = c * nsb + coarse_of_fine[fb]
            k = np.array([table.get(int(x), -1) for x in keys], np.int64)
            loc = bit - seed_side.off[np.maximum(c, 0)]
            ok = (c >= 0) & (k >= 0)
            ok[ok] &= loc[ok] < seed_side.nfine[k[ok]]
            got_seed.append(seed_side.first[k[ok]] + loc[ok])
            got_sens.append(fb[ok])
        fs = np.concatenate(got_seed) if got_seed else np.zeros(0, np.int64)
        ft = np.concatenate(got_sens) if got_sens else np.zeros(0, np.int64)
        pin, pout = (fs, ft) if forward else (ft, fs)
        part_in, part_out = lin.fine, lout.fine
        if stats is not None:
            stats["levels"] += 1
            stats["words"] += seed_side.n_words
        if len(part_in) == n_in + 1 and len(part_out) == n_out + 1:
            break
    return K.Pattern.from_triplets(n_out, n_in, pout, pin)


def _device_sweeper(tape, out, wrt):
    """Sparsity sweeps of ``tape`` (a runtime.CudaTape) on the device, one instance per word."""
    import torch

    def sweep(forward, seeds):
        n = seeds.shape[1]
        dev = torch.from_numpy(np.ascontiguousarray(seeds).view(np.int64)).cuda()
        if forward:
            args = [None] * len(tape.nnz_in)
            args[wrt] = dev
            return tape.sp_forward(args, n=n)[out].cpu().numpy().view(np.uint64)
        args = [torch.zeros((k, n), dtype=torch.int64, device="cuda") for k in tape.nnz_in]
        res = [None] * len(tape.nnz_out)
        res[out] = dev
        tape.sp_reverse(args, res, n=n)
        return args[wrt].cpu().numpy().view(np.uint64)

    return sweep


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
