"""Graph colourings that compress sparse Jacobians and Hessians into few directional
derivatives, and the recovery of their nonzeros (host code, numpy).

Sparsity patterns are compressed-column (CCS) arrays ``(nrow, ncol, colind, row)`` with
sorted rows, as CasADi's ``Sparsity``. The colourings run in the C++
library (``casadi_gb300_uni_coloring`` / ``casadi_gb300_star_coloring``, restating the
reference's ``SparsityInternal::uni_coloring``, ``::star_coloring`` and ``::largest_first``,
casadi/core/sparsity_internal.cpp:2959-3045, :3398-3509, :3511-3545), so they give the
reference's seed matrices; no device is needed.

Recovery: for a column colouring, nonzero (i, j) of J is entry (i, colour(j)) of the
compressed J*D. For a star colouring of a symmetric H, nonzero (i, j) is read from
(i, colour(j)) when no other column of colour(j) has a nonzero in row i, else from
(j, colour(i)) (the star property guarantees one of the two).
"""
import numpy as np


class Pattern:
    """A sparsity pattern in compressed-column storage."""

    def __init__(self, nrow, ncol, colind, row):
        self.nrow, self.ncol = int(nrow), int(ncol)
        self.colind = np.asarray(colind, dtype=np.int64)
        self.row = np.asarray(row, dtype=np.int64)

    @staticmethod
    def from_dense(mask):
        mask = np.asarray(mask, dtype=bool)
        nrow, ncol = mask.shape
        colind = np.zeros(ncol + 1, np.int64)
        rows = []
        for j in range(ncol):
            r = np.flatnonzero(mask[:, j])
            rows.append(r)
            colind[j + 1] = colind[j] + r.size
        row = np.concatenate(rows) if rows else np.zeros(0, np.int64)
        return Pattern(nrow, ncol, colind, row)

    @staticmethod
    def from_triplets(nrow, ncol, rows, cols):
        """Pattern of the (row, col) pairs given (duplicates merged), rows sorted per column."""
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        key = np.unique(cols * max(1, int(nrow)) + rows)
        c, r = np.divmod(key, max(1, int(nrow)))
        colind = np.zeros(int(ncol) + 1, np.int64)
        np.add.at(colind, c + 1, 1)
        return Pattern(nrow, ncol, np.cumsum(colind), r)

    @property
    def nnz(self):
        return int(self.colind[-1])

    def col(self):
        """Column index of every nonzero."""
        return np.repeat(np.arange(self.ncol), np.diff(self.colind))

    def T(self):
        mask = np.zeros((self.ncol, self.nrow), dtype=bool)
        mask[self.col(), self.row] = True
        return Pattern.from_dense(mask)

    def dense(self):
        m = np.zeros((self.nrow, self.ncol), dtype=bool)
        m[self.row, self.col()] = True
        return m

    def lower(self):
        """Nonzeros (row >= col) of a symmetric pattern, as (rows, cols)."""
        c = self.col()
        keep = self.row >= c
        return self.row[keep], c[keep]


def _ccs_args(A):
    import ctypes as ct
    colind = np.ascontiguousarray(A.colind, dtype=np.int32)
    row = np.ascontiguousarray(A.row if A.row.size else np.zeros(1), dtype=np.int32)
    return colind, row, ct


def uni_coloring(A):
    """Colour of every column of A such that columns of one colour share no row (the
    library's restatement of the reference's uni_coloring)."""
    from . import runtime as R
    colind, row, ct = _ccs_args(A)
    color = np.zeros(max(1, A.ncol), dtype=np.int32)
    R.check(R.load().casadi_gb300_uni_coloring(A.nrow, A.ncol, colind.ctypes.data,
                                               row.ctypes.data, color.ctypes.data))
    return color[:A.ncol].astype(np.int64)


def star_coloring(A, ordering=1):
    """Star colouring of a symmetric pattern (colour of every column); ordering 1 =
    largest-first, as the reference's default."""
    from . import runtime as R
    colind, row, ct = _ccs_args(A)
    color = np.zeros(max(1, A.ncol), dtype=np.int32)
    R.check(R.load().casadi_gb300_star_coloring(A.ncol, colind.ctypes.data, row.ctypes.data,
                                                ordering, color.ctypes.data))
    return color[:A.ncol].astype(np.int64)


def seed_matrix(color, n_colors=None):
    """Dense seed matrix D (ncol x n_colors): D[j, colour(j)] = 1."""
    n_colors = int(color.max()) + 1 if n_colors is None and color.size else (n_colors or 0)
    D = np.zeros((color.size, n_colors))
    D[np.arange(color.size), color] = 1.0
    return D


def jacobian_recovery(A, color):
    """For every nonzero of A (CCS order): the compressed row index d*nrow + i that holds it
    in J*D (D the seed matrix of the column colouring ``color``)."""
    return color[A.col()] * A.nrow + A.row


def hessian_recovery(A, color):
    """For every lower-triangle nonzero (i >= j) of a symmetric A, in CCS order of the lower
    triangle: the compressed index d*n + r of H*D (D from the star colouring ``color``) that
    holds H[i, j] with no other term mixed in. Returns (rows, cols, index)."""
    n = A.ncol
    dense = A.dense()
    rows, cols = A.lower()
    idx = np.empty(rows.size, np.int64)
    for k, (i, j) in enumerate(zip(rows, cols)):
        # row i of H*D at colour(j) holds sum of H[i, l] over l of that colour
        same = np.flatnonzero(color == color[j])
        if dense[i, same].sum() == 1:
            idx[k] = color[j] * n + i
            continue
        same = np.flatnonzero(color == color[i])
        if dense[j, same].sum() == 1:
            idx[k] = color[i] * n + j
            continue
        raise ValueError("colouring is not a star colouring at (%d, %d)" % (i, j))
    return rows, cols, idx
