"""Seed colourings (host code of the C ABI, no device): validity of the column and star
colourings on random and structured patterns, exact recovery of the nonzeros from the
compressed products, and agreement with hand-checked small cases of the reference's
algorithms."""
import numpy as np
import pytest

from casadi_gb300 import coloring as K


def _random_pattern(rng, nrow, ncol, density):
    return K.Pattern.from_dense(rng.random((nrow, ncol)) < density)


def _random_symmetric(rng, n, density):
    m = rng.random((n, n)) < density
    m = m | m.T
    np.fill_diagonal(m, True)
    return K.Pattern.from_dense(m)


def _banded_symmetric(n, bw):
    i, j = np.indices((n, n))
    return K.Pattern.from_dense(np.abs(i - j) <= bw)


def is_star_coloring(A, color):
    """Adjacent vertices differ, and every path on four vertices v-w-x-y with
    colour(v) == colour(x) and colour(w) == colour(y) is forbidden."""
    dense = A.dense()
    n = A.ncol
    adj = [np.flatnonzero(dense[:, v] & (np.arange(n) != v)) for v in range(n)]
    for v in range(n):
        if np.any(color[adj[v]] == color[v]):
            return False
    for v in range(n):
        for w in adj[v]:
            for x in adj[w]:
                if x == v or color[x] != color[v]:
                    continue
                for y in adj[x]:
                    if y != w and color[y] == color[w]:
                        return False
    return True


@pytest.mark.parametrize("seed", range(5))
def test_uni_coloring_columns_of_one_colour_share_no_row(seed):
    rng = np.random.default_rng(seed)
    A = _random_pattern(rng, 40, 60, 0.08)
    color = K.uni_coloring(A)
    dense = A.dense()
    for c in range(color.max() + 1):
        assert dense[:, color == c].sum(axis=1).max(initial=0) <= 1
    # greedy in column order: column 0 gets colour 0, colours are used contiguously
    assert color[0] == 0 and set(color) == set(range(color.max() + 1))


def test_uni_coloring_small_case_by_hand():
    # columns 0 and 2 share row 1, 1 and 2 share nothing, 3 is empty
    m = np.array([[1, 0, 0, 0],
                  [1, 0, 1, 0],
                  [0, 1, 0, 0]], bool)
    color = K.uni_coloring(K.Pattern.from_dense(m))
    assert color.tolist() == [0, 0, 1, 0]


@pytest.mark.parametrize("seed", range(5))
def test_star_coloring_is_a_star_coloring(seed):
    rng = np.random.default_rng(seed)
    A = _random_symmetric(rng, 30, 0.08)
    for ordering in (0, 1):
        color = K.star_coloring(A, ordering)
        assert is_star_coloring(A, color)


def test_star_coloring_banded():
    A = _banded_symmetric(50, 2)
    color = K.star_coloring(A)
    assert is_star_coloring(A, color)
    assert color.max() + 1 <= 9


@pytest.mark.parametrize("seed", range(3))
def test_recovery_is_exact(seed):
    rng = np.random.default_rng(seed)
    # Jacobian: J*D then pick each nonzero
    A = _random_pattern(rng, 25, 35, 0.1)
    J = np.zeros((A.nrow, A.ncol))
    J[A.row, A.col()] = rng.standard_normal(A.nnz)
    color = K.uni_coloring(A)
    comp = (J @ K.seed_matrix(color)).T.reshape(-1)  # [colour][row]
    idx = K.jacobian_recovery(A, color)
    assert np.array_equal(comp[idx], J[A.row, A.col()])
    # Hessian: H*D then the star recovery of the lower triangle
    S = _random_symmetric(rng, 30, 0.1)
    H = np.zeros((30, 30))
    r, c = S.lower()
    vals = rng.standard_normal(r.size)
    H[r, c] = vals
    H[c, r] = vals
    color = K.star_coloring(S)
    comp = (H @ K.seed_matrix(color)).T.reshape(-1)
    rows, cols, idx = K.hessian_recovery(S, color)
    assert np.array_equal(comp[idx], H[rows, cols])


def test_bad_patterns_are_refused():
    from casadi_gb300 import runtime as R
    import ctypes as ct
    colind = np.array([0, 2, 1], np.int32)  # decreasing
    row = np.array([0, 1], np.int32)
    color = np.zeros(2, np.int32)
    assert R.load().casadi_gb300_uni_coloring(2, 2, colind.ctypes.data, row.ctypes.data,
                                              color.ctypes.data) == -2
    colind = np.array([0, 2], np.int32)
    row = np.array([1, 0], np.int32)  # unsorted
    assert R.load().casadi_gb300_star_coloring(2, colind.ctypes.data, row.ctypes.data, 1,
                                               color.ctypes.data) == -2
