"""The in-place Gauss-Jordan inversion of the coarsest multigrid levels
(`gj_invert_cta` in xcore.jl_gb300/csrc/xc_stokes.cu), restated step for step
in numpy and checked against numpy's inverse on CPU: pivot search with ties
to the lower row, row interchange, scaling of the pivot row with its pivot
entry turned into 1/p, elimination of every other row with the saved column,
and the row interchanges undone as column interchanges, last first.  The GPU
tests check the solver that uses it end to end."""
import numpy as np
import pytest


def gj_invert(A, thr_rel=1e-12):
    M = np.array(A, dtype=np.float64, copy=True)
    n = M.shape[0]
    ok = True
    amax = np.abs(M).max()
    piv = np.zeros(n, dtype=int)
    for k in range(n):
        col = np.abs(M[k:, k])
        bi = k + int(np.argmax(col))          # argmax takes the first of equal values
        piv[k] = bi
        if not col.max() > thr_rel * amax:
            ok = False
        if bi != k:
            M[[k, bi], :] = M[[bi, k], :]
        pv = M[k, k]
        fcol = M[:, k].copy()
        M[k, :] = np.where(np.arange(n) == k, 1.0, M[k, :]) / pv
        for i in range(n):
            if i != k:
                M[i, :] = np.where(np.arange(n) == k, 0.0, M[i, :]) - fcol[i] * M[k, :]
    for k in range(n - 1, -1, -1):
        p = piv[k]
        if p != k:
            M[:, [k, p]] = M[:, [p, k]]
    return M, ok


@pytest.mark.parametrize("n", [1, 4, 17, 60, 64])
def test_inverse_of_pivoting_matrices(n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    # a small leading diagonal forces row interchanges at every step
    A[np.arange(n), np.arange(n)] *= 1e-3
    inv, ok = gj_invert(A)
    assert ok
    np.testing.assert_allclose(inv @ A, np.eye(n), atol=1e-9)
    np.testing.assert_allclose(inv, np.linalg.inv(A), rtol=1e-8, atol=1e-10)


def test_identity_and_ghost_like_rows():
    """Rows like the levels' ghost rows (x_g + s x_i = b, unit diagonal)
    mixed with diagonally dominant interior rows."""
    n = 12
    rng = np.random.default_rng(3)
    A = np.diag(4.0 + rng.random(n))
    A += np.diag(-1.0 * np.ones(n - 1), 1) + np.diag(-1.0 * np.ones(n - 1), -1)
    A[0, :] = 0.0
    A[0, 0], A[0, n - 2] = 1.0, -1.0      # a periodic ghost row
    inv, ok = gj_invert(A)
    assert ok
    np.testing.assert_allclose(inv @ A, np.eye(n), atol=1e-12)


def test_singular_matrix_flagged():
    """A zero pivot clears ok (the kernel then keeps the Jacobi sweeps); the
    values it leaves are not used."""
    A = np.ones((5, 5))
    with np.errstate(all="ignore"):
        _, ok = gj_invert(A)
    assert not ok
