"""The Householder column signs the Rayleigh-mixed entry applies to its
CholQR basis (ipt_block_householder_signs, host code) against LAPACK's
Householder QR (numpy.linalg.qr = dgeqrf + dorgqr, the convention of the
reference's cusolverDnDgeqrf/Dorgqr, ipt_rayleigh_mixed_cuda.cu:141-254)."""
import numpy as np

from block_ipt_gb300 import api


def cholqr(X):
    L = np.linalg.cholesky(X.T @ X)
    return np.linalg.solve(L, X.T).T


def test_signs_match_lapack_householder(lib):
    rng = np.random.default_rng(0)
    checked = 0
    for t in range(600):
        n = int(rng.integers(2, 70))
        k = int(rng.integers(1, min(n, 16) + 1))
        X = rng.standard_normal((n, k))
        if t % 3 == 0:
            # IPT-like blocks: unit diagonal dominating
            X[:k, :k] += np.eye(k) * rng.uniform(0, 5)
        if t % 5 == 0:
            X[:k, :k] -= 2 * np.eye(k)
        Qh, Rh = np.linalg.qr(X)
        Qc = cholqr(X)
        s = api.householder_signs(Qc[:k, :k], n)
        np.testing.assert_array_equal(s, np.sign(np.diag(Rh)))
        np.testing.assert_allclose(Qc * s[None, :], Qh, atol=1e-9)
        checked += 1
    assert checked == 600


def test_ipt_block_signs_square_and_invalid(lib):
    # a square block: the last column is not reflected (LAPACK dlarfg with a
    # single entry keeps its sign)
    X = np.array([[2.0, 1.0], [0.5, 3.0]])
    _, Rh = np.linalg.qr(X)
    s = api.householder_signs(cholqr(X)[:2, :2], 2)
    np.testing.assert_array_equal(s, np.sign(np.diag(Rh)))
    import ctypes as C
    out = np.zeros(2)
    assert lib.ipt_block_householder_signs(C.c_void_p(X.ctypes.data), 2, 1,
                                           C.c_void_p(out.ctypes.data)) == 1
