"""The projected-matrix eigensolver (ipt_block_symmetric_eig) vs LAPACK."""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib

pytestmark = pytest.mark.gpu


def run(torch, T):
    m = T.shape[0]
    dT = torch.from_numpy(np.asfortranarray(T).T.copy()).cuda()
    dw = torch.empty(m, dtype=torch.float64, device="cuda")
    dZ = torch.empty((m, m), dtype=torch.float64, device="cuda")
    st = _lib.load().ipt_block_symmetric_eig(C.c_void_p(dT.data_ptr()), m,
                                             C.c_void_p(dw.data_ptr()), C.c_void_p(dZ.data_ptr()),
                                             C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    return dw.cpu().numpy(), dZ.T.cpu().numpy()


def spectrum_matrix(lam, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((len(lam), len(lam))))
    return (Q * lam) @ Q.T


@pytest.mark.parametrize("m", [1, 2, 7, 32, 48, 96, 112])
def test_random_symmetric(cuda, m):
    rng = np.random.default_rng(m)
    A = rng.standard_normal((m, m))
    T = 0.5 * (A + A.T) + np.diag(np.arange(m) * 0.3)
    w, Z = run(cuda, T)
    ref = np.linalg.eigvalsh(T)
    nrm = np.abs(T).sum(axis=1).max()
    assert np.abs(w - ref).max() <= 1e-13 * nrm
    assert np.abs(Z.T @ Z - np.eye(m)).max() <= 1e-13
    assert np.abs(T @ Z - Z * w).max() <= 1e-12 * nrm


def test_clustered_and_degenerate(cuda):
    lam = np.concatenate([[1.0, 1.0, 1.0], [2.0, 2.0 + 1e-9], [3.0, 3.0 + 1e-6, 3.0 + 2e-6],
                          np.linspace(5.0, 40.0, 88)])
    T = spectrum_matrix(lam, 3)
    w, Z = run(cuda, T)
    nrm = np.abs(T).sum(axis=1).max()
    assert np.abs(w - np.sort(lam)).max() <= 1e-12 * nrm
    assert np.abs(Z.T @ Z - np.eye(len(lam))).max() <= 1e-13
    assert np.abs(T @ Z - Z * w).max() <= 1e-12 * nrm


def test_nearly_diagonal_projected_matrix(cuda):
    """The shape of a Davidson projected matrix: Ritz values on the diagonal
    plus small couplings to new directions."""
    rng = np.random.default_rng(9)
    m = 80
    T = np.diag(np.sort(rng.uniform(10, 12, m)))
    B = 1e-4 * rng.standard_normal((m, m))
    T += B + B.T
    w, Z = run(cuda, T)
    assert np.abs(w - np.linalg.eigvalsh(T)).max() <= 1e-13 * np.abs(T).sum(1).max()
    assert np.abs(Z.T @ Z - np.eye(m)).max() <= 1e-13


@pytest.mark.parametrize("kind", ["scalar", "geometric", "tight_cluster"])
def test_hard_spectra(cuda, kind):
    """Spectra that leave many pairs to the FP64 polish: a multiple of the
    identity (one eigenvalue of multiplicity m), eigenvalues spread over nine
    decades, and m - 4 eigenvalues inside a window of width 1e-2 next to a
    few far ones."""
    m = 96
    rng = np.random.default_rng(21)
    if kind == "scalar":
        T = 3.0 * np.eye(m)
        lam = np.full(m, 3.0)
    else:
        if kind == "geometric":
            lam = np.geomspace(1e-6, 1e3, m)
        else:
            lam = np.sort(np.concatenate([rng.uniform(0.0, 0.01, m - 4), [5.0, 6.0, 7.0, 100.0]]))
        T = spectrum_matrix(lam, 22)
    w, Z = run(cuda, T)
    nrm = np.abs(T).sum(axis=1).max()
    assert np.abs(w - np.sort(lam)).max() <= 1e-13 * nrm
    assert np.abs(Z.T @ Z - np.eye(m)).max() <= 1e-13
    assert np.abs(T @ Z - Z * w).max() <= 1e-12 * nrm


def test_invalid_sizes(cuda):
    torch = cuda
    d = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = C.c_void_p(d.data_ptr())
    lib = _lib.load()
    assert lib.ipt_block_symmetric_eig(p, 0, p, p, None) == 1
    assert lib.ipt_block_symmetric_eig(p, 113, p, p, None) == 1
    assert lib.ipt_block_symmetric_eig(None, 2, p, p, None) == 1


def chol_inv(torch, G, precision=0):
    """(status, Rinv, shifts) of ipt_block_cholesky_inverse on the GPU."""
    m = G.shape[0]
    dG = torch.from_numpy(np.asfortranarray(G).T.copy()).cuda()
    dR = torch.zeros((m, m), dtype=torch.float64, device="cuda")
    shifts = C.c_int(-7)
    st = _lib.load().ipt_block_cholesky_inverse(
        C.c_void_p(dG.data_ptr()), m, C.c_void_p(dR.data_ptr()), C.byref(shifts), precision,
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, dR.T.cpu().numpy(), shifts.value


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("m", [1, 5, 31, 32, 33, 64, 112])
def test_cholesky_inverse_spd(cuda, m, precision):
    """One-warp register kernels (m <= 32: FP64, or double-float ~48 bits) and
    the FP64 shared-memory kernel (m > 32) against LAPACK's Cholesky: R^{-1}
    upper triangular with R^{-T} G R^{-1} = I.  Tolerances: FP64 as LAPACK;
    double-float 64x looser (its unit roundoff 2^-47)."""
    rng = np.random.default_rng(100 + m)
    X = rng.standard_normal((4 * m + 8, m)) * (1.0 + np.arange(m))  # columns of mixed scale
    G = X.T @ X
    st, Rinv, shifts = chol_inv(cuda, G, precision)
    assert st == 0 and shifts == 0
    assert np.all(np.tril(Rinv, -1) == 0.0)
    R_ref = np.linalg.cholesky(G).T
    loose = 64.0 if (precision == 1 and m <= 32) else 1.0
    np.testing.assert_allclose(Rinv, np.linalg.inv(R_ref), rtol=1e-10 * loose,
                               atol=1e-12 * loose * np.abs(np.linalg.inv(R_ref)).max())
    assert np.abs(Rinv.T @ G @ Rinv - np.eye(m)).max() <= 1e-12 * loose


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("m", [8, 40])
def test_cholesky_inverse_shift_retries(cuda, m, precision):
    """An indefinite Gram-like matrix (two eigenvalues at -1e-9 trace) is
    factored with the first shift of the sequence 1e-14 trace * 100^j that
    works (both kernels)."""
    rng = np.random.default_rng(7 + m)
    X = rng.standard_normal((2 * m, m - 2))
    X = np.hstack([X, X[:, :2]])  # two repeated columns
    G = X.T @ X
    G -= 1e-9 * np.trace(G) * np.eye(m)
    st, Rinv, shifts = chol_inv(cuda, G, precision)
    assert st == 0 and shifts >= 3
    shift = 1e-14 * np.trace(np.abs(G)) * 100.0 ** (shifts - 1)
    Gs = G + shift * np.eye(m)
    assert np.all(np.isfinite(Rinv)) and np.all(np.tril(Rinv, -1) == 0.0)
    tol = 1e-15 * 10 * m * np.linalg.cond(Gs)
    assert np.abs(Rinv.T @ Gs @ Rinv - np.eye(m)).max() <= tol


def test_cholesky_inverse_invalid(cuda):
    G = np.eye(4)
    G[1, 1] = np.nan
    for precision in (0, 1):
        st, _, shifts = chol_inv(cuda, G, precision)
        assert st == _lib.IPT_CUDA_INVALID_ARGUMENT and shifts == -1  # no shift worked
    st, _, _ = chol_inv(cuda, np.eye(113))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
    st, _, _ = chol_inv(cuda, np.eye(4), precision=2)
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
