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
