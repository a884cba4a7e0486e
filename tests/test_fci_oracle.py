"""The CPU restatement of the matrix-free FCI-like Hamiltonian against the
FCI-like CSR workload it mirrors (same strings, links, hashes; FP32 instead
of FP64 normal deviates), and its sigma against its own CSR."""
import numpy as np
import pytest
from scipy.sparse import csr_matrix

from block_ipt_gb300 import workloads
from oracle import oracle


@pytest.mark.parametrize("norb,na,nb", [(6, 3, 3), (8, 4, 4), (7, 3, 2)])
def test_matches_csr_workload(norb, na, nb):
    rp, ci, va, d = oracle.fci_matrix(norb, na, nb, seed=0)
    rp2, ci2, va2, d2 = workloads.fci_like_csr(norb, na, nb, seed=0)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2)
    assert np.abs(va - va2).max() <= 1e-7 * np.abs(va2).max()
    assert np.abs(d - d2).max() <= 1e-7 * np.abs(d2).max()
    H = csr_matrix((va, ci, rp), shape=(len(d), len(d)))
    assert abs(H - H.T).max() == 0.0


def test_row_length_and_dimension():
    L = oracle._fci_lib()
    assert L.oracle_fci_dimension(14, 7, 7) == 11778624
    assert L.oracle_fci_row_length(14, 7, 7) == 3381
    assert L.oracle_fci_row_length(10, 5, 5) == 875


def test_sigma_matches_csr_product():
    rp, ci, va, d = oracle.fci_matrix(6, 3, 3, seed=5)
    n = len(d)
    X = np.random.default_rng(0).standard_normal((n, 3))
    Y = oracle.fci_sigma(6, 3, 3, X, seed=5)
    H = csr_matrix((va, ci, rp), shape=(n, n))
    assert np.abs(Y - H @ X).max() <= 1e-13 * np.abs(Y).max()
