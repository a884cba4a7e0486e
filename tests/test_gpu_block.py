"""GPU block solver (IPT -> CholQR2 -> Rayleigh-Ritz -> Davidson) against the
LAPACK eigen-oracle, through the C ABI.

Acceptance: |d lambda| <= 1e-10 ||H||, scaled residual <= 1e-8 (FP64 check).
"""
import os

import numpy as np
import pytest

from block_ipt_gb300 import api, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

LAMBDA_TOL = 1e-10
RES_TOL = 1e-8


def check_pairs(H, X, v, k, w=None):
    hn = np.abs(H).sum(axis=1).max()
    if w is None:
        w, _ = oracle.eigh_lowest(H, k)
    assert np.all(np.diff(v) >= -1e-12)
    assert np.abs(v - w).max() <= LAMBDA_TOL * hn, np.abs(v - w).max() / hn
    nrm = np.linalg.norm(X, axis=0)
    np.testing.assert_allclose(nrm, 1.0, atol=1e-10)
    r = np.linalg.norm(H @ X - X * v[None, :], axis=0) / max(1.0, hn)
    assert r.max() <= RES_TOL, r.max()


STRATEGIES = {"refine": 0, "davidson": 1}


@pytest.mark.parametrize("strategy", ["refine", "davidson"])
def test_block_fp64_config0(cuda, strategy):
    H, _ = workloads.dense_config0(1024, seed=1)
    X, v, rep = api.block_solve_dense(H, 8, "fp64", strategy=STRATEGIES[strategy])
    assert rep["converged"] == 1
    w, _ = oracle.dsyevd_lowest(H, 8)
    check_pairs(H, X, v, 8, w)


@pytest.mark.parametrize("strategy", ["refine", "davidson"])
def test_block_fp64_config1_shape_small(cuda, strategy):
    """The n=8192 construction at n=2048 (same spacing/decay), k=32."""
    H, _ = workloads.dense_config1(2048, seed=2)
    X, v, rep = api.block_solve_dense(H, 32, "fp64", ipt_maxiter=40,
                                      strategy=STRATEGIES[strategy])
    assert rep["converged"] == 1
    check_pairs(H, X, v, 32)


def test_block_fp64_unsorted_diagonal(cuda):
    H, _ = workloads.dense_config0(512, seed=3)
    P = np.random.default_rng(0).permutation(512)
    Hp = np.asfortranarray(H[np.ix_(P, P)])
    X, v, rep = api.block_solve_dense(Hp, 6, "fp64")
    assert rep["converged"] == 1
    check_pairs(Hp, X, v, 6)


def test_block_reference_dense_cases(cuda):
    for n, k, sym in [(32, 5, 1), (96, 16, 1)]:
        H = oracle.perturbative_matrix(n, sym)
        X, v, rep = api.block_solve_dense(H, k, "fp64", oversample=4)
        check_pairs(H, X, v, k)


def test_block_csr_banded(cuda):
    cp, ri, va = oracle.banded_csc(64)
    X, v, rep = api.block_solve_csr(cp, ri, va, 64, 5, "fp64")
    Hd = oracle.csc_to_dense(cp, ri, va, 64)
    check_pairs(Hd, X, v, 5)


def test_refine_falls_back_to_davidson_on_near_degenerate_targets(cuda):
    """Targets 1 and 2 nearly degenerate and strongly coupled: the IPT map
    does not contract there, so the refinement hands over to Davidson, which
    still returns the FP64-accurate pairs."""
    H, _ = workloads.dense_config0(400, seed=7)
    H = np.array(H)
    H[1, 1] = H[2, 2] = 1.5
    H[1, 2] = H[2, 1] = 0.3
    H = np.asfortranarray(H)
    X, v, rep = api.block_solve_dense(H, 6, "fp64")
    assert rep["converged"] == 1
    check_pairs(H, X, v, 6)


def test_block_csr_random_sparse(cuda):
    from scipy.sparse import csr_matrix, random as sprandom
    rng = np.random.default_rng(5)
    n = 3000
    A = sprandom(n, n, density=0.004, random_state=rng, format="csr") * 0.05
    A = A + A.T
    d = np.sort(rng.uniform(0, 300, n))
    H = (A + csr_matrix((d, (np.arange(n), np.arange(n))), shape=(n, n))).tocsr()
    H.sort_indices()
    X, v, rep = api.block_solve_csr(H.indptr, H.indices, H.data, n, 12, "fp64")
    assert rep["converged"] == 1
    Hd = H.toarray()
    check_pairs(Hd, X, v, 12)


def test_block_cluster_env_path(cuda, monkeypatch):
    """ipt_cuda_sparse_csc_tol with IPT_BLOCK_CLUSTER + IPT_DAVIDSON_ENRICH runs
    the block path: ascending Ritz values, unit vectors (ipt_cuda.cu:5070-5075)."""
    monkeypatch.setenv("IPT_BLOCK_CLUSTER", "1")
    monkeypatch.setenv("IPT_DAVIDSON_ENRICH", "1")
    monkeypatch.setenv("IPT_DAVIDSON_STEPS", "20")
    cp, ri, va = oracle.banded_csc(64)
    X, v, info = api.ipt_cuda_sparse_csc_tol(cp, ri, va, 64, 5, 1e-12, 200)
    Hd = oracle.csc_to_dense(cp, ri, va, 64)
    w, _ = oracle.eigh_lowest(Hd, 5)
    np.testing.assert_allclose(v, w, atol=1e-9)
    np.testing.assert_allclose(np.linalg.norm(X, axis=0), 1.0, atol=1e-10)
    assert info["basis_cols"] >= 5


@pytest.mark.parametrize("prec", ["fp64", "fp16"])
def test_block_dense_diagonal_order_cases(cuda, prec):
    """The one-pass statistics decide whether H is permuted: a permuted
    (descending somewhere) diagonal, and ties (a stable sort keeps them)."""
    H, _ = workloads.dense_config0(512, seed=4)
    P = np.random.default_rng(1).permutation(512)
    Hp = np.asfortranarray(H[np.ix_(P, P)])
    X, v, rep = api.block_solve_dense(Hp, 6, prec)
    assert rep["converged"] == 1
    check_pairs(Hp, X, v, 6)
    Ht = np.array(H)
    Ht[np.arange(200, 210), np.arange(200, 210)] = H[200, 200]  # a run of equal entries
    X, v, rep = api.block_solve_dense(np.asfortranarray(Ht), 6, prec)
    assert rep["converged"] == 1
    check_pairs(Ht, X, v, 6)


def test_trace_marks(cuda):
    """Phase marks of a dense mixed solve: every phase present, the GPU
    timestamps in stream order, no marks once tracing is off."""
    import torch
    H, _ = workloads.dense_config1(1024, seed=5)
    dev = torch.device("cuda", 0)
    dH = torch.from_numpy(np.asfortranarray(H).T.copy()).to(dev)
    dX = torch.empty((16, 1024), dtype=torch.float64, device=dev)
    dv = torch.empty(16, dtype=torch.float64, device=dev)
    api.trace_enable(True)
    rep = api.block_solve_dense_device(dH.data_ptr(), 1024, 16, dX.data_ptr(), dv.data_ptr(),
                                       "fp16")
    torch.cuda.synchronize()
    marks = api.trace_read()
    api.trace_enable(False)
    assert rep["converged"] == 1
    labels = [m[0] for m in marks]
    for want in ("dense:start", "dense:stats_done", "dense:operator_done", "ipt:start",
                 "refine:start", "refine:defect", "refine:rayleigh_ritz", "refine:end",
                 "dense:end"):
        assert want in labels, (want, labels)
    assert labels[0] == "dense:start" and labels[-1] == "dense:end"
    gpu = np.array([m[2] for m in marks], dtype=np.int64)
    host = np.array([m[1] for m in marks], dtype=np.int64)
    assert np.all(np.diff(gpu) >= 0) and np.all(np.diff(host) >= 0)
    api.block_solve_dense_device(dH.data_ptr(), 1024, 16, dX.data_ptr(), dv.data_ptr(), "fp16")
    assert api.trace_read() == []


@pytest.mark.parametrize("df", ["0", "1"])
def test_block_csr_davidson_products_fp64_and_double_float(cuda, monkeypatch, df):
    """The Davidson solve with its Gram/tall products in FP64 and in
    double-float (the default from 16384 rows) reaches the LAPACK pairs."""
    from scipy.sparse import csr_matrix, random as sprandom
    monkeypatch.setenv("IPT_GB300_DF_DAVIDSON", df)
    rng = np.random.default_rng(15)
    n = 2500
    A = sprandom(n, n, density=0.004, random_state=rng, format="csr") * 0.05
    A = A + A.T
    d = np.sort(rng.uniform(0, 250, n))
    H = (A + csr_matrix((d, (np.arange(n), np.arange(n))), shape=(n, n))).tocsr()
    H.sort_indices()
    X, v, rep = api.block_solve_csr(H.indptr, H.indices, H.data, n, 10, "fp64", strategy=1)
    assert rep["converged"] == 1
    check_pairs(H.toarray(), X, v, 10)
