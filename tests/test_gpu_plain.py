"""GPU parity of the plain IPT path against the oracle and the reference's
golden outputs, through the C ABI (host and device entry points)."""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, api
from oracle import oracle
from tests.conftest import device_to_host

pytestmark = pytest.mark.gpu

# The reference's own acceptance tolerances (runtests.cu:233-234,
# runtests_sparse.cu:422-428).
DENSE_TOL = 5e-9


def test_dense_reference_cases(cuda, golden):
    arrays, meta = golden
    for case in meta["dense"]:
        H = oracle.perturbative_matrix(case["n"], case["symmetric"])
        X, v, info = api.ipt_cuda(H, case["k"], case["iterations"])
        assert info["iterations"] == case["iterations"]
        gx = arrays["dense_%s_vectors" % case["name"]]
        gv = arrays["dense_%s_values" % case["name"]]
        assert np.abs(X - gx).max() <= DENSE_TOL, case["name"]
        assert np.abs(v - gv).max() <= DENSE_TOL, case["name"]
        assert oracle.max_relative_residual(H, X, v) <= 5e-9, case["name"]


def test_dense_with_initial_matches_oracle(cuda):
    H = oracle.perturbative_matrix(96, 1)
    rng = np.random.default_rng(3)
    X0 = np.eye(96, 12) + 1e-3 * rng.standard_normal((96, 12))
    X, v, _ = api.ipt_cuda(H, 12, 15, initial_vectors=X0)
    Xo, vo, _, _ = oracle.ipt_dense(H, 12, 15, x0=X0)
    assert np.abs(X - Xo).max() <= 1e-12
    assert np.abs(v - vo).max() <= 1e-12


def test_dense_tol_mode_matches_oracle(cuda):
    H = oracle.perturbative_matrix(96, 0)
    X, v, info = api.ipt_cuda_tol(H, 16, 1e-12, 300)
    Xo, vo, it, fp = oracle.ipt_dense(H, 16, 300, tol=1e-12, use_tol=True)
    assert abs(info["iterations"] - it) <= 1
    assert info["fixed_point_residual"] <= 1e-12
    assert np.abs(X - Xo).max() <= 1e-12
    assert np.abs(v - vo).max() <= 1e-11


def test_dense_tol_unconverged_returns_last_block(cuda):
    H = oracle.perturbative_matrix(32, 1)
    X, v, info = api.ipt_cuda_tol(H, 5, 1e-300, 4)
    Xo, vo, _, _ = oracle.ipt_dense(H, 5, 4)
    assert info["iterations"] == 4
    assert np.abs(X - Xo).max() <= 1e-14


def test_config0_plain_ipt_vs_dsyevd(cuda):
    from block_ipt_gb300 import workloads
    H, d = workloads.dense_config0(1024, seed=0)
    X, v, info = api.ipt_cuda_tol(H, 8, 1e-14, 200)
    w, _ = oracle.dsyevd_lowest(H, 8)
    hn = np.abs(H).sum(axis=1).max()
    assert np.abs(np.sort(v) - w).max() <= 1e-10 * hn
    Xn = X / np.linalg.norm(X, axis=0)
    r = np.linalg.norm(H @ Xn - Xn * v[None, :], axis=0)
    assert r.max() <= 1e-8 * hn


def _device_handle(torch):
    return C.c_void_p(torch.cuda.current_blas_handle())


def test_dense_device_entry(cuda):
    torch = cuda
    lib = _lib.load()
    H = oracle.perturbative_matrix(96, 1)
    dH = torch.from_numpy(H.T.copy()).cuda()  # column-major bytes: H^T row-major
    dvec = C.c_void_p()
    dval = C.c_void_p()
    it = C.c_int()
    fp = C.c_double()
    st = lib.ipt_cuda_device_tol(C.c_void_p(dH.data_ptr()), 96, 16, 1e-12, 300,
                                 _device_handle(torch), C.byref(dvec), C.byref(dval),
                                 C.byref(it), C.byref(fp))
    assert st == 0
    torch.cuda.synchronize()
    X = np.zeros((96, 16), order="F")
    v = np.zeros(16)
    device_to_host(dvec, X)
    device_to_host(dval, v)
    lib.ipt_cuda_free_device_result(dvec, dval)
    Xo, vo, ito, _ = oracle.ipt_dense(H, 16, 300, tol=1e-12, use_tol=True)
    assert abs(it.value - ito) <= 1
    assert np.abs(X - Xo).max() <= 1e-12
    assert np.abs(v - vo).max() <= 1e-11


def test_device_entry_invalid_arguments(cuda):
    torch = cuda
    lib = _lib.load()
    dvec = C.c_void_p(1)
    dval = C.c_void_p(1)
    st = lib.ipt_cuda_device(None, 8, 2, 3, _device_handle(torch), C.byref(dvec), C.byref(dval))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
    assert not dvec.value and not dval.value


def test_sparse_reference_cases(cuda, golden):
    arrays, meta = golden
    tolerances = {"synthetic_banded_k5": (1e-8, 1e-8), "h20_fci_w_k1": (1e-8, 1e-10)}
    for case in meta["sparse"]:
        name = case["name"]
        cp = arrays["sparse_%s_col_ptr" % name]
        ri = arrays["sparse_%s_row_ind" % name]
        va = arrays["sparse_%s_values_csc" % name]
        X, v, info = api.ipt_cuda_sparse_csc(cp, ri, va, case["n"], case["k"], case["iterations"])
        diff_tol, res_tol = tolerances[name]
        assert np.abs(X - arrays["sparse_%s_vectors" % name]).max() <= diff_tol, name
        assert np.abs(v - arrays["sparse_%s_values" % name]).max() <= diff_tol, name
        Hd = oracle.csc_to_dense(cp, ri, va, case["n"])
        assert oracle.max_relative_residual(Hd, X, v) <= res_tol, name


def test_sparse_unsorted_diagonal_is_permuted_back(cuda):
    """Reverse the banded matrix: targets are found after the sort and the
    vectors come back in the caller's row order."""
    n, k = 64, 5
    cp, ri, va = oracle.banded_csc(n)
    Hd = oracle.csc_to_dense(cp, ri, va, n)
    P = np.arange(n)[::-1]
    Hp = Hd[np.ix_(P, P)]
    from scipy.sparse import csc_matrix
    S = csc_matrix(Hp)
    X, v, _ = api.ipt_cuda_sparse_csc(S.indptr, S.indices, S.data, n, k, 80)
    Xo, vo, _, _ = oracle.ipt_dense(Hd, k, 80)
    np.testing.assert_allclose(v, vo, atol=1e-10)
    np.testing.assert_allclose(X, Xo[P, :], atol=1e-10)


def test_sparse_tol_mode(cuda):
    cp, ri, va = oracle.banded_csc(64)
    X, v, info = api.ipt_cuda_sparse_csc_tol(cp, ri, va, 64, 5, 1e-13, 500)
    rp, ci, vv, d, _ = oracle.prepare_sorted_csc(cp, ri, va, 64)
    Xo, vo, it, _ = oracle.ipt_csr(rp, ci, vv, d, 64, 5, 500, tol=1e-13, use_tol=True)
    assert abs(info["iterations"] - it) <= 1
    assert np.abs(X - Xo).max() <= 1e-12


def test_sparse_device_entry(cuda, golden):
    torch = cuda
    lib = _lib.load()
    arrays, _ = golden
    name = "synthetic_banded_k5"
    cp = torch.from_numpy(arrays["sparse_%s_col_ptr" % name].astype(np.int32)).cuda()
    ri = torch.from_numpy(arrays["sparse_%s_row_ind" % name].astype(np.int32)).cuda()
    va = torch.from_numpy(arrays["sparse_%s_values_csc" % name]).cuda()
    dvec = C.c_void_p()
    dval = C.c_void_p()
    st = lib.ipt_cuda_sparse_csc_device(C.c_void_p(cp.data_ptr()), C.c_void_p(ri.data_ptr()),
                                        C.c_void_p(va.data_ptr()), 64, 5, int(ri.numel()), 80,
                                        _device_handle(torch), C.byref(dvec), C.byref(dval))
    assert st == 0
    torch.cuda.synchronize()
    X = np.zeros((64, 5), order="F")
    v = np.zeros(5)
    device_to_host(dvec, X)
    device_to_host(dval, v)
    lib.ipt_cuda_free_device_result(dvec, dval)
    assert np.abs(X - arrays["sparse_%s_vectors" % name]).max() <= 1e-8
    assert np.abs(v - arrays["sparse_%s_values" % name]).max() <= 1e-8


def test_sparse_lifted_degenerate_targets(cuda):
    """Degenerate targets: the plain sparse path lifts them as the reference
    does (ipt_cuda.cu:5077-5090, fixtures from the reference's preparation):
    the result is the oracle's IPT on the prepared (rotated) matrix, rotated
    back; a matrix whose preparation the reference rejects is rejected."""
    import os
    from scipy.sparse import csc_matrix
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "lift_kat.npz"))
    lifted = 0
    for c in [str(x) for x in z["cases"]]:
        n, k, ncp, nri = (int(x) for x in z[c + "_params"])
        cp, ri = z[c + "_in"][:ncp], z[c + "_in"][ncp:ncp + nri]
        va = z[c + "_in_values"]
        if int(z[c + "_status"][0]) != 0:
            with pytest.raises(Exception):
                api.ipt_cuda_sparse_csc(cp, ri, va, n, k, 40)
            continue
        X, v, _ = api.ipt_cuda_sparse_csc(cp, ri, va, n, k, 40)
        Hp = csc_matrix((z[c + "_values"], z[c + "_row_ind"], z[c + "_col_ptr"]),
                        shape=(n, n)).tocsr()
        Hp.sort_indices()
        Xo, vo, _, _ = oracle.ipt_csr(Hp.indptr, Hp.indices, Hp.data, z[c + "_diag"], n, k, 40)
        Xb = oracle.unprepare_vectors(Xo, z[c + "_perm"], z[c + "_rot_first"],
                                      z[c + "_rot_size"], z[c + "_rot_values"])
        assert np.abs(X - Xb).max() <= 1e-10, c
        assert np.abs(v - vo).max() <= 1e-10, c
        H = oracle.csc_to_dense(cp, ri, va, n)
        assert oracle.max_relative_residual(H, X, v) <= 1e-8, c
        lifted += len(z[c + "_rot_first"]) > 0
    assert lifted >= 4


def test_sparse_general_lift_nonsymmetric(cuda, monkeypatch):
    """IPT_GB300_GENERAL_LIFT on the plain sparse path: a non-symmetric
    matrix with a degenerate target group is lifted by a general similarity
    (V^-1 H V on the group) and solved; the result is the oracle's IPT on
    the prepared matrix, transformed back, and satisfies H X = X diag(v)."""
    from scipy.sparse import csc_matrix
    from tests.test_prepare_lift import nonsymmetric_cluster_matrix
    monkeypatch.setenv("IPT_GB300_GENERAL_LIFT", "1")
    lifted = 0
    for seed, m in ((0, 2), (1, 3), (2, 5), (3, 8)):
        n, k = 40, 6
        cp, ri, va, H = nonsymmetric_cluster_matrix(n, m, 2, seed)
        prep = api.prepare_csc(cp, ri, va, n, k)
        X, v, _ = api.ipt_cuda_sparse_csc_tol(cp, ri, va, n, k, 1e-13, 200)
        Hp = csc_matrix((prep["values"], prep["row_ind"], prep["col_ptr"]), shape=(n, n)).tocsr()
        Hp.sort_indices()
        Xo, vo, _, _ = oracle.ipt_csr(Hp.indptr, Hp.indices, Hp.data, prep["diag"], n, k, 200,
                                      tol=1e-13, use_tol=True)
        Xb = oracle.unprepare_vectors(Xo, prep["perm"], prep["rot_first"], prep["rot_size"],
                                      prep["rot_values"])
        assert np.abs(v - vo).max() <= 1e-10
        assert np.abs(X - Xb).max() <= 1e-8
        assert oracle.max_relative_residual(H, X, v) <= 1e-8
        lifted += len(prep["rot_first"]) > 0
    assert lifted >= 3
