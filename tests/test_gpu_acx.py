"""ACX extrapolation over the dense FP64 IPT map (acx_cuda_device_tol)
against the oracle's restatement of IPT_C_GPU/src/ACX/acx_cuda.cu:390-620:
same step and map-evaluation counts, the same fixed point to rounding, the
reference's status codes."""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib
from oracle import oracle
from tests.conftest import device_to_host

pytestmark = pytest.mark.gpu


def run_acx(torch, H, k, tol, maxiter):
    lib = _lib.load()
    n = H.shape[0]
    dH = torch.from_numpy(np.ascontiguousarray(H.T)).cuda()  # column-major H
    res = _lib.ACXCudaResult()
    st = lib.acx_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, tol, maxiter, None,
                                 C.byref(res))
    if st != 0:
        assert not res.d_vectors and not res.d_values
        return st, None, None, res
    X = device_to_host(C.c_void_p(res.d_vectors), np.zeros((k, n))).T
    v = device_to_host(C.c_void_p(res.d_values), np.zeros(k))
    info = {f: getattr(res, f) for f in ("iterations", "f_calls", "converged", "max_residual",
                                          "fixed_point_residual", "n", "k")}
    lib.acx_cuda_free_result(C.byref(res))
    assert not res.d_vectors
    return st, X, v, info


@pytest.mark.parametrize("n,k,eps", [(300, 8, 0.06), (256, 256, 0.06), (513, 33, 0.2)])
def test_acx_matches_oracle(cuda, n, k, eps):
    H = oracle.acx_test_matrix(n, eps, seed=n + k)
    st, X, v, info = run_acx(cuda, H, k, 1e-12, 200)
    Xo, vo, io, so = oracle.acx_dense(H, k, 1e-12, 200)
    assert st == 0 and so == 0
    assert info["converged"] == 1 == io["converged"]
    assert (info["iterations"], info["f_calls"]) == (io["iterations"], io["f_calls"])
    assert info["n"] == n and info["k"] == k
    assert np.abs(X - Xo).max() <= 1e-10
    assert np.abs(v - vo).max() <= 1e-10 * np.abs(H).sum(1).max()
    assert info["fixed_point_residual"] < 1e-12
    # the eigenpairs continued from the diagonal: H x = lambda x
    R = H @ X - X * v
    assert np.abs(R).max() <= 1e-9 * np.abs(H).sum(1).max()


def test_acx_maxiter_without_convergence(cuda):
    H = oracle.acx_test_matrix(200, 0.5, seed=3)
    st, X, v, info = run_acx(cuda, H, 6, 1e-14, 2)
    Xo, vo, io, so = oracle.acx_dense(H, 6, 1e-14, 2)
    assert st == 0 == so
    assert info["converged"] == 0 == io["converged"]
    assert (info["iterations"], info["f_calls"]) == (2, 5) == (io["iterations"], io["f_calls"])
    assert np.abs(X - Xo).max() <= 1e-10


def test_acx_status_codes(cuda):
    lib = _lib.load()
    H = oracle.acx_test_matrix(64, 0.06, seed=1)
    H[5, 5] = H[2, 2]  # equal diagonal entries: the map's denominator vanishes
    st, _, _, res = run_acx(cuda, H, 4, 1e-12, 50)
    assert st == 5 and oracle.acx_dense(H, 4, 1e-12, 50)[3] == 5
    assert lib.acx_cuda_status_string(5) == b"zero diagonal denominator"
    assert np.isnan(res.max_residual) and res.d_vectors is None
    for n, k, tol, it in ((64, 0, 1e-12, 10), (64, 65, 1e-12, 10), (64, 4, 0.0, 10),
                          (64, 4, 1e-12, 0)):
        res = _lib.ACXCudaResult()
        assert lib.acx_cuda_device_tol(C.c_void_p(1), n, k, tol, it, None, C.byref(res)) == 1
    assert lib.acx_cuda_device_tol(None, 8, 2, 1e-12, 10, None, C.byref(res)) == 1


def run_mixed(torch, H, k, tf32_tol, tf32_maxiter, fp64_tol, fp64_maxiter, handle=True):
    lib = _lib.load()
    n = H.shape[0]
    dH = torch.from_numpy(np.ascontiguousarray(H.T)).cuda()
    res = _lib.ACXMixedTF32CudaResult()
    h = C.c_void_p(torch.cuda.current_blas_handle()) if handle else None
    st = lib.acx_mixed_precision_tf32_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, tf32_tol,
                                                      tf32_maxiter, fp64_tol, fp64_maxiter, h,
                                                      C.byref(res))
    torch.cuda.synchronize()
    if st != 0:
        assert not res.d_vectors and not res.d_values
        return st, None, None, res
    X = device_to_host(C.c_void_p(res.d_vectors), np.zeros((k, n))).T
    v = device_to_host(C.c_void_p(res.d_values), np.zeros(k))
    info = {f: getattr(res, f) for f, _ in _lib.ACXMixedTF32CudaResult._fields_
            if not f.startswith("d_")}
    lib.acx_mixed_precision_tf32_cuda_free_result(C.byref(res))
    return st, X, v, info


@pytest.mark.parametrize("n,k,eps", [(300, 8, 0.06), (400, 40, 0.2)])
def test_mixed_acx_matches_oracle(cuda, n, k, eps):
    """FP32 stage, then FP64 from its block: the oracle's counts (the FP32
    stage within one step, its sums run in another order) and the same FP64
    fixed point as the plain ACX."""
    H = oracle.acx_test_matrix(n, eps, seed=n + 7)
    st, X, v, info = run_mixed(cuda, H, k, 1e-5, 100, 1e-12, 100)
    Xo, vo, io, so = oracle.acx_mixed(H, k, 1e-5, 100, 1e-12, 100)
    assert st == 0 and so == 0
    assert info["tf32_converged"] == 1 == io["tf32_converged"]
    assert info["fp64_converged"] == 1 == io["fp64_converged"]
    assert abs(info["tf32_iterations"] - io["tf32_iterations"]) <= 1
    assert np.abs(X - Xo).max() <= 1e-10
    Xp, vp, _, _ = oracle.acx_dense(H, k, 1e-12, 200)
    assert np.abs(X - Xp).max() <= 1e-10
    assert np.abs(v - vp).max() <= 1e-10 * np.abs(H).sum(1).max()
    assert info["fp64_f_calls"] < oracle.acx_dense(H, k, 1e-12, 200)[2]["f_calls"]


def test_mixed_acx_status_codes(cuda):
    H = oracle.acx_test_matrix(64, 0.06, seed=1)
    st, _, _, res = run_mixed(cuda, H, 4, 1e-5, 50, 1e-12, 50, handle=False)
    assert st == 1 and np.isnan(res.tf32_time_sec)
    st, _, _, _ = run_mixed(cuda, H, 4, 0.0, 50, 1e-12, 50)
    assert st == 1
    H[5, 5] = H[2, 2]
    st, _, _, _ = run_mixed(cuda, H, 4, 1e-5, 50, 1e-12, 50)
    assert st == 5 and oracle.acx_mixed(H, 4, 1e-5, 50, 1e-12, 50)[3] == 5
