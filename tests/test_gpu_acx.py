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


def published_cases():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acx_published.json")
    with open(path) as f:
        return json.load(f)["cases"]


def run_ipt_device(torch, H, k, tol, maxiter):
    lib = _lib.load()
    n = H.shape[0]
    dH = torch.from_numpy(np.ascontiguousarray(H.T)).cuda()
    vec = C.c_void_p()
    val = C.c_void_p()
    it = C.c_int(0)
    fp = C.c_double(0.0)
    st = lib.ipt_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, tol, maxiter,
                                 C.c_void_p(torch.cuda.current_blas_handle()), C.byref(vec),
                                 C.byref(val), C.byref(it), C.byref(fp))
    assert st == 0, _lib.status_string(st)
    lib.ipt_cuda_free_device_result(vec, val)
    return it.value, fp.value


@pytest.mark.parametrize("which", [0, 1, 10])
def test_acx_and_plain_ipt_match_the_published_runs(cuda, which):
    """Parity pin against the reference's own runs (its ACX sweep benchmark
    on an A100, results/ACX): on the sweep's matrices, regenerated bit for
    bit (N = 64 smoke case; N = 4096 at eps = 0.06 and 0.12; k = n, tol
    1e-12), the GPU ACX takes the published number of steps and map
    evaluations and the GPU plain IPT the published number of iterations,
    and both fixed-point residuals end below the tolerance."""
    case = published_cases()[which]
    n, eps = case["n"], case["epsilon"]
    assert which == 0 or n == 4096
    H = oracle.acx_sweep_matrix(n, eps)
    st, X, v, info = run_acx(cuda, H, n, case["tol"], case["maxiter"])
    assert st == 0 and info["converged"] == 1
    assert (info["iterations"], info["f_calls"]) == (case["acx"]["iterations"],
                                                     case["acx"]["f_calls"])
    assert info["fixed_point_residual"] <= case["tol"]
    it, fp = run_ipt_device(cuda, H, n, case["tol"], case["maxiter"])
    assert it == case["ipt"]["iterations"]
    assert fp <= case["tol"]


def run_acx_rayleigh(torch, H, k, tf32_tol, tf32_maxiter, fp64_tol, fp64_maxiter):
    lib = _lib.load()
    n = H.shape[0]
    dH = torch.from_numpy(np.ascontiguousarray(H.T)).cuda()
    res = _lib.ACXRayleighMixedTF32CudaResult()
    st = lib.acx_rayleigh_mixed_tf32_cuda_device_tol(
        C.c_void_p(dH.data_ptr()), n, k, tf32_tol, tf32_maxiter, fp64_tol, fp64_maxiter,
        C.c_void_p(torch.cuda.current_blas_handle()), C.byref(res))
    if st != 0:
        assert not res.d_vectors and not res.d_values
        return st, None, None, None
    X = device_to_host(C.c_void_p(res.d_vectors), np.zeros((k, n))).T
    v = device_to_host(C.c_void_p(res.d_values), np.zeros(k))
    info = {f[0]: getattr(res, f[0]) for f in res._fields_ if not f[0].startswith("d_")}
    lib.acx_rayleigh_mixed_tf32_cuda_free_result(C.byref(res))
    assert not res.d_vectors and res.n == 0
    return st, X, v, info


@pytest.mark.parametrize("n,k,eps", [(96, 8, 0.06), (300, 32, 0.1), (64, 64, 0.06)])
def test_acx_rayleigh_against_oracle_and_lapack(cuda, n, k, eps):
    """The Rayleigh ACX entry (acx_rayleigh_mixed_precision_cuda.cu:289-434)
    against the oracle's restatement with an FP64 first stage: the FP32 ACX
    block spans the target subspace to within its rounding, so the Ritz
    values agree with the oracle's and LAPACK's to 1e-10 ||H||, the vectors to
    1e-4 of their size, the column signs of the Householder QR exactly; the
    FP64 stage on the k x k matrix converges like the oracle's."""
    H = oracle.acx_sweep_matrix(n, eps)
    st, X, v, info = run_acx_rayleigh(cuda, H, k, 1e-6, 100, 1e-12, 100)
    assert st == 0
    Xo, vo, Qo, io, so = oracle.acx_rayleigh(H, k, 1e-6, 100, 1e-12, 100)
    assert so == 0
    hn = np.abs(H).sum(1).max()
    assert info["n"] == n and info["k"] == k
    assert info["tf32_iterations"] > 0 and info["fp64_converged"] == 1 == io["converged"]
    assert info["fp64_iterations"] <= io["iterations"] + 2
    assert np.abs(v - vo).max() <= 1e-10 * hn
    w, _ = oracle.dsyevd_lowest(H, k)
    assert np.abs(np.sort(v) - w).max() <= 1e-10 * hn
    np.testing.assert_array_equal(np.sign(np.diag(X[:k, :k])), np.sign(np.diag(Xo[:k, :k])))
    assert np.abs(X - Xo).max() <= 1e-4 * np.abs(Xo).max()
    parts = ("tf32_time_sec", "orthogonalize_time_sec", "rayleigh_transform_time_sec",
             "fp64_time_sec", "backtransform_time_sec")
    assert abs(sum(info[p] for p in parts) - info["total_time_sec"]) <= 1e-9


def test_acx_rayleigh_invalid_arguments(cuda):
    torch = cuda
    lib = _lib.load()
    h = C.c_void_p(torch.cuda.current_blas_handle())
    dH = torch.eye(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dH.data_ptr())
    res = _lib.ACXRayleighMixedTF32CudaResult()
    f = lib.acx_rayleigh_mixed_tf32_cuda_device_tol
    assert f(None, 8, 2, 1e-6, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 9, 1e-6, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 2, 0.0, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, 1e-12, 0, h, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, 1e-12, 5, None, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, 1e-12, 5, h, None) == 1
    assert not res.d_vectors and np.isnan(res.total_time_sec)
