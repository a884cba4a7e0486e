"""The Rayleigh-mixed entry point ipt_rayleigh_mixed_tf32_cuda_device_tol
(IPT_C_GPU/src/mixed_precision/ipt_rayleigh_mixed_cuda.cu:274-400) through
the C ABI, against the oracle's restatement of the same driver with an FP64
first stage (oracle.rayleigh_mixed) and against LAPACK dsyevd.

Tolerances: the TF32 stage leaves the block within the operand rounding
(2^-11 relative per entry of Delta) of the FP64 iterate, so the subspace the
Rayleigh-Ritz step sees differs from the oracle's by an angle theta of that
order times ||Delta|| / gap.  Ritz values move by O(theta^2 ||H||) and the
vectors by O(theta): values within 1e-10 ||H||_inf of the oracle's and of
dsyevd, vectors within 5e-3 max|V| (the tensor-core stage's bar), the
column signs of the Householder QR exactly, and the FP64 stage to fp64_tol.
"""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, api, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def run(torch, H, k, tf32_tol=1e-6, tf32_maxiter=200, fp64_tol=1e-12, fp64_maxiter=300):
    from tests.conftest import device_to_host
    n = H.shape[0]
    dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()
    res = api.rayleigh_mixed_tf32_device(dH.data_ptr(), n, k, tf32_tol, tf32_maxiter, fp64_tol,
                                         fp64_maxiter, torch.cuda.current_blas_handle())
    torch.cuda.synchronize()
    V = np.zeros((n, k), order="F")
    v = np.zeros(k)
    device_to_host(C.c_void_p(res.d_vectors), V)
    device_to_host(C.c_void_p(res.d_values), v)
    info = {f[0]: getattr(res, f[0]) for f in res._fields_ if not f[0].startswith("d_")}
    api.free_rayleigh_result(res)
    assert not res.d_vectors and not res.d_values and res.n == 0
    return V, v, info


def check(H, k, V, v, info, fp64_tol=1e-12):
    hn = np.abs(H).sum(axis=1).max()
    Vo, vo, Qo, _, _ = oracle.rayleigh_mixed(H, k, 1e-6, 200, fp64_tol, 300)
    assert info["n"] == H.shape[0] and info["k"] == k
    assert info["tf32_iterations"] > 0 and info["fp64_iterations"] > 0
    assert info["fp64_fixed_point_residual"] <= fp64_tol
    parts = ("tf32_time_sec", "orthogonalize_time_sec", "rayleigh_transform_time_sec",
             "fp64_time_sec", "backtransform_time_sec")
    assert all(np.isfinite(info[p]) and info[p] >= 0 for p in parts)
    assert abs(sum(info[p] for p in parts) - info["total_time_sec"]) <= 1e-9
    # the values: Ritz values of the TF32 block, against the oracle's and LAPACK's
    assert np.abs(v - vo).max() <= 1e-10 * hn, np.abs(v - vo).max() / hn
    w, _ = oracle.dsyevd_lowest(H, k)
    assert np.abs(np.sort(v) - w).max() <= 1e-10 * hn
    # the vectors: the Householder column signs, then the entries
    np.testing.assert_array_equal(np.sign(np.diag(V[:k, :k])), np.sign(np.diag(Vo[:k, :k])))
    assert np.abs(V - Vo).max() <= 5e-3 * np.abs(Vo).max(), np.abs(V - Vo).max()
    # Q Z with Z_jj = 1 and Q orthonormal: every column has norm >= 1
    assert (np.linalg.norm(V, axis=0) >= 1.0 - 1e-12).all()
    return np.abs(v - vo).max() / hn


@pytest.mark.parametrize("k", [1, 5, 16, 32])
def test_reference_dense_cases(cuda, k):
    """The reference's n = 96 symmetric test matrix (runtests.cu:46-80)."""
    H = oracle.perturbative_matrix(96, 1)
    V, v, info = run(cuda, H, k)
    check(H, k, V, v, info)


def test_headline_construction_n2048(cuda):
    """The dense mixed-precision construction (d_i = i/8 + U(0,0.1),
    h_ij ~ N(0, 0.02^2) exp(-|i-j|/256)) at n = 2048, k = 32."""
    H, _ = workloads.dense_config1(2048, seed=0)
    V, v, info = run(cuda, H, 32)
    check(H, 32, V, v, info)


def test_k_equals_n(cuda):
    """Full spectrum of a small matrix (the reference's sweeps use k = n): the
    last Householder column is not reflected."""
    H = oracle.perturbative_matrix(32, 1)
    V, v, info = run(cuda, H, 32)
    check(H, 32, V, v, info)


def test_invalid_arguments(cuda):
    torch = cuda
    lib = _lib.load()
    h = C.c_void_p(torch.cuda.current_blas_handle())
    dH = torch.eye(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dH.data_ptr())
    res = _lib.IPTRayleighMixedCudaDeviceResult()
    f = lib.ipt_rayleigh_mixed_tf32_cuda_device_tol
    assert f(None, 8, 2, 1e-6, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 9, 1e-6, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 0, 1e-6, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 2, 0.0, 5, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, -1.0, 5, h, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 0, 1e-12, 5, h, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, 1e-12, 0, h, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, 1e-12, 5, None, C.byref(res)) == 1
    assert f(p, 8, 2, 1e-6, 5, 1e-12, 5, h, None) == 1
    assert not res.d_vectors and not res.d_values and np.isnan(res.total_time_sec)
