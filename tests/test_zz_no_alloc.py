"""The allocation-free FP64 dense solve (ipt_cuda_device_tol_noalloc).

Callers that cannot let a library allocate device memory (their own memory
pool, no allocation after start-up, pipelines that cudaFree's device-wide
synchronisation would stall) use this entry point: they pass H and the
output buffers, and the library works in one static 16 MiB device array.
The test runs it twice in a row on different problems, so the second call
sees the scratch the first one left behind, and checks each result against
the allocating entry point ipt_cuda_device_tol through the C ABI.  It is
collected last and passes alone in a fresh process or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, workloads
from oracle import oracle
from tests.conftest import device_to_host

pytestmark = pytest.mark.gpu

VEC_TOL = 1e-12
VAL_TOL = 1e-11


def _allocating(torch, lib, dH, n, k, tol, maxiter):
    dvec = C.c_void_p()
    dval = C.c_void_p()
    it = C.c_int()
    fp = C.c_double()
    st = lib.ipt_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, tol, maxiter,
                                 C.c_void_p(torch.cuda.current_blas_handle()), C.byref(dvec),
                                 C.byref(dval), C.byref(it), C.byref(fp))
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    X = device_to_host(dvec, np.zeros((n, k), order="F"))
    v = device_to_host(dval, np.zeros(k))
    lib.ipt_cuda_free_device_result(dvec, dval)
    return X, v, it.value, fp.value


def _noalloc(torch, lib, dH, n, k, tol, maxiter):
    dX = torch.full((k, n), float("nan"), dtype=torch.float64, device="cuda")
    dv = torch.full((k,), float("nan"), dtype=torch.float64, device="cuda")
    it = C.c_int()
    fp = C.c_double()
    st = lib.ipt_cuda_device_tol_noalloc(C.c_void_p(dH.data_ptr()), n, k, tol, maxiter,
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                         C.c_void_p(dX.data_ptr()), C.c_void_p(dv.data_ptr()),
                                         C.byref(it), C.byref(fp))
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    return dX.T.cpu().numpy(), dv.cpu().numpy(), it.value, fp.value


def test_noalloc_matches_allocating_entry_twice(cuda):
    torch = cuda
    lib = _lib.load()
    H1 = oracle.perturbative_matrix(96, 1)
    H2, _ = workloads.dense_config0(1024, seed=5)
    for H, k, tol in [(H1, 16, 1e-12), (H2, 8, 1e-13)]:
        n = H.shape[0]
        dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()
        Xa, va, ita, fpa = _allocating(torch, lib, dH, n, k, tol, 400)
        Xb, vb, itb, fpb = _noalloc(torch, lib, dH, n, k, tol, 400)
        assert itb == ita
        assert fpb <= tol
        assert np.abs(Xb - Xa).max() <= VEC_TOL
        assert np.abs(vb - va).max() <= VAL_TOL


def test_noalloc_rejects_sizes_beyond_the_scratch(cuda):
    torch = cuda
    lib = _lib.load()
    n, k = 4096, 512  # n*k = 2.1e6 > the ~1.0e6 limit
    it = C.c_int()
    fp = C.c_double()
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    st = lib.ipt_cuda_device_tol_noalloc(p, n, k, 1e-10, 10, None, p, p, C.byref(it),
                                         C.byref(fp))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
    assert it.value == 0
