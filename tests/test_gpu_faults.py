"""Failure paths through the C ABI, with faults made on the host (no GPU
fault, trap or hang): non-finite entries and zero gaps in H, broken CSC
arrays, and a tensor-core pipeline wait that is told to give up.

Status codes are the reference's (IPT_C_GPU/src/ipt_cuda.cu:82-90): 1 =
invalid argument, 3 = CUDA runtime error.  A tolerance-mode IPT whose iterate
stops being finite ends with "invalid argument" (ipt_cuda.cu:1676-1679), in
fixed-iteration mode the non-finite block is returned (no check); the oracle
restatement does the same (status -2)."""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, api, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def with_nonfinite(H, value, i=7, j=3):
    H = H.copy()
    H[i, j] = value
    H[j, i] = value
    return H


@pytest.mark.parametrize("value", [np.nan, np.inf])
def test_nonfinite_entry_tolerance_mode(cuda, value):
    H = with_nonfinite(oracle.perturbative_matrix(96, 1), value)
    with pytest.raises(_lib.IPTError) as exc:
        api.ipt_cuda_tol(H, 8, 1e-12, 50)
    assert exc.value.status == 1
    with pytest.raises(RuntimeError):
        oracle.ipt_dense(H, 8, 50, tol=1e-12, use_tol=True)


def test_nonfinite_entry_fixed_iterations_returns_the_block(cuda):
    H = with_nonfinite(oracle.perturbative_matrix(96, 1), np.nan)
    X, v, info = api.ipt_cuda(H, 8, 5)
    Xo, vo, _, _ = oracle.ipt_dense(H, 8, 5)
    assert info["iterations"] == 5
    np.testing.assert_array_equal(np.isfinite(X), np.isfinite(Xo))
    np.testing.assert_array_equal(np.isfinite(v), np.isfinite(vo))


def test_zero_gap_tolerance_mode(cuda):
    """Two equal diagonal entries among the targets: G has a 1/0, the iterate
    stops being finite and the tolerance loop reports invalid argument."""
    H = oracle.perturbative_matrix(96, 1)
    H[4, 4] = H[2, 2]
    with pytest.raises(_lib.IPTError) as exc:
        api.ipt_cuda_tol(H, 8, 1e-12, 50)
    assert exc.value.status == 1
    with pytest.raises(RuntimeError):
        oracle.ipt_dense(H, 8, 50, tol=1e-12, use_tol=True)


def test_sparse_nonfinite_value(cuda):
    cp, ri, va = oracle.banded_csc(64)
    va = va.copy()
    va[len(va) // 2] = np.nan
    with pytest.raises(_lib.IPTError) as exc:
        api.ipt_cuda_sparse_csc_tol(cp, ri, va, 64, 5, 1e-12, 200)
    assert exc.value.status == 1


@pytest.mark.parametrize("kind", ["decreasing_col_ptr", "row_out_of_range", "negative_row",
                                  "nnz_mismatch", "k_gt_n"])
def test_broken_csc_is_rejected(cuda, kind):
    """The reference's CSC validation (IPT_C_GPU/src/ipt_preparation.cu:148-169)
    and argument checks (ipt_cuda.cu:1816-1828): invalid argument, nothing
    computed."""
    cp, ri, va = oracle.banded_csc(64)
    cp, ri, va = cp.copy(), ri.copy(), va.copy()
    n, k = 64, 5
    if kind == "decreasing_col_ptr":
        cp[10] = cp[12] + 1
    elif kind == "row_out_of_range":
        ri[5] = 64
    elif kind == "negative_row":
        ri[5] = -1
    elif kind == "nnz_mismatch":
        cp[-1] = cp[-1] - 1
    else:
        k = 65
    with pytest.raises(_lib.IPTError) as exc:
        api.ipt_cuda_sparse_csc_tol(cp, ri, va, n, k, 1e-12, 200)
    assert exc.value.status == 1


def test_block_solver_nonfinite_matrix_does_not_converge(cuda):
    """The mixed block solve on an H with a NaN: no pair is reported
    converged (or the call fails); the process and the context stay usable."""
    H, _ = workloads.dense_config0(512, seed=3)
    Hn = with_nonfinite(H, np.nan, 100, 7)
    try:
        _, _, rep = api.block_solve_dense(Hn, 8, "fp16")
        assert rep["converged"] == 0
    except _lib.IPTError as exc:
        assert exc.status in (1, 3)
    X, v, rep = api.block_solve_dense(H, 8, "fp16")
    w, _ = oracle.eigh_lowest(H, 8)
    assert rep["converged"] == 1
    assert np.abs(v - w).max() <= 1e-10 * np.abs(H).sum(1).max()


def run_mixed_fp16(torch, H, k):
    lib = _lib.load()
    n = H.shape[0]
    dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()
    res = _lib._MixedResult()
    st = lib.ipt_mixed_precision_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, 1e-4, 50,
                                                 1e-12, 100,
                                                 C.c_void_p(torch.cuda.current_blas_handle()),
                                                 C.byref(res))
    torch.cuda.synchronize()
    lib.ipt_mixed_precision_cuda_free_device_result(C.byref(res))
    return st


def test_tensor_core_wait_limit_gives_error_status(cuda, monkeypatch):
    """The tensor-core product's pipeline waits give up after a single poll
    (IPT_GB300_SPIN_LIMIT=1): the kernel sets its error flag, waits with the
    full bound for its own MMAs and copies, releases TMEM and returns; the
    mixed entry reports the CUDA-error status, and the next call on the same
    context succeeds."""
    torch = cuda
    H, _ = workloads.dense_config0(2048, seed=5)
    monkeypatch.setenv("IPT_GB300_SPIN_LIMIT", "1")
    assert run_mixed_fp16(torch, H, 16) == 3
    monkeypatch.delenv("IPT_GB300_SPIN_LIMIT")
    assert run_mixed_fp16(torch, H, 16) == 0
    X, v, rep = api.block_solve_dense(H, 16, "fp16")
    assert rep["converged"] == 1
