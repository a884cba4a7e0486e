"""GPU parity of the tensor-core (tcgen05/TMA) low-precision IPT stage and of
the mixed-precision solvers, through the C ABI.

Tolerances: a low-precision IPT iterate differs from the FP64 iterate by the
operand rounding (FP16 2^-11, BF16 2^-8, TF32 2^-11 relative per entry), so
after a few iterations max|X_lp - X_64| <= 5e-3 (FP16/TF32) and 3e-2 (BF16)
times max|X|.  After FP64 refinement / Davidson the results meet the FP64
bars: 1e-9 on refined IPT vectors, |dlambda| <= 1e-10 ||H||, scaled residual
<= 1e-8.
"""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, api, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu

KINDS = {"fp16": ("ipt_mixed_precision_cuda_device_tol", 5e-3),
         "fp32": ("ipt_mixed_precision_fp32_cuda_device_tol", 1e-5),
         "tf32": ("ipt_mixed_precision_tf32_cuda_device_tol", 5e-3)}
FREE = {"fp16": "ipt_mixed_precision_cuda_free_device_result",
        "fp32": "ipt_mixed_precision_fp32_cuda_free_device_result",
        "tf32": "ipt_mixed_precision_tf32_cuda_free_device_result"}


def run_mixed(torch, H, k, kind, lp_tol, lp_maxiter, fp64_tol, fp64_maxiter):
    from tests.conftest import device_to_host
    lib = _lib.load()
    n = H.shape[0]
    dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()
    res = _lib._MixedResult()
    fn = getattr(lib, KINDS[kind][0])
    st = fn(C.c_void_p(dH.data_ptr()), n, k, lp_tol, lp_maxiter, fp64_tol, fp64_maxiter,
            C.c_void_p(torch.cuda.current_blas_handle()), C.byref(res))
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    X = np.zeros((n, k), order="F")
    v = np.zeros(k)
    device_to_host(C.c_void_p(res.d_vectors), X)
    device_to_host(C.c_void_p(res.d_values), v)
    info = {"lowp_iterations": res.lowp_iterations, "fp64_iterations": res.fp64_iterations,
            "lowp_fpres": res.lowp_fixed_point_residual, "fp64_fpres": res.fp64_fixed_point_residual,
            "lowp_time": res.lowp_time_sec, "fp64_time": res.fp64_time_sec}
    getattr(lib, FREE[kind])(C.byref(res))
    assert not res.d_vectors
    return X, v, info


@pytest.mark.parametrize("kind", ["fp16", "tf32", "fp32"])
@pytest.mark.parametrize("n,k", [(256, 8), (1000, 5), (777, 40)])
def test_lowp_iterates_track_fp64(cuda, kind, n, k):
    """m low-precision steps + one FP64 step vs m+1 FP64 steps."""
    H, _ = workloads.dense_config0(n, seed=11, sigma=0.05)
    m = 4
    X, v, info = run_mixed(cuda, H, k, kind, 1e-300, m, 1e300, 1)
    assert info["lowp_iterations"] == m and info["fp64_iterations"] == 1
    Xo, vo, _, _ = oracle.ipt_dense(H, k, m + 1)
    tol = KINDS[kind][1]
    err = np.abs(X - Xo).max() / np.abs(Xo).max()
    assert err <= tol, err


@pytest.mark.parametrize("kind", ["fp16", "tf32"])
@pytest.mark.parametrize("n,k", [(300, 8), (777, 40), (2048, 33), (4100, 16)])
def test_stream_and_split_schedules(cuda, monkeypatch, kind, n, k):
    """The persistent stream-K product with two CTAs per SM (default) or one
    (IPT_GB300_TC_STREAMK=1) and the split-K grid (=0) all track the FP64
    iterates; the stream-K result is the same bits on a second run (fixed
    slot order)."""
    H, _ = workloads.dense_config0(n, seed=5, sigma=0.05)
    m = 4
    Xo, _, _, _ = oracle.ipt_dense(H, k, m + 1)
    tol = KINDS[kind][1]
    got = {}
    for mode in ("2", "1", "0"):
        monkeypatch.setenv("IPT_GB300_TC_STREAMK", mode)
        X, v, info = run_mixed(cuda, H, k, kind, 1e-300, m, 1e300, 1)
        assert info["lowp_iterations"] == m
        err = np.abs(X - Xo).max() / np.abs(Xo).max()
        assert err <= tol, (mode, err)
        got[mode] = X
    monkeypatch.setenv("IPT_GB300_TC_STREAMK", "2")
    X2, _, _ = run_mixed(cuda, H, k, kind, 1e-300, m, 1e300, 1)
    assert np.array_equal(X2, got["2"])



@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("n", [700, 2085, 6200])
def test_symmetric_product_solve(cuda, monkeypatch, prec, n):
    """The block solver's symmetric product (Delta's upper 128 x 128 tiles,
    each used as A and, through an MN-major descriptor, as A^T; enabled with
    IPT_GB300_TC_SYM=2) gives the certified eigenpairs of the stream-K
    product, the same bits on a second run, and about the same IPT
    iteration count."""
    H, _ = workloads.dense_config1(n, seed=31)
    k = 24
    monkeypatch.setenv("IPT_GB300_TC_SYM", "0")
    X0, v0, r0 = api.block_solve_dense(H, k, prec)
    monkeypatch.setenv("IPT_GB300_TC_SYM", "2")
    X1, v1, r1 = api.block_solve_dense(H, k, prec)
    X2, v2, r2 = api.block_solve_dense(H, k, prec)
    assert r0["converged"] == 1 and r1["converged"] == 1
    check_pairs(H, X1, v1, k)
    hn = np.abs(H).sum(axis=1).max()
    assert np.abs(v1 - v0).max() <= 1e-10 * hn
    assert np.array_equal(X1, X2) and np.array_equal(v1, v2)
    assert abs(r1["ipt_iterations"] - r0["ipt_iterations"]) <= 8


@pytest.mark.parametrize("kind", ["fp16", "tf32", "fp32"])
def test_mixed_converges_to_fp64_fixed_point(cuda, kind):
    H = oracle.perturbative_matrix(96, 1)
    X, v, info = run_mixed(cuda, H, 16, kind, 1e-3, 100, 1e-12, 300)
    Xo, vo, _, _ = oracle.ipt_dense(H, 16, 300, tol=1e-12, use_tol=True)
    assert info["fp64_fpres"] <= 1e-12
    assert np.abs(X - Xo).max() <= 1e-9
    assert np.abs(v - vo).max() <= 1e-9
    assert oracle.max_relative_residual(H, X, v) <= 5e-9


def test_mixed_invalid_arguments(cuda):
    torch = cuda
    lib = _lib.load()
    res = _lib._MixedResult()
    h = C.c_void_p(torch.cuda.current_blas_handle())
    assert lib.ipt_mixed_precision_cuda_device_tol(None, 8, 2, 1e-3, 5, 1e-9, 5, h,
                                                   C.byref(res)) == 1
    dH = torch.zeros(8, 8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dH.data_ptr())
    assert lib.ipt_mixed_precision_tf32_cuda_device_tol(p, 8, 9, 1e-3, 5, 1e-9, 5, h,
                                                        C.byref(res)) == 1
    assert lib.ipt_mixed_precision_fp32_cuda_device_tol(p, 8, 2, 0.0, 5, 1e-9, 5, h,
                                                        C.byref(res)) == 1
    assert not res.d_vectors


def check_pairs(H, X, v, k):
    hn = np.abs(H).sum(axis=1).max()
    w, _ = oracle.eigh_lowest(H, k)
    assert np.abs(v - w).max() <= 1e-10 * hn, np.abs(v - w).max() / hn
    r = np.linalg.norm(H @ X - X * v[None, :], axis=0) / max(1.0, hn)
    assert r.max() <= 1e-8, r.max()


@pytest.mark.parametrize("prec", ["fp16", "bf16", "tf32"])
@pytest.mark.parametrize("n", [2048, 3000])
def test_anderson_mixing_saves_low_precision_steps(cuda, monkeypatch, prec, n):
    """The refinement's Anderson-mixed low-precision iterations reach the
    plain map's eigenpairs (LAPACK's, to 1e-10 ||H||) in fewer low-precision
    products, with no more FP64-accurate ones.  n = 3000 is not a multiple of
    1024: its inner products come from a kernel of their own."""
    H, _ = workloads.dense_config1(n, seed=21)
    runs = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("IPT_GB300_ANDERSON", mode)
        X, v, rep = api.block_solve_dense(H, 32, prec, ipt_maxiter=60, ipt_check_every=8)
        assert rep["converged"] == 1
        check_pairs(H, X, v, 32)
        runs[mode] = rep
    assert runs["1"]["lowp_matvecs"] < runs["0"]["lowp_matvecs"], runs
    assert runs["1"]["fp64_matvecs"] <= runs["0"]["fp64_matvecs"], runs


@pytest.mark.parametrize("strategy", [0, 1])
@pytest.mark.parametrize("prec", ["fp16", "bf16", "tf32"])
def test_block_mixed_config1_shape_small(cuda, prec, strategy):
    H, _ = workloads.dense_config1(2048, seed=4)
    X, v, rep = api.block_solve_dense(H, 32, prec, ipt_maxiter=60, ipt_check_every=4,
                                      strategy=strategy)
    assert rep["converged"] == 1
    assert rep["lowp_matvecs"] > 0
    check_pairs(H, X, v, 32)


def test_block_mixed_config1_full(cuda):
    """The n = 8192, k = 32 workload: FP16 tensor-core IPT + FP64 recovery."""
    H, _ = workloads.dense_config1(8192, seed=0)
    X, v, rep = api.block_solve_dense(H, 32, "fp16", ipt_maxiter=80, ipt_check_every=8)
    assert rep["converged"] == 1
    check_pairs(H, X, v, 32)
    # the refinement needs only a few FP64 block products
    assert rep["fp64_matvecs"] <= 4 * 32


def test_mixed_refine_uses_fewer_fp64_products_than_plain(cuda):
    H, _ = workloads.dense_config1(2048, seed=9)
    _, _, rep_mixed = api.block_solve_dense(H, 16, "fp16", ipt_maxiter=60, ipt_check_every=4)
    _, _, rep_plain = api.block_solve_dense(H, 16, "fp64")
    assert rep_mixed["converged"] == 1 and rep_plain["converged"] == 1
    assert rep_mixed["fp64_matvecs"] * 3 <= rep_plain["fp64_matvecs"]


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_device_stop_matches_host_checks(cuda, monkeypatch, prec):
    """The device-side stop (per-step norm history; the steps after the one
    that meets the tolerance pass the block through) gives the same pairs as
    host checks every few steps, and its IPT stage stops no later.  (Stopping
    exactly at the tolerance can cost the refinement an extra step, so the
    total count of low-precision products is not compared.)"""
    H, _ = workloads.dense_config1(2048, seed=12)
    runs = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("IPT_GB300_DEVICE_STOP", mode)
        X, v, rep = api.block_solve_dense(H, 16, prec, ipt_maxiter=60, ipt_check_every=8)
        assert rep["converged"] == 1
        check_pairs(H, X, v, 16)
        runs[mode] = rep
    assert runs["1"]["ipt_iterations"] <= runs["0"]["ipt_iterations"]


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_host_entry_pinned_matches_pageable(cuda, prec):
    """ipt_block_solve_dense on pinned host memory reads H over the host link
    inside its first (fused) pass; on pageable memory it copies H first.  Both
    run the same kernels on the same numbers: identical results."""
    import ctypes as C
    from block_ipt_gb300 import _lib
    torch = cuda
    n, k = 1536, 12
    H, _ = workloads.dense_config1(n, seed=21)
    H = np.asfortranarray(H)
    X1, v1, r1 = api.block_solve_dense(H, k, prec)
    pinned = torch.from_numpy(H.T.copy()).pin_memory()  # row-major H^T = column-major H
    opt = api.block_options(prec)
    X2 = np.zeros((n, k), order="F")
    v2 = np.zeros(k)
    rep = _lib.IPTBlockReport()
    st = _lib.load().ipt_block_solve_dense(C.c_void_p(pinned.data_ptr()), n, k, C.byref(opt),
                                           C.c_void_p(X2.ctypes.data), C.c_void_p(v2.ctypes.data),
                                           C.byref(rep))
    assert st == 0
    assert r1["converged"] == 1 and rep.converged == 1
    assert np.array_equal(v1, v2)
    assert np.array_equal(X1, X2)
    check_pairs(H, X2, v2, k)


@pytest.mark.parametrize("n", [1000, 2085])
def test_host_entry_pinned_reads_only_the_upper_triangle(cuda, n):
    """From pinned host memory the mixed solve moves only the upper triangle
    of H across the host link (column chunks mirrored on the device): with
    NaN in every entry below the diagonal of the host copy it returns the
    same bits as the solve of the symmetric matrix from pageable memory."""
    import ctypes as C
    from block_ipt_gb300 import _lib
    torch = cuda
    k = 12
    H, _ = workloads.dense_config1(n, seed=23)
    H = np.asfortranarray(H)
    X1, v1, r1 = api.block_solve_dense(H, k, "fp16")
    Hu = H.copy(order="F")
    Hu[np.tril_indices(n, -1)] = np.nan
    pinned = torch.from_numpy(Hu.T.copy()).pin_memory()  # row-major H^T = column-major H
    opt = api.block_options("fp16")
    X2 = np.zeros((n, k), order="F")
    v2 = np.zeros(k)
    rep = _lib.IPTBlockReport()
    st = _lib.load().ipt_block_solve_dense(C.c_void_p(pinned.data_ptr()), n, k, C.byref(opt),
                                           C.c_void_p(X2.ctypes.data), C.c_void_p(v2.ctypes.data),
                                           C.byref(rep))
    assert st == 0 and rep.converged == 1 and r1["converged"] == 1
    assert np.array_equal(v1, v2)
    assert np.array_equal(X1, X2)
    check_pairs(H, X2, v2, k)


def test_fused_setup_matches_two_pass(cuda, monkeypatch):
    """The fused setup pass (per-row FP16 scales) and the two-pass setup (one
    global scale) reach the same certified eigenpairs."""
    H, _ = workloads.dense_config1(2048, seed=22)
    monkeypatch.setenv("IPT_GB300_FUSED_SETUP", "1")
    X1, v1, r1 = api.block_solve_dense(H, 16, "fp16")
    monkeypatch.setenv("IPT_GB300_FUSED_SETUP", "0")
    X2, v2, r2 = api.block_solve_dense(H, 16, "fp16")
    assert r1["converged"] == 1 and r2["converged"] == 1
    check_pairs(H, X1, v1, 16)
    check_pairs(H, X2, v2, 16)
    hn = np.abs(H).sum(axis=1).max()
    assert np.abs(v1 - v2).max() <= 1e-10 * hn
    assert abs(r1["matrix_norm_inf"] - hn) <= 1e-12 * hn
