"""The CPU oracle pinned against the reference's own outputs (no GPU)."""
import numpy as np
import pytest

from oracle import oracle


def test_dense_generator_matches_reference(golden):
    arrays, meta = golden
    for case in meta["dense"]:
        H = oracle.perturbative_matrix(case["n"], case["symmetric"])
        assert H.sum() == case["matrix_sum"]
        assert (H * H).sum() == case["matrix_sumsq"]
        np.testing.assert_array_equal(H.ravel(order="F")[::7], arrays["dense_%s_sample" % case["name"]])


def test_dense_ipt_bit_exact_vs_reference(golden):
    arrays, meta = golden
    for case in meta["dense"]:
        H = oracle.perturbative_matrix(case["n"], case["symmetric"])
        X, v, it, _ = oracle.ipt_dense(H, case["k"], case["iterations"])
        assert it == case["iterations"]
        np.testing.assert_array_equal(X, arrays["dense_%s_vectors" % case["name"]])
        np.testing.assert_array_equal(v, arrays["dense_%s_values" % case["name"]])


def test_dense_reference_cases_converge(golden):
    """The reference's acceptance rule (runtests.cu:233-234): residual <= 5e-9."""
    arrays, meta = golden
    for case in meta["dense"]:
        H = oracle.perturbative_matrix(case["n"], case["symmetric"])
        X = arrays["dense_%s_vectors" % case["name"]]
        v = arrays["dense_%s_values" % case["name"]]
        assert oracle.max_relative_residual(H, X, v) <= 5e-9


def test_banded_csc_matches_reference(golden):
    arrays, _ = golden
    cp, ri, va = oracle.banded_csc(64)
    np.testing.assert_array_equal(cp, arrays["sparse_synthetic_banded_k5_col_ptr"])
    np.testing.assert_array_equal(ri, arrays["sparse_synthetic_banded_k5_row_ind"])
    np.testing.assert_array_equal(va, arrays["sparse_synthetic_banded_k5_values_csc"])


def test_sparse_ipt_vs_reference(golden):
    arrays, meta = golden
    for case in meta["sparse"]:
        name = case["name"]
        cp = arrays["sparse_%s_col_ptr" % name]
        ri = arrays["sparse_%s_row_ind" % name]
        va = arrays["sparse_%s_values_csc" % name]
        H = oracle.csc_to_dense(cp, ri, va, case["n"])
        X, v, _, _ = oracle.ipt_dense(H, case["k"], case["iterations"])
        np.testing.assert_array_equal(X, arrays["sparse_%s_vectors" % name])
        np.testing.assert_array_equal(v, arrays["sparse_%s_values" % name])


def test_sparse_preparation_vs_reference(golden):
    """Sorted CSR from the oracle == the reference preparation (as CSR)."""
    arrays, meta = golden
    for case in meta["sparse"]:
        name = case["name"]
        n = case["n"]
        cp = arrays["sparse_%s_col_ptr" % name]
        ri = arrays["sparse_%s_row_ind" % name]
        va = arrays["sparse_%s_values_csc" % name]
        rp, ci, vv, d, perm = oracle.prepare_sorted_csc(cp, ri, va, n)
        np.testing.assert_array_equal(perm, arrays["sparse_%s_prep_perm" % name])
        np.testing.assert_array_equal(d, arrays["sparse_%s_prep_diag" % name])
        Hr = oracle.csc_to_dense(arrays["sparse_%s_prep_col_ptr" % name],
                                 arrays["sparse_%s_prep_row_ind" % name],
                                 arrays["sparse_%s_prep_values" % name], n)
        Ho = np.zeros((n, n))
        for r in range(n):
            for p in range(rp[r], rp[r + 1]):
                Ho[r, ci[p]] += vv[p]
        np.testing.assert_array_equal(Ho, Hr)


def test_csr_ipt_matches_dense_ipt():
    cp, ri, va = oracle.banded_csc(64)
    rp, ci, vv, d, _ = oracle.prepare_sorted_csc(cp, ri, va, 64)
    X1, v1, _, _ = oracle.ipt_csr(rp, ci, vv, d, 64, 5, 80)
    X2, v2, _, _ = oracle.ipt_dense(oracle.csc_to_dense(cp, ri, va, 64), 5, 80)
    np.testing.assert_allclose(X1, X2, atol=1e-15)
    np.testing.assert_allclose(v1, v2, rtol=1e-14)


def test_tol_mode_semantics():
    """Tolerance mode returns F(X) of the step that met the tolerance."""
    H = oracle.perturbative_matrix(96, 1)
    X, v, it, fp = oracle.ipt_dense(H, 16, 500, tol=1e-12, use_tol=True)
    assert fp <= 1e-12
    X_fixed, v_fixed, _, _ = oracle.ipt_dense(H, 16, it)
    np.testing.assert_array_equal(X, X_fixed)
    np.testing.assert_array_equal(v, v_fixed)


def test_oracle_matches_reference_library_directly():
    """Extra sizes against the reference's compiled CPU function, where built."""
    if not oracle.ref_available():
        pytest.skip("reference tree not present on this host")
    import ctypes as C
    L = oracle.ref_lib("dense")
    for n, k, it in [(17, 3, 7), (64, 64, 12), (128, 9, 25)]:
        H = oracle.perturbative_matrix(n, 1)
        Xr = np.zeros((n, k), order="F")
        vr = np.zeros(k)
        assert L.ref_ipt_cpu_reference(C.c_void_p(H.ctypes.data), n, k, it,
                                       C.c_void_p(Xr.ctypes.data), C.c_void_p(vr.ctypes.data)) == 0
        X, v, _, _ = oracle.ipt_dense(H, k, it)
        np.testing.assert_array_equal(X, Xr)
        np.testing.assert_array_equal(v, vr)


def test_eigen_oracle_agrees_with_dsyevd():
    H = oracle.perturbative_matrix(96, 1)
    w1, _ = oracle.eigh_lowest(H, 8)
    w2, _ = oracle.dsyevd_lowest(H, 8)
    np.testing.assert_allclose(w1, w2, atol=1e-12)
