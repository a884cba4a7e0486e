"""The ACX oracle (a restatement of IPT_C_GPU/src/ACX/acx_cuda.cu, whose
reference has no CPU code to run against) tied to the pinned plain-IPT
oracle: both iterate the same map F from the identity, so ACX must land on
the plain iteration's fixed point, in fewer map evaluations."""
import numpy as np
import pytest

from oracle import oracle


@pytest.mark.parametrize("n,k,eps", [(64, 4, 0.06), (96, 96, 0.06), (120, 10, 0.2)])
def test_acx_fixed_point_is_the_plain_ipt_fixed_point(n, k, eps):
    H = oracle.acx_test_matrix(n, eps, seed=n)
    X, v, info, st = oracle.acx_dense(H, k, 1e-12, 200)
    assert st == 0 and info["converged"] == 1
    Xp, vp, iters, _ = oracle.ipt_dense(H, k, 2000, tol=1e-13, use_tol=True)
    assert np.abs(X - Xp).max() <= 1e-10
    assert np.abs(v - vp).max() <= 1e-10 * np.abs(H).sum(1).max()
    assert info["f_calls"] < iters


def test_acx_oracle_status_codes():
    H = oracle.acx_test_matrix(32, 0.06, seed=2)
    assert oracle.acx_dense(H, 0, 1e-12, 10)[3] == 1
    assert oracle.acx_dense(H, 4, 0.0, 10)[3] == 1
    H[7, 7] = H[3, 3]
    assert oracle.acx_dense(H, 4, 1e-12, 10)[3] == 5


def test_mixed_acx_oracle_reaches_the_fp64_fixed_point():
    H = oracle.acx_test_matrix(96, 0.06, seed=5)
    X, v, info, st = oracle.acx_mixed(H, 8, 1e-5, 100, 1e-12, 100)
    Xp, vp, ip, sp = oracle.acx_dense(H, 8, 1e-12, 100)
    assert st == 0 == sp and info["fp64_converged"] == 1 and info["tf32_converged"] == 1
    assert np.abs(X - Xp).max() <= 1e-11
    assert info["fp64_f_calls"] < ip["f_calls"]
    assert oracle.acx_mixed(H, 8, 0.0, 100, 1e-12, 100)[3] == 1
