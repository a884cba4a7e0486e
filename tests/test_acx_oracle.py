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


def published():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "acx_published.json")
    with open(path) as f:
        return json.load(f)


def test_acx_oracle_reproduces_the_published_smoke_run():
    """Parity pin: on the matrix of the reference's ACX sweep (regenerated
    bit for bit, N = 64, eps = 0.06, k = n), the oracle's ACX takes the
    reference's iterations and map evaluations, and its plain IPT the
    reference's iterations; the fixed-point residuals agree to the rounding
    of the different summation orders (results/ACX/smoke_fcalls)."""
    case = published()["cases"][0]
    assert case["n"] == 64
    H = oracle.acx_sweep_matrix(case["n"], case["epsilon"])
    X, v, info, st = oracle.acx_dense(H, case["n"], case["tol"], case["maxiter"])
    assert st == 0 and info["converged"] == 1
    assert info["iterations"] == case["acx"]["iterations"]
    assert info["f_calls"] == case["acx"]["f_calls"]
    assert abs(info["fixed_point_residual"] / case["acx"]["fixed_point_residual"] - 1) < 0.01
    assert abs(info["max_residual"] / case["acx"]["max_apply_residual"] - 1) < 0.01
    Xp, vp, it, fp = oracle.ipt_dense(H, case["n"], case["maxiter"], tol=case["tol"],
                                      use_tol=True)
    assert it == case["ipt"]["iterations"]
    assert abs(fp / case["ipt"]["fixed_point_residual"] - 1) < 0.01


def test_acx_sweep_matrix_matches_the_reference_generator():
    """Spot values of the regenerated sweep matrix from the reference's hash
    (benchmark_acx_cuda_sweep.cu:256-313), computed with Python integers."""
    import struct
    M = (1 << 64) - 1

    def sm(x):
        x = (x + 0x9E3779B97F4A7C15) & M
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M
        return x ^ (x >> 31)

    n, eps = 100, 0.08
    seed = 20260615 + n + sm(struct.unpack("<Q", struct.pack("<d", eps))[0]) % 1000000007

    def u(r, c):
        x = (seed + n * 0xD1B54A32D192ED03) & M
        x ^= ((r + 1) * 0x9E3779B97F4A7C15) & M
        x ^= ((c + 1) * 0xBF58476D1CE4E5B9) & M
        return (sm(x) >> 11) * (1.0 / 9007199254740992.0)

    H = oracle.acx_sweep_matrix(n, eps)
    for r, c in [(0, 0), (3, 17), (99, 0), (42, 42), (7, 93)]:
        want = (r + 1) + eps * u(r, r) if r == c else 0.5 * eps * (u(r, c) + u(c, r))
        assert H[r, c] == want and H[c, r] == want
