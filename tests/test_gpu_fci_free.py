"""Matrix-free FCI-like sigma and Davidson (k_fci.cu) through the C ABI,
against the CPU restatement (oracle/fci_oracle.c): the diagonal bit for
bit, the FP64 sigma to FP64 rounding (the elements are bit-identical, only
the summation order differs), the FP32 / BF16 sigmas to their operand
rounding, and the eigenpairs against the CSR solver on the oracle's CSR and
against LAPACK."""
import numpy as np
import pytest
from scipy.sparse import csr_matrix

from block_ipt_gb300 import api
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_diagonal_bit_exact(cuda):
    torch = cuda
    spec = api.fci_spec(8, 4, 4, seed=3)
    n = api.fci_dimension(spec)
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    api.fci_diagonal(spec, d.data_ptr())
    ref = oracle.fci_matrix(8, 4, 4, seed=3, csr=False)
    assert np.array_equal(d.cpu().numpy(), ref)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 2e-6), ("bf16", 1e-2)])
@pytest.mark.parametrize("k", [5, 12])
def test_sigma_matches_oracle(cuda, prec, tol, k):
    torch = cuda
    spec = api.fci_spec(8, 4, 4, seed=1)
    n = api.fci_dimension(spec)
    X = np.random.default_rng(k).standard_normal((n, k))
    dX = torch.from_numpy(X.T.copy()).cuda()  # column-major n x k
    dY = torch.empty((k, n), dtype=torch.float64, device="cuda")
    api.fci_sigma(spec, dX.data_ptr(), k, dY.data_ptr(), prec)
    Y = dY.T.cpu().numpy()
    ref = oracle.fci_sigma(8, 4, 4, X, seed=1)
    assert np.abs(Y - ref).max() <= tol * np.abs(ref).max()


def solve(torch, spec, k, prec, **kw):
    n = api.fci_dimension(spec)
    dX = torch.empty((k, n), dtype=torch.float64, device="cuda")
    dv = torch.empty(k, dtype=torch.float64, device="cuda")
    rep = api.block_solve_fci(spec, k, dX.data_ptr(), dv.data_ptr(), prec, **kw)
    return dX.T.cpu().numpy(), dv.cpu().numpy(), rep


@pytest.mark.parametrize("prec", ["fp64", "bf16", "fp32"])
def test_small_solve_vs_lapack(cuda, prec):
    torch = cuda
    rp, ci, va, d = oracle.fci_matrix(6, 3, 3, seed=2)
    H = csr_matrix((va, ci, rp), shape=(len(d), len(d))).toarray()
    spec = api.fci_spec(6, 3, 3, seed=2)
    X, v, rep = solve(torch, spec, 8, prec, strategy=1, davidson_maxsteps=100)
    assert rep["converged"] == 1
    hn = np.abs(H).sum(axis=1).max()
    assert abs(rep["matrix_norm_inf"] - hn) <= 1e-12 * hn
    w = np.linalg.eigvalsh(H)[:8]
    assert np.abs(v - w).max() <= 1e-10 * hn
    r = np.linalg.norm(H @ X - X * v[None, :], axis=0) / max(1.0, hn)
    assert r.max() <= 1e-8


def test_solve_matches_csr_solver(cuda):
    torch = cuda
    rp, ci, va, d = oracle.fci_matrix(8, 4, 4, seed=4)
    n = len(d)
    Xc, vc, rc = api.block_solve_csr(rp, ci, va, n, 8, "fp64", strategy=1,
                                     davidson_maxsteps=100)
    spec = api.fci_spec(8, 4, 4, seed=4)
    X, v, rep = solve(torch, spec, 8, "bf16", strategy=1, davidson_maxsteps=100)
    assert rc["converged"] == 1 and rep["converged"] == 1
    assert np.abs(v - vc).max() <= 1e-10 * rc["matrix_norm_inf"]
    H = csr_matrix((va, ci, rp), shape=(n, n))
    r = np.linalg.norm(H @ X - X * v[None, :], axis=0) / max(1.0, rc["matrix_norm_inf"])
    assert r.max() <= 1e-8


def test_two_term_correction_saves_steps(cuda):
    """The second-order Davidson correction of the learned preconditioner at
    weight 1 on every row (its output bias alone), its second-order term
    from the FP32 sigma: the same eigenpairs as the plain FP64-accurate
    Davidson in fewer steps and FP64 sigma columns (10 orbitals)."""
    torch = cuda
    spec = api.fci_spec(10, 5, 5, seed=0)
    P = torch.zeros(api.mlp_param_count(), dtype=torch.float32, device="cuda")
    P[-1] = 30.0
    Xp, vp, rp = solve(torch, spec, 8, "fp64", strategy=1, davidson_maxsteps=60)
    Xl, vl, rl = solve(torch, spec, 8, "fp64", strategy=1, davidson_maxsteps=60,
                       preconditioner=1, mlp_params=P.data_ptr())
    assert rp["converged"] == 1 and rl["converged"] == 1
    assert rl["max_scaled_residual"] <= 1e-8
    assert np.abs(vl - vp).max() <= 1e-10 * rp["matrix_norm_inf"]
    assert rl["mlp_steps_accepted"] > 0 and rl["precond_matvecs"] > 0
    assert rl["davidson_steps"] < rp["davidson_steps"]
    assert rl["fp64_matvecs"] < rp["fp64_matvecs"]


def test_invalid_arguments(cuda):
    torch = cuda
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(api.IPTError):
        api.fci_sigma(api.fci_spec(20, 4, 4), x.data_ptr(), 1, x.data_ptr())
    with pytest.raises(api.IPTError):
        api.fci_sigma(api.fci_spec(6, 3, 3), x.data_ptr(), 0, x.data_ptr())
    with pytest.raises(api.IPTError):
        api.fci_dimension(api.fci_spec(6, 6, 3))
