"""GPU block solver on the FCI-like sparse CSR workloads vs the ARPACK
eigen-oracle fixture (tests/golden/fci_eigs.json).

Acceptance: |d lambda| <= 1e-10 ||H||_inf and scaled FP64 residual <= 1e-8.
"""
import json
import os

import numpy as np
import pytest

from block_ipt_gb300 import api, workloads

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "fci_eigs.json")) as f:
    FCI = json.load(f)


def solve_and_check(name, **kw):
    from scipy.sparse import csr_matrix
    case = FCI[name]
    rp, ci, v, d = workloads.fci_like_csr(case["norb"], case["nalpha"], case["nbeta"],
                                          seed=case["seed"])
    n, k = case["n"], case["k"]
    X, w, rep = api.block_solve_csr(rp, ci, v, n, k, "fp64", **kw)
    H = csr_matrix((v, ci, rp), shape=(n, n))
    hn = case["norm_inf"]
    ref = np.array(case["eigenvalues"])
    assert rep["converged"] == 1
    assert np.abs(w - ref).max() <= 1e-10 * hn, np.abs(w - ref).max() / hn
    r = np.linalg.norm(H @ X - X * w[None, :], axis=0) / max(1.0, hn)
    assert r.max() <= 1e-8, r.max()
    np.testing.assert_allclose(np.linalg.norm(X, axis=0), 1.0, atol=1e-10)
    return rep


@pytest.mark.parametrize("name", ["fci_6o_3a3b_seed1", "fci_8o_4a4b_seed0", "fci_8o_4a4b_seed5"])
@pytest.mark.parametrize("strategy", [0, 1])
def test_fci_small(cuda, name, strategy):
    solve_and_check(name, strategy=strategy)


def test_fci_config3_full(cuda):
    """n = 63,504 (10 orbitals, 5 alpha + 5 beta), nnz = 55.6M, k = 16."""
    rep = solve_and_check("fci_10o_5a5b_seed0")
    assert rep["fp64_matvecs"] > 0


def test_fci_device_entry_unsorted_diagonal(cuda):
    """The device CSR entry point on an unsorted FCI-like matrix: the targets
    are still the lowest diagonal positions and the rows come back in the
    caller's order."""
    torch = cuda
    from block_ipt_gb300 import api
    from scipy.sparse import csr_matrix
    case = FCI["fci_8o_4a4b_seed0"]
    rp, ci, v, d = workloads.fci_like_csr(8, 4, 4, seed=0)
    n, k = case["n"], case["k"]
    assert not np.all(np.diff(d) >= 0)
    drp = torch.from_numpy(rp).cuda()
    dci = torch.from_numpy(ci).cuda()
    dv = torch.from_numpy(v).cuda()
    dX = torch.empty((k, n), dtype=torch.float64, device="cuda")
    dw = torch.empty(k, dtype=torch.float64, device="cuda")
    import ctypes as C
    from block_ipt_gb300 import _lib
    opt = api.block_options("fp64", stream=torch.cuda.current_stream().cuda_stream)
    rep = _lib.IPTBlockReport()
    st = _lib.load().ipt_block_solve_csr_device(
        C.c_void_p(drp.data_ptr()), C.c_void_p(dci.data_ptr()), C.c_void_p(dv.data_ptr()), n,
        len(ci), k, C.byref(opt), C.c_void_p(dX.data_ptr()), C.c_void_p(dw.data_ptr()),
        C.byref(rep))
    assert st == 0
    torch.cuda.synchronize()
    X = dX.T.cpu().numpy()
    w = dw.cpu().numpy()
    H = csr_matrix((v, ci, rp), shape=(n, n))
    hn = case["norm_inf"]
    assert np.abs(w - np.array(case["eigenvalues"])).max() <= 1e-10 * hn
    r = np.linalg.norm(H @ X - X * w[None, :], axis=0) / max(1.0, hn)
    assert r.max() <= 1e-8
