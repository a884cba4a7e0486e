"""The FP64-accurate block product on the tensor cores
(ipt_block_accurate_product: six 8-bit digit slices per operand, exact
integer accumulation on the FP16 tensor cores, double-float drains) through
the C ABI.

Checks:
  * against the oracle's exact-integer emulation of the same split
    (oracle.accurate_product_emulated): the only differences are the
    double-float combination of the drains and the final FP64 sums,
    |Y - Y_emu| <= 2^-46 (n 2^(e_i + f_c)) with 2^e_i > max_l |Delta_il|
    and 2^f_c > max_l |X_lc|;
  * against the true product (long double): every entry within
    1e-14 * sum_l |H_il| max_l |X_lc|, the accuracy bar of the
    double-float product this kernel replaces.  The split is fixed-point per
    row of Delta, so a row whose entries span many decades is accurate
    relative to its largest entry instead: for the wide-range case the bar
    is 2^-44 sqrt(n) max_l |Delta_il| max_l |X_lc| (random rounding errors of
    2^-49 of the row scale over n terms).
"""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def run(torch, H, X):
    lib = _lib.load()
    n, c = X.shape
    dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()  # row-major H^T = col-major H
    dX = torch.from_numpy(np.asfortranarray(X).T.copy()).cuda()
    dY = torch.empty((c, n), dtype=torch.float64, device="cuda")
    st = lib.ipt_block_accurate_product(C.c_void_p(dH.data_ptr()), n, C.c_void_p(dX.data_ptr()),
                                        c, C.c_void_p(dY.data_ptr()), None)
    assert st == 0, _lib.status_string(st)
    torch.cuda.synchronize()
    return dY.cpu().numpy().T.copy()


def true_product(H, X):
    return (H.astype(np.longdouble) @ X.astype(np.longdouble)).astype(np.float64)


def cases():
    rng = np.random.default_rng(5)
    H, _ = workloads.dense_config1(1024, seed=2)
    yield "config1_n1024_ipt_block", H, np.eye(1024, 40) + 0.01 * rng.standard_normal((1024, 40))
    H = rng.standard_normal((300, 300))
    yield "general_300x300_c17", H, rng.standard_normal((300, 17))
    H = rng.standard_normal((513, 513)) * np.exp(-rng.uniform(0, 30, (513, 513)))
    yield "wide_range_513_c64", H, rng.standard_normal((513, 64)) * np.exp(-rng.uniform(0, 20, (513, 64)))
    H, _ = workloads.dense_config0(777, seed=4)
    yield "config0_777_c70", H, rng.standard_normal((777, 70))
    H = rng.standard_normal((128, 128))
    yield "one_tile_c1", H, rng.standard_normal((128, 1))


@pytest.mark.parametrize("name,H,X", list(cases()), ids=[c[0] for c in cases()])
def test_against_emulation_and_truth(cuda, name, H, X):
    Y = run(cuda, H, X)
    n = H.shape[0]
    D = np.abs(H - np.diag(np.diag(H)))
    rmax = D.max(axis=1)
    cmax = np.abs(X).max(axis=0)
    fixed_scale = n * np.outer(2.0 * np.maximum(rmax, 1e-300), 2.0 * np.maximum(cmax, 1e-300))
    Ye = oracle.accurate_product_emulated(H, X)
    assert (np.abs(Y - Ye) <= 2.0 ** -46 * fixed_scale + 1e-15 * np.abs(Ye)).all(), \
        (np.abs(Y - Ye) / fixed_scale).max()
    Yt = true_product(H, X)
    if name.startswith("wide_range"):
        scale = 2.0 ** -44 * np.sqrt(n) * np.outer(rmax, cmax) + 1e-14 * np.abs(Yt)
        assert (np.abs(Y - Yt) <= scale).all(), (np.abs(Y - Yt) / scale).max()
    else:
        scale = np.abs(H).sum(axis=1)[:, None] * cmax[None, :]
        rel = (np.abs(Y - Yt) / scale).max()
        assert rel <= 1e-14, rel


def test_nonfinite_row_gives_nan(cuda):
    H = np.eye(64) * 3.0
    H[5, 9] = np.nan
    X = np.ones((64, 3))
    Y = run(cuda, H, X)
    assert np.isnan(Y[5]).all()
    assert np.isfinite(np.delete(Y, 5, axis=0)).all()
    np.testing.assert_array_equal(np.delete(Y, 5, axis=0), 3.0)


def test_invalid_arguments(cuda):
    lib = _lib.load()
    assert lib.ipt_block_accurate_product(None, 8, None, 2, None, None) == 1
