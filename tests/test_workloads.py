"""Seeded workload generators (no GPU)."""
import numpy as np
import pytest

from block_ipt_gb300 import workloads


def test_dense_generators_are_symmetric_and_seeded():
    H1, d1 = workloads.dense_config0(200, seed=3)
    H2, d2 = workloads.dense_config0(200, seed=3)
    np.testing.assert_array_equal(H1, H2)
    assert np.abs(H1 - H1.T).max() == 0.0
    assert np.all(np.diff(d1) > 0)
    np.testing.assert_array_equal(np.diag(H1), d1)
    H3, _ = workloads.dense_config0(200, seed=4)
    assert np.abs(H3 - H1).max() > 0
    G, e = workloads.dense_config1(512, seed=0)
    assert np.abs(G - G.T).max() == 0.0
    assert np.all(np.diff(e) > 0)


def test_uniform_and_normal_moments():
    idx = np.arange(200000)
    u = workloads.uniform(7, 1, idx)
    assert 0.0 < u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 5e-3
    z = workloads.normal(7, 2, idx, idx * 3 + 1)
    assert abs(z.mean()) < 1e-2 and abs(z.std() - 1.0) < 1e-2


def test_batch_instances_in_range():
    inst = workloads.batch_config2(64, seed=1)
    assert len(inst) == 64
    for n, k, s, _ in inst:
        assert 64 <= n <= 2048 and 4 <= k <= 16 and 0.01 <= s <= 0.1


def test_fci_like_structure():
    from scipy.sparse import csr_matrix
    rp, ci, v, d = workloads.fci_like_csr(8, 4, 4, seed=0)
    n = workloads.fci_like_dims(8, 4, 4)
    assert len(rp) == n + 1 == 4901
    # 4*4 singles per spin = 16+16, doubles C(4,2)^2 = 36+36, ab = 256, + diagonal
    assert np.all(np.diff(rp) == 16 + 16 + 36 + 36 + 256 + 1)
    H = csr_matrix((v, ci, rp), shape=(n, n))
    assert abs(H - H.T).max() == 0.0
    np.testing.assert_allclose(H.diagonal(), d)
    assert np.all(np.diff(ci.reshape(n, -1), axis=1) > 0)  # rows sorted, no duplicates


def test_fci_config3_row_count():
    assert workloads.fci_like_dims(10, 5, 5) == 63504
    # 25 + 25 single, 100 + 100 same-spin double, 625 alpha-beta double = 875 per row
    assert 25 + 25 + 100 + 100 + 625 == 875


def test_torch_generator_matches_numpy():
    torch = pytest.importorskip("torch")
    for n, sig, seed in [(64, 0.05, 3), (333, 0.1, 17)]:
        H, d = workloads.batch_instance(n, sig, seed)
        Ht, dt = workloads.batch_instance_torch(torch, n, sig, seed, device="cpu")
        assert np.array_equal(d, dt.numpy())
        assert np.abs(H - Ht.numpy()).max() <= 1e-15
