"""Block-cluster path on the GPU: the update kernel bit for bit against the
oracle's restatement, the basis solve against the oracle and the
reference's own CPU solve (committed fixtures), and the IPT_BLOCK_CLUSTER
entry end to end."""
import os

import numpy as np
import pytest

from block_ipt_gb300 import api
from oracle import oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cluster_kat.npz")


def dev(torch, a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a.T if a.ndim == 2 else a))
    return t.cuda() if dtype is None else t.to(dtype).cuda()


def to_f(torch, t, n, m):
    return t.cpu().numpy().T.copy(order="F") if m > 0 else t.cpu().numpy()


def update_case(rng, n, m, first):
    d = np.sort(rng.uniform(0, n, n))
    X = rng.standard_normal((n, m))
    Y = rng.standard_normal((n, m)) * 0.5 + d[:, None] * X
    return d, np.asfortranarray(X), np.asfortranarray(Y)


@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 7, 8, 9, 16, 17, 31, 32, 33, 48, 64])
@pytest.mark.parametrize("damping", [1.0, 0.6])
def test_update_bit_exact(cuda, m, damping):
    torch = cuda
    rng = np.random.default_rng(100 + m)
    n = 300
    first = int(rng.integers(0, n - m))
    d, X, Y = update_case(rng, n, m, first)
    want, sing = oracle.cluster_update(X, Y, d, first, damping)
    assert not sing
    dX, dY, dd = dev(torch, X), dev(torch, Y), dev(torch, d)
    dN = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    s = api.cluster_update(dX.data_ptr(), dY.data_ptr(), dd.data_ptr(), n, first, m, dN.data_ptr(),
                           damping)
    got = dN.cpu().numpy().T
    assert not s
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), np.abs(got - want).max()
    np.testing.assert_array_equal(got[first:first + m], np.eye(m))


@pytest.mark.parametrize("m", [1, 3, 40])
def test_update_singular_flag(cuda, m):
    """A row whose system is singular (d_i I - h^T with a zero pivot) or whose
    solution is not finite sets the flag, as in the oracle."""
    torch = cuda
    rng = np.random.default_rng(7)
    n = 120
    first = 10
    d, X, Y = update_case(rng, n, m, first)
    # h = Y[first:first+m, :] = diag(d[50]) makes row 50's matrix exactly zero
    Y[first:first + m, :] = 0.0
    Y[np.arange(first, first + m), np.arange(m)] = d[50]
    want, sing = oracle.cluster_update(X, Y, d, first)
    assert sing
    dX, dY, dd = dev(torch, X), dev(torch, Y), dev(torch, d)
    dN = torch.zeros((m, n), dtype=torch.float64, device="cuda")
    assert api.cluster_update(dX.data_ptr(), dY.data_ptr(), dd.data_ptr(), n, first, m,
                              dN.data_ptr())
    # a NaN on the right side: the value is not finite
    d, X, Y = update_case(rng, n, m, first)
    Y[77, 0] = np.nan
    want, sing = oracle.cluster_update(X, Y, d, first)
    assert sing
    dX, dY = dev(torch, X), dev(torch, Y)
    assert api.cluster_update(dX.data_ptr(), dY.data_ptr(), dd.data_ptr(), n, first, m,
                              dN.data_ptr())


def run_basis(torch, cp, ri, va, diag, ranges, maxiter, tol, damping):
    n = cp.size - 1
    cols = int(sum(b - a + 1 for a, b in ranges))
    drp, dci = dev(torch, cp.astype(np.int32)), dev(torch, ri.astype(np.int32))
    dva, dd = dev(torch, va), dev(torch, diag)
    dB = torch.zeros((cols, n), dtype=torch.float64, device="cuda")
    it, res = api.cluster_basis(drp.data_ptr(), dci.data_ptr(), dva.data_ptr(), n, ri.size,
                                dd.data_ptr(), ranges, maxiter, tol, dB.data_ptr(), damping)
    return dB.cpu().numpy().T.copy(order="F"), it, res


def test_basis_matches_reference_fixtures(cuda):
    """Each fixture (the reference's own CPU solve): the GPU basis and
    iteration counts against it and against the oracle."""
    kat = np.load(GOLDEN)
    for c in [str(x) for x in kat["cases"]]:
        k, adaptive, damping, maxiter, tol = kat[c + "_params"]
        cp, ri, va = kat[c + "_prep_col_ptr"], kat[c + "_prep_row_ind"], kat[c + "_prep_values"]
        diag = kat[c + "_prep_diag"]
        ranges = [tuple(r) for r in kat[c + "_ranges"].tolist()]
        X, it, res = run_basis(cuda, cp, ri, va, diag, ranges, int(maxiter), tol, damping)
        Xo, ito, reso, st = oracle.cluster_basis(cp, ri, va, diag, ranges, int(maxiter), tol,
                                                 damping)
        assert st == 0
        ref = kat[c + "_basis"]
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(X - ref).max() / scale <= 1e-11, c
        assert np.abs(X - Xo).max() / scale <= 1e-12, c
        np.testing.assert_array_equal(it, kat[c + "_iterations"])
        np.testing.assert_array_equal(it, ito)
        # the residuals near convergence are differences at rounding level
        np.testing.assert_allclose(res, reso, rtol=1e-3, atol=1e-14)


def test_basis_sweep_against_oracle(cuda):
    worst = 0.0
    for seed in range(10):
        for coupling in (0.01, 0.3):
            n = 80 + 7 * seed
            cp, ri, va, H = oracle.cluster_test_matrix(n, seed, coupling)
            ranges, _, _, _ = oracle.cluster_ranges(cp, ri, va, n, 8,
                                                    adaptive=bool(seed % 2))
            diag = np.diag(H).copy()
            for damping in (1.0, 0.8):
                X, it, _ = run_basis(cuda, cp, ri, va, diag, ranges, 50, 1e-12, damping)
                Xo, ito, _, st = oracle.cluster_basis(cp, ri, va, diag, ranges, 50, 1e-12,
                                                      damping)
                assert st == 0
                err = np.abs(X - Xo).max() / max(1.0, np.abs(Xo).max())
                worst = max(worst, err)
                assert np.all(np.abs(it - ito) <= 1), (it, ito)
    assert worst <= 1e-12, worst


def test_basis_rejects_bad_ranges(cuda):
    torch = cuda
    cp, ri, va, H = oracle.cluster_test_matrix(30, 1, 0.1)
    for ranges in ([(3, 2)], [(0, 4), (4, 6)], [(0, 64)], [(28, 30)]):
        with pytest.raises(Exception):
            run_basis(torch, cp, ri, va, np.diag(H).copy(), ranges, 10, 1e-12, 1.0)


@pytest.mark.parametrize("adaptive,n,seed,k", [("0", 90, 5, 6), ("1", 56, 5, 4)])
def test_block_cluster_entry_degenerate(cuda, monkeypatch, adaptive, n, seed, k):
    """ipt_cuda_sparse_csc_tol with IPT_BLOCK_CLUSTER on a matrix with planted
    degeneracies: the cluster basis, Rayleigh-Ritz and the Davidson
    enrichment give the lowest eigenpairs (ipt_cuda.cu:4712-5016)."""
    monkeypatch.setenv("IPT_BLOCK_CLUSTER", "1")
    monkeypatch.setenv("IPT_BLOCK_CLUSTER_ADAPTIVE", adaptive)
    monkeypatch.setenv("IPT_DAVIDSON_ENRICH", "1")
    monkeypatch.setenv("IPT_DAVIDSON_STEPS", "40")
    cp, ri, va, H = oracle.cluster_test_matrix(n, seed, 0.3)
    X, v, info = api.ipt_cuda_sparse_csc_tol(cp, ri, va, n, k, 1e-12, 200)
    w, _ = oracle.eigh_lowest(H, k)
    scale = np.abs(H).sum(1).max()
    np.testing.assert_allclose(v, w, atol=1e-9 * scale)
    np.testing.assert_allclose(np.linalg.norm(X, axis=0), 1.0, atol=1e-10)
    assert np.abs(H @ X - X * v).max() <= 1e-7 * scale
    assert info["iterations"] > 0 and info["basis_cols"] >= k
    want = oracle.cluster_ranges(cp, ri, va, n, k, adaptive=adaptive == "1")
    added = ";".join(str(i) for i in want[1]) or "none"
    assert info["adaptive_added_indices"] == added


def orthogonality(B):
    """(Frobenius norm, largest entry) of B^T B - I, the reference's
    host statistics (ipt_cuda.cu:2489-2524)."""
    E = B.T @ B - np.eye(B.shape[1])
    return np.sqrt((E * E).sum()), np.abs(E).max()


@pytest.mark.parametrize("qr", ["0", "1"])
def test_block_cluster_orthogonality_stats(cuda, monkeypatch, qr):
    """IPT_RR_HOST_ORTHOGONALITY_STATS and IPT_BLOCK_CLUSTER_QR on the
    block-cluster entry: rayleigh_ritz_used_qr follows the knob; the basis
    figures describe the cluster basis as built (against the oracle's basis)
    or, with QR, its orthonormalised form; the Ritz vectors' figures are at
    rounding level; with the statistics off the figures stay NaN."""
    monkeypatch.setenv("IPT_BLOCK_CLUSTER", "1")
    monkeypatch.setenv("IPT_BLOCK_CLUSTER_QR", qr)
    monkeypatch.setenv("IPT_RR_HOST_ORTHOGONALITY_STATS", "1")
    n, k = 90, 6
    cp, ri, va, H = oracle.cluster_test_matrix(n, 5, 0.3)
    X, v, info = api.ipt_cuda_sparse_csc_tol(cp, ri, va, n, k, 1e-12, 200)
    assert info["rayleigh_ritz_used_qr"] == int(qr)
    fro, mx, bad = info["basis_orthogonality"]
    assert bad == 0 and np.isfinite(fro) and mx <= fro
    if qr == "0":
        ranges, _, _, _ = oracle.cluster_ranges(cp, ri, va, n, k)
        # symmetric: the CSC arrays are also the CSR arrays
        B, _, _, st = oracle.cluster_basis(cp, ri, va, np.diag(H).copy(), ranges, 200, 1e-12)
        assert st == 0
        wf, wm = orthogonality(B)
        assert wf > 1e-6  # the cluster basis is not orthonormal
        assert abs(fro - wf) <= 1e-8 * wf and abs(mx - wm) <= 1e-8 * wm
    else:
        assert fro <= 1e-12
    rf, rm, rbad = info["ritz_vectors_orthogonality"]
    assert rbad == 0 and rf <= 1e-12 and rm <= rf
    wf, _ = orthogonality(X)
    assert abs(rf - wf) <= 1e-12
    monkeypatch.setenv("IPT_RR_HOST_ORTHOGONALITY_STATS", "0")
    _, v2, info = api.ipt_cuda_sparse_csc_tol(cp, ri, va, n, k, 1e-12, 200)
    assert np.isnan(info["basis_orthogonality"][0]) and np.isnan(info["ritz_vectors_orthogonality"][1])
    assert info["rayleigh_ritz_used_qr"] == int(qr)
    np.testing.assert_array_equal(v2, v)


def test_block_cluster_entry_singular_block(cuda, monkeypatch):
    """A cluster whose row system turns singular makes the entry fail with
    an invalid argument, as the oracle's (and the reference's) block solve
    does (ipt_cuda.cu:2994-3000, 4872-4881: no identity fallback)."""
    monkeypatch.setenv("IPT_BLOCK_CLUSTER", "1")
    n, k = 90, 6
    cp, ri, va, H = oracle.cluster_test_matrix(n, 2, 0.3)
    ranges, _, _, _ = oracle.cluster_ranges(cp, ri, va, n, k)
    assert oracle.cluster_basis(cp, ri, va, np.diag(H).copy(), ranges, 200, 1e-12)[3] != 0
    with pytest.raises(Exception):
        api.ipt_cuda_sparse_csc_tol(cp, ri, va, n, k, 1e-12, 200)


def one_sided_storage(cp, ri, va, n, seed):
    """The same matrix stored unevenly: some entries above the diagonal split
    into two duplicates (their mirror stays one entry), explicit zeros added
    on one side only, a 1e-15 entry whose mirror is absent, and shuffled
    columns."""
    rng = np.random.default_rng(seed)
    ncp, nri, nva = [0], [], []
    for c in range(n):
        ents = []
        for p in range(cp[c], cp[c + 1]):
            r, v = int(ri[p]), float(va[p])
            if r < c and rng.uniform() < 0.3:
                a = rng.uniform()
                ents += [(r, v * a), (r, v - v * a)]
            else:
                ents.append((r, v))
        if c + 2 < n and rng.uniform() < 0.2:
            ents.append((c + 2, 0.0))
        if c == n // 2:
            ents.append((n - 1, 1e-15))
        rng.shuffle(ents)
        nri += [e[0] for e in ents]
        nva += [e[1] for e in ents]
        ncp.append(len(nri))
    return np.array(ncp, np.int32), np.array(nri, np.int32), np.array(nva)


@pytest.mark.parametrize("adaptive", ["0", "1"])
def test_block_cluster_entry_uneven_storage(cuda, monkeypatch, adaptive):
    """A symmetric matrix stored with one-sided duplicates and explicit zeros
    passes the entry's symmetry check (the reference merges the columns and
    compares values by lookup, ipt_preparation.cu:860-883) and gives the
    same eigenpairs as its clean storage, whether or not the diagonal needs
    sorting."""
    monkeypatch.setenv("IPT_BLOCK_CLUSTER", "1")
    monkeypatch.setenv("IPT_BLOCK_CLUSTER_ADAPTIVE", adaptive)
    monkeypatch.setenv("IPT_DAVIDSON_ENRICH", "1")
    monkeypatch.setenv("IPT_DAVIDSON_STEPS", "40")
    n, k = 90, 6
    cp, ri, va, H = oracle.cluster_test_matrix(n, 5, 0.3)
    for shuffle_diag in (False, True):
        if shuffle_diag:
            # a diagonal out of ascending order takes the permuted preparation
            perm = np.random.default_rng(1).permutation(n)
            Hp = H[perm][:, perm]
            cols = [np.nonzero(Hp[:, c])[0] for c in range(n)]
            cp = np.cumsum([0] + [len(x) for x in cols]).astype(np.int32)
            ri = np.concatenate(cols).astype(np.int32)
            va = np.concatenate([Hp[x, c] for c, x in enumerate(cols)])
            Href = Hp
        else:
            Href = H
        ucp, uri, uva = one_sided_storage(cp, ri, va, n, 7)
        X, v, info = api.ipt_cuda_sparse_csc_tol(ucp, uri, uva, n, k, 1e-12, 200)
        w, _ = oracle.eigh_lowest(Href, k)
        scale = np.abs(Href).sum(1).max()
        np.testing.assert_allclose(v, w, atol=1e-9 * scale)
        assert np.abs(Href @ X - X * v).max() <= 1e-7 * scale


def device_csr(torch, cp, ri, va):
    """A symmetric CSC matrix is its own CSR: the three arrays on the GPU."""
    return (torch.from_numpy(np.asarray(cp, np.int32)).cuda(),
            torch.from_numpy(np.asarray(ri, np.int32)).cuda(),
            torch.from_numpy(np.asarray(va, np.float64)).cuda())


@pytest.mark.parametrize("adaptive", [False, True])
def test_device_ranges_match_host(cuda, adaptive):
    """ipt_block_cluster_ranges_device gives the host entry's ranges and
    limit flag on seeded matrices with planted exact and near degeneracies,
    weak to strong coupling, and several target counts."""
    torch = cuda
    multi = 0
    for seed in range(10):
        for coupling in (0.01, 0.3, 2.0):
            n = 40 + 5 * seed
            cp, ri, va, _ = oracle.cluster_test_matrix(n, seed, coupling)
            drp, dci, dvv = device_csr(torch, cp, ri, va)
            for k in (1, 4, 9):
                for rk in sorted({1, k}):
                    want = api.cluster_ranges(cp, ri, va, n, k, requested_k=rk,
                                              adaptive=adaptive)
                    got = api.cluster_ranges_device(drp.data_ptr(), dci.data_ptr(),
                                                    dvv.data_ptr(), n, len(ri), k,
                                                    requested_k=rk, adaptive=adaptive)
                    assert got == want, (seed, coupling, k, rk)
                    multi += any(b > a for a, b in want[0])
    assert multi >= 10


def test_device_ranges_match_reference_fixtures(cuda):
    """The committed fixtures of the reference's own detection: the device
    entry finds its ranges on every prepared matrix."""
    torch = cuda
    kat = np.load(GOLDEN)
    for c in [str(x) for x in kat["cases"]]:
        k, adaptive = int(kat[c + "_params"][0]), int(kat[c + "_params"][1])
        cp, ri, va = kat[c + "_prep_col_ptr"], kat[c + "_prep_row_ind"], kat[c + "_prep_values"]
        drp, dci, dvv = device_csr(torch, cp, ri, va)
        got, lim = api.cluster_ranges_device(drp.data_ptr(), dci.data_ptr(), dvv.data_ptr(),
                                             cp.size - 1, len(ri), k, adaptive=bool(adaptive))
        assert got == [tuple(r) for r in kat[c + "_ranges"].tolist()], c
        assert int(lim) == int(kat[c + "_limit_hit"][0]), c


def test_device_ranges_large_sparse(cuda):
    """A 200000-row banded matrix with a planted degenerate group: the device
    scans and the host entry agree."""
    torch = cuda
    sp = pytest.importorskip("scipy.sparse")
    n, k = 200000, 12
    rng = np.random.default_rng(3)
    d = np.sort(rng.uniform(0, 100, n))
    d[3:6] = d[3]
    off = rng.normal(scale=0.05, size=n - 1)
    H = sp.diags([off, d, off], [-1, 0, 1], format="csc")
    H.sort_indices()
    want = api.cluster_ranges(H.indptr, H.indices, H.data, n, k, adaptive=True)
    drp, dci, dvv = device_csr(torch, H.indptr, H.indices, H.data)
    got = api.cluster_ranges_device(drp.data_ptr(), dci.data_ptr(), dvv.data_ptr(), n,
                                    int(H.nnz), k, adaptive=True)
    assert got == want
    assert any(b > a for a, b in got[0])


def test_device_ranges_invalid_arguments(cuda):
    torch = cuda
    cp, ri, va, _ = oracle.cluster_test_matrix(30, 1, 0.1)
    drp, dci, dvv = device_csr(torch, cp, ri, va)
    for k, rk in ((0, 1), (31, 1), (4, 5), (4, 0)):
        with pytest.raises(RuntimeError):
            api.cluster_ranges_device(drp.data_ptr(), dci.data_ptr(), dvv.data_ptr(), 30,
                                      len(ri), k, requested_k=rk)
    with pytest.raises(RuntimeError):
        api.cluster_ranges_device(0, dci.data_ptr(), dvv.data_ptr(), 30, len(ri), 4)
