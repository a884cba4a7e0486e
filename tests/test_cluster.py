"""Block-cluster path on the host: the cluster ranges of the library
(ipt_block_cluster_ranges) against the oracle's restatement, and the
oracle's cluster ranges and basis solve against the reference's own CPU
code (the committed fixtures, and oracle/_ref where it was built)."""
import os

import numpy as np
import pytest

from block_ipt_gb300 import api
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cluster_kat.npz")


@pytest.fixture(scope="module")
def kat():
    return np.load(GOLDEN)


def cases(kat):
    return [str(c) for c in kat["cases"]]


def test_oracle_ranges_match_reference_fixtures(kat):
    for c in cases(kat):
        k, adaptive = int(kat[c + "_params"][0]), int(kat[c + "_params"][1])
        cp, ri, va = kat[c + "_prep_col_ptr"], kat[c + "_prep_row_ind"], kat[c + "_prep_values"]
        ranges, added, lim, too_large = oracle.cluster_ranges(cp, ri, va, cp.size - 1, k,
                                                              adaptive=bool(adaptive))
        assert not too_large
        assert ranges == [tuple(r) for r in kat[c + "_ranges"].tolist()], c
        assert added == kat[c + "_added"].tolist(), c
        assert int(lim) == int(kat[c + "_limit_hit"][0]), c


def test_oracle_basis_matches_reference_fixtures(kat):
    """The oracle restates the GPU update (Gauss-Jordan); the reference's CPU
    solve inverts the m x m matrix: the same basis to rounding."""
    for c in cases(kat):
        k, adaptive, damping, maxiter, tol = kat[c + "_params"]
        cp, ri, va = kat[c + "_prep_col_ptr"], kat[c + "_prep_row_ind"], kat[c + "_prep_values"]
        X, its, res, st = oracle.cluster_basis(cp, ri, va, kat[c + "_prep_diag"],
                                               kat[c + "_ranges"], int(maxiter), tol, damping)
        assert st == 0, c
        ref = kat[c + "_basis"]
        err = np.abs(X - ref).max() / max(1.0, np.abs(ref).max())
        assert err <= 1e-11, (c, err)
        np.testing.assert_array_equal(its, kat[c + "_iterations"])


@pytest.mark.parametrize("adaptive", [False, True])
def test_library_ranges_match_oracle(lib, adaptive):
    """The library's host ranges against the oracle on seeded matrices with
    planted exact / near degeneracies and weak to strong coupling."""
    seen_multi = 0
    for seed in range(12):
        for coupling in (0.01, 0.3, 2.0):
            n = 40 + 3 * seed
            cp, ri, va, _ = oracle.cluster_test_matrix(n, seed, coupling)
            for k in (1, 4, 9):
                want = oracle.cluster_ranges(cp, ri, va, n, k, adaptive=adaptive)
                got, lim = api.cluster_ranges(cp, ri, va, n, k, adaptive=adaptive)
                assert got == want[0], (seed, coupling, k)
                assert lim == want[2]
                seen_multi += any(b > a for a, b in got)
    assert seen_multi > 20


def test_library_ranges_oversampled_targets(lib):
    """Ranges for k + oversample targets, the adaptive expansion keyed on the
    requested k (ipt_cuda.cu:4602-4641)."""
    cp, ri, va, _ = oracle.cluster_test_matrix(60, 3, 0.3)
    got, _ = api.cluster_ranges(cp, ri, va, 60, 12, requested_k=5)
    want = oracle.cluster_ranges(cp, ri, va, 60, 12, requested_k=5)
    assert got == want[0]
    assert sum(b - a + 1 for a, b in got) >= 12


def test_library_ranges_reject_wide_cluster(lib, monkeypatch):
    """A cluster wider than IPT_MAX_LIFT_BLOCK_SIZE is an invalid argument
    (ipt_cuda.cu:4619-4632)."""
    cp, ri, va, _ = oracle.cluster_test_matrix(56, 25, 2.0)
    want = oracle.cluster_ranges(cp, ri, va, 56, 9, max_block=3)
    assert want[3]
    monkeypatch.setenv("IPT_MAX_LIFT_BLOCK_SIZE", "3")
    with pytest.raises(Exception):
        api.cluster_ranges(cp, ri, va, 56, 9)


def test_library_ranges_invalid_input(lib):
    cp, ri, va, _ = oracle.cluster_test_matrix(20, 1, 0.1)
    for k in (0, 21):
        with pytest.raises(Exception):
            api.cluster_ranges(cp, ri, va, 20, k)
    bad = cp.copy()
    bad[-1] += 1
    with pytest.raises(Exception):
        api.cluster_ranges(bad, ri, va, 20, 3)


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built here")
def test_oracle_against_reference_code_sweep(monkeypatch):
    """Where the reference was compiled (oracle/_ref): ranges (with and
    without the adaptive expansion) and per-cluster bases on a sweep."""
    for seed in range(8):
        for coupling in (0.01, 0.3, 2.0):
            n = 40 + seed
            cp, ri, va, H = oracle.cluster_test_matrix(n, seed, coupling)
            for k in (4, 9):
                for adaptive in (0, 1):
                    monkeypatch.setenv("IPT_BLOCK_CLUSTER_ADAPTIVE", str(adaptive))
                    ref = oracle.ref_cluster_prepare(cp, ri, va, n, k)
                    mine = oracle.cluster_ranges(cp, ri, va, n, k, adaptive=bool(adaptive))
                    assert (ref[0], ref[1], ref[2]) == (mine[0], mine[1], mine[2])
                if coupling > 1.0:
                    continue
                ranges = mine[0]
                diag = np.diag(H).copy()
                X, its, _, st = oracle.cluster_basis(cp, ri, va, diag, ranges, 60, 1e-12)
                assert st == 0
                off = 0
                for c, (a, b) in enumerate(ranges):
                    Xr, itr = oracle.ref_cluster_solve_basis(cp, ri, va, diag, a, b, 60, 1e-12)
                    m = b - a + 1
                    err = np.abs(X[:, off:off + m] - Xr).max() / max(1.0, np.abs(Xr).max())
                    assert err <= 1e-11 and itr == its[c]
                    off += m


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built here")
def test_ranges_with_duplicates_and_unsorted_columns_against_reference(lib, monkeypatch):
    """Split (duplicate) entries and shuffled columns: the library merges the
    columns first, as the reference's block-cluster preparation does, and
    finds the reference's clusters."""
    checked = 0
    for seed in range(16):
        rng = np.random.default_rng(seed)
        n = 30 + seed % 10
        _, _, _, H = oracle.cluster_test_matrix(n, seed, [0.01, 0.3, 2.0][seed % 3])
        cp, ri, va = [0], [], []
        for c in range(n):
            ents = []
            for r in range(n):
                v = H[r, c]
                if v != 0 or r == c:
                    if rng.uniform() < 0.2 and r != c:
                        a = rng.uniform()
                        ents += [(r, v * a), (r, v * (1 - a))]
                    else:
                        ents.append((r, v))
            if seed % 4 == 3:
                rng.shuffle(ents)
            ri += [e[0] for e in ents]
            va += [e[1] for e in ents]
            cp.append(len(ri))
        cp, ri, va = np.array(cp, np.int32), np.array(ri, np.int32), np.array(va)
        for k in (3, 6):
            for adaptive in (0, 1):
                monkeypatch.setenv("IPT_BLOCK_CLUSTER_ADAPTIVE", str(adaptive))
                ref = oracle.ref_cluster_prepare(cp, ri, va, n, k)
                if isinstance(ref, int):
                    continue
                got, lim = api.cluster_ranges(cp, ri, va, n, k, adaptive=bool(adaptive))
                assert got == ref[0] and lim == ref[2], (seed, k, adaptive)
                checked += 1
    assert checked >= 40


def test_host_ranges_large_matrix_threaded_scans(lib):
    """A matrix of 8.8 M nonzeros, where the host entry's scans over the
    nonzeros (validation, merged-column check, diagonal, strongest couplings)
    run in parts on host threads: the planted degenerate pair (3, 4) forms
    the only multi-index cluster, the other targets are singletons, the
    same input with unsorted columns (merged first) gives the same ranges,
    and a row index out of range near the end is rejected."""
    from scipy.sparse import csc_matrix, diags
    n, k = 40000, 6
    d = np.arange(n, dtype=float)
    d[4] = d[3]
    rng = np.random.default_rng(7)
    half = 110 * n
    R = csc_matrix((np.full(half, 1e-9), (rng.integers(0, n, half), rng.integers(0, n, half))),
                   shape=(n, n))
    H = (R + R.T + diags(d)).tocsc()
    H.sort_indices()
    assert H.nnz > 8_000_000
    ranges, _ = api.cluster_ranges(H.indptr, H.indices, H.data, n, k)
    assert ranges == [(0, 0), (1, 1), (2, 2), (3, 4), (5, 5)]
    ri = H.indices.copy()
    c = n // 2
    a, b = H.indptr[c], H.indptr[c + 1]
    ri[a:b] = ri[a:b][::-1].copy()
    va = H.data.copy()
    va[a:b] = va[a:b][::-1].copy()
    assert api.cluster_ranges(H.indptr, ri, va, n, k)[0] == ranges
    ri[-1] = n
    with pytest.raises(api.IPTError):
        api.cluster_ranges(H.indptr, ri, va, n, k)
