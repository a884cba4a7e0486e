"""The plain sparse path's host preparation with degeneracy lifting
(ipt_block_prepare_csc) against the reference's own preparation, bit for
bit: the committed fixtures (tests/golden/make_lift_golden.py) and, where
oracle/_ref was built, a sweep; the oracle's back-transform against the
reference's."""
import os

import numpy as np
import pytest
from scipy.sparse import csc_matrix

from block_ipt_gb300 import api
from oracle import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lift_kat.npz")
KEYS = ("col_ptr", "row_ind", "values", "diag", "perm", "rot_first", "rot_size", "rot_values")


def bits(a):
    a = np.asarray(a)
    return a.view(np.uint64) if a.dtype == np.float64 else a.astype(np.int64)


def case_input(z, c):
    n, k, ncp, nri = (int(x) for x in z[c + "_params"])
    ints = z[c + "_in"]
    return ints[:ncp], ints[ncp:ncp + nri], z[c + "_in_values"], n, k


@pytest.fixture(scope="module")
def kat():
    return np.load(GOLDEN)


def test_lifted_preparation_matches_reference_fixtures(lib, kat):
    rotated = 0
    for c in [str(x) for x in kat["cases"]]:
        cp, ri, va, n, k = case_input(kat, c)
        if int(kat[c + "_status"][0]) != 0:
            with pytest.raises(Exception):
                api.prepare_csc(cp, ri, va, n, k)
            continue
        got = api.prepare_csc(cp, ri, va, n, k)
        for key in KEYS:
            want = kat[c + "_" + key]
            assert np.array_equal(bits(got[key]), bits(want)), (c, key)
        rotated += len(got["rot_first"]) > 0
    assert rotated >= 4


def test_oracle_back_transform_matches_reference(kat):
    for c in [str(x) for x in kat["cases"]]:
        if int(kat[c + "_status"][0]) != 0:
            continue
        out = oracle.unprepare_vectors(kat[c + "_vectors_in"], kat[c + "_perm"],
                                       kat[c + "_rot_first"], kat[c + "_rot_size"],
                                       kat[c + "_rot_values"])
        assert np.array_equal(bits(out), bits(kat[c + "_vectors_out"])), c


def test_no_lifting_on_the_reference_test_matrices(lib, golden):
    """The reference's own sparse cases (banded n = 64, H2O "W") have no
    degenerate targets: lifting leaves them as the sort-only preparation."""
    arrays, meta = golden
    for case in meta["sparse"]:
        name = case["name"]
        cp = arrays["sparse_%s_col_ptr" % name]
        ri = arrays["sparse_%s_row_ind" % name]
        va = arrays["sparse_%s_values_csc" % name]
        got = api.prepare_csc(cp, ri, va, case["n"], case["k"])
        assert len(got["rot_first"]) == 0
        np.testing.assert_array_equal(got["diag"], arrays["sparse_%s_prep_diag" % name])
        np.testing.assert_array_equal(got["perm"], arrays["sparse_%s_prep_perm" % name])


def test_lifted_blocks_are_orthogonal_rotations(lib, kat):
    for c in [str(x) for x in kat["cases"]]:
        if int(kat[c + "_status"][0]) != 0:
            continue
        cp, ri, va, n, k = case_input(kat, c)
        got = api.prepare_csc(cp, ri, va, n, k)
        ofs = 0
        for m in got["rot_size"]:
            Q = got["rot_values"][ofs:ofs + m * m].reshape((m, m), order="F")
            np.testing.assert_allclose(Q.T @ Q, np.eye(m), atol=1e-13)
            ofs += m * m
        # the prepared matrix is the rotated, permuted input (eigenvalues kept)
        H = csc_matrix((va, ri, cp), shape=(n, n)).toarray()
        Hp = csc_matrix((got["values"], got["row_ind"], got["col_ptr"]), shape=(n, n)).toarray()
        np.testing.assert_allclose(np.linalg.eigvalsh(0.5 * (Hp + Hp.T)),
                                   np.linalg.eigvalsh(H), atol=1e-12 * np.abs(H).max())


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built here")
def test_lifted_preparation_sweep_against_reference(lib):
    ok = rotated = rejected = 0
    for seed in range(20):
        for coupling in (0.01, 0.3, 2.0):
            n = 30 + seed
            _, _, _, H = oracle.cluster_test_matrix(n, seed, coupling)
            P = np.random.default_rng(seed).permutation(n)
            S = csc_matrix(H[np.ix_(P, P)])
            S.sort_indices()
            for k in (1, 3, 6):
                ref = oracle.ref_prepare_lifted(S.indptr, S.indices, S.data, n, k)
                if isinstance(ref, int):
                    with pytest.raises(Exception):
                        api.prepare_csc(S.indptr, S.indices, S.data, n, k)
                    rejected += 1
                    continue
                got = api.prepare_csc(S.indptr, S.indices, S.data, n, k)
                for key in KEYS:
                    assert np.array_equal(bits(got[key]), bits(ref[key])), (seed, coupling, k, key)
                ok += 1
                rotated += len(ref["rot_first"]) > 0
    assert ok > 50 and rotated > 10 and rejected > 10


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built here")
def test_non_symmetric_matrices_against_reference(lib):
    """A non-symmetric matrix whose targets need a lift is rejected, as the
    reference rejects it without LAPACK dgeev; one without degenerate
    targets is prepared as the reference prepares it."""
    rejected = accepted = 0
    for seed in range(6):
        n = 30
        _, _, _, H = oracle.cluster_test_matrix(n, seed, 0.3)
        H = H.copy()
        H[0, 5] += 0.01
        S = csc_matrix(H)
        S.sort_indices()
        for k in (1, 3, 6):
            ref = oracle.ref_prepare_lifted(S.indptr, S.indices, S.data, n, k)
            if isinstance(ref, int):
                with pytest.raises(Exception):
                    api.prepare_csc(S.indptr, S.indices, S.data, n, k)
                rejected += 1
            else:
                got = api.prepare_csc(S.indptr, S.indices, S.data, n, k)
                for key in KEYS:
                    assert np.array_equal(bits(got[key]), bits(ref[key])), (seed, k, key)
                accepted += 1
    assert rejected >= 3 and accepted >= 6


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built here")
def test_duplicates_zeros_and_unsorted_columns_against_reference(lib):
    """Inputs with split (duplicate) entries, explicit zeros and shuffled
    columns, permuted or not: the same prepared arrays as the reference."""
    ok = 0
    for seed in range(24):
        rng = np.random.default_rng(seed)
        n = 30 + seed % 10
        _, _, _, H = oracle.cluster_test_matrix(n, seed, [0.01, 0.3, 2.0][seed % 3])
        P = rng.permutation(n) if seed % 2 else np.arange(n)
        H = H[np.ix_(P, P)]
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
            if rng.uniform() < 0.3:
                ents.append((int(rng.integers(0, n)), 0.0))
            if seed % 4 == 3:
                rng.shuffle(ents)
            ri += [e[0] for e in ents]
            va += [e[1] for e in ents]
            cp.append(len(ri))
        cp, ri, va = np.array(cp, np.int32), np.array(ri, np.int32), np.array(va)
        for k in (1, 3, 6):
            ref = oracle.ref_prepare_lifted(cp, ri, va, n, k)
            if isinstance(ref, int):
                with pytest.raises(Exception):
                    api.prepare_csc(cp, ri, va, n, k)
                continue
            got = api.prepare_csc(cp, ri, va, n, k)
            for key in KEYS:
                assert np.array_equal(bits(got[key]), bits(ref[key])), (seed, k, key)
            ok += 1
    assert ok >= 15


def prep_debug_lines(capfd, monkeypatch, cp, ri, va, n, k):
    monkeypatch.setenv("IPT_DEBUG_PREPARATION", "1")
    capfd.readouterr()
    try:
        api.prepare_csc(cp, ri, va, n, k)
    except Exception:
        pass
    out = capfd.readouterr().out
    return [line for line in out.splitlines() if line.startswith("[IPT preparation]")]


def test_debug_preparation_lines_match_reference(lib, kat, capfd, monkeypatch):
    """IPT_DEBUG_PREPARATION: the diagnostic lines of the detection and the
    lift rounds (unions, candidate summary, rounds and blocks, post-lift
    diagonal, the rejection of a block wider than the limit) are the
    reference's, character for character (tests/golden/prep_debug_kat.json,
    recorded from the reference's own preparation)."""
    import json
    with open(os.path.join(os.path.dirname(GOLDEN), "prep_debug_kat.json")) as f:
        want = json.load(f)
    for c in [str(x) for x in kat["cases"]]:
        cp, ri, va, n, k = case_input(kat, c)
        assert prep_debug_lines(capfd, monkeypatch, cp, ri, va, n, k) == want[c], c
    assert any("lift succeeded" in line for lines in want.values() for line in lines)
    assert any("unresolved target gap" in line for line in want["reject"])
    monkeypatch.setenv("IPT_MAX_LIFT_BLOCK_SIZE", "2")
    cp, ri, va, n, k = case_input(kat, "lift_5")
    got = prep_debug_lines(capfd, monkeypatch, cp, ri, va, n, k)
    assert got == want["lift_5_max_block_2"]
    assert "exceeds max_block_size=2" in got[-1]


def test_debug_preparation_off_prints_nothing(lib, kat, capfd, monkeypatch):
    cp, ri, va, n, k = case_input(kat, "lift_5")
    for value in ("0", "no", ""):
        monkeypatch.setenv("IPT_DEBUG_PREPARATION", value)
        capfd.readouterr()
        api.prepare_csc(cp, ri, va, n, k)
        assert "[IPT preparation]" not in capfd.readouterr().out


def nonsymmetric_cluster_matrix(n, m, first, seed, spread=1e-3):
    """A non-symmetric matrix whose diagonal is degenerate at positions
    first..first+m-1 (shuffled), coupled there by a real-spectrum block
    S D S^-1 (D: m distinct values within `spread`), with weak symmetric
    couplings elsewhere."""
    rng = np.random.default_rng(seed)
    d = np.arange(n, dtype=float) + 0.5
    d[first:first + m] = d[first]
    H = np.diag(d)
    for _ in range(3 * n):
        i, j = rng.integers(0, n, 2)
        if i != j and not (first <= i < first + m and first <= j < first + m):
            v = rng.uniform(-1e-3, 1e-3)
            H[i, j] += v
            H[j, i] += v
    S = rng.standard_normal((m, m)) + 3 * np.eye(m)
    D = np.diag(np.sort(rng.uniform(-1, 1, m)) * spread)
    H[first:first + m, first:first + m] += S @ D @ np.linalg.inv(S)
    P = rng.permutation(n)
    S = csc_matrix(H[np.ix_(P, P)])
    S.sort_indices()
    return S.indptr, S.indices, S.data, H[np.ix_(P, P)]


def test_general_lift_of_nonsymmetric_groups(lib, monkeypatch):
    """IPT_GB300_GENERAL_LIFT: a degenerate group of a non-symmetric matrix
    is lifted with this build's real eigensolver, where the reference uses
    LAPACK dgeev when linked: the block's eigenvectors agree with dgeev's
    (scipy.linalg.eig) up to sign, the left factor is their inverse (the
    lifted block is diagonal), the spectrum is kept, and the back-transform
    of the prepared matrix's eigenvectors gives the input's.  Without the
    switch the same inputs are rejected, as the reference's own build
    without dgeev rejects them."""
    scipy_linalg = pytest.importorskip("scipy.linalg")
    lifted = 0
    for seed in range(5):
        for m in (2, 3, 5, 8):
            n, k = 40, 6
            cp, ri, va, H = nonsymmetric_cluster_matrix(n, m, 2, seed)
            monkeypatch.setenv("IPT_GB300_GENERAL_LIFT", "1")
            got = api.prepare_csc(cp, ri, va, n, k)
            if len(got["rot_first"]) == 0:
                continue
            lifted += 1
            scale = np.abs(H).sum(axis=1).max()
            Hp = csc_matrix((got["values"], got["row_ind"], got["col_ptr"]), shape=(n, n)).toarray()
            np.testing.assert_allclose(np.sort(np.linalg.eigvals(Hp).real),
                                       np.sort(np.linalg.eigvals(H).real), atol=1e-11 * scale)
            pre = api.prepare_csc(cp, ri, va, n, k, lift=False)
            Hs = csc_matrix((pre["values"], pre["row_ind"], pre["col_ptr"]), shape=(n, n)).toarray()
            f, b = int(got["rot_first"][0]), int(got["rot_size"][0])
            w, Vl = scipy_linalg.eig(Hs[f:f + b, f:f + b])
            Vl = Vl[:, np.argsort(w.real)].real
            V = got["rot_values"][:b * b].reshape((b, b), order="F")
            np.testing.assert_allclose(np.linalg.norm(V, axis=0), 1.0, atol=1e-13)
            cos = np.abs((V * Vl).sum(axis=0)) / np.linalg.norm(Vl, axis=0)
            assert cos.min() >= 1 - 1e-10, (seed, m, cos)
            off = Hp[f:f + b, f:f + b] - np.diag(np.diag(Hp[f:f + b, f:f + b]))
            assert np.abs(off).max() <= 1e-12 * scale
            w, Y = np.linalg.eig(Hp)
            X = oracle.unprepare_vectors(np.asfortranarray(Y.real), got["perm"], got["rot_first"],
                                         got["rot_size"], got["rot_values"])
            assert np.abs(H @ X - X * w.real).max() <= 1e-11 * scale
            monkeypatch.setenv("IPT_GB300_GENERAL_LIFT", "0")
            with pytest.raises(Exception):
                api.prepare_csc(cp, ri, va, n, k)
            if oracle.ref_available():
                assert isinstance(oracle.ref_prepare_lifted(cp, ri, va, n, k), int)
    assert lifted >= 15


def test_general_lift_rejects_complex_eigenvalues(lib, monkeypatch, capfd):
    """A degenerate group whose block has complex eigenvalues cannot be
    lifted by a real similarity: rejected even with the general lift, with
    the reference's diagnostic."""
    n = 12
    H = np.diag(np.arange(n, dtype=float))
    H[1, 1] = H[2, 2] = 0.5
    H[1, 2], H[2, 1] = 1e-3, -1e-3
    S = csc_matrix(H)
    S.sort_indices()
    monkeypatch.setenv("IPT_GB300_GENERAL_LIFT", "1")
    monkeypatch.setenv("IPT_DEBUG_PREPARATION", "1")
    capfd.readouterr()
    with pytest.raises(Exception):
        api.prepare_csc(S.indptr, S.indices, S.data, n, 3)
    assert "[IPT preparation] lift failed status=1" in capfd.readouterr().out
