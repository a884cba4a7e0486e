"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Every random number is a pure function of (seed, stream, i, j) through a
splitmix64 hash, so matrices are identical on any host and any thread count,
and symmetric entries come from the canonical pair (min(i,j), max(i,j)).

  dense_config0(n=1024, seed)  d_i = i + U(0,0.5) sorted ascending,
                               h_ij ~ N(0, 0.05^2) * exp(-|d_i - d_j| / 64)
  dense_config1(n=8192, seed)  d_i = i/8 + U(0,0.1),
                               h_ij ~ N(0, 0.02^2) * exp(-|i - j| / 256)
  batch_config2(count, seed)   per instance: n ~ U{64..2048}, k ~ U{4..16},
                               sigma ~ U(0.01, 0.1), config-0 construction
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x):
    with np.errstate(over="ignore"):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = x
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def _key(seed, stream):
    return _splitmix(np.uint64((seed * 0x10001 + stream) & 0xFFFFFFFFFFFFFFFF))


def _hash2(key, a, b):
    with np.errstate(over="ignore"):
        h = _splitmix(key ^ a.astype(np.uint64))
        return _splitmix(h ^ (b.astype(np.uint64) * np.uint64(0xD1B54A32D192ED03) & _M64))


def _u01(h):
    """Uniform in the open interval (0, 1) from the top 53 bits."""
    return ((h >> np.uint64(11)).astype(np.float64) + 0.5) * (2.0 ** -53)


def uniform(seed, stream, a, b=None):
    a = np.asarray(a)
    b = np.zeros_like(a) if b is None else np.asarray(b)
    return _u01(_hash2(_key(seed, stream), a, b))


def normal(seed, stream, a, b):
    """Standard normal via Box-Muller from two independent hashes."""
    u1 = uniform(seed, stream, a, b)
    u2 = uniform(seed, stream + 7919, a, b)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def _symmetric_offdiag(n, seed, sigma, decay, chunk=1024):
    """sigma * N(0,1)_{min(i,j),max(i,j)} * decay(i, j), zero diagonal."""
    H = np.empty((n, n), dtype=np.float64)
    cols = np.arange(n, dtype=np.int64)
    for r0 in range(0, n, chunk):
        rows = np.arange(r0, min(n, r0 + chunk), dtype=np.int64)[:, None]
        lo = np.minimum(rows, cols[None, :])
        hi = np.maximum(rows, cols[None, :])
        H[r0:r0 + len(rows), :] = sigma * normal(seed, 2, lo, hi) * decay(rows, cols[None, :])
    np.fill_diagonal(H, 0.0)
    return H


def dense_config0(n=1024, seed=0, sigma=0.05):
    """Plain-IPT dense case: sorted d_i = i + U(0,0.5), exp(-|d_i-d_j|/64) decay."""
    d = np.sort(np.arange(n, dtype=np.float64) + 0.5 * uniform(seed, 1, np.arange(n)))
    H = _symmetric_offdiag(n, seed, sigma, lambda i, j: np.exp(-np.abs(d[i] - d[j]) / 64.0))
    H[np.arange(n), np.arange(n)] = d
    return np.asfortranarray(H), d


def dense_config1(n=8192, seed=0, sigma=0.02):
    """Mixed-precision dense case: d_i = i/8 + U(0,0.1), exp(-|i-j|/256) decay."""
    d = np.arange(n, dtype=np.float64) / 8.0 + 0.1 * uniform(seed, 1, np.arange(n))
    H = _symmetric_offdiag(n, seed, sigma, lambda i, j: np.exp(-np.abs(i - j) / 256.0))
    H[np.arange(n), np.arange(n)] = d
    return np.asfortranarray(H), d


def batch_config2(count=512, seed=0):
    """Instance list [(n, k, sigma, seed_b)] of the batched dense workload."""
    idx = np.arange(count)
    n = 64 + np.floor(uniform(seed, 11, idx) * (2048 - 64 + 1)).astype(np.int64)
    k = 4 + np.floor(uniform(seed, 12, idx) * 13).astype(np.int64)
    sig = 0.01 + 0.09 * uniform(seed, 13, idx)
    seeds = (seed * 1000003 + idx * 7 + 1).astype(np.int64)
    return [(int(a), int(b), float(c), int(s)) for a, b, c, s in zip(n, k, sig, seeds)]


def batch_instance(n, sigma, seed):
    return dense_config0(n=n, seed=seed, sigma=sigma)


# ---------------------------------------------------------------------------
# FCI-like sparse Hamiltonians
# ---------------------------------------------------------------------------
def _strings(norb, nel):
    """Occupation bitstrings of nel electrons in norb orbitals, lexicographic."""
    from itertools import combinations
    return [sum(1 << o for o in occ) for occ in combinations(range(norb), nel)]


def _links(strings, norb, eps):
    """Single and double excitation links of every string:
    (targets, delta_eps) arrays of shape (ns, n_singles) and (ns, n_doubles),
    delta_eps = sum(eps[particles]) - sum(eps[holes])."""
    index = {s: i for i, s in enumerate(strings)}
    st, sd, dt, dd = [], [], [], []
    for s in strings:
        occ = [o for o in range(norb) if s >> o & 1]
        vir = [o for o in range(norb) if not s >> o & 1]
        t1, e1, t2, e2 = [], [], [], []
        for h in occ:
            for p in vir:
                t1.append(index[s ^ (1 << h) ^ (1 << p)])
                e1.append(eps[p] - eps[h])
        for ia in range(len(occ)):
            for ib in range(ia + 1, len(occ)):
                for pa in range(len(vir)):
                    for pb in range(pa + 1, len(vir)):
                        h1, h2, p1, p2 = occ[ia], occ[ib], vir[pa], vir[pb]
                        t2.append(index[s ^ (1 << h1) ^ (1 << h2) ^ (1 << p1) ^ (1 << p2)])
                        e2.append(eps[p1] + eps[p2] - eps[h1] - eps[h2])
        st.append(t1)
        sd.append(e1)
        dt.append(t2)
        dd.append(e2)
    return (np.array(st, np.int64), np.array(sd), np.array(dt, np.int64), np.array(dd))


def fci_like_csr(norb=10, nalpha=5, nbeta=5, seed=0, sigma=0.05):
    """FCI-like symmetric CSR matrix over all (alpha, beta) string pairs.

    Determinant I = ia * n_beta_strings + ib.  Orbital energies
    eps_p = 0.5 p + N(0, 0.05); H_II = sum of occupied eps (both spins) +
    N(0, 0.01).  H_IJ != 0 only for single and double excitations (alpha,
    beta, alpha-alpha, beta-beta, alpha-beta); its value is
    sigma * N(0,1)[seed, min(I,J), max(I,J)] * exp(-|d eps|), with d eps the
    particle-minus-hole orbital energy of the excitation (the difference of
    the two determinants' occupied-orbital energies), so H is exactly
    symmetric.  Returns (row_ptr, col_ind, values, diag) with rows sorted by
    column (int32 indices, float64 values); the diagonal is stored in the rows.
    """
    eps = 0.5 * np.arange(norb) + 0.05 * normal(seed, 31, np.arange(norb), np.zeros(norb, np.int64))
    sa = _strings(norb, nalpha)
    sb = _strings(norb, nbeta)
    na, nb = len(sa), len(sb)
    a_st, a_sd, a_dt, a_dd = _links(sa, norb, eps)
    if nbeta == nalpha:
        b_st, b_sd, b_dt, b_dd = a_st, a_sd, a_dt, a_dd
    else:
        b_st, b_sd, b_dt, b_dd = _links(sb, norb, eps)
    occ_a = np.array([sum(eps[o] for o in range(norb) if s >> o & 1) for s in sa])
    occ_b = np.array([sum(eps[o] for o in range(norb) if s >> o & 1) for s in sb])
    N = na * nb
    I = np.arange(N, dtype=np.int64)
    ia = I // nb
    ib = I % nb
    diag = occ_a[ia] + occ_b[ib] + 0.01 * normal(seed, 32, I, np.zeros(N, np.int64))
    # connected columns and d eps, grouped by excitation class
    cols = [a_st[ia] * nb + ib[:, None],                      # alpha singles
            ia[:, None] * nb + b_st[ib],                      # beta singles
            a_dt[ia] * nb + ib[:, None],                      # alpha-alpha doubles
            ia[:, None] * nb + b_dt[ib],                      # beta-beta doubles
            (a_st[ia][:, :, None] * nb + b_st[ib][:, None, :]).reshape(N, -1)]  # alpha-beta
    C = np.concatenate(cols, axis=1)
    del cols
    # |d eps| of the excitation = |E_occ(J) - E_occ(I)|, written as a
    # difference of the two determinants' occupied-orbital energies so that
    # it is bit-identical for (I, J) and (J, I)
    eocc = occ_a[ia] + occ_b[ib]
    DE = eocc[C] - eocc[:, None]
    lo = np.minimum(I[:, None], C)
    hi = np.maximum(I[:, None], C)
    V = sigma * normal(seed, 33, lo, hi) * np.exp(-np.abs(DE))
    del lo, hi, DE
    C = np.concatenate([C, I[:, None]], axis=1)
    V = np.concatenate([V, diag[:, None]], axis=1)
    order = np.argsort(C, axis=1, kind="stable")
    C = np.take_along_axis(C, order, axis=1)
    V = np.take_along_axis(V, order, axis=1)
    per = C.shape[1]
    row_ptr = (np.arange(N + 1, dtype=np.int64) * per).astype(np.int32)
    return row_ptr, C.reshape(-1).astype(np.int32), V.reshape(-1), diag


def fci_like_dims(norb, nalpha, nbeta):
    from math import comb
    return comb(norb, nalpha) * comb(norb, nbeta)


def sort_by_diagonal(row_ptr, col_ind, values, diag):
    """Symmetric permutation of a CSR matrix that makes its diagonal ascending
    (stable order), column indices sorted within rows.  Returns
    (row_ptr, col_ind, values, diag, perm) with new row r = old row perm[r]."""
    from scipy.sparse import csr_matrix
    n = len(row_ptr) - 1
    perm = np.argsort(diag, kind="stable")
    H = csr_matrix((values, col_ind, row_ptr), shape=(n, n))[perm][:, perm].tocsr()
    H.sort_indices()
    return (H.indptr.astype(np.int32), H.indices.astype(np.int32), H.data.copy(),
            np.asarray(diag)[perm], perm)


# ---------------------------------------------------------------------------
# The same constructions generated on the GPU with torch integer arithmetic
# (for benchmark-sized batches; numpy generation of the 6 GB batch takes
# tens of seconds).  Hashes and uniforms are bit-identical to the numpy
# versions; log/cos/exp round as the device's libm does (~1 ulp).
# ---------------------------------------------------------------------------
def _t_signed(v):
    """The int64 with the bits of the uint64 v."""
    v &= 0xFFFFFFFFFFFFFFFF
    return v - (1 << 64) if v >= (1 << 63) else v


_T_GOLD = _t_signed(0x9E3779B97F4A7C15)
_T_M1 = _t_signed(0xBF58476D1CE4E5B9)
_T_M2 = _t_signed(0x94D049BB133111EB)
_T_M3 = _t_signed(0xD1B54A32D192ED03)


def _t_srl(x, s):
    """Logical right shift of int64 tensors."""
    return (x >> s) & ((1 << (64 - s)) - 1)


def _t_splitmix(x):
    x = x + _T_GOLD
    z = (x ^ _t_srl(x, 30)) * _T_M1
    z = (z ^ _t_srl(z, 27)) * _T_M2
    return z ^ _t_srl(z, 31)


def _t_uniform(torch, seed, stream, a, b):
    key = int(_key(seed, stream))
    h = _t_splitmix(torch.bitwise_xor(a, _t_signed(key)))
    h = _t_splitmix(h ^ (b * _T_M3))
    return (_t_srl(h, 11).to(torch.float64) + 0.5) * (2.0 ** -53)


def batch_instance_torch(torch, n, sigma, seed, device="cuda"):
    """dense_config0(n, seed, sigma) built on the device: (H column-major as an
    n x n tensor whose storage is H^T = H, d)."""
    i = torch.arange(n, dtype=torch.int64, device=device)
    d = i.to(torch.float64) + 0.5 * _t_uniform(torch, seed, 1, i, torch.zeros_like(i))
    # d is increasing by construction (i + U(0, 0.5)), so the sort is the identity
    lo = torch.minimum(i[:, None], i[None, :])
    hi = torch.maximum(i[:, None], i[None, :])
    u1 = _t_uniform(torch, seed, 2, lo, hi)
    u2 = _t_uniform(torch, seed, 2 + 7919, lo, hi)
    H = sigma * torch.sqrt(-2.0 * torch.log(u1)) * torch.cos(2.0 * torch.pi * u2)
    H *= torch.exp(-torch.abs(d[:, None] - d[None, :]) / 64.0)
    H.fill_diagonal_(0.0)
    H += torch.diag(d)
    return H, d
