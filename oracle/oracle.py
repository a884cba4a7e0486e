"""Python access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker of the CUDA solver and the CPU baseline of
bench.py; the product (block_ipt_gb300) never imports it.  It offers:

  * the C restatement of the reference IPT path (oracle/ipt_oracle.c, built
    into oracle/_build/liboracle.so), each function citing the reference;
  * the reference's own CPU test code compiled from its sources into
    oracle/_ref/ (only where the reference tree exists, see build_ref.py);
  * FP64 numpy references for the block path: CholQR, Rayleigh-Ritz and the
    LAPACK (scipy) dsyevd eigenpairs used as the eigen-oracle.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DENSE = os.path.join(HERE, "_ref", "libref_dense.so")
REF_SPARSE = os.path.join(HERE, "_ref", "libref_sparse.so")

_lib = None
_ref = {}


def build():
    """Compile the C oracle (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        L.oracle_deterministic_noise.restype = d
        L.oracle_deterministic_noise.argtypes = [i, i]
        L.oracle_fill_perturbative_matrix.argtypes = [vp, i, i]
        L.oracle_build_banded_csc.restype = i
        L.oracle_build_banded_csc.argtypes = [i, vp, vp, vp]
        L.oracle_ipt_dense.restype = i
        L.oracle_ipt_dense.argtypes = [vp, i, i, i, d, i, vp, vp, vp, vp, vp]
        L.oracle_ipt_csr.restype = i
        L.oracle_ipt_csr.argtypes = [vp, vp, vp, vp, i, i, i, d, i, vp, vp, vp, vp, vp]
        L.oracle_matmul.argtypes = [vp, vp, vp, i, i]
        L.oracle_csc_to_dense.argtypes = [vp, vp, vp, vp, i]
        L.oracle_max_relative_residual.restype = d
        L.oracle_max_relative_residual.argtypes = [vp, vp, vp, i, i]
        L.oracle_validate_csc.restype = i
        L.oracle_validate_csc.argtypes = [vp, vp, i, i]
        L.oracle_csc_diagonal.argtypes = [vp, vp, vp, i, vp]
        L.oracle_stable_sort_permutation.argtypes = [vp, i, vp]
        L.oracle_csc_matmul.argtypes = [vp, vp, vp, i, vp, i, vp]
        L.oracle_csr_matmul.argtypes = [vp, vp, vp, i, vp, i, vp]
        L.oracle_ipt_dense_products_to_residual.restype = i
        L.oracle_ipt_dense_products_to_residual.argtypes = [vp, i, i, i, d, d, vp]
        L.oracle_num_threads.restype = i
        L.oracle_set_num_threads.argtypes = [i]
        L.oracle_acx_mixed.restype = i
        L.oracle_acx_mixed.argtypes = [vp, i, i, d, i, d, i, vp, vp, vp, vp]
        L.oracle_acx_dense.restype = i
        L.oracle_acx_dense.argtypes = [vp, i, i, d, i, vp, vp, vp, vp]
        L.oracle_cluster_update.restype = i
        L.oracle_cluster_update.argtypes = [vp, vp, vp, i, i, i, d, vp]
        L.oracle_cluster_basis.restype = i
        L.oracle_cluster_basis.argtypes = [vp, vp, vp, vp, i, vp, i, i, d, d, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


# ---- reference test inputs -------------------------------------------------
def perturbative_matrix(n, symmetric):
    """IPT_C_GPU/test_temp/runtests.cu:60-80."""
    H = np.zeros((n, n), dtype=np.float64, order="F")
    lib().oracle_fill_perturbative_matrix(_p(H), n, int(symmetric))
    return H


def banded_csc(n):
    """IPT_C_GPU/test/sparse/runtests_sparse.cu:224-268."""
    nnz = n + 2 * (n - 1)
    cp = np.zeros(n + 1, dtype=np.int32)
    ri = np.zeros(nnz, dtype=np.int32)
    va = np.zeros(nnz, dtype=np.float64)
    got = lib().oracle_build_banded_csc(n, _p(cp), _p(ri), _p(va))
    assert got == nnz
    return cp, ri, va


def csc_to_dense(cp, ri, va, n):
    H = np.zeros((n, n), dtype=np.float64, order="F")
    lib().oracle_csc_to_dense(_p(H), _p(np.ascontiguousarray(cp, np.int32)),
                              _p(np.ascontiguousarray(ri, np.int32)),
                              _p(np.ascontiguousarray(va, np.float64)), n)
    return H


# ---- plain IPT ---------------------------------------------------------------
def ipt_dense(H, k, maxiter, tol=0.0, use_tol=False, x0=None):
    """Plain IPT (runtests.cu:98-174; tolerance rule of ipt_cuda.cu:1883-1932).
    Returns (vectors n x k, values k, iterations, fixed_point_residual)."""
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    X = np.zeros((n, k), dtype=np.float64, order="F")
    v = np.zeros(k, dtype=np.float64)
    it = C.c_int(0)
    fp = C.c_double(0.0)
    x0a = None if x0 is None else np.asfortranarray(x0, dtype=np.float64)
    st = lib().oracle_ipt_dense(_p(H), n, k, maxiter, float(tol), int(use_tol), _p(x0a), _p(X),
                                _p(v), C.byref(it), C.byref(fp))
    if st != 0:
        raise RuntimeError("oracle_ipt_dense failed: %d" % st)
    return X, v, it.value, fp.value


def ipt_csr(row_ptr, col_ind, vals, diag, n, k, maxiter, tol=0.0, use_tol=False, x0=None):
    rp = np.ascontiguousarray(row_ptr, np.int32)
    ci = np.ascontiguousarray(col_ind, np.int32)
    va = np.ascontiguousarray(vals, np.float64)
    dg = np.ascontiguousarray(diag, np.float64)
    X = np.zeros((n, k), dtype=np.float64, order="F")
    v = np.zeros(k, dtype=np.float64)
    it = C.c_int(0)
    fp = C.c_double(0.0)
    x0a = None if x0 is None else np.asfortranarray(x0, dtype=np.float64)
    st = lib().oracle_ipt_csr(_p(rp), _p(ci), _p(va), _p(dg), n, k, maxiter, float(tol),
                              int(use_tol), _p(x0a), _p(X), _p(v), C.byref(it), C.byref(fp))
    if st != 0:
        raise RuntimeError("oracle_ipt_csr failed: %d" % st)
    return X, v, it.value, fp.value


def products_to_residual(H, k, maxiter, res_tol=1e-8):
    """Block products plain IPT needs until the scaled eigen-residual of its
    iterate is <= res_tol (-1 if not within maxiter); see ipt_oracle.c."""
    H = np.asfortranarray(H, dtype=np.float64)
    hn = float(np.abs(H).sum(axis=1).max())
    fr = C.c_double(0.0)
    got = lib().oracle_ipt_dense_products_to_residual(_p(H), H.shape[0], k, maxiter, hn,
                                                      float(res_tol), C.byref(fr))
    return got, fr.value


def num_threads():
    return lib().oracle_num_threads()


def set_num_threads(threads):
    """Thread count of the oracle's following calls."""
    lib().oracle_set_num_threads(int(threads))


def max_relative_residual(H, X, v):
    """IPT_C_GPU/test_temp/runtests.cu:191-229."""
    H = np.asfortranarray(H, dtype=np.float64)
    X = np.asfortranarray(X, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    return lib().oracle_max_relative_residual(_p(H), _p(X), _p(v), H.shape[0], X.shape[1])


def prepare_sorted_csc(cp, ri, va, n):
    """Stable diagonal sort + symmetric permutation with duplicate merge and
    zero drop (IPT_C_GPU/src/ipt_preparation.cu:190-262, 1375-1431).
    Returns (row_ptr, col_ind, vals) as CSR of the sorted matrix, the summed
    sorted diagonal, and perm (perm[sorted] = original)."""
    cp = np.ascontiguousarray(cp, np.int32)
    ri = np.ascontiguousarray(ri, np.int32)
    va = np.ascontiguousarray(va, np.float64)
    diag = np.zeros(n)
    lib().oracle_csc_diagonal(_p(cp), _p(ri), _p(va), n, _p(diag))
    perm = np.zeros(n, dtype=np.int32)
    lib().oracle_stable_sort_permutation(_p(diag), n, _p(perm))
    inv = np.empty(n, dtype=np.int64)
    inv[perm] = np.arange(n)
    cols = np.repeat(np.arange(n), np.diff(cp))
    nr = inv[ri]
    nc = inv[cols]
    A = {}
    for r, c, v in zip(nr.tolist(), nc.tolist(), va.tolist()):
        A[(r, c)] = A.get((r, c), 0.0) + v
    keys = sorted(k for k, v in A.items() if v != 0.0 or (perm == np.arange(n)).all())
    rp = np.zeros(n + 1, dtype=np.int32)
    for r, _ in keys:
        rp[r + 1] += 1
    rp = np.cumsum(rp).astype(np.int32)
    ci = np.array([c for _, c in keys], dtype=np.int32)
    vv = np.array([A[k] for k in keys], dtype=np.float64)
    d = np.zeros(n)
    for (r, c), v in A.items():
        if r == c:
            d[r] += v
    return rp, ci, vv, d, perm


# ---- FP64 eigen-oracle and block references ------------------------------------
def eigh_lowest(H, k):
    """LAPACK (scipy) symmetric eigensolver: k lowest pairs, ascending."""
    import scipy.linalg as sl
    w, V = sl.eigh(np.asarray(H, dtype=np.float64), subset_by_index=[0, k - 1], driver="evr")
    return w, V


def dsyevd_lowest(H, k):
    """LAPACK dsyevd (divide and conquer), full spectrum, the k lowest."""
    from scipy.linalg import lapack
    w, V, info = lapack.dsyevd(np.asarray(H, dtype=np.float64), compute_v=1, lower=1)
    if info != 0:
        raise RuntimeError("dsyevd info=%d" % info)
    return w[:k], V[:, :k]


def rayleigh_mixed(H, k, lowp_tol, lowp_maxiter, fp64_tol, fp64_maxiter):
    """The reference's Rayleigh-mixed driver
    (IPT_C_GPU/src/mixed_precision/ipt_rayleigh_mixed_cuda.cu:274-400) with an
    FP64 first stage in place of its TF32 one: plain IPT to lowp_tol, the
    Householder QR of that block (LAPACK dgeqrf/dorgqr through numpy, the
    convention of its cusolverDnDgeqrf/Dorgqr, :141-254), B = sym(Q^T H Q)
    (:84-106, :338-343), plain IPT on the k x k matrix B to fp64_tol (:358)
    and the vectors Q Z (:370).  Returns (vectors, values, Q, fp64 iterations,
    fp64 fixed-point residual)."""
    X0, _, _, _ = ipt_dense(H, k, lowp_maxiter, tol=lowp_tol, use_tol=True)
    Q, _ = np.linalg.qr(X0)
    B = Q.T @ (np.asarray(H, dtype=np.float64) @ Q)
    B = 0.5 * (B + B.T)
    Z, vals, it, fp = ipt_dense(B, k, fp64_maxiter, tol=fp64_tol, use_tol=True)
    return Q @ Z, vals, Q, it, fp


# ---- split-operand FP64-accurate product ------------------------------------
# Restatement of the library's error-free split (block_ipt_gb300/csrc/oz.cuh),
# itself the fixed-point form of Ozaki, Ogita, Oishi and Rump (Numer.
# Algorithms 59, 2012): checker only.
OZ_SLICES = 6
OZ_NONFINITE = 0x7FFFFFFF


def accurate_exponent(max_abs):
    """Smallest e with |max_abs| < 2^e (0 for 0, OZ_NONFINITE for Inf/NaN)."""
    b = int(np.array([max_abs], dtype=np.float64).view(np.uint64)[0]) & 0x7FFFFFFFFFFFFFFF
    if b == 0:
        return 0
    E = b >> 52
    if E == 2047:
        return OZ_NONFINITE
    if E == 0:
        return b.bit_length() + 0 - 1074
    return E - 1022


def accurate_fixed(values, e):
    """round(v 2^(48 - e)) (half away from zero) as int64; 0 for non-finite."""
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    out = np.zeros(v.size, dtype=np.int64)
    if e == OZ_NONFINITE:
        return out
    for idx, b in enumerate(v.view(np.uint64).tolist()):
        neg = b >> 63
        b &= 0x7FFFFFFFFFFFFFFF
        E = b >> 52
        if E == 2047 or b == 0:
            continue
        if E == 0:
            M, x = b, -1074
        else:
            M, x = (b & 0xFFFFFFFFFFFFF) | (1 << 52), E - 1075
        sh = e - 48 - x
        if sh >= 60:
            q = 0
        elif sh > 0:
            q = (M >> sh) + ((M >> (sh - 1)) & 1)
        else:
            q = M << (-sh)
        out[idx] = -q if neg else q
    return out


def accurate_digits(q):
    """Balanced base-256 digits [count, 6] of fixed-point values (s = 0 most
    significant; digit 0 in [-256, 256], the others in [-128, 127])."""
    q = np.array(q, dtype=np.int64)
    d = np.zeros((q.size, OZ_SLICES), dtype=np.int64)
    for s in range(OZ_SLICES - 1, 0, -1):
        r = ((q + 128) & 255) - 128
        d[:, s] = r
        q = (q - r) >> 8
    d[:, 0] = q
    return d


def accurate_product_emulated(H, X):
    """The split-operand product as the library defines it, in exact
    integer arithmetic rounded once at the end: Delta = H - diag(H) split
    per row, X per column, the digit pairs of levels 0..5 summed exactly,
    plus diag(H) X in FP64."""
    H = np.asarray(H, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    n, c = H.shape[0], X.shape[1]
    D = H.copy()
    np.fill_diagonal(D, 0.0)
    er = [accurate_exponent(np.abs(D[i]).max()) for i in range(n)]
    fc = [accurate_exponent(np.abs(X[:, j]).max()) for j in range(c)]
    A = np.stack([accurate_digits(accurate_fixed(D[i], er[i])) for i in range(n)])  # n, n, 6
    B = np.stack([accurate_digits(accurate_fixed(X[:, j], fc[j])) for j in range(c)])  # c, n, 6
    levels = [np.zeros((n, c)) for _ in range(OZ_SLICES)]
    for s in range(OZ_SLICES):
        for t in range(OZ_SLICES - s):
            # digit products < 2^16, sums over n < 2^53: exact in FP64
            levels[s + t] += A[:, :, s].astype(np.float64) @ B[:, :, t].T.astype(np.float64)
    Y = np.empty((n, c))
    d = np.diag(H)
    for i in range(n):
        for j in range(c):
            if er[i] == OZ_NONFINITE or fc[j] == OZ_NONFINITE:
                Y[i, j] = np.nan
                continue
            V = 0
            for l in range(OZ_SLICES):
                V += int(levels[l][i, j]) << (8 * (OZ_SLICES - 1 - l))
            y = float(np.ldexp(float(V), er[i] + fc[j] - 16 - 8 * (OZ_SLICES - 1)))
            Y[i, j] = y + d[i] * X[i, j]
    return Y


def cholqr(X):
    """CholQR: X = Q R with R from the FP64 Gram matrix."""
    G = X.T @ X
    R = np.linalg.cholesky(G).T
    return np.linalg.solve(R.T, X.T).T


def rayleigh_ritz(H, V, k):
    """Ritz pairs of H on span(V) (V orthonormal): ascending values."""
    T = V.T @ (H @ V)
    T = 0.5 * (T + T.T)
    w, Z = np.linalg.eigh(T)
    return w[:k], V @ Z[:, :k]


def scaled_residuals(H_apply, X, w, hnorm):
    """||H x_j - w_j x_j|| / (max(1,||H||_inf) max(1,||x_j||))
    (IPT_C_GPU/src/ipt_cuda.cu:2684-2697)."""
    R = H_apply(X) - X * w[None, :]
    return np.linalg.norm(R, axis=0) / (max(1.0, hnorm) * np.maximum(1.0, np.linalg.norm(X, axis=0)))


# ---- the reference's own compiled CPU code (checker only) -------------------------
def ref_available():
    return os.path.exists(REF_DENSE) and os.path.exists(REF_SPARSE)


def ref_lib(which):
    if which not in _ref:
        path = REF_DENSE if which == "dense" else REF_SPARSE
        L = C.CDLL(path)
        vp, i = C.c_void_p, C.c_int
        if which == "dense":
            L.ref_ipt_cpu_reference.restype = i
            L.ref_ipt_cpu_reference.argtypes = [vp, i, i, i, vp, vp]
            L.ref_fill_perturbative_matrix.argtypes = [vp, i, i]
            L.ref_result_layout.restype = i
            L.ref_result_layout.argtypes = [vp, i]
        else:
            L.ref_sparse_ipt_cpu_reference.restype = i
            L.ref_sparse_ipt_cpu_reference.argtypes = [vp, i, i, i, vp, vp]
            L.ref_build_banded_csc.restype = i
            L.ref_build_banded_csc.argtypes = [i, vp, vp, vp]
            L.ref_h20_w_csc.restype = i
            L.ref_h20_w_csc.argtypes = [vp, vp, vp]
            L.ref_prepare_sparse_csc_sorted.restype = i
            L.ref_prepare_sparse_csc_sorted.argtypes = [vp, vp, vp, i, i, i, vp, vp, vp, vp, vp]
            L.ref_prepare_sparse_csc_lifted.restype = i
            L.ref_prepare_sparse_csc_lifted.argtypes = [vp, vp, vp, i, i, i, C.c_double, vp, vp,
                                                        vp, i, vp, vp, vp, vp, vp, i, i, vp, vp,
                                                        i]
            L.ref_block_cluster_prepare.restype = i
            L.ref_block_cluster_prepare.argtypes = [vp, vp, vp, i, i, i, vp, i, vp, vp, i, vp]
            L.ref_block_cluster_solve_basis.restype = i
            L.ref_block_cluster_solve_basis.argtypes = [vp, vp, vp, i, i, vp, i, i, i,
                                                        C.c_double, C.c_double, vp, vp]
        _ref[which] = L
    return _ref[which]


# ---- ACX extrapolation ------------------------------------------------------------
def acx_dense(H, k, tol, maxiter):
    """ACX over the dense IPT map (oracle_acx_dense): (vectors, values, info,
    status) with info = iterations, f_calls, converged, max_residual,
    fixed_point_residual."""
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    X = np.zeros((n, k), dtype=np.float64, order="F")
    v = np.zeros(k)
    info = np.zeros(3, dtype=np.int32)
    res = np.zeros(2)
    st = lib().oracle_acx_dense(_p(H), n, k, tol, maxiter, _p(X), _p(v), _p(info), _p(res))
    return X, v, {"iterations": int(info[0]), "f_calls": int(info[1]),
                  "converged": int(info[2]), "max_residual": float(res[0]),
                  "fixed_point_residual": float(res[1])}, st


def acx_mixed(H, k, tf32_tol, tf32_maxiter, fp64_tol, fp64_maxiter):
    """Mixed ACX (oracle_acx_mixed): (vectors, values, info, status)."""
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[0]
    X = np.zeros((n, k), dtype=np.float64, order="F")
    v = np.zeros(k)
    info = np.zeros(6, dtype=np.int32)
    res = np.zeros(3)
    st = lib().oracle_acx_mixed(_p(H), n, k, tf32_tol, tf32_maxiter, fp64_tol, fp64_maxiter,
                                _p(X), _p(v), _p(info), _p(res))
    keys = ("tf32_iterations", "tf32_f_calls", "tf32_converged", "fp64_iterations",
            "fp64_f_calls", "fp64_converged")
    out = {kk: int(x) for kk, x in zip(keys, info)}
    out.update({"tf32_fixed_point_residual": float(res[0]), "fp64_max_residual": float(res[1]),
                "fp64_fixed_point_residual": float(res[2])})
    return X, v, out, st


def acx_rayleigh(H, k, lowp_tol, lowp_maxiter, fp64_tol, fp64_maxiter):
    """The reference's Rayleigh ACX driver
    (IPT_C_GPU/src/ACX/acx_rayleigh_mixed_precision_cuda.cu:289-434) with an
    FP64 first stage in place of its TF32 one: ACX to lowp_tol, Householder
    QR of that block (numpy = LAPACK dgeqrf/dorgqr, the convention of its
    cusolverDnDgeqrf/Dorgqr), B = sym(Q^T H Q), FP64 ACX on B to fp64_tol
    and the vectors Q Z.  Returns (vectors, values, Q, info of the FP64 stage,
    status)."""
    X0, _, _, st = acx_dense(H, k, lowp_tol, lowp_maxiter)
    if st != 0:
        return None, None, None, None, st
    Q, _ = np.linalg.qr(X0)
    B = Q.T @ (np.asarray(H, dtype=np.float64) @ Q)
    B = 0.5 * (B + B.T)
    Z, vals, info, st = acx_dense(B, k, fp64_tol, fp64_maxiter)
    return (Q @ Z if st == 0 else None), vals, Q, info, st


def acx_test_matrix(n, epsilon, seed):
    """Symmetric dense matrix of the reference's ACX benchmark shape
    (IPT_C_GPU/test/ACX/benchmark_acx_cuda_sweep.cu:284-313): diagonal
    row + 1 + eps u, off-diagonal eps (u_ij + u_ji) / 2, with u uniform in
    [0, 1) from numpy's seeded generator standing in for its hash."""
    rng = np.random.default_rng(seed)
    U = rng.uniform(size=(n, n))
    H = 0.5 * epsilon * (U + U.T)
    H[np.diag_indices(n)] = np.arange(1, n + 1) + epsilon * np.diag(U)
    return np.asfortranarray(H)


def _splitmix64_u64(x):
    """splitmix64 on numpy uint64 arrays (wrapping arithmetic)."""
    x = x + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


ACX_SWEEP_SEED = 20260615


def acx_sweep_matrix(n, epsilon, base_seed=ACX_SWEEP_SEED):
    """The matrix of the reference's ACX sweep benchmark, bit for bit:
    seed = base_seed + n + splitmix64(bits(epsilon)) mod 1000000007
    (IPT_C_GPU/test/ACX/benchmark_acx_cuda_sweep.cu:25,273-282,880-882);
    u(row, col) = splitmix64(seed + n c1 ^ (row+1) c2 ^ (col+1) c3) >> 11
    scaled to [0, 1) (:256-271); diagonal row + 1 + eps u(row, row),
    off-diagonal eps (u(row, col) + u(col, row)) / 2 (:284-313)."""
    with np.errstate(over="ignore"):
        ebits = np.array([epsilon], dtype=np.float64).view(np.uint64)
        off = int(_splitmix64_u64(ebits)[0]) % 1000000007
        seed = np.uint64((base_seed + n + off) & 0xFFFFFFFFFFFFFFFF)
        base = seed + np.uint64(n) * np.uint64(0xD1B54A32D192ED03)
        r = (np.arange(n, dtype=np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        c = (np.arange(n, dtype=np.uint64) + np.uint64(1)) * np.uint64(0xBF58476D1CE4E5B9)
        x = (base ^ r[:, None]) ^ c[None, :]  # x[row, col]
        U = (_splitmix64_u64(x) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    H = 0.5 * epsilon * (U + U.T)
    H[np.diag_indices(n)] = np.arange(1, n + 1) + epsilon * np.diag(U)
    return np.asfortranarray(H)


# ---- the reference's binary CSC matrix cache -------------------------------------
def reference_csc_cache_bytes(magic, cp, ri, va, dg, norm, counts=(0, 0, 0, 0, 0, 0), version=1):
    """A cache file as the reference's benchmarks write it: the header struct
    (IPT_C_GPU/test/sparse/CH4/benchmark_ch4_sto6g_fci_15876_ipt.cu:182-194,
    natural alignment: four zero bytes after nnz, 56 bytes) and the arrays in
    the order of its writer (:1015-1066)."""
    import struct
    n, nnz = len(cp) - 1, len(ri)
    head = struct.pack("<8sIii4xd6i", magic, version, n, nnz, norm, *counts)
    return (head + np.asarray(cp, "<i4").tobytes() + np.asarray(ri, "<i4").tobytes()
            + np.asarray(va, "<f8").tobytes() + np.asarray(dg, "<f8").tobytes())


def parse_reference_csc_cache(data):
    """Parse cache bytes the way the reference's inspection script does
    (IPT_C_GPU/results/sparse/CH4_K30_debug/inspect_csc_bin.py:7-57)."""
    import struct
    magic, mol, version, n = struct.unpack_from("<4s4sii", data, 0)
    nnz = struct.unpack_from("<q", data, 16)[0]
    norm = struct.unpack_from("<d", data, 24)[0]
    counts = struct.unpack_from("<iiiiii", data, 32)
    o = 56
    cp = np.frombuffer(data, "<i4", n + 1, o)
    o += 4 * (n + 1)
    ri = np.frombuffer(data, "<i4", nnz, o)
    o += 4 * nnz
    va = np.frombuffer(data, "<f8", nnz, o)
    o += 8 * nnz
    dg = np.frombuffer(data, "<f8", n, o)
    assert o + 8 * n == len(data)
    return {"magic": (magic + mol).decode(), "version": version, "n": n, "nnz": nnz,
            "norm": norm, "counts": counts, "col_ptr": cp, "row_ind": ri, "values": va,
            "diag": dg}


# ---- block-cluster path ---------------------------------------------------------
def cluster_test_matrix(n, seed, coupling=0.05, groups=3, density=0.05):
    """Symmetric CSC test matrix for the block-cluster path: ascending
    diagonal with planted exact and near (1e-13) degeneracies among the
    lowest entries, random symmetric off-diagonal entries of the given
    scale.  Returns (col_ptr, row_ind, values, dense H)."""
    rng = np.random.default_rng(seed)
    d = np.sort(rng.uniform(0, n, n))
    for g in range(groups):
        i = int(rng.integers(0, min(n - 4, 12)))
        w = int(rng.integers(2, 4))
        d[i:i + w] = d[i] + (rng.uniform(0, 1e-13, w) if g % 2 else 0.0)
    d = np.sort(d)
    mask = rng.uniform(size=(n, n)) < density
    A = np.triu(np.where(mask, rng.normal(scale=coupling, size=(n, n)), 0.0), 1)
    H = np.diag(d) + A + A.T
    cp, ri, va = [0], [], []
    for c in range(n):
        for r in range(n):
            if H[r, c] != 0.0 or r == c:
                ri.append(r)
                va.append(H[r, c])
        cp.append(len(ri))
    return (np.array(cp, np.int32), np.array(ri, np.int32), np.array(va, np.float64),
            np.asfortranarray(H))


def cluster_update(basis, y, diag, first, damping=1.0):
    """One block-cluster update (oracle_cluster_update); returns (next, singular)."""
    basis = np.asfortranarray(basis, dtype=np.float64)
    y = np.asfortranarray(y, dtype=np.float64)
    diag = np.ascontiguousarray(diag, dtype=np.float64)
    n, m = basis.shape
    nxt = np.zeros((n, m), dtype=np.float64, order="F")
    s = lib().oracle_cluster_update(_p(basis), _p(y), _p(diag), n, first, m, damping, _p(nxt))
    return nxt, bool(s)


def cluster_basis(row_ptr, col_ind, vals, diag, ranges, maxiter, tol, damping=1.0):
    """Block-cluster basis of every cluster (oracle_cluster_basis); returns
    (basis, iterations, residuals, status) with status 0 or 1 + the failing
    cluster."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_ind, dtype=np.int32)
    va = np.ascontiguousarray(vals, dtype=np.float64)
    dg = np.ascontiguousarray(diag, dtype=np.float64)
    rg = np.ascontiguousarray(np.asarray(ranges, dtype=np.int32).reshape(-1))
    C_ = rg.size // 2
    n = rp.size - 1
    cols = int(sum(rg[2 * c + 1] - rg[2 * c] + 1 for c in range(C_)))
    X = np.zeros((n, cols), dtype=np.float64, order="F")
    it = np.zeros(C_, dtype=np.int32)
    res = np.zeros(C_, dtype=np.float64)
    st = lib().oracle_cluster_basis(_p(rp), _p(ci if ci.size else np.zeros(1, np.int32)),
                                    _p(va if va.size else np.zeros(1)), _p(dg), n, _p(rg), C_,
                                    maxiter, tol, damping, _p(X), _p(it), _p(res))
    return X, it, res, st


def cluster_ranges(cp, ri, va, n, k, requested_k=None, threshold=0.0, adaptive=False,
                   tau=0.1, eps_multiplier=1000.0, rel_gap_tol=1e-12, ratio_tol=0.2,
                   eta=0.02, max_block=64):
    """Cluster ranges of the block-cluster path for a CSC matrix with
    ascending diagonal, restated in Python (small n): degenerate-subspace
    detection IPT_C_GPU/src/ipt_preparation.cu:345-644, singleton targets
    IPT_C_GPU/src/ipt_cuda.cu:4114-4132, adaptive expansion :4134-4272.
    Returns (ranges, added, limit_hit, too_large)."""
    import math
    requested_k = k if requested_k is None else requested_k
    eps = np.finfo(np.float64).eps
    diag = [0.0] * n
    for c in range(n):
        for p_ in range(cp[c], cp[c + 1]):
            if ri[p_] == c:
                diag[c] = float(va[p_])
                break
    tau_num = eps_multiplier * eps * max(1.0, max(abs(x) for x in diag))
    rt = max(ratio_tol, eps)
    cs = [0.0] * n
    rs = [0.0] * n
    for c in range(n):
        for p_ in range(cp[c], cp[c + 1]):
            r = int(ri[p_])
            if r != c:
                cs[c] = max(cs[c], abs(va[p_]))
                rs[r] = max(rs[r], abs(va[p_]))
    off = [max(cs[i], rs[i]) for i in range(n)]

    def floor_(a, b):
        return max(max(threshold, tau_num), rel_gap_tol * max(1.0, abs(a), abs(b)))

    def entry(r, c):
        for p_ in range(cp[c], cp[c + 1]):
            if ri[p_] == r:
                return float(va[p_])
        return 0.0

    parent = list(range(n))
    rank = [0] * n

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    def unite(a, b):
        a, b = find(a), find(b)
        if a == b:
            return
        if rank[a] < rank[b]:
            a, b = b, a
        parent[b] = a
        if rank[a] == rank[b]:
            rank[a] += 1

    order = sorted(range(n), key=lambda i: (diag[i], i))
    for col in range(min(k, n)):
        dc = diag[col]
        w = max(floor_(dc, dc), off[col] / rt)
        for row in order:
            dr = diag[row]
            if row == col or dr < dc - w or dr > dc + w:
                continue
            cpl = max(abs(entry(row, col)), abs(entry(col, row)))
            if not cpl > 0.0:
                cpl = eta * min(off[row], off[col])
            gap = abs(dr - dc)
            fl = floor_(dr, dc)
            if gap <= fl or (cpl > 0.0 and cpl / max(gap, fl) >= rt):
                unite(row, col)
    comp = {}
    for i in range(n):
        r = find(i)
        lo, hi, t = comp.get(r, (n, -1, False))
        comp[r] = (min(lo, i), max(hi, i), t or i < k)
    rg = sorted((lo, hi) for lo, hi, t in comp.values() if t and lo < hi)
    merged = []
    for a, b in rg:
        if merged and a <= merged[-1][1] + 1:
            merged[-1] = (merged[-1][0], max(merged[-1][1], b))
        else:
            merged.append((a, b))
    too_large = any(b - a + 1 > max_block for a, b in merged)
    covered = set()
    for a, b in merged:
        covered.update(range(a, b + 1))
    merged += [(t, t) for t in range(min(k, n)) if t not in covered]
    ranges = sorted(merged)
    added, limit_hit = [], False
    if adaptive and not too_large:
        def degenerate(a, b):
            g = max(1e-14, 1000.0 * eps * max(1.0, abs(diag[a]), abs(diag[b])))
            return abs(diag[a] - diag[b]) <= g
        while True:
            tid = next((i for i, (a, b) in enumerate(ranges) if a <= requested_k - 1 <= b), -1)
            if tid < 0:
                break
            first, last = ranges[tid]
            best, best_row = 0.0, -1
            for col in range(first, last + 1):
                for p_ in range(cp[col], cp[col + 1]):
                    row = int(ri[p_])
                    if first <= row <= last:
                        continue
                    ratio = abs(va[p_]) / max(abs(diag[col] - diag[row]), 1e-14)
                    if max(last, row) - min(first, row) + 1 > max_block:
                        limit_hit = limit_hit or ratio > tau
                        continue
                    if ratio > best:
                        best, best_row = ratio, row
            if best_row < 0 or best <= tau:
                break
            pf, pl = min(first, best_row), max(last, best_row)
            grew = True
            while grew:
                grew = False
                if pf > 0 and degenerate(pf, pf - 1):
                    pf -= 1
                    grew = True
                if pl + 1 < n and degenerate(pl, pl + 1):
                    pl += 1
                    grew = True
            if pl - pf + 1 > max_block:
                limit_hit = True
                break
            added += [i for i in range(pf, pl + 1) if i < first or i > last]
            ranges[tid] = (pf, pl)
            ranges.sort()
            m2 = []
            for a, b in ranges:
                if not m2 or a > m2[-1][1]:
                    m2.append((a, b))
                else:
                    m2[-1] = (m2[-1][0], max(m2[-1][1], b))
            ranges = m2
    del math
    return ranges, sorted(set(added)), limit_hit, too_large


def ref_cluster_prepare(cp, ri, va, n, k):
    """The reference's own block-cluster preparation (needs oracle/_ref):
    ranges of the diagonal-sorted matrix, (ranges, added, limit_hit) or a
    negative status."""
    L = ref_lib("sparse")
    cp = np.ascontiguousarray(cp, dtype=np.int32)
    ri = np.ascontiguousarray(ri, dtype=np.int32)
    va = np.ascontiguousarray(va, dtype=np.float64)
    cap = n
    rg = np.zeros(2 * cap, dtype=np.int32)
    lim = np.zeros(1, dtype=np.int32)
    added = np.zeros(n, dtype=np.int32)
    na = np.zeros(1, dtype=np.int32)
    cnt = L.ref_block_cluster_prepare(_p(cp), _p(ri), _p(va), n, k, int(cp[-1]), _p(rg), cap,
                                      _p(lim), _p(added), n, _p(na))
    if cnt < 0:
        return cnt
    return ([(int(rg[2 * i]), int(rg[2 * i + 1])) for i in range(cnt)],
            [int(x) for x in added[:na[0]]], bool(lim[0]))


def ref_prepare_lifted(cp, ri, va, n, k, threshold=0.0, vectors=None):
    """The reference's plain-path preparation with degeneracy lifting (needs
    oracle/_ref): a dict of the prepared CSC, diagonal, permutation and
    rotations, with the back-transformed copy of `vectors` (prepared basis ->
    caller's basis) when given; a negative status when it fails."""
    L = ref_lib("sparse")
    cp = np.ascontiguousarray(cp, dtype=np.int32)
    ri = np.ascontiguousarray(ri, dtype=np.int32)
    va = np.ascontiguousarray(va, dtype=np.float64)
    cap = max(4 * ri.size, n * n, 16)
    ocp = np.zeros(n + 1, np.int32)
    ori = np.zeros(cap, np.int32)
    ova = np.zeros(cap)
    od = np.zeros(n)
    op = np.zeros(n, np.int32)
    rf = np.zeros(n, np.int32)
    rs = np.zeros(n, np.int32)
    rv = np.zeros(max(1, 64 * 64 * n))
    rc = np.zeros(1, np.int32)
    V = None if vectors is None else np.array(vectors, dtype=np.float64, order="F", copy=True)
    nnz = L.ref_prepare_sparse_csc_lifted(_p(cp), _p(ri), _p(va), n, k, int(cp[-1]), threshold,
                                          _p(ocp), _p(ori), _p(ova), cap, _p(od), _p(op), _p(rf),
                                          _p(rs), _p(rv), n, rv.size, _p(rc), _p(V),
                                          0 if V is None else V.shape[1])
    if nnz < 0:
        return nnz
    r = int(rc[0])
    return {"col_ptr": ocp, "row_ind": ori[:nnz], "values": ova[:nnz], "diag": od, "perm": op,
            "rot_first": rf[:r], "rot_size": rs[:r],
            "rot_values": rv[:int(sum(int(m) * int(m) for m in rs[:r]))], "vectors": V}


def unprepare_vectors(X, perm, rot_first, rot_size, rot_values):
    """Prepared-basis vectors back to the caller's basis: the lifting
    rotations last first (v[block] <- Q v[block]), then basis_to_original
    (restates IPT_C_GPU/src/ipt_preparation.cu:1222-1293)."""
    X = np.array(X, dtype=np.float64, order="F", copy=True)
    ofs = int(sum(int(m) * int(m) for m in rot_size))
    for first, m in reversed(list(zip(rot_first, rot_size))):
        first, m = int(first), int(m)
        ofs -= m * m
        Q = np.asarray(rot_values[ofs:ofs + m * m]).reshape((m, m), order="F")
        for j in range(X.shape[1]):
            blk = X[first:first + m, j].copy()
            X[first:first + m, j] = [sum(Q[i, l] * blk[l] for l in range(m)) for i in range(m)]
    out = np.empty_like(X)
    out[np.asarray(perm), :] = X
    return out


def ref_cluster_solve_basis(cp, ri, va, diag, first, last, maxiter, tol, damping=1.0):
    """The reference's CPU block-cluster basis solve of one cluster (needs
    oracle/_ref); (basis, iterations) or None when it reports failure."""
    L = ref_lib("sparse")
    cp = np.ascontiguousarray(cp, dtype=np.int32)
    ri = np.ascontiguousarray(ri, dtype=np.int32)
    va = np.ascontiguousarray(va, dtype=np.float64)
    dg = np.ascontiguousarray(diag, dtype=np.float64)
    n = cp.size - 1
    m = last - first + 1
    X = np.zeros((n, m), dtype=np.float64, order="F")
    it = np.zeros(1, dtype=np.int32)
    ok = L.ref_block_cluster_solve_basis(_p(cp), _p(ri), _p(va), n, int(cp[-1]), _p(dg), first,
                                         last, maxiter, tol, damping, _p(X), _p(it))
    return (X, int(it[0])) if ok else None


# ---- matrix-free FCI-like construction (fci_oracle.c) -------------------------
def _fci_lib():
    L = lib()
    if not hasattr(L, "_fci_ready"):
        L.oracle_fci_dimension.restype = C.c_longlong
        L.oracle_fci_dimension.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oracle_fci_row_length.restype = C.c_int
        L.oracle_fci_row_length.argtypes = [C.c_int, C.c_int, C.c_int]
        L.oracle_fci_matrix.restype = C.c_int
        L.oracle_fci_matrix.argtypes = [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_double,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_fci_sigma.restype = C.c_int
        L.oracle_fci_sigma.argtypes = [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_double,
                                       C.c_void_p, C.c_int, C.c_void_p]
        L._fci_ready = True
    return L


def fci_matrix(norb, na, nb, seed=0, sigma=0.05, csr=True):
    """Diagonal and (optionally) the CSR of the matrix-free FCI-like H."""
    L = _fci_lib()
    n = L.oracle_fci_dimension(norb, na, nb)
    diag = np.zeros(n)
    if not csr:
        L.oracle_fci_matrix(norb, na, nb, seed, sigma, _p(diag), None, None, None)
        return diag
    per = L.oracle_fci_row_length(norb, na, nb) + 1
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(n * per, np.int32)
    va = np.zeros(n * per)
    st = L.oracle_fci_matrix(norb, na, nb, seed, sigma, _p(diag), _p(rp), _p(ci), _p(va))
    if st != 0:
        raise RuntimeError("oracle_fci_matrix failed")
    return rp, ci, va, diag


def fci_sigma(norb, na, nb, X, seed=0, sigma=0.05):
    L = _fci_lib()
    X = np.asfortranarray(X, dtype=np.float64)
    Y = np.zeros_like(X, order="F")
    L.oracle_fci_sigma(norb, na, nb, seed, sigma, _p(X), X.shape[1], _p(Y))
    return Y
