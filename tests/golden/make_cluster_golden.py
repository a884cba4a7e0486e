"""Generate the block-cluster fixtures from the reference's own CPU code.

Run in a container where the reference tree exists:
    python oracle/build_ref.py && python tests/golden/make_cluster_golden.py

It loads oracle/_ref/libref_sparse.so (the reference's sparse test driver,
which compiles IPT_C_GPU/src/ipt_cuda.cu, built from its sources) and
records, for seeded symmetric test matrices with planted degeneracies
(oracle.cluster_test_matrix) and the reference's H2O FCI "W" fixture
(IPT_C_GPU/test/sparse/h20_w_csc.h):

  * the cluster ranges of ipt_block_cluster_prepare (ipt_cuda.cu:4555-4688),
    without and with the adaptive expansion (IPT_BLOCK_CLUSTER_ADAPTIVE);
  * the basis and iteration count of every cluster from the reference's CPU
    block-cluster solve (ipt_block_cluster_solve_basis, ipt_cuda.cu:4274-4395).

Output: tests/golden/cluster_kat.npz (matrices included, so the tests need
neither the reference nor this script).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle  # noqa: E402

CASES = [  # (name, n, seed, coupling, k, adaptive, damping)
    ("deg_small", 48, 3, 0.3, 4, 0, 1.0),
    ("deg_adaptive", 56, 2, 0.3, 9, 1, 1.0),
    ("wide_adaptive", 56, 25, 2.0, 9, 1, 1.0),
    ("weak_coupling", 64, 11, 0.01, 9, 0, 1.0),
    ("damped", 52, 5, 0.3, 4, 0, 0.7),
]
MAXITER = 60
TOL = 1e-12


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref not built (python oracle/build_ref.py)")
    out = {}
    names = []
    L = oracle.ref_lib("sparse")
    cases = list(CASES)
    for name, n, seed, coupling, k, adaptive, damping in cases:
        cp, ri, va, H = oracle.cluster_test_matrix(n, seed, coupling)
        out[name + "_col_ptr"], out[name + "_row_ind"], out[name + "_values"] = cp, ri, va
        names.append((name, k, adaptive, damping))
    # H2O W fixture, k = 3 (its own diagonal order is prepared by the test)
    cp = np.zeros(11, np.int32)
    ri = np.zeros(100, np.int32)
    va = np.zeros(100)
    nnz = L.ref_h20_w_csc(oracle._p(cp), oracle._p(ri), oracle._p(va))
    out["h2o_w_col_ptr"], out["h2o_w_row_ind"], out["h2o_w_values"] = cp, ri[:nnz], va[:nnz]
    names.append(("h2o_w", 3, 0, 1.0))
    for name, k, adaptive, damping in names:
        cp, ri, va = out[name + "_col_ptr"], out[name + "_row_ind"], out[name + "_values"]
        n = cp.size - 1
        os.environ["IPT_BLOCK_CLUSTER_ADAPTIVE"] = str(adaptive)
        ranges, added, lim = oracle.ref_cluster_prepare(cp, ri, va, n, k)
        os.environ.pop("IPT_BLOCK_CLUSTER_ADAPTIVE")
        # the prepared (diagonal-sorted) matrix the ranges refer to
        pcp = np.zeros(n + 1, np.int32)
        pri = np.zeros(ri.size, np.int32)
        pva = np.zeros(ri.size)
        pd = np.zeros(n)
        perm = np.zeros(n, np.int32)
        pnnz = L.ref_prepare_sparse_csc_sorted(oracle._p(cp), oracle._p(ri), oracle._p(va), n, k,
                                               ri.size, oracle._p(pcp), oracle._p(pri),
                                               oracle._p(pva), oracle._p(pd), oracle._p(perm))
        pri, pva = pri[:pnnz], pva[:pnnz]
        bases, its = [], []
        for a, b in ranges:
            r = oracle.ref_cluster_solve_basis(pcp, pri, pva, pd, a, b, MAXITER, TOL, damping)
            assert r is not None, (name, a, b)
            X, it = r
            bases.append(X)
            its.append(it)
        out[name + "_prep_col_ptr"], out[name + "_prep_row_ind"] = pcp, pri
        out[name + "_prep_values"], out[name + "_prep_diag"] = pva, pd
        out[name + "_ranges"] = np.array(ranges, np.int32).reshape(-1, 2)
        out[name + "_added"] = np.array(added, np.int32)
        out[name + "_limit_hit"] = np.array([int(lim)], np.int32)
        out[name + "_basis"] = np.asfortranarray(np.hstack(bases))
        out[name + "_iterations"] = np.array(its, np.int32)
        out[name + "_params"] = np.array([k, adaptive, damping, MAXITER, TOL])
    out["cases"] = np.array([c[0] for c in names])
    np.savez_compressed(os.path.join(HERE, "cluster_kat.npz"), **out)
    print("wrote", len(names), "cases")


if __name__ == "__main__":
    main()
