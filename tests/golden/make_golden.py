"""Generate the golden fixtures from the reference's own CPU code.

Run in a container where the reference tree exists:
    python oracle/build_ref.py && python tests/golden/make_golden.py

It loads oracle/_ref/libref_{dense,sparse}.so (the reference's test drivers
IPT_C_GPU/test_temp/runtests.cu and IPT_C_GPU/test/sparse/runtests_sparse.cu
compiled from their sources) and records, for the reference's own test cases:

  * dense: the 8 cases of runtests.cu:304-313 (n, k, symmetric), a checksum
    and strided sample of the generated matrix (runtests.cu:46-80), and the
    vectors/values of ipt_cpu_reference after 20 iterations (runtests.cu:98-174);
  * sparse: the banded n=64 CSC (runtests_sparse.cu:224-268) and the 10x10
    H2O FCI "W" fixture (test/sparse/h20_w_csc.h), with the CPU reference's
    vectors/values after 80 iterations (runtests_sparse.cu:422-428), and the
    reference preparation's sorted arrays for both;
  * the binary layout (sizes and field offsets) of IPTCudaResult and the
    Davidson history structs.
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle  # noqa: E402

DENSE_CASES = [(32, 1, 0, "random_k1"), (32, 5, 0, "random_k5"), (32, 32, 0, "random_full"),
               (32, 1, 1, "symmetric_k1"), (32, 5, 1, "symmetric_k5"),
               (32, 32, 1, "symmetric_full"), (96, 5, 0, "random_medium"),
               (96, 16, 1, "symmetric_medium")]


def p(a):
    return C.c_void_p(a.ctypes.data)


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref not built (python oracle/build_ref.py)")
    dense = oracle.ref_lib("dense")
    sparse = oracle.ref_lib("sparse")
    out = {}
    meta = {"dense": [], "sparse": []}
    for n, k, sym, name in DENSE_CASES:
        H = np.zeros((n, n), dtype=np.float64, order="F")
        dense.ref_fill_perturbative_matrix(p(H), n, sym)
        X = np.zeros((n, k), dtype=np.float64, order="F")
        v = np.zeros(k, dtype=np.float64)
        assert dense.ref_ipt_cpu_reference(p(H), n, k, 20, p(X), p(v)) == 0
        out["dense_%s_vectors" % name] = X
        out["dense_%s_values" % name] = v
        out["dense_%s_sample" % name] = H.ravel(order="F")[::7].copy()
        meta["dense"].append({"name": name, "n": n, "k": k, "symmetric": sym, "iterations": 20,
                              "matrix_sum": float(H.sum()), "matrix_sumsq": float((H * H).sum())})
    # banded n = 64, k = 5, 80 iterations
    n = 64
    nnz = 3 * n - 2
    cp = np.zeros(n + 1, np.int32)
    ri = np.zeros(nnz, np.int32)
    va = np.zeros(nnz, np.float64)
    assert sparse.ref_build_banded_csc(n, p(cp), p(ri), p(va)) == nnz
    cases = [("synthetic_banded_k5", n, 5, cp, ri, va)]
    # H2O W 10 x 10, k = 1
    wn = 10
    wcp = np.zeros(wn + 1, np.int32)
    wri = np.zeros(100, np.int32)
    wva = np.zeros(100, np.float64)
    assert sparse.ref_h20_w_csc(p(wcp), p(wri), p(wva)) == 100
    cases.append(("h20_fci_w_k1", wn, 1, wcp, wri, wva))
    for name, n, k, cp, ri, va in cases:
        Hd = oracle.csc_to_dense(cp, ri, va, n)
        X = np.zeros((n, k), dtype=np.float64, order="F")
        v = np.zeros(k, dtype=np.float64)
        assert sparse.ref_sparse_ipt_cpu_reference(p(Hd), n, k, 80, p(X), p(v)) == 0
        pcp = np.zeros(n + 1, np.int32)
        pri = np.zeros(len(ri), np.int32)
        pva = np.zeros(len(ri), np.float64)
        pd = np.zeros(n, np.float64)
        pperm = np.zeros(n, np.int32)
        pnnz = sparse.ref_prepare_sparse_csc_sorted(p(cp), p(ri), p(va), n, k, len(ri), p(pcp),
                                                    p(pri), p(pva), p(pd), p(pperm))
        assert pnnz >= 0
        out["sparse_%s_col_ptr" % name] = cp
        out["sparse_%s_row_ind" % name] = ri
        out["sparse_%s_values_csc" % name] = va
        out["sparse_%s_vectors" % name] = X
        out["sparse_%s_values" % name] = v
        out["sparse_%s_prep_col_ptr" % name] = pcp
        out["sparse_%s_prep_row_ind" % name] = pri[:pnnz]
        out["sparse_%s_prep_values" % name] = pva[:pnnz]
        out["sparse_%s_prep_diag" % name] = pd
        out["sparse_%s_prep_perm" % name] = pperm
        meta["sparse"].append({"name": name, "n": n, "k": k, "nnz": int(len(ri)),
                               "iterations": 80})
    lay = np.zeros(32, dtype=np.int64)
    cnt = dense.ref_result_layout(p(lay), 32)
    meta["layout"] = {
        "names": ["sizeof_IPTCudaResult", "sizeof_IPTDavidsonHistoryEntry",
                  "sizeof_IPTDavidsonSelectionEntry", "sizeof_IPTDavidsonBlockHistoryEntry",
                  "vectors", "values", "matvecs", "fixed_point_residual",
                  "adaptive_added_indices", "davidson_history", "davidson_block_history",
                  "best_so_far_source", "cluster_soft_locked_count"],
        "values": [int(x) for x in lay[:cnt]],
    }
    np.savez_compressed(os.path.join(HERE, "reference_kat.npz"), **out)
    with open(os.path.join(HERE, "reference_kat.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
