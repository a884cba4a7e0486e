"""Generate the degeneracy-lifting fixtures from the reference's own code.

Run in a container where the reference tree exists:
    python oracle/build_ref.py && python tests/golden/make_lift_golden.py

It loads oracle/_ref/libref_sparse.so (the reference's sparse test driver,
which compiles IPT_C_GPU/src/ipt_cuda.cu and src/ipt_preparation.cu, built
from their sources) and records, for seeded symmetric matrices with planted
exact and near degeneracies (oracle.cluster_test_matrix, rows and columns
shuffled so that the diagonal sort matters):

  * the plain path's preparation with degeneracy lifting
    (ipt_prepare_sparse_csc with lift = 1, ipt_preparation.cu:1375-1648):
    the prepared CSC, its diagonal, basis_to_original and the rotations;
  * the reference's back-transform (ipt_apply_prepared_q_to_vectors,
    ipt_preparation.cu:1222-1294) of a seeded n x 3 block;
  * cases the preparation rejects (status recorded).

Output: tests/golden/lift_kat.npz.
"""
import os
import sys

import numpy as np
from scipy.sparse import csc_matrix

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle  # noqa: E402

CASES = [  # (name, n, seed, coupling, k)
    ("lift_5", 37, 7, 0.01, 6),
    ("lift_5b", 38, 8, 0.3, 3),
    ("lift_7", 44, 14, 0.3, 6),
    ("lift_3", 36, 6, 0.3, 6),
    ("lift_17", 32, 2, 2.0, 3),
    ("plain", 30, 0, 0.01, 1),
    ("reject", 31, 1, 2.0, 6),
]


def shuffled(n, seed, coupling):
    _, _, _, H = oracle.cluster_test_matrix(n, seed, coupling)
    P = np.random.default_rng(seed).permutation(n)
    S = csc_matrix(H[np.ix_(P, P)])
    S.sort_indices()
    return S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.copy()


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref not built (python oracle/build_ref.py)")
    out = {}
    for name, n, seed, coupling, k in CASES:
        cp, ri, va = shuffled(n, seed, coupling)
        V = np.random.default_rng(seed + 1000).standard_normal((n, 3))
        r = oracle.ref_prepare_lifted(cp, ri, va, n, k, vectors=V)
        out[name + "_in"] = np.concatenate([cp, ri]).astype(np.int32)
        out[name + "_in_values"] = va
        out[name + "_params"] = np.array([n, k, len(cp), len(ri)], np.int32)
        if isinstance(r, int):
            out[name + "_status"] = np.array([-r], np.int32)
            continue
        out[name + "_status"] = np.array([0], np.int32)
        for key in ("col_ptr", "row_ind", "values", "diag", "perm", "rot_first", "rot_size",
                    "rot_values"):
            out[name + "_" + key] = np.asarray(r[key])
        out[name + "_vectors_in"] = np.asfortranarray(V)
        out[name + "_vectors_out"] = r["vectors"]
        print(name, "rotations", len(r["rot_first"]), list(r["rot_size"]))
    out["cases"] = np.array([c[0] for c in CASES])
    np.savez_compressed(os.path.join(HERE, "lift_kat.npz"), **out)


if __name__ == "__main__":
    main()
