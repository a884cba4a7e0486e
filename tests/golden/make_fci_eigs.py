"""Eigen-oracle fixtures for the FCI-like sparse workloads.

The k lowest eigenvalues of block_ipt_gb300.workloads.fci_like_csr matrices,
from scipy's ARPACK (eigsh, which='SA', tol 1e-13) with every pair's FP64
residual checked; a converged FP64 Krylov run is the eigen-oracle where n is
too large for a dense LAPACK solve.

    python tests/golden/make_fci_eigs.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(os.path.dirname(HERE))

from block_ipt_gb300 import workloads  # noqa: E402

CASES = [("fci_6o_3a3b_seed1", 6, 3, 3, 1, 6), ("fci_8o_4a4b_seed0", 8, 4, 4, 0, 8),
         ("fci_8o_4a4b_seed5", 8, 4, 4, 5, 8), ("fci_10o_5a5b_seed0", 10, 5, 5, 0, 16)]


def main():
    from scipy.sparse import csr_matrix
    from scipy.sparse.linalg import eigsh
    out = {}
    for name, norb, na, nb, seed, k in CASES:
        rp, ci, v, d = workloads.fci_like_csr(norb, na, nb, seed=seed)
        n = len(rp) - 1
        H = csr_matrix((v, ci, rp), shape=(n, n))
        w, V = eigsh(H, k=k, which="SA", tol=1e-13, ncv=max(4 * k, 40))
        order = np.argsort(w)
        w, V = w[order], V[:, order]
        hn = float(abs(H).sum(axis=1).max())
        res = np.linalg.norm(H @ V - V * w[None, :], axis=0) / max(1.0, hn)
        assert res.max() < 1e-11, res.max()
        out[name] = {"norb": norb, "nalpha": na, "nbeta": nb, "seed": seed, "k": k, "n": n,
                     "nnz": int(len(ci)), "norm_inf": hn, "eigenvalues": w.tolist(),
                     "max_scaled_residual": float(res.max())}
        print(name, n, w[:4])
    with open(os.path.join(HERE, "fci_eigs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
