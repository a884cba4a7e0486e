"""Count the block products plain IPT needs on the benchmark matrices.

TEST INFRASTRUCTURE ONLY.  For each seeded benchmark workload this runs the
oracle's plain IPT (oracle_ipt_dense_products_to_residual) until the scaled
eigen-residual max_j ||H x_j - lambda_j x_j|| / (max(1,||H||_inf) max(1,||x_j||))
reaches 1e-8, and records the count in oracle/plain_ipt_products.json.  The
count scales the timed CPU sample of bench.py (one IPT iteration) to the
time the reference's CPU path needs to reach the same residual.

    python oracle/count_plain_products.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)

from block_ipt_gb300 import workloads  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = os.path.join(HERE, "plain_ipt_products.json")


def main():
    out = {}
    for name, n, k, seed, gen in [("dense_config0_n1024_k8_seed0", 1024, 8, 0, workloads.dense_config0),
                                  ("dense_config1_n8192_k32_seed0", 8192, 32, 0, workloads.dense_config1)]:
        H, _ = gen(n, seed=seed)
        t = time.time()
        cnt, res = oracle.products_to_residual(H, k, 2000, 1e-8)
        out[name] = {"n": n, "k": k, "seed": seed, "res_tol": 1e-8, "products": cnt,
                     "final_scaled_residual": res, "oracle_seconds": time.time() - t,
                     "threads": oracle.num_threads()}
        print(name, out[name], flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
