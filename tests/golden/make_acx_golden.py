"""Record the reference's published ACX / plain-IPT sweep results as a
fixture (tests/golden/acx_published.json).

TEST INFRASTRUCTURE ONLY.  Reads the result files the reference ships
(IPT_C_GPU/results/ACX/smoke_fcalls/acx_cuda_sweep_epsilon_0_06.csv and
IPT_C_GPU/results/ACX/acx_vs_original_ipt_summary.csv), which its ACX sweep
benchmark (IPT_C_GPU/test/ACX/benchmark_acx_cuda_sweep.cu) wrote on an A100
for the matrices that oracle.acx_sweep_matrix regenerates: ACX and plain IPT
from the identity, k = n, tol 1e-12.

    python tests/golden/make_acx_golden.py [IPT_C_GPU root]
"""
import csv
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("IPT_REFERENCE_ROOT",
                                                             "/root/reference/IPT_C_GPU")


def main():
    out = {"source": "IPT_C_GPU/results/ACX (A100-SXM4-80GB runs of benchmark_acx_cuda_sweep.cu)",
           "base_seed": 20260615, "cases": []}
    smoke = os.path.join(ROOT, "results", "ACX", "smoke_fcalls", "acx_cuda_sweep_epsilon_0_06.csv")
    rows = list(csv.DictReader(open(smoke)))
    case = {}
    for r in rows:
        key = "acx" if r["method"] == "acx_gpu_fp64" else "ipt"
        case.update({"n": int(r["N"]), "epsilon": float(r["epsilon"]), "tol": float(r["tol"]),
                     "maxiter": int(r["maxiter"])})
        case[key] = {"iterations": int(r["iterations"]), "f_calls": int(r["f_calls"]),
                     "fixed_point_residual": float(r["fixed_point_residual"]),
                     "max_apply_residual": (float(r["max_apply_residual"])
                                            if r["max_apply_residual"] != "nan" else None)}
    out["cases"].append(case)
    summary = os.path.join(ROOT, "results", "ACX", "acx_vs_original_ipt_summary.csv")
    for r in csv.DictReader(open(summary)):
        out["cases"].append({
            "n": int(r["N"]), "epsilon": float(r["epsilon"]), "tol": 1e-12, "maxiter": 1000,
            "acx": {"iterations": int(r["acx_iterations"]), "f_calls": int(r["acx_f_calls"]),
                    "fixed_point_residual": float(r["acx_fixed_point_residual"])},
            "ipt": {"iterations": int(r["original_ipt_iterations"]),
                    "f_calls": int(r["original_ipt_f_calls"]),
                    "fixed_point_residual": float(r["original_ipt_fixed_point_residual"])}})
    with open(os.path.join(HERE, "acx_published.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
