"""Record the reference's IPT_DEBUG_PREPARATION diagnostic lines for the
degeneracy-lifting fixtures (tests/golden/lift_kat.npz).

Run in a container where the reference tree exists:
    python oracle/build_ref.py && python tests/golden/make_prep_debug_golden.py

For every case of lift_kat.npz it runs the reference's own preparation with
lifting (ipt_prepare_sparse_csc, IPT_C_GPU/src/ipt_preparation.cu:1375-1648,
compiled from its sources into oracle/_ref/libref_sparse.so) in a child
process with IPT_DEBUG_PREPARATION=1 and keeps the "[IPT preparation]" lines
it prints (ipt_preparation.cu:601-613, 1448-1610); once more for case
lift_5 with IPT_MAX_LIFT_BLOCK_SIZE=2, where the block of three is too wide
(key "lift_5_max_block_2").

Output: tests/golden/prep_debug_kat.json, {case: [line, ...]}.
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")

CHILD = r'''
import sys
import numpy as np
sys.path.insert(0, %(root)r)
from oracle import oracle
z = np.load(%(kat)r)
c = %(case)r
n, k, ncp, nri = (int(x) for x in z[c + "_params"])
ints = z[c + "_in"]
oracle.ref_prepare_lifted(ints[:ncp], ints[ncp:ncp + nri], z[c + "_in_values"], n, k)
'''


def debug_lines(code, env_extra=None):
    """Run `code` in a child interpreter with the diagnostics switched on and
    return its "[IPT preparation]" lines."""
    env = dict(os.environ, IPT_DEBUG_PREPARATION="1", **(env_extra or {}))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         check=True).stdout
    return [line for line in out.splitlines() if line.startswith("[IPT preparation]")]


def main():
    sys.path.insert(0, ROOT)
    import numpy as np
    from oracle import oracle
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref not built (python oracle/build_ref.py)")
    kat = os.path.join(HERE, "lift_kat.npz")
    out = {}
    for case in [str(c) for c in np.load(kat)["cases"]]:
        out[case] = debug_lines(CHILD % {"root": os.path.abspath(ROOT), "kat": kat, "case": case})
        print(case, len(out[case]), "lines")
    out["lift_5_max_block_2"] = debug_lines(
        CHILD % {"root": os.path.abspath(ROOT), "kat": kat, "case": "lift_5"},
        {"IPT_MAX_LIFT_BLOCK_SIZE": "2"})
    with open(os.path.join(HERE, "prep_debug_kat.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
