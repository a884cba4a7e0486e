"""Build libipt_gb300.so (the C-ABI library) from block_ipt_gb300/csrc.

Every translation unit is compiled for sm_103a only, in parallel, and linked
into block_ipt_gb300/_build/libipt_gb300.so.  Only the entry points marked
for export (include/ipt_cuda.h, include/ipt_block.h) are visible.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libipt_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _compile(nvcc, src, obj, verbose):
    # host code without contraction: host-side FP arithmetic (workload tables)
    # must match the CPU oracle bit for bit
    cmd = [nvcc, "-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler",
           "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-Xptxas", "-warn-spills",
           "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc, "-O3", "-std=c++17", "-Xcompiler",
               "-fPIC,-fvisibility=hidden,-ffp-contract=off", "-c", src, "-o", obj]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or proc.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    return proc.returncode


def build(verbose=False, force=False):
    """Compile and link; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(PKG, "..", "include", f)
                for f in os.listdir(os.path.join(PKG, "..", "include"))]
    newest_header = max(os.path.getmtime(h) for h in headers)
    jobs = []
    objs = []
    for src in srcs:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        stale = (force or not os.path.exists(obj)
                 or os.path.getmtime(obj) < max(os.path.getmtime(src), newest_header))
        if stale:
            jobs.append((src, obj))
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(workers) as ex:
            rcs = list(ex.map(lambda j: _compile(nvcc, j[0], j[1], verbose), jobs))
        if any(rcs):
            raise RuntimeError("nvcc failed for: " + ", ".join(
                os.path.basename(j[0]) for j, rc in zip(jobs, rcs) if rc))
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-lcublas", "-lcudart"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("link failed:\n" + proc.stdout + proc.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
