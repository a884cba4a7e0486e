"""Benchmark: time to the k lowest eigenpairs at ||r|| <= 1e-8 ||H||_inf.

Workload (one step = one solve): dense symmetric n = 8192, k = 32 with
d_i = i/8 + U(0,0.1) and h_ij ~ N(0, 0.02^2) exp(-|i-j|/256) (seeded synthetic
matrix, block_ipt_gb300.workloads.dense_config1).  Our arm solves it with
the block solver: FP16 tensor-core IPT (tcgen05/TMA), refinement of the IPT
fixed point by FP16 tensor-core correction solves against FP64-accurate
(double-FP32) defects, and a final FP64 CholQR2 + Rayleigh-Ritz; each result
is checked in FP64 (torch DGEMM residual, LAPACK eigenvalues).

  value        device time per solve, H already resident in HBM (ms)
  e2e          the same solve through the host C-ABI entry point
               (ipt_block_solve_dense): H copied in from pinned host memory
               and the pairs copied back inside the timed region (ms)
  plain_fp64   the same code with an FP64 IPT stage (ms), and the speed-up
  roofline     dominant kernel of the timed region, from live CUDA-event
               timings of every launch (ipt_block_profile_*)
  cpu_baseline the oracle restatement of the reference's CPU IPT: one
               complete solve of this matrix on all host cores, stopped at
               the scaled residual 1e-8; beside it one iteration on one core
               and LAPACK dsyevd (scipy, all host cores)
  fci_config3  FCI-like CSR (n = 63,504, k = 16), plain and learned Davidson
  batched_config2      512 dense instances, persistent kernel under a graph
  matrix_free_config4  matrix-free FCI-like sigma, 14 orbitals (n = 11.8M)

`--impl reference` times the reference's CPU path alone (rank 0 only): every
step is one complete tolerance-stopped plain-IPT solve of the same matrix.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to k eigenpairs at ||r||<=1e-8, mixed+learned vs plain FP64 IPT, 1xGB300"
METHOD = ("FP16 tcgen05 IPT + refinement against FP64-accurate defects, FP64-accurate "
          "CholQR/Rayleigh-Ritz, to scaled residual 1e-8")
REFERENCE_PATH = ("the reference's CPU plain IPT (runtests.cu:98-174 semantics, oracle port) "
                  "stopped at the scaled residual 1e-8")
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# DRAM bytes (read + write) per launch from one ncu capture of each kernel on
# this workload (profiles/dense64_partial_fp64_n8192_k32.md,
# profiles/df64_partial_n8192_k32.md, profiles/tc_partial_fp16_n8192_k32.md);
# keyed by (kernel, n, k, precision).
NCU_TRAFFIC = {("dense64_partial", 8192, 32, "fp16"): 567.5e6,
               ("df64_partial", 8192, 32, "fp16"): 1111.3e6,
               # launches inside 30-step FP16 runs of the n = 8192 / 16384
               # matrices with the L2-kept share of Delta, caches not flushed
               # between launches (profiles/tc_stream_fp16_n8192_k32.md); the
               # same figure stands for the product inside the dense solve
               ("tc_stream", 8192, 32, "fp16"): 95.7e6,
               ("tc_stream", 8192, "default"): 95.7e6,
               ("tc_stream", 8192, "0"): 141.9e6,
               ("tc_stream", 16384, "default"): 554.4e6,
               # one cold launch at n = 8192, 32 columns
               # (profiles/oz_product_n4096_n8192_c32.md)
               ("oz_product", 8192, 32, "fp16"): 811.5e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--k", type=int, default=32)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", default="fp16", choices=["fp16", "bf16", "tf32"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-lapack", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fci", action="store_true")
    ap.add_argument("--fci-steps", type=int, default=2)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-fci-free", action="store_true")
    ap.add_argument("--no-acx", action="store_true")
    ap.add_argument("--no-lowp-sweep", action="store_true")
    ap.add_argument("--fci-free-orbitals", type=int, default=14)
    ap.add_argument("--batch", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--trace", default=None,
                    help="write the phase marks of one more dense solve to this file")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, world, device="cpu"):
    """The N > 1 rule of the timed region: every rank's time, then the
    maximum over ranks (all ranks receive it).  World size 1 needs no
    process group."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
    return float(t.item())


def replica_seed(seed, rank):
    """Replicas only: each rank solves its own instance of the workload."""
    return seed + rank


def workload_name(n, k, seed):
    return ("dense symmetric n=%d k=%d, d_i=i/8+U(0,0.1), h_ij~N(0,0.02^2)exp(-|i-j|/256), seed %d"
            % (n, k, seed))


def bench_config(args):
    """The workload description both arms print (identical dictionaries)."""
    return {"workload": workload_name(args.n, args.k, args.seed), "n": args.n, "k": args.k,
            "seed": args.seed, "target": "k lowest eigenpairs, scaled residual <= 1e-8",
            "l2": "256 MB buffer written between timed GPU steps (inputs also > L2)",
            "parallelism": "replicas only (one instance per GPU)"}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's CPU IPT (oracle port or oracle/_ref)
# ---------------------------------------------------------------------------
def cpu_solve(H, k):
    """One complete plain-IPT solve of H by the reference's CPU algorithm
    (the oracle's restatement of runtests.cu:98-174, on all host cores),
    iterated until the scaled eigen-residual of every column is <= 1e-8.
    Returns (ms, block products, final scaled residual)."""
    from oracle import oracle
    t0 = time.perf_counter()
    cnt, res = oracle.products_to_residual(H, k, 2000, 1e-8)
    ms = (time.perf_counter() - t0) * 1e3
    if cnt <= 0:
        raise RuntimeError("CPU plain IPT did not reach the scaled residual 1e-8")
    return ms, cnt, res


def cpu_one_core_iteration(H, k):
    """One plain-IPT iteration of the same CPU code on a single host core:
    one block product and the update, plus the product that returns the
    eigenvalues (ms)."""
    from oracle import oracle
    cores = oracle.num_threads()
    oracle.set_num_threads(1)
    try:
        t0 = time.perf_counter()
        oracle.ipt_dense(H, k, 1)
        return (time.perf_counter() - t0) * 1e3
    finally:
        oracle.set_num_threads(cores)


def blas_threads():
    try:
        import threadpoolctl
        info = threadpoolctl.threadpool_info()
        if info:
            return max(int(x.get("num_threads", 0)) for x in info)
    except ImportError:
        pass
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
        if os.environ.get(var):
            return int(os.environ[var])
    return os.cpu_count()


def dsyevd_leg(H, k):
    """LAPACK dsyevd (scipy, divide and conquer, all eigenpairs) on the
    same matrix, timed once; returns the report and the k lowest values."""
    from oracle import oracle
    t0 = time.perf_counter()
    w, _ = oracle.dsyevd_lowest(H, k)
    ms = (time.perf_counter() - t0) * 1e3
    return {"ms": ms, "threads": blas_threads(),
            "routine": "scipy.linalg.lapack.dsyevd, compute_v=1 (full spectrum)"}, w


def cpu_sample_text(n, k, cnt):
    return ("one complete solve per step: plain IPT from the identity block (n=%d, k=%d) until "
            "every scaled residual is <= 1e-8 (%d block products)" % (n, k, cnt))


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from block_ipt_gb300 import workloads
    from oracle import oracle
    oracle.build()
    H, _ = workloads.dense_config1(args.n, seed=args.seed)
    H = np.asfortranarray(H)
    for _ in range(args.warmup):
        cpu_solve(H, args.k)
    samples, cnt, res = [], 0, None
    for _ in range(args.steps):
        ms, cnt, res = cpu_solve(H, args.k)
        samples.append(ms)
    value = statistics.mean(samples)
    cores = oracle.num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "ms",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": value,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": bench_config(args), "path": REFERENCE_PATH,
        "cpu_baseline": {"value": value, "unit": "ms", "cores": cores, "kind": "port",
                         "sample": cpu_sample_text(args.n, args.k, cnt),
                         "final_scaled_residual": res},
        "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def fp64_check(torch, dH, dX, dv, hnorm):
    R = dH @ dX - dX * dv[None, :]
    r = (torch.linalg.vector_norm(R, dim=0) / max(1.0, hnorm)).max().item()
    return r


def write_trace(path, api, torch, solve, flush):
    """Phase marks (GPU global timer and host clock) of one solve, as a table."""
    flush.zero_()
    torch.cuda.synchronize()
    api.trace_enable(True)
    solve()
    torch.cuda.synchronize()
    marks = api.trace_read()
    api.trace_enable(False)
    g0, h0 = marks[0][2], marks[0][1]
    with open(path, "w") as f:
        f.write("%-30s %10s %10s %10s %10s\n" % ("mark", "gpu_us", "host_us", "gpu-host", "d_gpu"))
        prev = g0
        for label, host, gpu in marks:
            f.write("%-30s %10.1f %10.1f %10.1f %10.1f\n" % (
                label, (gpu - g0) / 1e3, (host - h0) / 1e3, ((gpu - g0) - (host - h0)) / 1e3,
                (gpu - prev) / 1e3))
            prev = gpu


def profile_snapshot(lib):
    out = {}
    name = C.c_char_p()
    ms = C.c_double()
    cnt = C.c_longlong()
    for kid in range(10):
        lib.ipt_block_profile_read(kid, C.byref(name), C.byref(ms), C.byref(cnt))
        out[name.value.decode()] = (ms.value, cnt.value)
    return out


def fci_section(args, torch, lib, stream, flush, dev):
    """The FCI-like sparse workload (10 orbitals, 5+5 electrons, n = 63,504,
    nnz = 55.6M, k = 16): FP64 CSR block solve, device-resident input."""
    from scipy.sparse import csr_matrix

    from block_ipt_gb300 import _lib, api, workloads
    rp, ci, v, d = workloads.fci_like_csr(10, 5, 5, seed=0)
    n, k = len(rp) - 1, 16
    perm = np.argsort(d, kind="stable")
    Hs = csr_matrix((v, ci, rp), shape=(n, n))[perm][:, perm].tocsr()
    Hs.sort_indices()
    drp = torch.from_numpy(Hs.indptr.astype(np.int32)).to(dev)
    dci = torch.from_numpy(Hs.indices.astype(np.int32)).to(dev)
    dvv = torch.from_numpy(Hs.data).to(dev)
    dX = torch.empty((k, n), dtype=torch.float64, device=dev)
    dw = torch.empty(k, dtype=torch.float64, device=dev)
    opt = api.block_options("fp64", stream=stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def solve():
        rep = _lib.IPTBlockReport()
        st = lib.ipt_block_solve_csr_device(C.c_void_p(drp.data_ptr()), C.c_void_p(dci.data_ptr()),
                                            C.c_void_p(dvv.data_ptr()), n, int(Hs.nnz), k,
                                            C.byref(opt), C.c_void_p(dX.data_ptr()),
                                            C.c_void_p(dw.data_ptr()), C.byref(rep))
        assert st == 0, _lib.status_string(st)
        return rep.as_dict()

    solve()
    times, rep = [], None
    for _ in range(max(1, args.fci_steps)):
        flush.zero_()
        e0.record(stream)
        rep = solve()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    # per-kernel event timings over a second, instrumented pass
    lib.ipt_block_profile_reset()
    lib.ipt_block_profile_enable(1)
    for _ in range(len(times)):
        flush.zero_()
        solve()
    torch.cuda.synchronize()
    lib.ipt_block_profile_enable(0)
    prof = profile_snapshot(lib)
    X = dX.T.cpu().numpy()
    w = dw.cpu().numpy()
    hn = float(abs(Hs).sum(axis=1).max())
    res = float((np.linalg.norm(Hs @ X - X * w[None, :], axis=0) / max(1.0, hn)).max())
    dl = None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "fci_eigs.json")) as f:
            ref = np.array(json.load(f)["fci_10o_5a5b_seed0"]["eigenvalues"])
        dl = float(np.abs(w - ref).max() / hn)
    except (OSError, KeyError):
        pass
    cp_ms, cp_cnt = prof["csr_product"]
    cols = rep["fp64_matvecs"]
    learned_part = None
    if not args.no_learned:
        learned_part = learned_section(args, torch, dev, stream, flush, solve, opt, e0, e1,
                                       times, rep)
    achieved = (2.0 * Hs.nnz * cols * len(times)) / (cp_ms * 1e-3) / 1e12 if cp_ms else None
    cluster = cluster_part(args, torch, lib, stream, flush, dev, Hs, drp, dci, dvv, k, e0, e1)
    cpu = None if args.no_cpu else fci_cpu_baseline(Hs, k, hn)
    return {"workload": "FCI-like CSR, 10 orbitals 5a/5b, n=%d nnz=%d, k=%d, seed 0" % (n, Hs.nnz, k),
            "cpu_baseline": cpu,
            "ms": statistics.mean(times), "report": {kk: rep[kk] for kk in (
                "converged", "ipt_iterations", "davidson_steps", "restarts", "basis_cols",
                "fp64_matvecs", "total_ms")},
            "check": {"max_scaled_residual": res, "max_abs_dlambda_over_norm_inf": dl},
            "csr_product": {"launches": cp_cnt, "ms_per_solve": cp_ms / len(times),
                            "achieved_fp64_tflops": achieved},
            "kernel_ms": {kk: round(val[0] / len(times), 4) for kk, val in prof.items() if val[1]},
            "learned": learned_part, "block_cluster": cluster}


def fci_cpu_baseline(Hs, k, hn):
    """The FCI-like workload on the host: ARPACK's implicitly restarted
    Lanczos (scipy.sparse.linalg.eigsh) for the k lowest pairs of the same
    CSR matrix, relative tolerance 1e-10 (the reference's plain CPU IPT does
    not converge on this family: its map diverges from the first step).
    One complete solve, timed; the scaled residual of its pairs is checked."""
    from scipy.sparse.linalg import eigsh
    t0 = time.perf_counter()
    w, X = eigsh(Hs, k=k, which="SA", tol=1e-10)
    s = time.perf_counter() - t0
    res = float((np.linalg.norm(Hs @ X - X * w[None, :], axis=0) / max(1.0, hn)).max())
    return {"s": s, "max_scaled_residual": res, "threads": 1,
            "routine": "scipy.sparse.linalg.eigsh (ARPACK Lanczos), which='SA', tol 1e-10; "
                       "the CSR products run on one thread"}


def batch_cpu_baseline(specs, budget_s=6.0):
    """The batched workload on the host cores, over the leading instances of
    the batch (its order is random in n) until budget_s is spent: the
    reference's CPU IPT (the oracle port, all cores) from the identity block
    until every scaled residual is <= 1e-8, and LAPACK dsyevd on each of them;
    reported as instances per second of each."""
    from block_ipt_gb300 import workloads
    from oracle import oracle
    ipt_s = lap_s = 0.0
    done = 0
    unconverged = 0
    for n, k, sig, seed in specs:
        H, _ = workloads.batch_instance(n, sig, seed)
        t0 = time.perf_counter()
        cnt, _ = oracle.products_to_residual(H, k, 500, 1e-8)
        ipt_s += time.perf_counter() - t0
        if cnt <= 0:
            unconverged += 1
        t0 = time.perf_counter()
        oracle.dsyevd_lowest(H, k)
        lap_s += time.perf_counter() - t0
        done += 1
        if ipt_s + lap_s >= budget_s:
            break
    return {"instances": done, "of": len(specs),
            "ipt_port": {"s": ipt_s, "instances_per_s": done / ipt_s if ipt_s else None,
                         "cores": oracle.num_threads(), "unconverged": unconverged},
            "dsyevd": {"s": lap_s, "instances_per_s": done / lap_s if lap_s else None,
                       "threads": blas_threads()},
            "sample": "the first %d instances of the batch, each solved completely" % done}


def lowp_sweep_section(torch, lib, dev, k, peak):
    """The low-precision tensor-core product on its own, per launch, inside
    30-step fixed-iteration FP16 IPT runs (ipt_mixed_precision_cuda_device_tol):
    n = 8192 (FP16 Delta 134 MB, about L2's size) and n = 16384 (537 MB, four
    times L2), with the default L2 hint and without it (IPT_GB300_L2_KEEP_PCT=0:
    every byte of Delta from DRAM).  Synthetic matrices of the headline
    family (diagonal i/8, off-diagonal 0.02 N(0,1) exp(-|i-j|/256)), made on
    the device."""
    import os
    from block_ipt_gb300 import _lib
    out = []
    for n in (8192, 16384):
        g = torch.Generator(device=dev)
        g.manual_seed(n)
        idx = torch.arange(n, device=dev, dtype=torch.float64)
        H = torch.empty((n, n), dtype=torch.float64, device=dev)
        for r0 in range(0, n, 2048):
            r1 = min(n, r0 + 2048)
            H[r0:r1] = 0.02 * torch.randn((r1 - r0, n), generator=g, device=dev,
                                          dtype=torch.float64) * torch.exp(
                -(idx[r0:r1, None] - idx[None, :]).abs() / 256.0)
        H = torch.triu(H, 1)
        H = H + H.T
        H.diagonal().copy_(idx / 8.0)
        ldp = (n + 63) // 64 * 64
        alg = 2 * n * ldp + 2 * ldp * ((k + 15) // 16 * 16)
        for keep in (None, "0"):
            old = os.environ.pop("IPT_GB300_L2_KEEP_PCT", None)
            if keep is not None:
                os.environ["IPT_GB300_L2_KEEP_PCT"] = keep
            try:
                res = _lib._MixedResult()

                def run():
                    st = lib.ipt_mixed_precision_cuda_device_tol(
                        C.c_void_p(H.data_ptr()), n, k, 1e-300, 30, 1e300, 1,
                        C.c_void_p(torch.cuda.current_blas_handle()), C.byref(res))
                    if st != 0:
                        raise RuntimeError("mixed IPT status %d" % st)
                    lib.ipt_mixed_precision_cuda_free_device_result(C.byref(res))

                run()
                torch.cuda.synchronize()
                lib.ipt_block_profile_reset()
                lib.ipt_block_profile_enable(1)
                run()
                run()
                torch.cuda.synchronize()
                lib.ipt_block_profile_enable(0)
                ms, cnt = profile_snapshot(lib)["lowp_product"]
            finally:
                os.environ.pop("IPT_GB300_L2_KEEP_PCT", None)
                if old is not None:
                    os.environ["IPT_GB300_L2_KEEP_PCT"] = old
            per = ms / max(1, cnt)
            ach = alg / (per * 1e-3) / 1e9
            traffic = NCU_TRAFFIC.get(("tc_stream", n, keep or "default"))
            out.append({"n": n, "l2_keep": "default" if keep is None else "off",
                        "us_per_launch": per * 1e3, "launches": cnt,
                        "algorithmic_bytes": alg, "achieved_gbs": ach, "frac": ach / peak,
                        "dram_bytes_per_launch": traffic,
                        "dram_only_frac": (traffic / (per * 1e-3) / 1e9 / peak) if traffic else None})
        del H
        torch.cuda.empty_cache()
    return out


def acx_section(torch, lib, dH, n, k):
    """ACX extrapolation over the FP64 IPT map (the reference's
    acx_cuda_device_tol) on the headline matrix: steps, map evaluations,
    wall time as the reference reports it (result->time_sec), the FP64 check."""
    res = _lib_mod().ACXCudaResult()
    lib.acx_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, 1e-12, 200, None, C.byref(res))
    lib.acx_cuda_free_result(C.byref(res))  # warm-up
    torch.cuda.synchronize()
    res = _lib_mod().ACXCudaResult()
    st = lib.acx_cuda_device_tol(C.c_void_p(dH.data_ptr()), n, k, 1e-12, 200, None, C.byref(res))
    if st != 0:
        return {"status": st}
    X = torch.empty((k, n), dtype=torch.float64, device=dH.device)
    v = torch.empty(k, dtype=torch.float64, device=dH.device)
    rt = _cudart()
    rt.cudaMemcpy(C.c_void_p(X.data_ptr()), C.c_void_p(res.d_vectors), C.c_size_t(8 * n * k), 3)
    rt.cudaMemcpy(C.c_void_p(v.data_ptr()), C.c_void_p(res.d_values), C.c_size_t(8 * k), 3)
    Xc = X.T
    R = dH @ Xc - Xc * v[None, :]
    hn = float(dH.abs().sum(dim=1).max())
    check = float((R.norm(dim=0) / (torch.clamp(Xc.norm(dim=0), min=1.0) * max(1.0, hn))).max())
    out = {"workload": "dense n=%d, k=%d (the headline matrix), tol 1e-12" % (n, k),
           "ms": res.time_sec * 1e3, "iteration_ms": res.iteration_time_sec * 1e3,
           "iterations": res.iterations, "f_calls": res.f_calls, "converged": res.converged,
           "fixed_point_residual": res.fixed_point_residual, "max_scaled_residual": check}
    lib.acx_cuda_free_result(C.byref(res))
    return out


def _lib_mod():
    from block_ipt_gb300 import _lib
    return _lib


def _cudart():
    for name in ("libcudart.so", "/usr/local/cuda/lib64/libcudart.so", "libcudart.so.13",
                 "libcudart.so.12"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise OSError("libcudart not found")


def gj_fmas(m):
    """FMAs of one row's Gauss-Jordan elimination of an m x (m+1) system."""
    return (m - 1) * ((m + 1) * (m + 2) // 2 - 1)


def cluster_part(args, torch, lib, stream, flush, dev, Hs, drp, dci, dvv, k, e0, e1):
    """The block-cluster basis (the reference's IPT_BLOCK_CLUSTER stage) of
    the same matrix: cluster ranges of the k targets from the device CSR
    (scans on the GPU, detection rules on the host), the basis solve on the
    device (CSR products + the Gauss-Jordan update kernel), and the update
    kernel's FP64 roofline."""
    from block_ipt_gb300 import api
    n = Hs.shape[0]

    def detect():
        return api.cluster_ranges_device(drp.data_ptr(), dci.data_ptr(), dvv.data_ptr(), n,
                                         int(Hs.nnz), k, stream=stream.cuda_stream)

    ranges, _ = detect()
    host_ranges, _ = api.cluster_ranges(Hs.indptr, Hs.indices, Hs.data, n, k)
    if ranges != host_ranges:
        raise RuntimeError("device cluster ranges differ from the host entry's")
    detect_ms = []
    for _ in range(3):
        t0 = time.perf_counter()
        detect()
        detect_ms.append((time.perf_counter() - t0) * 1e3)
    t0 = time.perf_counter()
    api.cluster_ranges(Hs.indptr, Hs.indices, Hs.data, n, k)
    host_detect_ms = (time.perf_counter() - t0) * 1e3
    dd = torch.from_numpy(Hs.diagonal().copy()).to(dev)
    cols = sum(b - a + 1 for a, b in ranges)
    dB = torch.empty((cols, n), dtype=torch.float64, device=dev)

    def run():
        return api.cluster_basis(drp.data_ptr(), dci.data_ptr(), dvv.data_ptr(), n, int(Hs.nnz),
                                 dd.data_ptr(), ranges, 100, 1e-12, dB.data_ptr(),
                                 stream=stream.cuda_stream)

    run()
    times = []
    for _ in range(max(1, args.fci_steps)):
        flush.zero_()
        e0.record(stream)
        its, res = run()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    lib.ipt_block_profile_reset()
    lib.ipt_block_profile_enable(1)
    run()
    torch.cuda.synchronize()
    lib.ipt_block_profile_enable(0)
    prof = profile_snapshot(lib)
    up_ms, up_cnt = prof["cluster_update"]
    flops = sum(2.0 * gj_fmas(b - a + 1) * (n - (b - a + 1)) * int(its[c])
                for c, (a, b) in enumerate(ranges))
    peak = C.c_double(0.0)
    lib.ipt_block_measure_fp64_peak(C.byref(peak))
    ach = flops / (up_ms * 1e-3) / 1e12 if up_ms else None
    return {"ranges": [list(r) for r in ranges if r[1] > r[0]], "clusters": len(ranges),
            "basis_cols": cols, "iterations": [int(x) for x in its],
            "detect_ms": min(detect_ms), "host_detect_ms": host_detect_ms,
            "max_fixed_point_residual": float(np.nanmax(res)), "ms": statistics.mean(times),
            "update": {"launches": up_cnt, "ms_per_solve": up_ms, "fp64_tflops": ach,
                       "peak_tflops": peak.value, "frac": ach / peak.value if ach else None,
                       "bound": "fp64",
                       "flops_per_solve": flops},
            "csr_product_ms_per_solve": prof["csr_product"][0]}


def learned_section(args, torch, dev, stream, flush, solve, opt, e0, e1, plain_times, plain_rep):
    """Learned Davidson preconditioner on the FCI-like workload: trained (outside
    any timed region) on 6- and 8-orbital instances of the family by the
    library's own kernels, then the same solve timed with it."""
    from block_ipt_gb300 import learned
    t0 = time.perf_counter()
    params, info = learned.build(torch, device=dev)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    # what the network gains on a held-out instance of the training family
    held = learned.device_csr(torch, 8, 4, 4, 9, device=dev)
    rows = torch.empty((1_500_000, learned.ROW), dtype=torch.float32, device=dev)
    got = learned.collect(torch, held, 16, rows, 0)
    loss_plain, loss_neumann, loss_mlp = learned.correction_losses(torch, params, rows, got)
    del rows
    def timed_with(p):
        opt.preconditioner = 1
        opt.mlp_params = C.c_void_p(p.data_ptr())
        solve()
        ts, r = [], None
        for _ in range(max(1, args.fci_steps)):
            flush.zero_()
            e0.record(stream)
            r = solve()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        opt.preconditioner = 0
        opt.mlp_params = None
        return ts, r

    times, rep = timed_with(params)
    # ablation: the unweighted two-term correction (weight 1 on every row)
    two = torch.zeros_like(params)
    two[-1] = 30.0
    two_times, two_rep = timed_with(two)
    return {"ms": statistics.mean(times), "plain_ms": statistics.mean(plain_times),
            "two_term_ms": statistics.mean(two_times), "two_term_steps": two_rep["davidson_steps"],
            "two_term_fp64_matvecs": two_rep["fp64_matvecs"],
            "two_term_precond_matvecs": two_rep["precond_matvecs"],
            "selected": info.get("selected"), "validation_steps": info.get("validation_steps"),
            "steps": rep["davidson_steps"], "plain_steps": plain_rep["davidson_steps"],
            "fp64_matvecs": rep["fp64_matvecs"], "plain_fp64_matvecs": plain_rep["fp64_matvecs"],
            "precond_matvecs": rep["precond_matvecs"],
            "converged": rep["converged"], "max_scaled_residual": rep["max_scaled_residual"],
            "mlp_steps_accepted": rep["mlp_steps_accepted"],
            "mlp_steps_rejected": rep["mlp_steps_rejected"],
            "train_s": train_s, "train_rows": info["rows_total"],
            "heldout_correction_error": {"plain": loss_plain, "two_term_neumann": loss_neumann,
                                         "learned": loss_mlp,
                                         "instance": "8 orbitals 4a/4b seed 9"},
            "_params": params}


def batch_section(args, torch, dev):
    """The batched dense workload: 512 independent instances, n ~ U{64..2048},
    k ~ U{4..16}, sigma ~ U(0.01, 0.1), configs[0] construction per instance
    (generated on the device, same hashes as block_ipt_gb300.workloads), solved
    by the persistent batched kernel replayed as one CUDA graph, launch shape
    autotuned: FP64 sweeps on the FP64 pipe, the same sweeps in double-float
    arithmetic, and mixed (FP32 sweeps, then double-float or FP64-pipe
    certifying sweeps)."""
    from block_ipt_gb300 import api, workloads
    specs = workloads.batch_config2(args.batch, seed=args.seed)
    bufs, inst = [], []
    for n, k, sig, seed in specs:
        H, _ = workloads.batch_instance_torch(torch, n, sig, seed, device=dev)
        dX = torch.empty((k, n), dtype=torch.float64, device=dev)
        dv = torch.empty(k, dtype=torch.float64, device=dev)
        bufs.append((H, dX, dv))
        inst.append((H.data_ptr(), n, k, dX.data_ptr(), dv.data_ptr()))
    torch.cuda.synchronize()
    out = {"workload": "%d dense instances, n~U{64..2048}, k~U{4..16}, sigma~U(0.01,0.1), "
                       "seed %d" % (len(specs), args.seed),
           "fp64_bytes_of_H": int(sum(8 * n * n for n, _, _, _ in specs))}
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream(dev)
    from block_ipt_gb300 import _lib
    for name, prec, cert in (("fp64", "fp64", _lib.IPT_BLOCK_FP64),
                             ("fp64_double_float", "fp64", _lib.IPT_BLOCK_DF64),
                             ("mixed", "fp32", _lib.IPT_BLOCK_DF64),
                             ("mixed_fp64_certify", "fp32", _lib.IPT_BLOCK_FP64)):
        plan = api.BatchPlan(inst, prec, certify_precision=cert)
        threads, chunk, _ = plan.autotune(stream.cuda_stream)
        plan.run(stream.cuda_stream)
        times = []
        for _ in range(max(1, args.batch_steps)):
            e0.record(stream)
            plan.run(stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        reps = plan.reports()
        shape = plan.shape()
        plan.close()
        lat = np.array([r["latency_ms"] for r in reps])
        ms = statistics.median(times)
        out[name] = {
            "ms_per_batch": ms, "instances_per_s": len(specs) / (ms * 1e-3),
            "p50_latency_ms": float(np.percentile(lat, 50)),
            "p99_latency_ms": float(np.percentile(lat, 99)),
            "converged": int(sum(r["converged"] for r in reps)),
            "max_scaled_residual": float(max(r["max_scaled_residual"] for r in reps)),
            "mean_sweeps": float(np.mean([r["iterations"] for r in reps])),
            "mean_fp64_sweeps": float(np.mean([r["fp64_iterations"] for r in reps])),
            "autotuned": shape, "graph_launches": len(times) + 1}
    # eigenvalue check of a few instances against LAPACK
    worst = 0.0
    for b in range(0, len(specs), max(1, len(specs) // 4)):
        H, _, dv = bufs[b]
        Hn = H.cpu().numpy()
        k = specs[b][1]
        w = np.linalg.eigvalsh(Hn)[:k]
        worst = max(worst, float(np.abs(np.sort(dv.cpu().numpy()) - w).max()
                                 / np.abs(Hn).sum(axis=1).max()))
    out["check"] = {"max_abs_dlambda_over_norm_inf_sampled": worst}
    if not args.no_cpu:
        out["cpu_baseline"] = batch_cpu_baseline(specs)
    del bufs
    torch.cuda.empty_cache()
    return out


def fci_free_section(args, torch, dev, mlp_params=None):
    """The matrix-free FCI-like workload: norb orbitals with norb/2 alpha and
    norb/2 beta electrons (14 -> 11,778,624 determinants, 3,381 couplings per
    row), k = 8, H regenerated from hashes inside every sigma build.  Plain
    FP64-accurate Davidson vs a BF16-sigma phase followed by the FP64 one
    (and the learned preconditioner when trained), each to the scaled
    residual 1e-8; sigma timed alone per precision."""
    from block_ipt_gb300 import api
    norb = args.fci_free_orbitals
    spec = api.fci_spec(norb, norb // 2, norb // 2, seed=args.seed)
    n = api.fci_dimension(spec)
    k = 8
    couplings = 2 * (norb // 2) ** 2 + 2 * ((norb // 2) * (norb // 2 - 1) // 2) ** 2 \
        + (norb // 2) ** 4
    out = {"workload": "matrix-free FCI-like, %d orbitals %d+%d electrons, n=%d, %d couplings "
                       "per row, k=%d, seed %d" % (norb, norb // 2, norb // 2, n, couplings, k,
                                                   args.seed)}
    X = torch.randn((k, n), dtype=torch.float64, device=dev)
    Y = torch.empty_like(X)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    sig = {}
    for prec in ("fp64", "fp32", "bf16"):
        api.fci_sigma(spec, X.data_ptr(), k, Y.data_ptr(), prec)
        torch.cuda.synchronize()
        e0.record()
        api.fci_sigma(spec, X.data_ptr(), k, Y.data_ptr(), prec)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        esize = {"fp64": 8, "fp32": 4, "bf16": 2}[prec]
        # minimal bytes: X once (k values per determinant), Y once (FP64), diagonal
        minimal = n * k * esize + n * k * 8 + n * 8
        sig[prec] = {"ms_incl_setup": ms, "couplings_per_s": n * couplings / (ms * 1e-3),
                     "achieved_gflops": 2.0 * n * couplings * k / (ms * 1e-3) / 1e9,
                     "minimal_bytes": minimal,
                     "gbs_of_minimal_bytes": minimal / (ms * 1e-3) / 1e9}
    out["sigma_k8"] = sig
    del X, Y
    dX = torch.empty((k, n), dtype=torch.float64, device=dev)
    dv = torch.empty(k, dtype=torch.float64, device=dev)
    runs = [("fp64", {}), ("bf16", {})]
    if mlp_params is not None:
        # the learned correction on the FP64-accurate Davidson (its second-order
        # term from the FP32 sigma); after the BF16 phase its first steps are
        # rejected and the solve falls back to the plain correction
        runs.append(("fp64_learned", {"preconditioner": 1, "mlp_params": mlp_params.data_ptr()}))
    for name, extra in runs:
        prec = "bf16" if name.startswith("bf16") else "fp64"
        t0 = time.perf_counter()
        rep = api.block_solve_fci(spec, k, dX.data_ptr(), dv.data_ptr(), prec, strategy=1,
                                  davidson_maxsteps=60, **extra)
        torch.cuda.synchronize()
        out[name] = {"s": time.perf_counter() - t0, "converged": rep["converged"],
                     "davidson_steps": rep["davidson_steps"], "fp64_matvecs": rep["fp64_matvecs"],
                     "lowp_matvecs": rep["lowp_matvecs"],
                     "max_scaled_residual": rep["max_scaled_residual"],
                     "mlp_steps_accepted": rep["mlp_steps_accepted"],
                     "mlp_steps_rejected": rep["mlp_steps_rejected"],
                     "precond_matvecs": rep["precond_matvecs"],
                     "lowest": dv.cpu().numpy()[:3].tolist()}
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    from block_ipt_gb300 import _lib, api, workloads

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    lib = _lib.load()
    dev = torch.device("cuda", local)
    n, k = args.n, args.k
    # one independent instance per rank ("replicas only": the dense solve is
    # not sharded), seeded by rank
    H, _ = workloads.dense_config1(n, seed=replica_seed(args.seed, rank))
    H = np.asfortranarray(H)
    hnorm = float(np.abs(H).sum(axis=1).max())
    H_pinned = torch.from_numpy(H.T.copy()).pin_memory()  # row-major view of H^T = col-major H
    dH = H_pinned.to(dev)
    dHsym = dH  # symmetric: the same buffer is H in either order for the check
    dX = torch.empty((k, n), dtype=torch.float64, device=dev)  # column-major n x k
    dv = torch.empty(k, dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    stream = torch.cuda.current_stream(dev)
    kw = dict(ipt_maxiter=80, ipt_check_every=8, stream=stream.cuda_stream)

    def solve(prec, **extra):
        opts = dict(kw)
        opts.update(extra)
        return api.block_solve_dense_device(dH.data_ptr(), n, k, dX.data_ptr(), dv.data_ptr(),
                                            prec, **opts)

    for _ in range(args.warmup):
        solve(args.precision)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    lib.ipt_block_profile_enable(0)
    launches0 = lib.ipt_block_launch_count()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    times, reports, worst_res = [], [], 0.0
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        flush.zero_()
        e0.record(stream)
        rep = solve(args.precision)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        reports.append(rep)
        worst_res = max(worst_res, fp64_check(torch, dHsym.T, dX.T, dv, hnorm))
    torch.cuda.synchronize()
    launches = lib.ipt_block_launch_count() - launches0
    clocks = sampler.stop()
    # per-kernel CUDA-event timings over a second pass of the same K solves:
    # the events around every instrumented launch cost ~0.4 ms of host time per
    # solve, so the headline pass above runs without them
    lib.ipt_block_profile_reset()
    lib.ipt_block_profile_enable(1)
    prof_reports = []
    for _ in range(args.steps):
        flush.zero_()
        prof_reports.append(solve(args.precision))
    torch.cuda.synchronize()
    lib.ipt_block_profile_enable(0)
    prof = profile_snapshot(lib)
    if args.trace and rank == 0:
        write_trace(args.trace, api, torch, lambda: solve(args.precision), flush)
    ms = max_over_ranks(statistics.mean(times), world, dev)

    # eigenvalues against LAPACK dsyevd (once, outside the timed region; its
    # time is reported beside the CPU baseline)
    vals = dv.cpu().numpy()
    dlambda = None
    dsyevd = None
    if not args.no_lapack and rank == 0:
        dsyevd, w = dsyevd_leg(H, k)
        dlambda = float(np.abs(vals - w).max() / hnorm)

    # plain FP64 IPT path of the same code (FP64 IPT steps to the same
    # residual, then the same Rayleigh-Ritz), and the FP64 Davidson strategy
    def timed_runs(count, prec, **extra):
        ms_list, last = [], None
        for _ in range(count):
            flush.zero_()
            e0.record(stream)
            last = solve(prec, **extra)
            e1.record(stream)
            e1.synchronize()
            ms_list.append(e0.elapsed_time(e1))
        return (statistics.mean(ms_list) if ms_list else None), last

    plain, plain_rep = timed_runs(args.plain_steps, "fp64", strategy=0)
    fp64_dav, fp64_dav_rep = timed_runs(args.plain_steps, "fp64", strategy=1)

    # end to end through the host entry point (pinned H in, pairs out)
    Xh = np.zeros((n, k), order="F")
    vh = np.zeros(k)
    Hptr = C.c_void_p(H_pinned.data_ptr())
    opt = api.block_options(args.precision, **kw)

    def e2e_call():
        rep = _lib.IPTBlockReport()
        st = lib.ipt_block_solve_dense(Hptr, n, k, C.byref(opt), C.c_void_p(Xh.ctypes.data),
                                       C.c_void_p(vh.ctypes.data), C.byref(rep))
        assert st == 0, _lib.status_string(st)
        return rep

    # untimed warm-up of the host entry point: its first call grows the
    # stream-ordered pool by the device copy of H (steady-state serving
    # reuses it)
    for _ in range(min(2, args.e2e_steps)):
        e2e_call()
    torch.cuda.synchronize()
    e2e = []
    for _ in range(args.e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rep = _lib.IPTBlockReport()
        st = lib.ipt_block_solve_dense(Hptr, n, k, C.byref(opt), C.c_void_p(Xh.ctypes.data),
                                       C.c_void_p(vh.ctypes.data), C.byref(rep))
        torch.cuda.synchronize()
        e2e.append((time.perf_counter() - t0) * 1e3)
        assert st == 0, _lib.status_string(st)
        assert rep.converged == 1
    e2e_ms = statistics.mean(e2e) if e2e else None

    # roofline of the dominant kernel of the timed region (the larger of the
    # low-precision product and the FP64-accurate product, by total time)
    steps = args.steps
    avg_rep = reports[-1]
    with open(MEASURED_PEAKS) as f:
        peaks = json.load(f)
    lp_ms, lp_cnt = prof["lowp_product"]
    ldp = (n + 63) // 64 * 64
    esize = 2 if args.precision in ("fp16", "bf16") else 4
    lp_bytes = n * ldp * esize + ldp * ((k + 8 + 15) // 16 * 16) * esize
    lp_ach = lp_bytes / (lp_ms / max(1, lp_cnt) * 1e-3) / 1e9 if lp_cnt else None
    lp_traffic = NCU_TRAFFIC.get(("tc_stream", n, k, args.precision))
    lp_dram = (lp_traffic / (lp_ms / max(1, lp_cnt) * 1e-3) / 1e9) if (lp_traffic and lp_cnt) else None
    roofline_lowp = {"kernel": "tc_stream_kernel (tcgen05 + TMA, persistent stream-K, %s)"
                               % args.precision,
                     "bound": "hbm", "achieved": lp_ach, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": (lp_ach / peaks["hbm_gbs"]) if lp_ach else None,
                     "traffic": lp_traffic,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + write.sum)",
                     "dram_only_achieved": lp_dram,
                     "dram_only_frac": (lp_dram / peaks["hbm_gbs"]) if lp_dram else None,
                     "dram_only_note": "DRAM bytes of a launch inside the solve (the L2-kept share "
                                       "of Delta is not counted) over the same live launch time",
                     "launches": lp_cnt,
                     "avg_launch_ms": lp_ms / max(1, lp_cnt),
                     "algorithmic_bytes_per_launch": lp_bytes,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    # the FP64-accurate products of the refinement (k columns each): six FP16
    # digit slices of Delta streamed once per product, the X slices written
    # and read, X read and H X written (k_oz.cu); bound: HBM.  Its timer spans
    # the X split, the tensor-core product and the finish kernel.
    fp_ms, fp_cnt = prof["fp64_product"]
    cp = (k + 15) // 16 * 16
    acc_bytes = 12 * n * ldp + 24 * cp * ldp + 16 * n * k
    acc_ach = acc_bytes / (fp_ms / max(1, fp_cnt) * 1e-3) / 1e9 if fp_cnt else None
    # MMA work: slice s times B rows (6 - s) cp, over every (row, K) pair
    mma_flops = 2.0 * ((n + 127) // 128 * 128) * ldp * sum((6 - s) * cp for s in range(6))
    roofline_accurate = {
        "kernel": "oz_product_kernel (FP64-accurate product: 6+6 FP16 digit slices, tcgen05 "
                  "+ TMA, persistent)",
        "bound": "hbm", "achieved": acc_ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": (acc_ach / peaks["hbm_gbs"]) if acc_ach else None,
        "traffic": NCU_TRAFFIC.get(("oz_product", n, k, args.precision)),
        "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + write.sum)",
        "launches": fp_cnt, "avg_launch_ms": fp_ms / max(1, fp_cnt),
        "algorithmic_bytes_per_launch": acc_bytes,
        "tensor_tflops": (mma_flops / (fp_ms / max(1, fp_cnt) * 1e-3) / 1e12) if fp_cnt else None,
        "tensor_peak_tflops": peaks["bf16_tflops"],
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
    roofline = roofline_accurate if fp_ms > lp_ms else roofline_lowp

    fci = None
    mlp_params = None
    if not args.no_fci and rank == 0:
        fci = fci_section(args, torch, lib, stream, flush, dev)
        if fci.get("learned"):
            mlp_params = fci["learned"].pop("_params", None)
    batched = None
    if not args.no_batch and rank == 0:
        batched = batch_section(args, torch, dev)
    fci_free = None
    if not args.no_fci_free and rank == 0:
        fci_free = fci_free_section(args, torch, dev, mlp_params)

    lowp_sweep = None
    if not args.no_lowp_sweep and rank == 0:
        try:
            lowp_sweep = lowp_sweep_section(torch, lib, dev, k, peaks["hbm_gbs"])
        except Exception as exc:  # a side measurement never takes the headline line down
            lowp_sweep = {"error": repr(exc)}

    acx = None
    if not args.no_acx and rank == 0:
        try:
            acx = acx_section(torch, lib, dH, n, k)
        except Exception as exc:  # a side measurement never takes the headline line down
            acx = {"error": repr(exc)}

    cpu = None
    if not args.no_cpu and rank == 0:
        from oracle import oracle
        cpu_ms, cnt, cres = cpu_solve(H, k)
        cpu = {"value": cpu_ms, "unit": "ms", "cores": oracle.num_threads(), "kind": "port",
               "sample": cpu_sample_text(n, k, cnt), "final_scaled_residual": cres,
               "one_core": {"ms": cpu_one_core_iteration(H, k), "cores": 1,
                            "sample": "one plain-IPT iteration (one block product and the "
                                      "update) plus the eigenvalue product, n=%d k=%d" % (n, k)},
               "dsyevd": dsyevd}

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "%s+f64" % args.precision,
            "data": "synthetic",
            "config": bench_config(args),
            "method": METHOD.replace("FP16", args.precision.upper()),
            "learned_preconditioner": "acts on Davidson steps; this workload converges in the "
                                      "mixed refinement, so it is timed on the FCI-like "
                                      "workload (fci_config3.learned)",
            # the host entry moves the upper triangle of H (symmetric) across the link
            "e2e": ({"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 4 * n * (n + 1),
                     "d2h_bytes_per_step": 8 * n * k + 8 * k} if e2e_ms is not None else None),
            "gpu_launches": launches,
            "roofline": roofline,
            "roofline_lowp": roofline_lowp,
            "roofline_accurate": roofline_accurate,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "plain_fp64_ms": plain,
            "speedup_vs_plain_fp64": (plain / ms) if plain else None,
            "fp64_davidson_ms": fp64_dav,
            "speedup_vs_fp64_davidson": (fp64_dav / ms) if fp64_dav else None,
            "check": {"max_scaled_residual": worst_res, "max_abs_dlambda_over_norm_inf": dlambda,
                      "converged": all(r["converged"] == 1 for r in reports)},
            "report": {kk: avg_rep[kk] for kk in ("ipt_iterations", "davidson_steps", "restarts",
                                                  "basis_cols", "fp64_matvecs", "lowp_matvecs",
                                                  "ipt_ms", "rayleigh_ritz_ms", "davidson_ms",
                                                  "total_ms")},
            "plain_report": ({kk: plain_rep[kk] for kk in ("ipt_iterations", "davidson_steps",
                                                           "fp64_matvecs", "total_ms", "converged")}
                             if plain_rep else None),
            "fp64_davidson_report": ({kk: fp64_dav_rep[kk] for kk in (
                "ipt_iterations", "davidson_steps", "fp64_matvecs", "total_ms", "converged")}
                if fp64_dav_rep else None),
            "kernel_ms": {kk: round(v[0] / steps, 4) for kk, v in prof.items() if v[1]},
            "fci_config3": fci,
            "batched_config2": batched,
            "matrix_free_config4": fci_free,
            "acx_fp64": acx,
            "lowp_product_sweep": lowp_sweep,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
