"""Small fixed workloads for timing and profiling single kernels of the
library on cuda:0 (each prints one line and exits 0 on success):

    python -m block_ipt_gb300.microbench accurate N C
        ipt_block_accurate_product on a random symmetric N x N H and C
        columns, three calls, checked against the FP64 product of torch;
    python -m block_ipt_gb300.microbench lowp N [K] [STEPS]
        ipt_mixed_precision_cuda_device_tol with STEPS (30) fixed FP16 IPT
        steps on the N x N headline-family matrix (workloads.dense_config1),
        three runs; prints the per-launch time of the low-precision product;
    python -m block_ipt_gb300.microbench solve N [K]
        two FP16 mixed dense solves (ipt_block_solve_dense_device) of the
        headline-family matrix;
    python -m block_ipt_gb300.microbench solve_host N [K]
        FP16 mixed solves of it through the host entry from pinned memory,
        with the phase marks of the last;
    python -m block_ipt_gb300.microbench batch COUNT [MIXED] [THREADS] [RUNS]
        the batched solver on the first COUNT instances of the 512-instance
        batched workload (MIXED = 1: FP32 sweeps and double-float
        certification, 0: FP64 sweeps), default launch shape with THREADS
        (256) per CTA, RUNS (2) graph launches, the last one timed.

Environment knobs of the library (IPT_GB300_*) apply as usual."""
import ctypes as C
import sys

import numpy as np


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("microbench needs a CUDA device")
    return torch


def accurate(n, c):
    torch = _torch()
    from . import _lib
    lib = _lib.load()
    rng = np.random.default_rng(0)
    H = rng.standard_normal((n, n))
    H = H + H.T
    dH = torch.from_numpy(H).cuda()
    dX = torch.from_numpy(rng.standard_normal((c, n))).cuda()
    dY = torch.empty((c, n), dtype=torch.float64, device="cuda")
    for _ in range(3):
        st = lib.ipt_block_accurate_product(C.c_void_p(dH.data_ptr()), n,
                                            C.c_void_p(dX.data_ptr()), c,
                                            C.c_void_p(dY.data_ptr()), None)
        if st != 0:
            raise SystemExit("ipt_block_accurate_product status %d" % st)
    torch.cuda.synchronize()
    ref = (dH @ dX.T).T
    err = ((dY - ref).abs().max() / ref.abs().max()).item()
    print("accurate product n=%d c=%d: max|Y - Y_fp64| / max|Y| = %.3g" % (n, c, err))
    if not err <= 1e-13:
        raise SystemExit(1)


def dense_headline(torch, n):
    from . import workloads
    H, _ = workloads.dense_config1(n, seed=0)
    dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()
    return dH


def lowp(n, k=32, steps=30):
    torch = _torch()
    from . import _lib
    lib = _lib.load()
    dH = dense_headline(torch, n)
    res = _lib._MixedResult()

    def run():
        st = lib.ipt_mixed_precision_cuda_device_tol(
            C.c_void_p(dH.data_ptr()), n, k, 1e-300, steps, 1e300, 1,
            C.c_void_p(torch.cuda.current_blas_handle()), C.byref(res))
        if st != 0:
            raise SystemExit("ipt_mixed_precision_cuda_device_tol status %d" % st)
        lib.ipt_mixed_precision_cuda_free_device_result(C.byref(res))

    run()
    torch.cuda.synchronize()
    lib.ipt_block_profile_reset()
    lib.ipt_block_profile_enable(1)
    run()
    run()
    torch.cuda.synchronize()
    lib.ipt_block_profile_enable(0)
    name, ms, cnt = C.c_char_p(), C.c_double(), C.c_longlong()
    lib.ipt_block_profile_read(0, C.byref(name), C.byref(ms), C.byref(cnt))
    print("%s n=%d k=%d: %.2f us per launch over %d launches"
          % (name.value.decode(), n, k, 1e3 * ms.value / max(1, cnt.value), cnt.value))


def solve(n, k=32):
    torch = _torch()
    from . import api
    dH = dense_headline(torch, n)
    dX = torch.empty((k, n), dtype=torch.float64, device="cuda")
    dv = torch.empty(k, dtype=torch.float64, device="cuda")
    rep = None
    for _ in range(2):
        rep = api.block_solve_dense_device(dH.data_ptr(), n, k, dX.data_ptr(), dv.data_ptr(),
                                           "fp16")
    torch.cuda.synchronize()
    print("dense FP16 solve n=%d k=%d: converged %d, max scaled residual %.3g"
          % (n, k, rep["converged"], rep["max_scaled_residual"]))
    if rep["converged"] != 1:
        raise SystemExit(1)


def solve_host(n, k=32):
    """Three FP16 mixed solves through the host entry with H in pinned memory
    (ipt_block_solve_dense); prints the wall time of the last and its phase
    marks (GPU global timer and host clock)."""
    torch = _torch()
    import time
    from . import _lib, api, workloads
    lib = _lib.load()
    H, _ = workloads.dense_config1(n, seed=0)
    pinned = torch.from_numpy(np.asfortranarray(H).T.copy()).pin_memory()
    del H
    opt = api.block_options("fp16")
    X = np.zeros((n, k), order="F")
    v = np.zeros(k)
    rep = _lib.IPTBlockReport()

    def run():
        st = lib.ipt_block_solve_dense(C.c_void_p(pinned.data_ptr()), n, k, C.byref(opt),
                                       C.c_void_p(X.ctypes.data), C.c_void_p(v.ctypes.data),
                                       C.byref(rep))
        if st != 0:
            raise SystemExit("ipt_block_solve_dense status %d" % st)

    run()
    run()
    api.trace_enable(True)
    t0 = time.perf_counter()
    run()
    ms = (time.perf_counter() - t0) * 1e3
    marks = api.trace_read()
    api.trace_enable(False)
    print("host dense FP16 solve n=%d k=%d from pinned memory: %.3f ms, converged %d"
          % (n, k, ms, rep.converged))
    g0 = marks[0][2] if marks else 0
    h0 = marks[0][1] if marks else 0
    for label, host_ns, gpu_ns in marks:
        print("  %-32s gpu %9.1f us  host %9.1f us" % (label, (gpu_ns - g0) / 1e3,
                                                     (host_ns - h0) / 1e3))


def batch(count, mixed=1, threads=256, runs=2):
    torch = _torch()
    from . import api, workloads
    specs = workloads.batch_config2(512, seed=0)[:count]
    bufs, inst = [], []
    for n, k, sig, seed in specs:
        H, _ = workloads.batch_instance_torch(torch, n, sig, seed)
        dX = torch.empty((k, n), dtype=torch.float64, device="cuda")
        dv = torch.empty(k, dtype=torch.float64, device="cuda")
        bufs.append((H, dX, dv))
        inst.append((H.data_ptr(), n, k, dX.data_ptr(), dv.data_ptr()))
    plan = api.BatchPlan(inst, "fp32" if mixed else "fp64", threads=threads)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(max(1, runs)):
        torch.cuda.synchronize()
        e0.record()
        plan.run(torch.cuda.current_stream().cuda_stream)
        e1.record()
        e1.synchronize()
    reps = plan.reports()
    shape = plan.shape()
    plan.close()
    conv = sum(r["converged"] for r in reps)
    print("batch of %d (%s): %.3f ms, converged %d, shape %s"
          % (count, "mixed" if mixed else "fp64", e0.elapsed_time(e1), conv, shape))
    if conv != count:
        raise SystemExit(1)


def main(argv):
    cmds = {"accurate": accurate, "lowp": lowp, "solve": solve, "solve_host": solve_host,
            "batch": batch}
    if len(argv) < 2 or argv[0] not in cmds:
        raise SystemExit(__doc__)
    args = [int(a) for a in argv[1:]]
    cmds[argv[0]](*args)


if __name__ == "__main__":
    main(sys.argv[1:])
