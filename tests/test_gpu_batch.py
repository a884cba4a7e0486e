"""Batched dense solver (k_batch.cu) through the C ABI: every instance against
the oracle's plain IPT (same block, same number of products), eigenvalues
against LAPACK, the mixed-precision mode, graph replay, the autotuner, and
argument checks.  Instances use the batched construction of
workloads.batch_config2 (configs[0] matrices with per-instance n, k, sigma)."""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib, api, workloads
from oracle import oracle

pytestmark = pytest.mark.gpu


def make_batch(torch, specs):
    """specs: [(n, k, sigma, seed)] -> (host matrices, device tensors, instance tuples)."""
    Hs, dev, inst = [], [], []
    for n, k, sig, seed in specs:
        H, _ = workloads.batch_instance(n, sig, seed)
        dH = torch.from_numpy(np.asfortranarray(H).T.copy()).cuda()  # column-major
        dX = torch.zeros((k, n), dtype=torch.float64, device="cuda")
        dv = torch.zeros(k, dtype=torch.float64, device="cuda")
        Hs.append(H)
        dev.append((dH, dX, dv))
        inst.append((dH.data_ptr(), n, k, dX.data_ptr(), dv.data_ptr()))
    return Hs, dev, inst


SMALL = [(64, 4, 0.05, 11), (97, 16, 0.1, 12), (130, 7, 0.01, 13), (256, 16, 0.08, 14),
         (300, 5, 0.03, 15), (77, 9, 0.06, 16), (200, 12, 0.1, 17), (150, 16, 0.02, 18)]


def test_batch_fp64_matches_oracle(cuda):
    torch = cuda
    Hs, dev, inst = make_batch(torch, SMALL)
    plan = api.BatchPlan(inst, "fp64", threads=256)
    plan.run()
    torch.cuda.synchronize()
    reps = plan.reports()
    for (n, k, _, _), H, (_, dX, dv), rep in zip(SMALL, Hs, dev, reps):
        assert rep["converged"] == 1 and rep["max_scaled_residual"] <= 1e-8
        prods, _ = oracle.products_to_residual(H, k, 500, 1e-8)
        assert rep["fp64_iterations"] == prods
        Xo, _, _, _ = oracle.ipt_dense(H, k, prods - 1)
        X = dX.T.cpu().numpy()
        v = dv.cpu().numpy()
        assert np.abs(X - Xo).max() <= 1e-12
        rq = np.einsum("ij,ij->j", Xo, H @ Xo) / np.einsum("ij,ij->j", Xo, Xo)
        assert np.abs(v - rq).max() <= 1e-12 * max(1.0, np.abs(rq).max())
        hn = np.abs(H).sum(axis=1).max()
        w = np.linalg.eigvalsh(H)[:k]
        assert np.abs(np.sort(v) - w).max() <= 1e-10 * hn
    plan.close()


def test_batch_mixed_precision(cuda):
    torch = cuda
    Hs, dev, inst = make_batch(torch, SMALL)
    plan64 = api.BatchPlan(inst, "fp64")
    plan64.run()
    torch.cuda.synchronize()
    r64 = plan64.reports()
    v64 = [d[2].cpu().numpy().copy() for d in dev]
    plan32 = api.BatchPlan(inst, "fp32")
    plan32.run()
    torch.cuda.synchronize()
    r32 = plan32.reports()
    for (n, k, _, _), H, (_, dX, dv), a, b, v in zip(SMALL, Hs, dev, r64, r32, v64):
        assert b["converged"] == 1 and b["max_scaled_residual"] <= 1e-8
        assert b["fp64_iterations"] < a["fp64_iterations"]
        hn = np.abs(H).sum(axis=1).max()
        assert np.abs(dv.cpu().numpy() - v).max() <= 1e-10 * hn
        X = dX.T.cpu().numpy()
        r = H @ X - X * dv.cpu().numpy()[None, :]
        sc = np.linalg.norm(r, axis=0) / (max(1.0, hn) * np.maximum(1.0, np.linalg.norm(X, axis=0)))
        assert sc.max() <= 1e-8
    plan64.close()
    plan32.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_certifying_sweeps_fp64_and_double_float(cuda, precision):
    """The certifying sweeps on the FP64 pipe and in double-float arithmetic
    reach the same certified eigenpairs (scaled residual <= 1e-8 checked on
    the host, eigenvalues within 1e-10 ||H||_inf of each other)."""
    torch = cuda
    Hs, dev, inst = make_batch(torch, SMALL)
    vals = {}
    for cert in (_lib.IPT_BLOCK_FP64, _lib.IPT_BLOCK_DF64):
        plan = api.BatchPlan(inst, precision, certify_precision=cert)
        plan.run()
        torch.cuda.synchronize()
        reps = plan.reports()
        plan.close()
        vals[cert] = [d[2].cpu().numpy().copy() for d in dev]
        for H, (_, dX, dv), r in zip(Hs, dev, reps):
            assert r["converged"] == 1 and r["max_scaled_residual"] <= 1e-8
            hn = np.abs(H).sum(axis=1).max()
            X = dX.T.cpu().numpy()
            res = H @ X - X * dv.cpu().numpy()[None, :]
            sc = np.linalg.norm(res, axis=0) / (max(1.0, hn) *
                                                 np.maximum(1.0, np.linalg.norm(X, axis=0)))
            assert sc.max() <= 1e-8
    for H, a, b in zip(Hs, vals[_lib.IPT_BLOCK_FP64], vals[_lib.IPT_BLOCK_DF64]):
        assert np.abs(a - b).max() <= 1e-10 * np.abs(H).sum(axis=1).max()


def test_batch_graph_replay_and_autotune_are_deterministic(cuda):
    torch = cuda
    Hs, dev, inst = make_batch(torch, SMALL)
    plan = api.BatchPlan(inst, "fp32")
    plan.run()
    torch.cuda.synchronize()
    first = [d[1].cpu().numpy().copy() for d in dev]
    t, c, ms = plan.autotune()
    assert t in (128, 256, 512) and c in (64, 128) and ms > 0
    plan.run()
    plan.run()
    torch.cuda.synchronize()
    for f, d in zip(first, dev):
        assert np.array_equal(f, d[1].cpu().numpy())
    reps = plan.reports()
    assert all(r["latency_ms"] > 0 and r["completion_ms"] >= r["latency_ms"] - 1e-6 for r in reps)
    plan.close()


def test_batch_config2_shape(cuda):
    """64 instances drawn like the 512-instance batch (n <= 2048, k <= 16)."""
    torch = cuda
    specs = workloads.batch_config2(64, seed=3)
    Hs, dev, inst = make_batch(torch, specs)
    plan = api.BatchPlan(inst, "fp32")
    plan.autotune()
    plan.run()
    torch.cuda.synchronize()
    reps = plan.reports()
    assert all(r["converged"] == 1 for r in reps)
    for b in (0, 17, 40):
        H = Hs[b]
        k = specs[b][1]
        w = np.linalg.eigvalsh(H)[:k]
        v = np.sort(dev[b][2].cpu().numpy())
        assert np.abs(v - w).max() <= 1e-10 * np.abs(H).sum(axis=1).max()
    plan.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_cluster_teams_match_single_cta_solves(cuda, monkeypatch, precision):
    """The most expensive instances are solved by a whole thread-block cluster
    (rows split over its CTAs, sums exchanged through distributed shared
    memory): the same blocks, sweep counts and eigenpairs as when every
    instance runs on one CTA, and the LAPACK eigenvalues."""
    torch = cuda
    specs = [(2048, 16, 0.05, 31), (1536, 9, 0.1, 32), (1100, 13, 0.02, 33), (640, 4, 0.08, 34),
             (300, 16, 0.06, 35), (96, 5, 0.03, 36), (257, 12, 0.1, 37), (64, 4, 0.01, 38)]
    Hs, dev, inst = make_batch(torch, specs)
    results = {}
    for pct in ("25", "0"):
        monkeypatch.setenv("IPT_GB300_BATCH_TEAM_PCT", pct)
        plan = api.BatchPlan(inst, precision)
        shape = plan.shape()
        plan.run()
        torch.cuda.synchronize()
        reps = plan.reports()
        plan.close()
        if pct == "0":
            assert shape["cluster"] == 1 and shape["team_instances"] == 0
        else:
            assert shape["cluster"] > 1 and shape["team_instances"] >= 2, shape
        results[pct] = ([d[1].cpu().numpy().copy() for d in dev],
                        [d[2].cpu().numpy().copy() for d in dev], reps)
    (Xt, vt, rt), (Xs, vs, rs) = results["25"], results["0"]
    for (n, k, _, _), H, a, b, va, vb, ra, rb in zip(specs, Hs, Xt, Xs, vt, vs, rt, rs):
        assert ra["converged"] == 1 and rb["converged"] == 1
        assert ra["iterations"] == rb["iterations"]
        assert ra["fp64_iterations"] == rb["fp64_iterations"]
        assert np.abs(a - b).max() <= 1e-12
        hn = np.abs(H).sum(axis=1).max()
        assert np.abs(va - vb).max() <= 1e-12 * hn
        w = np.linalg.eigvalsh(H)[:k]
        assert np.abs(np.sort(va) - w).max() <= 1e-10 * hn


def test_batch_invalid_arguments(cuda):
    torch = cuda
    lib = _lib.load()
    dH = torch.eye(8, dtype=torch.float64, device="cuda")
    dX = torch.zeros(8 * 17, dtype=torch.float64, device="cuda")
    for n, k in ((8, 9), (8, 0), (0, 1), (20, 17)):
        with pytest.raises(_lib.IPTError):
            api.BatchPlan([(dH.data_ptr(), n, k, dX.data_ptr(), dX.data_ptr())])
    with pytest.raises(_lib.IPTError):
        api.BatchPlan([(dH.data_ptr(), 8, 2, dX.data_ptr(), dX.data_ptr())], threads=300)
    plan = C.c_void_p()
    assert lib.ipt_block_batch_plan_create(None, 1, None, C.byref(plan)) == 1
    assert lib.ipt_block_batch_plan_run(None, None) == 1
