"""GPU tests of the learned Davidson preconditioner (k_mlp.cu) through the C
ABI: forward, gradient and Adam kernels against the CPU oracle
(oracle/mlp_oracle.py, float64; tolerances cover the kernels' FP32
arithmetic), training, the collector, what the trained network gains over
the plain diagonal correction, and the FP64 rejection fallback."""
import numpy as np
import pytest

from block_ipt_gb300 import api, learned
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

MASK = (1 << 64) - 1


def splitmix(x):
    x = (x + 0x9E3779B97F4A7C15) & MASK
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & MASK
    return x ^ (x >> 31)


def random_rows(rng, count):
    F = rng.standard_normal((count, 6))
    return np.column_stack([F, rng.standard_normal(count), rng.uniform(0.1, 2.0, count)])


def gpu_params(torch, seed):
    P = torch.empty(api.mlp_param_count(), dtype=torch.float32, device="cuda")
    api.mlp_init(P.data_ptr(), seed)
    torch.cuda.synchronize()
    return P


def test_init(cuda):
    P = gpu_params(cuda, 3).cpu().numpy().astype(np.float64)
    d = M.unpack(P)
    assert d["b3"][0] == 4.0  # o = sigmoid(z) starts near 1, the two-term correction
    assert np.all(d["b1"] == 0) and np.all(d["b2"] == 0)
    assert np.abs(d["W1"]).max() <= 1.0 and 0 < np.abs(d["W2"]).max() <= np.sqrt(6 / 64)


def test_forward_matches_oracle(cuda):
    torch = cuda
    rng = np.random.default_rng(4)
    P = gpu_params(torch, 5)
    rows = random_rows(rng, 3000)
    dR = torch.from_numpy(rows.astype(np.float32)).cuda()
    out = torch.empty(3000, dtype=torch.float32, device="cuda")
    api.mlp_forward(P.data_ptr(), dR.data_ptr(), 3000, 8, out.data_ptr())
    ref, _ = M.forward(P.cpu().numpy(), rows.astype(np.float32)[:, :6])
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_gradient_matches_oracle(cuda):
    """Gradient check of the fused forward/backward kernel against the CPU oracle."""
    torch = cuda
    rng = np.random.default_rng(6)
    P = gpu_params(torch, 8)
    # non-trivial output layer so that every gradient block is exercised
    P[4608:4672] = torch.from_numpy(rng.standard_normal(64).astype(np.float32) * 0.3).cuda()
    rows = random_rows(rng, 1000).astype(np.float32)
    dR = torch.from_numpy(rows).cuda()
    g = torch.empty(api.mlp_param_count() + 1, dtype=torch.float32, device="cuda")
    api.mlp_loss_grad(P.data_ptr(), dR.data_ptr(), 1000, g.data_ptr())
    g = g.cpu().numpy().astype(np.float64)
    loss, gref = M.loss_grad(P.cpu().numpy(), rows)
    assert abs(g[-1] - loss) <= 1e-5 * max(1.0, loss)
    scale = np.abs(gref).max()
    assert np.abs(g[:-1] - gref).max() <= 1e-4 * scale
    for name, (lo, hi) in {"W1": (0, 384), "W2": (448, 4544), "W3": (4608, 4672)}.items():
        blk = gref[lo:hi]
        assert np.linalg.norm(g[lo:hi] - blk) <= 1e-4 * np.linalg.norm(blk), name


def test_adam_trajectory_matches_oracle(cuda):
    """Three Adam steps on hash-sampled batches, GPU (FP32) vs oracle (FP64)."""
    torch = cuda
    rng = np.random.default_rng(9)
    nrows, batch, steps, lr, seed = 5000, 512, 3, 1e-3, 77
    rows = random_rows(rng, nrows).astype(np.float32)
    P = gpu_params(torch, 10)
    p0 = P.cpu().numpy().astype(np.float64)
    dR = torch.from_numpy(rows).cuda()
    L = torch.empty(steps, dtype=torch.float32, device="cuda")
    api.mlp_train(P.data_ptr(), dR.data_ptr(), nrows, steps, batch, lr, seed, L.data_ptr())
    batches = []
    for step in range(1, steps + 1):
        idx = [splitmix(seed ^ (step << 32) ^ b) % nrows for b in range(batch)]
        batches.append(rows[idx].astype(np.float64))
    pref, losses = M.adam_steps(p0, batches, lr)
    assert np.allclose(L.cpu().numpy(), losses, rtol=1e-4)
    _, g1 = M.loss_grad(p0, batches[0])
    live = np.abs(g1) > 1e-3 * np.abs(g1).max()  # sign-stable Adam updates
    diff = np.abs(P.cpu().numpy() - pref)
    assert diff[live].max() <= 0.05 * lr * steps


def test_training_reduces_loss(cuda):
    torch = cuda
    rng = np.random.default_rng(11)
    F = rng.standard_normal((20000, 6))
    rows = np.column_stack([F, 0.6 + 0.3 * np.tanh(F[:, 3]) - 0.2 * F[:, 4] ** 2 / (1 + F[:, 4] ** 2),
                            np.ones(20000)]).astype(np.float32)
    dR = torch.from_numpy(rows).cuda()
    P, L = learned.train(torch, dR, 20000, steps=1500, batch=2048, lr=2e-3)
    L = L.cpu().numpy()
    assert np.isfinite(L).all()
    assert L[-50:].mean() < 0.1 * L[:5].mean()


def test_collector_rows(cuda):
    torch = cuda
    csr = learned.device_csr(torch, 6, 3, 3, 1)
    rows = torch.empty((400_000, 8), dtype=torch.float32, device="cuda")
    got = learned.collect(torch, csr, 16, rows, 0)
    assert got > 0 and got % csr["n"] == 0
    R = rows[:got].cpu().numpy()
    assert np.isfinite(R).all()
    # f0 is a unit-RMS normalisation of each pair's plain correction; the
    # row weight is the square of the second-order term projected out of the
    # search space, in the units of f1 (the unprojected term), so per pair
    # the weights add up to at most the sum of f1^2
    per_pair = (R[:, 0] ** 2).reshape(-1, csr["n"]).mean(axis=1)
    assert np.allclose(per_pair, 1.0, rtol=2e-2)
    assert (R[:, 7] >= 0).all()
    wsum = R[:, 7].reshape(-1, csr["n"]).sum(axis=1)
    f1sum = (R[:, 1].astype(np.float64) ** 2).reshape(-1, csr["n"]).sum(axis=1)
    assert (wsum <= f1sum * (1 + 1e-4) + 1e-6).all()
    assert (wsum > 0).any()


@pytest.fixture(scope="module")
def trained(cuda):
    torch = cuda
    params, info = learned.build(torch, steps=2000)
    return params, info


def learned_vs_plain(torch, params, spec):
    csr = learned.device_csr(torch, *spec)
    _, wp, rp = learned.solve_csr(torch, csr, 16, strategy=1, davidson_maxsteps=100)
    _, wl, rl = learned.solve_csr(torch, csr, 16, strategy=1, davidson_maxsteps=100,
                                  preconditioner=1, mlp_params=params.data_ptr())
    assert rp["converged"] == 1 and rl["converged"] == 1
    assert rl["max_scaled_residual"] <= 1e-8
    assert (wl - wp).abs().max().item() <= 1e-10 * rp["matrix_norm_inf"]
    assert rl["mlp_steps_accepted"] > 0
    # each learned correction costs one more block-product column (its
    # second-order term), counted apart from the FP64 products
    assert rl["precond_matvecs"] > 0
    return rl, rp


def test_learned_correction_beats_plain_on_held_out(cuda, trained):
    """What the learned preconditioner gains on a held-out instance of the
    size it was trained at (8 orbitals, seed 9): its corrections are closer
    to the exact corrections (outside the search space) than the plain
    diagonal ones, about as close as the two-term series, and the learned
    Davidson solve reaches the same eigenpairs in fewer steps and block
    products than the plain one."""
    torch = cuda
    params, info = trained
    assert info["loss_last"] < info["loss_first"]
    assert info["selected"] in ("trained", "two_term")
    csr = learned.device_csr(torch, 8, 4, 4, 9)
    rows = torch.empty((1_500_000, 8), dtype=torch.float32, device="cuda")
    got = learned.collect(torch, csr, 16, rows, 0)
    plain, neumann, mlp = learned.correction_losses(torch, params, rows, got)
    assert mlp < 0.9 * plain and mlp < 1.05 * neumann, (plain, neumann, mlp)
    del rows
    rl, rp = learned_vs_plain(torch, params, (8, 4, 4, 9))
    assert rl["davidson_steps"] < rp["davidson_steps"], (rl, rp)
    assert rl["fp64_matvecs"] < rp["fp64_matvecs"], (rl, rp)


def test_learned_solve_at_an_untrained_size(cuda, trained):
    """At 10 orbitals (n = 63,504, a size the training never saw) the learned
    solve reaches the plain solve's eigenpairs in fewer Davidson steps."""
    rl, rp = learned_vs_plain(cuda, trained[0], (10, 5, 5, 4))
    assert rl["davidson_steps"] < rp["davidson_steps"], (rl, rp)


def test_saturated_network_is_the_plain_preconditioner(cuda, monkeypatch):
    """A network whose weight is 0 everywhere (o = sigmoid(-120)) gives the
    plain diagonal correction: with every step accepted
    (IPT_GB300_MLP_ACCEPT), the learned solve follows the plain solve step
    for step."""
    torch = cuda
    monkeypatch.setenv("IPT_GB300_MLP_ACCEPT", "1e30")
    P = torch.zeros(api.mlp_param_count(), dtype=torch.float32, device="cuda")
    P[-1] = -120.0
    csr = learned.device_csr(torch, 6, 3, 3, 2)
    _, wp, rp = learned.solve_csr(torch, csr, 16, strategy=1, davidson_maxsteps=100)
    _, wl, rl = learned.solve_csr(torch, csr, 16, strategy=1, davidson_maxsteps=100,
                                  preconditioner=1, mlp_params=P.data_ptr())
    assert rl["converged"] == 1
    assert rl["davidson_steps"] == rp["davidson_steps"]
    assert rl["fp64_matvecs"] == rp["fp64_matvecs"]
    assert (wl - wp).abs().max().item() <= 1e-10 * rp["matrix_norm_inf"]


def test_rejected_learned_steps_fall_back_to_plain(cuda, trained, monkeypatch):
    """With an acceptance bar no step can meet (IPT_GB300_MLP_ACCEPT), every
    learned step is rejected by the FP64 residual test, the learned
    correction is switched off after two rejections, and the plain
    correction finishes the solve with the same eigenpairs."""
    torch = cuda
    params, _ = trained
    monkeypatch.setenv("IPT_GB300_MLP_ACCEPT", "1e-30")
    csr = learned.device_csr(torch, 6, 3, 3, 2)
    _, wp, rp = learned.solve_csr(torch, csr, 16, strategy=1, davidson_maxsteps=100)
    _, wl, rl = learned.solve_csr(torch, csr, 16, strategy=1, davidson_maxsteps=100,
                                  preconditioner=1, mlp_params=params.data_ptr())
    assert rl["converged"] == 1
    assert rl["mlp_steps_rejected"] == 2 and rl["mlp_steps_accepted"] == 0
    assert (wl - wp).abs().max().item() <= 1e-10 * rp["matrix_norm_inf"]


def test_invalid_arguments(cuda):
    torch = cuda
    P = gpu_params(torch, 1)
    assert api._lib.load().ipt_block_mlp_train(None, None, 10, 1, 1, 1e-3, 0, None, None) == 1
    with pytest.raises(api.IPTError):
        api.mlp_train(P.data_ptr(), P.data_ptr(), 0, 1, 1, 1e-3)
    with pytest.raises(api.IPTError):
        api.mlp_forward(P.data_ptr(), P.data_ptr(), 5, 3, P.data_ptr())
