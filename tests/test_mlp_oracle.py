"""The CPU oracle of the learned preconditioner's network: its backward pass
against central finite differences, and its Adam loop on a toy problem."""
import numpy as np

from oracle import mlp_oracle as M


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(M.N_PARAMS) * 0.3
    rows = np.column_stack([rng.standard_normal((60, 6)), rng.standard_normal(60),
                            rng.uniform(0.1, 2.0, 60)])
    _, g = M.loss_grad(p, rows)
    idx = rng.choice(M.N_PARAMS, 60, replace=False)
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = M.loss_grad(q, rows)
        q[i] -= 2 * eps
        lm, _ = M.loss_grad(q, rows)
        assert abs((lp - lm) / (2 * eps) - g[i]) <= 1e-7 * max(1.0, abs(g[i]))


def test_adam_reduces_loss():
    rng = np.random.default_rng(1)
    F = rng.standard_normal((512, 6))
    y = 0.5 + 0.3 * np.tanh(F[:, 3])
    rows = np.column_stack([F, y, np.ones(512)])
    p = rng.standard_normal(M.N_PARAMS) * 0.1
    _, losses = M.adam_steps(p, [rows] * 200, lr=3e-3)
    assert losses[-1] < 0.1 * losses[0]


def test_layout():
    assert M.N_PARAMS == 4673
    d = M.unpack(np.arange(M.N_PARAMS, dtype=np.float64))
    assert d["W1"].shape == (64, 6) and d["W2"].shape == (64, 64) and d["W3"].shape == (64,)
    assert d["b3"][0] == M.N_PARAMS - 1
