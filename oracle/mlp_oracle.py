"""CPU restatement of the learned preconditioner's network (TEST INFRASTRUCTURE
ONLY: the checker of block_ipt_gb300/csrc/k_mlp.cu's forward, backward and Adam
kernels; the product never imports it).

The network has no counterpart in the reference, which uses the diagonal
Davidson correction (IPT_C_GPU/src/ipt_cuda.cu:2449-2465).  Parameter layout
(FP32 vector of 4673): W1[64][6], b1[64], W2[64][64], b2[64], W3[64], b3.
Rows are [6 features | target | weight]; the network's weight of the
second-order term is o = sigmoid(z), z its linear output;
loss = mean of weight * (o - target)^2.
Everything here is float64; finite differences pin the backward pass.
"""
import numpy as np

N_IN = 6
N_H = 64
SIZES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)),
         ("W3", (N_H,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        size = int(np.prod(shape))
        out[name] = p[o:o + size].reshape(shape)
        o += size
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in SIZES])


def forward(p, F):
    w = unpack(p)
    F = np.asarray(F, np.float64)
    z1 = F @ w["W1"].T + w["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(z2, 0.0)
    z = h2 @ w["W3"] + w["b3"][0]
    return 1.0 / (1.0 + np.exp(-z)), (F, z1, h1, z2, h2)


def loss_grad(p, rows):
    """(loss, grad) of the weighted squared error over rows [features | target | weight]."""
    rows = np.asarray(rows, np.float64)
    F, y, wt = rows[:, :N_IN], rows[:, N_IN], rows[:, N_IN + 1]
    w = unpack(p)
    o, (F, z1, h1, z2, h2) = forward(p, F)
    B = len(y)
    err = o - y
    loss = float(np.mean(wt * err ** 2))
    # through o = sigmoid(z): do/dz = o (1 - o)
    dO = 2.0 * wt * err * o * (1.0 - o) / B
    g = {}
    g["W3"] = dO @ h2
    g["b3"] = np.array([dO.sum()])
    d2 = np.outer(dO, w["W3"]) * (z2 > 0)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(axis=0)
    d1 = (d2 @ w["W2"]) * (z1 > 0)
    g["W1"] = d1.T @ F
    g["b1"] = d1.sum(axis=0)
    return loss, pack(g)


def adam_steps(p, rows_list, lr, b1=0.9, b2=0.999, eps=1e-8):
    """Adam (Kingma & Ba 2015) over a list of batches, float64."""
    p = np.array(p, np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    losses = []
    for t, rows in enumerate(rows_list, start=1):
        loss, g = loss_grad(p, rows)
        losses.append(loss)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p = p - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, losses
