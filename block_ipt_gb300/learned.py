"""Training pipeline of the learned Davidson preconditioner (k_mlp.cu).

Everything runs on the GPU through the C ABI: the plain solver produces the
converged eigenvectors of small FCI-like instances, the collector records
(features, exact-correction target, weight) rows while the plain solver runs
(and, for a second round, while the learned one runs), and the library's
own forward/backward/Adam kernels train the network.  torch is used only to
hold device buffers.

The training family is the FCI-like construction of workloads.fci_like_csr
at 6 orbitals (3+3 electrons, n = 400) and 8 orbitals (4+4, n = 4900).
"""
import numpy as np

from . import api, workloads

ROW = 8  # floats per training row: 6 features, target weight of the second-order term, row weight
TRAIN_SPECS = ((6, 3, 3, 1), (6, 3, 3, 2), (6, 3, 3, 3), (8, 4, 4, 1), (8, 4, 4, 2))


def device_csr(torch, norb, nalpha, nbeta, seed, device="cuda"):
    """FCI-like CSR with an ascending diagonal, as device tensors."""
    rp, ci, v, d = workloads.fci_like_csr(norb, nalpha, nbeta, seed=seed)
    rp, ci, v, d, _ = workloads.sort_by_diagonal(rp, ci, v, d)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
    return {"row_ptr": t(rp), "col_ind": t(ci), "values": t(v), "n": len(rp) - 1, "nnz": len(ci)}


def solve_csr(torch, csr, k, **opts):
    """(X (k x n tensor, row j = vector j), values, report) of the block solver."""
    n = csr["n"]
    X = torch.empty((k, n), dtype=torch.float64, device=csr["values"].device)
    w = torch.empty(k, dtype=torch.float64, device=csr["values"].device)
    rep = api.block_solve_csr_device(csr["row_ptr"].data_ptr(), csr["col_ind"].data_ptr(),
                                     csr["values"].data_ptr(), n, csr["nnz"], k, X.data_ptr(),
                                     w.data_ptr(), "fp64", **opts)
    return X, w, rep


def collect(torch, csr, k, rows, offset, params=None, extra=8):
    """Append training rows for one instance at rows[offset:]; returns the
    number of rows written.  params = None follows the plain trajectory."""
    n = csr["n"]
    kstar = min(n, k + extra)
    Xs, _, rep = solve_csr(torch, csr, kstar, strategy=1, residual_tol=1e-12,
                           davidson_maxsteps=200)
    if rep["converged"] != 1:
        return 0
    opts = dict(strategy=1, residual_tol=1e-10, davidson_maxsteps=60)
    if params is not None:
        opts.update(preconditioner=1, mlp_params=params.data_ptr())
    got, _ = api.mlp_collect_csr(csr["row_ptr"].data_ptr(), csr["col_ind"].data_ptr(),
                                 csr["values"].data_ptr(), n, csr["nnz"], k, Xs.data_ptr(), kstar,
                                 rows[offset:].data_ptr(), rows.shape[0] - offset, **opts)
    return got


def train(torch, rows, count, steps=3000, batch=4096, lr=1e-3, seed=11, init_seed=7):
    """Fresh network trained on rows[:count]; returns (params, loss history)."""
    P = torch.empty(api.mlp_param_count(), dtype=torch.float32, device=rows.device)
    api.mlp_init(P.data_ptr(), init_seed)
    L = torch.empty(max(1, steps), dtype=torch.float32, device=rows.device)
    api.mlp_train(P.data_ptr(), rows.data_ptr(), count, steps, batch, lr, seed, L.data_ptr())
    return P, L


def correction_losses(torch, params, rows, count):
    """Weighted correction error, on rows[:count], of the plain preconditioner
    (weight 0 on the second-order term), of the two-term Neumann correction
    (weight 1) and of the network (its weight sigmoid(z), as the solver
    applies it)."""
    R = rows[:count]
    out = torch.empty(count, dtype=torch.float32, device=rows.device)
    api.mlp_forward(params.data_ptr(), R.data_ptr(), count, ROW, out.data_ptr())
    w, y = R[:, 7], R[:, 6]
    plain = torch.mean(w * y ** 2).item()
    neumann = torch.mean(w * (1.0 - y) ** 2).item()
    mlp = torch.mean(w * (out - y) ** 2).item()
    return plain, neumann, mlp


VALIDATION_SPECS = ((8, 4, 4, 5), (8, 4, 4, 6))


def davidson_steps(torch, csr, params, k=16):
    """Davidson steps of the learned solve of one instance (the library's
    FP64-accurate Davidson strategy, residual 1e-8)."""
    _, _, rep = solve_csr(torch, csr, min(k, csr["n"] // 4), strategy=1,
                          davidson_maxsteps=60, preconditioner=1, mlp_params=params.data_ptr())
    return rep["davidson_steps"] if rep["converged"] == 1 else 10 ** 6


def build(torch, k=16, specs=TRAIN_SPECS, dagger=True, capacity=8_000_000, steps=3000,
          device="cuda", validation=VALIDATION_SPECS):
    """Train the preconditioner on the FCI-like family; returns (params, info).

    Model selection: the trained network and the untrained one (the output
    bias alone, o = sigmoid(4) = 0.98 on every row: the two-term correction)
    each solve the validation instances (held out from training); the trained
    one is returned only if it takes fewer Davidson steps in total.  The
    per-row targets only approximate what a Davidson step needs, so a lower
    training loss does not guarantee fewer steps: on the FCI-like family the
    trained network matches the two-term correction at the training sizes
    and can take many more steps than it at 10 orbitals."""
    rows = torch.empty((capacity, ROW), dtype=torch.float32, device=device)
    total = 0
    csrs = [device_csr(torch, *spec, device=device) for spec in specs]
    for csr in csrs:
        total += collect(torch, csr, min(k, csr["n"] // 4), rows, total)
    first = total
    params, hist = train(torch, rows, total, steps=steps)
    if dagger:
        for csr in csrs:
            total += collect(torch, csr, min(k, csr["n"] // 4), rows, total, params=params)
        params, hist = train(torch, rows, total, steps=steps, seed=12)
    # batch losses are noisy: compare the first and last stretches of training
    info = {"rows_plain_trajectory": first, "rows_total": total,
            "loss_first": float(hist[:20].mean().item()),
            "loss_last": float(hist[-200:].mean().item())}
    if validation:
        base = torch.zeros_like(params)
        base[-1] = 4.0  # output bias only: the two-term correction's weight
        vcsr = [device_csr(torch, *spec, device=device) for spec in validation]
        trained_steps = sum(davidson_steps(torch, c, params, k) for c in vcsr)
        base_steps = sum(davidson_steps(torch, c, base, k) for c in vcsr)
        info["validation_steps"] = {"trained": trained_steps, "two_term": base_steps}
        info["selected"] = "trained" if trained_steps < base_steps else "two_term"
        if trained_steps >= base_steps:
            params = base
    return params, info
