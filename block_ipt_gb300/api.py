"""Python mirror of the reference solver interface, on top of the C ABI.

Function names, argument meaning and error behaviour follow the reference's
`ipt_cuda*` entry points (IPT_C_GPU/src/ipt_cuda.cu:262-308): a non-zero
status raises IPTError carrying the status code.  Dense matrices are taken
as 2-D numpy arrays (copied to column-major doubles); sparse input is CSC.
Every call goes through libipt_gb300.so; nothing here computes on the CPU.
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import IPTBlockOptions, IPTBlockReport, IPTCudaResult, IPTError


def _f64(a):
    return np.asfortranarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _take_result(res, status, what):
    lib = _lib.load()
    if status != _lib.IPT_CUDA_SUCCESS:
        lib.ipt_cuda_free_result(C.byref(res))
        raise IPTError(status, what)
    n, k = res.n, res.k
    vec = np.ctypeslib.as_array(res.vectors, shape=(n * k,)).reshape((n, k), order="F").copy()
    val = np.ctypeslib.as_array(res.values, shape=(k,)).copy()
    info = {
        "iterations": res.iterations,
        "basis_cols": res.basis_cols,
        "matvecs": res.matvecs,
        "fixed_point_residual": res.fixed_point_residual,
        "solve_time_sec": res.solve_time_sec,
        "iteration_time_sec": res.iteration_time_sec,
        "rayleigh_ritz_time_sec": res.rayleigh_ritz_time_sec,
        "davidson_time_sec": res.davidson_time_sec,
        "davidson_residual_after": res.davidson_residual_after,
        "adaptive_added_indices": res.adaptive_added_indices.decode(),
        "adaptive_target_block": (res.adaptive_target_block_start, res.adaptive_target_block_end),
        "rayleigh_ritz_used_qr": res.rayleigh_ritz_used_qr,
        "basis_orthogonality": (res.basis_orthogonality_frobenius_error,
                                res.basis_orthogonality_max_abs_error, res.basis_has_nan_or_inf),
        "ritz_vectors_orthogonality": (res.ritz_vectors_orthogonality_frobenius_error,
                                       res.ritz_vectors_orthogonality_max_abs_error,
                                       res.ritz_vectors_has_nan_or_inf),
    }
    lib.ipt_cuda_free_result(C.byref(res))
    return vec, val, info


# ---- dense, host buffers --------------------------------------------------
def ipt_cuda(matrix, k, iterations, initial_vectors=None):
    """Fixed-iteration plain IPT (ipt_cuda / ipt_cuda_with_initial)."""
    H = _f64(matrix)
    n = H.shape[0]
    X0 = None if initial_vectors is None else _f64(initial_vectors)
    res = IPTCudaResult()
    lib = _lib.load()
    if X0 is None:
        st = lib.ipt_cuda(_ptr(H), n, k, iterations, C.byref(res))
    else:
        st = lib.ipt_cuda_with_initial(_ptr(H), _ptr(X0), n, k, iterations, C.byref(res))
    return _take_result(res, st, "ipt_cuda")


def ipt_cuda_tol(matrix, k, tol, maxiter, initial_vectors=None):
    """Tolerance-stopped plain IPT (ipt_cuda_tol / ipt_cuda_with_initial_tol)."""
    H = _f64(matrix)
    n = H.shape[0]
    X0 = None if initial_vectors is None else _f64(initial_vectors)
    res = IPTCudaResult()
    lib = _lib.load()
    if X0 is None:
        st = lib.ipt_cuda_tol(_ptr(H), n, k, tol, maxiter, C.byref(res))
    else:
        st = lib.ipt_cuda_with_initial_tol(_ptr(H), _ptr(X0), n, k, tol, maxiter, C.byref(res))
    return _take_result(res, st, "ipt_cuda_tol")


# ---- sparse CSC, host buffers ------------------------------------------------
def ipt_cuda_sparse_csc(col_ptr, row_ind, values, n, k, iterations, initial_vectors=None):
    cp, ri, va = _i32(col_ptr), _i32(row_ind), np.ascontiguousarray(values, dtype=np.float64)
    res = IPTCudaResult()
    lib = _lib.load()
    if initial_vectors is None:
        st = lib.ipt_cuda_sparse_csc(_ptr(cp), _ptr(ri), _ptr(va), n, k, len(ri), iterations,
                                     C.byref(res))
    else:
        X0 = _f64(initial_vectors)
        st = lib.ipt_cuda_sparse_csc_with_initial(_ptr(cp), _ptr(ri), _ptr(va), _ptr(X0), n, k,
                                                  len(ri), iterations, C.byref(res))
    return _take_result(res, st, "ipt_cuda_sparse_csc")


def ipt_cuda_sparse_csc_tol(col_ptr, row_ind, values, n, k, tol, maxiter, initial_vectors=None):
    cp, ri, va = _i32(col_ptr), _i32(row_ind), np.ascontiguousarray(values, dtype=np.float64)
    res = IPTCudaResult()
    lib = _lib.load()
    if initial_vectors is None:
        st = lib.ipt_cuda_sparse_csc_tol(_ptr(cp), _ptr(ri), _ptr(va), n, k, len(ri), tol,
                                         maxiter, C.byref(res))
    else:
        X0 = _f64(initial_vectors)
        st = lib.ipt_cuda_sparse_csc_with_initial_tol(_ptr(cp), _ptr(ri), _ptr(va), _ptr(X0), n,
                                                      k, len(ri), tol, maxiter, C.byref(res))
    return _take_result(res, st, "ipt_cuda_sparse_csc_tol")


# ---- block solver (include/ipt_block.h) ----------------------------------------
PRECISIONS = {"fp64": _lib.IPT_BLOCK_FP64, "fp16": _lib.IPT_BLOCK_FP16,
              "bf16": _lib.IPT_BLOCK_BF16, "tf32": _lib.IPT_BLOCK_TF32}


def block_options(precision="fp64", stream=None, **kw):
    opt = IPTBlockOptions()
    _lib.load().ipt_block_default_options(C.byref(opt))
    opt.ipt_precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    if stream is not None:
        opt.stream = C.c_void_p(int(stream))
    for key, val in kw.items():
        if not hasattr(opt, key):
            raise TypeError("unknown block option %r" % key)
        if key == "mlp_params":
            val = C.c_void_p(int(val)) if val is not None else None
        setattr(opt, key, val)
    return opt


def block_solve_dense(matrix, k, precision="fp64", **kw):
    """k lowest eigenpairs of a dense symmetric matrix held in host memory."""
    H = _f64(matrix)
    n = H.shape[0]
    opt = block_options(precision, **kw)
    vec = np.zeros((n, k), dtype=np.float64, order="F")
    val = np.zeros(k, dtype=np.float64)
    rep = IPTBlockReport()
    st = _lib.load().ipt_block_solve_dense(_ptr(H), n, k, C.byref(opt), _ptr(vec), _ptr(val),
                                           C.byref(rep))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_block_solve_dense")
    return vec, val, rep.as_dict()


def block_solve_dense_device(d_matrix_ptr, n, k, d_vectors_ptr, d_values_ptr, precision="fp64",
                             **kw):
    """Device-pointer variant; pointers are integers (e.g. torch data_ptr())."""
    opt = block_options(precision, **kw)
    rep = IPTBlockReport()
    st = _lib.load().ipt_block_solve_dense_device(C.c_void_p(d_matrix_ptr), n, k, C.byref(opt),
                                                  C.c_void_p(d_vectors_ptr),
                                                  C.c_void_p(d_values_ptr), C.byref(rep))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_block_solve_dense_device")
    return rep.as_dict()


def block_solve_csr(row_ptr, col_ind, values, n, k, precision="fp64", **kw):
    """k lowest eigenpairs of a symmetric CSR matrix held in host memory."""
    rp, ci = _i32(row_ptr), _i32(col_ind)
    va = np.ascontiguousarray(values, dtype=np.float64)
    opt = block_options(precision, **kw)
    vec = np.zeros((n, k), dtype=np.float64, order="F")
    val = np.zeros(k, dtype=np.float64)
    rep = IPTBlockReport()
    st = _lib.load().ipt_block_solve_csr(_ptr(rp), _ptr(ci), _ptr(va), n, len(ci), k,
                                         C.byref(opt), _ptr(vec), _ptr(val), C.byref(rep))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_block_solve_csr")
    return vec, val, rep.as_dict()


def block_solve_csr_device(d_row_ptr, d_col_ind, d_vals, n, nnz, k, d_vectors_ptr, d_values_ptr,
                           precision="fp64", **kw):
    """Device-pointer CSR variant (diagonal need not be sorted)."""
    opt = block_options(precision, **kw)
    rep = IPTBlockReport()
    st = _lib.load().ipt_block_solve_csr_device(C.c_void_p(d_row_ptr), C.c_void_p(d_col_ind),
                                                C.c_void_p(d_vals), n, nnz, k, C.byref(opt),
                                                C.c_void_p(d_vectors_ptr),
                                                C.c_void_p(d_values_ptr), C.byref(rep))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_block_solve_csr_device")
    return rep.as_dict()


# ---------------------------------------------------------------------------
# learned preconditioner
# ---------------------------------------------------------------------------
def _check(status, what="ipt_block_mlp"):
    if status != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(status, what)


def _stream_ptr(stream):
    return C.c_void_p(stream) if stream else None


def mlp_param_count():
    return _lib.load().ipt_block_mlp_param_count()


def mlp_init(d_params_ptr, seed=0, stream=None):
    st = _lib.load().ipt_block_mlp_init(C.c_void_p(d_params_ptr), seed, _stream_ptr(stream))
    _check(st)


def mlp_loss_grad(d_params_ptr, d_rows_ptr, rows, d_grad_ptr, stream=None):
    st = _lib.load().ipt_block_mlp_loss_grad(C.c_void_p(d_params_ptr), C.c_void_p(d_rows_ptr),
                                             rows, C.c_void_p(d_grad_ptr), _stream_ptr(stream))
    _check(st)


def mlp_forward(d_params_ptr, d_rows_ptr, rows, row_stride, d_out_ptr, stream=None):
    st = _lib.load().ipt_block_mlp_forward(C.c_void_p(d_params_ptr), C.c_void_p(d_rows_ptr), rows,
                                           row_stride, C.c_void_p(d_out_ptr), _stream_ptr(stream))
    _check(st)


def mlp_train(d_params_ptr, d_rows_ptr, rows, steps, batch, lr, seed=0, d_loss_ptr=None,
              stream=None):
    st = _lib.load().ipt_block_mlp_train(C.c_void_p(d_params_ptr), C.c_void_p(d_rows_ptr), rows,
                                         steps, batch, lr, seed,
                                         C.c_void_p(d_loss_ptr) if d_loss_ptr else None,
                                         _stream_ptr(stream))
    _check(st)


def mlp_collect_csr(d_row_ptr, d_col_ind, d_vals, n, nnz, k, d_exact_ptr, exact_cols,
                    d_rows_ptr, capacity, **opts):
    """Run the diagonal-preconditioned Davidson solver on device CSR arrays and
    record (features, exact-correction target) rows; returns (rows, report)."""
    lib = _lib.load()
    opts.setdefault("strategy", 1)
    opt = block_options("fp64", **opts)
    rep = _lib.IPTBlockReport()
    written = C.c_longlong(0)
    st = lib.ipt_block_mlp_collect_csr(C.c_void_p(d_row_ptr), C.c_void_p(d_col_ind),
                                       C.c_void_p(d_vals), n, nnz, k, C.byref(opt),
                                       C.c_void_p(d_exact_ptr), exact_cols, C.c_void_p(d_rows_ptr),
                                       capacity, C.byref(written), C.byref(rep))
    _check(st)
    return written.value, rep.as_dict()


# ---------------------------------------------------------------------------
# batched dense solver
# ---------------------------------------------------------------------------
class BatchPlan:
    """Many independent dense instances solved by one persistent kernel under a
    captured CUDA graph (include/ipt_block.h, ipt_block_batch_*).

    instances: sequence of (d_H, n, k, d_vectors, d_values) device pointers
    (integers); they must stay valid while the plan lives."""

    def __init__(self, instances, precision="fp64", **opts):
        lib = _lib.load()
        self._lib = lib
        self.count = len(instances)
        arr = (_lib.IPTBatchInstance * self.count)()
        for b, (h, n, k, vec, val) in enumerate(instances):
            arr[b] = _lib.IPTBatchInstance(C.c_void_p(h), n, k, C.c_void_p(vec), C.c_void_p(val))
        opt = _lib.IPTBatchOptions()
        lib.ipt_block_batch_default_options(C.byref(opt))
        opt.precision = _lib.IPT_BLOCK_FP32 if precision == "fp32" else _lib.IPT_BLOCK_FP64
        for key, val in opts.items():
            if not hasattr(opt, key):
                raise TypeError("unknown batch option %r" % key)
            setattr(opt, key, val)
        self._plan = C.c_void_p()
        _check(lib.ipt_block_batch_plan_create(arr, self.count, C.byref(opt),
                                               C.byref(self._plan)), "ipt_block_batch_plan_create")

    def run(self, stream=None):
        _check(self._lib.ipt_block_batch_plan_run(self._plan, _stream_ptr(stream)),
               "ipt_block_batch_plan_run")

    def autotune(self, stream=None):
        t, c, ms = C.c_int(0), C.c_int(0), C.c_double(0.0)
        _check(self._lib.ipt_block_batch_plan_autotune(self._plan, _stream_ptr(stream), C.byref(t),
                                                       C.byref(c), C.byref(ms)),
               "ipt_block_batch_plan_autotune")
        return t.value, c.value, ms.value

    def reports(self):
        arr = (_lib.IPTBatchReport * self.count)()
        _check(self._lib.ipt_block_batch_plan_reports(self._plan, arr),
               "ipt_block_batch_plan_reports")
        return [{f: getattr(r, f) for f, _ in _lib.IPTBatchReport._fields_} for r in arr]

    def shape(self):
        v = [C.c_int(0) for _ in range(5)]
        _check(self._lib.ipt_block_batch_plan_shape(self._plan, *[C.byref(x) for x in v]),
               "ipt_block_batch_plan_shape")
        return dict(zip(("threads", "chunk", "cluster", "ctas", "team_instances"),
                        (x.value for x in v)))

    def close(self):
        if self._plan:
            self._lib.ipt_block_batch_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# matrix-free FCI-like Hamiltonians
# ---------------------------------------------------------------------------
PRECISION_CODES = {"fp64": _lib.IPT_BLOCK_FP64, "fp32": _lib.IPT_BLOCK_FP32,
                   "bf16": _lib.IPT_BLOCK_BF16}


def fci_spec(norb, nalpha, nbeta, seed=0, sigma=0.05):
    return _lib.IPTFciSpec(norb, nalpha, nbeta, seed, sigma)


def fci_dimension(spec):
    n = C.c_longlong(0)
    _check(_lib.load().ipt_fci_dimension(C.byref(spec), C.byref(n)), "ipt_fci_dimension")
    return n.value


def fci_diagonal(spec, d_diag_ptr, stream=None):
    _check(_lib.load().ipt_fci_diagonal(C.byref(spec), C.c_void_p(d_diag_ptr),
                                        _stream_ptr(stream)), "ipt_fci_diagonal")


def fci_sigma(spec, d_x_ptr, k, d_y_ptr, precision="fp64", stream=None):
    _check(_lib.load().ipt_fci_sigma(C.byref(spec), C.c_void_p(d_x_ptr), k, C.c_void_p(d_y_ptr),
                                     PRECISION_CODES[precision], _stream_ptr(stream)),
           "ipt_fci_sigma")


def block_solve_fci(spec, k, d_vectors_ptr, d_values_ptr, precision="fp64", **kw):
    """k lowest eigenpairs of the matrix-free FCI-like H by Davidson; precision
    "bf16"/"fp32" runs a low-precision sigma phase before the FP64 one."""
    opt = block_options("fp64", **kw)
    opt.ipt_precision = PRECISION_CODES[precision]
    rep = IPTBlockReport()
    st = _lib.load().ipt_block_solve_fci(C.byref(spec), k, C.byref(opt), C.c_void_p(d_vectors_ptr),
                                         C.c_void_p(d_values_ptr), C.byref(rep))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_block_solve_fci")
    return rep.as_dict()


def trace_enable(on=True):
    """Start (clearing earlier marks) or stop the solvers' phase marks."""
    _check(_lib.load().ipt_block_trace_enable(1 if on else 0), "ipt_block_trace_enable")


def trace_read():
    """[(label, host_ns, gpu_ns)] of the marks recorded since trace_enable()."""
    lib = _lib.load()
    m = lib.ipt_block_trace_count()
    labels = (C.c_char_p * max(1, m))()
    host = (C.c_longlong * max(1, m))()
    gpu = (C.c_longlong * max(1, m))()
    _check(lib.ipt_block_trace_read(m, labels, host, gpu), "ipt_block_trace_read")
    return [(labels[i].decode(), host[i], gpu[i]) for i in range(m)]


# ---- block-cluster path (include/ipt_block.h) ------------------------------------
def cluster_ranges(col_ptr, row_ind, values, n, k, requested_k=None, threshold=0.0,
                   adaptive=False, coupling_tau=0.1):
    """Cluster ranges of a symmetric CSC matrix with ascending diagonal
    (ipt_block_cluster_ranges): ([(first, last), ...], limit_hit)."""
    cp, ri, va = _i32(col_ptr), _i32(row_ind), _f64(values)
    lib = _lib.load()
    cap = max(1, n)
    out = np.zeros(2 * cap, dtype=np.int32)
    cnt, lim = C.c_int(0), C.c_int(0)
    st = lib.ipt_block_cluster_ranges(_ptr(cp), _ptr(ri), _ptr(va), n, len(ri), k,
                                      k if requested_k is None else requested_k, threshold,
                                      int(bool(adaptive)), coupling_tau, _ptr(out), cap,
                                      C.byref(cnt), C.byref(lim))
    _check(st, "ipt_block_cluster_ranges")
    return [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(cnt.value)], bool(lim.value)


def cluster_ranges_device(d_row_ptr, d_col_ind, d_vals, n, nnz, k, requested_k=None,
                          threshold=0.0, adaptive=False, coupling_tau=0.1, stream=None):
    """Cluster ranges of a prepared symmetric device CSR
    (ipt_block_cluster_ranges_device): ([(first, last), ...], limit_hit)."""
    lib = _lib.load()
    cap = max(1, n)
    out = np.zeros(2 * cap, dtype=np.int32)
    cnt, lim = C.c_int(0), C.c_int(0)
    st = lib.ipt_block_cluster_ranges_device(d_row_ptr, d_col_ind, d_vals, n, nnz, k,
                                             k if requested_k is None else requested_k,
                                             threshold, int(bool(adaptive)), coupling_tau,
                                             _ptr(out), cap, C.byref(cnt), C.byref(lim),
                                             _stream_ptr(stream))
    _check(st, "ipt_block_cluster_ranges_device")
    return [(int(out[2 * i]), int(out[2 * i + 1])) for i in range(cnt.value)], bool(lim.value)


def cluster_basis(d_row_ptr, d_col_ind, d_vals, n, nnz, d_diag, ranges, maxiter, tol,
                  d_basis, damping=1.0, stream=None):
    """Block-cluster basis on the device (ipt_block_cluster_basis); returns
    (iterations, residuals) per cluster."""
    rg = np.ascontiguousarray(np.asarray(ranges, dtype=np.int32).reshape(-1))
    nc = rg.size // 2
    it = np.zeros(nc, dtype=np.int32)
    res = np.zeros(nc, dtype=np.float64)
    st = _lib.load().ipt_block_cluster_basis(d_row_ptr, d_col_ind, d_vals, n, nnz, d_diag,
                                             _ptr(rg), nc, maxiter, tol, damping, d_basis,
                                             _ptr(it), _ptr(res), _stream_ptr(stream))
    _check(st, "ipt_block_cluster_basis")
    return it, res


def cluster_update(d_basis, d_y, d_diag, n, first, m, d_next, damping=1.0, stream=None):
    """One block-cluster update of cluster [first, first+m) on the device
    (ipt_block_cluster_update); returns the singular flag."""
    sing = C.c_int(0)
    st = _lib.load().ipt_block_cluster_update(d_basis, d_y, d_diag, n, first, m, damping,
                                              d_next, C.byref(sing), _stream_ptr(stream))
    _check(st, "ipt_block_cluster_update")
    return bool(sing.value)


def prepare_csc(col_ptr, row_ind, values, n, k, lift=True, threshold=0.0):
    """The plain sparse path's host preparation (ipt_block_prepare_csc): a dict
    of the prepared CSC, diagonal, permutation and lifting rotations."""
    cp, ri, va = _i32(col_ptr), _i32(row_ind), _f64(values)
    lib = _lib.load()
    cap = max(4 * len(ri), n * n, 16)
    ocp = np.zeros(n + 1, np.int32)
    ori = np.zeros(cap, np.int32)
    ova = np.zeros(cap)
    od = np.zeros(n)
    op = np.zeros(n, np.int32)
    rf = np.zeros(n, np.int32)
    rs = np.zeros(n, np.int32)
    rv = np.zeros(max(1, 64 * 64 * n))
    nnz, rc = C.c_int(0), C.c_int(0)
    st = lib.ipt_block_prepare_csc(_ptr(cp), _ptr(ri), _ptr(va), n, k, len(ri), int(bool(lift)),
                                   threshold, _ptr(ocp), _ptr(ori), _ptr(ova), cap, C.byref(nnz),
                                   _ptr(od), _ptr(op), _ptr(rf), _ptr(rs), n, _ptr(rv), rv.size,
                                   C.byref(rc))
    _check(st, "ipt_block_prepare_csc")
    r = rc.value
    return {"col_ptr": ocp, "row_ind": ori[:nnz.value], "values": ova[:nnz.value], "diag": od,
            "perm": op, "rot_first": rf[:r], "rot_size": rs[:r],
            "rot_values": rv[:int(sum(int(m) * int(m) for m in rs[:r]))]}


# ---- the reference's binary CSC matrix cache (include/ipt_block.h) -------------
_CACHE_FIELDS = ("norb", "nelec", "neleca", "nelecb", "na", "nb")


def read_csc_cache(path):
    """A cache file of the reference's molecule benchmarks: (col_ptr, row_ind,
    values, diagonal, info dict)."""
    lib = _lib.load()
    info = _lib.IPTCscCacheInfo()
    p = os.fsencode(path)
    _check(lib.ipt_block_csc_cache_info(p, C.byref(info)), "ipt_block_csc_cache_info")
    n, nnz = info.n, info.nnz
    cp = np.zeros(n + 1, np.int32)
    ri = np.zeros(max(1, nnz), np.int32)
    va = np.zeros(max(1, nnz))
    dg = np.zeros(n)
    _check(lib.ipt_block_csc_cache_read(p, _ptr(cp), _ptr(ri), _ptr(va), _ptr(dg), n, nnz,
                                        C.byref(info)), "ipt_block_csc_cache_read")
    meta = {"magic": info.magic.decode(), "version": info.version, "n": n, "nnz": nnz,
            "matrix_inf_norm": info.matrix_inf_norm}
    meta.update({f: getattr(info, f) for f in _CACHE_FIELDS})
    return cp, ri[:nnz], va[:nnz], dg, meta


def write_csc_cache(path, col_ptr, row_ind, values, diagonal, magic="IPTGENC1",
                    matrix_inf_norm=None, **counts):
    """Write a cache file in the reference's layout (counts: norb, nelec,
    neleca, nelecb, na, nb; the norm defaults to max row sum of |H|)."""
    cp, ri, va, dg = _i32(col_ptr), _i32(row_ind), _f64(values), _f64(diagonal)
    n = len(cp) - 1
    if matrix_inf_norm is None:
        rows = np.zeros(n)
        np.add.at(rows, ri, np.abs(va))
        matrix_inf_norm = float(rows.max()) if n else 0.0
    info = _lib.IPTCscCacheInfo()
    info.magic = magic.encode()[:8]
    info.version = 1
    info.n, info.nnz = n, len(ri)
    info.matrix_inf_norm = matrix_inf_norm
    for f in _CACHE_FIELDS:
        setattr(info, f, int(counts.get(f, 0)))
    _check(_lib.load().ipt_block_csc_cache_write(os.fsencode(path), C.byref(info), _ptr(cp),
                                                 _ptr(ri), _ptr(va), _ptr(dg)),
           "ipt_block_csc_cache_write")


# ---- Rayleigh-mixed (device buffers) ---------------------------------------
def householder_signs(top, n):
    """Column signs of a LAPACK Householder QR from the top k x k block of
    an orthonormal CholQR factor (ipt_block_householder_signs)."""
    T = _f64(top)
    k = T.shape[0]
    out = np.zeros(k)
    st = _lib.load().ipt_block_householder_signs(_ptr(T), k, n, _ptr(out))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_block_householder_signs")
    return out


def rayleigh_mixed_tf32_device(d_matrix_ptr, n, k, tf32_tol, tf32_maxiter, fp64_tol,
                               fp64_maxiter, handle):
    """ipt_rayleigh_mixed_tf32_cuda_device_tol on a device matrix; returns the
    result struct (device vectors/values owned by the caller, released by
    free_rayleigh_result)."""
    res = _lib.IPTRayleighMixedCudaDeviceResult()
    st = _lib.load().ipt_rayleigh_mixed_tf32_cuda_device_tol(
        C.c_void_p(d_matrix_ptr), n, k, float(tf32_tol), int(tf32_maxiter), float(fp64_tol),
        int(fp64_maxiter), C.c_void_p(handle), C.byref(res))
    if st != _lib.IPT_CUDA_SUCCESS:
        raise IPTError(st, "ipt_rayleigh_mixed_tf32_cuda_device_tol")
    return res


def free_rayleigh_result(res):
    _lib.load().ipt_rayleigh_mixed_cuda_free_device_result(C.byref(res))

