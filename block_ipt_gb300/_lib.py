"""ctypes binding of libipt_gb300.so (the C ABI in include/ipt_cuda.h and
include/ipt_block.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared object has not been built.
"""
import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libipt_gb300.so")

# status codes (include/ipt_cuda.h)
IPT_CUDA_SUCCESS = 0
IPT_CUDA_INVALID_ARGUMENT = 1
IPT_CUDA_ALLOCATION_FAILED = 2
IPT_CUDA_CUDA_ERROR = 3
IPT_CUDA_CUBLAS_ERROR = 4
IPT_CUDA_CUSPARSE_ERROR = 5
IPT_CUDA_CUSOLVER_ERROR = 6

IPT_BLOCK_FP64 = 0
IPT_BLOCK_FP16 = 1
IPT_BLOCK_BF16 = 2
IPT_BLOCK_TF32 = 3
IPT_BLOCK_FP32 = 4
IPT_BLOCK_DF64 = 5
IPT_BLOCK_STRATEGY_REFINE = 0
IPT_BLOCK_STRATEGY_DAVIDSON = 1
IPT_BLOCK_PRECOND_DIAGONAL = 0
IPT_BLOCK_PRECOND_MLP = 1

_d = C.c_double
_i = C.c_int
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class IPTDavidsonHistoryEntry(C.Structure):
    _fields_ = [
        ("davidson_step", _i), ("active_pair_index", _i), ("residual_before", _d),
        ("residual_after", _d), ("accepted", _i), ("basis_cols", _i),
        ("max_relative_eigen_residual", _d), ("max_relative_eigen_residual_index", _i),
        ("pair_28_residual", _d), ("pair_29_residual", _d),
        ("orthogonality_max_abs_error", _d), ("restarted", _i), ("best_so_far_updated", _i),
        ("best_so_far_step", _i), ("best_so_far_max_residual", _d),
        ("pair28_best_residual", _d), ("pair29_best_residual", _d), ("accept_global_ok", _i),
        ("accept_active_ok", _i), ("accept_locked_safe", _i), ("accept_reason", C.c_char * 64),
        ("accepted_steps", _i), ("rejected_steps", _i), ("early_jump_to_continuation", _i),
        ("gap28_29", _d), ("relative_gap28_29", _d), ("cluster_residual_fro_before", _d),
        ("cluster_residual_fro_after", _d), ("cluster_residual_max_before", _d),
        ("cluster_residual_max_after", _d), ("ritz_overlap_28_28", _d),
        ("ritz_overlap_28_29", _d), ("ritz_overlap_29_28", _d), ("ritz_overlap_29_29", _d),
        ("ritz_overlap_swap_detected", _i), ("pair28_lock_state", C.c_char * 16),
        ("pair29_lock_state", C.c_char * 16), ("cluster_hard_locked", _i),
        ("cluster_soft_locked_count", _i),
    ]


class IPTDavidsonSelectionEntry(C.Structure):
    _fields_ = [
        ("davidson_step", _i), ("pair_index", _i), ("residual", _d),
        ("selected_by_residual", _i), ("selected_forced", _i), ("selected_auto_cluster", _i),
        ("skipped_converged_in_cluster", _i), ("skipped_linear_dependent", _i),
        ("skipped_locked_old_logic_should_not_happen", _i),
        ("correction_norm_before_ortho", _d), ("correction_norm_after_ortho", _d),
    ]


class IPTDavidsonBlockHistoryEntry(C.Structure):
    _fields_ = [
        ("davidson_step", _i), ("active_pairs", C.c_char * 64), ("accepted_corrections", _i),
        ("rejected_corrections", _i), ("correction_norm_before_ortho", C.c_char * 256),
        ("correction_norm_after_ortho", C.c_char * 256), ("residual_before_global", _d),
        ("residual_after_global", _d), ("pair_28_before", _d), ("pair_28_after", _d),
        ("pair_29_before", _d), ("pair_29_after", _d), ("accepted", _i),
        ("reject_reason", C.c_char * 64), ("basis_cols_before", _i), ("basis_cols_after", _i),
        ("orthogonality_error_before", _d), ("orthogonality_error_after", _d),
        ("best_so_far_updated", _i), ("best_so_far_step", _i), ("best_so_far_max_residual", _d),
        ("pair28_best_residual", _d), ("pair29_best_residual", _d), ("accept_global_ok", _i),
        ("accept_active_ok", _i), ("accept_locked_safe", _i), ("accept_reason", C.c_char * 64),
        ("accepted_steps", _i), ("rejected_steps", _i), ("early_jump_to_continuation", _i),
        ("gap28_29", _d), ("relative_gap28_29", _d), ("cluster_residual_fro_before", _d),
        ("cluster_residual_fro_after", _d), ("cluster_residual_max_before", _d),
        ("cluster_residual_max_after", _d), ("ritz_overlap_28_28", _d),
        ("ritz_overlap_28_29", _d), ("ritz_overlap_29_28", _d), ("ritz_overlap_29_29", _d),
        ("ritz_overlap_swap_detected", _i), ("pair28_lock_state", C.c_char * 16),
        ("pair29_lock_state", C.c_char * 16), ("cluster_hard_locked", _i),
        ("cluster_soft_locked_count", _i),
    ]


class IPTCudaResult(C.Structure):
    _fields_ = [
        ("n", _i), ("k", _i), ("iterations", _i), ("vectors", _dp), ("values", _dp),
        ("basis_cols", _i), ("matvecs", C.c_longlong), ("preparation_time_sec", _d),
        ("transfer_setup_time_sec", _d), ("iteration_time_sec", _d),
        ("rayleigh_ritz_time_sec", _d), ("davidson_time_sec", _d), ("solve_time_sec", _d),
        ("fixed_point_residual", _d), ("oversample", _i), ("rayleigh_ritz_used_qr", _i),
        ("basis_orthogonality_frobenius_error", _d), ("basis_orthogonality_max_abs_error", _d),
        ("ritz_vectors_orthogonality_frobenius_error", _d),
        ("ritz_vectors_orthogonality_max_abs_error", _d), ("basis_has_nan_or_inf", _i),
        ("ritz_vectors_has_nan_or_inf", _i), ("davidson_attempted", _i),
        ("davidson_accepted", _i), ("davidson_target_index", _i),
        ("davidson_residual_before", _d), ("davidson_residual_after", _d),
        ("davidson_denom_clip", _d), ("adaptive_block_enabled", _i),
        ("adaptive_coupling_tau", _d), ("adaptive_limit_hit", _i),
        ("adaptive_target_block_start", _i), ("adaptive_target_block_end", _i),
        ("adaptive_added_indices", C.c_char * 256), ("davidson_history_count", _i),
        ("davidson_history", C.POINTER(IPTDavidsonHistoryEntry)),
        ("davidson_restart_count", _i), ("davidson_selection_history_count", _i),
        ("davidson_selection_history", C.POINTER(IPTDavidsonSelectionEntry)),
        ("davidson_block_history_count", _i),
        ("davidson_block_history", C.POINTER(IPTDavidsonBlockHistoryEntry)),
        ("best_so_far_enabled", _i), ("best_so_far_updated", _i),
        ("best_so_far_update_count", _i), ("best_so_far_step", _i),
        ("best_so_far_source", C.c_char * 32), ("best_so_far_basis_cols", _i),
        ("best_so_far_max_residual", _d), ("best_so_far_max_residual_index", _i),
        ("final_returned_from_best_so_far", _i), ("pair28_best_residual", _d),
        ("pair29_best_residual", _d), ("accepted_steps", _i), ("rejected_steps", _i),
        ("early_jump_to_continuation", _i), ("gap28_29", _d), ("relative_gap28_29", _d),
        ("cluster_residual_fro", _d), ("cluster_residual_max", _d),
        ("pair28_lock_state", C.c_char * 16), ("pair29_lock_state", C.c_char * 16),
        ("cluster_hard_locked", _i), ("cluster_soft_locked_count", _i),
    ]


class _MixedResult(C.Structure):
    _fields_ = [
        ("n", _i), ("k", _i), ("lowp_iterations", _i), ("fp64_iterations", _i),
        ("lowp_time_sec", _d), ("fp64_time_sec", _d), ("total_time_sec", _d),
        ("lowp_fixed_point_residual", _d), ("fp64_fixed_point_residual", _d),
        ("d_vectors", C.c_void_p), ("d_values", C.c_void_p),
    ]


class IPTRayleighMixedCudaDeviceResult(C.Structure):
    _fields_ = [
        ("n", _i), ("k", _i), ("tf32_iterations", _i), ("fp64_iterations", _i),
        ("tf32_time_sec", _d), ("orthogonalize_time_sec", _d),
        ("rayleigh_transform_time_sec", _d), ("fp64_time_sec", _d),
        ("backtransform_time_sec", _d), ("total_time_sec", _d),
        ("tf32_fixed_point_residual", _d), ("fp64_fixed_point_residual", _d),
        ("d_vectors", C.c_void_p), ("d_values", C.c_void_p),
    ]


class IPTBlockOptions(C.Structure):
    _fields_ = [
        ("ipt_precision", _i), ("oversample", _i), ("ipt_maxiter", _i), ("ipt_tol", _d),
        ("ipt_check_every", _i), ("residual_tol", _d), ("davidson_maxsteps", _i),
        ("max_basis", _i), ("preconditioner", _i), ("mlp_params", C.c_void_p),
        ("stream", C.c_void_p), ("strategy", _i), ("refine_maxiter", _i),
        ("inner_maxiter", _i), ("inner_tol", _d),
    ]


class IPTBlockReport(C.Structure):
    _fields_ = [
        ("n", _i), ("k", _i), ("converged", _i), ("ipt_iterations", _i),
        ("davidson_steps", _i), ("restarts", _i), ("basis_cols", _i),
        ("fp64_matvecs", C.c_longlong), ("lowp_matvecs", C.c_longlong),
        ("ipt_fixed_point_residual", _d), ("max_scaled_residual", _d),
        ("matrix_norm_inf", _d), ("ipt_ms", _d), ("rayleigh_ritz_ms", _d),
        ("davidson_ms", _d), ("total_ms", _d), ("mlp_steps_accepted", _i),
        ("mlp_steps_rejected", _i), ("precond_matvecs", C.c_longlong),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class IPTFciSpec(C.Structure):
    _fields_ = [("norb", C.c_int), ("nalpha", C.c_int), ("nbeta", C.c_int),
                ("seed", C.c_ulonglong), ("offdiag_sigma", C.c_double)]


class IPTBatchInstance(C.Structure):
    _fields_ = [("H", C.c_void_p), ("n", C.c_int), ("k", C.c_int), ("vectors", C.c_void_p),
                ("values", C.c_void_p)]


class IPTBatchOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("residual_tol", C.c_double), ("maxiter", C.c_int),
                ("lowp_maxiter", C.c_int), ("lowp_tol", C.c_double), ("threads", C.c_int),
                ("chunk", C.c_int), ("certify_precision", C.c_int)]


class IPTBatchReport(C.Structure):
    _fields_ = [("converged", C.c_int), ("status", C.c_int), ("iterations", C.c_int),
                ("fp64_iterations", C.c_int), ("max_scaled_residual", C.c_double),
                ("latency_ms", C.c_double), ("completion_ms", C.c_double)]


class IPTCscCacheInfo(C.Structure):
    _fields_ = [("magic", C.c_char * 9), ("version", C.c_int), ("n", C.c_int), ("nnz", C.c_int),
                ("matrix_inf_norm", C.c_double), ("norb", C.c_int), ("nelec", C.c_int),
                ("neleca", C.c_int), ("nelecb", C.c_int), ("na", C.c_int), ("nb", C.c_int)]


class ACXCudaResult(C.Structure):
    _fields_ = [("n", C.c_int), ("k", C.c_int), ("iterations", C.c_int), ("f_calls", C.c_int),
                ("converged", C.c_int), ("time_sec", C.c_double),
                ("iteration_time_sec", C.c_double), ("finalization_time_sec", C.c_double),
                ("max_residual", C.c_double), ("fixed_point_residual", C.c_double),
                ("d_vectors", C.c_void_p), ("d_values", C.c_void_p)]


class ACXRayleighMixedTF32CudaResult(C.Structure):
    _fields_ = [
        ("n", _i), ("k", _i), ("tf32_iterations", _i), ("fp64_iterations", _i),
        ("tf32_f_calls", _i), ("fp64_f_calls", _i), ("tf32_converged", _i),
        ("fp64_converged", _i), ("tf32_time_sec", _d), ("orthogonalize_time_sec", _d),
        ("rayleigh_transform_time_sec", _d), ("fp64_time_sec", _d),
        ("finalization_time_sec", _d), ("backtransform_time_sec", _d), ("total_time_sec", _d),
        ("tf32_fixed_point_residual", _d), ("fp64_fixed_point_residual", _d),
        ("fp64_max_residual", _d), ("d_vectors", C.c_void_p), ("d_values", C.c_void_p),
    ]


class ACXMixedTF32CudaResult(C.Structure):
    _fields_ = [("n", C.c_int), ("k", C.c_int), ("tf32_iterations", C.c_int),
                ("fp64_iterations", C.c_int), ("tf32_f_calls", C.c_int),
                ("fp64_f_calls", C.c_int), ("tf32_converged", C.c_int),
                ("fp64_converged", C.c_int), ("tf32_time_sec", C.c_double),
                ("fp64_time_sec", C.c_double), ("total_time_sec", C.c_double),
                ("finalization_time_sec", C.c_double),
                ("tf32_fixed_point_residual", C.c_double),
                ("fp64_fixed_point_residual", C.c_double), ("fp64_max_residual", C.c_double),
                ("d_vectors", C.c_void_p), ("d_values", C.c_void_p)]


# (name, restype, argtypes) of every exported entry point
_vp = C.c_void_p
SIGNATURES = [
    ("ipt_cuda_status_string", C.c_char_p, [_i]),
    ("ipt_cuda_free_result", None, [C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_free_device_result", None, [_vp, _vp]),
    ("ipt_cuda", _i, [_vp, _i, _i, _i, C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_tol", _i, [_vp, _i, _i, _d, _i, C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_with_initial", _i, [_vp, _vp, _i, _i, _i, C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_with_initial_tol", _i, [_vp, _vp, _i, _i, _d, _i, C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_device", _i, [_vp, _i, _i, _i, _vp, C.POINTER(_vp), C.POINTER(_vp)]),
    ("ipt_cuda_device_tol", _i, [_vp, _i, _i, _d, _i, _vp, C.POINTER(_vp), C.POINTER(_vp),
                                 _ip, _dp]),
    ("ipt_cuda_sparse_csc", _i, [_vp, _vp, _vp, _i, _i, _i, _i, C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_sparse_csc_tol", _i, [_vp, _vp, _vp, _i, _i, _i, _d, _i,
                                     C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_sparse_csc_with_initial", _i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i,
                                              C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_sparse_csc_with_initial_tol", _i, [_vp, _vp, _vp, _vp, _i, _i, _i, _d, _i,
                                                  C.POINTER(IPTCudaResult)]),
    ("ipt_cuda_sparse_csc_device", _i, [_vp, _vp, _vp, _i, _i, _i, _i, _vp, C.POINTER(_vp),
                                        C.POINTER(_vp)]),
    ("ipt_cuda_sparse_csc_device_tol", _i, [_vp, _vp, _vp, _i, _i, _i, _d, _i, _vp,
                                            C.POINTER(_vp), C.POINTER(_vp), _ip, _dp]),
    ("ipt_mixed_precision_cuda_device_tol", _i, [_vp, _i, _i, _d, _i, _d, _i, _vp,
                                                 C.POINTER(_MixedResult)]),
    ("ipt_mixed_precision_fp32_cuda_device_tol", _i, [_vp, _i, _i, _d, _i, _d, _i, _vp,
                                                      C.POINTER(_MixedResult)]),
    ("ipt_mixed_precision_tf32_cuda_device_tol", _i, [_vp, _i, _i, _d, _i, _d, _i, _vp,
                                                      C.POINTER(_MixedResult)]),
    ("ipt_mixed_precision_cuda_free_device_result", None, [C.POINTER(_MixedResult)]),
    ("ipt_mixed_precision_fp32_cuda_free_device_result", None, [C.POINTER(_MixedResult)]),
    ("ipt_mixed_precision_tf32_cuda_free_device_result", None, [C.POINTER(_MixedResult)]),
    ("ipt_rayleigh_mixed_tf32_cuda_device_tol", _i, [_vp, _i, _i, _d, _i, _d, _i, _vp,
                                                     C.POINTER(IPTRayleighMixedCudaDeviceResult)]),
    ("ipt_rayleigh_mixed_cuda_free_device_result", None,
     [C.POINTER(IPTRayleighMixedCudaDeviceResult)]),
    ("ipt_block_householder_signs", _i, [_vp, _i, _i, _vp]),
    ("ipt_block_accurate_product", _i, [_vp, _i, _vp, _i, _vp, _vp]),
    ("ipt_block_accurate_split_host", _i, [_vp, C.c_longlong, _d, C.POINTER(_i), _vp]),
    ("ipt_block_default_options", None, [C.POINTER(IPTBlockOptions)]),
    ("ipt_block_cholesky_inverse", _i, [_vp, _i, _vp, C.POINTER(C.c_int), _i, _vp]),
    ("ipt_block_split_double", _i, [_vp, C.c_longlong, _vp, _vp, _vp]),
    ("ipt_block_cluster_ranges", _i, [_vp, _vp, _vp, _i, _i, _i, _i, C.c_double, _i,
                                      C.c_double, _vp, _i, C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]),
    ("ipt_block_cluster_ranges_device", _i, [_vp, _vp, _vp, _i, _i, _i, _i, C.c_double, _i,
                                             C.c_double, _vp, _i, C.POINTER(C.c_int),
                                             C.POINTER(C.c_int), _vp]),
    ("acx_cuda_status_string", C.c_char_p, [_i]),
    ("acx_cuda_reset_result", None, [C.POINTER(ACXCudaResult)]),
    ("acx_cuda_free_result", None, [C.POINTER(ACXCudaResult)]),
    ("acx_mixed_precision_tf32_cuda_reset_result", None, [C.POINTER(ACXMixedTF32CudaResult)]),
    ("acx_mixed_precision_tf32_cuda_free_result", None, [C.POINTER(ACXMixedTF32CudaResult)]),
    ("acx_mixed_precision_tf32_cuda_device_tol", _i, [_vp, _i, _i, C.c_double, _i, C.c_double,
                                                      _i, _vp,
                                                      C.POINTER(ACXMixedTF32CudaResult)]),
    ("acx_cuda_device_tol", _i, [_vp, _i, _i, C.c_double, _i, _vp, C.POINTER(ACXCudaResult)]),
    ("acx_rayleigh_mixed_tf32_cuda_reset_result", None,
     [C.POINTER(ACXRayleighMixedTF32CudaResult)]),
    ("acx_rayleigh_mixed_tf32_cuda_free_result", None,
     [C.POINTER(ACXRayleighMixedTF32CudaResult)]),
    ("acx_rayleigh_mixed_tf32_cuda_device_tol", _i, [_vp, _i, _i, _d, _i, _d, _i, _vp,
                                                     C.POINTER(ACXRayleighMixedTF32CudaResult)]),
    ("ipt_block_csc_cache_info", _i, [C.c_char_p, C.POINTER(IPTCscCacheInfo)]),
    ("ipt_block_csc_cache_read", _i, [C.c_char_p, _vp, _vp, _vp, _vp, _i, _i,
                                      C.POINTER(IPTCscCacheInfo)]),
    ("ipt_block_csc_cache_write", _i, [C.c_char_p, C.POINTER(IPTCscCacheInfo), _vp, _vp, _vp,
                                       _vp]),
    ("ipt_block_prepare_csc", _i, [_vp, _vp, _vp, _i, _i, _i, _i, C.c_double, _vp, _vp, _vp,
                                   _i, C.POINTER(C.c_int), _vp, _vp, _vp, _vp, _i, _vp, _i,
                                   C.POINTER(C.c_int)]),
    ("ipt_block_cluster_basis", _i, [_vp, _vp, _vp, _i, _i, _vp, _vp, _i, _i, C.c_double,
                                     C.c_double, _vp, _vp, _vp, _vp]),
    ("ipt_block_cluster_update", _i, [_vp, _vp, _vp, _i, _i, _i, C.c_double, _vp,
                                      C.POINTER(C.c_int), _vp]),
    ("ipt_block_split_double_host", _i, [_vp, C.c_longlong, _vp, _vp]),
    ("ipt_block_symmetric_eig", _i, [_vp, _i, _vp, _vp, _vp]),
    ("ipt_block_mlp_param_count", _i, []),
    ("ipt_block_batch_default_options", None, [C.POINTER(IPTBatchOptions)]),
    ("ipt_fci_dimension", _i, [C.POINTER(IPTFciSpec), C.POINTER(C.c_longlong)]),
    ("ipt_fci_diagonal", _i, [C.POINTER(IPTFciSpec), _vp, _vp]),
    ("ipt_fci_sigma", _i, [C.POINTER(IPTFciSpec), _vp, _i, _vp, _i, _vp]),
    ("ipt_block_solve_fci", _i, [C.POINTER(IPTFciSpec), _i, C.POINTER(IPTBlockOptions), _vp, _vp,
                                 C.POINTER(IPTBlockReport)]),
    ("ipt_block_batch_plan_create", _i, [C.POINTER(IPTBatchInstance), _i,
                                         C.POINTER(IPTBatchOptions), C.POINTER(C.c_void_p)]),
    ("ipt_block_batch_plan_run", _i, [_vp, _vp]),
    ("ipt_block_batch_plan_autotune", _i, [_vp, _vp, C.POINTER(_i), C.POINTER(_i),
                                           C.POINTER(_d)]),
    ("ipt_block_batch_plan_reports", _i, [_vp, C.POINTER(IPTBatchReport)]),
    ("ipt_block_batch_plan_shape", _i, [_vp] + [C.POINTER(C.c_int)] * 5),
    ("ipt_block_batch_plan_destroy", _i, [_vp]),
    ("ipt_block_mlp_init", _i, [_vp, C.c_ulonglong, _vp]),
    ("ipt_block_mlp_forward", _i, [_vp, _vp, C.c_longlong, _i, _vp, _vp]),
    ("ipt_block_mlp_loss_grad", _i, [_vp, _vp, C.c_longlong, _vp, _vp]),
    ("ipt_block_mlp_train", _i, [_vp, _vp, C.c_longlong, _i, _i, C.c_float, C.c_ulonglong, _vp,
                                 _vp]),
    ("ipt_block_mlp_collect_csr", _i, [_vp, _vp, _vp, _i, _i, _i, C.POINTER(IPTBlockOptions), _vp,
                                       _i, _vp, C.c_longlong, C.POINTER(C.c_longlong),
                                       C.POINTER(IPTBlockReport)]),
    ("ipt_cuda_device_tol_noalloc", _i, [_vp, _i, _i, _d, _i, _vp, _vp, _vp, _ip, _dp]),
    ("ipt_block_launch_count", C.c_longlong, []),
    ("ipt_block_profile_enable", None, [_i]),
    ("ipt_block_profile_reset", None, []),
    ("ipt_block_profile_read", _i, [_i, C.POINTER(C.c_char_p), _dp, C.POINTER(C.c_longlong)]),
    ("ipt_block_trace_enable", _i, [_i]),
    ("ipt_block_trace_count", _i, []),
    ("ipt_block_trace_read", _i, [_i, C.POINTER(C.c_char_p), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_longlong)]),
    ("ipt_block_measure_fp64_peak", _i, [_dp]),
    ("ipt_block_measure_fp32_peak", _i, [_dp]),
    ("ipt_block_solve_dense_device", _i, [_vp, _i, _i, C.POINTER(IPTBlockOptions), _vp, _vp,
                                          C.POINTER(IPTBlockReport)]),
    ("ipt_block_solve_dense", _i, [_vp, _i, _i, C.POINTER(IPTBlockOptions), _vp, _vp,
                                   C.POINTER(IPTBlockReport)]),
    ("ipt_block_solve_csr_device", _i, [_vp, _vp, _vp, _i, _i, _i, C.POINTER(IPTBlockOptions),
                                        _vp, _vp, C.POINTER(IPTBlockReport)]),
    ("ipt_block_solve_csr", _i, [_vp, _vp, _vp, _i, _i, _i, C.POINTER(IPTBlockOptions), _vp,
                                 _vp, C.POINTER(IPTBlockReport)]),
]

_LIB = None


def load(path=None):
    """Load libipt_gb300.so and bind every exported entry point."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "libipt_gb300.so is not built (%s); run `python -c \"import __graft_entry__ as g; "
            "g.build()\"` first" % p)
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def status_string(code):
    return load().ipt_cuda_status_string(code).decode()


class IPTError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (what or "ipt call", status_string(status),
                                                        status))
