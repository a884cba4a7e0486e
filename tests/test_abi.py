"""The C-ABI library: exports, struct layout, argument validation (no GPU)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from block_ipt_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for fn in os.listdir(INCLUDE):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(?:int|void|long long|const char \*)\s*\*?\s*([a-z_][a-z0-9_]*)\s*\(", text):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "ipt_cuda" in names and "ipt_block_solve_dense" in names
    for name in sorted(names):
        assert hasattr(lib, name), name


def test_exported_set_is_the_declared_set():
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert exported == declared_functions()


def test_ctypes_signatures_cover_declarations():
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert declared_functions() - bound == set()


def _c_layout():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "ipt_block.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(IPTCudaResult), sizeof(IPTDavidsonHistoryEntry),
         sizeof(IPTDavidsonSelectionEntry), sizeof(IPTDavidsonBlockHistoryEntry));
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", offsetof(IPTCudaResult, vectors),
         offsetof(IPTCudaResult, values), offsetof(IPTCudaResult, matvecs),
         offsetof(IPTCudaResult, fixed_point_residual),
         offsetof(IPTCudaResult, adaptive_added_indices), offsetof(IPTCudaResult, davidson_history),
         offsetof(IPTCudaResult, davidson_block_history), offsetof(IPTCudaResult, best_so_far_source),
         offsetof(IPTCudaResult, cluster_soft_locked_count));
  printf("%zu %zu %zu\n", sizeof(IPTBlockOptions), sizeof(IPTBlockReport), sizeof(IPTMixedCudaDeviceResult));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", INCLUDE, "-o", exe, c], check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    return [list(map(int, ln.split())) for ln in lines if ln.strip()]


def test_struct_layout_matches_reference(golden):
    _, meta = golden
    ref = meta["layout"]["values"]
    sizes, offsets, ext = _c_layout()
    assert sizes + offsets == ref
    # ctypes mirror agrees with the C header
    assert C.sizeof(_lib.IPTCudaResult) == sizes[0]
    assert C.sizeof(_lib.IPTDavidsonHistoryEntry) == sizes[1]
    assert C.sizeof(_lib.IPTDavidsonSelectionEntry) == sizes[2]
    assert C.sizeof(_lib.IPTDavidsonBlockHistoryEntry) == sizes[3]
    assert C.sizeof(_lib.IPTBlockOptions) == ext[0]
    assert C.sizeof(_lib.IPTBlockReport) == ext[1]
    assert C.sizeof(_lib._MixedResult) == ext[2]
    names = meta["layout"]["names"][4:]
    for name, off in zip(names, offsets):
        assert getattr(_lib.IPTCudaResult, name).offset == off, name


def test_status_strings(lib):
    expect = ["success", "invalid argument", "allocation failed", "CUDA runtime error",
              "cuBLAS error", "cuSPARSE error", "cuSOLVER error"]
    for code, text in enumerate(expect):
        assert lib.ipt_cuda_status_string(code).decode() == text
    assert lib.ipt_cuda_status_string(99).decode() == "unknown error"


@pytest.mark.parametrize("n,k,it,tol", [(0, 1, 5, 0.0), (4, 0, 5, 0.0), (4, 5, 5, 0.0),
                                        (4, 2, -1, 0.0)])
def test_invalid_arguments_rejected_before_device_work(lib, n, k, it, tol):
    """Validation mirrors ipt_cuda.cu:1816-1828; returns before any CUDA call."""
    res = _lib.IPTCudaResult()
    H = (C.c_double * 16)()
    st = lib.ipt_cuda(C.cast(H, C.c_void_p), n, k, it, C.byref(res))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
    assert not res.vectors and not res.values
    st = lib.ipt_cuda_tol(C.cast(H, C.c_void_p), 4, 2, 0.0, 10, C.byref(res))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
    st = lib.ipt_cuda(None, 4, 2, 3, C.byref(res))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT
    st = lib.ipt_cuda_sparse_csc(None, None, None, 4, 2, 0, 3, C.byref(res))
    assert st == _lib.IPT_CUDA_INVALID_ARGUMENT


def test_free_result_resets_fields(lib):
    res = _lib.IPTCudaResult()
    res.n = 7
    res.iterations = 3
    lib.ipt_cuda_free_result(C.byref(res))
    assert res.n == 0 and res.iterations == 0
    assert res.fixed_point_residual != res.fixed_point_residual  # NaN
    assert res.best_so_far_step == -1
    assert res.pair28_lock_state == b"unknown"
    lib.ipt_cuda_free_result(None)


def test_new_entries_reject_bad_arguments_before_device_work(lib):
    """The block-cluster, ACX and cache entries validate their arguments on
    the host before any CUDA call (fake device pointers are never touched)."""
    fake = C.c_void_p(16)
    it = (C.c_int * 4)()
    rs = (C.c_double * 4)()
    for ranges in ([3, 2], [0, 4, 4, 6], [0, 64], [28, 30]):
        rg = (C.c_int * len(ranges))(*ranges)
        st = lib.ipt_block_cluster_basis(fake, fake, fake, 30, 10, fake, rg, len(ranges) // 2, 10,
                                         1e-12, 1.0, fake, it, rs, None)
        assert st == _lib.IPT_CUDA_INVALID_ARGUMENT, ranges
    rg = (C.c_int * 2)(0, 1)
    assert lib.ipt_block_cluster_basis(None, fake, fake, 30, 10, fake, rg, 1, 10, 1e-12, 1.0,
                                       fake, it, rs, None) == _lib.IPT_CUDA_INVALID_ARGUMENT
    sing = C.c_int(0)
    for first, m in ((0, 0), (0, 65), (-1, 2), (29, 2)):
        assert lib.ipt_block_cluster_update(fake, fake, fake, 30, first, m, 1.0, fake,
                                            C.byref(sing), None) == _lib.IPT_CUDA_INVALID_ARGUMENT
    res = _lib.ACXCudaResult()
    for n, k, tol, mi in ((0, 1, 1e-12, 5), (8, 9, 1e-12, 5), (8, 2, -1.0, 5), (8, 2, 1e-12, 0)):
        assert lib.acx_cuda_device_tol(fake, n, k, tol, mi, None, C.byref(res)) == 1
    assert lib.acx_cuda_status_string(5) == b"zero diagonal denominator"
    mres = _lib.ACXMixedTF32CudaResult()
    assert lib.acx_mixed_precision_tf32_cuda_device_tol(fake, 8, 2, 1e-5, 10, 1e-12, 10, None,
                                                        C.byref(mres)) == 1
    assert mres.tf32_time_sec != mres.tf32_time_sec  # reset to NaN
    info = _lib.IPTCscCacheInfo()
    assert lib.ipt_block_csc_cache_info(b"", C.byref(info)) == _lib.IPT_CUDA_INVALID_ARGUMENT
