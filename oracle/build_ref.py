"""Compile the reference's own CPU test paths into oracle/_ref/ (checker only).

TEST INFRASTRUCTURE ONLY.  The reference ships its CPU IPT inside its test
drivers (IPT_C_GPU/test_temp/runtests.cu:98-174 and
IPT_C_GPU/test/sparse/runtests_sparse.cu:91-167), which #include the solver
translation unit IPT_C_GPU/src/ipt_cuda.cu.  This recipe compiles those
files where they lie, through a tiny generated wrapper that renames their
main() and exports the static CPU helpers with C linkage, into two shared
libraries:

  oracle/_ref/libref_dense.so   ref_ipt_cpu_reference, ref_fill_perturbative_matrix,
                                ref_max_relative_residual
  oracle/_ref/libref_sparse.so  ref_sparse_ipt_cpu_reference, ref_build_banded_csc,
                                ref_h20_w_csc, ref_prepare_sparse_csc_sorted,
                                ref_block_cluster_prepare, ref_block_cluster_solve_basis,
                                ref_prepare_sparse_csc_lifted

Nothing from the reference is copied into the repository; the outputs are
git-ignored.  The reference tree is found through the IPT_REFERENCE_ROOT
environment variable (the IPT_C_GPU directory), or the first command-line
argument, falling back to /root/reference/IPT_C_GPU; where it is absent the
recipe is skipped (returns False).
"""
import os
import shutil
import subprocess
import sys

DEFAULT_REF_ROOT = "/root/reference/IPT_C_GPU"


def ref_root(argv=None):
    """The reference's IPT_C_GPU directory: argument, environment, default."""
    if argv:
        return argv[0]
    return os.environ.get("IPT_REFERENCE_ROOT", DEFAULT_REF_ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

DENSE_WRAP = r'''
#define main ipt_ref_dense_main
#include "%(ref)s/test_temp/runtests.cu"
#undef main
extern "C" int ref_ipt_cpu_reference(const double *m, int n, int k, int iterations,
                                     double *vectors, double *values) {
    double *v = NULL, *w = NULL;
    int s = ipt_cpu_reference(m, n, k, iterations, &v, &w);
    if (s == 0) {
        memcpy(vectors, v, (size_t)n * (size_t)k * sizeof(double));
        memcpy(values, w, (size_t)k * sizeof(double));
    }
    free(v); free(w);
    return s;
}
extern "C" void ref_fill_perturbative_matrix(double *m, int n, int symmetric) {
    fill_perturbative_matrix(m, n, symmetric);
}
extern "C" double ref_max_relative_residual(const double *m, const double *v,
                                            const double *w, int n, int k) {
    return max_relative_residual(m, v, w, n, k);
}
/* Binary layout of the result structs: sizes, then field offsets. */
#include <stddef.h>
extern "C" int ref_result_layout(long long *out, int cap) {
    long long v[] = {
        (long long)sizeof(IPTCudaResult), (long long)sizeof(IPTDavidsonHistoryEntry),
        (long long)sizeof(IPTDavidsonSelectionEntry), (long long)sizeof(IPTDavidsonBlockHistoryEntry),
        (long long)offsetof(IPTCudaResult, vectors), (long long)offsetof(IPTCudaResult, values),
        (long long)offsetof(IPTCudaResult, matvecs), (long long)offsetof(IPTCudaResult, fixed_point_residual),
        (long long)offsetof(IPTCudaResult, adaptive_added_indices),
        (long long)offsetof(IPTCudaResult, davidson_history),
        (long long)offsetof(IPTCudaResult, davidson_block_history),
        (long long)offsetof(IPTCudaResult, best_so_far_source),
        (long long)offsetof(IPTCudaResult, cluster_soft_locked_count)};
    int cnt = (int)(sizeof(v) / sizeof(v[0]));
    for (int i = 0; i < cnt && i < cap; ++i) out[i] = v[i];
    return cnt;
}
'''

SPARSE_WRAP = r'''
#define main ipt_ref_sparse_main
#include "%(ref)s/test/sparse/runtests_sparse.cu"
#undef main
extern "C" int ref_sparse_ipt_cpu_reference(const double *m, int n, int k, int iterations,
                                            double *vectors, double *values) {
    double *v = NULL, *w = NULL;
    int s = ipt_cpu_reference(m, n, k, iterations, &v, &w);
    if (s == 0) {
        memcpy(vectors, v, (size_t)n * (size_t)k * sizeof(double));
        memcpy(values, w, (size_t)k * sizeof(double));
    }
    free(v); free(w);
    return s;
}
extern "C" int ref_build_banded_csc(int n, int *col_ptr, int *row_ind, double *values) {
    int *cp = NULL, *ri = NULL; double *va = NULL; int nnz = 0;
    if (build_banded_csc(n, &cp, &ri, &va, &nnz) != 0) return -1;
    memcpy(col_ptr, cp, (size_t)(n + 1) * sizeof(int));
    memcpy(row_ind, ri, (size_t)nnz * sizeof(int));
    memcpy(values, va, (size_t)nnz * sizeof(double));
    free(cp); free(ri); free(va);
    return nnz;
}
extern "C" int ref_h20_w_csc(int *col_ptr, int *row_ind, double *values) {
    if (col_ptr) memcpy(col_ptr, H20_W_CSC_COL_PTR, sizeof(H20_W_CSC_COL_PTR));
    if (row_ind) memcpy(row_ind, H20_W_CSC_ROW_IND, sizeof(H20_W_CSC_ROW_IND));
    if (values) memcpy(values, H20_W_CSC_VALUES, sizeof(H20_W_CSC_VALUES));
    return H20_W_CSC_NNZ;
}
/* Sort/permute only (no degeneracy lifting): returns prepared nnz, fills the
 * sorted CSC, its diagonal and basis_to_original (identity if unchanged). */
extern "C" int ref_prepare_sparse_csc_sorted(const int *col_ptr, const int *row_ind,
                                             const double *values, int n, int k, int nnz,
                                             int *out_col_ptr, int *out_row_ind,
                                             double *out_values, double *out_diag,
                                             int *out_perm) {
    IPTPreparedCsc p;
    int s = ipt_prepare_sparse_csc(col_ptr, row_ind, values, n, k, nnz, 1, 0, 0.0, &p);
    if (s != 0) return -s;
    memcpy(out_col_ptr, p.col_ptr, (size_t)(n + 1) * sizeof(int));
    if (p.nnz > 0) {
        memcpy(out_row_ind, p.row_ind, (size_t)p.nnz * sizeof(int));
        memcpy(out_values, p.values, (size_t)p.nnz * sizeof(double));
    }
    memcpy(out_diag, p.diagonal, (size_t)n * sizeof(double));
    for (int i = 0; i < n; ++i) out_perm[i] = p.basis_to_original ? p.basis_to_original[i] : i;
    int out = p.nnz;
    ipt_prepared_csc_free(&p);
    return out;
}
/* The plain path's preparation with degeneracy lifting (ipt_prepare_sparse_csc
 * with lift = 1): returns the prepared nnz (or -status) and fills the CSC,
 * diagonal, basis_to_original and the rotations; when vectors is not NULL the
 * reference's back-transform (ipt_apply_prepared_q_to_vectors) is applied to
 * them in place (n x kv, prepared basis -> caller's basis). */
extern "C" int ref_prepare_sparse_csc_lifted(const int *col_ptr, const int *row_ind,
                                             const double *values, int n, int k, int nnz,
                                             double threshold, int *out_col_ptr,
                                             int *out_row_ind, double *out_values, int capacity,
                                             double *out_diag, int *out_perm, int *rot_first,
                                             int *rot_size, double *rot_values, int rot_cap,
                                             int rot_values_cap, int *rot_count,
                                             double *vectors, int kv) {
    IPTPreparedCsc p;
    int s = ipt_prepare_sparse_csc(col_ptr, row_ind, values, n, k, nnz, 1, 1, threshold, &p);
    if (s != 0) return -s;
    int out = p.nnz;
    *rot_count = p.rotation_count;
    if (p.nnz <= capacity && p.rotation_count <= rot_cap &&
        p.rotation_values_count <= rot_values_cap) {
        memcpy(out_col_ptr, p.col_ptr, (size_t)(n + 1) * sizeof(int));
        if (p.nnz > 0) {
            memcpy(out_row_ind, p.row_ind, (size_t)p.nnz * sizeof(int));
            memcpy(out_values, p.values, (size_t)p.nnz * sizeof(double));
        }
        memcpy(out_diag, p.diagonal, (size_t)n * sizeof(double));
        for (int i = 0; i < n; ++i) out_perm[i] = p.basis_to_original ? p.basis_to_original[i] : i;
        if (p.rotation_count > 0) {
            memcpy(rot_first, p.rotation_starts, (size_t)p.rotation_count * sizeof(int));
            memcpy(rot_size, p.rotation_sizes, (size_t)p.rotation_count * sizeof(int));
            memcpy(rot_values, p.rotation_values, (size_t)p.rotation_values_count * sizeof(double));
        }
        if (vectors != NULL && kv > 0) ipt_apply_prepared_q_to_vectors(&p, vectors, kv);
    } else {
        out = -1000;
    }
    ipt_prepared_csc_free(&p);
    return out;
}
/* Block-cluster preparation (ipt_block_cluster_prepare, ipt_cuda.cu:4555-4688):
 * the cluster ranges of the diagonal-sorted matrix; returns the range count,
 * or -status. */
extern "C" int ref_block_cluster_prepare(const int *col_ptr, const int *row_ind,
                                         const double *values, int n, int k, int nnz,
                                         int *out_ranges, int capacity, int *out_limit_hit,
                                         int *out_added, int added_capacity, int *out_added_count) {
    IPTCudaResult r;
    memset(&r, 0, sizeof(r));
    IPTBlockClusterPreparation p;
    int s = ipt_block_cluster_prepare(col_ptr, row_ind, values, n, k, nnz, 100, 0.0, 0, &r, &p);
    if (s != 0) return -s;
    int cnt = (int)p.ranges.size();
    for (int i = 0; i < cnt && i < capacity; ++i) {
        out_ranges[2 * i] = p.ranges[i].first;
        out_ranges[2 * i + 1] = p.ranges[i].second;
    }
    *out_limit_hit = p.adaptive_limit_hit;
    *out_added_count = (int)p.adaptive_added_indices.size();
    for (int i = 0; i < *out_added_count && i < added_capacity; ++i) {
        out_added[i] = p.adaptive_added_indices[i];
    }
    return cnt;
}
/* The reference's CPU block-cluster basis solve of one cluster
 * (ipt_block_cluster_solve_basis, ipt_cuda.cu:4274-4395) on a sorted CSC;
 * returns 1 on success, 0 when a row system is singular or an entry is not
 * finite. */
extern "C" int ref_block_cluster_solve_basis(const int *col_ptr, const int *row_ind,
                                             const double *values, int n, int nnz,
                                             const double *diag, int first, int last,
                                             int maxiter, double tol, double damping,
                                             double *basis_out, int *iterations) {
    std::vector<int> cp(col_ptr, col_ptr + n + 1), ri(row_ind, row_ind + nnz);
    std::vector<double> va(values, values + nnz), d(diag, diag + n), b;
    int it = 0;
    int ok = ipt_block_cluster_solve_basis(cp, ri, va, d, first, last, maxiter, tol, damping,
                                           &b, &it);
    if (ok) memcpy(basis_out, b.data(), b.size() * sizeof(double));
    *iterations = it;
    return ok;
}
'''


def build(verbose=False, root=None):
    """Build oracle/_ref/*.so from the reference sources; False if absent."""
    root = root or ref_root()
    if not os.path.isdir(root):
        return False
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for name, text in (("dense", DENSE_WRAP), ("sparse", SPARSE_WRAP)):
        src = os.path.join(OUT, "ref_%s_wrap.cu" % name)
        lib = os.path.join(OUT, "libref_%s.so" % name)
        with open(src, "w") as f:
            f.write(text % {"ref": root})
        cmd = [nvcc, "-O2", "-std=c++14", "-shared", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-w",
               "-gencode", "arch=compute_103a,code=sm_103a",
               "-o", lib, src, "-lcublas", "-lcusparse", "-lcusolver"]
        jobs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                           stderr=subprocess.STDOUT)))
    ok = True
    for cmd, proc in jobs:
        out, _ = proc.communicate()
        if proc.returncode != 0:
            ok = False
            sys.stderr.write(out.decode(errors="replace")[-4000:])
        elif verbose:
            print(" ".join(cmd))
    return ok


if __name__ == "__main__":
    sys.exit(0 if build(verbose=True, root=ref_root(sys.argv[1:])) else 1)
