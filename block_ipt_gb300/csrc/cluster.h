// cluster.h - the block-cluster path (internal): cluster ranges on the host
// (prep.cpp) and the block-cluster basis solve on the device (k_cluster.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <utility>
#include <vector>

namespace iptgb {

// The reference's default limit on a cluster's width (IPT_MAX_LIFT_BLOCK_SIZE,
// IPT_C_GPU/src/ipt_preparation.cu:20); the update kernel holds one m x (m+1)
// system per row in shared memory up to this width.
constexpr int kClusterMaxWidth = 64;

struct ClusterRanges {
    std::vector<std::pair<int, int>> ranges;  // inclusive, ascending, disjoint
    std::vector<int> added;                   // indices added by the adaptive expansion
    int limit_hit = 0;
    int too_large = 0;                        // a cluster exceeds max_block_size
    int max_block_size = kClusterMaxWidth;
};

// How the cluster-range rules read the matrix: the first stored entry of
// CSC column col at row (0 if absent), and the stored entries of a column
// in storage order.
struct ClusterMatrixView {
    virtual ~ClusterMatrixView() = default;
    virtual double entry(int row, int col) = 0;
    virtual void column(int col, std::vector<std::pair<int, double>> *entries) = 0;
};

// Cluster ranges of the k targets (the basis target: requested + oversample)
// of a symmetric CSC matrix whose diagonal is ascending and whose columns are
// merged (sorted by row, no duplicates: merge_csc_columns) (prep.cpp;
// ipt_preparation.cu:502-644, ipt_cuda.cu:4114-4272); the adaptive expansion
// grows the cluster of target requested_k - 1.
void cluster_ranges(const int *col_ptr, const int *row_ind, const double *vals, int n, int k,
                    int requested_k, double degeneracy_threshold, int adaptive,
                    double coupling_tau, ClusterRanges *out);

// The same rules on a matrix read through `view`, with its diagonal (sum of
// duplicates) and the largest off-diagonal magnitude of every row/column
// already formed (by the host scan above, or by a device pass over a
// symmetric CSR, k_cluster.cu).
void cluster_ranges_from(ClusterMatrixView &view, int n, const std::vector<double> &diag,
                         const std::vector<double> &offmax, int k, int requested_k,
                         double degeneracy_threshold, int adaptive, double coupling_tau,
                         ClusterRanges *out);

// cluster_ranges_from on a symmetric device CSR (rows sorted by column, no
// duplicates): diagonal and off-diagonal maxima from a device pass, the rows
// the rules read fetched on demand (k_cluster.cu).
int cluster_ranges_device(const int *row_ptr, const int *col_ind, const double *vals, int n,
                          int k, int requested_k, double degeneracy_threshold, int adaptive,
                          double coupling_tau, ClusterRanges *out, cudaStream_t s);

size_t cluster_update_smem(int m);

// One update launch over C clusters (info4: {first, m, column offset, 0}).
int launch_cluster_update(const double *X, const double *Y, const double *d, int n,
                          const int *info4, const int *active, int C, int max_m, size_t smem,
                          double damping, double *Xn, int *flags, cudaStream_t s);

// The block-cluster basis (n x sum of widths, column-major, cluster after
// cluster) of a CSR matrix with ascending diagonal d (products in
// double-float from 16384 rows, davidson_df_products); ranges holds C
// inclusive (first, last) pairs.  iterations / residuals (host, C entries)
// receive each cluster's iteration count and last fixed-point residual.
// IPT_CUDA_INVALID_ARGUMENT for a singular row system or a non-finite
// iterate, with the first such cluster in *first_error_cluster.
int cluster_basis_solve(const int *row_ptr, const int *col_ind, const double *vals, int n,
                        int nnz, const double *d, const int *ranges, int C, int maxiter, double tol,
                        double damping, double *X, int *iterations, double *residuals,
                        int *first_error_cluster, cudaStream_t s);

}  // namespace iptgb
