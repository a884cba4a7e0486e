// prep.h - host preparation of sparse input (internal).
#pragma once

#include <vector>

namespace iptgb {

// A sparse matrix ready for the CSR gather kernels.  When `permuted` is set
// the rows/columns are in ascending-diagonal order and perm[sorted] gives the
// original index (the reference's basis_to_original).
struct PreparedCsr {
    int n = 0;
    int nnz = 0;
    std::vector<int> row_ptr;
    std::vector<int> col_ind;
    std::vector<double> vals;
    std::vector<double> diag;
    std::vector<int> perm;
    bool permuted = false;
    // degeneracy lifting: block r covers [rot_first[r], rot_first[r] + rot_size[r])
    // and its rotation (column-major) follows the previous ones in rot_values
    std::vector<int> rot_first, rot_size;
    std::vector<double> rot_values;
};

// CSC validation (IPT_C_GPU/src/ipt_preparation.cu:148-169).
bool validate_csc(const int *col_ptr, const int *row_ind, int n, int nnz);

// First stored diagonal entry of each CSC column (ipt_preparation.cu:171-188).
void csc_diagonal(const int *col_ptr, const int *row_ind, const double *vals, int n,
                  std::vector<double> *diag);

// Reference preparation without degeneracy lifting
// (IPT_C_GPU/src/ipt_preparation.cu:1375-1431): validate, stable sort of the
// diagonal, and, when the order changes, a symmetric permutation that merges
// duplicates and drops explicit zeros (ipt_permute_csc, :210-262).  The
// result is emitted as CSR of the same matrix (a transpose of the CSC arrays)
// so that the gather kernels compute H X for any sparsity pattern.
// With lift_k > 0 the groups of numerically close indices around the lift_k
// targets are then rotated into the eigenbasis of their diagonal blocks, in
// up to IPT_MAX_LIFT_ROUNDS rounds (ipt_preparation.cu:1436-1592; the plain
// sparse path of the reference always lifts).  Returns IPT_CUDA_SUCCESS or
// IPT_CUDA_INVALID_ARGUMENT (also when a group is too wide, the gaps stay
// unresolved, or a group of a non-symmetric matrix would need lifting).
int prepare_csc(const int *col_ptr, const int *row_ind, const double *vals, int n, int nnz,
                bool sort_diagonal, PreparedCsr *out, int lift_k = 0,
                double degeneracy_threshold = 0.0);

// Take prepared-basis rows back to the caller's basis, in place: the lifting
// rotations, then the permutation (ipt_apply_prepared_q_to_vectors,
// ipt_preparation.cu:1222-1293).
void unpermute_vectors(const PreparedCsr &prep, double *vectors_col_major, int k);

// Columns sorted by row, duplicates summed, exact zeros dropped (the
// reference's identity permutation, ipt_preparation.cu:210-262).
void merge_csc_columns(const int *col_ptr, const int *row_ind, const double *vals, int n,
                       std::vector<int> *cp, std::vector<int> *ri, std::vector<double> *va);
// Whether merge_csc_columns would return the arrays unchanged (every column
// strictly increasing in row, no stored zeros).
bool csc_columns_merged(const int *col_ptr, const int *row_ind, const double *vals, int n);

// Real-symmetry test of merged compressed arrays (sorted, no duplicates),
// by value lookup within 1e-12 * max(1, |a|, |b|) (ipt_preparation.cu:860-883).
bool merged_is_symmetric(const int *ptr, const int *idx, const double *vals, int n);

// CSC -> CSR transpose keeping duplicates and storage order (stable by column).
void csc_to_csr(const int *col_ptr, const int *row_ind, const double *vals, int n, int nnz,
                std::vector<int> *row_ptr, std::vector<int> *col_ind, std::vector<double> *out);

}  // namespace iptgb
