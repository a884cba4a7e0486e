// prep.cpp - host preparation of sparse CSC input.
#include "prep.h"

#include <algorithm>
#include <cstring>
#include <limits>
#include <numeric>
#include <utility>

#include "../../include/ipt_cuda.h"

namespace iptgb {

bool validate_csc(const int *col_ptr, const int *row_ind, int n, int nnz)
{
    if (col_ptr == nullptr || n <= 0 || nnz < 0 || (nnz > 0 && row_ind == nullptr) ||
        col_ptr[0] != 0 || col_ptr[n] != nnz) {
        return false;
    }
    for (int c = 0; c < n; ++c) {
        if (col_ptr[c] > col_ptr[c + 1]) {
            return false;
        }
    }
    for (int p = 0; p < nnz; ++p) {
        if (row_ind[p] < 0 || row_ind[p] >= n) {
            return false;
        }
    }
    return true;
}

void csc_diagonal(const int *col_ptr, const int *row_ind, const double *vals, int n,
                  std::vector<double> *diag)
{
    diag->assign((size_t)n, 0.0);
    for (int c = 0; c < n; ++c) {
        for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
            if (row_ind[p] == c) {
                (*diag)[(size_t)c] = vals[p];
                break;
            }
        }
    }
}

void csc_to_csr(const int *col_ptr, const int *row_ind, const double *vals, int n, int nnz,
                std::vector<int> *row_ptr, std::vector<int> *col_ind, std::vector<double> *out)
{
    row_ptr->assign((size_t)n + 1U, 0);
    col_ind->resize((size_t)nnz);
    out->resize((size_t)nnz);
    for (int p = 0; p < nnz; ++p) {
        ++(*row_ptr)[(size_t)row_ind[p] + 1U];
    }
    for (int r = 0; r < n; ++r) {
        (*row_ptr)[(size_t)r + 1U] += (*row_ptr)[(size_t)r];
    }
    std::vector<int> cursor(row_ptr->begin(), row_ptr->end() - 1);
    // columns in ascending order => entries of every row stay sorted by column
    for (int c = 0; c < n; ++c) {
        for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
            const int r = row_ind[p];
            const int dst = cursor[(size_t)r]++;
            (*col_ind)[(size_t)dst] = c;
            (*out)[(size_t)dst] = vals[p];
        }
    }
}

int prepare_csc(const int *col_ptr, const int *row_ind, const double *vals, int n, int nnz,
                bool sort_diagonal, PreparedCsr *out)
{
    if (out == nullptr || vals == nullptr || !validate_csc(col_ptr, row_ind, n, nnz)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    out->n = n;
    std::vector<double> diag;
    csc_diagonal(col_ptr, row_ind, vals, n, &diag);

    std::vector<int> perm((size_t)n);
    std::iota(perm.begin(), perm.end(), 0);
    bool changed = false;
    if (sort_diagonal) {
        std::stable_sort(perm.begin(), perm.end(),
                         [&diag](int a, int b) { return diag[(size_t)a] < diag[(size_t)b]; });
        for (int i = 0; i < n; ++i) {
            if (perm[(size_t)i] != i) {
                changed = true;
                break;
            }
        }
    }

    if (!changed) {
        csc_to_csr(col_ptr, row_ind, vals, n, nnz, &out->row_ptr, &out->col_ind, &out->vals);
        // The reference re-reads the prepared diagonal summing duplicate
        // entries (ipt_extract_csc_diagonal_vectors, ipt_preparation.cu:845-858).
        out->diag.assign((size_t)n, 0.0);
        for (int r = 0; r < n; ++r) {
            for (int p = out->row_ptr[(size_t)r]; p < out->row_ptr[(size_t)r + 1U]; ++p) {
                if (out->col_ind[(size_t)p] == r) {
                    out->diag[(size_t)r] += out->vals[(size_t)p];
                }
            }
        }
        out->perm.clear();
        out->permuted = false;
        out->nnz = nnz;
        return IPT_CUDA_SUCCESS;
    }

    // Symmetric permutation.  Entry (r, c, v) moves to (inv[r], inv[c]); within
    // each new row the entries are ordered by new column, duplicates are summed
    // and exact zeros dropped (ipt_permute_csc, ipt_preparation.cu:210-262,
    // written there per column; the merged set is identical per row).
    std::vector<int> inv((size_t)n);
    for (int s = 0; s < n; ++s) {
        inv[(size_t)perm[(size_t)s]] = s;
    }
    std::vector<int> count((size_t)n + 1U, 0);
    for (int p = 0; p < nnz; ++p) {
        ++count[(size_t)inv[(size_t)row_ind[p]] + 1U];
    }
    for (int r = 0; r < n; ++r) {
        count[(size_t)r + 1U] += count[(size_t)r];
    }
    std::vector<std::pair<int, double>> entries((size_t)nnz);
    {
        std::vector<int> cursor(count.begin(), count.end() - 1);
        for (int c = 0; c < n; ++c) {
            const int nc = inv[(size_t)c];
            for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
                const int nr = inv[(size_t)row_ind[p]];
                entries[(size_t)cursor[(size_t)nr]++] = std::make_pair(nc, vals[p]);
            }
        }
    }
    out->row_ptr.assign((size_t)n + 1U, 0);
    out->col_ind.clear();
    out->vals.clear();
    out->col_ind.reserve((size_t)nnz);
    out->vals.reserve((size_t)nnz);
    for (int r = 0; r < n; ++r) {
        auto b = entries.begin() + count[(size_t)r];
        auto e = entries.begin() + count[(size_t)r + 1U];
        std::stable_sort(b, e, [](const std::pair<int, double> &x,
                                  const std::pair<int, double> &y) { return x.first < y.first; });
        out->row_ptr[(size_t)r] = (int)out->col_ind.size();
        for (auto it = b; it != e; ++it) {
            const int c = it->first;
            double v = it->second;
            while (it + 1 != e && (it + 1)->first == c) {
                ++it;
                v += it->second;
            }
            if (v != 0.0) {
                out->col_ind.push_back(c);
                out->vals.push_back(v);
            }
        }
    }
    out->row_ptr[(size_t)n] = (int)out->col_ind.size();
    out->nnz = (int)out->col_ind.size();
    // duplicates are merged by now, so the stored diagonal entry is the sum
    out->diag.assign((size_t)n, 0.0);
    for (int r = 0; r < n; ++r) {
        for (int p = out->row_ptr[(size_t)r]; p < out->row_ptr[(size_t)r + 1U]; ++p) {
            if (out->col_ind[(size_t)p] == r) {
                out->diag[(size_t)r] = out->vals[(size_t)p];
            }
        }
    }
    out->perm = perm;
    out->permuted = true;
    return IPT_CUDA_SUCCESS;
}

void unpermute_vectors(const PreparedCsr &prep, double *vectors, int k)
{
    if (!prep.permuted) {
        return;
    }
    const int n = prep.n;
    std::vector<double> tmp((size_t)n);
    for (int j = 0; j < k; ++j) {
        double *v = vectors + (size_t)j * (size_t)n;
        for (int s = 0; s < n; ++s) {
            tmp[(size_t)prep.perm[(size_t)s]] = v[s];
        }
        std::memcpy(v, tmp.data(), (size_t)n * sizeof(double));
    }
}

}  // namespace iptgb
