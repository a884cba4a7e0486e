// prep.cpp - host preparation of sparse CSC input.
#include "prep.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>
#include <utility>

#include "../../include/ipt_cuda.h"
#include "cluster.h"

namespace iptgb {

double env_double(const char *name, double default_value);
int env_int(const char *name, int default_value);
int env_flag(const char *name, int default_value);
int lift_degeneracies(std::vector<int> *cp, std::vector<int> *ri, std::vector<double> *va, int n,
                      int k, double degeneracy_threshold, int sorted_changed,
                      std::vector<double> *diag, std::vector<int> *rot_first,
                      std::vector<int> *rot_size, std::vector<double> *rot_values);

// IPT_DEBUG_PREPARATION: the reference's diagnostic lines of the degeneracy
// detection and lifting on standard output, "[IPT preparation] ..." with the
// same fields (IPT_C_GPU/src/ipt_preparation.cu:69-82, 601-613, 1448-1610).
static bool prep_debug() { return env_flag("IPT_DEBUG_PREPARATION", 0) != 0; }

#define IPTGB_PREP_CHECK(expr)                  \
    do {                                        \
        const int prep_status_ = (expr);        \
        if (prep_status_ != IPT_CUDA_SUCCESS) { \
            return prep_status_;                \
        }                                       \
    } while (0)

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
    // row indices in range, checked in slices on host threads for large inputs
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int parts = std::max(1, std::min({nnz >> 22, hw, 16}));
    std::vector<char> ok((size_t)parts, 1);
    auto check = [&](int t) {
        const long long lo = (long long)nnz * t / parts, hi = (long long)nnz * (t + 1) / parts;
        for (long long p = lo; p < hi; ++p) {
            if (row_ind[p] < 0 || row_ind[p] >= n) {
                ok[(size_t)t] = 0;
                return;
            }
        }
    };
    if (parts == 1) {
        check(0);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < parts; ++t) pool.emplace_back(check, t);
        for (auto &th : pool) th.join();
    }
    return std::all_of(ok.begin(), ok.end(), [](char x) { return x != 0; });
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

static int prepare_sorted(const int *col_ptr, const int *row_ind, const double *vals, int n,
                          int nnz, bool sort_diagonal, PreparedCsr *out);

int prepare_csc(const int *col_ptr, const int *row_ind, const double *vals, int n, int nnz,
                bool sort_diagonal, PreparedCsr *out, int lift_k, double degeneracy_threshold)
{
    IPTGB_PREP_CHECK(prepare_sorted(col_ptr, row_ind, vals, n, nnz, sort_diagonal, out));
    out->rot_first.clear();
    out->rot_size.clear();
    out->rot_values.clear();
    if (lift_k <= 0) return IPT_CUDA_SUCCESS;
    // the lifting works on the CSC arrays of the sorted matrix: the input as
    // given when the order did not change, else the permuted matrix
    std::vector<int> cp, ri;
    std::vector<double> va;
    if (!out->permuted) {
        cp.assign(col_ptr, col_ptr + (size_t)n + 1U);
        ri.assign(row_ind, row_ind + (size_t)nnz);
        va.assign(vals, vals + (size_t)nnz);
    } else {
        csc_to_csr(out->row_ptr.data(), out->col_ind.data(), out->vals.data(), n, out->nnz, &cp,
                   &ri, &va);
    }
    std::vector<double> diag;
    IPTGB_PREP_CHECK(lift_degeneracies(&cp, &ri, &va, n, lift_k, degeneracy_threshold,
                                       out->permuted ? 1 : 0, &diag, &out->rot_first,
                                       &out->rot_size, &out->rot_values));
    if (!out->rot_first.empty()) {
        csc_to_csr(cp.data(), ri.data(), va.data(), n, (int)ri.size(), &out->row_ptr,
                   &out->col_ind, &out->vals);
        out->nnz = (int)out->col_ind.size();
        out->diag = diag;
    }
    return IPT_CUDA_SUCCESS;
}

static int prepare_sorted(const int *col_ptr, const int *row_ind, const double *vals, int n,
                          int nnz, bool sort_diagonal, PreparedCsr *out)
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
    const int n = prep.n;
    // the lifting rotations, last first: v[block] <- Q v[block]
    // (ipt_apply_prepared_q_to_vectors, ipt_preparation.cu:1222-1268)
    size_t vofs = prep.rot_values.size();
    for (size_t r = prep.rot_first.size(); r-- > 0;) {
        const int first = prep.rot_first[r], m = prep.rot_size[r];
        vofs -= (size_t)m * (size_t)m;
        const double *q = prep.rot_values.data() + vofs;
        std::vector<double> t((size_t)m);
        for (int j = 0; j < k; ++j) {
            double *v = vectors + (size_t)j * (size_t)n + first;
            for (int i = 0; i < m; ++i) {
                double s = 0.0;
                for (int l = 0; l < m; ++l) s += q[(size_t)i + (size_t)l * (size_t)m] * v[l];
                t[(size_t)i] = s;
            }
            std::memcpy(v, t.data(), (size_t)m * sizeof(double));
        }
    }
    if (!prep.permuted) {
        return;
    }
    std::vector<double> tmp((size_t)n);
    for (int j = 0; j < k; ++j) {
        double *v = vectors + (size_t)j * (size_t)n;
        for (int s = 0; s < n; ++s) {
            tmp[(size_t)prep.perm[(size_t)s]] = v[s];
        }
        std::memcpy(v, tmp.data(), (size_t)n * sizeof(double));
    }
}

// Each column sorted by row, duplicates summed in that order, exact zeros
// dropped: the reference's permutation step with the identity order
// (ipt_permute_csc, ipt_preparation.cu:210-262), which its block-cluster
// preparation always applies (ipt_cuda.cu:4568-4575).
// Runs fn(first, last, part) over `parts` column ranges of about equal
// nonzero counts on host threads (the scans of large matrices are
// memory-bound passes over every nonzero); every column is visited by one
// part, so per-column results do not depend on the split.
template <class Fn>
static void for_column_parts(const int *col_ptr, int n, int parts, Fn fn)
{
    if (parts <= 1) {
        fn(0, n, 0);
        return;
    }
    const long long nnz = col_ptr[n];
    std::vector<int> cut((size_t)parts + 1U, n);
    cut[0] = 0;
    for (int t = 1; t < parts; ++t) {
        const long long want = nnz * t / parts;
        cut[(size_t)t] = (int)(std::lower_bound(col_ptr, col_ptr + n + 1, want) - col_ptr);
        cut[(size_t)t] = std::max(cut[(size_t)t - 1], std::min(cut[(size_t)t], n));
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < parts; ++t) {
        pool.emplace_back(fn, cut[(size_t)t], cut[(size_t)t + 1], t);
    }
    for (auto &th : pool) th.join();
}

// Host threads for a scan over nnz nonzeros: one per 4 M nonzeros, at most
// the hardware threads and 16.
static int scan_parts(long long nnz)
{
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    return (int)std::max(1LL, std::min<long long>({nnz >> 22, (long long)hw, 16LL}));
}

static bool column_merged(const int *col_ptr, const int *row_ind, const double *vals, int c)
{
    for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
        if (vals[p] == 0.0 || (p > col_ptr[c] && row_ind[p - 1] >= row_ind[p])) return false;
    }
    return true;
}

bool csc_columns_merged(const int *col_ptr, const int *row_ind, const double *vals, int n)
{
    const int parts = scan_parts(col_ptr[n]);
    std::vector<char> ok((size_t)parts, 1);
    for_column_parts(col_ptr, n, parts, [&](int c0, int c1, int t) {
        for (int c = c0; c < c1 && ok[(size_t)t]; ++c) ok[(size_t)t] = column_merged(col_ptr, row_ind, vals, c);
    });
    return std::all_of(ok.begin(), ok.end(), [](char x) { return x != 0; });
}

void merge_csc_columns(const int *col_ptr, const int *row_ind, const double *vals, int n,
                       std::vector<int> *cp, std::vector<int> *ri, std::vector<double> *va)
{
    cp->assign((size_t)n + 1U, 0);
    ri->clear();
    va->clear();
    ri->reserve((size_t)col_ptr[n]);
    va->reserve((size_t)col_ptr[n]);
    std::vector<std::pair<int, double>> e;
    for (int c = 0; c < n; ++c) {
        // a column already sorted by row, without duplicates or stored
        // zeros, is its own merged form
        if (column_merged(col_ptr, row_ind, vals, c)) {
            (*cp)[(size_t)c] = (int)ri->size();
            ri->insert(ri->end(), row_ind + col_ptr[c], row_ind + col_ptr[c + 1]);
            va->insert(va->end(), vals + col_ptr[c], vals + col_ptr[c + 1]);
            continue;
        }
        e.clear();
        for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) e.emplace_back(row_ind[p], vals[p]);
        std::sort(e.begin(), e.end(), [](const std::pair<int, double> &x,
                                         const std::pair<int, double> &y) { return x.first < y.first; });
        (*cp)[(size_t)c] = (int)ri->size();
        for (size_t i = 0; i < e.size(); ++i) {
            const int r = e[i].first;
            double v = e[i].second;
            while (i + 1 < e.size() && e[i + 1].first == r) v += e[++i].second;
            if (v != 0.0) {
                ri->push_back(r);
                va->push_back(v);
            }
        }
    }
    (*cp)[(size_t)n] = (int)ri->size();
}

// Real-symmetry test of a merged compressed matrix (every column - or row -
// sorted, no duplicates): each stored entry (r, c) against the value stored
// at (c, r), 0 when absent, within 1e-12 * max(1, |a|, |b|).  The test is
// the reference's (ipt_csc_is_hermitian_real, ipt_preparation.cu:860-883,
// which scans the merged, permuted CSC of its block-cluster preparation);
// the lookup is a binary search in the sorted column instead of a scan.  The
// test reads the same whether the arrays are CSC or CSR, since a matrix is
// symmetric exactly when its transpose is.
bool merged_is_symmetric(const int *ptr, const int *idx, const double *vals, int n)
{
    for (int c = 0; c < n; ++c) {
        for (int p = ptr[c]; p < ptr[c + 1]; ++p) {
            const int r = idx[p];
            const double a = vals[p];
            double b = 0.0;
            const int *lo = idx + ptr[r], *hi = idx + ptr[r + 1];
            const int *it = std::lower_bound(lo, hi, c);
            if (it != hi && *it == c) b = vals[it - idx];
            const double scale = std::max(1.0, std::max(fabs(a), fabs(b)));
            if (fabs(a - b) > 1e-12 * scale) return false;
        }
    }
    return true;
}

// ---- block-cluster ranges ---------------------------------------------------
// Restated from the reference's degenerate-subspace detection
// (IPT_C_GPU/src/ipt_preparation.cu:345-644) and the block-cluster
// preparation (IPT_C_GPU/src/ipt_cuda.cu:4114-4272, 4597-4640).

namespace {

struct GapOptions {
    double absolute_gap;
    double eps_multiplier;
    double rel_gap_tol;
    double ratio_tol;
    double eta;
    int max_block_size;
};

// ipt_preparation.cu:127-146 (defaults :16-20, environment names kept)
GapOptions gap_options(double degeneracy_threshold)
{
    GapOptions o;
    o.absolute_gap = degeneracy_threshold > 0.0 ? degeneracy_threshold : 0.0;
    o.eps_multiplier = env_double("IPT_EPS_MULTIPLIER", 1000.0);
    o.rel_gap_tol = env_double("IPT_REL_GAP_TOL", 1.0e-12);
    o.ratio_tol = std::max(env_double("IPT_COUPLING_GAP_RATIO_TOL", 0.2),
                           std::numeric_limits<double>::epsilon());
    o.eta = env_double("IPT_COUPLING_ETA", 0.02);
    const int mb = env_int("IPT_MAX_LIFT_BLOCK_SIZE", kClusterMaxWidth);
    o.max_block_size = mb > 0 ? mb : kClusterMaxWidth;
    return o;
}

// the gap below which two diagonal entries count as equal
// (ipt_preparation.cu:345-351, 412-423)
double gap_floor(double a, double b, double tau_num, const GapOptions &o)
{
    const double scale = std::max(1.0, std::max(std::fabs(a), std::fabs(b)));
    return std::max(std::max(o.absolute_gap, tau_num), o.rel_gap_tol * scale);
}

// |H[row, col]| as the first stored entry of CSC column col, 0 if absent
double csc_entry(const int *col_ptr, const int *row_ind, const double *vals, int row, int col)
{
    for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) {
        if (row_ind[p] == row) return vals[p];
    }
    return 0.0;
}

struct DisjointSets {
    std::vector<int> parent, rank;
    explicit DisjointSets(int n) : parent((size_t)n), rank((size_t)n, 0)
    {
        std::iota(parent.begin(), parent.end(), 0);
    }
    int find(int x)
    {
        int r = x;
        while (parent[(size_t)r] != r) r = parent[(size_t)r];
        while (parent[(size_t)x] != r) {
            const int next = parent[(size_t)x];
            parent[(size_t)x] = r;
            x = next;
        }
        return r;
    }
    void unite(int a, int b)
    {
        a = find(a);
        b = find(b);
        if (a == b) return;
        if (rank[(size_t)a] < rank[(size_t)b]) std::swap(a, b);
        parent[(size_t)b] = a;
        if (rank[(size_t)a] == rank[(size_t)b]) ++rank[(size_t)a];
    }
};

}  // namespace

// Grow the cluster of the last requested target by its most strongly
// coupled outside row while |H[row, col]| / gap > coupling_tau, taking the
// degenerate neighbours along (IPT_C_GPU/src/ipt_cuda.cu:4134-4272).
static void adaptive_expand(ClusterMatrixView &view, const std::vector<double> &diag,
                            int requested_k, int max_block, double tau, ClusterRanges *out)
{
    std::vector<std::pair<int, double>> colv;
    const double eps_gap = 1.0e-14;
    const int n = (int)diag.size();
    auto &ranges = out->ranges;
    auto degenerate = [&](int a, int b) {
        const double scale = std::max(1.0, std::max(std::fabs(diag[(size_t)a]), std::fabs(diag[(size_t)b])));
        const double g = std::max(eps_gap, 1000.0 * std::numeric_limits<double>::epsilon() * scale);
        return std::fabs(diag[(size_t)a] - diag[(size_t)b]) <= g;
    };
    for (;;) {
        int tid = -1;
        for (size_t i = 0; i < ranges.size(); ++i) {
            if (ranges[i].first <= requested_k - 1 && requested_k - 1 <= ranges[i].second) {
                tid = (int)i;
                break;
            }
        }
        if (tid < 0) break;
        const int first = ranges[(size_t)tid].first, last = ranges[(size_t)tid].second;
        int best_row = -1;
        double best = 0.0;
        for (int col = first; col <= last; ++col) {
            view.column(col, &colv);
            for (const auto &ev : colv) {
                const int row = ev.first;
                if (first <= row && row <= last) continue;
                const double gap = std::fabs(diag[(size_t)col] - diag[(size_t)row]);
                const double ratio = std::fabs(ev.second) / std::max(gap, eps_gap);
                if (std::max(last, row) - std::min(first, row) + 1 > max_block) {
                    if (ratio > tau) out->limit_hit = 1;
                    continue;
                }
                if (ratio > best) {
                    best = ratio;
                    best_row = row;
                }
            }
        }
        if (best_row < 0 || best <= tau) break;
        int pf = std::min(first, best_row), pl = std::max(last, best_row);
        for (bool grew = true; grew;) {
            grew = false;
            if (pf > 0 && degenerate(pf, pf - 1)) {
                --pf;
                grew = true;
            }
            if (pl + 1 < n && degenerate(pl, pl + 1)) {
                ++pl;
                grew = true;
            }
        }
        if (pl - pf + 1 > max_block) {
            out->limit_hit = 1;
            break;
        }
        for (int i = pf; i <= pl; ++i) {
            if (i < first || i > last) out->added.push_back(i);
        }
        ranges[(size_t)tid] = std::make_pair(pf, pl);
        std::sort(ranges.begin(), ranges.end());
        std::vector<std::pair<int, int>> merged;
        for (const auto &r : ranges) {
            if (merged.empty() || r.first > merged.back().second) {
                merged.push_back(r);
            } else {
                merged.back().second = std::max(merged.back().second, r.second);
            }
        }
        ranges.swap(merged);
    }
    std::sort(out->added.begin(), out->added.end());
    out->added.erase(std::unique(out->added.begin(), out->added.end()), out->added.end());
}

// Sum of the stored entries at (row, col) of a CSC matrix (duplicates add,
// ipt_preparation.cu:830-843) and the diagonal read that way (:845-858).
static double csc_value_sum(const int *col_ptr, const int *row_ind, const double *vals, int row,
                            int col)
{
    double v = 0.0;
    for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) {
        if (row_ind[p] == row) v += vals[p];
    }
    return v;
}

static void csc_diagonal_sum(const int *col_ptr, const int *row_ind, const double *vals, int n,
                             std::vector<double> *diag)
{
    diag->assign((size_t)n, 0.0);
    double *dg = diag->data();
    for_column_parts(col_ptr, n, scan_parts(col_ptr[n]), [&](int c0, int c1, int) {
        for (int c = c0; c < c1; ++c) dg[c] = csc_value_sum(col_ptr, row_ind, vals, c, c);
    });
}

namespace {

// What the subspace detection and the gap check share: the numeric gap
// scale, the strongest off-diagonal entry of every index, and the indices
// in ascending diagonal order.
struct GapScan {
    double tau_num = 0.0;
    std::vector<double> off, sorted_diag;
    std::vector<int> order;
};

// strongest off-diagonal entry of each row and column (ipt_preparation.cu:353-380)
std::vector<double> offdiag_max(const int *col_ptr, const int *row_ind, const double *vals, int n)
{
    // column maxima per column; row maxima per part, then combined (a
    // maximum does not depend on the order; NaN entries never win a
    // comparison either way); parts limited so their row arrays stay small
    int parts = scan_parts(col_ptr[n]);
    parts = std::max(1, std::min(parts, (int)((32LL << 20) / std::max(1, n))));
    std::vector<double> cs((size_t)n, 0.0), rs((size_t)n * (size_t)parts, 0.0), off((size_t)n);
    for_column_parts(col_ptr, n, parts, [&](int c0, int c1, int t) {
        double *rt = rs.data() + (size_t)t * (size_t)n;
        for (int c = c0; c < c1; ++c) {
            for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
                const int r = row_ind[p];
                if (r == c) continue;
                const double a = std::fabs(vals[p]);
                cs[(size_t)c] = std::max(cs[(size_t)c], a);
                rt[r] = std::max(rt[r], a);
            }
        }
    });
    for (int i = 0; i < n; ++i) {
        double m = cs[(size_t)i];
        for (int t = 0; t < parts; ++t) m = std::max(m, rs[(size_t)t * (size_t)n + (size_t)i]);
        off[(size_t)i] = m;
    }
    return off;
}

GapScan gap_scan_from(int n, const std::vector<double> &diag, std::vector<double> off,
                      const GapOptions &o)
{
    GapScan g;
    double dmax = 0.0;
    for (double v : diag) dmax = std::max(dmax, std::fabs(v));
    g.tau_num = o.eps_multiplier * std::numeric_limits<double>::epsilon() * std::max(1.0, dmax);
    g.off = std::move(off);
    g.order.resize((size_t)n);
    std::iota(g.order.begin(), g.order.end(), 0);
    std::stable_sort(g.order.begin(), g.order.end(),
                     [&](int a, int b) { return diag[(size_t)a] < diag[(size_t)b]; });
    g.sorted_diag.resize((size_t)n);
    for (int i = 0; i < n; ++i) g.sorted_diag[(size_t)i] = diag[(size_t)g.order[(size_t)i]];
    return g;
}

GapScan gap_scan(const int *col_ptr, const int *row_ind, const double *vals, int n,
                 const std::vector<double> &diag, const GapOptions &o)
{
    return gap_scan_from(n, diag, offdiag_max(col_ptr, row_ind, vals, n), o);
}

// The view of host CSC arrays.  `merged`: every column sorted by row without
// duplicates, so an entry is found by binary search; otherwise the first
// stored entry of the row is taken, scanning the column as the reference does.
struct HostCscView final : ClusterMatrixView {
    const int *col_ptr;
    const int *row_ind;
    const double *vals;
    bool merged;
    HostCscView(const int *cp, const int *ri, const double *va, bool merged_ = false)
        : col_ptr(cp), row_ind(ri), vals(va), merged(merged_)
    {
    }
    double entry(int row, int col) override
    {
        if (!merged) return csc_entry(col_ptr, row_ind, vals, row, col);
        const int *lo = row_ind + col_ptr[col], *hi = row_ind + col_ptr[col + 1];
        const int *it = std::lower_bound(lo, hi, row);
        return it != hi && *it == row ? vals[it - row_ind] : 0.0;
    }
    void column(int col, std::vector<std::pair<int, double>> *e) override
    {
        e->clear();
        for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) e->emplace_back(row_ind[p], vals[p]);
    }
};

// A candidate pair's figures: |d_row - d_col|, the gap counted as zero, the
// coupling, coupling / max(gap, floor) and the largest gap at which the pair
// still joins (ipt_preparation.cu:443-478).
struct ClosePair {
    double gap, floor, coupling, ratio, allowed;
};
// Candidates seen by a scan and the one with the largest coupling/gap ratio
// (the diagnostics of ipt_preparation.cu:519-613).
struct CandidateScan {
    int candidates = 0;
    double max_ratio = 0.0;
    int col = -1, row = -1;
    double gap = 0.0, coupling = 0.0;
};

// Calls join(row, col, pair) for every target col < k and every other index
// row whose gap to it is numerically zero or small against their coupling
// (ipt_preparation.cu:383-455 and the candidate loops of :502-611, 658-757).
template <class Join>
void for_each_close_pair(ClusterMatrixView &view, int n, const std::vector<double> &diag, int k,
                         const GapOptions &o, const GapScan &g, Join join,
                         CandidateScan *scan = nullptr)
{
    for (int col = 0; col < std::min(k, n); ++col) {
        const double dc = diag[(size_t)col];
        const double window =
            std::max(gap_floor(dc, dc, g.tau_num, o), g.off[(size_t)col] / o.ratio_tol);
        const auto &sd = g.sorted_diag;
        const size_t lo = (size_t)(std::lower_bound(sd.begin(), sd.end(), dc - window) - sd.begin());
        const size_t hi = (size_t)(std::upper_bound(sd.begin(), sd.end(), dc + window) - sd.begin());
        for (size_t q = lo; q < hi; ++q) {
            const int row = g.order[q];
            if (row == col) continue;
            const double dr = diag[(size_t)row];
            double coupling = std::max(std::fabs(view.entry(row, col)),
                                       std::fabs(view.entry(col, row)));
            if (!(coupling > 0.0)) {
                coupling = o.eta * std::min(g.off[(size_t)row], g.off[(size_t)col]);
            }
            const double gap = std::fabs(dr - dc);
            const double fl = gap_floor(dr, dc, g.tau_num, o);
            const double ratio = coupling > 0.0 ? coupling / std::max(gap, fl) : 0.0;
            if (scan != nullptr) {
                ++scan->candidates;
                if (ratio > scan->max_ratio) {
                    scan->max_ratio = ratio;
                    scan->col = col;
                    scan->row = row;
                    scan->gap = gap;
                    scan->coupling = coupling;
                }
            }
            if (gap <= fl || (coupling > 0.0 && ratio >= o.ratio_tol)) {
                join(row, col, ClosePair{gap, fl, coupling, ratio,
                                         std::max(fl, coupling / o.ratio_tol)});
            }
        }
    }
}

// The index ranges spanned by the groups of close indices that contain a
// target, merged when they overlap or touch (ipt_preparation.cu:502-645).
std::vector<std::pair<int, int>> degenerate_subspaces(ClusterMatrixView &view, int n,
                                                      const std::vector<double> &diag,
                                                      const GapScan &g, int k,
                                                      const GapOptions &o, int *too_large)
{
    DisjointSets sets(n);
    const bool debug = prep_debug();
    CandidateScan scan;
    int unions = 0;
    constexpr int kUnionLines = 64;
    for_each_close_pair(
        view, n, diag, k, o, g,
        [&](int row, int col, const ClosePair &c) {
            sets.unite(row, col);
            if (debug && unions < kUnionLines) {
                printf("[IPT preparation] union target=%d row=%d gap=%.17g gap_floor=%.17g "
                       "coupling=%.17g coupling_gap_ratio=%.17g ratio_tol=%.17g "
                       "allowed_gap=%.17g\n",
                       col, row, c.gap, c.floor, c.coupling, c.ratio, o.ratio_tol, c.allowed);
            }
            ++unions;
        },
        debug ? &scan : nullptr);
    if (debug) {
        printf("[IPT preparation] target_vs_all_candidates=%d unions=%d "
               "max_coupling_gap_ratio=%.17g at target=%d row=%d gap=%.17g coupling=%.17g\n",
               scan.candidates, unions, scan.max_ratio, scan.col, scan.row, scan.gap,
               scan.coupling);
        if (unions > kUnionLines) {
            printf("[IPT preparation] union log truncated after %d pairs\n", kUnionLines);
        }
        fflush(stdout);
    }
    std::vector<int> cmin((size_t)n, n), cmax((size_t)n, -1), target((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
        const int r = sets.find(i);
        cmin[(size_t)r] = std::min(cmin[(size_t)r], i);
        cmax[(size_t)r] = std::max(cmax[(size_t)r], i);
        if (i < k) target[(size_t)r] = 1;
    }
    std::vector<std::pair<int, int>> rg;
    for (int r = 0; r < n; ++r) {
        if (target[(size_t)r] && cmin[(size_t)r] < cmax[(size_t)r]) {
            rg.emplace_back(cmin[(size_t)r], cmax[(size_t)r]);
        }
    }
    std::sort(rg.begin(), rg.end());
    std::vector<std::pair<int, int>> merged;
    for (const auto &r : rg) {
        if (!merged.empty() && r.first <= merged.back().second + 1) {
            merged.back().second = std::max(merged.back().second, r.second);
        } else {
            merged.push_back(r);
        }
    }
    *too_large = 0;
    for (const auto &r : merged) {
        if (r.second - r.first + 1 > o.max_block_size) *too_large = 1;
    }
    return merged;
}

std::vector<std::pair<int, int>> degenerate_subspaces_host(const int *col_ptr,
                                                           const int *row_ind, const double *vals,
                                                           int n, const std::vector<double> &diag,
                                                           int k, const GapOptions &o,
                                                           int *too_large)
{
    const GapScan g = gap_scan(col_ptr, row_ind, vals, n, diag, o);
    HostCscView view(col_ptr, row_ind, vals);
    return degenerate_subspaces(view, n, diag, g, k, o, too_large);
}

// The (target, index) pairs still close after lifting: their number, the
// first one, and the smallest gap of a target to a close index or to its
// neighbours in diagonal order (ipt_validate_target_gaps,
// ipt_preparation.cu:658-757).
struct GapCheck {
    int bad = 0;
    double min_abs_gap = std::numeric_limits<double>::infinity();
    int first_col = -1, first_row = -1;
    ClosePair first{0.0, 0.0, 0.0, 0.0, 0.0};
};

GapCheck target_gap_check(const int *col_ptr, const int *row_ind, const double *vals, int n,
                          const std::vector<double> &diag, int k, const GapOptions &o)
{
    const GapScan g = gap_scan(col_ptr, row_ind, vals, n, diag, o);
    HostCscView view(col_ptr, row_ind, vals);
    GapCheck check;
    std::vector<int> rank((size_t)n);
    for (int i = 0; i < n; ++i) rank[(size_t)g.order[(size_t)i]] = i;
    for (int col = 0; col < std::min(k, n); ++col) {
        const int r = rank[(size_t)col];
        const double dc = diag[(size_t)col];
        if (r > 0) {
            check.min_abs_gap = std::min(check.min_abs_gap, std::fabs(dc - g.sorted_diag[(size_t)r - 1]));
        }
        if (r + 1 < n) {
            check.min_abs_gap = std::min(check.min_abs_gap, std::fabs(dc - g.sorted_diag[(size_t)r + 1]));
        }
    }
    for_each_close_pair(view, n, diag, k, o, g, [&](int row, int col, const ClosePair &c) {
        check.min_abs_gap = std::min(check.min_abs_gap, c.gap);
        if (check.bad++ == 0) {
            check.first_col = col;
            check.first_row = row;
            check.first = c;
        }
    });
    return check;
}

int target_gap_violations(const int *col_ptr, const int *row_ind, const double *vals, int n,
                          const std::vector<double> &diag, int k, const GapOptions &o)
{
    return target_gap_check(col_ptr, row_ind, vals, n, diag, k, o).bad;
}

}  // namespace

void cluster_ranges(const int *col_ptr, const int *row_ind, const double *vals, int n, int k,
                    int requested_k, double degeneracy_threshold, int adaptive,
                    double coupling_tau, ClusterRanges *out)
{
    std::vector<double> diag;
    csc_diagonal_sum(col_ptr, row_ind, vals, n, &diag);
    HostCscView view(col_ptr, row_ind, vals, true);
    cluster_ranges_from(view, n, diag, offdiag_max(col_ptr, row_ind, vals, n), k, requested_k,
                        degeneracy_threshold, adaptive, coupling_tau, out);
}

void cluster_ranges_from(ClusterMatrixView &view, int n, const std::vector<double> &diag,
                         const std::vector<double> &offmax, int k, int requested_k,
                         double degeneracy_threshold, int adaptive, double coupling_tau,
                         ClusterRanges *out)
{
    *out = ClusterRanges();
    const GapOptions o = gap_options(degeneracy_threshold);
    out->max_block_size = o.max_block_size;
    const GapScan g = gap_scan_from(n, diag, offmax, o);
    std::vector<std::pair<int, int>> merged =
        degenerate_subspaces(view, n, diag, g, k, o, &out->too_large);
    // singleton clusters for the targets not covered (ipt_cuda.cu:4114-4132)
    std::vector<char> covered((size_t)n, 0);
    for (const auto &r : merged) {
        for (int i = std::max(0, r.first); i <= r.second && i < n; ++i) covered[(size_t)i] = 1;
    }
    for (int t = 0; t < std::min(k, n); ++t) {
        if (!covered[(size_t)t]) merged.emplace_back(t, t);
    }
    std::sort(merged.begin(), merged.end());
    out->ranges = merged;
    if (adaptive && !out->too_large) {
        adaptive_expand(view, diag, requested_k, o.max_block_size, coupling_tau, out);
    }
}

// ---- degeneracy lifting -------------------------------------------------------
// The reference's plain sparse path rotates every group of close target
// indices into the eigenbasis of its diagonal block before the IPT
// iteration and rotates the result back (ipt_preparation.cu:1296-1338,
// 1222-1294, driven by :1436-1592).  The rotated matrix must carry the same
// bits as the reference's, so the local Jacobi eigensolver, the order in
// which the similarity transform emits and merges entries, and the
// summation orders follow the reference step for step.

// Classical Jacobi on a symmetric m x m block: rotate away the largest
// off-diagonal entry until none exceeds 1e-14 or 64 m^2 rotations were made
// (ipt_preparation.cu:759-828).  V receives the accumulated rotations.
static void jacobi_symmetric(const std::vector<double> &block, int m, std::vector<double> *V)
{
    std::vector<double> a = block;
    auto A = [&](int r, int c) -> double & { return a[(size_t)r + (size_t)c * (size_t)m]; };
    V->assign((size_t)m * (size_t)m, 0.0);
    for (int i = 0; i < m; ++i) (*V)[(size_t)i * (size_t)(m + 1)] = 1.0;
    for (int rot = 0; rot < 64 * m * m; ++rot) {
        int p = 0, q = 1;
        double big = 0.0;
        for (int c = 1; c < m; ++c) {
            for (int r = 0; r < c; ++r) {
                if (std::fabs(A(r, c)) > big) {
                    big = std::fabs(A(r, c));
                    p = r;
                    q = c;
                }
            }
        }
        if (big <= 1.0e-14) break;
        const double app = A(p, p), aqq = A(q, q), apq = A(p, q);
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(1.0 + theta * theta));
        const double cs = 1.0 / std::sqrt(1.0 + t * t);
        const double sn = t * cs;
        for (int r = 0; r < m; ++r) {
            if (r == p || r == q) continue;
            const double arp = A(r, p), arq = A(r, q);
            const double np_ = cs * arp - sn * arq;
            const double nq = sn * arp + cs * arq;
            A(r, p) = np_;
            A(p, r) = np_;
            A(r, q) = nq;
            A(q, r) = nq;
        }
        A(p, p) = cs * cs * app - 2.0 * sn * cs * apq + sn * sn * aqq;
        A(q, q) = sn * sn * app + 2.0 * sn * cs * apq + cs * cs * aqq;
        A(p, q) = 0.0;
        A(q, p) = 0.0;
        for (int r = 0; r < m; ++r) {
            double &vp = (*V)[(size_t)r + (size_t)p * (size_t)m];
            double &vq = (*V)[(size_t)r + (size_t)q * (size_t)m];
            const double x = vp, y = vq;
            vp = cs * x - sn * y;
            vq = sn * x + cs * y;
        }
    }
}

// Eigenvectors of a symmetric block in ascending order of their Rayleigh
// quotients v^T B v (ipt_preparation.cu:916-977).
static void sorted_symmetric_eigenvectors(const std::vector<double> &block, int m,
                                          std::vector<double> *V)
{
    jacobi_symmetric(block, m, V);
    std::vector<double> lam((size_t)m, 0.0);
    for (int j = 0; j < m; ++j) {
        const double *v = V->data() + (size_t)j * (size_t)m;
        double s = 0.0;
        for (int r = 0; r < m; ++r) {
            for (int i = 0; i < m; ++i) s += v[r] * block[(size_t)r + (size_t)i * (size_t)m] * v[i];
        }
        lam[(size_t)j] = s;
    }
    std::vector<int> idx((size_t)m);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[(size_t)a] < lam[(size_t)b]; });
    std::vector<double> sorted((size_t)m * (size_t)m);
    for (int j = 0; j < m; ++j) {
        std::copy(V->begin() + (size_t)idx[(size_t)j] * (size_t)m,
                  V->begin() + (size_t)(idx[(size_t)j] + 1) * (size_t)m,
                  sorted.begin() + (size_t)j * (size_t)m);
    }
    V->swap(sorted);
}

// ---- general (non-symmetric) blocks -------------------------------------------
// The reference lifts a degenerate group of a non-symmetric matrix with the
// eigenvectors LAPACK dgeev returns (all eigenvalues real: |Im| <= 1e-12
// max(1, |Re|), else the preparation fails), sorted by eigenvalue, and the
// inverse of that eigenvector matrix as the left factor
// (ipt_preparation.cu:979-1030, 1032-1107, 1313-1324).  This build computes
// the eigenvectors itself: Householder reduction to Hessenberg form, Francis
// double-shift QR to real Schur form with the transformations accumulated,
// real 2 x 2 blocks split by a rotation, and back substitution on the
// triangular factor (Golub & Van Loan, Matrix Computations, 4th ed.,
// Algorithms 7.4.2 and 7.5.1-7.5.2, section 7.6.4).  The vectors agree with
// dgeev's to rounding and up to sign; they are not its bits.

namespace {

struct Dense {
    std::vector<double> a;
    int m;
    Dense(int m_, double fill = 0.0) : a((size_t)m_ * (size_t)m_, fill), m(m_) {}
    double &operator()(int i, int j) { return a[(size_t)i + (size_t)j * (size_t)m]; }
};

// Reflect rows r0..r0+len-1 of H (columns c0..m-1) and columns r0.. of H
// (rows 0..rmax) and of Z by I - beta v v^T.
void apply_reflector(Dense &H, Dense &Z, const double *v, int len, double beta, int r0, int c0,
                     int rmax)
{
    const int m = H.m;
    for (int j = c0; j < m; ++j) {
        double t = 0.0;
        for (int q = 0; q < len; ++q) t += v[q] * H(r0 + q, j);
        t *= beta;
        for (int q = 0; q < len; ++q) H(r0 + q, j) -= t * v[q];
    }
    for (int i = 0; i <= rmax; ++i) {
        double t = 0.0;
        for (int q = 0; q < len; ++q) t += H(i, r0 + q) * v[q];
        t *= beta;
        for (int q = 0; q < len; ++q) H(i, r0 + q) -= t * v[q];
    }
    for (int i = 0; i < m; ++i) {
        double t = 0.0;
        for (int q = 0; q < len; ++q) t += Z(i, r0 + q) * v[q];
        t *= beta;
        for (int q = 0; q < len; ++q) Z(i, r0 + q) -= t * v[q];
    }
}

// Householder vector v (v[0] = x[0] - alpha) and beta = 2 / v^T v mapping x
// to alpha e_1; beta = 0 when x is already a multiple of e_1.
double householder(const double *x, int len, double *v)
{
    double nrm = 0.0;
    for (int q = 0; q < len; ++q) nrm += x[q] * x[q];
    nrm = std::sqrt(nrm);
    for (int q = 0; q < len; ++q) v[q] = x[q];
    if (nrm == 0.0) return 0.0;
    const double alpha = x[0] > 0.0 ? -nrm : nrm;
    v[0] -= alpha;
    double vv = 0.0;
    for (int q = 0; q < len; ++q) vv += v[q] * v[q];
    return vv > 0.0 ? 2.0 / vv : 0.0;
}

// Rotate rows and columns p, p+1 so that the real 2 x 2 diagonal block at p
// becomes upper triangular; false when its eigenvalues are complex beyond
// the reference's tolerance.
bool split_block(Dense &H, Dense &Z, int p)
{
    const int m = H.m;
    const double a = H(p, p), b = H(p, p + 1), c = H(p + 1, p), d = H(p + 1, p + 1);
    const double half = 0.5 * (a - d);
    const double disc = half * half + b * c;
    const double mean = 0.5 * (a + d);
    double lam;
    if (disc < 0.0) {
        const double im = std::sqrt(-disc);
        if (im > 1.0e-12 * std::max(1.0, std::fabs(mean))) return false;
        lam = mean;  // a numerically double real eigenvalue
    } else {
        const double r = std::sqrt(disc);
        lam = mean + (half >= 0.0 ? r : -r);  // the root without cancellation
    }
    // eigenvector of the block for lam: (b, lam - a) or (lam - d, c)
    double u0 = b, u1 = lam - a;
    const double w0 = lam - d, w1 = c;
    if (w0 * w0 + w1 * w1 > u0 * u0 + u1 * u1) {
        u0 = w0;
        u1 = w1;
    }
    const double nu = std::hypot(u0, u1);
    if (nu == 0.0) return true;  // already triangular
    const double cs = u0 / nu, sn = u1 / nu;
    // G = [[cs, -sn], [sn, cs]]: H <- G^T H G, Z <- Z G
    for (int j = 0; j < m; ++j) {
        const double x = H(p, j), y = H(p + 1, j);
        H(p, j) = cs * x + sn * y;
        H(p + 1, j) = -sn * x + cs * y;
    }
    for (int i = 0; i < m; ++i) {
        const double x = H(i, p), y = H(i, p + 1);
        H(i, p) = cs * x + sn * y;
        H(i, p + 1) = -sn * x + cs * y;
        const double zx = Z(i, p), zy = Z(i, p + 1);
        Z(i, p) = cs * zx + sn * zy;
        Z(i, p + 1) = -sn * zx + cs * zy;
    }
    H(p + 1, p) = 0.0;
    return true;
}

// Real Schur form T = Z^T A Z (upper triangular: every eigenvalue real);
// false on complex eigenvalues or no convergence.
bool real_schur(Dense &H, Dense &Z)
{
    const int m = H.m;
    const double eps = std::numeric_limits<double>::epsilon();
    for (int i = 0; i < m; ++i) Z(i, i) = 1.0;
    std::vector<double> v((size_t)std::max(m, 3));
    // Hessenberg reduction
    for (int k = 0; k + 2 < m; ++k) {
        std::vector<double> x((size_t)(m - k - 1));
        for (int q = 0; q < m - k - 1; ++q) x[(size_t)q] = H(k + 1 + q, k);
        const double beta = householder(x.data(), m - k - 1, v.data());
        if (beta == 0.0) continue;
        apply_reflector(H, Z, v.data(), m - k - 1, beta, k + 1, k, m - 1);
        for (int q = 2; q < m - k; ++q) H(k + q, k) = 0.0;
    }
    double anorm = 0.0;
    for (double e : H.a) anorm = std::max(anorm, std::fabs(e));
    int hi = m - 1, iter = 0, total = 0;
    while (hi >= 0) {
        int l = hi;
        while (l > 0) {
            double sc = std::fabs(H(l - 1, l - 1)) + std::fabs(H(l, l));
            if (sc == 0.0) sc = anorm;
            if (std::fabs(H(l, l - 1)) <= eps * sc) {
                H(l, l - 1) = 0.0;
                break;
            }
            --l;
        }
        if (l == hi) {
            --hi;
            iter = 0;
            continue;
        }
        if (l == hi - 1) {
            if (!split_block(H, Z, hi - 1)) return false;
            hi -= 2;
            iter = 0;
            continue;
        }
        if (++total > 60 * m) return false;
        ++iter;
        // shifts: the eigenvalues of the trailing 2 x 2 block, or an
        // exceptional pair after 10 and 20 fruitless sweeps
        double sum = H(hi - 1, hi - 1) + H(hi, hi);
        double prod = H(hi - 1, hi - 1) * H(hi, hi) - H(hi - 1, hi) * H(hi, hi - 1);
        if (iter == 10 || iter == 20) {
            const double w = std::fabs(H(hi, hi - 1)) + std::fabs(H(hi - 1, hi - 2));
            sum = 1.5 * w + H(hi, hi);
            prod = w * w;
        }
        // first column of (H - s1 I)(H - s2 I) on the active window
        double x = H(l, l) * H(l, l) + H(l, l + 1) * H(l + 1, l) - sum * H(l, l) + prod;
        double y = H(l + 1, l) * (H(l, l) + H(l + 1, l + 1) - sum);
        double z = H(l + 1, l) * H(l + 2, l + 1);
        for (int k = l; k <= hi - 2; ++k) {
            const double xv[3] = {x, y, z};
            const double beta = householder(xv, 3, v.data());
            if (beta != 0.0) {
                apply_reflector(H, Z, v.data(), 3, beta, k, std::max(l, k - 1), std::min(k + 3, hi));
            }
            if (k > l) {
                H(k + 1, k - 1) = 0.0;
                H(k + 2, k - 1) = 0.0;
            }
            x = H(k + 1, k);
            y = H(k + 2, k);
            if (k + 3 <= hi) z = H(k + 3, k);
        }
        const double xv[2] = {x, y};
        const double beta = householder(xv, 2, v.data());
        if (beta != 0.0) apply_reflector(H, Z, v.data(), 2, beta, hi - 1, hi - 2, hi);
        H(hi, hi - 2) = 0.0;
    }
    return true;
}

}  // namespace

// Eigenvectors of a general real m x m block, unit 2-norm columns sorted by
// ascending eigenvalue (stable); false when an eigenvalue is complex or the
// iteration fails, as the reference's dgeev path fails.
static bool general_real_eigenvectors(const std::vector<double> &block, int m,
                                      std::vector<double> *V)
{
    Dense T(m), Z(m);
    T.a = block;
    if (!real_schur(T, Z)) return false;
    double tnorm = 0.0;
    for (double e : T.a) tnorm = std::max(tnorm, std::fabs(e));
    const double small = std::max(std::numeric_limits<double>::epsilon() * tnorm,
                                  std::numeric_limits<double>::min());
    std::vector<double> lam((size_t)m), vecs((size_t)m * (size_t)m, 0.0), y((size_t)m);
    for (int i = 0; i < m; ++i) {
        const double li = T(i, i);
        lam[(size_t)i] = li;
        std::fill(y.begin(), y.end(), 0.0);
        y[(size_t)i] = 1.0;
        for (int j = i - 1; j >= 0; --j) {
            double s = 0.0;
            for (int q = j + 1; q <= i; ++q) s += T(j, q) * y[(size_t)q];
            double den = T(j, j) - li;
            if (std::fabs(den) < small) den = den < 0.0 ? -small : small;
            y[(size_t)j] = -s / den;
            if (std::fabs(y[(size_t)j]) > 1e150) {  // keep the back substitution finite
                const double r = 1.0 / std::fabs(y[(size_t)j]);
                for (int q = j; q <= i; ++q) y[(size_t)q] *= r;
            }
        }
        double nrm = 0.0;
        double *x = vecs.data() + (size_t)i * (size_t)m;
        for (int r = 0; r < m; ++r) {
            double t = 0.0;
            for (int q = 0; q <= i; ++q) t += Z(r, q) * y[(size_t)q];
            x[r] = t;
            nrm += t * t;
        }
        nrm = std::sqrt(nrm);
        if (!(nrm > 0.0) || !std::isfinite(nrm)) return false;
        for (int r = 0; r < m; ++r) x[r] /= nrm;
    }
    std::vector<int> idx((size_t)m);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[(size_t)a] < lam[(size_t)b]; });
    V->resize((size_t)m * (size_t)m);
    for (int j = 0; j < m; ++j) {
        std::copy(vecs.begin() + (size_t)idx[(size_t)j] * (size_t)m,
                  vecs.begin() + (size_t)(idx[(size_t)j] + 1) * (size_t)m,
                  V->begin() + (size_t)j * (size_t)m);
    }
    return true;
}

// Inverse of an m x m matrix by Gauss-Jordan elimination with partial
// pivoting; false when a pivot is at most 1e-14 in magnitude, the
// reference's rule (ipt_preparation.cu:1032-1107).  Writes W = (A^{-1})^T.
static bool inverse_transposed(const std::vector<double> &A, int m, std::vector<double> *W)
{
    // rows of [A | I] as row-major strips
    const int w = 2 * m;
    std::vector<double> g((size_t)m * (size_t)w, 0.0);
    for (int r = 0; r < m; ++r) {
        for (int c = 0; c < m; ++c) g[(size_t)r * w + c] = A[(size_t)r + (size_t)c * (size_t)m];
        g[(size_t)r * w + m + r] = 1.0;
    }
    for (int c = 0; c < m; ++c) {
        int piv = c;
        for (int r = c + 1; r < m; ++r) {
            if (std::fabs(g[(size_t)r * w + c]) > std::fabs(g[(size_t)piv * w + c])) piv = r;
        }
        if (std::fabs(g[(size_t)piv * w + c]) <= 1.0e-14) return false;
        if (piv != c) {
            for (int j = 0; j < w; ++j) std::swap(g[(size_t)c * w + j], g[(size_t)piv * w + j]);
        }
        const double inv = 1.0 / g[(size_t)c * w + c];
        for (int j = 0; j < w; ++j) g[(size_t)c * w + j] *= inv;
        for (int r = 0; r < m; ++r) {
            if (r == c) continue;
            const double f = g[(size_t)r * w + c];
            if (f == 0.0) continue;
            for (int j = 0; j < w; ++j) g[(size_t)r * w + j] -= f * g[(size_t)c * w + j];
        }
    }
    // W(r, c) = (A^{-1})(c, r)
    W->resize((size_t)m * (size_t)m);
    for (int r = 0; r < m; ++r) {
        for (int c = 0; c < m; ++c) (*W)[(size_t)r + (size_t)c * (size_t)m] = g[(size_t)c * w + m + r];
    }
    return true;
}

// H <- W^T H V on the block [first, first + m), with W = V for an orthogonal
// V (the symmetric lift: Q^T H Q) or W = (V^{-1})^T for a general one: column
// lists rebuilt entry by entry, then sorted by row, duplicates summed in
// that order and exact zeros dropped (ipt_preparation.cu:1109-1220).
static void rotate_block_csc(std::vector<int> *col_ptr, std::vector<int> *row_ind,
                             std::vector<double> *vals, int n, int first, int m,
                             const std::vector<double> &V, const std::vector<double> &W)
{
    std::vector<std::vector<std::pair<int, double>>> cols((size_t)n);
    auto Q = [&](int r, int c) { return W[(size_t)r + (size_t)c * (size_t)m]; };
    for (int c = 0; c < n; ++c) {
        const int cl = c - first;
        const bool c_in = cl >= 0 && cl < m;
        for (int p = (*col_ptr)[(size_t)c]; p < (*col_ptr)[(size_t)c + 1]; ++p) {
            const int r = (*row_ind)[(size_t)p];
            const int rl = r - first;
            const bool r_in = rl >= 0 && rl < m;
            const double v = (*vals)[(size_t)p];
            if (!r_in && !c_in) {
                cols[(size_t)c].emplace_back(r, v);
            } else if (!r_in) {
                for (int j = 0; j < m; ++j) {
                    const double w = v * V[(size_t)cl + (size_t)j * (size_t)m];
                    if (w != 0.0) cols[(size_t)(first + j)].emplace_back(r, w);
                }
            } else if (!c_in) {
                for (int i = 0; i < m; ++i) {
                    const double w = Q(rl, i) * v;  // (W^T)[i, rl]
                    if (w != 0.0) cols[(size_t)c].emplace_back(first + i, w);
                }
            } else {
                for (int j = 0; j < m; ++j) {
                    const double qj = V[(size_t)cl + (size_t)j * (size_t)m];
                    if (qj == 0.0) continue;
                    for (int i = 0; i < m; ++i) {
                        const double w = Q(rl, i) * v * qj;
                        if (w != 0.0) cols[(size_t)(first + j)].emplace_back(first + i, w);
                    }
                }
            }
        }
    }
    col_ptr->assign((size_t)n + 1U, 0);
    row_ind->clear();
    vals->clear();
    for (int c = 0; c < n; ++c) {
        auto &e = cols[(size_t)c];
        std::sort(e.begin(), e.end(), [](const std::pair<int, double> &x,
                                         const std::pair<int, double> &y) { return x.first < y.first; });
        (*col_ptr)[(size_t)c] = (int)row_ind->size();
        for (size_t i = 0; i < e.size(); ++i) {
            const int r = e[i].first;
            double v = e[i].second;
            while (i + 1 < e.size() && e[i + 1].first == r) v += e[++i].second;
            if (v != 0.0) {
                row_ind->push_back(r);
                vals->push_back(v);
            }
        }
    }
    (*col_ptr)[(size_t)n] = (int)row_ind->size();
}

// Real symmetric within 1e-12 relative, entry by entry (ipt_preparation.cu:860-883):
// each stored (r, c, v) against the sum of the stored entries at (c, r).  The
// sums come from a copy of every column sorted by row (stable, so duplicates
// add in storage order, as a scan of the column would), found by binary
// search: O(nnz log) instead of a column scan per entry.
static bool csc_is_symmetric(const std::vector<int> &cp, const std::vector<int> &ri,
                             const std::vector<double> &va, int n)
{
    const size_t nnz = ri.size();
    std::vector<std::pair<int, double>> sorted(nnz);
    for (size_t p = 0; p < nnz; ++p) sorted[p] = std::make_pair(ri[p], va[p]);
    for (int c = 0; c < n; ++c) {
        std::stable_sort(sorted.begin() + cp[(size_t)c], sorted.begin() + cp[(size_t)c + 1],
                         [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
                             return a.first < b.first;
                         });
    }
    auto sum_at = [&](int row, int col) {
        auto b = sorted.begin() + cp[(size_t)col], e = sorted.begin() + cp[(size_t)col + 1];
        auto it = std::lower_bound(b, e, row, [](const std::pair<int, double> &a, int r) {
            return a.first < r;
        });
        double v = 0.0;
        for (; it != e && it->first == row; ++it) v += it->second;
        return v;
    };
    for (int c = 0; c < n; ++c) {
        for (int p = cp[(size_t)c]; p < cp[(size_t)c + 1]; ++p) {
            const int r = ri[(size_t)p];
            const double v = va[(size_t)p];
            const double t = sum_at(c, r);
            const double scale = std::max(1.0, std::max(std::fabs(v), std::fabs(t)));
            if (std::fabs(v - t) > 1.0e-12 * scale) return false;
        }
    }
    return true;
}

// the first `count` diagonal entries with their gaps to the next one
static void print_diagonal(const char *label, const char *gap_label,
                           const std::vector<double> &diag, int count)
{
    for (int i = 0; i < count; ++i) {
        if (i + 1 < count) {
            printf("[IPT preparation] %s[%d]=%.17g %s=%.17g\n", label, i, diag[(size_t)i], gap_label,
                   diag[(size_t)i + 1] - diag[(size_t)i]);
        } else {
            printf("[IPT preparation] %s[%d]=%.17g\n", label, i, diag[(size_t)i]);
        }
    }
}

int lift_degeneracies(std::vector<int> *cp, std::vector<int> *ri, std::vector<double> *va, int n,
                      int k, double degeneracy_threshold, int sorted_changed,
                      std::vector<double> *diag, std::vector<int> *rot_first,
                      std::vector<int> *rot_size, std::vector<double> *rot_values)
{
    const GapOptions o = gap_options(degeneracy_threshold);
    const int mr = env_int("IPT_MAX_LIFT_ROUNDS", 3);
    const int rounds = mr > 0 ? mr : 3;
    const bool debug = prep_debug();
    const bool general = env_flag("IPT_GB300_GENERAL_LIFT", 0) != 0;
    // symmetry of the matrix as it enters the rounds; only a lift needs it
    // (and the diagnostics, which report it first)
    int symmetric = debug ? (csc_is_symmetric(*cp, *ri, *va, n) ? 1 : 0) : -1;
    if (debug) {
        printf("[IPT preparation] n=%d k=%d abs_threshold=%.17g eps_multiplier=%.17g "
               "rel_gap_tol=%.17g coupling_gap_ratio_tol=%.17g eta=%.17g max_block_size=%d "
               "max_lift_rounds=%d sorted_changed=%d hermitian=%d\n",
               n, k, o.absolute_gap, o.eps_multiplier, o.rel_gap_tol, o.ratio_tol, o.eta,
               o.max_block_size, rounds, sorted_changed, symmetric);
        fflush(stdout);
    }
    bool clean = false;
    for (int round = 0; round < rounds; ++round) {
        csc_diagonal_sum(cp->data(), ri->data(), va->data(), n, diag);
        int too_large = 0;
        const auto subspaces =
            degenerate_subspaces_host(cp->data(), ri->data(), va->data(), n, *diag, k, o,
                                      &too_large);
        if (debug) {
            printf("[IPT preparation] round=%d target_vs_all_blocks=%zu\n", round + 1,
                   subspaces.size());
            print_diagonal("diag", "gap_to_next_index", *diag, std::min(n, 10));
            for (size_t b = 0; b < subspaces.size(); ++b) {
                const int first = subspaces[b].first, last = subspaces[b].second;
                double max_gap = 0.0;
                for (int i = first; i < last; ++i) {
                    max_gap = std::max(max_gap, std::fabs((*diag)[(size_t)i + 1] - (*diag)[(size_t)i]));
                }
                printf("[IPT preparation] block[%zu]=%d:%d size=%d diag_first=%.17g "
                       "diag_last=%.17g max_adjacent_index_gap=%.17g\n",
                       b, first, last, last - first + 1, (*diag)[(size_t)first],
                       (*diag)[(size_t)last], max_gap);
            }
            fflush(stdout);
        }
        if (too_large) {
            if (debug) {
                printf("[IPT preparation] near-degenerate block exceeds max_block_size=%d; "
                       "fallback eigensolver needed\n",
                       o.max_block_size);
                fflush(stdout);
            }
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        if (subspaces.empty()) {
            clean = target_gap_violations(cp->data(), ri->data(), va->data(), n, *diag, k, o) == 0;
            break;
        }
        // a non-symmetric block needs a general real eigensolver: the
        // reference calls LAPACK dgeev when it is linked in and fails the
        // preparation otherwise (its own test build); this build does the
        // latter unless IPT_GB300_GENERAL_LIFT asks for its own eigensolver
        if (symmetric < 0) symmetric = csc_is_symmetric(*cp, *ri, *va, n) ? 1 : 0;
        if (symmetric == 0 && !general) {
            if (debug) {
                printf("[IPT preparation] lift failed status=%d\n", 1);
                fflush(stdout);
            }
            return IPT_CUDA_INVALID_ARGUMENT;
        }
        for (const auto &sub : subspaces) {
            const int first = sub.first, m = sub.second - sub.first + 1;
            std::vector<double> block((size_t)m * (size_t)m, 0.0);
            for (int c = 0; c < m; ++c) {
                for (int p = (*cp)[(size_t)(first + c)]; p < (*cp)[(size_t)(first + c) + 1]; ++p) {
                    const int r = (*ri)[(size_t)p] - first;
                    if (r >= 0 && r < m) block[(size_t)r + (size_t)c * (size_t)m] += (*va)[(size_t)p];
                }
            }
            std::vector<double> V, W;
            if (symmetric) {
                sorted_symmetric_eigenvectors(block, m, &V);
                rotate_block_csc(cp, ri, va, n, first, m, V, V);
            } else {
                if (!general_real_eigenvectors(block, m, &V) || !inverse_transposed(V, m, &W)) {
                    if (debug) {
                        printf("[IPT preparation] lift failed status=%d\n", 1);
                        fflush(stdout);
                    }
                    return IPT_CUDA_INVALID_ARGUMENT;
                }
                rotate_block_csc(cp, ri, va, n, first, m, V, W);
            }
            rot_first->push_back(first);
            rot_size->push_back(m);
            rot_values->insert(rot_values->end(), V.begin(), V.end());
        }
        csc_diagonal_sum(cp->data(), ri->data(), va->data(), n, diag);
        const GapCheck check = target_gap_check(cp->data(), ri->data(), va->data(), n, *diag, k, o);
        if (debug) {
            printf("[IPT preparation] round=%d lift succeeded total_rotations=%zu bad_gaps=%d "
                   "min_abs_gap=%.17g\n",
                   round + 1, rot_first->size(), check.bad, check.min_abs_gap);
            print_diagonal("post_lift_diag", "gap_to_next", *diag, std::min(n, std::min(k, 10)));
            if (check.bad > 0) {
                printf("[IPT preparation] first_bad_gap col=%d row=%d gap=%.17g allowed=%.17g "
                       "coupling=%.17g coupling_gap_ratio=%.17g\n",
                       check.first_col, check.first_row, check.first.gap, check.first.allowed,
                       check.first.coupling, check.first.ratio);
            }
            fflush(stdout);
        }
        if (check.bad == 0) {
            clean = true;
            break;
        }
    }
    if (!clean) {
        csc_diagonal_sum(cp->data(), ri->data(), va->data(), n, diag);
        const GapCheck check = target_gap_check(cp->data(), ri->data(), va->data(), n, *diag, k, o);
        if (check.bad > 0) {
            if (debug) {
                printf("[IPT preparation] unresolved target gap after %d lift rounds: bad_gaps=%d "
                       "min_abs_gap=%.17g first_col=%d first_row=%d gap=%.17g allowed=%.17g "
                       "coupling=%.17g coupling_gap_ratio=%.17g\n",
                       rounds, check.bad, check.min_abs_gap, check.first_col, check.first_row,
                       check.first.gap, check.first.allowed, check.first.coupling,
                       check.first.ratio);
                fflush(stdout);
            }
            return IPT_CUDA_INVALID_ARGUMENT;
        }
    }
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb

#define IPT_API extern "C" __attribute__((visibility("default")))

// Host only: the cluster ranges of the block-cluster path for a symmetric
// CSC matrix with ascending diagonal (columns merged and sorted first).
// Returns IPT_CUDA_INVALID_ARGUMENT for invalid input, a cluster wider than
// the limit (ipt_cuda.cu:4619-4632), or a capacity below the cluster count
// (*count is set either way).
IPT_API int ipt_block_cluster_ranges(const int *col_ptr, const int *row_ind, const double *vals,
                                     int n, int nnz, int k, int requested_k,
                                     double degeneracy_threshold, int adaptive,
                                     double coupling_tau, int *ranges, int capacity, int *count,
                                     int *limit_hit)
{
    if (count != nullptr) *count = 0;
    if (limit_hit != nullptr) *limit_hit = 0;
    if (vals == nullptr || count == nullptr || k <= 0 || k > n || requested_k <= 0 ||
        requested_k > k || !iptgb::validate_csc(col_ptr, row_ind, n, nnz)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    // merged and sorted first, as the reference's block-cluster preparation
    // always does (a no-op for a prepared matrix)
    std::vector<int> mcp, mri;
    std::vector<double> mva;
    const bool merged = iptgb::csc_columns_merged(col_ptr, row_ind, vals, n);
    if (!merged) iptgb::merge_csc_columns(col_ptr, row_ind, vals, n, &mcp, &mri, &mva);
    iptgb::ClusterRanges cr;
    iptgb::cluster_ranges(merged ? col_ptr : mcp.data(), merged ? row_ind : mri.data(),
                          merged ? vals : mva.data(), n, k, requested_k, degeneracy_threshold,
                          adaptive, coupling_tau, &cr);
    *count = (int)cr.ranges.size();
    if (limit_hit != nullptr) *limit_hit = cr.limit_hit;
    if (cr.too_large || *count > capacity || ranges == nullptr) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    for (size_t i = 0; i < cr.ranges.size(); ++i) {
        ranges[2 * i] = cr.ranges[i].first;
        ranges[2 * i + 1] = cr.ranges[i].second;
    }
    return IPT_CUDA_SUCCESS;
}

// Host only: the sparse preparation of the plain path (ipt_prepare_sparse_csc,
// IPT_C_GPU/src/ipt_preparation.cu:1375-1648) for checking: the prepared
// matrix as CSC, its diagonal, basis_to_original, and the lifting rotations.
IPT_API int ipt_block_prepare_csc(const int *col_ptr, const int *row_ind, const double *vals,
                                  int n, int k, int nnz, int lift, double degeneracy_threshold,
                                  int *out_col_ptr, int *out_row_ind, double *out_vals,
                                  int capacity, int *out_nnz, double *out_diag, int *out_perm,
                                  int *rot_first, int *rot_size, int rot_capacity,
                                  double *rot_values, int rot_values_capacity, int *rot_count)
{
    if (out_nnz != nullptr) *out_nnz = 0;
    if (rot_count != nullptr) *rot_count = 0;
    if (out_nnz == nullptr || rot_count == nullptr || k <= 0 || k > n) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    iptgb::PreparedCsr prep;
    const int st = iptgb::prepare_csc(col_ptr, row_ind, vals, n, nnz, true, &prep,
                                      lift ? k : 0, degeneracy_threshold);
    if (st != IPT_CUDA_SUCCESS) return st;
    // the prepared CSC: the input arrays themselves when neither the sort nor
    // a lift changed the matrix (the reference keeps them as given), else the
    // transpose of the prepared CSR (columns sorted by row, as the reference
    // rebuilds them)
    std::vector<int> cp, ri;
    std::vector<double> va;
    if (!prep.permuted && prep.rot_first.empty()) {
        cp.assign(col_ptr, col_ptr + (size_t)n + 1U);
        ri.assign(row_ind, row_ind + (size_t)nnz);
        va.assign(vals, vals + (size_t)nnz);
    } else {
        iptgb::csc_to_csr(prep.row_ptr.data(), prep.col_ind.data(), prep.vals.data(), n,
                          prep.nnz, &cp, &ri, &va);
    }
    *out_nnz = prep.nnz;
    *rot_count = (int)prep.rot_first.size();
    if (prep.nnz > capacity || *rot_count > rot_capacity ||
        (int)prep.rot_values.size() > rot_values_capacity || out_col_ptr == nullptr ||
        out_diag == nullptr || out_perm == nullptr) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    std::copy(cp.begin(), cp.end(), out_col_ptr);
    std::copy(ri.begin(), ri.end(), out_row_ind);
    std::copy(va.begin(), va.end(), out_vals);
    std::copy(prep.diag.begin(), prep.diag.end(), out_diag);
    for (int i = 0; i < n; ++i) out_perm[i] = prep.permuted ? prep.perm[(size_t)i] : i;
    std::copy(prep.rot_first.begin(), prep.rot_first.end(), rot_first);
    std::copy(prep.rot_size.begin(), prep.rot_size.end(), rot_size);
    std::copy(prep.rot_values.begin(), prep.rot_values.end(), rot_values);
    return IPT_CUDA_SUCCESS;
}
