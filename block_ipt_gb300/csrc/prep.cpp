// prep.cpp - host preparation of sparse CSC input.
#include "prep.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <utility>

#include "../../include/ipt_cuda.h"
#include "cluster.h"

namespace iptgb {

double env_double(const char *name, double default_value);
int env_int(const char *name, int default_value);

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
static void adaptive_expand(const int *col_ptr, const int *row_ind, const double *vals,
                            const std::vector<double> &diag, int requested_k, int max_block,
                            double tau, ClusterRanges *out)
{
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
            for (int p = col_ptr[col]; p < col_ptr[col + 1]; ++p) {
                const int row = row_ind[p];
                if (first <= row && row <= last) continue;
                const double gap = std::fabs(diag[(size_t)col] - diag[(size_t)row]);
                const double ratio = std::fabs(vals[p]) / std::max(gap, eps_gap);
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

void cluster_ranges(const int *col_ptr, const int *row_ind, const double *vals, int n, int k,
                    int requested_k, double degeneracy_threshold, int adaptive,
                    double coupling_tau, ClusterRanges *out)
{
    *out = ClusterRanges();
    const GapOptions o = gap_options(degeneracy_threshold);
    out->max_block_size = o.max_block_size;
    std::vector<double> diag;
    csc_diagonal(col_ptr, row_ind, vals, n, &diag);
    double dmax = 0.0;
    for (double v : diag) dmax = std::max(dmax, std::fabs(v));
    const double tau_num = o.eps_multiplier * std::numeric_limits<double>::epsilon() *
                           std::max(1.0, dmax);
    // strongest off-diagonal entry of each row and column (ipt_preparation.cu:353-380)
    std::vector<double> cs((size_t)n, 0.0), rs((size_t)n, 0.0), off((size_t)n);
    for (int c = 0; c < n; ++c) {
        for (int p = col_ptr[c]; p < col_ptr[c + 1]; ++p) {
            const int r = row_ind[p];
            if (r == c) continue;
            const double a = std::fabs(vals[p]);
            cs[(size_t)c] = std::max(cs[(size_t)c], a);
            rs[(size_t)r] = std::max(rs[(size_t)r], a);
        }
    }
    for (int i = 0; i < n; ++i) off[(size_t)i] = std::max(cs[(size_t)i], rs[(size_t)i]);
    std::vector<int> order((size_t)n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return diag[(size_t)a] < diag[(size_t)b]; });
    std::vector<double> sd((size_t)n);
    for (int i = 0; i < n; ++i) sd[(size_t)i] = diag[(size_t)order[(size_t)i]];
    // union every target with the rows whose gap is numerically zero or small
    // against their coupling (ipt_preparation.cu:425-455, 502-611)
    DisjointSets sets(n);
    for (int col = 0; col < std::min(k, n); ++col) {
        const double dc = diag[(size_t)col];
        const double window =
            std::max(gap_floor(dc, dc, tau_num, o), off[(size_t)col] / o.ratio_tol);
        const size_t lo = (size_t)(std::lower_bound(sd.begin(), sd.end(), dc - window) - sd.begin());
        const size_t hi = (size_t)(std::upper_bound(sd.begin(), sd.end(), dc + window) - sd.begin());
        for (size_t q = lo; q < hi; ++q) {
            const int row = order[q];
            if (row == col) continue;
            const double dr = diag[(size_t)row];
            double coupling = std::max(std::fabs(csc_entry(col_ptr, row_ind, vals, row, col)),
                                       std::fabs(csc_entry(col_ptr, row_ind, vals, col, row)));
            if (!(coupling > 0.0)) {
                coupling = o.eta * std::min(off[(size_t)row], off[(size_t)col]);
            }
            const double gap = std::fabs(dr - dc);
            const double fl = gap_floor(dr, dc, tau_num, o);
            const bool join =
                gap <= fl || (coupling > 0.0 && coupling / std::max(gap, fl) >= o.ratio_tol);
            if (join) sets.unite(row, col);
        }
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
    // merge overlapping or touching ranges (ipt_preparation.cu:480-500)
    std::sort(rg.begin(), rg.end());
    std::vector<std::pair<int, int>> merged;
    for (const auto &r : rg) {
        if (!merged.empty() && r.first <= merged.back().second + 1) {
            merged.back().second = std::max(merged.back().second, r.second);
        } else {
            merged.push_back(r);
        }
    }
    for (const auto &r : merged) {
        if (r.second - r.first + 1 > o.max_block_size) out->too_large = 1;
    }
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
        adaptive_expand(col_ptr, row_ind, vals, diag, requested_k, o.max_block_size,
                        coupling_tau, out);
    }
}

}  // namespace iptgb

#define IPT_API extern "C" __attribute__((visibility("default")))

// Host only: the cluster ranges of the block-cluster path for a symmetric
// CSC matrix with ascending diagonal.  Returns IPT_CUDA_INVALID_ARGUMENT for
// invalid input, a cluster wider than the limit (ipt_cuda.cu:4619-4632), or a
// capacity below the cluster count (*count is set either way).
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
    iptgb::ClusterRanges cr;
    iptgb::cluster_ranges(col_ptr, row_ind, vals, n, k, requested_k, degeneracy_threshold,
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
