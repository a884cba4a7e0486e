// block_solver.cu - block IPT + CholQR2 + Rayleigh-Ritz + Davidson driver.
//
// Steps follow the reference's block path (IPT_C_GPU/src/ipt_cuda.cu:4712-5016):
//   1. IPT on the p = k + oversample lowest diagonal positions (the
//      reference iterates per near-degenerate cluster, :2871-3037; here one
//      IPT block covers all targets and Rayleigh-Ritz resolves the clusters);
//   2. orthonormal basis of the IPT block (CholQR2 with FP64 Gram matrices,
//      the reference's mixed CholQR, IPT_C_GPU/mixed/ipt_rayleigh_mixed_mpqr_cuda.cu:169-386);
//   3. Rayleigh-Ritz: T = V^T H V in FP64, symmetric eigensolve, Ritz pairs
//      (ipt_cuda.cu:3039-3316);
//   4. residual-driven Davidson: corrections r_j / (d - theta_j) with the
//      clipped denominator for every unconverged pair, CGS2 against the basis,
//      thick restart once the basis is full, a new Rayleigh-Ritz per step, the
//      best-so-far Ritz set kept (ipt_cuda.cu:3318-3982, 485-701).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "block_solver.h"
#include "common.cuh"

namespace iptgb {

// A learned Davidson step is kept when the largest scaled residual drops at
// least as much as a plain diagonal step is expected to: the geometric mean
// of the drops of this solve's plain steps, kPlainDropPrior before the first
// plain step, and in any case below kLearnedDrop of its value.  Tuning knob
// IPT_GB300_MLP_ACCEPT replaces the required factor.
constexpr double kLearnedDrop = 0.75;
constexpr double kPlainDropPrior = 0.5;

// Rows from which the Davidson products switch to double-float.
constexpr int kDfDavidsonMinRows = 16384;

bool davidson_df_products(int n)
{
    const int knob = env_int("IPT_GB300_DF_DAVIDSON", -1);
    return knob >= 0 ? knob != 0 : n >= kDfDavidsonMinRows;
}

void fill_default_options(IPTBlockOptions *opt)
{
    memset(opt, 0, sizeof(*opt));
    opt->ipt_precision = IPT_BLOCK_FP64;
    opt->oversample = -1;  // automatic
    opt->ipt_maxiter = 60;
    opt->ipt_tol = 1e-4;
    opt->ipt_check_every = 8;  // each read-back idles the GPU for a host round trip
    opt->residual_tol = 1e-8;
    opt->davidson_maxsteps = 40;
    opt->max_basis = 0;
    opt->preconditioner = IPT_BLOCK_PRECOND_DIAGONAL;
    opt->mlp_params = nullptr;
    opt->stream = nullptr;
    opt->strategy = IPT_BLOCK_STRATEGY_REFINE;
    opt->refine_maxiter = 300;
    opt->inner_maxiter = 64;
    opt->inner_tol = 3e-3;
}

namespace {

struct Events {
    cudaEvent_t e[8] = {};
    int create()
    {
        for (auto &x : e) {
            IPTGB_CUDA(cudaEventCreate(&x));
        }
        return IPT_CUDA_SUCCESS;
    }
    ~Events()
    {
        for (auto &x : e) {
            if (x != nullptr) cudaEventDestroy(x);
        }
    }
};

float elapsed_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// Orthonormalise the n x c block B into dst (CholQR: G = B^T B = R^T R,
// dst = B R^{-1}).  G, Rinv: c x c scratch; st: device int.
int cholqr(BlockOps &ops, const double *B, int n, int c, double *dst, double *G, double *Rinv,
           int *st_dev, int *st_host, cudaStream_t s)
{
    IPTGB_CHECK(ops.gram(B, n, c, B, n, c, n, G, c));
    // the factor in double-float with the double-float products (the FP64
    // one-CTA factorisation is latency-bound on GB300's FP64 pipe)
    IPTGB_CHECK(ops.chol_inverse(G, c, Rinv, st_dev, nullptr, ops.df_products));
    IPTGB_CHECK(ops.tall_gemm(B, n, Rinv, c, dst, n, n, c, c));
    IPTGB_CUDA(cudaMemcpyAsync(st_host, st_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    if (*st_host < 0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    return IPT_CUDA_SUCCESS;
}

// Orthogonality of the n x c columns C: G = C^T C with FP64 products into
// the c x c scratch G, then the Frobenius norm and the largest entry of
// G - I on the host.  A non-finite entry of C makes its column's diagonal
// entry of G non-finite (an entry of magnitude above ~1e154 does too, which
// the reference's host scan would not flag).  Reference:
// IPT_C_GPU/src/ipt_cuda.cu:2489-2524.
int orth_figure(BlockOps &ops, const double *C, int n, int c, double *G, cudaStream_t s,
                OrthFigure *out)
{
    const bool df = ops.df_products;
    ops.df_products = false;
    const int st = ops.gram(C, n, c, C, n, c, n, G, c);
    ops.df_products = df;
    IPTGB_CHECK(st);
    std::vector<double> h((size_t)c * c);
    IPTGB_CUDA(cudaMemcpyAsync(h.data(), G, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    IPTGB_CUDA(cudaStreamSynchronize(s));
    double fro = 0.0, mx = 0.0;
    int invalid = 0;
    for (int j = 0; j < c && !invalid; ++j) {
        invalid = !isfinite(h[(size_t)j * c + j]);
    }
    for (int j = 0; j < c && !invalid; ++j) {
        for (int i = 0; i < c; ++i) {
            const double e = h[(size_t)j * c + i] - (i == j ? 1.0 : 0.0);
            fro += e * e;
            mx = std::max(mx, fabs(e));
        }
    }
    out->invalid = invalid;
    out->frobenius = invalid ? NAN : sqrt(fro);
    out->max_abs = invalid ? NAN : mx;
    return IPT_CUDA_SUCCESS;
}

}  // namespace

int block_solve(const BlockSolveInput &in, double *X_out, double *values_out,
                IPTBlockReport *rep, cudaStream_t s)
{
    const int n = in.n;
    const int k = in.k;
    IPTBlockOptions opt = in.opt;
    int p = opt.oversample < 0 ? std::min(n, k + std::max(8, k / 4)) : std::min(n, k + opt.oversample);
    if (p < k) p = k;
    // Basis up to 6k columns (at least the reference's k + max(16, (2k+2)/3),
    // ipt_cuda.cu:3335-3338): a larger basis converges clustered spectra in
    // far fewer steps, and the projected eigensolve stays cheap.
    int maxb = opt.max_basis > 0 ? opt.max_basis
                                 : std::max(p + k, std::max(6 * k, k + std::max(16, (2 * k + 2) / 3)));
    maxb = std::min(maxb, n);
    maxb = std::max(maxb, p);
    if (maxb > 112) {
        // the projected eigensolve holds two maxb x maxb FP64 matrices in shared memory
        maxb = std::max(112, p);
    }
    if (maxb > 112 || k > 64) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    const double tol = opt.residual_tol > 0.0 ? opt.residual_tol : 1e-8;

    memset(rep, 0, sizeof(*rep));
    rep->n = n;
    rep->k = k;
    rep->matrix_norm_inf = in.hnorm;
    rep->max_scaled_residual = NAN;
    rep->ipt_fixed_point_residual = NAN;

    BlockOps ops;
    ops.stream = s;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&ops.sms, cudaDevAttrMultiProcessorCount, dev);
    ops.df_products = davidson_df_products(n);

    const size_t nb = (size_t)n * (size_t)maxb;
    DeviceBuffer<double> V, AV, Vt, AVt, Xr, AXr, R, Xbest, small;
    IPTGB_CHECK(V.alloc(nb, s));
    IPTGB_CHECK(AV.alloc(nb, s));
    IPTGB_CHECK(Vt.alloc(nb, s));
    IPTGB_CHECK(AVt.alloc(nb, s));
    IPTGB_CHECK(Xr.alloc((size_t)n * k, s));
    IPTGB_CHECK(AXr.alloc((size_t)n * k, s));
    IPTGB_CHECK(R.alloc((size_t)n * k, s));
    IPTGB_CHECK(Xbest.alloc((size_t)n * k, s));
    const size_t mm = (size_t)maxb * maxb;
    const size_t small_head = 4 * mm + 4 * (size_t)maxb + 4 * (size_t)k + 64;
    IPTGB_CHECK(small.alloc(small_head + mm, s));
    double *Tf = small.ptr + small_head;  // V^T H V of the current basis, ld maxb
    double *Tm = small.ptr;
    double *Zm = Tm + mm;
    double *Gm = Zm + mm;
    double *Rinv = Gm + mm;
    double *theta = Rinv + mm;
    double *theta_best = theta + maxb;
    double *cnorm0 = theta_best + maxb;
    double *cnorm1 = cnorm0 + maxb;
    double *rnorm = cnorm1 + maxb;
    double *scaled = rnorm + k;
    int *sel = (int *)(scaled + k);           // k ints
    int *st_dev = (int *)(scaled + 2 * k);    // a few ints
    std::vector<double> h_scaled((size_t)k), h_theta((size_t)maxb), h_c0((size_t)maxb),
        h_c1((size_t)maxb);
    std::vector<int> h_sel((size_t)k);
    int h_status = 0;

    Events ev;
    IPTGB_CHECK(ev.create());
    IPTGB_CUDA(cudaEventRecord(ev.e[0], s));

    // ---- 1. IPT stage ------------------------------------------------------
    int ipt_iters = 0;
    double ipt_res = NAN;
    long long lowp_mv = 0;
    if (in.initial != nullptr) {
        // start block given (e.g. from the refinement driver): its columns,
        // then unit vectors of the next diagonal positions up to p
        IPTGB_CHECK(launch_set_identity(Vt.ptr, n, p, s));
        IPTGB_CUDA(cudaMemcpyAsync(Vt.ptr, in.initial,
                                   (size_t)n * std::min(p, in.initial_cols) * sizeof(double),
                                   cudaMemcpyDeviceToDevice, s));
    } else {
        IPTGB_CHECK(in.ipt->run(p, opt.ipt_maxiter, opt.ipt_tol, std::max(1, opt.ipt_check_every),
                                Vt.ptr, &ipt_iters, &ipt_res, &lowp_mv));
    }
    rep->ipt_iterations = ipt_iters;
    rep->ipt_fixed_point_residual = ipt_res;
    if (in.lowp) {
        rep->lowp_matvecs += lowp_mv;
    } else {
        rep->fp64_matvecs += lowp_mv;
    }
    IPTGB_CUDA(cudaEventRecord(ev.e[1], s));

    // ---- 2. CholQR2 of the IPT block ---------------------------------------
    int m = p;
    OrthFigure basis_now, ritz_now, basis_best, ritz_best;
    bool raw_basis_pending = false;
    if (in.orth != nullptr && in.orth->raw_first_basis) {
        IPTGB_CHECK(orth_figure(ops, Vt.ptr, n, m, Gm, s, &basis_now));
        raw_basis_pending = true;
    }
    {
        int st = cholqr(ops, Vt.ptr, n, m, V.ptr, Gm, Rinv, st_dev, &h_status, s);
        if (st == IPT_CUDA_SUCCESS) {
            st = cholqr(ops, V.ptr, n, m, Vt.ptr, Gm, Rinv, st_dev, &h_status, s);
        }
        if (st != IPT_CUDA_SUCCESS) {
            // IPT block numerically rank deficient (e.g. a diverged column):
            // restart from the unit vectors of the target positions.
            IPTGB_CHECK(launch_set_identity(Vt.ptr, n, m, s));
        }
        std::swap(V.ptr, Vt.ptr);
    }

    // ---- 3. Rayleigh-Ritz ---------------------------------------------------
    // The projection is kept incrementally: appending c columns at m0 costs
    // one (m0+c) x c Gram block instead of the full m x m one.
    auto project_new = [&](int m0, int c) -> int {
        IPTGB_CHECK(ops.gram(V.ptr, n, m0 + c, AV.ptr + (size_t)m0 * n, n, c, n, Gm, m0 + c));
        return ops.proj_insert(Gm, m0, c, Tf, maxb);
    };
    IPTGB_CHECK(in.apply->apply(V.ptr, m, AV.ptr));
    rep->fp64_matvecs += m;
    IPTGB_CHECK(project_new(0, m));
    auto rayleigh_ritz = [&]() -> int {
        IPTGB_CHECK(ops.proj_compact(Tf, maxb, m, Tm));
        IPTGB_CHECK(ops.symmetric_eig(Tm, m, theta, Zm, st_dev));
        IPTGB_CHECK(ops.tall_gemm(V.ptr, n, Zm, m, Xr.ptr, n, n, m, k));
        IPTGB_CHECK(ops.tall_gemm(AV.ptr, n, Zm, m, AXr.ptr, n, n, m, k));
        IPTGB_CHECK(ops.residuals(Xr.ptr, AXr.ptr, theta, n, k, n, in.hnorm, R.ptr, rnorm, scaled));
        IPTGB_CUDA(cudaMemcpyAsync(h_scaled.data(), scaled, (size_t)k * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaMemcpyAsync(h_theta.data(), theta, (size_t)m * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        IPTGB_CUDA(cudaStreamSynchronize(s));
        if (in.orth != nullptr) {
            if (!raw_basis_pending) {
                IPTGB_CHECK(orth_figure(ops, V.ptr, n, m, Gm, s, &basis_now));
            }
            raw_basis_pending = false;
            IPTGB_CHECK(orth_figure(ops, Xr.ptr, n, k, Gm, s, &ritz_now));
        }
        return IPT_CUDA_SUCCESS;
    };
    IPTGB_CHECK(rayleigh_ritz());
    IPTGB_CUDA(cudaEventRecord(ev.e[2], s));

    auto max_res = [&]() -> double {
        double mx = 0.0;
        for (int j = 0; j < k; ++j) {
            const double r = h_scaled[(size_t)j];
            if (!isfinite(r)) return (double)INFINITY;
            mx = std::max(mx, r);
        }
        return mx;
    };
    double best = INFINITY;
    auto note_best = [&]() -> int {
        const double mx = max_res();
        if (mx < best) {
            best = mx;
            IPTGB_CUDA(cudaMemcpyAsync(Xbest.ptr, Xr.ptr, (size_t)n * k * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s));
            IPTGB_CUDA(cudaMemcpyAsync(theta_best, theta, (size_t)k * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s));
            basis_best = basis_now;
            ritz_best = ritz_now;
        }
        return IPT_CUDA_SUCCESS;
    };
    IPTGB_CHECK(note_best());

    // ---- 4. Davidson ----------------------------------------------------------
    int steps = 0;
    int restarts = 0;
    bool learned_on = true;
    int learned_rejects = 0;
    double plain_log_drop = 0.0;
    int plain_drops = 0;
    const double forced_accept = env_double("IPT_GB300_MLP_ACCEPT", 0.0);
    const int restart_keep = env_int("IPT_GB300_RESTART_KEEP", in.restart_keep);
    auto required_drop = [&]() -> double {
        if (forced_accept > 0.0) return forced_accept;
        const double expect =
            plain_drops > 0 ? exp(plain_log_drop / plain_drops) : kPlainDropPrior;
        return std::min(kLearnedDrop, expect);
    };
    while (best > tol && steps < opt.davidson_maxsteps) {
        // pairs that still need a correction (ipt_cuda.cu:774-797)
        int nsel = 0;
        for (int j = 0; j < k; ++j) {
            const double r = h_scaled[(size_t)j];
            if (!isfinite(r) || r > tol) {
                h_sel[(size_t)nsel++] = j;
            }
        }
        if (nsel == 0) {
            break;
        }
        // thick restart: keep the lowest Ritz vectors so the new block fits,
        // at most restart_keep of them when that is set
        if (m + nsel > maxb) {
            const int room = restart_keep > 0 ? std::min(restart_keep, maxb - nsel) : maxb - nsel;
            const int kr = std::max(k, std::min(m, room));
            IPTGB_CHECK(ops.tall_gemm(V.ptr, n, Zm, m, Vt.ptr, n, n, m, kr));
            IPTGB_CHECK(ops.tall_gemm(AV.ptr, n, Zm, m, AVt.ptr, n, n, m, kr));
            std::swap(V.ptr, Vt.ptr);
            std::swap(AV.ptr, AVt.ptr);
            m = kr;
            IPTGB_CHECK(ops.proj_diag(theta, m, Tf, maxb));
            ++restarts;
            if (m + nsel > maxb) {
                nsel = maxb - m;
            }
        }
        if (nsel <= 0) {
            break;
        }
        // clip scale: eps^(2/3) * max(1, ||H||, max|theta|) (ipt_cuda.cu:3389-3403)
        double scale = std::max(1.0, fabs(in.hnorm));
        for (int j = 0; j < k; ++j) {
            if (isfinite(h_theta[(size_t)j])) scale = std::max(scale, fabs(h_theta[(size_t)j]));
        }
        const double clip = pow(2.220446049250313e-16, 2.0 / 3.0) * scale;
        IPTGB_CUDA(cudaMemcpyAsync(sel, h_sel.data(), (size_t)nsel * sizeof(int),
                                   cudaMemcpyHostToDevice, s));
        // A learned step is judged by the FP64 residual: unless the largest
        // scaled residual drops by at least kLearnedDrop, the appended
        // directions are discarded, the previous Rayleigh-Ritz state is
        // restored and the step is redone with the plain diagonal
        // correction.  Two rejections in a row switch the learned correction
        // off for the rest of the solve.
        bool stop = false;
        for (int attempt = 0; attempt < 2; ++attempt) {
            const bool use_learned = attempt == 0 && in.learned != nullptr && learned_on;
            double *T = Vt.ptr;  // n x nsel scratch
            if (in.learned != nullptr && (use_learned || !in.learned->learned())) {
                CorrectionArgs ca;
                ca.apply = in.precond_apply != nullptr ? in.precond_apply : in.apply;
                ca.V = V.ptr;
                ca.m = m;
                ca.R = R.ptr;
                ca.X = Xr.ptr;
                ca.d = in.d;
                ca.theta = theta;
                ca.rnorm = rnorm;
                ca.sel = sel;
                ca.nsel = nsel;
                ca.n = n;
                ca.clip = clip;
                IPTGB_CHECK(in.learned->correct(ca, T));
                rep->precond_matvecs += nsel;
            } else {
                IPTGB_CHECK(ops.diag_correction(R.ptr, in.d, theta, sel, nsel, n, clip, T));
            }
            const bool judged = use_learned && in.learned->learned();
            // CGS2 against the basis, then drop numerically dependent directions
            IPTGB_CHECK(ops.column_norms(T, n, n, nsel, cnorm0));
            for (int pass = 0; pass < 2; ++pass) {
                IPTGB_CHECK(ops.gram(V.ptr, n, m, T, n, nsel, n, Gm, m));
                IPTGB_CHECK(ops.tall_gemm(V.ptr, n, Gm, m, T, n, n, m, nsel, -1.0, 1.0));
            }
            IPTGB_CHECK(ops.column_norms(T, n, n, nsel, cnorm1));
            IPTGB_CUDA(cudaMemcpyAsync(h_c0.data(), cnorm0, (size_t)nsel * sizeof(double),
                                       cudaMemcpyDeviceToHost, s));
            IPTGB_CUDA(cudaMemcpyAsync(h_c1.data(), cnorm1, (size_t)nsel * sizeof(double),
                                       cudaMemcpyDeviceToHost, s));
            IPTGB_CUDA(cudaStreamSynchronize(s));
            std::vector<int> keep;
            std::vector<double> inv;
            for (int c = 0; c < nsel; ++c) {
                const double a = h_c0[(size_t)c], b = h_c1[(size_t)c];
                if (isfinite(a) && isfinite(b) && b > 1e-10 * a && b > 1e-300) {
                    keep.push_back(c);
                    inv.push_back(1.0 / b);
                }
            }
            ++steps;
            auto reject_learned = [&]() {
                ++rep->mlp_steps_rejected;
                if (++learned_rejects >= 2) learned_on = false;
            };
            if (keep.empty()) {
                if (judged) {
                    reject_learned();
                    continue;
                }
                stop = true;
                break;
            }
            const int c = (int)keep.size();
            // normalised kept columns -> V[:, m:m+c] (via the sel/norm scratch);
            // sel is re-uploaded for a retry below
            IPTGB_CUDA(cudaMemcpyAsync(cnorm1, inv.data(), (size_t)c * sizeof(double),
                                       cudaMemcpyHostToDevice, s));
            int *keep_dev = st_dev + 4;
            IPTGB_CUDA(cudaMemcpyAsync(keep_dev, keep.data(), (size_t)c * sizeof(int),
                                       cudaMemcpyHostToDevice, s));
            double *Vnew = V.ptr + (size_t)m * n;
            IPTGB_CHECK(ops.gather_columns(T, n, keep_dev, cnorm1, n, c, Vnew, n));
            // CholQR of the new block, one more projection pass, CholQR again
            int st = cholqr(ops, Vnew, n, c, T, Gm, Rinv, st_dev, &h_status, s);
            if (st == IPT_CUDA_SUCCESS) {
                IPTGB_CHECK(ops.gram(V.ptr, n, m, T, n, c, n, Gm, m));
                IPTGB_CHECK(ops.tall_gemm(V.ptr, n, Gm, m, T, n, n, m, c, -1.0, 1.0));
                st = cholqr(ops, T, n, c, Vnew, Gm, Rinv, st_dev, &h_status, s);
            }
            if (st != IPT_CUDA_SUCCESS) {
                if (judged) {
                    reject_learned();
                    continue;
                }
                stop = true;
                break;
            }
            IPTGB_CHECK(in.apply->apply(Vnew, c, AV.ptr + (size_t)m * n));
            rep->fp64_matvecs += c;
            IPTGB_CHECK(project_new(m, c));
            const double before = max_res();
            m += c;
            IPTGB_CHECK(rayleigh_ritz());
            const double after = max_res();
            if (!judged && isfinite(before) && before > 0.0 && isfinite(after) && after > 0.0) {
                plain_log_drop += log(std::min(1.0, after / before));
                ++plain_drops;
            }
            if (judged) {
                if (!(after < required_drop() * before)) {
                    // reject: restore the basis and the previous Ritz state
                    reject_learned();
                    m -= c;
                    IPTGB_CHECK(rayleigh_ritz());
                    continue;
                }
                ++rep->mlp_steps_accepted;
                learned_rejects = 0;
            }
            IPTGB_CHECK(note_best());
            break;
        }
        if (stop) {
            break;
        }
    }
    IPTGB_CUDA(cudaEventRecord(ev.e[3], s));

    IPTGB_CUDA(cudaMemcpyAsync(X_out, Xbest.ptr, (size_t)n * k * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    IPTGB_CUDA(cudaMemcpyAsync(values_out, theta_best, (size_t)k * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    IPTGB_CUDA(cudaEventRecord(ev.e[4], s));
    IPTGB_CUDA(cudaEventSynchronize(ev.e[4]));
    ops.release();
    if (in.orth != nullptr) {
        in.orth->basis = basis_best;
        in.orth->ritz = ritz_best;
    }
    rep->davidson_steps = steps;
    rep->restarts = restarts;
    rep->basis_cols = m;
    rep->max_scaled_residual = best;
    rep->converged = best <= tol ? 1 : 0;
    rep->ipt_ms = elapsed_ms(ev.e[0], ev.e[1]);
    rep->rayleigh_ritz_ms = elapsed_ms(ev.e[1], ev.e[2]);
    rep->davidson_ms = elapsed_ms(ev.e[2], ev.e[3]);
    rep->total_ms = elapsed_ms(ev.e[0], ev.e[4]);
    return IPT_CUDA_SUCCESS;
}

}  // namespace iptgb
