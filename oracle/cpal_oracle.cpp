/*
 * cpal_oracle.cpp -- CPU restatement of the CP_AL (LP) restarted reflected
 * Halpern augmented primal-dual solver.  TEST INFRASTRUCTURE ONLY: it is the
 * checker of the CUDA library, never part of the product path.  Only tests/,
 * __graft_entry__.smoke() and bench.py (its CPU-baseline legs) load it.
 *
 * It follows the reference's operation order in plain FP64 loops:
 *   - setup            LP/CP_AL/src/solver.cu:1795-2273
 *   - equilibration    LP/CP_AL/src/preconditioner.cu:128-160, 273-475, 477-736
 *   - power iteration  LP/CP_AL/src/utils.cu:87-228 (std::mt19937(1) start)
 *   - step schedule    LP/CP_AL/src/solver.cu:3103-3164, 3538-3609
 *   - iteration        LP/CP_AL/src/solver.cu:2340-2479 (kernels), 2523-2661 (op order)
 *   - block loop       LP/CP_AL/src/solver.cu:1270-1736
 *   - fixed point err  LP/CP_AL/src/solver.cu:3611-3686
 *   - residual/KKT     LP/CP_AL/src/utils.cu:649-682, 812-917
 *   - termination      LP/CP_AL/src/utils.cu:275-317
 *   - restart rule     LP/CP_AL/src/utils.cu:319-359
 *   - restart / PID    LP/CP_AL/src/solver.cu:2821-3101
 *   - result           LP/CP_AL/src/solver.cu:1768-1793, 2481-2500, 3828-3909
 * The third-party reductions of the reference (cuBLAS Dnrm2/Ddot, CUB sums,
 * cuSPARSE CSR SpMV) are restated as sequential sums.
 *
 * Built with -ffp-contract=off so x86 and Arm hosts produce the same bits.
 * With oracle_set_threads(n > 1) the vector loops use OpenMP (timing only:
 * the sums then depend on the thread count).
 */
#include "../include/cp_al_gb300.h"
#include "../include/cp_al_types.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

int g_threads = 1;
int g_polish_status[2] = {-1, -1};
int g_restart_targets[3] = {0, 0, 0};
int g_controllers[4] = {-1, 0, 0, 0}; /* pulse start iteration, pulse gate, sigma trigger and dynamic evaluation iterations */

struct Csr {
    int nr = 0, nc = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
};

/* Column-major copy of A (rows of A^T ordered by increasing row of A), the
 * ordering cusparseCsr2cscEx2 produces (LP/CP_AL/src/solver.cu:1859-1890). */
Csr transpose(const Csr &A) {
    Csr T;
    T.nr = A.nc;
    T.nc = A.nr;
    T.rp.assign(A.nc + 1, 0);
    T.ci.resize(A.v.size());
    T.v.resize(A.v.size());
    for (size_t k = 0; k < A.ci.size(); ++k) T.rp[A.ci[k] + 1]++;
    for (int j = 0; j < A.nc; ++j) T.rp[j + 1] += T.rp[j];
    std::vector<int> next(T.rp.begin(), T.rp.end() - 1);
    for (int i = 0; i < A.nr; ++i)
        for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            int p = next[A.ci[k]]++;
            T.ci[p] = i;
            T.v[p] = A.v[k];
        }
    return T;
}

void spmv(const Csr &M, const double *x, double *y) {
#pragma omp parallel for schedule(static) if (g_threads > 1) num_threads(g_threads)
    for (int i = 0; i < M.nr; ++i) {
        double s = 0.0;
        for (int k = M.rp[i]; k < M.rp[i + 1]; ++k) s += M.v[k] * x[M.ci[k]];
        y[i] = s;
    }
}

double dot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0.0;
    const int n = (int)a.size();
#pragma omp parallel for reduction(+ : s) schedule(static) if (g_threads > 1) num_threads(g_threads)
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

double nrm2(const std::vector<double> &a) { return std::sqrt(dot(a, a)); }

double amax(const std::vector<double> &a) {
    double m = 0.0;
    for (double v : a) m = std::fmax(m, std::fabs(v));
    return m;
}

double clampd(double v, double lo, double hi) { return std::fmax(lo, std::fmin(v, hi)); }

struct Solver {
    const cp_al_parameters_t *P;
    cp_al_gb300_options_t O;
    int n = 0, m = 0;
    Csr A, At;
    std::vector<double> c, vlb, vub, clb, cub, clb_fin, cub_fin;
    std::vector<double> x0, x, xh, xbar, y0, y, yh, ybar, dprod, pprod, lam;
    std::vector<double> dcum, rcum, dx, dy, rp, rd, contrib;
    double cbr = 1.0, ovr = 1.0, obj_const = 0.0;
    double obj_norm = 0.0, bnd_norm = 0.0;

    /* scalar state (internal_types.h cp_al_solver_state_t) */
    double step = 0.0, pw = 1.0, al_lambda = 0.0, beta = 0.0, lambda_est = 1.0;
    bool sigma_mode = false, sigma_adaptive = false;
    double sigma = 0, sigma_base = 0, sigma_min = 0, sigma_max = 0, sigma_best = 0, sigma_esum = 0, sigma_last = 0;
    double lambda_param = 0;
    double pw_esum = 0, pw_last = 0, best_pw = 1, best_gap = INFINITY;
    int total = 0, inner = 0;
    double fp = 0, fp0 = 0, fp_last = INFINITY;
    double abs_p = 0, abs_d = 0, rel_p = 0, rel_d = 0, pobj = 0, dobj = 0, gap = 0, rel_gap = 0;
    termination_reason_t reason = TERMINATION_REASON_UNSPECIFIED;
    int power_iters = 0, restarts = 0;
    int restarts_to[3] = {0, 0, 0}; /* restarts by target: current point, reflected, plain Halpern */
    /* benchmark controllers (LP/CP_AL/src/solver.cu:198-272 state): the
     * alpha pulse's phase (0 idle, 1 positive block, 2 over) and gate (0 not
     * evaluated, 1 passed, 2 rejected), the epoch being measured and the last
     * two zero-alpha epochs; the sigma trigger's iteration */
    int pulse_phase = 0, pulse_gate = 0, pulse_start = -1;
    bool epoch_valid = false;
    int epoch_total = 0, hist_count = 0;
    int hist_k[2] = {0, 0};
    double hist_rate[2] = {0.0, 0.0};
    double epoch_p = 0, epoch_d = 0, epoch_g = 0;
    int trigger_iter = 0;
    /* the dynamic evaluation frequency (solver.cu:1229-1255): the next
     * block's length, whether the switch to short blocks was taken and at
     * which iteration */
    int F_cur = 0, dyn_iter = 0;
    bool dyn_latched = false, cr_early_stopped = false;
    struct Dyn {
        bool on = false, resid = false;
        int fast = 0, min_iters = 0, boot = 0, after_iters = -1;
        double after_sec = -1.0, small = 0, large = 0, ratio = 0;
    } dyn;
    void dyn_setup() {
        const int F = P->termination_evaluation_frequency;
        dyn.fast = std::min(std::max(O.dynamic_eval_fast, 3), F);
        dyn.resid = O.dynamic_eval != 0;
        dyn.after_sec = O.dynamic_eval_after_sec;
        dyn.after_iters = O.dynamic_eval_after_iters;
        dyn.on = (dyn.resid || dyn.after_sec > 0.0 || dyn.after_iters > 0) && dyn.fast < F;
        dyn.min_iters = std::max(O.dynamic_eval_min_iters > 0 ? O.dynamic_eval_min_iters : F, F);
        dyn.small = O.dynamic_eval_small_res;
        dyn.large = O.dynamic_eval_large_res;
        dyn.ratio = O.dynamic_eval_ratio;
        dyn.boot = std::max(O.dynamic_eval_bootstrap_iters, 0);
        F_cur = (dyn.on && dyn.boot > 0) ? dyn.fast : F;
    }
    /* solver.cu:1529-1583, after an evaluation */
    void dyn_update(double elapsed) {
        if (!dyn.on || sigma_mode) return;
        if (!(total >= dyn.min_iters || (dyn.boot > 0 && total >= dyn.boot))) return;
        const double rpr = std::fmax(rel_p, 1e-300), rdr = std::fmax(rel_d, 1e-300);
        const double lo = std::fmin(rpr, rdr), hi = std::fmax(rpr, rdr);
        const bool one_sided = lo <= dyn.small && hi >= dyn.large;
        const bool lag = hi / lo >= dyn.ratio && hi >= dyn.large;
        const bool tgate = dyn.after_sec > 0.0 && !cr_early_stopped && elapsed >= dyn.after_sec;
        const bool igate = dyn.after_iters > 0 && !cr_early_stopped && total >= dyn.after_iters;
        if (tgate || igate || (dyn.resid && (one_sided || lag))) {
            if (!dyn_latched) dyn_iter = total;
            dyn_latched = true;
            F_cur = dyn.fast;
        } else if (!dyn_latched && dyn.boot > 0 && F_cur == dyn.fast && total >= dyn.boot) {
            F_cur = P->termination_evaluation_frequency;
        }
    }

    static double metric(double v) { return std::fmax(std::fabs(v), 1e-300); } /* solver.cu:415-418 */
    static double log_rate(double a, double b, int k) {                        /* solver.cu:420-428 */
        if (k <= 0 || !std::isfinite(a) || !std::isfinite(b)) return NAN;
        const double r = std::log(metric(a) / metric(b)) / (double)k;
        return std::isfinite(r) ? r : NAN;
    }
    /* solver.cu:616-678, at a restart before the restart itself */
    void record_epoch() {
        if (!epoch_valid || al_lambda > 0.0) return;
        const int k = total - epoch_total;
        const double fr = log_rate(fp0, fp, k);
        const double pr = log_rate(epoch_p, rel_p, k), dr = log_rate(epoch_d, rel_d, k);
        const double gr = log_rate(epoch_g, rel_gap, k);
        const double kr = log_rate(std::fmax(epoch_p, std::fmax(epoch_d, epoch_g)),
                                   std::fmax(metric(rel_p), std::fmax(metric(rel_d), metric(rel_gap))), k);
        const bool ok = k > 0 && std::isfinite(fr) && std::isfinite(pr) && std::isfinite(dr) && std::isfinite(gr) &&
                        std::isfinite(kr);
        if (!ok) return;
        if (hist_count < 2) {
            hist_k[hist_count] = k;
            hist_rate[hist_count] = fr;
            ++hist_count;
        } else {
            hist_k[0] = hist_k[1];
            hist_rate[0] = hist_rate[1];
            hist_k[1] = k;
            hist_rate[1] = fr;
        }
    }
    void epoch_start() { /* solver.cu:605-614 */
        epoch_valid = true;
        epoch_total = total;
        epoch_p = metric(rel_p);
        epoch_d = metric(rel_d);
        epoch_g = metric(rel_gap);
    }
    /* solver.cu:899-988: evaluated once, after a restart */
    void pulse_gate_eval(int F, int limit) {
        if (!O.alpha_direct_pulse || pulse_gate || pulse_phase || hist_count < 2 || total < 10000 || F != 200) return;
        if (limit - total < 400) return;
        for (int i = 0; i < 2; ++i)
            if (hist_k[i] <= 0 || !std::isfinite(hist_rate[i])) return;
        pulse_gate = O.pulse_force ? 1 : 2;
        if (!O.pulse_force) return;
        pulse_phase = 1;
        pulse_start = total;
        sigma_mode = false;
        al_lambda = 0.002;
        refresh_step_schedule();
    }

    double kp() const { return std::isnan(O.sigma_kp) ? P->restart_params.k_p : O.sigma_kp; }

    /* ---------------- equilibration (preconditioner.cu) ---------------- */
    void scale_problem(const std::vector<double> &r, const std::vector<double> &d) {
        /* preconditioner.cu:128-160 + kernels 476-530 */
        for (int j = 0; j < n; ++j) {
            double dj = d[j], inv = 1.0 / d[j];
            c[j] *= inv;
            vlb[j] *= dj;
            vub[j] *= dj;
            x0[j] *= dj;
        }
        for (int i = 0; i < m; ++i) {
            double inv = 1.0 / r[i], ei = r[i];
            clb[i] *= inv;
            cub[i] *= inv;
            y0[i] *= ei;
        }
        for (int i = 0; i < m; ++i)
            for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) A.v[k] *= (1.0 / d[A.ci[k]]) * (1.0 / r[i]);
        for (int j = 0; j < n; ++j)
            for (int k = At.rp[j]; k < At.rp[j + 1]; ++k) At.v[k] *= (1.0 / d[j]) * (1.0 / r[At.ci[k]]);
    }
    /* preconditioner.cu:128-160 + kernels 476-530 with the inverses given
     * (the Curtis-Reid pass hands over f, not 1/(1/f)) */
    void scale_problem_inv(const std::vector<double> &r, const std::vector<double> &rinv, const std::vector<double> &d,
                           const std::vector<double> &dinv) {
        for (int j = 0; j < n; ++j) {
            c[j] *= dinv[j];
            vlb[j] *= d[j];
            vub[j] *= d[j];
            x0[j] *= d[j];
        }
        for (int i = 0; i < m; ++i) {
            clb[i] *= rinv[i];
            cub[i] *= rinv[i];
            y0[i] *= r[i];
        }
        for (int i = 0; i < m; ++i)
            for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) A.v[k] *= dinv[A.ci[k]] * rinv[i];
        for (int j = 0; j < n; ++j)
            for (int k = At.rp[j]; k < At.rp[j + 1]; ++k) At.v[k] *= dinv[j] * rinv[At.ci[k]];
    }
    /* Curtis-Reid (preconditioner.cu:162-270, 553-624): alternating passes
     * set each row's log scale to the mean of -log|a| - (column log scale)
     * over its nonzeros, then each column's from the rows; the scales are
     * 1 / clamp(exp(log), 1e-30, 1e30).  With early stop (20 passes) the
     * passes end after the fifth when the largest change of a scaled entry's
     * log, |delta_row + delta_col|, is at most the threshold. */
    int cr_passes = 0;
    void curtis_reid() {
        const int iters = O.cr_iterations;
        const bool early = O.cr_early_stop != 0 && iters == 20;
        std::vector<double> lr(m, 0.0), lc(n, 0.0), dr(m, 0.0), dc(n, 0.0);
        auto update = [](const Csr &M, const std::vector<double> &other, std::vector<double> &ls,
                         std::vector<double> &delta) {
            for (int i = 0; i < M.nr; ++i) {
                const int k0 = M.rp[i], k1 = M.rp[i + 1];
                double acc = 0.0;
                for (int k = k0; k < k1; ++k) {
                    double v = std::fabs(M.v[k]);
                    if (!std::isfinite(v) || v < 1e-300) v = 1e-300;
                    acc += -std::log(v) - other[M.ci[k]];
                }
                const double u = k1 > k0 ? acc / (double)(k1 - k0) : 0.0;
                delta[i] = u - ls[i];
                ls[i] = u;
            }
        };
        for (int it = 0; it < iters; ++it) {
            update(A, lc, lr, dr);
            update(At, lr, lc, dc);
            cr_passes = it + 1;
            if (early && it + 1 == 5) {
                /* a maximum over no rows is the lowest double: below any threshold */
                if (m == 0) break;
                double mx = 0.0;
                for (int i = 0; i < m; ++i)
                    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) {
                        const double e = std::fabs(dr[i] + dc[A.ci[k]]);
                        if (std::isfinite(e) && e > mx) mx = e;
                    }
                if (mx <= O.cr_early_stop_threshold) break;
            }
        }
        cr_early_stopped = early && cr_passes < iters; /* preconditioner.cu:246 */
        std::vector<double> rinv(m), dinv(n);
        for (int i = 0; i < m; ++i) {
            const double f = std::fmin(std::fmax(std::exp(lr[i]), 1e-30), 1e30);
            lr[i] = 1.0 / f;
            rinv[i] = f;
            rcum[i] *= lr[i];
        }
        for (int j = 0; j < n; ++j) {
            const double f = std::fmin(std::fmax(std::exp(lc[j]), 1e-30), 1e30);
            lc[j] = 1.0 / f;
            dinv[j] = f;
            dcum[j] *= lc[j];
        }
        scale_problem_inv(lr, rinv, lc, dinv);
    }
    static void clamp_sqrt_accum(std::vector<double> &s, std::vector<double> &cum) {
        /* preconditioner.cu:653-667 */
        for (size_t t = 0; t < s.size(); ++t) {
            double v = s[t];
            double q = (v < 1e-12) ? 1.0 : std::sqrt(v);
            cum[t] *= q;
            s[t] = q;
        }
    }
    static void row_absmax(const Csr &M, std::vector<double> &out) {
        /* preconditioner.cu:532-550 */
        for (int i = 0; i < M.nr; ++i) {
            double mx = 0.0;
            for (int k = M.rp[i]; k < M.rp[i + 1]; ++k) {
                double v = std::fabs(M.v[k]);
                if (!std::isfinite(v)) v = 0.0;
                if (v > mx) mx = v;
            }
            out[i] = mx;
        }
    }
    static double pow_fast(double v, double p) {
        if (p == 2.0) return v * v;
        if (p == 1.0) return v;
        if (p == 0.5) return std::sqrt(v);
        return std::pow(v, p);
    }
    static void row_powsum(const Csr &M, double deg, std::vector<double> &out) {
        /* preconditioner.cu:634-651 */
        for (int i = 0; i < M.nr; ++i) {
            double acc = 0.0;
            for (int k = M.rp[i]; k < M.rp[i + 1]; ++k) {
                double v = std::fabs(M.v[k]);
                if (!std::isfinite(v)) v = 0.0;
                acc += pow_fast(v, deg);
            }
            out[i] = acc;
        }
    }
    void rescale() {
        /* preconditioner.cu:379-475 */
        std::vector<double> r(m), d(n);
        dcum.assign(n, 1.0);
        rcum.assign(m, 1.0);
        if (O.cr_iterations > 0) curtis_reid(); /* 403-425: before Ruiz */
        for (int it = 0; it < P->l_inf_ruiz_iterations; ++it) { /* 273-299 */
            row_absmax(A, r);
            clamp_sqrt_accum(r, rcum);
            row_absmax(At, d);
            clamp_sqrt_accum(d, dcum);
            scale_problem(r, d);
        }
        if (P->has_pock_chambolle_alpha) { /* 301-327 */
            row_powsum(A, P->pock_chambolle_alpha, r);
            clamp_sqrt_accum(r, rcum);
            row_powsum(At, 2.0 - P->pock_chambolle_alpha, d);
            clamp_sqrt_accum(d, dcum);
            scale_problem(r, d);
        }
        cbr = 1.0;
        ovr = 1.0;
        if (P->bound_objective_rescaling) { /* 329-377, 669-691 */
            double s = 0.0;
            for (int i = 0; i < m; ++i) {
                double L = clb[i], U = cub[i];
                bool fL = std::isfinite(L), fU = std::isfinite(U);
                double acc = 0.0;
                if (fL && (!fU || std::fabs(L - U) > 1e-12)) acc += L * L;
                if (fU) acc += U * U;
                s += acc;
            }
            double bnd = std::sqrt(s);
            double objn = nrm2(c);
            cbr = 1.0 / (bnd + 1.0);
            ovr = 1.0 / (objn + 1.0);
            for (int i = 0; i < m; ++i) {
                clb[i] *= cbr;
                cub[i] *= cbr;
                y0[i] *= ovr;
            }
            for (int j = 0; j < n; ++j) {
                vlb[j] *= cbr;
                vub[j] *= cbr;
                c[j] *= ovr;
                x0[j] *= cbr;
            }
        }
    }

    /* ---------------- power iteration (utils.cu:87-228) ---------------- */
    double max_singular_value() {
        std::mt19937 gen(1);
        std::normal_distribution<double> dist(0.0, 1.0);
        std::vector<double> v(m), nv(m), dp(n);
        for (int i = 0; i < m; ++i) v[i] = dist(gen);
        double s2 = 1.0;
        for (int it = 0; it < P->sv_max_iter; ++it) {
            power_iters = it + 1;
            nv = v;
            double inv = 1.0 / nrm2(nv);
            for (int i = 0; i < m; ++i) nv[i] = inv * nv[i];
            spmv(At, nv.data(), dp.data());
            spmv(A, dp.data(), v.data());
            s2 = dot(nv, v);
            for (int i = 0; i < m; ++i) nv[i] = (-s2 * nv[i]) + v[i];
            if (nrm2(nv) < P->sv_tol) break;
        }
        return std::sqrt(s2);
    }

    /* ---------------- step schedule (solver.cu:3103-3164) ---------------- */
    void refresh_step_schedule() {
        const double margin = O.step_margin;
        if (sigma_mode) {
            const double s = std::fmax(sigma, 0.0);
            if (s <= 0.0) {
                beta = 0.0;
                lambda_param = 0.0;
                step = std::sqrt(std::fmax(margin / std::fmax(lambda_est, 1e-12), 1e-24));
                al_lambda = 0.0;
                return;
            }
            if (!std::isfinite(lambda_param) || lambda_param <= 0.0) {
                lambda_param = O.lambda_param_set ? O.lambda_param : O.lambda_factor * std::fmax(lambda_est, 1e-12);
            }
            lambda_param = std::fmax(lambda_param, (2.0 + 1e-12) * std::fmax(lambda_est, 1e-12));
            const double tau = 1.0 / (s * lambda_param);
            const double rho = s;
            beta = s;
            step = std::sqrt(std::fmax(tau * rho, 1e-24));
            pw = std::sqrt(std::fmax(rho / tau, 1e-24));
            al_lambda = 0.0;
            return;
        }
        al_lambda = std::fmin(std::fmax(al_lambda, 0.0), 0.95);
        const double eta_sq = margin * (1.0 - al_lambda) / std::fmax(lambda_est, 1e-12);
        step = std::sqrt(std::fmax(eta_sq, 1e-24));
        const double dual_step = step * std::fmax(pw, 1e-12);
        beta = dual_step * al_lambda / std::fmax(1.0 - al_lambda, 1e-12);
    }
    void initialize_sigma_parameters() {
        lambda_param = O.lambda_param_set ? O.lambda_param : O.lambda_factor * std::fmax(lambda_est, 1e-12);
        lambda_param = std::fmax(lambda_param, (2.0 + 1e-12) * std::fmax(lambda_est, 1e-12));
        sigma_base = 1.0 / std::sqrt(std::fmax(lambda_param, 1e-16));
        sigma_min = O.sigma_min_factor * sigma_base;
        sigma_max = O.sigma_max_factor * sigma_base;
        sigma = O.sigma_set ? O.sigma : O.sigma_init_factor * sigma_base;
        sigma = std::fmin(std::fmax(sigma, sigma_min), sigma_max);
        sigma_best = sigma;
        sigma_esum = 0.0;
        sigma_last = 0.0;
        sigma_adaptive = O.sigma_adaptive != 0;
        sigma_mode = true;
    }
    void initialize_step_size_and_primal_weight() { /* solver.cu:3538-3609 */
        lambda_est = (A.v.empty()) ? 1.0 : [&] {
            double s = max_singular_value();
            return s * s;
        }();
        pw = P->bound_objective_rescaling ? 1.0 : (obj_norm + 1.0) / (bnd_norm + 1.0);
        sigma_mode = O.sigma_mode != 0;
        if (sigma_mode) initialize_sigma_parameters();
        al_lambda = O.al_lambda;
        refresh_step_schedule();
        best_pw = pw;
    }

    /* ---------------- one iteration (solver.cu:2523-2661) ---------------- */
    void primal(int koff, bool major) {
        const double tau = step / pw;
        const double r = P->reflection_coefficient;
        const double *u = y.data();
        if (beta > 0.0) { /* 2528-2554 + kernel 2459-2479 */
            spmv(A, x.data(), pprod.data());
            for (int i = 0; i < m; ++i) {
                double zz = clampd(pprod[i] - y[i] / beta, clb[i], cub[i]);
                ybar[i] = y[i] - beta * (pprod[i] - zz);
            }
            u = ybar.data();
        }
        spmv(At, u, dprod.data());
        const int k = inner + koff;
        const double w = (double)k / (double)(k + 1);
#pragma omp parallel for schedule(static) if (g_threads > 1) num_threads(g_threads)
        for (int j = 0; j < n; ++j) { /* kernels 2340-2397 */
            double t = x[j] - tau * (c[j] - dprod[j]);
            double proj = std::fmax(vlb[j], std::fmin(t, vub[j]));
            if (major) {
                xh[j] = proj;
                lam[j] = (proj - t) / tau;
            }
            xbar[j] = 2.0 * proj - x[j];
            double refl = r * xbar[j] + (1.0 - r) * x[j];
            x[j] = w * refl + (1.0 - w) * x0[j];
        }
    }
    void dual(int koff, bool major) {
        const double rho = step * pw;
        const double r = P->reflection_coefficient;
        spmv(A, xbar.data(), pprod.data());
        const int k = inner + koff;
        const double w = (double)k / (double)(k + 1);
        const double prox = rho + beta;
#pragma omp parallel for schedule(static) if (g_threads > 1) num_threads(g_threads)
        for (int i = 0; i < m; ++i) { /* kernels 2399-2457 */
            double zb = std::fmax(clb[i], std::fmin(pprod[i] - y[i] / prox, cub[i]));
            double yn = y[i] - rho * (pprod[i] - zb);
            double refl;
            if (major) {
                yh[i] = yn;
                ybar[i] = 2.0 * yn - y[i];
                refl = r * ybar[i] + (1.0 - r) * y[i];
            } else {
                refl = r * (2.0 * yn - y[i]) + (1.0 - r) * y[i];
            }
            y[i] = w * refl + (1.0 - w) * y0[i];
        }
    }

    /* ---------------- evaluation ---------------- */
    void fixed_point_error() { /* solver.cu:3611-3686 */
        for (int j = 0; j < n; ++j) dx[j] = xbar[j] - xh[j];
        for (int i = 0; i < m; ++i) dy[i] = ybar[i] - yh[i];
        spmv(At, dy.data(), dprod.data());
        spmv(A, dx.data(), pprod.data());
        double dn = nrm2(dy), pn = nrm2(dx), axn = nrm2(pprod);
        if (sigma_mode && sigma > 0.0 && lambda_param > 0.0) {
            double val = sigma * (lambda_param * pn * pn - axn * axn) + dn * dn / std::fmax(sigma, 1e-16);
            fp = std::sqrt(std::fmax(val, 0.0));
            return;
        }
        double movement = pn * pn * pw + dn * dn / pw;
        double cross = dot(dprod, dx);
        double interaction = 2 * step * cross;
        double aug = step * beta * axn * axn;
        fp = std::sqrt(std::fmax(movement + interaction - aug, 0.0));
    }
    void compute_residual() { /* utils.cu:812-917 */
        spmv(A, xh.data(), pprod.data());
        spmv(At, yh.data(), dprod.data());
        for (int i = 0; i < m; ++i) {
            double cl = std::fmax(clb[i], std::fmin(pprod[i], cub[i]));
            rp[i] = (pprod[i] - cl) * rcum[i];
            contrib[i] = std::fmax(yh[i], 0.0) * clb_fin[i] + std::fmin(yh[i], 0.0) * cub_fin[i];
        }
        for (int j = 0; j < n; ++j) rd[j] = (c[j] - dprod[j] - lam[j]) * dcum[j];
        if (P->optimality_norm == NORM_TYPE_L_INF) {
            abs_p = amax(rp);
            abs_d = amax(rd);
        } else {
            abs_p = nrm2(rp) / cbr;
            abs_d = nrm2(rd);
        }
        abs_d /= ovr;
        pobj = dot(c, xh) / (cbr * ovr) + obj_const;
        double base = dot(lam, xh);
        double csum = 0.0;
        for (int i = 0; i < m; ++i) csum += contrib[i];
        dobj = (base + csum) / (cbr * ovr) + obj_const;
        rel_p = abs_p / (1.0 + bnd_norm);
        rel_d = abs_d / (1.0 + obj_norm);
        gap = std::fabs(pobj - dobj);
        rel_gap = gap / (1.0 + std::fabs(pobj) + std::fabs(dobj));
    }
    bool should_restart(int F) { /* utils.cu:319-359 */
        const auto &R = P->restart_params;
        const double suff = std::isnan(O.restart_sufficient) ? R.sufficient_reduction_for_restart : O.restart_sufficient;
        const double nec = std::isnan(O.restart_necessary) ? R.necessary_reduction_for_restart : O.restart_necessary;
        const double art = std::isnan(O.restart_artificial) ? R.artificial_restart_threshold : O.restart_artificial;
        bool rs = false;
        if (total == F) {
            rs = true;
        } else if (total > F) {
            if (fp <= suff * fp0) rs = true;
            if (fp <= nec * fp0 && fp > fp_last) rs = true;
            if (inner >= art * total) rs = true;
        }
        fp_last = fp;
        return rs;
    }
    /* solver.cu:2663-2747: fixed-point score of candidate (x^, y^) against a
     * reference point (rx, ry) */
    double restart_delta_score(const std::vector<double> &rx, const std::vector<double> &ry) {
        std::vector<double> ddx(n), ddy(m), dp(n), pp(m);
        for (int j = 0; j < n; ++j) ddx[j] = xh[j] - rx[j];
        for (int i = 0; i < m; ++i) ddy[i] = yh[i] - ry[i];
        spmv(At, ddy.data(), dp.data());
        spmv(A, ddx.data(), pp.data());
        const double pn = nrm2(ddx), dn = nrm2(ddy), axn = nrm2(pp);
        if (sigma_mode && sigma > 0.0 && lambda_param > 0.0) {
            const double val = sigma * (lambda_param * pn * pn - axn * axn) + dn * dn / std::fmax(sigma, 1e-16);
            return std::sqrt(std::fmax(val, 0.0));
        }
        const double movement = pn * pn * pw + dn * dn / pw;
        const double interaction = 2 * step * dot(dp, ddx);
        const double aug = step * beta * axn * axn;
        return std::sqrt(std::fmax(movement + interaction - aug, 0.0));
    }
    /* the plain Halpern point of the last (major) iteration of the block,
     * w x^ + (1 - w) x0 with that iteration's weight (solver.cu:2392) */
    std::vector<double> xhal, yhal;
    void halpern_point() {
        const double w = (double)inner / (double)(inner + 1);
        xhal.resize(n);
        yhal.resize(m);
        for (int j = 0; j < n; ++j) xhal[j] = w * xh[j] + (1.0 - w) * x0[j];
        for (int i = 0; i < m; ++i) yhal[i] = w * yh[i] + (1.0 - w) * y0[i];
    }
    /* solver.cu:2749-2819: target 1 is the reflected Halpern iterate (x, y),
     * target 2 the plain Halpern point (three-point mode); the best score
     * wins when it is within the margin of the current point's (mode 1, 3),
     * or target 1 is taken always (mode 2) */
    int restart_target = 0;
    void choose_restart_candidate(double elapsed) {
        restart_target = 0;
        if (O.restart_select == 0) return;
        if (total < O.restart_select_min_iters || elapsed < O.restart_select_min_time) return;
        const double cur = fp;
        const double avg = restart_delta_score(x, y);
        const bool three = O.restart_select == 3 || O.restart_select_threepoint != 0;
        double hal = INFINITY;
        if (three) {
            halpern_point();
            hal = restart_delta_score(xhal, yhal);
        }
        if (O.restart_select == 2) {
            restart_target = 1;
            fp = avg;
        } else if (std::isfinite(cur)) {
            int best = 0;
            double best_score = cur;
            if (std::isfinite(avg) && avg < best_score) {
                best = 1;
                best_score = avg;
            }
            if (three && std::isfinite(hal) && hal < best_score) {
                best = 2;
                best_score = hal;
            }
            if (best != 0 && best_score <= O.restart_select_margin * cur) {
                restart_target = best;
                fp = best_score;
            }
        }
    }
    void perform_restart() { /* solver.cu:2821-3101 */
        const bool to_current = O.restart_select != 0 && restart_target == 1;
        const bool to_halpern = O.restart_select != 0 && restart_target == 2;
        const std::vector<double> &rx = to_current ? x : to_halpern ? xhal : xh;
        const std::vector<double> &ry = to_current ? y : to_halpern ? yhal : yh;
        std::vector<double> ddx(n), ddy(m);
        for (int j = 0; j < n; ++j) ddx[j] = rx[j] - x0[j];
        for (int i = 0; i < m; ++i) ddy[i] = ry[i] - y0[i];
        const double pd = nrm2(ddx), dd = nrm2(ddy);
        const double ratio = rel_d / std::fmax(rel_p, 1e-300);
        const auto &R = P->restart_params;
        if (sigma_mode) {
            if (sigma_adaptive) {
                std::vector<double> ad(m);
                spmv(A, ddx.data(), ad.data());
                const double axd = nrm2(ad);
                const double dxm = lambda_param * pd * pd - axd * axd;
                if (dd > 1e-16 && dd < 1e12 && dxm > 1e-24 && dxm < 1e24 && std::isfinite(sigma) && sigma > 1e-16 &&
                    ratio > 1e-8 && ratio < 1e8) {
                    const double ism = std::isnan(O.sigma_i_smooth) ? R.i_smooth : O.sigma_i_smooth;
                    const double ki = std::isnan(O.sigma_ki) ? R.k_i : O.sigma_ki;
                    const double kd = std::isnan(O.sigma_kd) ? R.k_d : O.sigma_kd;
                    double err = std::log(std::fmax(dd, 1e-300)) - 0.5 * std::log(std::fmax(dxm, 1e-300)) -
                                 std::log(std::fmax(sigma, 1e-300));
                    double bal = 0.5 * std::log(std::fmax(ratio, 1e-300));
                    bal = std::fmax(-2.0, std::fmin(bal, 2.0));
                    err += O.sigma_balance_gain * bal;
                    sigma_esum = ism * sigma_esum + err;
                    const double de = err - sigma_last;
                    double sr = std::exp(kp() * err + ki * sigma_esum + kd * de);
                    sr = std::fmin(std::fmax(sr, O.sigma_update_min), O.sigma_update_max);
                    sigma *= sr;
                    sigma_last = err;
                } else {
                    sigma = sigma_best;
                    sigma_esum = 0.0;
                    sigma_last = 0.0;
                }
            }
            if (!std::isfinite(sigma) || sigma <= 1e-16) {
                sigma = sigma_best;
                sigma_esum = 0.0;
                sigma_last = 0.0;
            }
            sigma = std::fmin(std::fmax(sigma, sigma_min), sigma_max);
            double g = std::fabs(std::log10(std::fmax(rel_d, 1e-300) / std::fmax(rel_p, 1e-300)));
            if (std::isfinite(g) && g < best_gap) {
                best_gap = g;
                sigma_best = sigma;
            }
            pw_esum = 0.0;
            pw_last = 0.0;
        } else {
            if (pd > 1e-16 && dd > 1e-16 && pd < 1e12 && dd < 1e12 && ratio > 1e-8 && ratio < 1e8) {
                double err = std::log(dd) - std::log(pd) - std::log(pw);
                pw_esum *= R.i_smooth;
                pw_esum += err;
                double de = err - pw_last;
                pw *= std::exp(R.k_p * err + R.k_i * pw_esum + R.k_d * de);
                pw_last = err;
            } else {
                pw = best_pw;
                pw_esum = 0.0;
                pw_last = 0.0;
            }
            double g = std::fabs(std::log10(std::fmax(rel_d, 1e-300) / std::fmax(rel_p, 1e-300)));
            if (g < best_gap) {
                best_gap = g;
                best_pw = pw;
            }
        }
        refresh_step_schedule();
        if (to_current) { /* solver.cu:3015-3040 */
            xbar = xh;
            ybar = yh;
            x0 = x;
            xh = x;
            y0 = y;
            yh = y;
        } else if (to_halpern) { /* solver.cu:3043-3068 */
            xbar = xh;
            ybar = yh;
            x0 = xhal;
            x = xhal;
            xh = xhal;
            y0 = yhal;
            y = yhal;
            yh = yhal;
        } else {
            x0 = xh;
            x = xh;
            y0 = yh;
            y = yh;
        }
        inner = 0;
        fp_last = INFINITY;
        restarts++;
        restarts_to[to_current ? 1 : to_halpern ? 2 : 0]++;
    }
    /* Infeasibility certificates: an opt-in extension of this library.  The
     * reference computes these quantities (compute_infeasibility_information,
     * LP/CP_AL/src/utils.cu:919-1029) but never calls that function, and its
     * termination test (utils.cu:298-317) checks only optimality and the
     * limits.  The ray estimates are the iterates' displacement from the
     * restart anchor, dx = x^ - x0 and dy = y^ - y0, projected onto the
     * recession cones as utils.cu:684-720 does; the certificate tests are
     * utils.cu:281-297 with tolerance eps_infeasible.  Both ratios are
     * invariant to the rays' scale, so the raw displacements are used, and
     * the reported values are normalised as utils.cu:929-1028 normalises
     * them (primal ray by its max norm, dual ray by the larger of its max
     * norm and its largest dual-slack violation). */
    double ray_pinf = 0, ray_dinf = 0, ray_pobj = 0, ray_dobj = 0;
    void infeasibility_information() {
        std::vector<double> dxr(n), dyr(m), adx(m), aty(n);
        for (int j = 0; j < n; ++j) {
            double d = xh[j] - x0[j];
            if (std::isfinite(vlb[j])) d = std::fmax(d, 0.0);
            if (std::isfinite(vub[j])) d = std::fmin(d, 0.0);
            dxr[j] = d;
        }
        for (int i = 0; i < m; ++i) {
            double d = yh[i] - y0[i];
            if (!std::isfinite(clb[i])) d = std::fmin(d, 0.0);
            if (!std::isfinite(cub[i])) d = std::fmax(d, 0.0);
            dyr[i] = d;
        }
        spmv(A, dxr.data(), adx.data());
        spmv(At, dyr.data(), aty.data());
        double pviol = 0.0, rowsum = 0.0, dy_inf = 0.0;
        for (int i = 0; i < m; ++i) {
            const double a = adx[i];
            pviol = std::fmax(pviol, (std::fmax(0.0, -a) * (std::isfinite(clb[i]) ? 1.0 : 0.0) +
                                      std::fmax(0.0, a) * (std::isfinite(cub[i]) ? 1.0 : 0.0)) *
                                         rcum[i]);
            rowsum += std::fmax(dyr[i], 0.0) * clb_fin[i] + std::fmin(dyr[i], 0.0) * cub_fin[i];
            dy_inf = std::fmax(dy_inf, std::fabs(dyr[i]));
        }
        double dviol = 0.0, colsum = 0.0, dx_inf = 0.0, cdx = 0.0;
        for (int j = 0; j < n; ++j) {
            const double q = -aty[j];
            const bool lf = std::isfinite(vlb[j]), uf = std::isfinite(vub[j]);
            dviol = std::fmax(dviol, (std::fmax(0.0, q) * (lf ? 0.0 : 1.0) - std::fmin(0.0, q) * (uf ? 0.0 : 1.0)) *
                                         dcum[j]);
            colsum += std::fmax(q, 0.0) * (lf ? vlb[j] : 0.0) + std::fmin(q, 0.0) * (uf ? vub[j] : 0.0);
            dx_inf = std::fmax(dx_inf, std::fabs(dxr[j]));
            cdx += c[j] * dxr[j];
        }
        ray_pinf = dx_inf > 0.0 ? pviol / dx_inf : pviol;
        ray_pobj = (dx_inf > 0.0 ? cdx / dx_inf : cdx) / (cbr * ovr);
        const double sc = std::fmax(dy_inf, dviol);
        ray_dinf = sc > 0.0 ? dviol / sc : 0.0;
        ray_dobj = sc > 0.0 ? (rowsum + colsum) / (cbr * ovr) / sc : 0.0;
    }
    void check_termination(double elapsed) { /* utils.cu:275-317 */
        const auto &T = P->termination_criteria;
        if (rel_d < T.eps_feasible_relative && rel_p < T.eps_feasible_relative && rel_gap < T.eps_optimal_relative) {
            reason = TERMINATION_REASON_OPTIMAL;
            return;
        }
        if (O.infeasibility_detection) {
            infeasibility_information();
            /* utils.cu:281-288: a dual ray certifies primal infeasibility */
            if (ray_dobj > 0.0 && ray_dinf / ray_dobj <= O.eps_infeasible) {
                reason = TERMINATION_REASON_PRIMAL_INFEASIBLE;
                return;
            }
            /* utils.cu:290-297: a primal ray certifies dual infeasibility */
            if (ray_pobj < 0.0 && ray_pinf / (-ray_pobj) <= O.eps_infeasible) {
                reason = TERMINATION_REASON_DUAL_INFEASIBLE;
                return;
            }
        }
        if (total >= T.iteration_limit) {
            reason = TERMINATION_REASON_ITERATION_LIMIT;
            return;
        }
        if (elapsed >= T.time_sec_limit) {
            reason = TERMINATION_REASON_TIME_LIMIT;
            return;
        }
    }
};

double norm_of(const double *v, int len, norm_type_t nt) {
    double s = 0.0, mx = 0.0;
    for (int i = 0; i < len; ++i) {
        if (nt == NORM_TYPE_L_INF)
            mx = std::fmax(mx, std::fabs(v[i]));
        else
            s += v[i] * v[i];
    }
    return nt == NORM_TYPE_L_INF ? mx : std::sqrt(s);
}

} // namespace

extern "C" {

/* The reference defaults of the CP_AL_* environment plane
 * (LP/CP_AL/src/solver.cu:3141-3164, 3563-3579, 2862-2880, 3105;
 * LP/CP_AL/src/utils.cu:324-332, 2751-2760), environment ignored. */
void oracle_cpal_default_options(cp_al_gb300_options_t *o) {
    memset(o, 0, sizeof(*o));
    o->al_lambda = 0.05;
    o->sigma_mode = 0;
    o->sigma_set = 0;
    o->sigma = 0.0;
    o->sigma_adaptive = 1;
    o->sigma_init_factor = 6.0;
    o->sigma_min_factor = 1e-4;
    o->sigma_max_factor = 100.0;
    o->lambda_factor = 2.01;
    o->lambda_param_set = 0;
    o->lambda_param = 0.0;
    o->sigma_balance_gain = 0.15;
    o->sigma_i_smooth = NAN;
    o->sigma_kp = NAN;
    o->sigma_ki = NAN;
    o->sigma_kd = NAN;
    o->sigma_update_min = 0.60;
    o->sigma_update_max = 1.70;
    o->step_margin = 0.998 * 0.998;
    o->restart_sufficient = NAN;
    o->restart_necessary = NAN;
    o->restart_artificial = NAN;
    o->restart_select = 0;
    o->restart_select_margin = 1.0;
    o->restart_select_min_iters = 0;
    o->restart_select_threepoint = 0;
    o->restart_select_min_time = 0.0;
    o->cr_iterations = 0;
    o->cr_early_stop = 0;
    o->cr_early_stop_threshold = 0.1;
    o->precision = CP_AL_GB300_FP64;
    o->fp32_switch_tol = 1e-5;
    o->fp32_max_iterations = -1;
    o->spmv_nnz_per_block = 0;
    o->device = -1;
    o->graph_blocks = 1;
    o->timing = 0;
    o->fp32_stall_evals = 25;
    /* device-only choices of the library (the oracle has one arithmetic) */
    o->dual_panels = -1;
    o->panel_width = 0;
    o->primal_hot_rows = -1;
    o->power_method = -1;
    o->primal_staged = -1;
    o->infeasibility_detection = 0;
    o->eps_infeasible = 1e-8;
    o->persistent_loop = -1;
    o->dual_fused_finish = -1;
    o->device_transpose = -1;
    o->alpha_direct_pulse = 0;
    o->pulse_force = 0;
    o->pulse_trace = 0;
    o->pulse_test_limit = 0;
    o->sigma_trigger = 0;
    o->sigma_trigger_min_iters = 200;
    o->sigma_trigger_primal = 1e-2;
    o->sigma_trigger_dual = 1e-6;
    o->sigma_trigger_ratio = 1e6;
    o->dynamic_eval = 0;
    o->dynamic_eval_fast = 50;
    o->dynamic_eval_after_sec = -1.0;
    o->dynamic_eval_after_iters = -1;
    o->dynamic_eval_min_iters = 0;
    o->dynamic_eval_small_res = 1e-6;
    o->dynamic_eval_large_res = 1e-4;
    o->dynamic_eval_ratio = 1e4;
    o->dynamic_eval_bootstrap_iters = 0;
    o->dual_concurrent = -1;
}

/* LP/CP_AL/src/utils.cu:361-394 (reflection coefficient without the
 * CP_AL_REFLECTION_COEFFICIENT override). */
void oracle_cpal_default_parameters(cp_al_parameters_t *p) {
    memset(p, 0, sizeof(*p));
    p->l_inf_ruiz_iterations = 10;
    p->has_pock_chambolle_alpha = true;
    p->pock_chambolle_alpha = 1.0;
    p->bound_objective_rescaling = true;
    p->verbose = false;
    p->termination_evaluation_frequency = 200;
    p->feasibility_polishing = false;
    p->reflection_coefficient = 1.0;
    p->sv_max_iter = 5000;
    p->sv_tol = 1e-4;
    p->termination_criteria.eps_optimal_relative = 1e-4;
    p->termination_criteria.eps_feasible_relative = 1e-4;
    p->termination_criteria.time_sec_limit = 3600.0;
    p->termination_criteria.iteration_limit = 2147483647;
    p->termination_criteria.eps_feas_polish_relative = 1e-6;
    p->restart_params.artificial_restart_threshold = 0.36;
    p->restart_params.sufficient_reduction_for_restart = 0.2;
    p->restart_params.necessary_reduction_for_restart = 0.5;
    p->restart_params.k_p = 0.99;
    p->restart_params.k_i = 0.01;
    p->restart_params.k_d = 0.0;
    p->restart_params.i_smooth = 0.3;
    p->optimality_norm = NORM_TYPE_L2;
    p->presolve = true;
    p->matrix_zero_tol = 1e-9;
}

void oracle_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"

namespace {

/* setup of a solve: solver.cu:1795-2273 and 3538-3609 */
Solver *oracle_setup(const lp_problem_t *prob, const cp_al_parameters_t *params, const cp_al_gb300_options_t *opts) {
    Solver *SP = new Solver();
    Solver &S = *SP;
    S.P = params;
    S.O = *opts;
    S.n = prob->num_variables;
    S.m = prob->num_constraints;
    const int n = S.n, m = S.m, nnz = prob->constraint_matrix_num_nonzeros;
    S.A.nr = m;
    S.A.nc = n;
    S.A.rp.assign(prob->constraint_matrix_row_pointers, prob->constraint_matrix_row_pointers + m + 1);
    S.A.ci.assign(prob->constraint_matrix_col_indices, prob->constraint_matrix_col_indices + nnz);
    S.A.v.assign(prob->constraint_matrix_values, prob->constraint_matrix_values + nnz);
    S.At = transpose(S.A);
    S.c.assign(prob->objective_vector, prob->objective_vector + n);
    S.vlb.assign(prob->variable_lower_bound, prob->variable_lower_bound + n);
    S.vub.assign(prob->variable_upper_bound, prob->variable_upper_bound + n);
    S.clb.assign(prob->constraint_lower_bound, prob->constraint_lower_bound + m);
    S.cub.assign(prob->constraint_upper_bound, prob->constraint_upper_bound + m);
    S.obj_const = prob->objective_constant;
    S.x0.assign(n, 0.0);
    S.y0.assign(m, 0.0);
    if (prob->primal_start) S.x0.assign(prob->primal_start, prob->primal_start + n);
    if (prob->dual_start) S.y0.assign(prob->dual_start, prob->dual_start + m);
    for (auto *v : {&S.x, &S.xh, &S.xbar, &S.dprod, &S.lam, &S.dx, &S.rd}) v->assign(n, 0.0);
    for (auto *v : {&S.y, &S.yh, &S.ybar, &S.pprod, &S.dy, &S.rp, &S.contrib}) v->assign(m, 0.0);
    S.rescale();
    S.x = S.x0;
    S.y = S.y0;
    S.xh = S.x0;
    S.yh = S.y0;
    S.clb_fin.resize(m);
    S.cub_fin.resize(m);
    for (int i = 0; i < m; ++i) { /* solver.cu:2323-2338 */
        S.clb_fin[i] = std::isfinite(S.clb[i]) ? S.clb[i] : 0.0;
        S.cub_fin[i] = std::isfinite(S.cub[i]) ? S.cub[i] : 0.0;
    }
    /* norms of the unscaled problem, solver.cu:1999-2067 */
    S.obj_norm = norm_of(prob->objective_vector, n, params->optimality_norm);
    {
        double s = 0.0, mx = 0.0;
        for (int i = 0; i < m; ++i) {
            double lo = prob->constraint_lower_bound[i], up = prob->constraint_upper_bound[i];
            if (params->optimality_norm == NORM_TYPE_L_INF) {
                if (std::isfinite(lo) && lo != up) mx = std::fmax(mx, std::fabs(lo));
                if (std::isfinite(up)) mx = std::fmax(mx, std::fabs(up));
            } else {
                if (std::isfinite(lo) && lo != up) s += lo * lo;
                if (std::isfinite(up)) s += up * up;
            }
        }
        S.bnd_norm = params->optimality_norm == NORM_TYPE_L_INF ? mx : std::sqrt(s);
    }
    S.initialize_step_size_and_primal_weight();
    S.dyn_setup();
    return SP;
}

/* one evaluation block of the loop, solver.cu:1270-1697; returns true when
 * the solve has terminated */
bool oracle_block(Solver &S, bool &do_restart, int &charged, double elapsed, int limit) {
    const int F = S.F_cur; /* this block's length */
    if (do_restart) {
        S.fixed_point_error();
        S.fp0 = S.fp;
        do_restart = false;
    }
    S.primal(1, true);
    S.dual(1, true);
    for (int i = 2; i <= F - 1; ++i) {
        S.primal(i, false);
        S.dual(i, false);
    }
    S.primal(F, true);
    S.dual(F, true);
    S.fixed_point_error();
    S.compute_residual();
    S.inner += F;
    S.total += F;
    charged += F;
    if (S.P->verbose) {
        printf("%8d %.2e | %+.6e %+.6e | %.1e %.1e %.1e | %.1e | pw %.3e eta %.3e beta %.3e rs %d oracle\n", S.total,
               elapsed, S.pobj, S.dobj, S.rel_p, S.rel_d, S.rel_gap, S.fp, S.pw, S.step, S.beta, S.restarts);
        fflush(stdout);
    }
    S.check_termination(elapsed);
    if (S.reason == TERMINATION_REASON_UNSPECIFIED && charged >= limit) S.reason = TERMINATION_REASON_ITERATION_LIMIT;
    const cp_al_gb300_options_t &O = S.O;
    if (O.alpha_direct_pulse && S.pulse_phase == 1) {
        /* solver.cu:990-1007: alpha back to 0 and the fixed-point error
         * taken again with the refreshed steps, terminated or not */
        S.sigma_mode = false;
        S.al_lambda = 0.0;
        S.refresh_step_schedule();
        S.fixed_point_error();
        S.pulse_phase = 2;
    }
    if (S.reason == TERMINATION_REASON_UNSPECIFIED && O.alpha_direct_pulse && O.pulse_test_limit > 0 &&
        S.pulse_phase == 2 && S.total >= O.pulse_test_limit) /* solver.cu:1386-1391, 1418-1424 */
        S.reason = TERMINATION_REASON_ITERATION_LIMIT;
    if (S.reason != TERMINATION_REASON_UNSPECIFIED) return true;
    S.choose_restart_candidate(elapsed);
    /* solver.cu:1496-1527: the sigma trigger; a forced restart skips the
     * restart rule */
    bool forced = false;
    if (O.sigma_trigger && !S.sigma_mode && S.total >= O.sigma_trigger_min_iters) {
        const double rpr = std::fmax(S.rel_p, 1e-300), rdr = std::fmax(S.rel_d, 1e-300);
        if (rpr >= O.sigma_trigger_primal && rdr <= O.sigma_trigger_dual && rpr / rdr >= O.sigma_trigger_ratio) {
            S.initialize_sigma_parameters();
            S.trigger_iter = S.total;
            forced = true;
        }
    }
    S.dyn_update(elapsed);
    do_restart = forced || S.should_restart(F);
    if (do_restart) {
        if (O.alpha_direct_pulse) S.record_epoch();
        S.perform_restart();
        if (O.alpha_direct_pulse) {
            S.epoch_start();
            S.pulse_gate_eval(F, limit);
        }
    }
    return false;
}

/* ---------------- feasibility polishing (LP/CP_AL/src/solver.cu:3912-4456) ----------------
 * Primal polishing solves the feasibility problem (c = 0) from the final
 * primal iterates with the dual iterates at zero; dual polishing solves the
 * problem with every finite bound set to zero from the final dual iterates
 * with the primal iterates at zero.  Both keep the step size and the AL /
 * sigma state of the solve, take the primal weight of the start of the
 * solve, run the iteration in blocks of F with the restart rule on a
 * one-sided fixed-point error (|x^ - x_bar|^2 w, or |y^ - y_bar|^2 / w), and
 * stop when their relative residual is below eps_feas_polish_relative.  A
 * successful phase replaces the solve's primal (dual) solution, residuals and
 * objective; the primal objective is then taken without the objective
 * constant (utils.cu:1388-1391 adds the polishing state's constant, which is
 * zero). */
struct PolishOut {
    termination_reason_t reason = TERMINATION_REASON_UNSPECIFIED;
    int total = 0;
};

static PolishOut polish_phase(const Solver &S, bool primal, Solver &W,
                              std::chrono::steady_clock::time_point solve_start) {
    const int F = S.P->termination_evaluation_frequency;
    const int n = S.n, m = S.m;
    W = S;
    if (primal) { /* solver.cu:4147-4200 */
        std::fill(W.c.begin(), W.c.end(), 0.0);
        for (auto *v : {&W.y0, &W.y, &W.yh, &W.ybar}) std::fill(v->begin(), v->end(), 0.0);
        std::fill(W.dprod.begin(), W.dprod.end(), 0.0);
    } else { /* solver.cu:4245-4330 */
        auto zero_finite = [](std::vector<double> &v) {
            for (double &x : v)
                if (std::isfinite(x)) x = 0.0;
        };
        zero_finite(W.clb);
        zero_finite(W.cub);
        zero_finite(W.vlb);
        zero_finite(W.vub);
        std::fill(W.clb_fin.begin(), W.clb_fin.end(), 0.0);
        std::fill(W.cub_fin.begin(), W.cub_fin.end(), 0.0);
        for (auto *v : {&W.x0, &W.x, &W.xh, &W.xbar}) std::fill(v->begin(), v->end(), 0.0);
        std::fill(W.pprod.begin(), W.pprod.end(), 0.0);
    }
    if (primal) std::fill(W.lam.begin(), W.lam.end(), 0.0);
    W.pw_esum = W.pw_last = 0.0;
    W.fp = W.fp0 = W.fp_last = INFINITY;
    W.total = W.inner = 0;
    W.reason = TERMINATION_REASON_UNSPECIFIED;
    W.best_gap = INFINITY;
    const double pw0 = S.P->bound_objective_rescaling ? 1.0 : (S.obj_norm + 1.0) / (S.bnd_norm + 1.0);
    W.pw = pw0;
    W.best_pw = pw0;
    auto fpe = [&]() {
        double acc = 0.0;
        if (primal) {
            for (int j = 0; j < n; ++j) acc += (W.xh[j] - W.xbar[j]) * (W.xh[j] - W.xbar[j]);
            return acc * W.pw;
        }
        for (int i = 0; i < m; ++i) acc += (W.yh[i] - W.ybar[i]) * (W.yh[i] - W.ybar[i]);
        return acc / W.pw;
    };
    const double eps = S.P->termination_criteria.eps_feas_polish_relative;
    const int limit = S.P->termination_criteria.iteration_limit;
    bool do_restart = false;
    PolishOut out;
    while (W.reason == TERMINATION_REASON_UNSPECIFIED) { /* solver.cu:3988-4051, 4063-4126 */
        W.primal(1, true);
        W.dual(1, true);
        if (do_restart) {
            W.fp = fpe();
            W.fp0 = W.fp;
            do_restart = false;
        }
        for (int i = 2; i <= F - 1; ++i) {
            W.primal(i, false);
            W.dual(i, false);
        }
        W.primal(F, true);
        W.dual(F, true);
        W.fp = fpe();
        if (primal) { /* utils.cu:1341-1392 */
            spmv(W.A, W.xh.data(), W.pprod.data());
            for (int i = 0; i < m; ++i)
                W.rp[i] = (W.pprod[i] - std::fmax(W.clb[i], std::fmin(W.pprod[i], W.cub[i]))) * W.rcum[i];
            W.abs_p = (S.P->optimality_norm == NORM_TYPE_L_INF ? amax(W.rp) : nrm2(W.rp)) / W.cbr;
            W.rel_p = W.abs_p / (1.0 + W.bnd_norm);
            W.pobj = dot(S.c, W.xh) / (W.cbr * W.ovr);
        } else { /* utils.cu:1394-1453 */
            spmv(W.At, W.yh.data(), W.dprod.data());
            for (int j = 0; j < n; ++j) W.rd[j] = (W.c[j] - W.dprod[j] - W.lam[j]) * W.dcum[j];
            double csum = 0.0;
            for (int i = 0; i < m; ++i)
                csum += std::fmax(W.yh[i], 0.0) * S.clb_fin[i] + std::fmin(W.yh[i], 0.0) * S.cub_fin[i];
            W.abs_d = (S.P->optimality_norm == NORM_TYPE_L_INF ? amax(W.rd) : nrm2(W.rd)) / W.ovr;
            W.rel_d = W.abs_d / (1.0 + W.obj_norm);
            W.dobj = (dot(W.lam, S.xh) + csum) / (W.cbr * W.ovr) + W.obj_const;
        }
        W.inner += F;
        W.total += F;
        /* utils.cu:1194-1226; the time limit counts from the start of the solve */
        const double since = std::chrono::duration<double>(std::chrono::steady_clock::now() - solve_start).count();
        if ((primal ? W.rel_p : W.rel_d) <= eps)
            W.reason = TERMINATION_REASON_FEAS_POLISH_SUCCESS;
        else if (W.total >= limit)
            W.reason = TERMINATION_REASON_ITERATION_LIMIT;
        else if (since >= S.P->termination_criteria.time_sec_limit)
            W.reason = TERMINATION_REASON_TIME_LIMIT;
        if (W.reason != TERMINATION_REASON_UNSPECIFIED) break;
        do_restart = W.should_restart(F);
        if (do_restart) { /* solver.cu:4376-4404 */
            if (primal) {
                W.x0 = W.xh;
                W.x = W.xh;
            } else {
                W.y0 = W.yh;
                W.y = W.yh;
            }
            W.inner = 0;
            W.fp_last = INFINITY;
        }
    }
    out.reason = W.reason;
    out.total = W.total;
    return out;
}

/* returns the iterations the two phases add to feasibility_iteration */
static int oracle_polish(Solver &S, int *primal_status, int *dual_status,
                         std::chrono::steady_clock::time_point solve_start) {
    *primal_status = *dual_status = -1;
    const double eps = S.P->termination_criteria.eps_feas_polish_relative;
    if (S.rel_p < eps && S.rel_d < eps) return 0; /* solver.cu:3915-3920 */
    int iters = 0;
    {
        std::unique_ptr<Solver> W(new Solver());
        PolishOut o = polish_phase(S, true, *W, solve_start);
        *primal_status = (int)o.reason;
        if (o.reason == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
            S.xh = W->xh;
            S.abs_p = W->abs_p;
            S.rel_p = W->rel_p;
            S.pobj = W->pobj;
        }
        iters += o.total - 1;
    }
    {
        std::unique_ptr<Solver> W(new Solver());
        PolishOut o = polish_phase(S, false, *W, solve_start);
        *dual_status = (int)o.reason;
        if (o.reason == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
            S.yh = W->yh;
            S.abs_d = W->abs_d;
            S.rel_d = W->rel_d;
            S.dobj = W->dobj;
        }
        iters += o.total - 1;
    }
    S.gap = std::fabs(S.pobj - S.dobj);
    S.rel_gap = S.gap / (1.0 + std::fabs(S.pobj) + std::fabs(S.dobj));
    return iters;
}

/* result: solver.cu:3828-3909 */
cp_al_result_t *oracle_result(Solver &S, double rescale_sec, double elapsed) {
    const int n = S.n, m = S.m;
    cp_al_result_t *res = (cp_al_result_t *)calloc(1, sizeof(cp_al_result_t));
    res->primal_solution = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    res->dual_solution = (double *)malloc(sizeof(double) * (m > 0 ? m : 1));
    res->reduced_cost = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    spmv(S.At, S.yh.data(), S.dprod.data());
    for (int j = 0; j < n; ++j) {
        double rc = (S.c[j] - S.dprod[j]) * S.dcum[j] / S.ovr;
        if (!std::isfinite(S.vlb[j])) rc = std::fmin(rc, 0.0);
        if (!std::isfinite(S.vub[j])) rc = std::fmax(rc, 0.0);
        res->reduced_cost[j] = rc;
        res->primal_solution[j] = S.xh[j] / S.dcum[j] / S.cbr;
    }
    for (int i = 0; i < m; ++i) res->dual_solution[i] = S.yh[i] / S.rcum[i] / S.ovr;
    res->num_variables = n;
    res->num_constraints = m;
    res->num_nonzeros = (int)S.A.v.size();
    res->total_count = S.total;
    res->rescaling_time_sec = rescale_sec;
    res->cumulative_time_sec = elapsed;
    res->absolute_primal_residual = S.abs_p;
    res->relative_primal_residual = S.rel_p;
    res->absolute_dual_residual = S.abs_d;
    res->relative_dual_residual = S.rel_d;
    res->primal_objective_value = S.pobj;
    res->dual_objective_value = S.dobj;
    res->objective_gap = S.gap;
    res->relative_objective_gap = S.rel_gap;
    res->termination_reason = S.reason;
    res->max_primal_ray_infeasibility = S.ray_pinf;
    res->max_dual_ray_infeasibility = S.ray_dinf;
    res->primal_ray_linear_objective = S.ray_pobj;
    res->dual_ray_objective = S.ray_dobj;
    return res;
}

struct OracleSession {
    Solver *S = nullptr;
    cp_al_parameters_t P;
    bool do_restart = false;
    int charged = 0;
};

} // namespace

extern "C" {

cp_al_result_t *oracle_cpal_solve(const lp_problem_t *prob, const cp_al_parameters_t *params,
                                  const cp_al_gb300_options_t *opts, int *power_iterations_out) {
    if (!prob || !params || !opts) return nullptr;
    if (params->termination_evaluation_frequency < 3) return nullptr;
    auto t0 = std::chrono::steady_clock::now();
    std::unique_ptr<Solver> S(oracle_setup(prob, params, opts));
    double rescale_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    auto t_start = std::chrono::steady_clock::now();
    const int limit = params->termination_criteria.iteration_limit;
    bool do_restart = false;
    int charged = 0;
    double elapsed = 0.0;
    while (charged < limit) {
        elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        if (oracle_block(*S, do_restart, charged, elapsed, limit)) break;
    }
    elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    if (S->reason == TERMINATION_REASON_UNSPECIFIED) {
        S->reason = TERMINATION_REASON_ITERATION_LIMIT;
        S->compute_residual();
    }
    if (power_iterations_out) *power_iterations_out = S->power_iters;
    for (int t = 0; t < 3; ++t) g_restart_targets[t] = S->restarts_to[t];
    g_controllers[0] = S->pulse_start;
    g_controllers[1] = S->pulse_gate;
    g_controllers[2] = S->trigger_iter;
    g_controllers[3] = S->dyn_iter;
    int polish_iters = 0, pst = -1, dst = -1;
    double polish_sec = 0.0;
    if (params->feasibility_polishing && S->reason != TERMINATION_REASON_PRIMAL_INFEASIBLE &&
        S->reason != TERMINATION_REASON_DUAL_INFEASIBLE) { /* solver.cu:1715-1719 */
        auto tp = std::chrono::steady_clock::now();
        polish_iters = oracle_polish(*S, &pst, &dst, t_start);
        polish_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count();
    }
    cp_al_result_t *r = oracle_result(*S, rescale_sec, elapsed);
    if (r && params->feasibility_polishing) {
        r->feasibility_iteration = polish_iters;
        r->feasibility_polishing_time = polish_sec;
    }
    g_polish_status[0] = pst;
    g_polish_status[1] = dst;
    return r;
}

/* statuses of the last solve's primal and dual polishing phases (-1: not run) */
void oracle_cpal_polish_status(int *primal, int *dual) {
    *primal = g_polish_status[0];
    *dual = g_polish_status[1];
}

/* restarts of the last solve by target: the current point, the reflected
 * Halpern iterate, the plain Halpern point */
void oracle_cpal_restart_targets(int *counts) {
    for (int t = 0; t < 3; ++t) counts[t] = g_restart_targets[t];
}

/* benchmark controllers of the last solve: the iteration at which the alpha
 * pulse's positive block started (-1: never), its gate (0 not evaluated, 1
 * passed, 2 rejected), the iteration at which the sigma trigger fired (0:
 * never), the iteration at which the dynamic evaluation frequency switched to
 * short blocks (0: never) */
void oracle_cpal_controllers(int *out) {
    for (int t = 0; t < 4; ++t) out[t] = g_controllers[t];
}

/* Session form for timing: setup once, then blocks of iterations. */
void *oracle_cpal_session_create(const lp_problem_t *prob, const cp_al_parameters_t *params,
                                 const cp_al_gb300_options_t *opts) {
    if (!prob || !params || !opts || params->termination_evaluation_frequency < 3) return nullptr;
    OracleSession *s = new OracleSession();
    s->P = *params;
    s->S = oracle_setup(prob, &s->P, opts);
    s->S->P = &s->P;
    return s;
}

/* Runs ceil(iterations / F) evaluation blocks; returns the iterations run. */
int oracle_cpal_session_iterate(void *h, int iterations) {
    OracleSession *s = (OracleSession *)h;
    if (!s) return -1;
    int done = 0;
    while (done < iterations) {
        s->S->reason = TERMINATION_REASON_UNSPECIFIED;
        const int F = s->S->F_cur; /* this block's length */
        if (oracle_block(*s->S, s->do_restart, s->charged, 0.0, 2147483647) &&
            s->S->reason == TERMINATION_REASON_OPTIMAL)
            break;
        done += F;
    }
    return done;
}

void oracle_cpal_session_free(void *h) {
    OracleSession *s = (OracleSession *)h;
    if (!s) return;
    delete s->S;
    delete s;
}

void oracle_cpal_result_free(cp_al_result_t *r) {
    if (!r) return;
    free(r->primal_solution);
    free(r->dual_solution);
    free(r->reduced_cost);
    free(r);
}

/* Equilibration alone, for tests: writes the cumulative row/column scales and
 * the bound/objective factors of the reference's rescale_problem. */
int oracle_cpal_rescale(const lp_problem_t *prob, const cp_al_parameters_t *params, const cp_al_gb300_options_t *opts,
                        double *row_scale, double *col_scale, double *cbr_ovr, double *scaled_vals) {
    Solver S;
    S.P = params;
    if (opts)
        S.O = *opts;
    else
        oracle_cpal_default_options(&S.O);
    S.n = prob->num_variables;
    S.m = prob->num_constraints;
    const int nnz = prob->constraint_matrix_num_nonzeros;
    S.A.nr = S.m;
    S.A.nc = S.n;
    S.A.rp.assign(prob->constraint_matrix_row_pointers, prob->constraint_matrix_row_pointers + S.m + 1);
    S.A.ci.assign(prob->constraint_matrix_col_indices, prob->constraint_matrix_col_indices + nnz);
    S.A.v.assign(prob->constraint_matrix_values, prob->constraint_matrix_values + nnz);
    S.At = transpose(S.A);
    S.c.assign(prob->objective_vector, prob->objective_vector + S.n);
    S.vlb.assign(prob->variable_lower_bound, prob->variable_lower_bound + S.n);
    S.vub.assign(prob->variable_upper_bound, prob->variable_upper_bound + S.n);
    S.clb.assign(prob->constraint_lower_bound, prob->constraint_lower_bound + S.m);
    S.cub.assign(prob->constraint_upper_bound, prob->constraint_upper_bound + S.m);
    S.x0.assign(S.n, 0.0);
    S.y0.assign(S.m, 0.0);
    S.rescale();
    for (int i = 0; i < S.m; ++i) row_scale[i] = S.rcum[i];
    for (int j = 0; j < S.n; ++j) col_scale[j] = S.dcum[j];
    cbr_ovr[0] = S.cbr;
    cbr_ovr[1] = S.ovr;
    if (scaled_vals)
        for (int k = 0; k < nnz; ++k) scaled_vals[k] = S.A.v[k];
    return S.cr_passes; /* Curtis-Reid passes run (0 when off) */
}

/* Power iteration alone: sigma_max(A) of the (unscaled) CSR matrix given. */
double oracle_power_iteration(int m, int n, const int *rp, const int *ci, const double *v, int max_iter, double tol,
                              int *iters) {
    Solver S;
    cp_al_parameters_t P;
    memset(&P, 0, sizeof(P));
    P.sv_max_iter = max_iter;
    P.sv_tol = tol;
    S.P = &P;
    S.m = m;
    S.n = n;
    S.A.nr = m;
    S.A.nc = n;
    S.A.rp.assign(rp, rp + m + 1);
    S.A.ci.assign(ci, ci + rp[m]);
    S.A.v.assign(v, v + rp[m]);
    S.At = transpose(S.A);
    double s = S.max_singular_value();
    if (iters) *iters = S.power_iters;
    return s;
}

} // extern "C"
