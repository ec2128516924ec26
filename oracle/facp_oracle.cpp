/*
 * facp_oracle.cpp -- CPU restatement of the FA_CP (convex QP) restarted
 * reflected Halpern primal-dual solver.  TEST INFRASTRUCTURE ONLY: the checker
 * of the CUDA library, never part of the product path.
 *
 * It follows the reference's operation order in plain FP64 loops, including
 * the places where buffers are shared between stages:
 *   - host equilibration     QP/FA_CP/src/preconditioner.c:92-331
 *   - state setup            QP/FA_CP/src/solver_state.cu:494-877, 220-303
 *   - power iterations       QP/FA_CP/src/utils.cu:65-315
 *   - outer loop             QP/FA_CP/src/solver.cu:74-165
 *   - update, BB inner solve QP/FA_CP/src/fa_cp_core_op.cu:68-640
 *   - sigma rules, restart   QP/FA_CP/src/fa_cp_core_op.cu:650-1020
 *   - fixed-point error      QP/FA_CP/src/fa_cp_core_op.cu:1042-1089
 *   - residual, rays         QP/FA_CP/src/utils.cu:705-1132
 *   - termination, restart   QP/FA_CP/src/utils.cu:413-492
 *   - result                 QP/FA_CP/src/fa_cp_core_op.cu:1171-1239
 * cuBLAS/cuSPARSE reductions are restated as sequential sums; the Q
 * eigenvalue start vectors use the C library's rand() from its default seed,
 * as a fresh reference process does.  Built with -ffp-contract=off.
 */
#include "../include/fa_cp_types.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

namespace {

struct Csr {
    int nr = 0, nc = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
    int nnz() const { return (int)v.size(); }
};

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
    for (int i = 0; i < M.nr; ++i) {
        double s = 0.0;
        for (int k = M.rp[i]; k < M.rp[i + 1]; ++k) s += M.v[k] * x[M.ci[k]];
        y[i] = s;
    }
}

double dot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}
double nrm2(const std::vector<double> &a) { return std::sqrt(dot(a, a)); }
double amax(const std::vector<double> &a) {
    double m = 0.0;
    for (double v : a) m = std::fmax(m, std::fabs(v));
    return m;
}
double vsum(const std::vector<double> &a) {
    double s = 0.0;
    for (double v : a) s += v;
    return s;
}

int g_trace = 0;
int g_polish_status[2] = {-1, -1};

int print_frequency(int iter) { /* utils.cu:636-647 */
    int step = 10;
    long long threshold = 1000;
    while (iter >= threshold) {
        step *= 10;
        threshold *= 10;
    }
    return step;
}

Csr from_component(const CsrComponent *c, int nrows, int ncols, int nnz) {
    Csr M;
    M.nr = nrows;
    M.nc = ncols;
    M.rp.assign(nrows + 1, 0);
    if (c && c->row_ptr && nnz > 0) {
        M.rp.assign(c->row_ptr, c->row_ptr + nrows + 1);
        M.ci.assign(c->col_ind, c->col_ind + nnz);
        M.v.assign(c->val, c->val + nnz);
    }
    return M;
}

double sane_positive(double v, double fb) { return (std::isfinite(v) && v > 0.0) ? v : fb; }
double score_component(double v) { return std::isfinite(v) ? std::fmax(v, 1e-300) : INFINITY; }

struct QP {
    const fa_cp_parameters_t *P;
    int n = 0, m = 0, nr = 0;
    Csr A, At, Q, R, Rt;
    quad_obj_type_t qtype = FA_CP_NON_Q;
    bool is_lp = true;
    std::vector<double> c, vlb, vub, clb, cub, clb_fin, cub_fin, vlb_fin, vub_fin, diag;
    std::vector<double> x0, x, xh, xbar, y0, y, yh, ybar;
    std::vector<double> dprod, pprod, dslack, pslack, dx, dy, qx, rx, grad, dir, pbuf, aldual, rres, dres;
    std::vector<double> dcum, rcum;
    double cbr = 1, ovr = 1, c0 = 0, obj_norm = 0, bnd_norm = 0;
    double qnorm = 0, nonconvexity = 0;
    double step = 0, pw = 1, best_pw = 1, pw_esum = 0, pw_last = 0, best_gap = INFINITY;
    double fp = INFINITY, fp0 = INFINITY, fp_last = INFINITY;
    int total = 0, inner = 0;
    bool major = false;
    double abs_p = 0, abs_d = 0, rel_p = 0, rel_d = 0, pobj = 0, dobj = 0, gap = 0, rel_gap = 0;
    double max_pray = 0, max_dray = 0, pray_lin = 0, dray_obj = 0;
    termination_reason_t reason = TERMINATION_REASON_UNSPECIFIED;
    /* AL sigma */
    bool al_available = false, use_al = false;
    double al_sigma = 0, best_al_sigma = 0, best_sigma_score = INFINITY, last_sigma_score = INFINITY;
    double last_rp = INFINITY, last_rd = INFINITY, last_rg = INFINITY;
    int sigma_updates = 0, sigma_dir = 1;
    /* inner solver */
    bool has_inner = false;
    int inner_limit = 1000;
    double inner_tol = 1e-3;
    int inner_total = 0;

    /* ---------- equilibration (preconditioner.c) ---------- */
    void scale(const std::vector<double> &r, const std::vector<double> &d) { /* 92-131 */
        for (int i = 0; i < n; ++i) {
            c[i] /= d[i];
            vub[i] *= d[i];
            vlb[i] *= d[i];
        }
        for (int i = 0; i < m; ++i) {
            clb[i] /= r[i];
            cub[i] /= r[i];
        }
        for (int row = 0; row < m; ++row)
            for (int k = A.rp[row]; k < A.rp[row + 1]; ++k) A.v[k] /= (r[row] * d[A.ci[k]]);
        for (int qr = 0; qr < n; ++qr)
            for (int k = Q.rp[qr]; k < Q.rp[qr + 1]; ++k) Q.v[k] /= (d[qr] * d[Q.ci[k]]);
        if (R.nnz() > 0)
            for (int rr = 0; rr < nr; ++rr)
                for (int k = R.rp[rr]; k < R.rp[rr + 1]; ++k) R.v[k] /= d[R.ci[k]];
    }
    void rescale() {
        dcum.assign(n, 1.0);
        rcum.assign(m, 1.0);
        std::vector<double> cr(m), vr(n);
        for (int it = 0; it < P->l_inf_ruiz_iterations; ++it) { /* 136-198 */
            std::fill(vr.begin(), vr.end(), 0.0);
            std::fill(cr.begin(), cr.end(), 0.0);
            for (int row = 0; row < m; ++row)
                for (int k = A.rp[row]; k < A.rp[row + 1]; ++k) {
                    const double v = std::fabs(A.v[k]);
                    if (v > vr[A.ci[k]]) vr[A.ci[k]] = v;
                    if (v > cr[row]) cr[row] = v;
                }
            for (int qr = 0; qr < n; ++qr)
                for (int k = Q.rp[qr]; k < Q.rp[qr + 1]; ++k) {
                    const double v = std::fabs(Q.v[k]);
                    if (v > vr[Q.ci[k]]) vr[Q.ci[k]] = v;
                }
            for (int i = 0; i < n; ++i) vr[i] = (vr[i] < 1e-12) ? 1.0 : std::sqrt(vr[i]);
            for (int i = 0; i < m; ++i) cr[i] = (cr[i] < 1e-12) ? 1.0 : std::sqrt(cr[i]);
            scale(cr, vr);
            for (int i = 0; i < n; ++i) dcum[i] *= vr[i];
            for (int i = 0; i < m; ++i) rcum[i] *= cr[i];
        }
        if (P->has_pock_chambolle_alpha) { /* 200-243 */
            const double a = P->pock_chambolle_alpha;
            std::fill(vr.begin(), vr.end(), 0.0);
            std::fill(cr.begin(), cr.end(), 0.0);
            for (int row = 0; row < m; ++row)
                for (int k = A.rp[row]; k < A.rp[row + 1]; ++k) {
                    const double v = std::fabs(A.v[k]);
                    vr[A.ci[k]] += std::pow(v, 2.0 - a);
                    cr[row] += std::pow(v, a);
                }
            for (int qr = 0; qr < n; ++qr)
                for (int k = Q.rp[qr]; k < Q.rp[qr + 1]; ++k) vr[Q.ci[k]] += std::pow(std::fabs(Q.v[k]), 2.0 - a);
            for (int i = 0; i < n; ++i) vr[i] = (vr[i] < 1e-12) ? 1.0 : std::sqrt(vr[i]);
            for (int i = 0; i < m; ++i) cr[i] = (cr[i] < 1e-12) ? 1.0 : std::sqrt(cr[i]);
            scale(cr, vr);
            for (int i = 0; i < n; ++i) dcum[i] *= vr[i];
            for (int i = 0; i < m; ++i) rcum[i] *= cr[i];
        }
        if (P->bound_objective_rescaling) { /* 245-289 */
            double bsq = 0.0;
            for (int i = 0; i < m; ++i) {
                if (std::isfinite(clb[i]) && clb[i] != cub[i]) bsq += clb[i] * clb[i];
                if (std::isfinite(cub[i])) bsq += cub[i] * cub[i];
            }
            double csq = 0.0;
            for (int i = 0; i < n; ++i) csq += c[i] * c[i];
            cbr = 1.0 / (std::sqrt(bsq) + 1.0);
            ovr = 1.0 / (std::sqrt(csq) + 1.0);
            for (int i = 0; i < m; ++i) {
                clb[i] *= cbr;
                cub[i] *= cbr;
            }
            for (int i = 0; i < n; ++i) {
                vlb[i] *= cbr;
                vub[i] *= cbr;
                c[i] *= ovr;
            }
            for (double &v : Q.v) v *= ovr / cbr;
            if (R.nnz() > 0) {
                const double f = std::sqrt(ovr / cbr);
                for (double &v : R.v) v *= f;
            }
        } else {
            cbr = 1.0;
            ovr = 1.0;
        }
    }

    /* ---------- objective products (solver_state.cu:371-442) ---------- */
    void obj_product(const std::vector<double> &v) {
        switch (qtype) {
        case FA_CP_NON_Q:
            return;
        case FA_CP_SPARSE_Q:
            spmv(Q, v.data(), qx.data());
            return;
        case FA_CP_DIAG_Q:
            for (int i = 0; i < n; ++i) qx[i] = diag[i] * v[i];
            return;
        case FA_CP_LOW_RANK_Q:
            spmv(R, v.data(), rx.data());
            spmv(Rt, rx.data(), qx.data());
            return;
        case FA_CP_LOW_RANK_PLUS_SPARSE_Q: {
            spmv(Q, v.data(), qx.data());
            spmv(R, v.data(), rx.data());
            std::vector<double> t(n);
            spmv(Rt, rx.data(), t.data());
            for (int i = 0; i < n; ++i) qx[i] = t[i] + qx[i];
            return;
        }
        }
    }

    /* ---------- power iterations (utils.cu:65-315) ---------- */
    double max_singular_value() {
        std::mt19937 gen(1);
        std::normal_distribution<double> dist(0.0, 1.0);
        std::vector<double> v(m), nv(m), dp(n);
        for (int i = 0; i < m; ++i) v[i] = dist(gen);
        double s2 = 1.0;
        for (int it = 0; it < P->sv_max_iter; ++it) {
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
    double q_max_eig() {
        std::vector<double> v(n), av(n);
        for (int i = 0; i < n; ++i) v[i] = (double)rand() / RAND_MAX;
        double lam = 0.0;
        for (int it = 0; it < P->sv_max_iter; ++it) {
            double inv = 1.0 / nrm2(v);
            for (int i = 0; i < n; ++i) v[i] = inv * v[i];
            spmv(Q, v.data(), av.data());
            double old = lam;
            lam = dot(v, av);
            if (it > 0 && std::fabs(lam - old) < P->sv_tol) break;
            v = av;
        }
        return lam;
    }
    double q_min_eig(double lmax) {
        std::vector<double> v(n), av(n), sv(n);
        for (int i = 0; i < n; ++i) v[i] = (double)rand() / RAND_MAX;
        double mu = 0.0;
        for (int it = 0; it < P->sv_max_iter; ++it) {
            double inv = 1.0 / nrm2(v);
            for (int i = 0; i < n; ++i) v[i] = inv * v[i];
            spmv(Q, v.data(), av.data());
            for (int i = 0; i < n; ++i) sv[i] = lmax * v[i] + (-1.0 * av[i]);
            double old = mu;
            mu = dot(v, sv);
            if (it > 0 && std::fabs(mu - old) < P->sv_tol) break;
            v = sv;
        }
        return lmax - mu;
    }

    /* ---------- update (fa_cp_core_op.cu:531-630) ---------- */
    bool write_major() const { return major || ((total + 2) % print_frequency(total + 2)) == 0; }
    void al_effective_dual(const std::vector<double> &xv, double sigma) { /* 275-303 */
        spmv(A, xv.data(), pprod.data());
        for (int i = 0; i < m; ++i) {
            const double shifted = pprod[i] - y[i] / sigma;
            const double proj = std::fmax(clb[i], std::fmin(shifted, cub[i]));
            aldual[i] = y[i] - sigma * (pprod[i] - proj);
        }
        spmv(At, aldual.data(), dprod.data());
    }
    void bb(double tau, double sigma) { /* 445-503 */
        const double inv = 1.0 / tau;
        int it = 1;
        double alpha = 1.0 / inv;
        if (use_al) al_effective_dual(x, sigma);
        obj_product(x);
        for (int i = 0; i < n; ++i) {
            const double g = qx[i] + c[i] - dprod[i];
            double nx = x[i] - alpha * g;
            nx = std::fmax(vlb[i], std::fmin(nx, vub[i]));
            xh[i] = nx;
            grad[i] = g;
            dir[i] = nx - x[i];
        }
        while (it < inner_limit) {
            const double ng = nrm2(dir);
            if (ng <= inner_tol) break;
            if (use_al) al_effective_dual(xh, sigma);
            obj_product(xh);
            for (int i = 0; i < n; ++i) {
                const double last = grad[i];
                const double cur = qx[i] + c[i] - dprod[i] + inv * (xh[i] - x[i]);
                pbuf[i] = cur - last;
                grad[i] = cur;
            }
            const double tmp = dot(dir, pbuf);
            alpha = ng * ng / tmp;
            for (int i = 0; i < n; ++i) {
                const double cur = xh[i];
                double nx = cur - alpha * grad[i];
                nx = std::fmax(vlb[i], std::fmin(nx, vub[i]));
                dir[i] = nx - cur;
                xh[i] = nx;
            }
            it++;
        }
        for (int i = 0; i < n; ++i) xbar[i] = 2.0 * xh[i] - x[i];
        inner_total += (it - 1);
    }
    void update() {
        double tau = step / pw;
        if (nonconvexity < 0) {
            tau = std::fmax(tau, -1.01 * std::fmin(0.0, nonconvexity));
            tau /= 2;
        }
        const double rho = step * pw;
        const double sigma = use_al ? al_sigma : 0.0;
        if (!use_al) spmv(At, y.data(), dprod.data());
        const bool wm = write_major();
        if (use_al) {
            bb(tau, sigma);
        } else if (qtype == FA_CP_NON_Q) { /* 93-122, 305-324 */
            for (int i = 0; i < n; ++i) {
                const double xi = x[i];
                const double t = xi - tau * (c[i] - dprod[i]);
                const double pr = std::fmax(vlb[i], std::fmin(t, vub[i]));
                xbar[i] = 2.0 * pr - xi;
                if (wm) {
                    xh[i] = pr;
                    dslack[i] = (pr - t) / tau;
                }
            }
        } else if (qtype == FA_CP_DIAG_Q) { /* 124-154, 326-347 */
            for (int i = 0; i < n; ++i) {
                const double xi = x[i];
                const double t = (xi - tau * (c[i] - dprod[i])) / (1.0 + tau * diag[i]);
                const double pr = std::fmax(vlb[i], std::fmin(t, vub[i]));
                xbar[i] = 2.0 * pr - xi;
                if (wm) xh[i] = pr;
            }
        } else {
            bb(tau, 0.0);
        }
        spmv(A, xbar.data(), pprod.data());
        for (int i = 0; i < m; ++i) {
            if (use_al) { /* 194-223 */
                const double denom = sigma + rho;
                const double shifted = pprod[i] - y[i] / denom;
                const double proj = std::fmax(clb[i], std::fmin(shifted, cub[i]));
                const double nd = y[i] + rho * (proj - pprod[i]);
                if (wm) yh[i] = nd;
                ybar[i] = 2.0 * nd - y[i];
            } else { /* 156-179 */
                const double t = y[i] / rho - pprod[i];
                const double tp = std::fmax(-cub[i], std::fmin(t, -clb[i]));
                if (wm) {
                    yh[i] = (t - tp) * rho;
                    ybar[i] = 2.0 * yh[i] - y[i];
                } else {
                    ybar[i] = 2.0 * (t - tp) * rho - y[i];
                }
            }
        }
    }
    void halpern() { /* 632-640, 226-242 */
        const double w = (double)(inner + 1) / (inner + 2);
        const double r = P->reflection_coefficient;
        for (int i = 0; i < n; ++i) {
            const double refl = r * xbar[i] + (1.0 - r) * x[i];
            x[i] = w * refl + (1.0 - w) * x0[i];
        }
        for (int i = 0; i < m; ++i) {
            const double refl = r * ybar[i] + (1.0 - r) * y[i];
            y[i] = w * refl + (1.0 - w) * y0[i];
        }
    }
    void fixed_point_error() { /* 1042-1089 */
        for (int i = 0; i < n; ++i) dx[i] = xbar[i] - x[i];
        for (int i = 0; i < m; ++i) dy[i] = ybar[i] - y[i];
        spmv(At, dy.data(), dprod.data());
        const double dn = nrm2(dy), pn = nrm2(dx);
        const double movement = pn * pn * pw + dn * dn / pw;
        const double cross = dot(dprod, dx);
        const double interaction = 2 * step * cross;
        fp = std::sqrt(std::fmax(movement + interaction, 0.0));
        if (has_inner) inner_tol = std::fmin(inner_tol, std::fmax(0.0005 * pn / step * pw, 1e-9));
    }

    /* ---------- evaluation (utils.cu:889-1026) ---------- */
    void residual() {
        const bool linf = P->optimality_norm == NORM_TYPE_L_INF;
        spmv(A, xh.data(), pprod.data());
        spmv(At, yh.data(), dprod.data());
        obj_product(xh);
        const double tau = step / pw;
        for (int i = 0; i < m; ++i) {
            const double cl = std::fmax(clb[i], std::fmin(pprod[i], cub[i]));
            rres[i] = (pprod[i] - cl) * rcum[i];
            pslack[i] = std::fmax(yh[i], 0.0) * clb_fin[i] + std::fmin(yh[i], 0.0) * cub_fin[i];
        }
        for (int j = 0; j < n; ++j) {
            if (is_lp) {
                dres[j] = (c[j] - dprod[j] - dslack[j]) * dcum[j];
            } else {
                const double g = qx[j] + c[j] - dprod[j];
                const double t = xh[j] - tau * g;
                const double pt = std::fmax(vlb[j], std::fmin(vub[j], t));
                const double ds = (pt - t) / tau;
                dres[j] = (g - ds) * dcum[j];
                dslack[j] = ds;
            }
        }
        abs_p = (linf ? amax(rres) : nrm2(rres)) / cbr;
        abs_d = (linf ? amax(dres) : nrm2(dres)) / ovr;
        const double half = (qtype == FA_CP_NON_Q) ? 0.0 : 0.5 * dot(xh, qx);
        pobj = (dot(c, xh) + half) / (cbr * ovr) + c0;
        const double base = dot(dslack, xh);
        dobj = (base + vsum(pslack) - half) / (cbr * ovr) + c0;
        rel_p = abs_p / (1.0 + bnd_norm);
        if (is_lp) {
            rel_d = abs_d / (1.0 + obj_norm);
        } else {
            for (int j = 0; j < n; ++j) {
                dprod[j] = dprod[j] * dcum[j];
                qx[j] = qx[j] * dcum[j];
            }
            const double qn = linf ? amax(qx) : nrm2(qx);
            const double an = linf ? amax(dprod) : nrm2(dprod);
            rel_d = abs_d / (1.0 + std::fmax(obj_norm, std::fmax(qn / ovr, an / ovr)));
        }
        gap = std::fabs(pobj - dobj);
        rel_gap = gap / (1.0 + std::fabs(pobj) + std::fabs(dobj));
    }
    void infeasibility() { /* 1028-1132 */
        for (int j = 0; j < n; ++j) {
            if (std::isfinite(vlb[j])) dx[j] = std::fmax(dx[j], 0.0);
            if (std::isfinite(vub[j])) dx[j] = std::fmin(dx[j], 0.0);
        }
        for (int i = 0; i < m; ++i) {
            if (!std::isfinite(clb[i])) dy[i] = std::fmin(dy[i], 0.0);
            if (!std::isfinite(cub[i])) dy[i] = std::fmax(dy[i], 0.0);
        }
        const double pnorm = amax(dx);
        if (pnorm > 0.0) {
            const double s = 1.0 / pnorm;
            for (double &v : dx) v = s * v;
        }
        const double dnorm = amax(dy);
        spmv(A, dx.data(), pprod.data());
        spmv(At, dy.data(), dprod.data());
        pray_lin = dot(c, dx) / (cbr * ovr);
        for (int i = 0; i < m; ++i)
            pslack[i] = std::fmax(dy[i], 0.0) * clb_fin[i] + std::fmin(dy[i], 0.0) * cub_fin[i];
        for (int j = 0; j < n; ++j)
            dslack[j] = std::fmax(-dprod[j], 0.0) * vlb_fin[j] + std::fmin(-dprod[j], 0.0) * vub_fin[j];
        dray_obj = (vsum(pslack) + vsum(dslack)) / (cbr * ovr);
        for (int i = 0; i < m; ++i) {
            const double p = pprod[i];
            pslack[i] = (std::fmax(0.0, -p) * (double)std::isfinite(clb[i]) +
                         std::fmax(0.0, p) * (double)std::isfinite(cub[i])) *
                        rcum[i];
        }
        for (int j = 0; j < n; ++j) {
            const double d = -dprod[j];
            dslack[j] = (std::fmax(0.0, d) * (double)!std::isfinite(vlb[j]) -
                         std::fmin(0.0, d) * (double)!std::isfinite(vub[j])) *
                        dcum[j];
        }
        max_pray = amax(pslack);
        if (!is_lp && qtype != FA_CP_NON_Q) {
            obj_product(dx);
            max_pray = std::fmax(max_pray, amax(qx) / ovr);
        }
        const double dsn = amax(dslack);
        max_dray = dsn;
        const double sf = std::fmax(dnorm, dsn);
        if (sf > 0.0) {
            max_dray /= sf;
            dray_obj /= sf;
        } else {
            max_dray = 0.0;
            dray_obj = 0.0;
        }
    }
    void check_termination(double elapsed) { /* utils.cu:438-462 */
        const auto &T = P->termination_criteria;
        if (rel_d < T.eps_feasible_relative && rel_p < T.eps_feasible_relative && rel_gap < T.eps_optimal_relative) {
            reason = TERMINATION_REASON_OPTIMAL;
            return;
        }
        if (dray_obj > 0.0 && max_dray / dray_obj <= T.eps_infeasible) {
            reason = TERMINATION_REASON_PRIMAL_INFEASIBLE;
            return;
        }
        if (pray_lin < 0.0 && max_pray / (-pray_lin) <= T.eps_infeasible) {
            reason = TERMINATION_REASON_DUAL_INFEASIBLE;
            return;
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
    bool should_restart() { /* utils.cu:464-492 */
        const auto &R = P->restart_params;
        const int F = P->termination_evaluation_frequency;
        bool rs = false;
        if (total == F) {
            rs = true;
        } else if (total > F) {
            if (fp <= R.sufficient_reduction_for_restart * fp0) rs = true;
            if (fp <= R.necessary_reduction_for_restart * fp0 && fp > fp_last) rs = true;
            if (inner >= R.artificial_restart_threshold * total) rs = true;
        }
        fp_last = fp;
        return rs;
    }

    /* ---------- sigma rules (fa_cp_core_op.cu:650-906) ---------- */
    void set_sigma_active(double s, double zt) {
        if (!std::isfinite(s) || s <= zt) {
            al_sigma = 0.0;
            use_al = false;
        } else {
            al_sigma = s;
            use_al = al_available;
        }
    }
    double clipped(double cur, double ratio) const {
        double gain = sane_positive(P->sigma_update_gain, 0.5);
        double lo = sane_positive(P->sigma_clip_low, 0.6), hi = sane_positive(P->sigma_clip_high, 1.7);
        if (lo > hi) std::swap(lo, hi);
        ratio = sane_positive(ratio, 1.0);
        double f = std::pow(ratio, gain);
        f = std::fmin(std::fmax(f, lo), hi);
        return cur * f;
    }
    void update_sigma(double pd, double dd, double normal) {
        const auto rule = P->sigma_update_rule;
        const bool bal = rule == FA_CP_SIGMA_UPDATE_BALANCED_GUARDED;
        const bool guarded = rule == FA_CP_SIGMA_UPDATE_GUARDED || bal;
        if (!al_available || rule == FA_CP_SIGMA_UPDATE_FIXED) return;
        if (!guarded && !use_al) return;
        const double ref = bal ? sane_positive(step * pw, 1.0) : 1.0;
        double smin = sane_positive(P->sigma_min, 1e-8) * ref;
        double smax = sane_positive(P->sigma_max, 10.0) * ref;
        const double zt = sane_positive(P->sigma_zero_threshold, sane_positive(P->sigma_min, 1e-8)) * ref;
        if (smin > smax) std::swap(smin, smax);
        if (zt > smin) smin = zt;
        const double cur = use_al ? std::fmin(std::fmax(sane_positive(al_sigma, smin), smin), smax) : 0.0;
        set_sigma_active(cur, zt);
        const double eps = 1e-300;
        const double rp = sane_positive(rel_p, eps), rd = sane_positive(rel_d, eps), rg = sane_positive(rel_gap, eps);
        const double score = std::fmax(score_component(rel_p), std::fmax(score_component(rel_d), score_component(rel_gap)));
        if (!std::isfinite(score)) return;
        if (!std::isfinite(best_sigma_score) || score < best_sigma_score) {
            best_sigma_score = score;
            best_al_sigma = cur;
        }
        if (P->sigma_rollback_tol > 0.0 && (!guarded || cur > zt) && std::isfinite(best_sigma_score) &&
            best_sigma_score > 0.0 && score > P->sigma_rollback_tol * best_sigma_score &&
            std::isfinite(best_al_sigma) && (guarded ? best_al_sigma >= 0.0 : best_al_sigma > 0.0)) {
            const double bs = (guarded && best_al_sigma <= zt) ? 0.0 : std::fmin(std::fmax(best_al_sigma, smin), smax);
            set_sigma_active(bs, zt);
            last_sigma_score = score;
            last_rp = rp;
            last_rd = rd;
            last_rg = rg;
            sigma_updates++;
            return;
        }
        double prop = cur;
        switch (rule) {
        case FA_CP_SIGMA_UPDATE_RESIDUAL_BALANCE:
            prop = clipped(cur, rp / rd);
            break;
        case FA_CP_SIGMA_UPDATE_KKT_BALANCE:
            prop = clipped(cur, rp / std::fmax(rd, rg));
            break;
        case FA_CP_SIGMA_UPDATE_DISPLACEMENT:
            if (std::isfinite(pd) && std::isfinite(dd) && pd > 1e-16 && dd > 1e-16) {
                const double target = std::fmin(std::fmax(dd / pd, smin), smax);
                prop = clipped(cur, target / cur);
            }
            break;
        case FA_CP_SIGMA_UPDATE_PROGRESS: {
            const double last_other = std::fmax(last_rd, last_rg);
            const double other = std::fmax(rd, rg);
            if (std::isfinite(last_rp) && std::isfinite(last_other) && last_rp > 0.0 && last_other > 0.0)
                prop = clipped(cur, (last_other / other) / (last_rp / rp));
            else
                prop = clipped(cur, rp / std::fmax(rd, rg));
            break;
        }
        case FA_CP_SIGMA_UPDATE_GREEDY_SCORE:
            if (sigma_updates == 0)
                sigma_dir = (rp >= std::fmax(rd, rg)) ? 1 : -1;
            else if (std::isfinite(score) && std::isfinite(last_sigma_score) && score > last_sigma_score)
                sigma_dir *= -1;
            prop = clipped(cur, sigma_dir > 0 ? P->sigma_clip_high : P->sigma_clip_low);
            break;
        case FA_CP_SIGMA_UPDATE_GUARDED:
        case FA_CP_SIGMA_UPDATE_BALANCED_GUARDED: {
            const bool normal_ok = !std::isfinite(normal) || normal > sane_positive(P->sigma_normal_motion_threshold, 1e-10);
            const bool zero_ok =
                !std::isfinite(normal) || normal > std::fmax(sane_positive(P->sigma_normal_motion_threshold, 1e-10), 2e-1);
            const bool bottleneck = rp >= sane_positive(P->sigma_activation_threshold, 2.0) *
                                              sane_positive(std::fmax(rd, rg), 1e-300);
            const bool zero_stalled = cur <= zt && std::isfinite(last_sigma_score) && score > 0.9 * last_sigma_score;
            const bool primal_signal = rp >= 0.5 * sane_positive(rd, 1e-300);
            const double act = sane_positive(P->sigma_activation_value, 0.1) * ref;
            const bool scale_ok = !bal || act >= 1e-6;
            const bool activate =
                cur <= zt ? (zero_ok && zero_stalled && primal_signal && scale_ok) : (normal_ok && bottleneck);
            if (cur <= zt)
                prop = activate ? act : 0.0;
            else if (!normal_ok)
                prop = clipped(cur, P->sigma_clip_low);
            else if (activate)
                prop = clipped(cur, rp / std::fmax(rd, rg));
            else
                prop = clipped(cur, P->sigma_clip_low);
            break;
        }
        default:
            break;
        }
        if (prop > zt)
            prop = std::fmin(std::fmax(prop, smin), smax);
        else
            prop = 0.0;
        set_sigma_active(prop, zt);
        last_sigma_score = score;
        last_rp = rp;
        last_rd = rd;
        last_rg = rg;
        sigma_updates++;
    }
    void perform_restart() { /* 908-1020, target "current" */
        for (int j = 0; j < n; ++j) dx[j] = xh[j] - x0[j];
        for (int i = 0; i < m; ++i) dy[i] = yh[i] - y0[i];
        const double pd = nrm2(dx), dd = nrm2(dy);
        double normal = INFINITY;
        if (pd > 1e-16 && std::isfinite(pd)) {
            spmv(A, dx.data(), pprod.data());
            normal = nrm2(pprod) / pd;
        }
        const double ratio = rel_d / rel_p;
        const auto &R = P->restart_params;
        if (pd > 1e-16 && dd > 1e-16 && pd < 1e12 && dd < 1e12 && ratio > 1e-8 && ratio < 1e8) {
            const double err = std::log(dd) - std::log(pd) - std::log(pw);
            pw_esum *= R.i_smooth;
            pw_esum += err;
            const double de = err - pw_last;
            pw *= std::exp(R.k_p * err + R.k_i * pw_esum + R.k_d * de);
            pw_last = err;
        } else {
            pw = best_pw;
            pw_esum = 0.0;
            pw_last = 0.0;
        }
        const double g = std::fabs(std::log10(rel_d / rel_p));
        if (g < best_gap) {
            best_gap = g;
            best_pw = pw;
        }
        update_sigma(pd, dd, normal);
        x0 = xh;
        y0 = yh;
        x = xh;
        y = yh;
        inner = 0;
        fp_last = INFINITY;
    }
};

/* ---------- feasibility polishing (fa_cp_core_op.cu:1241-1735) ----------
 * Two phases after the solve, each the same iteration and loop as the solve
 * on a feasibility problem: the primal phase drops the objective (c = 0,
 * constant 0) and starts from the solve's primal iterates with the dual
 * iterates at zero; the dual phase sets every finite bound to zero and starts
 * from the solve's dual iterates (and dual slack) with the primal iterates
 * at zero.  Both take the primal weight of the start of the solve, restart by
 * the solve's rule on a one-sided fixed-point error (|x_bar - x|^2 w, or
 * |y_bar - y|^2 / w, no square root) by moving the anchor to the current
 * point (no weight or sigma update), and stop when their relative residual is
 * at most eps_feas_polish_relative (utils.cu:1360-1384).  Like the
 * reference's loop, a phase runs one more iteration after its stopping test
 * and reports total - 1 iterations. */
struct PolishOut {
    termination_reason_t reason;
    int total;
    double abs_r, rel_r, obj;
    std::vector<double> sol; /* the phase's primal (dual) solution */
};

void polish_residual(QP &S, const QP &ori, bool primal) { /* utils.cu:1491-1574 */
    const bool linf = S.P->optimality_norm == NORM_TYPE_L_INF;
    if (primal) {
        spmv(S.A, S.xh.data(), S.pprod.data());
        for (int i = 0; i < S.m; ++i) {
            const double cl = std::fmax(S.clb[i], std::fmin(S.pprod[i], S.cub[i]));
            S.rres[i] = (S.pprod[i] - cl) * S.rcum[i];
        }
        S.abs_p = (linf ? amax(S.rres) : nrm2(S.rres)) / S.cbr;
        S.rel_p = S.abs_p / (1.0 + S.bnd_norm);
        S.pobj = dot(ori.c, S.xh) / (S.cbr * S.ovr) + S.c0;
    } else {
        spmv(S.At, S.yh.data(), S.dprod.data());
        for (int j = 0; j < S.n; ++j) S.dres[j] = (S.c[j] - S.dprod[j] - S.dslack[j]) * S.dcum[j];
        for (int i = 0; i < S.m; ++i)
            S.pslack[i] = std::fmax(S.yh[i], 0.0) * ori.clb_fin[i] + std::fmin(S.yh[i], 0.0) * ori.cub_fin[i];
        S.abs_d = (linf ? amax(S.dres) : nrm2(S.dres)) / S.ovr;
        S.rel_d = S.abs_d / (1.0 + S.obj_norm);
        S.dobj = (dot(S.dslack, ori.xh) + vsum(S.pslack)) / (S.cbr * S.ovr) + S.c0;
    }
}

PolishOut polish_phase(const QP &ori, bool primal, double pw0, std::chrono::steady_clock::time_point t0) {
    QP S = ori; /* *state copy (fa_cp_core_op.cu:1410-1478, 1525-1607) */
    const int n = S.n, m = S.m;
    auto zero = [](std::vector<double> &v) { std::fill(v.begin(), v.end(), 0.0); };
    if (primal) {
        zero(S.c);
        S.c0 = 0.0;
        zero(S.y0), zero(S.y), zero(S.yh), zero(S.ybar), zero(S.dprod);
        zero(S.dslack);
    } else {
        auto zf = [](std::vector<double> &v) {
            for (double &e : v)
                if (std::isfinite(e)) e = 0.0;
        };
        zf(S.clb), zf(S.cub), zf(S.vlb), zf(S.vub);
        zero(S.clb_fin), zero(S.cub_fin), zero(S.vlb_fin), zero(S.vub_fin);
        zero(S.x0), zero(S.x), zero(S.xh), zero(S.xbar), zero(S.pprod);
    }
    zero(S.aldual), zero(S.pslack), zero(S.dres), zero(S.rres), zero(S.dx), zero(S.dy);
    (void)n, (void)m;
    S.pw_esum = 0.0;
    S.pw_last = 0.0;
    S.fp = S.fp0 = S.fp_last = INFINITY;
    S.major = false;
    S.total = S.inner = 0;
    S.reason = TERMINATION_REASON_UNSPECIFIED;
    S.best_gap = INFINITY;
    if (primal) {
        S.rel_d = S.abs_d = S.rel_gap = S.gap = 0.0;
    } else {
        S.rel_p = S.abs_p = S.rel_gap = S.gap = 0.0;
    }
    S.pw = S.best_pw = pw0;
    const auto &T = S.P->termination_criteria;
    const int F = S.P->termination_evaluation_frequency;
    const auto tp = std::chrono::steady_clock::now();
    (void)t0;
    bool do_restart = false;
    while (S.reason == TERMINATION_REASON_UNSPECIFIED) { /* fa_cp_core_op.cu:1313-1355, 1362-1404 */
        if (S.major || S.total == 0 || S.total % print_frequency(S.total) == 0) {
            polish_residual(S, ori, primal);
            const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count();
            if ((primal ? S.rel_p : S.rel_d) <= T.eps_feas_polish_relative)
                S.reason = TERMINATION_REASON_FEAS_POLISH_SUCCESS;
            else if (S.total >= T.iteration_limit)
                S.reason = TERMINATION_REASON_ITERATION_LIMIT;
            else if (elapsed >= T.time_sec_limit)
                S.reason = TERMINATION_REASON_TIME_LIMIT;
        }
        if (S.major || S.total == 0) {
            do_restart = S.should_restart();
            if (do_restart) { /* fa_cp_core_op.cu:1649-1668 */
                if (primal) {
                    S.x0 = S.xh;
                    S.x = S.xh;
                } else {
                    S.y0 = S.yh;
                    S.y = S.yh;
                }
                S.inner = 0;
                S.fp_last = INFINITY;
            }
        }
        S.major = ((S.total + 1) % F) == 0;
        S.update();
        if (S.major || do_restart) { /* fa_cp_core_op.cu:1705-1735 */
            double s = 0.0;
            if (primal) {
                for (int j = 0; j < S.n; ++j) s += (S.xbar[j] - S.x[j]) * (S.xbar[j] - S.x[j]);
                S.fp = s * S.pw;
            } else {
                for (int i = 0; i < S.m; ++i) s += (S.ybar[i] - S.y[i]) * (S.ybar[i] - S.y[i]);
                S.fp = s / S.pw;
            }
            if (do_restart) {
                S.fp0 = S.fp;
                do_restart = false;
            }
        }
        S.halpern();
        S.inner++;
        S.total++;
    }
    return PolishOut{S.reason, S.total, primal ? S.abs_p : S.abs_d, primal ? S.rel_p : S.rel_d,
                     primal ? S.pobj : S.dobj, primal ? S.xh : S.yh};
}

quad_obj_type_t detect_q_type(const Csr &Q, const Csr &R) { /* utils.cu:1576-1616 */
    if (Q.nnz() == 0 && R.nnz() == 0) return FA_CP_NON_Q;
    if (R.nnz() > 0) return Q.nnz() > 0 ? FA_CP_LOW_RANK_PLUS_SPARSE_Q : FA_CP_LOW_RANK_Q;
    for (int i = 0; i < Q.nr; ++i)
        for (int k = Q.rp[i]; k < Q.rp[i + 1]; ++k)
            if (Q.ci[k] != i) return FA_CP_SPARSE_Q;
    return FA_CP_DIAG_Q;
}

double norm_of(const double *v, int len, bool linf) {
    double s = 0.0, mx = 0.0;
    for (int i = 0; i < len; ++i) {
        if (linf)
            mx = std::fmax(mx, std::fabs(v[i]));
        else
            s += v[i] * v[i];
    }
    return linf ? mx : std::sqrt(s);
}

} // namespace

extern "C" {

void oracle_facp_default_parameters(fa_cp_parameters_t *p) { /* QP/FA_CP/src/utils.cu:494-537 */
    memset(p, 0, sizeof(*p));
    p->l_inf_ruiz_iterations = 10;
    p->has_pock_chambolle_alpha = true;
    p->pock_chambolle_alpha = 1.0;
    p->bound_objective_rescaling = true;
    p->trajectory_csv = nullptr;
    p->use_al_qp = true;
    p->al_sigma = 0.0;
    p->sigma_update_rule = FA_CP_SIGMA_UPDATE_GUARDED;
    p->sigma_update_gain = 0.5;
    p->sigma_clip_low = 0.6;
    p->sigma_clip_high = 1.7;
    p->sigma_min = 1e-8;
    p->sigma_max = 10.0;
    p->sigma_rollback_tol = 1.25;
    p->sigma_zero_threshold = 1e-8;
    p->sigma_activation_threshold = 2.0;
    p->sigma_normal_motion_threshold = 1e-10;
    p->sigma_activation_value = 0.1;
    p->verbose = 1;
    p->termination_evaluation_frequency = 200;
    p->feasibility_polishing = false;
    p->reflection_coefficient = 1.0;
    p->sv_max_iter = 5000;
    p->sv_tol = 1e-4;
    p->termination_criteria.eps_optimal_relative = 1e-4;
    p->termination_criteria.eps_feasible_relative = 1e-4;
    p->termination_criteria.eps_infeasible = 1e-10;
    p->termination_criteria.time_sec_limit = 3600.0;
    p->termination_criteria.iteration_limit = 2147483647;
    p->termination_criteria.eps_feas_polish_relative = 1e-6;
    p->restart_params.artificial_restart_threshold = 0.36;
    p->restart_params.sufficient_reduction_for_restart = 0.2;
    p->restart_params.necessary_reduction_for_restart = 0.8;
    p->restart_params.k_p = 0.99;
    p->restart_params.k_i = 0.01;
    p->restart_params.k_d = 0.0;
    p->restart_params.i_smooth = 0.3;
    p->optimality_norm = NORM_TYPE_L_INF;
}

fa_cp_result_t *oracle_facp_solve(const qp_problem_t *prob, const fa_cp_parameters_t *params) {
    g_polish_status[0] = g_polish_status[1] = -1;
    if (!prob || !params || params->termination_evaluation_frequency < 1) return nullptr;
    auto t0 = std::chrono::steady_clock::now();
    std::unique_ptr<QP> SP(new QP());
    QP &S = *SP;
    S.P = params;
    S.n = prob->num_variables;
    S.m = prob->num_constraints;
    S.nr = prob->num_rank_lowrank_obj;
    const int n = S.n, m = S.m;
    S.A = from_component(prob->constraint_matrix, m, n, prob->constraint_matrix_num_nonzeros);
    S.Q = from_component(prob->objective_sparse_matrix, n, n, prob->objective_sparse_matrix_num_nonzeros);
    S.R = from_component(prob->objective_lowrank_matrix, S.nr, n, prob->objective_lowrank_matrix_num_nonzeros);
    S.c.assign(prob->objective_vector, prob->objective_vector + n);
    S.vlb.assign(prob->variable_lower_bound, prob->variable_lower_bound + n);
    S.vub.assign(prob->variable_upper_bound, prob->variable_upper_bound + n);
    S.clb.assign(prob->constraint_lower_bound, prob->constraint_lower_bound + m);
    S.cub.assign(prob->constraint_upper_bound, prob->constraint_upper_bound + m);
    S.c0 = prob->objective_constant;
    S.rescale();
    S.At = transpose(S.A);
    S.Rt = transpose(S.R);
    double rescale_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    /* state (solver_state.cu:494-877) */
    for (auto *v : {&S.x0, &S.x, &S.xh, &S.xbar, &S.dprod, &S.dslack, &S.dres, &S.dx, &S.qx, &S.grad, &S.dir,
                    &S.pbuf})
        v->assign(n, 0.0);
    for (auto *v : {&S.y0, &S.y, &S.yh, &S.ybar, &S.pprod, &S.aldual, &S.pslack, &S.rres, &S.dy}) v->assign(m, 0.0);
    S.rx.assign(S.nr, 0.0);
    if (prob->primal_start)
        for (int i = 0; i < n; ++i) S.x0[i] = S.x[i] = S.xh[i] = prob->primal_start[i] * S.dcum[i] * S.cbr;
    if (prob->dual_start)
        for (int i = 0; i < m; ++i) S.y0[i] = S.y[i] = S.yh[i] = prob->dual_start[i] * S.rcum[i] * S.ovr;
    S.clb_fin.resize(m);
    S.cub_fin.resize(m);
    S.vlb_fin.resize(n);
    S.vub_fin.resize(n);
    for (int i = 0; i < m; ++i) {
        S.clb_fin[i] = std::isfinite(S.clb[i]) ? S.clb[i] : 0.0;
        S.cub_fin[i] = std::isfinite(S.cub[i]) ? S.cub[i] : 0.0;
    }
    for (int i = 0; i < n; ++i) {
        S.vlb_fin[i] = std::isfinite(S.vlb[i]) ? S.vlb[i] : 0.0;
        S.vub_fin[i] = std::isfinite(S.vub[i]) ? S.vub[i] : 0.0;
    }
    const bool linf = params->optimality_norm == NORM_TYPE_L_INF;
    S.obj_norm = norm_of(prob->objective_vector, n, linf);
    {
        double s = 0.0, mx = 0.0;
        for (int i = 0; i < m; ++i) {
            const double lo = prob->constraint_lower_bound[i], up = prob->constraint_upper_bound[i];
            if (linf) {
                if (std::isfinite(lo) && lo != up) mx = std::fmax(mx, std::fabs(lo));
                if (std::isfinite(up)) mx = std::fmax(mx, std::fabs(up));
            } else {
                if (std::isfinite(lo) && lo != up) s += lo * lo;
                if (std::isfinite(up)) s += up * up;
            }
        }
        S.bnd_norm = linf ? mx : std::sqrt(s);
    }
    S.al_available = params->use_al_qp;
    S.use_al = params->use_al_qp;
    S.al_sigma = params->al_sigma;
    S.best_al_sigma = params->al_sigma;
    S.qtype = detect_q_type(S.Q, S.R);
    S.is_lp = S.qtype == FA_CP_NON_Q;
    if (S.qtype == FA_CP_DIAG_Q) { /* solver_state.cu:252-270 */
        S.diag.assign(n, 0.0);
        for (int i = 0; i < n; ++i)
            for (int k = S.Q.rp[i]; k < S.Q.rp[i + 1]; ++k)
                if (S.Q.ci[k] < n) S.diag[S.Q.ci[k]] = S.Q.v[k] + 1e-12;
        double mx = 0.0, mn = 0.0;
        for (int i = 0; i < n; ++i) {
            mx = std::fmax(mx, std::fabs(S.diag[i]));
            mn = std::fmin(mn, S.diag[i]);
        }
        S.qnorm = mx;
        S.nonconvexity = mn;
    } else if (S.qtype == FA_CP_SPARSE_Q) { /* solver_state.cu:462-475 */
        srand(1);
        S.qnorm = S.q_max_eig();
        S.nonconvexity = S.q_min_eig(S.qnorm);
    }
    if (S.al_available && params->al_sigma <= params->sigma_zero_threshold) {
        S.use_al = false;
        S.al_sigma = 0.0;
    }
    /* initialize_inner_solver (solver_state.cu:305-360) */
    S.has_inner = S.use_al || S.al_available || !(S.qtype == FA_CP_NON_Q || S.qtype == FA_CP_DIAG_Q);
    S.inner_limit = 1000;
    S.inner_tol = 1e-3;
    if (S.nonconvexity < 0) S.inner_limit = 1;
    /* initialize_step_size_and_primal_weight (fa_cp_core_op.cu:1022-1040) */
    S.step = (S.A.nnz() == 0) ? 1.0 : 0.998 / S.max_singular_value();
    S.pw = params->bound_objective_rescaling ? 1.0 : (S.obj_norm + 1.0) / (S.bnd_norm + 1.0);
    S.best_pw = S.pw;

    const auto t_start = std::chrono::steady_clock::now();
    const int F = params->termination_evaluation_frequency;
    bool do_restart = false;
    double elapsed = 0.0;
    while (S.total < params->termination_criteria.iteration_limit) { /* solver.cu:94-144 */
        const bool consider = S.major || S.total == 0;
        bool planned = false;
        if (consider || (S.total % print_frequency(S.total) == 0)) {
            S.residual();
            if (S.major && S.total < 3 * F) S.infeasibility();
            elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
            S.check_termination(elapsed);
            if (g_trace)
                fprintf(stderr, "[facp-oracle] it %d rp %.6e rd %.6e gap %.6e pobj %.12e dobj %.12e fp %.6e pw %.6e sigma %.3e inner %d\n",
                        S.total, S.rel_p, S.rel_d, S.rel_gap, S.pobj, S.dobj, S.fp, S.pw, S.al_sigma, S.inner_total);
            if (consider && S.reason == TERMINATION_REASON_UNSPECIFIED) planned = S.should_restart();
            if (S.reason != TERMINATION_REASON_UNSPECIFIED) break;
        }
        if (consider) {
            do_restart = planned;
            if (do_restart) S.perform_restart();
        }
        S.major = ((S.total + 1) % F) == 0;
        S.update();
        if (S.major || do_restart) {
            S.fixed_point_error();
            if (do_restart) {
                S.fp0 = S.fp;
                do_restart = false;
            }
        }
        S.halpern();
        S.inner++;
        S.total++;
    }
    if (S.reason == TERMINATION_REASON_UNSPECIFIED) {
        S.reason = TERMINATION_REASON_ITERATION_LIMIT;
        S.residual();
    }
    elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();

    /* solver.cu:156-160: polishing after the solve, except after an
     * infeasibility status; built for problems without Q (for a QP the
     * reference's dual phase keeps a stale dual slack and does not converge) */
    int polish_iters = 0;
    double polish_sec = 0.0;
    if (params->feasibility_polishing && S.reason != TERMINATION_REASON_DUAL_INFEASIBLE &&
        S.reason != TERMINATION_REASON_PRIMAL_INFEASIBLE && S.qtype == FA_CP_NON_Q) {
        const auto &T = params->termination_criteria;
        const auto tp = std::chrono::steady_clock::now();
        /* fa_cp_core_op.cu:1244-1252: nothing to do when already feasible */
        if (!(S.rel_p < T.eps_feas_polish_relative && S.rel_d < T.eps_feas_polish_relative)) {
            const double pw0 = params->bound_objective_rescaling ? 1.0 : (S.obj_norm + 1.0) / (S.bnd_norm + 1.0);
            PolishOut po = polish_phase(S, true, pw0, tp);
            if (po.reason == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
                S.xh = po.sol;
                S.abs_p = po.abs_r;
                S.rel_p = po.rel_r;
                S.pobj = po.obj;
            }
            polish_iters += po.total - 1;
            PolishOut pd = polish_phase(S, false, pw0, tp);
            if (pd.reason == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
                S.yh = pd.sol;
                S.abs_d = pd.abs_r;
                S.rel_d = pd.rel_r;
                S.dobj = pd.obj;
            }
            polish_iters += pd.total - 1;
            S.gap = std::fabs(S.pobj - S.dobj);
            S.rel_gap = S.gap / (1.0 + std::fabs(S.pobj) + std::fabs(S.dobj));
            g_polish_status[0] = po.reason;
            g_polish_status[1] = pd.reason;
        }
        polish_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - tp).count();
    }

    /* result (fa_cp_core_op.cu:1171-1239) */
    fa_cp_result_t *r = (fa_cp_result_t *)calloc(1, sizeof(fa_cp_result_t));
    r->primal_solution = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    r->dual_solution = (double *)malloc(sizeof(double) * (m > 0 ? m : 1));
    r->reduced_cost = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    spmv(S.At, S.yh.data(), S.dprod.data());
    for (int j = 0; j < n; ++j) {
        r->reduced_cost[j] = (S.c[j] - S.dprod[j]) * S.dcum[j] / S.ovr;
        r->primal_solution[j] = S.xh[j] / S.dcum[j] / S.cbr;
    }
    for (int i = 0; i < m; ++i) r->dual_solution[i] = S.yh[i] / S.rcum[i] / S.ovr;
    r->num_variables = n;
    r->num_constraints = m;
    r->num_nonzeros = prob->constraint_matrix_num_nonzeros;
    r->total_count = S.total;
    r->total_inner_count = S.inner_total;
    r->rescaling_time_sec = rescale_sec;
    r->cumulative_time_sec = elapsed;
    r->absolute_primal_residual = S.abs_p;
    r->relative_primal_residual = S.rel_p;
    r->absolute_dual_residual = S.abs_d;
    r->relative_dual_residual = S.rel_d;
    r->primal_objective_value = S.pobj;
    r->dual_objective_value = S.dobj;
    r->objective_gap = S.gap;
    r->relative_objective_gap = S.rel_gap;
    r->max_primal_ray_infeasibility = S.max_pray;
    r->max_dual_ray_infeasibility = S.max_dray;
    r->primal_ray_linear_objective = S.pray_lin;
    r->dual_ray_objective = S.dray_obj;
    r->final_al_sigma = S.al_sigma;
    r->sigma_update_count = S.sigma_updates;
    r->sigma_update_rule = S.al_available ? params->sigma_update_rule : FA_CP_SIGMA_UPDATE_FIXED;
    r->termination_reason = S.reason;
    r->feasibility_iteration = polish_iters;
    r->feasibility_polishing_time = polish_sec;
    return r;
}

/* Only the equilibration of oracle_facp_solve: column and row scales and
 * {cbr, ovr}. */
int oracle_facp_scaling(const qp_problem_t *prob, const fa_cp_parameters_t *params, double *dcum, double *rcum,
                        double *cbr_ovr) {
    if (!prob || !params) return -1;
    std::unique_ptr<QP> SP(new QP());
    QP &S = *SP;
    S.P = params;
    S.n = prob->num_variables;
    S.m = prob->num_constraints;
    S.nr = prob->num_rank_lowrank_obj;
    const int n = S.n, m = S.m;
    S.A = from_component(prob->constraint_matrix, m, n, prob->constraint_matrix_num_nonzeros);
    S.Q = from_component(prob->objective_sparse_matrix, n, n, prob->objective_sparse_matrix_num_nonzeros);
    S.R = from_component(prob->objective_lowrank_matrix, S.nr, n, prob->objective_lowrank_matrix_num_nonzeros);
    S.c.assign(prob->objective_vector, prob->objective_vector + n);
    S.vlb.assign(prob->variable_lower_bound, prob->variable_lower_bound + n);
    S.vub.assign(prob->variable_upper_bound, prob->variable_upper_bound + n);
    S.clb.assign(prob->constraint_lower_bound, prob->constraint_lower_bound + m);
    S.cub.assign(prob->constraint_upper_bound, prob->constraint_upper_bound + m);
    S.rescale();
    std::copy(S.dcum.begin(), S.dcum.end(), dcum);
    std::copy(S.rcum.begin(), S.rcum.end(), rcum);
    cbr_ovr[0] = S.cbr;
    cbr_ovr[1] = S.ovr;
    return 0;
}

void oracle_facp_set_trace(int on) { g_trace = on; }

/* statuses of the last solve's primal and dual polishing phases (-1: not run) */
void oracle_facp_polish_status(int *primal, int *dual) {
    *primal = g_polish_status[0];
    *dual = g_polish_status[1];
}

void oracle_facp_result_free(fa_cp_result_t *r) {
    if (!r) return;
    free(r->primal_solution);
    free(r->dual_solution);
    free(r->reduced_cost);
    free(r);
}

} // extern "C"
