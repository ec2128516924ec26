/*
 * cpal_control.h -- scalar control logic of the CP_AL iteration, compiled for
 * both the host (initial step schedule) and the device (the single-thread
 * controller kernel that ends every evaluation block).
 *
 * Running the decisions on the device is what lets the loop replay as a CUDA
 * graph: the reference does the same work on the host after about ten
 * host-synchronising cuBLAS reductions per block (LP/CP_AL/src/solver.cu:
 * 1343-1697).  The rules themselves are the reference's:
 *   step schedule      LP/CP_AL/src/solver.cu:3103-3139
 *   sigma parameters   LP/CP_AL/src/solver.cu:3141-3164
 *   fixed-point error  LP/CP_AL/src/solver.cu:3611-3686
 *   residual / KKT     LP/CP_AL/src/utils.cu:812-917
 *   termination        LP/CP_AL/src/utils.cu:275-317
 *   restart rule       LP/CP_AL/src/utils.cu:319-359
 *   restart (PID, sigma PID, best weight)  LP/CP_AL/src/solver.cu:2821-3101
 */
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define PDAL_HD __host__ __device__ __forceinline__
#else
#define PDAL_HD inline
#endif

namespace pdal {

/* Parameters the controller needs, resolved on the host once per solve. */
struct CpalParams {
    int F;                 /* termination_evaluation_frequency */
    int iteration_limit;
    double time_limit;
    double eps_opt, eps_feas;
    int norm_linf;
    double refl;           /* reflection coefficient */
    double suff, nec, art; /* restart thresholds (environment overrides applied) */
    double kp, ki, kd, ismooth;
    int sigma_mode, sigma_adaptive;
    double s_kp, s_ki, s_kd, s_ismooth, s_gain, s_umin, s_umax;
    double step_margin, lambda_factor;
    int lambda_param_set;
    double lambda_param_opt;
    double obj_norm, bnd_norm, obj_const;
    /* restart target selection (LP/CP_AL/src/solver.cu:2749-2819, two-point
     * modes): 0 off, 1 restart to the Halpern iterate when its score beats
     * the averaged point's within the margin, 2 always */
    int restart_select;
    int restart_select_min_iters;
    double restart_select_margin;
    double restart_select_min_time;
    int restart_threepoint; /* also score the plain Halpern point (mode 3 or the three-point switch) */
    /* infeasibility certificates (an opt-in extension: the reference never
     * evaluates them) */
    int infeas;
    double eps_infeas;
    /* benchmark controllers of the reference, off by default there and here.
     * Alpha pulse (LP/CP_AL/src/solver.cu:885-1032): once, at a restart after
     * 10,000 iterations with two recorded zero-alpha epochs, run one
     * evaluation block at alpha = 0.002 when the gate passes (pulse_force);
     * pulse_test_limit ends the solve once the pulse is over and this many
     * iterations are done. */
    int pulse, pulse_force, pulse_test_limit;
    /* sigma trigger (solver.cu:1496-1527): outside sigma mode, switch sigma
     * mode on and restart when the primal residual lags the dual one */
    int trigger, trigger_min_iters;
    double trigger_p, trigger_d, trigger_ratio;
    /* sigma initialisation the trigger repeats (solver.cu:3141-3164) */
    int sigma_set;
    double sigma_value, sigma_init_f, sigma_min_f, sigma_max_f;
    /* dynamic evaluation frequency (solver.cu:1229-1255, 1529-1583): blocks
     * of dyn_fast iterations instead of F once the residuals are lopsided
     * (dyn_resid), after dyn_sec seconds or dyn_iters iterations (unless
     * Curtis-Reid stopped early), or from the start until dyn_boot
     * iterations */
    int dyn, dyn_resid, dyn_fast, dyn_min_iters, dyn_boot, dyn_iters, cr_early_stopped;
    double dyn_sec, dyn_small, dyn_large, dyn_ratio;
};

/* Solver scalars, resident in device memory during the loop. */
struct CpalState {
    /* coefficients read by the iteration kernels */
    double tau, rho, beta, inv_tau, inv_prox, inv_beta, refl;
    /* the same coefficients rounded once to FP32 for the FP32 phase (the FP64
     * pipe of GB300 is too narrow to convert them in every thread) */
    float tau_f, rho_f, beta_f, inv_tau_f, inv_prox_f, inv_beta_f, refl_f, pad_f;
    int inner;   /* Halpern counter at the start of the current block */
    int status;  /* 0 while running, else termination_reason_t */
    int restart; /* 1 when the last evaluation restarted */
    int total;
    /* controller state */
    double step, pw, al_lambda, lambda_est;
    double sigma, sigma_base, sigma_min, sigma_max, sigma_best, sigma_esum, sigma_last, lambda_param;
    double pw_esum, pw_last, best_pw, best_gap;
    double fp, fp0, fp_last;
    double abs_p, abs_d, rel_p, rel_d, pobj, dobj, gap, rel_gap;
    double cbr, ovr;
    double elapsed;
    unsigned long long t_start_ns;
    int restarts;
    int sigma_on;
    int sigma_adapt;
    int phase_switch;      /* 1: the FP32 phase reached its switch tolerance or stalled */
    double fp32_switch_tol; /* < 0: no FP32 phase running */
    int iter_limit;        /* iteration limit (device copy, a session may extend it) */
    int fp32_stall_limit;  /* evaluations without a 2x KKT gain that end the FP32 phase */
    int fp32_stall;        /* evaluations since the FP32 phase last halved its best KKT */
    int restart_target; /* 1: the last restart went to the reflected Halpern iterate, 2: to the
                           plain Halpern point */
    double fp32_best_kkt;
    double restart_w; /* Halpern weight of the block's last iteration, for a restart to the plain
                         Halpern point w x^ + (1 - w) x0 */
    /* the last evaluation's ray quantities, normalised as the reference
     * reports them (infeasibility detection only) */
    double ray_pinf, ray_dinf, ray_pobj, ray_dobj;
    /* alpha pulse: phase 0 idle, 1 running its positive block, 2 over; gate 0
     * not evaluated, 1 passed, 2 rejected; the epoch being measured (valid
     * after the first restart) and the last two zero-alpha epochs */
    int pulse_phase, pulse_gate, pulse_start, pulse_status;
    int epoch_valid, epoch_total, hist_count;
    int hist_iters[2];
    double hist_fp_rate[2];
    double epoch_p, epoch_d, epoch_g;
    double pulse_fp, pulse_p, pulse_d, pulse_g;
    int trigger_iter; /* iteration at which the sigma trigger fired (0: never) */
    int F;            /* iterations of the next evaluation block */
    int dyn_latched;  /* the dynamic evaluation frequency switched to its fast value */
    int dyn_iter;     /* at this iteration (0: never) */
};

/* Reduction terms of one evaluation (finished sums / maxima). */
struct CpalEval {
    /* rows of A */
    double rp2, contrib, adx2, dy2, ddy2, axd2, rpmax;
    /* rows of A^T */
    double rd2, dx2, cross, cx, lx, ddx2, rdmax;
    /* restart target selection only: |A(x^ - x)|^2, |y^ - y|^2, |x^ - x|^2,
     * <A^T(y^ - y), x^ - x>, and the distances of the Halpern iterate from
     * the anchors |x - x0|^2, |y - y0|^2, |A x - A x0|^2 */
    double sel_ax2, sel_dy2, sel_dx2, sel_cross, cur_dx2, cur_dy2, cur_axd2;
    /* three-point selection only: <A^T(y^ - y0), x^ - x0> */
    double h_cross;
    /* infeasibility detection only, for the projected displacements
     * dx = P(x^ - x0), dy = P(y^ - y0): the largest unscaled violation of
     * A dx, max|dx|, c'dx; the largest unscaled dual-slack violation of
     * A^T dy, max|dy|, and the two dual-objective sums */
    double ray_pviol, ray_dxinf, ray_cdx, ray_dviol, ray_dyinf, ray_rowsum, ray_colsum;
};

PDAL_HD void cpal_set_coefficients(CpalState &s) {
    s.tau = s.step / s.pw;
    s.rho = s.step * s.pw;
    s.inv_tau = 1.0 / s.tau;
    s.inv_prox = 1.0 / (s.rho + s.beta);
    s.inv_beta = s.beta > 0.0 ? 1.0 / s.beta : 0.0;
    s.tau_f = (float)s.tau;
    s.rho_f = (float)s.rho;
    s.beta_f = (float)s.beta;
    s.inv_tau_f = (float)s.inv_tau;
    s.inv_prox_f = (float)s.inv_prox;
    s.inv_beta_f = (float)s.inv_beta;
    s.refl_f = (float)s.refl;
}

/* Halpern weights of the block that starts with counter `inner`:
 * entry i (1..F) holds w = k/(k+1) and 1 - w for k = inner + i
 * (LP/CP_AL/src/solver.cu:2355-2356), in FP64 and rounded to FP32. */
struct HalpernW {
    double w, omw;
};
struct HalpernWf {
    float w, omw;
};
PDAL_HD void cpal_halpern_entry(int inner, int i, HalpernW &d, HalpernWf &f) {
    const int k = inner + i;
    d.w = (double)k / (double)(k + 1);
    d.omw = 1.0 - d.w;
    f.w = (float)d.w;
    f.omw = (float)d.omw;
}

/* LP/CP_AL/src/solver.cu:3103-3139 */
PDAL_HD void cpal_refresh_step_schedule(CpalState &s, const CpalParams &p) {
    const double margin = p.step_margin;
    if (s.sigma_on) {
        const double sg = fmax(s.sigma, 0.0);
        if (sg <= 0.0) {
            s.beta = 0.0;
            s.lambda_param = 0.0;
            s.step = sqrt(fmax(margin / fmax(s.lambda_est, 1e-12), 1e-24));
            s.al_lambda = 0.0;
            return;
        }
        if (!isfinite(s.lambda_param) || s.lambda_param <= 0.0) {
            s.lambda_param = p.lambda_param_set ? p.lambda_param_opt : p.lambda_factor * fmax(s.lambda_est, 1e-12);
        }
        s.lambda_param = fmax(s.lambda_param, (2.0 + 1e-12) * fmax(s.lambda_est, 1e-12));
        const double tau = 1.0 / (sg * s.lambda_param);
        const double rho = sg;
        s.beta = sg;
        s.step = sqrt(fmax(tau * rho, 1e-24));
        s.pw = sqrt(fmax(rho / tau, 1e-24));
        s.al_lambda = 0.0;
        return;
    }
    s.al_lambda = fmin(fmax(s.al_lambda, 0.0), 0.95);
    const double eta_sq = margin * (1.0 - s.al_lambda) / fmax(s.lambda_est, 1e-12);
    s.step = sqrt(fmax(eta_sq, 1e-24));
    const double dual_step = s.step * fmax(s.pw, 1e-12);
    s.beta = dual_step * s.al_lambda / fmax(1.0 - s.al_lambda, 1e-12);
}

/* LP/CP_AL/src/solver.cu:3611-3686; the arguments are squared norms, taken
 * through sqrt and squared again as the reference does with nrm2 results. */
PDAL_HD double cpal_fixed_point_error(const CpalState &s, double pn2, double dn2, double axn2, double cross) {
    const double pn = sqrt(pn2), dn = sqrt(dn2), axn = sqrt(axn2);
    if (s.sigma_on && s.sigma > 0.0 && s.lambda_param > 0.0) {
        const double val = s.sigma * (s.lambda_param * pn * pn - axn * axn) + dn * dn / fmax(s.sigma, 1e-16);
        return sqrt(fmax(val, 0.0));
    }
    const double movement = pn * pn * s.pw + dn * dn / s.pw;
    const double interaction = 2 * s.step * cross;
    const double augmentation = s.step * s.beta * axn * axn;
    return sqrt(fmax(movement + interaction - augmentation, 0.0));
}

/* LP/CP_AL/src/utils.cu:812-917 (scalar tail of compute_residual) */
PDAL_HD void cpal_residual_scalars(CpalState &s, const CpalParams &p, const CpalEval &e) {
    if (p.norm_linf) {
        s.abs_p = e.rpmax;
        s.abs_d = e.rdmax;
    } else {
        s.abs_p = sqrt(e.rp2) / s.cbr;
        s.abs_d = sqrt(e.rd2);
    }
    s.abs_d /= s.ovr;
    s.pobj = e.cx / (s.cbr * s.ovr) + p.obj_const;
    s.dobj = (e.lx + e.contrib) / (s.cbr * s.ovr) + p.obj_const;
    s.rel_p = s.abs_p / (1.0 + p.bnd_norm);
    s.rel_d = s.abs_d / (1.0 + p.obj_norm);
    s.gap = fabs(s.pobj - s.dobj);
    s.rel_gap = s.gap / (1.0 + fabs(s.pobj) + fabs(s.dobj));
}

/* LP/CP_AL/src/utils.cu:319-359, F the iterations of the block just run */
PDAL_HD bool cpal_should_restart(CpalState &s, const CpalParams &p, int F) {
    bool rs = false;
    if (s.total == F) {
        rs = true;
    } else if (s.total > F) {
        if (s.fp <= p.suff * s.fp0) rs = true;
        if (s.fp <= p.nec * s.fp0 && s.fp > s.fp_last) rs = true;
        if (s.inner >= p.art * s.total) rs = true;
    }
    s.fp_last = s.fp;
    return rs;
}

/* Scalar part of LP/CP_AL/src/solver.cu:2821-3101 (restart target "current");
 * pd2/dd2 are the squared distances of (x^, y^) from the anchors, axd2 the
 * squared norm of A(x^ - x0). */
PDAL_HD void cpal_restart_scalars(CpalState &s, const CpalParams &p, double pd2, double dd2, double axd2) {
    const double pd = sqrt(pd2), dd = sqrt(dd2);
    const double ratio = s.rel_d / fmax(s.rel_p, 1e-300);
    if (s.sigma_on) {
        if (s.sigma_adapt) {
            const double axd = sqrt(axd2);
            const double dxm = s.lambda_param * pd * pd - axd * axd;
            if (dd > 1e-16 && dd < 1e12 && dxm > 1e-24 && dxm < 1e24 && isfinite(s.sigma) && s.sigma > 1e-16 &&
                ratio > 1e-8 && ratio < 1e8) {
                double err = log(fmax(dd, 1e-300)) - 0.5 * log(fmax(dxm, 1e-300)) - log(fmax(s.sigma, 1e-300));
                double bal = 0.5 * log(fmax(ratio, 1e-300));
                bal = fmax(-2.0, fmin(bal, 2.0));
                err += p.s_gain * bal;
                s.sigma_esum = p.s_ismooth * s.sigma_esum + err;
                const double de = err - s.sigma_last;
                double sr = exp(p.s_kp * err + p.s_ki * s.sigma_esum + p.s_kd * de);
                sr = fmin(fmax(sr, p.s_umin), p.s_umax);
                s.sigma *= sr;
                s.sigma_last = err;
            } else {
                s.sigma = s.sigma_best;
                s.sigma_esum = 0.0;
                s.sigma_last = 0.0;
            }
        }
        if (!isfinite(s.sigma) || s.sigma <= 1e-16) {
            s.sigma = s.sigma_best;
            s.sigma_esum = 0.0;
            s.sigma_last = 0.0;
        }
        s.sigma = fmin(fmax(s.sigma, s.sigma_min), s.sigma_max);
        const double g = fabs(log10(fmax(s.rel_d, 1e-300) / fmax(s.rel_p, 1e-300)));
        if (isfinite(g) && g < s.best_gap) {
            s.best_gap = g;
            s.sigma_best = s.sigma;
        }
        s.pw_esum = 0.0;
        s.pw_last = 0.0;
    } else {
        if (pd > 1e-16 && dd > 1e-16 && pd < 1e12 && dd < 1e12 && ratio > 1e-8 && ratio < 1e8) {
            const double err = log(dd) - log(pd) - log(s.pw);
            s.pw_esum *= p.ismooth;
            s.pw_esum += err;
            const double de = err - s.pw_last;
            s.pw *= exp(p.kp * err + p.ki * s.pw_esum + p.kd * de);
            s.pw_last = err;
        } else {
            s.pw = s.best_pw;
            s.pw_esum = 0.0;
            s.pw_last = 0.0;
        }
        const double g = fabs(log10(fmax(s.rel_d, 1e-300) / fmax(s.rel_p, 1e-300)));
        if (g < s.best_gap) {
            s.best_gap = g;
            s.best_pw = s.pw;
        }
    }
    cpal_refresh_step_schedule(s, p);
    s.inner = 0;
    s.fp_last = INFINITY;
    s.restarts++;
}

/* LP/CP_AL/src/solver.cu:415-428: the controllers' guarded magnitude and
 * log-rate per iteration */
PDAL_HD double ctl_metric(double v) { return fmax(fabs(v), 1e-300); }
PDAL_HD double ctl_log_rate(double a, double b, int k) {
    if (k <= 0 || !isfinite(a) || !isfinite(b)) return NAN;
    const double r = log(ctl_metric(a) / ctl_metric(b)) / (double)k;
    return isfinite(r) ? r : NAN;
}

/* LP/CP_AL/src/solver.cu:616-678: at a restart, an epoch run at alpha = 0 is
 * kept (the last two) when all of its rates are finite */
PDAL_HD void cpal_record_epoch(CpalState &s) {
    if (!s.epoch_valid || s.al_lambda > 0.0) return;
    const int k = s.total - s.epoch_total;
    const double fr = ctl_log_rate(s.fp0, s.fp, k);
    const double pr = ctl_log_rate(s.epoch_p, s.rel_p, k);
    const double dr = ctl_log_rate(s.epoch_d, s.rel_d, k);
    const double gr = ctl_log_rate(s.epoch_g, s.rel_gap, k);
    const double k0 = fmax(s.epoch_p, fmax(s.epoch_d, s.epoch_g));
    const double k1 = fmax(ctl_metric(s.rel_p), fmax(ctl_metric(s.rel_d), ctl_metric(s.rel_gap)));
    const double kr = ctl_log_rate(k0, k1, k);
    if (!(k > 0 && isfinite(fr) && isfinite(pr) && isfinite(dr) && isfinite(gr) && isfinite(kr))) return;
    if (s.hist_count < 2) {
        s.hist_iters[s.hist_count] = k;
        s.hist_fp_rate[s.hist_count] = fr;
        s.hist_count++;
    } else {
        s.hist_iters[0] = s.hist_iters[1];
        s.hist_fp_rate[0] = s.hist_fp_rate[1];
        s.hist_iters[1] = k;
        s.hist_fp_rate[1] = fr;
    }
}

/* solver.cu:605-614 */
PDAL_HD void cpal_epoch_start(CpalState &s) {
    s.epoch_valid = 1;
    s.epoch_total = s.total;
    s.epoch_p = ctl_metric(s.rel_p);
    s.epoch_d = ctl_metric(s.rel_d);
    s.epoch_g = ctl_metric(s.rel_gap);
}

/* solver.cu:899-966 (gate) and 968-988 (start), after a restart: the gate is
 * evaluated once; with force it passes and the next block runs at alpha =
 * 0.002 outside sigma mode */
PDAL_HD void cpal_pulse_gate(CpalState &s, const CpalParams &p, int F) {
    if (!p.pulse || s.pulse_gate || s.pulse_phase != 0 || s.hist_count < 2 || s.total < 10000 || F != 200) return;
    if (s.iter_limit - s.total < 400) return;
    for (int i = 0; i < 2; ++i)
        if (s.hist_iters[i] <= 0 || !isfinite(s.hist_fp_rate[i])) return;
    s.pulse_gate = p.pulse_force ? 1 : 2;
    if (!p.pulse_force) return;
    s.pulse_phase = 1;
    s.pulse_start = s.total;
    s.sigma_on = 0;
    s.al_lambda = 0.002;
    cpal_refresh_step_schedule(s, p);
}

/* solver.cu:3141-3164, as the sigma trigger runs it: the sigma parameters
 * from the step's lambda estimate; the step sizes follow at the restart the
 * trigger forces */
PDAL_HD void cpal_init_sigma(CpalState &s, const CpalParams &p) {
    const double le = fmax(s.lambda_est, 1e-12);
    s.lambda_param = p.lambda_param_set ? p.lambda_param_opt : p.lambda_factor * le;
    s.lambda_param = fmax(s.lambda_param, (2.0 + 1e-12) * le);
    s.sigma_base = 1.0 / sqrt(fmax(s.lambda_param, 1e-16));
    s.sigma_min = p.sigma_min_f * s.sigma_base;
    s.sigma_max = p.sigma_max_f * s.sigma_base;
    s.sigma = p.sigma_set ? p.sigma_value : p.sigma_init_f * s.sigma_base;
    s.sigma = fmin(fmax(s.sigma, s.sigma_min), s.sigma_max);
    s.sigma_best = s.sigma;
    s.sigma_esum = 0.0;
    s.sigma_last = 0.0;
    s.sigma_adapt = p.sigma_adaptive;
    s.sigma_on = 1;
}

/* Termination tests (LP/CP_AL/src/utils.cu:299-317, then the ray
 * certificates, the iteration limit, the FP32 phase's switch and the time
 * limit), then the end of an alpha pulse's positive block
 * (LP/CP_AL/src/solver.cu:990-1032), which the reference runs whether or not
 * that block ended the solve: alpha back to 0, the step schedule refreshed and
 * the fixed-point error taken again with the new coefficients. */
PDAL_HD bool cpal_terminated(CpalState &s, const CpalParams &p, const CpalEval &e) {
    int st = 0;
    if (s.rel_d < p.eps_feas && s.rel_p < p.eps_feas && s.rel_gap < p.eps_opt) st = 1; /* OPTIMAL */
    if (!st && p.infeas) {
        /* LP/CP_AL/src/utils.cu:919-1029 normalisation and 281-297 tests */
        const double cs = s.cbr * s.ovr;
        s.ray_pinf = e.ray_dxinf > 0.0 ? e.ray_pviol / e.ray_dxinf : e.ray_pviol;
        s.ray_pobj = (e.ray_dxinf > 0.0 ? e.ray_cdx / e.ray_dxinf : e.ray_cdx) / cs;
        const double sc = fmax(e.ray_dyinf, e.ray_dviol);
        s.ray_dinf = sc > 0.0 ? e.ray_dviol / sc : 0.0;
        s.ray_dobj = sc > 0.0 ? (e.ray_rowsum + e.ray_colsum) / cs / sc : 0.0;
        if (s.ray_dobj > 0.0 && s.ray_dinf / s.ray_dobj <= p.eps_infeas)
            st = 2; /* PRIMAL_INFEASIBLE */
        else if (s.ray_pobj < 0.0 && s.ray_pinf / (-s.ray_pobj) <= p.eps_infeas)
            st = 3; /* DUAL_INFEASIBLE */
    }
    if (!st && s.total >= s.iter_limit) st = 6; /* ITERATION_LIMIT */
    if (!st) {
        if (s.fp32_switch_tol > 0.0) {
            /* the FP32 phase ends at its tolerance, or when the KKT error has
             * not halved over fp32_stall_limit evaluations (FP32 rounding
             * floor) */
            const double kkt = fmax(s.rel_p, fmax(s.rel_d, s.rel_gap));
            if (kkt < 0.5 * s.fp32_best_kkt) {
                s.fp32_best_kkt = kkt;
                s.fp32_stall = 0;
            } else {
                s.fp32_stall++;
            }
            if (kkt < s.fp32_switch_tol || (s.fp32_stall_limit > 0 && s.fp32_stall >= s.fp32_stall_limit))
                s.phase_switch = 1;
        }
        if (s.elapsed >= p.time_limit) st = 5; /* TIME_LIMIT */
    }
    if (p.pulse && s.pulse_phase == 1) {
        s.pulse_p = ctl_metric(s.rel_p);
        s.pulse_d = ctl_metric(s.rel_d);
        s.pulse_g = ctl_metric(s.rel_gap);
        s.pulse_status = st;
        s.sigma_on = 0;
        s.al_lambda = 0.0;
        cpal_refresh_step_schedule(s, p);
        s.fp = cpal_fixed_point_error(s, e.dx2, e.dy2, e.adx2, e.cross);
        s.pulse_fp = ctl_metric(s.fp);
        s.pulse_phase = 2;
    }
    /* solver.cu:1386-1391, 1418-1424 */
    if (!st && p.pulse && p.pulse_test_limit > 0 && s.pulse_phase == 2 && s.total >= p.pulse_test_limit) st = 6;
    s.status = st;
    return st != 0;
}

/*
 * Everything the reference does between two graph launches
 * (LP/CP_AL/src/solver.cu:1343-1697 with the default controllers off):
 * fixed-point error, KKT, counters, termination, restart decision, restart.
 * Returns true when the solve has terminated (s.status set).
 */
PDAL_HD bool cpal_end_of_block(CpalState &s, const CpalParams &p, const CpalEval &e) {
    const int F = s.F; /* this block's iterations */
    s.fp = cpal_fixed_point_error(s, e.dx2, e.dy2, e.adx2, e.cross);
    cpal_residual_scalars(s, p, e);
    s.inner += F;
    s.total += F;
    s.restart = 0;
    if (cpal_terminated(s, p, e)) return true;
    /* LP/CP_AL/src/solver.cu:2749-2819: the scores of the reflected Halpern
     * iterate (x, y) and, in the three-point mode, of the plain Halpern point
     * h = w x^ + (1 - w) x0 against (x^, y^), by the fixed-point error's
     * formula.  x^ - h = (1 - w)(x^ - x0) and the score is homogeneous of
     * degree one in the difference, so h's score is (1 - w) times the score of
     * x^ - x0, whose terms the evaluation already holds. */
    s.restart_target = 0;
    const double w = (double)s.inner / (double)(s.inner + 1);
    s.restart_w = w;
    if (p.restart_select != 0 && s.total >= p.restart_select_min_iters && s.elapsed >= p.restart_select_min_time) {
        const double cur = s.fp;
        const double avg = cpal_fixed_point_error(s, e.sel_dx2, e.sel_dy2, e.sel_ax2, e.sel_cross);
        const double hal =
            p.restart_threepoint ? (1.0 - w) * cpal_fixed_point_error(s, e.ddx2, e.ddy2, e.axd2, e.h_cross) : INFINITY;
        if (p.restart_select == 2) {
            s.restart_target = 1;
            s.fp = avg;
        } else if (isfinite(cur)) {
            int best = 0;
            double best_score = cur;
            if (isfinite(avg) && avg < best_score) {
                best = 1;
                best_score = avg;
            }
            if (p.restart_threepoint && isfinite(hal) && hal < best_score) {
                best = 2;
                best_score = hal;
            }
            if (best != 0 && best_score <= p.restart_select_margin * cur) {
                s.restart_target = best;
                s.fp = best_score;
            }
        }
    }
    /* LP/CP_AL/src/solver.cu:1496-1527: the sigma trigger forces a restart
     * (the restart rule is then not evaluated) */
    bool forced = false;
    if (p.trigger && !s.sigma_on && s.total >= p.trigger_min_iters) {
        const double rpr = fmax(s.rel_p, 1e-300), rdr = fmax(s.rel_d, 1e-300);
        if (rpr >= p.trigger_p && rdr <= p.trigger_d && rpr / rdr >= p.trigger_ratio) {
            cpal_init_sigma(s, p);
            s.trigger_iter = s.total;
            forced = true;
        }
    }
    /* LP/CP_AL/src/solver.cu:1529-1583: the next blocks' length */
    if (p.dyn && !s.sigma_on && (s.total >= p.dyn_min_iters || (p.dyn_boot > 0 && s.total >= p.dyn_boot))) {
        const double rpr = fmax(s.rel_p, 1e-300), rdr = fmax(s.rel_d, 1e-300);
        const double lo = fmin(rpr, rdr), hi = fmax(rpr, rdr);
        const bool one_sided = lo <= p.dyn_small && hi >= p.dyn_large;
        const bool lag = hi / lo >= p.dyn_ratio && hi >= p.dyn_large;
        const bool tgate = p.dyn_sec > 0.0 && !p.cr_early_stopped && s.elapsed >= p.dyn_sec;
        const bool igate = p.dyn_iters > 0 && !p.cr_early_stopped && s.total >= p.dyn_iters;
        if (tgate || igate || (p.dyn_resid && (one_sided || lag))) {
            if (!s.dyn_latched) s.dyn_iter = s.total;
            s.dyn_latched = 1;
            s.F = p.dyn_fast;
        } else if (!s.dyn_latched && p.dyn_boot > 0 && s.F == p.dyn_fast && s.total >= p.dyn_boot) {
            s.F = p.F;
        }
    }
    if (forced || cpal_should_restart(s, p, F)) {
        /* the PID distances run from the anchors to the restart point:
         * h - x0 = w (x^ - x0) for the plain Halpern point */
        const int tg = s.restart_target;
        const double w2 = w * w;
        if (p.pulse) cpal_record_epoch(s);
        if (tg == 1)
            cpal_restart_scalars(s, p, e.cur_dx2, e.cur_dy2, e.cur_axd2);
        else if (tg == 2)
            cpal_restart_scalars(s, p, w2 * e.ddx2, w2 * e.ddy2, w2 * e.axd2);
        else
            cpal_restart_scalars(s, p, e.ddx2, e.ddy2, e.axd2);
        if (p.pulse) {
            cpal_epoch_start(s);
            cpal_pulse_gate(s, p, F);
        }
        s.restart = 1;
        /* the reference recomputes the fixed-point error of the unchanged
         * iterates with the new coefficients at the start of the next block
         * (solver.cu:1279-1284).  A restart to the reflected Halpern iterate
         * first sets x-bar = x^ and x^ = x (solver.cu:3016-3042), so the
         * deltas are then x^ - x; one to the plain Halpern point sets x-bar =
         * x^ and x^ = h (solver.cu:3043-3075), so they are (1 - w)(x^ - x0). */
        if (tg == 1)
            s.fp0 = cpal_fixed_point_error(s, e.sel_dx2, e.sel_dy2, e.sel_ax2, e.sel_cross);
        else if (tg == 2)
            s.fp0 = (1.0 - w) * cpal_fixed_point_error(s, e.ddx2, e.ddy2, e.axd2, e.h_cross);
        else
            s.fp0 = cpal_fixed_point_error(s, e.dx2, e.dy2, e.adx2, e.cross);
    }
    cpal_set_coefficients(s);
    return false;
}

} // namespace pdal
