/*
 * batch_kernels.cuh -- thousands of independent CP_AL LPs in ONE persistent
 * launch (sm_103a).
 *
 * Each resident CUDA block takes the next instance from a global queue (an
 * atomic counter over instances ordered by decreasing size), solves it
 * completely -- equilibration, power iteration, the Halpern blocks, the
 * evaluations, restarts and termination -- and takes the next one, so a
 * finished instance frees its block for a queued one.  All synchronisation
 * inside an instance is __syncthreads(); no block ever waits on another.
 *
 * The arithmetic is the single-instance solver's: the same row-block products
 * and fused epilogues (cpal_kernels.cuh), the same controller
 * (cpal_control.h), run by one block over the instance's own row blocks.
 * Rows longer than one row block are summed piece by piece in the block, in
 * piece order.  Per-instance state (step, weight, sigma, restart and
 * termination state) is a CpalState in shared memory.
 */
#pragma once

#include "cpal_control.h"
#include "cpal_kernels.cuh"
#include "rowblock.cuh"

namespace pdal {
namespace batch {

constexpr int kBS = 1024; /* nonzeros per row block */

/* One instance: its arrays (device pointers into the batch arena). */
struct BInst {
    int m, n, nnz;
    int nbA, nlA, nbAt, nlAt;
    int pad;
    const int *Arp, *Aci, *Atrp, *Atci;
    double *Av, *Atv;
    const int4 *Adesc, *Alinfo, *Atdesc, *Atlinfo;
    double *Alpart, *Atlpart;
    unsigned *Alcount, *Atlcount;
    double *c, *vlb, *vub, *clb, *cub, *x0, *y0;
    double *x, *xbar, *xh, *lam, *y, *yh, *ybar, *ax, *u, *ax0, *phat;
    double *dsc, *rsc, *clbf, *cubf, *tn, *tm, *tm2;
    const double *pv0; /* power-iteration start vector (m) */
    double *out_x, *out_y, *out_rc;
    double obj_norm, bnd_norm, obj_const;
    double sigma0; /* > 0: initial sigma of this instance (sigma mode) */
};

/* Per-instance outcome. */
struct BOut {
    int status, iterations, restarts, power_iters;
    double pobj, dobj, rel_p, rel_d, rel_gap, abs_p, abs_d;
    double lambda_est, pw, step, elapsed;
    double setup_sec;
    double sigma, sigma_best;
};

/* Batch-wide options resolved on the host. */
struct BOpts {
    int ruiz, pc;
    double pc_alpha;
    int boundobj;
    int sv_max_iter;
    double sv_tol;
    double al_lambda;
    int sigma_mode, sigma_set, sigma_adaptive, lambda_param_set;
    double sigma, sigma_init_factor, sigma_min_factor, sigma_max_factor, lambda_param;
};

/* Shared-memory staging reused by every phase (the evaluation of the rows
 * gathers three vectors, the largest user). */
union BSmem {
    RowBlockSmem<kBS, 1, double> one;
    RowBlockSmem<kBS, 2, double> two;
    RowBlockSmem<kBS, 3, double> three;
};

template <class F>
__device__ __forceinline__ void blk_for(int count, F f) {
    for (int i = threadIdx.x; i < count; i += kThreads) f(i);
}

/* warp per row over the rows of one matrix, inside the block */
template <class F>
__device__ __forceinline__ void blk_rows(int nr, F f) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int row = warp; row < nr; row += kThreads / 32) f(row, lane);
}

/* The instance's row blocks of one matrix, run by this block. */
template <int NP, class Gat, class Epi, class R>
__device__ __forceinline__ void blk_spmv(int nblocks, const int4 *desc, const int4 *linfo, double *lpart,
                                         unsigned *lcount, int nlong, const int *rp, const int *ci, const double *val,
                                         Gat &gat, Epi &epi, R &red, RowBlockSmem<kBS, NP, double> &sm) {
    RowPlanDev plan;
    plan.desc = desc;
    plan.linfo = linfo;
    plan.lpart = lpart;
    plan.lcount = lcount;
    plan.nblocks = nblocks;
    plan.nlong = nlong;
    for (int b = 0; b < nblocks; ++b) {
        rowblock_run_at<kBS, NP, double>(b, plan, rp, ci, val, gat, epi, red, sm);
        __syncthreads();
    }
}

/* Long-row reduction terms go to a shared accumulator (thread 0 runs every
 * long-row epilogue in the block, so the order is the piece order). */
template <int NS, int NM>
struct LongAcc {
    Red<NS, NM> *acc;
    __device__ __forceinline__ void add(const Red<NS, NM> &r) const {
#pragma unroll
        for (int i = 0; i < NS; ++i) acc->s[i] += r.s[i];
#pragma unroll
        for (int i = 0; i < NM; ++i) acc->mx[i] = fmax(acc->mx[i], r.mx[i]);
    }
};

template <class Base>
struct EvalRowsB : Base {
    LongAcc<6, 1> la;
    __device__ __forceinline__ void long_red(int, Red<6, 1> &r) const { la.add(r); }
};

/* ------------------------------------------------------------------ setup */

/* Ruiz (mode 0) or Pock-Chambolle (mode 1) pass, the block-level form of
 * k_row_scale / k_scale_matrix / k_scale_vectors (same operation order). */
__device__ void blk_scale_pass(const BInst &I, int mode, double deg_rows, double deg_cols) {
    auto row_scale = [&](int nr, const int *rp, const double *val, double deg, double *scale, double *cum) {
        blk_rows(nr, [&](int row, int lane) {
            double acc = 0.0;
            for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) {
                double v = fabs(val[k]);
                if (!isfinite(v)) v = 0.0;
                if (mode == 0) {
                    acc = fmax(acc, v);
                } else {
                    double pv;
                    if (deg == 2.0)
                        pv = v * v;
                    else if (deg == 1.0)
                        pv = v;
                    else if (deg == 0.5)
                        pv = sqrt(v);
                    else
                        pv = pow(v, deg);
                    acc += pv;
                }
            }
            acc = mode == 0 ? warp_max(acc) : warp_sum(acc);
            if (lane == 0) {
                const double s = (acc < 1e-12) ? 1.0 : sqrt(acc);
                cum[row] *= s;
                scale[row] = s;
            }
        });
    };
    row_scale(I.m, I.Arp, I.Av, deg_rows, I.tm, I.rsc);
    row_scale(I.n, I.Atrp, I.Atv, deg_cols, I.tn, I.dsc);
    __syncthreads();
    blk_rows(I.m, [&](int row, int lane) {
        const double inv_row = 1.0 / I.tm[row];
        for (int k = I.Arp[row] + lane; k < I.Arp[row + 1]; k += 32) {
            const double inv_col = 1.0 / I.tn[I.Aci[k]];
            I.Av[k] *= inv_col * inv_row;
        }
    });
    blk_rows(I.n, [&](int row, int lane) {
        const double inv_row = 1.0 / I.tn[row];
        for (int k = I.Atrp[row] + lane; k < I.Atrp[row + 1]; k += 32) {
            const double inv_col = 1.0 / I.tm[I.Atci[k]];
            I.Atv[k] *= inv_row * inv_col;
        }
    });
    blk_for(I.n, [&](int t) {
        const double dj = I.tn[t], inv = 1.0 / I.tn[t];
        I.c[t] *= inv;
        I.vlb[t] *= dj;
        I.vub[t] *= dj;
        I.x0[t] *= dj;
    });
    blk_for(I.m, [&](int t) {
        const double inv = 1.0 / I.tm[t], ei = I.tm[t];
        I.clb[t] *= inv;
        I.cub[t] *= inv;
        I.y0[t] *= ei;
    });
    __syncthreads();
}

__device__ void blk_equilibrate(const BInst &I, const BOpts &o, CpalState &s, double *sbuf) {
    blk_for(I.n, [&](int t) { I.dsc[t] = 1.0; });
    blk_for(I.m, [&](int t) { I.rsc[t] = 1.0; });
    __syncthreads();
    for (int it = 0; it < o.ruiz; ++it) blk_scale_pass(I, 0, 0.0, 0.0);
    if (o.pc) blk_scale_pass(I, 1, o.pc_alpha, 2.0 - o.pc_alpha);
    Red<2, 0> r;
    r.zero();
    blk_for(I.m, [&](int t) {
        const double L = I.clb[t], U = I.cub[t];
        const bool fL = isfinite(L), fU = isfinite(U);
        double acc = 0.0;
        if (fL && (!fU || fabs(L - U) > 1e-12)) acc += L * L;
        if (fU) acc += U * U;
        r.s[0] += acc;
    });
    blk_for(I.n, [&](int t) { r.s[1] += I.c[t] * I.c[t]; });
    block_reduce<kThreads, 2, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        if (o.boundobj) {
            s.cbr = 1.0 / (sqrt(r.s[0]) + 1.0);
            s.ovr = 1.0 / (sqrt(r.s[1]) + 1.0);
        } else {
            s.cbr = 1.0;
            s.ovr = 1.0;
        }
    }
    __syncthreads();
    if (o.boundobj) {
        const double cs = s.cbr, os = s.ovr;
        blk_for(I.m, [&](int t) {
            I.clb[t] *= cs;
            I.cub[t] *= cs;
            I.y0[t] *= os;
        });
        blk_for(I.n, [&](int t) {
            I.vlb[t] *= cs;
            I.vub[t] *= cs;
            I.c[t] *= os;
            I.x0[t] *= cs;
        });
    }
    blk_for(I.m, [&](int t) {
        I.clbf[t] = isfinite(I.clb[t]) ? I.clb[t] : 0.0;
        I.cubf[t] = isfinite(I.cub[t]) ? I.cub[t] : 0.0;
    });
    __syncthreads();
}

struct PowColEpiB : NoLongRed {
    double *dp;
    __device__ __forceinline__ void operator()(int j, const double *s, Red<0, 0> &) const { dp[j] = s[0]; }
};
struct PowRowEpiB {
    const double *v;
    double *vn;
    double inv;
    LongAcc<1, 0> la;
    __device__ __forceinline__ void operator()(int i, const double *s, Red<1, 0> &r) const {
        vn[i] = s[0];
        r.s[0] += (inv * v[i]) * s[0];
    }
    __device__ __forceinline__ void long_red(int, Red<1, 0> &r) const { la.add(r); }
};

/* sigma_max(A)^2 by the power iteration of k_power_* (start vector in tm). */
__device__ double blk_power(const BInst &I, const BOpts &o, BSmem &sm, double *sbuf, Red<1, 0> *lacc,
                            double *sh, int &iters) {
    double *v = I.tm, *vn = I.tm2, *dp = I.tn;
    blk_for(I.m, [&](int i) { v[i] = I.pv0[i]; });
    __syncthreads();
    Red<1, 0> r;
    r.zero();
    blk_for(I.m, [&](int i) { r.s[0] += v[i] * v[i]; });
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) sh[0] = 1.0 / sqrt(r.s[0]);
    __syncthreads();
    double inv = sh[0], s2 = 0.0;
    int it = 0;
    bool done = o.sv_max_iter <= 0;
    while (!done) {
        {
            PowColEpiB e;
            e.dp = dp;
            auto g = [&](int c, double *out) { out[0] = inv * v[c]; };
            Red<0, 0> z;
            blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, I.Atv, g, e, z,
                        sm.one);
        }
        {
            if (threadIdx.x == 0) lacc->zero();
            __syncthreads();
            PowRowEpiB e;
            e.v = v;
            e.vn = vn;
            e.inv = inv;
            e.la.acc = lacc;
            auto g = [&](int c, double *out) { out[0] = dp[c]; };
            Red<1, 0> rr;
            rr.zero();
            blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, I.Av, g, e, rr, sm.one);
            block_reduce<kThreads, 1, 0>(rr, sbuf);
            if (threadIdx.x == 0) sh[1] = rr.s[0] + lacc->s[0];
            __syncthreads();
            s2 = sh[1];
        }
        Red<2, 0> q;
        q.zero();
        blk_for(I.m, [&](int i) {
            const double nv = inv * v[i];
            const double vni = vn[i];
            const double d = (-s2 * nv) + vni;
            q.s[0] += d * d;
            q.s[1] += vni * vni;
            v[i] = vni;
        });
        block_reduce<kThreads, 2, 0>(q, sbuf);
        if (threadIdx.x == 0) {
            sh[2] = sqrt(q.s[0]);
            sh[0] = 1.0 / sqrt(q.s[1]);
        }
        __syncthreads();
        ++it;
        inv = sh[0];
        done = sh[2] < o.sv_tol || it >= o.sv_max_iter;
    }
    iters = it;
    const double smax = sqrt(s2);
    return smax * smax;
}

/* ------------------------------------------------------------------ one instance */

__device__ void blk_solve(const BInst &I, CpalParams p, const BOpts &o, BOut *out, BSmem &sm, double *sbuf,
                          CpalState &s, Red<6, 1> *lacc6, Red<1, 0> *lacc1, double *sh) {
    const unsigned long long t0 = globaltimer_ns();
    p.obj_norm = I.obj_norm;
    p.bnd_norm = I.bnd_norm;
    p.obj_const = I.obj_const;
    if (threadIdx.x == 0) {
        s = CpalState{};
    }
    __syncthreads();
    blk_equilibrate(I, o, s, sbuf);
    int piters = 0;
    double lambda_est = 1.0;
    if (I.nnz > 0) lambda_est = blk_power(I, o, sm, sbuf, lacc1, sh, piters);
    if (threadIdx.x == 0) { /* the setup of CpalSolver::setup_device */
        s.lambda_est = lambda_est;
        s.pw = o.boundobj ? 1.0 : (I.obj_norm + 1.0) / (I.bnd_norm + 1.0);
        s.sigma_on = o.sigma_mode;
        s.sigma_adapt = 0;
        if (s.sigma_on) {
            s.lambda_param = o.lambda_param_set ? o.lambda_param : p.lambda_factor * fmax(s.lambda_est, 1e-12);
            s.lambda_param = fmax(s.lambda_param, (2.0 + 1e-12) * fmax(s.lambda_est, 1e-12));
            s.sigma_base = 1.0 / sqrt(fmax(s.lambda_param, 1e-16));
            s.sigma_min = o.sigma_min_factor * s.sigma_base;
            s.sigma_max = o.sigma_max_factor * s.sigma_base;
            s.sigma = I.sigma0 > 0.0 ? I.sigma0 : (o.sigma_set ? o.sigma : o.sigma_init_factor * s.sigma_base);
            s.sigma = fmin(fmax(s.sigma, s.sigma_min), s.sigma_max);
            s.sigma_best = s.sigma;
            s.sigma_adapt = o.sigma_adaptive != 0;
        }
        s.al_lambda = o.al_lambda;
        cpal_refresh_step_schedule(s, p);
        s.best_pw = s.pw;
        s.best_gap = INFINITY;
        s.fp_last = INFINITY;
        s.refl = p.refl;
        s.fp32_switch_tol = -1.0;
        s.iter_limit = p.iteration_limit;
        cpal_set_coefficients(s);
        s.t_start_ns = globaltimer_ns();
        sh[3] = (double)(s.t_start_ns - t0) * 1e-9;
    }
    __syncthreads();
    const bool beta_on = s.beta > 0.0;
    /* iterates start at the scaled warm start */
    blk_for(I.n, [&](int j) {
        I.x[j] = I.x0[j];
        I.xh[j] = I.x0[j];
        I.lam[j] = 0.0;
        I.xbar[j] = 0.0;
    });
    blk_for(I.m, [&](int i) {
        I.y[i] = I.y0[i];
        I.yh[i] = I.y0[i];
        I.ybar[i] = 0.0;
        I.u[i] = 0.0;
    });
    __syncthreads();
    auto init_ax = [&]() {
        if (beta_on) {
            InitAxEpi<double, true> e;
            e.ax = I.ax;
            e.u = I.u;
            e.ax0 = I.ax0;
            e.ax0f = nullptr;
            e.y = I.y;
            e.lb = I.clb;
            e.ub = I.cub;
            e.beta = s.beta;
            e.inv_beta = s.inv_beta;
            auto g = [&](int c, double *o2) { o2[0] = I.x0[c]; };
            Red<0, 0> z;
            blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, I.Av, g, e, z, sm.one);
        } else {
            InitAxEpi<double, false> e;
            e.ax = I.ax;
            e.u = I.u;
            e.ax0 = I.ax0;
            e.ax0f = nullptr;
            e.y = I.y;
            e.lb = I.clb;
            e.ub = I.cub;
            e.beta = 0.0;
            e.inv_beta = 0.0;
            auto g = [&](int c, double *o2) { o2[0] = I.x0[c]; };
            Red<0, 0> z;
            blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, I.Av, g, e, z, sm.one);
        }
    };
    init_ax();

    const int F = p.F;
    for (;;) {
        Coefs<double> k;
        k.tau = s.tau;
        k.inv_tau = s.inv_tau;
        k.rho = s.rho;
        k.inv_prox = s.inv_prox;
        k.beta = s.beta;
        k.inv_beta = s.inv_beta;
        k.r = s.refl;
        const int inner = s.inner;
        for (int i = 1; i <= F; ++i) {
            const int kk = inner + i;
            const double w = (double)kk / (double)(kk + 1);
            const double omw = 1.0 - w;
            const double *gat = beta_on ? I.u : I.y;
            auto gp = [&](int c, double *o2) { o2[0] = gat[c]; };
            PrimalArgs<double> pa{I.x, I.xbar, I.xh, I.lam, I.x0, I.c, I.vlb, I.vub};
            Red<0, 0> z;
            if (i == F) {
                PrimalEpi<double, true> e;
                e.a = pa;
                e.k = k;
                e.w = w;
                e.omw = omw;
                blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, I.Atv, gp, e,
                            z, sm.one);
            } else {
                PrimalEpi<double, false> e;
                e.a = pa;
                e.k = k;
                e.w = w;
                e.omw = omw;
                blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, I.Atv, gp, e,
                            z, sm.one);
            }
            if (I.m > 0) {
                DualArgs<double> da{I.y, I.yh, I.ybar, I.ax, I.u, I.y0, I.ax0, I.clb, I.cub};
                auto gd = [&](int c, double *o2) { o2[0] = I.xbar[c]; };
#define PDAL_BATCH_DUAL(MAJ, BET)                                                                                      \
    {                                                                                                                  \
        DualEpi<double, MAJ, BET> e;                                                                                   \
        e.a = da;                                                                                                      \
        e.k = k;                                                                                                       \
        e.w = w;                                                                                                       \
        e.omw = omw;                                                                                                   \
        blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, I.Av, gd, e, z, sm.one);     \
    }
                if (i == F) {
                    if (beta_on)
                        PDAL_BATCH_DUAL(true, true)
                    else
                        PDAL_BATCH_DUAL(true, false)
                } else {
                    if (beta_on)
                        PDAL_BATCH_DUAL(false, true)
                    else
                        PDAL_BATCH_DUAL(false, false)
                }
#undef PDAL_BATCH_DUAL
            }
        }
        /* evaluation (k_eval_rows / k_eval_cols / k_control) */
        CpalEval e{};
        if (threadIdx.x == 0) lacc6->zero();
        __syncthreads();
        {
            EvalRowsB<EvalRowEpi<double>> ep;
            ep.a = EvalRowArgs<double>{I.xh, I.xbar, I.yh, I.ybar, I.x0, I.y0, I.ax0, I.clb, I.cub, I.clbf, I.cubf,
                                       I.rsc, I.phat, nullptr, 0};
            ep.la.acc = lacc6;
            auto g = [&](int c, double *o2) {
                const double xhc = I.xh[c];
                o2[0] = xhc;
                o2[1] = I.xbar[c] - xhc;
                o2[2] = xhc - I.x0[c];
            };
            Red<6, 1> r;
            r.zero();
            blk_spmv<3>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, I.Av, g, ep, r, sm.three);
            block_reduce<kThreads, 6, 1>(r, sbuf);
            if (threadIdx.x == 0) {
                for (int q = 0; q < 6; ++q) r.s[q] += lacc6->s[q];
                r.mx[0] = fmax(r.mx[0], lacc6->mx[0]);
                sh[4] = r.s[0];
                sh[5] = r.s[1];
                sh[6] = r.s[2];
                sh[7] = r.s[3];
                sh[8] = r.s[4];
                sh[9] = r.s[5];
                sh[10] = r.mx[0];
                lacc6->zero();
            }
            __syncthreads();
        }
        {
            EvalRowsB<EvalColEpi<double>> ec;
            ec.a = EvalColArgs<double>{I.xh, I.xbar, I.yh, I.ybar, I.lam, I.x0, I.c, I.dsc, nullptr, 0};
            ec.la.acc = lacc6;
            auto g = [&](int c, double *o2) {
                const double yhc = I.yh[c];
                o2[0] = yhc;
                o2[1] = I.ybar[c] - yhc;
            };
            Red<6, 1> r;
            r.zero();
            blk_spmv<2>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, I.Atv, g, ec, r,
                        sm.two);
            block_reduce<kThreads, 6, 1>(r, sbuf);
            if (threadIdx.x == 0) {
                for (int q = 0; q < 6; ++q) r.s[q] += lacc6->s[q];
                r.mx[0] = fmax(r.mx[0], lacc6->mx[0]);
                e.rp2 = sh[4];
                e.contrib = sh[5];
                e.adx2 = sh[6];
                e.dy2 = sh[7];
                e.ddy2 = sh[8];
                e.axd2 = sh[9];
                e.rpmax = sh[10];
                e.rd2 = r.s[0];
                e.dx2 = r.s[1];
                e.cross = r.s[2];
                e.cx = r.s[3];
                e.lx = r.s[4];
                e.ddx2 = r.s[5];
                e.rdmax = r.mx[0];
                s.elapsed = (double)(globaltimer_ns() - s.t_start_ns) * 1e-9;
                cpal_end_of_block(s, p, e);
            }
            __syncthreads();
        }
        if (s.status) break;
        if (s.restart) { /* k_restart */
            blk_for(I.n, [&](int j) {
                const double v = I.xh[j];
                I.x[j] = v;
                I.x0[j] = v;
            });
            const double beta = s.beta, inv_beta = s.inv_beta;
            blk_for(I.m, [&](int i) {
                const double v = I.yh[i];
                I.y[i] = v;
                I.y0[i] = v;
                const double ph = I.phat[i];
                I.ax0[i] = ph;
                I.ax[i] = ph;
                if (beta_on) {
                    const double z2 = fmax(I.clb[i], fmin(ph - v * inv_beta, I.cub[i]));
                    I.u[i] = v - beta * (ph - z2);
                }
            });
            __syncthreads();
        }
    }
    /* result (k_result_cols / k_result_rows) */
    {
        ResultColEpi re;
        re.xh = I.xh;
        re.c = I.c;
        re.cscale = I.dsc;
        re.vlb = I.vlb;
        re.vub = I.vub;
        re.st = &s;
        re.x_out = I.out_x;
        re.rc_out = I.out_rc;
        auto g = [&](int c, double *o2) { o2[0] = I.yh[c]; };
        Red<0, 0> z;
        blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, I.Atv, g, re, z,
                    sm.one);
        const double ovr = s.ovr;
        blk_for(I.m, [&](int i) { I.out_y[i] = I.yh[i] / I.rsc[i] / ovr; });
    }
    if (threadIdx.x == 0) {
        BOut r;
        r.status = s.status;
        r.iterations = s.total;
        r.restarts = s.restarts;
        r.power_iters = piters;
        r.pobj = s.pobj;
        r.dobj = s.dobj;
        r.rel_p = s.rel_p;
        r.rel_d = s.rel_d;
        r.rel_gap = s.rel_gap;
        r.abs_p = s.abs_p;
        r.abs_d = s.abs_d;
        r.lambda_est = s.lambda_est;
        r.pw = s.pw;
        r.step = s.step;
        r.elapsed = (double)(globaltimer_ns() - s.t_start_ns) * 1e-9;
        r.setup_sec = sh[3];
        r.sigma = s.sigma_on ? s.sigma : 0.0;
        r.sigma_best = s.sigma_on ? s.sigma_best : 0.0;
        *out = r;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 2) k_batch_lp(const BInst *__restrict__ insts, int count,
                                                          const int *__restrict__ order, unsigned *queue, CpalParams p,
                                                          BOpts o, BOut *outs) {
    __shared__ BSmem sm;
    __shared__ CpalState s;
    __shared__ double sbuf[8 * (kThreads / 32)];
    __shared__ Red<6, 1> lacc6;
    __shared__ Red<1, 0> lacc1;
    __shared__ double sh[16];
    __shared__ int slot;
    for (;;) {
        if (threadIdx.x == 0) slot = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int q = slot;
        __syncthreads();
        if (q >= count) return;
        const int idx = order[q];
        const BInst &I = insts[idx];
        blk_solve(I, p, o, outs + idx, sm, sbuf, s, &lacc6, &lacc1, sh);
    }
}

} // namespace batch
} // namespace pdal
