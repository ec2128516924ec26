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
    /* the FP32 phase: matrix values, bounds and iterates rounded to FP32,
     * the FP64 anchors as (hi, lo) float pairs */
    float *Avf, *Atvf, *cf, *vlbf, *vubf, *clbF, *cubF;
    float *xf, *xbarf, *xhf, *lamf, *yf, *yhf, *ybarf, *axf, *uf;
    float2 *x0f, *y0f, *ax0f;
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
    int fp32_iterations, pad;
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
    int fp32;              /* run the FP32 phase first */
    int fp32_stall_evals;
    double fp32_switch_tol;
};

/* Shared-memory staging reused by every phase (the evaluation of the rows
 * gathers three vectors, the largest user). */
template <int BS>
union BSmem {
    RowBlockSmem<BS, 1, float> onef;
    RowBlockSmem<BS, 1, double> one;
    RowBlockSmem<BS, 2, double> two;
    RowBlockSmem<BS, 3, double> three;
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
template <int NP, int BS, typename T, class Gat, class Epi, class R>
__device__ __forceinline__ void blk_spmv(int nblocks, const int4 *desc, const int4 *linfo, double *lpart,
                                         unsigned *lcount, int nlong, const int *rp, const int *ci, const T *val,
                                         Gat &gat, Epi &epi, R &red, RowBlockSmem<BS, NP, T> &sm) {
    RowPlanDev plan;
    plan.desc = desc;
    plan.linfo = linfo;
    plan.lpart = lpart;
    plan.lcount = lcount;
    plan.nblocks = nblocks;
    plan.nlong = nlong;
    for (int b = 0; b < nblocks; ++b) {
        rowblock_run_at<BS, NP, T>(b, plan, rp, ci, val, gat, epi, red, sm);
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
 * k_row_scale / k_scale_matrix / k_scale_vectors (same operation order: the
 * Pock-Chambolle sums in row order in one lane, as the reference adds them). */
__device__ void blk_scale_pass(const BInst &I, int mode, double deg_rows, double deg_cols) {
    auto row_scale = [&](int nr, const int *rp, const double *val, double deg, double *scale, double *cum) {
        blk_rows(nr, [&](int row, int lane) {
            if (mode != 0) {
                if (lane == 0) {
                    double acc = 0.0;
                    for (int k = rp[row]; k < rp[row + 1]; ++k) {
                        double v = fabs(val[k]);
                        if (!isfinite(v)) v = 0.0;
                        acc += deg == 2.0 ? v * v : deg == 1.0 ? v : deg == 0.5 ? sqrt(v) : pow(v, deg);
                    }
                    const double s = (acc < 1e-12) ? 1.0 : sqrt(acc);
                    cum[row] *= s;
                    scale[row] = s;
                }
                return;
            }
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
template <int BS>
__device__ double blk_power(const BInst &I, const BOpts &o, BSmem<BS> &sm, double *sbuf, Red<1, 0> *lacc,
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

/* The arrays one precision phase iterates on. */
template <typename T>
struct BVec {
    T *x, *xbar, *xh, *lam, *y, *yh, *ybar, *ax, *u;
    const T *c, *vlb, *vub, *clb, *cub, *Av, *Atv;
    const typename AnchorT<T>::type *x0, *y0, *ax0;
};
__device__ __forceinline__ BVec<double> bvec64(const BInst &I) {
    return BVec<double>{I.x,   I.xbar, I.xh,  I.lam, I.y,  I.yh, I.ybar, I.ax, I.u,  I.c,  I.vlb,
                        I.vub, I.clb,  I.cub, I.Av,  I.Atv, I.x0, I.y0,   I.ax0};
}
__device__ __forceinline__ BVec<float> bvec32(const BInst &I) {
    return BVec<float>{I.xf,   I.xbarf, I.xhf, I.lamf, I.yf,   I.yhf, I.ybarf, I.axf, I.uf,  I.cf,  I.vlbf,
                       I.vubf, I.clbF,  I.cubF, I.Avf, I.Atvf, I.x0f, I.y0f,   I.ax0f};
}

template <typename T>
__device__ __forceinline__ BVec<T> bvec(const BInst &I);
template <>
__device__ __forceinline__ BVec<double> bvec<double>(const BInst &I) {
    return bvec64(I);
}
template <>
__device__ __forceinline__ BVec<float> bvec<float>(const BInst &I) {
    return bvec32(I);
}

template <typename T>
__device__ __forceinline__ float2 *anchor_split(const BInst &I, int which);
template <>
__device__ __forceinline__ float2 *anchor_split<double>(const BInst &, int) {
    return nullptr;
}
template <>
__device__ __forceinline__ float2 *anchor_split<float>(const BInst &I, int which) {
    return which == 0 ? I.x0f : (which == 1 ? I.y0f : I.ax0f);
}

/* A x0 (FP64 matrix) and the first predictor of a phase (k_init_ax). */
template <typename T, int BS>
__device__ void blk_init_ax(const BInst &I, const BVec<T> &v, const CpalState &s, bool beta_on, BSmem<BS> &sm) {
    Coefs<T> k;
    load_coefs(&s, k);
    auto g = [&](int c, double *o2) { o2[0] = I.x0[c]; };
    Red<0, 0> z;
    if (beta_on) {
        InitAxEpi<T, true> e;
        e.ax = v.ax;
        e.u = v.u;
        e.ax0 = I.ax0;
        e.ax0f = anchor_split<T>(I, 2);
        e.y = v.y;
        e.lb = v.clb;
        e.ub = v.cub;
        e.beta = k.beta;
        e.inv_beta = k.inv_beta;
        blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, (const double *)I.Av, g, e, z,
                    sm.one);
    } else {
        InitAxEpi<T, false> e;
        e.ax = v.ax;
        e.u = v.u;
        e.ax0 = I.ax0;
        e.ax0f = anchor_split<T>(I, 2);
        e.y = v.y;
        e.lb = v.clb;
        e.ub = v.cub;
        e.beta = k.beta;
        e.inv_beta = k.inv_beta;
        blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, (const double *)I.Av, g, e, z,
                    sm.one);
    }
}

template <int BS>
__device__ __forceinline__ RowBlockSmem<BS, 1, double> &smem1(BSmem<BS> &sm, double) {
    return sm.one;
}
template <int BS>
__device__ __forceinline__ RowBlockSmem<BS, 1, float> &smem1(BSmem<BS> &sm, float) {
    return sm.onef;
}

/* One precision phase: evaluation blocks until the controller terminates the
 * solve or (FP32) ends the phase.  The arithmetic of k_primal / k_dual /
 * k_eval_rows / k_eval_cols / k_control / k_restart. */
template <typename T, int BS>
__device__ void blk_phase(const BInst &I, const CpalParams &p, BSmem<BS> &sm, double *sbuf, CpalState &s,
                          Red<6, 1> *lacc6, double *sh, bool beta_on) {
    const BVec<T> v = bvec<T>(I);
    const int F = p.F;
    for (;;) {
        Coefs<T> k;
        load_coefs(&s, k);
        const int inner = s.inner;
        for (int i = 1; i <= F; ++i) {
            HalpernW wd;
            HalpernWf wf;
            cpal_halpern_entry(inner, i, wd, wf);
            const T w = sizeof(T) == 8 ? (T)wd.w : (T)wf.w;
            const T omw = sizeof(T) == 8 ? (T)wd.omw : (T)wf.omw;
            const T *gat = beta_on ? v.u : v.y;
            auto gp = [&](int c, T *o2) { o2[0] = gat[c]; };
            PrimalArgs<T> pa{v.x, v.xbar, v.xh, v.lam, v.x0, v.c, v.vlb, v.vub};
            Red<0, 0> z;
            if (i == F) {
                PrimalEpi<T, true> e;
                e.a = pa;
                e.k = k;
                e.w = w;
                e.omw = omw;
                blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, v.Atv, gp, e,
                            z, smem1(sm, T(0)));
            } else {
                PrimalEpi<T, false> e;
                e.a = pa;
                e.k = k;
                e.w = w;
                e.omw = omw;
                blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci, v.Atv, gp, e,
                            z, smem1(sm, T(0)));
            }
            if (I.m > 0) {
                DualArgs<T> da{v.y, v.yh, v.ybar, v.ax, v.u, v.y0, v.ax0, v.clb, v.cub};
                auto gd = [&](int c, T *o2) { o2[0] = v.xbar[c]; };
#define PDAL_BATCH_DUAL(MAJ, BET)                                                                                      \
    {                                                                                                                  \
        DualEpi<T, MAJ, BET> e;                                                                                        \
        e.a = da;                                                                                                      \
        e.k = k;                                                                                                       \
        e.w = w;                                                                                                       \
        e.omw = omw;                                                                                                   \
        blk_spmv<1>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, v.Av, gd, e, z, smem1(sm, T(0))); \
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
        /* evaluation in FP64 over the FP64 matrices */
        CpalEval e{};
        if (threadIdx.x == 0) lacc6->zero();
        __syncthreads();
        {
            EvalRowsB<EvalRowEpi<T>> ep;
            ep.a = EvalRowArgs<T>{v.xh, v.xbar, v.yh, v.ybar, I.x0, I.y0, I.ax0, I.clb, I.cub, I.clbf, I.cubf,
                                  I.rsc, I.phat, nullptr, 0};
            ep.la.acc = lacc6;
            auto g = [&](int c, double *o2) {
                const double xhc = (double)v.xh[c];
                o2[0] = xhc;
                o2[1] = (double)v.xbar[c] - xhc;
                o2[2] = xhc - I.x0[c];
            };
            Red<6, 1> r;
            r.zero();
            blk_spmv<3>(I.nbA, I.Adesc, I.Alinfo, I.Alpart, I.Alcount, I.nlA, I.Arp, I.Aci, (const double *)I.Av, g,
                        ep, r, sm.three);
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
            EvalRowsB<EvalColEpi<T>> ec;
            ec.a = EvalColArgs<T>{v.xh, v.xbar, v.yh, v.ybar, v.lam, I.x0, I.c, I.dsc, nullptr, 0};
            ec.la.acc = lacc6;
            auto g = [&](int c, double *o2) {
                const double yhc = (double)v.yh[c];
                o2[0] = yhc;
                o2[1] = (double)v.ybar[c] - yhc;
            };
            Red<6, 1> r;
            r.zero();
            blk_spmv<2>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci,
                        (const double *)I.Atv, g, ec, r, sm.two);
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
        if (s.status) return;
        if (s.restart) { /* k_restart */
            Coefs<T> kr;
            load_coefs(&s, kr);
            float2 *x0s = anchor_split<T>(I, 0), *y0s = anchor_split<T>(I, 1), *ax0s = anchor_split<T>(I, 2);
            blk_for(I.n, [&](int j) {
                const T val = v.xh[j];
                v.x[j] = val;
                I.x0[j] = (double)val;
                if (x0s) x0s[j] = split_anchor((double)val);
            });
            blk_for(I.m, [&](int i) {
                const T val = v.yh[i];
                v.y[i] = val;
                I.y0[i] = (double)val;
                if (y0s) y0s[i] = split_anchor((double)val);
                const double ph = I.phat[i];
                I.ax0[i] = ph;
                if (ax0s) ax0s[i] = split_anchor(ph);
                const T axv = (T)ph;
                v.ax[i] = axv;
                if (beta_on) {
                    const T z2 = vmax(v.clb[i], vmin(axv - val * kr.inv_beta, v.cub[i]));
                    v.u[i] = val - kr.beta * (axv - z2);
                }
            });
            __syncthreads();
        }
        if (sizeof(T) == 4 && s.phase_switch) return;
    }
}

template <int BS>
__device__ void blk_solve(const BInst &I, CpalParams p, const BOpts &o, BOut *out, BSmem<BS> &sm, double *sbuf,
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
        s.fp32_switch_tol = o.fp32 ? o.fp32_switch_tol : -1.0;
        s.fp32_stall_limit = o.fp32_stall_evals;
        s.fp32_best_kkt = INFINITY;
        s.iter_limit = p.iteration_limit;
        s.F = p.F;
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
    int fp32_iters = 0;
    if (o.fp32) {
        /* FP32 copies of the scaled problem and the starting point */
        for (int k = threadIdx.x; k < I.nnz; k += kThreads) {
            I.Avf[k] = (float)I.Av[k];
            I.Atvf[k] = (float)I.Atv[k];
        }
        blk_for(I.n, [&](int j) {
            I.cf[j] = (float)I.c[j];
            I.vlbf[j] = (float)I.vlb[j];
            I.vubf[j] = (float)I.vub[j];
            const float xv = (float)I.x0[j];
            I.xf[j] = xv;
            I.xhf[j] = xv;
            I.lamf[j] = 0.f;
            I.xbarf[j] = 0.f;
            I.x0f[j] = split_anchor(I.x0[j]);
        });
        blk_for(I.m, [&](int i) {
            I.clbF[i] = (float)I.clb[i];
            I.cubF[i] = (float)I.cub[i];
            const float yv = (float)I.y0[i];
            I.yf[i] = yv;
            I.yhf[i] = yv;
            I.ybarf[i] = 0.f;
            I.uf[i] = 0.f;
            I.y0f[i] = split_anchor(I.y0[i]);
        });
        __syncthreads();
        blk_init_ax<float, BS>(I, bvec32(I), s, beta_on, sm);
        blk_phase<float, BS>(I, p, sm, sbuf, s, lacc6, sh, beta_on);
        fp32_iters = s.total;
        if (!s.status) {
            /* FP64 refinement from the FP32 iterate (switch_to_fp64) */
            blk_for(I.n, [&](int j) {
                const double xv = (double)I.xhf[j];
                I.xh[j] = xv;
                I.x[j] = xv;
                I.x0[j] = xv;
                I.xbar[j] = (double)I.xbarf[j];
                I.lam[j] = (double)I.lamf[j];
            });
            blk_for(I.m, [&](int i) {
                const double yv = (double)I.yhf[i];
                I.yh[i] = yv;
                I.y[i] = yv;
                I.y0[i] = yv;
                I.ybar[i] = (double)I.ybarf[i];
            });
            if (threadIdx.x == 0) {
                s.inner = 0;
                s.fp_last = INFINITY;
                if (!s.restart) s.fp0 = s.fp;
                s.phase_switch = 0;
                s.fp32_switch_tol = -1.0;
                s.restart = 0;
            }
            __syncthreads();
            blk_init_ax<double, BS>(I, bvec64(I), s, beta_on, sm);
            blk_phase<double, BS>(I, p, sm, sbuf, s, lacc6, sh, beta_on);
        } else {
            blk_for(I.n, [&](int j) { I.xh[j] = (double)I.xhf[j]; });
            blk_for(I.m, [&](int i) { I.yh[i] = (double)I.yhf[i]; });
            __syncthreads();
        }
    } else {
        __syncthreads();
        blk_init_ax<double, BS>(I, bvec64(I), s, beta_on, sm);
        blk_phase<double, BS>(I, p, sm, sbuf, s, lacc6, sh, beta_on);
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
        blk_spmv<1>(I.nbAt, I.Atdesc, I.Atlinfo, I.Atlpart, I.Atlcount, I.nlAt, I.Atrp, I.Atci,
                    (const double *)I.Atv, g, re, z, sm.one);
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
        r.fp32_iterations = fp32_iters;
        r.pad = 0;
        *out = r;
    }
    __syncthreads();
}

/* MINB: resident blocks per SM the register allocation targets (more
 * resident instances hide more of each block's load latency). */
template <int MINB, int BS>
__global__ void __launch_bounds__(kThreads, MINB) k_batch_lp(const BInst *__restrict__ insts, int count,
                                                             const int *__restrict__ order, unsigned *queue,
                                                             CpalParams p, BOpts o, BOut *outs) {
    extern __shared__ __align__(16) unsigned char batch_dyn_smem[];
    BSmem<BS> &sm = *reinterpret_cast<BSmem<BS> *>(batch_dyn_smem);
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
        blk_solve<BS>(I, p, o, outs + idx, sm, sbuf, s, &lacc6, &lacc1, sh);
    }
}

} // namespace batch
} // namespace pdal
