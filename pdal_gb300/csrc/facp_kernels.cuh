/*
 * facp_kernels.cuh -- the FA_CP (convex QP) iteration as ONE persistent
 * cooperative kernel (sm_103a).
 *
 * The reference drives every step from the host: per outer iteration a
 * cuSPARSE SpMV plus elementwise kernels, and per projected Barzilai-Borwein
 * (BB) inner step two host-synchronising cuBLAS reductions
 * (QP/FA_CP/src/fa_cp_core_op.cu:445-503, 531-630).  Here a launch runs a
 * whole segment of iterations between two evaluation points -- the BB inner
 * loop with its data-dependent stop included -- with every block resident
 * (cooperative launch) and the phases separated by grid barriers:
 *
 *   phase                         work                              barrier
 *   dual product  q = A'y         row-block SpMV over A'            yes
 *   closed-form primal            fused into the A' SpMV epilogue   -
 *   BB init / gradient            Q (or R, R') SpMV + epilogue      reduce
 *   BB direction                  elementwise + |d|^2               reduce
 *   reflection + Halpern on x     elementwise                       yes
 *   dual step + Halpern on y      row-block SpMV over A + epilogue  yes
 *   fixed-point cross term        A' SpMV of dy (major iterations)  reduce
 *
 * Grid reductions are deterministic: every block writes one partial slot,
 * and after the barrier every block adds the slots in the same fixed order,
 * so all blocks hold the same total without a second barrier.  Terms of rows
 * longer than one row block are accumulated in per-row slots (in phase
 * order) and added after the block slots.
 *
 * Every barrier wait is bounded: after kSpinLimit polls a block records an
 * error in the barrier word and returns; blocks that see the error return at
 * their next barrier, and the host reports the failure.
 *
 * Vectors written during a launch are read with plain (coherent) loads, never
 * through the read-only path; only the matrices use streaming loads.
 */
#pragma once

#include "rowblock.cuh"

#include <cuda_runtime.h>

namespace pdal {
namespace facp {

constexpr int kS = 1024;       /* nonzeros per row block */
constexpr int kSlot = 16;      /* doubles per reduction slot */
constexpr long long kSpinLimit = 1ll << 25;

enum : int { MAT_A = 0, MAT_AT = 1, MAT_Q = 2, MAT_R = 3, MAT_RT = 4, NMAT = 5 };
enum : int { Q_SPARSE = 0, Q_DIAG = 1, Q_LOWRANK_SPARSE = 2, Q_LOWRANK = 3, Q_NONE = 4 };

enum : int {
    MODE_SEGMENT = 0,
    MODE_EVAL = 1,
    MODE_RESTART = 2,
    MODE_DELTA_SCORE = 3,
    MODE_RESULT = 4,
    MODE_POWER_A = 5,
    MODE_POWER_QMAX = 6,
    MODE_POWER_QMIN = 7,
};

struct DMat {
    const int *rp;
    const int *ci;
    const double *v;
    RowPlanDev plan;
    int rows;
    int lbase; /* first long-row reduction slot of this matrix */
};

struct GridBar {
    unsigned int count;
    unsigned int gen;
    int err;
    int pad;
};

/* Scalars the kernel produces (device memory, read by the host after a launch). */
struct Ctl {
    double inner_tol;
    double fp;       /* last fixed-point error */
    double fp_first; /* fixed-point error of the first iteration of the segment */
    long long inner_total;
    int status;
    int pad;
    double abs_p, abs_d, pobj, dobj, rel_p, rel_d, gap, rel_gap;
    double max_pray, max_dray, pray_lin, dray_obj;
    double pd, dd, normal_dist, score;
    double power_value;
    int power_iters;
    int pad2;
};

struct Prob {
    int n, m, nr, qtype;
    DMat M[NMAT];
    const double *c, *vlb, *vub, *clb, *cub, *clb_fin, *cub_fin, *vlb_fin, *vub_fin, *diag, *dcum, *rcum;
    double *x0, *x, *xh, *xbar, *y0, *y, *yh, *ybar;
    double *dprod, *dslack, *dx, *dy, *qx, *rx, *grad, *dir, *aldual;
    double *pv, *pv2, *pv3; /* power-iteration vectors, max(m, n) each */
    double *part;           /* 3 windows x grid x kSlot */
    double *lpart;          /* 3 windows x nlong_total x kSlot (zero at launch) */
    int nlong_total;
    int pad;
    GridBar *bar;
    Ctl *ctl;
    double *out_x, *out_y, *out_rc;
};

struct Args {
    int mode;
    int t0, t1, inner0, F;
    int fp_first, has_inner, inner_limit, use_al;
    int linf, infeas;
    int max_iter;
    double tau, rho, step, pw, sigma, refl;
    double tau_eval;
    double cbr, ovr, c0, obj_norm, bnd_norm;
    double tol, lam_max;
};

__device__ __forceinline__ int print_frequency(int iter) { /* QP/FA_CP/src/utils.cu:694-703 */
    int step = 10;
    long long threshold = 1000;
    while (iter >= threshold) {
        step *= 10;
        threshold *= 10;
    }
    return step;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ double clampd(double v, double lo, double hi) { return fmax(lo, fmin(v, hi)); }

/* Per-block context. */
struct Cx {
    const Prob &P;
    const Args &a;
    RowBlockSmem<kS, 1, double> &sm;
    double *stot; /* shared: totals of the last reduction */
    int *sok;     /* shared: barrier status */
    unsigned nb;
    int parity;
};

__device__ bool gsync(Cx &cx) {
    GridBar *b = cx.P.bar;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned g = ld_acquire(&b->gen);
        __threadfence();
        const unsigned prev = atomicAdd(&b->count, 1u);
        if (prev == cx.nb - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            long long spins = 0;
            while (ld_acquire(&b->gen) == g) {
                if (*(volatile int *)&b->err) {
                    ok = 0;
                    break;
                }
                if (++spins > kSpinLimit) {
                    atomicExch(&b->err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*(volatile int *)&b->err) ok = 0;
        *cx.sok = ok;
    }
    __syncthreads();
    return *cx.sok != 0;
}

#define FACP_SYNC(cx)                                                                                                  \
    do {                                                                                                               \
        if (!gsync(cx)) return false;                                                                                  \
    } while (0)

/* Slot of long row `lid` of matrix `mat` in the current reduction window
 * (cx.parity cycles over three buffers). */
__device__ __forceinline__ double *long_slot(const Cx &cx, int mat, int lid) {
    const int nl = cx.P.nlong_total > 0 ? cx.P.nlong_total : 1;
    return cx.P.lpart + ((size_t)cx.parity * nl + (size_t)(cx.P.M[mat].lbase + lid)) * kSlot;
}

/*
 * Deterministic grid reduction of NS sums and NM maxima.  lmask selects the
 * matrices whose long-row slots (filled by SpMV epilogues since the previous
 * reduction) are added after the block slots.  Totals land in cx.stot and in
 * `tot` for every thread of every block.
 */
template <int NS, int NM>
__device__ bool greduce(Cx &cx, Red<NS, NM> &r, unsigned lmask, double (&tot)[NS + NM]) {
    static_assert(NS + NM <= kSlot, "too many reduction terms");
    constexpr int NQ = NS + NM;
    const Prob &P = cx.P;
    double *buf = P.part + (size_t)cx.parity * cx.nb * kSlot;
    block_reduce<kThreads, NS, NM>(r, cx.sm.red);
    if (threadIdx.x == 0) {
        double *s = buf + (size_t)blockIdx.x * kSlot;
#pragma unroll
        for (int i = 0; i < NS; ++i) s[i] = r.s[i];
#pragma unroll
        for (int i = 0; i < NM; ++i) s[NS + i] = r.mx[i];
    }
    FACP_SYNC(cx);
    const int nl = P.nlong_total > 0 ? P.nlong_total : 1;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int q = 0; q < NQ; ++q) {
            const bool is_max = q >= NS;
            double acc = 0.0;
            for (unsigned b = lane; b < cx.nb; b += 32) {
                const double v = buf[(size_t)b * kSlot + q];
                acc = is_max ? fmax(acc, v) : acc + v;
            }
            for (int mat = 0; mat < NMAT; ++mat) {
                if (!(lmask & (1u << mat))) continue;
                const int nlong = P.M[mat].plan.nlong;
                for (int l = lane; l < nlong; l += 32) {
                    const double v = P.lpart[((size_t)cx.parity * nl + (size_t)(P.M[mat].lbase + l)) * kSlot + q];
                    acc = is_max ? fmax(acc, v) : acc + v;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double w = __shfl_xor_sync(0xffffffffu, acc, o);
                acc = is_max ? fmax(acc, w) : acc + w;
            }
            if (lane == 0) cx.stot[q] = acc;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; ++q) tot[q] = cx.stot[q];
    /* Buffers rotate over three reduction windows.  The one of window W-1
     * was read by every block before this barrier and is written next in
     * window W+2, whose epilogues start after the barrier of window W+1:
     * clear it now. */
    {
        double *old_buf = P.lpart + (size_t)((cx.parity + 2) % 3) * nl * kSlot;
        const size_t cnt = (size_t)P.nlong_total * kSlot;
        for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < cnt; i += (size_t)cx.nb * kThreads)
            old_buf[i] = 0.0;
    }
    cx.parity = (cx.parity + 1) % 3;
    __syncthreads();
    return true;
}

/* Runs the row blocks of M owned by this block. */
template <class Gat, class Epi, class R>
__device__ __forceinline__ void spmv(Cx &cx, const DMat &M, Gat &gat, Epi &epi, R &red) {
    for (int b = blockIdx.x; b < M.plan.nblocks; b += gridDim.x) {
        rowblock_run_at<kS, 1, double>(b, M.plan, M.rp, M.ci, M.v, gat, epi, red, cx.sm);
        __syncthreads();
    }
}

struct Gat {
    const double *v;
    __device__ __forceinline__ void operator()(int col, double (&o)[1]) const { o[0] = v[col]; }
};

template <class F>
__device__ __forceinline__ void foreach_elem(const Cx &cx, int count, F f) {
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < count; i += cx.nb * kThreads) f(i);
}

/* Epilogue that stores the row sum (no reduction terms). */
struct EpiStore {
    double *out;
    __device__ __forceinline__ void operator()(int row, const double (&s)[1], Red<1, 0> &) const { out[row] = s[0]; }
    __device__ __forceinline__ void long_red(int, Red<1, 0> &) const {}
};

/* Adds the long-row reduction terms of `lr` to the row's slot. */
template <int NS, int NM>
__device__ __forceinline__ void add_long(const Cx &cx, int mat, int lid, const Red<NS, NM> &lr) {
    double *s = long_slot(cx, mat, lid);
#pragma unroll
    for (int i = 0; i < NS; ++i) s[i] += lr.s[i];
#pragma unroll
    for (int i = 0; i < NM; ++i) s[NS + i] = fmax(s[NS + i], lr.mx[i]);
}

/* ------------------------------------------------------------------ objective product */

/* y = Q v for the objective term (solver_state.cu:371-442 of the reference):
 * SPARSE Q v; DIAG d.*v; LOW_RANK R'(R v); LOW_RANK_SPARSE Q v + R'(R v).
 * The final product of each row goes through `epi` (which may fuse more work);
 * `qtmp` receives Q v first in the LOW_RANK_SPARSE form. */
template <class Epi, class R>
__device__ bool obj_product(Cx &cx, const double *v, Epi &epi, R &red, unsigned &lmask) {
    const Prob &P = cx.P;
    switch (P.qtype) {
    case Q_SPARSE: {
        Gat g{v};
        spmv(cx, P.M[MAT_Q], g, epi, red);
        lmask |= 1u << MAT_Q;
        return true;
    }
    case Q_DIAG: {
        foreach_elem(cx, P.n, [&](int j) {
            const double s[1] = {P.diag[j] * v[j]};
            epi(j, s, red);
        });
        return true;
    }
    case Q_LOWRANK:
    case Q_LOWRANK_SPARSE: {
        Red<1, 0> dummy;
        if (P.qtype == Q_LOWRANK_SPARSE) {
            Gat g{v};
            EpiStore st{P.qx};
            spmv(cx, P.M[MAT_Q], g, st, dummy);
        }
        {
            Gat g{v};
            EpiStore st{P.rx};
            spmv(cx, P.M[MAT_R], g, st, dummy);
        }
        FACP_SYNC(cx);
        Gat g{P.rx};
        spmv(cx, P.M[MAT_RT], g, epi, red);
        lmask |= 1u << MAT_RT;
        return true;
    }
    default: /* Q_NONE: the product buffer keeps its contents (zeros) */
        foreach_elem(cx, P.n, [&](int j) {
            const double s[1] = {P.qx[j]};
            epi(j, s, red);
        });
        return true;
    }
}

/* In the LOW_RANK_SPARSE form the R'R v row sum is added to the stored Q v
 * (cuSPARSE's beta = 1 accumulation in the reference); every other form
 * passes the row sum through. */
__device__ __forceinline__ double q_total(const Prob &P, int j, double s) {
    return P.qtype == Q_LOWRANK_SPARSE ? s + P.qx[j] : s;
}

/* ------------------------------------------------------------------ iteration pieces */

/* u = y - sigma (p - P(p - y/sigma)), p = A v   (fa_cp_core_op.cu:181-192, 275-303) */
struct EpiAlDual {
    const Prob *P;
    double sigma;
    __device__ __forceinline__ void operator()(int i, const double (&s)[1], Red<1, 0> &) const {
        const double p = s[0];
        const double yi = P->y[i];
        const double shifted = p - yi / sigma;
        const double proj = fmax(P->clb[i], fmin(shifted, P->cub[i]));
        P->aldual[i] = yi - sigma * (p - proj);
    }
    __device__ __forceinline__ void long_red(int, Red<1, 0> &) const {}
};

/* dprod = A' u with u = y (plain) or the AL effective dual at v. */
__device__ bool dual_product(Cx &cx, const double *v, bool al) {
    const Prob &P = cx.P;
    Red<1, 0> dummy;
    const double *u = P.y;
    if (al) {
        Gat g{v};
        EpiAlDual e{&P, cx.a.sigma};
        spmv(cx, P.M[MAT_A], g, e, dummy);
        FACP_SYNC(cx);
        u = P.aldual;
    }
    Gat g{u};
    EpiStore st{P.dprod};
    spmv(cx, P.M[MAT_AT], g, st, dummy);
    FACP_SYNC(cx);
    return true;
}

/* BB init (fa_cp_core_op.cu:398-417): g = Qx + c - q; x' = P(x - alpha g). */
struct EpiBBInit {
    const Prob *P;
    double alpha;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<1, 0> &r) const {
        const double qxj = q_total(*P, j, s[0]);
        P->qx[j] = qxj;
        const double g = qxj + P->c[j] - P->dprod[j];
        const double xj = P->x[j];
        double nx = xj - alpha * g;
        nx = fmax(P->vlb[j], fmin(nx, P->vub[j]));
        P->xh[j] = nx;
        P->grad[j] = g;
        const double d = nx - xj;
        P->dir[j] = d;
        r.s[0] += d * d;
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<1, 0> &lr) const { add_long(*cx, mat, lid, lr); }
};

/* BB gradient (fa_cp_core_op.cu:401-417): g' = Qx' + c - q + (x' - x)/tau;
 * dg = g' - g; dot(d, dg) accumulates. */
struct EpiBBGrad {
    const Prob *P;
    double inv;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<1, 0> &r) const {
        const double qxj = q_total(*P, j, s[0]);
        P->qx[j] = qxj;
        const double last = P->grad[j];
        const double cur = qxj + P->c[j] - P->dprod[j] + inv * (P->xh[j] - P->x[j]);
        const double dg = cur - last;
        P->grad[j] = cur;
        r.s[0] += P->dir[j] * dg;
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<1, 0> &lr) const { add_long(*cx, mat, lid, lr); }
};

__device__ __forceinline__ int obj_long_mat(int qtype) {
    return (qtype == Q_LOWRANK || qtype == Q_LOWRANK_SPARSE) ? MAT_RT : MAT_Q;
}

/* Projected BB on the primal subproblem (fa_cp_core_op.cu:445-503).  Leaves
 * x' in xh; returns false on a barrier failure. */
__device__ bool bb_solve(Cx &cx, double tau, bool al, double &inner_tol, long long &inner_total) {
    const Prob &P = cx.P;
    const double inv = 1.0 / tau;
    double alpha = 1.0 / inv;
    int it = 1;
    if (!dual_product(cx, P.x, al)) return false;
    double tot[1];
    {
        Red<1, 0> r;
        r.zero();
        unsigned lmask = 0;
        EpiBBInit e{&P, alpha, &cx, obj_long_mat(P.qtype)};
        if (!obj_product(cx, P.x, e, r, lmask)) return false;
        if (!greduce<1, 0>(cx, r, lmask, tot)) return false;
    }
    double ng = sqrt(tot[0]);
    while (it < cx.a.inner_limit) {
        if (ng <= inner_tol) break;
        if (al && !dual_product(cx, P.xh, true)) return false;
        {
            Red<1, 0> r;
            r.zero();
            unsigned lmask = 0;
            EpiBBGrad e{&P, inv, &cx, obj_long_mat(P.qtype)};
            if (!obj_product(cx, P.xh, e, r, lmask)) return false;
            if (!greduce<1, 0>(cx, r, lmask, tot)) return false;
        }
        alpha = ng * ng / tot[0];
        {
            Red<1, 0> r;
            r.zero();
            foreach_elem(cx, P.n, [&](int j) {
                const double cur = P.xh[j];
                double nx = cur - alpha * P.grad[j];
                nx = fmax(P.vlb[j], fmin(nx, P.vub[j]));
                const double d = nx - cur;
                P.dir[j] = d;
                P.xh[j] = nx;
                r.s[0] += d * d;
            });
            if (!greduce<1, 0>(cx, r, 0u, tot)) return false;
        }
        ng = sqrt(tot[0]);
        it++;
    }
    inner_total += it - 1;
    return true;
}

/* Closed-form primal step (LP and diagonal Q without AL) fused into the A'y
 * SpMV (fa_cp_core_op.cu:93-154, 305-347), with the reflection, the fixed-point
 * delta and the Halpern average of x. */
struct EpiPrimalClosed {
    const Prob *P;
    double tau, w, refl;
    int wm, fp, diag;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<3, 0> &r) const {
        const double xj = P->x[j];
        double t = xj - tau * (P->c[j] - s[0]);
        if (diag) t = t / (1.0 + tau * P->diag[j]);
        const double pr = fmax(P->vlb[j], fmin(t, P->vub[j]));
        const double xb = 2.0 * pr - xj;
        P->xbar[j] = xb;
        if (wm) {
            P->xh[j] = pr;
            if (!diag) P->dslack[j] = (pr - t) / tau;
        }
        if (fp) {
            const double d = xb - xj;
            P->dx[j] = d;
            r.s[0] += d * d;
        }
        const double refl_v = refl * xb + (1.0 - refl) * xj;
        P->x[j] = w * refl_v + (1.0 - w) * P->x0[j];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<3, 0> &lr) const { add_long(*cx, MAT_AT, lid, lr); }
};

/* Dual step (AL form fa_cp_core_op.cu:194-223 or the Moreau form 156-179)
 * fused into the A x-bar SpMV, with the fixed-point delta and Halpern on y. */
struct EpiDual {
    const Prob *P;
    double rho, sigma, w, refl;
    int wm, fp, al;
    __device__ __forceinline__ void operator()(int i, const double (&s)[1], Red<3, 0> &r) const {
        const double p = s[0];
        const double yi = P->y[i];
        double yb;
        if (al) {
            const double denom = sigma + rho;
            const double shifted = p - yi / denom;
            const double proj = fmax(P->clb[i], fmin(shifted, P->cub[i]));
            const double nd = yi + rho * (proj - p);
            if (wm) P->yh[i] = nd;
            yb = 2.0 * nd - yi;
        } else {
            const double t = yi / rho - p;
            const double tp = fmax(-P->cub[i], fmin(t, -P->clb[i]));
            if (wm) {
                const double yhi = (t - tp) * rho;
                P->yh[i] = yhi;
                yb = 2.0 * yhi - yi;
            } else {
                yb = 2.0 * (t - tp) * rho - yi;
            }
        }
        P->ybar[i] = yb;
        if (fp) {
            const double d = yb - yi;
            P->dy[i] = d;
            r.s[1] += d * d;
        }
        const double refl_v = refl * yb + (1.0 - refl) * yi;
        P->y[i] = w * refl_v + (1.0 - w) * P->y0[i];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<3, 0> &lr) const { add_long(*cx, MAT_A, lid, lr); }
};

/* <A'dy, dx> of the fixed-point error (fa_cp_core_op.cu:1042-1089). */
struct EpiCross {
    const Prob *P;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<3, 0> &r) const {
        P->dprod[j] = s[0];
        r.s[2] += s[0] * P->dx[j];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<3, 0> &lr) const { add_long(*cx, MAT_AT, lid, lr); }
};

/* One outer iteration at total count k.  The Halpern average of x and y is
 * applied as soon as the reflected point is known: the fixed-point error only
 * needs the deltas, which are taken from the pre-update values. */
__device__ bool iteration(Cx &cx, int k, int inner, bool fp, double &inner_tol, long long &inner_total,
                          double &fp_out) {
    const Prob &P = cx.P;
    const Args &a = cx.a;
    const bool major = ((k + 1) % a.F) == 0;
    const bool wm = major || ((k + 2) % print_frequency(k + 2)) == 0;
    const double w = (double)(inner + 1) / (inner + 2);
    const bool al = a.use_al != 0;
    const bool closed = !al && (P.qtype == Q_NONE || P.qtype == Q_DIAG);
    Red<3, 0> fr;
    fr.zero();
    unsigned fmask = 0;
    if (closed) {
        Gat g{P.y};
        EpiPrimalClosed e{&P, a.tau, w, a.refl, wm ? 1 : 0, fp ? 1 : 0, P.qtype == Q_DIAG ? 1 : 0, &cx};
        spmv(cx, P.M[MAT_AT], g, e, fr);
        if (fp) fmask |= 1u << MAT_AT;
        FACP_SYNC(cx);
    } else {
        if (!bb_solve(cx, a.tau, al, inner_tol, inner_total)) return false;
        foreach_elem(cx, P.n, [&](int j) {
            const double xj = P.x[j];
            const double xb = 2.0 * P.xh[j] - xj;
            P.xbar[j] = xb;
            if (fp) {
                const double d = xb - xj;
                P.dx[j] = d;
                fr.s[0] += d * d;
            }
            const double refl_v = a.refl * xb + (1.0 - a.refl) * xj;
            P.x[j] = w * refl_v + (1.0 - w) * P.x0[j];
        });
        FACP_SYNC(cx);
    }
    {
        Gat g{P.xbar};
        EpiDual e{&P, a.rho, a.sigma, w, a.refl, wm ? 1 : 0, fp ? 1 : 0, al ? 1 : 0, &cx};
        spmv(cx, P.M[MAT_A], g, e, fr);
        if (fp) fmask |= 1u << MAT_A;
        FACP_SYNC(cx);
    }
    if (fp) {
        Gat g{P.dy};
        EpiCross e{&P, &cx};
        spmv(cx, P.M[MAT_AT], g, e, fr);
        fmask |= 1u << MAT_AT;
        double tot[3];
        if (!greduce<3, 0>(cx, fr, fmask, tot)) return false;
        const double pn = sqrt(tot[0]), dn = sqrt(tot[1]);
        const double movement = pn * pn * a.pw + dn * dn / a.pw;
        const double interaction = 2 * a.step * tot[2];
        fp_out = sqrt(fmax(movement + interaction, 0.0));
        if (a.has_inner) inner_tol = fmin(inner_tol, fmax(0.0005 * pn / a.step * a.pw, 1e-9));
    }
    return true;
}

__device__ bool run_segment(Cx &cx) {
    const Args &a = cx.a;
    Ctl *ctl = cx.P.ctl;
    double inner_tol = ctl->inner_tol;
    long long inner_total = ctl->inner_total;
    double fp = ctl->fp, fp_first = ctl->fp_first;
    int inner = a.inner0;
    for (int k = a.t0; k < a.t1; ++k, ++inner) {
        const bool major = ((k + 1) % a.F) == 0;
        const bool first = (k == a.t0) && a.fp_first;
        const bool need_fp = major || first;
        double f = fp;
        if (!iteration(cx, k, inner, need_fp, inner_tol, inner_total, f)) return false;
        if (need_fp) {
            fp = f;
            if (first) fp_first = f;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->inner_tol = inner_tol;
        ctl->inner_total = inner_total;
        ctl->fp = fp;
        ctl->fp_first = fp_first;
    }
    return true;
}

/* ------------------------------------------------------------------ evaluation */

/* Primal residual terms of A x-hat (utils.cu:705-770): s0 |r_p|^2, s1 sum of
 * the dual-objective contributions, mx0 |r_p|. */
struct EpiEvalRows {
    const Prob *P;
    __device__ __forceinline__ void operator()(int i, const double (&s)[1], Red<2, 1> &r) const {
        const double p = s[0];
        const double cl = fmax(P->clb[i], fmin(p, P->cub[i]));
        const double res = (p - cl) * P->rcum[i];
        r.s[0] += res * res;
        r.mx[0] = fmax(r.mx[0], fabs(res));
        const double yi = P->yh[i];
        r.s[1] += fmax(yi, 0.0) * P->clb_fin[i] + fmin(yi, 0.0) * P->cub_fin[i];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<2, 1> &lr) const { add_long(*cx, MAT_A, lid, lr); }
};

/* Dual residual terms (LP form utils.cu:705-733 uses the stored dual slack;
 * QP form 735-770 recomputes it): sums |r_d|^2, c'x, slack'x, x'Qx,
 * |A'y .* d|^2, |Qx .* d|^2; maxima |r_d|, |A'y .* d|, |Qx .* d|. */
struct EpiEvalCols {
    const Prob *P;
    double tau;
    int lp;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<6, 3> &r) const {
        const double xj = P->xh[j];
        const double dj = P->dcum[j];
        double res;
        if (lp) {
            const double q = s[0];
            res = (P->c[j] - q - P->dslack[j]) * dj;
            r.s[2] += P->dslack[j] * xj;
        } else {
            const double qxj = q_total(*P, j, s[0]);
            const double q = P->dprod[j];
            const double g = qxj + P->c[j] - q;
            const double t = xj - tau * g;
            const double pt = fmax(P->vlb[j], fmin(P->vub[j], t));
            const double ds = (pt - t) / tau;
            res = (g - ds) * dj;
            P->dslack[j] = ds;
            r.s[2] += ds * xj;
            r.s[3] += xj * qxj;
            const double aq = q * dj, qq = qxj * dj;
            r.s[4] += aq * aq;
            r.s[5] += qq * qq;
            r.mx[1] = fmax(r.mx[1], fabs(aq));
            r.mx[2] = fmax(r.mx[2], fabs(qq));
        }
        r.s[0] += res * res;
        r.mx[0] = fmax(r.mx[0], fabs(res));
        r.s[1] += P->c[j] * xj;
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<6, 3> &lr) const { add_long(*cx, mat, lid, lr); }
};

/* Infeasibility rays (utils.cu:1028-1132) from the last fixed-point deltas. */
struct EpiRayRows {
    const Prob *P;
    __device__ __forceinline__ void operator()(int i, const double (&s)[1], Red<2, 1> &r) const {
        const double p = s[0];
        const double pinf = (fmax(0.0, -p) * (double)isfinite(P->clb[i]) + fmax(0.0, p) * (double)isfinite(P->cub[i])) *
                            P->rcum[i];
        r.mx[0] = fmax(r.mx[0], fabs(pinf));
        const double dyi = P->dy[i];
        r.s[0] += fmax(dyi, 0.0) * P->clb_fin[i] + fmin(dyi, 0.0) * P->cub_fin[i];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<2, 1> &lr) const { add_long(*cx, MAT_A, lid, lr); }
};

struct EpiRayCols {
    const Prob *P;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<2, 1> &r) const {
        const double dp = s[0];
        P->dprod[j] = dp;
        r.s[0] += fmax(-dp, 0.0) * P->vlb_fin[j] + fmin(-dp, 0.0) * P->vub_fin[j];
        r.s[1] += P->c[j] * P->dx[j];
        const double d = -dp;
        const double dinf = (fmax(0.0, d) * (double)!isfinite(P->vlb[j]) - fmin(0.0, d) * (double)!isfinite(P->vub[j])) *
                            P->dcum[j];
        P->dslack[j] = dinf;
        r.mx[0] = fmax(r.mx[0], fabs(dinf));
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<2, 1> &lr) const { add_long(*cx, MAT_AT, lid, lr); }
};

struct EpiQRay {
    const Prob *P;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<0, 1> &r) const {
        const double q = q_total(*P, j, s[0]);
        P->qx[j] = q;
        r.mx[0] = fmax(r.mx[0], fabs(q));
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<0, 1> &lr) const { add_long(*cx, mat, lid, lr); }
};

__device__ bool run_eval(Cx &cx) {
    const Prob &P = cx.P;
    const Args &a = cx.a;
    const bool lp = P.qtype == Q_NONE;
    double rowt[3], colt[9];
    {
        Red<2, 1> r;
        r.zero();
        Gat g{P.xh};
        EpiEvalRows e{&P, &cx};
        spmv(cx, P.M[MAT_A], g, e, r);
        if (!greduce<2, 1>(cx, r, 1u << MAT_A, rowt)) return false;
    }
    {
        Red<6, 3> r;
        r.zero();
        unsigned lmask = 0;
        Gat g{P.yh};
        if (lp) {
            EpiEvalCols e{&P, a.tau_eval, 1, &cx, MAT_AT};
            spmv(cx, P.M[MAT_AT], g, e, r);
            lmask |= 1u << MAT_AT;
        } else {
            Red<1, 0> dummy;
            EpiStore st{P.dprod};
            spmv(cx, P.M[MAT_AT], g, st, dummy);
            FACP_SYNC(cx);
            EpiEvalCols e{&P, a.tau_eval, 0, &cx, obj_long_mat(P.qtype)};
            if (!obj_product(cx, P.xh, e, r, lmask)) return false;
        }
        if (!greduce<6, 3>(cx, r, lmask, colt)) return false;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctl *c = P.ctl;
        double ap = a.linf ? rowt[2] : sqrt(rowt[0]);
        double ad = a.linf ? colt[6] : sqrt(colt[0]);
        if (P.m == 0) ap = 0.0;
        c->abs_p = ap / a.cbr;
        c->abs_d = ad / a.ovr;
        const double half = lp ? 0.0 : 0.5 * colt[3];
        c->pobj = (colt[1] + half) / (a.cbr * a.ovr) + a.c0;
        c->dobj = (colt[2] + rowt[1] - half) / (a.cbr * a.ovr) + a.c0;
        c->rel_p = c->abs_p / (1.0 + a.bnd_norm);
        if (lp) {
            c->rel_d = c->abs_d / (1.0 + a.obj_norm);
        } else {
            const double qn = a.linf ? colt[8] : sqrt(colt[5]);
            const double an = a.linf ? colt[7] : sqrt(colt[4]);
            c->rel_d = c->abs_d / (1.0 + fmax(a.obj_norm, fmax(qn / a.ovr, an / a.ovr)));
        }
        c->gap = fabs(c->pobj - c->dobj);
        c->rel_gap = c->gap / (1.0 + fabs(c->pobj) + fabs(c->dobj));
    }
    if (!a.infeas) return true;
    /* rays: project the deltas, normalise the primal one */
    double nt[2];
    {
        Red<0, 2> r;
        r.zero();
        foreach_elem(cx, P.n, [&](int j) {
            double v = P.dx[j];
            if (isfinite(P.vlb[j])) v = fmax(v, 0.0);
            if (isfinite(P.vub[j])) v = fmin(v, 0.0);
            P.dx[j] = v;
            r.mx[0] = fmax(r.mx[0], fabs(v));
        });
        foreach_elem(cx, P.m, [&](int i) {
            double v = P.dy[i];
            if (!isfinite(P.clb[i])) v = fmin(v, 0.0);
            if (!isfinite(P.cub[i])) v = fmax(v, 0.0);
            P.dy[i] = v;
            r.mx[1] = fmax(r.mx[1], fabs(v));
        });
        if (!greduce<0, 2>(cx, r, 0u, nt)) return false;
    }
    const double pnorm = nt[0], dnorm = nt[1];
    if (pnorm > 0.0) {
        const double sc = 1.0 / pnorm;
        foreach_elem(cx, P.n, [&](int j) { P.dx[j] = sc * P.dx[j]; });
        FACP_SYNC(cx);
    }
    double rt[3], ct[3];
    {
        Red<2, 1> r;
        r.zero();
        Gat g{P.dx};
        EpiRayRows e{&P, &cx};
        spmv(cx, P.M[MAT_A], g, e, r);
        if (!greduce<2, 1>(cx, r, 1u << MAT_A, rt)) return false;
    }
    {
        Red<2, 1> r;
        r.zero();
        Gat g{P.dy};
        EpiRayCols e{&P, &cx};
        spmv(cx, P.M[MAT_AT], g, e, r);
        if (!greduce<2, 1>(cx, r, 1u << MAT_AT, ct)) return false;
    }
    double qray = 0.0;
    if (!lp) {
        Red<0, 1> r;
        r.zero();
        unsigned lmask = 0;
        EpiQRay e{&P, &cx, obj_long_mat(P.qtype)};
        if (!obj_product(cx, P.dx, e, r, lmask)) return false;
        double qt[1];
        if (!greduce<0, 1>(cx, r, lmask, qt)) return false;
        qray = qt[0];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctl *c = P.ctl;
        c->pray_lin = ct[1] / (a.cbr * a.ovr);
        c->dray_obj = (rt[0] + ct[0]) / (a.cbr * a.ovr);
        double mp = P.m > 0 ? rt[2] : 0.0;
        if (!lp) mp = fmax(mp, qray / a.ovr);
        c->max_pray = mp;
        const double dsn = P.n > 0 ? ct[2] : 0.0;
        double md = dsn, dro = c->dray_obj;
        const double sf = fmax(dnorm, dsn);
        if (sf > 0.0) {
            md /= sf;
            dro /= sf;
        } else {
            md = 0.0;
            dro = 0.0;
        }
        c->max_dray = md;
        c->dray_obj = dro;
    }
    return true;
}

/* ------------------------------------------------------------------ restart support */

struct EpiSumSq {
    double *store;
    __device__ __forceinline__ void operator()(int row, const double (&s)[1], Red<1, 0> &r) const {
        if (store) store[row] = s[0];
        r.s[0] += s[0] * s[0];
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<1, 0> &lr) const { add_long(*cx, mat, lid, lr); }
};

/* |xh - x0|, |yh - y0| and |A (xh - x0)| (fa_cp_core_op.cu:908-962). */
__device__ bool run_restart(Cx &cx) {
    const Prob &P = cx.P;
    double t[2];
    {
        Red<2, 0> r;
        r.zero();
        foreach_elem(cx, P.n, [&](int j) {
            const double d = P.xh[j] - P.x0[j];
            P.dx[j] = d;
            r.s[0] += d * d;
        });
        foreach_elem(cx, P.m, [&](int i) {
            const double d = P.yh[i] - P.y0[i];
            P.dy[i] = d;
            r.s[1] += d * d;
        });
        if (!greduce<2, 0>(cx, r, 0u, t)) return false;
    }
    double nm[1];
    {
        Red<1, 0> r;
        r.zero();
        Gat g{P.dx};
        EpiSumSq e{nullptr, &cx, MAT_A};
        spmv(cx, P.M[MAT_A], g, e, r);
        if (!greduce<1, 0>(cx, r, 1u << MAT_A, nm)) return false;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.ctl->pd = sqrt(t[0]);
        P.ctl->dd = sqrt(t[1]);
        P.ctl->normal_dist = sqrt(nm[0]);
    }
    return true;
}

/* Fixed-point score of the Halpern point against the current iterate
 * (fa_cp_core_op.cu:1091-1128). */
__device__ bool run_delta_score(Cx &cx) {
    const Prob &P = cx.P;
    const Args &a = cx.a;
    Red<3, 0> r;
    r.zero();
    foreach_elem(cx, P.n, [&](int j) {
        const double d = P.xh[j] - P.x[j];
        P.dx[j] = d;
        r.s[0] += d * d;
    });
    foreach_elem(cx, P.m, [&](int i) {
        const double d = P.yh[i] - P.y[i];
        P.dy[i] = d;
        r.s[1] += d * d;
    });
    FACP_SYNC(cx);
    Gat g{P.dy};
    EpiCross e{&P, &cx};
    spmv(cx, P.M[MAT_AT], g, e, r);
    double t[3];
    if (!greduce<3, 0>(cx, r, 1u << MAT_AT, t)) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double pn = sqrt(t[0]), dn = sqrt(t[1]);
        const double movement = pn * pn * a.pw + dn * dn / a.pw;
        const double interaction = 2.0 * a.step * t[2];
        P.ctl->score = sqrt(fmax(movement + interaction, 0.0));
    }
    return true;
}

/* Unscaled solution and reduced cost (fa_cp_core_op.cu:1171-1239). */
struct EpiResult {
    const Prob *P;
    double ovr, cbr;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<1, 0> &) const {
        P->out_rc[j] = (P->c[j] - s[0]) * P->dcum[j] / ovr;
        P->out_x[j] = P->xh[j] / P->dcum[j] / cbr;
    }
    __device__ __forceinline__ void long_red(int, Red<1, 0> &) const {}
};

__device__ bool run_result(Cx &cx) {
    const Prob &P = cx.P;
    Red<1, 0> dummy;
    Gat g{P.yh};
    EpiResult e{&P, cx.a.ovr, cx.a.cbr};
    spmv(cx, P.M[MAT_AT], g, e, dummy);
    foreach_elem(cx, P.m, [&](int i) { P.out_y[i] = P.yh[i] / P.rcum[i] / cx.a.ovr; });
    return true;
}

/* ------------------------------------------------------------------ power iterations */

/* sigma_max(A) by power iteration on A A' (QP/FA_CP/src/utils.cu:65-170):
 * pv holds the start vector on entry. */
__device__ bool run_power_a(Cx &cx) {
    const Prob &P = cx.P;
    const Args &a = cx.a;
    double *v = P.pv, *nv = P.pv2, *dp = P.pv3;
    double s2 = 1.0;
    int it = 0;
    for (; it < a.max_iter; ++it) {
        double t[1];
        {
            Red<1, 0> r;
            r.zero();
            foreach_elem(cx, P.m, [&](int i) {
                const double vi = v[i];
                nv[i] = vi;
                r.s[0] += vi * vi;
            });
            if (!greduce<1, 0>(cx, r, 0u, t)) return false;
        }
        const double inv = 1.0 / sqrt(t[0]);
        foreach_elem(cx, P.m, [&](int i) { nv[i] = inv * nv[i]; });
        FACP_SYNC(cx);
        {
            Red<1, 0> dummy;
            Gat g{nv};
            EpiStore st{dp};
            spmv(cx, P.M[MAT_AT], g, st, dummy);
            FACP_SYNC(cx);
        }
        {
            Red<1, 0> r;
            r.zero();
            struct E {
                double *v;
                const double *nv;
                __device__ void operator()(int i, const double (&s)[1], Red<1, 0> &rr) const {
                    v[i] = s[0];
                    rr.s[0] += nv[i] * s[0];
                }
                const Cx *cx;
                __device__ void long_red(int lid, Red<1, 0> &lr) const { add_long(*cx, MAT_A, lid, lr); }
            } e{v, nv, &cx};
            Gat g{dp};
            spmv(cx, P.M[MAT_A], g, e, r);
            if (!greduce<1, 0>(cx, r, 1u << MAT_A, t)) return false;
        }
        s2 = t[0];
        {
            Red<1, 0> r;
            r.zero();
            foreach_elem(cx, P.m, [&](int i) {
                const double w = (-s2 * nv[i]) + v[i];
                nv[i] = w;
                r.s[0] += w * w;
            });
            if (!greduce<1, 0>(cx, r, 0u, t)) return false;
        }
        if (sqrt(t[0]) < a.tol) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.ctl->power_value = sqrt(s2);
        P.ctl->power_iters = it;
    }
    return true;
}

/* Largest eigenvalue of Q (utils.cu:172-238) or, with lam_max given, the
 * smallest through the shift lam_max I - Q (240-315); pv holds the start. */
__device__ bool run_power_q(Cx &cx, bool shifted) {
    const Prob &P = cx.P;
    const Args &a = cx.a;
    double *v = P.pv, *av = P.pv2;
    double lam = 0.0;
    int it = 0;
    for (; it < a.max_iter; ++it) {
        double t[1];
        {
            Red<1, 0> r;
            r.zero();
            foreach_elem(cx, P.n, [&](int j) { r.s[0] += v[j] * v[j]; });
            if (!greduce<1, 0>(cx, r, 0u, t)) return false;
        }
        const double inv = 1.0 / sqrt(t[0]);
        foreach_elem(cx, P.n, [&](int j) { v[j] = inv * v[j]; });
        FACP_SYNC(cx);
        {
            Red<1, 0> r;
            r.zero();
            struct E {
                double *av;
                const double *v;
                double lmax;
                int shifted;
                __device__ void operator()(int j, const double (&s)[1], Red<1, 0> &rr) const {
                    const double q = shifted ? lmax * v[j] + (-1.0 * s[0]) : s[0];
                    av[j] = q;
                    rr.s[0] += v[j] * q;
                }
                const Cx *cx;
                __device__ void long_red(int lid, Red<1, 0> &lr) const { add_long(*cx, MAT_Q, lid, lr); }
            } e{av, v, a.lam_max, shifted ? 1 : 0, &cx};
            Gat g{v};
            spmv(cx, P.M[MAT_Q], g, e, r);
            if (!greduce<1, 0>(cx, r, 1u << MAT_Q, t)) return false;
        }
        const double old = lam;
        lam = t[0];
        if (it > 0 && fabs(lam - old) < a.tol) break;
        foreach_elem(cx, P.n, [&](int j) { v[j] = av[j]; });
        FACP_SYNC(cx);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.ctl->power_value = shifted ? a.lam_max - lam : lam;
        P.ctl->power_iters = it;
    }
    return true;
}

/* ------------------------------------------------------------------ the kernel */

__global__ void __launch_bounds__(kThreads, 2) k_facp(Prob P, Args a) {
    __shared__ RowBlockSmem<kS, 1, double> sm;
    __shared__ double stot[kSlot];
    __shared__ int sok;
    Cx cx{P, a, sm, stot, &sok, gridDim.x, 0};
    bool ok = true;
    switch (a.mode) {
    case MODE_SEGMENT:
        ok = run_segment(cx);
        break;
    case MODE_EVAL:
        ok = run_eval(cx);
        break;
    case MODE_RESTART:
        ok = run_restart(cx);
        break;
    case MODE_DELTA_SCORE:
        ok = run_delta_score(cx);
        break;
    case MODE_RESULT:
        ok = run_result(cx);
        break;
    case MODE_POWER_A:
        ok = run_power_a(cx);
        break;
    case MODE_POWER_QMAX:
        ok = run_power_q(cx, false);
        break;
    case MODE_POWER_QMIN:
        ok = run_power_q(cx, true);
        break;
    default:
        ok = false;
    }
    if (!ok && threadIdx.x == 0) atomicExch(&P.ctl->status, 1);
}

} // namespace facp
} // namespace pdal
