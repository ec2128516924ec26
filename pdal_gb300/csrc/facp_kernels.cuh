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
    MODE_POLISH_EVAL_P = 8, /* feasibility polishing: primal-phase residual */
    MODE_POLISH_EVAL_D = 9, /* feasibility polishing: dual-phase residual */
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

/* The segment (iteration) path runs in T: FP64, or FP32 in the first phase
 * of the chosen form.  SegV<T> holds what that path reads and writes in T;
 * in FP32 the Halpern anchors stay FP64-accurate as unevaluated (hi, lo)
 * float pairs, and every reduction still accumulates in FP64.  The FP64
 * vectors of Prob are the state between launches: an FP32 segment converts
 * them in at its start and back at its end. */
template <typename T>
struct AnchorOf {
    using type = double;
};
template <>
struct AnchorOf<float> {
    using type = float2;
};

template <typename T>
struct SegV {
    const T *c, *vlb, *vub, *clb, *cub, *diag;
    T *x, *xh, *xbar, *y, *yh, *ybar, *dprod, *dslack, *dx, *dy, *qx, *rx, *grad, *dir, *aldual;
    typename AnchorOf<T>::type *x0, *y0;
    const T *mv[NMAT]; /* matrix values */
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
    int bar_extra;          /* blocks a barrier waits for beyond the launch (failure-path test only) */
    long long spin_limit;   /* polls before a barrier wait gives up */
    GridBar *bar;
    Ctl *ctl;
    double *out_x, *out_y, *out_rc;
    SegV<float> f; /* FP32 mirror (chosen form only; null pointers otherwise) */
    /* feasibility polishing phases: the solve's objective, finite bounds and
     * primal solution, which the phase residuals read (null otherwise) */
    const double *ref_c, *ref_clb_fin, *ref_cub_fin, *ref_xh;
};

struct Args {
    int mode;
    int t0, t1, inner0, F;
    int fp_first, has_inner, inner_limit, use_al;
    int linf, infeas;
    int max_iter;
    int fp32; /* MODE_SEGMENT: run the segment in FP32 */
    int polish; /* MODE_SEGMENT: 0 the solve; 1 (2) a primal (dual) polishing phase, whose
                   fixed-point error is |x_bar - x|^2 w (|y_bar - y|^2 / w) */
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
    RowBlockSmem<kS, 1, float> &smf; /* the same shared bytes, typed for FP32 */
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
        if (prev == cx.nb + (unsigned)cx.P.bar_extra - 1) {
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
                if (++spins > cx.P.spin_limit) {
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

/* Runs the row blocks of matrix `mat` owned by this block, with values `val`
 * in the arithmetic type T. */
template <typename T, class Gat, class Epi, class R>
__device__ __forceinline__ void spmv_t(Cx &cx, int mat, const T *val, Gat &gat, Epi &epi, R &red) {
    const DMat &M = cx.P.M[mat];
    RowBlockSmem<kS, 1, T> *sm;
    if constexpr (sizeof(T) == sizeof(double))
        sm = &cx.sm;
    else
        sm = &cx.smf;
    for (int b = blockIdx.x; b < M.plan.nblocks; b += gridDim.x) {
        rowblock_run_at<kS, 1, T>(b, M.plan, M.rp, M.ci, val, gat, epi, red, *sm);
        __syncthreads();
    }
}

/* FP64 products of the evaluation, restart and power paths. */
template <class Gat, class Epi, class R>
__device__ __forceinline__ void spmv(Cx &cx, const DMat &M, Gat &gat, Epi &epi, R &red) {
    for (int b = blockIdx.x; b < M.plan.nblocks; b += gridDim.x) {
        rowblock_run_at<kS, 1, double>(b, M.plan, M.rp, M.ci, M.v, gat, epi, red, cx.sm);
        __syncthreads();
    }
}

template <typename T>
struct GatT {
    const T *v;
    __device__ __forceinline__ void operator()(int col, T (&o)[1]) const { o[0] = v[col]; }
};
using Gat = GatT<double>;

template <class F>
__device__ __forceinline__ void foreach_elem(const Cx &cx, int count, F f) {
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < count; i += cx.nb * kThreads) f(i);
}

/* Epilogue that stores the row sum (no reduction terms). */
template <typename T>
struct EpiStoreT {
    T *out;
    __device__ __forceinline__ void operator()(int row, const T (&s)[1], Red<1, 0> &) const { out[row] = s[0]; }
    __device__ __forceinline__ void long_red(int, Red<1, 0> &) const {}
};
using EpiStore = EpiStoreT<double>;

/* Adds the long-row reduction terms of `lr` to the row's slot. */
template <int NS, int NM>
__device__ __forceinline__ void add_long(const Cx &cx, int mat, int lid, const Red<NS, NM> &lr) {
    double *s = long_slot(cx, mat, lid);
#pragma unroll
    for (int i = 0; i < NS; ++i) s[i] += lr.s[i];
#pragma unroll
    for (int i = 0; i < NM; ++i) s[NS + i] = fmax(s[NS + i], lr.mx[i]);
}

__device__ __forceinline__ double tmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ double tmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float tmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float tmin(float a, float b) { return fminf(a, b); }

/* Halpern average w * r + (1 - w) * anchor; the FP32 form keeps the anchor
 * as (hi, lo) and adds both parts (FP64-accurate anchor, FP32 arithmetic). */
__device__ __forceinline__ double halpern_avg(double w, double rv, double a) { return w * rv + (1.0 - w) * a; }
__device__ __forceinline__ float halpern_avg(float w, float rv, float2 a) {
    const float omw = 1.0f - w;
    return fmaf(w, rv, fmaf(omw, a.x, omw * a.y));
}
__device__ __forceinline__ float2 split_anchor(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

__device__ __forceinline__ SegV<double> seg64(const Prob &P) {
    SegV<double> v;
    v.c = P.c;
    v.vlb = P.vlb;
    v.vub = P.vub;
    v.clb = P.clb;
    v.cub = P.cub;
    v.diag = P.diag;
    v.x = P.x;
    v.xh = P.xh;
    v.xbar = P.xbar;
    v.y = P.y;
    v.yh = P.yh;
    v.ybar = P.ybar;
    v.dprod = P.dprod;
    v.dslack = P.dslack;
    v.dx = P.dx;
    v.dy = P.dy;
    v.qx = P.qx;
    v.rx = P.rx;
    v.grad = P.grad;
    v.dir = P.dir;
    v.aldual = P.aldual;
    v.x0 = P.x0;
    v.y0 = P.y0;
    for (int k = 0; k < NMAT; ++k) v.mv[k] = P.M[k].v;
    return v;
}

/* ------------------------------------------------------------------ objective product */

/* In the LOW_RANK_SPARSE form the R'R v row sum is added to the stored Q v
 * (cuSPARSE's beta = 1 accumulation in the reference); every other form
 * passes the row sum through. */
template <typename T>
__device__ __forceinline__ T q_total_t(int qtype, const T *qx, int j, T s) {
    return qtype == Q_LOWRANK_SPARSE ? s + qx[j] : s;
}
__device__ __forceinline__ double q_total(const Prob &P, int j, double s) { return q_total_t(P.qtype, P.qx, j, s); }

/* y = Q v for the objective term (solver_state.cu:371-442 of the reference):
 * SPARSE Q v; DIAG d.*v; LOW_RANK R'(R v); LOW_RANK_SPARSE Q v + R'(R v).
 * The final product of each row goes through `epi` (which may fuse more work);
 * `qx` receives Q v first in the LOW_RANK_SPARSE form. */
template <typename T, class Epi, class R>
__device__ bool obj_product_t(Cx &cx, const SegV<T> &V, const T *v, Epi &epi, R &red, unsigned &lmask) {
    const Prob &P = cx.P;
    switch (P.qtype) {
    case Q_SPARSE: {
        GatT<T> g{v};
        spmv_t<T>(cx, MAT_Q, V.mv[MAT_Q], g, epi, red);
        lmask |= 1u << MAT_Q;
        return true;
    }
    case Q_DIAG: {
        foreach_elem(cx, P.n, [&](int j) {
            const T s[1] = {V.diag[j] * v[j]};
            epi(j, s, red);
        });
        return true;
    }
    case Q_LOWRANK:
    case Q_LOWRANK_SPARSE: {
        Red<1, 0> dummy;
        if (P.qtype == Q_LOWRANK_SPARSE) {
            GatT<T> g{v};
            EpiStoreT<T> st{V.qx};
            spmv_t<T>(cx, MAT_Q, V.mv[MAT_Q], g, st, dummy);
        }
        {
            GatT<T> g{v};
            EpiStoreT<T> st{V.rx};
            spmv_t<T>(cx, MAT_R, V.mv[MAT_R], g, st, dummy);
        }
        FACP_SYNC(cx);
        GatT<T> g{(const T *)V.rx};
        spmv_t<T>(cx, MAT_RT, V.mv[MAT_RT], g, epi, red);
        lmask |= 1u << MAT_RT;
        return true;
    }
    default: /* Q_NONE: the product buffer keeps its contents (zeros) */
        foreach_elem(cx, P.n, [&](int j) {
            const T s[1] = {V.qx[j]};
            epi(j, s, red);
        });
        return true;
    }
}

template <class Epi, class R>
__device__ bool obj_product(Cx &cx, const double *v, Epi &epi, R &red, unsigned &lmask) {
    const SegV<double> V = seg64(cx.P);
    return obj_product_t<double>(cx, V, v, epi, red, lmask);
}

/* ------------------------------------------------------------------ iteration pieces */

/* u = y - sigma (p - P(p - y/sigma)), p = A v   (fa_cp_core_op.cu:181-192, 275-303) */
template <typename T>
struct EpiAlDual {
    const SegV<T> *V;
    T sigma;
    __device__ __forceinline__ void operator()(int i, const T (&s)[1], Red<1, 0> &) const {
        const T p = s[0];
        const T yi = V->y[i];
        const T shifted = p - yi / sigma;
        const T proj = tmax(V->clb[i], tmin(shifted, V->cub[i]));
        V->aldual[i] = yi - sigma * (p - proj);
    }
    __device__ __forceinline__ void long_red(int, Red<1, 0> &) const {}
};

/* dprod = A' u with u = y (plain) or the AL effective dual at v. */
template <typename T>
__device__ bool dual_product(Cx &cx, const SegV<T> &V, const T *v, bool al) {
    Red<1, 0> dummy;
    const T *u = V.y;
    if (al) {
        GatT<T> g{v};
        EpiAlDual<T> e{&V, (T)cx.a.sigma};
        spmv_t<T>(cx, MAT_A, V.mv[MAT_A], g, e, dummy);
        FACP_SYNC(cx);
        u = V.aldual;
    }
    GatT<T> g{u};
    EpiStoreT<T> st{V.dprod};
    spmv_t<T>(cx, MAT_AT, V.mv[MAT_AT], g, st, dummy);
    FACP_SYNC(cx);
    return true;
}

/* BB init (fa_cp_core_op.cu:398-417): g = Qx + c - q; x' = P(x - alpha g).
 * s1 accumulates |x|^2 (the FP32 form's floor of the inner tolerance). */
template <typename T>
struct EpiBBInit {
    const SegV<T> *V;
    int qtype;
    T alpha;
    __device__ __forceinline__ void operator()(int j, const T (&s)[1], Red<2, 0> &r) const {
        const T qxj = q_total_t(qtype, (const T *)V->qx, j, s[0]);
        V->qx[j] = qxj;
        const T g = qxj + V->c[j] - V->dprod[j];
        const T xj = V->x[j];
        T nx = xj - alpha * g;
        nx = tmax(V->vlb[j], tmin(nx, V->vub[j]));
        V->xh[j] = nx;
        V->grad[j] = g;
        const T d = nx - xj;
        V->dir[j] = d;
        r.s[0] += (double)d * (double)d;
        r.s[1] += (double)xj * (double)xj;
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<2, 0> &lr) const { add_long(*cx, mat, lid, lr); }
};

/* BB gradient (fa_cp_core_op.cu:401-417): g' = Qx' + c - q + (x' - x)/tau;
 * dg = g' - g; dot(d, dg) accumulates. */
template <typename T>
struct EpiBBGrad {
    const SegV<T> *V;
    int qtype;
    T inv;
    __device__ __forceinline__ void operator()(int j, const T (&s)[1], Red<1, 0> &r) const {
        const T qxj = q_total_t(qtype, (const T *)V->qx, j, s[0]);
        V->qx[j] = qxj;
        const T last = V->grad[j];
        const T cur = qxj + V->c[j] - V->dprod[j] + inv * (V->xh[j] - V->x[j]);
        const T dg = cur - last;
        V->grad[j] = cur;
        r.s[0] += (double)V->dir[j] * (double)dg;
    }
    const Cx *cx;
    int mat;
    __device__ __forceinline__ void long_red(int lid, Red<1, 0> &lr) const { add_long(*cx, mat, lid, lr); }
};

__device__ __forceinline__ int obj_long_mat(int qtype) {
    return (qtype == Q_LOWRANK || qtype == Q_LOWRANK_SPARSE) ? MAT_RT : MAT_Q;
}

/* FP32 form: the BB loop also stops once |d| is at the FP32 resolution of
 * the iterate (kF32Floor |x|), below which the FP32 step cannot make progress. */
constexpr double kF32Floor = 1e-6;

/* Projected BB on the primal subproblem (fa_cp_core_op.cu:445-503).  Leaves
 * x' in xh; returns false on a barrier failure. */
template <typename T>
__device__ bool bb_solve(Cx &cx, const SegV<T> &V, double tau, bool al, double &inner_tol, long long &inner_total) {
    const Prob &P = cx.P;
    const double inv = 1.0 / tau;
    double alpha = 1.0 / inv;
    int it = 1;
    if (!dual_product<T>(cx, V, V.x, al)) return false;
    double tol = inner_tol;
    double ng;
    {
        Red<2, 0> r;
        r.zero();
        unsigned lmask = 0;
        EpiBBInit<T> e{&V, P.qtype, (T)alpha, &cx, obj_long_mat(P.qtype)};
        if (!obj_product_t<T>(cx, V, V.x, e, r, lmask)) return false;
        double tot[2];
        if (!greduce<2, 0>(cx, r, lmask, tot)) return false;
        ng = sqrt(tot[0]);
        if (sizeof(T) == sizeof(float)) tol = fmax(tol, kF32Floor * sqrt(tot[1]));
    }
    double tot[1];
    while (it < cx.a.inner_limit) {
        if (ng <= tol) break;
        if (al && !dual_product<T>(cx, V, V.xh, true)) return false;
        {
            Red<1, 0> r;
            r.zero();
            unsigned lmask = 0;
            EpiBBGrad<T> e{&V, P.qtype, (T)inv, &cx, obj_long_mat(P.qtype)};
            if (!obj_product_t<T>(cx, V, V.xh, e, r, lmask)) return false;
            if (!greduce<1, 0>(cx, r, lmask, tot)) return false;
        }
        alpha = ng * ng / tot[0];
        {
            Red<1, 0> r;
            r.zero();
            const T al_t = (T)alpha;
            foreach_elem(cx, P.n, [&](int j) {
                const T cur = V.xh[j];
                T nx = cur - al_t * V.grad[j];
                nx = tmax(V.vlb[j], tmin(nx, V.vub[j]));
                const T d = nx - cur;
                V.dir[j] = d;
                V.xh[j] = nx;
                r.s[0] += (double)d * (double)d;
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
template <typename T>
struct EpiPrimalClosed {
    const SegV<T> *V;
    T tau, w, refl;
    int wm, fp, diag;
    __device__ __forceinline__ void operator()(int j, const T (&s)[1], Red<3, 0> &r) const {
        const T xj = V->x[j];
        T t = xj - tau * (V->c[j] - s[0]);
        if (diag) t = t / (T(1) + tau * V->diag[j]);
        const T pr = tmax(V->vlb[j], tmin(t, V->vub[j]));
        const T xb = T(2) * pr - xj;
        V->xbar[j] = xb;
        if (wm) {
            V->xh[j] = pr;
            if (!diag) V->dslack[j] = (pr - t) / tau;
        }
        if (fp) {
            const T d = xb - xj;
            V->dx[j] = d;
            r.s[0] += (double)d * (double)d;
        }
        const T refl_v = refl * xb + (T(1) - refl) * xj;
        V->x[j] = halpern_avg(w, refl_v, V->x0[j]);
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<3, 0> &lr) const { add_long(*cx, MAT_AT, lid, lr); }
};

/* Dual step (AL form fa_cp_core_op.cu:194-223 or the Moreau form 156-179)
 * fused into the A x-bar SpMV, with the fixed-point delta and Halpern on y. */
template <typename T>
struct EpiDual {
    const SegV<T> *V;
    T rho, sigma, w, refl;
    int wm, fp, al;
    __device__ __forceinline__ void operator()(int i, const T (&s)[1], Red<3, 0> &r) const {
        const T p = s[0];
        const T yi = V->y[i];
        T yb;
        if (al) {
            const T denom = sigma + rho;
            const T shifted = p - yi / denom;
            const T proj = tmax(V->clb[i], tmin(shifted, V->cub[i]));
            const T nd = yi + rho * (proj - p);
            if (wm) V->yh[i] = nd;
            yb = T(2) * nd - yi;
        } else {
            const T t = yi / rho - p;
            const T tp = tmax(-V->cub[i], tmin(t, -V->clb[i]));
            if (wm) {
                const T yhi = (t - tp) * rho;
                V->yh[i] = yhi;
                yb = T(2) * yhi - yi;
            } else {
                yb = T(2) * (t - tp) * rho - yi;
            }
        }
        V->ybar[i] = yb;
        if (fp) {
            const T d = yb - yi;
            V->dy[i] = d;
            r.s[1] += (double)d * (double)d;
        }
        const T refl_v = refl * yb + (T(1) - refl) * yi;
        V->y[i] = halpern_avg(w, refl_v, V->y0[i]);
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<3, 0> &lr) const { add_long(*cx, MAT_A, lid, lr); }
};

/* <A'dy, dx> of the fixed-point error (fa_cp_core_op.cu:1042-1089). */
template <typename T>
struct EpiCrossT {
    const SegV<T> *V;
    __device__ __forceinline__ void operator()(int j, const T (&s)[1], Red<3, 0> &r) const {
        V->dprod[j] = s[0];
        r.s[2] += (double)s[0] * (double)V->dx[j];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<3, 0> &lr) const { add_long(*cx, MAT_AT, lid, lr); }
};

/* One outer iteration at total count k.  The Halpern average of x and y is
 * applied as soon as the reflected point is known: the fixed-point error only
 * needs the deltas, which are taken from the pre-update values. */
template <typename T>
__device__ bool iteration(Cx &cx, const SegV<T> &V, int k, int inner, bool fp, double &inner_tol,
                          long long &inner_total, double &fp_out) {
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
        GatT<T> g{(const T *)V.y};
        EpiPrimalClosed<T> e{&V, (T)a.tau, (T)w, (T)a.refl, wm ? 1 : 0, fp ? 1 : 0, P.qtype == Q_DIAG ? 1 : 0, &cx};
        spmv_t<T>(cx, MAT_AT, V.mv[MAT_AT], g, e, fr);
        if (fp) fmask |= 1u << MAT_AT;
        FACP_SYNC(cx);
    } else {
        if (!bb_solve<T>(cx, V, a.tau, al, inner_tol, inner_total)) return false;
        const T w_t = (T)w, refl_t = (T)a.refl;
        foreach_elem(cx, P.n, [&](int j) {
            const T xj = V.x[j];
            const T xb = T(2) * V.xh[j] - xj;
            V.xbar[j] = xb;
            if (fp) {
                const T d = xb - xj;
                V.dx[j] = d;
                fr.s[0] += (double)d * (double)d;
            }
            const T refl_v = refl_t * xb + (T(1) - refl_t) * xj;
            V.x[j] = halpern_avg(w_t, refl_v, V.x0[j]);
        });
        FACP_SYNC(cx);
    }
    {
        GatT<T> g{(const T *)V.xbar};
        EpiDual<T> e{&V, (T)a.rho, (T)a.sigma, (T)w, (T)a.refl, wm ? 1 : 0, fp ? 1 : 0, al ? 1 : 0, &cx};
        spmv_t<T>(cx, MAT_A, V.mv[MAT_A], g, e, fr);
        if (fp) fmask |= 1u << MAT_A;
        FACP_SYNC(cx);
    }
    if (fp) {
        GatT<T> g{(const T *)V.dy};
        EpiCrossT<T> e{&V, &cx};
        spmv_t<T>(cx, MAT_AT, V.mv[MAT_AT], g, e, fr);
        fmask |= 1u << MAT_AT;
        double tot[3];
        if (!greduce<3, 0>(cx, fr, fmask, tot)) return false;
        const double pn = sqrt(tot[0]), dn = sqrt(tot[1]);
        const double movement = pn * pn * a.pw + dn * dn / a.pw;
        const double interaction = 2 * a.step * tot[2];
        /* fa_cp_core_op.cu:1705-1735 in a polishing phase (no square root) */
        fp_out = a.polish == 1 ? tot[0] * a.pw : a.polish == 2 ? tot[1] / a.pw : sqrt(fmax(movement + interaction, 0.0));
        if (a.has_inner) inner_tol = fmin(inner_tol, fmax(0.0005 * pn / a.step * a.pw, 1e-9));
    }
    return true;
}

template <typename T>
__device__ bool run_segment_t(Cx &cx, const SegV<T> &V) {
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
        if (!iteration<T>(cx, V, k, inner, need_fp, inner_tol, inner_total, f)) return false;
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

/* The FP64 state between launches is converted into the FP32 mirror at the
 * start of an FP32 segment (iterates, anchors as (hi, lo), the buffers the
 * evaluation and restart read or modify) and back at its end. */
__device__ bool run_segment(Cx &cx) {
    const Prob &P = cx.P;
    if (!cx.a.fp32) {
        const SegV<double> V = seg64(P);
        return run_segment_t<double>(cx, V);
    }
    const SegV<float> &F = P.f;
    foreach_elem(cx, P.n, [&](int j) {
        F.x[j] = (float)P.x[j];
        F.xh[j] = (float)P.xh[j];
        F.dslack[j] = (float)P.dslack[j];
        F.dx[j] = (float)P.dx[j];
        F.x0[j] = split_anchor(P.x0[j]);
    });
    foreach_elem(cx, P.m, [&](int i) {
        F.y[i] = (float)P.y[i];
        F.yh[i] = (float)P.yh[i];
        F.dy[i] = (float)P.dy[i];
        F.y0[i] = split_anchor(P.y0[i]);
    });
    FACP_SYNC(cx);
    if (!run_segment_t<float>(cx, F)) return false;
    FACP_SYNC(cx);
    foreach_elem(cx, P.n, [&](int j) {
        P.x[j] = (double)F.x[j];
        P.xh[j] = (double)F.xh[j];
        P.dslack[j] = (double)F.dslack[j];
        P.dx[j] = (double)F.dx[j];
    });
    foreach_elem(cx, P.m, [&](int i) {
        P.y[i] = (double)F.y[i];
        P.yh[i] = (double)F.yh[i];
        P.dy[i] = (double)F.dy[i];
    });
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

/* ------------------------------------------------------------------ feasibility polishing */

/* primal phase (utils.cu:1456-1470, 1491-1529): |A x^ clamped-residual .* r|
 * and the solve's objective at x^ */
struct EpiPolishRows {
    const Prob *P;
    __device__ __forceinline__ void operator()(int i, const double (&s)[1], Red<2, 1> &r) const {
        const double p = s[0];
        const double cl = fmax(P->clb[i], fmin(p, P->cub[i]));
        const double res = (p - cl) * P->rcum[i];
        r.s[0] += res * res;
        r.mx[0] = fmax(r.mx[0], fabs(res));
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<2, 1> &lr) const { add_long(*cx, MAT_A, lid, lr); }
};

/* dual phase (utils.cu:1472-1489, 1531-1574): |(c - A'y^ - slack) .* d| and
 * the slack's product with the solve's primal solution */
struct EpiPolishCols {
    const Prob *P;
    __device__ __forceinline__ void operator()(int j, const double (&s)[1], Red<2, 1> &r) const {
        const double res = (P->c[j] - s[0] - P->dslack[j]) * P->dcum[j];
        r.s[0] += res * res;
        r.mx[0] = fmax(r.mx[0], fabs(res));
        r.s[1] += P->dslack[j] * P->ref_xh[j];
    }
    const Cx *cx;
    __device__ __forceinline__ void long_red(int lid, Red<2, 1> &lr) const { add_long(*cx, MAT_AT, lid, lr); }
};

__device__ bool run_polish_eval(Cx &cx, bool primal) {
    const Prob &P = cx.P;
    const Args &a = cx.a;
    double t[3], o[2];
    {
        Red<2, 1> r;
        r.zero();
        if (primal) {
            Gat g{P.xh};
            EpiPolishRows e{&P, &cx};
            spmv(cx, P.M[MAT_A], g, e, r);
            if (!greduce<2, 1>(cx, r, 1u << MAT_A, t)) return false;
        } else {
            Gat g{P.yh};
            EpiPolishCols e{&P, &cx};
            spmv(cx, P.M[MAT_AT], g, e, r);
            if (!greduce<2, 1>(cx, r, 1u << MAT_AT, t)) return false;
        }
    }
    {
        Red<2, 0> r;
        r.zero();
        if (primal) {
            foreach_elem(cx, P.n, [&](int j) { r.s[0] += P.ref_c[j] * P.xh[j]; });
        } else {
            foreach_elem(cx, P.m, [&](int i) {
                const double yi = P.yh[i];
                r.s[1] += fmax(yi, 0.0) * P.ref_clb_fin[i] + fmin(yi, 0.0) * P.ref_cub_fin[i];
            });
        }
        if (!greduce<2, 0>(cx, r, 0u, o)) return false;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctl *c = P.ctl;
        if (primal) {
            const double ap = P.m > 0 ? (a.linf ? t[2] : sqrt(t[0])) : 0.0;
            c->abs_p = ap / a.cbr;
            c->rel_p = c->abs_p / (1.0 + a.bnd_norm);
            c->pobj = o[0] / (a.cbr * a.ovr) + a.c0;
        } else {
            const double ad = a.linf ? t[2] : sqrt(t[0]);
            c->abs_d = ad / a.ovr;
            c->rel_d = c->abs_d / (1.0 + a.obj_norm);
            c->dobj = (t[1] + o[1]) / (a.cbr * a.ovr) + a.c0;
        }
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
    const SegV<double> V = seg64(P);
    EpiCrossT<double> e{&V, &cx};
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
    static_assert(sizeof(RowBlockSmem<kS, 1, float>) <= sizeof(RowBlockSmem<kS, 1, double>), "shared staging");
    __shared__ __align__(16) unsigned char smraw[sizeof(RowBlockSmem<kS, 1, double>)];
    __shared__ double stot[kSlot];
    __shared__ int sok;
    Cx cx{P, a, *reinterpret_cast<RowBlockSmem<kS, 1, double> *>(smraw),
          *reinterpret_cast<RowBlockSmem<kS, 1, float> *>(smraw), stot, &sok, gridDim.x, 0};
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
    case MODE_POLISH_EVAL_P:
        ok = run_polish_eval(cx, true);
        break;
    case MODE_POLISH_EVAL_D:
        ok = run_polish_eval(cx, false);
        break;
    default:
        ok = false;
    }
    if (!ok && threadIdx.x == 0) atomicExch(&P.ctl->status, 1);
}

} // namespace facp
} // namespace pdal
