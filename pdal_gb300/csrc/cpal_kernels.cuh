/*
 * cpal_kernels.cuh -- device kernels of the CP_AL (LP) solver.
 *
 * One iteration is two launches, each streaming one matrix once:
 *   k_primal  rows of A^T:  q = A^T u  ->  projected primal step, reflection,
 *             Halpern averaging (LP/CP_AL/src/solver.cu:2340-2397, 2561-2606)
 *   k_dual    rows of A:    p = A xbar ->  dual step, reflection, Halpern
 *             averaging (solver.cu:2399-2457, 2617-2661), and, when the
 *             augmentation beta > 0, the next iteration's predictor
 *             u = y - beta (Ax - P(Ax - y/beta)) (solver.cu:2459-2479).
 * The predictor needs A x for the *next* x.  Since
 *   x+ = w (r xbar + (1-r) x) + (1-w) x0,
 * A x+ = w (r A xbar + (1-r) A x) + (1-w) A x0 is formed from the product the
 * dual kernel already holds and the anchor product A x0 (recomputed exactly at
 * every restart).  This removes the reference's third matrix stream per
 * iteration (solver.cu:2528-2554).
 *
 * Every evaluation block ends with
 *   k_eval_rows / k_eval_cols  the KKT, gap and fixed-point reductions
 *             (utils.cu:812-917, solver.cu:3611-3686) as fused products over
 *             the FP64 matrices,
 *   k_control the scalar controller (cpal_control.h), one block,
 *   k_restart the anchor reset of a restart (solver.cu:3078-3095).
 *
 * T is the arithmetic type of the iteration (double, or float in the FP32
 * phase).  Anchors x0, y0, A x0 and every reduction stay in FP64.
 */
#pragma once

#include "cpal_control.h"
#include "bulk_copy.cuh"
#include "rowblock.cuh"

#include <type_traits>

namespace pdal {

template <typename T>
__device__ __forceinline__ T vmax(T a, T b) {
    return fmax(a, b);
}
template <>
__device__ __forceinline__ float vmax<float>(float a, float b) {
    return fmaxf(a, b);
}
template <typename T>
__device__ __forceinline__ T vmin(T a, T b) {
    return fmin(a, b);
}
template <>
__device__ __forceinline__ float vmin<float>(float a, float b) {
    return fminf(a, b);
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct NoLongRed {
    __device__ __forceinline__ void long_red(int, Red<0, 0> &) const {}
};

/* Programmatic dependent launch of the iteration and FP32 power kernels: the
 * launch of a kernel is prepared while the one before it finishes, and each
 * block waits here until every write of that kernel is visible before it
 * reads anything.  The dependents launch as the blocks exit (no explicit
 * early trigger: blocks dispatched early and parked in the wait made the
 * short kernels of small LPs almost twice as slow).  Without the launch
 * attribute the wait is a no-op. */
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

/* ------------------------------------------------------------------ */
/* iteration                                                           */
/* ------------------------------------------------------------------ */

/* Storage of an FP64 anchor (x0, y0, A x0) as the iteration kernels read it:
 * a double in the FP64 phase, an unevaluated (hi, lo) float pair in the FP32
 * phase so that the anchor keeps FP64 accuracy while all arithmetic stays on
 * the FP32 pipes. */
template <typename T>
struct AnchorT;
template <>
struct AnchorT<double> {
    using type = double;
};
template <>
struct AnchorT<float> {
    using type = float2;
};
template <typename T>
struct WeightT;
template <>
struct WeightT<double> {
    using type = HalpernW;
};
template <>
struct WeightT<float> {
    using type = HalpernWf;
};

__device__ __forceinline__ double halpern(double w, double omw, double refl, double a) { return w * refl + omw * a; }
__device__ __forceinline__ float halpern(float w, float omw, float refl, float2 a) {
    return fmaf(w, refl, fmaf(omw, a.x, omw * a.y));
}

__device__ __forceinline__ float2 split_anchor(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

template <typename T>
struct Coefs {
    T tau, inv_tau, rho, inv_prox, beta, inv_beta, r;
};
__device__ __forceinline__ void load_coefs(const CpalState *s, Coefs<double> &c) {
    c.tau = s->tau;
    c.inv_tau = s->inv_tau;
    c.rho = s->rho;
    c.inv_prox = s->inv_prox;
    c.beta = s->beta;
    c.inv_beta = s->inv_beta;
    c.r = s->refl;
}
__device__ __forceinline__ void load_coefs(const CpalState *s, Coefs<float> &c) {
    c.tau = s->tau_f;
    c.inv_tau = s->inv_tau_f;
    c.rho = s->rho_f;
    c.inv_prox = s->inv_prox_f;
    c.beta = s->beta_f;
    c.inv_beta = s->inv_beta_f;
    c.r = s->refl_f;
}

template <typename T>
struct PrimalArgs {
    T *x, *xbar, *xh, *lam;
    const typename AnchorT<T>::type *x0;
    const T *c, *lb, *ub;
};

template <typename T, bool MAJOR>
struct PrimalEpi : NoLongRed {
    PrimalArgs<T> a;
    Coefs<T> k;
    T w, omw;
    /* row j with product entry s and its inputs x, c, lb, ub, x0 already read
     * (from global memory, or from a staged copy in shared memory) */
    __device__ __forceinline__ void apply(int j, T s, T xj, T cj, T lbj, T ubj,
                                          typename AnchorT<T>::type x0j) const {
        const T t = xj - k.tau * (cj - s);
        const T proj = vmax(lbj, vmin(t, ubj));
        const T xb = T(2) * proj - xj;
        a.xbar[j] = xb;
        if (MAJOR) {
            a.xh[j] = proj;
            a.lam[j] = (proj - t) * k.inv_tau;
        }
        const T refl = k.r * xb + (T(1) - k.r) * xj;
        a.x[j] = halpern(w, omw, refl, x0j);
    }
    __device__ __forceinline__ void operator()(int j, const T *s, Red<0, 0> &) const {
        apply(j, s[0], a.x[j], a.c[j], a.lb[j], a.ub[j], a.x0[j]);
    }
};

template <typename T, int S, bool MAJOR>
__global__ void __launch_bounds__(kThreads) k_primal(RowPlanDev plan, const int *__restrict__ rp,
                                                     const int *__restrict__ ci, const T *__restrict__ val,
                                                     const T *__restrict__ gat, PrimalArgs<T> a,
                                                     const CpalState *__restrict__ st,
                                                     const typename WeightT<T>::type *__restrict__ wt, int koff) {
    pdl_enter();
    if (st->status) return;
    __shared__ RowBlockSmem<S, 1, T> sm;
    PrimalEpi<T, MAJOR> epi;
    epi.a = a;
    load_coefs(st, epi.k);
    epi.w = wt[koff].w;
    epi.omw = wt[koff].omw;
    auto g = [&](int c, T *out) { out[0] = __ldg(gat + c); };
    Red<0, 0> red;
    rowblock_run<S, 1, T>(plan, rp, ci, val, g, epi, red, sm);
}

/* ------------------------------------------------------------------ */
/* the primal product with TMA-staged row blocks                       */
/* ------------------------------------------------------------------ */

/* Row-vector entries staged per row block: rows [r0, r1) are copied from
 * r0 rounded down to a multiple of 4, so at most kMaxRowsPerBlock + 7. */
constexpr int kStageRows = kMaxRowsPerBlock + 8;

/* the epilogue's inputs of a staged row block (ROWS), or nothing */
template <typename T, bool ROWS>
struct StageRows {
    T x[kStageRows], c[kStageRows], lb[kStageRows], ub[kStageRows];
    typename AnchorT<T>::type x0[kStageRows];
};
template <typename T>
struct StageRows<T, false> {};

/* One staged row block: the slice of A^T (column indices, values, row
 * pointers) and, with ROWS, the epilogue's inputs for its rows, each copied
 * by one bulk copy from a 16-byte-aligned start (nonzero k sits at
 * k - (k0 & ~3), row j at j - (r0 & ~3)). */
template <int S, typename T, bool ROWS>
struct __align__(16) PrimalStage {
    int ci[S + 8];
    T val[S + 8];
    int rp[kStageRows];
    StageRows<T, ROWS> rows;
};

template <int S, typename T, bool ROWS>
struct __align__(16) PrimalTmaSmem {
    PrimalStage<S, T, ROWS> st[2];
    /* the gathered entries; in FP32 they overwrite the stage's column
     * indices in place (each thread rewrites only the entries it read) */
    T g[sizeof(T) == 4 ? 4 : S + 8];
    double red[kThreads / 32];
    uint64_t bar[2];
    int last;
    int stop;
};

/* Thread 0 arms `bar` and issues the bulk copies of row block `blk`. */
template <int S, typename T, bool ROWS>
__device__ __forceinline__ void primal_stage_issue(const RowPlanDev &plan, const int *__restrict__ rp,
                                                   const int *__restrict__ ci, const T *__restrict__ val,
                                                   const PrimalArgs<T> &a, int blk, PrimalStage<S, T, ROWS> &s,
                                                   uint64_t *bar) {
    using A = typename AnchorT<T>::type;
    const int4 d = plan.desc[blk];
    const int kb = d.z & ~3, ke = (d.w + 3) & ~3;
    const bool rows = d.y >= d.x;
    const int rb = rows ? (d.x & ~3) : 0, re = rows ? ((d.y + 3) & ~3) : 0, rpe = rows ? ((d.y + 4) & ~3) : 0;
    const unsigned nk = (unsigned)(ke - kb), nr = ROWS ? (unsigned)(re - rb) : 0u, np = (unsigned)(rpe - rb);
    mbar_arrive_expect_tx(bar, nk * (unsigned)(sizeof(int) + sizeof(T)) + np * (unsigned)sizeof(int) +
                                   nr * (unsigned)(4 * sizeof(T) + sizeof(A)));
    if (nk) {
        bulk_g2s(s.ci, ci + kb, nk * sizeof(int), bar);
        bulk_g2s(s.val, val + kb, nk * sizeof(T), bar);
    }
    if (np) bulk_g2s(s.rp, rp + rb, np * sizeof(int), bar);
    if constexpr (ROWS) {
        if (nr) {
            bulk_g2s(s.rows.x, a.x + rb, nr * sizeof(T), bar);
            bulk_g2s(s.rows.c, a.c + rb, nr * sizeof(T), bar);
            bulk_g2s(s.rows.lb, a.lb + rb, nr * sizeof(T), bar);
            bulk_g2s(s.rows.ub, a.ub + rb, nr * sizeof(T), bar);
            bulk_g2s(s.rows.x0, a.x0 + rb, nr * sizeof(A), bar);
        }
    }
}

/* The iteration's A^T u + primal epilogue as a grid of one wave: each block
 * walks row blocks blockIdx.x, blockIdx.x + gridDim.x, ... and, while it
 * gathers, reduces and finishes one, the TMA engine copies the next one's
 * matrix slice (and, with ROWS, its rows' epilogue inputs) into the other
 * stage buffer.  Same lane grouping, fused multiply-add chains and epilogue
 * as k_primal, so the results are bit-identical to it.  A staging wait that
 * runs out sets st->status = kStatusDeviceError and *err, and the block
 * returns. */
constexpr int kStatusDeviceError = 100;

template <typename T, int S, bool MAJOR, bool ROWS>
__global__ void __launch_bounds__(kThreads) k_primal_tma(RowPlanDev plan, const int *__restrict__ rp,
                                                         const int *__restrict__ ci, const T *__restrict__ val,
                                                         const T *__restrict__ gat, PrimalArgs<T> a, CpalState *st,
                                                         const typename WeightT<T>::type *__restrict__ wt, int koff,
                                                         int *err) {
    constexpr int NT = kThreads;
    constexpr int GIT = (S + 8 + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char tma_smem[];
    auto &sm = *reinterpret_cast<PrimalTmaSmem<S, T, ROWS> *>(tma_smem);
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        fence_mbar_init();
    }
    pdl_enter();
    /* one read of the status for the whole block: another block may set it
     * while this one starts */
    if (tid == 0) sm.stop = st->status;
    __syncthreads();
    if (sm.stop) return;
    PrimalEpi<T, MAJOR> epi;
    epi.a = a;
    load_coefs(st, epi.k);
    epi.w = wt[koff].w;
    epi.omw = wt[koff].omw;
    int blk = blockIdx.x;
    if (tid == 0 && blk < plan.nblocks)
        primal_stage_issue<S, T, ROWS>(plan, rp, ci, val, a, blk, sm.st[0], &sm.bar[0]);
    uint32_t parity = 0; /* bit b: the phase of bar[b] to wait for next */
    for (int i = 0; blk < plan.nblocks; ++i, blk += gridDim.x) {
        const int b = i & 1;
        const int nxt = blk + gridDim.x;
        if (tid == 0 && nxt < plan.nblocks) {
            fence_proxy_async_smem();
            primal_stage_issue<S, T, ROWS>(plan, rp, ci, val, a, nxt, sm.st[b ^ 1], &sm.bar[b ^ 1]);
        }
        const uint32_t pb = (parity >> b) & 1u;
        const bool ok = mbar_wait(&sm.bar[b], pb, kStageWaitNs);
        parity ^= 1u << b;
        if (!__syncthreads_and(ok)) {
            if (tid == 0) {
                atomicExch(err, 1);
                atomicExch(&st->status, kStatusDeviceError);
                /* let the copies still in flight land before the block exits */
                mbar_wait(&sm.bar[b], pb, kStageWaitNs);
                if (nxt < plan.nblocks) mbar_wait(&sm.bar[b ^ 1], (parity >> (b ^ 1)) & 1u, kStageWaitNs);
            }
            return;
        }
        PrimalStage<S, T, ROWS> &s = sm.st[b];
        T *gbuf = sizeof(T) == 4 ? reinterpret_cast<T *>(s.ci) : sm.g;
        const int4 d = plan.desc[blk];
        const int k0 = d.z, k1 = d.w, kb = k0 & ~3;
        {
            /* every column index first, then every gather, so that a thread
             * has all its loads of u in flight at once */
            int cols[GIT];
            T gv[GIT];
#pragma unroll
            for (int it = 0; it < GIT; ++it) {
                const int e = kb + it * NT + tid;
                cols[it] = (e >= k0 && e < k1) ? s.ci[it * NT + tid] : -1;
            }
#pragma unroll
            for (int it = 0; it < GIT; ++it) gv[it] = cols[it] >= 0 ? __ldg(gat + cols[it]) : T(0);
#pragma unroll
            for (int it = 0; it < GIT; ++it)
                if (it * NT + tid < S + 8) gbuf[it * NT + tid] = gv[it];
        }
        __syncthreads();
        if (d.y >= d.x) {
            const int r0 = d.x, nrows = d.y - d.x, ro = r0 - (r0 & ~3);
            auto finish = [&](int row, T acc) {
                if constexpr (ROWS) {
                    const int q = ro + row;
                    epi.apply(r0 + row, acc, s.rows.x[q], s.rows.c[q], s.rows.lb[q], s.rows.ub[q], s.rows.x0[q]);
                } else {
                    const T sv[1] = {acc};
                    Red<0, 0> lr;
                    epi(r0 + row, sv, lr);
                }
            };
            if (nrows <= NT) {
                int g = 32;
                while (g > 1 && g * nrows > NT) g >>= 1;
                const int row = tid / g, lane = tid & (g - 1);
                T acc = T(0);
                if (row < nrows) {
                    const int e = s.rp[ro + row + 1] - kb;
                    for (int kk = s.rp[ro + row] - kb + lane; kk < e; kk += g) acc = vfma(s.val[kk], gbuf[kk], acc);
                }
                for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, g);
                if (row < nrows && lane == 0) finish(row, acc);
            } else {
                for (int row = tid; row < nrows; row += NT) {
                    T acc = T(0);
                    const int e = s.rp[ro + row + 1] - kb;
                    for (int kk = s.rp[ro + row] - kb; kk < e; ++kk) acc = vfma(s.val[kk], gbuf[kk], acc);
                    finish(row, acc);
                }
            }
        } else {
            /* one S-slice of a long row: as rowblock_run_at's LONG piece */
            const int lid = ~d.y;
            const int4 li = plan.linfo[lid];
            const int piece = (k0 - li.w) / S;
            T acc[1] = {T(0)};
            for (int kk = k0 - kb + tid; kk < k1 - kb; kk += NT) acc[0] = vfma(s.val[kk], gbuf[kk], acc[0]);
            block_sum_t<1, T>(acc, reinterpret_cast<T *>(sm.red));
            if (tid == 0) {
                plan.lpart[(size_t)(li.z + piece) * kLongStride] = (double)acc[0];
                __threadfence();
                const unsigned prev = atomicAdd(&plan.lcount[lid], 1u);
                sm.last = (prev == (unsigned)(li.y - 1));
            }
            __syncthreads();
            if (sm.last && tid == 0) {
                __threadfence();
                double tot = 0.0;
                for (int q = 0; q < li.y; ++q) tot += __ldcg(&plan.lpart[(size_t)(li.z + q) * kLongStride]);
                plan.lcount[lid] = 0u;
                const T sv[1] = {(T)tot};
                Red<0, 0> lr;
                epi(li.x, sv, lr);
            }
        }
        __syncthreads(); /* stage b and the gathered entries are free for the next refill */
    }
}

template <typename T>
struct DualArgs {
    T *y, *yh, *ybar, *ax, *u;
    const typename AnchorT<T>::type *y0, *ax0;
    const T *lb, *ub;
};

/* Per-row inputs of the dual epilogue, loaded apart from the product so that
 * a kernel can issue them for several rows before any product is ready. */
template <typename T>
struct DualIn {
    T y, lo, hi, ax;
    typename AnchorT<T>::type y0, ax0;
};

template <typename T, bool MAJOR, bool BETA>
struct DualEpi : NoLongRed {
    DualArgs<T> a;
    Coefs<T> k;
    T w, omw;
    __device__ __forceinline__ DualIn<T> fetch(int i) const {
        DualIn<T> d;
        d.y = a.y[i];
        d.lo = a.lb[i];
        d.hi = a.ub[i];
        d.y0 = a.y0[i];
        if (BETA) {
            d.ax = (k.r != T(1)) ? a.ax[i] : T(0);
            d.ax0 = a.ax0[i];
        }
        return d;
    }
    __device__ __forceinline__ void finish(int i, T p, const DualIn<T> &d) const {
        const T yi = d.y;
        const T zb = vmax(d.lo, vmin(p - yi * k.inv_prox, d.hi));
        const T yn = yi - k.rho * (p - zb);
        const T yb = T(2) * yn - yi;
        if (MAJOR) {
            a.yh[i] = yn;
            a.ybar[i] = yb;
        }
        const T refl = k.r * yb + (T(1) - k.r) * yi;
        const T ynew = halpern(w, omw, refl, d.y0);
        a.y[i] = ynew;
        if (BETA) {
            T mix = p;
            if (k.r != T(1)) mix = k.r * p + (T(1) - k.r) * d.ax;
            const T axn = halpern(w, omw, mix, d.ax0);
            a.ax[i] = axn;
            const T z2 = vmax(d.lo, vmin(axn - ynew * k.inv_beta, d.hi));
            a.u[i] = ynew - k.beta * (axn - z2);
        }
    }
    __device__ __forceinline__ void operator()(int i, const T *s, Red<0, 0> &) const { finish(i, s[0], fetch(i)); }
};

template <typename T, int S, bool MAJOR, bool BETA>
__global__ void __launch_bounds__(kThreads) k_dual(RowPlanDev plan, const int *__restrict__ rp,
                                                   const int *__restrict__ ci, const T *__restrict__ val,
                                                   const T *__restrict__ xbar, DualArgs<T> a,
                                                   const CpalState *__restrict__ st,
                                                   const typename WeightT<T>::type *__restrict__ wt, int koff) {
    pdl_enter();
    if (st->status) return;
    __shared__ RowBlockSmem<S, 1, T> sm;
    DualEpi<T, MAJOR, BETA> epi;
    epi.a = a;
    load_coefs(st, epi.k);
    epi.w = wt[koff].w;
    epi.omw = wt[koff].omw;
    /* x-bar gathers bypass L1: the random column gathers of a large LP hit
     * L2, and caching them in L1 only adds L1TEX pressure (measured 3.5%
     * faster for this kernel; the same load in k_primal is slower) */
    auto g = [&](int c, T *out) { out[0] = __ldcg(xbar + c); };
    Red<0, 0> red;
    rowblock_run<S, 1, T>(plan, rp, ci, val, g, epi, red, sm);
}

/* ------------------------------------------------------------------ */
/* the other rows of the dual product, split by length                 */
/* ------------------------------------------------------------------ */
/* With the long rows on panels, the rows of A with at most one nonzero (most
 * rows of a power-law LP) run one thread per row from a compact copy -- row,
 * column and value of the single entry (an empty row has value 0) -- so a row
 * costs three coalesced loads, one gather and its epilogue; a thread takes
 * kShortUnroll rows and issues every load of them before using any.  Rows of
 * 2..kShortMidLen nonzeros run 8 lanes per row, longer rows (up to S) a warp
 * per row, over the CSR arrays.  One launch, each part a fixed number of
 * blocks looping over its rows (one wave, no tail of short-lived blocks). */
constexpr int kShortUnroll = 2;
constexpr int kShortMidLen = 64; /* rows up to this length: 8 lanes each; longer rows: a warp */

template <typename T>
struct ShortDev {
    const int *__restrict__ r1; /* rows with at most one entry, ascending */
    const int *__restrict__ c1; /* its column (0 for an empty row) */
    const T *__restrict__ v1;   /* its value (0 for an empty row) */
    const int *__restrict__ r2; /* rows of 2..kShortMidLen entries, ascending */
    const int *__restrict__ r3; /* rows of kShortMidLen+1..S entries, longest first */
    int n1, n2, n3;             /* row counts */
    int b1, b2, b3;             /* blocks of each part (in that order) */
};

template <typename T, bool MAJOR, bool BETA>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 6 : 4) k_dual_short(ShortDev<T> sd, const int *__restrict__ rp,
                                                         const int *__restrict__ ci, const T *__restrict__ val,
                                                         const T *__restrict__ xbar, DualArgs<T> a,
                                                         const CpalState *__restrict__ st,
                                                         const typename WeightT<T>::type *__restrict__ wt,
                                                         int koff) {
    pdl_enter();
    if (st->status) return;
    DualEpi<T, MAJOR, BETA> epi;
    epi.a = a;
    load_coefs(st, epi.k);
    epi.w = wt[koff].w;
    epi.omw = wt[koff].omw;
    const int b = blockIdx.x;
    const int lane = threadIdx.x & 31;
    if (b < sd.b1) {
        /* one thread per row, kShortUnroll rows per thread at a time */
        const int stride = sd.b1 * kThreads * kShortUnroll;
        for (int base = b * kThreads * kShortUnroll + threadIdx.x; base < sd.n1; base += stride) {
            int row[kShortUnroll], col[kShortUnroll];
            T v[kShortUnroll], g[kShortUnroll];
            DualIn<T> in[kShortUnroll];
#pragma unroll
            for (int u = 0; u < kShortUnroll; ++u) {
                const int t = base + u * kThreads;
                if (t < sd.n1) {
                    row[u] = __ldcs(sd.r1 + t);
                    col[u] = __ldcs(sd.c1 + t);
                    v[u] = __ldcs(sd.v1 + t);
                }
            }
#pragma unroll
            for (int u = 0; u < kShortUnroll; ++u) {
                if (base + u * kThreads < sd.n1) {
                    g[u] = __ldcg(xbar + col[u]);
                    in[u] = epi.fetch(row[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < kShortUnroll; ++u)
                if (base + u * kThreads < sd.n1) epi.finish(row[u], v[u] * g[u], in[u]);
        }
        return;
    }
    if (b < sd.b1 + sd.b2) {
        /* 8 lanes per row, four rows per warp at a time */
        const int sub = lane >> 3, li = lane & 7;
        const int w0 = (b - sd.b1) * (kThreads / 32) + ((int)threadIdx.x >> 5);
        const int nw = sd.b2 * (kThreads / 32);
        const unsigned mask = 0xffu << (8 * sub);
        for (int g0 = w0 * 4; g0 < sd.n2; g0 += nw * 4) {
            const int t = g0 + sub;
            if (t >= sd.n2) continue; /* whole 8-lane groups skip together */
            const int i = __ldcs(sd.r2 + t);
            const int k0 = rp[i], k1 = rp[i + 1];
            DualIn<T> in;
            if (li == 0) in = epi.fetch(i);
            T acc = T(0);
            for (int k = k0 + li; k < k1; k += 8) acc = vfma(__ldcs(val + k), __ldcg(xbar + __ldcs(ci + k)), acc);
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) acc += __shfl_xor_sync(mask, acc, o, 8);
            if (li == 0) epi.finish(i, acc, in);
        }
        return;
    }
    /* a warp per row */
    const int w0 = (b - sd.b1 - sd.b2) * (kThreads / 32) + ((int)threadIdx.x >> 5);
    const int nw = sd.b3 * (kThreads / 32);
    for (int w = w0; w < sd.n3; w += nw) {
        const int i = __ldcs(sd.r3 + w);
        const int k0 = rp[i], k1 = rp[i + 1];
        DualIn<T> in;
        if (lane == 0) in = epi.fetch(i);
        T acc = T(0);
        constexpr int U3 = 8;
        for (int k = k0 + lane; k < k1; k += 32 * U3) {
            T vv[U3];
            int cc[U3];
#pragma unroll
            for (int u = 0; u < U3; ++u) {
                const bool in_row = k + 32 * u < k1;
                vv[u] = in_row ? __ldcs(val + k + 32 * u) : T(0);
                cc[u] = in_row ? __ldcs(ci + k + 32 * u) : 0;
            }
            T g[U3];
#pragma unroll
            for (int u = 0; u < U3; ++u) g[u] = (k + 32 * u < k1) ? __ldcg(xbar + cc[u]) : T(0);
#pragma unroll
            for (int u = 0; u < U3; ++u) acc = vfma(vv[u], g[u], acc);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) epi.finish(i, acc, in);
    }
}

/* ------------------------------------------------------------------ */
/* the long rows of the dual product, by column panels                 */
/* ------------------------------------------------------------------ */
/* Device side of HostPanels (common.h): the long rows' nonzeros in panel
 * order (values in the iteration's type, 16-bit column offsets), the
 * segments {h, k0, k1, p}, the blocks {p, first segment, end segment} and
 * one partial sum per (long row, panel). */
template <typename T>
struct PanelDev {
    const int *__restrict__ rows;
    const int4 *__restrict__ seg;
    const int4 *__restrict__ piece; /* {panel, first segment, end segment} */
    const int4 *__restrict__ cta;   /* {first piece, end piece} per block */
    const T *__restrict__ val;
    const uint16_t *__restrict__ off;
    T *part;
    T *hot; /* the long rows' entries of the primal product's gathered vector (or null) */
    int H, P, W, nblocks;
    /* the row's last segment finishes it (k_dual_panels with FUSE): arrivals
     * per long row (zero between launches) and segments per long row */
    unsigned *cnt;
    const int *nseg;
};

constexpr int kPanelThreads = 512;
constexpr int kPanelLanes = 8;  /* lanes per segment */
constexpr int kPanelUnroll = 2; /* groups of four nonzeros per segment a lane loads before using them */

/* dynamic shared memory of a panel block: the x-bar panel */
template <typename T>
__host__ __device__ constexpr size_t panel_smem_bytes(int W) {
    return (size_t)W * sizeof(T);
}

/* panel values from the CSR values (after equilibration, in each precision) */
template <typename T>
__global__ void k_panel_gather(const int *__restrict__ pmap, const double *__restrict__ src, T *dst, long long len) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
        const int k = pmap[i];
        dst[i] = k >= 0 ? (T)src[k] : T(0);
    }
}

__device__ __forceinline__ void load4_stream(const uint16_t *p, int (&c)[4]) {
    const uint2 t = __ldcs(reinterpret_cast<const uint2 *>(p));
    c[0] = (int)(t.x & 0xffffu);
    c[1] = (int)(t.x >> 16);
    c[2] = (int)(t.y & 0xffffu);
    c[3] = (int)(t.y >> 16);
}

/* One block per range of segments (about equal nonzero counts, one wave).
 * For each panel its range touches, the block stages x-bar[pW, pW + W) in
 * shared memory; then each group of kPanelLanes lanes takes two of the
 * panel's segments at a time.  A lane loads up to kPanelUnroll groups of four
 * nonzeros of each (values with 128-bit streaming loads, 16-bit offsets with
 * 64-bit loads) before using any, gathers from shared memory, and the
 * group's lanes add their sums in a fixed tree into the segments' partial
 * slots.  The sum order is fixed, so results are deterministic. */
template <typename T>
__device__ __forceinline__ void panel_stage(T *sx, const T *__restrict__ xbar, int col0, int wlen) {
    /* x-bar starts 256-byte aligned and W is a multiple of 4, so a panel
     * starts on a 16-byte boundary */
    constexpr int V = 16 / sizeof(T);
    const int nvec = wlen / V;
    using Vec = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    const Vec *src = reinterpret_cast<const Vec *>(xbar + col0);
    Vec *dst = reinterpret_cast<Vec *>(sx);
    for (int i = threadIdx.x; i < nvec; i += 4 * kPanelThreads) {
        Vec t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * kPanelThreads < nvec) t[u] = __ldcg(src + i + u * kPanelThreads);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (i + u * kPanelThreads < nvec) dst[i + u * kPanelThreads] = t[u];
    }
    for (int i = nvec * V + threadIdx.x; i < wlen; i += kPanelThreads) sx[i] = __ldcg(xbar + col0 + i);
}

/* The long rows' partial sums of one launch; with FUSE the group that writes
 * a row's last partial (an arrival counter per row) also adds the row's P
 * partials in FP64 in a fixed order -- 8 lanes over the panels, then a fixed
 * shuffle tree -- and runs the dual epilogue, so that no separate launch is
 * needed (k_dual_long_finish does the same in its own launch). */
template <typename T, bool FUSE, bool MAJOR, bool BETA>
__global__ void __launch_bounds__(kPanelThreads, sizeof(T) == 4 ? 2 : 1) k_dual_panels(PanelDev<T> pd,
                                                                                      const T *__restrict__ xbar,
                                                                                      int n,
                                                                                      const CpalState *__restrict__ st,
                                                                                      DualArgs<T> a,
                                                                                      const typename WeightT<T>::type
                                                                                          *__restrict__ wt,
                                                                                      int koff) {
    pdl_enter();
    if (st->status) return;
    extern __shared__ __align__(16) unsigned char panel_smem[];
    T *sx = reinterpret_cast<T *>(panel_smem);
    const int4 c = pd.cta[blockIdx.x];
    constexpr int NG = kPanelThreads / kPanelLanes;
    const int grp = threadIdx.x / kPanelLanes, li = threadIdx.x % kPanelLanes;
    constexpr int STEP = 4 * kPanelLanes; /* nonzeros a group covers per group of loads */
    /* the groups of a warp may run different numbers of segments: each
     * shuffles among its own lanes only */
    const unsigned mask = ((1u << kPanelLanes) - 1u) << ((threadIdx.x & 31) & ~(kPanelLanes - 1));
    auto finish_row = [&](int h) {
        __threadfence();
        double s = 0.0;
        for (int q = li; q < pd.P; q += kPanelLanes) s += (double)__ldcg(&pd.part[(size_t)h * pd.P + q]);
#pragma unroll
        for (int o = kPanelLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(mask, s, o, kPanelLanes);
        if (li == 0) {
            DualEpi<T, MAJOR, BETA> epi;
            epi.a = a;
            load_coefs(st, epi.k);
            epi.w = wt[koff].w;
            epi.omw = wt[koff].omw;
            const int i = pd.rows[h];
            epi.finish(i, (T)s, epi.fetch(i));
            if (pd.hot) pd.hot[h] = BETA ? a.u[i] : a.y[i];
            pd.cnt[h] = 0u;
        }
    };
    for (int pc = c.x; pc < c.y; ++pc) {
        /* the segments of this block in panel p: [sbeg, send) */
        const int4 pie = pd.piece[pc];
        const int p = pie.x, sbeg = pie.y, send = pie.z;
        const int col0 = p * pd.W;
        __syncthreads(); /* the previous panel's gathers are done */
        panel_stage(sx, xbar, col0, min(pd.W, n - col0));
        __syncthreads();
        for (int s = sbeg + grp; s < send; s += 2 * NG) {
            const bool two = s + NG < send;
            const int4 sa = pd.seg[s];
            const int4 sb = two ? pd.seg[s + NG] : make_int4(0, 0, 0, 0);
            T acc_a = T(0), acc_b = T(0);
            const int la = sa.z - sa.y, lb = two ? sb.z - sb.y : 0;
            const int len = max(la, lb);
            for (int d = 4 * li; d < len; d += kPanelUnroll * STEP) {
                T va[kPanelUnroll][4], vb[kPanelUnroll][4];
                int oa[kPanelUnroll][4], ob[kPanelUnroll][4];
#pragma unroll
                for (int u = 0; u < kPanelUnroll; ++u) {
                    const int e = d + u * STEP;
                    if (e < la) {
                        load4_stream(pd.val + sa.y + e, va[u]);
                        load4_stream(pd.off + sa.y + e, oa[u]);
                    }
                    if (e < lb) {
                        load4_stream(pd.val + sb.y + e, vb[u]);
                        load4_stream(pd.off + sb.y + e, ob[u]);
                    }
                }
#pragma unroll
                for (int u = 0; u < kPanelUnroll; ++u) {
                    const int e = d + u * STEP;
                    if (e < la) {
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc_a = vfma(va[u][q], sx[oa[u][q]], acc_a);
                    }
                    if (e < lb) {
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc_b = vfma(vb[u][q], sx[ob[u][q]], acc_b);
                    }
                }
            }
#pragma unroll
            for (int o = kPanelLanes / 2; o > 0; o >>= 1) {
                acc_a += __shfl_xor_sync(mask, acc_a, o, kPanelLanes);
                acc_b += __shfl_xor_sync(mask, acc_b, o, kPanelLanes);
            }
            int last_a = 0, last_b = 0;
            if (li == 0) {
                pd.part[(size_t)sa.x * pd.P + sa.w] = acc_a;
                if (two) pd.part[(size_t)sb.x * pd.P + sb.w] = acc_b;
                if (FUSE) {
                    __threadfence();
                    last_a = atomicAdd(&pd.cnt[sa.x], 1u) == (unsigned)(pd.nseg[sa.x] - 1);
                    if (two) last_b = atomicAdd(&pd.cnt[sb.x], 1u) == (unsigned)(pd.nseg[sb.x] - 1);
                }
            }
            if (FUSE) {
                last_a = __shfl_sync(mask, last_a, 0, kPanelLanes);
                last_b = __shfl_sync(mask, last_b, 0, kPanelLanes);
                if (last_a) finish_row(sa.x);
                if (last_b) finish_row(sb.x);
            }
        }
    }
}

/* One warp per long row: the row's panel partials summed in FP64 in a fixed
 * order, then the dual epilogue of k_dual. */
template <typename T, bool MAJOR, bool BETA>
__global__ void __launch_bounds__(kThreads) k_dual_long_finish(PanelDev<T> pd, DualArgs<T> a,
                                                                const CpalState *__restrict__ st,
                                                                const typename WeightT<T>::type *__restrict__ wt,
                                                                int koff) {
    pdl_enter();
    if (st->status) return;
    const int h = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (h >= pd.H) return;
    double s = 0.0;
    for (int p = lane; p < pd.P; p += 32) s += (double)pd.part[(size_t)h * pd.P + p];
    s = warp_sum(s);
    if (lane == 0) {
        DualEpi<T, MAJOR, BETA> epi;
        epi.a = a;
        load_coefs(st, epi.k);
        epi.w = wt[koff].w;
        epi.omw = wt[koff].omw;
        const int i = pd.rows[h];
        epi.finish(i, (T)s, epi.fetch(i));
        /* the value the next primal product gathers for this row */
        if (pd.hot) pd.hot[h] = BETA ? a.u[i] : a.y[i];
    }
}

/* hot[h] = gat[rows[h]]: the compact copy of the long rows' gathered values,
 * rebuilt at the start of every evaluation block (restarts, phase switches
 * and polishing rewrite the vector between blocks; within a block only the
 * dual step writes it, and k_dual_long_finish keeps the copy current) */
template <typename T>
__global__ void k_hot_refresh(int H, const int *__restrict__ rows, const T *__restrict__ gat, T *hot,
                              const CpalState *__restrict__ st) {
    pdl_enter();
    if (st->status) return;
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < H; h += gridDim.x * blockDim.x) hot[h] = gat[rows[h]];
}

/* The primal product with the long rows' gathered values in shared memory:
 * every column of a power-law LP meets the long rows, so most of A^T's
 * gathers land on those few entries.  Each block stages their compact copy
 * once (one coalesced read) and then walks row blocks blockIdx.x,
 * blockIdx.x + gridDim.x, ... (a grid of one wave), taking those entries from
 * shared memory: a warp's 32 gathers into the copy cost a few bank cycles
 * instead of up to 32 L1 tag lookups.  A^T's column indices come in a copy
 * where an entry of long row h is stored as -1 - h. */
constexpr int kHotRows = 1536;

template <typename T, int S, bool MAJOR>
__global__ void __launch_bounds__(kThreads) k_primal_hot(RowPlanDev plan, const int *__restrict__ rp,
                                                         const int *__restrict__ ci_hot, const T *__restrict__ val,
                                                         const T *__restrict__ gat, const T *__restrict__ hot,
                                                         int nhot, PrimalArgs<T> a, const CpalState *__restrict__ st,
                                                         const typename WeightT<T>::type *__restrict__ wt, int koff) {
    pdl_enter();
    if (st->status) return;
    __shared__ RowBlockSmem<S, 1, T> sm;
    __shared__ T shot[kHotRows];
    for (int h = threadIdx.x; h < nhot; h += kThreads) shot[h] = __ldcg(hot + h);
    __syncthreads();
    PrimalEpi<T, MAJOR> epi;
    epi.a = a;
    load_coefs(st, epi.k);
    epi.w = wt[koff].w;
    epi.omw = wt[koff].omw;
    auto g = [&](int c, T *out) { out[0] = c >= 0 ? __ldg(gat + c) : shot[-1 - c]; };
    Red<0, 0> red;
    for (int blk = blockIdx.x; blk < plan.nblocks; blk += gridDim.x) {
        rowblock_run_at<S, 1, T>(blk, plan, rp, ci_hot, val, g, epi, red, sm);
        __syncthreads(); /* the next row block restages sm */
    }
}

/* Halpern weights for the block starting at st->inner (one block). */
static __global__ void k_fill_weights(const CpalState *__restrict__ st, HalpernW *wt, HalpernWf *wtf, int F) {
    const int inner = st->inner;
    for (int i = threadIdx.x + 1; i <= F; i += blockDim.x) cpal_halpern_entry(inner, i, wt[i], wtf[i]);
}

/* FP64 vector -> (hi, lo) float pairs */
static __global__ void k_split(const double *__restrict__ src, float2 *dst, int len) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) dst[i] = split_anchor(src[i]);
}

/* A x0 at the start of a solve (or of a precision phase), with the first
 * predictor u = y - beta (A x - P(A x - y/beta)). */
template <typename T, bool BETA>
struct InitAxEpi : NoLongRed {
    T *ax, *u;
    double *ax0;
    float2 *ax0f;
    const T *y, *lb, *ub;
    T beta, inv_beta;
    __device__ __forceinline__ void operator()(int i, const double *s, Red<0, 0> &) const {
        ax0[i] = s[0];
        if (ax0f) ax0f[i] = split_anchor(s[0]);
        const T axv = (T)s[0];
        ax[i] = axv;
        if (BETA) {
            const T yi = y[i];
            const T z = vmax(lb[i], vmin(axv - yi * inv_beta, ub[i]));
            u[i] = yi - beta * (axv - z);
        }
    }
};

template <typename T, int S, bool BETA>
__global__ void __launch_bounds__(kThreads) k_init_ax(RowPlanDev plan, const int *__restrict__ rp,
                                                      const int *__restrict__ ci, const double *__restrict__ val,
                                                      const double *__restrict__ x0, T *ax, double *ax0, float2 *ax0f,
                                                      T *u, const T *y, const T *lb, const T *ub,
                                                      const CpalState *__restrict__ st) {
    __shared__ RowBlockSmem<S, 1, double> sm;
    InitAxEpi<T, BETA> epi;
    epi.ax = ax;
    epi.u = u;
    epi.ax0 = ax0;
    epi.ax0f = ax0f;
    epi.y = y;
    epi.lb = lb;
    epi.ub = ub;
    Coefs<T> k;
    load_coefs(st, k);
    epi.beta = k.beta;
    epi.inv_beta = k.inv_beta;
    auto g = [&](int c, double *out) { out[0] = __ldg(x0 + c); };
    Red<0, 0> red;
    rowblock_run<S, 1, double>(plan, rp, ci, val, g, epi, red, sm);
}

/* ------------------------------------------------------------------ */
/* evaluation                                                          */
/* ------------------------------------------------------------------ */
constexpr int kEvalStride = 12; /* doubles per partial slot: 6 sums, the maximum, up to 4 extra sums */

/* rows of A: p^ = A x^, A dx, A (x^ - x0); primal residual, dual-objective
 * contribution, |A dx|^2, |dy|^2, |y^ - y0|^2, |A(x^ - x0)|^2. */
template <typename T>
struct EvalRowArgs {
    const T *xh, *xbar, *yh, *ybar;
    const double *x0, *y0, *ax0, *clb, *cub, *clb_fin, *cub_fin, *rscale;
    double *phat;
    double *part; /* (nblocks + nlong) * kEvalStride */
    int nblocks;
    const T *x, *y, *ax; /* restart target selection: the Halpern iterate and its tracked A x */
};

/* SEL (restart target selection on): also A(x^ - x), |y^ - y|^2, |y - y0|^2
 * and |A x - A x0|^2 in extra sums 6..9 (slot indices 7..10). */
template <typename T, bool SEL = false>
struct EvalRowEpi {
    EvalRowArgs<T> a;
    __device__ __forceinline__ void operator()(int i, const double *s, Red<SEL ? 10 : 6, 1> &r) const {
        const double ph = s[0];
        a.phat[i] = ph;
        const double cl = fmax(a.clb[i], fmin(ph, a.cub[i]));
        const double rpv = (ph - cl) * a.rscale[i];
        r.s[0] += rpv * rpv;
        r.mx[0] = fmax(r.mx[0], fabs(rpv));
        const double yhi = (double)a.yh[i];
        r.s[1] += fmax(yhi, 0.0) * a.clb_fin[i] + fmin(yhi, 0.0) * a.cub_fin[i];
        r.s[2] += s[1] * s[1];
        const double dyv = (double)a.ybar[i] - yhi;
        r.s[3] += dyv * dyv;
        const double ddy = yhi - a.y0[i];
        r.s[4] += ddy * ddy;
        r.s[5] += s[2] * s[2];
        if (SEL) {
            r.s[SEL ? 6 : 0] += s[SEL ? 3 : 0] * s[SEL ? 3 : 0];
            const double yc = (double)a.y[i];
            const double d1 = yhi - yc, d2 = yc - a.y0[i], d3 = (double)a.ax[i] - a.ax0[i];
            r.s[SEL ? 7 : 0] += d1 * d1;
            r.s[SEL ? 8 : 0] += d2 * d2;
            r.s[SEL ? 9 : 0] += d3 * d3;
        }
    }
    __device__ __forceinline__ void long_red(int lid, Red<SEL ? 10 : 6, 1> &r) const {
        double *d = a.part + (size_t)(a.nblocks + lid) * kEvalStride;
        for (int q = 0; q < 6; ++q) d[q] = r.s[q];
        d[6] = r.mx[0];
        for (int q = 6; q < (SEL ? 10 : 6); ++q) d[q + 1] = r.s[q];
    }
};

template <typename T, int S, bool SEL = false>
__device__ __forceinline__ void eval_rows_at(int blk, const RowPlanDev &plan, const int *__restrict__ rp,
                                             const int *__restrict__ ci, const double *__restrict__ val,
                                             const EvalRowArgs<T> &a, RowBlockSmem<S, SEL ? 4 : 3, double> &sm) {
    constexpr int NP = SEL ? 4 : 3, NS = SEL ? 10 : 6;
    EvalRowEpi<T, SEL> epi;
    epi.a = a;
    const T *xh = a.xh;
    const T *xb = a.xbar;
    const T *xc = a.x;
    const double *x0 = a.x0;
    auto g = [&](int c, double *out) {
        const double xhc = (double)xh[c];
        out[0] = xhc;
        out[1] = (double)xb[c] - xhc;
        out[2] = xhc - x0[c];
        if (SEL) out[SEL ? 3 : 0] = xhc - (double)xc[c];
    };
    Red<NS, 1> red;
    red.zero();
    rowblock_run_at<S, NP, double>(blk, plan, rp, ci, val, g, epi, red, sm);
    block_reduce<kThreads, NS, 1>(red, sm.red);
    if (threadIdx.x == 0) {
        double *d = a.part + (size_t)blk * kEvalStride;
        for (int q = 0; q < 6; ++q) d[q] = red.s[q];
        d[6] = red.mx[0];
        for (int q = 6; q < NS; ++q) d[q + 1] = red.s[q];
    }
}

template <typename T, int S, bool SEL = false>
__global__ void __launch_bounds__(kThreads) k_eval_rows(RowPlanDev plan, const int *__restrict__ rp,
                                                        const int *__restrict__ ci, const double *__restrict__ val,
                                                        EvalRowArgs<T> a, const CpalState *__restrict__ st) {
    if (st->status) return;
    __shared__ RowBlockSmem<S, SEL ? 4 : 3, double> sm;
    eval_rows_at<T, S, SEL>((int)blockIdx.x, plan, rp, ci, val, a, sm);
}

/* rows of A^T: q^ = A^T y^, A^T dy; dual residual, |dx|^2, <A^T dy, dx>,
 * c'x^, lambda'x^, |x^ - x0|^2. */
template <typename T>
struct EvalColArgs {
    const T *xh, *xbar, *yh, *ybar, *lam;
    const double *x0, *c, *cscale;
    double *part;
    int nblocks;
    const T *x, *y; /* restart target selection: the Halpern iterate */
    const double *y0; /* three-point selection: the dual anchor */
};

/* SEL: also <A^T(y^ - y), x^ - x>, |x^ - x|^2 and |x - x0|^2 in extra sums
 * 6..8 (slot indices 7..9); H3 (three-point selection, with SEL): also
 * <A^T(y^ - y0), x^ - x0> in extra sum 9 (slot index 10). */
template <typename T, bool SEL = false, bool H3 = false>
struct EvalColEpi {
    static constexpr int NS = SEL ? (H3 ? 10 : 9) : 6;
    EvalColArgs<T> a;
    __device__ __forceinline__ void operator()(int j, const double *s, Red<NS, 1> &r) const {
        const double xhj = (double)a.xh[j];
        const double lj = (double)a.lam[j];
        const double cj = a.c[j];
        const double rdv = (cj - s[0] - lj) * a.cscale[j];
        r.s[0] += rdv * rdv;
        r.mx[0] = fmax(r.mx[0], fabs(rdv));
        const double dxv = (double)a.xbar[j] - xhj;
        r.s[1] += dxv * dxv;
        r.s[2] += s[1] * dxv;
        r.s[3] += cj * xhj;
        r.s[4] += lj * xhj;
        const double ddx = xhj - a.x0[j];
        r.s[5] += ddx * ddx;
        if (SEL) {
            const double xc = (double)a.x[j];
            const double d1 = xhj - xc, d2 = xc - a.x0[j];
            r.s[SEL ? 6 : 0] += s[SEL ? 2 : 0] * d1;
            r.s[SEL ? 7 : 0] += d1 * d1;
            r.s[SEL ? 8 : 0] += d2 * d2;
        }
        if (H3) r.s[H3 ? 9 : 0] += s[H3 ? 3 : 0] * ddx;
    }
    __device__ __forceinline__ void long_red(int lid, Red<NS, 1> &r) const {
        double *d = a.part + (size_t)(a.nblocks + lid) * kEvalStride;
        for (int q = 0; q < 6; ++q) d[q] = r.s[q];
        d[6] = r.mx[0];
        for (int q = 6; q < NS; ++q) d[q + 1] = r.s[q];
    }
};

template <typename T, int S, bool SEL = false, bool H3 = false>
__device__ __forceinline__ void eval_cols_at(int blk, const RowPlanDev &plan, const int *__restrict__ rp,
                                             const int *__restrict__ ci, const double *__restrict__ val,
                                             const EvalColArgs<T> &a,
                                             RowBlockSmem<S, SEL ? (H3 ? 4 : 3) : 2, double> &sm) {
    static_assert(SEL || !H3, "three-point selection extends the two-point terms");
    constexpr int NP = SEL ? (H3 ? 4 : 3) : 2, NS = EvalColEpi<T, SEL, H3>::NS;
    EvalColEpi<T, SEL, H3> epi;
    epi.a = a;
    const T *yh = a.yh;
    const T *yb = a.ybar;
    const T *yc = a.y;
    const double *y0 = a.y0;
    auto g = [&](int c, double *out) {
        const double yhc = (double)yh[c];
        out[0] = yhc;
        out[1] = (double)yb[c] - yhc;
        if (SEL) out[SEL ? 2 : 0] = yhc - (double)yc[c];
        if (H3) out[H3 ? 3 : 0] = yhc - y0[c];
    };
    Red<NS, 1> red;
    red.zero();
    rowblock_run_at<S, NP, double>(blk, plan, rp, ci, val, g, epi, red, sm);
    block_reduce<kThreads, NS, 1>(red, sm.red);
    if (threadIdx.x == 0) {
        double *d = a.part + (size_t)blk * kEvalStride;
        for (int q = 0; q < 6; ++q) d[q] = red.s[q];
        d[6] = red.mx[0];
        for (int q = 6; q < NS; ++q) d[q + 1] = red.s[q];
    }
}

template <typename T, int S, bool SEL = false, bool H3 = false>
__global__ void __launch_bounds__(kThreads) k_eval_cols(RowPlanDev plan, const int *__restrict__ rp,
                                                        const int *__restrict__ ci, const double *__restrict__ val,
                                                        EvalColArgs<T> a, const CpalState *__restrict__ st) {
    if (st->status) return;
    __shared__ RowBlockSmem<S, SEL ? (H3 ? 4 : 3) : 2, double> sm;
    eval_cols_at<T, S, SEL, H3>((int)blockIdx.x, plan, rp, ci, val, a, sm);
}

/* ---- infeasibility certificates (opt-in) ------------------------------- */
/* The projected displacements from the restart anchor (the ray estimates of
 * LP/CP_AL/src/utils.cu:684-720): dx_j = x^_j - x0_j clipped to >= 0 where
 * the lower bound is finite and to <= 0 where the upper bound is finite;
 * dy_i = y^_i - y0_i clipped to <= 0 where the row's lower bound is
 * infinite and to >= 0 where its upper bound is infinite. */
__device__ __forceinline__ double ray_dx(double xh, double x0, double lb, double ub) {
    double d = xh - x0;
    if (isfinite(lb)) d = fmax(d, 0.0);
    if (isfinite(ub)) d = fmin(d, 0.0);
    return d;
}
__device__ __forceinline__ double ray_dy(double yh, double y0, double lb, double ub) {
    double d = yh - y0;
    if (!isfinite(lb)) d = fmin(d, 0.0);
    if (!isfinite(ub)) d = fmax(d, 0.0);
    return d;
}

template <typename T>
struct RayArgs {
    const T *xh, *yh;
    const double *x0, *y0, *vlb, *vub, *clb, *cub, *clb_fin, *cub_fin, *rscale, *cscale, *c;
    double *part; /* (nblocks + nlong) * kEvalStride */
    int nblocks;
};

/* rows of A: s = (A dx)_i; sum 0: the dual-objective row term of dy, max 0:
 * the unscaled violation of A dx (utils.cu:722-737), max 1: |dy_i| */
template <typename T>
struct RayRowEpi {
    RayArgs<T> a;
    __device__ __forceinline__ void operator()(int i, const double *s, Red<1, 2> &r) const {
        const double lb = a.clb[i], ub = a.cub[i], v = s[0];
        r.mx[0] = fmax(r.mx[0], (fmax(0.0, -v) * (isfinite(lb) ? 1.0 : 0.0) + fmax(0.0, v) * (isfinite(ub) ? 1.0 : 0.0)) *
                                    a.rscale[i]);
        const double dy = ray_dy((double)a.yh[i], a.y0[i], lb, ub);
        r.s[0] += fmax(dy, 0.0) * a.clb_fin[i] + fmin(dy, 0.0) * a.cub_fin[i];
        r.mx[1] = fmax(r.mx[1], fabs(dy));
    }
    __device__ __forceinline__ void long_red(int lid, Red<1, 2> &r) const {
        double *d = a.part + (size_t)(a.nblocks + lid) * kEvalStride;
        d[0] = r.s[0];
        d[1] = 0.0;
        d[2] = r.mx[0];
        d[3] = r.mx[1];
    }
};

/* rows of A^T: q = (A^T dy)_j; sum 0: the dual-objective slack term, sum 1:
 * c_j dx_j, max 0: the unscaled dual-slack violation (utils.cu:739-754),
 * max 1: |dx_j| */
template <typename T>
struct RayColEpi {
    RayArgs<T> a;
    __device__ __forceinline__ void operator()(int j, const double *s, Red<2, 2> &r) const {
        const double lb = a.vlb[j], ub = a.vub[j], q = -s[0];
        const bool lf = isfinite(lb), uf = isfinite(ub);
        r.mx[0] = fmax(r.mx[0], (fmax(0.0, q) * (lf ? 0.0 : 1.0) - fmin(0.0, q) * (uf ? 0.0 : 1.0)) * a.cscale[j]);
        r.s[0] += fmax(q, 0.0) * (lf ? lb : 0.0) + fmin(q, 0.0) * (uf ? ub : 0.0);
        const double dx = ray_dx((double)a.xh[j], a.x0[j], lb, ub);
        r.s[1] += a.c[j] * dx;
        r.mx[1] = fmax(r.mx[1], fabs(dx));
    }
    __device__ __forceinline__ void long_red(int lid, Red<2, 2> &r) const {
        double *d = a.part + (size_t)(a.nblocks + lid) * kEvalStride;
        d[0] = r.s[0];
        d[1] = r.s[1];
        d[2] = r.mx[0];
        d[3] = r.mx[1];
    }
};

template <typename T, int S>
__global__ void __launch_bounds__(kThreads) k_ray_rows(RowPlanDev plan, const int *__restrict__ rp,
                                                       const int *__restrict__ ci, const double *__restrict__ val,
                                                       RayArgs<T> a, const CpalState *__restrict__ st) {
    if (st->status) return;
    __shared__ RowBlockSmem<S, 1, double> sm;
    RayRowEpi<T> epi;
    epi.a = a;
    auto g = [&](int c, double *out) { out[0] = ray_dx((double)a.xh[c], a.x0[c], a.vlb[c], a.vub[c]); };
    Red<1, 2> red;
    red.zero();
    rowblock_run<S, 1, double>(plan, rp, ci, val, g, epi, red, sm);
    block_reduce<kThreads, 1, 2>(red, sm.red);
    if (threadIdx.x == 0) {
        double *d = a.part + (size_t)blockIdx.x * kEvalStride;
        d[0] = red.s[0];
        d[1] = 0.0;
        d[2] = red.mx[0];
        d[3] = red.mx[1];
    }
}

template <typename T, int S>
__global__ void __launch_bounds__(kThreads) k_ray_cols(RowPlanDev plan, const int *__restrict__ rp,
                                                       const int *__restrict__ ci, const double *__restrict__ val,
                                                       RayArgs<T> a, const CpalState *__restrict__ st) {
    if (st->status) return;
    __shared__ RowBlockSmem<S, 1, double> sm;
    RayColEpi<T> epi;
    epi.a = a;
    auto g = [&](int c, double *out) { out[0] = ray_dy((double)a.yh[c], a.y0[c], a.clb[c], a.cub[c]); };
    Red<2, 2> red;
    red.zero();
    rowblock_run<S, 1, double>(plan, rp, ci, val, g, epi, red, sm);
    block_reduce<kThreads, 2, 2>(red, sm.red);
    if (threadIdx.x == 0) {
        double *d = a.part + (size_t)blockIdx.x * kEvalStride;
        d[0] = red.s[0];
        d[1] = red.s[1];
        d[2] = red.mx[0];
        d[3] = red.mx[1];
    }
}

/* Sums (slots 0, 1) and maxima (slots 2, 3) of the ray partials, in a fixed
 * order. */
__device__ __forceinline__ void reduce_ray_slots(const double *part, int nslots, Red<2, 2> &r, double *sbuf) {
    r.zero();
    for (int b = threadIdx.x; b < nslots; b += kThreads) {
        const double *d = part + (size_t)b * kEvalStride;
        r.s[0] += d[0];
        r.s[1] += d[1];
        r.mx[0] = fmax(r.mx[0], d[2]);
        r.mx[1] = fmax(r.mx[1], d[3]);
    }
    block_reduce<kThreads, 2, 2>(r, sbuf);
}

/* Sums the partial slots of one evaluation kernel in a fixed order. */
__device__ __forceinline__ void reduce_slots(const double *part, int nslots, Red<10, 1> &r, double *sbuf) {
    r.zero();
    for (int b = threadIdx.x; b < nslots; b += kThreads) {
        const double *d = part + (size_t)b * kEvalStride;
        for (int q = 0; q < 6; ++q) r.s[q] += d[q];
        r.mx[0] = fmax(r.mx[0], d[6]);
        for (int q = 6; q < 10; ++q) r.s[q] += d[q + 1];
    }
    block_reduce<kThreads, 10, 1>(r, sbuf);
}

/* The controller of one evaluation, run by one block: the partial sums in a
 * fixed order, the end-of-block decisions, the next block's Halpern weights. */
__device__ __forceinline__ void control_block(const double *__restrict__ prow, int nrow_slots,
                                              const double *__restrict__ pcol, int ncol_slots,
                                              const double *__restrict__ pray_row, int nray_row,
                                              const double *__restrict__ pray_col, int nray_col, CpalState *st,
                                              const CpalParams &p, HalpernW *wt, HalpernWf *wtf, double *sbuf) {
    Red<10, 1> r1, r2;
    reduce_slots(prow, nrow_slots, r1, sbuf);
    reduce_slots(pcol, ncol_slots, r2, sbuf);
    Red<2, 2> q1, q2;
    q1.zero();
    q2.zero();
    if (p.infeas) {
        reduce_ray_slots(pray_row, nray_row, q1, sbuf);
        reduce_ray_slots(pray_col, nray_col, q2, sbuf);
    }
    if (threadIdx.x == 0) {
        CpalEval e;
        e.rp2 = r1.s[0];
        e.contrib = r1.s[1];
        e.adx2 = r1.s[2];
        e.dy2 = r1.s[3];
        e.ddy2 = r1.s[4];
        e.axd2 = r1.s[5];
        e.rpmax = r1.mx[0];
        e.rd2 = r2.s[0];
        e.dx2 = r2.s[1];
        e.cross = r2.s[2];
        e.cx = r2.s[3];
        e.lx = r2.s[4];
        e.ddx2 = r2.s[5];
        e.rdmax = r2.mx[0];
        e.sel_ax2 = r1.s[6];
        e.sel_dy2 = r1.s[7];
        e.cur_dy2 = r1.s[8];
        e.cur_axd2 = r1.s[9];
        e.sel_cross = r2.s[6];
        e.sel_dx2 = r2.s[7];
        e.cur_dx2 = r2.s[8];
        e.h_cross = r2.s[9];
        e.ray_rowsum = q1.s[0];
        e.ray_pviol = q1.mx[0];
        e.ray_dyinf = q1.mx[1];
        e.ray_colsum = q2.s[0];
        e.ray_cdx = q2.s[1];
        e.ray_dviol = q2.mx[0];
        e.ray_dxinf = q2.mx[1];
        CpalState s = *st;
        s.elapsed = (double)(globaltimer_ns() - s.t_start_ns) * 1e-9;
        cpal_end_of_block(s, p, e);
        *st = s;
    }
    __syncthreads();
    /* Halpern weights of the next block (the counter may have been reset) */
    const int inner = st->inner;
    for (int i = threadIdx.x + 1; i <= p.F; i += kThreads) cpal_halpern_entry(inner, i, wt[i], wtf[i]);
}

static __global__ void __launch_bounds__(kThreads) k_control(const double *__restrict__ prow, int nrow_slots,
                                                      const double *__restrict__ pcol, int ncol_slots,
                                                      const double *__restrict__ pray_row, int nray_row,
                                                      const double *__restrict__ pray_col, int nray_col,
                                                      CpalState *st, CpalParams p, HalpernW *wt, HalpernWf *wtf) {
    if (st->status) return;
    __shared__ double sbuf[11 * (kThreads / 32)];
    control_block(prow, nrow_slots, pcol, ncol_slots, pray_row, nray_row, pray_col, nray_col, st, p, wt, wtf, sbuf);
}

/* ------------------------------------------------------------------ */
/* feasibility polishing (LP/CP_AL/src/solver.cu:3912-4456)           */
/* ------------------------------------------------------------------ */
/* The terms a polishing phase reads from the evaluation partials. */
struct PolishEval {
    double rp2, rpmax, rd2, rdmax, dx2, dy2, contrib, lx, cx;
};

static __global__ void __launch_bounds__(kThreads) k_polish_reduce(const double *__restrict__ prow, int nrow_slots,
                                                                  const double *__restrict__ pcol, int ncol_slots,
                                                                  PolishEval *out) {
    __shared__ double sbuf[11 * (kThreads / 32)];
    Red<10, 1> r1, r2;
    reduce_slots(prow, nrow_slots, r1, sbuf);
    reduce_slots(pcol, ncol_slots, r2, sbuf);
    if (threadIdx.x == 0) {
        out->rp2 = r1.s[0];
        out->contrib = r1.s[1];
        out->dy2 = r1.s[3];
        out->rpmax = r1.mx[0];
        out->rd2 = r2.s[0];
        out->dx2 = r2.s[1];
        out->cx = r2.s[3];
        out->lx = r2.s[4];
        out->rdmax = r2.mx[0];
    }
}

/* the AL predictor u = y - beta (A x - P(A x - y / beta)) from the stored
 * A x, after the dual iterate changed alone */
static __global__ void __launch_bounds__(kThreads) k_predictor(int m, const double *__restrict__ ax,
                                                              const double *__restrict__ y,
                                                              const double *__restrict__ lb,
                                                              const double *__restrict__ ub, double *u,
                                                              const CpalState *__restrict__ st) {
    Coefs<double> k;
    load_coefs(st, k);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double z = fmax(lb[i], fmin(ax[i] - y[i] * k.inv_beta, ub[i]));
        u[i] = y[i] - k.beta * (ax[i] - z);
    }
}

/* every finite entry of v becomes 0 (solver.cu:4237-4245) */
static __global__ void __launch_bounds__(kThreads) k_zero_finite(int len, double *v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
        if (isfinite(v[i])) v[i] = 0.0;
}

/* a . b over len entries by one block in a fixed order */
static __global__ void __launch_bounds__(kThreads) k_dot_block(int len, const double *__restrict__ a,
                                                              const double *__restrict__ b, double *out) {
    __shared__ double sbuf[kThreads / 32];
    Red<1, 0> r;
    r.zero();
    for (int i = threadIdx.x; i < len; i += kThreads) r.s[0] += a[i] * b[i];
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) *out = r.s[0];
}

/* Anchor reset after a restart: x0 = x = x^, y0 = y = y^, A x0 = A x = p^,
 * and the next predictor from the new beta.  The FP64 anchors are written
 * together with the (hi, lo) copies the FP32 phase reads. */
template <typename T, bool BETA>
__device__ __forceinline__ void restart_all(const CpalState *__restrict__ st, int n, int m, const T *xh, T *x,
                                            double *x0, float2 *x0f, const T *yh, T *y, double *y0, float2 *y0f,
                                            const double *__restrict__ phat, T *ax, double *ax0, float2 *ax0f, T *u,
                                            const T *__restrict__ lb, const T *__restrict__ ub, T *xbar, T *ybar) {
    if (st->status || !st->restart) return;
    Coefs<T> k;
    load_coefs(st, k);
    const int total = n > m ? n : m;
    if (st->restart_target == 2) {
        /* restart to the plain Halpern point h = w x^ + (1 - w) x0 of the
         * block's last iteration (LP/CP_AL/src/solver.cu:2392, 2452,
         * 3043-3075): x-bar = x^, then x^ = x = x0 = h; the same for y;
         * A x0 = A x = w p^ + (1 - w) A x0 */
        const double w = st->restart_w, omw = 1.0 - w;
        T *xh_w = const_cast<T *>(xh), *yh_w = const_cast<T *>(yh);
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
            if (t < n) {
                const T xo = xh_w[t];
                const T v = (T)(w * (double)xo + omw * x0[t]);
                xbar[t] = xo;
                xh_w[t] = v;
                x[t] = v;
                x0[t] = (double)v;
                if (x0f) x0f[t] = split_anchor((double)v);
            }
            if (t < m) {
                const T yo = yh_w[t];
                const T v = (T)(w * (double)yo + omw * y0[t]);
                ybar[t] = yo;
                yh_w[t] = v;
                y[t] = v;
                y0[t] = (double)v;
                if (y0f) y0f[t] = split_anchor((double)v);
                const double axh = w * phat[t] + omw * ax0[t];
                ax0[t] = axh;
                if (ax0f) ax0f[t] = split_anchor(axh);
                const T axv = (T)axh;
                ax[t] = axv;
                if (BETA) {
                    const T z = vmax(lb[t], vmin(axv - v * k.inv_beta, ub[t]));
                    u[t] = v - k.beta * (axv - z);
                }
            }
        }
        return;
    }
    if (st->restart_target == 1) {
        /* restart to the Halpern iterate (LP/CP_AL/src/solver.cu:3015-3040):
         * x-bar = x^, x^ = x, x0 = x; the same for y; A x0 = the tracked A x */
        T *xh_w = const_cast<T *>(xh), *yh_w = const_cast<T *>(yh);
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
            if (t < n) {
                const T v = x[t];
                xbar[t] = xh_w[t];
                xh_w[t] = v;
                x0[t] = (double)v;
                if (x0f) x0f[t] = split_anchor((double)v);
            }
            if (t < m) {
                const T v = y[t];
                ybar[t] = yh_w[t];
                yh_w[t] = v;
                y0[t] = (double)v;
                if (y0f) y0f[t] = split_anchor((double)v);
                const T axv = ax[t];
                ax0[t] = (double)axv;
                if (ax0f) ax0f[t] = split_anchor((double)axv);
                if (BETA) {
                    const T z = vmax(lb[t], vmin(axv - v * k.inv_beta, ub[t]));
                    u[t] = v - k.beta * (axv - z);
                }
            }
        }
        return;
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < n) {
            const T v = xh[t];
            x[t] = v;
            x0[t] = (double)v;
            if (x0f) x0f[t] = split_anchor((double)v);
        }
        if (t < m) {
            const T v = yh[t];
            y[t] = v;
            y0[t] = (double)v;
            if (y0f) y0f[t] = split_anchor((double)v);
            const double ph = phat[t];
            ax0[t] = ph;
            if (ax0f) ax0f[t] = split_anchor(ph);
            const T axv = (T)ph;
            ax[t] = axv;
            if (BETA) {
                const T z = vmax(lb[t], vmin(axv - v * k.inv_beta, ub[t]));
                u[t] = v - k.beta * (axv - z);
            }
        }
    }
}

/* the restart as a launch of its own (the evaluation blocks of the graph) */
template <typename T, bool BETA>
__global__ void k_restart(const CpalState *__restrict__ st, int n, int m, const T *xh, T *x, double *x0,
                          float2 *x0f, const T *yh, T *y, double *y0, float2 *y0f, const double *__restrict__ phat,
                          T *ax, double *ax0, float2 *ax0f, T *u, const T *__restrict__ lb,
                          const T *__restrict__ ub, T *xbar, T *ybar) {
    restart_all<T, BETA>(st, n, m, xh, x, x0, x0f, yh, y, y0, y0f, phat, ax, ax0, ax0f, u, lb, ub, xbar, ybar);
}


static __global__ void k_start_clock(CpalState *st) { st->t_start_ns = globaltimer_ns(); }

/* ------------------------------------------------------------------ */
/* small LPs: the whole loop in one cooperative launch                 */
/* ------------------------------------------------------------------ */
/* A small LP's iteration is a few microseconds of work spread over a few
 * hundred blocks, so two kernel launches per iteration (even inside a CUDA
 * graph) cost as much as the work.  k_cpal_loop runs evaluation blocks
 * entirely on the device: every block of the grid (all co-resident, launched
 * cooperatively) walks the row blocks of each product, and a grid barrier
 * separates the primal product, the dual product, the evaluation, the
 * controller (block 0) and the restart.  The row-block bodies, epilogues,
 * controller and restart are the graph path's, with one difference: vectors
 * written inside the launch are gathered through L2 (__ldcg), never through
 * the read-only path. */
struct LoopBar {
    unsigned int count, gen;
    int err, pad;
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

/* Grid barrier number `k` (1, 2, ... within the launch; the counter is zero
 * at launch): one release-add per block on a monotonic counter, then an
 * acquire spin until all blocks of the k-th barrier have arrived.  False,
 * with the barrier marked failed for every block, when a wait exceeds
 * `limit` polls. */
__device__ __forceinline__ bool loop_sync(LoopBar *b, unsigned k, long long limit, int *sok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned target = k * gridDim.x;
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&b->count) : "memory");
        long long spins = 0;
        while (ld_acquire_gpu(&b->count) < target) {
            if (++spins > limit) {
                atomicExch(&b->err, 1);
                ok = 0;
                break;
            }
            if ((spins & 1023) == 0 && *(volatile int *)&b->err) {
                ok = 0;
                break;
            }
        }
        *sok = ok;
    }
    __syncthreads();
    return *sok != 0;
}

template <typename T>
struct LoopArgs {
    RowPlanDev at_it, a_it, at_ev, a_ev;
    const int *at_rp, *at_ci, *a_rp, *a_ci;
    const T *at_val, *a_val;      /* iteration values (the form's precision) */
    const double *at_v64, *a_v64; /* evaluation values */
    PrimalArgs<T> pa;
    DualArgs<T> da;
    const T *gat; /* gathered by the primal product: u (beta > 0) or y */
    EvalRowArgs<T> ra;
    EvalColArgs<T> ca;
    CpalState *st;
    CpalParams p;
    HalpernW *wt;
    HalpernWf *wtf;
    int nrow_slots, ncol_slots;
    int n, m;
    double *x0, *y0, *ax0;
    float2 *x0f, *y0f, *ax0f;
    const double *phat;
    LoopBar *bar;
    long long spin_limit;
    int max_blocks; /* evaluation blocks before the launch returns to the host */
    int *err;
};

template <typename T>
__device__ __forceinline__ const typename WeightT<T>::type &loop_weight(const LoopArgs<T> &L, int i);
template <>
__device__ __forceinline__ const HalpernW &loop_weight<double>(const LoopArgs<double> &L, int i) {
    return L.wt[i];
}
template <>
__device__ __forceinline__ const HalpernWf &loop_weight<float>(const LoopArgs<float> &L, int i) {
    return L.wtf[i];
}

template <typename T, int S, bool MAJOR>
__device__ __forceinline__ void loop_primal(const LoopArgs<T> &L, const Coefs<T> &k, int i,
                                            RowBlockSmem<S, 1, T> &sm) {
    PrimalEpi<T, MAJOR> epi;
    epi.a = L.pa;
    epi.k = k;
    epi.w = loop_weight<T>(L, i).w;
    epi.omw = loop_weight<T>(L, i).omw;
    const T *gat = L.gat;
    auto g = [&](int c, T *out) { out[0] = __ldcg(gat + c); };
    Red<0, 0> red;
    for (int blk = blockIdx.x; blk < L.at_it.nblocks; blk += gridDim.x) {
        rowblock_run_at<S, 1, T>(blk, L.at_it, L.at_rp, L.at_ci, L.at_val, g, epi, red, sm);
        __syncthreads();
    }
}

template <typename T, int S, bool MAJOR, bool BETA>
__device__ __forceinline__ void loop_dual(const LoopArgs<T> &L, const Coefs<T> &k, int i,
                                          RowBlockSmem<S, 1, T> &sm) {
    DualEpi<T, MAJOR, BETA> epi;
    epi.a = L.da;
    epi.k = k;
    epi.w = loop_weight<T>(L, i).w;
    epi.omw = loop_weight<T>(L, i).omw;
    const T *xbar = L.pa.xbar;
    auto g = [&](int c, T *out) { out[0] = __ldcg(xbar + c); };
    Red<0, 0> red;
    for (int blk = blockIdx.x; blk < L.a_it.nblocks; blk += gridDim.x) {
        rowblock_run_at<S, 1, T>(blk, L.a_it, L.a_rp, L.a_ci, L.a_val, g, epi, red, sm);
        __syncthreads();
    }
}

template <typename T, int S, int SE, bool BETA>
__global__ void __launch_bounds__(kThreads) k_cpal_loop(LoopArgs<T> L) {
    constexpr size_t B1 = sizeof(RowBlockSmem<S, 1, T>), B2 = sizeof(RowBlockSmem<SE, 3, double>),
                     B3 = sizeof(RowBlockSmem<SE, 2, double>);
    constexpr size_t BM = B1 > B2 ? (B1 > B3 ? B1 : B3) : (B2 > B3 ? B2 : B3);
    __shared__ __align__(16) unsigned char raw[BM];
    __shared__ double sbuf[11 * (kThreads / 32)];
    __shared__ int sok, sflag;
    auto &smi = *reinterpret_cast<RowBlockSmem<S, 1, T> *>(raw);
    auto &smr = *reinterpret_cast<RowBlockSmem<SE, 3, double> *>(raw);
    auto &smc = *reinterpret_cast<RowBlockSmem<SE, 2, double> *>(raw);
    const int F = L.p.F;
    auto give_up = [&]() {
        if (threadIdx.x == 0) {
            atomicExch(L.err, 2);
            atomicExch(&L.st->status, kStatusDeviceError);
        }
    };
    unsigned nsync = 0;
#define PDAL_LOOP_SYNC()                                                                                               \
    do {                                                                                                               \
        if (!loop_sync(L.bar, ++nsync, L.spin_limit, &sok)) {                                                          \
            give_up();                                                                                                 \
            return;                                                                                                    \
        }                                                                                                              \
    } while (0)
    for (int blocks = 0; blocks < L.max_blocks; ++blocks) {
        /* every block reads the state after the same barrier */
        if (threadIdx.x == 0) sflag = L.st->status;
        __syncthreads();
        if (sflag) return;
        Coefs<T> k;
        load_coefs(L.st, k);
        for (int i = 1; i <= F; ++i) {
            if (i == F)
                loop_primal<T, S, true>(L, k, i, smi);
            else
                loop_primal<T, S, false>(L, k, i, smi);
            PDAL_LOOP_SYNC();
            if (i == F)
                loop_dual<T, S, true, BETA>(L, k, i, smi);
            else
                loop_dual<T, S, false, BETA>(L, k, i, smi);
            PDAL_LOOP_SYNC();
        }
        for (int blk = blockIdx.x; blk < L.a_ev.nblocks; blk += gridDim.x) {
            eval_rows_at<T, SE, false>(blk, L.a_ev, L.a_rp, L.a_ci, L.a_v64, L.ra, smr);
            __syncthreads();
        }
        for (int blk = blockIdx.x; blk < L.at_ev.nblocks; blk += gridDim.x) {
            eval_cols_at<T, SE, false, false>(blk, L.at_ev, L.at_rp, L.at_ci, L.at_v64, L.ca, smc);
            __syncthreads();
        }
        PDAL_LOOP_SYNC();
        if (blockIdx.x == 0)
            control_block(L.ra.part, L.nrow_slots, L.ca.part, L.ncol_slots, nullptr, 0, nullptr, 0, L.st, L.p, L.wt,
                          L.wtf, sbuf);
        PDAL_LOOP_SYNC();
        restart_all<T, BETA>(L.st, L.n, L.m, L.pa.xh, L.pa.x, L.x0, L.x0f, L.da.yh, L.da.y, L.y0, L.y0f, L.phat,
                             L.da.ax, L.ax0, L.ax0f, L.da.u, L.da.lb, L.da.ub, L.pa.xbar, L.da.ybar);
        PDAL_LOOP_SYNC();
        /* the end of the FP32 phase is the host's to carry out */
        if (threadIdx.x == 0) sflag = L.st->phase_switch;
        __syncthreads();
        if (sflag) return;
    }
#undef PDAL_LOOP_SYNC
}

/* ------------------------------------------------------------------ */
/* result (LP/CP_AL/src/solver.cu:1768-1793, 2481-2500)                 */
/* ------------------------------------------------------------------ */
struct ResultColEpi : NoLongRed {
    const double *xh, *c, *cscale, *vlb, *vub;
    const CpalState *st;
    double *x_out, *rc_out;
    __device__ __forceinline__ void operator()(int j, const double *s, Red<0, 0> &) const {
        double rc = (c[j] - s[0]) * cscale[j] / st->ovr;
        if (!isfinite(vlb[j])) rc = fmin(rc, 0.0);
        if (!isfinite(vub[j])) rc = fmax(rc, 0.0);
        rc_out[j] = rc;
        x_out[j] = xh[j] / cscale[j] / st->cbr;
    }
};

template <int S>
__global__ void __launch_bounds__(kThreads) k_result_cols(RowPlanDev plan, const int *__restrict__ rp,
                                                          const int *__restrict__ ci, const double *__restrict__ val,
                                                          const double *__restrict__ yh, ResultColEpi epi) {
    __shared__ RowBlockSmem<S, 1, double> sm;
    auto g = [&](int c, double *out) { out[0] = yh[c]; };
    Red<0, 0> red;
    rowblock_run<S, 1, double>(plan, rp, ci, val, g, epi, red, sm);
}

static __global__ void k_result_rows(int m, const double *__restrict__ yh, const double *__restrict__ rscale,
                              const CpalState *__restrict__ st, double *y_out) {
    const double ovr = st->ovr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
        y_out[i] = yh[i] / rscale[i] / ovr;
}

/* Promotes / demotes a vector between the FP32 phase and FP64. */
template <typename A, typename B>
__global__ void k_convert(const A *__restrict__ src, B *dst, int len) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) dst[i] = (B)src[i];
}

/* ------------------------------------------------------------------ */
/* setup: equilibration (LP/CP_AL/src/preconditioner.cu)               */
/* ------------------------------------------------------------------ */

/* warp per row: s = clamp_sqrt(max |a| or sum |a|^deg), cum *= s
 * (preconditioner.cu:532-550, 634-667). mode 0 = abs max, 1 = power sum. */
/* ------------------------------------------------------------------ */
/* the transpose A^T built on the device                               */
/* ------------------------------------------------------------------ */
/* With the transpose's row pointers from the host (column counts), each
 * nonzero of A is placed in its column's segment by an atomic cursor -- rows
 * of at most kEqShort nonzeros one thread each, the listed longer rows a warp
 * each -- and every segment is then sorted by row index, moving the values
 * along.  Row indices within a column are distinct, so the result is exactly
 * the host transpose (rows in increasing order in every column), whatever
 * order the atomics took.  Columns of up to 32 entries are sorted by one
 * thread (insertion sort), the listed longer ones (up to kTransposeSort) by a
 * block (bitonic sort in shared memory). */
constexpr int kTransposeSort = 2048;
/* rows (columns) longer than this take a warp (a block) in the passes below */
constexpr int kEqShort = 32;

static __global__ void k_transpose_scatter(int nr, const int *__restrict__ rp, const int *__restrict__ ci,
                                           const double *__restrict__ v, int *cursor, int *tci, double *tv,
                                           const int *__restrict__ lrows, int nlong) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (int row = t; row < nr; row += nt) {
        const int k0 = rp[row], k1 = rp[row + 1];
        if (k1 - k0 > kEqShort) continue;
        for (int k = k0; k < k1; ++k) {
            const int p = atomicAdd(&cursor[ci[k]], 1);
            tci[p] = row;
            tv[p] = v[k];
        }
    }
    const int lane = threadIdx.x & 31;
    for (int q = t >> 5; q < nlong; q += nt >> 5) {
        const int row = lrows[q];
        for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) {
            const int p = atomicAdd(&cursor[ci[k]], 1);
            tci[p] = row;
            tv[p] = v[k];
        }
    }
}

/* columns of at most kEqShort entries: insertion sort by row, one thread each */
static __global__ void k_transpose_sort_short(int nc, const int *__restrict__ trp, int *tci, double *tv) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nc; j += gridDim.x * blockDim.x) {
        const int k0 = trp[j], k1 = trp[j + 1];
        if (k1 - k0 > kEqShort) continue;
        for (int k = k0 + 1; k < k1; ++k) {
            const int key = tci[k];
            const double val = tv[k];
            int q = k - 1;
            while (q >= k0 && tci[q] > key) {
                tci[q + 1] = tci[q];
                tv[q + 1] = tv[q];
                --q;
            }
            tci[q + 1] = key;
            tv[q + 1] = val;
        }
    }
}

/* the listed longer columns: a block each, bitonic sort of the segment
 * (padded to a power of two with keys above every row) in shared memory */
static __global__ void __launch_bounds__(kThreads) k_transpose_sort_long(const int *__restrict__ trp, int *tci,
                                                                          double *tv, const int *__restrict__ lcols,
                                                                          int nlong) {
    __shared__ int key[kTransposeSort];
    __shared__ double val[kTransposeSort];
    for (int q = blockIdx.x; q < nlong; q += gridDim.x) {
        const int j = lcols[q], k0 = trp[j], len = trp[j + 1] - k0;
        int n2 = 1;
        while (n2 < len) n2 <<= 1;
        for (int i = threadIdx.x; i < n2; i += blockDim.x) {
            key[i] = i < len ? tci[k0 + i] : 0x7fffffff;
            val[i] = i < len ? tv[k0 + i] : 0.0;
        }
        __syncthreads();
        for (int size = 2; size <= n2; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                    const int p = i ^ stride;
                    if (p > i) {
                        const bool up = (i & size) == 0;
                        if ((key[i] > key[p]) == up) {
                            const int tk = key[i];
                            key[i] = key[p];
                            key[p] = tk;
                            const double tvv = val[i];
                            val[i] = val[p];
                            val[p] = tvv;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            tci[k0 + i] = key[i];
            tv[k0 + i] = val[i];
        }
        __syncthreads();
    }
}

/* A^T's column indices with the long rows of A (hot_id >= 0) as -1 - h */
static __global__ void k_hot_indices(long long nnz, const int *__restrict__ ci, const int *__restrict__ hot_id,
                                     int *ci_hot) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nnz;
         k += (long long)gridDim.x * blockDim.x) {
        const int r = ci[k], h = hot_id[r];
        ci_hot[k] = h >= 0 ? -1 - h : r;
    }
}

/* Equilibration passes over the rows of a CSR matrix.  Rows of at most
 * kEqShort nonzeros (nearly all rows of a sparse LP) run one thread per row;
 * the longer rows, listed once at upload (`lrows`), run one warp per row in
 * the same launch.  (A warp per row for every row left 31 lanes idle on the
 * one-entry rows of a power-law LP and made each pass latency-bound.) */
__device__ __forceinline__ double row_scale_term(double v, int mode, double deg) {
    v = fabs(v);
    if (!isfinite(v)) v = 0.0;
    if (mode == 0) return v;
    if (deg == 2.0) return v * v;
    if (deg == 1.0) return v;
    if (deg == 0.5) return sqrt(v);
    return pow(v, deg);
}

__device__ __forceinline__ void row_scale_store(int row, double acc, double *scale, double *cum, double *inv) {
    const double s = (acc < 1e-12) ? 1.0 : sqrt(acc);
    cum[row] *= s;
    scale[row] = s;
    inv[row] = 1.0 / s;
}

/* Ruiz (mode 0: max |a|) or Pock-Chambolle (mode 1: sum |a|^deg) row scale
 * (LP/CP_AL/src/preconditioner.cu:273-378, 600-657).  The sums run in row
 * order in one thread, as the reference's kernel adds them (a long row too);
 * the maxima of the long rows take a warp (the order does not matter). */
static __global__ void k_row_scale(int nr, const int *__restrict__ rp, const double *__restrict__ val, int mode, double deg,
                            double *scale, double *cum, double *inv, const int *__restrict__ lrows, int nlong) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (int row = t; row < nr; row += nt) {
        const int k0 = rp[row], k1 = rp[row + 1];
        if (k1 - k0 > kEqShort) continue;
        double acc = 0.0;
        for (int k = k0; k < k1; ++k) {
            const double pv = row_scale_term(val[k], mode, deg);
            acc = mode == 0 ? fmax(acc, pv) : acc + pv;
        }
        row_scale_store(row, acc, scale, cum, inv);
    }
    if (mode != 0) {
        for (int q = t; q < nlong; q += nt) {
            const int row = lrows[q];
            double acc = 0.0;
            for (int k = rp[row]; k < rp[row + 1]; ++k) acc += row_scale_term(val[k], mode, deg);
            row_scale_store(row, acc, scale, cum, inv);
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    for (int q = t >> 5; q < nlong; q += nt >> 5) {
        const int row = lrows[q];
        double acc = 0.0;
        for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) acc = fmax(acc, row_scale_term(val[k], 0, deg));
        acc = warp_max(acc);
        if (lane == 0) row_scale_store(row, acc, scale, cum, inv);
    }
}

/* A values *= (1/d[j]) * (1/r[i]); rows of this matrix are scaled by
 * row_is_var ? d : r (preconditioner.cu:514-530).  The reciprocals come from
 * k_row_scale (the same 1/s, computed once per row instead of once per
 * nonzero: the FP64 divisions dominated this kernel on GB300's FP64 pipe). */
static __global__ void k_scale_matrix(int nr, const int *__restrict__ rp, const int *__restrict__ ci, double *val,
                               const double *__restrict__ inv_rowscale, const double *__restrict__ inv_colscale,
                               int row_is_var, const int *__restrict__ lrows, int nlong) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    for (int row = t; row < nr; row += nt) {
        const int k0 = rp[row], k1 = rp[row + 1];
        if (k1 - k0 > kEqShort) continue;
        const double inv_row = inv_rowscale[row];
        for (int k = k0; k < k1; ++k) {
            const double inv_col = inv_colscale[ci[k]];
            val[k] *= row_is_var ? inv_row * inv_col : inv_col * inv_row;
        }
    }
    const int lane = threadIdx.x & 31;
    for (int q = t >> 5; q < nlong; q += nt >> 5) {
        const int row = lrows[q];
        const double inv_row = inv_rowscale[row];
        for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) {
            const double inv_col = inv_colscale[ci[k]];
            val[k] *= row_is_var ? inv_row * inv_col : inv_col * inv_row;
        }
    }
}

/* Curtis-Reid log scales (LP/CP_AL/src/preconditioner.cu:553-588), warp per
 * row: the mean over the row's nonzeros of -log|a| - other[col] (|a| below
 * 1e-300 or not finite counts as 1e-300); an empty row gets 0.  delta, when
 * given, receives the change of the row's log scale. */
static __global__ void k_cr_log_update(int nr, const int *__restrict__ rp, const int *__restrict__ ci,
                                       const double *__restrict__ val, const double *__restrict__ other, double *ls,
                                       double *delta) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nr; row += warps) {
        const int k0 = rp[row], k1 = rp[row + 1];
        double acc = 0.0;
        for (int k = k0 + lane; k < k1; k += 32) {
            double v = fabs(val[k]);
            if (!isfinite(v) || v < 1e-300) v = 1e-300;
            acc += -log(v) - other[ci[k]];
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            const double u = k1 > k0 ? acc / (double)(k1 - k0) : 0.0;
            if (delta) delta[row] = u - ls[row];
            ls[row] = u;
        }
    }
}

/* per-block maximum over the nonzeros of |delta_row + delta_col|, the change
 * of a scaled entry's log (preconditioner.cu:590-609) */
static __global__ void __launch_bounds__(kThreads) k_cr_edge_change(int nr, const int *__restrict__ rp,
                                                                    const int *__restrict__ ci,
                                                                    const double *__restrict__ rd,
                                                                    const double *__restrict__ cd, double *part) {
    __shared__ double sbuf[kThreads / 32];
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    double mx = 0.0;
    for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nr; row += warps)
        for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) {
            const double e = fabs(rd[row] + cd[ci[k]]);
            if (isfinite(e) && e > mx) mx = e;
        }
    mx = warp_max(mx);
    if (lane == 0) sbuf[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) b = fmax(b, sbuf[w]);
        part[blockIdx.x] = b;
    }
}

/* log scale -> scaling 1/f and its inverse f = clamp(exp(log), 1e-30, 1e30);
 * cum *= 1/f (preconditioner.cu:611-624) */
static __global__ void k_cr_exp(int len, double *ls, double *inv, double *cum) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        const double f = fmin(fmax(exp(ls[i]), 1e-30), 1e30);
        const double s = 1.0 / f;
        ls[i] = s;
        inv[i] = f;
        cum[i] *= s;
    }
}

/* preconditioner.cu:476-512 with the inverses given (the Curtis-Reid pass
 * hands over f itself, not 1/(1/f)) */
static __global__ void k_scale_vectors_inv(int n, int m, const double *__restrict__ d, const double *__restrict__ dinv,
                                           const double *__restrict__ r, const double *__restrict__ rinv, double *c,
                                           double *vlb, double *vub, double *x0, double *clb, double *cub, double *y0) {
    const int total = n > m ? n : m;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < n) {
            const double dj = d[t];
            c[t] *= dinv[t];
            vlb[t] *= dj;
            vub[t] *= dj;
            x0[t] *= dj;
        }
        if (t < m) {
            clb[t] *= rinv[t];
            cub[t] *= rinv[t];
            y0[t] *= r[t];
        }
    }
}

/* preconditioner.cu:476-512 */
static __global__ void k_scale_vectors(int n, int m, const double *__restrict__ d, const double *__restrict__ r, double *c,
                                double *vlb, double *vub, double *x0, double *clb, double *cub, double *y0) {
    const int total = n > m ? n : m;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < n) {
            const double dj = d[t], inv = 1.0 / d[t];
            c[t] *= inv;
            vlb[t] *= dj;
            vub[t] *= dj;
            x0[t] *= dj;
        }
        if (t < m) {
            const double inv = 1.0 / r[t], ei = r[t];
            clb[t] *= inv;
            cub[t] *= inv;
            y0[t] *= ei;
        }
    }
}

/* bound/objective norms (preconditioner.cu:329-377, 669-691): partial sums of
 * the bound contributions and of c^2 per block. */
static __global__ void __launch_bounds__(kThreads) k_boundobj_partials(int n, int m, const double *__restrict__ clb,
                                                                const double *__restrict__ cub,
                                                                const double *__restrict__ c, double *part) {
    __shared__ double sbuf[2 * (kThreads / 32)];
    Red<2, 0> r;
    r.zero();
    const int total = n > m ? n : m;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < m) {
            const double L = clb[t], U = cub[t];
            const bool fL = isfinite(L), fU = isfinite(U);
            double acc = 0.0;
            if (fL && (!fU || fabs(L - U) > 1e-12)) acc += L * L;
            if (fU) acc += U * U;
            r.s[0] += acc;
        }
        if (t < n) r.s[1] += c[t] * c[t];
    }
    block_reduce<kThreads, 2, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        part[blockIdx.x * 2 + 0] = r.s[0];
        part[blockIdx.x * 2 + 1] = r.s[1];
    }
}

static __global__ void __launch_bounds__(kThreads) k_boundobj_finish(const double *__restrict__ part, int nparts,
                                                              CpalState *st, int enabled) {
    __shared__ double sbuf[2 * (kThreads / 32)];
    Red<2, 0> r;
    r.zero();
    for (int b = threadIdx.x; b < nparts; b += kThreads) {
        r.s[0] += part[b * 2];
        r.s[1] += part[b * 2 + 1];
    }
    block_reduce<kThreads, 2, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        if (enabled) {
            st->cbr = 1.0 / (sqrt(r.s[0]) + 1.0);
            st->ovr = 1.0 / (sqrt(r.s[1]) + 1.0);
        } else {
            st->cbr = 1.0;
            st->ovr = 1.0;
        }
    }
}

static __global__ void k_scale_boundobj(int n, int m, const CpalState *__restrict__ st, double *c, double *vlb, double *vub,
                                 double *x0, double *clb, double *cub, double *y0) {
    const double cs = st->cbr, os = st->ovr;
    const int total = n > m ? n : m;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        if (t < m) {
            clb[t] *= cs;
            cub[t] *= cs;
            y0[t] *= os;
        }
        if (t < n) {
            vlb[t] *= cs;
            vub[t] *= cs;
            c[t] *= os;
            x0[t] *= cs;
        }
    }
}

/* finite-bound copies (LP/CP_AL/src/solver.cu:2323-2338) */
static __global__ void k_finite_bounds(int m, const double *__restrict__ lb, const double *__restrict__ ub, double *lbf,
                                double *ubf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        lbf[i] = isfinite(lb[i]) ? lb[i] : 0.0;
        ubf[i] = isfinite(ub[i]) ? ub[i] : 0.0;
    }
}

/* ------------------------------------------------------------------ */
/* setup: power iteration on A A^T (LP/CP_AL/src/utils.cu:87-228)      */
/* ------------------------------------------------------------------ */
struct PowerState {
    double inv;  /* 1/|v| of the current vector */
    double s2;   /* Rayleigh quotient, sigma_max^2 estimate */
    double res;  /* residual norm */
    int done;    /* converged or out of iterations */
    int iters;
    int max_iter;
    double tol;
    double vsq;  /* |v|^2 of the current (unnormalised) vector */
};

/* The power iteration runs in the arithmetic type T: FP64 in the plain form
 * (the reference's arithmetic), FP32 in the chosen form, where its SpMVs
 * stream half the bytes; the Rayleigh quotient, the residual and the norms
 * are accumulated in FP64 either way. */
template <typename T>
struct PowerColEpi : NoLongRed {
    T *dp;
    __device__ __forceinline__ void operator()(int j, const T *s, Red<0, 0> &) const { dp[j] = s[0]; }
};

/* dp = A^T (inv * v) */
template <int S, typename T>
__global__ void __launch_bounds__(kThreads) k_power_at(RowPlanDev plan, const int *__restrict__ rp,
                                                       const int *__restrict__ ci, const T *__restrict__ val,
                                                       const T *__restrict__ v, T *dp,
                                                       const PowerState *__restrict__ ps) {
    pdl_enter();
    if (ps->done) return;
    __shared__ RowBlockSmem<S, 1, T> sm;
    const T inv = (T)ps->inv;
    PowerColEpi<T> epi;
    epi.dp = dp;
    auto g = [&](int c, T *out) { out[0] = inv * v[c]; };
    Red<0, 0> red;
    rowblock_run<S, 1, T>(plan, rp, ci, val, g, epi, red, sm);
}

/* vn = A dp, partial sums of (inv * v) . vn; with W2 also |vn|^2, slot
 * pairs (the fused FP32 step: the residual and the next normalisation then
 * follow from the two sums, see k_power_fin) */
template <typename T, bool W2 = false>
struct PowerRowEpi {
    static constexpr int NS = W2 ? 2 : 1;
    const T *v;
    T *vn;
    double inv;
    double *part;
    int nblocks;
    __device__ __forceinline__ void operator()(int i, const T *s, Red<NS, 0> &r) const {
        vn[i] = s[0];
        const double w = (double)s[0];
        r.s[0] += (inv * (double)v[i]) * w;
        if (W2) r.s[W2 ? 1 : 0] += w * w;
    }
    __device__ __forceinline__ void long_red(int lid, Red<NS, 0> &r) const {
#pragma unroll
        for (int q = 0; q < NS; ++q) part[NS * (nblocks + lid) + q] = r.s[q];
    }
};

template <int S, typename T, bool W2 = false>
__global__ void __launch_bounds__(kThreads) k_power_a(RowPlanDev plan, const int *__restrict__ rp,
                                                      const int *__restrict__ ci, const T *__restrict__ val,
                                                      const T *__restrict__ dp, const T *__restrict__ v,
                                                      T *vn, double *part, const PowerState *__restrict__ ps) {
    pdl_enter();
    if (ps->done) return;
    constexpr int NS = PowerRowEpi<T, W2>::NS;
    __shared__ RowBlockSmem<S, 1, T> sm;
    PowerRowEpi<T, W2> epi;
    epi.v = v;
    epi.vn = vn;
    epi.inv = ps->inv;
    epi.part = part;
    epi.nblocks = plan.nblocks;
    /* dp gathers bypass L1: the random column gathers of a large LP hit L2
     * (measured faster; the same load in k_power_at is slower) */
    auto g = [&](int c, T *out) { out[0] = __ldcg(dp + c); };
    Red<NS, 0> red;
    red.zero();
    rowblock_run<S, 1, T>(plan, rp, ci, val, g, epi, red, sm);
    block_reduce<kThreads, NS, 0>(red, sm.red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NS; ++q) part[NS * blockIdx.x + q] = red.s[q];
    }
}

/* Fused FP32 step, after k_power_a<..., true>: the Rayleigh quotient
 * s2 = (inv v) . vn, the residual |vn - s2 (inv v)| from
 * |vn|^2 - 2 s2 (inv v) . vn + s2^2 |inv v|^2 (no pass over the vectors;
 * FP64 sums, absolute error ~1e-16 |vn|^2 against the 1e-4 tolerance), the
 * next normalisation 1/|vn| and the stopping test.  The vectors alternate
 * between two buffers instead of being copied. */
static __global__ void __launch_bounds__(kThreads) k_power_fin(const double *__restrict__ part, int nparts,
                                                               PowerState *ps) {
    pdl_enter();
    if (ps->done) return;
    __shared__ double sbuf[2 * (kThreads / 32)];
    Red<2, 0> r;
    r.zero();
    for (int b = threadIdx.x; b < nparts; b += kThreads) {
        r.s[0] += part[2 * b];
        r.s[1] += part[2 * b + 1];
    }
    block_reduce<kThreads, 2, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        const double s2 = r.s[0], w2 = r.s[1];
        const double nv2 = ps->inv * ps->inv * ps->vsq;
        ps->s2 = s2;
        ps->iters += 1;
        ps->res = sqrt(fmax(w2 - 2.0 * s2 * s2 + s2 * s2 * nv2, 0.0));
        ps->inv = 1.0 / sqrt(w2);
        ps->vsq = w2;
        if (ps->res < ps->tol || ps->iters >= ps->max_iter) ps->done = 1;
    }
}

/* s2 = sum(part) */
static __global__ void __launch_bounds__(kThreads) k_power_dot(const double *__restrict__ part, int nparts, PowerState *ps) {
    if (ps->done) return;
    __shared__ double sbuf[kThreads / 32];
    Red<1, 0> r;
    r.zero();
    for (int b = threadIdx.x; b < nparts; b += kThreads) r.s[0] += part[b];
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) ps->s2 = r.s[0];
}

/* residual vn - s2 * (inv v) and |vn|^2; then v <- vn */
template <typename T>
__global__ void __launch_bounds__(kThreads) k_power_resid(int m, T *v, const T *__restrict__ vn, double *part,
                                                          const PowerState *__restrict__ ps) {
    if (ps->done) return;
    __shared__ double sbuf[2 * (kThreads / 32)];
    const double inv = ps->inv, s2 = ps->s2;
    Red<2, 0> r;
    r.zero();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double nv = inv * (double)v[i];
        const double vni = (double)vn[i];
        const double q = (-s2 * nv) + vni;
        r.s[0] += q * q;
        r.s[1] += vni * vni;
        v[i] = vn[i];
    }
    block_reduce<kThreads, 2, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        part[blockIdx.x * 2] = r.s[0];
        part[blockIdx.x * 2 + 1] = r.s[1];
    }
}

/* residual test and the normalisation of the next vector */
static __global__ void __launch_bounds__(kThreads) k_power_check(const double *__restrict__ part, int nparts,
                                                          PowerState *ps) {
    if (ps->done) return;
    __shared__ double sbuf[2 * (kThreads / 32)];
    Red<2, 0> r;
    r.zero();
    for (int b = threadIdx.x; b < nparts; b += kThreads) {
        r.s[0] += part[b * 2];
        r.s[1] += part[b * 2 + 1];
    }
    block_reduce<kThreads, 2, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        ps->iters += 1;
        ps->res = sqrt(r.s[0]);
        ps->inv = 1.0 / sqrt(r.s[1]);
        if (ps->res < ps->tol || ps->iters >= ps->max_iter) ps->done = 1;
    }
}

/* ------------------------------------------------------------------ */
/* Lanczos estimate of sigma_max(A)^2 (chosen form)                    */
/* ------------------------------------------------------------------ */
/* Lanczos on A A^T: q_1 = v0/|v0|, then for j = 1, 2, ...
 *   w = A (A^T q_j)                      (FP32 products: k_power_at and
 *                                         k_power_a with inv = 1, which also
 *                                         give the partials of q_j . w)
 *   alpha_j = q_j . w
 *   r = w - alpha_j q_j - beta_{j-1} q_{j-1},  beta_j = |r|,  q_{j+1} = r / beta_j
 * (vectors and reductions in FP64).  The largest eigenvalue of the
 * tridiagonal (alpha, beta) matrix -- computed on the host -- is a lower
 * bound of sigma_max^2 that converges much faster than the power iteration's
 * Rayleigh quotient (Golub and Van Loan, Matrix Computations, ch. 10).  The
 * step counter and the coefficients live in LanczosDev. */
struct LanczosDev {
    double *alpha, *beta; /* per step */
    int *j;               /* steps done */
};

/* alpha_j = sum of the partials of q_j . w */
static __global__ void __launch_bounds__(kThreads) k_lz_alpha(const double *__restrict__ part, int nparts,
                                                              LanczosDev lz) {
    pdl_enter();
    __shared__ double sbuf[kThreads / 32];
    Red<1, 0> r;
    r.zero();
    for (int b = threadIdx.x; b < nparts; b += kThreads) r.s[0] += part[b];
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) lz.alpha[*lz.j] = r.s[0];
}

/* p <- w - alpha_j q - beta_{j-1} p (p holds q_{j-1}), partials of |p|^2 */
template <typename T>
__global__ void __launch_bounds__(kThreads) k_lz_update(int m, const T *__restrict__ w, const double *__restrict__ q,
                                                        double *p, LanczosDev lz, double *part) {
    pdl_enter();
    __shared__ double sbuf[kThreads / 32];
    const int j = *lz.j;
    const double a = lz.alpha[j], b = j > 0 ? lz.beta[j - 1] : 0.0;
    Red<1, 0> r;
    r.zero();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double v = (double)w[i] - a * q[i] - b * p[i];
        p[i] = v;
        r.s[0] += v * v;
    }
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) part[blockIdx.x] = r.s[0];
}

/* beta_j = |r|, then j <- j + 1 */
static __global__ void __launch_bounds__(kThreads) k_lz_beta(const double *__restrict__ part, int nparts,
                                                             LanczosDev lz) {
    pdl_enter();
    __shared__ double sbuf[kThreads / 32];
    Red<1, 0> r;
    r.zero();
    for (int b = threadIdx.x; b < nparts; b += kThreads) r.s[0] += part[b];
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        const int j = *lz.j;
        lz.beta[j] = sqrt(r.s[0]);
        *lz.j = j + 1;
    }
}

/* q_{j+1} = r / beta_j into p (a zero beta -- an invariant subspace -- leaves
 * a zero vector, so the later coefficients are zero) and its FP32 copy for
 * the next products */
template <typename T>
__global__ void __launch_bounds__(kThreads) k_lz_next(int m, double *p, T *qf, LanczosDev lz) {
    pdl_enter();
    const double b = lz.beta[*lz.j - 1];
    const double inv = b > 0.0 ? 1.0 / b : 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double v = p[i] * inv;
        p[i] = v;
        qf[i] = (T)v;
    }
}

/* q_1 = v0 / |v0| (one block; v0 in q), q_0 = 0 in p */
template <typename T>
__global__ void __launch_bounds__(kThreads) k_lz_start(int m, double *q, T *qf, double *p) {
    __shared__ double sbuf[kThreads / 32];
    __shared__ double inv;
    Red<1, 0> r;
    r.zero();
    for (int i = threadIdx.x; i < m; i += kThreads) r.s[0] += q[i] * q[i];
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) inv = r.s[0] > 0.0 ? 1.0 / sqrt(r.s[0]) : 0.0;
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += kThreads) {
        const double v = q[i] * inv;
        q[i] = v;
        qf[i] = (T)v;
        p[i] = 0.0;
    }
}

/* 1/|v| of the start vector */
template <typename T>
__global__ void __launch_bounds__(kThreads) k_power_start(int m, const T *__restrict__ v, PowerState *ps) {
    __shared__ double sbuf[kThreads / 32];
    Red<1, 0> r;
    r.zero();
    for (int i = threadIdx.x; i < m; i += kThreads) r.s[0] += (double)v[i] * (double)v[i];
    block_reduce<kThreads, 1, 0>(r, sbuf);
    if (threadIdx.x == 0) {
        ps->inv = 1.0 / sqrt(r.s[0]);
        ps->vsq = r.s[0];
    }
}

} // namespace pdal
