/*
 * rowblock.cuh -- the sparse-product engine of the solver (sm_103a).
 *
 * One launch streams a CSR matrix exactly once.  The rows are cut on the host
 * into "row blocks" of at most S nonzeros (one CUDA block each):
 *
 *   STREAM block  rows [r0, r1) whose nonzeros [k0, k1) fit in S.  The block
 *                 loads every nonzero once, coalesced, forms val*gather in
 *                 shared memory, then a power-of-two group of lanes reduces
 *                 each row and its leader applies the fused epilogue.
 *   LONG piece    one S-slice of a row longer than S.  Each piece reduces its
 *                 slice, stores the partial in its own slot, and the block that
 *                 arrives last (atomic counter) adds the slots in piece order
 *                 and runs the epilogue.  The sum order is fixed, so results
 *                 are deterministic, and no block ever waits on another.
 *
 * This replaces cusparseSpMV(CSR_ALG2) plus the separate elementwise kernel of
 * the reference (LP/CP_AL/src/solver.cu:2523-2661): the epilogue (projection,
 * reflection, Halpern averaging, residual terms) runs while the row sum is in
 * a register, so the product vector never goes to HBM.
 *
 * The epilogue may also produce per-block reduction terms (sums and maxima)
 * that are written to a partial array and finished by a single-block kernel in
 * a fixed order.
 */
#pragma once

#include "rowblock_config.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace pdal {

/* Plan of one matrix, in device memory. */
struct RowPlanDev {
    const int4 *__restrict__ desc;  /* {r0, r1 (or ~long_id), k0, k1} per block */
    const int4 *__restrict__ linfo; /* {row, pieces, slot_base, row_start} per long row */
    double *__restrict__ lpart;     /* kLongStride doubles per long piece */
    unsigned int *__restrict__ lcount; /* arrival counter per long row (kept at 0 between launches) */
    int nblocks;
    int nlong;
};

/* Reduction terms carried by an epilogue: NS sums and NM maxima. */
template <int NS, int NM>
struct Red {
    double s[NS > 0 ? NS : 1];
    double mx[NM > 0 ? NM : 1];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < (NS > 0 ? NS : 1); ++i) s[i] = 0.0;
#pragma unroll
        for (int i = 0; i < (NM > 0 ? NM : 1); ++i) mx[i] = 0.0;
    }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

/* Deterministic block reduction of NS sums and NM maxima; thread 0 gets the
 * totals.  sbuf needs (NS+NM)*(NT/32) doubles. */
template <int NT, int NS, int NM>
__device__ __forceinline__ void block_reduce(Red<NS, NM> &r, double *sbuf) {
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        double v = warp_sum(r.s[i]);
        if (lane == 0) sbuf[i * NW + wid] = v;
    }
#pragma unroll
    for (int i = 0; i < NM; ++i) {
        double v = warp_max(r.mx[i]);
        if (lane == 0) sbuf[(NS + i) * NW + wid] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            double t = 0.0;
            for (int w = 0; w < NW; ++w) t += sbuf[i * NW + w];
            r.s[i] = t;
        }
#pragma unroll
        for (int i = 0; i < NM; ++i) {
            double t = 0.0;
            for (int w = 0; w < NW; ++w) t = fmax(t, sbuf[(NS + i) * NW + w]);
            r.mx[i] = t;
        }
    }
    __syncthreads();
}

/* 128-bit streaming loads of four consecutive elements (the matrix is read
 * once per launch: evict-first keeps the gathered vector resident in L2). */
__device__ __forceinline__ void load4_stream(const int *p, int (&v)[4]) {
    const int4 t = __ldcs(reinterpret_cast<const int4 *>(p));
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
}
__device__ __forceinline__ void load4_stream(const float *p, float (&v)[4]) {
    const float4 t = __ldcs(reinterpret_cast<const float4 *>(p));
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
}
__device__ __forceinline__ void load4_stream(const double *p, double (&v)[4]) {
    const double2 a = __ldcs(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcs(reinterpret_cast<const double2 *>(p + 2));
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}

template <typename T>
__device__ __forceinline__ T vfma(T a, T b, T c) {
    return fma(a, b, c);
}
template <>
__device__ __forceinline__ float vfma<float>(float a, float b, float c) {
    return fmaf(a, b, c);
}

/* Shared memory of one row-block launch: the block's matrix values and the
 * NP gathered vector entries of each nonzero, staged in nonzero order.
 * Element e of the block sits at index e - kb, kb = k0 rounded down to a
 * multiple of 4, so every thread writes its four elements with one 128-bit
 * store (no bank conflicts). */
template <int S, int NP, typename T>
struct RowBlockSmem {
    __align__(16) T val[S + 4];
    __align__(16) T g[NP][S + 4];
    int rp[kMaxRowsPerBlock + 1];
    double red[8 * (kThreads / 32) * 2];
    int last;
};

__device__ __forceinline__ void store4_shared(float *dst, const float (&v)[4]) {
    *reinterpret_cast<float4 *>(dst) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void store4_shared(double *dst, const double (&v)[4]) {
    reinterpret_cast<double2 *>(dst)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2 *>(dst)[1] = make_double2(v[2], v[3]);
}

/* Stages nonzeros [k0, k1) (at most S) at smem index e - (k0 & ~3): values
 * with 128-bit streaming loads, the gathered entries through the read-only
 * path.  Arrays are padded so that the four-element window may extend three
 * elements past k1; elements outside [k0, k1) are staged as zeros and never
 * read. */
template <int S, int NP, typename T, class Gat>
__device__ __forceinline__ void rowblock_stage(int k0, int k1, const int *__restrict__ ci, const T *__restrict__ val,
                                               Gat &gat, RowBlockSmem<S, NP, T> &sm) {
    constexpr int NT = kThreads;
    constexpr int MAXIT = (S / 4 + 1 + NT - 1) / NT;
    const int kb = k0 & ~3;
    const int nch = (k1 - kb + 3) >> 2;
#pragma unroll
    for (int it = 0; it < MAXIT; ++it) {
        const int c = it * NT + (int)threadIdx.x;
        if (c < nch) {
            const int kc = kb + 4 * c;
            int cols[4];
            T vals[4];
            load4_stream(ci + kc, cols);
            load4_stream(val + kc, vals);
            T gv[NP][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = kc + q;
                if (e >= k0 && e < k1) {
                    T t[NP];
                    gat(cols[q], t);
#pragma unroll
                    for (int p = 0; p < NP; ++p) gv[p][q] = t[p];
                } else {
#pragma unroll
                    for (int p = 0; p < NP; ++p) gv[p][q] = T(0);
                    vals[q] = T(0);
                }
            }
            store4_shared(&sm.val[4 * c], vals);
#pragma unroll
            for (int p = 0; p < NP; ++p) store4_shared(&sm.g[p][4 * c], gv[p]);
        }
    }
}

/* Sum over the block in the arithmetic type T; thread 0 gets the totals. */
template <int NP, typename T>
__device__ __forceinline__ void block_sum_t(T (&s)[NP], T *sbuf) {
    constexpr int NW = kThreads / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[p] += __shfl_xor_sync(0xffffffffu, s[p], o);
        if (lane == 0) sbuf[p * NW + wid] = s[p];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            T t = T(0);
            for (int w = 0; w < NW; ++w) t += sbuf[p * NW + w];
            s[p] = t;
        }
    }
    __syncthreads();
}

/*
 * Runs row block `blk` of `plan` (rowblock_run below: blk = blockIdx.x).
 *   gat(col, T out[NP])         the NP vector entries a nonzero in column col
 *                               multiplies (one per simultaneous product)
 *   epi(row, const T s[NP], R&) the fused row epilogue; may add to R
 *   epi.long_red(long_id, R&)   stores the reduction terms of a long row
 * Each row sum is a chain of fused multiply-adds in T (one per nonzero and
 * product).  Returns the per-thread reduction terms in `red` (STREAM rows
 * only; long rows are stored through long_red so their slot does not depend
 * on which block finished last).
 */
template <int S, int NP, typename T, class R, class Gat, class Epi>
__device__ __forceinline__ void rowblock_run_at(int blk, const RowPlanDev &plan, const int *__restrict__ rp,
                                                const int *__restrict__ ci, const T *__restrict__ val, Gat &gat,
                                                Epi &epi, R &red, RowBlockSmem<S, NP, T> &sm) {
    constexpr int NT = kThreads;
    static_assert(S % NT == 0, "S must be a multiple of the block size");
    static_assert(NP <= kLongStride, "too many products per nonzero");
    const int4 d = plan.desc[blk];
    const int tid = threadIdx.x;
    if (d.y >= d.x) {
        const int r0 = d.x, nrows = d.y - d.x, k0 = d.z, k1 = d.w;
        const int kb = k0 & ~3;
        for (int t = tid; t <= nrows; t += NT) sm.rp[t] = rp[r0 + t] - kb;
        rowblock_stage<S, NP, T>(k0, k1, ci, val, gat, sm);
        __syncthreads();
        if (nrows <= NT) {
            /* group of g lanes per row, g a power of two, g <= 32 */
            int g = 32;
            while (g > 1 && g * nrows > NT) g >>= 1;
            const int row = tid / g, lane = tid & (g - 1);
            T s[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) s[p] = T(0);
            if (row < nrows) {
                const int e = sm.rp[row + 1];
                for (int kk = sm.rp[row] + lane; kk < e; kk += g) {
                    const T v = sm.val[kk];
#pragma unroll
                    for (int p = 0; p < NP; ++p) s[p] = vfma(v, sm.g[p][kk], s[p]);
                }
            }
            for (int o = g >> 1; o > 0; o >>= 1) {
#pragma unroll
                for (int p = 0; p < NP; ++p) s[p] += __shfl_down_sync(0xffffffffu, s[p], o, g);
            }
            if (row < nrows && lane == 0) epi(r0 + row, s, red);
        } else {
            for (int row = tid; row < nrows; row += NT) {
                T s[NP];
#pragma unroll
                for (int p = 0; p < NP; ++p) s[p] = T(0);
                const int e = sm.rp[row + 1];
                for (int kk = sm.rp[row]; kk < e; ++kk) {
                    const T v = sm.val[kk];
#pragma unroll
                    for (int p = 0; p < NP; ++p) s[p] = vfma(v, sm.g[p][kk], s[p]);
                }
                epi(r0 + row, s, red);
            }
        }
    } else {
        const int lid = ~d.y;
        const int4 li = plan.linfo[lid];
        const int piece = (d.z - li.w) / S;
        rowblock_stage<S, NP, T>(d.z, d.w, ci, val, gat, sm);
        __syncthreads();
        T s[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) s[p] = T(0);
        const int lo = d.z - (d.z & ~3), hi = d.w - (d.z & ~3);
        for (int kk = lo + tid; kk < hi; kk += NT) {
            const T v = sm.val[kk];
#pragma unroll
            for (int p = 0; p < NP; ++p) s[p] = vfma(v, sm.g[p][kk], s[p]);
        }
        block_sum_t<NP, T>(s, reinterpret_cast<T *>(sm.red));
        if (tid == 0) {
#pragma unroll
            for (int p = 0; p < NP; ++p) plan.lpart[(size_t)(li.z + piece) * kLongStride + p] = (double)s[p];
            __threadfence();
            const unsigned prev = atomicAdd(&plan.lcount[lid], 1u);
            sm.last = (prev == (unsigned)(li.y - 1));
        }
        __syncthreads();
        if (sm.last && tid == 0) {
            __threadfence();
            double tot[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) tot[p] = 0.0;
            for (int q = 0; q < li.y; ++q) {
#pragma unroll
                for (int p = 0; p < NP; ++p) tot[p] += __ldcg(&plan.lpart[(size_t)(li.z + q) * kLongStride + p]);
            }
            plan.lcount[lid] = 0u;
            T st[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) st[p] = (T)tot[p];
            R lr;
            lr.zero();
            epi(li.x, st, lr);
            epi.long_red(lid, lr);
        }
    }
}

template <int S, int NP, typename T, class R, class Gat, class Epi>
__device__ __forceinline__ void rowblock_run(const RowPlanDev &plan, const int *__restrict__ rp,
                                             const int *__restrict__ ci, const T *__restrict__ val, Gat &gat, Epi &epi,
                                             R &red, RowBlockSmem<S, NP, T> &sm) {
    rowblock_run_at<S, NP, T>((int)blockIdx.x, plan, rp, ci, val, gat, epi, red, sm);
}

} // namespace pdal
