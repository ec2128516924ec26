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

/* Shared memory of one row-block launch. */
template <int S, int NP, typename Acc>
struct RowBlockSmem {
    Acc prod[NP][S];
    int rp[kMaxRowsPerBlock + 1];
    double red[8 * (kThreads / 32) * 2];
    int last;
};

/*
 * Runs the row block blockIdx.x of `plan`.
 *   prod(k, Acc out[NP])          products of nonzero k (val * gathered vector)
 *   epi(row, const Acc s[NP], R&) the fused row epilogue; may add to R
 *   epi.long_red(long_id, R&)     stores the reduction terms of a long row
 * Returns the per-thread reduction terms in `red` (STREAM rows only; long rows
 * are stored through long_red so their slot does not depend on which block
 * finished last).
 */
template <int S, int NP, typename Acc, class R, class Prod, class Epi>
__device__ __forceinline__ void rowblock_run(const RowPlanDev &plan, const int *__restrict__ rp, Prod &prod, Epi &epi,
                                             R &red, RowBlockSmem<S, NP, Acc> &sm) {
    constexpr int NT = kThreads;
    static_assert(S % NT == 0, "S must be a multiple of the block size");
    static_assert(NP <= kLongStride, "too many products per nonzero");
    const int4 d = plan.desc[blockIdx.x];
    const int tid = threadIdx.x;
    if (d.y >= d.x) {
        const int r0 = d.x, nrows = d.y - d.x, k0 = d.z, k1 = d.w;
        for (int t = tid; t <= nrows; t += NT) sm.rp[t] = rp[r0 + t] - k0;
#pragma unroll
        for (int it = 0; it < S / NT; ++it) {
            const int kk = it * NT + tid;
            const int k = k0 + kk;
            if (k < k1) {
                Acc pv[NP];
                prod(k, pv);
#pragma unroll
                for (int p = 0; p < NP; ++p) sm.prod[p][kk] = pv[p];
            }
        }
        __syncthreads();
        if (nrows <= NT) {
            /* group of g lanes per row, g a power of two, g <= 32 */
            int g = 32;
            while (g > 1 && g * nrows > NT) g >>= 1;
            const int row = tid / g, lane = tid & (g - 1);
            Acc s[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) s[p] = Acc(0);
            if (row < nrows) {
                const int e = sm.rp[row + 1];
                for (int kk = sm.rp[row] + lane; kk < e; kk += g) {
#pragma unroll
                    for (int p = 0; p < NP; ++p) s[p] += sm.prod[p][kk];
                }
            }
            for (int o = g >> 1; o > 0; o >>= 1) {
#pragma unroll
                for (int p = 0; p < NP; ++p) s[p] += __shfl_down_sync(0xffffffffu, s[p], o, g);
            }
            if (row < nrows && lane == 0) epi(r0 + row, s, red);
        } else {
            for (int row = tid; row < nrows; row += NT) {
                Acc s[NP];
#pragma unroll
                for (int p = 0; p < NP; ++p) s[p] = Acc(0);
                const int e = sm.rp[row + 1];
                for (int kk = sm.rp[row]; kk < e; ++kk) {
#pragma unroll
                    for (int p = 0; p < NP; ++p) s[p] += sm.prod[p][kk];
                }
                epi(r0 + row, s, red);
            }
        }
    } else {
        const int lid = ~d.y;
        const int4 li = plan.linfo[lid];
        const int piece = (d.z - li.w) / S;
        Red<NP, 0> acc;
        acc.zero();
        for (int k = d.z + tid; k < d.w; k += NT) {
            Acc pv[NP];
            prod(k, pv);
#pragma unroll
            for (int p = 0; p < NP; ++p) acc.s[p] += (double)pv[p];
        }
        block_reduce<NT, NP, 0>(acc, sm.red);
        if (tid == 0) {
#pragma unroll
            for (int p = 0; p < NP; ++p) plan.lpart[(size_t)(li.z + piece) * kLongStride + p] = acc.s[p];
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
            Acc s[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) s[p] = (Acc)tot[p];
            R lr;
            lr.zero();
            epi(li.x, s, lr);
            epi.long_red(lid, lr);
        }
    }
}

} // namespace pdal
