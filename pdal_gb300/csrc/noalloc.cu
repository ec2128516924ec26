/*
 * noalloc.cu -- primal KKT evaluation of a candidate point without any memory
 * allocation.
 *
 * Some callers cannot allocate device memory: code that runs while another
 * library owns the allocator (a framework caching allocator or a memory pool
 * that forbids cudaMalloc/cudaFree while it is active), code called between
 * the launches of a latency-critical loop where cudaMalloc would synchronise
 * the device, and embedded hosts with a fixed device-memory budget.  They can
 * still check a candidate solution with this entry point: it evaluates the
 * primal feasibility residual and the objective of x for
 *     min c'x  s.t.  con_lb <= A x <= con_ub
 * on the caller's own device buffers, the same terms the solver's row
 * evaluation kernel reduces (k_eval_rows in cpal_kernels.cuh, following
 * LP/CP_AL/src/utils.cu:812-917), but on the unscaled problem.
 *
 * Its only scratch is g_partials below: one slot of partial sums per CUDA
 * block, a fixed kNoAllocMaxBlocks slots (2 MiB), held by every device that
 * loads the library until the process exits.  One warp reduces one row, so a
 * call accepts at most kNoAllocMaxRows rows.
 */
#include "../../include/cp_al_gb300.h"
#include "cpal_setup.h"
#include "rowblock.cuh"

#include <cuda.h> /* driver types only: the two driver calls are fetched through the runtime */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

namespace pdal {
namespace {

constexpr int kNoAllocRowsPerBlock = kThreads / 32;
constexpr int kNoAllocMaxBlocks = 65536;
constexpr int kNoAllocMaxRows = kNoAllocMaxBlocks * kNoAllocRowsPerBlock; /* 524,288 */
constexpr int kNoAllocSlot = 4; /* doubles per block: sum r^2, max |r|, sum c_j x_j, spare */
constexpr int kNoAllocMaxDevices = 64;

/* The scratch of every call on this device: no call ever allocates. */
static __device__ __align__(256) double g_partials[kNoAllocMaxBlocks * kNoAllocSlot];

/* Maximum that keeps a NaN: a NaN anywhere in x, A or the bounds must show in
 * max |r| as well as in the norm, or a broken candidate could look feasible. */
__device__ __forceinline__ double nan_max(double a, double b) { return (a != a || b != b) ? a + b : fmax(a, b); }

/* Deterministic block reduction of (sum, sum, NaN-keeping max); thread 0
 * gets the totals.  sbuf holds 3 * (kThreads / 32) doubles. */
__device__ __forceinline__ void reduce3(double &s0, double &s1, double &mx, double *sbuf) {
    constexpr int NW = kThreads / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        mx = nan_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
        sbuf[wid] = s0;
        sbuf[NW + wid] = s1;
        sbuf[2 * NW + wid] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s0 = s1 = mx = 0.0;
        for (int w = 0; w < NW; ++w) {
            s0 += sbuf[w];
            s1 += sbuf[NW + w];
            mx = nan_max(mx, sbuf[2 * NW + w]);
        }
    }
    __syncthreads();
}

/* Per block: rows (warp per row) give |A x - P(A x)|^2 and its maximum; the
 * threads also sum c_j x_j over a block-strided share of the columns. Every
 * slot a launch uses is rewritten, so nothing carries over between calls. */
__global__ void __launch_bounds__(kThreads) k_primal_kkt_partials(int m, int n, const int *__restrict__ rp,
                                                                  const int *__restrict__ ci,
                                                                  const double *__restrict__ vals,
                                                                  const double *__restrict__ lb,
                                                                  const double *__restrict__ ub,
                                                                  const double *__restrict__ c,
                                                                  const double *__restrict__ x, double *partials) {
    __shared__ double sbuf[3 * (kThreads / 32)];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row = blockIdx.x * kNoAllocRowsPerBlock + warp;
    double rsq = 0.0, cx = 0.0, rmax = 0.0;
    if (row < m) {
        double s = 0.0;
        for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) s = fma(vals[k], x[ci[k]], s);
        s = warp_sum(s);
        if (lane == 0) {
            const double res = s - fmax(lb[row], fmin(s, ub[row]));
            rsq = res * res;
            /* a NaN row sum gives a NaN residual: fmax/fmin of the projection
             * would turn it into a bound, so carry it explicitly */
            rmax = (s != s) ? s : fabs(res);
        }
    }
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) cx += c[j] * x[j];
    reduce3(rsq, cx, rmax, sbuf);
    if (threadIdx.x == 0) {
        double *slot = partials + (size_t)blockIdx.x * kNoAllocSlot;
        slot[0] = rsq;
        slot[1] = rmax;
        slot[2] = cx;
        slot[3] = 0.0;
    }
}

__global__ void __launch_bounds__(kThreads) k_primal_kkt_finish(int nblocks, const double *__restrict__ partials,
                                                                double *out) {
    __shared__ double sbuf[3 * (kThreads / 32)];
    double rsq = 0.0, cx = 0.0, rmax = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kThreads) {
        const double *slot = partials + (size_t)b * kNoAllocSlot;
        rsq += slot[0];
        rmax = nan_max(rmax, slot[1]);
        cx += slot[2];
    }
    reduce3(rsq, cx, rmax, sbuf);
    if (threadIdx.x == 0) {
        out[0] = sqrt(rsq);
        out[1] = rmax;
        out[2] = cx;
    }
}

/* The scratch address is cached per device together with the id of the
 * context it was taken in: after cudaDeviceReset (or under another context on
 * the same device) the id differs and the address is taken again, so a call
 * never uses an address of a context that is gone.  Context ids are unique
 * for the life of the process (cuCtxGetId).  The two driver calls are
 * fetched through the runtime, so the library needs no link to libcuda. */
struct ScratchCache {
    unsigned long long ctx_id = 0;
    double *ptr = nullptr;
};
std::mutex g_setup_mutex;
ScratchCache g_scratch[kNoAllocMaxDevices];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_driver_fns_tried = false;

/* id of the current context, or 0 when there is none yet (or the driver
 * entry points are unavailable: then nothing is cached) */
unsigned long long current_context_id() {
    if (!g_driver_fns_tried) {
        g_driver_fns_tried = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError();
    }
    if (!g_ctx_get_current || !g_ctx_get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

int fail(const std::string &msg) {
    set_last_error("primal_kkt_noalloc: " + msg);
    return -1;
}

} // namespace
} // namespace pdal

extern "C" {

int cp_al_gb300_primal_kkt_noalloc(int m, int n, const int *row_ptr, const int *col_ind, const double *vals,
                                   const double *con_lb, const double *con_ub, const double *c, const double *x,
                                   double *out, void *stream) {
    using namespace pdal;
    clear_last_error();
    if (m < 0 || n <= 0) return fail("m must be >= 0 and n > 0");
    if (m > kNoAllocMaxRows)
        return fail(std::to_string(m) + " rows exceed the " + std::to_string(kNoAllocMaxRows) +
                    " rows its fixed scratch supports");
    if (!c || !x || !out || (m > 0 && (!row_ptr || !col_ind || !vals || !con_lb || !con_ub)))
        return fail("missing device pointer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail("device ordinal out of range");
    double *scratch = nullptr;
    {
        /* once per device and context, with that device current: the device
         * address of the scratch array (its host-side name is only a
         * stand-in) */
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        const unsigned long long id = current_context_id();
        ScratchCache &sc = g_scratch[dev];
        if (!sc.ptr || id == 0 || id != sc.ctx_id) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_partials);
            if (e != cudaSuccess) return fail(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            sc.ptr = static_cast<double *>(p);
            sc.ctx_id = current_context_id(); /* the context exists now */
        }
        scratch = sc.ptr;
    }
    const int nblocks = m > 0 ? (m + kNoAllocRowsPerBlock - 1) / kNoAllocRowsPerBlock : 1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_primal_kkt_partials<<<nblocks, kThreads, 0, s>>>(m, n, row_ptr, col_ind, vals, con_lb, con_ub, c, x, scratch);
    k_primal_kkt_finish<<<1, kThreads, 0, s>>>(nblocks, scratch, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("launch: ") + cudaGetErrorString(e));
    return 0;
}

} // extern "C"
