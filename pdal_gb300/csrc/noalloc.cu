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
#include "rowblock.cuh"

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
    Red<2, 1> r;
    r.zero();
    if (row < m) {
        double s = 0.0;
        for (int k = rp[row] + lane; k < rp[row + 1]; k += 32) s = fma(vals[k], x[ci[k]], s);
        s = warp_sum(s);
        if (lane == 0) {
            const double res = s - fmax(lb[row], fmin(s, ub[row]));
            r.s[0] = res * res;
            r.mx[0] = fabs(res);
        }
    }
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) r.s[1] += c[j] * x[j];
    block_reduce<kThreads, 2, 1>(r, sbuf);
    if (threadIdx.x == 0) {
        double *slot = partials + (size_t)blockIdx.x * kNoAllocSlot;
        slot[0] = r.s[0];
        slot[1] = r.mx[0];
        slot[2] = r.s[1];
        slot[3] = 0.0;
    }
}

__global__ void __launch_bounds__(kThreads) k_primal_kkt_finish(int nblocks, const double *__restrict__ partials,
                                                                double *out) {
    __shared__ double sbuf[3 * (kThreads / 32)];
    Red<2, 1> r;
    r.zero();
    for (int b = threadIdx.x; b < nblocks; b += kThreads) {
        const double *slot = partials + (size_t)b * kNoAllocSlot;
        r.s[0] += slot[0];
        r.mx[0] = fmax(r.mx[0], slot[1]);
        r.s[1] += slot[2];
    }
    block_reduce<kThreads, 2, 1>(r, sbuf);
    if (threadIdx.x == 0) {
        out[0] = sqrt(r.s[0]);
        out[1] = r.mx[0];
        out[2] = r.s[1];
    }
}

std::mutex g_setup_mutex;
double *g_scratch_ptr[kNoAllocMaxDevices] = {nullptr};

thread_local std::string g_noalloc_error;

int fail(const std::string &msg) {
    g_noalloc_error = msg;
    fprintf(stderr, "[cp_al_gb300] %s\n", msg.c_str());
    return -1;
}

} // namespace
} // namespace pdal

extern "C" {

int cp_al_gb300_primal_kkt_noalloc(int m, int n, const int *row_ptr, const int *col_ind, const double *vals,
                                   const double *con_lb, const double *con_ub, const double *c, const double *x,
                                   double *out, void *stream) {
    using namespace pdal;
    if (m < 0 || n <= 0) return fail("primal_kkt_noalloc: m must be >= 0 and n > 0");
    if (m > kNoAllocMaxRows)
        return fail("primal_kkt_noalloc: " + std::to_string(m) + " rows exceed the " +
                    std::to_string(kNoAllocMaxRows) + " rows its fixed scratch supports");
    if (!c || !x || !out || (m > 0 && (!row_ptr || !con_lb || !con_ub)))
        return fail("primal_kkt_noalloc: missing device pointer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(std::string("primal_kkt_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail("primal_kkt_noalloc: device ordinal out of range");
    double *scratch = nullptr;
    {
        /* once per device, with that device current: the device address of
         * the scratch array (its host-side name is only a stand-in) */
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_partials);
            if (e != cudaSuccess)
                return fail(std::string("primal_kkt_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_ptr[dev] = static_cast<double *>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    const int nblocks = m > 0 ? (m + kNoAllocRowsPerBlock - 1) / kNoAllocRowsPerBlock : 1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_primal_kkt_partials<<<nblocks, kThreads, 0, s>>>(m, n, row_ptr, col_ind, vals, con_lb, con_ub, c, x, scratch);
    k_primal_kkt_finish<<<1, kThreads, 0, s>>>(nblocks, scratch, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("primal_kkt_noalloc: launch: ") + cudaGetErrorString(e));
    return 0;
}

} // extern "C"
