/*
 * mlp.cu -- training and inference of the warm-start MLP (include/pdal_learn.h)
 * with the library's own CUDA kernels (sm_103a).
 *
 * The network is three layers of width 256.  Training runs in FP32 on
 * register-tiled SIMT GEMMs (64 x 64 output tile per block, 4 x 4 per
 * thread) with fused bias / ReLU epilogues, plus elementwise backward, Adam
 * and reduction kernels.  BF16 inference runs its three products on the
 * tensor cores (mma.sync m16n8k16, FP32 accumulation, k_gemm_bf16_tc), each
 * layer writing the next one's BF16 operand.  All reductions run in a fixed
 * order, so a training run and a prediction are reproducible bit for bit.
 */
#include "../../include/pdal_learn.h"
#include "common.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <random>
#include <string>
#include <vector>

namespace pdal {
namespace {

thread_local std::string g_mlp_error;

constexpr int TM = 64, TN = 64, TK = 16, GT = 256;

__device__ __forceinline__ float to_f(float v) { return v; }

/* C[m, n] = sum_k A(m, k) B(k, n) (+ C) (+ bias[n]) (ReLU); A(m, k) is
 * A[k*lda + m] when TA, else A[m*lda + k]; B(k, n) is B[n*ldb + k] when TB,
 * else B[k*ldb + n]. */
template <typename TI, bool TA, bool TB>
__global__ void __launch_bounds__(GT) k_gemm(int M, int N, int K, const TI *__restrict__ A, long long lda,
                                             const TI *__restrict__ B, long long ldb, float *C, long long ldc,
                                             const float *__restrict__ bias, int relu, int accumulate) {
    __shared__ float As[TK][TM + 4];
    __shared__ float Bs[TK][TN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += TK) {
        for (int e = threadIdx.x; e < TM * TK; e += GT) {
            int mm, kk;
            if (TA) {
                kk = e / TM;
                mm = e % TM;
            } else {
                mm = e / TK;
                kk = e % TK;
            }
            const int gm = m0 + mm, gk = k0 + kk;
            float v = 0.f;
            if (gm < M && gk < K) v = to_f(TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk]);
            As[kk][mm] = v;
        }
        for (int e = threadIdx.x; e < TN * TK; e += GT) {
            int nn, kk;
            if (TB) {
                nn = e / TK;
                kk = e % TK;
            } else {
                kk = e / TN;
                nn = e % TN;
            }
            const int gn = n0 + nn, gk = k0 + kk;
            float v = 0.f;
            if (gn < N && gk < K) v = to_f(TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn]);
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N) continue;
            float v = acc[i][j];
            float *c = C + (size_t)gm * ldc + gn;
            if (accumulate) v += *c;
            if (bias) v += bias[gn];
            if (relu) v = fmaxf(v, 0.f);
            *c = v;
        }
    }
}

/* ---- BF16 inference on the tensor cores ------------------------------ */

/* C = A B with A [M][K] and B [K][N] in BF16 (row-major, leading dimensions
 * lda, ldb) and FP32 accumulation in mma.sync m16n8k16 tensor-core
 * instructions.  Block tile 64 x 64 x 32 (four warps of 32 x 32), operands
 * staged in shared memory by cp.async in two buffers and fed to the tensor
 * cores by ldmatrix (B transposed on the fly, so both operands stay in their
 * row-major storage).  Split-K: block z sums k in [z*kchunk, (z+1)*kchunk)
 * into slice z of `part` ([gridDim.z][M][N]); k_tc_finish adds the slices in
 * order, so the result does not depend on the split's timing. */
constexpr int TCM = 64, TCN = 64, TCK = 32, TCT = 128;

__device__ __forceinline__ uint32_t tc_smem(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(tc_smem(p)));
}
__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(tc_smem(p)));
}
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc_smem(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

struct TcSmem {
    __nv_bfloat16 a[2][TCM][TCK + 8]; /* rows of 80 bytes: ldmatrix rows fall in distinct banks */
    __nv_bfloat16 b[2][TCK][TCN + 8]; /* rows of 144 bytes */
};

/* Stages the 64 x 32 tile of A at (m0, k) and the 32 x 64 tile of B at
 * (k, n0); 16-byte copies where a whole aligned chunk is inside the matrix,
 * element by element (zero outside) elsewhere. */
__device__ __forceinline__ void tc_stage(TcSmem &sm, int buf, int M, int N, int kend, int m0, int n0, int k,
                                         const __nv_bfloat16 *__restrict__ A, long long lda,
                                         const __nv_bfloat16 *__restrict__ B, long long ldb, bool avec, bool bvec) {
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int idx = threadIdx.x; idx < TCM * TCK / 8; idx += TCT) {
        const int r = idx / (TCK / 8), c = (idx % (TCK / 8)) * 8;
        const int gm = m0 + r, gk = k + c;
        __nv_bfloat16 *dst = &sm.a[buf][r][c];
        if (avec && gm < M && gk + 8 <= kend) {
            cp_async16(dst, A + (size_t)gm * lda + gk);
        } else {
            for (int q = 0; q < 8; ++q) dst[q] = (gm < M && gk + q < kend) ? A[(size_t)gm * lda + gk + q] : zero;
        }
    }
    for (int idx = threadIdx.x; idx < TCK * TCN / 8; idx += TCT) {
        const int r = idx / (TCN / 8), c = (idx % (TCN / 8)) * 8;
        const int gk = k + r, gn = n0 + c;
        __nv_bfloat16 *dst = &sm.b[buf][r][c];
        if (bvec && gk < kend && gn + 8 <= N) {
            cp_async16(dst, B + (size_t)gk * ldb + gn);
        } else {
            for (int q = 0; q < 8; ++q) dst[q] = (gk < kend && gn + q < N) ? B[(size_t)gk * ldb + gn + q] : zero;
        }
    }
}

__global__ void __launch_bounds__(TCT) k_gemm_bf16_tc(int M, int N, int K, int kchunk,
                                                      const __nv_bfloat16 *__restrict__ A, long long lda,
                                                      const __nv_bfloat16 *__restrict__ B, long long ldb,
                                                      float *part) {
    __shared__ __align__(128) TcSmem sm;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int m0 = blockIdx.y * TCM, n0 = blockIdx.x * TCN;
    const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
    /* 16-byte copies need 16-byte aligned rows */
    const bool avec = (lda % 8) == 0 && ((uintptr_t)A % 16) == 0;
    const bool bvec = (ldb % 8) == 0 && ((uintptr_t)B % 16) == 0;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
    const int ntiles = kend > kbeg ? (kend - kbeg + TCK - 1) / TCK : 0;
    if (ntiles > 0) tc_stage(sm, 0, M, N, kend, m0, n0, kbeg, A, lda, B, ldb, avec, bvec);
    cp_async_commit();
    for (int t = 0; t < ntiles; ++t) {
        const int buf = t & 1;
        if (t + 1 < ntiles) tc_stage(sm, buf ^ 1, M, N, kend, m0, n0, kbeg + (t + 1) * TCK, A, lda, B, ldb, avec, bvec);
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < TCK; ks += 16) {
            uint32_t af[2][4], bfr[2][4];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi) ldsm_x4(af[mi], &sm.a[buf][wm + mi * 16 + (lane & 15)][ks + (lane >> 4) * 8]);
#pragma unroll
            for (int nj = 0; nj < 2; ++nj)
                ldsm_x4_trans(bfr[nj], &sm.b[buf][ks + (lane & 15)][wn + nj * 16 + (lane >> 4) * 8]);
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt)
                    mma_bf16_16816(acc[mi][nt], af[mi], bfr[nt >> 1][(nt & 1) * 2], bfr[nt >> 1][(nt & 1) * 2 + 1]);
        }
        __syncthreads();
    }
    cp_async_wait<0>();
    float *out = part + (size_t)blockIdx.z * M * N;
    const int g = lane >> 2, tq = lane & 3;
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = m0 + wm + mi * 16 + g + (q >> 1) * 8, c = n0 + wn + nt * 8 + tq * 2 + (q & 1);
                if (r < M && c < N) out[(size_t)r * N + c] = acc[mi][nt][q];
            }
}

/* C[m][n] = sum over slices z (in order) of part[z][m][n], + bias[n], ReLU;
 * written in FP32 to C and, when Cb is given, in BF16 to Cb (the next
 * layer's input) */
__global__ void k_tc_finish(const float *__restrict__ part, int Z, int M, int N, const float *__restrict__ bias,
                            int relu, float *C, __nv_bfloat16 *Cb) {
    const size_t total = (size_t)M * N;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        for (int z = 0; z < Z; ++z) v += part[(size_t)z * total + t];
        if (bias) v += bias[t % N];
        if (relu) v = fmaxf(v, 0.f);
        if (C) C[t] = v;
        if (Cb) Cb[t] = __float2bfloat16(v);
    }
}

__global__ void k_gather_rows(float *dst, const float *__restrict__ src, const int *__restrict__ idx, int rows,
                              long long cols) {
    const size_t total = (size_t)rows * cols;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t r = t / cols, c = t % cols;
        dst[t] = src[(size_t)idx[r] * cols + c];
    }
}

/* db[n] = sum over rows of dY[:, n] (fixed row order) */
__global__ void k_colsum(const float *__restrict__ dY, int M, int N, float *db) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += dY[(size_t)m * N + n];
    db[n] = s;
}

__global__ void k_relu_bwd(float *dH, const float *__restrict__ H, size_t count) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        if (!(H[t] > 0.f)) dH[t] = 0.f;
}

/* dP = scale * (P - Y); per-block partial sums of (P - Y)^2 in FP64 */
__global__ void __launch_bounds__(GT) k_mse(const float *__restrict__ P, const float *__restrict__ Y, float *dP,
                                            size_t count, float scale, double *part) {
    __shared__ double sb[GT / 32];
    double s = 0.0;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x) {
        const float d = P[t] - Y[t];
        if (dP) dP[t] = scale * d;
        s += (double)d * (double)d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < GT / 32; ++w) t += sb[w];
        part[blockIdx.x] = t;
    }
}

__global__ void k_adam(float *p, const float *__restrict__ g, float *m, float *v, size_t count, float lr, float b1,
                       float b2, float eps, float bc1, float bc2) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[t];
        const float mi = b1 * m[t] + (1.f - b1) * gi;
        const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
        m[t] = mi;
        v[t] = vi;
        p[t] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

__global__ void k_to_bf16(const float *__restrict__ src, __nv_bfloat16 *dst, size_t count) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        dst[t] = __float2bfloat16(src[t]);
}

/* ---- the transportation family on the device --------------------------- */

/* standardised network input of B instances (FP64 arithmetic, rounded once
 * to FP32) */
__global__ void k_tr_features(int B, int S, int D, const double *__restrict__ c, const double *__restrict__ cap,
                              const double *__restrict__ b, const double *__restrict__ xm,
                              const double *__restrict__ xs, float *X) {
    const long long n = (long long)S * D, m = S + D, in = 2 * n + m;
    const long long total = (long long)B * in;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long r = t / in, f = t % in;
        double v;
        if (f < n)
            v = c[r * n + f] / 100.0;
        else if (f < 2 * n)
            v = cap[r * n + f - n] / 200.0;
        else
            v = b[r * m + f - 2 * n] / 100.0;
        X[t] = (float)(__dsub_rn(v, xm[f]) / xs[f]);
    }
}

/* t = T * ys + ym (two roundings, no fused multiply-add), then the warm
 * start it encodes */
__global__ void k_tr_decode(int B, int S, int D, const float *__restrict__ T, const double *__restrict__ ym,
                            const double *__restrict__ ys, const double *__restrict__ cap, double *x, double *y,
                            double *sigma) {
    const long long n = (long long)S * D, m = S + D, out = n + m + 1;
    const long long total = (long long)B * out;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long r = t / out, f = t % out;
        const double v = __dadd_rn(__dmul_rn((double)T[t], ys[f]), ym[f]);
        if (f < n)
            x[r * n + f] = fmin(fmax(v, 0.0), 1.0) * cap[r * n + f];
        else if (f < n + m)
            y[r * m + f - n] = v * 100.0;
        else
            sigma[r] = exp(v);
    }
}

__device__ __forceinline__ double tr_block_sum(double v, double *sb) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sb[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sb[i];
    return t;
}

/* relative KKT error of (x, y) per instance, one block each (cold: x = y = 0) */
__global__ void __launch_bounds__(GT) k_tr_kkt(int S, int D, const double *__restrict__ x,
                                               const double *__restrict__ y, const double *__restrict__ c,
                                               const double *__restrict__ cap, const double *__restrict__ b,
                                               int cold, double *kkt) {
    __shared__ double sb[GT / 32];
    const long long n = (long long)S * D, m = S + D, r = blockIdx.x;
    const double *xr = x ? x + r * n : nullptr, *yr = y ? y + r * m : nullptr;
    const double *cr = c + r * n, *ur = cap + r * n, *br = b + r * m;
    double pobj = 0.0, dterm = 0.0, res2 = 0.0, b2 = 0.0, by = 0.0;
    for (long long a = threadIdx.x; a < n; a += blockDim.x) {
        const double xa = cold ? 0.0 : fmin(fmax(xr[a], 0.0), ur[a]);
        const int i = (int)(a / D), j = (int)(a % D);
        const double rc = cold ? cr[a] : cr[a] - yr[i] - yr[S + j];
        pobj += cr[a] * xa;
        dterm += fmin(rc, 0.0) * ur[a];
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double s = 0.0;
        if (!cold) {
            if (i < S)
                for (int j = 0; j < D; ++j) s += fmin(fmax(xr[(long long)i * D + j], 0.0), ur[(long long)i * D + j]);
            else
                for (int q = 0; q < S; ++q) {
                    const long long a = (long long)q * D + (i - S);
                    s += fmin(fmax(xr[a], 0.0), ur[a]);
                }
        }
        const double ri = s - br[i];
        res2 += ri * ri;
        b2 += br[i] * br[i];
        by += cold ? 0.0 : br[i] * yr[i];
    }
    pobj = tr_block_sum(pobj, sb);
    dterm = tr_block_sum(dterm, sb);
    res2 = tr_block_sum(res2, sb);
    b2 = tr_block_sum(b2, sb);
    by = tr_block_sum(by, sb);
    if (threadIdx.x == 0) {
        const double dobj = by + dterm;
        const double rel_p = sqrt(res2) / (1.0 + sqrt(b2));
        const double gap = fabs(pobj - dobj) / (1.0 + fabs(pobj) + fabs(dobj));
        kkt[r] = fmax(rel_p, gap);
    }
}

int grid1(size_t count) { return (int)std::min<size_t>((count + GT - 1) / GT, 152 * 16); }

template <typename TI, bool TA, bool TB>
void gemm(cudaStream_t s, int M, int N, int K, const TI *A, long long lda, const TI *B, long long ldb, float *C,
          long long ldc, const float *bias, bool relu, bool accumulate) {
    if (M <= 0 || N <= 0) return;
    dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM);
    k_gemm<TI, TA, TB><<<grid, GT, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu ? 1 : 0, accumulate ? 1 : 0);
}

template <typename T>
struct DevBuf;

/* the tensor-core product of one BF16 layer: split-K when the output tiles
 * alone would not fill two waves of the GPU's SMs */
void gemm_tc(cudaStream_t s, int M, int N, int K, const __nv_bfloat16 *A, long long lda, const __nv_bfloat16 *B,
             long long ldb, float *C, __nv_bfloat16 *Cb, const float *bias, bool relu, DevBuf<float> &part);

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    void ensure(size_t count) {
        if (count <= n) return;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        PDAL_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(count, 1)));
        n = count;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

void gemm_tc(cudaStream_t s, int M, int N, int K, const __nv_bfloat16 *A, long long lda, const __nv_bfloat16 *B,
             long long ldb, float *C, __nv_bfloat16 *Cb, const float *bias, bool relu, DevBuf<float> &part) {
    if (M <= 0 || N <= 0) return;
    int dev = 0, sms = 0;
    PDAL_CUDA(cudaGetDevice(&dev));
    PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long tiles = (long long)((N + TCN - 1) / TCN) * ((M + TCM - 1) / TCM);
    int Z = 1;
    if (tiles < 2LL * sms) Z = (int)std::min<long long>((2LL * sms + tiles - 1) / tiles, std::max(1, K / 512));
    int kchunk = (K + Z - 1) / Z;
    kchunk = (kchunk + TCK - 1) / TCK * TCK;
    Z = std::max(1, (K + kchunk - 1) / kchunk);
    part.ensure((size_t)Z * M * N);
    dim3 grid((N + TCN - 1) / TCN, (M + TCM - 1) / TCM, Z);
    k_gemm_bf16_tc<<<grid, TCT, 0, s>>>(M, N, K, kchunk, A, lda, B, ldb, part.p);
    k_tc_finish<<<grid1((size_t)M * N), GT, 0, s>>>(part.p, Z, M, N, bias, relu ? 1 : 0, C, Cb);
}

} // namespace

struct Mlp {
    int in, h, out, device;
    size_t oW1, ob1, oW2, ob2, oW3, ob3, np;
    cudaStream_t s = nullptr;
    DevBuf<float> P, G, Ma, Va;
    DevBuf<float> Xb, Yb, H1, H2, Yp, dY, dH1, dH2;
    DevBuf<int> idx;
    DevBuf<double> part;
    DevBuf<float> Xd, Yd;
    DevBuf<__nv_bfloat16> Pb, Xbb, H1b, H2b;
    DevBuf<float> Tp; /* split-K slices of the tensor-core products */
    int ndata = 0;
    long long adam_t = 0;

    Mlp(int in_, int h_, int out_, unsigned seed, int dev) : in(in_), h(h_), out(out_), device(dev) {
        if (device >= 0) PDAL_CUDA(cudaSetDevice(device));
        oW1 = 0;
        ob1 = oW1 + (size_t)in * h;
        oW2 = ob1 + h;
        ob2 = oW2 + (size_t)h * h;
        oW3 = ob2 + h;
        ob3 = oW3 + (size_t)h * out;
        np = ob3 + out;
        PDAL_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        P.ensure(np);
        G.ensure(np);
        Ma.ensure(np);
        Va.ensure(np);
        std::vector<float> init(np, 0.f);
        std::mt19937 gen(seed);
        auto fill = [&](size_t off, size_t count, int fan_in) {
            const float a = std::sqrt(6.0f / (float)fan_in);
            std::uniform_real_distribution<float> U(-a, a);
            for (size_t i = 0; i < count; ++i) init[off + i] = U(gen);
        };
        fill(oW1, (size_t)in * h, in);
        fill(oW2, (size_t)h * h, h);
        fill(oW3, (size_t)h * out, h);
        PDAL_CUDA(cudaMemcpy(P.p, init.data(), np * 4, cudaMemcpyHostToDevice));
        PDAL_CUDA(cudaMemset(Ma.p, 0, np * 4));
        PDAL_CUDA(cudaMemset(Va.p, 0, np * 4));
    }
    ~Mlp() {
        if (s) cudaStreamDestroy(s);
    }

    void buffers(int B) {
        Xb.ensure((size_t)B * in);
        Yb.ensure((size_t)B * out);
        H1.ensure((size_t)B * h);
        H2.ensure((size_t)B * h);
        Yp.ensure((size_t)B * out);
        dY.ensure((size_t)B * out);
        dH1.ensure((size_t)B * h);
        dH2.ensure((size_t)B * h);
        part.ensure((size_t)152 * 16);
    }

    /* inference of B rows of X (device, FP32) into Yp: FP32 SIMT, or BF16
     * operands on the tensor cores (the weights' BF16 copy made by
     * prepare_bf16) */
    void prepare_bf16(int chunk) {
        Pb.ensure(np);
        Xbb.ensure((size_t)chunk * in);
        H1b.ensure((size_t)chunk * h);
        H2b.ensure((size_t)chunk * h);
        k_to_bf16<<<grid1(np), GT, 0, s>>>(P.p, Pb.p, np);
    }
    void infer(int B, const float *X, bool bf16) {
        if (!bf16) {
            forward(B, X);
            return;
        }
        const __nv_bfloat16 *W1 = Pb.p + oW1, *W2 = Pb.p + oW2, *W3 = Pb.p + oW3;
        const float *b1 = P.p + ob1, *b2 = P.p + ob2, *b3 = P.p + ob3;
        k_to_bf16<<<grid1((size_t)B * in), GT, 0, s>>>(X, Xbb.p, (size_t)B * in);
        /* each layer's BF16 output is the next layer's tensor-core operand */
        gemm_tc(s, B, h, in, Xbb.p, in, W1, h, nullptr, H1b.p, b1, true, Tp);
        gemm_tc(s, B, h, h, H1b.p, h, W2, h, nullptr, H2b.p, b2, true, Tp);
        gemm_tc(s, B, out, h, H2b.p, h, W3, out, Yp.p, nullptr, b3, false, Tp);
    }

    /* forward of B rows of X (device) into Yp */
    void forward(int B, const float *X) {
        const float *W1 = P.p + oW1, *b1 = P.p + ob1, *W2 = P.p + oW2, *b2 = P.p + ob2, *W3 = P.p + oW3,
                    *b3 = P.p + ob3;
        gemm<float, false, false>(s, B, h, in, X, in, W1, h, H1.p, h, b1, true, false);
        gemm<float, false, false>(s, B, h, h, H1.p, h, W2, h, H2.p, h, b2, true, false);
        gemm<float, false, false>(s, B, out, h, H2.p, h, W3, out, Yp.p, out, b3, false, false);
    }

    /* loss of B rows against Y (device); gradient into G when grad */
    double loss_backward(int B, const float *X, const float *Y, bool grad) {
        const size_t cnt = (size_t)B * out;
        const int g = grid1(cnt);
        k_mse<<<g, GT, 0, s>>>(Yp.p, Y, grad ? dY.p : nullptr, cnt, 2.0f / (float)cnt, part.p);
        std::vector<double> hp(g);
        if (grad) {
            const float *W2 = P.p + oW2, *W3 = P.p + oW3;
            /* layer 3 */
            gemm<float, true, false>(s, h, out, B, H2.p, h, dY.p, out, G.p + oW3, out, nullptr, false, false);
            k_colsum<<<(out + GT - 1) / GT, GT, 0, s>>>(dY.p, B, out, G.p + ob3);
            gemm<float, false, true>(s, B, h, out, dY.p, out, W3, out, dH2.p, h, nullptr, false, false);
            k_relu_bwd<<<grid1((size_t)B * h), GT, 0, s>>>(dH2.p, H2.p, (size_t)B * h);
            /* layer 2 */
            gemm<float, true, false>(s, h, h, B, H1.p, h, dH2.p, h, G.p + oW2, h, nullptr, false, false);
            k_colsum<<<(h + GT - 1) / GT, GT, 0, s>>>(dH2.p, B, h, G.p + ob2);
            gemm<float, false, true>(s, B, h, h, dH2.p, h, W2, h, dH1.p, h, nullptr, false, false);
            k_relu_bwd<<<grid1((size_t)B * h), GT, 0, s>>>(dH1.p, H1.p, (size_t)B * h);
            /* layer 1 */
            gemm<float, true, false>(s, in, h, B, X, in, dH1.p, h, G.p + oW1, h, nullptr, false, false);
            k_colsum<<<(h + GT - 1) / GT, GT, 0, s>>>(dH1.p, B, h, G.p + ob1);
        }
        PDAL_CUDA(cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * g, cudaMemcpyDeviceToHost, s));
        PDAL_CUDA(cudaStreamSynchronize(s));
        PDAL_CUDA(cudaGetLastError());
        double t = 0.0;
        for (double v : hp) t += v;
        return t / (double)cnt;
    }
};

} // namespace pdal

struct pdal_mlp {
    pdal::Mlp *m;
};

namespace {
int fail(const std::string &msg) {
    pdal::g_mlp_error = msg;
    fprintf(stderr, "[pdal_learn] %s\n", msg.c_str());
    return -1;
}
} // namespace

extern "C" {

pdal_mlp_t *pdal_mlp_create(int in, int hidden, int out, unsigned seed, int device) {
    if (in <= 0 || hidden <= 0 || out <= 0) {
        fail("pdal_mlp_create: dimensions must be positive");
        return nullptr;
    }
    try {
        pdal_mlp_t *h = new pdal_mlp_t;
        h->m = new pdal::Mlp(in, hidden, out, seed, device);
        return h;
    } catch (const std::exception &e) {
        fail(e.what());
        return nullptr;
    }
}

void pdal_mlp_free(pdal_mlp_t *h) {
    if (!h) return;
    delete h->m;
    delete h;
}

long long pdal_mlp_num_params(const pdal_mlp_t *h) { return h ? (long long)h->m->np : -1; }

int pdal_mlp_get_params(const pdal_mlp_t *h, float *params) {
    if (!h || !params) return fail("pdal_mlp_get_params: NULL argument");
    try {
        PDAL_CUDA(cudaMemcpy(params, h->m->P.p, h->m->np * 4, cudaMemcpyDeviceToHost));
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

int pdal_mlp_set_params(pdal_mlp_t *h, const float *params) {
    if (!h || !params) return fail("pdal_mlp_set_params: NULL argument");
    try {
        PDAL_CUDA(cudaMemcpy(h->m->P.p, params, h->m->np * 4, cudaMemcpyHostToDevice));
        PDAL_CUDA(cudaMemset(h->m->Ma.p, 0, h->m->np * 4));
        PDAL_CUDA(cudaMemset(h->m->Va.p, 0, h->m->np * 4));
        h->m->adam_t = 0;
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

int pdal_mlp_set_data(pdal_mlp_t *h, int n, const float *X, const float *Y) {
    if (!h || n <= 0 || !X || !Y) return fail("pdal_mlp_set_data: invalid arguments");
    try {
        pdal::Mlp &m = *h->m;
        m.Xd.ensure((size_t)n * m.in);
        m.Yd.ensure((size_t)n * m.out);
        PDAL_CUDA(cudaMemcpy(m.Xd.p, X, (size_t)n * m.in * 4, cudaMemcpyHostToDevice));
        PDAL_CUDA(cudaMemcpy(m.Yd.p, Y, (size_t)n * m.out * 4, cudaMemcpyHostToDevice));
        m.ndata = n;
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

double pdal_mlp_train(pdal_mlp_t *h, int epochs, int batch, float lr, unsigned seed) {
    if (!h || epochs <= 0 || batch <= 0 || h->m->ndata <= 0) return fail("pdal_mlp_train: invalid arguments");
    try {
        pdal::Mlp &m = *h->m;
        const int n = m.ndata;
        const int B = std::min(batch, n);
        m.buffers(B);
        m.idx.ensure(n);
        std::vector<int> perm(n);
        std::iota(perm.begin(), perm.end(), 0);
        std::mt19937 gen(seed);
        double last = 0.0;
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        for (int ep = 0; ep < epochs; ++ep) {
            std::shuffle(perm.begin(), perm.end(), gen);
            PDAL_CUDA(cudaMemcpyAsync(m.idx.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m.s));
            double sum = 0.0;
            int batches = 0;
            for (int b0 = 0; b0 + B <= n; b0 += B) {
                pdal::k_gather_rows<<<pdal::grid1((size_t)B * m.in), pdal::GT, 0, m.s>>>(m.Xb.p, m.Xd.p, m.idx.p + b0,
                                                                                        B, m.in);
                pdal::k_gather_rows<<<pdal::grid1((size_t)B * m.out), pdal::GT, 0, m.s>>>(
                    m.Yb.p, m.Yd.p, m.idx.p + b0, B, m.out);
                m.forward(B, m.Xb.p);
                sum += m.loss_backward(B, m.Xb.p, m.Yb.p, true);
                ++batches;
                ++m.adam_t;
                const float bc1 = 1.f - std::pow(b1, (float)m.adam_t), bc2 = 1.f - std::pow(b2, (float)m.adam_t);
                pdal::k_adam<<<pdal::grid1(m.np), pdal::GT, 0, m.s>>>(m.P.p, m.G.p, m.Ma.p, m.Va.p, m.np, lr, b1, b2,
                                                                      eps, bc1, bc2);
            }
            last = batches ? sum / batches : 0.0;
        }
        PDAL_CUDA(cudaStreamSynchronize(m.s));
        PDAL_CUDA(cudaGetLastError());
        return last;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

double pdal_mlp_loss_grad(pdal_mlp_t *h, int n, const float *X, const float *Y, float *grad) {
    if (!h || n <= 0 || !X || !Y) return fail("pdal_mlp_loss_grad: invalid arguments");
    try {
        pdal::Mlp &m = *h->m;
        m.buffers(n);
        PDAL_CUDA(cudaMemcpyAsync(m.Xb.p, X, (size_t)n * m.in * 4, cudaMemcpyHostToDevice, m.s));
        PDAL_CUDA(cudaMemcpyAsync(m.Yb.p, Y, (size_t)n * m.out * 4, cudaMemcpyHostToDevice, m.s));
        m.forward(n, m.Xb.p);
        const double loss = m.loss_backward(n, m.Xb.p, m.Yb.p, grad != nullptr);
        if (grad) PDAL_CUDA(cudaMemcpy(grad, m.G.p, m.np * 4, cudaMemcpyDeviceToHost));
        return loss;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

int pdal_mlp_predict(pdal_mlp_t *h, int n, const float *X, float *Y, int bf16) {
    if (!h || n <= 0 || !X || !Y) return fail("pdal_mlp_predict: invalid arguments");
    try {
        pdal::Mlp &m = *h->m;
        const int chunk = std::min(n, 1024);
        m.buffers(chunk);
        if (bf16) m.prepare_bf16(chunk);
        for (int r0 = 0; r0 < n; r0 += chunk) {
            const int B = std::min(chunk, n - r0);
            PDAL_CUDA(cudaMemcpyAsync(m.Xb.p, X + (size_t)r0 * m.in, (size_t)B * m.in * 4, cudaMemcpyHostToDevice,
                                      m.s));
            m.infer(B, m.Xb.p, bf16 != 0);
            PDAL_CUDA(cudaMemcpyAsync(Y + (size_t)r0 * m.out, m.Yp.p, (size_t)B * m.out * 4, cudaMemcpyDeviceToHost,
                                      m.s));
        }
        PDAL_CUDA(cudaStreamSynchronize(m.s));
        PDAL_CUDA(cudaGetLastError());
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

int pdal_transport_warm_start(pdal_mlp_t *h, int S, int D, int count, const double *costs, const double *caps,
                              const double *rhs, const double *xm, const double *xs, const double *ym,
                              const double *ys, int bf16, double *x, double *y, double *sigma, double *kkt_pred,
                              double *kkt_cold) {
    if (!h || S <= 0 || D <= 0 || count <= 0 || !costs || !caps || !rhs || !xm || !xs || !ym || !ys || !x || !y ||
        !sigma || !kkt_pred || !kkt_cold)
        return fail("pdal_transport_warm_start: invalid arguments");
    try {
        pdal::Mlp &m = *h->m;
        const long long n = (long long)S * D, mm = S + D;
        if (m.in != 2 * n + mm || m.out != n + mm + 1)
            return fail("pdal_transport_warm_start: the network's sizes do not match the S x D family");
        const int chunk = std::min(count, 1024);
        m.buffers(chunk);
        if (bf16) m.prepare_bf16(chunk);
        pdal::DevBuf<double> dc, du, db, dx, dy, ds, dk0, dk1, st;
        dc.ensure((size_t)chunk * n);
        du.ensure((size_t)chunk * n);
        db.ensure((size_t)chunk * mm);
        dx.ensure((size_t)chunk * n);
        dy.ensure((size_t)chunk * mm);
        ds.ensure(chunk);
        dk0.ensure(chunk);
        dk1.ensure(chunk);
        st.ensure((size_t)2 * m.in + 2 * m.out);
        double *dxm = st.p, *dxs = st.p + m.in, *dym = st.p + 2 * m.in, *dys = st.p + 2 * m.in + m.out;
        PDAL_CUDA(cudaMemcpyAsync(dxm, xm, sizeof(double) * m.in, cudaMemcpyHostToDevice, m.s));
        PDAL_CUDA(cudaMemcpyAsync(dxs, xs, sizeof(double) * m.in, cudaMemcpyHostToDevice, m.s));
        PDAL_CUDA(cudaMemcpyAsync(dym, ym, sizeof(double) * m.out, cudaMemcpyHostToDevice, m.s));
        PDAL_CUDA(cudaMemcpyAsync(dys, ys, sizeof(double) * m.out, cudaMemcpyHostToDevice, m.s));
        for (int r0 = 0; r0 < count; r0 += chunk) {
            const int B = std::min(chunk, count - r0);
            PDAL_CUDA(cudaMemcpyAsync(dc.p, costs + (size_t)r0 * n, sizeof(double) * B * n, cudaMemcpyHostToDevice,
                                      m.s));
            PDAL_CUDA(cudaMemcpyAsync(du.p, caps + (size_t)r0 * n, sizeof(double) * B * n, cudaMemcpyHostToDevice,
                                      m.s));
            PDAL_CUDA(cudaMemcpyAsync(db.p, rhs + (size_t)r0 * mm, sizeof(double) * B * mm, cudaMemcpyHostToDevice,
                                      m.s));
            pdal::k_tr_features<<<pdal::grid1((size_t)B * m.in), pdal::GT, 0, m.s>>>(B, S, D, dc.p, du.p, db.p, dxm,
                                                                                    dxs, m.Xb.p);
            m.infer(B, m.Xb.p, bf16 != 0);
            pdal::k_tr_decode<<<pdal::grid1((size_t)B * m.out), pdal::GT, 0, m.s>>>(B, S, D, m.Yp.p, dym, dys, du.p,
                                                                                   dx.p, dy.p, ds.p);
            pdal::k_tr_kkt<<<B, pdal::GT, 0, m.s>>>(S, D, dx.p, dy.p, dc.p, du.p, db.p, 0, dk0.p);
            pdal::k_tr_kkt<<<B, pdal::GT, 0, m.s>>>(S, D, nullptr, nullptr, dc.p, du.p, db.p, 1, dk1.p);
            PDAL_CUDA(cudaGetLastError());
            PDAL_CUDA(cudaMemcpyAsync(x + (size_t)r0 * n, dx.p, sizeof(double) * B * n, cudaMemcpyDeviceToHost, m.s));
            PDAL_CUDA(cudaMemcpyAsync(y + (size_t)r0 * mm, dy.p, sizeof(double) * B * mm, cudaMemcpyDeviceToHost,
                                      m.s));
            PDAL_CUDA(cudaMemcpyAsync(sigma + r0, ds.p, sizeof(double) * B, cudaMemcpyDeviceToHost, m.s));
            PDAL_CUDA(cudaMemcpyAsync(kkt_pred + r0, dk0.p, sizeof(double) * B, cudaMemcpyDeviceToHost, m.s));
            PDAL_CUDA(cudaMemcpyAsync(kkt_cold + r0, dk1.p, sizeof(double) * B, cudaMemcpyDeviceToHost, m.s));
            /* the chunk's device buffers are reused by the next chunk */
            PDAL_CUDA(cudaStreamSynchronize(m.s));
        }
        return 0;
    } catch (const std::exception &e) {
        return fail(e.what());
    }
}

const char *pdal_mlp_last_error(void) { return pdal::g_mlp_error.c_str(); }

} // extern "C"
