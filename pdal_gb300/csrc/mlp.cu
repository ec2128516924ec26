/*
 * mlp.cu -- training and inference of the warm-start MLP (include/pdal_learn.h)
 * with the library's own CUDA kernels (sm_103a).
 *
 * The network is small (three layers, width 256) and every step is a few
 * dense products, so the kernels are plain register-tiled SIMT GEMMs
 * (64 x 64 output tile per block, 4 x 4 per thread, FP32 accumulation) with
 * fused bias / ReLU epilogues, plus elementwise backward, Adam and reduction
 * kernels.  The BF16 inference path stores weights and activations in BF16
 * and accumulates in FP32 in the same GEMM.  All reductions run in a fixed
 * order, so a training run is reproducible bit for bit.
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
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

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

int grid1(size_t count) { return (int)std::min<size_t>((count + GT - 1) / GT, 152 * 16); }

template <typename TI, bool TA, bool TB>
void gemm(cudaStream_t s, int M, int N, int K, const TI *A, long long lda, const TI *B, long long ldb, float *C,
          long long ldc, const float *bias, bool relu, bool accumulate) {
    if (M <= 0 || N <= 0) return;
    dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM);
    k_gemm<TI, TA, TB><<<grid, GT, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, relu ? 1 : 0, accumulate ? 1 : 0);
}

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
        if (bf16) {
            m.Pb.ensure(m.np);
            m.Xbb.ensure((size_t)chunk * m.in);
            m.H1b.ensure((size_t)chunk * m.h);
            m.H2b.ensure((size_t)chunk * m.h);
            pdal::k_to_bf16<<<pdal::grid1(m.np), pdal::GT, 0, m.s>>>(m.P.p, m.Pb.p, m.np);
        }
        for (int r0 = 0; r0 < n; r0 += chunk) {
            const int B = std::min(chunk, n - r0);
            PDAL_CUDA(cudaMemcpyAsync(m.Xb.p, X + (size_t)r0 * m.in, (size_t)B * m.in * 4, cudaMemcpyHostToDevice,
                                      m.s));
            if (!bf16) {
                m.forward(B, m.Xb.p);
            } else {
                const __nv_bfloat16 *W1 = m.Pb.p + m.oW1, *W2 = m.Pb.p + m.oW2, *W3 = m.Pb.p + m.oW3;
                const float *b1 = m.P.p + m.ob1, *b2 = m.P.p + m.ob2, *b3 = m.P.p + m.ob3;
                pdal::k_to_bf16<<<pdal::grid1((size_t)B * m.in), pdal::GT, 0, m.s>>>(m.Xb.p, m.Xbb.p,
                                                                                    (size_t)B * m.in);
                pdal::gemm<__nv_bfloat16, false, false>(m.s, B, m.h, m.in, m.Xbb.p, m.in, W1, m.h, m.H1.p, m.h, b1,
                                                        true, false);
                pdal::k_to_bf16<<<pdal::grid1((size_t)B * m.h), pdal::GT, 0, m.s>>>(m.H1.p, m.H1b.p,
                                                                                   (size_t)B * m.h);
                pdal::gemm<__nv_bfloat16, false, false>(m.s, B, m.h, m.h, m.H1b.p, m.h, W2, m.h, m.H2.p, m.h, b2,
                                                        true, false);
                pdal::k_to_bf16<<<pdal::grid1((size_t)B * m.h), pdal::GT, 0, m.s>>>(m.H2.p, m.H2b.p,
                                                                                   (size_t)B * m.h);
                pdal::gemm<__nv_bfloat16, false, false>(m.s, B, m.out, m.h, m.H2b.p, m.h, W3, m.out, m.Yp.p, m.out,
                                                        b3, false, false);
            }
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

const char *pdal_mlp_last_error(void) { return pdal::g_mlp_error.c_str(); }

} // extern "C"
