// mlp.cu -- the learned warm start's network and its training on the GPU.
//
// A per-pair MLP, 40 -> 128 -> 128 -> 16 with ReLU, maps the statistics of a
// locus pair (r, n) to an initial 4 x 4 coupling block J_rn (the inputs are
// built in warmstart.cu).  Every layer, forward and backward, is one launch
// of a tiled FP32 kernel C = op(A) op(B) written here; Adam and the loss are
// elementwise kernels.  The parameter blob (MLP_* offsets in engine.h) holds
// the input normalisation, the weights and the output scale.
//
// SuperDCA has no learned component: its solver starts every locus from
// zero (SuperDCA/include/plmDCA.hpp:298).  The warm start only moves the
// starting point of a strictly convex problem.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels_common.cuh"
#include "superdca_gb300.h"

namespace sdca {
namespace {

constexpr int TM = 64, TN = 64, TK = 16;

// C[M x N] (=, or += with atomics when split along K) op(A)[M x K] . op(B)[K x N]
//   op(A)(m,k) = TA ? A[k*lda + m] : A[m*lda + k]
//   op(B)(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n]
// epilogue: + bias[n], ReLU, or * [mask(m,n) > 0]
template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
k_mm(int M, int N, int K, const float *__restrict__ A, int lda, const float *__restrict__ B, int ldb,
     float *__restrict__ C, int ldc, const float *__restrict__ bias, int relu, const float *__restrict__ mask,
     int k_per_split)
{
    __shared__ float sA[TK][TM + 4];
    __shared__ float sB[TK][TN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int kbeg = blockIdx.z * k_per_split, kend = min(K, kbeg + k_per_split);
    float acc[4][4] = {};
    for (int k0 = kbeg; k0 < kend; k0 += TK) {
        for (int e = threadIdx.x; e < TM * TK; e += 256) {
            int mm, kk;
            if (TA) { mm = e % TM; kk = e / TM; } else { kk = e % TK; mm = e / TK; }
            const int m = m0 + mm, k = k0 + kk;
            float v = 0.f;
            if (m < M && k < kend) v = TA ? A[(int64_t)k * lda + m] : A[(int64_t)m * lda + k];
            sA[kk][mm] = v;
        }
        for (int e = threadIdx.x; e < TN * TK; e += 256) {
            int nn, kk;
            if (TB) { kk = e % TK; nn = e / TK; } else { nn = e % TN; kk = e / TN; }
            const int n = n0 + nn, k = k0 + kk;
            float v = 0.f;
            if (n < N && k < kend) v = TB ? B[(int64_t)n * ldb + k] : B[(int64_t)k * ldb + n];
            sB[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sA[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    const bool split = gridDim.z > 1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n >= N) continue;
            float v = acc[i][j];
            float *c = C + (int64_t)m * ldc + n;
            if (split) {
                atomicAdd(c, v);
                continue;
            }
            if (bias) v += bias[n];
            if (relu) v = fmaxf(v, 0.f);
            if (mask && !(mask[(int64_t)m * ldc + n] > 0.f)) v = 0.f;
            *c = v;
        }
    }
}

template <bool TA, bool TB>
void mm(cudaStream_t st, int M, int N, int K, const float *A, int lda, const float *B, int ldb, float *C, int ldc,
        const float *bias, int relu, const float *mask, int splits = 1)
{
    const int kps = ((K + splits - 1) / splits + TK - 1) / TK * TK;
    splits = (K + kps - 1) / kps;
    // rows in pieces that keep grid.y within its limit (row-major A only)
    const int rows = TA ? M : std::min(M, 65535 * TM);
    for (int m0 = 0; m0 < M; m0 += rows) {
        const int mr = std::min(rows, M - m0);
        dim3 grid((N + TN - 1) / TN, (mr + TM - 1) / TM, splits);
        k_mm<TA, TB><<<grid, 256, 0, st>>>(mr, N, K, A + (TA ? 0 : (int64_t)m0 * lda), lda, B, ldb,
                                           C + (int64_t)m0 * ldc, ldc, bias, relu,
                                           mask ? mask + (int64_t)m0 * ldc : nullptr, kps);
    }
}

// (x - mean) * scale, row-major M x MLP_IN
__global__ void k_normalise(int64_t M, const float *__restrict__ X, const float *__restrict__ p,
                            float *__restrict__ Xn)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M * MLP_IN) return;
    const int c = (int)(t % MLP_IN);
    Xn[t] = (X[t] - p[MLP_IN_MEAN + c]) * p[MLP_IN_SCALE + c];
}

// rows of src picked by idx -> dst
__global__ void k_gather_rows(int64_t M, int width, const int32_t *__restrict__ idx, const float *__restrict__ src,
                              float *__restrict__ dst)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M * width) return;
    const int64_t m = t / width;
    const int c = (int)(t % width);
    dst[t] = src[(int64_t)idx[m] * width + c];
}

// mean squared error over M x MLP_OUT; dOut = 2 (out - t) / M
__global__ void k_mse(int64_t M, const float *__restrict__ out, const float *__restrict__ t, float *__restrict__ dout,
                      double *__restrict__ loss)
{
    double s = 0.0;
    const float inv = 2.f / (float)M;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < M * MLP_OUT;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float r = out[e] - t[e];
        dout[e] = inv * r;
        s += (double)r * r;
    }
    s = warp_sum(s);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) atomicAdd(loss, v / (double)M);
    }
}

// column sums of dC (M x N) into g[n]
__global__ void k_colsum(int64_t M, int N, const float *__restrict__ dC, float *__restrict__ g)
{
    const int n = threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int64_t m = blockIdx.x; m < M; m += gridDim.x) s += dC[m * N + n];
    atomicAdd(g + n, s);
}

__global__ void k_adam(int n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                       float *__restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

struct Dev {
    std::vector<void *> ptrs;
    bool ok = true;
    ~Dev() { for (void *q : ptrs) cudaFree(q); }
    template <typename T> T *alloc(size_t n)
    {
        void *q = nullptr;
        if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
            ok = false;
            return nullptr;
        }
        ptrs.push_back(q);
        return (T *)q;
    }
};

struct Scratch {
    float *h1, *h2, *out;
};

// forward over M normalised rows; activations kept for the backward
void forward(cudaStream_t st, const float *p, const float *Xn, int64_t M, const Scratch &s)
{
    mm<false, true>(st, (int)M, MLP_H, MLP_IN, Xn, MLP_IN, p + MLP_W1, MLP_IN, s.h1, MLP_H, p + MLP_B1, 1, nullptr);
    mm<false, true>(st, (int)M, MLP_H, MLP_H, s.h1, MLP_H, p + MLP_W2, MLP_H, s.h2, MLP_H, p + MLP_B2, 1, nullptr);
    mm<false, true>(st, (int)M, MLP_OUT, MLP_H, s.h2, MLP_H, p + MLP_W3, MLP_H, s.out, MLP_OUT, p + MLP_B3, 0,
                    nullptr);
}

// gradient of the loss whose output gradient is dout (M x MLP_OUT), into g
// (blob layout, zeroed by the caller); d1/d2 are M x MLP_H scratch
void backward(cudaStream_t st, const float *p, const float *Xn, int64_t M, const Scratch &s, const float *dout,
              float *d1, float *d2, float *g)
{
    const int splits = (int)std::min<int64_t>(64, std::max<int64_t>(1, M / 2048));
    const int cs_blocks = (int)std::min<int64_t>(256, std::max<int64_t>(1, M / 64));
    // layer 3
    mm<true, false>(st, MLP_OUT, MLP_H, (int)M, dout, MLP_OUT, s.h2, MLP_H, g + MLP_W3, MLP_H, nullptr, 0, nullptr,
                    splits);
    k_colsum<<<cs_blocks, 128, 0, st>>>(M, MLP_OUT, dout, g + MLP_B3);
    mm<false, false>(st, (int)M, MLP_H, MLP_OUT, dout, MLP_OUT, p + MLP_W3, MLP_H, d2, MLP_H, nullptr, 0, s.h2);
    // layer 2
    mm<true, false>(st, MLP_H, MLP_H, (int)M, d2, MLP_H, s.h1, MLP_H, g + MLP_W2, MLP_H, nullptr, 0, nullptr, splits);
    k_colsum<<<cs_blocks, 128, 0, st>>>(M, MLP_H, d2, g + MLP_B2);
    mm<false, false>(st, (int)M, MLP_H, MLP_H, d2, MLP_H, p + MLP_W2, MLP_H, d1, MLP_H, nullptr, 0, s.h1);
    // layer 1
    mm<true, false>(st, MLP_H, MLP_IN, (int)M, d1, MLP_H, Xn, MLP_IN, g + MLP_W1, MLP_IN, nullptr, 0, nullptr,
                    splits);
    k_colsum<<<cs_blocks, 128, 0, st>>>(M, MLP_H, d1, g + MLP_B1);
}

thread_local std::string t_err;

int mfail(const std::string &m)
{
    t_err = m;
    return SDCA_E_CUDA;
}

#define MK(call)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return mfail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int check_blob(const float *params)
{
    if (!params) return SDCA_E_ARG;
    if (params[MLP_VERSION] != (float)MLP_BLOB_VERSION) return SDCA_E_ARG;
    return SDCA_OK;
}

} // namespace

// inference for the engine: raw features (M x MLP_IN) -> normalised outputs
// (M x MLP_OUT); Xn, h1, h2 are scratch of M x {MLP_IN, MLP_H, MLP_H}
void mlp_infer(const float *p_dev, const float *X, int64_t M, float *Xn, float *h1, float *h2, float *out,
               cudaStream_t st)
{
    if (M <= 0) return;
    k_normalise<<<(unsigned)((M * MLP_IN + 255) / 256), 256, 0, st>>>(M, X, p_dev, Xn);
    forward(st, p_dev, Xn, M, Scratch{h1, h2, out});
}

} // namespace sdca

using namespace sdca;

extern "C" {

int sdca_mlp_blob_size(void) { return MLP_BLOB_SIZE; }

int sdca_mlp_grad(const float *params, const float *X, const float *T, int64_t M, double *loss, float *grad)
{
    if (check_blob(params) || !X || !T || M < 1 || !loss || !grad) return SDCA_E_ARG;
    cudaStream_t st = 0;
    Dev d;
    float *p = d.alloc<float>(MLP_BLOB_SIZE), *x = d.alloc<float>(M * MLP_IN), *xn = d.alloc<float>(M * MLP_IN);
    float *t = d.alloc<float>(M * MLP_OUT), *h1 = d.alloc<float>(M * MLP_H), *h2 = d.alloc<float>(M * MLP_H);
    float *out = d.alloc<float>(M * MLP_OUT), *dout = d.alloc<float>(M * MLP_OUT);
    float *d1 = d.alloc<float>(M * MLP_H), *d2 = d.alloc<float>(M * MLP_H), *g = d.alloc<float>(MLP_BLOB_SIZE);
    double *l = d.alloc<double>(1);
    if (!d.ok) return mfail("device allocation failed"), SDCA_E_NOMEM;
    MK(cudaMemcpy(p, params, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyHostToDevice));
    MK(cudaMemcpy(x, X, sizeof(float) * M * MLP_IN, cudaMemcpyHostToDevice));
    MK(cudaMemcpy(t, T, sizeof(float) * M * MLP_OUT, cudaMemcpyHostToDevice));
    MK(cudaMemset(g, 0, sizeof(float) * MLP_BLOB_SIZE));
    MK(cudaMemset(l, 0, sizeof(double)));
    k_normalise<<<(unsigned)((M * MLP_IN + 255) / 256), 256, 0, st>>>(M, x, p, xn);
    const Scratch s{h1, h2, out};
    forward(st, p, xn, M, s);
    k_mse<<<(unsigned)std::min<int64_t>(1024, (M * MLP_OUT + 255) / 256), 256, 0, st>>>(M, out, t, dout, l);
    backward(st, p, xn, M, s, dout, d1, d2, g);
    MK(cudaGetLastError());
    MK(cudaMemcpy(grad, g, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyDeviceToHost));
    MK(cudaMemcpy(loss, l, sizeof(double), cudaMemcpyDeviceToHost));
    return SDCA_OK;
}

int sdca_mlp_predict(const float *params, const float *X, int64_t M, float *out)
{
    if (check_blob(params) || !X || M < 1 || !out) return SDCA_E_ARG;
    Dev d;
    float *p = d.alloc<float>(MLP_BLOB_SIZE), *x = d.alloc<float>(M * MLP_IN), *xn = d.alloc<float>(M * MLP_IN);
    float *h1 = d.alloc<float>(M * MLP_H), *h2 = d.alloc<float>(M * MLP_H), *o = d.alloc<float>(M * MLP_OUT);
    if (!d.ok) return mfail("device allocation failed"), SDCA_E_NOMEM;
    MK(cudaMemcpy(p, params, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyHostToDevice));
    MK(cudaMemcpy(x, X, sizeof(float) * M * MLP_IN, cudaMemcpyHostToDevice));
    mlp_infer(p, x, M, xn, h1, h2, o, 0);
    MK(cudaGetLastError());
    MK(cudaMemcpy(out, o, sizeof(float) * M * MLP_OUT, cudaMemcpyDeviceToHost));
    return SDCA_OK;
}

int sdca_mlp_train(float *params, const float *X, const float *T, int64_t M, int epochs, int batch, float lr,
                   uint64_t seed, double *losses)
{
    if (check_blob(params) || !X || !T || M < 1 || epochs < 1 || batch < 1 || !(lr > 0.f)) return SDCA_E_ARG;
    cudaStream_t st = 0;
    const int64_t Bm = std::min<int64_t>(batch, M);
    Dev d;
    float *p = d.alloc<float>(MLP_BLOB_SIZE), *x = d.alloc<float>(M * MLP_IN), *xn = d.alloc<float>(M * MLP_IN);
    float *t = d.alloc<float>(M * MLP_OUT);
    float *bx = d.alloc<float>(Bm * MLP_IN), *bt = d.alloc<float>(Bm * MLP_OUT);
    float *h1 = d.alloc<float>(Bm * MLP_H), *h2 = d.alloc<float>(Bm * MLP_H), *out = d.alloc<float>(Bm * MLP_OUT);
    float *dout = d.alloc<float>(Bm * MLP_OUT), *d1 = d.alloc<float>(Bm * MLP_H), *d2 = d.alloc<float>(Bm * MLP_H);
    float *g = d.alloc<float>(MLP_BLOB_SIZE), *m1 = d.alloc<float>(MLP_BLOB_SIZE), *m2 = d.alloc<float>(MLP_BLOB_SIZE);
    int32_t *perm_d = d.alloc<int32_t>(M);
    double *l = d.alloc<double>(1);
    if (!d.ok) return mfail("device allocation failed"), SDCA_E_NOMEM;
    MK(cudaMemcpy(p, params, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyHostToDevice));
    MK(cudaMemcpy(x, X, sizeof(float) * M * MLP_IN, cudaMemcpyHostToDevice));
    MK(cudaMemcpy(t, T, sizeof(float) * M * MLP_OUT, cudaMemcpyHostToDevice));
    MK(cudaMemset(m1, 0, sizeof(float) * MLP_BLOB_SIZE));
    MK(cudaMemset(m2, 0, sizeof(float) * MLP_BLOB_SIZE));
    k_normalise<<<(unsigned)((M * MLP_IN + 255) / 256), 256, 0, st>>>(M, x, p, xn);
    std::mt19937_64 rng(seed);
    std::vector<int32_t> perm((size_t)M);
    const float b1 = 0.9f, b2 = 0.999f;
    float c1 = 1.f, c2 = 1.f;
    const Scratch s{h1, h2, out};
    for (int ep = 0; ep < epochs; ++ep) {
        for (int64_t i = 0; i < M; ++i) perm[i] = (int32_t)i;
        std::shuffle(perm.begin(), perm.end(), rng);
        MK(cudaMemcpy(perm_d, perm.data(), sizeof(int32_t) * M, cudaMemcpyHostToDevice));
        MK(cudaMemset(l, 0, sizeof(double)));
        int64_t nb = 0;
        for (int64_t b0 = 0; b0 + Bm <= M; b0 += Bm, ++nb) {
            k_gather_rows<<<(unsigned)((Bm * MLP_IN + 255) / 256), 256, 0, st>>>(Bm, MLP_IN, perm_d + b0, xn, bx);
            k_gather_rows<<<(unsigned)((Bm * MLP_OUT + 255) / 256), 256, 0, st>>>(Bm, MLP_OUT, perm_d + b0, t, bt);
            forward(st, p, bx, Bm, s);
            k_mse<<<(unsigned)std::min<int64_t>(1024, (Bm * MLP_OUT + 255) / 256), 256, 0, st>>>(Bm, out, bt, dout, l);
            MK(cudaMemsetAsync(g, 0, sizeof(float) * MLP_BLOB_SIZE, st));
            backward(st, p, bx, Bm, s, dout, d1, d2, g);
            c1 *= b1;
            c2 *= b2;
            k_adam<<<(MLP_TRAIN_END - MLP_W1 + 255) / 256, 256, 0, st>>>(MLP_TRAIN_END - MLP_W1, p + MLP_W1,
                                                                       g + MLP_W1, m1 + MLP_W1, m2 + MLP_W1, lr,
                                                                       b1, b2, 1e-8f, 1.f - c1, 1.f - c2);
        }
        MK(cudaGetLastError());
        double lsum = 0.0;
        MK(cudaMemcpy(&lsum, l, sizeof(double), cudaMemcpyDeviceToHost));
        if (losses) losses[ep] = nb ? lsum / (double)nb : 0.0;
    }
    MK(cudaMemcpy(params, p, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyDeviceToHost));
    return SDCA_OK;
}

const char *sdca_mlp_last_error(void) { return t_err.c_str(); }

} // extern "C"
