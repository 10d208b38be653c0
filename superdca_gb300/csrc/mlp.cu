// mlp.cu -- the learned warm start's network and its training on the GPU.
//
// An MLP, 40 -> 128 -> 128 -> 16 with ReLU, maps the statistics of a locus
// pair (r, n), or of one sequence at a target column (the dual form's start),
// to a starting point (the inputs are built in warmstart.cu).
//
// Inference, and the forward pass of training, is one fused tcgen05 kernel
// (k_mlp_tc): BF16 weights and activations, FP32 accumulators in TMEM, all
// three layers of a 128-row tile without leaving the SM.  The backward pass
// is tiled FP32 kernels C = op(A) op(B) on the FP32 master weights from the
// saved FP32 activations (mixed-precision training); Adam and the loss are
// elementwise kernels.  sdca_mlp_grad takes the FP32 forward, the exact
// derivative the CPU oracle checks.  The parameter blob (MLP_* offsets in
// engine.h) holds the input normalisation, the FP32 weights and the output
// scale; the BF16 weight image is made from it (k_mlp_pack).
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
#include <cuda_bf16.h>

#include "kernels_common.cuh"
#include "superdca_gb300.h"
#include "tcgen05.cuh"

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

// ---- the fused tensor-core forward (BF16 weights, FP32 accumulators)
//
// One CTA of 128 threads owns the three BF16 weight matrices in shared
// memory (128-byte swizzled K-major tiles: W1 128 x 64 with the 40 inputs
// zero-padded, W2 128 x 128 as two 64-column atoms, W3 16 x 128 likewise)
// and walks 128-row tiles of the input.  Per tile: thread r normalises row
// r, rounds it to BF16 into the A tile; one thread issues the layer's
// tcgen05.mma (M128, K16 steps) into TMEM and commits to an mbarrier; every
// thread reads its row's accumulators back (tcgen05.ld, TMEM lane = row),
// adds the bias, applies ReLU and writes the next layer's BF16 A tile.
// Layer 3 (N = 16) writes the outputs.  h1, h2 (optional) receive the FP32
// activations for the backward pass.
constexpr int MT_THREADS = 128;
constexpr int MT_K1 = 64;                                       // layer-1 K, padded
constexpr int MT_W1_ELEMS = MLP_H * MT_K1, MT_W2_ELEMS = MLP_H * MLP_H, MT_W3_ELEMS = MLP_OUT * MLP_H;
constexpr int MT_WB_ELEMS = MT_W1_ELEMS + MT_W2_ELEMS + MT_W3_ELEMS;   // BF16 weight image
constexpr uint32_t MT_SW1 = 0, MT_SW2 = 16384, MT_SW3 = 49152, MT_SA1 = 53248, MT_SA2 = 69632;
constexpr uint32_t MT_SBAR = 102400;
constexpr int MT_SMEM = (int)MT_SBAR + 64 + 1024;
constexpr uint32_t MT_TMEM_COLS = 256;                          // layer 1/3 at 0, layer 2 at 128
// kind::f16 instruction descriptor: D = F32, A = B = BF16, K-major, M = 128
constexpr uint32_t mt_idesc(int n) { return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | (8u << 24); }
static_assert(MLP_IN <= MT_K1 && MLP_H == 128 && MLP_OUT == 16, "tile shapes of k_mlp_tc");
static_assert(MT_WB_ELEMS == MLP_WB_ELEMS, "weight image size");
static_assert(MT_SW2 - MT_SW1 == 2 * MT_W1_ELEMS && MT_SW3 - MT_SW2 == 2 * MT_W2_ELEMS &&
              MT_SA1 - MT_SW3 == 2 * MT_W3_ELEMS && MT_SBAR - MT_SA2 == 2 * 128 * 128,
              "shared-memory map");

__device__ __forceinline__ void mt_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ uint32_t bf2(float a, float b)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// rows x (64 * atoms) BF16, row-major in global -> 128-byte swizzled atoms
__device__ void mt_stage_weights(const __nv_bfloat16 *__restrict__ w, int rows, int atoms, uint32_t dst)
{
    for (int e = threadIdx.x; e < rows * atoms * 8; e += blockDim.x) {
        const int c = e & 7, r = (e >> 3) % rows, a = (e >> 3) / rows;
        const uint4 v = *reinterpret_cast<const uint4 *>(w + (int64_t)r * 64 * atoms + a * 64 + c * 8);
        tc::st_shared_v4(tc::sw128(dst + (uint32_t)(a * rows * 128), r, c), v);
    }
}

// 32 accumulator columns of this thread's row: + bias, ReLU, into the BF16 A
// tile (4 chunks of 8 at column c0) and, when given, the FP32 activations
__device__ __forceinline__ void mt_hidden(const float (&v)[32], const float *__restrict__ bias, int c0, uint32_t a2,
                                         int r, float *__restrict__ h)
{
    float x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = fmaxf(v[j] + bias[c0 + j], 0.f);
    if (h) {
#pragma unroll
        for (int j = 0; j < 32; j += 4)
            *reinterpret_cast<float4 *>(h + c0 + j) = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
    }
    const int atom = c0 >> 6;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int c = ((c0 & 63) >> 3) + q;
        tc::st_shared_v4(tc::sw128(a2 + (uint32_t)(atom * 16384), r, c),
                         make_uint4(bf2(x[8 * q], x[8 * q + 1]), bf2(x[8 * q + 2], x[8 * q + 3]),
                                    bf2(x[8 * q + 4], x[8 * q + 5]), bf2(x[8 * q + 6], x[8 * q + 7])));
    }
}

__global__ void __launch_bounds__(MT_THREADS, 2)
k_mlp_tc(int64_t M, const float *__restrict__ X, const float *__restrict__ p, const __nv_bfloat16 *__restrict__ wb,
         float *__restrict__ out, float *__restrict__ h1, float *__restrict__ h2, int *__restrict__ err)
{
    extern __shared__ uint8_t smem_raw[];
    const uint32_t s0 = tc::smem_u32(smem_raw);
    const uint32_t sb = (s0 + 1023u) & ~1023u;
    uint8_t *const sg = smem_raw + (sb - s0);
    const uint32_t bar = sb + MT_SBAR, slot = bar + 8;
    const int t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                     "r"(MT_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    mt_stage_weights(wb, MLP_H, 1, sb + MT_SW1);
    mt_stage_weights(wb + MT_W1_ELEMS, MLP_H, 2, sb + MT_SW2);
    mt_stage_weights(wb + MT_W1_ELEMS + MT_W2_ELEMS, MLP_OUT, 2, sb + MT_SW3);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *reinterpret_cast<const uint32_t *>(sg + MT_SBAR + 8);
    const uint32_t lanes = (uint32_t)(warp * 32) << 16;
    const float *b1 = p + MLP_B1, *b2 = p + MLP_B2, *b3 = p + MLP_B3;
    uint32_t phase = 0;
    bool failed = false;
    // one layer: MMAs by thread 0, commit, bounded wait by every thread
    auto layer = [&](uint32_t d, uint32_t a, uint32_t w, int atoms, int a_stride, int w_stride, int n) -> bool {
        // the A tile's generic-proxy stores and this thread's TMEM reads come
        // before the MMAs that read the tile and overwrite the accumulators
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (t == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int at = 0; at < atoms; ++at)
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    mt_mma(tmem + d, tc::smem_desc_sw128(a + (uint32_t)(at * a_stride + kk * 32)),
                           tc::smem_desc_sw128(w + (uint32_t)(at * w_stride + kk * 32)), mt_idesc(n),
                           (at > 0 || kk > 0) ? 1u : 0u);
            tc::mma_commit(bar);
        }
        const bool ok = tc::mbar_wait(bar, phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        return __syncthreads_and(ok ? 1 : 0) != 0;
    };
    const int64_t tiles = (M + 127) / 128;
    for (int64_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const int64_t row = tile * 128 + t;
        const bool live = row < M;
        {
            // input row -> normalised BF16, K padded to 64
            float x[MT_K1];
#pragma unroll
            for (int k = 0; k < MT_K1; ++k) x[k] = 0.f;
            if (live) {
#pragma unroll
                for (int k = 0; k < MLP_IN; k += 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(X + row * MLP_IN + k);
                    x[k] = (v.x - p[MLP_IN_MEAN + k]) * p[MLP_IN_SCALE + k];
                    x[k + 1] = (v.y - p[MLP_IN_MEAN + k + 1]) * p[MLP_IN_SCALE + k + 1];
                    x[k + 2] = (v.z - p[MLP_IN_MEAN + k + 2]) * p[MLP_IN_SCALE + k + 2];
                    x[k + 3] = (v.w - p[MLP_IN_MEAN + k + 3]) * p[MLP_IN_SCALE + k + 3];
                }
            }
#pragma unroll
            for (int c = 0; c < 8; ++c)
                tc::st_shared_v4(tc::sw128(sb + MT_SA1, t, c),
                                 make_uint4(bf2(x[8 * c], x[8 * c + 1]), bf2(x[8 * c + 2], x[8 * c + 3]),
                                            bf2(x[8 * c + 4], x[8 * c + 5]), bf2(x[8 * c + 6], x[8 * c + 7])));
        }
        if (!layer(0, sb + MT_SA1, sb + MT_SW1, 1, 0, 0, MLP_H)) { failed = true; break; }
#pragma unroll 1
        for (int c0 = 0; c0 < MLP_H; c0 += 32) {
            float v[32];
            tc::tmem_ld32(tmem + lanes + (uint32_t)c0, v);
            mt_hidden(v, b1, c0, sb + MT_SA2, t, live && h1 ? h1 + row * MLP_H : nullptr);
        }
        if (!layer(128, sb + MT_SA2, sb + MT_SW2, 2, 16384, 16384, MLP_H)) { failed = true; break; }
        // layer-2 activations replace layer-1's in the A tile (the MMA that read them is complete)
#pragma unroll 1
        for (int c0 = 0; c0 < MLP_H; c0 += 32) {
            float v[32];
            tc::tmem_ld32(tmem + lanes + (uint32_t)(128 + c0), v);
            mt_hidden(v, b2, c0, sb + MT_SA2, t, live && h2 ? h2 + row * MLP_H : nullptr);
        }
        if (!layer(0, sb + MT_SA2, sb + MT_SW3, 2, 16384, 2048, MLP_OUT)) { failed = true; break; }
        float v0[8], v1[8];
        tc::tmem_ld8(tmem + lanes, v0);
        tc::tmem_ld8(tmem + lanes + 8u, v1);
        if (live) {
            float4 *o = reinterpret_cast<float4 *>(out + row * MLP_OUT);
            o[0] = make_float4(v0[0] + b3[0], v0[1] + b3[1], v0[2] + b3[2], v0[3] + b3[3]);
            o[1] = make_float4(v0[4] + b3[4], v0[5] + b3[5], v0[6] + b3[6], v0[7] + b3[7]);
            o[2] = make_float4(v1[0] + b3[8], v1[1] + b3[9], v1[2] + b3[10], v1[3] + b3[11]);
            o[3] = make_float4(v1[4] + b3[12], v1[5] + b3[13], v1[6] + b3[14], v1[7] + b3[15]);
        }
        // the next tile overwrites the A tiles and layer 1's accumulators
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (failed && t == 0 && err) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(MT_TMEM_COLS)
                     : "memory");
    }
}

// FP32 weights of the blob -> the BF16 image k_mlp_tc reads (W1 zero-padded to 64 inputs)
__global__ void k_mlp_pack(const float *__restrict__ p, __nv_bfloat16 *__restrict__ wb)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < MT_WB_ELEMS; e += gridDim.x * blockDim.x) {
        float v;
        if (e < MT_W1_ELEMS) {
            const int r = e / MT_K1, k = e % MT_K1;
            v = k < MLP_IN ? p[MLP_W1 + r * MLP_IN + k] : 0.f;
        } else if (e < MT_W1_ELEMS + MT_W2_ELEMS) {
            v = p[MLP_W2 + (e - MT_W1_ELEMS)];
        } else {
            v = p[MLP_W3 + (e - MT_W1_ELEMS - MT_W2_ELEMS)];
        }
        wb[e] = __float2bfloat16_rn(v);
    }
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
    // version 1 (per-pair start) and 2 (the dual form's per-sequence start) share the network
    if (params[MLP_VERSION] != (float)MLP_BLOB_VERSION && params[MLP_VERSION] != (float)MLP_BLOB_VERSION_DUAL)
        return SDCA_E_ARG;
    return SDCA_OK;
}

} // namespace

void mlp_pack(const float *p_dev, void *wb, cudaStream_t st)
{
    k_mlp_pack<<<(MT_WB_ELEMS + 255) / 256, 256, 0, st>>>(p_dev, static_cast<__nv_bfloat16 *>(wb));
}

namespace {

cudaError_t mt_configure()
{
    static std::once_flag once;
    static cudaError_t e = cudaSuccess;
    std::call_once(once, [] { e = cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, MT_SMEM); });
    return e;
}

// the fused forward over M rows: outputs, and the FP32 activations when h1, h2 are given
void mt_forward(const float *p_dev, const void *wb, const float *X, int64_t M, float *out, float *h1, float *h2,
                int *err, cudaStream_t st)
{
    if (M <= 0) return;
    if (mt_configure() != cudaSuccess) return;   // the caller's launch check reports it
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
    const int64_t tiles = (M + 127) / 128;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, 2 * (int64_t)sms);
    k_mlp_tc<<<grid, MT_THREADS, MT_SMEM, st>>>(M, X, p_dev, static_cast<const __nv_bfloat16 *>(wb), out, h1, h2,
                                                  err);
}

} // namespace

void mlp_infer(const float *p_dev, const void *wb, const float *X, int64_t M, float *out, int *err, cudaStream_t st)
{
    mt_forward(p_dev, wb, X, M, out, nullptr, nullptr, err, st);
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
    float *p = d.alloc<float>(MLP_BLOB_SIZE), *x = d.alloc<float>(M * MLP_IN), *o = d.alloc<float>(M * MLP_OUT);
    __nv_bfloat16 *wb = d.alloc<__nv_bfloat16>(MT_WB_ELEMS);
    int *err = d.alloc<int>(1);
    if (!d.ok) return mfail("device allocation failed"), SDCA_E_NOMEM;
    MK(cudaMemcpy(p, params, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyHostToDevice));
    MK(cudaMemcpy(x, X, sizeof(float) * M * MLP_IN, cudaMemcpyHostToDevice));
    MK(cudaMemset(err, 0, sizeof(int)));
    mlp_pack(p, wb, 0);
    mlp_infer(p, wb, x, M, o, err, 0);
    MK(cudaGetLastError());
    int e = 0;
    MK(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return mfail("tensor-core forward: a pipeline wait gave up");
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
    float *braw = d.alloc<float>(Bm * MLP_IN);
    __nv_bfloat16 *wb = d.alloc<__nv_bfloat16>(MT_WB_ELEMS);
    int *err = d.alloc<int>(1);
    if (!d.ok) return mfail("device allocation failed"), SDCA_E_NOMEM;
    MK(cudaMemset(err, 0, sizeof(int)));
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
            // forward on the tensor cores (BF16 image of the current weights),
            // backward in FP32 from its saved activations
            k_gather_rows<<<(unsigned)((Bm * MLP_IN + 255) / 256), 256, 0, st>>>(Bm, MLP_IN, perm_d + b0, x, braw);
            k_gather_rows<<<(unsigned)((Bm * MLP_IN + 255) / 256), 256, 0, st>>>(Bm, MLP_IN, perm_d + b0, xn, bx);
            k_gather_rows<<<(unsigned)((Bm * MLP_OUT + 255) / 256), 256, 0, st>>>(Bm, MLP_OUT, perm_d + b0, t, bt);
            mlp_pack(p, wb, st);
            mt_forward(p, wb, braw, Bm, out, h1, h2, err, st);
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
        int e = 0;
        MK(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) return mfail("tensor-core forward: a pipeline wait gave up");
        double lsum = 0.0;
        MK(cudaMemcpy(&lsum, l, sizeof(double), cudaMemcpyDeviceToHost));
        if (losses) losses[ep] = nb ? lsum / (double)nb : 0.0;
    }
    MK(cudaMemcpy(params, p, sizeof(float) * MLP_BLOB_SIZE, cudaMemcpyDeviceToHost));
    return SDCA_OK;
}

const char *sdca_mlp_last_error(void) { return t_err.c_str(); }

} // extern "C"
