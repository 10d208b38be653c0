// warmstart.cu -- the learned warm start's inputs and its start point.
//
// At the optimum of locus r the stationarity of the objective gives
//   2 lambda_J J_rn[s][a] = -sum_i w_i [s_i(n) = s] (p_i(a) - [s_i(r) = a]),
// a joint frequency of (n, r) weighted by each sequence's residual.  The
// residuals are not known before the solve; each sequence's k nearest
// neighbours in Hamming distance (the distance of the reweighting) predict
// its state at r:  p^_i(a) = (#{neighbours with state a} + eps f_r(a)) / (k + eps).
// The pair statistics fed to the per-pair MLP (mlp.cu) are, for every n,
//   joint[s][a] = sum_i w_i [s_i(n)=s][s_i(r)=a] / B_eff            (16)
//   resid[s][a] = sum_i w_i [s_i(n)=s] (p^_i(a) - [s_i(r)=a]) / B_eff (16)
//   f_n[s], f_r[a] (marginals)                                       (8)
// and its 16 outputs, times the output scale and B_eff / (2 lambda_J), are
// the start block J_rn.  h starts from 0, or (blob flag) is fitted by
// Newton's method with J fixed.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "engine.h"
#include "kernels_common.cuh"

namespace sdca {
namespace {

constexpr int WS_NB = 8;            // values of R per sequence: joint (4) and residual (4)

__device__ __forceinline__ bool before(int d, int j, int d2, int j2) { return d < d2 || (d == d2 && j < j2); }

// k nearest neighbours of each sequence (ties by lower index); one warp per row
__global__ void k_knn(const int32_t *__restrict__ dist, int N, int k, int32_t *__restrict__ knn,
                      int32_t *__restrict__ knn_d)
{
    const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= N) return;
    int bd[WS_MAX_K], bj[WS_MAX_K];
    for (int t = 0; t < WS_MAX_K; ++t) { bd[t] = INT_MAX; bj[t] = INT_MAX; }
    for (int j = lane; j < N; j += 32) {
        if (j == i) continue;
        const int d = dist[(int64_t)i * N + j];
        int pos = k - 1;
        if (!before(d, j, bd[pos], bj[pos])) continue;
        while (pos > 0 && before(d, j, bd[pos - 1], bj[pos - 1])) {
            bd[pos] = bd[pos - 1];
            bj[pos] = bj[pos - 1];
            --pos;
        }
        bd[pos] = d;
        bj[pos] = j;
    }
    for (int t = 0; t < k; ++t) {
        int d = bd[0], j = bj[0];
        for (int off = 16; off > 0; off >>= 1) {
            const int od = __shfl_xor_sync(0xffffffffu, d, off), oj = __shfl_xor_sync(0xffffffffu, j, off);
            if (before(od, oj, d, j)) { d = od; j = oj; }
        }
        if (bj[0] == j && bd[0] == d && j != INT_MAX) {
            for (int s = 0; s + 1 < k; ++s) { bd[s] = bd[s + 1]; bj[s] = bj[s + 1]; }
            bd[k - 1] = INT_MAX;
            bj[k - 1] = INT_MAX;
        }
        if (lane == 0) {
            knn[(int64_t)i * k + t] = j == INT_MAX ? -1 : j;
            if (knn_d) knn_d[(int64_t)i * k + t] = j == INT_MAX ? -1 : d;
        }
    }
}

// weighted state frequencies f_r of the block's locus (all threads get them)
__device__ void locus_frequencies(const uint8_t *__restrict__ y, int N, const double *__restrict__ w, float fr[4])
{
    __shared__ double sf[5];
    if (threadIdx.x < 5) sf[threadIdx.x] = 0.0;
    __syncthreads();
    double c[5] = {0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        c[y[i] & 3] += w[i];
        c[4] += w[i];
    }
    for (int a = 0; a < 5; ++a) {
        const double v = warp_sum(c[a]);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sf[a], v);
    }
    __syncthreads();
    for (int a = 0; a < 4; ++a) fr[a] = sf[4] > 0.0 ? (float)(sf[a] / sf[4]) : 0.25f;
}

// the two R rows of sequence i < N: w_i onehot(y_i) and w_i (p^_i - onehot(y_i))
__device__ __forceinline__ void sequence_r(const uint8_t *__restrict__ y, int i, const double *__restrict__ w,
                                           const int32_t *__restrict__ knn, int k, float eps, const float fr[4],
                                           float v[WS_NB])
{
    float cnt[4] = {0, 0, 0, 0};
    int kk = 0;
    for (int t = 0; t < k; ++t) {
        const int j = knn[(int64_t)i * k + t];
        if (j < 0) continue;
        cnt[y[j] & 3] += 1.f;
        ++kk;
    }
    const int yi = y[i] & 3;
    const float wi = (float)w[i];
    for (int a = 0; a < 4; ++a) {
        const float oh = a == yi ? 1.f : 0.f;
        const float ph = (cnt[a] + eps * fr[a]) / ((float)kk + eps);
        v[a] = wi * oh;
        v[4 + a] = wi * (ph - oh);
    }
}

// ---- the dual form's learned start (blob version 2).  From a zero start
// the dual iteration's x is (Phi^T a, eta), and at the optimum a* = -rho* /
// (2 lambda_J) with rho*_i = w_i (p*_i - onehot(y_i)), p*_i the fitted state
// probabilities of sequence i at the target column.  The network predicts
// p*_i - onehot(y_i) from statistics of the sequence and its DWS_K nearest
// neighbours in Hamming distance; the start is a0 = -alpha rho^ / (2
// lambda_J), eta0 = 0, with K a0 formed exactly (the K rho product of the
// iteration).  Statistics per sequence i of target column y (MLP_IN = 40):
//   [0, 4)   onehot(y_i)
//   [4, 8)   weighted state frequencies of the column
//   [8, 24)  state frequencies among the 1, 3, 8 and 16 nearest neighbours
//   [24, 28) Hamming distances of neighbours 1, 3, 8 and 16, over L
//   [28, 40) 0
__global__ void __launch_bounds__(256)
k_dual_ws_feats(const uint8_t *__restrict__ cols, const int32_t *__restrict__ idx, int N, int64_t Nx, int L,
                const double *__restrict__ w, const int32_t *__restrict__ knn, const int32_t *__restrict__ knn_d,
                float *__restrict__ feats)
{
    const int g = blockIdx.x;
    const uint8_t *y = cols + (int64_t)idx[g] * Nx;
    float fr[4];
    locus_frequencies(y, N, w, fr);
    const float invL = 1.f / (float)L;
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) {
        float f[MLP_IN];
#pragma unroll
        for (int t = 0; t < MLP_IN; ++t) f[t] = 0.f;
        if (i < N) {
            const int yi = y[i] & 3;
            float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                f[a] = a == yi ? 1.f : 0.f;
                f[4 + a] = fr[a];
            }
            int kk = 0;
            const int marks[4] = {1, 3, 8, 16};
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                for (; kk < marks[m]; ++kk) {
                    const int j = knn[(int64_t)i * DWS_K + kk];
                    if (j >= 0) {
                        const int yj = y[j] & 3;
#pragma unroll
                        for (int a = 0; a < 4; ++a) c[a] += a == yj ? 1.f : 0.f;
                    }
                }
#pragma unroll
                for (int a = 0; a < 4; ++a) f[8 + 4 * m + a] = c[a] / (float)marks[m];
                const int d = knn_d[(int64_t)i * DWS_K + marks[m] - 1];
                f[24 + m] = d < 0 ? 1.f : (float)d * invL;
            }
        }
        float4 *o4 = reinterpret_cast<float4 *>(feats + ((int64_t)g * Nx + i) * MLP_IN);
#pragma unroll
        for (int t = 0; t < MLP_IN / 4; ++t) o4[t] = make_float4(f[4 * t], f[4 * t + 1], f[4 * t + 2], f[4 * t + 3]);
    }
}

// The predicted residual rows of slots[g]: R_i = alpha w_i c_i with c_i the
// network's first four outputs in the blob's output units, centred (a
// residual p - onehot sums to zero over the states) and scaled down to
// max |c_ia| <= 1 where larger (a residual's entries lie in [-1, 1]), so that
// |R| <= w_max keeps the exact K rho product in its digit range; rows
// N..Nx-1 are zero
__global__ void k_dual_ws_r(const int32_t *__restrict__ slots, int N, int64_t Nx, const float *__restrict__ out,
                            const float *__restrict__ p, float alpha, const float *__restrict__ w,
                            float4 *__restrict__ R)
{
    const int g = blockIdx.y, b = slots[g];
    const float s0 = p[MLP_OUT_SCALE], s1 = p[MLP_OUT_SCALE + 1], s2 = p[MLP_OUT_SCALE + 2], s3 = p[MLP_OUT_SCALE + 3];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x) {
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < N) {
            const float *o = out + ((int64_t)g * Nx + i) * MLP_OUT;
            float c0 = o[0] * s0, c1 = o[1] * s1, c2 = o[2] * s2, c3 = o[3] * s3;
            const float m = 0.25f * (c0 + c1 + c2 + c3);
            c0 -= m;
            c1 -= m;
            c2 -= m;
            c3 -= m;
            const float mx = fmaxf(fmaxf(fabsf(c0), fabsf(c1)), fmaxf(fabsf(c2), fabsf(c3)));
            const float c = alpha * w[i] / fmaxf(mx, 1.f);
            r = isfinite(c * mx) ? make_float4(c * c0, c * c1, c * c2, c * c3) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        R[(int64_t)b * Nx + i] = r;
    }
}

// R values per sequence for one warm-start locus (block g), both rows side
// by side ([g][Nx][8]); rows N..Nx-1 are zero
__global__ void __launch_bounds__(256)
k_ws_residual(const uint8_t *__restrict__ XT, int64_t Nx, int N, const int32_t *__restrict__ loci,
              const double *__restrict__ w, const int32_t *__restrict__ knn, int k, float eps,
              float *__restrict__ Rws)
{
    const int g = blockIdx.x;
    const uint8_t *y = XT + (int64_t)loci[g] * Nx;
    float fr[4];
    locus_frequencies(y, N, w, fr);
    float *out = Rws + (int64_t)g * Nx * WS_NB;
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) {
        float v[WS_NB] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (i < N) sequence_r(y, i, w, knn, k, eps, fr, v);
        float4 *o4 = reinterpret_cast<float4 *>(out + (int64_t)i * WS_NB);
        o4[0] = make_float4(v[0], v[1], v[2], v[3]);
        o4[1] = make_float4(v[4], v[5], v[6], v[7]);
    }
}

// the same rows for the tensor-core path: the first into the slot's R rows
// (slots[g]), the second into R2[g]
__global__ void __launch_bounds__(256)
k_ws_residual_split(const uint8_t *__restrict__ XT, int64_t Nx, int N, const int32_t *__restrict__ loci,
                    const int32_t *__restrict__ slots, const double *__restrict__ w, const int32_t *__restrict__ knn,
                    int k, float eps, float4 *__restrict__ R, float4 *__restrict__ R2)
{
    const int g = blockIdx.x;
    const uint8_t *y = XT + (int64_t)loci[g] * Nx;
    float fr[4];
    locus_frequencies(y, N, w, fr);
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) {
        float v[WS_NB] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (i < N) sequence_r(y, i, w, knn, k, eps, fr, v);
        R[(int64_t)slots[g] * Nx + i] = make_float4(v[0], v[1], v[2], v[3]);
        R2[(int64_t)g * Nx + i] = make_float4(v[4], v[5], v[6], v[7]);
    }
}

__global__ void k_ws_copy_r(int64_t Nx, const int32_t *__restrict__ slots, const float4 *__restrict__ R2,
                            float4 *__restrict__ R)
{
    const int g = blockIdx.y;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x)
        R[(int64_t)slots[g] * Nx + i] = R2[(int64_t)g * Nx + i];
}

// features from the two contractions left in the slot's gradient buffers:
// joint in buffer 2b+1, residual-weighted in buffer 2b
__global__ void k_ws_assemble(int L, int64_t Dp, const int32_t *__restrict__ slots, const float *__restrict__ gpool,
                              float inv_beff, float *__restrict__ feats)
{
    const int g = blockIdx.y, b = slots[g];
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= L) return;
    const float4 *jt = reinterpret_cast<const float4 *>(gpool + (int64_t)(2 * b + 1) * Dp + (int64_t)QQ * n);
    const float4 *rs = reinterpret_cast<const float4 *>(gpool + (int64_t)(2 * b) * Dp + (int64_t)QQ * n);
    float *f = feats + ((int64_t)g * L + n) * MLP_IN;
    float fr[4] = {0, 0, 0, 0};
#pragma unroll
    for (int st = 0; st < 4; ++st) {
        const float4 a = jt[st], c = rs[st];
        f[4 * st + 0] = a.x * inv_beff; f[4 * st + 1] = a.y * inv_beff;
        f[4 * st + 2] = a.z * inv_beff; f[4 * st + 3] = a.w * inv_beff;
        f[16 + 4 * st + 0] = c.x * inv_beff; f[16 + 4 * st + 1] = c.y * inv_beff;
        f[16 + 4 * st + 2] = c.z * inv_beff; f[16 + 4 * st + 3] = c.w * inv_beff;
        f[32 + st] = (a.x + a.y + a.z + a.w) * inv_beff;
        fr[0] += a.x; fr[1] += a.y; fr[2] += a.z; fr[3] += a.w;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) f[36 + c] = fr[c] * inv_beff;
}

constexpr int PT = 128;   // loci per CTA
constexpr int PG = 2;     // warm-start loci per CTA
constexpr int PSUB = 64;  // sequences per shared-memory sub-tile

// pair statistics of PG loci against every locus n (one thread per n)
__global__ void __launch_bounds__(PT)
k_ws_pairs(const uint8_t *__restrict__ XT, int64_t Nx, int N, int L, int G, const float *__restrict__ Rws,
           float inv_beff, float *__restrict__ feats)
{
    __shared__ float4 sR[PG][PSUB][2];
    const int n = blockIdx.x * PT + threadIdx.x;
    int gs[PG];
#pragma unroll
    for (int q = 0; q < PG; ++q) {
        const int g = blockIdx.y * PG + q;
        gs[q] = g < G ? g : -1;
    }
    float a[PG][32];
#pragma unroll
    for (int q = 0; q < PG; ++q)
#pragma unroll
        for (int e = 0; e < 32; ++e) a[q][e] = 0.f;

    for (int i0 = 0; i0 < N; i0 += PSUB) {
        for (int e = threadIdx.x; e < PG * PSUB * 2; e += PT) {
            const int q = e / (PSUB * 2), r = e % (PSUB * 2), ii = r / 2, h = r % 2;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gs[q] >= 0)
                v = reinterpret_cast<const float4 *>(Rws + ((int64_t)gs[q] * Nx + i0 + ii) * WS_NB)[h];
            sR[q][ii][h] = v;
        }
        __syncthreads();
        if (n < L) {
            const uint4 *xp = reinterpret_cast<const uint4 *>(XT + (int64_t)n * Nx + i0);
#pragma unroll
            for (int q4 = 0; q4 < PSUB / 16; ++q4) {
                const uint4 wv = xp[q4];
                const uint32_t words[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
                for (int wd = 0; wd < 4; ++wd) {
#pragma unroll
                    for (int bt = 0; bt < 4; ++bt) {
                        const int ii = q4 * 16 + wd * 4 + bt;
                        const int s = (words[wd] >> (8 * bt)) & 0x3;
                        const float m[4] = {s == 0 ? 1.f : 0.f, s == 1 ? 1.f : 0.f, s == 2 ? 1.f : 0.f,
                                            s == 3 ? 1.f : 0.f};
#pragma unroll
                        for (int q = 0; q < PG; ++q) {
                            const float4 r1 = sR[q][ii][0], r2 = sR[q][ii][1];
#pragma unroll
                            for (int st = 0; st < 4; ++st) {
                                a[q][4 * st + 0] = fmaf(m[st], r1.x, a[q][4 * st + 0]);
                                a[q][4 * st + 1] = fmaf(m[st], r1.y, a[q][4 * st + 1]);
                                a[q][4 * st + 2] = fmaf(m[st], r1.z, a[q][4 * st + 2]);
                                a[q][4 * st + 3] = fmaf(m[st], r1.w, a[q][4 * st + 3]);
                                a[q][16 + 4 * st + 0] = fmaf(m[st], r2.x, a[q][16 + 4 * st + 0]);
                                a[q][16 + 4 * st + 1] = fmaf(m[st], r2.y, a[q][16 + 4 * st + 1]);
                                a[q][16 + 4 * st + 2] = fmaf(m[st], r2.z, a[q][16 + 4 * st + 2]);
                                a[q][16 + 4 * st + 3] = fmaf(m[st], r2.w, a[q][16 + 4 * st + 3]);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    if (n >= L) return;
#pragma unroll
    for (int q = 0; q < PG; ++q) {
        if (gs[q] < 0) continue;
        float *f = feats + ((int64_t)gs[q] * L + n) * MLP_IN;
        float fn[4] = {0, 0, 0, 0}, fr[4] = {0, 0, 0, 0};
#pragma unroll
        for (int e = 0; e < 32; ++e) f[e] = a[q][e] * inv_beff;
#pragma unroll
        for (int st = 0; st < 4; ++st)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                fn[st] += a[q][4 * st + c];
                fr[c] += a[q][4 * st + c];
            }
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            f[32 + e] = fn[e] * inv_beff;
            f[36 + e] = fr[e] * inv_beff;
        }
    }
}

// network outputs -> start point of slot slots[g]: J blocks (zero at n = r), h = 0
__global__ void k_ws_scatter(int L, int64_t Dp, const int32_t *__restrict__ slots, const int32_t *__restrict__ loci,
                             const float *__restrict__ out, const float *__restrict__ p, float out_mult,
                             float *__restrict__ wa, double *__restrict__ xmax)
{
    const int g = blockIdx.y;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float v = 0.f;
    if (e < Dp) {
        const int64_t n = e / QQ;
        const int k = (int)(e % QQ);
        if (n < L && n != loci[g]) v = out[((int64_t)g * L + n) * MLP_OUT + k] * p[MLP_OUT_SCALE + k] * out_mult;
        wa[(int64_t)slots[g] * Dp + e] = v;
    }
    float m = fabsf(v);
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomic_max_nonneg(xmax + g, (double)m);
}

// h with J fixed: Newton on sum_i w_i (lse(l_i + h) - (l_i + h)[y_i]) + lambda_h |h|^2
// from the logits l_i at the start point (which has h = 0); one block per slot
__global__ void __launch_bounds__(256)
k_ws_hfit(int N, int64_t Nx, int64_t Dp, int L, double lambda_h, const int32_t *__restrict__ slots,
          const uint8_t *__restrict__ rstate, const double *__restrict__ w, float *__restrict__ wa,
          double *__restrict__ lbase, double *__restrict__ xmax)
{
    const int g = blockIdx.x, b = slots[g];
    const uint8_t *y = rstate + (int64_t)b * Nx;
    double *lb = lbase + (int64_t)b * Nx * 4;
    __shared__ double red[14];
    __shared__ double sh[4];
    __shared__ int done;
    if (threadIdx.x < 4) sh[threadIdx.x] = 0.0;
    for (int it = 0; it < 40; ++it) {
        if (threadIdx.x < 14) red[threadIdx.x] = 0.0;
        __syncthreads();
        double acc[14] = {};
        const double h0 = sh[0], h1 = sh[1], h2 = sh[2], h3 = sh[3];
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double l[4] = {lb[4 * i] + h0, lb[4 * i + 1] + h1, lb[4 * i + 2] + h2, lb[4 * i + 3] + h3};
            const double mx = fmax(fmax(l[0], l[1]), fmax(l[2], l[3]));
            double pr[4], z = 0.0;
            for (int a = 0; a < 4; ++a) { pr[a] = exp(l[a] - mx); z += pr[a]; }
            const double wi = w[i];
            const int yi = y[i] & 3;
            int t = 4;
            for (int a = 0; a < 4; ++a) {
                pr[a] /= z;
                acc[a] += wi * (pr[a] - (a == yi ? 1.0 : 0.0));
            }
            for (int a = 0; a < 4; ++a)
                for (int c = a; c < 4; ++c) acc[t++] += wi * ((a == c ? pr[a] : 0.0) - pr[a] * pr[c]);
        }
        for (int e = 0; e < 14; ++e) {
            const double v = warp_sum(acc[e]);
            if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&red[e], v);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double gr[4], H[4][4];
            int t = 4;
            for (int a = 0; a < 4; ++a) gr[a] = red[a] + 2.0 * lambda_h * sh[a];
            for (int a = 0; a < 4; ++a)
                for (int c = a; c < 4; ++c) {
                    H[a][c] = H[c][a] = red[t++] + (a == c ? 2.0 * lambda_h : 0.0);
                }
            // Cholesky solve H dx = gr (H is positive definite: lambda_h > 0)
            double Lc[4][4] = {};
            bool ok = true;
            for (int a = 0; a < 4 && ok; ++a) {
                double s = H[a][a];
                for (int c = 0; c < a; ++c) s -= Lc[a][c] * Lc[a][c];
                if (!(s > 0.0)) { ok = false; break; }
                Lc[a][a] = sqrt(s);
                for (int r = a + 1; r < 4; ++r) {
                    double t2 = H[r][a];
                    for (int c = 0; c < a; ++c) t2 -= Lc[r][c] * Lc[a][c];
                    Lc[r][a] = t2 / Lc[a][a];
                }
            }
            double step = 0.0;
            if (ok) {
                double z[4], dx[4];
                for (int a = 0; a < 4; ++a) {
                    double s = gr[a];
                    for (int c = 0; c < a; ++c) s -= Lc[a][c] * z[c];
                    z[a] = s / Lc[a][a];
                }
                for (int a = 3; a >= 0; --a) {
                    double s = z[a];
                    for (int c = a + 1; c < 4; ++c) s -= Lc[c][a] * dx[c];
                    dx[a] = s / Lc[a][a];
                }
                for (int a = 0; a < 4; ++a) {
                    sh[a] -= dx[a];
                    step = fmax(step, fabs(dx[a]));
                }
            }
            done = !ok || step < 1e-13;
        }
        __syncthreads();
        if (done) break;
    }
    // store h in single precision and move the logits by exactly that amount
    const float hf[4] = {(float)sh[0], (float)sh[1], (float)sh[2], (float)sh[3]};
    if (threadIdx.x < 4) wa[(int64_t)b * Dp + (int64_t)QQ * L + threadIdx.x] = hf[threadIdx.x];
    for (int64_t i = threadIdx.x; i < Nx; i += blockDim.x)
        for (int a = 0; a < 4; ++a) lb[4 * i + a] += (double)hf[a];
    if (threadIdx.x == 0) {
        const double m = fmax(fmax(fabs((double)hf[0]), fabs((double)hf[1])), fmax(fabs((double)hf[2]), fabs((double)hf[3])));
        if (m > 0.0) atomic_max_nonneg(xmax + g, m);
    }
}

} // namespace

void launch_knn(const int32_t *dist, int N, int k, int32_t *knn, cudaStream_t st, int32_t *knn_d)
{
    const int64_t threads = (int64_t)N * 32;
    k_knn<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(dist, N, k, knn, knn_d);
}

void launch_dual_ws_feats(const uint8_t *cols, const int32_t *idx, int n, int N, int64_t Nx, int L, const double *w,
                          const int32_t *knn, const int32_t *knn_d, float *feats, cudaStream_t st)
{
    if (n <= 0) return;
    k_dual_ws_feats<<<n, 256, 0, st>>>(cols, idx, N, Nx, L, w, knn, knn_d, feats);
}

void launch_dual_ws_r(const int32_t *slots, int n, int N, int64_t Nx, const float *out, const float *p_dev, float alpha,
                      const float *w, float *R, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g((unsigned)((Nx + 255) / 256), (unsigned)n);
    k_dual_ws_r<<<g, 256, 0, st>>>(slots, N, Nx, out, p_dev, alpha, w, reinterpret_cast<float4 *>(R));
}

void launch_ws_residual(const uint8_t *XT, int64_t Nx, int N, const int32_t *loci, int G, const double *w,
                        const int32_t *knn, int k, float eps, float *Rws, cudaStream_t st)
{
    k_ws_residual<<<G, 256, 0, st>>>(XT, Nx, N, loci, w, knn, k, eps, Rws);
}

void launch_ws_residual_split(const uint8_t *XT, int64_t Nx, int N, const int32_t *loci, const int32_t *slots, int G,
                              const double *w, const int32_t *knn, int k, float eps, float *R, float *R2,
                              cudaStream_t st)
{
    k_ws_residual_split<<<G, 256, 0, st>>>(XT, Nx, N, loci, slots, w, knn, k, eps, reinterpret_cast<float4 *>(R),
                                           reinterpret_cast<float4 *>(R2));
}

void launch_ws_copy_r(int64_t Nx, const int32_t *slots, int G, const float *R2, float *R, cudaStream_t st)
{
    dim3 grid((unsigned)std::min<int64_t>((Nx + 255) / 256, 64), G);
    k_ws_copy_r<<<grid, 256, 0, st>>>(Nx, slots, reinterpret_cast<const float4 *>(R2), reinterpret_cast<float4 *>(R));
}

void launch_ws_assemble(int L, int64_t Dp, const int32_t *slots, int G, const float *gpool, double b_eff,
                        float *feats, cudaStream_t st)
{
    dim3 grid((L + 127) / 128, G);
    k_ws_assemble<<<grid, 128, 0, st>>>(L, Dp, slots, gpool, (float)(1.0 / b_eff), feats);
}

void launch_ws_pairs(const uint8_t *XT, int64_t Nx, int N, int L, int G, const float *Rws, double b_eff,
                     float *feats, cudaStream_t st)
{
    dim3 grid((L + PT - 1) / PT, (G + PG - 1) / PG);
    k_ws_pairs<<<grid, PT, 0, st>>>(XT, Nx, N, L, G, Rws, (float)(1.0 / b_eff), feats);
}

void launch_ws_scatter(int L, int64_t Dp, const int32_t *slots, const int32_t *loci, int G, const float *out,
                       const float *p_dev, double out_mult, float *wa, double *xmax, cudaStream_t st)
{
    dim3 grid((unsigned)((Dp + 255) / 256), G);
    k_ws_scatter<<<grid, 256, 0, st>>>(L, Dp, slots, loci, out, p_dev, (float)out_mult, wa, xmax);
}

void launch_ws_hfit(const Problem &P, const int32_t *slots, const uint8_t *rstate, const double *w, int G,
                    float *wa, double *lbase, double *xmax, cudaStream_t st)
{
    k_ws_hfit<<<G, 256, 0, st>>>((int)P.N, P.Nx, P.Dp, (int)P.L, P.lambda_h, slots, rstate, w, wa, lbase, xmax);
}

} // namespace sdca
