// kernels_gather.cu -- the plain contraction form: FP32 gather (forward) and
// masked accumulation (backward) on CUDA cores.
//
// forward   u_b[i][a] = sum_n v_b[n][X_in][a]                 (X one-hot . v_J)
// backward  g_b[n][s][a] = sum_{i: X_in = s} R_b[i][a] + 2 lambda_J x_b[n][s][a]
//
// These are SuperDCA's block gather (SuperDCA/include/plmDCA_objective.hpp:86-121,
// Coupling_matrix_view.hpp:59-86) and gradient scatter (plmDCA_objective.hpp:
// 153-190, Coupling_matrix_view.hpp:88-111) for a batch of target loci that
// share one alignment read.  Both are bound by shared-memory / FP32 issue
// (one 16-byte shared load or 16 FMAs per (sequence, locus, slot)).
#include "engine.h"
#include "kernels_common.cuh"

namespace sdca {

namespace {

constexpr int FWD_THREADS = 256;  // sequences per CTA
constexpr int FWD_G = 8;          // slots per CTA
constexpr int FWD_SUB = 32;       // loci per shared-memory sub-tile

__global__ void __launch_bounds__(FWD_THREADS)
k_fwd_gather(const uint8_t *__restrict__ X, int64_t Lx, int N, int L, int64_t LC,
             const int32_t *__restrict__ list, int nlist, const float *__restrict__ vecs,
             int64_t Dp, float4 *__restrict__ partial, int Bmax, int64_t Nx)
{
    __shared__ float4 sJ[FWD_G][FWD_SUB][Q];
    const int i = blockIdx.x * FWD_THREADS + threadIdx.x;
    const int c = blockIdx.z;
    const int64_t n_begin = (int64_t)c * LC;
    const int64_t n_end = min((int64_t)L, n_begin + LC);
    int slot[FWD_G];
#pragma unroll
    for (int g = 0; g < FWD_G; ++g) {
        const int k = blockIdx.y * FWD_G + g;
        slot[g] = k < nlist ? list[k] : -1;
    }
    float4 acc[FWD_G];
#pragma unroll
    for (int g = 0; g < FWD_G; ++g) acc[g] = make_float4(0.f, 0.f, 0.f, 0.f);

    for (int64_t n0 = n_begin; n0 < n_end; n0 += FWD_SUB) {
        for (int k = threadIdx.x; k < FWD_G * FWD_SUB * Q; k += FWD_THREADS) {
            const int g = k / (FWD_SUB * Q), rem = k % (FWD_SUB * Q);
            const int nl = rem / Q, s = rem % Q;
            const int64_t n = n0 + nl;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (slot[g] >= 0 && n < n_end)
                v = reinterpret_cast<const float4 *>(vecs + (int64_t)slot[g] * Dp)[n * Q + s];
            sJ[g][nl][s] = v;
        }
        __syncthreads();
        if (i < N) {
            const uint4 *xp = reinterpret_cast<const uint4 *>(X + (int64_t)i * Lx + n0);
            const uint4 w0 = xp[0], w1 = xp[1];
            const uint32_t words[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
            for (int wd = 0; wd < 8; ++wd) {
#pragma unroll
                for (int bt = 0; bt < 4; ++bt) {
                    const int nl = wd * 4 + bt;
                    const int s = (words[wd] >> (8 * bt)) & 0x3;
#pragma unroll
                    for (int g = 0; g < FWD_G; ++g) {
                        const float4 j = sJ[g][nl][s];
                        acc[g].x += j.x;
                        acc[g].y += j.y;
                        acc[g].z += j.z;
                        acc[g].w += j.w;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (i < N) {
#pragma unroll
        for (int g = 0; g < FWD_G; ++g)
            if (slot[g] >= 0) partial[((int64_t)c * Bmax + slot[g]) * Nx + i] = acc[g];
    }
}

// Logits at a stored point, for the start of a locus and for the objective a
// converged locus reports.  The sequences of an alignment share most of their
// states, so rounding errors of long FP32 locus sums are correlated across
// sequences and add up over the N terms of the objective; here FP32 sums run
// over 64-locus stretches only and the stretches accumulate in FP64.
constexpr int EX_G = 4;

__global__ void __launch_bounds__(FWD_THREADS)
k_fwd_gather_exact(const uint8_t *__restrict__ X, int64_t Lx, int N, int L, int64_t LC,
                   const int32_t *__restrict__ list, int nlist, const float *__restrict__ vecs,
                   int64_t Dp, double4 *__restrict__ partial, int Bmax, int64_t Nx)
{
    __shared__ float4 sJ[EX_G][FWD_SUB][Q];
    const int i = blockIdx.x * FWD_THREADS + threadIdx.x;
    const int c = blockIdx.z;
    const int64_t n_begin = (int64_t)c * LC;
    const int64_t n_end = min((int64_t)L, n_begin + LC);
    int slot[EX_G];
#pragma unroll
    for (int g = 0; g < EX_G; ++g) {
        const int k = blockIdx.y * EX_G + g;
        slot[g] = k < nlist ? list[k] : -1;
    }
    float4 acc[EX_G];
    double a64[EX_G][4];
#pragma unroll
    for (int g = 0; g < EX_G; ++g) {
        acc[g] = make_float4(0.f, 0.f, 0.f, 0.f);
        a64[g][0] = a64[g][1] = a64[g][2] = a64[g][3] = 0.0;
    }
    int sub = 0;
    for (int64_t n0 = n_begin; n0 < n_end; n0 += FWD_SUB, ++sub) {
        for (int k = threadIdx.x; k < EX_G * FWD_SUB * Q; k += FWD_THREADS) {
            const int g = k / (FWD_SUB * Q), rem = k % (FWD_SUB * Q);
            const int nl = rem / Q, s = rem % Q;
            const int64_t n = n0 + nl;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (slot[g] >= 0 && n < n_end)
                v = reinterpret_cast<const float4 *>(vecs + (int64_t)slot[g] * Dp)[n * Q + s];
            sJ[g][nl][s] = v;
        }
        __syncthreads();
        if (i < N) {
            const uint4 *xp = reinterpret_cast<const uint4 *>(X + (int64_t)i * Lx + n0);
            const uint4 w0 = xp[0], w1 = xp[1];
            const uint32_t words[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
            for (int wd = 0; wd < 8; ++wd) {
#pragma unroll
                for (int bt = 0; bt < 4; ++bt) {
                    const int nl = wd * 4 + bt;
                    const int s = (words[wd] >> (8 * bt)) & 0x3;
#pragma unroll
                    for (int g = 0; g < EX_G; ++g) {
                        const float4 j = sJ[g][nl][s];
                        acc[g].x += j.x;
                        acc[g].y += j.y;
                        acc[g].z += j.z;
                        acc[g].w += j.w;
                    }
                }
            }
            if (sub & 1) {
#pragma unroll
                for (int g = 0; g < EX_G; ++g) {
                    a64[g][0] += acc[g].x; a64[g][1] += acc[g].y;
                    a64[g][2] += acc[g].z; a64[g][3] += acc[g].w;
                    acc[g] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
        }
        __syncthreads();
    }
    if (i < N) {
#pragma unroll
        for (int g = 0; g < EX_G; ++g)
            if (slot[g] >= 0)
                partial[((int64_t)c * Bmax + slot[g]) * Nx + i] =
                    make_double4(a64[g][0] + acc[g].x, a64[g][1] + acc[g].y, a64[g][2] + acc[g].z,
                                 a64[g][3] + acc[g].w);
    }
}

__global__ void k_reduce_partial64(const double4 *__restrict__ partial, int C, int Bmax, int64_t Nx,
                                   int N, const int32_t *__restrict__ list,
                                   const float *__restrict__ vecs, int64_t Dp, int64_t hoff,
                                   double *__restrict__ out_d)
{
    const int b = list[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float *h = vecs + (int64_t)b * Dp + hoff;
    double s0 = h[0], s1 = h[1], s2 = h[2], s3 = h[3];
    for (int c = 0; c < C; ++c) {
        const double4 p = partial[((int64_t)c * Bmax + b) * Nx + i];
        s0 += p.x; s1 += p.y; s2 += p.z; s3 += p.w;
    }
    const int64_t o = (int64_t)b * Nx + i;
    out_d[o * 4 + 0] = s0; out_d[o * 4 + 1] = s1;
    out_d[o * 4 + 2] = s2; out_d[o * 4 + 3] = s3;
}

// Sums the partial slices into u (float) or logits (double).  With R given,
// also reduces sum_i R_i . u_i per slot into acc[ACC_DG0]: the slope at
// step 0 of the line the next search walks, from the same numbers the
// trial steps will use.
__global__ void k_reduce_partial(const float4 *__restrict__ partial, int C, int Bmax, int64_t Nx,
                                 int N, const int32_t *__restrict__ list,
                                 const float *__restrict__ vecs, int64_t Dp, int64_t hoff,
                                 int add_h, float4 *__restrict__ out_f, double *__restrict__ out_d,
                                 const float4 *__restrict__ R, double *__restrict__ acc)
{
    const int b = list[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (R) {
        // every thread of the block takes part in the reduction
        double ru = 0.0;
        if (i < N) {
            double t[4] = {0, 0, 0, 0};
            if (add_h) {
                const float *h = vecs + (int64_t)b * Dp + hoff;
                t[0] = h[0]; t[1] = h[1]; t[2] = h[2]; t[3] = h[3];
            }
            for (int c = 0; c < C; ++c) {
                const float4 p = partial[((int64_t)c * Bmax + b) * Nx + i];
                t[0] += p.x; t[1] += p.y; t[2] += p.z; t[3] += p.w;
            }
            const float4 uf = make_float4((float)t[0], (float)t[1], (float)t[2], (float)t[3]);
            out_f[(int64_t)b * Nx + i] = uf;
            const float4 r = R[(int64_t)b * Nx + i];
            ru = (double)r.x * uf.x + (double)r.y * uf.y + (double)r.z * uf.z + (double)r.w * uf.w;
        }
        double v[1] = {ru};
        const int idx[1] = {ACC_DG0};
        block_sum_atomic<1>(v, acc + (int64_t)b * NACC, idx);
        return;
    }
    if (i >= N) return;
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    if (add_h) {
        const float *h = vecs + (int64_t)b * Dp + hoff;
        s0 = h[0]; s1 = h[1]; s2 = h[2]; s3 = h[3];
    }
    for (int c = 0; c < C; ++c) {
        const float4 p = partial[((int64_t)c * Bmax + b) * Nx + i];
        s0 += p.x; s1 += p.y; s2 += p.z; s3 += p.w;
    }
    const int64_t o = (int64_t)b * Nx + i;
    if (out_f) out_f[o] = make_float4((float)s0, (float)s1, (float)s2, (float)s3);
    if (out_d) {
        out_d[o * 4 + 0] = s0; out_d[o * 4 + 1] = s1;
        out_d[o * 4 + 2] = s2; out_d[o * 4 + 3] = s3;
    }
}

constexpr int BWD_THREADS = 128;  // loci per CTA
constexpr int BWD_G = 4;          // slots per CTA
constexpr int BWD_SUB = 64;       // sequences per shared-memory sub-tile

__global__ void __launch_bounds__(BWD_THREADS)
k_bwd_gather(const uint8_t *__restrict__ XT, int64_t Nx, int N, int L,
             const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int nlist,
             const float4 *__restrict__ R, const float *__restrict__ wa, float *__restrict__ gpool,
             void *__restrict__ Ypool, const void *__restrict__ Spool, int hist_bf16, int m,
             int64_t Dp, double lambda_J, double *__restrict__ acc)
{
    __shared__ float4 sR[BWD_G][BWD_SUB];
    const int n = blockIdx.x * BWD_THREADS + threadIdx.x;
    int slot[BWD_G];
#pragma unroll
    for (int g = 0; g < BWD_G; ++g) {
        const int k = blockIdx.y * BWD_G + g;
        slot[g] = k < nlist ? list[k] : -1;
    }
    float a[BWD_G][QQ];
#pragma unroll
    for (int g = 0; g < BWD_G; ++g)
#pragma unroll
        for (int k = 0; k < QQ; ++k) a[g][k] = 0.f;

    for (int i0 = 0; i0 < N; i0 += BWD_SUB) {
        for (int k = threadIdx.x; k < BWD_G * BWD_SUB; k += BWD_THREADS) {
            const int g = k / BWD_SUB, ii = k % BWD_SUB;
            const int i = i0 + ii;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (slot[g] >= 0 && i < N) v = R[(int64_t)slot[g] * Nx + i];
            sR[g][ii] = v;
        }
        __syncthreads();
        if (n < L) {
            const uint4 *xp = reinterpret_cast<const uint4 *>(XT + (int64_t)n * Nx + i0);
#pragma unroll
            for (int q4 = 0; q4 < BWD_SUB / 16; ++q4) {
                const uint4 w = xp[q4];
                const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int wd = 0; wd < 4; ++wd) {
#pragma unroll
                    for (int bt = 0; bt < 4; ++bt) {
                        const int ii = q4 * 16 + wd * 4 + bt;
                        const int s = (words[wd] >> (8 * bt)) & 0x3;
                        const float m0 = s == 0, m1 = s == 1, m2 = s == 2, m3 = s == 3;
#pragma unroll
                        for (int g = 0; g < BWD_G; ++g) {
                            const float4 r = sR[g][ii];
                            a[g][0] += m0 * r.x; a[g][1] += m0 * r.y; a[g][2] += m0 * r.z; a[g][3] += m0 * r.w;
                            a[g][4] += m1 * r.x; a[g][5] += m1 * r.y; a[g][6] += m1 * r.z; a[g][7] += m1 * r.w;
                            a[g][8] += m2 * r.x; a[g][9] += m2 * r.y; a[g][10] += m2 * r.z; a[g][11] += m2 * r.w;
                            a[g][12] += m3 * r.x; a[g][13] += m3 * r.y; a[g][14] += m3 * r.z; a[g][15] += m3 * r.w;
                        }
                    }
                }
            }
        }
        __syncthreads();
    }

    // epilogue: + 2 lambda_J x, zero the J_rr block, push y, reductions
    const float l2 = (float)(2.0 * lambda_J);
#pragma unroll
    for (int g = 0; g < BWD_G; ++g) {
        if (slot[g] < 0) continue;  // uniform across the block
        const int b = slot[g];
        GradRed red;
        if (n < L) grad_locus(sd[b], b, n, a[g], wa, gpool, Ypool, Spool, hist_bf16, m, Dp, l2, red);
        double v[5] = {red.g2, red.x2, red.sy, red.yy, red.ss};
        const int idx[5] = {ACC_G2, ACC_X2J, ACC_SY, ACC_YY, ACC_SS};
        block_sum_atomic<5>(v, acc + (int64_t)b * NACC, idx);
        const float wm = warp_max(red.gmax);
        if ((threadIdx.x & 31) == 0 && wm > 0.f) atomic_max_nonneg(acc + (int64_t)b * NACC + ACC_GMAX, (double)wm);
    }
}

// The tensor-core backward leaves X^T R (scaled back) in the new-gradient
// buffer; this adds the L2 part and does the same bookkeeping.
__global__ void __launch_bounds__(BWD_THREADS)
k_grad_finalize(int L, const SlotDev *__restrict__ sd, const int32_t *__restrict__ list,
                const float *__restrict__ wa, float *__restrict__ gpool, void *__restrict__ Ypool,
                const void *__restrict__ Spool, int hist_bf16, int m, int64_t Dp, double lambda_J,
                double *__restrict__ acc)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const float l2 = (float)(2.0 * lambda_J);
    GradRed red;
    for (int64_t n = (int64_t)blockIdx.x * BWD_THREADS + threadIdx.x; n < L; n += (int64_t)gridDim.x * BWD_THREADS) {
        const float4 *gr = reinterpret_cast<const float4 *>(gpool + (int64_t)(2 * b + 1 - S.gcur) * Dp + n * QQ);
        float c[16];
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4) {
            const float4 v = gr[k4];
            c[4 * k4] = v.x; c[4 * k4 + 1] = v.y; c[4 * k4 + 2] = v.z; c[4 * k4 + 3] = v.w;
        }
        grad_locus(S, b, n, c, wa, gpool, Ypool, Spool, hist_bf16, m, Dp, l2, red);
    }
    double v[5] = {red.g2, red.x2, red.sy, red.yy, red.ss};
    const int idx[5] = {ACC_G2, ACC_X2J, ACC_SY, ACC_YY, ACC_SS};
    block_sum_atomic<5>(v, acc + (int64_t)b * NACC, idx);
    const float wm = warp_max(red.gmax);
    if ((threadIdx.x & 31) == 0 && wm > 0.f) atomic_max_nonneg(acc + (int64_t)b * NACC + ACC_GMAX, (double)wm);
}

} // namespace

void launch_fwd_gather(const Problem &P, const uint8_t *X, const int32_t *list, int n,
                       const float *vecs, float *partial, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 grid((unsigned)((P.N + FWD_THREADS - 1) / FWD_THREADS), (unsigned)((n + FWD_G - 1) / FWD_G),
              (unsigned)P.Cg);
    k_fwd_gather<<<grid, FWD_THREADS, 0, st>>>(X, P.Lx, (int)P.N, (int)P.L, P.LC, list, n, vecs, P.Dp,
                                               reinterpret_cast<float4 *>(partial), P.Bmax, P.Nx);
}

void launch_fwd_exact(const Problem &P, const uint8_t *X, const int32_t *list, int n, const float *vecs,
                      double *partial64, double *lbase, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 grid((unsigned)((P.N + FWD_THREADS - 1) / FWD_THREADS), (unsigned)((n + EX_G - 1) / EX_G),
              (unsigned)P.Cg);
    k_fwd_gather_exact<<<grid, FWD_THREADS, 0, st>>>(X, P.Lx, (int)P.N, (int)P.L, P.LC, list, n, vecs, P.Dp,
                                                     reinterpret_cast<double4 *>(partial64), P.Bmax, P.Nx);
    dim3 g2((unsigned)((P.N + 255) / 256), (unsigned)n);
    k_reduce_partial64<<<g2, 256, 0, st>>>(reinterpret_cast<const double4 *>(partial64), (int)P.Cg, P.Bmax,
                                           P.Nx, (int)P.N, list, vecs, P.Dp, QQ * P.L, lbase);
}

void launch_reduce_partial(const Problem &P, const int32_t *list, int n, const float *partial,
                           const float *vecs, int add_h, float *out_f, double *out_d,
                           cudaStream_t st, int C, const float *R, double *acc)
{
    if (n <= 0) return;
    dim3 grid((unsigned)((P.N + 255) / 256), (unsigned)n);
    k_reduce_partial<<<grid, 256, 0, st>>>(reinterpret_cast<const float4 *>(partial), C > 0 ? C : (int)P.Cg,
                                           P.Bmax, P.Nx, (int)P.N, list, vecs, P.Dp, QQ * P.L, add_h,
                                           reinterpret_cast<float4 *>(out_f), out_d,
                                           reinterpret_cast<const float4 *>(R), acc);
}

void launch_grad_finalize(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                          const float *wa, float *gpool, void *Ypool, const void *Spool, int hist_bf16,
                          double *acc, cudaStream_t st)
{
    if (n <= 0) return;
    const int64_t need = (P.L + BWD_THREADS - 1) / BWD_THREADS;
    dim3 grid((unsigned)(need < 512 ? need : 512), (unsigned)n);
    k_grad_finalize<<<grid, BWD_THREADS, 0, st>>>((int)P.L, sd, list, wa, gpool, Ypool, Spool, hist_bf16,
                                                   P.ring, P.Dp, P.lambda_J, acc);
}

void launch_bwd_gather(const Problem &P, const uint8_t *XT, const SlotDev *sd,
                       const int32_t *list, int n, const float *R, const float *wa,
                       float *gpool, void *Ypool, const void *Spool, int hist_bf16,
                       double *acc, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 grid((unsigned)((P.L + BWD_THREADS - 1) / BWD_THREADS), (unsigned)((n + BWD_G - 1) / BWD_G));
    k_bwd_gather<<<grid, BWD_THREADS, 0, st>>>(XT, P.Nx, (int)P.N, (int)P.L, sd, list, n,
                                               reinterpret_cast<const float4 *>(R), wa, gpool, Ypool,
                                               Spool, hist_bf16, P.ring, P.Dp, P.lambda_J, acc);
}

} // namespace sdca
