// kernels_solver.cu -- per-slot solver kernels shared by every contraction
// form: line-search trials, iterate update, L-BFGS history and direction,
// and coupling scores.
//
// Line-search trials never run a contraction.  The logits of sequence i are
// affine in the step along d: l_i(stp) = lbase_i + stp * u_i with
// u_i = X_i . d_J + d_h, so a trial needs O(N q) work per slot.  This is
// exactly SuperDCA's objective along the search line (plmDCA_objective.hpp:
// 126-151 for the pseudo-likelihood part; the L2 part is a quadratic in stp
// that the host evaluates from x.d and d.d).
#include <algorithm>

#include "df.cuh"
#include "engine.h"
#include "kernels_common.cuh"

namespace sdca {

namespace {

constexpr int TRIAL_THREADS = 256;

// the direction's logits u and the base logits: float4 / FP64
__device__ __forceinline__ double4 load4(const float4 *u, int64_t o)
{
    const float4 v = u[o];
    return make_double4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ double4 load4(const double *v, int64_t o)
{
    const double2 a = reinterpret_cast<const double2 *>(v + o * 4)[0];
    const double2 b = reinterpret_cast<const double2 *>(v + o * 4)[1];
    return make_double4(a.x, a.y, b.x, b.y);
}

template <typename UT, typename LT>
__global__ void __launch_bounds__(TRIAL_THREADS)
k_trial(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int N, int64_t Nx,
        const LT *__restrict__ lbase, const UT *__restrict__ u,
        const uint8_t *__restrict__ rstate, const double *__restrict__ w, float4 *__restrict__ R,
        double *__restrict__ acc)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const double stp = S.stp;
    const bool use_u = S.flags & SLOT_F_USE_U;
    double f = 0, dg = 0, rs0 = 0, rs1 = 0, rs2 = 0, rs3 = 0;
    for (int i = blockIdx.x * TRIAL_THREADS + threadIdx.x; i < N; i += gridDim.x * TRIAL_THREADS) {
        const int64_t o = (int64_t)b * Nx + i;
        const double4 lb = load4(lbase, o);
        const double4 uu = use_u ? load4(u, o) : make_double4(0.0, 0.0, 0.0, 0.0);
        double l[4] = {lb.x + stp * uu.x, lb.y + stp * uu.y, lb.z + stp * uu.z, lb.w + stp * uu.w};
        const double mx = fmax(fmax(l[0], l[1]), fmax(l[2], l[3]));
        double e[4], z = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            e[a] = exp(l[a] - mx);
            z += e[a];
        }
        const double lse = mx + log(z);
        const int sr = rstate[o];
        const double wi = w[i];
        f += wi * (lse - l[sr]);
        double r[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) r[a] = wi * (e[a] / z) - (a == sr ? wi : 0.0);
        dg += r[0] * uu.x + r[1] * uu.y + r[2] * uu.z + r[3] * uu.w;
        rs0 += r[0]; rs1 += r[1]; rs2 += r[2]; rs3 += r[3];
        R[o] = make_float4((float)r[0], (float)r[1], (float)r[2], (float)r[3]);
    }
    double v[6] = {f, dg, rs0, rs1, rs2, rs3};
    const int idx[6] = {ACC_F, ACC_DG, ACC_RS0, ACC_RS1, ACC_RS2, ACC_RS3};
    block_sum_atomic<6>(v, acc + (int64_t)b * NACC, idx);
}

// x <- x + stp d; with a history push, s = x_new - x_old goes to ring_new.
__global__ void k_accept(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list,
                         int64_t Dp, int m, float *__restrict__ wa, const float *__restrict__ d,
                         void *__restrict__ Spool, int hist_bf16)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const float stp = (float)S.stp;
    const bool push = (S.flags & SLOT_F_PUSH) && S.ring_new >= 0;
    for (int64_t e = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); e < Dp;
         e += 4 * (int64_t)gridDim.x * blockDim.x) {
        float4 *xp = reinterpret_cast<float4 *>(wa + (int64_t)b * Dp + e);
        const float4 x = *xp;
        const float4 dv = *reinterpret_cast<const float4 *>(d + (int64_t)b * Dp + e);
        float4 xn;
        xn.x = fmaf(stp, dv.x, x.x);
        xn.y = fmaf(stp, dv.y, x.y);
        xn.z = fmaf(stp, dv.z, x.z);
        xn.w = fmaf(stp, dv.w, x.w);
        if (push)
            store_hist4(Spool, ((int64_t)b * m + S.ring_new) * Dp + e,
                        make_float4(xn.x - x.x, xn.y - x.y, xn.z - x.z, xn.w - x.w), hist_bf16);
        *xp = xn;
    }
}

__global__ void k_lbase_update(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list,
                               int N, int64_t Nx, double *__restrict__ lbase,
                               const float4 *__restrict__ u)
{
    const int b = list[blockIdx.y];
    const double stp = sd[b].stp;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || stp == 0.0) return;
    const int64_t o = (int64_t)b * Nx + i;
    const float4 uu = u[o];
    double *lb = lbase + o * 4;
    lb[0] += stp * uu.x;
    lb[1] += stp * uu.y;
    lb[2] += stp * uu.z;
    lb[3] += stp * uu.w;
}

// gradient of h_r: sum_i R_i + 2 lambda_h h (plmDCA_objective.hpp:149,198)
__global__ void k_hpart(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list,
                        int64_t L, int64_t Dp, int m, double lambda_h, const float *__restrict__ wa,
                        float *__restrict__ gpool, void *__restrict__ Ypool,
                        const void *__restrict__ Spool, int hist_bf16, double *__restrict__ acc)
{
    const int b = list[blockIdx.x];
    if (threadIdx.x != 0) return;
    const SlotDev &S = sd[b];
    const int64_t hoff = QQ * L;
    const float *x = wa + (int64_t)b * Dp + hoff;
    float *gn = gpool + (int64_t)(2 * b + 1 - S.gcur) * Dp + hoff;
    const float *go = gpool + (int64_t)(2 * b + S.gcur) * Dp + hoff;
    const bool push = (S.flags & SLOT_F_PUSH) && S.ring_new >= 0;
    double g2 = 0, x2 = 0, sy = 0, yy = 0, ss = 0, gmax = 0;
    float4 gv, yv;
    float *gp = &gv.x, *yp = &yv.x;
    for (int a = 0; a < 4; ++a) {
        const double g = S.rs[a] + 2.0 * lambda_h * (double)x[a];
        gp[a] = (float)g;
        gn[a] = gp[a];
        g2 += (double)gp[a] * gp[a];
        x2 += (double)x[a] * x[a];
        gmax = fmax(gmax, fabs((double)gp[a]));
        yp[a] = gp[a] - go[a];
    }
    if (push) {
        const int64_t off = ((int64_t)b * m + S.ring_new) * Dp + hoff;
        yv = store_hist4(Ypool, off, yv, hist_bf16);
        const float4 sv = load_hist4(Spool, off, hist_bf16);
        sy = (double)dot4(sv, yv);
        yy = (double)dot4(yv, yv);
        ss = (double)dot4(sv, sv);
    }
    double *A = acc + (int64_t)b * NACC;
    atomicAdd(A + ACC_G2, g2);
    atomicAdd(A + ACC_X2H, x2);
    if (push) {
        atomicAdd(A + ACC_SY, sy);
        atomicAdd(A + ACC_YY, yy);
        atomicAdd(A + ACC_SS, ss);
    }
    if (gmax > 0) atomic_max_nonneg(A + ACC_GMAX, gmax);
}

constexpr int DOT_THREADS = 256;
constexpr int DOT_U = 4;  // float4 groups per thread per tile: 16 KB runs per stream per block

// dots[b] = [S_j.g | Y_j.g | S_j.y_new | Y_j.y_new], j over the history.
// Blocks walk tiles of DOT_THREADS x DOT_U float4 groups; within a tile g and
// y_new stay in registers while the history vectors stream through one at a
// time, so every stream is read in long contiguous runs.
__global__ void __launch_bounds__(DOT_THREADS)
k_hist_dots(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int64_t Dp, int m,
            const float *__restrict__ gpool, const void *__restrict__ Spool,
            const void *__restrict__ Ypool, int hist_bf16, double *__restrict__ dots)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const int nh = S.nhist;
    const float4 *g4 = reinterpret_cast<const float4 *>(gpool + (int64_t)(2 * b + S.gcur) * Dp);
    const bool has_new = S.ring_new >= 0;
    const int64_t ybase = ((int64_t)b * m + (has_new ? S.ring_new : 0)) * Dp;
    const int64_t nv4 = Dp / 4, tile = (int64_t)DOT_THREADS * DOT_U;
    float aSg[MAXHIST], aYg[MAXHIST], aSy[MAXHIST], aYy[MAXHIST];
#pragma unroll
    for (int j = 0; j < MAXHIST; ++j) aSg[j] = aYg[j] = aSy[j] = aYy[j] = 0.f;
    for (int64_t tb = (int64_t)blockIdx.x * tile; tb < nv4; tb += (int64_t)gridDim.x * tile) {
        float4 gv[DOT_U], yn[DOT_U];
#pragma unroll
        for (int u = 0; u < DOT_U; ++u) {
            const int64_t v = tb + u * DOT_THREADS + threadIdx.x;
            const bool ok = v < nv4;
            gv[u] = ok ? g4[v] : make_float4(0.f, 0.f, 0.f, 0.f);
            yn[u] = (ok && has_new) ? load_hist4(Ypool, ybase + 4 * v, hist_bf16) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < MAXHIST; ++j) {
            if (j < nh) {
                const int64_t base = ((int64_t)b * m + S.ring[j]) * Dp;
                float4 sv[DOT_U], yv[DOT_U];
#pragma unroll
                for (int u = 0; u < DOT_U; ++u) {
                    const int64_t v = tb + u * DOT_THREADS + threadIdx.x;
                    const bool ok = v < nv4;
                    sv[u] = ok ? load_hist4(Spool, base + 4 * v, hist_bf16) : make_float4(0.f, 0.f, 0.f, 0.f);
                    yv[u] = ok ? load_hist4(Ypool, base + 4 * v, hist_bf16) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < DOT_U; ++u) {
                    aSg[j] += dot4(sv[u], gv[u]);
                    aYg[j] += dot4(yv[u], gv[u]);
                    aSy[j] += dot4(sv[u], yn[u]);
                    aYy[j] += dot4(yv[u], yn[u]);
                }
            }
        }
    }
    float v[4 * MAXHIST];
    int idx[4 * MAXHIST];
#pragma unroll
    for (int j = 0; j < MAXHIST; ++j) {
        v[j] = aSg[j];
        v[MAXHIST + j] = aYg[j];
        v[2 * MAXHIST + j] = aSy[j];
        v[3 * MAXHIST + j] = aYy[j];
    }
#pragma unroll
    for (int k = 0; k < 4 * MAXHIST; ++k) idx[k] = k;
    block_sum_atomic_f<4 * MAXHIST>(v, dots + (int64_t)b * 4 * MAXHIST, idx);
}

// d = coef_g g + sum_j (coefS_j s_j + coefY_j y_j), J_rr block zero;
// reductions g.d, d.d and x.d split into the J and h parts, and max|d|.
// Same tiling as k_hist_dots: d and g of a tile stay in registers while the
// history streams through.
__global__ void __launch_bounds__(DOT_THREADS)
k_direction(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int64_t L,
            int64_t Dp, int m, const float *__restrict__ gpool, const void *__restrict__ Spool,
            const void *__restrict__ Ypool, int hist_bf16, const float *__restrict__ wa,
            float *__restrict__ d, double *__restrict__ acc)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const int nh = S.nhist;
    const float4 *g4 = reinterpret_cast<const float4 *>(gpool + (int64_t)(2 * b + S.gcur) * Dp);
    const float4 *x4 = reinterpret_cast<const float4 *>(wa + (int64_t)b * Dp);
    float4 *d4 = reinterpret_cast<float4 *>(d + (int64_t)b * Dp);
    const float cg = (float)S.coef_g;
    const int64_t hoff4 = QQ * L / 4;
    const int64_t rlo4 = (int64_t)S.locus * QQ / 4, rhi4 = rlo4 + QQ / 4;
    const int64_t nv4 = Dp / 4, tile = (int64_t)DOT_THREADS * DOT_U;
    float gd = 0.f, ddJ = 0.f, ddH = 0.f, xdJ = 0.f, xdH = 0.f, dmax = 0.f;
    for (int64_t tb = (int64_t)blockIdx.x * tile; tb < nv4; tb += (int64_t)gridDim.x * tile) {
        float4 gv[DOT_U], dv[DOT_U];
#pragma unroll
        for (int u = 0; u < DOT_U; ++u) {
            const int64_t v = tb + u * DOT_THREADS + threadIdx.x;
            gv[u] = v < nv4 ? g4[v] : make_float4(0.f, 0.f, 0.f, 0.f);
            dv[u] = make_float4(cg * gv[u].x, cg * gv[u].y, cg * gv[u].z, cg * gv[u].w);
        }
#pragma unroll
        for (int j = 0; j < MAXHIST; ++j) {
            if (j < nh) {
                const int64_t base = ((int64_t)b * m + S.ring[j]) * Dp;
                const float cs = (float)S.coefS[j], cy = (float)S.coefY[j];
                float4 sv[DOT_U], yv[DOT_U];
#pragma unroll
                for (int u = 0; u < DOT_U; ++u) {
                    const int64_t v = tb + u * DOT_THREADS + threadIdx.x;
                    const bool ok = v < nv4;
                    sv[u] = ok ? load_hist4(Spool, base + 4 * v, hist_bf16) : make_float4(0.f, 0.f, 0.f, 0.f);
                    yv[u] = ok ? load_hist4(Ypool, base + 4 * v, hist_bf16) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < DOT_U; ++u) {
                    dv[u].x += cs * sv[u].x + cy * yv[u].x;
                    dv[u].y += cs * sv[u].y + cy * yv[u].y;
                    dv[u].z += cs * sv[u].z + cy * yv[u].z;
                    dv[u].w += cs * sv[u].w + cy * yv[u].w;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < DOT_U; ++u) {
            const int64_t v = tb + u * DOT_THREADS + threadIdx.x;
            if (v >= nv4) continue;
            if (v >= rlo4 && v < rhi4) dv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            d4[v] = dv[u];
            const float4 xv = x4[v];
            gd += dot4(gv[u], dv[u]);
            dmax = fmaxf(dmax, fmaxf(fmaxf(fabsf(dv[u].x), fabsf(dv[u].y)), fmaxf(fabsf(dv[u].z), fabsf(dv[u].w))));
            if (v < hoff4) {
                ddJ += dot4(dv[u], dv[u]);
                xdJ += dot4(xv, dv[u]);
            } else {
                ddH += dot4(dv[u], dv[u]);
                xdH += dot4(xv, dv[u]);
            }
        }
    }
    float v[5] = {gd, ddJ, ddH, xdJ, xdH};
    const int idx[5] = {ACC_GD, ACC_DDJ, ACC_DDH, ACC_XDJ, ACC_XDH};
    block_sum_atomic_f<5>(v, acc + (int64_t)b * NACC, idx);
    const float wm = warp_max(dmax);
    if ((threadIdx.x & 31) == 0 && wm > 0.f) atomic_max_nonneg(acc + (int64_t)b * NACC + ACC_DMAX, (double)wm);
}

// S[r][n] = || gauge(M) ||_F without GAP, M = J_rn (transposed for n < r):
// SuperDCA/include/plmDCA.hpp:378-393, plmDCA_utility.hpp:57-83,
// Matrix_math.hpp:166-213.  G[i][j] = ((M[i][j] - rowmean(M)[j]) -
// colmean(M)[i]) + mean(rowmean(M)), evaluated in FP64 like the reference.
__global__ void k_score(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list,
                        int64_t L, int64_t Dp, const float *__restrict__ wa, int gap,
                        float *__restrict__ rows)
{
    const int k = blockIdx.y;
    const int b = list[k];
    const int64_t r = sd[b].locus;
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= L) return;
    float *row = rows + (int64_t)k * L;
    if (n == r) {
        row[n] = __int_as_float(0x7fc00000);
        return;
    }
    const float4 *jp = reinterpret_cast<const float4 *>(wa + (int64_t)b * Dp + n * QQ);
    // single precision: the block is stored in FP32 and the score is written
    // as FP32 (GB300's FP64 rate is a small fraction of its FP32 rate)
    float J[4][4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const float4 v = jp[s];
        const float t[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (n < r) J[a][s] = t[a];
            else J[s][a] = t[a];
        }
    }
    float rm[4], cm[4], gm = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float t = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) t = t + J[i][j];
        rm[i] = t * 0.25f;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float t = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) t = t + J[i][j];
        cm[j] = t * 0.25f;
    }
    {
        float t = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) t += rm[i];
        gm = t * 0.25f;
    }
    float sum = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i == gap) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j == gap) continue;
            const float gij = ((J[i][j] - rm[j]) - cm[i]) + gm;
            sum = fmaf(gij, gij, sum);
        }
    }
    row[n] = sqrtf(sum);
}

// blocks per slot for the D-length passes: at most `cap`, so that every
// thread streams many float4 before the per-block reduction
unsigned dgrid(int64_t Dp, int threads, int64_t cap = 256)
{
    const int64_t need = (Dp / 4 + threads - 1) / threads;
    return (unsigned)(need < cap ? need : cap);
}

} // namespace

void launch_trial(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                  const double *lbase, const float *u, const uint8_t *rstate, const double *w,
                  float *R, double *acc, cudaStream_t st)
{
    if (n <= 0) return;
    int gx = (int)((P.N + TRIAL_THREADS - 1) / TRIAL_THREADS);
    if (gx > 32) gx = 32;
    dim3 grid((unsigned)gx, (unsigned)n);
    k_trial<float4, double><<<grid, TRIAL_THREADS, 0, st>>>(sd, list, (int)P.N, P.Nx, lbase,
                                                    reinterpret_cast<const float4 *>(u), rstate, w,
                                                    reinterpret_cast<float4 *>(R), acc);
}

void launch_accept(const Problem &P, const SlotDev *sd, const int32_t *list, int n, float *wa,
                   const float *d, void *Spool, int hist_bf16, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 grid(dgrid(P.Dp, 256), (unsigned)n);
    k_accept<<<grid, 256, 0, st>>>(sd, list, P.Dp, P.ring, wa, d, Spool, hist_bf16);
}

void launch_lbase_update(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                         double *lbase, const float *u, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 grid((unsigned)((P.N + 255) / 256), (unsigned)n);
    k_lbase_update<<<grid, 256, 0, st>>>(sd, list, (int)P.N, P.Nx, lbase,
                                         reinterpret_cast<const float4 *>(u));
}

void launch_hpart(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                  const float *wa, float *gpool, void *Ypool, const void *Spool, int hist_bf16,
                  double *acc, cudaStream_t st)
{
    if (n <= 0) return;
    k_hpart<<<n, 32, 0, st>>>(sd, list, P.L, P.Dp, P.ring, P.lambda_h, wa, gpool, Ypool, Spool,
                              hist_bf16, acc);
}

void launch_hist_dots(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                      const float *gpool, const void *Spool, const void *Ypool, int hist_bf16,
                      double *dots, cudaStream_t st)
{
    if (n <= 0) return;
    // enough blocks for about two waves in total, each thread streaming
    // hundreds of float4 before the block reduction
    const int64_t per_slot = std::max<int64_t>(4, std::min<int64_t>(64, (4 * 152 + n - 1) / n));
    dim3 grid(dgrid(P.Dp, DOT_THREADS * DOT_U, per_slot), (unsigned)n);
    k_hist_dots<<<grid, DOT_THREADS, 0, st>>>(sd, list, P.Dp, P.ring, gpool, Spool, Ypool, hist_bf16,
                                              dots);
}

void launch_direction(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                      const float *gpool, const void *Spool, const void *Ypool, int hist_bf16,
                      const float *wa, float *d, double *acc, cudaStream_t st)
{
    if (n <= 0) return;
    const int64_t per_slot = std::max<int64_t>(4, std::min<int64_t>(128, (4 * 152 + n - 1) / n));
    dim3 grid(dgrid(P.Dp, DOT_THREADS * DOT_U, per_slot), (unsigned)n);
    k_direction<<<grid, DOT_THREADS, 0, st>>>(sd, list, P.L, P.Dp, P.ring, gpool, Spool, Ypool,
                                              hist_bf16, wa, d, acc);
}

void launch_score(const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                  const float *wa, int gap, float *rows, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 grid((unsigned)((P.L + 127) / 128), (unsigned)n);
    k_score<<<grid, 128, 0, st>>>(sd, list, P.L, P.Dp, wa, gap, rows);
}

} // namespace sdca
