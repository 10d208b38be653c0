// kernels_dual.cu -- the per-locus solve in the span of the sequences.
//
// For target locus r let phi_i be sequence i's one-hot features over the
// loci n != r (4 per locus).  The logits are l_i = h + J^T phi_i, and from
// x = 0 every L-BFGS vector of SuperDCA's solve (gradient, direction, steps,
// gradient differences) has the form v = (Phi^T a_v, eta_v) with a_v an
// N x 4 coefficient matrix and eta_v a 4-vector: the J gradient is
// Phi^T rho + 2 lambda_J J with rho_i = w_i (p_i - onehot(s_i(r))), and the
// iteration only forms linear combinations.  With K = Phi Phi^T
// (K_ij = number of loci n != r where s_i(n) = s_j(n)) a vector's logit
// image is K a_v + eta_v and inner products are a_v . K a_w + eta_v . eta_w.
// So the same iteration runs on N x 4 coefficients; a vector is kept as the
// pair (a, k = K a) in double-float (df.cuh: ~48 bits on the FP32 pipe) and
// its eta (4 values, FP64) in the slot's device state (DualCtl).
//
// The one product per iteration, K rho, is exact: rho is rounded to integers
// rho_q = round(rho * 2^QB / w_max) (the rounded value is the one used, so
// the pair (a, K a) stays consistent), K is an integer matrix, and the sums
// are taken in 64-bit integers; QB keeps them below 2^62.  K = K_all minus
// the agreement at r itself, a class sum per state of r.
#include <cstdint>
#include <cstdlib>
#include <new>

#include "df.cuh"
#include "engine.h"
#include "kernels_common.cuh"
#include "lbfgs_host.h"
#include "linesearch.h"

namespace sdca {
namespace {

__global__ void k_dual_kmat(const int32_t *__restrict__ dist, int N, int64_t Nx, int L, int32_t *__restrict__ K)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < Nx * Nx; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Nx, j = t % Nx;
        K[t] = (i < N && j < N) ? L - dist[i * N + j] : 0;
    }
}

// rho_q = round(R * qscale) (R is FP32, so a single-precision product loses
// nothing: the rounded value is the one every later step uses), with the
// entry at the sequence's own state set to minus the sum of the other three,
// so that every row sums to zero exactly (a residual w (p - onehot) does; the
// K rho product then needs three columns); class sums csum[b][a][c] = sum
// over i with s_i(r) = a
__global__ void __launch_bounds__(256)
k_dual_quant(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int N, int64_t Nx,
             const float4 *__restrict__ R, const uint8_t *__restrict__ rstate, float qscale, int4 *__restrict__ rq,
             unsigned long long *__restrict__ csum, const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.y >= *cnt) return;
    const int b = list[blockIdx.y];
    const bool own = sd[b].locus >= 0;   // scan mode: no own-agreement correction
    __shared__ unsigned long long red[16];
    if (threadIdx.x < 16) red[threadIdx.x] = 0ull;
    __syncthreads();
    long long cs[4][4] = {};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x) {
        int4 q = make_int4(0, 0, 0, 0);
        if (i < N) {
            const float4 v = R[(int64_t)b * Nx + i];
            q = make_int4(__float2int_rn(v.x * qscale), __float2int_rn(v.y * qscale), __float2int_rn(v.z * qscale),
                          __float2int_rn(v.w * qscale));
            const int ys = rstate[(int64_t)b * Nx + i] & 3;
            if (ys == 0) q.x = -(q.y + q.z + q.w);
            else if (ys == 1) q.y = -(q.x + q.z + q.w);
            else if (ys == 2) q.z = -(q.x + q.y + q.w);
            else q.w = -(q.x + q.y + q.z);
            const int y = own ? ys : -1;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                if (a != y) continue;
                cs[a][0] += q.x; cs[a][1] += q.y; cs[a][2] += q.z; cs[a][3] += q.w;
            }
        }
        rq[(int64_t)b * Nx + i] = q;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            long long v = cs[a][c];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(&red[a * 4 + c], (unsigned long long)v);
        }
    __syncthreads();
    if (threadIdx.x < 16 && red[threadIdx.x] != 0ull) atomicAdd(csum + (int64_t)b * 16 + threadIdx.x, red[threadIdx.x]);
}

constexpr int KP_M = 64;   // rows (sequences i) per CTA
constexpr int KP_S = 16;   // slots per CTA (64 columns: 16 slots x 4 states)
constexpr int KP_J = 16;   // sequences j per shared-memory stage

// KR[b][i][c] = (sum_j K_ij rho_q[b][j][c] - csum[b][s_i(r)][c]) / qscale
__global__ void __launch_bounds__(256)
k_dual_kprod(const int32_t *__restrict__ K, int64_t Nx, int N, const int32_t *__restrict__ list, int nlist,
             const int4 *__restrict__ rq, const long long *__restrict__ csum, const uint8_t *__restrict__ rstate,
             double inv_qscale, float2 *__restrict__ KR, const int *__restrict__ cnt)
{
    if (cnt) {
        nlist = *cnt;
        if ((int)blockIdx.y * KP_S >= nlist) return;
    }
    __shared__ __align__(16) int32_t sK[KP_J][KP_M];
    __shared__ __align__(16) int32_t sR[KP_J][KP_S * 4];
    const int t = threadIdx.x;
    const int ty = t >> 4, tx = t & 15;
    const int64_t i0 = (int64_t)blockIdx.x * KP_M;
    const int s0 = blockIdx.y * KP_S;
    const int my_slot = (s0 + tx < nlist) ? list[s0 + tx] : -1;
    const int ld_jj = t >> 4, ld_part = t & 15;
    const int ld_slot = my_slot;  // the loader of sR row ld_jj, slot column ld_part = tx
    long long acc[4][4] = {};
    for (int64_t j0 = 0; j0 < Nx; j0 += KP_J) {
        *reinterpret_cast<int4 *>(&sK[ld_jj][ld_part * 4]) =
            *reinterpret_cast<const int4 *>(K + (j0 + ld_jj) * Nx + i0 + ld_part * 4);
        int4 rv = make_int4(0, 0, 0, 0);
        if (ld_slot >= 0) rv = rq[(int64_t)ld_slot * Nx + j0 + ld_jj];
        *reinterpret_cast<int4 *>(&sR[ld_jj][ld_part * 4]) = rv;
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < KP_J; ++jj) {
            const int4 kv = *reinterpret_cast<const int4 *>(&sK[jj][ty * 4]);
            const int4 r4 = *reinterpret_cast<const int4 *>(&sR[jj][tx * 4]);
            const int k[4] = {kv.x, kv.y, kv.z, kv.w};
            const int r[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[a][c] += (long long)k[a] * (long long)r[c];
        }
        __syncthreads();
    }
    if (my_slot < 0) return;
    const int b = my_slot;
    const float2 iq = df_from_d(inv_qscale);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int64_t i = i0 + ty * 4 + a;
        float2 *o = KR + ((int64_t)b * Nx + i) * 4;
        if (i >= N) {
            o[0] = o[1] = o[2] = o[3] = df_zero();
            continue;
        }
        const int y = rstate[(int64_t)b * Nx + i] & 3;
        const long long *cs = csum + (int64_t)b * 16 + y * 4;
#pragma unroll
        for (int c = 0; c < 4; ++c) o[c] = df_mul(df_from_ll(acc[a][c] - cs[c]), iq);
    }
}

__device__ __forceinline__ int64_t dvo(int64_t b, int v, int part, int NV, int64_t Nx)
{
    return (((b * NV + v) * 2 + part) * Nx) * 4;
}

// two consecutive double-float entries (t: the pair's index) in one 16-byte access
__device__ __forceinline__ void df2_load(const float2 *p, int64_t t, float2 (&v)[2])
{
    const float4 q = reinterpret_cast<const float4 *>(p)[t];
    v[0] = make_float2(q.x, q.y);
    v[1] = make_float2(q.z, q.w);
}

__device__ __forceinline__ void df2_store(float2 *p, int64_t t, const float2 (&v)[2])
{
    reinterpret_cast<float4 *>(p)[t] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
}

// The accept of a slot that searched this round and the gradient pass at
// its new point, in one pass over the slot's vectors (a slot entering
// with its start point has no accept):
//   accept: x += stp d (a and k parts), s = x_new - x_old into the history
//   on a push (the logits k_x + eta_x follow with x);
//   gradient (a, k) = (rho_q / qscale + 2 lambda_J a_x, K rho + 2 lambda_J k_x),
//   y = g_new - g_old into the history on a push;
//   J-part sums: g.g, x.x, s.y, y.y, s.s; max |a_g| and max |a_x|.
// Nothing between the line search and this kernel reads x of a searching
// slot (the residual quantiser and K rho take the search's R rows), so the
// accept can wait until here.
__global__ void __launch_bounds__(256)
k_dual_grad(const DualCtl *__restrict__ ctl, const int32_t *__restrict__ list, int64_t Nx, int NV, int ring,
            float2 l2, const int32_t *__restrict__ rq, float2 iq, const float2 *__restrict__ KR,
            float2 *__restrict__ dv, double *__restrict__ acc, double *__restrict__ amax,
            const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.y >= *cnt) return;
    const int b = list[blockIdx.y];
    const DualCtl &S = ctl[b];
    if (S.phase == DC_STOP) return;
    const bool step = S.phase == DC_STEP;   // searched this round: accept first
    const bool push = S.push && S.ring_new >= 0;
    const float2 sf = S.stp_df;
    // the slot's vectors as entry pairs (float4) from one base, each part at
    // a 32-bit offset (a part; its k part follows at + P): fewer registers
    // than a pointer per stream, so more blocks fit on an SM
    const int P = (int)(Nx * 2);
    float4 *base = reinterpret_cast<float4 *>(dv + dvo(b, 0, 0, NV, Nx));
    const int ps = push ? S.ring_new : 0;
    const int o_x = DV_X * 2 * P, o_d = DV_D * 2 * P, o_go = (DV_G + S.gcur) * 2 * P,
              o_gn = (DV_G + 1 - S.gcur) * 2 * P, o_s = (DV_S + ps) * 2 * P, o_y = (DV_S + ring + ps) * 2 * P;
    const int2 *rq2 = reinterpret_cast<const int2 *>(rq + (int64_t)b * Nx * 4);
    const float4 *KRb = reinterpret_cast<const float4 *>(KR + (int64_t)b * Nx * 4);
    auto ld = [&](int o, int t, float2 (&v)[2]) {
        const float4 q = base[o + t];
        v[0] = make_float2(q.x, q.y);
        v[1] = make_float2(q.z, q.w);
    };
    auto st = [&](int o, int t, const float2 (&v)[2]) { base[o + t] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y); };
    float2 g2 = df_zero(), x2 = df_zero(), sy = df_zero(), yy = df_zero(), ss = df_zero();
    float mg = 0.f, mx = 0.f;
    // entry pairs (2t, 2t+1): 16-byte loads of every stream
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < P; t += gridDim.x * blockDim.x) {
        float2 a_x[2], k_x[2], kr[2], a_g[2], k_g[2], a_s[2], k_s[2];
        ld(o_x, t, a_x);
        ld(o_x + P, t, k_x);
        {
            const float4 q = KRb[t];
            kr[0] = make_float2(q.x, q.y);
            kr[1] = make_float2(q.z, q.w);
        }
        const int2 r2 = rq2[t];
        const int rr[2] = {r2.x, r2.y};
        if (step) {
            float2 a_d[2], k_d[2];
            ld(o_d, t, a_d);
            ld(o_d + P, t, k_d);
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float2 a1 = df_fma(sf, a_d[q], a_x[q]), k1 = df_fma(sf, k_d[q], k_x[q]);
                a_s[q] = df_sub(a1, a_x[q]);
                k_s[q] = df_sub(k1, k_x[q]);
                a_x[q] = a1;
                k_x[q] = k1;
            }
            st(o_x, t, a_x);
            st(o_x + P, t, k_x);
            if (push) {
                st(o_s, t, a_s);
                st(o_s + P, t, k_s);
            }
        } else if (push) {
            ld(o_s, t, a_s);
            ld(o_s + P, t, k_s);
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            a_g[q] = df_fma(l2, a_x[q], df_mul(df_from_int(rr[q]), iq));
            k_g[q] = df_fma(l2, k_x[q], kr[q]);
            g2 = df_fma(a_g[q], k_g[q], g2);
            x2 = df_fma(a_x[q], k_x[q], x2);
            mg = fmaxf(mg, fabsf(a_g[q].x));
            mx = fmaxf(mx, fabsf(a_x[q].x));
        }
        if (push) {
            float2 a_o[2], k_o[2], a_y[2], k_y[2];
            ld(o_go, t, a_o);
            ld(o_go + P, t, k_o);
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                a_y[q] = df_sub(a_g[q], a_o[q]);
                k_y[q] = df_sub(k_g[q], k_o[q]);
                sy = df_fma(a_s[q], k_y[q], sy);
                yy = df_fma(a_y[q], k_y[q], yy);
                ss = df_fma(a_s[q], k_s[q], ss);
            }
            st(o_y, t, a_y);
            st(o_y + P, t, k_y);
        }
        st(o_gn, t, a_g);
        st(o_gn + P, t, k_g);
    }
    float2 v[5] = {g2, x2, sy, yy, ss};
    const int idx[5] = {ACC_G2, ACC_X2J, ACC_SY, ACC_YY, ACC_SS};
    block_sum_df<5>(v, acc + (int64_t)b * NACC, idx);
    mg = warp_max(mg);
    mx = warp_max(mx);
    if ((threadIdx.x & 31) == 0) {
        if (mg > 0.f) atomic_max_nonneg(amax + 2 * b, (double)mg);
        if (mx > 0.f) atomic_max_nonneg(amax + 2 * b + 1, (double)mx);
    }
}

// J-part dots of the live history pairs (and the pair the last accept
// pushed) with a gradient, stored by ring position p: dots[b][p] =
// a_sp . k_g, dots[b][DOT_Y + p] = a_yp . k_g.  newg: the gradient just
// formed (buffer 1 - gcur) instead of the accepted one.  (The dots with the
// newest y follow in the control kernel from these and the previous
// iteration's: S^T y = S^T g - S^T g_old.)
// A block takes DOT_CHUNK entries of one slot: k_g staged in shared memory;
// the work is cut into (history vector, quarter of the chunk) units, taken
// by the warps in turn, so every warp gets the same number of units whatever
// the history length (8k units for 8 warps); 16-byte loads, eight in flight
// per lane, one accumulator per lane.
constexpr int DOT_CHUNK = 2048;
constexpr int DOT_SUBS = 4;                       // units per vector and chunk
constexpr int DOT_SUB_Q = DOT_CHUNK / 2 / DOT_SUBS;   // float4 pairs per unit (256)

__global__ void __launch_bounds__(256)
k_dual_dots(const DualCtl *__restrict__ ctl, const int32_t *__restrict__ list, int64_t Nx, int NV, int ring,
            int newg, const float2 *__restrict__ dv, double *__restrict__ dots, const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.y >= *cnt) return;
    const int b = list[blockIdx.y];
    const DualCtl &S = ctl[b];
    if (S.phase == DC_STOP) return;
    // the live history and the pair the last accept pushed
    const bool pushed = S.push && S.ring_new >= 0;
    const int k = S.nhist + (pushed ? 1 : 0);
    const int64_t E = Nx * 4, e0 = (int64_t)blockIdx.x * DOT_CHUNK;
    const int ne = E - e0 < DOT_CHUNK ? (int)(E - e0) : DOT_CHUNK;   // a multiple of 4 (Nx is of 64)
    const int nq = ne / 2;                                            // float4 pairs
    __shared__ float4 g[DOT_CHUNK / 2];
    const float2 *kg = dv + dvo(b, DV_G + (newg ? 1 - S.gcur : S.gcur), 1, NV, Nx) + e0;   // (gcur flips in the control kernel)
    for (int t = threadIdx.x; t < nq; t += blockDim.x) g[t] = reinterpret_cast<const float4 *>(kg)[t];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int u = warp; u < 2 * k * DOT_SUBS; u += nw) {
        const int qv = u / DOT_SUBS, t0 = (u % DOT_SUBS) * DOT_SUB_Q;
        const bool isy = qv >= k;
        const int j = isy ? qv - k : qv;
        const int pos = j < S.nhist ? S.hist[j] : S.ring_new;
        const float4 *v = reinterpret_cast<const float4 *>(dv + dvo(b, DV_S + (isy ? ring : 0) + pos, 0, NV, Nx) + e0);
        const int t1 = min(nq, t0 + DOT_SUB_Q);
        float2 acc = df_zero();
#pragma unroll 8
        for (int t = t0 + lane; t < t1; t += 32) {
            const float4 x = v[t], y = g[t];
            acc = df_fma(make_float2(x.x, x.y), make_float2(y.x, y.y), acc);
            acc = df_fma(make_float2(x.z, x.w), make_float2(y.z, y.w), acc);
        }
        const float2 sum = df_warp_sum(acc);
        if (lane == 0 && (sum.x != 0.f || sum.y != 0.f))
            atomicAdd(dots + (int64_t)b * 4 * MAXHIST + (isy ? DOT_Y : 0) + pos, df_to_d(sum));
    }
}

// A step trial of one sequence with a large step (|t| >= 30), from its
// double-float logits without FP64 arithmetic: l0 = k_x + eta_x,
// u = k_d + eta_d, l1 = l0 + stp u in double-float, each log-sum-exp shifted by its largest high part and taken
// in FP32 (the shifted terms are O(1)), the change of w (lse(l) - l_y)
// assembled in double-float.  Returns the change of w (lse - l_y), the
// slope change and the residual row r (by value: nothing of the common path
// has to live in memory for this rare call).
struct BigTrial {
    float4 r;
    float2 df, ddg;
};

__device__ __noinline__ BigTrial trial_big(const float2 *kx, const float2 *kd, const float2 *ex, const float2 *ed,
                                           float2 stp, int y, float wi, float4 p0v)
{
    const float p0[4] = {p0v.x, p0v.y, p0v.z, p0v.w};
    float r[4];
    float2 fbig = df_zero(), dgbig = df_zero();
    float2 l0[4], l1[4], uu[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        l0[a] = df_add(kx[a], ex[a]);
        uu[a] = df_add(kd[a], ed[a]);
        l1[a] = df_fma(stp, uu[a], l0[a]);
    }
    const float m0 = fmaxf(fmaxf(l0[0].x, l0[1].x), fmaxf(l0[2].x, l0[3].x));
    const float m1 = fmaxf(fmaxf(l1[0].x, l1[1].x), fmaxf(l1[2].x, l1[3].x));
    float z0 = 0.f, z1 = 0.f, e1[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        z0 += expf(df_f(df_sub(l0[a], make_float2(m0, 0.f))));
        e1[a] = expf(df_f(df_sub(l1[a], make_float2(m1, 0.f))));
        z1 += e1[a];
    }
    float2 l0y = l0[0], l1y = l1[0], uy = uu[0];
#pragma unroll
    for (int a = 1; a < 4; ++a)
        if (a == y) {
            l0y = l0[a];
            l1y = l1[a];
            uy = uu[a];
        }
    float2 d = df_sub(df_sub(make_float2(m1, 0.f), l1y), df_sub(make_float2(m0, 0.f), l0y));
    d = df_add(d, make_float2(logf(z1) - logf(z0), 0.f));
    fbig = df_fma(make_float2(wi, 0.f), d, fbig);
    const float iz1 = 1.f / z1;
    float ro = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const float p1 = e1[a] * iz1;
        dgbig = df_fma(make_float2(wi * (p1 - p0[a]), 0.f), df_sub(uu[a], uy), dgbig);
        const float ra = a == y ? 0.f : wi * p1;
        r[a] = ra;
        ro += ra;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
        if (a == y) r[a] = -ro;
    BigTrial o;
    o.r = make_float4(r[0], r[1], r[2], r[3]);
    o.df = fbig;
    o.ddg = dgbig;
    return o;
}

// A line-search trial as a change from the current point.  With p0 the base
// probabilities (computed from the logits at the current point), y the
// sequence's state at r and t_a = stp (u_a - u_y), per sequence
//   l(stp) - l(0) = log(Z),  Z = sum_a p0_a exp(t_a) = 1 + q,
//   q = sum_a p0_a expm1(t_a),  p_a(stp) = p0_a exp(t_a) / Z,
// and the slope changes by sum_a w (p_a(stp) - p0_a) (u_a - u_y), with
// p_a(stp) - p0_a = p0_a (expm1(t_a) - q) / Z.  Every term is a difference
// from the sequence's own state, so single precision gives the change with
// ~1e-7 relative error of the change itself, which is what the line search
// compares; the base values (objective, slope at 0) are FP64.  Z is a sum of
// positive terms and the new probabilities are products, so a probability
// that has become small keeps its relative precision.  Sequences whose step
// is large take a log-sum-exp of the double-float logits (trial_big).  Per trial:
// the sums of w dl, of the slope change and of R(stp), and the rows
// R <- R(stp) = w (p(stp) - onehot(y)), the y entry as minus the sum of the
// others (trial_seq, in the line-search kernel below).
// d = coef_g g + sum_j coefS_j s_j + coefY_j y_j (a and k parts); the trial
// logits direction u = k_d + eta_d, kept only as its single-precision
// differences u - u_y; the base probabilities P0 of the step trials from the
// double-float logits k_x + eta_x at the current point (fresh every iteration,
// so that rounding does not carry from one iteration to the next); sums g.d,
// d.d, x.d (J parts) and the slope of the search line at 0 from the trials'
// own numbers, sum_i w_i sum_c p0_ic (u_ic - u_iy).
// Each thread takes two consecutive entries (16-byte loads of every stream);
// a sequence's four states sit in a lane pair.  History loads of two vectors
// are issued before their multiply-adds.  One pass per thread: the grid
// covers the slot's N x 4 entries.
constexpr int DIR_THREADS = 256;

__global__ void __launch_bounds__(DIR_THREADS, 5)
k_dual_direction(const DualCtl *__restrict__ ctl, const int32_t *__restrict__ list, int64_t Nx, int N, int NV,
                 int ring, float2 *__restrict__ dv, float *__restrict__ P0, const float *__restrict__ w,
                 const uint8_t *__restrict__ rstate, float *__restrict__ ud, double *__restrict__ dacc,
                 const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.y >= *cnt) return;
    const int b = list[blockIdx.y];
    const DualCtl &S = ctl[b];
    if (S.phase == DC_STOP) return;
    const int k = S.nhist;
    __shared__ float2 cf[2 * MAXHIST + 1 + Q];   // the slot's coefficients and eta_d (double-float)
    __shared__ float2 ex[Q];                     // eta_x (double-float): logits = k_x + eta_x
    __shared__ int64_t hoff[2 * MAXHIST];        // history vector offsets (a parts; k part at + Nx*4)
    if (threadIdx.x < 2 * MAXHIST + 1 + Q) cf[threadIdx.x] = S.cdf[threadIdx.x];
    if (threadIdx.x < Q) ex[threadIdx.x] = df_from_d(S.eta_x[threadIdx.x]);
    if (threadIdx.x < k) {
        hoff[threadIdx.x] = dvo(b, DV_S + S.hist[threadIdx.x], 0, NV, Nx);
        hoff[MAXHIST + threadIdx.x] = dvo(b, DV_S + ring + S.hist[threadIdx.x], 0, NV, Nx);
    }
    __syncthreads();
    const int64_t part = Nx * 4;                 // a part -> k part, in float2 entries
    const int64_t t = (int64_t)blockIdx.x * DIR_THREADS + threadIdx.x;   // entry pair: entries 2t, 2t+1
    const bool live = t < Nx * 2;
    float2 gd = df_zero(), dd = df_zero(), xd = df_zero(), dg0 = df_zero();
    // (the whole warp reaches the shuffles below: Nx*2 is a multiple of 128)
    if (live) {
        const float2 *ag = dv + dvo(b, DV_G + S.gcur, 0, NV, Nx), *kg = ag + part;
        const float2 *ax = dv + dvo(b, DV_X, 0, NV, Nx);
        float2 *ad = dv + dvo(b, DV_D, 0, NV, Nx), *kd = ad + part;
        const float2 cg = cf[2 * MAXHIST];
        float2 g_a[2], g_k[2], a[2], kk[2];
        df2_load(ag, t, g_a);
        df2_load(kg, t, g_k);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            a[q] = df_mul(cg, g_a[q]);
            kk[q] = df_mul(cg, g_k[q]);
        }
        int j = 0;
        for (; j + 1 < k; j += 2) {
            float2 sa0[2], sk0[2], ya0[2], yk0[2], sa1[2], sk1[2], ya1[2], yk1[2];
            const float2 *s0 = dv + hoff[j], *y0 = dv + hoff[MAXHIST + j];
            const float2 *s1 = dv + hoff[j + 1], *y1 = dv + hoff[MAXHIST + j + 1];
            df2_load(s0, t, sa0);
            df2_load(s0 + part, t, sk0);
            df2_load(y0, t, ya0);
            df2_load(y0 + part, t, yk0);
            df2_load(s1, t, sa1);
            df2_load(s1 + part, t, sk1);
            df2_load(y1, t, ya1);
            df2_load(y1 + part, t, yk1);
            const float2 cs0 = cf[j], cy0 = cf[MAXHIST + j], cs1 = cf[j + 1], cy1 = cf[MAXHIST + j + 1];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                a[q] = df_fma(cy0, ya0[q], df_fma(cs0, sa0[q], a[q]));
                kk[q] = df_fma(cy0, yk0[q], df_fma(cs0, sk0[q], kk[q]));
                a[q] = df_fma(cy1, ya1[q], df_fma(cs1, sa1[q], a[q]));
                kk[q] = df_fma(cy1, yk1[q], df_fma(cs1, sk1[q], kk[q]));
            }
        }
        if (j < k) {
            float2 sa0[2], sk0[2], ya0[2], yk0[2];
            const float2 *s0 = dv + hoff[j], *y0 = dv + hoff[MAXHIST + j];
            df2_load(s0, t, sa0);
            df2_load(s0 + part, t, sk0);
            df2_load(y0, t, ya0);
            df2_load(y0 + part, t, yk0);
            const float2 cs0 = cf[j], cy0 = cf[MAXHIST + j];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                a[q] = df_fma(cy0, ya0[q], df_fma(cs0, sa0[q], a[q]));
                kk[q] = df_fma(cy0, yk0[q], df_fma(cs0, sk0[q], kk[q]));
            }
        }
        df2_store(ad, t, a);
        df2_store(kd, t, kk);
        float2 x_a[2], l[2];
        df2_load(ax, t, x_a);
        df2_load(ax + part, t, l);
        const int c0 = (int)((2 * t) & 3);        // state of the first entry: 0 or 2
        const int64_t i = t >> 1;                  // the sequence
        float2 uu[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            gd = df_fma(g_a[q], kk[q], gd);
            dd = df_fma(a[q], kk[q], dd);
            xd = df_fma(x_a[q], kk[q], xd);
            uu[q] = df_add(kk[q], cf[2 * MAXHIST + 1 + c0 + q]);
            l[q] = df_add(l[q], ex[c0 + q]);       // logits k_x + eta_x
        }
        // u at the sequence's own state y, from whichever lane of the pair holds it
        const int y = rstate[(int64_t)b * Nx + i] & 3;
        const float2 mine = (y & 1) ? uu[1] : uu[0];
        const float2 other = make_float2(__shfl_xor_sync(0xffffffffu, mine.x, 1), __shfl_xor_sync(0xffffffffu, mine.y, 1));
        const float2 uy = ((y & 2) == c0) ? mine : other;
        float2 du[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) du[q] = df_sub(uu[q], uy);
        reinterpret_cast<float2 *>(ud + (int64_t)b * Nx * 4)[t] = make_float2(df_f(du[0]), df_f(du[1]));
        // p0 = softmax of the sequence's four logits, shifted by the largest high part
        float m = fmaxf(l[0].x, l[1].x);
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
        const float e0 = expf(df_f(df_sub(l[0], make_float2(m, 0.f))));
        const float e1 = expf(df_f(df_sub(l[1], make_float2(m, 0.f))));
        float z = e0 + e1;
        z += __shfl_xor_sync(0xffffffffu, z, 1);
        const float p00 = e0 / z, p01 = e1 / z;
        reinterpret_cast<float2 *>(P0 + (int64_t)b * Nx * 4)[t] = make_float2(p00, p01);
        if (i < N) {
            const float wi = w[i];
            dg0 = df_fma(make_float2(wi * p00, 0.f), du[0], dg0);
            dg0 = df_fma(make_float2(wi * p01, 0.f), du[1], dg0);
        }
    }
    float2 v[4] = {gd, dd, xd, dg0};
    const int idx[4] = {DA_GD, DA_DDJ, DA_XDJ, DA_DG0};
    block_sum_df<4>(v, dacc + (int64_t)b * NDACC, idx);
}

// FP32 copy of a vector's a part (the current gradient, or x) as the R rows
// of a tensor-core backward contraction, scaled by `scale`
__global__ void k_dual_to_r(const DualCtl *__restrict__ ctl, const int32_t *__restrict__ list, int64_t Nx, int N,
                            int NV, int which, const float2 *__restrict__ dv, float4 *__restrict__ R)
{
    const int b = list[blockIdx.y];
    const int v = which == 0 ? DV_G + ctl[b].gcur : DV_X;
    const float2 *a = dv + dvo(b, v, 0, NV, Nx);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x) {
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < N) r = make_float4(df_f(a[4 * i]), df_f(a[4 * i + 1]), df_f(a[4 * i + 2]), df_f(a[4 * i + 3]));
        R[(int64_t)b * Nx + i] = r;
    }
}

// Digit d (0: high) of a_x rounded to 32 bits of the slot's scale (the
// slot's tc_scale field): A = round(a qa), A = D0 2^22 + D1 2^11 + D2 with
// |D| <= 2^10.  Digits are exact in fp16 and their sums over fewer than
// 2^14 sequences are exact in FP32, so X^T D is exact on the tensor cores.
__global__ void k_dual_digits(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int64_t Nx, int N,
                              int NV, int d, const float2 *__restrict__ dv, float4 *__restrict__ R)
{
    const int b = list[blockIdx.y];
    const double qa = sd[b].tc_scale;
    const float2 *a = dv + dvo(b, DV_X, 0, NV, Nx);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x) {
        float v[4] = {0.f, 0.f, 0.f, 0.f};
        if (i < N) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const long long A = llrint(df_to_d(a[4 * i + c]) * qa);
                const long long d0 = (A + (1ll << 21)) >> 22;          // round(A / 2^22)
                const long long r0 = A - (d0 << 22);
                const long long d1 = (r0 + (1ll << 10)) >> 11;         // round(r0 / 2^11)
                const long long d2 = r0 - (d1 << 11);
                v[c] = (float)(d == 0 ? d0 : d == 1 ? d1 : d2);
            }
        }
        R[(int64_t)b * Nx + i] = make_float4(v[0], v[1], v[2], v[3]);
    }
}

// The three digits at once: plane d of list position s into R row d n + s.
__global__ void k_dual_digits3(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int n, int64_t Nx,
                               int N, int NV, const float2 *__restrict__ dv, float4 *__restrict__ R)
{
    const int s = blockIdx.y, b = list[s];
    const double qa = sd[b].tc_scale;
    const float2 *a = dv + dvo(b, DV_X, 0, NV, Nx);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x) {
        float v[3][4] = {};
        if (i < N) {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const long long A = llrint(df_to_d(a[4 * i + c]) * qa);
                const long long d0 = (A + (1ll << 21)) >> 22;          // round(A / 2^22)
                const long long r0 = A - (d0 << 22);
                const long long d1 = (r0 + (1ll << 10)) >> 11;         // round(r0 / 2^11)
                v[0][c] = (float)d0;
                v[1][c] = (float)d1;
                v[2][c] = (float)(r0 - (d1 << 11));
            }
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) R[((int64_t)d * n + s) * Nx + i] = make_float4(v[d][0], v[d][1], v[d][2], v[d][3]);
    }
}

// The solution from its three digit planes in one pass: J = (2^22 X^T D0 +
// 2^11 X^T D1 + X^T D2) / tc_scale, the integer sum exact in 64 bits (below
// 2^47), converted to double-float exactly, scaled in double-float and
// rounded once to FP32 (no FP64 arithmetic: GB300's FP64 pipe is narrow);
// J_rr = 0, h = eta, padding 0.  The products come from gpool buffers s,
// n + s, 2n + s.
__global__ void k_dual_planes_to_wa(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int n, int L,
                                    int64_t Dp, const float *__restrict__ gpool, float *__restrict__ wa)
{
    const int s = blockIdx.y, b = list[s];
    const SlotDev &S = sd[b];
    __shared__ float2 s_inv;
    if (threadIdx.x == 0) s_inv = df_from_d(1.0 / S.tc_scale);   // one FP64 division per block
    __syncthreads();
    const float2 inv = s_inv;
    const float *g0 = gpool + (int64_t)s * Dp, *g1 = gpool + (int64_t)(n + s) * Dp, *g2 = gpool + (int64_t)(2 * n + s) * Dp;
    const int64_t nJ = (int64_t)QQ * L, own0 = (int64_t)S.locus * QQ;
    float *o = wa + (int64_t)b * Dp;
    for (int64_t e4 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e4 < Dp / 4; e4 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = 4 * e4;   // Dp and nJ are multiples of 4: a float4 is all J, all h or all padding
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (e < nJ) {
            if (e < own0 || e >= own0 + QQ) {
                const float4 a = reinterpret_cast<const float4 *>(g0)[e4], bb = reinterpret_cast<const float4 *>(g1)[e4],
                             c = reinterpret_cast<const float4 *>(g2)[e4];
                const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {bb.x, bb.y, bb.z, bb.w}, cv[4] = {c.x, c.y, c.z, c.w};
                float r[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const long long J = ((long long)__float2int_rn(av[k]) << 22) +
                                        ((long long)__float2int_rn(bv[k]) << 11) + (long long)__float2int_rn(cv[k]);
                    r[k] = df_f(df_mul(df_from_ll_fast(J), inv));
                }
                v = make_float4(r[0], r[1], r[2], r[3]);
            }
        } else if (e < nJ + Q) {
            v = make_float4((float)S.eta[0], (float)S.eta[1], (float)S.eta[2], (float)S.eta[3]);
        }
        reinterpret_cast<float4 *>(o)[e4] = v;
    }
}

// J (=, or +=) 2^(22, 11, 0) (X^T D) in 64-bit integers: every X^T D is an
// integer below 2^24, exact in the FP32 backward output
__global__ void k_dual_digit_acc(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int64_t Dp,
                                 int d, const float *__restrict__ gpool, long long *__restrict__ J64)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const float *g = gpool + (int64_t)(2 * b + 1 - S.gcur) * Dp;
    const long long wgt = 1ll << (d == 0 ? 22 : d == 1 ? 11 : 0);
    long long *o = J64 + (int64_t)b * Dp;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < Dp; e += (int64_t)gridDim.x * blockDim.x)
        o[e] = (d == 0 ? 0ll : o[e]) + (long long)__float2int_rn(g[e]) * wgt;
}

// x in the engine layout from the combined digits: J blocks (J_rr = 0) =
// the integer sum / tc_scale, rounded once to FP32; h = eta (the slot's eta
// field), padding 0
__global__ void k_dual_to_wa(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int L, int64_t Dp,
                             const long long *__restrict__ J64, float *__restrict__ wa)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const long long *g = J64 + (int64_t)b * Dp;
    const double inv = 1.0 / S.tc_scale;
    // (the integer is below 2^47, so its FP64 value is exact)
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < Dp; e += (int64_t)gridDim.x * blockDim.x) {
        float v = 0.f;
        if (e < (int64_t)QQ * L) v = (e / QQ == S.locus) ? 0.f : (float)((double)g[e] * inv);
        else if (e < (int64_t)QQ * L + Q) v = (float)S.eta[e - (int64_t)QQ * L];
        wa[(int64_t)b * Dp + e] = v;
    }
}

// ---- the per-iteration decisions on the device

// What a step trial reads of one sequence: u_a - u_y, the base
// probabilities, the state at r and the weight (constant through a search).
struct TrialIn {
    float4 du, p0;
    int y;
    float w;
};

__device__ __forceinline__ TrialIn trial_load(int64_t o, int i, const float4 *__restrict__ ud,
                                              const uint8_t *__restrict__ rstate, const float *__restrict__ w,
                                              const float4 *__restrict__ P0)
{
    TrialIn t;
    t.du = ud[o];
    t.p0 = P0[o];
    t.y = rstate[o] & 3;
    t.w = w[i];
    return t;
}

// One sequence of a step trial as a change from the current point (the
// derivation above): adds w dl, the slope change and the new residual row's
// sums, and writes the row.
__device__ __forceinline__ void trial_seq(int64_t o, int i, const TrialIn &in, float2 stp, float stpf,
                                          const float2 *__restrict__ kx, const float2 *__restrict__ kd,
                                          const float2 *ex, const float2 *ed, float4 *__restrict__ R, float &f,
                                          float &dg, float (&rs)[4], float2 &fbig, float2 &dgbig)
{
    const float du[4] = {in.du.x, in.du.y, in.du.z, in.du.w};   // u_a - u_y
    const int y = in.y;
    const float wi = in.w;
    const float p0[4] = {in.p0.x, in.p0.y, in.p0.z, in.p0.w};
    float t[4], tmax = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        t[a] = stpf * du[a];
        tmax = fmaxf(tmax, fabsf(t[a]));
    }
    float r[4];
    if (tmax < 30.f) {
        float e[4], x[4], q = 0.f, z = 0.f;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            e[a] = expm1f(t[a]);
            x[a] = p0[a] * expf(t[a]);
            q = fmaf(p0[a], e[a], q);
            z += x[a];
        }
        const float iz = 1.f / z;
        f = fmaf(wi, fabsf(q) < 0.5f ? log1pf(q) : logf(z), f);
        float ro = 0.f;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            dg = fmaf(wi * (p0[a] * (e[a] - q) * iz), du[a], dg);
            r[a] = a == y ? 0.f : wi * (x[a] * iz);
            ro += r[a];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
            if (a == y) r[a] = -ro;
    } else {
        const BigTrial bt = trial_big(kx + 4 * (int64_t)i, kd + 4 * (int64_t)i, ex, ed, stp, y, wi, in.p0);
        r[0] = bt.r.x;
        r[1] = bt.r.y;
        r[2] = bt.r.z;
        r[3] = bt.r.w;
        fbig = df_add(fbig, bt.df);
        dgbig = df_add(dgbig, bt.ddg);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) rs[a] += r[a];
    R[o] = make_float4(r[0], r[1], r[2], r[3]);
}

__device__ __forceinline__ double dot4d(const double *a, const double *b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

// Threads per search block (LS_THREADS, 128 by default): the search is
// latency-bound (short passes over the slot's sequences between block
// reductions and the FP64 state machine of one thread), so smaller blocks
// let more searches share an SM.

// The whole line search of one slot in one thread block (SuperDCA: the
// More-Thuente search of CppNumericalSolvers' LbfgsSolver, one
// value_and_gradient per trial, LBFGS_interface_CppNumericalSolvers.hpp:
// 111-117).  Thread 0 holds the More-Thuente state machine (FP64, in shared
// memory); all threads evaluate each trial over the slot's sequences and
// reduce it (FP32 per thread and warp, FP64 across warps).
//   1. Restart test: a direction that is not downhill in angle
//      (cos(g, d) >= -1e-10), or one the last search asked to restart,
//      becomes steepest descent: d = -g, its logit direction, differences
//      and slope at 0 are formed here and the history is dropped.
//   2. More-Thuente start from f, the slope at 0 (data part from the
//      direction kernel's base probabilities, L2 part exact) and the initial
//      step (1 after a restart, else 1 / ||g||).  A start that is not downhill
//      evaluates the point itself (step 0) and marks the slot to restart, or
//      to stop when it has no history.
//   3. Trials until the search accepts one: the accepted point is the last
//      trial, so R holds its residual rows, acc[ACC_RS*] their sums and the
//      slot's f, stp the point's objective and step.
template <int LS_THREADS>
__global__ void __launch_bounds__(LS_THREADS, 768 / LS_THREADS)
k_dual_linesearch(DualCtl *__restrict__ ctl, const int32_t *__restrict__ list, int N, int64_t Nx, int NV,
                  double lambda_J, double lambda_h, const double *__restrict__ dacc, float2 *__restrict__ dv,
                  float4 *__restrict__ ud,
                  const uint8_t *__restrict__ rstate, const float *__restrict__ w, const float4 *__restrict__ P0,
                  float4 *__restrict__ R, double *__restrict__ acc, const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.x >= *cnt) return;
    const int b = list[blockIdx.x];
    DualCtl &S = ctl[b];
    if (S.phase != DC_STEP) return;   // (the same for the whole block)
    __shared__ __align__(16) unsigned char mt_raw[sizeof(MoreThuente)];
    __shared__ double red[LS_THREADS / 32][8];
    __shared__ double s_stp;
    __shared__ float2 s_stp_df;
    __shared__ double s_tot[8];
    __shared__ int s_restart, s_done;
    __shared__ float2 s_ex[Q], s_ed[Q];   // eta_x, eta_d as double-float (the h parts of the logits and of u)
    MoreThuente &mt = *reinterpret_cast<MoreThuente *>(mt_raw);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const double *da = dacc + (int64_t)b * NDACC;
    // FP64 scalars of the search, thread 0's (in shared memory, so that they
    // hold no registers of the other threads through the trial loop)
    __shared__ double sc[9];
    double &xdJ = sc[0], &xdH = sc[1], &ddJ = sc[2], &ddH = sc[3], &dg0 = sc[4], &f0d = sc[5], &dg0d = sc[6],
           &x2H = sc[7];
    __shared__ int s_mode;   // 0 searching, 1 evaluating the current point (start not downhill)
    if (tid == 0) {
        const double *eg = S.eta_g[S.gcur];
        const double gd = da[DA_GD] + dot4d(eg, S.eta_d);
        ddJ = da[DA_DDJ];
        ddH = dot4d(S.eta_d, S.eta_d);
        const double cosgd = gd / sqrt(fmax(S.g2, 0.0) * fmax(ddJ + ddH, 0.0));
        s_restart = (S.nhist > 0 && (S.force_restart || !(cosgd < -1e-10))) ? 1 : 0;
        S.force_restart = 0;
        xdJ = da[DA_XDJ];
        dg0 = da[DA_DG0];
        s_mode = 0;
    }
    __syncthreads();
    const bool restart = s_restart != 0;
    if (restart) {
        const int gc = S.gcur;
        float2 ed[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) ed[c] = df_from_d(-S.eta_g[gc][c]);
        const float2 *ag = dv + dvo(b, DV_G + gc, 0, NV, Nx), *kg = dv + dvo(b, DV_G + gc, 1, NV, Nx);
        const float2 *ax = dv + dvo(b, DV_X, 0, NV, Nx);
        float2 *ad = dv + dvo(b, DV_D, 0, NV, Nx), *kd = dv + dvo(b, DV_D, 1, NV, Nx);
        float2 xd = df_zero(), d0 = df_zero();
        for (int64_t i = tid; i < Nx; i += LS_THREADS) {
            const int64_t o = (int64_t)b * Nx + i;
            float2 uu[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float2 a_d = df_neg(ag[4 * i + c]), k_d = df_neg(kg[4 * i + c]);
                ad[4 * i + c] = a_d;
                kd[4 * i + c] = k_d;
                uu[c] = df_add(k_d, ed[c]);
                xd = df_fma(ax[4 * i + c], k_d, xd);
            }
            const int y = rstate[o] & 3;
            float2 uy = uu[0];
#pragma unroll
            for (int c = 1; c < 4; ++c)
                if (c == y) uy = uu[c];
            float du[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) du[c] = df_f(df_sub(uu[c], uy));
            ud[o] = make_float4(du[0], du[1], du[2], du[3]);
            if (i < N) {
                const float4 pv = P0[o];
                const float p0[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                for (int c = 0; c < 4; ++c) d0 = df_fma(make_float2(w[i] * p0[c], 0.f), df_sub(uu[c], uy), d0);
            }
        }
        const float2 sx = df_warp_sum(xd), s0 = df_warp_sum(d0);
        if (lane == 0) {
            red[wid][0] = df_to_d(sx);
            red[wid][1] = df_to_d(s0);
        }
        __syncthreads();
        if (tid == 0) {
            double t0 = 0, t1 = 0;
            for (int k = 0; k < LS_THREADS / 32; ++k) {
                t0 += red[k][0];
                t1 += red[k][1];
            }
            xdJ = t0;
            dg0 = t1;
            ddJ = S.g2J;
            for (int c = 0; c < 4; ++c) {
                S.eta_d[c] = -S.eta_g[gc][c];
                S.cdf[2 * MAXHIST + 1 + c] = df_from_d(S.eta_d[c]);
            }
            ddH = dot4d(S.eta_d, S.eta_d);
            S.nhist = 0;
            S.iter = 0;
            S.restarts++;
            S.coef_g = -1.0;
            S.cdf[2 * MAXHIST] = make_float2(-1.f, 0.f);
        }
        __syncthreads();
    }
    if (tid == 0) {
        for (int c = 0; c < Q; ++c) {
            s_ex[c] = df_from_d(S.eta_x[c]);
            s_ed[c] = df_from_d(S.eta_d[c]);
        }
        xdH = dot4d(S.eta_x, S.eta_d);
        x2H = dot4d(S.eta_x, S.eta_x);
        const double l20 = lambda_J * S.x2J + lambda_h * x2H;
        const double d0 = dg0 + 2.0 * lambda_J * xdJ + 2.0 * lambda_h * xdH;
        f0d = S.f - l20;
        dg0d = dg0;
        const double alpha = restart ? 1.0 : 1.0 / sqrt(S.g2);
        S.trials = 0;
        new (mt_raw) MoreThuente();
        if (mt.start(S.f, d0, alpha) == MoreThuente::NEED_EVAL) {
            s_stp = mt.stp;
            s_stp_df = df_from_d(mt.stp);
        } else {
            s_stp = 0.0;
            s_stp_df = df_zero();
            s_mode = 1;
            S.weak++;
            if (S.nhist == 0) S.stalled = 1;
            else S.force_restart = 1;
        }
        s_done = 0;
    }
    // More-Thuente stops within 20 trials; the bound only guards the loop
    for (int it = 0; it < 64; ++it) {
        __syncthreads();
        const double stp = s_stp;
        const float2 stpd = s_stp_df;
        const float stpf = stpd.x + stpd.y;
        float f = 0.f, dg = 0.f, rs[4] = {0.f, 0.f, 0.f, 0.f};
        float2 fbig = df_zero(), dgbig = df_zero();
        const float2 *kxs = dv + dvo(b, DV_X, 1, NV, Nx), *kds = dv + dvo(b, DV_D, 1, NV, Nx);
        // two sequences per pass, both sequences' loads in flight before
        // either is computed (the search has few warps per SM to hide
        // latency with)
#pragma unroll 1
        for (int i0 = tid; i0 < N; i0 += 2 * LS_THREADS) {
            const int i1 = i0 + LS_THREADS;
            const bool two = i1 < N;
            const int64_t o0 = (int64_t)b * Nx + i0, o1 = (int64_t)b * Nx + (two ? i1 : i0);
            const TrialIn t0 = trial_load(o0, i0, ud, rstate, w, P0);
            const TrialIn t1 = trial_load(o1, two ? i1 : i0, ud, rstate, w, P0);
            trial_seq(o0, i0, t0, stpd, stpf, kxs, kds, s_ex, s_ed, R, f, dg, rs, fbig, dgbig);
            if (two) trial_seq(o1, i1, t1, stpd, stpf, kxs, kds, s_ex, s_ed, R, f, dg, rs, fbig, dgbig);
        }
        // FP32 sums per warp (each lane's value is an FP32 partial over a few
        // sequences), double-float for the large-step terms, FP64 across warps
        const float v[6] = {warp_sum_f(f), warp_sum_f(dg), warp_sum_f(rs[0]), warp_sum_f(rs[1]), warp_sum_f(rs[2]),
                            warp_sum_f(rs[3])};
        fbig = df_warp_sum(fbig);
        dgbig = df_warp_sum(dgbig);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < 6; ++k) red[wid][k] = (double)v[k];
            red[wid][6] = df_to_d(fbig);
            red[wid][7] = df_to_d(dgbig);
        }
        __syncthreads();
        if (tid < 8) {
            double t = 0.0;
            for (int k = 0; k < LS_THREADS / 32; ++k) t += red[k][tid];
            s_tot[tid] = t;
        }
        __syncthreads();
        if (tid == 0) {
            const double *tot = s_tot;
            const double l2 = lambda_J * (S.x2J + 2.0 * stp * xdJ + stp * stp * ddJ) +
                              lambda_h * (x2H + 2.0 * stp * xdH + stp * stp * ddH);
            const double dl2 = 2.0 * lambda_J * (xdJ + stp * ddJ) + 2.0 * lambda_h * (xdH + stp * ddH);
            const double ff = f0d + (tot[0] + tot[6]) + l2;
            const double dd = dg0d + (tot[1] + tot[7]) + dl2;
            S.trials++;
            bool done = s_mode == 1 || it == 63;
            if (!done && (!isfinite(ff) || !isfinite(dd))) done = true;
            if (!done) {
                if (mt.feed(ff, dd) == MoreThuente::DONE) {
                    done = true;
                    if (mt.info != 1) S.weak++;
                    S.max_trials = max(S.max_trials, S.trials);
                } else {
                    s_stp = mt.stp;
                    s_stp_df = df_from_d(mt.stp);
                }
            }
            if (done) {
                S.stp = stp;   // the accepted point is the last trial
                S.stp_df = stpd;
                S.f = ff;
                double *ac = acc + (int64_t)b * NACC;
                for (int a = 0; a < 4; ++a) ac[ACC_RS0 + a] = tot[2 + a];
                s_done = 1;
            }
        }
        __syncthreads();
        if (s_done) break;
    }
}

constexpr int CTL_WORDS = (int)(sizeof(DualCtl) / 8);
static_assert(sizeof(DualCtl) % 8 == 0, "DualCtl is copied as 8-byte words");

__device__ void write_summary(const DualCtl &S, DualSum &o)
{
    o.phase = S.phase;
    o.status = S.status;
    o.want_check = S.want_check;
    o.chk_wait = S.chk_wait;
    o.releps_stop = S.releps_stop;
    o.iterations = S.iterations;
    o.nfeval = S.nfeval;
    o.restarts = S.restarts;
    o.skipped = S.skipped;
    o.weak = S.weak;
    o.max_trials = S.max_trials;
    o.f = S.f;
    o.gmax = S.gmax;
    o.amax_g = S.amax_g;
    o.amax_x = S.amax_x;
    o.x2J = S.x2J;
    for (int a = 0; a < Q; ++a) o.eta_x[a] = S.eta_x[a];
}

// After the gradient pass: the L-BFGS bookkeeping of one slot per warp, in
// FP64 by lane 0 on a shared-memory copy of the slot's state (SuperDCA's
// LbfgsSolver iteration, driven from plmDCA.hpp:298-304; stop on max|g| <
// threshold or the iteration limit, plmDCA.hpp:218-221):
//   h gradient from the residual sums, the (s, y) pair kept when
//   s.y > 1e-3 |s| |y|, the iteration limit and stall stops, the wish for an
//   exact max-norm check (the host batches those), the newest column of the
//   Gram matrices S^T Y and Y^T Y from the history dots, the compact-form
//   coefficients of the next direction and its h part, and the ring
//   position the next accepted step will fill.
__global__ void __launch_bounds__(32)
k_dual_control(DualCtl *__restrict__ ctl, DualSum *__restrict__ sum, const int32_t *__restrict__ list, int m,
               int max_iterations, double gtol, double lambda_J, double lambda_h, const double *__restrict__ acc,
               const double *__restrict__ amax, const double *__restrict__ dots, const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.x >= *cnt) return;
    const int b = list[blockIdx.x];
    __shared__ DualCtl S;
    __shared__ double s_eg[Q], s_dt[2 * MAXHIST], s_R[MAXHIST * MAXHIST], s_YY[MAXHIST * MAXHIST];
    __shared__ int s_go;
    {
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(ctl + b);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(&S);
        for (int k = threadIdx.x; k < CTL_WORDS; k += 32) dst[k] = src[k];
    }
    if (threadIdx.x == 0) s_go = 0;
    __syncwarp();
    int &go = s_go;
    if (threadIdx.x == 0 && S.phase != DC_STOP) {
        const double *ac = acc + (int64_t)b * NACC;
        const bool init = S.phase == DC_EVAL0;
        if (!init) {
            // the accepted step's h part: x_h += stp d_h, s_h
            for (int a = 0; a < Q; ++a) {
                const double xn = S.eta_x[a] + S.stp * S.eta_d[a];
                if (S.push && S.ring_new >= 0) S.eta_s[S.ring_new][a] = xn - S.eta_x[a];
                S.eta_x[a] = xn;
            }
        }
        const int gn = 1 - S.gcur;
        double eg[Q];
        for (int a = 0; a < Q; ++a) eg[a] = ac[ACC_RS0 + a] + 2.0 * lambda_h * S.eta_x[a];
        const bool pushed = S.push && S.ring_new >= 0;
        if (pushed)
            for (int a = 0; a < Q; ++a) S.eta_y[S.ring_new][a] = eg[a] - S.eta_g[S.gcur][a];
        for (int a = 0; a < Q; ++a) S.eta_g[gn][a] = eg[a];
        S.gcur = gn;
        S.g2J = ac[ACC_G2];
        S.g2 = S.g2J + dot4d(eg, eg);
        S.x2J = ac[ACC_X2J];
        const double x2H = dot4d(S.eta_x, S.eta_x);
        S.amax_g = amax[2 * b];
        S.amax_x = amax[2 * b + 1];
        const double gnorm = sqrt(fmax(S.g2, 0.0));
        S.gmax = S.chk_ratio > 0.0 ? S.chk_ratio * gnorm : gnorm;   // estimate until checked
        bool st = false;
        if (init) {
            S.f = ac[ACC_F] + lambda_J * S.x2J + lambda_h * x2H;
            S.nfeval = 1;
        } else {
            S.iterations++;
            S.nfeval += 2 + S.trials;
            const int pr = S.ring_new >= 0 ? S.ring_new : 0;
            const double sy = ac[ACC_SY] + (pushed ? dot4d(S.eta_s[pr], S.eta_y[pr]) : 0.0);
            const double yy = ac[ACC_YY] + (pushed ? dot4d(S.eta_y[pr], S.eta_y[pr]) : 0.0);
            const double ss = ac[ACC_SS] + (pushed ? dot4d(S.eta_s[pr], S.eta_s[pr]) : 0.0);
            if (pushed && sy > 1e-3 * sqrt(ss * yy) && yy > 0.0 && isfinite(sy) && isfinite(yy)) {
                if (S.nhist == m) {
                    for (int j = 1; j < m; ++j) S.hist[j - 1] = S.hist[j];
                    S.nhist--;
                }
                S.hist[S.nhist++] = S.ring_new;
                S.gamma = sy / yy;
                S.sy_new = sy;
                S.yy_new = yy;
                S.iter++;
            } else {
                S.ring_new = -1;
                S.skipped++;
            }
            if (S.iterations > max_iterations) {
                S.status = 1;
                st = true;
            } else if (S.stalled) {
                S.status = 2;
                st = true;
            }
        }
        if (!isfinite(S.f) || !isfinite(S.g2)) {
            S.status = -1;
            st = true;
        }
        if (st) {
            S.phase = DC_STOP;
            S.want_check = 0;
        } else {
            // the relative-norm stop is decided after the max-norm test (by the host's check pass)
            const double releps = 1e-4 * fmax(1.0, sqrt(S.x2J + x2H));
            S.releps_stop = gnorm < releps;
            // the max-norm test needs J = Phi^T a_g: wanted when the last check's
            // ratio max|g| / ||g|| predicts a pass, and every 15 iterations
            const bool due = S.iterations - S.last_check >= 15 && (S.chk_ratio > 0.0 || gnorm < 150.0 * gtol);
            const bool near = S.chk_ratio > 0.0 && S.chk_ratio * gnorm < 1.1 * gtol;
            S.want_check = (due || near || gnorm < gtol || S.releps_stop) ? 1 : 0;
            S.chk_wait = S.want_check ? S.chk_wait + 1 : 0;
            S.coef_g = -1.0;
            for (int a = 0; a < Q; ++a) s_eg[a] = eg[a];
            go = 1;
        }
    }
    __syncwarp();
    // compact-form coefficients of the next direction: the per-pair work on
    // the warp's lanes (lane j: history pair j), the small triangular solve
    // on one thread
    if (go) {
        const int lane = threadIdx.x, k = S.nhist;
        const double *dp = dots + (int64_t)b * 4 * MAXHIST;
        if (lane < k) {
            const int pj = S.hist[lane];
            s_dt[lane] = dp[pj] + dot4d(S.eta_s[pj], s_eg);
            s_dt[MAXHIST + lane] = dp[DOT_Y + pj] + dot4d(S.eta_y[pj], s_eg);
        }
        __syncwarp();
        if (lane < k) {
            const int pj = S.hist[lane];
            if (S.ring_new >= 0) {
                // the newest pair's column: s_j.y = s_j.g - s_j.g_old, y_j.y likewise,
                // and its own s.y, y.y from the gradient pass
                const int pn = S.ring_new;
                const double syj = pj == pn ? S.sy_new : s_dt[lane] - S.sg_prev[pj];
                const double yyj = pj == pn ? S.yy_new : s_dt[MAXHIST + lane] - S.yg_prev[pj];
                S.SY[pj][pn] = syj;
                S.YY[pj][pn] = yyj;
                S.YY[pn][pj] = yyj;
            }
        }
        __syncwarp();
        if (lane < k) {
            S.sg_prev[S.hist[lane]] = s_dt[lane];
            S.yg_prev[S.hist[lane]] = s_dt[MAXHIST + lane];
        }
        for (int e = lane; e < k * k; e += 32) {
            const int ra = e / k, rc = e % k;
            s_R[e] = (ra <= rc) ? S.SY[S.hist[ra]][S.hist[rc]] : 0.0;
            s_YY[e] = S.YY[S.hist[ra]][S.hist[rc]];
        }
        __syncwarp();
        if (lane == 0 && k > 0) {
            double cg, cS[MAXHIST], cY[MAXHIST];
            if (lbfgs_compact_coeffs(k, s_R, s_YY, s_dt, s_dt + MAXHIST, S.gamma, &cg, cS, cY)) {
                S.coef_g = cg;
                for (int a = 0; a < k; ++a) {
                    S.coefS[a] = cS[a];
                    S.coefY[a] = cY[a];
                }
            } else {
                S.nhist = 0;
                S.iter = 0;
            }
        }
        __syncwarp();
        const int kk = S.nhist;
        if (lane < Q) {
            double v = S.coef_g * s_eg[lane];
            for (int j = 0; j < kk; ++j)
                v += S.coefS[j] * S.eta_s[S.hist[j]][lane] + S.coefY[j] * S.eta_y[S.hist[j]][lane];
            S.eta_d[lane] = v;
            S.cdf[2 * MAXHIST + 1 + lane] = df_from_d(v);
        }
        if (lane < kk) {
            S.cdf[lane] = df_from_d(S.coefS[lane]);
            S.cdf[MAXHIST + lane] = df_from_d(S.coefY[lane]);
        }
        if (lane == 0) {
            S.cdf[2 * MAXHIST] = df_from_d(S.coef_g);
            // the next accepted step fills a ring position outside the live history
            int pos = 0;
            for (bool used = true; used;) {
                used = false;
                for (int j = 0; j < kk; ++j) used = used || S.hist[j] == pos;
                if (used) ++pos;
            }
            S.ring_new = pos;
            S.push = 1;
            S.phase = DC_STEP;
        }
    }
    __syncwarp();
    {
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(ctl + b);
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&S);
        for (int k = threadIdx.x; k < CTL_WORDS; k += 32) dst[k] = src[k];
    }
    if (threadIdx.x == 0) write_summary(S, sum[b]);
}

// After an exact max-norm check (the tensor-core backward X^T a_g with its
// max-only epilogue): the slot's max|g| is the J part's maximum and |g_h|;
// stop with status 0 below the threshold, or with
// status 2 on a pending relative-norm stop (SuperDCA: plmDCA.hpp:218-221).
__global__ void k_dual_check_apply(DualCtl *__restrict__ ctl, DualSum *__restrict__ sum,
                                   const int32_t *__restrict__ list, int n, double gtol,
                                   const double *__restrict__ acc)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int b = list[t];
    DualCtl &S = ctl[b];
    if (S.phase == DC_STOP) return;
    const double *eg = S.eta_g[S.gcur];
    double gm = acc[(int64_t)b * NACC + ACC_GMAX];
    for (int a = 0; a < Q; ++a) gm = fmax(gm, fabs(eg[a]));
    const double gnorm = sqrt(fmax(S.g2, 0.0));
    S.gmax = gm;
    S.chk_ratio = gnorm > 0.0 ? gm / gnorm : 0.0;
    S.last_check = S.iterations;
    S.chk_wait = 0;
    S.want_check = 0;
    if (gm < gtol) {
        S.status = 0;
        S.phase = DC_STOP;
    } else if (S.releps_stop) {
        S.status = 2;
        S.phase = DC_STOP;
    }
    write_summary(S, sum[b]);
}

// The learned start of a slot from its predicted residual rows (already
// through k_dual_quant and the exact K rho product): a_x = c rho_q / qscale,
// k_x = c K rho (KR is K rho / qscale), c = -1 / (2 lambda_J); the logits
// are k_x (eta = 0).  The pair (a_x, k_x) is consistent to the double-float
// rounding of one product by c.
__global__ void __launch_bounds__(256)
k_dual_ws_init(const int32_t *__restrict__ list, int64_t Nx, int NV, double c, double inv_qscale,
               const int32_t *__restrict__ rq, const float2 *__restrict__ KR, float2 *__restrict__ dv,
               const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.y >= *cnt) return;
    const int b = list[blockIdx.y];
    const float2 cd = df_from_d(c), cq = df_from_d(c * inv_qscale);
    float2 *ax = dv + dvo(b, DV_X, 0, NV, Nx), *kx = ax + Nx * 4;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < Nx * 4; e += (int64_t)gridDim.x * blockDim.x) {
        const float2 a = df_mul(cq, df_from_int(rq[(int64_t)b * Nx * 4 + e]));
        const float2 k = df_mul(cd, KR[(int64_t)b * Nx * 4 + e]);
        ax[e] = a;
        kx[e] = k;
    }
}

// The start and final evaluations of the dual form: objective terms, R rows
// and their sums at the slot's current point, from the logits k_x + eta
// (eta: the SlotDev field, the h part of x; zero at a start) with an FP64
// log-sum-exp (SuperDCA's objective, plmDCA_objective.hpp:86-151, at x).
constexpr int EVAL_THREADS = 256;

__global__ void __launch_bounds__(EVAL_THREADS)
k_dual_eval(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int N, int64_t Nx, int NV,
            const float2 *__restrict__ dv, const uint8_t *__restrict__ rstate, const double *__restrict__ w,
            float4 *__restrict__ R, double *__restrict__ acc)
{
    const int b = list[blockIdx.y];
    const SlotDev &S = sd[b];
    const double eta[4] = {S.eta[0], S.eta[1], S.eta[2], S.eta[3]};
    const float2 *kx = dv + dvo(b, DV_X, 1, NV, Nx);
    double f = 0, rs0 = 0, rs1 = 0, rs2 = 0, rs3 = 0;
    for (int i = blockIdx.x * EVAL_THREADS + threadIdx.x; i < N; i += gridDim.x * EVAL_THREADS) {
        const int64_t o = (int64_t)b * Nx + i;
        double l[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) l[a] = df_to_d(kx[4 * (int64_t)i + a]) + eta[a];
        const double mx = fmax(fmax(l[0], l[1]), fmax(l[2], l[3]));
        double e[4], z = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            e[a] = exp(l[a] - mx);
            z += e[a];
        }
        const int sr = rstate[o] & 3;
        const double wi = w[i];
        f += wi * (mx + log(z) - l[sr]);
        double r[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) r[a] = wi * (e[a] / z) - (a == sr ? wi : 0.0);
        rs0 += r[0]; rs1 += r[1]; rs2 += r[2]; rs3 += r[3];
        R[o] = make_float4((float)r[0], (float)r[1], (float)r[2], (float)r[3]);
    }
    double v[6] = {f, 0.0, rs0, rs1, rs2, rs3};
    const int idx[6] = {ACC_F, ACC_DG, ACC_RS0, ACC_RS1, ACC_RS2, ACC_RS3};
    block_sum_atomic<6>(v, acc + (int64_t)b * NACC, idx);
}

unsigned grid_for(int64_t elems, int per_block_elems, int cap)
{
    const int64_t g = (elems + per_block_elems - 1) / per_block_elems;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

// Entry pairs per thread of the gradient and accept kernels: each block ends
// with reductions and atomics, which eight passes amortise (measured: 8 %
// less time than two passes, 2048 loci at 3000 x 94,000)
constexpr int STREAM_PASSES = 8;

} // namespace

void launch_dual_kmat(const int32_t *dist, int N, int64_t Nx, int L, int32_t *K, cudaStream_t st)
{
    k_dual_kmat<<<grid_for(Nx * Nx, 256 * 8, 4096), 256, 0, st>>>(dist, N, Nx, L, K);
}

void launch_dual_quant(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float *R,
                       const uint8_t *rstate, double qscale, int32_t *rq, long long *csum, cudaStream_t st,
                       const int *cnt)
{
    if (n <= 0) return;
    dim3 gq(grid_for(P.Nx, 256 * 4, 64), n);
    k_dual_quant<<<gq, 256, 0, st>>>(sd, list, (int)P.N, P.Nx, reinterpret_cast<const float4 *>(R), rstate,
                                     (float)qscale, reinterpret_cast<int4 *>(rq),
                                     reinterpret_cast<unsigned long long *>(csum), cnt);
}

// K rho on the CUDA cores (64-bit integer multiply-adds): any N
void launch_dual_kprod(const Problem &P, const int32_t *list, int n, const uint8_t *rstate, const int32_t *K,
                       double qscale, const int32_t *rq, const long long *csum, float2 *KR, cudaStream_t st,
                       const int *cnt)
{
    if (n <= 0) return;
    dim3 gk((unsigned)(P.Nx / KP_M), (unsigned)((n + KP_S - 1) / KP_S));
    k_dual_kprod<<<gk, 256, 0, st>>>(K, P.Nx, (int)P.N, list, n, reinterpret_cast<const int4 *>(rq), csum, rstate,
                                     1.0 / qscale, KR, cnt);
}

void launch_dual_grad(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, double qscale,
                      const int32_t *rq, const float2 *KR, float2 *dv, double *acc, double *amax, cudaStream_t st,
                      const int *cnt)
{
    if (n <= 0) return;
    const int NV = DV_S + 2 * P.ring;
    dim3 gg(grid_for(P.Nx * 2, 256 * STREAM_PASSES, 64), n);
    k_dual_grad<<<gg, 256, 0, st>>>(ctl, list, P.Nx, NV, P.ring, df_host(2.0 * P.lambda_J), rq, df_host(1.0 / qscale),
                                    KR, dv, acc, amax, cnt);
}

void launch_dual_dots(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, int newg, const float2 *dv,
                      double *dots, cudaStream_t st, const int *cnt)
{
    if (n <= 0) return;
    dim3 g((unsigned)((P.Nx * 4 + DOT_CHUNK - 1) / DOT_CHUNK), n);
    k_dual_dots<<<g, 256, 0, st>>>(ctl, list, P.Nx, DV_S + 2 * P.ring, P.ring, newg, dv, dots, cnt);
}

void launch_dual_direction(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, float2 *dv,
                           float *P0, const float *w, const uint8_t *rstate, float *ud, double *dacc,
                           cudaStream_t st, const int *cnt)
{
    if (n <= 0) return;
    dim3 g((unsigned)((P.Nx * 2 + DIR_THREADS - 1) / DIR_THREADS), n);
    k_dual_direction<<<g, DIR_THREADS, 0, st>>>(ctl, list, P.Nx, (int)P.N, DV_S + 2 * P.ring, P.ring, dv, P0, w,
                                                rstate, ud, dacc, cnt);
}

void launch_dual_eval(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float2 *dv,
                      const uint8_t *rstate, const double *w, float *R, double *acc, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.N, EVAL_THREADS, 32), n);
    k_dual_eval<<<g, EVAL_THREADS, 0, st>>>(sd, list, (int)P.N, P.Nx, DV_S + 2 * P.ring, dv, rstate, w,
                                            reinterpret_cast<float4 *>(R), acc);
}


void launch_dual_ws_init(const Problem &P, const int32_t *list, int n, double c, double qscale, const int32_t *rq,
                         const float2 *KR, float2 *dv, cudaStream_t st, const int *cnt)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Nx * 4, 256 * 4, 64), n);
    k_dual_ws_init<<<g, 256, 0, st>>>(list, P.Nx, DV_S + 2 * P.ring, c, 1.0 / qscale, rq, KR, dv, cnt);
}

void launch_dual_to_r(const Problem &P, const DualCtl *ctl, const int32_t *list, int n, int which,
                      const float2 *dv, float *R, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Nx, 256 * 4, 64), n);
    k_dual_to_r<<<g, 256, 0, st>>>(ctl, list, P.Nx, (int)P.N, DV_S + 2 * P.ring, which, dv,
                                   reinterpret_cast<float4 *>(R));
}

void launch_dual_digits(const Problem &P, const SlotDev *sd, const int32_t *list, int n, int d, const float2 *dv,
                        float *R, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Nx, 256 * 4, 64), n);
    k_dual_digits<<<g, 256, 0, st>>>(sd, list, P.Nx, (int)P.N, DV_S + 2 * P.ring, d, dv,
                                     reinterpret_cast<float4 *>(R));
}

void launch_dual_digit_acc(const Problem &P, const SlotDev *sd, const int32_t *list, int n, int d,
                           const float *gpool, double *J64, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Dp, 256 * 16, 256), n);
    k_dual_digit_acc<<<g, 256, 0, st>>>(sd, list, P.Dp, d, gpool, reinterpret_cast<long long *>(J64));
}

void launch_dual_digits3(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float2 *dv, float *R,
                         cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Nx, 256 * 4, 64), n);
    k_dual_digits3<<<g, 256, 0, st>>>(sd, list, n, P.Nx, (int)P.N, DV_S + 2 * P.ring, dv,
                                      reinterpret_cast<float4 *>(R));
}

void launch_dual_planes_to_wa(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const float *gpool,
                              float *wa, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Dp / 4, 256 * 8, 256), n);
    k_dual_planes_to_wa<<<g, 256, 0, st>>>(sd, list, n, (int)P.L, P.Dp, gpool, wa);
}

void launch_dual_to_wa(const Problem &P, const SlotDev *sd, const int32_t *list, int n, const double *J64,
                       float *wa, cudaStream_t st)
{
    if (n <= 0) return;
    dim3 g(grid_for(P.Dp, 256 * 16, 256), n);
    k_dual_to_wa<<<g, 256, 0, st>>>(sd, list, (int)P.L, P.Dp, reinterpret_cast<const long long *>(J64), wa);
}

void launch_dual_linesearch(const Problem &P, DualCtl *ctl, const int32_t *list, int n, const double *dacc,
                            float2 *dv, float *ud, const uint8_t *rstate,
                            const float *w, const float *P0, float *R, double *acc, cudaStream_t st, const int *cnt)
{
    if (n <= 0) return;
    static const int threads = [] {
        const char *e = std::getenv("SDCA_LS_THREADS");
        const int v = e ? std::atoi(e) : 128;
        return (v == 64 || v == 256) ? v : 128;
    }();
#define SDCA_LS_LAUNCH(T)                                                                                          \
    k_dual_linesearch<T><<<n, T, 0, st>>>(ctl, list, (int)P.N, P.Nx, DV_S + 2 * P.ring, P.lambda_J, P.lambda_h,   \
                                          dacc, dv, reinterpret_cast<float4 *>(ud), rstate, w,                    \
                                          reinterpret_cast<const float4 *>(P0), reinterpret_cast<float4 *>(R), acc, \
                                          cnt)
    if (threads == 64) SDCA_LS_LAUNCH(64);
    else if (threads == 256) SDCA_LS_LAUNCH(256);
    else SDCA_LS_LAUNCH(128);
#undef SDCA_LS_LAUNCH
}

void launch_dual_control(const Problem &P, DualCtl *ctl, DualSum *sum, const int32_t *list, int n,
                         int max_iterations, double gtol, const double *acc, const double *amax, const double *dots,
                         cudaStream_t st, const int *cnt)
{
    if (n <= 0) return;
    k_dual_control<<<n, 32, 0, st>>>(ctl, sum, list, P.m, max_iterations, gtol, P.lambda_J, P.lambda_h, acc, amax,
                                     dots, cnt);
}

void launch_dual_check_apply(DualCtl *ctl, DualSum *sum, const int32_t *list, int n, double gtol, const double *acc,
                             cudaStream_t st)
{
    if (n <= 0) return;
    k_dual_check_apply<<<(n + 63) / 64, 64, 0, st>>>(ctl, sum, list, n, gtol, acc);
}

} // namespace sdca
