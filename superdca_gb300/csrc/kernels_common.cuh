// kernels_common.cuh -- small device helpers shared by the engine kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sdca {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max_d(double v)
{
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    return v;
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum K per-thread values over the block; thread 0 adds them to dst[idx[k]].
// Warp sums run in FP32 (each thread's value is itself an FP32 partial over
// a stretch of one vector), the cross-warp sum in FP64.
// Requires blockDim.x a multiple of 32 and <= 1024.
template <int K>
__device__ __forceinline__ void block_sum_atomic_f(float (&v)[K], double *dst, const int *idx)
{
    __shared__ double redf[32][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum_f(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) redf[wid][k] = (double)v[k];
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < K; ++k) {
            double t = lane < nw ? redf[lane][k] : 0.0;
            t = warp_sum(t);
            if (lane == 0 && t != 0.0) atomicAdd(dst + idx[k], t);
        }
    }
    __syncthreads();
}

// Sum K per-thread values over the block; thread 0 adds them to dst[0..K-1].
// Requires blockDim.x a multiple of 32 and <= 1024.
template <int K>
__device__ __forceinline__ void block_sum_atomic(double (&v)[K], double *dst, const int *idx)
{
    __shared__ double red[32][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[wid][k] = v[k];
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double t = lane < nw ? red[lane][k] : 0.0;
            t = warp_sum(t);
            if (lane == 0 && t != 0.0) atomicAdd(dst + idx[k], t);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v)
{
    // ordering of non-negative IEEE doubles equals the ordering of their bits
    atomicMax(reinterpret_cast<unsigned long long *>(addr),
              static_cast<unsigned long long>(__double_as_longlong(v)));
}

// history vectors are stored as float or as bf16
__device__ __forceinline__ float4 load_hist4(const void *base, int64_t off, int bf16)
{
    if (bf16) {
        // one 8-byte load for four values (off is a multiple of 4)
        const uint2 raw = *reinterpret_cast<const uint2 *>(reinterpret_cast<const __nv_bfloat16 *>(base) + off);
        return make_float4(__uint_as_float(raw.x << 16), __uint_as_float(raw.x & 0xFFFF0000u),
                           __uint_as_float(raw.y << 16), __uint_as_float(raw.y & 0xFFFF0000u));
    }
    return *reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(base) + off);
}

// store and return the value as it reads back
__device__ __forceinline__ float4 store_hist4(void *base, int64_t off, float4 v, int bf16)
{
    if (bf16) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
        const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
        uint2 raw;
        raw.x = *reinterpret_cast<const uint32_t *>(&a);
        raw.y = *reinterpret_cast<const uint32_t *>(&b);
        *reinterpret_cast<uint2 *>(reinterpret_cast<__nv_bfloat16 *>(base) + off) = raw;
        const float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
        return make_float4(fa.x, fa.y, fb.x, fb.y);
    }
    *reinterpret_cast<float4 *>(reinterpret_cast<float *>(base) + off) = v;
    return v;
}

__device__ __forceinline__ float dot4(float4 a, float4 b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
}

struct GradRed {
    float gmax = 0.f, g2 = 0.f, x2 = 0.f, sy = 0.f, yy = 0.f, ss = 0.f;
};

// Gradient of the 16 J entries of locus n for one slot: g = c + 2 lambda_J x
// (c the contraction X^T R), zero for the J_rr block; writes g to the new
// gradient buffer and, with a history push, y = g - g_old to the ring.
// SuperDCA: plmDCA_objective.hpp:153-190 (scatter) and 192-244 (L2 part).
template <typename SlotT>
__device__ __forceinline__ void grad_locus(const SlotT &S, int b, int64_t n, const float (&c)[16],
                                           const float *__restrict__ wa, float *__restrict__ gpool,
                                           void *__restrict__ Ypool, const void *__restrict__ Spool,
                                           int hist_bf16, int ring, int64_t Dp, float l2, GradRed &red)
{
    const float *x = wa + (int64_t)b * Dp + n * 16;
    float *gn = gpool + (int64_t)(2 * b + 1 - S.gcur) * Dp + n * 16;
    const float *go = gpool + (int64_t)(2 * b + S.gcur) * Dp + n * 16;
    const bool zero = (n == S.locus);
    const bool push = (S.flags & 2) && S.ring_new >= 0;
    const int64_t hoff = ((int64_t)b * ring + (push ? S.ring_new : 0)) * Dp + n * 16;
#pragma unroll
    for (int k4 = 0; k4 < 4; ++k4) {
        const float4 xv = reinterpret_cast<const float4 *>(x)[k4];
        float4 gv;
        gv.x = zero ? 0.f : c[4 * k4 + 0] + l2 * xv.x;
        gv.y = zero ? 0.f : c[4 * k4 + 1] + l2 * xv.y;
        gv.z = zero ? 0.f : c[4 * k4 + 2] + l2 * xv.z;
        gv.w = zero ? 0.f : c[4 * k4 + 3] + l2 * xv.w;
        reinterpret_cast<float4 *>(gn)[k4] = gv;
        red.gmax = fmaxf(red.gmax, fmaxf(fmaxf(fabsf(gv.x), fabsf(gv.y)), fmaxf(fabsf(gv.z), fabsf(gv.w))));
        red.g2 += dot4(gv, gv);
        red.x2 += dot4(xv, xv);
        if (push) {
            const float4 ov = reinterpret_cast<const float4 *>(go)[k4];
            float4 yv = make_float4(gv.x - ov.x, gv.y - ov.y, gv.z - ov.z, gv.w - ov.w);
            yv = store_hist4(Ypool, hoff + 4 * k4, yv, hist_bf16);
            const float4 sv = load_hist4(Spool, hoff + 4 * k4, hist_bf16);
            red.sy += dot4(sv, yv);
            red.yy += dot4(yv, yv);
            red.ss += dot4(sv, sv);
        }
    }
}

} // namespace sdca
