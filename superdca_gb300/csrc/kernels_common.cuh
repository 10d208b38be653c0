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

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
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
        const __nv_bfloat162 *p = reinterpret_cast<const __nv_bfloat162 *>(
            reinterpret_cast<const __nv_bfloat16 *>(base) + off);
        const float2 a = __bfloat1622float2(p[0]);
        const float2 b = __bfloat1622float2(p[1]);
        return make_float4(a.x, a.y, b.x, b.y);
    }
    return *reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(base) + off);
}

// store and return the value as it reads back
__device__ __forceinline__ float4 store_hist4(void *base, int64_t off, float4 v, int bf16)
{
    if (bf16) {
        __nv_bfloat162 *p = reinterpret_cast<__nv_bfloat162 *>(
            reinterpret_cast<__nv_bfloat16 *>(base) + off);
        const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
        const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
        p[0] = a;
        p[1] = b;
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

} // namespace sdca
