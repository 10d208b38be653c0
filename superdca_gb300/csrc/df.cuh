// df.cuh -- double-float arithmetic: a value is the unevaluated sum hi + lo
// of two floats (float2 {x = hi, y = lo}, |lo| <= ulp(hi) / 2), about 48
// significant bits, computed on the FP32 pipe.  GB300 runs FP64 at a small
// fraction of its FP32 rate, so the dual form keeps its coefficient vectors
// in this format: the same 8 bytes per value as a double.
//
// Error-free transformations: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum
// (Dekker 1971, |a| >= |b|), and TwoProd by a fused multiply-add.  Sums use
// the "sloppy" double-float addition (Dekker): its error is within a few
// units of 2^-48 of the larger operand, which is the scale every use here
// needs (sums of terms, not of cancelled results).  No -use_fast_math: the
// transformations rely on IEEE round-to-nearest and no reassociation.
#pragma once

#include <cstdint>

namespace sdca {

__device__ __forceinline__ float2 df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return make_float2(s, e);
}

__device__ __forceinline__ float2 df_fast_two_sum(float a, float b)
{
    const float s = a + b;
    return make_float2(s, b - (s - a));
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    float2 s = df_two_sum(a.x, b.x);
    s.y += a.y + b.y;
    return df_fast_two_sum(s.x, s.y);
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_fast_two_sum(p, e);
}

// acc + c x
__device__ __forceinline__ float2 df_fma(float2 c, float2 x, float2 acc)
{
    const float p = c.x * x.x;
    float e = fmaf(c.x, x.x, -p);
    e = fmaf(c.x, x.y, e);
    e = fmaf(c.y, x.x, e);
    float2 s = df_two_sum(acc.x, p);
    s.y += acc.y + e;
    return df_fast_two_sum(s.x, s.y);
}

// conversions (FP64 instructions: for per-block scalars and the few values
// that meet FP64 data)
__device__ __forceinline__ float2 df_from_d(double x)
{
    const float hi = __double2float_rn(x);
    return make_float2(hi, __double2float_rn(x - (double)hi));
}

__device__ __forceinline__ double df_to_d(float2 a) { return (double)a.x + (double)a.y; }

// the same split on the host, for kernel arguments
__host__ __device__ __forceinline__ float2 df_host(double x)
{
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// exact for |v| < 2^31
__device__ __forceinline__ float2 df_from_int(int v)
{
    const float hi = __int2float_rn(v);
    return make_float2(hi, __int2float_rn(v - __float2int_rn(hi)));
}

// 48 bits of a 64-bit integer (|v| < 2^62)
__device__ __forceinline__ float2 df_from_ll(long long v)
{
    const float hi = __ll2float_rn(v);
    return make_float2(hi, __ll2float_rn(v - __float2ll_rn(hi)));
}

// 48 bits of a 64-bit integer (|v| < 2^62) from its 32-bit halves, with
// 32-bit conversions and FP32 arithmetic only: v = hi 2^32 + lo, lo in
// [0, 2^32) as 2^16 lo_h + lo_l, each part exact as a float or a
// double-float, summed in double-float.
__device__ __forceinline__ float2 df_from_ll_fast(long long v)
{
    const int hi = (int)(v >> 32);
    const unsigned lo = (unsigned)(v & 0xffffffffll);
    const float hh = __int2float_rn(hi);
    const float hl = __int2float_rn(hi - __float2int_rn(hh));        // hi = hh + hl exactly (|hi| < 2^30)
    const float lh = __uint2float_rn(lo >> 16) * 65536.0f;           // exact: < 2^32, 16 significant bits
    const float ll = __uint2float_rn(lo & 0xffffu);                  // exact
    float2 r = df_two_sum(hh * 4294967296.0f, hl * 4294967296.0f);   // powers of two: exact products
    r = df_add(r, df_two_sum(lh, ll));
    return r;
}

__device__ __forceinline__ float2 df_zero() { return make_float2(0.f, 0.f); }

// value as a float (rounded)
__device__ __forceinline__ float df_f(float2 a) { return a.x + a.y; }

// sum over the warp, in double-float (lane 0 holds it)
__device__ __forceinline__ float2 df_warp_sum(float2 v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, v.x, off), __shfl_xor_sync(0xffffffffu, v.y, off));
        v = df_add(v, o);
    }
    return v;
}

// Sum K per-thread double-float values over the block and add them to
// dst[idx[k]] (FP64 atomics): warp sums in double-float, the warps' sums in
// double-float by the first warp, one conversion and one atomic per value
// (GB300's FP64 pipe is narrow: only the conversion and the atomic use it).
template <int K>
__device__ __forceinline__ void block_sum_df(float2 (&v)[K], double *dst, const int *idx)
{
    __shared__ float2 red_df[32][K];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float2 s = df_warp_sum(v[k]);
        if (lane == 0) red_df[wid][k] = s;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 t = df_warp_sum(lane < nw ? red_df[lane][k] : df_zero());
            if (lane == 0 && (t.x != 0.f || t.y != 0.f)) atomicAdd(dst + idx[k], df_to_d(t));
        }
    }
    __syncthreads();
}

} // namespace sdca
