// Double-word FP32 ("hi + lo") helpers on packed f32x2 lanes, shared by the
// Celio and Lindblad double-word kernels.  A complex value is a float4
// (re_hi, im_hi, re_lo, im_lo); lanes of a 64-bit register carry (re, im).
#pragma once

#include "msp_common.cuh"

namespace msp {

typedef unsigned long long u64;

__device__ __forceinline__ u64 add2(u64 a, u64 b) {
    u64 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 sub2(u64 a, u64 b) {
    u64 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ float4 dw_split(double2 v) {
    const float hr = (float)v.x, hi = (float)v.y;
    return make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

__device__ __forceinline__ double2 dw_join(float4 v) {
    return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
}

// s + p = t + err exactly (both lanes, no ordering needed); err goes into c
__device__ __forceinline__ void two_sum2(u64 &s, u64 p, u64 &c) {
    const u64 t = add2(s, p);
    const u64 bb = sub2(t, s);
    const u64 err = add2(sub2(s, sub2(t, bb)), sub2(p, bb));
    s = t;
    c = add2(c, err);
}

// (a, b) -> (-b, a): multiplication by i of a lane pair
__device__ __forceinline__ u64 times_i(u64 v) {
    float a, b;
    split_f32x2(v, a, b);
    return f32x2(-b, a);
}

// y = S1 + i S2 from the two anchored sums (s already minus the anchor K,
// c their compensations), then hi = s + c and lo = its rounding error;
// returned as (re_hi, im_hi, re_lo, im_lo).
__device__ __forceinline__ float4 dw_finish(u64 s1, u64 c1, u64 s2, u64 c2) {
    two_sum2(s1, times_i(s2), c1);
    c1 = add2(c1, times_i(c2));
    u64 hi = s1, lo = 0ull;
    two_sum2(hi, c1, lo);
    float hr, him, lr, lim;
    split_f32x2(hi, hr, him);
    split_f32x2(lo, lr, lim);
    return make_float4(hr, him, lr, lim);
}

// Smallest power of two above b >= 0 (2^-126 for b = 0).
__device__ __forceinline__ float pow2_above(float b) {
    const unsigned e = (__float_as_uint(b) >> 23) & 0xffu;
    return __uint_as_float((e + 1u) << 23);
}

}  // namespace msp
