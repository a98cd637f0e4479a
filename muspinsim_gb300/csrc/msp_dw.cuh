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

// ---- anchored double-word product sums (shared by the refinement kernels)
//
// A sum of products starts at an anchor K, a power of two >= 4.01 times a
// bound on the sum's magnitude (|row| |column| by Cauchy-Schwarz), so every
// partial sum stays within a factor of two of K: s - fl(s + p) is then
// exact, and fma(a, b, s - t) is the rounding error of t = fl(s + a b).
// Errors accumulate in a compensation term; the anchor is subtracted
// exactly at the end.

__device__ __forceinline__ u64 lm_anchor(float bound) {
    const float K = pow2_above(4.01f * bound);
    return f32x2(K, K);
}

// Anchored double-word product-sum step for one complex product a b:
// ah = (a.re, a.im) as stored (one 64-bit register pair), bx = (b.re,
// b.re), by = (b.im, b.im) (duplicated once per k and shared by a
// thread's four outputs):
//   S1 += ah bx = (a.re b.re, a.im b.re),  S2 += ah by = (a.re b.im, a.im b.im),
// so that a b = S1 + i S2 (lane-wise: re = S1.x - S2.y, im = S1.y + S2.x)
// and conj(a) b = conj(S1) + i conj(S2); rounding errors into c1, c2.  The
// lo parts: al (A's, ALO) times bx, by; ah times blx, bly (B's, BLO).
template <bool ALO, bool BLO>
__device__ __forceinline__ void lm_step(u64 &s1, u64 &c1, u64 &s2, u64 &c2, u64 ah, u64 al, u64 bx,
                                        u64 by, u64 blx, u64 bly) {
    const u64 t1 = fma_f32x2(ah, bx, s1);
    const u64 t2 = fma_f32x2(ah, by, s2);
    c1 = add2(c1, fma_f32x2(ah, bx, sub2(s1, t1)));
    c2 = add2(c2, fma_f32x2(ah, by, sub2(s2, t2)));
    s1 = t1;
    s2 = t2;
    if (BLO) {
        c1 = fma_f32x2(ah, blx, c1);
        c2 = fma_f32x2(ah, bly, c2);
    }
    if (ALO) {
        c1 = fma_f32x2(al, bx, c1);
        c2 = fma_f32x2(al, by, c2);
    }
}

// (re, im) -> (re, -im) on a lane pair: the sign bit of the upper lane
__device__ __forceinline__ u64 lm_conj2(u64 v) { return v ^ 0x8000000000000000ull; }

// The double-word value of an anchored sum pair (a b, or conj(a) b when
// CONJ), anchor K removed: (re_hi, im_hi, re_lo, im_lo).
template <bool CONJ>
__device__ __forceinline__ float4 lm_dw(u64 s1, u64 c1, u64 s2, u64 c2, u64 K) {
    s1 = sub2(s1, K);  // exact
    s2 = sub2(s2, K);
    if (CONJ) {
        s1 = lm_conj2(s1);
        c1 = lm_conj2(c1);
        s2 = lm_conj2(s2);
        c2 = lm_conj2(c2);
    }
    return dw_finish(s1, c1, s2, c2);
}

// The FP32 value of a plain sum pair (a b, or conj(a) b when CONJ).
template <bool CONJ>
__device__ __forceinline__ cx<float> lm_plain(u64 s1, u64 s2) {
    float ax, ay, bx, by;
    split_f32x2(s1, ax, ay);
    split_f32x2(s2, bx, by);
    return CONJ ? mk<float>(ax + by, bx - ay) : mk<float>(ax - by, ay + bx);
}

}  // namespace msp
