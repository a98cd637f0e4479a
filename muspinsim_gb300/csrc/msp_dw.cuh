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

// ---- double-word scalars: a value hi + lo as a float2 (x = hi, y = lo),
// normalised (|lo| <= half an ulp of hi) unless stated otherwise.  About
// 2^-48 relative accuracy: eigenvalues and phase increments of the
// mixed-precision paths are kept in this form so that those paths need no
// FP64 arithmetic (FP64 runs at a small fraction of the FP32 rate here).

#define MSP_TWOPI_HI 6.28318548202514648f      // fl32(2 pi)
#define MSP_TWOPI_LO (-1.7484555314695172e-07f)  // 2 pi - MSP_TWOPI_HI

// (h, l) <- (h + l) reduced modulo 2 pi, then renormalised (|l| <= half an
// ulp of h).  k * MSP_TWOPI_HI is split exactly by an FMA and h - p is
// exact (Sterbenz), so only the low-word sum rounds; the _rn intrinsics keep
// the compiler from contracting the split.
__device__ __forceinline__ void dw_reduce_2pi(float &h, float &l) {
    const float k = rintf(h * 0.15915494309189535f);
    const float p = __fmul_rn(k, MSP_TWOPI_HI);
    const float e = fmaf(k, MSP_TWOPI_HI, -p);
    const float t = __fsub_rn(h, p);
    const float lo = (l - e) - k * MSP_TWOPI_LO;
    const float s = __fadd_rn(t, lo);
    const float bb = __fsub_rn(s, t);
    l = __fadd_rn(__fsub_rn(t, __fsub_rn(s, bb)), __fsub_rn(lo, bb));
    h = s;
}

// (h, l) += (h2, l2), the high sum split exactly (TwoSum).
__device__ __forceinline__ void dw_add(float &h, float &l, float h2, float l2) {
    const float s = __fadd_rn(h, h2);
    const float bb = __fsub_rn(s, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
    h = s;
    l = l + l2 + err;
}

// a + b exactly as hi + lo (TwoSum, Knuth)
__device__ __forceinline__ float2 dw_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}

// a + b (double-word plus float), normalised
__device__ __forceinline__ float2 dw_add_f(float2 a, float b) {
    const float2 t = dw_two_sum(a.x, b);
    return dw_two_sum(t.x, __fadd_rn(t.y, a.y));
}

// a - b as a double-word
__device__ __forceinline__ float2 dw_sub(float2 a, float2 b) {
    const float2 t = dw_two_sum(a.x, -b.x);
    return dw_two_sum(t.x, __fadd_rn(t.y, __fsub_rn(a.y, b.y)));
}

// a - b rounded to FP32 (the high words' difference is exact when they are
// within a factor of two of each other, and FP32-accurate otherwise)
__device__ __forceinline__ float dw_sub_f(float2 a, float2 b) {
    return __fadd_rn(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}

// a < b for normalised double-words
__device__ __forceinline__ bool dw_less(float2 a, float2 b) {
    return a.x < b.x || (a.x == b.x && a.y < b.y);
}

__device__ __forceinline__ bool dw_equal(float2 a, float2 b) { return a.x == b.x && a.y == b.y; }

__host__ __device__ __forceinline__ float2 dw_of(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

__device__ __forceinline__ double dw_to_double(float2 a) { return (double)a.x + (double)a.y; }

// Rayleigh quotient S / (1 + g) of a refinement step for double-words S
// and g = G - 1 (|g| << 1: X^H X close to I), as S - S g + S g^2 / (1 + g)
// with S.hi g.hi split exactly by an FMA and every smaller term summed in
// FP32: ~2e-14 relative for |g| <= 3e-5, 3e-13 at |g| = 1e-3 (an FP32
// quotient would lose |g| 2^-24 relative: 1e-12 of l at |g| ~ 1e-5).
__device__ __forceinline__ float2 dw_rayleigh(float2 S, float2 g) {
    const float p = __fmul_rn(S.x, g.x);
    const float pe = fmaf(S.x, g.x, -p);
    const float gs = g.x + g.y;
    const float q2 = gs * gs / (1.0f + gs);
    const float c = S.y - pe - S.x * g.y - S.y * g.x + S.x * q2;
    const float2 t = dw_two_sum(S.x, -p);
    return dw_two_sum(t.x, __fadd_rn(t.y, c));
}

// d * c reduced modulo 2 pi (double-words d, c): the phase step of a level
// pair, d the level gap and c = 2 pi dt.
__device__ __forceinline__ float2 dw_phase_mod2pi(float2 d, float2 c) {
    float h = __fmul_rn(d.x, c.x);
    float l = fmaf(d.x, c.y, fmaf(d.y, c.x, fmaf(d.x, c.x, -h)));
    dw_reduce_2pi(h, l);
    return make_float2(h, l);
}

// Warp sum of double-words (every lane gets the total).
__device__ __forceinline__ float2 dw_warp_sum(float2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_xor_sync(0xffffffffu, v.x, o);
        const float l = __shfl_xor_sync(0xffffffffu, v.y, o);
        const float2 t = dw_two_sum(v.x, h);
        v = dw_two_sum(t.x, __fadd_rn(t.y, __fadd_rn(v.y, l)));
    }
    return v;
}

// CTA sum of every thread's double-word v; red holds one float2 per warp.
// All threads call it; the result is valid in every thread.  Begins and
// ends with a barrier (red may be reused right after).
__device__ __forceinline__ double dw_block_sum(float2 v, float2 *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = dw_warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float2 t = make_float2(0.f, 0.f);
    for (int w = 0; w < nw; ++w) {
        const float2 u = dw_two_sum(t.x, red[w].x);
        t = dw_two_sum(u.x, __fadd_rn(u.y, __fadd_rn(t.y, red[w].y)));
    }
    __syncthreads();
    return dw_to_double(t);
}

}  // namespace msp
