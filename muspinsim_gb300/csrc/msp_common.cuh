// Shared device helpers for the muon polarisation kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mspgpu.h"

namespace msp {

template <typename T>
struct cx {
    T re, im;
};

template <typename T>
__device__ __forceinline__ cx<T> mk(T re, T im) {
    cx<T> r;
    r.re = re;
    r.im = im;
    return r;
}

template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mk<T>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}

// conj(a) * b
template <typename T>
__device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
    return mk<T>(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}

template <typename T>
__device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) {
    return mk<T>(a.re + b.re, a.im + b.im);
}

template <typename T>
__device__ __forceinline__ cx<T> cscale(T s, cx<T> a) {
    return mk<T>(s * a.re, s * a.im);
}

template <typename T>
__device__ __forceinline__ T cabs2(cx<T> a) {
    return a.re * a.re + a.im * a.im;
}

template <typename T>
__device__ __forceinline__ cx<T> conj(cx<T> a) {
    return mk<T>(a.re, -a.im);
}

// Phase reduction: x mod 2 pi into [-pi, pi], in double.  Two-term 2 pi so
// that phases of order 1e5 rad keep ~1e-16 absolute accuracy.
__device__ __forceinline__ double reduce_2pi(double x) {
    const double inv2pi = 0.15915494309189533577;
    const double twopi_hi = 6.28318530717958623200;
    const double twopi_lo = 2.44929359829470635445e-16;
    double k = rint(x * inv2pi);
    double r = fma(-k, twopi_hi, x);
    return fma(-k, twopi_lo, r);
}

// x / d by multiply and shift with c = ceil(2^20 / d): exact whenever
// 0 <= x < 2^20 / d (x * c then fits 32 bits and the rounding excess stays
// below 1/d), which covers every index of an m x m matrix with m <= 64.
struct FastDiv {
    unsigned int c;
    __device__ __forceinline__ explicit FastDiv(int d)
        : c(((1u << 20) + (unsigned)d - 1u) / (unsigned)d) {}
    __device__ __forceinline__ int div(int x) const {
        return (int)(((unsigned)x * c) >> 20);
    }
};

// Double-word ("df32") accumulation on the FP32 pipe: (hi, lo) += a * b with
// the product split exactly (TwoProduct via FMA) and the running sum kept by
// TwoSum (Knuth), the low words summed plainly.  About 2^-44 relative
// accuracy for short dot products; the _rn intrinsics keep the compiler
// from contracting or reassociating the error terms.
__device__ __forceinline__ void dw_acc(float &hi, float &lo, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = fmaf(a, b, -p);
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
}

// Packed FP32 pairs (Blackwell f32x2 instructions): two lanes in one 64-bit
// register, one instruction for both.
__device__ __forceinline__ unsigned long long f32x2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void split_f32x2(unsigned long long v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long fma_f32x2(unsigned long long a, unsigned long long b,
                                                        unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long mul_f32x2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// Block-wide sum of two values; every thread receives the totals.  `red`
// needs 2 * (blockDim.x / 32) entries of shared memory.
template <typename T>
__device__ __forceinline__ void block_sum2(T &a, T &b, T *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __syncthreads();
    if (lane == 0) {
        red[warp] = a;
        red[nw + warp] = b;
    }
    __syncthreads();
    a = 0;
    b = 0;
    for (int w = 0; w < nw; ++w) {
        a += red[w];
        b += red[nw + w];
    }
    __syncthreads();
}

}  // namespace msp
