// Cyclic two-sided Jacobi for one complex Hermitian matrix held in shared
// memory by one CTA.  Replaces the LAPACK zheevd call of Hermitian.diag
// (muspinsim/spinop.py:51-82).
//
// Schedule: round-robin ("circle") ordering over m = even padded dimension,
// m-1 steps per sweep, m/2 disjoint rotations per step.  Pair k of step r is
// (a_k, b_k) = (r, m-1) for k = 0 and ((r+k) mod (m-1), (r-k) mod (m-1))
// otherwise; each pair of the next step takes one member from each of two
// pairs of this step, by a rule that does not depend on r (jacobi_succ).
//
// One step is one phase between two __syncthreads():
//   * H <- G^dag H G on 2x2 blocks (rows of pair k1, columns of pair k2,
//     k1 <= k2); H is kept as its upper triangle, an element below the
//     diagonal being read and written as the conjugate of its mirror;
//     diagonal blocks become diag(a', b') exactly.  The block that holds the element (a'_j, b'_j) of next-step
//     pair j also computes that pair's rotation, from the new element and
//     the new diagonal entries (known from this step's rotations), so no
//     separate rotation phase and barrier are needed.
//   * U <- U G on the eigenvector matrix, kept as separate real and
//     imaginary column planes: a task updates 4 consecutive rows of the two
//     columns of one pair with 128-bit loads and (FP32) packed f32x2 FMAs.
// A sweep starts with a block reduction of the off-diagonal and total
// Frobenius norms; the loop stops when off <= tol^2 * total, when a sweep
// no longer shrinks off (rounding floor, FP32), or at max_sweeps (status
// MSP_ITEM_NOT_CONVERGED).  Padding: when n is odd, index m-1 = n is a zero
// row/column; its rotations are the identity.
//
// On return the eigenvectors are interleaved complex columns of w.U (row
// stride m + 1) and w.diag holds the eigenvalues (unsorted); w.H and w.U
// have swapped buffers, and the buffer now at w.H is free.
#pragma once

#include "msp_common.cuh"

namespace msp {

// Rotation G = [[c, s], [-conj(s), c]] on the ordered pair (a, b), packed
// ab = a | b << 16 (16 bytes in FP32: one 128-bit load).
template <typename T>
struct __align__(16) JRot {
    T c, sr, si;
    int ab;
    __device__ __forceinline__ int a() const { return ab & 0xffff; }
    __device__ __forceinline__ int b() const { return ab >> 16; }
};

template <typename T>
struct JacobiWork {
    // H and U are two buffers of jacobi_buffer(m) complex entries each.
    cx<T> *H;      // the matrix: interleaved, row-major, row stride
                   // jacobi_ldh(m); the sweeps keep the upper triangle only
    cx<T> *U;      // during the sweeps: the eigenvector planes (real part,
                   // column c row r at c * ldu + r, then the imaginary
                   // part); on return: eigenvectors, interleaved, row
                   // stride m + 1
    JRot<T> *rot;  // 2 x m/2 (double-buffered by step parity)
    T *dia;        // 2 x m/2 x 2: new diagonal entries (a', b') of each pair
    uint2 *tab;    // m/2 (m/2 + 1) / 2 block tasks: (k1 | k2 << 8, successor entries)
    T *red;        // 2 * warps scratch
    T *diag;       // m eigenvalues on return
};

template <typename T>
struct JacobiConst;
template <>
struct JacobiConst<double> {
    static constexpr double tol = 4e-15;
    static constexpr double floor_tol = 1e-13;
    static constexpr double big = 1e150;
};
template <>
struct JacobiConst<float> {
    static constexpr float tol = 4e-7f;
    static constexpr float floor_tol = 2e-5f;
    static constexpr float big = 1e18f;
};

// Column stride of the eigenvector planes: m rounded up to a multiple of 4
// (16-byte aligned 4-row groups for 128-bit loads).  Rows m .. ldu-1 stay
// zero.  Consecutive pairs rotate consecutive columns, so a quarter-warp of
// 4-row tasks mostly reads one contiguous 128-byte span.
__host__ __device__ inline int jacobi_ldu(int m) { return (m + 3) & ~3; }

// Row stride of the matrix during the sweeps (even: with the 2x2 block
// access pattern of the circle schedule it spreads 8-byte elements over the
// banks best).
__host__ __device__ inline int jacobi_ldh(int m) { return m + 2; }

// Elements per Jacobi buffer (complex): the matrix (row stride
// jacobi_ldh(m)), an m x m result with row stride m + 1, or the two
// eigenvector planes.
__host__ __device__ inline int jacobi_buffer(int m) {
    const int a = m * jacobi_ldh(m), b = m * jacobi_ldu(m);
    return a > b ? a : b;
}

// Next-step pair j <- (first member: pair p1 role r1, second: pair p2 role
// r2); role 0 = a, 1 = b.  Packed as p1 | r1 << 7 | p2 << 8 | r2 << 15.
__device__ __forceinline__ unsigned jacobi_succ(int j, int half) {
    int p1, r1, p2, r2;
    if (half == 1) {
        p1 = 0; r1 = 0; p2 = 0; r2 = 1;
    } else if (j == 0) {
        p1 = 1; r1 = 0; p2 = 0; r2 = 1;
    } else if (half == 2) {
        p1 = 1; r1 = 1; p2 = 0; r2 = 0;
    } else if (j == 1) {
        p1 = 2; r1 = 0; p2 = 0; r2 = 0;
    } else if (j <= half - 2) {
        p1 = j + 1; r1 = 0; p2 = j - 1; r2 = 1;
    } else {
        p1 = half - 1; r1 = 1; p2 = half - 2; r2 = 1;
    }
    return (unsigned)p1 | ((unsigned)r1 << 7) | ((unsigned)p2 << 8) | ((unsigned)r2 << 15);
}

// Whether block (k1 <= k2) holds the element of a next-step pair: the
// blocks of jacobi_succ in closed form.
__device__ __forceinline__ bool jacobi_produces(int k1, int k2, int half) {
    if (half == 1) return false;
    if (k1 == 0 && k2 == 1) return true;
    if (half < 3) return false;
    return (k1 == 0 && k2 == 2) || (k2 == k1 + 2 && k1 >= 1 && k1 <= half - 3) ||
           (k1 == half - 2 && k2 == half - 1);
}

// Rotation that zeroes apq = H[a][b] given app = H[a][a], aqq = H[b][b]:
// c, s and the new diagonal entries.  Couplings at or below `skip` are left.
template <typename T>
__device__ __forceinline__ void jacobi_rotation(T app, T aqq, cx<T> apq, T skip, int a, int b,
                                                JRot<T> &R, T &na, T &nb) {
    const T mag = sqrt(cabs2(apq));
    R.c = T(1);
    R.sr = T(0);
    R.si = T(0);
    R.ab = a | (b << 16);
    na = app;
    nb = aqq;
    if (mag > skip) {
        const T zeta = (aqq - app) / (T(2) * mag);
        T t;
        if (fabs(zeta) > JacobiConst<T>::big)
            t = T(0.5) / zeta;
        else
            t = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + t * t);
        const T f = t * c / mag;
        R.c = c;
        R.sr = f * apq.re;
        R.si = f * apq.im;
        na = app - t * mag;
        nb = aqq + t * mag;
    }
}

// U[:, a], U[:, b] <- (c x - conj(s) y, s x + c y) on rows r .. r+3.
__device__ __forceinline__ void jacobi_rotate_rows(float *Ur, float *Ui, int ia, int ib,
                                                   const JRot<float> &R) {
    const float4 xr = *reinterpret_cast<const float4 *>(Ur + ia);
    const float4 xi = *reinterpret_cast<const float4 *>(Ui + ia);
    const float4 yr = *reinterpret_cast<const float4 *>(Ur + ib);
    const float4 yi = *reinterpret_cast<const float4 *>(Ui + ib);
    const unsigned long long C = f32x2(R.c, R.c), SR = f32x2(R.sr, R.sr),
                             SI = f32x2(R.si, R.si), NSR = f32x2(-R.sr, -R.sr),
                             NSI = f32x2(-R.si, -R.si);
    float4 oxr, oxi, oyr, oyi;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const unsigned long long XR = h ? f32x2(xr.z, xr.w) : f32x2(xr.x, xr.y);
        const unsigned long long XI = h ? f32x2(xi.z, xi.w) : f32x2(xi.x, xi.y);
        const unsigned long long YR = h ? f32x2(yr.z, yr.w) : f32x2(yr.x, yr.y);
        const unsigned long long YI = h ? f32x2(yi.z, yi.w) : f32x2(yi.x, yi.y);
        // x' = c x - conj(s) y
        const unsigned long long AR = fma_f32x2(NSI, YI, fma_f32x2(NSR, YR, mul_f32x2(C, XR)));
        const unsigned long long AI = fma_f32x2(SI, YR, fma_f32x2(NSR, YI, mul_f32x2(C, XI)));
        // y' = s x + c y
        const unsigned long long BR = fma_f32x2(NSI, XI, fma_f32x2(SR, XR, mul_f32x2(C, YR)));
        const unsigned long long BI = fma_f32x2(SI, XR, fma_f32x2(SR, XI, mul_f32x2(C, YI)));
        if (h) {
            split_f32x2(AR, oxr.z, oxr.w);
            split_f32x2(AI, oxi.z, oxi.w);
            split_f32x2(BR, oyr.z, oyr.w);
            split_f32x2(BI, oyi.z, oyi.w);
        } else {
            split_f32x2(AR, oxr.x, oxr.y);
            split_f32x2(AI, oxi.x, oxi.y);
            split_f32x2(BR, oyr.x, oyr.y);
            split_f32x2(BI, oyi.x, oyi.y);
        }
    }
    *reinterpret_cast<float4 *>(Ur + ia) = oxr;
    *reinterpret_cast<float4 *>(Ui + ia) = oxi;
    *reinterpret_cast<float4 *>(Ur + ib) = oyr;
    *reinterpret_cast<float4 *>(Ui + ib) = oyi;
}

__device__ __forceinline__ void jacobi_rotate_rows(double *Ur, double *Ui, int ia, int ib,
                                                   const JRot<double> &R) {
#pragma unroll
    for (int h = 0; h < 4; h += 2) {
        const double2 xr = *reinterpret_cast<const double2 *>(Ur + ia + h);
        const double2 xi = *reinterpret_cast<const double2 *>(Ui + ia + h);
        const double2 yr = *reinterpret_cast<const double2 *>(Ur + ib + h);
        const double2 yi = *reinterpret_cast<const double2 *>(Ui + ib + h);
        double2 oxr, oxi, oyr, oyi;
        oxr.x = R.c * xr.x - R.sr * yr.x - R.si * yi.x;
        oxr.y = R.c * xr.y - R.sr * yr.y - R.si * yi.y;
        oxi.x = R.c * xi.x - R.sr * yi.x + R.si * yr.x;
        oxi.y = R.c * xi.y - R.sr * yi.y + R.si * yr.y;
        oyr.x = R.sr * xr.x - R.si * xi.x + R.c * yr.x;
        oyr.y = R.sr * xr.y - R.si * xi.y + R.c * yr.y;
        oyi.x = R.sr * xi.x + R.si * xr.x + R.c * yi.x;
        oyi.y = R.sr * xi.y + R.si * xr.y + R.c * yi.y;
        *reinterpret_cast<double2 *>(Ur + ia + h) = oxr;
        *reinterpret_cast<double2 *>(Ui + ia + h) = oxi;
        *reinterpret_cast<double2 *>(Ur + ib + h) = oyr;
        *reinterpret_cast<double2 *>(Ui + ib + h) = oyi;
    }
}

// This thread's share of the squared Frobenius norms of the Hermitian H
// from its upper triangle: off-diagonal (both triangles) and total.
template <typename T>
__device__ __forceinline__ void jacobi_norms(const cx<T> *H, int m, int ld, const FastDiv &fdm,
                                             T &off, T &fro) {
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
        const int i = fdm.div(e), j = e - i * m;
        if (j < i) continue;
        const T v = cabs2(H[i * ld + j]);
        if (i == j) {
            fro += v;
        } else {
            fro += T(2) * v;
            off += T(2) * v;
        }
    }
}

// Element (x, y) of the Hermitian matrix stored as its upper triangle.
template <typename T>
__device__ __forceinline__ cx<T> herm_load(const cx<T> *H, int ld, int x, int y) {
    const bool up = x <= y;
    cx<T> v = H[up ? x * ld + y : y * ld + x];
    if (!up) v.im = -v.im;
    return v;
}
template <typename T>
__device__ __forceinline__ void herm_store(cx<T> *H, int ld, int x, int y, cx<T> v) {
    const bool up = x <= y;
    if (!up) v.im = -v.im;
    H[up ? x * ld + y : y * ld + x] = v;
}

// Runs the sweeps on w.H (already loaded, m x m Hermitian, row stride
// jacobi_ldh(m); only the upper triangle is read).  All threads of
// the CTA must call it.  See the file comment for what it leaves where.
template <typename T>
__device__ int jacobi_sweeps(JacobiWork<T> &w, int m, int max_sweeps) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int half = m >> 1;
    const int nblk = half * (half + 1) / 2;
    const int ldu = jacobi_ldu(m);
    const int ngrp = (m + 3) >> 2;  // 4-row groups of a column
    const int ntask = nblk + half * ngrp;
    const T tol = JacobiConst<T>::tol;
    const int ld = jacobi_ldh(m);  // row stride of H during the sweeps
    const FastDiv fdm(m), fdg(ngrp);
    T *const Ur = reinterpret_cast<T *>(w.U);
    T *const Ui = Ur + m * ldu;

    for (int e = tid; e < m * ldu; e += nt) {
        const int c = e / ldu, r = e - c * ldu;
        Ur[e] = r == c ? T(1) : T(0);
        Ui[e] = T(0);
    }
    // Block tasks (k1 <= k2, packed k1 | k2 << 8) with their successor
    // entries: j | rr << 12 | cr << 13 | conj << 14 | valid << 15 for
    // next-step pair j, where rr / cr are the roles of the element's row in
    // pair k1 and column in pair k2, and conj means the element is the
    // mirror of the computed one (two entries per block at most: m = 4).
    // The blocks that hold next-step elements come first, so the rotation
    // arithmetic runs in as few warps as possible.
    if (tid == 0) {
        int pos = 0;
        for (int j = 0; j < half && half > 1; ++j) {
            const unsigned s = jacobi_succ(j, half);
            const int p1 = s & 127, r1 = (s >> 7) & 1, p2 = (s >> 8) & 127, r2 = (s >> 15) & 1;
            const int k1 = p1 < p2 ? p1 : p2, k2 = p1 < p2 ? p2 : p1;
            const unsigned cj = p1 < p2 ? 0u : 1u;
            const unsigned rr = p1 < p2 ? r1 : r2, cr = p1 < p2 ? r2 : r1;
            const unsigned ent = (unsigned)j | (rr << 12) | (cr << 13) | (cj << 14) | (1u << 15);
            const unsigned key = (unsigned)k1 | ((unsigned)k2 << 8);
            if (pos > 0 && w.tab[pos - 1].x == key)
                w.tab[pos - 1].y |= ent << 16;
            else
                w.tab[pos++] = make_uint2(key, ent);
        }
        for (int k2 = 0; k2 < half; ++k2)
            for (int k1 = 0; k1 <= k2; ++k1)
                if (!jacobi_produces(k1, k2, half))
                    w.tab[pos++] = make_uint2((unsigned)k1 | ((unsigned)k2 << 8), 0u);
    }
    T off = 0, fro = 0;
    jacobi_norms(w.H, m, ld, fdm, off, fro);
    block_sum2(off, fro, w.red);  // contains __syncthreads
    T skip = tol * sqrt(fro) / T(m);
    // rotations of step 0
    for (int k = tid; k < half; k += nt) {
        const int a = k == 0 ? 0 : k, b = k == 0 ? m - 1 : m - 1 - k;
        JRot<T> R;
        T na, nb;
        jacobi_rotation<T>(w.H[a * ld + a].re, w.H[b * ld + b].re, w.H[a * ld + b], skip, a, b, R,
                           na, nb);
        w.rot[k] = R;
        w.dia[2 * k] = na;
        w.dia[2 * k + 1] = nb;
    }
    __syncthreads();

    int status = MSP_ITEM_NOT_CONVERGED;
    T prev_off = T(-1);
    int cur = 0;
    for (int sweep = 0;; ++sweep) {
        if (sweep > 0) {
            off = 0;
            fro = 0;
            jacobi_norms(w.H, m, ld, fdm, off, fro);
            block_sum2(off, fro, w.red);
        }
        if (off <= tol * tol * fro) {
            status = MSP_ITEM_OK;
            break;
        }
        // rounding floor: already small, and a sweep no longer shrinks it
        {
            const T ft = JacobiConst<T>::floor_tol;
            if (prev_off >= T(0) && off > T(0.25) * prev_off && off <= ft * ft * fro) {
                status = MSP_ITEM_OK;
                break;
            }
        }
        if (sweep >= max_sweeps) break;
        prev_off = off;
        skip = tol * sqrt(fro) / T(m);

        for (int r = 0; r < m - 1; ++r) {
            const JRot<T> *rc = w.rot + cur * half;
            const T *dc = w.dia + cur * m;
            JRot<T> *rn = w.rot + (cur ^ 1) * half;
            T *dn = w.dia + (cur ^ 1) * m;
            for (int task = tid; task < ntask; task += nt) {
                if (task < nblk) {
                    const uint2 tb = w.tab[task];
                    const int k1 = (int)(tb.x & 0xffu), k2 = (int)(tb.x >> 8);
                    const JRot<T> R1 = rc[k1];
                    const int p = R1.a(), q = R1.b();
                    if (k1 == k2) {
                        const T na = dc[2 * k1], nb = dc[2 * k1 + 1];
                        w.H[p * ld + p] = mk<T>(na, T(0));
                        w.H[q * ld + q] = mk<T>(nb, T(0));
                        herm_store(w.H, ld, p, q, mk<T>(T(0), T(0)));
                        if (half == 1) {  // m = 2: the same pair again, already diagonal
                            JRot<T> Rn;
                            T a2, b2;
                            jacobi_rotation<T>(na, nb, mk<T>(T(0), T(0)), skip, p, q, Rn, a2, b2);
                            rn[0] = Rn;
                            dn[0] = a2;
                            dn[1] = b2;
                        }
                    } else {
                        const JRot<T> R2 = rc[k2];
                        const int p2 = R2.a(), q2 = R2.b();
                        const T c1 = R1.c, c2 = R2.c;
                        const cx<T> s1 = mk<T>(R1.sr, R1.si), s2 = mk<T>(R2.sr, R2.si);
                        const cx<T> b00 = herm_load(w.H, ld, p, p2), b01 = herm_load(w.H, ld, p, q2);
                        const cx<T> b10 = herm_load(w.H, ld, q, p2), b11 = herm_load(w.H, ld, q, q2);
                        // T = G1^dag B
                        const cx<T> t00 = cadd(cscale(c1, b00), cscale(T(-1), cmul(s1, b10)));
                        const cx<T> t01 = cadd(cscale(c1, b01), cscale(T(-1), cmul(s1, b11)));
                        const cx<T> t10 = cadd(cmulc(s1, b00), cscale(c1, b10));
                        const cx<T> t11 = cadd(cmulc(s1, b01), cscale(c1, b11));
                        // B' = T G2
                        const cx<T> n00 = cadd(cscale(c2, t00), cscale(T(-1), cmulc(s2, t01)));
                        const cx<T> n01 = cadd(cmul(s2, t00), cscale(c2, t01));
                        const cx<T> n10 = cadd(cscale(c2, t10), cscale(T(-1), cmulc(s2, t11)));
                        const cx<T> n11 = cadd(cmul(s2, t10), cscale(c2, t11));
                        herm_store(w.H, ld, p, p2, n00);
                        herm_store(w.H, ld, p, q2, n01);
                        herm_store(w.H, ld, q, p2, n10);
                        herm_store(w.H, ld, q, q2, n11);
                        // rotations of the next step whose element is in this block
                        unsigned ents = tb.y;
                        while (ents) {
                            const unsigned ent = ents & 0xffffu;
                            ents >>= 16;
                            if (!(ent & 0x8000u)) continue;
                            const int j = (int)(ent & 0xfffu);
                            const int rr = (ent >> 12) & 1, cr = (ent >> 13) & 1;
                            const bool cj = (ent >> 14) & 1;
                            cx<T> v = rr ? (cr ? n11 : n10) : (cr ? n01 : n00);
                            const int row = rr ? q : p, col = cr ? q2 : p2;
                            const T drow = dc[2 * k1 + rr], dcol = dc[2 * k2 + cr];
                            JRot<T> Rn;
                            T na, nb;
                            if (cj) {  // element (col, row) = conj(v)
                                jacobi_rotation<T>(dcol, drow, conj(v), skip, col, row, Rn, na, nb);
                            } else {
                                jacobi_rotation<T>(drow, dcol, v, skip, row, col, Rn, na, nb);
                            }
                            rn[j] = Rn;
                            dn[2 * j] = na;
                            dn[2 * j + 1] = nb;
                        }
                    }
                } else {
                    const int t2 = task - nblk;
                    const int k = fdg.div(t2), g = t2 - k * ngrp;
                    const JRot<T> R = rc[k];
                    jacobi_rotate_rows(Ur, Ui, R.a() * ldu + 4 * g, R.b() * ldu + 4 * g, R);
                }
            }
            __syncthreads();
            cur ^= 1;
        }
    }
    // eigenvalues; eigenvectors interleaved (row stride m + 1) into the H
    // buffer, then swap
    for (int i = tid; i < m; i += nt) w.diag[i] = w.H[i * ld + i].re;
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) {
        const int i = fdm.div(e), j = e - i * m;  // row i, column j
        w.H[i * (m + 1) + j] = mk<T>(Ur[j * ldu + i], Ui[j * ldu + i]);
    }
    __syncthreads();
    cx<T> *const t = w.H;
    w.H = w.U;
    w.U = t;
    return status;
}

}  // namespace msp
