// Cyclic two-sided Jacobi for one complex Hermitian matrix held in shared
// memory by one CTA.  Replaces the LAPACK zheevd call of Hermitian.diag
// (muspinsim/spinop.py:51-82).
//
// Schedule: round-robin ("circle") ordering over m = even padded dimension,
// m-1 steps per sweep, m/2 disjoint rotations per step.  Each step is two
// phases separated by __syncthreads():
//   1. one thread per pair computes the rotation G = [[c, s], [-conj(s), c]]
//      that zeroes H[p][q] (c real, s complex);
//   2. H <- G^dag H G on 2x2 blocks: only one block of each mirrored pair is
//      computed and its conjugate transpose written to the mirror, which
//      halves the work of a row pass followed by a column pass; the
//      diagonal blocks are set to diag(a', b') exactly.  U <- U G column
//      updates run in the same phase.
// A sweep starts with a block reduction of the off-diagonal and total
// Frobenius norms; the loop stops when off <= tol^2 * total, when a sweep
// no longer shrinks off (rounding floor, FP32), or at max_sweeps (status
// MSP_ITEM_NOT_CONVERGED).  Padding: when n is odd, index m-1 = n is a zero
// row/column that is never rotated.
#pragma once

#include "msp_common.cuh"

namespace msp {

template <typename T>
struct JacobiWork {
    cx<T> *H;   // m*m, row-major, leading dimension m
    cx<T> *U;   // m*m
    T *cs;      // m/2 rotation cosines
    cx<T> *sn;  // m/2 rotation sines (complex)
    T *da;      // m/2 new diagonal entries a'
    T *db;      // m/2 new diagonal entries b'
    int *pp;    // m/2 pair first index
    int *pq;    // m/2 pair second index
    T *red;     // 2 * warps scratch
    unsigned *tab;  // (m/2)(m/2+1)/2 block tasks: k1 | k2 << 16, k1 <= k2
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

// Runs the sweeps on w.H (already loaded, m x m Hermitian, row stride m + 1
// so that column walks hit distinct shared-memory banks) and sets w.U to
// the accumulated rotations.  All threads of the CTA must call it.  On
// return w.H holds the eigenvalues on its diagonal (unsorted) and w.U the
// eigenvectors in its columns.
template <typename T>
__device__ int jacobi_sweeps(const JacobiWork<T> &w, int m, int max_sweeps) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int half = m >> 1;
    const int nblk = half * (half + 1) / 2;
    const int ntask = nblk + half * m;
    const T tol = JacobiConst<T>::tol;
    const int ld = m + 1;  // padded row stride of H and U
    const FastDiv fdm(m);

    for (int e = tid; e < m * m; e += nt) {
        const int i = fdm.div(e), j = e - i * m;
        w.U[i * ld + j] = mk<T>(i == j ? T(1) : T(0), T(0));
    }
    // block task table, decoded once instead of at every step
    for (int task = tid; task < nblk; task += nt) {
        int k2 = (int)((sqrtf(8.0f * (float)task + 1.0f) - 1.0f) * 0.5f);
        while ((k2 + 1) * (k2 + 2) / 2 <= task) ++k2;
        while (k2 * (k2 + 1) / 2 > task) --k2;
        const int k1 = task - k2 * (k2 + 1) / 2;
        w.tab[task] = (unsigned)k1 | ((unsigned)k2 << 16);
    }

    int status = MSP_ITEM_NOT_CONVERGED;
    T prev_off = T(-1);
    for (int sweep = 0;; ++sweep) {
        T off = 0, fro = 0;
        for (int e = tid; e < m * m; e += nt) {
            const int i = fdm.div(e), j = e - i * m;
            const T v = cabs2(w.H[i * ld + j]);
            fro += v;
            if (i != j) off += v;
        }
        block_sum2(off, fro, w.red);  // contains __syncthreads
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
        const T skip = tol * sqrt(fro) / T(m);

        for (int r = 0; r < m - 1; ++r) {
            // phase 1: rotations of this step
            for (int k = tid; k < half; k += nt) {
                int a, b;
                if (k == 0) {
                    a = r;
                    b = m - 1;
                } else {
                    a = (r + k) % (m - 1);
                    b = (r - k + m - 1) % (m - 1);
                }
                const int p = a < b ? a : b, q = a < b ? b : a;
                const T app = w.H[p * ld + p].re, aqq = w.H[q * ld + q].re;
                const cx<T> apq = w.H[p * ld + q];
                const T mag = sqrt(cabs2(apq));
                T c = T(1), na = app, nb = aqq;
                cx<T> s = mk<T>(T(0), T(0));
                if (mag > skip) {
                    const T zeta = (aqq - app) / (T(2) * mag);
                    T t;
                    if (fabs(zeta) > JacobiConst<T>::big)
                        t = T(0.5) / zeta;
                    else
                        t = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
                    c = T(1) / sqrt(T(1) + t * t);
                    const T sr = t * c / mag;
                    s = mk<T>(sr * apq.re, sr * apq.im);
                    na = app - t * mag;
                    nb = aqq + t * mag;
                }
                w.pp[k] = p;
                w.pq[k] = q;
                w.cs[k] = c;
                w.sn[k] = s;
                w.da[k] = na;
                w.db[k] = nb;
            }
            __syncthreads();
            // phase 2: H <- G^dag H G (2x2 blocks), U <- U G
            for (int task = tid; task < ntask; task += nt) {
                if (task < nblk) {
                    const unsigned kk = w.tab[task];
                    const int k1 = (int)(kk & 0xffffu), k2 = (int)(kk >> 16);
                    const int p = w.pp[k1], q = w.pq[k1];
                    if (k1 == k2) {
                        w.H[p * ld + p] = mk<T>(w.da[k1], T(0));
                        w.H[q * ld + q] = mk<T>(w.db[k1], T(0));
                        w.H[p * ld + q] = mk<T>(T(0), T(0));
                        w.H[q * ld + p] = mk<T>(T(0), T(0));
                    } else {
                        const int p2 = w.pp[k2], q2 = w.pq[k2];
                        const T c1 = w.cs[k1], c2 = w.cs[k2];
                        const cx<T> s1 = w.sn[k1], s2 = w.sn[k2];
                        const cx<T> b00 = w.H[p * ld + p2], b01 = w.H[p * ld + q2];
                        const cx<T> b10 = w.H[q * ld + p2], b11 = w.H[q * ld + q2];
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
                        w.H[p * ld + p2] = n00;
                        w.H[p * ld + q2] = n01;
                        w.H[q * ld + p2] = n10;
                        w.H[q * ld + q2] = n11;
                        w.H[p2 * ld + p] = conj(n00);
                        w.H[q2 * ld + p] = conj(n01);
                        w.H[p2 * ld + q] = conj(n10);
                        w.H[q2 * ld + q] = conj(n11);
                    }
                } else {
                    const int t2 = task - nblk;
                    const int k = fdm.div(t2), row = t2 - k * m;
                    const int p = w.pp[k], q = w.pq[k];
                    const T c = w.cs[k];
                    const cx<T> s = w.sn[k];
                    const cx<T> x = w.U[row * ld + p], y = w.U[row * ld + q];
                    w.U[row * ld + p] = cadd(cscale(c, x), cscale(T(-1), cmulc(s, y)));
                    w.U[row * ld + q] = cadd(cmul(s, x), cscale(c, y));
                }
            }
            __syncthreads();
        }
    }
    return status;
}

}  // namespace msp
