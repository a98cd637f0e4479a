// Householder + QL Hermitian eigensolver for 64 < n <= MSP_MAX_DIM_LARGE,
// shared by the large-n kernels (msp_large.cu: FP64 fast path, eigensolver
// API and the general path; msp_large_mixed.cu: the solver in FP32 followed
// by double-word refinement).  One CTA per matrix, working matrices in
// global memory.  Replaces numpy.linalg.eigh in Hermitian.diag
// (muspinsim/spinop.py:51-82) where the shared-memory Jacobi does not fit:
//   1. Householder tridiagonalisation of the lower triangle (H = Q T Q^H,
//      T real symmetric tridiagonal, Q = H_0 H_1 ... H_{n-2},
//      H_k = I - tau_k v_k v_k^H), LAPACK zhetd2 order;
//   2. implicit-shift QL on T with the rotations accumulated into Z
//      (T = Z diag(l) Z^T; the EISPACK tql2 iteration): robust for
//      degenerate and clustered levels, orthogonal to working precision;
//   3. back-transformation U = Q Z.
// Parallelisation: column-parallel Hermitian matrix-vector products and
// 2-D rank-2 updates (1), the QL rotations computed by one thread one
// batch ahead of the other warps, which apply them to the rows of Z (2),
// column-parallel reflector products (3).  Step 2's rotation sequence is a
// serial chain (FP64 at 1/64 of the FP32 rate and long FP64 latency on
// GB300): d and e live in shared memory, each rotation takes one Newton
// reciprocal square root instead of a library hypot and two divisions, and
// small CTAs (128 threads) run several to an SM so that one matrix's
// serial QL overlaps other matrices' parallel phases.
#pragma once

#include <math_constants.h>
#include <stdio.h>

#include "msp_internal.cuh"

#ifndef MSP_DBL_EPS
#define MSP_DBL_EPS 2.220446049250313080847e-16  // 2^-52
#endif

namespace msp {

int record_error(int code, const char *msg);

// Per-CTA global scratch (doubles): A (2n^2), U (2n^2), Zt (n^2), d, e,
// lam (n each), tau (2n).
__host__ __device__ inline size_t large_scratch_doubles(int n) {
    return (size_t)5 * n * n + 5 * (size_t)n + 64;
}

template <typename T>
struct LargeScratchT {
    cx<T> *A, *U;
    T *Zt, *d, *e, *lam;
    cx<T> *tau;
};
using LargeScratch = LargeScratchT<double>;

template <typename T>
struct LargeEps;
template <>
struct LargeEps<double> {
    static constexpr double eps = MSP_DBL_EPS;
};
template <>
struct LargeEps<float> {
    static constexpr float eps = 1.1920928955078125e-7f;  // 2^-23
};

__device__ __forceinline__ LargeScratch large_carve(double *base, int n) {
    LargeScratch s;
    s.A = reinterpret_cast<cx<double> *>(base);
    s.U = s.A + (size_t)n * n;
    s.Zt = reinterpret_cast<double *>(s.U + (size_t)n * n);
    s.d = s.Zt + (size_t)n * n;
    s.e = s.d + n;
    s.lam = s.e + n;
    s.tau = reinterpret_cast<cx<double> *>(s.lam + n);
    return s;
}

template <typename T>
__device__ __forceinline__ T block_sum(T v, T *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    T t = 0;
    for (int w = 0; w < nw; ++w) t += red[w];
    __syncthreads();
    return t;
}

// Row parts of the column-parallel products: RW = min(threads, 64) rows
// (or columns) at a time, the reduction index split into G = threads / RW
// parts whose partial sums meet in shared memory.
__host__ __device__ inline int large_parts(int threads) {
    const int rw = threads < 64 ? threads : 64;
    return threads / rw;
}

// Shared memory of the solver: v, p (n complex each), part (G x (n + 32)
// complex partial sums), y (32 complex), qc, qs (2 n reals each: two
// rotation batches), d, e (n reals each), red (one real per warp).
template <typename T>
struct LargeSm {
    cx<T> *v, *p, *part, *y;
    T *qc, *qs, *d, *e, *red;
};

template <typename T>
__host__ __device__ inline size_t large_sm_bytes(int n, int threads) {
    const size_t c = sizeof(cx<T>), r = sizeof(T);
    return c * (2 * (size_t)n + (size_t)large_parts(threads) * (n + 32) + 32) +
           r * (6 * (size_t)n + threads / 32) + 64;
}

template <typename T>
__device__ __forceinline__ LargeSm<T> large_sm(char *smem, int n, int threads) {
    LargeSm<T> m;
    m.v = reinterpret_cast<cx<T> *>(smem);
    m.p = m.v + n;
    m.part = m.p + n;
    m.y = m.part + (size_t)large_parts(threads) * (n + 32);
    m.qc = reinterpret_cast<T *>(m.y + 32);  // two batches of n
    m.qs = m.qc + 2 * n;
    m.d = m.qs + 2 * n;  // diagonal and off-diagonal of the tridiagonal matrix
    m.e = m.d + n;
    m.red = m.e + n;
    return m;
}

// (The FP64 kernels' dynamic shared memory.)
__host__ __device__ inline size_t large_smem_bytes(int n, int threads) {
    return large_sm_bytes<double>(n, threads);
}

// 1 / sqrt(x) for x > 0 in FP64 by Newton's method on f(y) = 1/y^2 - x,
// y <- y (3 - x y^2) / 2, from a single-precision seed: each step squares
// the relative error (2^-23 -> 2^-46 -> 2^-92), so the result is correct to
// the last bit or two, in a dozen dependent FP64 operations.  Callers keep
// x inside the seed's range (1e-36 .. 1e36).
template <typename T>
__device__ __forceinline__ T rsqrt_newton(T x);
template <>
__device__ __forceinline__ double rsqrt_newton<double>(double x) {
    double y = (double)rsqrtf((float)x);
    const double h = 0.5 * x;
    y = y * fma(-h * y, y, 1.5);
    y = y * fma(-h * y, y, 1.5);
    return y;
}
// FP32: the hardware approximation and one Newton step
template <>
__device__ __forceinline__ float rsqrt_newton<float>(float x) {
    const float y = rsqrtf(x);
    return y * fmaf(-0.5f * x * y, y, 1.5f);
}

// Eigenpairs of the Hermitian matrix already in s.A (full, row-major):
// eigenvalues into s.lam, eigenvectors (columns) into s.U.  Returns
// MSP_ITEM_OK or MSP_ITEM_NOT_CONVERGED (QL iteration cap).  BACK = false
// stops after the QL step (s.Zt holds Z, s.A the reflectors, s.tau their
// scalars) for a caller that back-transforms by itself; TRI = false starts
// at the QL step (the caller left d and e in this layout's shared memory,
// the reflectors in s.A and s.tau).
template <typename T, bool BACK = true, bool TRI = true>
__device__ int large_eigh(LargeScratchT<T> s, int n, char *smem) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int nw = nt >> 5;
    const int RW = nt < 64 ? nt : 64, G = nt / RW, pr = tid % RW, pg = tid / RW;
    const LargeSm<T> sm = large_sm<T>(smem, n, nt);
    cx<T> *v = sm.v, *p = sm.p, *part = sm.part;
    T *qc = sm.qc, *qs = sm.qs, *dsm = sm.d, *esm = sm.e, *red = sm.red;
    cx<T> *A = s.A;

    // ---- 1. tridiagonalisation
    for (int k = 0; TRI && k + 1 < n; ++k) {
        const int m = n - k - 1;  // length of x = A[k+1.., k]
        T xn2 = T(0);
        for (int i = 1 + tid; i < m; i += nt) xn2 += cabs2(A[(size_t)(k + 1 + i) * n + k]);
        xn2 = block_sum(xn2, red);
        const cx<T> alpha = A[(size_t)(k + 1) * n + k];
        cx<T> tau = mk<T>(T(0), T(0));
        T beta = alpha.re;
        const bool reflect = !(xn2 == T(0) && alpha.im == T(0));
        if (reflect) {
            beta = -copysign(sqrt(alpha.re * alpha.re + alpha.im * alpha.im + xn2), alpha.re);
            tau = mk<T>((beta - alpha.re) / beta, -alpha.im / beta);
            // v = x / (alpha - beta), v_0 = 1
            const cx<T> den = mk<T>(alpha.re - beta, alpha.im);
            const T dd = T(1) / cabs2(den);
            const cx<T> sc = mk<T>(den.re * dd, -den.im * dd);
            for (int i = tid; i < m; i += nt)
                v[i] = i == 0 ? mk<T>(T(1), T(0)) : cmul(A[(size_t)(k + 1 + i) * n + k], sc);
        }
        if (tid == 0) {
            dsm[k] = A[(size_t)k * n + k].re;
            esm[k] = beta;
            s.tau[k] = tau;
        }
        __syncthreads();
        if (!reflect) continue;
        // p = tau * A22 v.  A22 is Hermitian, so p_i = sum_j conj(A22_ji) v_j
        // reads rows of A22 coalesced over i: thread (pr, pg) takes rows
        // i = pr, pr + RW, ... and the pg-th of G parts of the j range, two
        // independent accumulators, partial sums into `part`.
        if (pg < G) {
            const int jb = (int)((long long)m * pg / G), je = (int)((long long)m * (pg + 1) / G);
            for (int i = pr; i < m; i += RW) {
                const cx<T> *col = A + (size_t)(k + 1) * n + (k + 1 + i);
                T r0 = T(0), i0 = T(0), r1 = T(0), i1 = T(0);
                int j = jb;
#pragma unroll 4
                for (; j + 1 < je; j += 2) {
                    const cx<T> a0 = col[(size_t)j * n], a1 = col[(size_t)(j + 1) * n];
                    const cx<T> x0 = v[j], x1 = v[j + 1];
                    r0 += a0.re * x0.re + a0.im * x0.im;
                    i0 += a0.re * x0.im - a0.im * x0.re;
                    r1 += a1.re * x1.re + a1.im * x1.im;
                    i1 += a1.re * x1.im - a1.im * x1.re;
                }
                if (j < je) {
                    const cx<T> a0 = col[(size_t)j * n], x0 = v[j];
                    r0 += a0.re * x0.re + a0.im * x0.im;
                    i0 += a0.re * x0.im - a0.im * x0.re;
                }
                part[(size_t)pg * (n + 32) + i] = mk<T>(r0 + r1, i0 + i1);
            }
        }
        __syncthreads();
        for (int i = tid; i < m; i += nt) {
            T sr = T(0), si = T(0);
            for (int g = 0; g < G; ++g) {
                sr += part[(size_t)g * (n + 32) + i].re;
                si += part[(size_t)g * (n + 32) + i].im;
            }
            p[i] = cmul(tau, mk<T>(sr, si));
        }
        __syncthreads();
        // alpha2 = -1/2 tau (p^H v); w = p + alpha2 v (in p)
        T hr = T(0), hi = T(0);
        for (int i = tid; i < m; i += nt) {
            const cx<T> c = cmulc(p[i], v[i]);  // conj(p_i) v_i
            hr += c.re;
            hi += c.im;
        }
        hr = block_sum(hr, red);
        hi = block_sum(hi, red);
        const cx<T> a2 = cscale(-T(0.5), cmul(tau, mk<T>(hr, hi)));
        for (int i = tid; i < m; i += nt) p[i] = cadd(p[i], cmul(a2, v[i]));
        __syncthreads();
        // A22 -= v w^H + w v^H: warps over rows, lanes over columns
        for (int i = warp; i < m; i += nw) {
            const cx<T> vi = v[i], wi = p[i];
            cx<T> *row = A + (size_t)(k + 1 + i) * n + (k + 1);
#pragma unroll 4
            for (int j = lane; j < m; j += 32) {
                const cx<T> vj = v[j], wj = p[j], a = row[j];
                const cx<T> t1 = cmul(vi, conj(wj)), t2 = cmul(wi, conj(vj));
                row[j] = mk<T>(a.re - t1.re - t2.re, a.im - t1.im - t2.im);
            }
        }
        // keep v for the back-transformation (column k below the subdiagonal)
        for (int i = 1 + tid; i < m; i += nt) A[(size_t)(k + 1 + i) * n + k] = v[i];
        __syncthreads();
    }
    if (TRI && tid == 0) {
        dsm[n - 1] = A[(size_t)(n - 1) * n + (n - 1)].re;
        esm[n - 1] = T(0);
    }
    // Z = I (column-major: Zt[col * n + row])
    for (size_t e = tid; e < (size_t)n * n; e += nt) {
        const int c = (int)(e / n), r = (int)(e - (size_t)c * n);
        s.Zt[e] = r == c ? T(1) : T(0);
    }
    __syncthreads();

    // ---- 2. QL with implicit shifts; e[i] couples d[i], d[i+1].
    // Thread 0 runs the serial part (convergence tests, shifts and the
    // rotation chain of one QL step: a "batch" of rotations for columns
    // l .. m of Z) one batch ahead of the other warps, which apply the
    // previous batch to the rows of Z meanwhile; qc / qs hold two batches.
    __shared__ int s_bat[2][3];  // per batch: m, l, rotation count (-1: done)
    __shared__ int s_status;
    T *d = dsm, *e = esm;
    // producer state (thread 0 only)
    int pl = 0, piter = 0, pstatus = MSP_ITEM_OK;
    T pf = T(0), ptst = T(0);
    // Next batch into slot `slot`: deflates converged eigenvalues, then one
    // QL step (or marks the end).
    auto produce = [&](int slot) {
        T *bc = qc + slot * n, *bs = qs + slot * n;
        for (;;) {
            if (pl >= n) {
                s_bat[slot][2] = -1;
                s_status = pstatus;
                return;
            }
            const int l = pl;
            if (piter == 0) ptst = fmax(ptst, fabs(d[l]) + fabs(e[l]));
            int m = l;
            while (m < n - 1 && fabs(e[m]) > LargeEps<T>::eps * ptst) ++m;
            if (m == l || piter >= 60) {
                if (m != l) pstatus = MSP_ITEM_NOT_CONVERGED;
                d[l] += pf;
                e[l] = T(0);
                ++pl;
                piter = 0;
                continue;
            }
            // one QL step on rows l..m; rotations (c, s) for i = m-1 .. l
            T g = d[l];
            T pp = (d[l + 1] - g) / (T(2) * e[l]);
            T r = hypot(pp, T(1));
            d[l] = e[l] / (pp + copysign(r, pp));
            d[l + 1] = e[l] * (pp + copysign(r, pp));
            const T dl1 = d[l + 1];
            T h = g - d[l];
            for (int i = l + 2; i < n; ++i) d[i] -= h;
            pf += h;
            pp = d[m];
            T c = T(1), c2 = T(1), c3 = T(1), sn = T(0), s2 = T(0);
            const T el1 = e[l + 1];
            int cnt = 0;
            for (int i = m - 1; i >= l; --i) {
                c3 = c2;
                c2 = c;
                s2 = sn;
                const T ei = e[i];
                g = c * ei;
                h = c * pp;
                const T x2 = fma(pp, pp, ei * ei);
                if (x2 > T(1e-36) && x2 < T(1e36)) {
                    const T y = rsqrt_newton<T>(x2);
                    r = x2 * y;
                    e[i + 1] = sn * r;
                    sn = ei * y;
                    c = pp * y;
                } else {  // outside the seed's range: the library route
                    r = hypot(pp, ei);
                    e[i + 1] = sn * r;
                    sn = ei / r;
                    c = pp / r;
                }
                pp = c * d[i] - sn * g;
                d[i + 1] = h + sn * (c * g + sn * d[i]);
                bc[cnt] = c;
                bs[cnt] = sn;
                ++cnt;
            }
            pp = -sn * s2 * c3 * el1 * e[l] / dl1;
            e[l] = sn * pp;
            d[l] = c * pp;
            ++piter;
            s_bat[slot][0] = m;
            s_bat[slot][1] = l;
            s_bat[slot][2] = cnt;
            return;
        }
    };
    // appliers: warps 1.. (all threads when the CTA is one warp)
    const int a0 = nt >= 64 ? 32 : 0, na = nt - a0;
    if (tid == 0) produce(0);
    __syncthreads();
    for (int b = 0;; ++b) {
        const int cur = b & 1;
        if (s_bat[cur][2] < 0) break;  // the same in every thread
        const int m = s_bat[cur][0], l = s_bat[cur][1], cnt = s_bat[cur][2];
        if (tid == 0) produce(cur ^ 1);
        if (tid >= a0) {
            // apply the batch to every row of Z: columns (i, i+1), i = m-1 .. l
            const T *bc = qc + cur * n, *bs = qs + cur * n;
            T *__restrict__ Zt = s.Zt;
            for (int row = tid - a0; row < n; row += na) {
                T hcarry = Zt[(size_t)m * n + row];  // Z[row][i+1] for i = m-1
                int q = 0;
                // eight entries loaded ahead of the rotation chain: within a
                // batch every entry is read before it is written
                for (; q + 8 <= cnt; q += 8) {
                    T zi[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) zi[u] = Zt[(size_t)(m - 1 - q - u) * n + row];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = m - 1 - q - u;
                        const T c = bc[q + u], sn = bs[q + u];
                        Zt[(size_t)(i + 1) * n + row] = sn * zi[u] + c * hcarry;
                        hcarry = c * zi[u] - sn * hcarry;
                    }
                }
                for (; q < cnt; ++q) {
                    const int i = m - 1 - q;
                    const T zi = Zt[(size_t)i * n + row];
                    const T c = bc[q], sn = bs[q];
                    Zt[(size_t)(i + 1) * n + row] = sn * zi + c * hcarry;
                    hcarry = c * zi - sn * hcarry;
                }
                Zt[(size_t)l * n + row] = hcarry;
            }
        }
        __syncthreads();
    }
    const int status = s_status;


    // ---- 3. U = Q Z (complex), reflectors applied last to first
    if (BACK) {
        for (size_t x = tid; x < (size_t)n * n; x += nt) {
            const int i = (int)(x / n), j = (int)(x - (size_t)i * n);
            s.U[x] = mk<T>(s.Zt[(size_t)j * n + i], T(0));
        }
        __syncthreads();
        for (int k = n - 2; k >= 0; --k) {
            const cx<T> tau = s.tau[k];
            if (tau.re == T(0) && tau.im == T(0)) continue;  // the same in every thread
            const int m = n - k - 1;
            for (int i = tid; i < m; i += nt)
                v[i] = i == 0 ? mk<T>(T(1), T(0)) : A[(size_t)(k + 1 + i) * n + k];
            __syncthreads();
            // s_j = v^H U[k+1.., j]: thread (pr, pg) takes columns j = pr, pr + RW,
            // ... and the pg-th of G parts of the rows
            if (pg < G) {
                const int ib = (int)((long long)m * pg / G), ie = (int)((long long)m * (pg + 1) / G);
                for (int j = pr; j < n; j += RW) {
                    const cx<T> *col = s.U + (size_t)(k + 1) * n + j;
                    T r0 = T(0), i0 = T(0), r1 = T(0), i1 = T(0);
                    int i = ib;
#pragma unroll 4
                    for (; i + 1 < ie; i += 2) {
                        const cx<T> u0 = col[(size_t)i * n], u1 = col[(size_t)(i + 1) * n];
                        const cx<T> v0 = v[i], v1 = v[i + 1];
                        r0 += v0.re * u0.re + v0.im * u0.im;
                        i0 += v0.re * u0.im - v0.im * u0.re;
                        r1 += v1.re * u1.re + v1.im * u1.im;
                        i1 += v1.re * u1.im - v1.im * u1.re;
                    }
                    if (i < ie) {
                        const cx<T> u0 = col[(size_t)i * n], v0 = v[i];
                        r0 += v0.re * u0.re + v0.im * u0.im;
                        i0 += v0.re * u0.im - v0.im * u0.re;
                    }
                    part[(size_t)pg * (n + 32) + j] = mk<T>(r0 + r1, i0 + i1);
                }
            }
            __syncthreads();
            for (int j = tid; j < n; j += nt) {
                T sr = T(0), si = T(0);
                for (int g = 0; g < G; ++g) {
                    sr += part[(size_t)g * (n + 32) + j].re;
                    si += part[(size_t)g * (n + 32) + j].im;
                }
                p[j] = cmul(tau, mk<T>(sr, si));  // tau s_j
            }
            __syncthreads();
            // U[k+1.., j] -= v tau s_j: warps over rows, lanes over columns
            for (int i = warp; i < m; i += nw) {
                const cx<T> vi = v[i];
                cx<T> *row = s.U + (size_t)(k + 1 + i) * n;
#pragma unroll 4
                for (int j = lane; j < n; j += 32) {
                    const cx<T> t = cmul(vi, p[j]), u = row[j];
                    row[j] = mk<T>(u.re - t.re, u.im - t.im);
                }
            }
            __syncthreads();
        }
    }
    for (int i = tid; i < n; i += nt) s.lam[i] = d[i];
    __syncthreads();
    return status;
}

// ascending order of s.lam (ties by index): rank[j]
__device__ __forceinline__ int large_rank(const double *lam, int n, int j) {
    const double lj = lam[j];
    int r = 0;
    for (int k = 0; k < n; ++k) {
        const double lk = lam[k];
        r += (lk < lj) || (lk == lj && k < j);
    }
    return r;
}

// Pair record o: coefficient (cA, cB) (already scaled; cB = 0 on the fast
// path) and frequency w, as FP64 frequencies or, with pair_phase,
// double-word phase increments reduced modulo 2 pi.
__device__ __forceinline__ void large_store_pair(const SnapArgs &a, size_t o, double cA, double w,
                                                 double cB = 0.0) {
    if (a.pair_phase) {
        reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2((float)cA, (float)cB);
        const double psi = reduce_2pi(w * a.dt);
        const double ph0 = a.t0 == 0.0 ? 0.0 : reduce_2pi(w * a.t0);
        const float psh = (float)psi, p0h = (float)ph0;
        a.pair_phase[o] =
            make_float4(psh, (float)(psi - (double)psh), p0h, (float)(ph0 - (double)p0h));
    } else {
        if (a.coef_f32)
            reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2((float)cA, (float)cB);
        else
            reinterpret_cast<double2 *>(a.pair_coef)[o] = make_double2(cA, cB);
        a.pair_omega[o] = w;
    }
}

}  // namespace msp
