// Hermitian eigensolver for 64 < n <= MSP_MAX_DIM_LARGE (FP64; the fast
// path also in MIXED precision: the same solver in FP32 followed by
// double-word refinement, at the end of this file), one CTA per matrix,
// working matrices in global memory.  Replaces numpy.linalg.eigh in Hermitian.diag (muspinsim/spinop.py:
// 51-82) where the shared-memory Jacobi does not fit:
//   1. Householder tridiagonalisation of the lower triangle (H = Q T Q^H,
//      T real symmetric tridiagonal, Q = H_0 H_1 ... H_{n-2},
//      H_k = I - tau_k v_k v_k^H), LAPACK zhetd2 order;
//   2. implicit-shift QL on T with the rotations accumulated into Z
//      (T = Z diag(l) Z^T; the EISPACK tql2 iteration): robust for
//      degenerate and clustered levels, orthogonal to working precision;
//   3. back-transformation U = Q Z and ascending sort.
// Parallelisation: warp-per-row matrix-vector products and elementwise
// rank-2 updates (1), the QL rotations computed by one thread and applied to
// all rows of Z by all threads (2), one column of U per thread (3).
// Step 2's rotation sequence is a serial chain of FP64 operations, which on
// GB300 (FP64 at 1/64 of the FP32 rate, long FP64 latency) took two thirds
// of the solve: d and e live in shared memory, each rotation takes one
// Newton reciprocal square root instead of a library hypot and two
// divisions, and small CTAs (128 threads) run several to an SM so that one
// matrix's serial QL overlaps other matrices' parallel phases.
#include <math_constants.h>
#include <stdio.h>

#include "msp_dw.cuh"
#include "msp_internal.cuh"

#define MSP_DBL_EPS 2.220446049250313080847e-16  // 2^-52

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

// Shared memory: v, p (n complex each), qc, qs (n doubles each), red.
// (sized for T = double; the FP32 instance uses half of it)
__host__ __device__ inline size_t large_smem_bytes(int n, int threads) {
    return (size_t)n * 16 * 2 + (size_t)n * 8 * 4 + (size_t)(threads / 32) * 16 + 64;
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
// ascending eigenvalues into s.lam, eigenvectors (columns) into s.U.
// Returns MSP_ITEM_OK or MSP_ITEM_NOT_CONVERGED (QL iteration cap).
template <typename T>
__device__ int large_eigh(LargeScratchT<T> s, int n, char *smem) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int nw = nt >> 5;
    cx<T> *v = reinterpret_cast<cx<T> *>(smem);
    cx<T> *p = v + n;
    T *qc = reinterpret_cast<T *>(p + n);
    T *qs = qc + n;
    T *dsm = qs + n;  // diagonal and off-diagonal of the tridiagonal matrix
    T *esm = dsm + n;
    T *red = esm + n;
    cx<T> *A = s.A;

    // ---- 1. tridiagonalisation
    for (int k = 0; k + 1 < n; ++k) {
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
        // p = tau * A22 v  (warp per row)
        for (int i = warp; i < m; i += nw) {
            const cx<T> *row = A + (size_t)(k + 1 + i) * n + (k + 1);
            T pr = T(0), pi = T(0);
            for (int j = lane; j < m; j += 32) {
                const cx<T> a = row[j], x = v[j];
                pr += a.re * x.re - a.im * x.im;
                pi += a.re * x.im + a.im * x.re;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                pr += __shfl_xor_sync(0xffffffffu, pr, o);
                pi += __shfl_xor_sync(0xffffffffu, pi, o);
            }
            if (lane == 0) p[i] = cmul(tau, mk<T>(pr, pi));
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
        // A22 -= v w^H + w v^H
        for (int e = tid; e < m * m; e += nt) {
            const int i = e / m, j = e - i * m;  // FastDiv is exact only for m^3 < 2^20
            const cx<T> vi = v[i], wi = p[i], vj = v[j], wj = p[j];
            cx<T> &a = A[(size_t)(k + 1 + i) * n + (k + 1 + j)];
            const cx<T> t1 = cmul(vi, conj(wj)), t2 = cmul(wi, conj(vj));
            a = mk<T>(a.re - t1.re - t2.re, a.im - t1.im - t2.im);
        }
        // keep v for the back-transformation (column k below the subdiagonal)
        for (int i = 1 + tid; i < m; i += nt) A[(size_t)(k + 1 + i) * n + k] = v[i];
        __syncthreads();
    }
    if (tid == 0) {
        dsm[n - 1] = A[(size_t)(n - 1) * n + (n - 1)].re;
        esm[n - 1] = T(0);
    }
    // Z = I (column-major: Zt[col * n + row])
    for (size_t e = tid; e < (size_t)n * n; e += nt) {
        const int c = (int)(e / n), r = (int)(e - (size_t)c * n);
        s.Zt[e] = r == c ? T(1) : T(0);
    }
    __syncthreads();

    // ---- 2. QL with implicit shifts; e[i] couples d[i], d[i+1]
    int status = MSP_ITEM_OK;
    __shared__ int s_ctl[4];  // m, iteration flag, rotation count, status
    __shared__ T s_f, s_tst;
    if (tid == 0) {
        s_f = T(0);
        s_tst = T(0);
        s_ctl[3] = MSP_ITEM_OK;
    }
    __syncthreads();
    T *d = dsm, *e = esm;
    for (int l = 0; l < n; ++l) {
        for (int iter = 0;; ++iter) {
            if (tid == 0) {
                if (iter == 0) s_tst = fmax(s_tst, fabs(d[l]) + fabs(e[l]));
                int m = l;
                while (m < n - 1 && fabs(e[m]) > LargeEps<T>::eps * s_tst) ++m;
                s_ctl[0] = m;
                s_ctl[1] = 0;
                s_ctl[2] = 0;
                if (m > l && iter < 60) {
                    // one QL step on rows l..m; rotations (c, s) for i = m-1 .. l
                    T g = d[l];
                    T pp = (d[l + 1] - g) / (T(2) * e[l]);
                    T r = hypot(pp, T(1));
                    d[l] = e[l] / (pp + copysign(r, pp));
                    d[l + 1] = e[l] * (pp + copysign(r, pp));
                    const T dl1 = d[l + 1];
                    T h = g - d[l];
                    for (int i = l + 2; i < n; ++i) d[i] -= h;
                    s_f += h;
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
                        qc[cnt] = c;
                        qs[cnt] = sn;
                        ++cnt;
                    }
                    pp = -sn * s2 * c3 * el1 * e[l] / dl1;
                    e[l] = sn * pp;
                    d[l] = c * pp;
                    s_ctl[1] = 1;
                    s_ctl[2] = cnt;
                } else if (m > l) {
                    s_ctl[3] = MSP_ITEM_NOT_CONVERGED;
                }
            }
            __syncthreads();
            if (!s_ctl[1]) break;
            // apply the rotations to every row of Z: columns (i, i+1), i = m-1 .. l
            {
                const int m = s_ctl[0], cnt = s_ctl[2];
                T *__restrict__ Zt = s.Zt;
                for (int row = tid; row < n; row += nt) {
                    T hcarry = Zt[(size_t)m * n + row];  // Z[row][i+1] for i = m-1
                    int q = 0;
                    // eight entries loaded ahead of the rotation chain: within a
                    // sweep every entry is read before it is written
                    for (; q + 8 <= cnt; q += 8) {
                        T zi[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) zi[u] = Zt[(size_t)(m - 1 - q - u) * n + row];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int i = m - 1 - q - u;
                            const T c = qc[q + u], sn = qs[q + u];
                            Zt[(size_t)(i + 1) * n + row] = sn * zi[u] + c * hcarry;
                            hcarry = c * zi[u] - sn * hcarry;
                        }
                    }
                    for (; q < cnt; ++q) {
                        const int i = m - 1 - q;
                        const T zi = Zt[(size_t)i * n + row];
                        const T c = qc[q], sn = qs[q];
                        Zt[(size_t)(i + 1) * n + row] = sn * zi + c * hcarry;
                        hcarry = c * zi - sn * hcarry;
                    }
                    Zt[(size_t)l * n + row] = hcarry;
                }
            }
            __syncthreads();
        }
        if (tid == 0) {
            d[l] += s_f;
            e[l] = T(0);
        }
        __syncthreads();
    }
    status = s_ctl[3];

    // ---- 3. U = Q Z (complex), reflectors applied last to first; one column per thread
    for (size_t x = tid; x < (size_t)n * n; x += nt) {
        const int i = (int)(x / n), j = (int)(x - (size_t)i * n);
        s.U[x] = mk<T>(s.Zt[(size_t)j * n + i], T(0));
    }
    __syncthreads();
    for (int k = n - 2; k >= 0; --k) {
        const cx<T> tau = s.tau[k];
        if (tau.re == T(0) && tau.im == T(0)) continue;
        const int m = n - k - 1;
        for (int j = tid; j < n; j += nt) {
            // s_j = v^H U[k+1.., j]; U[k+1.., j] -= tau v s_j
            T sr = T(0), si = T(0);
            for (int i = 0; i < m; ++i) {
                const cx<T> vi = i == 0 ? mk<T>(T(1), T(0)) : A[(size_t)(k + 1 + i) * n + k];
                const cx<T> u = s.U[(size_t)(k + 1 + i) * n + j];
                sr += vi.re * u.re + vi.im * u.im;
                si += vi.re * u.im - vi.im * u.re;
            }
            const cx<T> ts = cmul(tau, mk<T>(sr, si));
            for (int i = 0; i < m; ++i) {
                const cx<T> vi = i == 0 ? mk<T>(T(1), T(0)) : A[(size_t)(k + 1 + i) * n + k];
                cx<T> &u = s.U[(size_t)(k + 1 + i) * n + j];
                const cx<T> t = cmul(vi, ts);
                u = mk<T>(u.re - t.re, u.im - t.im);
            }
        }
        __syncthreads();
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

__global__ void msp_eigh_large_kernel(const cx<double> *__restrict__ Hin, int n, int batch,
                                      double *__restrict__ evals, cx<double> *__restrict__ evecs,
                                      int *__restrict__ status, double *__restrict__ scratch) {
    extern __shared__ __align__(16) char smem[];
    LargeScratch s = large_carve(scratch + (size_t)blockIdx.x * large_scratch_doubles(n), n);
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        const cx<double> *Hb = Hin + (size_t)b * n * n;
        for (size_t x = threadIdx.x; x < (size_t)n * n; x += blockDim.x) s.A[x] = Hb[x];
        __syncthreads();
        const int st = large_eigh(s, n, smem);
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int r = large_rank(s.lam, n, j);
            evals[(size_t)b * n + r] = s.lam[j];
            cx<double> *V = evecs + (size_t)b * n * n;
            for (int i = 0; i < n; ++i) V[(size_t)i * n + r] = s.U[(size_t)i * n + j];
        }
        if (threadIdx.x == 0) status[b] = st;
        __syncthreads();
    }
}

// Pair record o of the fast path: coefficient cA (already scaled) and
// frequency w, as FP64 frequencies or, with pair_phase, double-word phase
// increments reduced modulo 2 pi.
__device__ __forceinline__ void large_store_pair(const SnapArgs &a, size_t o, double cA, double w) {
    if (a.pair_phase) {
        reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2((float)cA, 0.f);
        const double psi = reduce_2pi(w * a.dt);
        const double ph0 = a.t0 == 0.0 ? 0.0 : reduce_2pi(w * a.t0);
        const float psh = (float)psi, p0h = (float)ph0;
        a.pair_phase[o] =
            make_float4(psh, (float)(psi - (double)psh), p0h, (float)(ph0 - (double)p0h));
    } else {
        if (a.coef_f32)
            reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2((float)cA, 0.f);
        else
            reinterpret_cast<double2 *>(a.pair_coef)[o] = make_double2(cA, 0.0);
        a.pair_omega[o] = w;
    }
}

// Fast path per snapshot for n > 64 (muspinsim/hamiltonian.py:166-217), the
// large-n counterpart of msp_snap_fast_kernel: H = Hsys + b . Z, eigenpairs,
// M = U^H (sigma_p (x) 1_d) U, pair records and the constant part.
__global__ void msp_large_fast_kernel(SnapArgs a, double *__restrict__ scratch) {
    extern __shared__ __align__(16) char smem[];
    const int n = a.n, d = n / 2, P = n * (n - 1) / 2;
    LargeScratch s = large_carve(scratch + (size_t)blockIdx.x * large_scratch_doubles(n), n);
    const int tid = threadIdx.x, nt = blockDim.x;
    __shared__ double red[32];
    const size_t nn = (size_t)n * n;
    for (int sn = blockIdx.x; sn < a.num_snap; sn += gridDim.x) {
        const SnapSource src = snap_source(a, sn);
        const size_t g = (size_t)src.g;
        const double bx = a.field[3 * g], by = a.field[3 * g + 1], bz = a.field[3 * g + 2];
        for (size_t x = tid; x < nn; x += nt) {
            const cx<double> hs = src.Hsys[x], z0 = src.Z[x], z1 = src.Z[nn + x],
                             z2 = src.Z[2 * nn + x];
            s.A[x] = mk<double>(hs.re + bx * z0.re + by * z1.re + bz * z2.re,
                                hs.im + bx * z0.im + by * z1.im + bz * z2.im);
        }
        __syncthreads();
        const int st = large_eigh(s, n, smem);
        // W = (sigma_p (x) 1_d) U into A (free now)
        const double px = a.pol[3 * g], py = a.pol[3 * g + 1], pz = a.pol[3 * g + 2];
        for (size_t x = tid; x < nn; x += nt) {
            const int i = (int)(x / n);
            cx<double> val;
            if (i < d) {
                const cx<double> u0 = s.U[x], u1 = s.U[x + (size_t)d * n];
                val = mk<double>(pz * u0.re + px * u1.re + py * u1.im,
                                 pz * u0.im + px * u1.im - py * u1.re);
            } else {
                const cx<double> u0 = s.U[x - (size_t)d * n], u1 = s.U[x];
                val = mk<double>(px * u0.re - py * u0.im - pz * u1.re,
                                 px * u0.im + py * u0.re - pz * u1.im);
            }
            s.A[x] = val;
        }
        __syncthreads();
        const double scale = 0.5 * a.wscale[g] / (double)d;
        double diag = 0.0;
        // pairs j >= k: G = sum_i conj(U_ij) W_ik, A = |G|^2
        const size_t ntri = (size_t)n * (n + 1) / 2;
        for (size_t x = tid; x < ntri; x += nt) {
            int j = (int)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
            while ((size_t)(j + 1) * (j + 2) / 2 <= x) ++j;
            while ((size_t)j * (j + 1) / 2 > x) --j;
            const int k = (int)(x - (size_t)j * (j + 1) / 2);
            double gr = 0.0, gi = 0.0;
            for (int i = 0; i < n; ++i) {
                const cx<double> u = s.U[(size_t)i * n + j], w = s.A[(size_t)i * n + k];
                gr += u.re * w.re + u.im * w.im;
                gi += u.re * w.im - u.im * w.re;
            }
            const double Am = gr * gr + gi * gi;
            if (j == k)
                diag += Am;
            else
                large_store_pair(a, (size_t)sn * P + (size_t)j * (j - 1) / 2 + k, scale * Am,
                                 6.283185307179586476925 * (s.lam[j] - s.lam[k]));
        }
        diag = block_sum(diag, red);
        if (tid == 0) {
            a.snap_const[sn] = scale * 0.5 * diag;
            a.status[g] = st;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ mixed precision
//
// MIXED for n > 64: the solver above in FP32, then Ogita-Aishima refinement
// steps (T. Ogita and K. Aishima, Japan J. Indust. Appl. Math. 35 (2018)
// 1007, Algorithm 1, Hermitian form; the scheme of the n <= 64 MIXED
// kernels, with their exact 2 x 2 rotations for near-degenerate pairs):
//   R = I - X^H X,  S = X^H H X,  l_i = S_ii / (1 - R_ii),
//   E_ij = (S_ij + l_j R_ij) / (l_j - l_i),  E_ii = R_ii / 2,  X <- X + X E,
// eigenvalues l_i plus the second-order term.  H X, X^H (H X) and X^H X
// are accumulated in double-word FP32 from an anchor (the accumulator
// starts at a power of two K >= 4.01 |row| |column|, so every partial sum
// stays within a factor of two of K: s - fl(s + p) is exact and the
// rounding error of each product-sum goes into a compensation term), on
// packed f32x2 lanes; H itself is held as hi + lo.  Eigenvalues come out
// FP64-accurate, eigenvectors to FP32 rounding, as in the n <= 64 kernels.
// FP32 runs at ~60x GB300's FP64 rate and with ~15x shorter latency, which
// matters most in the serial QL rotation chain.

// Per-CTA scratch: H (double-word, 16 n^2 bytes), Y = H X (double-word,
// 16 n^2; the FP32 solver's A and Zt live there while it runs), X and X2
// (eigenvector matrices, 8 n^2 each), SR (S and R, then E; 8 n^2), the
// solver's eigenvalues and reflector scalars.
__host__ __device__ inline size_t lm_take(size_t &off, size_t bytes) {
    off = (off + 15) & ~size_t(15);
    const size_t o = off;
    off += bytes;
    return o;
}

struct LargeMixed {
    float4 *H, *Y;
    cx<float> *X, *X2, *SR;
    LargeScratchT<float> sol;
};

__host__ __device__ inline size_t lm_layout(int n, LargeMixed *s, char *base) {
    const size_t nn = (size_t)n * n;
    size_t off = 0;
    const size_t oH = lm_take(off, 16 * nn), oY = lm_take(off, 16 * nn);
    const size_t oX = lm_take(off, 8 * nn), oX2 = lm_take(off, 8 * nn);
    const size_t oSR = lm_take(off, 8 * nn), olam = lm_take(off, 4 * (size_t)n);
    const size_t otau = lm_take(off, 8 * (size_t)n);
    if (s) {
        s->H = reinterpret_cast<float4 *>(base + oH);
        s->Y = reinterpret_cast<float4 *>(base + oY);
        s->X = reinterpret_cast<cx<float> *>(base + oX);
        s->X2 = reinterpret_cast<cx<float> *>(base + oX2);
        s->SR = reinterpret_cast<cx<float> *>(base + oSR);
        s->sol.A = reinterpret_cast<cx<float> *>(base + oY);
        s->sol.Zt = reinterpret_cast<float *>(base + oY + 8 * nn);
        s->sol.U = s->X;
        s->sol.d = s->sol.e = nullptr;  // the solver keeps d and e in shared memory
        s->sol.lam = reinterpret_cast<float *>(base + olam);
        s->sol.tau = reinterpret_cast<cx<float> *>(base + otau);
    }
    return (off + 255) & ~size_t(255);
}

__host__ __device__ inline size_t lm_scratch_bytes(int n) { return lm_layout(n, nullptr, nullptr); }

// Refinement vectors in shared memory (the solver's shared memory is free
// once it returns): 48 n + 16 bytes <= large_smem_bytes(n, threads).
struct LmVec {
    double *lam, *sd, *rd;
    float *lamf, *corr, *ed, *rn, *cn, *yn;
    int *step;
};

__device__ __forceinline__ LmVec lm_vec(char *smem, int n) {
    LmVec v;
    v.lam = reinterpret_cast<double *>(smem);
    v.sd = v.lam + n;
    v.rd = v.sd + n;
    v.lamf = reinterpret_cast<float *>(v.rd + n);
    v.corr = v.lamf + n;
    v.ed = v.corr + n;
    v.rn = v.ed + n;
    v.cn = v.rn + n;
    v.yn = v.cn + n;
    v.step = reinterpret_cast<int *>(v.yn + n);
    return v;
}

// Anchored double-word accumulation of m * x into (s1 + i s2, c1 + i c2)
// for a real multiplier pair: s1 += mR x, s2 += mI x with x = (re, im) on
// the two lanes; the products' and sums' rounding errors go into c1, c2.
__device__ __forceinline__ void lm_acc(u64 &s1, u64 &c1, u64 &s2, u64 &c2, u64 mR, u64 mI,
                                       u64 x) {
    const u64 t1 = fma_f32x2(mR, x, s1);
    const u64 t2 = fma_f32x2(mI, x, s2);
    c1 = add2(c1, fma_f32x2(mR, x, sub2(s1, t1)));
    c2 = add2(c2, fma_f32x2(mI, x, sub2(s2, t2)));
    s1 = t1;
    s2 = t2;
}

__device__ __forceinline__ u64 lm_anchor(float bound) {
    const float K = pow2_above(4.01f * bound);
    return f32x2(K, K);
}

// One refinement step of the eigenvector columns X into X2 and of the
// eigenvalues v.lam.  Returns the largest first-order |E_ij| or rotation
// |s| (the size of the correction just applied).
__device__ float lm_refine(const LargeMixed &s, const cx<float> *__restrict__ X,
                           cx<float> *__restrict__ X2, const LmVec &v, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    float4 *__restrict__ Y = s.Y;
    cx<float> *__restrict__ SR = s.SR;
    for (int j = tid; j < n; j += nt) {
        float acc = 0.f;
        for (int k = 0; k < n; ++k) {
            const cx<float> x = X[(size_t)k * n + j];
            acc = fmaf(x.re, x.re, fmaf(x.im, x.im, acc));
        }
        v.cn[j] = sqrtf(acc);
    }
    if (tid == 0) *v.step = 0;
    __syncthreads();
    // Y = H X: a task is rows i0 .. i0 + 3 and column j (lanes take
    // consecutive j: H entries are broadcast, X rows coalesced)
    const int nb4 = (n + 3) >> 2;
    for (int task = tid; task < nb4 * n; task += nt) {
        const int ib = task / n, j = task - ib * n, i0 = 4 * ib;
        int row[4];
        u64 s1[4], c1[4], s2[4], c2[4], KK[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            row[q] = min(i0 + q, n - 1);
            KK[q] = lm_anchor(v.rn[row[q]] * v.cn[j]);
            s1[q] = s2[q] = KK[q];
            c1[q] = c2[q] = 0ull;
        }
#pragma unroll 1
        for (int k = 0; k < n; ++k) {
            const cx<float> x = X[(size_t)k * n + j];
            const u64 xh = f32x2(x.re, x.im);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 h = s.H[(size_t)row[q] * n + k];
                lm_acc(s1[q], c1[q], s2[q], c2[q], f32x2(h.x, h.x), f32x2(h.y, h.y), xh);
                c1[q] = fma_f32x2(f32x2(h.z, h.z), xh, c1[q]);  // lo part of H
                c2[q] = fma_f32x2(f32x2(h.w, h.w), xh, c2[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (i0 + q < n)
                Y[(size_t)(i0 + q) * n + j] =
                    dw_finish(sub2(s1[q], KK[q]), c1[q], sub2(s2[q], KK[q]), c2[q]);
    }
    __syncthreads();
    for (int j = tid; j < n; j += nt) {
        float acc = 0.f;
        for (int k = 0; k < n; ++k) {
            const float4 y = Y[(size_t)k * n + j];
            acc = fmaf(y.x, y.x, fmaf(y.y, y.y, acc));
        }
        v.yn[j] = sqrtf(acc);
    }
    __syncthreads();
    // S_ij = X_i^H Y_j and G_ij = X_i^H X_j for i <= j: a task is rows
    // i0, i0 + 1 and column j >= i0.  S_ij (i < j) goes to SR[i][j], R_ij =
    // -G_ij to SR[j][i]; S_ii and R_ii = 1 - G_ii to v.sd, v.rd.
    const int nb2 = (n + 1) >> 1;
    for (int task = tid; task < nb2 * n; task += nt) {
        const int ib = task / n, j = task - ib * n, i0 = 2 * ib;
        if (j < i0) continue;
        int col[2];
        u64 a1[2], ac1[2], a2[2], ac2[2], KS[2], g1[2], gc1[2], g2[2], gc2[2], KG[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            col[q] = min(i0 + q, n - 1);
            KS[q] = lm_anchor(v.cn[col[q]] * v.yn[j]);
            KG[q] = lm_anchor(v.cn[col[q]] * v.cn[j]);
            a1[q] = a2[q] = KS[q];
            g1[q] = g2[q] = KG[q];
            ac1[q] = ac2[q] = gc1[q] = gc2[q] = 0ull;
        }
#pragma unroll 1
        for (int k = 0; k < n; ++k) {
            const float4 y = Y[(size_t)k * n + j];
            const u64 yh = f32x2(y.x, y.y), yl = f32x2(y.z, y.w);
            const cx<float> xj = X[(size_t)k * n + j];
            const u64 xjh = f32x2(xj.re, xj.im);
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                // conj(a) y = a_re y + i (-a_im) y
                const cx<float> xa = X[(size_t)k * n + col[q]];
                const u64 mR = f32x2(xa.re, xa.re), mI = f32x2(-xa.im, -xa.im);
                lm_acc(a1[q], ac1[q], a2[q], ac2[q], mR, mI, yh);
                ac1[q] = fma_f32x2(mR, yl, ac1[q]);
                ac2[q] = fma_f32x2(mI, yl, ac2[q]);
                lm_acc(g1[q], gc1[q], g2[q], gc2[q], mR, mI, xjh);
            }
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int i = i0 + q;
            if (i >= n || i > j) continue;
            const float4 Sv = dw_finish(sub2(a1[q], KS[q]), ac1[q], sub2(a2[q], KS[q]), ac2[q]);
            const float4 Gv = dw_finish(sub2(g1[q], KG[q]), gc1[q], sub2(g2[q], KG[q]), gc2[q]);
            if (i == j) {
                v.sd[i] = (double)Sv.x + (double)Sv.z;
                v.rd[i] = (1.0 - (double)Gv.x) - (double)Gv.z;
            } else {
                SR[(size_t)i * n + j] = mk<float>(Sv.x + Sv.z, Sv.y + Sv.w);
                SR[(size_t)j * n + i] = mk<float>(-(Gv.x + Gv.z), -(Gv.y + Gv.w));
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        const double l = v.sd[i] / (1.0 - v.rd[i]);
        v.lam[i] = l;
        v.lamf[i] = (float)l;
        v.corr[i] = 0.f;
        v.ed[i] = 0.f;
    }
    __syncthreads();
    // E (both triangles) in place of S / R, second-order eigenvalue terms;
    // only the gap l_j - l_i needs FP64
    const int nup = n * (n - 1) / 2;
    float emax = 0.f;
    for (int e = tid; e < nup; e += nt) {
        int j = (int)((sqrtf(8.0f * (float)e + 1.0f) + 1.0f) * 0.5f);
        while (j * (j - 1) / 2 > e) --j;
        while ((j + 1) * j / 2 <= e) ++j;
        const int i = e - j * (j - 1) / 2;  // 0 <= i < j
        const cx<float> S = SR[(size_t)i * n + j], R = SR[(size_t)j * n + i];
        const float dl = (float)(v.lam[j] - v.lam[i]);
        const float lj_f = v.lamf[j], li_f = v.lamf[i];
        const float br = S.re + lj_f * R.re, bi = S.im + lj_f * R.im;  // S_ij + l_j R_ij
        const float ar = S.re + li_f * R.re, ai = S.im + li_f * R.im;  // S_ij + l_i R_ij
        cx<float> Eij, Eji;
        if (fmaxf(fmaxf(fabsf(br), fabsf(bi)), fmaxf(fabsf(ar), fabsf(ai))) < 1e-2f * fabsf(dl)) {
            const float inv = 1.0f / dl;
            Eij = mk<float>(br * inv, bi * inv);
            Eji = mk<float>(-ar * inv, ai * inv);
            atomicAdd(&v.corr[i], -(ar * ar + ai * ai) * inv);
            atomicAdd(&v.corr[j], (br * br + bi * bi) * inv);
            emax = fmaxf(emax, fmaxf(fmaxf(fabsf(Eij.re), fabsf(Eij.im)),
                                     fmaxf(fabsf(Eji.re), fabsf(Eji.im))));
        } else {
            // near-degenerate pair: exact rotation of the orthonormalised 2 x 2 block
            const float cr = 0.5f * (ar + br), ci = 0.5f * (ai + bi);
            const float mag = sqrtf(cr * cr + ci * ci);
            float sr = 0.f, si = 0.f;
            if (mag > 0.f) {
                const float zeta = dl / (2.0f * mag);
                const float t = fabsf(zeta) > 1e18f
                                    ? 0.5f / zeta
                                    : copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                const float qq = sqrtf(1.0f + t * t);  // 1 / k
                const float f = t / (qq * mag);
                sr = f * cr;
                si = f * ci;
                atomicAdd(&v.corr[i], -t * mag);
                atomicAdd(&v.corr[j], t * mag);
                const float km1 = -t * t / (qq * (1.0f + qq));  // k - 1 without cancellation
                atomicAdd(&v.ed[i], km1);
                atomicAdd(&v.ed[j], km1);
            }
            Eij = mk<float>(sr + 0.5f * R.re, si + 0.5f * R.im);
            Eji = mk<float>(-sr + 0.5f * R.re, si - 0.5f * R.im);
            emax = fmaxf(emax, fmaxf(fabsf(sr), fabsf(si)));
        }
        SR[(size_t)i * n + j] = Eij;
        SR[(size_t)j * n + i] = Eji;
    }
    atomicMax(v.step, __float_as_int(emax));  // non-negative: int order = float order
    __syncthreads();
    for (int j = tid; j < n; j += nt)
        SR[(size_t)j * n + j] = mk<float>((float)(0.5 * v.rd[j]) + v.ed[j], 0.f);
    __syncthreads();
    // X2 = X + X E: a task is rows k0 .. k0 + 3 and column j
    for (int task = tid; task < nb4 * (int)n; task += nt) {
        const int kb = task / n, j = task - kb * n, k0 = 4 * kb;
        int row[4];
        float ar[4], ai[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            row[q] = min(k0 + q, n - 1);
            const cx<float> x = X[(size_t)row[q] * n + j];
            ar[q] = x.re;
            ai[q] = x.im;
        }
#pragma unroll 1
        for (int i = 0; i < n; ++i) {
            const cx<float> E = SR[(size_t)i * n + j];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const cx<float> x = X[(size_t)row[q] * n + i];
                ar[q] = fmaf(x.re, E.re, fmaf(-x.im, E.im, ar[q]));
                ai[q] = fmaf(x.re, E.im, fmaf(x.im, E.re, ai[q]));
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (k0 + q < n) X2[(size_t)(k0 + q) * n + j] = mk<float>(ar[q], ai[q]);
    }
    for (int i = tid; i < n; i += nt) v.lam[i] += (double)v.corr[i];
    __syncthreads();
    const float step = __int_as_float(*v.step);
    __syncthreads();
    return step;
}

// The fast path for n > 64 in MIXED precision: H = Hsys + b . Z in FP64,
// split into hi + lo; the FP32 solver on hi; refinement steps until the
// correction drops below 2e-4 (at most four; one step leaves an error of
// order E^2); M = U^H (sigma_p (x) 1_d) U in FP32; pair records with FP64
// frequencies from the refined eigenvalues.
__global__ void __maxnreg__(96) msp_large_fast_mixed_kernel(SnapArgs a, char *scratch) {
    extern __shared__ __align__(16) char smem[];
    const int n = a.n, d = n / 2, P = n * (n - 1) / 2;
    LargeMixed s;
    lm_layout(n, &s, scratch + (size_t)blockIdx.x * lm_scratch_bytes(n));
    const LmVec v = lm_vec(smem, n);
    const int tid = threadIdx.x, nt = blockDim.x;
    __shared__ double red[32];
    const size_t nn = (size_t)n * n;
    for (int sn = blockIdx.x; sn < a.num_snap; sn += gridDim.x) {
        const SnapSource src = snap_source(a, sn);
        const size_t g = (size_t)src.g;
        const double bx = a.field[3 * g], by = a.field[3 * g + 1], bz = a.field[3 * g + 2];
        for (size_t x = tid; x < nn; x += nt) {
            const cx<double> hs = src.Hsys[x], z0 = src.Z[x], z1 = src.Z[nn + x],
                             z2 = src.Z[2 * nn + x];
            const double hr = hs.re + bx * z0.re + by * z1.re + bz * z2.re;
            const double hi = hs.im + bx * z0.im + by * z1.im + bz * z2.im;
            const float4 h = dw_split(make_double2(hr, hi));
            s.H[x] = h;
            s.sol.A[x] = mk<float>(h.x, h.y);
        }
        __syncthreads();
        const int st = large_eigh<float>(s.sol, n, smem);
        for (int i = tid; i < n; i += nt) {
            float acc = 0.f;
            for (int k = 0; k < n; ++k) {
                const float4 h = s.H[(size_t)i * n + k];
                acc = fmaf(h.x, h.x, fmaf(h.y, h.y, acc));
            }
            v.rn[i] = sqrtf(acc);
        }
        __syncthreads();
        cx<float> *X = s.X, *X2 = s.X2;
        for (int it = 0; it < 4; ++it) {
            const float step = lm_refine(s, X, X2, v, n);
            cx<float> *t = X;
            X = X2;
            X2 = t;
            if (step <= 2e-4f) break;
        }
        // W = (sigma_p (x) 1_d) X into X2
        const float px = (float)a.pol[3 * g], py = (float)a.pol[3 * g + 1],
                    pz = (float)a.pol[3 * g + 2];
        for (size_t x = tid; x < nn; x += nt) {
            const int i = (int)(x / n);
            cx<float> val;
            if (i < d) {
                const cx<float> u0 = X[x], u1 = X[x + (size_t)d * n];
                val = mk<float>(pz * u0.re + px * u1.re + py * u1.im,
                                pz * u0.im + px * u1.im - py * u1.re);
            } else {
                const cx<float> u0 = X[x - (size_t)d * n], u1 = X[x];
                val = mk<float>(px * u0.re - py * u0.im - pz * u1.re,
                                px * u0.im + py * u0.re - pz * u1.im);
            }
            X2[x] = val;
        }
        __syncthreads();
        const double scale = 0.5 * a.wscale[g] / (double)d;
        double diag = 0.0;
        const size_t ntri = (size_t)n * (n + 1) / 2;
        for (size_t x = tid; x < ntri; x += nt) {
            int j = (int)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
            while ((size_t)(j + 1) * (j + 2) / 2 <= x) ++j;
            while ((size_t)j * (j + 1) / 2 > x) --j;
            const int k = (int)(x - (size_t)j * (j + 1) / 2);
            float gr = 0.f, gi = 0.f;
            for (int i = 0; i < n; ++i) {
                const cx<float> u = X[(size_t)i * n + j], w = X2[(size_t)i * n + k];
                gr = fmaf(u.re, w.re, fmaf(u.im, w.im, gr));
                gi = fmaf(u.re, w.im, fmaf(-u.im, w.re, gi));
            }
            const double Am = (double)(gr * gr + gi * gi);
            if (j == k)
                diag += Am;
            else
                large_store_pair(a, (size_t)sn * P + (size_t)j * (j - 1) / 2 + k, scale * Am,
                                 6.283185307179586476925 * (v.lam[j] - v.lam[k]));
        }
        diag = block_sum(diag, red);
        if (tid == 0) {
            a.snap_const[sn] = scale * 0.5 * diag;
            a.status[g] = st;
        }
        __syncthreads();
    }
}

int large_threads(int n) { return 128; }

cudaError_t launch_eigh_large(const double *H, int n, int batch, double *evals, double *evecs,
                              int *status, double *scratch, int grid, cudaStream_t st) {
    const int threads = large_threads(n);
    const size_t smem = large_smem_bytes(n, threads);
    cudaError_t e = cudaFuncSetAttribute(msp_eigh_large_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    msp_eigh_large_kernel<<<grid, threads, smem, st>>>(
        reinterpret_cast<const cx<double> *>(H), n, batch, evals,
        reinterpret_cast<cx<double> *>(evecs), status, scratch);
    return cudaGetLastError();
}

cudaError_t launch_large_fast(const SnapArgs &a, double *scratch, int grid, cudaStream_t st,
                              int threads, int precision) {
    if (threads <= 0) threads = large_threads(a.n);
    const bool mixed = precision == MSP_PREC_MIXED;
    if ((threads & 31) || (mixed && threads > 256)) return cudaErrorInvalidValue;
    const size_t smem = large_smem_bytes(a.n, threads);
    const void *fn = mixed ? reinterpret_cast<const void *>(msp_large_fast_mixed_kernel)
                           : reinterpret_cast<const void *>(msp_large_fast_kernel);
    cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (mixed)
        msp_large_fast_mixed_kernel<<<grid, threads, smem, st>>>(a,
                                                                 reinterpret_cast<char *>(scratch));
    else
        msp_large_fast_kernel<<<grid, threads, smem, st>>>(a, scratch);
    return cudaGetLastError();
}

size_t large_scratch_bytes(int n, int grid, int precision) {
    const size_t per = precision == MSP_PREC_MIXED ? lm_scratch_bytes(n) : large_scratch_doubles(n) * 8;
    return per * (size_t)grid;
}

// Resident CTAs of the large-n kernels per SM with large_threads(n)
// threads, cut so that all CTAs' scratch stays within about 2 GB (large n
// keeps one CTA per SM).
int large_ctas_per_sm(int n, int precision) {
    const int threads = large_threads(n);
    int occ = 1;
    const bool mixed = precision == MSP_PREC_MIXED;
    const void *fn = mixed ? reinterpret_cast<const void *>(msp_large_fast_mixed_kernel)
                           : reinterpret_cast<const void *>(msp_large_fast_kernel);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads,
                                                      large_smem_bytes(n, threads)) !=
            cudaSuccess ||
        occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const size_t per = large_scratch_bytes(n, 1, precision), budget = (size_t)2 << 30;
    while (occ > 1 && (size_t)occ * sms * per > budget) --occ;
    return occ;
}

// A persistent grid of SMs x large_ctas_per_sm(n, precision) CTAs, at most
// one per matrix.
int large_grid(int batch, int n, int precision) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const int g = sms * large_ctas_per_sm(n, precision);
    return batch < g ? (batch > 0 ? batch : 1) : g;
}

}  // namespace msp
