// Hermitian eigensolver for 64 < n <= MSP_MAX_DIM_LARGE (FP64), one CTA per
// matrix, working matrices in global memory (one CTA per SM keeps them in
// L2).  Replaces numpy.linalg.eigh in Hermitian.diag (muspinsim/spinop.py:
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
            if (j == k) {
                diag += Am;
            } else {
                const size_t o = (size_t)sn * P + (size_t)j * (j - 1) / 2 + k;
                const double w = 6.283185307179586476925 * (s.lam[j] - s.lam[k]);
                if (a.pair_phase) {
                    reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2((float)(scale * Am), 0.f);
                    const double psi = reduce_2pi(w * a.dt);
                    const double ph0 = a.t0 == 0.0 ? 0.0 : reduce_2pi(w * a.t0);
                    const float psh = (float)psi, p0h = (float)ph0;
                    a.pair_phase[o] = make_float4(psh, (float)(psi - (double)psh), p0h,
                                                  (float)(ph0 - (double)p0h));
                } else {
                    if (a.coef_f32)
                        reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2((float)(scale * Am), 0.f);
                    else
                        reinterpret_cast<double2 *>(a.pair_coef)[o] = make_double2(scale * Am, 0.0);
                    a.pair_omega[o] = w;
                }
            }
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
                              int threads) {
    if (threads <= 0) threads = large_threads(a.n);
    const size_t smem = large_smem_bytes(a.n, threads);
    cudaError_t e = cudaFuncSetAttribute(msp_large_fast_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    msp_large_fast_kernel<<<grid, threads, smem, st>>>(a, scratch);
    return cudaGetLastError();
}

size_t large_scratch_bytes(int n, int grid) { return large_scratch_doubles(n) * 8 * (size_t)grid; }

// Resident CTAs of the large-n kernels per SM with large_threads(n)
// threads, cut so that all CTAs' scratch stays within about 2 GB (large n
// keeps one CTA per SM).
int large_ctas_per_sm(int n) {
    const int threads = large_threads(n);
    int occ = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_large_fast_kernel, threads,
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
    const size_t per = large_scratch_doubles(n) * 8, budget = (size_t)2 << 30;
    while (occ > 1 && (size_t)occ * sms * per > budget) --occ;
    return occ;
}

// A persistent grid of SMs x large_ctas_per_sm(n) CTAs, at most one per
// matrix.
int large_grid(int batch, int n) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    const int g = sms * large_ctas_per_sm(n);
    return batch < g ? (batch > 0 ? batch : 1) : g;
}

}  // namespace msp
