// Dissipative (Lindblad) propagation: the path ExperimentRunner takes when
// the configuration has dissipation terms (muspinsim/experiment.py:272-341)
// and the Lindbladian class it builds (muspinsim/lindbladian.py:17-173).
//
// The reference diagonalises the n^2 x n^2 superoperator L with a dense
// non-Hermitian eig and writes rho(t) = V exp(2 pi Lambda t) V^-1 rho0 and
// the decaying integral as sum_k rho'_k O'_k / (1/tau - 2 pi lambda_k).
// Both are functions of L alone, computed here without an eigensolver:
//   * evolution: E = exp(2 pi L dt) by scaling and squaring of a degree-13
//     Taylor polynomial (Horner form, ||2 pi L dt / 2^s||_1 <= 1/2, truncation
//     below 1e-15), then rho(t_{k+1}) = E rho(t_k); a uniform grid needs
//     exp(2 pi L t0) and exp(2 pi L dt) only, a non-uniform grid one
//     exponential per interval;
//   * integral: O^T-weighted solution of (1/tau - 2 pi L) x = rho0 by
//     Gaussian elimination with partial pivoting (the matrix is regular:
//     Re lambda <= 0 for a Lindbladian and 1/tau > 0).
// Same values up to rounding, and no ill-conditioned eigenvector matrix
// when L is (nearly) defective.  All FP64: the plain drop-in path.
//
// One CTA per superoperator problem; its N x N matrices (N = n^2) live in a
// per-CTA slice of the caller's workspace (L2-resident for N <= 64).
#include <math_constants.h>
#include <string.h>

#include <algorithm>

#include "msp_dw.cuh"
#include "msp_internal.cuh"
#include "msp_rho.cuh"

namespace msp {
int record_error(int code, const char *msg);
}

using namespace msp;

typedef cx<double> zd;

#define MSP_LB_THREADS 256
#define MSP_LB_MAX_N2 1024  // superoperator dimension (n <= 32)

namespace {

// Per-CTA scratch, complex entries: L, A (LU / spare), X, T (N x N);
// v, w (N); o (num_ops x N); H, Mx, Ax (n x n); pivot row indices (N ints,
// stored in N complex slots).
struct LbWork {
    zd *L, *A, *X, *T, *v, *w, *o, *H, *M, *D;
    int *piv;
};

__host__ __device__ inline size_t lb_entries(int n, int num_ops) {
    const size_t N = (size_t)n * n;
    return 4 * N * N + (2 + (size_t)num_ops) * N + 3 * (size_t)n * n + N + 32;
}

__device__ inline LbWork lb_carve(zd *base, int n, int num_ops) {
    const size_t N = (size_t)n * n;
    LbWork w;
    w.L = base;
    w.A = w.L + N * N;
    w.X = w.A + N * N;
    w.T = w.X + N * N;
    w.v = w.T + N * N;
    w.w = w.v + N;
    w.o = w.w + N;
    w.H = w.o + (size_t)num_ops * N;
    w.M = w.H + (size_t)n * n;
    w.D = w.M + (size_t)n * n;
    w.piv = reinterpret_cast<int *>(w.D + (size_t)n * n);
    return w;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ double warp_sumd(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide maximum (every thread gets it); red: >= 32 doubles.
__device__ double lb_block_max(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double m = 0.0;
    for (int k = 0; k < nw; ++k) m = fmax(m, red[k]);
    __syncthreads();
    return m;
}

// Block-wide complex sum (every thread gets it); red: >= 64 doubles.
__device__ zd lb_block_csum(zd v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v.re = warp_sumd(v.re);
    v.im = warp_sumd(v.im);
    __syncthreads();
    if (lane == 0) {
        red[warp] = v.re;
        red[32 + warp] = v.im;
    }
    __syncthreads();
    zd s = mk<double>(0.0, 0.0);
    for (int k = 0; k < nw; ++k) {
        s.re += red[k];
        s.im += red[32 + k];
    }
    __syncthreads();
    return s;
}

// C = A B (N x N, row-major); C aliases neither.
__device__ void lb_gemm(zd *C, const zd *A, const zd *B, int N) {
    const int NN = N * N;
    for (int e = threadIdx.x; e < NN; e += blockDim.x) {
        const int i = e / N, j = e - (e / N) * N;
        const zd *a = A + (size_t)i * N;
        double cr = 0.0, ci = 0.0;
        for (int k = 0; k < N; ++k) {
            const zd x = a[k], y = B[(size_t)k * N + j];
            cr = fma(x.re, y.re, cr);
            cr = fma(-x.im, y.im, cr);
            ci = fma(x.re, y.im, ci);
            ci = fma(x.im, y.re, ci);
        }
        C[e] = mk<double>(cr, ci);
    }
    __syncthreads();
}

// y = E x, a warp per row.
__device__ void lb_matvec(zd *y, const zd *E, const zd *x, int N) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = warp; i < N; i += nw) {
        const zd *row = E + (size_t)i * N;
        double cr = 0.0, ci = 0.0;
        for (int k = lane; k < N; k += 32) {
            const zd a = row[k], b = x[k];
            cr = fma(a.re, b.re, cr);
            cr = fma(-a.im, b.im, cr);
            ci = fma(a.re, b.im, ci);
            ci = fma(a.im, b.re, ci);
        }
        cr = warp_sumd(cr);
        ci = warp_sumd(ci);
        if (lane == 0) y[i] = mk<double>(cr, ci);
    }
    __syncthreads();
}

// exp(f L) into the returned buffer (w.X or w.T).
__device__ zd *lb_expm(LbWork &w, int N, double f, double *red) {
    const int tid = threadIdx.x, nt = blockDim.x, NN = N * N;
    double cmax = 0.0;
    for (int j = tid; j < N; j += nt) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) {
            const zd x = w.L[(size_t)i * N + j];
            s += sqrt(x.re * x.re + x.im * x.im);
        }
        cmax = fmax(cmax, s);
    }
    double nrm = lb_block_max(cmax, red) * fabs(f);
    int sq = 0;
    while (nrm > 0.5 && sq < 64) {
        nrm *= 0.5;
        ++sq;
    }
    const double g = ldexp(f, -sq);
    for (int e = tid; e < NN; e += nt) w.X[e] = mk<double>((e / N) == (e % N) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int k = 13; k >= 1; --k) {  // X <- I + (g / k) L X
        lb_gemm(w.T, w.L, w.X, N);
        const double c = g / (double)k;
        for (int e = tid; e < NN; e += nt) {
            const zd t = w.T[e];
            w.X[e] = mk<double>(((e / N) == (e % N) ? 1.0 : 0.0) + c * t.re, c * t.im);
        }
        __syncthreads();
    }
    zd *P = w.X, *Q = w.T;
    for (int s = 0; s < sq; ++s) {
        lb_gemm(Q, P, P, N);
        zd *t = P;
        P = Q;
        Q = t;
    }
    return P;
}

// Expectations (or states) of one time sample.
__device__ void lb_emit(const LbWork &w, int N, int num_ops, const zd *v, double *red,
                        zd *out_c, double *out_r, double weight) {
    if (num_ops == 0) {  // states
        for (int e = threadIdx.x; e < N; e += blockDim.x) out_c[e] = v[e];
        return;
    }
    for (int op = 0; op < num_ops; ++op) {
        zd acc = mk<double>(0.0, 0.0);
        for (int e = threadIdx.x; e < N; e += blockDim.x) acc = cadd(acc, cmul(w.o[(size_t)op * N + e], v[e]));
        const zd s = lb_block_csum(acc, red);
        if (threadIdx.x == 0) {
            if (out_c) out_c[op] = s;
            if (out_r) out_r[op] = s.re * weight;
        }
    }
}

// Time series of rho(t) = exp(2 pi L t) rho0 (w.L, w.v hold L and rho0):
// outputs per time through lb_emit.
__device__ void lb_evolve(LbWork &w, int N, int num_ops, const double *times, int num_times,
                          int uniform, double t0, double dt, double *red, zd *out_c,
                          double *out_r, double weight) {
    zd *v = w.v, *y = w.w;
    zd *E = nullptr;
    double t_prev = 0.0;
    if (uniform && t0 != 0.0) {  // to the first sample
        E = lb_expm(w, N, 2.0 * CUDART_PI * t0, red);
        lb_matvec(y, E, v, N);
        zd *t = v;
        v = y;
        y = t;
        E = nullptr;
    }
    for (int k = 0; k < num_times; ++k) {
        if (uniform) {
            if (k > 0) {
                if (E == nullptr) E = lb_expm(w, N, 2.0 * CUDART_PI * dt, red);
                lb_matvec(y, E, v, N);
                zd *t = v;
                v = y;
                y = t;
            }
        } else {
            const double tk = times[k], step = tk - t_prev;
            if (step != 0.0) {
                E = lb_expm(w, N, 2.0 * CUDART_PI * step, red);
                lb_matvec(y, E, v, N);
                zd *t = v;
                v = y;
                y = t;
            }
            t_prev = tk;
        }
        lb_emit(w, N, num_ops, v, red,
                out_c ? out_c + (size_t)k * (num_ops ? num_ops : N) : nullptr,
                out_r ? out_r + (size_t)k * num_ops : nullptr, weight);
        __syncthreads();
    }
}

// x = (1/tau - 2 pi L)^-1 rho0 into w.v; w.A holds the factors.
__device__ void lb_solve(LbWork &w, int N, double tau, double *red) {
    const int tid = threadIdx.x, nt = blockDim.x, NN = N * N;
    const double inv_tau = 1.0 / tau, tp = 2.0 * CUDART_PI;
    for (int e = tid; e < NN; e += nt) {
        const zd l = w.L[e];
        w.A[e] = mk<double>(((e / N) == (e % N) ? inv_tau : 0.0) - tp * l.re, -tp * l.im);
    }
    __syncthreads();
    __shared__ int s_piv;
    zd *M = w.A, *b = w.v, *f = w.w;
    for (int k = 0; k < N; ++k) {
        // pivot: largest |M[i][k]|, i >= k (warp 0 scans)
        if (threadIdx.x < 32) {
            double best = -1.0;
            int bi = k;
            for (int i = k + (int)threadIdx.x; i < N; i += 32) {
                const zd x = M[(size_t)i * N + k];
                const double a = x.re * x.re + x.im * x.im;
                if (a > best) {
                    best = a;
                    bi = i;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) {
                    best = ob;
                    bi = oi;
                }
            }
            if (threadIdx.x == 0) s_piv = bi;
        }
        __syncthreads();
        const int p = s_piv;
        if (p != k) {
            for (int j = tid; j < N; j += nt) {
                const zd t = M[(size_t)k * N + j];
                M[(size_t)k * N + j] = M[(size_t)p * N + j];
                M[(size_t)p * N + j] = t;
            }
            if (tid == 0) {
                const zd t = b[k];
                b[k] = b[p];
                b[p] = t;
            }
        }
        __syncthreads();
        const zd piv = M[(size_t)k * N + k];
        const double dd = 1.0 / (piv.re * piv.re + piv.im * piv.im);
        const zd inv = mk<double>(piv.re * dd, -piv.im * dd);
        for (int i = k + 1 + tid; i < N; i += nt) f[i] = cmul(M[(size_t)i * N + k], inv);
        __syncthreads();
        const int rows = N - k - 1, cols = N - k - 1;
        for (int e = tid; e < rows * (cols + 1); e += nt) {
            const int i = k + 1 + e / (cols + 1), jj = e - (e / (cols + 1)) * (cols + 1);
            if (jj == cols) {
                const zd t = cmul(f[i], b[k]);
                b[i] = mk<double>(b[i].re - t.re, b[i].im - t.im);
            } else {
                const int j = k + 1 + jj;
                const zd t = cmul(f[i], M[(size_t)k * N + j]);
                M[(size_t)i * N + j] = mk<double>(M[(size_t)i * N + j].re - t.re,
                                                  M[(size_t)i * N + j].im - t.im);
            }
        }
        __syncthreads();
    }
    // back substitution, column oriented
    for (int k = N - 1; k >= 0; --k) {
        if (tid == 0) {
            const zd piv = M[(size_t)k * N + k];
            const double dd = 1.0 / (piv.re * piv.re + piv.im * piv.im);
            b[k] = cmul(b[k], mk<double>(piv.re * dd, -piv.im * dd));
        }
        __syncthreads();
        const zd xk = b[k];
        for (int i = tid; i < k; i += nt) {
            const zd t = cmul(M[(size_t)i * N + k], xk);
            b[i] = mk<double>(b[i].re - t.re, b[i].im - t.im);
        }
        __syncthreads();
    }
    (void)red;
}

// o[op] = vec(O_op^T): o[i n + j] = O[j][i]
__device__ void lb_observables(LbWork &w, const zd *ops, int num_ops, int n) {
    const int N = n * n;
    for (int e = threadIdx.x; e < num_ops * N; e += blockDim.x) {
        const int op = e / N, r = e - op * N, i = r / n, j = r - (r / n) * n;
        w.o[e] = ops[(size_t)op * N + (size_t)j * n + i];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(MSP_LB_THREADS) msp_superop_kernel(
    const zd *__restrict__ L, int n, const zd *__restrict__ rho0, const zd *__restrict__ ops,
    int num_ops, const double *__restrict__ times, int num_times, int uniform, double t0,
    double dt, int integral, double tau, zd *__restrict__ out, zd *__restrict__ scratch) {
    __shared__ double red[64];
    const int N = n * n;
    LbWork w = lb_carve(scratch, n, num_ops);
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) w.L[e] = L[e];
    for (int e = threadIdx.x; e < N; e += blockDim.x) w.v[e] = rho0[e];
    __syncthreads();
    lb_observables(w, ops, num_ops, n);
    if (integral) {
        lb_solve(w, N, tau, red);
        lb_emit(w, N, num_ops, w.v, red, out, nullptr, 1.0);
    } else {
        lb_evolve(w, N, num_ops, times, num_times, uniform, t0, dt, red, out, nullptr, 1.0);
    }
}

// ---------------------------------------------------------------- batched driver path

struct LbArgs {
    SnapArgs sa;             // n, spins, field, pol, temperature, gammas (rho0 factors)
    const zd *spin_ops;      // num_spins x 3 x n x n: S^a_i embedded
    int num_diss;
    int diss_spin[MSP_MAX_SPINS];
    double diss_rate[MSP_MAX_SPINS];
    const double *times;
    int num_times, uniform;
    double t0, dt;
    int integral;
    double *res;             // num_snap x T (real part x wscale)
    zd *scratch;
    size_t scratch_entries;  // per CTA
    int build_only;          // write L, rho0 and vec(O^T) per snapshot, do not propagate
    zd *Lout, *vout, *oout;  // num_snap x N^2, N, N
};

// Two axes orthogonal to z (muspinsim/utils.py:71-93), z a unit vector.
__device__ inline void lb_get_xy(const double *z, double *x, double *y) {
    if (z[0] == 0.0 && z[1] == 0.0) {
        x[0] = 1.0; x[1] = 0.0; x[2] = 0.0;
        y[0] = 0.0; y[1] = z[2]; y[2] = 0.0;
        return;
    }
    const double r = sqrt(z[0] * z[0] + z[1] * z[1]);
    x[0] = z[1] / r; x[1] = -z[0] / r; x[2] = 0.0;
    y[0] = z[1] * x[2] - z[2] * x[1];
    y[1] = z[2] * x[0] - z[0] * x[2];
    y[2] = z[0] * x[1] - z[1] * x[0];
}

__global__ void __launch_bounds__(MSP_LB_THREADS) msp_lindblad_kernel(LbArgs a) {
    __shared__ double red[64];
    __shared__ zd fac[MSP_MAX_SPINS * MSP_FACTOR_MAXD * MSP_FACTOR_MAXD];
    __shared__ double axes[6];
    const SnapArgs &sa = a.sa;
    const int n = sa.n, N = n * n, tid = threadIdx.x, nt = blockDim.x;
    LbWork w = lb_carve(a.scratch + (size_t)blockIdx.x * a.scratch_entries, n, 1);
    const size_t nn = (size_t)n * n;
    for (int s = blockIdx.x; s < sa.num_snap; s += gridDim.x) {
        const double *b = sa.field + 3 * (size_t)s, *p = sa.pol + 3 * (size_t)s;
        const double Bn = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        const double T = sa.temperature ? sa.temperature[s] : CUDART_INF;
        // H = Hsys + b . Z; rho0 factors; dissipator axes
        for (size_t e = tid; e < nn; e += nt) {
            const zd hs = sa.Hsys[e], z0 = sa.Z[e], z1 = sa.Z[nn + e], z2 = sa.Z[2 * nn + e];
            w.H[e] = mk<double>(hs.re + b[0] * z0.re + b[1] * z1.re + b[2] * z2.re,
                                hs.im + b[0] * z0.im + b[1] * z1.im + b[2] * z2.im);
        }
        build_rho_factors(sa, s, fac);
        if (tid == 0) {
            double x[3] = {1.0, 0.0, 0.0}, y[3] = {0.0, 1.0, 0.0};
            if (Bn != 0.0) {
                const double z[3] = {b[0] / Bn, b[1] / Bn, b[2] / Bn};
                lb_get_xy(z, x, y);
            }
            for (int k = 0; k < 3; ++k) {
                axes[k] = x[k];
                axes[3 + k] = y[k];
            }
        }
        __syncthreads();
        // rho0 = Kronecker product of the factors (spin 0 the slowest digit)
        for (int e = tid; e < N; e += nt) {
            int i = e / n, j = e - (e / n) * n, off = 0;
            zd r = mk<double>(1.0, 0.0);
            int ri = i, rj = j, stride = n;
            for (int q = 0; q < sa.num_spins; ++q) {
                const int dq = sa.dims[q];
                stride /= dq;
                const int di = ri / stride, dj = rj / stride;
                ri -= di * stride;
                rj -= dj * stride;
                r = cmul(r, fac[off + di * dq + dj]);
                off += dq * dq;
            }
            w.v[e] = r;
        }
        // observable: O = p . S_mu, o = vec(O^T)
        const zd *Smu = a.spin_ops + (size_t)sa.mu_index * 3 * nn;
        for (int e = tid; e < N; e += nt) {
            const int i = e / n, j = e - (e / n) * n;
            const size_t q = (size_t)j * n + i;
            w.o[e] = mk<double>(p[0] * Smu[q].re + p[1] * Smu[nn + q].re + p[2] * Smu[2 * nn + q].re,
                                p[0] * Smu[q].im + p[1] * Smu[nn + q].im + p[2] * Smu[2 * nn + q].im);
        }
        __syncthreads();
        // L: -i (H (x) 1 - 1 (x) H^T)
        for (int e = tid; e < N * N; e += nt) {
            const int r = e / N, c = e - (e / N) * N;
            const int i = r / n, j = r - (r / n) * n, k = c / n, l = c - (c / n) * n;
            zd v = mk<double>(0.0, 0.0);
            if (j == l) v = cadd(v, w.H[(size_t)i * n + k]);
            if (i == k) {
                const zd h = w.H[(size_t)l * n + j];
                v = mk<double>(v.re - h.re, v.im - h.im);
            }
            w.L[e] = mk<double>(v.im, -v.re);  // -i v
        }
        __syncthreads();
        // dissipators: S+ and S- about the field of each dissipative spin
        for (int d = 0; d < a.num_diss; ++d) {
            const int si = a.diss_spin[d];
            const double rate = a.diss_rate[d];
            double Zu = 0.0;
            if (T > 0.0) Zu = exp(-6.62607015e-34 * sa.gammas[si] * Bn * 1e6 / (1.380649e-23 * T));
            const zd *S = a.spin_ops + (size_t)si * 3 * nn;
            for (int pm = 0; pm < 2; ++pm) {
                const double g = pm == 0 ? rate * Zu / (CUDART_PI * (1.0 + Zu))
                                         : rate / (CUDART_PI * (1.0 + Zu));
                const double sg = pm == 0 ? 1.0 : -1.0;
                if (g == 0.0) continue;
                // D = op_x +/- i op_y
                for (size_t e = tid; e < nn; e += nt) {
                    double xr = 0, xi = 0, yr = 0, yi = 0;
                    for (int c = 0; c < 3; ++c) {
                        const zd sc = S[c * nn + e];
                        xr += axes[c] * sc.re;
                        xi += axes[c] * sc.im;
                        yr += axes[3 + c] * sc.re;
                        yi += axes[3 + c] * sc.im;
                    }
                    w.D[e] = mk<double>(xr - sg * yi, xi + sg * yr);
                }
                __syncthreads();
                // M = D^H D
                for (size_t e = tid; e < nn; e += nt) {
                    const int i = (int)(e / n), j = (int)(e - (e / n) * n);
                    double mr = 0, mi = 0;
                    for (int k = 0; k < n; ++k) {
                        const zd x = w.D[(size_t)k * n + i], y = w.D[(size_t)k * n + j];
                        mr += x.re * y.re + x.im * y.im;
                        mi += x.re * y.im - x.im * y.re;
                    }
                    w.M[e] = mk<double>(mr, mi);
                }
                __syncthreads();
                // L += g [D (x) conj(D) - 1/2 (M (x) 1 + 1 (x) M^T)]
                for (int e = tid; e < N * N; e += nt) {
                    const int r = e / N, c = e - (e / N) * N;
                    const int i = r / n, j = r - (r / n) * n, k = c / n, l = c - (c / n) * n;
                    const zd dik = w.D[(size_t)i * n + k], djl = w.D[(size_t)j * n + l];
                    zd v = cmul(dik, mk<double>(djl.re, -djl.im));
                    if (j == l) {
                        const zd m = w.M[(size_t)i * n + k];
                        v = mk<double>(v.re - 0.5 * m.re, v.im - 0.5 * m.im);
                    }
                    if (i == k) {
                        const zd m = w.M[(size_t)l * n + j];
                        v = mk<double>(v.re - 0.5 * m.re, v.im - 0.5 * m.im);
                    }
                    const zd lv = w.L[e];
                    w.L[e] = mk<double>(lv.re + g * v.re, lv.im + g * v.im);
                }
                __syncthreads();
            }
        }
        if (a.build_only) {
            for (int e = tid; e < N * N; e += nt) a.Lout[(size_t)s * N * N + e] = w.L[e];
            for (int e = tid; e < N; e += nt) {
                a.vout[(size_t)s * N + e] = w.v[e];
                a.oout[(size_t)s * N + e] = w.o[e];
            }
            if (tid == 0 && sa.status) sa.status[s] = MSP_ITEM_OK;
            __syncthreads();
            continue;
        }
        const double weight = sa.wscale[s];
        double *res = a.res + (size_t)s * a.num_times;
        if (a.integral) {
            lb_solve(w, N, sa.tau, red);
            lb_emit(w, N, 1, w.v, red, nullptr, res, weight / sa.tau);
        } else {
            lb_evolve(w, N, 1, a.times, a.num_times, a.uniform, a.t0, a.dt, red, nullptr, res,
                      weight);
        }
        if (tid == 0 && sa.status) sa.status[s] = MSP_ITEM_OK;
        __syncthreads();
    }
}

// ---------------------------------------------------------------- double-word propagation
// The mixed precision of the evolution mode on a uniform grid, N = n^2 <= 64:
// L, the propagators and rho live in shared memory as double-word FP32
// (hi + lo pairs, about 48 significant bits), and every product runs on the
// FP32 pipe with the anchored compensated accumulation of the Celio kernels:
// each sum starts at a power of two K >= 4 ||row|| ||column|| (Cauchy-
// Schwarz bounds every partial sum), so fma(u, x, s), the exact s - t and
// fma(u, x, s - t) give the sum and its rounding error.  GB300 runs FP64 at
// 1/64 of the FP32 rate with a 64-cycle dependent-FMA latency; the FP64
// kernel above stays the reference form.
constexpr int LBW_MAXN = 64;

constexpr int LBW_THREADS = 256;  // one CTA per SM (shared memory); 512 measured slower
constexpr int LBW_CHUNK = 256;    // time steps recorded before they are measured

struct LbDwArgs {
    const zd *L, *v, *o;  // per snapshot: N x N, N, N (from the build-only pass)
    int n, num_snap, num_times;
    double t0, dt;
    const double *wscale;
    double *res;          // num_snap x T
    float4 *hist;         // per CTA: LBW_CHUNK x N states awaiting measurement
};

// <O> of the recorded states hist[0 .. cnt) into res[k0 ..): two threads per
// state, FP64 sums of the double-word values.
__device__ void lbw_measure_chunk(const float4 *hist, const double2 *os, int N, int cnt,
                                  double weight, double *res) {
    const int tid = threadIdx.x, half = tid & 1, j = tid >> 1;
    const int h = (N + 1) >> 1, e0 = half * h, e1 = min(N, e0 + h);
    const int per = blockDim.x >> 1;  // states per pass; every thread runs every pass
    for (int jj = j; jj < (cnt + per - 1) / per * per; jj += per) {
        double acc = 0.0;
        if (jj < cnt)
            for (int e = e0; e < e1; ++e) {
                const double2 r = dw_join(hist[(size_t)jj * N + e]), o = os[e];
                acc = fma(o.x, r.x, fma(-o.y, r.y, acc));
            }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if (jj < cnt && half == 0) res[jj] = acc * weight;
    }
}

// (h, l) * (ch, cl) for one real component, renormalised
__device__ __forceinline__ void lbw_mul(float &h, float &l, float ch, float cl) {
    const float p = h * ch;
    float e = fmaf(h, ch, -p);
    e = fmaf(h, cl, fmaf(l, ch, e));
    h = p + e;
    l = e - (h - p);
}

// (h, l) + 1 exactly to double-word precision
__device__ __forceinline__ void lbw_add1(float &h, float &l) {
    const float s = 1.0f + h;
    const float bb = s - 1.0f;
    const float err = (1.0f - (s - bb)) + (h - bb);
    const float e = l + err;
    h = s + e;
    l = e - (h - s);
}

// Shared-memory position of matrix entry (i, k): odd rows are XOR-swizzled
// by 4 entries (sw = 4 when N is a multiple of 8, else 0), so that the two
// rows a quarter-warp reads in the matrix-vector product fall in disjoint
// bank groups; a permutation inside every row.
__device__ __forceinline__ int lbw_at(int i, int k, int N, int sw) {
    return i * N + (k ^ ((i & 1) * sw));
}

__device__ __forceinline__ void lbw_step(u64 &s1, u64 &c1, u64 &s2, u64 &c2, float4 a, float4 b) {
    const u64 R = f32x2(a.x, a.x), I = f32x2(a.y, a.y), lR = f32x2(a.z, a.z),
              lI = f32x2(a.w, a.w);
    const u64 xh = f32x2(b.x, b.y), xl = f32x2(b.z, b.w);
    const u64 t1 = fma_f32x2(R, xh, s1);
    const u64 t2 = fma_f32x2(I, xh, s2);
    c1 = add2(c1, fma_f32x2(R, xh, sub2(s1, t1)));
    c2 = add2(c2, fma_f32x2(I, xh, sub2(s2, t2)));
    s1 = t1;
    s2 = t2;
    c1 = fma_f32x2(R, xl, c1);
    c2 = fma_f32x2(I, xl, c2);
    c1 = fma_f32x2(lR, xh, c1);
    c2 = fma_f32x2(lI, xh, c2);
}

// C = A B (N x N, shared memory); rn, cn: scratch for row / column norms
__device__ void lbw_gemm(float4 *C, const float4 *A, const float4 *B, int N, float *rn, float *cn,
                         int sw) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int q = tid; q < 2 * N; q += nt) {
        float acc = 0.f;
        if (q < N) {
            for (int k = 0; k < N; ++k) {
                const float4 a = A[q * N + k];  // a whole row, in any order
                acc = fmaf(a.x, a.x, fmaf(a.y, a.y, acc));
            }
            rn[q] = sqrtf(acc);
        } else {
            const int j = q - N;
            for (int k = 0; k < N; ++k) {
                const float4 b = B[lbw_at(k, j, N, sw)];
                acc = fmaf(b.x, b.x, fmaf(b.y, b.y, acc));
            }
            cn[j] = sqrtf(acc);
        }
    }
    __syncthreads();
    // a task is row i and the columns jb, jb + W, jb + 2W, jb + 3W (W = N / 4
    // rounded up): consecutive threads read consecutive columns of B
    const int W = (N + 3) >> 2;
    for (int task = tid; task < N * W; task += nt) {
        const int i = task / W, jb = task - i * W;
        u64 s1[4], s2[4], c1[4], c2[4], KK[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = jb + q * W < N ? jb + q * W : N - 1;
            const float K = pow2_above(4.01f * rn[i] * cn[j]);
            KK[q] = f32x2(K, K);
            s1[q] = s2[q] = KK[q];
            c1[q] = c2[q] = 0ull;
        }
        for (int k = 0; k < N; ++k) {
            const float4 a = A[lbw_at(i, k, N, sw)];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = jb + q * W < N ? jb + q * W : N - 1;
                lbw_step(s1[q], c1[q], s2[q], c2[q], a, B[lbw_at(k, j, N, sw)]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (jb + q * W < N)
                C[lbw_at(i, jb + q * W, N, sw)] =
                    dw_finish(sub2(s1[q], KK[q]), c1[q], sub2(s2[q], KK[q]), c2[q]);
    }
    __syncthreads();
}

// y = E x with P lanes per output (P the largest power of two <= 32 with
// N P <= threads; lane p of an output takes k = p, p + P, ...); xb bounds
// ||x||_2.
__device__ void lbw_matvec(float4 *y, const float4 *E, const float4 *x, int N, const float *rE,
                           float xb, int sw) {
    const int tid = threadIdx.x, nt = blockDim.x;
    int P = 1;
    while (P < 32 && N * P * 2 <= nt) P *= 2;
    const int part = tid & (P - 1);
    for (int i0 = 0; i0 < N; i0 += nt / P) {
        const int i = i0 + tid / P;
        const bool active = i < N;
        const int ii = active ? i : 0;
        const float K = pow2_above(4.01f * rE[ii] * xb);
        const u64 KK = f32x2(K, K);
        u64 s1 = KK, s2 = KK, c1 = 0ull, c2 = 0ull;
        if (active) {
#pragma unroll 4
            for (int k = part; k < N; k += P)
                lbw_step(s1, c1, s2, c2, E[lbw_at(ii, k, N, sw)], x[k]);
        }
        s1 = sub2(s1, KK);
        s2 = sub2(s2, KK);
        for (int off = 1; off < P; off <<= 1) {
            const u64 o1 = __shfl_xor_sync(0xffffffffu, s1, off);
            const u64 o2 = __shfl_xor_sync(0xffffffffu, s2, off);
            const u64 d1 = __shfl_xor_sync(0xffffffffu, c1, off);
            const u64 d2 = __shfl_xor_sync(0xffffffffu, c2, off);
            two_sum2(s1, o1, c1);
            two_sum2(s2, o2, c2);
            c1 = add2(c1, d1);
            c2 = add2(c2, d2);
        }
        if (active && part == 0) y[i] = dw_finish(s1, c1, s2, c2);
    }
    __syncthreads();
}

// row 2-norms of a matrix (any order inside a row), slightly rounded up
__device__ void lbw_row_norms(const float4 *E, int N, float *r) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        float q = 0.f;
        for (int k = 0; k < N; ++k)
            q = fmaf(E[i * N + k].x, E[i * N + k].x, fmaf(E[i * N + k].y, E[i * N + k].y, q));
        r[i] = sqrtf(q) * 1.0001f;
    }
    __syncthreads();
}

// exp(f L) by scaling, Horner Taylor-13 and squaring; returns X or T
__device__ float4 *lbw_expm(const float4 *Ls, float4 *X, float4 *T, int N, double f,
                            double lnorm, float *rn, float *cn, int sw) {
    const int tid = threadIdx.x, nt = blockDim.x, NN = N * N;
    double nrm = lnorm * fabs(f);
    int sq = 0;
    while (nrm > 0.5 && sq < 64) {
        nrm *= 0.5;
        ++sq;
    }
    const double g = ldexp(f, -sq);
    // logical column of physical entry e: the swizzle is its own inverse
    for (int e = tid; e < NN; e += nt) {
        const int i = e / N, j = (e - i * N) ^ ((i & 1) * sw);
        X[e] = make_float4(i == j ? 1.f : 0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    for (int k = 13; k >= 1; --k) {  // X <- I + (g / k) L X
        lbw_gemm(T, Ls, X, N, rn, cn, sw);
        const double c = g / (double)k;
        const float ch = (float)c, cl = (float)(c - (double)ch);
        for (int e = tid; e < NN; e += nt) {
            const int i = e / N, j = (e - i * N) ^ ((i & 1) * sw);
            float4 t = T[e];
            lbw_mul(t.x, t.z, ch, cl);
            lbw_mul(t.y, t.w, ch, cl);
            if (i == j) lbw_add1(t.x, t.z);
            X[e] = t;
        }
        __syncthreads();
    }
    float4 *P = X, *Q = T;
    for (int q = 0; q < sq; ++q) {
        lbw_gemm(Q, P, P, N, rn, cn, sw);
        float4 *t = P;
        P = Q;
        Q = t;
    }
    return P;
}

__global__ void __launch_bounds__(LBW_THREADS) msp_lindblad_dw_kernel(LbDwArgs a) {
    extern __shared__ __align__(16) unsigned char lbw_smem[];
    __shared__ double red[64];
    const int n = a.n, N = n * n, NN = N * N, tid = threadIdx.x, nt = blockDim.x;
    float4 *Ls = reinterpret_cast<float4 *>(lbw_smem);
    float4 *X = Ls + NN, *T = X + NN, *x0 = T + NN, *x1 = x0 + N;
    double2 *os = reinterpret_cast<double2 *>(x1 + N);
    float *rn = reinterpret_cast<float *>(os + N), *cn = rn + N, *rE = cn + N;
    const int sw = (N & 7) == 0 ? 4 : 0;
    for (int s = blockIdx.x; s < a.num_snap; s += gridDim.x) {
        const zd *Lg = a.L + (size_t)s * NN;
        for (int e = tid; e < NN; e += nt) {
            const int i = e / N, k = e - i * N;
            Ls[lbw_at(i, k, N, sw)] = dw_split(make_double2(Lg[e].re, Lg[e].im));
        }
        for (int e = tid; e < N; e += nt) {
            const zd v = a.v[(size_t)s * N + e], o = a.o[(size_t)s * N + e];
            x0[e] = dw_split(make_double2(v.re, v.im));
            os[e] = make_double2(o.re, o.im);
        }
        // ||L||_1 (largest column sum, FP64) and ||rho0||_2
        double cmax = 0.0, v2 = 0.0;
        for (int j = tid; j < N; j += nt) {
            double c = 0.0;
            for (int i = 0; i < N; ++i) c += sqrt(Lg[(size_t)i * N + j].re * Lg[(size_t)i * N + j].re +
                                                  Lg[(size_t)i * N + j].im * Lg[(size_t)i * N + j].im);
            cmax = fmax(cmax, c);
            const zd v = a.v[(size_t)s * N + j];
            v2 += v.re * v.re + v.im * v.im;
        }
        const double lnorm = lb_block_max(cmax, red);
        const zd vs = lb_block_csum(mk<double>(v2, 0.0), red);
        // a density matrix keeps ||vec(rho)||_2 = sqrt(Tr rho^2) <= 1
        const float xb = (float)(fmax(1.0, sqrt(vs.re)) * 1.01);
        float4 *cur = x0;
        if (a.t0 != 0.0) {
            float4 *E0 = lbw_expm(Ls, X, T, N, 2.0 * CUDART_PI * a.t0, lnorm, rn, cn, sw);
            lbw_row_norms(E0, N, rE);
            lbw_matvec(x1, E0, cur, N, rE, xb, sw);
            cur = x1;
        }
        const double weight = a.wscale[s];
        double *res = a.res + (size_t)s * a.num_times;
        float4 *hist = a.hist + (size_t)blockIdx.x * LBW_CHUNK * N;
        // state 0
        for (int e = tid; e < N; e += nt) hist[e] = cur[e];
        __syncthreads();
        lbw_measure_chunk(hist, os, N, 1, weight, res);
        __syncthreads();
        if (a.num_times > 1) {
            float4 *E = lbw_expm(Ls, X, T, N, 2.0 * CUDART_PI * a.dt, lnorm, rn, cn, sw);
            lbw_row_norms(E, N, rE);
            float4 *nxt = cur == x0 ? x1 : x0;
            for (int k0 = 1; k0 < a.num_times; k0 += LBW_CHUNK) {
                const int cnt = min(LBW_CHUNK, a.num_times - k0);
                for (int q = 0; q < cnt; ++q) {
                    lbw_matvec(nxt, E, cur, N, rE, xb, sw);
                    float4 *t = cur;
                    cur = nxt;
                    nxt = t;
                    // cur is only read until the next matvec, which writes nxt
                    for (int e = tid; e < N; e += nt) hist[(size_t)q * N + e] = cur[e];
                }
                __syncthreads();
                lbw_measure_chunk(hist, os, N, cnt, weight, res + k0);
                __syncthreads();
            }
        }
    }
}

static size_t lbw_smem_bytes(int n) {
    const size_t N = (size_t)n * n;
    return 3 * N * N * 16 + 2 * N * 16 + N * 16 + 3 * N * 4 + 64;
}

// out[slot][t] = sum of the slot's snapshot results, in snapshot order
__global__ void msp_lindblad_reduce_kernel(const double *__restrict__ res,
                                           const int *__restrict__ slot_first, int num_slots,
                                           int T, double *__restrict__ out) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (e >= (size_t)num_slots * T) return;
    const int sl = (int)(e / T), t = (int)(e - (e / T) * T);
    double acc = 0.0;
    for (int s = slot_first[sl]; s < slot_first[sl + 1]; ++s) acc += res[(size_t)s * T + t];
    out[e] = acc;
}

static int lb_grid(int jobs) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    return jobs < sms ? (jobs > 0 ? jobs : 1) : sms;
}

static int lb_fail(int code, const char *m) { return record_error(code, m); }

static int lb_cuda(cudaError_t e) {
    return e == cudaSuccess ? MSP_OK : record_error(MSP_ERR_CUDA, cudaGetErrorString(e));
}

}  // namespace

extern "C" {

int msp_superop_workspace(int n, int num_ops, size_t *bytes) {
    if (n < 1 || (size_t)n * n > MSP_LB_MAX_N2 || num_ops < 0 || bytes == NULL)
        return lb_fail(MSP_ERR_ARG, "msp_superop_workspace: n outside 1..32 or num_ops < 0");
    *bytes = lb_entries(n, num_ops) * sizeof(zd);
    return MSP_OK;
}

static int superop_common(const double *L, int n, const double *rho0, const double *ops,
                          int num_ops, void *workspace, size_t workspace_bytes) {
    size_t need = 0;
    int rc = msp_superop_workspace(n, num_ops, &need);
    if (rc != MSP_OK) return rc;
    if (L == NULL || rho0 == NULL || (num_ops > 0 && ops == NULL))
        return lb_fail(MSP_ERR_ARG, "msp_superop: a required pointer is NULL");
    if (workspace == NULL || workspace_bytes < need || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return lb_fail(MSP_ERR_WORKSPACE, "msp_superop: workspace too small or not 256-byte aligned");
    return MSP_OK;
}

int msp_superop_evolve(const double *L, int n, const double *rho0, const double *ops, int num_ops,
                       const double *times, int num_times, int uniform, double t0, double dt,
                       double *out, void *workspace, size_t workspace_bytes, void *stream) {
    int rc = superop_common(L, n, rho0, ops, num_ops, workspace, workspace_bytes);
    if (rc != MSP_OK) return rc;
    if (num_times < 0 || out == NULL || (!uniform && num_times > 0 && times == NULL))
        return lb_fail(MSP_ERR_ARG, "msp_superop_evolve: times / out");
    if (num_times == 0) return MSP_OK;
    msp_superop_kernel<<<1, MSP_LB_THREADS, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const zd *>(L), n, reinterpret_cast<const zd *>(rho0),
        reinterpret_cast<const zd *>(ops), num_ops, times, num_times, uniform, t0, dt, 0, 1.0,
        reinterpret_cast<zd *>(out), reinterpret_cast<zd *>(workspace));
    return lb_cuda(cudaGetLastError());
}

int msp_superop_integrate(const double *L, int n, const double *rho0, const double *ops,
                          int num_ops, double tau, double *out, void *workspace,
                          size_t workspace_bytes, void *stream) {
    int rc = superop_common(L, n, rho0, ops, num_ops, workspace, workspace_bytes);
    if (rc != MSP_OK) return rc;
    if (!(tau > 0.0) || num_ops < 1 || out == NULL)
        return lb_fail(MSP_ERR_ARG, "msp_superop_integrate: tau must be > 0, one operator at least");
    msp_superop_kernel<<<1, MSP_LB_THREADS, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const zd *>(L), n, reinterpret_cast<const zd *>(rho0),
        reinterpret_cast<const zd *>(ops), num_ops, nullptr, 0, 1, 0.0, 0.0, 1, tau,
        reinterpret_cast<zd *>(out), reinterpret_cast<zd *>(workspace));
    return lb_cuda(cudaGetLastError());
}

static int check_lindblad(const msp_lindblad_args *a) {
    if (a == NULL) return lb_fail(MSP_ERR_ARG, "msp_lindblad: args is NULL");
    if (a->n < 2 || (size_t)a->n * a->n > MSP_LB_MAX_N2)
        return lb_fail(MSP_ERR_UNSUPPORTED, "msp_lindblad: n outside 2..32");
    if (a->num_spins < 1 || a->num_spins > MSP_MAX_SPINS)
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: num_spins");
    long long prod = 1;
    for (int s = 0; s < a->num_spins; ++s) {
        if (a->dims[s] < 1 || a->dims[s] > MSP_FACTOR_MAXD)
            return lb_fail(MSP_ERR_UNSUPPORTED, "msp_lindblad: a spin multiplicity outside 1..10");
        prod *= a->dims[s];
    }
    if (prod != a->n) return lb_fail(MSP_ERR_ARG, "msp_lindblad: product of dims != n");
    if (a->mu_index < 0 || a->mu_index >= a->num_spins || a->dims[a->mu_index] != 2)
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: mu_index");
    if (a->num_dissipative < 0 || a->num_dissipative > a->num_spins)
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: num_dissipative");
    for (int d = 0; d < a->num_dissipative; ++d)
        if (a->dissipative_spin[d] < 0 || a->dissipative_spin[d] >= a->num_spins)
            return lb_fail(MSP_ERR_ARG, "msp_lindblad: dissipative_spin out of range");
    if (a->num_snap < 0 || a->num_slots < 1) return lb_fail(MSP_ERR_ARG, "msp_lindblad: sizes");
    if (a->mode != MSP_MODE_EVOLVE && a->mode != MSP_MODE_INTEGRAL)
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: mode must be EVOLVE or INTEGRAL");
    if (a->mode == MSP_MODE_INTEGRAL && !(a->tau > 0.0))
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: tau must be > 0");
    if (a->mode == MSP_MODE_EVOLVE && (a->num_times < 1 || (!a->uniform && a->times == NULL)))
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: times");
    if (a->precision != MSP_PREC_FP64 && a->precision != MSP_PREC_MIXED)
        return lb_fail(MSP_ERR_ARG, "msp_lindblad: precision");
    return MSP_OK;
}

// Upper bound of the double-word kernel's grid (SMs x 2): sizes the
// per-CTA history buffers.
static int lbw_grid_max() {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    return 2 * sms;
}

struct LbLayout {
    size_t res, slot_first, item_first, scratch, Lb, vb, ob, hb, total;
    int T, grid;
    bool dw;  // double-word propagation (mixed, evolve, uniform grid, n^2 <= 64)
};

static LbLayout lb_layout(const msp_lindblad_args *a) {
    LbLayout L;
    L.T = a->mode == MSP_MODE_INTEGRAL ? 1 : a->num_times;
    L.grid = lb_grid(a->num_snap);
    L.dw = a->precision == MSP_PREC_MIXED && a->mode == MSP_MODE_EVOLVE && a->uniform &&
           a->n * a->n <= LBW_MAXN;
    size_t off = 0;
    auto take = [&](size_t b) {
        const size_t o = off;
        off += (b + 255) & ~(size_t)255;
        return o;
    };
    L.res = take((size_t)a->num_snap * L.T * 8);
    L.slot_first = take((size_t)(a->num_slots + 1) * 4);
    L.item_first = take((size_t)(a->num_slots + 1) * 4);
    L.scratch = take(lb_entries(a->n, 1) * sizeof(zd) * L.grid);
    L.Lb = L.vb = L.ob = L.hb = 0;
    if (L.dw) {
        const size_t N = (size_t)a->n * a->n;
        L.Lb = take((size_t)a->num_snap * N * N * sizeof(zd));
        L.vb = take((size_t)a->num_snap * N * sizeof(zd));
        L.ob = take((size_t)a->num_snap * N * sizeof(zd));
        L.hb = take((size_t)lbw_grid_max() * LBW_CHUNK * N * 16);
    }
    L.total = off;
    return L;
}

int msp_lindblad_workspace(const msp_lindblad_args *a, size_t *bytes) {
    int rc = check_lindblad(a);
    if (rc != MSP_OK) return rc;
    if (bytes == NULL) return lb_fail(MSP_ERR_ARG, "msp_lindblad_workspace: bytes is NULL");
    *bytes = lb_layout(a).total;
    return MSP_OK;
}

int msp_lindblad_run(const msp_lindblad_args *a) {
    int rc = check_lindblad(a);
    if (rc != MSP_OK) return rc;
    if (a->out == NULL) return lb_fail(MSP_ERR_ARG, "msp_lindblad_run: out is NULL");
    if (a->num_snap > 0 && (!a->Hsys || !a->Z || !a->spin_ops || !a->field || !a->pol ||
                            !a->wscale || !a->slot || !a->status))
        return lb_fail(MSP_ERR_ARG, "msp_lindblad_run: a snapshot pointer is NULL");
    const LbLayout Lo = lb_layout(a);
    if (a->workspace == NULL || a->workspace_bytes < Lo.total ||
        (reinterpret_cast<uintptr_t>(a->workspace) & 255))
        return lb_fail(MSP_ERR_WORKSPACE, "msp_lindblad_run: workspace too small or misaligned");
    cudaStream_t st = (cudaStream_t)a->stream;
    char *ws = reinterpret_cast<char *>(a->workspace);
    LbArgs la;
    memset(&la, 0, sizeof(la));
    SnapArgs &sa = la.sa;
    sa.n = a->n;
    sa.num_snap = a->num_snap;
    sa.Hsys = reinterpret_cast<const zd *>(a->Hsys);
    sa.Z = reinterpret_cast<const zd *>(a->Z);
    sa.field = a->field;
    sa.pol = a->pol;
    sa.wscale = a->wscale;
    sa.num_spins = a->num_spins;
    sa.mu_index = a->mu_index;
    for (int s = 0; s < a->num_spins; ++s) {
        sa.dims[s] = a->dims[s];
        sa.gammas[s] = a->gammas[s];
    }
    sa.temperature = a->temperature;
    sa.tau = a->tau;
    sa.status = a->status;
    la.spin_ops = reinterpret_cast<const zd *>(a->spin_ops);
    la.num_diss = a->num_dissipative;
    for (int d = 0; d < a->num_dissipative; ++d) {
        la.diss_spin[d] = a->dissipative_spin[d];
        la.diss_rate[d] = a->dissipative_rate[d];
    }
    la.times = a->times;
    la.num_times = Lo.T;
    la.uniform = a->mode == MSP_MODE_INTEGRAL ? 1 : a->uniform;
    la.t0 = a->t0;
    la.dt = a->dt;
    la.integral = a->mode == MSP_MODE_INTEGRAL;
    la.res = reinterpret_cast<double *>(ws + Lo.res);
    la.scratch = reinterpret_cast<zd *>(ws + Lo.scratch);
    la.scratch_entries = lb_entries(a->n, 1);
    if (a->num_snap > 0 && Lo.dw) {
        la.build_only = 1;
        la.Lout = reinterpret_cast<zd *>(ws + Lo.Lb);
        la.vout = reinterpret_cast<zd *>(ws + Lo.vb);
        la.oout = reinterpret_cast<zd *>(ws + Lo.ob);
        msp_lindblad_kernel<<<Lo.grid, MSP_LB_THREADS, 0, st>>>(la);
        rc = lb_cuda(cudaGetLastError());
        if (rc != MSP_OK) return rc;
        LbDwArgs da;
        da.L = la.Lout;
        da.v = la.vout;
        da.o = la.oout;
        da.n = a->n;
        da.num_snap = a->num_snap;
        da.num_times = Lo.T;
        da.t0 = a->t0;
        da.dt = a->dt;
        da.wscale = a->wscale;
        da.res = la.res;
        da.hist = reinterpret_cast<float4 *>(ws + Lo.hb);
        const size_t smem = lbw_smem_bytes(a->n);
        rc = lb_cuda(cudaFuncSetAttribute(msp_lindblad_dw_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (rc != MSP_OK) return rc;
        int occ = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_lindblad_dw_kernel,
                                                          LBW_THREADS, smem) != cudaSuccess ||
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
        const int grid = (int)std::min<long long>(
            a->num_snap, std::min<long long>((long long)sms * occ, lbw_grid_max()));
        msp_lindblad_dw_kernel<<<grid, LBW_THREADS, smem, st>>>(da);
        rc = lb_cuda(cudaGetLastError());
        if (rc != MSP_OK) return rc;
    } else if (a->num_snap > 0) {
        msp_lindblad_kernel<<<Lo.grid, MSP_LB_THREADS, 0, st>>>(la);
        rc = lb_cuda(cudaGetLastError());
        if (rc != MSP_OK) return rc;
    }
    rc = lb_cuda(launch_schedule(a->slot, a->num_snap, a->num_slots, 1, 1, 0,
                                 reinterpret_cast<int *>(ws + Lo.slot_first),
                                 reinterpret_cast<int *>(ws + Lo.item_first), a->status, st));
    if (rc != MSP_OK) return rc;
    const size_t total = (size_t)a->num_slots * Lo.T;
    msp_lindblad_reduce_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
        la.res, reinterpret_cast<const int *>(ws + Lo.slot_first), a->num_slots, Lo.T, a->out);
    return lb_cuda(cudaGetLastError());
}

}  // extern "C"
