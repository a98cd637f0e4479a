// Celio's method: Trotter evolution without diagonalisation
// (muspinsim/celio.py:54-486; the reference's native kernels are
// muspinsim/cpp/parallel.cpp:126-262 and muspinsim/cpp/celio.cpp:23-64).
//
// The Hamiltonian is split into contributions H_c that each act on one or
// two spins; one time step is (prod_c U_c)^k with U_c = exp(-2 pi i H_c dt/k)
// a small dense D x D matrix.  The state is a tensor whose digits are spin
// multiplicities (spin 0 most significant):
//   * PURE    -- averaged random initial states psi = mu_psi (x)
//                exp(2 pi i r) / sqrt(d); per time: measure
//                Re <psi|(sigma (x) 1_d)|psi>, then psi <- U_c psi for every
//                factor, k times (the reference's fast variant);
//   * DENSITY -- rho(t_i) = T^dag rho0 T with T = E^i, E = (prod_c F_c)^k
//                (the reference's density-matrix variant), applied as
//                rho <- U_c^dag rho U_c factor by factor on the 2L digits of
//                rho (row digits, then column digits), measured as
//                sum rho .* O^T.
// Applying a factor is a gather / D x D matvec / scatter over the D-element
// groups of the digits it acts on ("M (x) 1_d through an index map" in the
// reference); the groups are enumerated arithmetically from the digit
// strides instead of a stored index table.
//
// Shared-memory path: one CTA owns one state for the whole run -- the
// state, every factor matrix of its snapshot and the group offsets live in
// shared memory, and each factor application is one pass followed by one
// barrier, so HBM sees only the inputs and the measured series.  States too
// large for one CTA's shared memory run the global-memory path: one launch
// per factor application over every state, then a two-level deterministic
// reduction per measurement.  All FP64 (the reference's precision).
#include <math_constants.h>
#include <string.h>

#include <vector>

#include "msp_dw.cuh"
#include "msp_internal.cuh"

namespace msp {
int record_error(int code, const char *msg);
}

namespace {
using namespace msp;

constexpr int CE_MAX_DIGITS = 32;
constexpr int CE_MAX_FACTORS = 1024;
constexpr int CE_MAX_D = 128;
constexpr int CE_THREADS = 256;
constexpr int CE_DW_THREADS = 512;  // double-word kernel: 16 warps, <= 128 registers
constexpr int CE_CHUNK = 8192;  // elements per CTA of the global measurement

// One factor application: the digits it acts on, sorted by stride (A the
// slower one), and where its matrix and group offsets are.
struct CeFactor {
    long long sA, sB;  // strides; sB = 1, DB = 1 for a one-digit factor
    long long M;       // sA / (sB * DB): digits strictly between A and B
    long long mat;     // offset (complex entries) of the matrix in a snapshot's block
    int DA, DB, D;     // digit dims and matrix dimension
    int two;           // acts on two digits
    int off;           // first of its D offsets in the offsets table
    int pad;
};

struct CeArgs {
    const CeFactor *fac;
    const long long *offs;
    int nf, noffs;
    const double2 *mats;
    long long mats_len;
    int mats_per_snap;
    int mode;  // MSP_CELIO_PURE / MSP_CELIO_DENSITY
    long long V;   // elements of one state
    long long half;
    int S, A, k, T;
    const double2 *mu_psi;
    const double2 *sigma;
    const double *phases;
    unsigned long long seed;
    const double2 *rho0;
    const double2 *meas;
    int nops, meas_per_snap;
    double *series_pure;   // [S*A][T]
    double2 *series_rho;   // [S][T][nops]
    double2 *state;        // global path: [S*A][V] (double2, or float4 hi/lo pairs when dw)
    double *partial;       // global path: [S*A][chunks][2 nops]
    int chunks;
    void *dwmats;          // global double-word path: factor entries in lane patterns
    float *rnorms;         // global double-word path: [blocks][nf] row 2-norm bounds
};

// First element of group g of factor f (the element whose involved digits
// are all zero), from the mixed-radix decomposition of g over the other
// digits.
template <typename I>
__device__ __forceinline__ I ce_base(const CeFactor &f, I g) {
    if (!f.two) {
        const I sA = (I)f.sA;
        const I q = g / sA;
        return q * sA * (I)f.DA + (g - q * sA);
    }
    const I sB = (I)f.sB, M = (I)f.M;
    const I q = g / sB;
    const I l = g - q * sB;
    const I t = q / M;
    const I m = q - t * M;
    return t * (I)f.sA * (I)f.DA + m * sB * (I)f.DB + l;
}

// SplitMix64 (Steele, Lea and Flood, OOPSLA 2014): uniform double in [0, 1)
// from a 64-bit counter, for random initial states when the caller passes
// no phases.
__device__ __forceinline__ double ce_uniform(unsigned long long seed, unsigned long long ctr) {
    unsigned long long z = seed + (ctr + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

__device__ __forceinline__ double2 ce_init_pure(const CeArgs &a, int st, long long x) {
    const int s = st / a.A;
    const int hi = x >= a.half;
    const long long kk = hi ? x - a.half : x;
    const double r = a.phases ? a.phases[(size_t)st * a.half + kk]
                              : ce_uniform(a.seed, (unsigned long long)st * a.half + kk);
    double sn, cs;
    sincospi(2.0 * r, &sn, &cs);
    const double2 m = a.mu_psi[2 * s + hi];
    const double inv = 1.0 / sqrt((double)a.half);
    return make_double2((m.x * cs - m.y * sn) * inv, (m.x * sn + m.y * cs) * inv);
}

// y = U x for one group, x held in registers (D known at compile time).
template <int D, typename I>
__device__ __forceinline__ void ce_group(double2 *__restrict__ V, const double2 *__restrict__ U,
                                         const CeFactor &f, const I *__restrict__ off, I g) {
    const I base = ce_base<I>(f, g);
    double2 x[D];
#pragma unroll
    for (int j = 0; j < D; ++j) x[j] = V[base + off[j]];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        double re = 0.0, im = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            const double2 u = U[i * D + j];
            re = fma(u.x, x[j].x, re);
            re = fma(-u.y, x[j].y, re);
            im = fma(u.x, x[j].y, im);
            im = fma(u.y, x[j].x, im);
        }
        V[base + off[i]] = make_double2(re, im);
    }
}

// y = U x for one group by one warp (any D <= 32 R): lane l holds x_j for
// j = l, l + 32, ...; x_j is broadcast by shuffle.
template <int R, typename I>
__device__ __forceinline__ void ce_group_warp(double2 *__restrict__ V,
                                              const double2 *__restrict__ U, const CeFactor &f,
                                              const I *__restrict__ off, I g, int lane) {
    const int D = f.D;
    const I base = ce_base<I>(f, g);
    double2 x[R], y[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = lane + 32 * r;
        x[r] = j < D ? V[base + off[j]] : make_double2(0.0, 0.0);
        y[r] = make_double2(0.0, 0.0);
    }
    __syncwarp();
#pragma unroll
    for (int r2 = 0; r2 < R; ++r2) {
        for (int jj = 0; jj < 32; ++jj) {
            const int j = 32 * r2 + jj;
            if (j >= D) break;
            const double xr = __shfl_sync(0xffffffffu, x[r2].x, jj);
            const double xi = __shfl_sync(0xffffffffu, x[r2].y, jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int i = lane + 32 * r;
                if (i < D) {
                    const double2 u = U[i * D + j];
                    y[r].x = fma(u.x, xr, fma(-u.y, xi, y[r].x));
                    y[r].y = fma(u.x, xi, fma(u.y, xr, y[r].y));
                }
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int i = lane + 32 * r;
        if (i < D) V[base + off[i]] = y[r];
    }
}

// Every group of one factor, distributed over `workers` threads (or warps).
template <typename I>
__device__ void ce_apply(double2 *__restrict__ V, const double2 *__restrict__ U,
                         const CeFactor &f, const I *__restrict__ off, I G, I first, I step) {
    switch (f.D) {
#define CE_CASE(DD)                                                       \
    case DD:                                                              \
        for (I g = first; g < G; g += step) ce_group<DD, I>(V, U, f, off, g); \
        return;
        CE_CASE(1)
        CE_CASE(2)
        CE_CASE(3)
        CE_CASE(4)
        CE_CASE(5)
        CE_CASE(6)
        CE_CASE(8)
        CE_CASE(9)
        CE_CASE(10)
        CE_CASE(12)
        CE_CASE(16)
#undef CE_CASE
        default:
            break;
    }
}

// The warp form for the other D; first / step count warps.
template <typename I>
__device__ void ce_apply_warp(double2 *__restrict__ V, const double2 *__restrict__ U,
                              const CeFactor &f, const I *__restrict__ off, I G, I first, I step,
                              int lane) {
    const int R = (f.D + 31) >> 5;
    for (I g = first; g < G; g += step) {
        if (R == 1)
            ce_group_warp<1, I>(V, U, f, off, g, lane);
        else if (R == 2)
            ce_group_warp<2, I>(V, U, f, off, g, lane);
        else if (R == 3)
            ce_group_warp<3, I>(V, U, f, off, g, lane);
        else
            ce_group_warp<4, I>(V, U, f, off, g, lane);
    }
}

__host__ __device__ __forceinline__ bool ce_thread_form(int D) {
    return D <= 6 || D == 8 || D == 9 || D == 10 || D == 12 || D == 16;
}

// Re <psi|(sigma (x) 1)|psi> over elements [lo, hi) of the half-blocks,
// with the upper triangle of sigma used twice, as the reference does.
__device__ __forceinline__ double ce_measure_pure(const double2 *__restrict__ V, long long half,
                                                  const double2 *sig, long long lo, long long hi,
                                                  long long step) {
    const double2 m00 = sig[0], m01 = sig[1], m11 = sig[3];
    double acc = 0.0;
    for (long long kk = lo; kk < hi; kk += step) {
        const double2 u = V[kk], d = V[half + kk];
        const double tr = m00.x * u.x - m00.y * u.y + 2.0 * (m01.x * d.x - m01.y * d.y);
        const double ti = m00.x * u.y + m00.y * u.x + 2.0 * (m01.x * d.y + m01.y * d.x);
        acc += u.x * tr + u.y * ti;
        const double sr = m11.x * d.x - m11.y * d.y, si = m11.x * d.y + m11.y * d.x;
        acc += d.x * sr + d.y * si;
    }
    return acc;
}

// ----------------------------------------------------------- shared-memory path
__global__ void __launch_bounds__(CE_THREADS) msp_celio_smem_kernel(CeArgs a) {
    extern __shared__ __align__(16) unsigned char ce_smem[];
    double2 *V = reinterpret_cast<double2 *>(ce_smem);
    double2 *Um = V + a.V;
    CeFactor *fac = reinterpret_cast<CeFactor *>(Um + a.mats_len);
    int *offs = reinterpret_cast<int *>(fac + a.nf);
    double *red = reinterpret_cast<double *>(offs + ((a.noffs + 3) & ~3));

    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int i = tid; i < a.nf; i += nt) fac[i] = a.fac[i];
    for (int i = tid; i < a.noffs; i += nt) offs[i] = (int)a.offs[i];

    const int V32 = (int)a.V;
    int loaded = -1;
    for (int st = blockIdx.x; st < a.S * a.A; st += gridDim.x) {
        const int s = st / a.A;
        const int blk = a.mats_per_snap ? s : 0;
        if (blk != loaded) {
            const double2 *src = a.mats + (size_t)blk * a.mats_len;
            for (long long i = tid; i < a.mats_len; i += nt) Um[i] = src[i];
            loaded = blk;
        }
        if (a.mode == MSP_CELIO_PURE) {
            for (int x = tid; x < V32; x += nt) V[x] = ce_init_pure(a, st, x);
        } else {
            const double2 *r0 = a.rho0 + (size_t)s * a.V;
            for (int x = tid; x < V32; x += nt) V[x] = r0[x];
        }
        __syncthreads();
        for (int t = 0; t < a.T; ++t) {
            if (a.mode == MSP_CELIO_PURE) {
                double m = ce_measure_pure(V, a.half, a.sigma + 4 * s, tid, a.half, nt), z = 0.0;
                block_sum2(m, z, red);
                if (tid == 0) a.series_pure[(size_t)st * a.T + t] = m;
            } else {
                const double2 *W0 = a.meas + (size_t)(a.meas_per_snap ? s : 0) * a.nops * a.V;
                for (int j = 0; j < a.nops; ++j) {
                    const double2 *W = W0 + (size_t)j * a.V;
                    double re = 0.0, im = 0.0;
                    for (int x = tid; x < V32; x += nt) {
                        const double2 r = V[x], w = W[x];
                        re += r.x * w.x - r.y * w.y;
                        im += r.x * w.y + r.y * w.x;
                    }
                    block_sum2(re, im, red);
                    if (tid == 0)
                        a.series_rho[((size_t)s * a.T + t) * a.nops + j] = make_double2(re, im);
                }
            }
            if (t + 1 == a.T) break;  // the evolution after the last sample is never read
            for (int r = 0; r < a.k; ++r) {
                for (int fi = 0; fi < a.nf; ++fi) {
                    const CeFactor &f = fac[fi];
                    const int G = V32 / f.D;
                    if (ce_thread_form(f.D))
                        ce_apply<int>(V, Um + f.mat, f, offs + f.off, G, tid, nt);
                    else
                        ce_apply_warp<int>(V, Um + f.mat, f, offs + f.off, G, warp, nw, lane);
                    __syncthreads();
                }
            }
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------- double-word FP32 path
// GB300 runs FP32 at 64x its FP64 rate, so the mixed form keeps every
// state entry and factor entry as an unevaluated sum hi + lo of two FP32
// numbers (about 48 significant bits) and evaluates each group product
// y_i = sum_j u_ij x_j on the FP32 pipe.  Lanes of packed f32x2 registers
// carry (re, im) of x; two sums run side by side,
//     S1 = sum (u_re, u_re) * (x_re, x_im),  S2 = sum (u_im, u_im) * (x_re, x_im),
// and y = S1 + (-S2_im, S2_re) is formed once per output.
//
// Anchored accumulation: each sum starts at a power of two K >= 4 ||u_i||
// ||x_group|| (Cauchy-Schwarz bounds every partial sum and every product
// by ||u_i|| ||x||), so the running value s stays in [3K/4, 5K/4]:
//     t = fma(u, x, s)       one rounding of s + u x,
//     s - t                  exact (Sterbenz: s and t within a factor 2),
//     r = fma(u, x, s - t)   that rounding error, rounded once more,
// and r goes into a plain FP32 compensation c together with the hi x lo
// and lo x hi cross terms; s - K is exact at the end.  Four packed
// instructions per real product instead of TwoProduct + TwoSum's seven, so
// a complex multiply-add costs 12 packed instructions.  The error of one
// group product is about 2^-44 K, i.e. ~2^-40 relative to the output.
// One factor entry as lane pairs: hi (u_re, u_re), (u_im, u_im) and lo.
struct DwU {
    u64 R, I, lR, lI;
};

__device__ __forceinline__ DwU dw_entry(double2 u) {
    const float hr = (float)u.x, hi = (float)u.y;
    const float lr = (float)(u.x - (double)hr), li = (float)(u.y - (double)hi);
    DwU e;
    e.R = f32x2(hr, hr);
    e.I = f32x2(hi, hi);
    e.lR = f32x2(lr, lr);
    e.lI = f32x2(li, li);
    return e;
}

// Shared-memory position of state entry x: the low three bits are XORed
// with bits 3..5 (msk = 7; msk = 0 leaves the layout alone), so that the
// eight 16-byte entries a quarter-warp reads at a stride of 8 entries (the
// groups of a factor on the last, stride-1 digit) fall in distinct banks
// while contiguous runs stay contiguous.  A permutation inside every
// aligned block of 8 entries.
template <typename I>
__device__ __forceinline__ I swz(I x, int msk) {
    return x ^ ((x >> 3) & (I)msk);
}

template <int D, typename I>
__device__ __forceinline__ void ce_group_dw(float4 *__restrict__ V, const DwU *__restrict__ U,
                                            float rnorm, const CeFactor &f,
                                            const I *__restrict__ off, I g, int msk) {
    const I base = ce_base<I>(f, g);
    u64 xh[D], xl[D];
    float n2 = 0.f;
#pragma unroll
    for (int j = 0; j < D; ++j) {
        const float4 v = V[swz<I>(base + off[j], msk)];
        xh[j] = f32x2(v.x, v.y);
        xl[j] = f32x2(v.z, v.w);
        n2 = fmaf(v.x, v.x, fmaf(v.y, v.y, n2));
    }
    // 4.01 covers the lo parts and the rounding of n2 and of the square root
    const float K = pow2_above(4.01f * rnorm * sqrtf(n2));
    const u64 KK = f32x2(K, K);
#pragma unroll 1
    for (int i = 0; i < D; ++i) {
        u64 s1 = KK, s2 = KK, c1 = 0ull, c2 = 0ull;
#pragma unroll
        for (int j = 0; j < D; ++j) {
            const DwU &u = U[i * D + j];
            const u64 t1 = fma_f32x2(u.R, xh[j], s1);
            const u64 t2 = fma_f32x2(u.I, xh[j], s2);
            c1 = add2(c1, fma_f32x2(u.R, xh[j], sub2(s1, t1)));
            c2 = add2(c2, fma_f32x2(u.I, xh[j], sub2(s2, t2)));
            s1 = t1;
            s2 = t2;
            c1 = fma_f32x2(u.R, xl[j], c1);
            c2 = fma_f32x2(u.I, xl[j], c2);
            c1 = fma_f32x2(u.lR, xh[j], c1);
            c2 = fma_f32x2(u.lI, xh[j], c2);
        }
        // sub2 with the anchor is exact
        V[swz<I>(base + off[i], msk)] = dw_finish(sub2(s1, KK), c1, sub2(s2, KK), c2);
    }
}

// Factors outside the register-resident set: one warp per group, FP64
// arithmetic on the double-word values (rare: D = 7, 11, 13-15, > 16).
template <int R, typename I>
__device__ __forceinline__ void ce_group_dw_warp(float4 *__restrict__ V,
                                                 const double2 *__restrict__ U,
                                                 const CeFactor &f, const I *__restrict__ off, I g,
                                                 int lane, int msk) {
    const int D = f.D;
    const I base = ce_base<I>(f, g);
    double2 x[R], y[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = lane + 32 * r;
        x[r] = j < D ? dw_join(V[swz<I>(base + off[j], msk)]) : make_double2(0.0, 0.0);
        y[r] = make_double2(0.0, 0.0);
    }
    __syncwarp();
#pragma unroll
    for (int r2 = 0; r2 < R; ++r2) {
        for (int jj = 0; jj < 32; ++jj) {
            const int j = 32 * r2 + jj;
            if (j >= D) break;
            const double xr = __shfl_sync(0xffffffffu, x[r2].x, jj);
            const double xi = __shfl_sync(0xffffffffu, x[r2].y, jj);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int i = lane + 32 * r;
                if (i < D) {
                    const double2 u = U[i * D + j];
                    y[r].x = fma(u.x, xr, fma(-u.y, xi, y[r].x));
                    y[r].y = fma(u.x, xi, fma(u.y, xr, y[r].y));
                }
            }
        }
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int i = lane + 32 * r;
        if (i < D) V[swz<I>(base + off[i], msk)] = dw_split(y[r]);
    }
}

template <typename I>
__device__ void ce_apply_dw(float4 *__restrict__ V, const DwU *__restrict__ U,
                            const double2 *__restrict__ Ud, float rnorm, const CeFactor &f,
                            const I *__restrict__ off, I G, int tid, int nt, int lane, int warp,
                            int nw, int msk) {
    switch (f.D) {
#define CE_DW_CASE(DD)                                                                    \
    case DD:                                                                              \
        for (I g = tid; g < G; g += nt) ce_group_dw<DD, I>(V, U, rnorm, f, off, g, msk);  \
        return;
        CE_DW_CASE(1)
        CE_DW_CASE(2)
        CE_DW_CASE(3)
        CE_DW_CASE(4)
        CE_DW_CASE(5)
        CE_DW_CASE(6)
        CE_DW_CASE(8)
        CE_DW_CASE(9)
        CE_DW_CASE(10)
        CE_DW_CASE(12)
        CE_DW_CASE(16)
#undef CE_DW_CASE
        default:
            break;
    }
    const int R = (f.D + 31) >> 5;
    for (I g = warp; g < G; g += nw) {
        if (R == 1)
            ce_group_dw_warp<1, I>(V, Ud, f, off, g, lane, msk);
        else if (R == 2)
            ce_group_dw_warp<2, I>(V, Ud, f, off, g, lane, msk);
        else if (R == 3)
            ce_group_dw_warp<3, I>(V, Ud, f, off, g, lane, msk);
        else
            ce_group_dw_warp<4, I>(V, Ud, f, off, g, lane, msk);
    }
}

// Shared memory of the double-word kernel: state (16 B per entry), factor
// entries in lane patterns (48 B) and, for the warp-form factors, in FP64.
__global__ void __launch_bounds__(CE_DW_THREADS) msp_celio_smem_dw_kernel(CeArgs a) {
    extern __shared__ __align__(16) unsigned char ce_smem[];
    float4 *V = reinterpret_cast<float4 *>(ce_smem);
    DwU *Uw = reinterpret_cast<DwU *>(V + a.V);
    double2 *Ud = reinterpret_cast<double2 *>(Uw + a.mats_len);
    CeFactor *fac = reinterpret_cast<CeFactor *>(Ud + a.mats_len);
    float *rnorm = reinterpret_cast<float *>(fac + a.nf);
    int *offs = reinterpret_cast<int *>(rnorm + ((a.nf + 3) & ~3));
    double *red = reinterpret_cast<double *>(offs + ((a.noffs + 3) & ~3));

    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    for (int i = tid; i < a.nf; i += nt) fac[i] = a.fac[i];
    for (int i = tid; i < a.noffs; i += nt) offs[i] = (int)a.offs[i];

    const int V32 = (int)a.V;
    const int msk = (V32 & 7) == 0 ? 7 : 0;
    int loaded = -1;
    for (int st = blockIdx.x; st < a.S * a.A; st += gridDim.x) {
        const int s = st / a.A;
        const int blk = a.mats_per_snap ? s : 0;
        if (blk != loaded) {
            const double2 *src = a.mats + (size_t)blk * a.mats_len;
            for (long long i = tid; i < a.mats_len; i += nt) {
                const double2 u = src[i];
                Uw[i] = dw_entry(u);
                Ud[i] = u;
            }
            // largest row 2-norm of each factor (1 for a unitary factor)
            for (int fi = tid; fi < a.nf; fi += nt) {
                const CeFactor &f = a.fac[fi];
                const double2 *m = src + f.mat;
                double best = 0.0;
                for (int r = 0; r < f.D; ++r) {
                    double q = 0.0;
                    for (int c = 0; c < f.D; ++c) q += m[r * f.D + c].x * m[r * f.D + c].x +
                                                       m[r * f.D + c].y * m[r * f.D + c].y;
                    best = fmax(best, q);
                }
                rnorm[fi] = (float)(sqrt(best) * (1.0 + 1e-6));
            }
            loaded = blk;
        }
        if (a.mode == MSP_CELIO_PURE) {
            for (int x = tid; x < V32; x += nt) V[swz(x, msk)] = dw_split(ce_init_pure(a, st, x));
        } else {
            const double2 *r0 = a.rho0 + (size_t)s * a.V;
            for (int x = tid; x < V32; x += nt) V[swz(x, msk)] = dw_split(r0[x]);
        }
        __syncthreads();
        for (int t = 0; t < a.T; ++t) {
            if (a.mode == MSP_CELIO_PURE) {
                const double2 *sg = a.sigma + 4 * s;
                const double2 m00 = sg[0], m01 = sg[1], m11 = sg[3];
                double m = 0.0, z = 0.0;
                for (int kk = tid; kk < (int)a.half; kk += nt) {
                    const double2 u = dw_join(V[swz(kk, msk)]);
                    const double2 d = dw_join(V[swz(kk + (int)a.half, msk)]);
                    const double tr = m00.x * u.x - m00.y * u.y + 2.0 * (m01.x * d.x - m01.y * d.y);
                    const double ti = m00.x * u.y + m00.y * u.x + 2.0 * (m01.x * d.y + m01.y * d.x);
                    m += u.x * tr + u.y * ti;
                    const double sr = m11.x * d.x - m11.y * d.y, si = m11.x * d.y + m11.y * d.x;
                    m += d.x * sr + d.y * si;
                }
                block_sum2(m, z, red);
                if (tid == 0) a.series_pure[(size_t)st * a.T + t] = m;
            } else {
                const double2 *W0 = a.meas + (size_t)(a.meas_per_snap ? s : 0) * a.nops * a.V;
                for (int j = 0; j < a.nops; ++j) {
                    const double2 *W = W0 + (size_t)j * a.V;
                    double re = 0.0, im = 0.0;
                    for (int x = tid; x < V32; x += nt) {
                        const double2 r = dw_join(V[swz(x, msk)]), w = W[x];
                        re += r.x * w.x - r.y * w.y;
                        im += r.x * w.y + r.y * w.x;
                    }
                    block_sum2(re, im, red);
                    if (tid == 0)
                        a.series_rho[((size_t)s * a.T + t) * a.nops + j] = make_double2(re, im);
                }
            }
            if (t + 1 == a.T) break;
            for (int r = 0; r < a.k; ++r) {
                for (int fi = 0; fi < a.nf; ++fi) {
                    const CeFactor &f = fac[fi];
                    ce_apply_dw<int>(V, Uw + f.mat, Ud + f.mat, rnorm[fi], f, offs + f.off,
                                     V32 / f.D, tid, nt, lane, warp, nw, msk);
                    __syncthreads();
                }
            }
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------- global-memory path
__device__ __forceinline__ double2 ce_ld(const double2 *V, long long x) { return V[x]; }
__device__ __forceinline__ double2 ce_ld(const float4 *V, long long x) { return dw_join(V[x]); }
__device__ __forceinline__ void ce_st(double2 *V, long long x, double2 v) { V[x] = v; }
__device__ __forceinline__ void ce_st(float4 *V, long long x, double2 v) { V[x] = dw_split(v); }

template <typename S>
__global__ void msp_celio_init_kernel(CeArgs a) {
    S *state = reinterpret_cast<S *>(a.state);
    const long long total = (long long)a.S * a.A * a.V;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int st = (int)(e / a.V);
        const long long x = e - (long long)st * a.V;
        ce_st(state, e, a.mode == MSP_CELIO_PURE ? ce_init_pure(a, st, x)
                                                 : a.rho0[(size_t)(st / a.A) * a.V + x]);
    }
}

// Global double-word path: factor entries in lane patterns and the row
// 2-norm bound of every factor, once per run.
__global__ void msp_celio_dw_prep_kernel(CeArgs a, int blocks) {
    DwU *dst = reinterpret_cast<DwU *>(a.dwmats);
    const long long total = (long long)blocks * a.mats_len;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x)
        dst[e] = dw_entry(a.mats[e]);
    const long long nfb = (long long)blocks * a.nf;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nfb;
         e += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(e / a.nf), fi = (int)(e - (long long)b * a.nf);
        const CeFactor &f = a.fac[fi];
        const double2 *m = a.mats + (size_t)b * a.mats_len + f.mat;
        double best = 0.0;
        for (int r = 0; r < f.D; ++r) {
            double q = 0.0;
            for (int c = 0; c < f.D; ++c)
                q += m[r * f.D + c].x * m[r * f.D + c].x + m[r * f.D + c].y * m[r * f.D + c].y;
            best = fmax(best, q);
        }
        a.rnorms[e] = (float)(sqrt(best) * (1.0 + 1e-6));
    }
}

__global__ void msp_celio_apply_dw_kernel(CeArgs a, CeFactor f, int fi) {
    const long long G = a.V / f.D;
    const long long *off = a.offs + f.off;
    const int states = a.S * a.A;
    const long long total = G * states;
    float4 *state = reinterpret_cast<float4 *>(a.state);
    const DwU *dw = reinterpret_cast<const DwU *>(a.dwmats);
    if (ce_thread_form(f.D)) {
        for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
             e += (long long)gridDim.x * blockDim.x) {
            const int st = (int)(e / G);
            const long long g = e - (long long)st * G;
            const int blk = a.mats_per_snap ? st / a.A : 0;
            float4 *V = state + (size_t)st * a.V;
            const DwU *U = dw + (size_t)blk * a.mats_len + f.mat;
            const float rn = a.rnorms[(size_t)blk * a.nf + fi];
            switch (f.D) {
#define CE_DWG_CASE(DD)                                          \
    case DD:                                                     \
        ce_group_dw<DD, long long>(V, U, rn, f, off, g, 0);      \
        break;
                CE_DWG_CASE(1)
                CE_DWG_CASE(2)
                CE_DWG_CASE(3)
                CE_DWG_CASE(4)
                CE_DWG_CASE(5)
                CE_DWG_CASE(6)
                CE_DWG_CASE(8)
                CE_DWG_CASE(9)
                CE_DWG_CASE(10)
                CE_DWG_CASE(12)
                CE_DWG_CASE(16)
#undef CE_DWG_CASE
                default:
                    break;
            }
        }
    } else {
        const int lane = threadIdx.x & 31;
        const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
        const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
        const int R = (f.D + 31) >> 5;
        for (long long e = wid; e < total; e += nwarps) {
            const int st = (int)(e / G);
            const long long g = e - (long long)st * G;
            const int blk = a.mats_per_snap ? st / a.A : 0;
            float4 *V = state + (size_t)st * a.V;
            const double2 *Ud = a.mats + (size_t)blk * a.mats_len + f.mat;
            if (R == 1)
                ce_group_dw_warp<1, long long>(V, Ud, f, off, g, lane, 0);
            else if (R == 2)
                ce_group_dw_warp<2, long long>(V, Ud, f, off, g, lane, 0);
            else if (R == 3)
                ce_group_dw_warp<3, long long>(V, Ud, f, off, g, lane, 0);
            else
                ce_group_dw_warp<4, long long>(V, Ud, f, off, g, lane, 0);
        }
    }
}

__global__ void msp_celio_apply_kernel(CeArgs a, CeFactor f) {
    const long long G = a.V / f.D;
    const long long *off = a.offs + f.off;
    const int states = a.S * a.A;
    if (ce_thread_form(f.D)) {
        const long long total = G * states;
        for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
             e += (long long)gridDim.x * blockDim.x) {
            const int st = (int)(e / G);
            const long long g = e - (long long)st * G;
            const int blk = a.mats_per_snap ? st / a.A : 0;
            double2 *V = a.state + (size_t)st * a.V;
            const double2 *U = a.mats + (size_t)blk * a.mats_len + f.mat;
            ce_apply<long long>(V, U, f, off, g + 1, g, 1);
        }
    } else {
        const int lane = threadIdx.x & 31;
        const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
        const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
        const long long total = G * states;
        for (long long e = wid; e < total; e += nwarps) {
            const int st = (int)(e / G);
            const long long g = e - (long long)st * G;
            const int blk = a.mats_per_snap ? st / a.A : 0;
            double2 *V = a.state + (size_t)st * a.V;
            const double2 *U = a.mats + (size_t)blk * a.mats_len + f.mat;
            ce_apply_warp<long long>(V, U, f, off, g + 1, g, 1, lane);
        }
    }
}

// Partial sums of one measurement: CTA (chunk c, state st).
template <typename S>
__global__ void __launch_bounds__(CE_THREADS) msp_celio_measure_kernel(CeArgs a) {
    __shared__ double red[2 * (CE_THREADS / 32)];
    const int c = blockIdx.x, st = blockIdx.y;
    const S *V = reinterpret_cast<const S *>(a.state) + (size_t)st * a.V;
    double *out = a.partial + ((size_t)st * a.chunks + c) * 2 * a.nops;
    if (a.mode == MSP_CELIO_PURE) {
        const long long lo = (long long)c * CE_CHUNK;
        const long long hi = lo + CE_CHUNK < a.half ? lo + CE_CHUNK : a.half;
        const double2 *sg = a.sigma + 4 * (st / a.A);
        const double2 m00 = sg[0], m01 = sg[1], m11 = sg[3];
        double m = 0.0, z = 0.0;
        for (long long kk = lo + threadIdx.x; kk < hi; kk += blockDim.x) {
            const double2 u = ce_ld(V, kk), d = ce_ld(V, a.half + kk);
            const double tr = m00.x * u.x - m00.y * u.y + 2.0 * (m01.x * d.x - m01.y * d.y);
            const double ti = m00.x * u.y + m00.y * u.x + 2.0 * (m01.x * d.y + m01.y * d.x);
            m += u.x * tr + u.y * ti;
            const double sr = m11.x * d.x - m11.y * d.y, si = m11.x * d.y + m11.y * d.x;
            m += d.x * sr + d.y * si;
        }
        block_sum2(m, z, red);
        if (threadIdx.x == 0) out[0] = m;
    } else {
        const int s = st;
        const long long lo = (long long)c * CE_CHUNK;
        const long long hi = lo + CE_CHUNK < a.V ? lo + CE_CHUNK : a.V;
        const double2 *W0 = a.meas + (size_t)(a.meas_per_snap ? s : 0) * a.nops * a.V;
        for (int j = 0; j < a.nops; ++j) {
            const double2 *W = W0 + (size_t)j * a.V;
            double re = 0.0, im = 0.0;
            for (long long x = lo + threadIdx.x; x < hi; x += blockDim.x) {
                const double2 r = ce_ld(V, x), w = W[x];
                re += r.x * w.x - r.y * w.y;
                im += r.x * w.y + r.y * w.x;
            }
            block_sum2(re, im, red);
            if (threadIdx.x == 0) {
                out[2 * j] = re;
                out[2 * j + 1] = im;
            }
        }
    }
}

// Chunk partials of time t summed in chunk order.
__global__ void msp_celio_measure_finish_kernel(CeArgs a, int t) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int states = a.S * a.A;
    if (e >= states * a.nops) return;
    const int st = e / a.nops, j = e - st * a.nops;
    const double *p = a.partial + (size_t)st * a.chunks * 2 * a.nops + 2 * j;
    double re = 0.0, im = 0.0;
    for (int c = 0; c < a.chunks; ++c) {
        re += p[(size_t)c * 2 * a.nops];
        im += p[(size_t)c * 2 * a.nops + 1];
    }
    if (a.mode == MSP_CELIO_PURE)
        a.series_pure[(size_t)st * a.T + t] = re;
    else
        a.series_rho[((size_t)st * a.T + t) * a.nops + j] = make_double2(re, im);
}

// rows[r][t] = sum over the snapshots of row r (in order) of wscale[s] *
// (PURE: 0.5 / A * sum_a series; DENSITY: Re series of operator 0).
__global__ void msp_celio_rows_kernel(CeArgs a, const double *__restrict__ wscale,
                                      const int *__restrict__ row_start, int num_rows,
                                      double *__restrict__ rows) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)num_rows * a.T) return;
    const int r = (int)(e / a.T), t = (int)(e - (long long)r * a.T);
    double acc = 0.0;
    for (int s = row_start[r]; s < row_start[r + 1]; ++s) {
        double v;
        if (a.mode == MSP_CELIO_PURE) {
            double m = 0.0;
            for (int av = 0; av < a.A; ++av) m += a.series_pure[((size_t)s * a.A + av) * a.T + t];
            v = m * (1.0 / a.A) * 0.5;
        } else {
            v = a.series_rho[((size_t)s * a.T + t) * a.nops].x;
        }
        acc += v * (wscale ? wscale[s] : 1.0);
    }
    rows[e] = acc;
}

// ----------------------------------------------------------- factor exponentials
constexpr int EX_WARPS = 4;
constexpr int EX_MAXD = 16;
constexpr int EX_TAYLOR = 16;
constexpr int EX_MAX_FACTORS = 64;

// Field-dependent factors of one call (host values, passed by value).
struct ExDesc {
    int nf;
    int dims[EX_MAX_FACTORS];
    long long hoff[EX_MAX_FACTORS];     // complex entries before factor f in H0 (x 3 in G)
    long long out[3 * EX_MAX_FACTORS];  // offsets of U, U^dagger, U^T in a block (-1: skip)
};

// out = A * B for D x D complex matrices in shared memory, one warp.
__device__ __forceinline__ void ex_matmul(double2 *out, const double2 *A, const double2 *B, int D,
                                          int lane) {
    for (int e = lane; e < D * D; e += 32) {
        const int i = e / D, j = e - (e / D) * D;
        double re = 0.0, im = 0.0;
        for (int q = 0; q < D; ++q) {
            const double2 x = A[i * D + q], y = B[q * D + j];
            re = fma(x.x, y.x, fma(-x.y, y.y, re));
            im = fma(x.x, y.y, fma(x.y, y.x, im));
        }
        out[e] = make_double2(re, im);
    }
    __syncwarp();
}

// U = exp(-2 pi i tau (H0 + sum_a B_a G_a)) for each (snapshot, factor), by
// scaling (||X||_1 <= 1/2), a degree-16 Taylor polynomial in Horner form
// (truncation < 1e-19) and squaring; written as U, U^dagger and / or U^T.
__global__ void __launch_bounds__(32 * EX_WARPS) msp_celio_expm_kernel(
    int S, ExDesc ex, const double2 *__restrict__ H0, const double2 *__restrict__ Gm,
    const double *__restrict__ B, double tau, double2 *__restrict__ mats, long long mats_len) {
    __shared__ double2 buf[EX_WARPS][3][EX_MAXD * EX_MAXD];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nf = ex.nf;
    const long long job = (long long)blockIdx.x * EX_WARPS + w;
    if (job >= (long long)S * nf) return;
    const int s = (int)(job / nf), f = (int)(job - (long long)s * nf);
    const int D = ex.dims[f];
    double2 *X = buf[w][0], *P = buf[w][1], *Y = buf[w][2];
    const double2 *h = H0 + ex.hoff[f];
    const double2 *g = Gm + 3 * ex.hoff[f];
    const double bx = B[3 * s], by = B[3 * s + 1], bz = B[3 * s + 2];
    const double c = -2.0 * CUDART_PI * tau;
    // X = -2 pi i tau H  =>  X = (c Im H ... ): (i c) * (hr + i hi) = -c hi + i c hr
    for (int e = lane; e < D * D; e += 32) {
        const double hr = h[e].x + bx * g[e].x + by * g[D * D + e].x + bz * g[2 * D * D + e].x;
        const double hi = h[e].y + bx * g[e].y + by * g[D * D + e].y + bz * g[2 * D * D + e].y;
        X[e] = make_double2(-c * hi, c * hr);
    }
    __syncwarp();
    double colmax = 0.0;
    for (int j = lane; j < D; j += 32) {
        double sum = 0.0;
        for (int i = 0; i < D; ++i) sum += hypot(X[i * D + j].x, X[i * D + j].y);
        colmax = fmax(colmax, sum);
    }
    for (int o = 16; o > 0; o >>= 1) colmax = fmax(colmax, __shfl_xor_sync(0xffffffffu, colmax, o));
    int sq = 0;
    double scale = 1.0;
    while (colmax * scale > 0.5 && sq < 60) {
        scale *= 0.5;
        ++sq;
    }
    for (int e = lane; e < D * D; e += 32) {
        X[e].x *= scale;
        X[e].y *= scale;
        P[e] = make_double2((e / D) == (e - (e / D) * D) ? 1.0 : 0.0, 0.0);
    }
    __syncwarp();
    for (int j = EX_TAYLOR; j >= 1; --j) {
        ex_matmul(Y, X, P, D, lane);
        const double inv = 1.0 / j;
        for (int e = lane; e < D * D; e += 32) {
            const bool diag = (e / D) == (e - (e / D) * D);
            P[e] = make_double2(Y[e].x * inv + (diag ? 1.0 : 0.0), Y[e].y * inv);
        }
        __syncwarp();
    }
    for (int q = 0; q < sq; ++q) {
        ex_matmul(Y, P, P, D, lane);
        for (int e = lane; e < D * D; e += 32) P[e] = Y[e];
        __syncwarp();
    }
    double2 *dst = mats + (size_t)s * mats_len;
    const long long oU = ex.out[3 * f], oH = ex.out[3 * f + 1], oT = ex.out[3 * f + 2];
    for (int e = lane; e < D * D; e += 32) {
        const int i = e / D, j = e - (e / D) * D;
        if (oU >= 0) dst[oU + e] = P[e];
        if (oH >= 0) dst[oH + j * D + i] = make_double2(P[e].x, -P[e].y);
        if (oT >= 0) dst[oT + j * D + i] = P[e];
    }
}

// ----------------------------------------------------------- host side
static int ce_fail(int code, const char *m) { return record_error(code, m); }

static int ce_cuda(cudaError_t e) {
    return e == cudaSuccess ? MSP_OK : record_error(MSP_ERR_CUDA, cudaGetErrorString(e));
}

static size_t ce_align(size_t x) { return (x + 255) & ~(size_t)255; }

struct CePlan {
    std::vector<CeFactor> fac;
    std::vector<long long> offs;
    long long V = 0, half = 0;
    int states = 0;
    int chunks = 1;
    size_t smem = 0;
    bool use_smem = false;
    bool dw = false;  // double-word FP32 shared-memory kernel
};

static int ce_plan(const msp_celio_args *a, CePlan &p) {
    if (a == NULL) return ce_fail(MSP_ERR_ARG, "msp_celio: args is NULL");
    if (a->mode != MSP_CELIO_PURE && a->mode != MSP_CELIO_DENSITY)
        return ce_fail(MSP_ERR_ARG, "msp_celio: mode must be MSP_CELIO_PURE or MSP_CELIO_DENSITY");
    if (a->num_digits < 1 || a->num_digits > CE_MAX_DIGITS || a->digit_dims == NULL)
        return ce_fail(MSP_ERR_ARG, "msp_celio: num_digits outside 1..32 or digit_dims NULL");
    if (a->num_factors < 0 || a->num_factors > CE_MAX_FACTORS ||
        (a->num_factors > 0 && (a->factor_digits == NULL || a->factor_mat == NULL)))
        return ce_fail(MSP_ERR_ARG, "msp_celio: num_factors outside 0..1024 or descriptors NULL");
    if (a->num_snapshots < 0 || a->states_per_snapshot < 1 || a->trotter_k < 1 ||
        a->num_times < 0)
        return ce_fail(MSP_ERR_ARG, "msp_celio: sizes (snapshots, states, k, times)");
    long long strides[CE_MAX_DIGITS];
    long long V = 1;
    for (int d = a->num_digits - 1; d >= 0; --d) {
        if (a->digit_dims[d] < 1) return ce_fail(MSP_ERR_ARG, "msp_celio: a digit dimension < 1");
        strides[d] = V;
        V *= a->digit_dims[d];
        if (V > (1ll << 34)) return ce_fail(MSP_ERR_UNSUPPORTED, "msp_celio: state larger than 2^34");
    }
    p.V = V;
    if (a->mode == MSP_CELIO_PURE) {
        if (a->digit_dims[0] != 2)
            return ce_fail(MSP_ERR_ARG, "msp_celio: PURE needs the muon (dimension 2) as digit 0");
        p.half = V / 2;
        if (a->mu_psi == NULL || a->sigma == NULL)
            return ce_fail(MSP_ERR_ARG, "msp_celio: PURE needs mu_psi and sigma");
    } else {
        if (a->states_per_snapshot != 1)
            return ce_fail(MSP_ERR_ARG, "msp_celio: DENSITY has one state per snapshot");
        if (a->rho0 == NULL || a->meas == NULL || a->num_ops < 1)
            return ce_fail(MSP_ERR_ARG, "msp_celio: DENSITY needs rho0, meas and num_ops >= 1");
    }
    if (a->num_factors > 0 && (a->mats == NULL || a->mats_len < 1))
        return ce_fail(MSP_ERR_ARG, "msp_celio: mats");
    p.fac.resize(a->num_factors);
    p.offs.clear();
    for (int fi = 0; fi < a->num_factors; ++fi) {
        const int d0 = a->factor_digits[2 * fi], d1 = a->factor_digits[2 * fi + 1];
        if (d0 < 0 || d0 >= a->num_digits || d1 >= a->num_digits || d1 == d0)
            return ce_fail(MSP_ERR_ARG, "msp_celio: factor digits out of range or repeated");
        CeFactor f;
        memset(&f, 0, sizeof(f));
        f.two = d1 >= 0;
        const int D0 = a->digit_dims[d0], D1 = f.two ? a->digit_dims[d1] : 1;
        f.D = D0 * D1;
        if (f.D > CE_MAX_D) return ce_fail(MSP_ERR_UNSUPPORTED, "msp_celio: factor dimension > 128");
        if (f.two) {
            const int a_ = strides[d0] > strides[d1] ? d0 : d1, b_ = a_ == d0 ? d1 : d0;
            f.sA = strides[a_];
            f.DA = a->digit_dims[a_];
            f.sB = strides[b_];
            f.DB = a->digit_dims[b_];
            f.M = f.sA / (f.sB * f.DB);
        } else {
            f.sA = strides[d0];
            f.DA = D0;
            f.sB = 1;
            f.DB = 1;
            f.M = 1;
        }
        f.mat = a->factor_mat[fi];
        if (f.mat < 0 || f.mat + (long long)f.D * f.D > a->mats_len)
            return ce_fail(MSP_ERR_ARG, "msp_celio: a factor matrix lies outside mats_len");
        f.off = (int)p.offs.size();
        // element j of a group in the factor's own order: j = j0 * D1 + j1
        for (int j = 0; j < f.D; ++j) {
            const int j0 = j / D1, j1 = j - (j / D1) * D1;
            p.offs.push_back(j0 * strides[d0] + (f.two ? j1 * strides[d1] : 0));
        }
        p.fac[fi] = f;
    }
    p.states = a->num_snapshots * a->states_per_snapshot;
    const long long span = a->mode == MSP_CELIO_PURE ? p.half : V;
    p.chunks = (int)((span + CE_CHUNK - 1) / CE_CHUNK);
    if (p.chunks < 1) p.chunks = 1;
    if (a->precision != MSP_PREC_FP64 && a->precision != MSP_PREC_MIXED)
        return ce_fail(MSP_ERR_ARG, "msp_celio: precision must be MSP_PREC_FP64 or MSP_PREC_MIXED");
    const size_t offs_pad = (p.offs.size() + 3) & ~(size_t)3;
    const bool mixed = a->precision == MSP_PREC_MIXED;
    const size_t mats_b = (size_t)a->mats_len * (mixed ? 48 : 16);
    const size_t rnorm_b = mixed ? ((p.fac.size() + 3) & ~(size_t)3) * 4 : 0;
    p.smem = (size_t)V * 16 + mats_b + p.fac.size() * sizeof(CeFactor) + rnorm_b +
             offs_pad * 4 + 2 * (CE_DW_THREADS / 32) * sizeof(double);
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        optin = 227 * 1024;
    }
    const bool fits = p.smem <= (size_t)optin && V < (1ll << 30);
    p.use_smem = a->path == 1 ? true : (a->path == 2 ? false : fits);
    if (p.use_smem && !fits)
        return ce_fail(MSP_ERR_UNSUPPORTED, "msp_celio: state does not fit in shared memory");
    p.dw = a->precision == MSP_PREC_MIXED;
    return MSP_OK;
}

static size_t ce_workspace(const msp_celio_args *a, const CePlan &p) {
    size_t b = ce_align(p.fac.size() * sizeof(CeFactor) + 16) + ce_align(p.offs.size() * 8 + 16);
    const size_t series = a->mode == MSP_CELIO_PURE
                              ? (size_t)p.states * a->num_times * sizeof(double)
                              : (size_t)a->num_snapshots * a->num_times * a->num_ops * 16;
    if (a->series == NULL) b += ce_align(series + 16);
    if (!p.use_smem) {
        b += ce_align((size_t)p.states * p.V * 16);
        const int nops = a->mode == MSP_CELIO_PURE ? 1 : a->num_ops;
        b += ce_align((size_t)p.states * p.chunks * 2 * nops * sizeof(double));
        if (p.dw) {
            const size_t blocks = a->mats_per_snapshot ? (size_t)a->num_snapshots : 1;
            b += ce_align(blocks * (size_t)a->mats_len * 32 + 16);
            b += ce_align(blocks * p.fac.size() * sizeof(float) + 16);
        }
    }
    return b;
}

static int ce_sms() {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        sms = 152;
    }
    return sms;
}

}  // namespace

extern "C" {

int msp_celio_workspace(const msp_celio_args *args, size_t *bytes) {
    CePlan p;
    const int rc = ce_plan(args, p);
    if (rc != MSP_OK) return rc;
    if (bytes == NULL) return ce_fail(MSP_ERR_ARG, "msp_celio_workspace: bytes is NULL");
    *bytes = ce_workspace(args, p);
    return MSP_OK;
}

int msp_celio_run(const msp_celio_args *a, void *workspace, size_t workspace_bytes,
                  void *stream) {
    CePlan p;
    int rc = ce_plan(a, p);
    if (rc != MSP_OK) return rc;
    if (a->num_snapshots == 0 || a->num_times == 0) return MSP_OK;
    if (workspace == NULL || ((uintptr_t)workspace & 255) != 0 ||
        workspace_bytes < ce_workspace(a, p))
        return ce_fail(MSP_ERR_WORKSPACE, "msp_celio_run: workspace too small or not 256-byte aligned");
    if (a->rows_out != NULL && (a->row_start == NULL || a->num_rows < 1))
        return ce_fail(MSP_ERR_ARG, "msp_celio_run: rows_out needs row_start and num_rows");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *w = (unsigned char *)workspace;
    CeArgs k;
    memset(&k, 0, sizeof(k));
    CeFactor *dfac = (CeFactor *)w;
    w += ce_align(p.fac.size() * sizeof(CeFactor) + 16);
    long long *doffs = (long long *)w;
    w += ce_align(p.offs.size() * 8 + 16);
    if (!p.fac.empty()) {
        rc = ce_cuda(cudaMemcpyAsync(dfac, p.fac.data(), p.fac.size() * sizeof(CeFactor),
                                     cudaMemcpyHostToDevice, st));
        if (rc != MSP_OK) return rc;
        rc = ce_cuda(cudaMemcpyAsync(doffs, p.offs.data(), p.offs.size() * 8,
                                     cudaMemcpyHostToDevice, st));
        if (rc != MSP_OK) return rc;
    }
    k.fac = dfac;
    k.offs = doffs;
    k.nf = (int)p.fac.size();
    k.noffs = (int)p.offs.size();
    k.mats = (const double2 *)a->mats;
    k.mats_len = a->num_factors > 0 ? a->mats_len : 0;
    k.mats_per_snap = a->mats_per_snapshot;
    k.mode = a->mode;
    k.V = p.V;
    k.half = p.half;
    k.S = a->num_snapshots;
    k.A = a->states_per_snapshot;
    k.k = a->trotter_k;
    k.T = a->num_times;
    k.mu_psi = (const double2 *)a->mu_psi;
    k.sigma = (const double2 *)a->sigma;
    k.phases = a->phases;
    k.seed = a->seed;
    k.rho0 = (const double2 *)a->rho0;
    k.meas = (const double2 *)a->meas;
    k.nops = a->mode == MSP_CELIO_PURE ? 1 : a->num_ops;
    k.meas_per_snap = a->meas_per_snapshot;
    void *series = a->series;
    if (series == NULL) {
        series = w;
        const size_t b = a->mode == MSP_CELIO_PURE
                             ? (size_t)p.states * a->num_times * sizeof(double)
                             : (size_t)a->num_snapshots * a->num_times * a->num_ops * 16;
        w += ce_align(b + 16);
    }
    k.series_pure = (double *)series;
    k.series_rho = (double2 *)series;
    k.chunks = p.chunks;
    const int sms = ce_sms();
    if (p.use_smem) {
        void (*kern)(CeArgs) = p.dw ? msp_celio_smem_dw_kernel : msp_celio_smem_kernel;
        rc = ce_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)p.smem));
        if (rc != MSP_OK) return rc;
        int occ = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern,
                                                          p.dw ? CE_DW_THREADS : CE_THREADS,
                                                          p.smem) !=
                cudaSuccess ||
            occ < 1) {
            cudaGetLastError();
            occ = 1;
        }
        const long long cap = (long long)sms * occ;
        const int grid = (int)(p.states < cap ? p.states : cap);
        kern<<<grid, p.dw ? CE_DW_THREADS : CE_THREADS, p.smem, st>>>(k);
        rc = ce_cuda(cudaGetLastError());
        if (rc != MSP_OK) return rc;
    } else {
        k.state = (double2 *)w;
        w += ce_align((size_t)p.states * p.V * 16);
        k.partial = (double *)w;
        {
            const int nops = a->mode == MSP_CELIO_PURE ? 1 : a->num_ops;
            w += ce_align((size_t)p.states * p.chunks * 2 * nops * sizeof(double));
        }
        const long long total = (long long)p.states * p.V;
        const int igrid = (int)((total + 255) / 256 < (long long)sms * 16 ? (total + 255) / 256
                                                                         : (long long)sms * 16);
        if (p.dw) {
            const int blocks = a->mats_per_snapshot ? a->num_snapshots : 1;
            k.dwmats = (void *)w;
            w += ce_align((size_t)blocks * (size_t)a->mats_len * 32 + 16);
            k.rnorms = (float *)w;
            w += ce_align((size_t)blocks * p.fac.size() * sizeof(float) + 16);
            if (!p.fac.empty())
                msp_celio_dw_prep_kernel<<<sms * 4, 256, 0, st>>>(k, blocks);
            msp_celio_init_kernel<float4><<<igrid, 256, 0, st>>>(k);
        } else {
            msp_celio_init_kernel<double2><<<igrid, 256, 0, st>>>(k);
        }
        rc = ce_cuda(cudaGetLastError());
        if (rc != MSP_OK) return rc;
        const dim3 mgrid(p.chunks, p.states);
        const int fin = (p.states * k.nops + 127) / 128;
        for (int t = 0; t < a->num_times; ++t) {
            if (p.dw)
                msp_celio_measure_kernel<float4><<<mgrid, CE_THREADS, 0, st>>>(k);
            else
                msp_celio_measure_kernel<double2><<<mgrid, CE_THREADS, 0, st>>>(k);
            msp_celio_measure_finish_kernel<<<fin, 128, 0, st>>>(k, t);
            if (t + 1 == a->num_times) break;
            for (int r = 0; r < a->trotter_k; ++r) {
                for (size_t fi = 0; fi < p.fac.size(); ++fi) {
                    const CeFactor &f = p.fac[fi];
                    const long long work = (long long)p.states * (p.V / f.D) *
                                           (ce_thread_form(f.D) ? 1 : 32);
                    const long long blocks = (work + 255) / 256;
                    const int grid = (int)(blocks < (long long)sms * 8 ? blocks : (long long)sms * 8);
                    if (p.dw)
                        msp_celio_apply_dw_kernel<<<grid, 256, 0, st>>>(k, f, (int)fi);
                    else
                        msp_celio_apply_kernel<<<grid, 256, 0, st>>>(k, f);
                }
            }
            rc = ce_cuda(cudaGetLastError());
            if (rc != MSP_OK) return rc;
        }
    }
    if (a->rows_out != NULL) {
        const long long n = (long long)a->num_rows * a->num_times;
        msp_celio_rows_kernel<<<(int)((n + 127) / 128), 128, 0, st>>>(k, a->wscale, a->row_start,
                                                                     a->num_rows, a->rows_out);
        rc = ce_cuda(cudaGetLastError());
        if (rc != MSP_OK) return rc;
    }
    return MSP_OK;
}

int msp_celio_expm(int num_snapshots, int num_factors, const int *dims, const double *H0,
                   const double *G, const double *fields, double tau,
                   const long long *out_offsets, double *mats, long long mats_len,
                   void *stream) {
    if (num_snapshots < 0 || num_factors < 0 || num_factors > EX_MAX_FACTORS)
        return ce_fail(MSP_ERR_ARG, "msp_celio_expm: sizes outside 0..num, 0..64");
    if (num_snapshots == 0 || num_factors == 0) return MSP_OK;
    if (dims == NULL || H0 == NULL || G == NULL || fields == NULL || out_offsets == NULL ||
        mats == NULL)
        return ce_fail(MSP_ERR_ARG, "msp_celio_expm: a required pointer is NULL");
    ExDesc ex;
    memset(&ex, 0, sizeof(ex));
    ex.nf = num_factors;
    long long h = 0;
    for (int f = 0; f < num_factors; ++f) {
        const int D = dims[f];
        if (D < 1 || D > EX_MAXD)
            return ce_fail(MSP_ERR_UNSUPPORTED, "msp_celio_expm: a factor dimension outside 1..16");
        ex.dims[f] = D;
        ex.hoff[f] = h;
        h += (long long)D * D;
        for (int q = 0; q < 3; ++q) {
            const long long o = out_offsets[3 * f + q];
            if (o >= 0 && o + (long long)D * D > mats_len)
                return ce_fail(MSP_ERR_ARG, "msp_celio_expm: an output offset lies outside mats_len");
            ex.out[3 * f + q] = o;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    const long long jobs = (long long)num_snapshots * num_factors;
    const int grid = (int)((jobs + EX_WARPS - 1) / EX_WARPS);
    msp_celio_expm_kernel<<<grid, 32 * EX_WARPS, 0, st>>>(num_snapshots, ex, (const double2 *)H0,
                                                           (const double2 *)G, fields, tau,
                                                           (double2 *)mats, mats_len);
    return ce_cuda(cudaGetLastError());
}

}  // extern "C"
