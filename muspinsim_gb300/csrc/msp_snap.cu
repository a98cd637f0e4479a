// Per-snapshot kernels: one CTA diagonalises one Hamiltonian in shared
// memory and turns its eigenbasis into the quantities the time evolution
// needs.  Replaces, per configuration snapshot, ExperimentRunner.Htot
// (muspinsim/experiment.py:332-341), Hermitian.diag (muspinsim/spinop.py:
// 51-82) and the eigenbasis part of Hamiltonian.fast_evolve / evolve /
// integrate_decaying (muspinsim/hamiltonian.py:76-87, 149-160, 195-211).
//
// Precision modes:
//   FP64  -- Jacobi sweeps, eigenvalues and eigenbasis products in FP64.
//   MIXED -- Jacobi sweeps in FP32, then one Ogita-Aishima refinement step
//            evaluated in double-word FP32 arithmetic (dw_acc): residual
//            products H X, X^H H X and X^H X to ~2^-44, eigenvalues to FP64
//            accuracy (Rayleigh quotient plus the second-order term), the
//            eigenvectors corrected to FP32 rounding.  GB300 runs FP32 at
//            ~60x its FP64 rate, so this costs about as much as the FP32
//            sweeps themselves instead of dominating as FP64 would.
#include "msp_internal.cuh"
#include "msp_cluster.cuh"
#include "msp_dw.cuh"
#include "msp_jacobi.cuh"
#include "msp_rho.cuh"

#include <math_constants.h>

namespace msp {

static_assert(sizeof(JRot<float>) == 16 && sizeof(JRot<double>) == 32, "JRot layout");

// ------------------------------------------------------------------ smem layout

struct SnapLayout {
    size_t H, U, rot, dia, red, tab, diag;     // Jacobi work
    size_t lam, acc, rank;                     // eigenvalues, reductions, sort
    size_t Hh, Hl, Yl, SR, corr, rd, lamf, rk, ord, cst, scal, rn, cn, yn;  // refinement (MIXED)
    size_t fac, facf, B2;                      // general path
    size_t total;
};

__host__ __device__ inline size_t lay_take(size_t &off, size_t bytes) {
    off = (off + 15) & ~size_t(15);
    const size_t o = off;
    off += bytes;
    return o;
}

// Byte offsets of every shared-memory buffer of a snapshot kernel.  The
// same function sizes the launch (host) and carves the buffers (device).
__host__ __device__ inline SnapLayout snap_layout(int n, int esize, bool refine, bool rho,
                                                  int fac_len, int nwarps) {
    SnapLayout L;
    const size_t m = (size_t)(n + (n & 1));
    const size_t mm = m * (m + 1);  // leading dimension m + 1 (odd): no bank conflicts
    // the two Jacobi buffers hold either a matrix with row stride m + 1 or
    // the eigenvector planes with column stride jacobi_ldu(m)
    const size_t mj = (size_t)jacobi_buffer((int)m);
    size_t off = 0;
    L.H = lay_take(off, mj * 2 * esize);
    L.U = lay_take(off, mj * 2 * esize);
    L.rot = lay_take(off, 2 * (m / 2) * (esize == 4 ? 16 : 32));  // sizeof(JRot<T>)
    L.dia = lay_take(off, 2 * m * esize);
    L.red = lay_take(off, 2 * (size_t)nwarps * esize);
    L.tab = lay_take(off, (m / 2) * (m / 2 + 1) / 2 * 8);
    L.diag = lay_take(off, m * esize);
    L.lam = lay_take(off, m * 8);
    L.acc = lay_take(off, 2 * 8);
    L.rank = lay_take(off, m * 4);
    L.Hh = L.Hl = L.Yl = L.SR = L.corr = L.rd = L.lamf = 0;
    L.rk = L.ord = L.cst = L.scal = L.rn = L.cn = L.yn = 0;
    if (refine) {
        L.Hh = lay_take(off, mm * 8);
        L.Hl = lay_take(off, mm * 8);
        L.Yl = lay_take(off, mm * 8);
        L.SR = lay_take(off, mm * 8);
        L.corr = lay_take(off, m * 4);
        L.rd = lay_take(off, m * 8);
        L.lamf = lay_take(off, m * 4);
        L.rk = lay_take(off, m * 4);
        L.ord = lay_take(off, m * 4);
        L.cst = lay_take(off, m * 4);
        L.scal = lay_take(off, 4 * 4);
        L.rn = lay_take(off, m * 4);
        L.cn = lay_take(off, m * 4);
        L.yn = lay_take(off, m * 4);
    }
    L.fac = L.facf = L.B2 = 0;
    if (rho) {
        L.fac = lay_take(off, (size_t)fac_len * 16);
        if (refine) L.facf = lay_take(off, (size_t)fac_len * 8);
        // MIXED: the second basis buffer reuses Hh (free after refinement)
        L.B2 = refine ? L.Hh : lay_take(off, mm * 2 * esize);
    }
    L.total = (off + 15) & ~size_t(15);
    return L;
}

static int jacobi_threads(int m) {
    if (m <= 8) return 32;
    if (m <= 16) return 64;
    if (m <= 32) return 128;
    return 256;
}

size_t snap_smem_bytes(int n, int mode, int precision, int fac_len) {
    const int m = n + (n & 1);
    const bool mixed = precision == MSP_PREC_MIXED;
    return snap_layout(n, mixed ? 4 : 8, mixed, mode != MSP_MODE_FAST, fac_len,
                       jacobi_threads(m) / 32)
        .total;
}

template <typename T>
struct SnapSmem {
    JacobiWork<T> w;
    double *lam, *acc;  // FP64 path: eigenvalues
    float2 *lw;         // MIXED: eigenvalues as double-words (msp_dw.cuh), over lam
    int *rank;
    cx<float> *Hh, *Hl, *Yl, *SR;
    float2 *gd;         // MIXED: x_i^H x_i - 1 of the refinement step (double-word)
    float *corr, *lamf;
    int *rk, *ord, *cst, *scal;  // refinement clusters
    float *rn, *cn, *yn;         // norms: rows of H, columns of X and of Y
    cx<double> *fac;
    cx<float> *facf;    // MIXED: FP32 copy of fac
    cx<T> *B2;
};

template <typename T, bool REFINE>
__device__ __forceinline__ SnapSmem<T> snap_carve(char *base, int n, bool rho, int fac_len) {
    const SnapLayout L =
        snap_layout(n, sizeof(T), REFINE, rho, fac_len, (blockDim.x + 31) >> 5);
    SnapSmem<T> s;
    s.w.H = reinterpret_cast<cx<T> *>(base + L.H);
    s.w.U = reinterpret_cast<cx<T> *>(base + L.U);
    s.w.rot = reinterpret_cast<JRot<T> *>(base + L.rot);
    s.w.dia = reinterpret_cast<T *>(base + L.dia);
    s.w.red = reinterpret_cast<T *>(base + L.red);
    s.w.tab = reinterpret_cast<uint2 *>(base + L.tab);
    s.w.diag = reinterpret_cast<T *>(base + L.diag);
    s.lam = reinterpret_cast<double *>(base + L.lam);
    s.lw = REFINE ? reinterpret_cast<float2 *>(base + L.lam) : nullptr;
    s.acc = reinterpret_cast<double *>(base + L.acc);
    s.rank = reinterpret_cast<int *>(base + L.rank);
    s.Hh = REFINE ? reinterpret_cast<cx<float> *>(base + L.Hh) : nullptr;
    s.Hl = REFINE ? reinterpret_cast<cx<float> *>(base + L.Hl) : nullptr;
    s.Yl = REFINE ? reinterpret_cast<cx<float> *>(base + L.Yl) : nullptr;
    s.SR = REFINE ? reinterpret_cast<cx<float> *>(base + L.SR) : nullptr;
    s.corr = REFINE ? reinterpret_cast<float *>(base + L.corr) : nullptr;
    s.gd = REFINE ? reinterpret_cast<float2 *>(base + L.rd) : nullptr;
    s.lamf = REFINE ? reinterpret_cast<float *>(base + L.lamf) : nullptr;
    s.rk = REFINE ? reinterpret_cast<int *>(base + L.rk) : nullptr;
    s.ord = REFINE ? reinterpret_cast<int *>(base + L.ord) : nullptr;
    s.cst = REFINE ? reinterpret_cast<int *>(base + L.cst) : nullptr;
    s.scal = REFINE ? reinterpret_cast<int *>(base + L.scal) : nullptr;
    s.rn = REFINE ? reinterpret_cast<float *>(base + L.rn) : nullptr;
    s.cn = REFINE ? reinterpret_cast<float *>(base + L.cn) : nullptr;
    s.yn = REFINE ? reinterpret_cast<float *>(base + L.yn) : nullptr;
    s.fac = rho ? reinterpret_cast<cx<double> *>(base + L.fac) : nullptr;
    s.facf = rho && REFINE ? reinterpret_cast<cx<float> *>(base + L.facf) : nullptr;
    s.B2 = rho ? reinterpret_cast<cx<T> *>(base + L.B2) : nullptr;
    return s;
}

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ void tri_index(int e, int &j, int &k) {
    // e -> (j, k) with j >= k, e = j (j + 1) / 2 + k
    j = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
    while ((j + 1) * (j + 2) / 2 <= e) ++j;
    while (j * (j + 1) / 2 > e) --j;
    k = e - j * (j + 1) / 2;
}

__device__ __forceinline__ int pair_index(int j, int k) { return j * (j - 1) / 2 + k; }

// Frequency record of pair o (FP64 snapshot kernels): the FP64 angular
// frequency w, or -- on a uniform grid in mixed precision -- the phases
// w dt and w t0 reduced modulo 2 pi in FP64 and stored as double-word
// floats.  The mixed kernels use store_frequency_dw instead.
__device__ __forceinline__ void store_frequency(const SnapArgs &a, size_t o, double w) {
    if (a.pair_phase) {
        const double psi = reduce_2pi(w * a.dt);
        const double ph0 = a.t0 == 0.0 ? 0.0 : reduce_2pi(w * a.t0);
        const float psh = (float)psi, p0h = (float)ph0;
        a.pair_phase[o] = make_float4(psh, (float)(psi - (double)psh), p0h,
                                      (float)(ph0 - (double)p0h));
    } else {
        a.pair_omega[o] = w;
    }
}

// Frequency record of pair o on the mixed path from its level gap d
// (double-word): the phases d (2 pi dt) and d (2 pi t0) reduced modulo 2 pi,
// or the FP64 angular frequency for arbitrary grids.  No FP64 arithmetic on
// a uniform grid.
__device__ __forceinline__ void store_frequency_dw(const SnapArgs &a, size_t o, float2 d) {
    if (a.pair_phase) {
        const float2 psi = dw_phase_mod2pi(d, a.c_dt);
        const float2 ph0 = a.t0_zero ? make_float2(0.f, 0.f) : dw_phase_mod2pi(d, a.c_t0);
        a.pair_phase[o] = make_float4(psi.x, psi.y, ph0.x, ph0.y);
    } else {
        a.pair_omega[o] = 6.283185307179586476925 * dw_to_double(d);
    }
}

// Row norms of H's hi part (bounds of the refinement's anchored sums).
template <typename T>
__device__ void hamiltonian_row_norms(SnapSmem<T> &s, int n, int m) {
    const int ld = m + 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float acc = 0.f;
        for (int k = 0; k < n; ++k) {
            const cx<float> h = s.Hh[i * ld + k];
            acc = fmaf(h.re, h.re, fmaf(h.im, h.im, acc));
        }
        s.rn[i] = sqrtf(acc);
    }
    __syncthreads();
}

// (s, c) += b z for a double-word b and z = zh + zl: the product's high
// part summed with its rounding error (TwoSum) and every low-order term
// into c.
__device__ __forceinline__ void dw_acc_prod(float &s, float &c, float2 b, float zh, float zl) {
    const float p = __fmul_rn(b.x, zh);
    const float e = fmaf(b.x, zh, -p);
    const float t = __fadd_rn(s, p);
    const float bb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, __fadd_rn(e, fmaf(b.x, zl, b.y * zh))));
}

// v[0..3) in precision T; FP32: converted by lanes 0..2 and shared across
// the warp (one FP64 conversion per warp instead of one per thread).
template <typename T>
__device__ __forceinline__ void load_vec3(const double *v, T &x, T &y, T &z) {
    if constexpr (sizeof(T) == 8) {
        x = v[0];
        y = v[1];
        z = v[2];
    } else {
        const int lane = threadIdx.x & 31;
        const float f = lane < 3 ? (float)v[lane] : 0.f;
        x = __shfl_sync(0xffffffffu, f, 0);
        y = __shfl_sync(0xffffffffu, f, 1);
        z = __shfl_sync(0xffffffffu, f, 2);
    }
}

// b[0..3) as double-words, computed by lanes 0..2 of the warp and shared.
__device__ __forceinline__ void field_dw(const double *b, float2 &bx, float2 &by, float2 &bz) {
    const int lane = threadIdx.x & 31;
    const float2 v = lane < 3 ? dw_of(b[lane]) : make_float2(0.f, 0.f);
    bx = make_float2(__shfl_sync(0xffffffffu, v.x, 0), __shfl_sync(0xffffffffu, v.y, 0));
    by = make_float2(__shfl_sync(0xffffffffu, v.x, 1), __shfl_sync(0xffffffffu, v.y, 1));
    bz = make_float2(__shfl_sync(0xffffffffu, v.x, 2), __shfl_sync(0xffffffffu, v.y, 2));
}

// H = Hsys + b . Z into the Jacobi buffer (precision T, padded to m); in
// MIXED mode also its split H = Hh + Hl into two FP32 matrices.  MIXED
// with Hdw / Zdw (Hsys and Z pre-split into double-words, (re_hi, im_hi,
// re_lo, im_lo) per entry) assembles in double-word FP32 (~2^-47 relative),
// otherwise in FP64 (split exactly).  blockDim.x is a multiple of 32.
template <typename T, bool REFINE, bool PRE = false>
__device__ void load_hamiltonian(const cx<double> *Hsys, const cx<double> *Z, const float4 *Hdw,
                                 const float4 *Zdw, const double *b, int n, int m,
                                 SnapSmem<T> &s) {
    const int tid = threadIdx.x, nt = blockDim.x, ld = m + 1, ldh = jacobi_ldh(m);
    const size_t nn = (size_t)n * n;
    if (REFINE && Hdw != nullptr) {
        float2 bx, by, bz;
        field_dw(b, bx, by, bz);
        for (int e = tid; e < m * m; e += nt) {
            const int i = FastDiv(m).div(e), j = e - i * m;
            float2 hr = make_float2(0.f, 0.f), hi = hr;
            if (i < n && j < n) {
                const size_t o = (size_t)i * n + j;
                const float4 hs = Hdw[o], z0 = Zdw[o], z1 = Zdw[nn + o], z2 = Zdw[2 * nn + o];
                float sr = hs.x, cr = hs.z, si = hs.y, ci = hs.w;
                dw_acc_prod(sr, cr, bx, z0.x, z0.z);
                dw_acc_prod(si, ci, bx, z0.y, z0.w);
                dw_acc_prod(sr, cr, by, z1.x, z1.z);
                dw_acc_prod(si, ci, by, z1.y, z1.w);
                dw_acc_prod(sr, cr, bz, z2.x, z2.z);
                dw_acc_prod(si, ci, bz, z2.y, z2.w);
                hr = dw_two_sum(sr, cr);
                hi = dw_two_sum(si, ci);
            }
            if (!PRE) s.w.H[i * ldh + j] = mk<T>((T)hr.x, (T)hi.x);
            s.Hh[i * ld + j] = mk<float>(hr.x, hi.x);
            s.Hl[i * ld + j] = mk<float>(hr.y, hi.y);
        }
    } else {
        const double bx = b[0], by = b[1], bz = b[2];
        for (int e = tid; e < m * m; e += nt) {
            const int i = FastDiv(m).div(e), j = e - i * m;
            cx<double> h = mk<double>(0.0, 0.0);
            if (i < n && j < n) {
                const size_t o = (size_t)i * n + j;
                const cx<double> hs = Hsys[o], z0 = Z[o], z1 = Z[nn + o], z2 = Z[2 * nn + o];
                h.re = hs.re + bx * z0.re + by * z1.re + bz * z2.re;
                h.im = hs.im + bx * z0.im + by * z1.im + bz * z2.im;
            }
            if (!PRE) s.w.H[i * ldh + j] = mk<T>((T)h.re, (T)h.im);
            if (REFINE) {
                const float hr = (float)h.re, hi = (float)h.im;
                s.Hh[i * ld + j] = mk<float>(hr, hi);
                s.Hl[i * ld + j] =
                    mk<float>((float)(h.re - (double)hr), (float)(h.im - (double)hi));
            }
        }
    }
    __syncthreads();
    if (REFINE) hamiltonian_row_norms(s, n, m);
}

// The eigensolve of a snapshot: FP64 or FP32 Jacobi in this CTA, or (PRE)
// the FP32 eigenvectors the warp Jacobi stage left in a.evec, with the
// status it wrote.  Leaves the eigenvectors in s.w.U (row stride m + 1).
template <typename T, bool PRE>
__device__ __forceinline__ int snap_eigvecs(const SnapArgs &a, int sn, int g, int n, int m,
                                            SnapSmem<T> &s) {
    if (!PRE) return jacobi_sweeps<T>(s.w, m, a.max_sweeps);
    const float2 *X = reinterpret_cast<const float2 *>(a.evec) + (size_t)sn * n * n;
    const int ld = m + 1;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = FastDiv(n).div(e), j = e - i * n;
        const float2 x = X[e];
        s.w.U[i * ld + j] = mk<T>((T)x.x, (T)x.y);
    }
    const int st = a.status[g];
    __syncthreads();
    return st;
}

// One Ogita-Aishima refinement step of the FP32 eigenvector matrix X
// (columns) against H = Hh + Hl (Ogita & Aishima, Japan J. Indust. Appl.
// Math. 35 (2018) 1007, Algorithm 1, Hermitian form):
//   R = I - X^H X,  S = X^H H X,  l_i = S_ii / (1 - R_ii),
//   E_ij = (S_ij + l_j R_ij) / (l_j - l_i)  (i != j),
//   E_ii = R_ii / 2,   X <- X + X E,
// with eigenvalues l_i plus the second-order term
// sum_j |S_ij + l_i R_ij|^2 / (l_i - l_j).  H X, X^H H X and X^H X use
// double-word FP32 accumulation and l_i is a double-word (S_ii over
// 1 - R_ii = 1 + g_i as S_ii - S_ii g_i / (1 + g_i)); E, the second-order
// terms and X E are FP32 (they are small corrections).  No FP64.
// Levels too close for the first-order E (near-degenerate clusters, e.g.
// at level anticrossings, and exactly degenerate multiplets) are resolved
// as clusters (msp_cluster.cuh).  Returns this step's largest correction.
// NN > 0: n = NN at compile time (the product loops unroll with constant
// shared-memory offsets); NN = 0: n from the argument.
template <int NN>
__device__ float oa_refine(SnapSmem<float> &s, int n_rt, int m_rt) {
    const int n = NN > 0 ? NN : n_rt, m = NN > 0 ? NN + (NN & 1) : m_rt;
    const int tid = threadIdx.x, nt = blockDim.x, ld = m + 1;
    cx<float> *X = s.w.U;
    cx<float> *Yh = s.w.H;  // Jacobi work matrix is free now
    if (tid < 4) s.scal[tid] = 0;  // [0]: amax, [1]: max|l|, [2]: step (float bits)
    // anchored double-word products (msp_dw.cuh): column norms of X bound
    // every partial sum
    for (int j = tid; j < n; j += nt) {
        float acc = 0.f;
        #pragma unroll

        for (int k = 0; k < n; ++k) acc = fmaf(X[k * ld + j].re, X[k * ld + j].re,
                                               fmaf(X[k * ld + j].im, X[k * ld + j].im, acc));
        s.cn[j] = sqrtf(acc);
    }
    __syncthreads();
    // Y = H X (H as hi + lo)
    for (int e = tid; e < n * n; e += nt) {
        const int i = FastDiv(n).div(e), j = e - i * n;
        const u64 K = lm_anchor(s.rn[i] * s.cn[j]);
        u64 s1 = K, s2 = K, c1 = 0ull, c2 = 0ull;
        const u64 *hh = reinterpret_cast<const u64 *>(s.Hh + i * ld);
        const u64 *hl = reinterpret_cast<const u64 *>(s.Hl + i * ld);
        #pragma unroll

        for (int k = 0; k < n; ++k) {
            const cx<float> x = X[k * ld + j];
            lm_step<true, false>(s1, c1, s2, c2, hh[k], hl[k], f32x2(x.re, x.re),
                                 f32x2(x.im, x.im), 0ull, 0ull);
        }
        const float4 r = lm_dw<false>(s1, c1, s2, c2, K);
        Yh[i * ld + j] = mk<float>(r.x, r.y);
        s.Yl[i * ld + j] = mk<float>(r.z, r.w);
    }
    __syncthreads();
    for (int j = tid; j < n; j += nt) {
        float acc = 0.f;
        #pragma unroll

        for (int k = 0; k < n; ++k) acc = fmaf(Yh[k * ld + j].re, Yh[k * ld + j].re,
                                               fmaf(Yh[k * ld + j].im, Yh[k * ld + j].im, acc));
        s.yn[j] = sqrtf(acc);
    }
    __syncthreads();
    // S_ij = X_i^H Y_j (i <= j) into SR upper triangle / sd; R_ij = -X_i^H X_j
    // (i < j) into SR lower triangle at (j, i); R_ii into rd
    const int ntri = n * (n + 1) / 2;
    for (int e = tid; e < ntri; e += nt) {
        int j, i;
        tri_index(e, j, i);  // j >= i
        const u64 KS = lm_anchor(s.cn[i] * s.yn[j]), KG = lm_anchor(s.cn[i] * s.cn[j]);
        u64 a1 = KS, a2 = KS, ac1 = 0ull, ac2 = 0ull;
        u64 g1 = KG, g2 = KG, gc1 = 0ull, gc2 = 0ull;
        #pragma unroll

        for (int k = 0; k < n; ++k) {
            const u64 xi = *reinterpret_cast<const u64 *>(X + k * ld + i);
            const cx<float> y = Yh[k * ld + j], yl = s.Yl[k * ld + j], xj = X[k * ld + j];
            lm_step<false, true>(a1, ac1, a2, ac2, xi, 0ull, f32x2(y.re, y.re), f32x2(y.im, y.im),
                                 f32x2(yl.re, yl.re), f32x2(yl.im, yl.im));
            lm_step<false, false>(g1, gc1, g2, gc2, xi, 0ull, f32x2(xj.re, xj.re),
                                  f32x2(xj.im, xj.im), 0ull, 0ull);
        }
        const float4 S = lm_dw<true>(a1, ac1, a2, ac2, KS);
        const float4 G = lm_dw<true>(g1, gc1, g2, gc2, KG);
        if (i == j) {
            s.gd[i] = make_float2(G.x - 1.0f, G.z);  // G_ii - 1 (G.x - 1 exact)
            s.lw[i] = make_float2(S.x, S.z);         // S_ii until l_i replaces it
        } else {
            s.SR[i * ld + j] = mk<float>(S.x + S.z, S.y + S.w);
            s.SR[j * ld + i] = mk<float>(-(G.x + G.z), -(G.y + G.w));  // R_ij = -G_ij
        }
    }
    __syncthreads();
    float lmax = 0.f;
    for (int i = tid; i < n; i += nt) {
        const float2 lw = dw_rayleigh(s.lw[i], s.gd[i]);
        const float l = lw.x;
        s.lw[i] = lw;
        s.lamf[i] = l;
        s.corr[i] = 0.f;
        lmax = fmaxf(lmax, fabsf(l));
    }
    atomicMax(&s.scal[1], __float_as_int(lmax));  // non-negative: int order = float order
    __syncthreads();
    // clusters; T in Yl (free now)
    OaCluster cl;
    cl.rank = s.rk;
    cl.order = s.ord;
    cl.cstart = s.cst;
    cl.scal = s.scal;
    cl.T = s.Yl;
    cl.ldt = ld;
    oa_clusters(s.SR, ld, s.lw, s.lamf, n, cl);
    float emax = 0.f;
    const int nup = n * (n - 1) / 2;
    for (int e = tid; e < nup; e += nt) {
        int i, j;
        oa_pair_of(e, i, j);
        oa_pair_correction(s.SR, ld, s.lw, s.lamf, cl, s.corr, i, j, emax);
    }
    __syncthreads();
    oa_cluster_diagonal(s.lw, s.corr, n, cl);
    // X' = X + X E  (into Yh), E_ii = R_ii / 2
    for (int e = tid; e < n * n; e += nt) {
        const int k = FastDiv(n).div(e), j = e - k * n;
        const cx<float> xkj = X[k * ld + j];
        const float hr = -0.5f * (s.gd[j].x + s.gd[j].y);  // R_jj / 2
        float ar = xkj.re + hr * xkj.re, ai = xkj.im + hr * xkj.im;
        #pragma unroll

        for (int i = 0; i < n; ++i) {
            if (i == j) continue;
            const cx<float> x = X[k * ld + i], E = s.SR[i * ld + j];
            ar = fmaf(x.re, E.re, fmaf(-x.im, E.im, ar));
            ai = fmaf(x.re, E.im, fmaf(x.im, E.re, ai));
        }
        Yh[k * ld + j] = mk<float>(ar, ai);
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {
        const int k = FastDiv(n).div(e), j = e - k * n;
        X[k * ld + j] = Yh[k * ld + j];
    }
    __syncthreads();
    emax = fmaxf(emax, oa_resolve_clusters(X, ld, n, s.lw, s.corr, n, cl,
                                           __int_as_float(s.scal[1])));
    atomicMax(&s.scal[2], __float_as_int(emax));  // non-negative: int order = float order
    __syncthreads();
    const float step = __int_as_float(s.scal[2]);
    __syncthreads();
    return step;
}

// Eigenvalues: the Jacobi diagonal into lam[0..n) (FP64), or the refined
// double-words into lw[0..n) (MIXED; also refines the eigenvectors in
// place).
// Returns status bits (MSP_ITEM_REFINE_LIMIT when the refinement ran out of
// steps).
template <typename T, bool REFINE>
__device__ int eigenpairs(SnapSmem<T> &s, int n, int m, int max_refine);

template <>
__device__ int eigenpairs<double, false>(SnapSmem<double> &s, int n, int m, int) {
    for (int j = threadIdx.x; j < n; j += blockDim.x) s.lam[j] = s.w.diag[j];
    __syncthreads();
    return MSP_ITEM_OK;
}

// One refinement step leaves an error of order E^2; a step whose largest
// correction exceeds 2e-4 (clusters resolved by large rotations, levels
// within ~1e3 FP32 resolutions) is followed by another, at most max_refine
// in all; a last step still above 2e-4 sets MSP_ITEM_REFINE_LIMIT.
template <>
__device__ int eigenpairs<float, true>(SnapSmem<float> &s, int n, int m, int max_refine) {
    if (max_refine <= 0) max_refine = 4;
    for (int it = 0; it < max_refine; ++it) {
        const float step = n == 24   ? oa_refine<24>(s, n, m)
                           : n == 32 ? oa_refine<32>(s, n, m)
                                     : oa_refine<0>(s, n, m);
        if (step <= 2e-4f) return MSP_ITEM_OK;
    }
    return MSP_ITEM_REFINE_LIMIT;
}

// ------------------------------------------------------------------ eigh

template <typename T, bool REFINE>
__global__ void msp_eigh_kernel(const cx<double> *__restrict__ Hin, int n, int batch,
                                int max_sweeps, double *__restrict__ evals,
                                cx<double> *__restrict__ evecs, int *__restrict__ status) {
    extern __shared__ __align__(16) char smem[];
    const int m = n + (n & 1), ld = m + 1, ldh = jacobi_ldh(m);
    SnapSmem<T> s = snap_carve<T, REFINE>(smem, n, false, 0);
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int bidx = blockIdx.x; bidx < batch; bidx += gridDim.x) {
        const cx<double> *Hb = Hin + (size_t)bidx * n * n;
        for (int e = tid; e < m * m; e += nt) {
            const int i = FastDiv(m).div(e), j = e - i * m;
            cx<double> h = mk<double>(0.0, 0.0);
            if (i < n && j < n) h = Hb[(size_t)i * n + j];
            s.w.H[i * ldh + j] = mk<T>((T)h.re, (T)h.im);
            if (REFINE) {
                const float hr = (float)h.re, hi = (float)h.im;
                s.Hh[i * ld + j] = mk<float>(hr, hi);
                s.Hl[i * ld + j] = mk<float>((float)(h.re - (double)hr), (float)(h.im - (double)hi));
            }
        }
        __syncthreads();
        if (REFINE) hamiltonian_row_norms(s, n, m);
        int st = jacobi_sweeps<T>(s.w, m, max_sweeps);
        st |= eigenpairs<T, REFINE>(s, n, m, 4);
        // ascending order, ties by index (stable)
        for (int j = tid; j < n; j += nt) {
            int r = 0;
            if constexpr (REFINE) {
                const float2 lj = s.lw[j];
                for (int k = 0; k < n; ++k) {
                    const float2 lk = s.lw[k];
                    r += dw_less(lk, lj) || (dw_equal(lk, lj) && k < j);
                }
                evals[(size_t)bidx * n + r] = dw_to_double(lj);
            } else {
                const double lj = s.lam[j];
                for (int k = 0; k < n; ++k) {
                    const double lk = s.lam[k];
                    r += (lk < lj) || (lk == lj && k < j);
                }
                evals[(size_t)bidx * n + r] = lj;
            }
            s.rank[j] = r;
        }
        __syncthreads();
        cx<double> *Vb = evecs + (size_t)bidx * n * n;
        for (int e = tid; e < n * n; e += nt) {
            const int i = FastDiv(n).div(e), j = e - i * n;
            const cx<T> u = s.w.U[i * ld + j];
            Vb[(size_t)i * n + s.rank[j]] = mk<double>((double)u.re, (double)u.im);
        }
        if (tid == 0) status[bidx] = st;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ fast path

// Mixed fast path: A_jk = |(U^H M)_jk|^2 over the lower triangle j >= k
// (FP32), pair records for j > k, and this thread's share of sum_j A_jj as
// a double-word.  NN > 0: n = NN at compile time.
template <int NN>
__device__ __forceinline__ float2 amplitudes_mixed(const SnapArgs &a, const SnapSmem<float> &s,
                                                   const cx<float> *U, const cx<float> *M,
                                                   int n_rt, int sn, float scale) {
    const int n = NN > 0 ? NN : n_rt, ld = n + (n & 1) + 1;
    const int P = n * (n - 1) / 2, ntri = n * (n + 1) / 2;
    float2 diag = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < ntri; e += blockDim.x) {
        int j, k;
        tri_index(e, j, k);
        float gr = 0.f, gi = 0.f;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const cx<float> u = U[i * ld + j], mm = M[i * ld + k];
            gr += u.re * mm.re + u.im * mm.im;
            gi += u.re * mm.im - u.im * mm.re;
        }
        const float A = gr * gr + gi * gi;
        if (j == k) {
            diag = dw_add_f(diag, A);
        } else {
            const size_t o = (size_t)sn * P + pair_index(j, k);
            reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2(scale * A, 0.f);
            store_frequency_dw(a, o, dw_sub(s.lw[j], s.lw[k]));
        }
    }
    return diag;
}

// One snapshot of the muon-first T = inf shortcut (muspinsim/hamiltonian.py:
// 166-217): A = |U^dag (sigma_p (x) 1_d) U|^2 and omega_jk = 2 pi (l_j - l_k)
// for j > k, scaled by 0.5 * w / (d * N_avg), plus the constant
// 0.5 * sum_j A_jj part.
// MIXED: at most 64 registers (no spills; ptxas would take ~88 and fit
// 5 instead of 7-8 CTAs of 128 threads per SM).
template <typename T, bool REFINE, bool PRE = false>
__global__ void __maxnreg__(REFINE ? 64 : 255) msp_snap_fast_kernel(SnapArgs a) {
    extern __shared__ __align__(16) char smem[];
    const int n = a.n, m = n + (n & 1), ld = m + 1, d = n / 2;
    SnapSmem<T> s = snap_carve<T, REFINE>(smem, n, false, 0);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int P = n * (n - 1) / 2;
    typedef typename PairCoef<T>::type coef_t;
    coef_t *coef = reinterpret_cast<coef_t *>(a.pair_coef);

    for (int sn = blockIdx.x; sn < a.num_snap; sn += gridDim.x) {
        const SnapSource src = snap_source(a, sn);
        const size_t g = (size_t)src.g;
        load_hamiltonian<T, REFINE, PRE>(src.Hsys, src.Z, src.Hdw, src.Zdw, a.field + 3 * g, n,
                                         m, s);
        int st = snap_eigvecs<T, PRE>(a, sn, (int)g, n, m, s);
        st |= eigenpairs<T, REFINE>(s, n, m, a.max_refine);

        // sigma_p = p . sigma (Pauli), applied on the muon (slowest) digit
        T px, py, pz;
        load_vec3<T>(a.pol + 3 * g, px, py, pz);
        const cx<T> s00 = mk<T>(pz, T(0)), s01 = mk<T>(px, -py);
        const cx<T> s10 = mk<T>(px, py), s11 = mk<T>(-pz, T(0));
        cx<T> *M = s.w.H;  // free buffer
        const cx<T> *U = s.w.U;
        for (int e = tid; e < n * n; e += nt) {
            const int i = FastDiv(n).div(e), k = e - i * n;
            cx<T> v;
            if (i < d)
                v = cadd(cmul(s00, U[i * ld + k]), cmul(s01, U[(i + d) * ld + k]));
            else
                v = cadd(cmul(s10, U[(i - d) * ld + k]), cmul(s11, U[i * ld + k]));
            M[i * ld + k] = v;
        }
        if (!REFINE && tid == 0) s.acc[0] = 0.0;
        __syncthreads();
        const int ntri = n * (n + 1) / 2;
        if constexpr (REFINE) {
            // FP32 amplitudes, double-word level gaps and diagonal sum
            const float scale = (float)a.wscale[g] * (0.5f / (float)d);
            const float2 diag = n == 24   ? amplitudes_mixed<24>(a, s, U, M, n, sn, scale)
                                : n == 32 ? amplitudes_mixed<32>(a, s, U, M, n, sn, scale)
                                          : amplitudes_mixed<0>(a, s, U, M, n, sn, scale);
            const double dsum = dw_block_sum(diag, reinterpret_cast<float2 *>(s.w.red));
            if (tid == 0) {
                a.snap_const[sn] = 0.25 * a.wscale[g] * dsum / (double)d;
                a.status[g] = st;
            }
        } else {
            const double scale = 0.5 * a.wscale[g] / (double)d;
            double diag_local = 0.0;
            for (int e = tid; e < ntri; e += nt) {
                int j, k;
                tri_index(e, j, k);
                T gr = 0, gi = 0;
                for (int i = 0; i < n; ++i) {
                    const cx<T> u = U[i * ld + j], mm = M[i * ld + k];
                    gr += u.re * mm.re + u.im * mm.im;
                    gi += u.re * mm.im - u.im * mm.re;
                }
                const double A = (double)(gr * gr + gi * gi);
                if (j == k) {
                    diag_local += A;
                } else {
                    const size_t o = (size_t)sn * P + pair_index(j, k);
                    coef[o] = PairCoef<T>::make(scale * A, 0.0);
                    store_frequency(a, o, 6.283185307179586476925 * (s.lam[j] - s.lam[k]));
                }
            }
            atomicAdd(&s.acc[0], diag_local);
            __syncthreads();
            if (tid == 0) {
                a.snap_const[sn] = scale * 0.5 * s.acc[0];
                a.status[g] = st;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ general path

// Applies the single-spin matrix F (dim x dim, complex FP64 or FP32) on
// digit `stride` of the row index of X (n x n, leading dim m) into Y:
// Y = (1 (x) F (x) 1) X.
template <typename T, typename TF>
__device__ void apply_digit(const cx<TF> *F, int dim, int stride, const cx<T> *X, cx<T> *Y, int n,
                            int m) {
    const int ld = m + 1;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = FastDiv(n).div(e), k = e - i * n;
        const int di = (i / stride) % dim;
        const int base = i - di * stride;
        T yr = 0, yi = 0;
        for (int l = 0; l < dim; ++l) {
            const cx<TF> f = F[di * dim + l];
            const cx<T> x = X[(base + l * stride) * ld + k];
            yr += (T)f.re * x.re - (T)f.im * x.im;
            yi += (T)f.re * x.im + (T)f.im * x.re;
        }
        Y[i * ld + k] = mk<T>(yr, yi);
    }
    __syncthreads();
}

// Y[j][k] = sum_i conj(U_ij) X_ik for j >= k (row stride ld = n + (n & 1) + 1);
// NN > 0: n = NN at compile time.
template <typename T, int NN>
__device__ __forceinline__ void tri_conj_products(const cx<T> *U, const cx<T> *X, cx<T> *Y,
                                                  int n_rt) {
    const int n = NN > 0 ? NN : n_rt, ld = n + (n & 1) + 1, ntri = n * (n + 1) / 2;
    for (int e = threadIdx.x; e < ntri; e += blockDim.x) {
        int j, k;
        tri_index(e, j, k);
        T gr = 0, gi = 0;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const cx<T> u = U[i * ld + j], x = X[i * ld + k];
            gr += u.re * x.re + u.im * x.im;
            gi += u.re * x.im - u.im * x.re;
        }
        Y[j * ld + k] = mk<T>(gr, gi);
    }
}

// Mixed general path: every term C_jk = rho'_jk O'_kj (j >= k, O'_kj =
// sum_i conj(U_ik) (O U)_ij): pair records (EVOLVE) or the decaying-integral
// terms (INTEGRAL); returns this thread's share of the constant / integral
// as a double-word.  NN > 0: n = NN at compile time.
template <bool INTEGRAL, int NN>
__device__ __forceinline__ float2 rho_terms_mixed(const SnapArgs &a, const SnapSmem<float> &s,
                                                  const cx<float> *U, const cx<float> *OU,
                                                  const cx<float> *Y, int n_rt, int sn,
                                                  float tau_f, float itau_f) {
    const int n = NN > 0 ? NN : n_rt, ld = n + (n & 1) + 1;
    const int P = n * (n - 1) / 2, ntri = n * (n + 1) / 2;
    const float scale2 = 2.0f * (float)a.wscale[sn];
    float2 local = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < ntri; e += blockDim.x) {
        int j, k;
        tri_index(e, j, k);
        float orr = 0.f, oii = 0.f;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const cx<float> u = U[i * ld + k], x = OU[i * ld + j];
            orr += u.re * x.re + u.im * x.im;
            oii += u.re * x.im - u.im * x.re;
        }
        const cx<float> r = Y[j * ld + k];
        const float cr = r.re * orr - r.im * oii;
        const float ci = r.re * oii + r.im * orr;
        if (INTEGRAL) {
            // term = C_jk (-1) / (2 pi i (l_k - l_j) - 1/tau); pairs count twice
            if (j == k) {
                local = dw_add_f(local, cr * tau_f);
            } else {
                const float gap = dw_sub_f(s.lw[k], s.lw[j]);
                const float x = fmaf(gap, MSP_TWOPI_HI, gap * MSP_TWOPI_LO);
                const float den = fmaf(x, x, itau_f * itau_f);
                local = dw_add_f(local, 2.0f * (cr * itau_f - ci * x) / den);
            }
        } else {
            if (j == k) {
                local = dw_add_f(local, cr);
            } else {
                const size_t o = (size_t)sn * P + pair_index(j, k);
                reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2(scale2 * cr, scale2 * ci);
                store_frequency_dw(a, o, dw_sub(s.lw[j], s.lw[k]));
            }
        }
    }
    return local;
}

// One snapshot of the general path: rho' = U^dag rho0 U, O' = U^dag O U with
// rho0 = (x)_s rho_s (Kronecker factors) and O = p . S_mu.  EVOLVE writes the
// pair coefficients of <O>(t) = sum_ij rho'_ij O'_ji exp(-i w_ij t)
// (muspinsim/hamiltonian.py:80-107); INTEGRAL writes the decaying integral
// divided by tau (muspinsim/hamiltonian.py:150-164, experiment.py:492-496).
// MIXED: at most 96 registers (shared memory limits these CTAs to ~4 per SM
// at n = 32 anyway).
template <typename T, bool REFINE, bool INTEGRAL, bool PRE = false>
__global__ void __maxnreg__(REFINE ? 96 : 255) msp_snap_rho_kernel(SnapArgs a) {
    extern __shared__ __align__(16) char smem[];
    const int n = a.n, m = n + (n & 1), ld = m + 1;
    SnapSmem<T> s = snap_carve<T, REFINE>(smem, n, true, a.fac_len);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int P = n * (n - 1) / 2;
    typedef typename PairCoef<T>::type coef_t;
    coef_t *coef = reinterpret_cast<coef_t *>(a.pair_coef);
    const double twopi = 6.283185307179586476925;
    // MIXED constants (FP32)
    const float tau_f = INTEGRAL ? (float)a.tau : 0.f;
    const float itau_f = INTEGRAL ? (float)(1.0 / a.tau) : 0.f;

    for (int sn = blockIdx.x; sn < a.num_snap; sn += gridDim.x) {
        if (a.rho_fac) {
            for (int e = tid; e < a.fac_len; e += nt)
                s.fac[e] = a.rho_fac[(size_t)sn * a.fac_len + e];
        } else {
            build_rho_factors(a, sn, s.fac);
        }
        load_hamiltonian<T, REFINE, PRE>(a.Hsys, a.Z, a.Hsys_dw, a.Z_dw, a.field + 3 * (size_t)sn,
                                         n, m, s);
        if (REFINE)  // made visible by the eigensolve's barriers
            for (int e = tid; e < a.fac_len; e += nt)
                s.facf[e] = mk<float>((float)s.fac[e].re, (float)s.fac[e].im);
        int st = snap_eigvecs<T, PRE>(a, sn, sn, n, m, s);
        st |= eigenpairs<T, REFINE>(s, n, m, a.max_refine);
        const cx<T> *U = s.w.U;

        // T1 = rho0 U by Kronecker factors: X ping-pongs between H and B2
        const cx<T> *X = U;
        cx<T> *Y = s.w.H;
        {
            int off = 0;
            for (int sp = 0; sp < a.num_spins; ++sp) {
                const int dim = a.dims[sp];
                if constexpr (REFINE)
                    apply_digit<T>(s.facf + off, dim, a.strides[sp], X, Y, n, m);
                else
                    apply_digit<T>(s.fac + off, dim, a.strides[sp], X, Y, n, m);
                off += dim * dim;
                X = Y;
                Y = (Y == s.w.H) ? s.B2 : s.w.H;
            }
        }
        // X holds rho0 U.  rho'_jk (j >= k) -> Y (the other buffer).
        const int ntri = n * (n + 1) / 2;
        if (REFINE && n == 24)
            tri_conj_products<T, 24>(U, X, Y, n);
        else if (REFINE && n == 32)
            tri_conj_products<T, 32>(U, X, Y, n);
        else
            tri_conj_products<T, 0>(U, X, Y, n);
        __syncthreads();
        // O U into the buffer X (free now): O = sum_a p_a S^a on the muon digit
        cx<T> *OU = const_cast<cx<T> *>(X);
        {
            T px, py, pz;
            load_vec3<T>(a.pol + 3 * (size_t)sn, px, py, pz);
            const T h = T(0.5);
            const int stride = a.strides[a.mu_index];
            const cx<T> o00 = mk<T>(h * pz, T(0));
            const cx<T> o01 = mk<T>(h * px, -h * py);
            const cx<T> o10 = mk<T>(h * px, h * py);
            const cx<T> o11 = mk<T>(-h * pz, T(0));
            for (int e = tid; e < n * n; e += nt) {
                const int i = FastDiv(n).div(e), k = e - i * n;
                const int di = (i / stride) & 1;
                const int base = i - di * stride;
                const cx<T> x0 = U[base * ld + k], x1 = U[(base + stride) * ld + k];
                OU[i * ld + k] = di == 0 ? cadd(cmul(o00, x0), cmul(o01, x1))
                                        : cadd(cmul(o10, x0), cmul(o11, x1));
            }
        }
        if (!REFINE && tid == 0) s.acc[0] = 0.0;
        __syncthreads();
        if constexpr (REFINE) {
            // FP32 terms, double-word level gaps and sums
            const float2 local =
                n == 24   ? rho_terms_mixed<INTEGRAL, 24>(a, s, U, OU, Y, n, sn, tau_f, itau_f)
                : n == 32 ? rho_terms_mixed<INTEGRAL, 32>(a, s, U, OU, Y, n, sn, tau_f, itau_f)
                          : rho_terms_mixed<INTEGRAL, 0>(a, s, U, OU, Y, n, sn, tau_f, itau_f);
            const double sum = dw_block_sum(local, reinterpret_cast<float2 *>(s.w.red));
            if (tid == 0) {
                a.snap_const[sn] = INTEGRAL ? a.wscale[sn] * sum / a.tau : a.wscale[sn] * sum;
                a.status[sn] = st;
            }
        } else {
            const double scale = a.wscale[sn];
            double local = 0.0;
            for (int e = tid; e < ntri; e += nt) {
                int j, k;
                tri_index(e, j, k);
                // O'_kj = sum_i conj(U_ik) (O U)_ij
                T orr = 0, oii = 0;
                for (int i = 0; i < n; ++i) {
                    const cx<T> u = U[i * ld + k], x = OU[i * ld + j];
                    orr += u.re * x.re + u.im * x.im;
                    oii += u.re * x.im - u.im * x.re;
                }
                const cx<T> r = Y[j * ld + k];
                // C_jk = rho'_jk O'_kj
                const double cr = (double)r.re * (double)orr - (double)r.im * (double)oii;
                const double ci = (double)r.re * (double)oii + (double)r.im * (double)orr;
                if (INTEGRAL) {
                    // term = C_jk * (-1) / (2 pi i (l_k - l_j) - 1/tau); pairs count twice
                    const double inv_tau = 1.0 / a.tau;
                    if (j == k) {
                        local += cr * a.tau;
                    } else {
                        const double x = twopi * (s.lam[k] - s.lam[j]);
                        // -C / (-1/tau + i x) = C (1/tau + i x) / (1/tau^2 + x^2)
                        const double den = inv_tau * inv_tau + x * x;
                        local += 2.0 * (cr * inv_tau - ci * x) / den;
                    }
                } else {
                    if (j == k) {
                        local += cr;
                    } else {
                        const size_t o = (size_t)sn * P + pair_index(j, k);
                        coef[o] = PairCoef<T>::make(2.0 * scale * cr, 2.0 * scale * ci);
                        store_frequency(a, o, twopi * (s.lam[j] - s.lam[k]));
                    }
                }
            }
            atomicAdd(&s.acc[0], local);
            __syncthreads();
            if (tid == 0) {
                a.snap_const[sn] = INTEGRAL ? scale * s.acc[0] / a.tau : scale * s.acc[0];
                a.status[sn] = st;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ launchers

int snap_default_threads(int n) { return jacobi_threads(n + (n & 1)); }

// Shared memory of a snapshot kernel launched with `threads` threads (the
// reduction scratch grows with the warp count).
static size_t snap_smem_threads(int n, int mode, int precision, int fac_len, int threads) {
    const bool mixed = precision == MSP_PREC_MIXED;
    return snap_layout(n, mixed ? 4 : 8, mixed, mode != MSP_MODE_FAST, fac_len, threads / 32)
        .total;
}

template <typename K>
static cudaError_t launch_snap(K kernel, const SnapArgs &a, int grid, int threads, size_t smem,
                               cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    kernel<<<grid, threads, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename K>
static int occupancy_of(K kernel, int threads, size_t smem) {
    int blocks = 0;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, smem) !=
            cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return blocks > 0 ? blocks : 1;
}

int snap_occupancy(int n, int mode, int precision, int threads) {
    if (threads <= 0) threads = snap_default_threads(n);
    const size_t smem = snap_smem_threads(n, mode, precision, 0, threads);
    const bool mixed = precision == MSP_PREC_MIXED;
    if (mode == MSP_MODE_FAST) {
        if (mixed && jacobi_warp_supported(n))
            return occupancy_of(msp_snap_fast_kernel<float, true, true>, threads, smem);
        return mixed ? occupancy_of(msp_snap_fast_kernel<float, true>, threads, smem)
                     : occupancy_of(msp_snap_fast_kernel<double, false>, threads, smem);
    }
    return 1;
}

size_t snap_evec_bytes(int n, long long num_snap, int precision) {
    if (precision != MSP_PREC_MIXED || !jacobi_warp_supported(n) || num_snap <= 0) return 0;
    return (size_t)num_snap * (size_t)n * (size_t)n * sizeof(float2);
}

// Second stage of the two-stage MIXED form: refinement and eigenbasis
// products from the eigenvectors the warp Jacobi left in a.evec.
cudaError_t launch_snapshots_refine(const SnapArgs &a, int mode, cudaStream_t st, int threads,
                                    int grid) {
    if (a.num_snap <= 0) return cudaSuccess;
    if (threads <= 0) threads = snap_default_threads(a.n);
    const size_t smem = snap_smem_threads(a.n, mode, MSP_PREC_MIXED, a.fac_len, threads);
    if (grid <= 0 || grid > a.num_snap) grid = a.num_snap;
    if (mode == MSP_MODE_FAST)
        return launch_snap(msp_snap_fast_kernel<float, true, true>, a, grid, threads, smem, st);
    if (mode == MSP_MODE_EVOLVE)
        return launch_snap(msp_snap_rho_kernel<float, true, false, true>, a, grid, threads, smem,
                           st);
    return launch_snap(msp_snap_rho_kernel<float, true, true, true>, a, grid, threads, smem, st);
}

// threads = 0: jacobi_threads(m); grid = 0: one CTA per snapshot.  Any
// other grid runs persistent CTAs that stride over the snapshots.
cudaError_t launch_snapshots(const SnapArgs &a, int mode, int precision, cudaStream_t st,
                             int threads, int grid) {
    if (a.num_snap <= 0) return cudaSuccess;
    if (threads <= 0) threads = snap_default_threads(a.n);
    const size_t smem = snap_smem_threads(a.n, mode, precision, a.fac_len, threads);
    if (grid <= 0 || grid > a.num_snap) grid = a.num_snap;
    const bool mixed = precision == MSP_PREC_MIXED;
    if (mixed && a.evec != nullptr && jacobi_warp_supported(a.n)) {
        // two stages: warp Jacobi, then refinement and eigenbasis products
        const cudaError_t e = launch_jacobi_warp(a, st);
        if (e != cudaSuccess) return e;
        return launch_snapshots_refine(a, mode, st, threads, grid);
    }
    if (mode == MSP_MODE_FAST) {
        return mixed ? launch_snap(msp_snap_fast_kernel<float, true>, a, grid, threads, smem, st)
                     : launch_snap(msp_snap_fast_kernel<double, false>, a, grid, threads, smem, st);
    } else if (mode == MSP_MODE_EVOLVE) {
        return mixed
                   ? launch_snap(msp_snap_rho_kernel<float, true, false>, a, grid, threads, smem, st)
                   : launch_snap(msp_snap_rho_kernel<double, false, false>, a, grid, threads, smem,
                                 st);
    }
    return mixed ? launch_snap(msp_snap_rho_kernel<float, true, true>, a, grid, threads, smem, st)
                 : launch_snap(msp_snap_rho_kernel<double, false, true>, a, grid, threads, smem,
                               st);
}

__global__ void msp_split_dw_kernel(const cx<double> *__restrict__ Hsys, size_t nh,
                                    const cx<double> *__restrict__ Z, size_t nz,
                                    float4 *__restrict__ dst) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nh + nz; i += stride) {
        const cx<double> v = i < nh ? Hsys[i] : Z[i - nh];
        dst[i] = dw_split(make_double2(v.re, v.im));
    }
}

cudaError_t launch_split_dw(const double *Hsys, size_t nh, const double *Z, size_t nz,
                            float4 *dst, cudaStream_t st) {
    const size_t total = nh + nz;
    if (total == 0) return cudaSuccess;
    size_t grid = (total + 255) / 256;
    if (grid > 1024) grid = 1024;
    msp_split_dw_kernel<<<(unsigned)grid, 256, 0, st>>>(
        reinterpret_cast<const cx<double> *>(Hsys), nh, reinterpret_cast<const cx<double> *>(Z),
        nz, dst);
    return cudaGetLastError();
}

cudaError_t launch_eigh(const double *H, int n, int batch, int precision, int max_sweeps,
                        double *evals, double *evecs, int *status, cudaStream_t st) {
    const int m = n + (n & 1);
    const size_t smem = snap_smem_bytes(n, MSP_MODE_FAST, precision, 0);
    const int grid = batch;
    const cx<double> *Hc = reinterpret_cast<const cx<double> *>(H);
    cx<double> *Vc = reinterpret_cast<cx<double> *>(evecs);
    cudaError_t e;
    if (precision == MSP_PREC_MIXED) {
        e = cudaFuncSetAttribute(msp_eigh_kernel<float, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        msp_eigh_kernel<float, true><<<grid, jacobi_threads(m), smem, st>>>(
            Hc, n, batch, max_sweeps, evals, Vc, status);
    } else {
        e = cudaFuncSetAttribute(msp_eigh_kernel<double, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        msp_eigh_kernel<double, false><<<grid, jacobi_threads(m), smem, st>>>(
            Hc, n, batch, max_sweeps, evals, Vc, status);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------ assemble / basis change

__global__ void msp_assemble_kernel(const cx<double> *__restrict__ Hsys,
                                    const cx<double> *__restrict__ Z,
                                    const double *__restrict__ fields, int n, int batch,
                                    cx<double> *__restrict__ H) {
    const size_t nn = (size_t)n * n;
    const size_t total = nn * batch;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t b = e / nn, o = e - b * nn;
        const double bx = fields[3 * b], by = fields[3 * b + 1], bz = fields[3 * b + 2];
        const cx<double> hs = Hsys[o], z0 = Z[o], z1 = Z[nn + o], z2 = Z[2 * nn + o];
        H[e] = mk<double>(hs.re + bx * z0.re + by * z1.re + bz * z2.re,
                          hs.im + bx * z0.im + by * z1.im + bz * z2.im);
    }
}

cudaError_t launch_assemble(const double *Hsys, const double *Z, const double *fields, int n,
                            int batch, double *H, cudaStream_t st) {
    const size_t total = (size_t)n * n * batch;
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    if (grid < 1) grid = 1;
    msp_assemble_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<const cx<double> *>(Hsys),
                                              reinterpret_cast<const cx<double> *>(Z), fields, n,
                                              batch, reinterpret_cast<cx<double> *>(H));
    return cudaGetLastError();
}

// out = U^dag M U (adjoint = 0) or U M U^dag (adjoint = 1), FP64, one CTA per
// matrix, n <= 64: U and M staged in shared memory, T = M U (or M U^dag)
// kept in shared memory, then out = U^dag T (or U T) written to global.
__global__ void msp_basis_change_kernel(const cx<double> *__restrict__ U, long long u_stride,
                                        const cx<double> *__restrict__ M, long long m_stride,
                                        int n, int batch, int adjoint,
                                        cx<double> *__restrict__ out) {
    extern __shared__ __align__(16) char smem[];
    cx<double> *sU = reinterpret_cast<cx<double> *>(smem);
    cx<double> *sM = sU + n * n;
    cx<double> *sT = sM + n * n;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int b = blockIdx.x; b < batch; b += gridDim.x) {
        const cx<double> *Ub = U + (size_t)b * u_stride;
        const cx<double> *Mb = M + (size_t)b * m_stride;
        for (int e = tid; e < n * n; e += nt) {
            sU[e] = Ub[e];
            sM[e] = Mb[e];
        }
        __syncthreads();
        for (int e = tid; e < n * n; e += nt) {
            const int i = FastDiv(n).div(e), k = e - i * n;
            double tr = 0, ti = 0;
            for (int l = 0; l < n; ++l) {
                const cx<double> mv = sM[i * n + l];
                // adjoint: (U^dag)_lk = conj(U_kl)
                const cx<double> uv = adjoint ? conj(sU[k * n + l]) : sU[l * n + k];
                tr += mv.re * uv.re - mv.im * uv.im;
                ti += mv.re * uv.im + mv.im * uv.re;
            }
            sT[e] = mk<double>(tr, ti);
        }
        __syncthreads();
        cx<double> *Ob = out + (size_t)b * n * n;
        for (int e = tid; e < n * n; e += nt) {
            const int j = FastDiv(n).div(e), k = e - j * n;
            double tr = 0, ti = 0;
            for (int i = 0; i < n; ++i) {
                // row j of U^dag = conj(U_ij); row j of U = U_ji
                const cx<double> uv = adjoint ? sU[j * n + i] : conj(sU[i * n + j]);
                const cx<double> tv = sT[i * n + k];
                tr += uv.re * tv.re - uv.im * tv.im;
                ti += uv.re * tv.im + uv.im * tv.re;
            }
            Ob[e] = mk<double>(tr, ti);
        }
        __syncthreads();
    }
}

// n > 64: the same product from global memory in two launches, one CTA
// per (column j, matrix): T = M op(U) into out (op(U) = U, or U^dag when
// adjoint), then out = op'(U) T (op'(U) = U^dag, or U).  Each CTA first
// stages its column (of op(U), then of T) in shared memory, so the second
// pass overwrites column j in place.
__global__ void msp_basis_change_col1_kernel(const cx<double> *__restrict__ U, long long u_stride,
                                             const cx<double> *__restrict__ M, long long m_stride,
                                             int n, int adjoint, int b0,
                                             cx<double> *__restrict__ out) {
    extern __shared__ __align__(16) char smem[];
    cx<double> *col = reinterpret_cast<cx<double> *>(smem);
    const int j = blockIdx.x, b = b0 + blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
    const cx<double> *Ub = U + (size_t)b * u_stride;
    const cx<double> *Mb = M + (size_t)b * m_stride;
    cx<double> *Ob = out + (size_t)b * n * n;
    for (int l = tid; l < n; l += nt)
        col[l] = adjoint ? conj(Ub[(size_t)j * n + l]) : Ub[(size_t)l * n + j];
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        const cx<double> *row = Mb + (size_t)i * n;
        double tr = 0, ti = 0;
        for (int l = 0; l < n; ++l) {
            const cx<double> mv = row[l], uv = col[l];
            tr += mv.re * uv.re - mv.im * uv.im;
            ti += mv.re * uv.im + mv.im * uv.re;
        }
        Ob[(size_t)i * n + j] = mk<double>(tr, ti);
    }
}

__global__ void msp_basis_change_col2_kernel(const cx<double> *__restrict__ U, long long u_stride,
                                             int n, int adjoint, int b0,
                                             cx<double> *__restrict__ out) {
    extern __shared__ __align__(16) char smem[];
    cx<double> *col = reinterpret_cast<cx<double> *>(smem);
    const int j = blockIdx.x, b = b0 + blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
    const cx<double> *Ub = U + (size_t)b * u_stride;
    cx<double> *Ob = out + (size_t)b * n * n;
    for (int k = tid; k < n; k += nt) col[k] = Ob[(size_t)k * n + j];
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        double tr = 0, ti = 0;
        for (int k = 0; k < n; ++k) {
            // row i of U^dag = conj(U_ki); row i of U = U_ik
            const cx<double> uv = adjoint ? Ub[(size_t)i * n + k] : conj(Ub[(size_t)k * n + i]);
            const cx<double> tv = col[k];
            tr += uv.re * tv.re - uv.im * tv.im;
            ti += uv.re * tv.im + uv.im * tv.re;
        }
        Ob[(size_t)i * n + j] = mk<double>(tr, ti);
    }
}

cudaError_t launch_basis_change(const double *U, long long u_stride, const double *M,
                                long long m_stride, int n, int batch, int adjoint, double *out,
                                cudaStream_t st) {
    if (n > MSP_MAX_DIM) {
        const size_t smem = (size_t)n * sizeof(cx<double>);
        const cx<double> *Uc = reinterpret_cast<const cx<double> *>(U);
        cx<double> *Oc = reinterpret_cast<cx<double> *>(out);
        for (int b0 = 0; b0 < batch; b0 += 65535) {
            const dim3 grid(n, batch - b0 < 65535 ? batch - b0 : 65535);
            msp_basis_change_col1_kernel<<<grid, 256, smem, st>>>(
                Uc, u_stride, reinterpret_cast<const cx<double> *>(M), m_stride, n, adjoint, b0,
                Oc);
            msp_basis_change_col2_kernel<<<grid, 256, smem, st>>>(Uc, u_stride, n, adjoint, b0,
                                                                  Oc);
        }
        return cudaGetLastError();
    }
    const size_t smem = (size_t)3 * n * n * sizeof(cx<double>);
    cudaError_t e = cudaFuncSetAttribute(msp_basis_change_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int grid = batch < 152 * 8 ? batch : 152 * 8;
    msp_basis_change_kernel<<<grid, n <= 16 ? 64 : 256, smem, st>>>(
        reinterpret_cast<const cx<double> *>(U), u_stride,
        reinterpret_cast<const cx<double> *>(M), m_stride, n, batch, adjoint,
        reinterpret_cast<cx<double> *>(out));
    return cudaGetLastError();
}

}  // namespace msp
