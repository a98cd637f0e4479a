// The MIXED fast path for n > 64: msp_large.cuh's solver in FP32, then
// double-word Ogita-Aishima refinement, with every O(n^3) product on one
// shared-memory tile engine (see the section comment below).
#include <type_traits>

#include "msp_cluster.cuh"
#include "msp_dw.cuh"
#include "msp_large.cuh"

namespace msp {

// ------------------------------------------------------------------ mixed precision
//
// MIXED for n > 64: msp_large.cuh's solver in FP32, then Ogita-Aishima refinement
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

// Refinement vectors and GEMM slabs in shared memory (the solver's shared
// memory is free once it returns).
constexpr int LM_KT = 16;  // k depth of a GEMM slab

struct LmVec {
    float2 *lam, *sd;  // eigenvalues and S_ii as double-words (msp_dw.cuh)
    float2 *gd;        // x_i^H x_i - 1 (double-word)
    int *rank, *order, *cstart;  // refinement clusters (msp_cluster.cuh)
    float *lamf, *corr, *rn, *cn, *yn;
    int *step;  // [0]: largest correction, [1]: largest |l_i|, [2]: amax (float bits)
    char *slab;  // two stages of GEMM slabs (A: TR x LM_KT, B: LM_KT x 32)
};

// Bytes of one slab stage: A and B at up to 16 bytes per element.
__host__ __device__ inline size_t lm_stage_bytes(int threads) {
    return ((size_t)4 * (threads / 32) * LM_KT + (size_t)LM_KT * 32) * 16;
}

// Bytes of the refinement vectors (also the back-transformation's two
// LM_KT x LM_KT complex matrices).
__host__ __device__ inline size_t lm_vec_bytes(int n) {
    size_t b = 56 * (size_t)n + 16;
    if (b < 2 * LM_KT * LM_KT * 8) b = 2 * LM_KT * LM_KT * 8;
    return (b + 15) & ~size_t(15);
}

// The slabs sit above both the refinement vectors and the FP32 solver's
// shared memory (the blocked tridiagonalisation uses both at once).
__host__ __device__ inline size_t lm_slab_offset(int n, int threads) {
    size_t o = lm_vec_bytes(n);
    const size_t sol = large_sm_bytes<float>(n, threads);
    if (sol > o) o = sol;
    return (o + 15) & ~size_t(15);
}

__host__ __device__ inline size_t lm_smem_bytes(int n, int threads) {
    return lm_slab_offset(n, threads) + 2 * lm_stage_bytes(threads);
}

__device__ __forceinline__ LmVec lm_vec(char *smem, int n) {
    LmVec v;
    v.lam = reinterpret_cast<float2 *>(smem);
    v.sd = v.lam + n;
    v.gd = v.sd + n;
    v.rank = reinterpret_cast<int *>(v.gd + n);
    v.order = v.rank + n;
    v.cstart = v.order + n;
    v.lamf = reinterpret_cast<float *>(v.cstart + n);
    v.corr = v.lamf + n;
    v.rn = v.corr + n;
    v.cn = v.rn + n;
    v.yn = v.cn + n;
    v.step = reinterpret_cast<int *>(v.yn + n);
    v.slab = smem + lm_slab_offset(n, blockDim.x);
    return v;
}

// Asynchronous global -> shared copies of one element (8 or 16 bytes);
// `valid` false writes zeros (nothing is read; src is still a valid
// address).  One commit group per slab; wait_group 1 leaves the newest
// group in flight.
__device__ __forceinline__ void lm_cp8(void *dst, const void *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src),
                 "r"(valid ? 8 : 0)
                 : "memory");
}
__device__ __forceinline__ void lm_cp16(void *dst, const void *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src),
                 "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void lm_cp(float4 *dst, const float4 *src, bool valid) {
    lm_cp16(dst, src, valid);
}
__device__ __forceinline__ void lm_cp(float2 *dst, const float2 *src, bool valid) {
    lm_cp8(dst, src, valid);
}
__device__ __forceinline__ void lm_cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void lm_cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// A stored element as its hi and lo lane pairs (lo = 0 for FP32 elements)
__device__ __forceinline__ void lm_pairs(const float4 *p, u64 &h, u64 &l) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(p);
    h = v.x;
    l = v.y;
}
__device__ __forceinline__ void lm_pairs(const float2 *p, u64 &h, u64 &l) {
    h = *reinterpret_cast<const u64 *>(p);
    l = 0ull;
}

// Tiled product C(i, j) = sum_k op(A)(i, k) B(k, j), i < M, j < N, k < K,
// as one CTA-wide kernel body.  The CTA walks output tiles of TR = 4 x
// warps rows by 32 columns; a thread owns rows 4 w .. 4 w + 3 (w its warp)
// of column `lane`.  A and B are staged in shared memory LM_KT deep as they
// are stored in global memory (no conversion), by cp.async in two stages:
// the next slab's copies are in flight while the current one is
// multiplied.  A(i, k) is read from Ag[k * lda + i] (A_KI) or
// Ag[i * lda + k], B(k, j) from Bg[k * ldb + j]; the A reads of the multiply
// are warp broadcasts.  Accumulation (ACC):
//   LM_DW_ALO   anchored double-word, A double-word (float4), B FP32
//   LM_DW_CBLO  anchored double-word, conj(A) FP32, B double-word
//   LM_DW_C     anchored double-word, conj(A) and B FP32
//   LM_PLAIN    FP32 sums of A B
//   LM_PLAIN_C  FP32 sums of conj(A) B
// (the pair (s1, s2) of lm_step; lm_dw / lm_plain turn it into the value).
// skip(i0, j0) drops a whole tile; init(i, j, s1, c1, s2, c2) seeds an
// accumulator (the anchor, or a start value); epi(i, j, s1, c1, s2, c2)
// consumes it (i < M, j < N only).
enum { LM_DW_ALO = 0, LM_DW_CBLO = 1, LM_DW_C = 2, LM_PLAIN = 3, LM_PLAIN_C = 4 };

template <int ACC, bool A_KI, typename AT, typename BT, typename Skip, typename Init, typename Epi>
__device__ void lm_tiles(int M, int N, int K, const AT *__restrict__ Ag, int lda,
                         const BT *__restrict__ Bg, int ldb, const LmVec &v, Skip skip, Init init,
                         Epi epi) {
    const int tid = threadIdx.x, nt = blockDim.x, w = tid >> 5, lane = tid & 31;
    const int TR = 4 * (nt >> 5);
    const int ti = (M + TR - 1) / TR, tj = (N + 31) >> 5, nslab = (K + LM_KT - 1) / LM_KT;
    const size_t stage = lm_stage_bytes(nt);
    char *A0 = v.slab, *B0 = v.slab + (size_t)TR * LM_KT * 16;
    auto issue = [&](int i0, int j0, int sl) {
        AT *As = reinterpret_cast<AT *>(A0 + (sl & 1) * stage);
        BT *Bs = reinterpret_cast<BT *>(B0 + (sl & 1) * stage);
        const int k0 = sl * LM_KT;
        for (int e = tid; e < TR * LM_KT; e += nt) {
            const int i = A_KI ? e % TR : e / LM_KT, k = A_KI ? e / TR : e % LM_KT;
            const int gi = i0 + i, gk = k0 + k;
            const bool ok = gi < M && gk < K;
            const size_t off = ok ? (A_KI ? (size_t)gk * lda + gi : (size_t)gi * lda + gk) : 0;
            lm_cp(As + e, Ag + off, ok);
        }
        for (int e = tid; e < LM_KT * 32; e += nt) {
            const int gk = k0 + (e >> 5), gj = j0 + (e & 31);
            const bool ok = gk < K && gj < N;
            lm_cp(Bs + e, Bg + (ok ? (size_t)gk * ldb + gj : 0), ok);
        }
        lm_cp_commit();
    };
    for (int t = 0; t < ti * tj; ++t) {  // the same sequence in every thread
        const int it = t / tj, i0 = it * TR, j0 = (t - it * tj) * 32;
        if (skip(i0, j0)) continue;
        const int j = j0 + lane;
        u64 s1[4], c1[4], s2[4], c2[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            s1[q] = c1[q] = s2[q] = c2[q] = 0ull;
            init(i0 + 4 * w + q, j, s1[q], c1[q], s2[q], c2[q]);
        }
        issue(i0, j0, 0);
        for (int sl = 0; sl < nslab; ++sl) {
            if (sl + 1 < nslab)
                issue(i0, j0, sl + 1);
            else
                lm_cp_commit();  // an empty group keeps wait_group 1 exact
            lm_cp_wait1();
            __syncthreads();
            const AT *As = reinterpret_cast<const AT *>(A0 + (sl & 1) * stage);
            const BT *Bs = reinterpret_cast<const BT *>(B0 + (sl & 1) * stage);
#pragma unroll 4
            for (int k = 0; k < LM_KT; ++k) {
                u64 bh, bl;
                lm_pairs(Bs + k * 32 + lane, bh, bl);
                float b0, b1;
                split_f32x2(bh, b0, b1);
                const u64 bx = f32x2(b0, b0), by = f32x2(b1, b1);
                u64 blx = 0ull, bly = 0ull;
                if (ACC == LM_DW_CBLO) {
                    split_f32x2(bl, b0, b1);
                    blx = f32x2(b0, b0);
                    bly = f32x2(b1, b1);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = 4 * w + q;
                    u64 ah, al;
                    lm_pairs(As + (A_KI ? k * TR + r : r * LM_KT + k), ah, al);
                    if (ACC == LM_DW_ALO) {
                        lm_step<true, false>(s1[q], c1[q], s2[q], c2[q], ah, al, bx, by, 0ull, 0ull);
                    } else if (ACC == LM_DW_CBLO) {
                        lm_step<false, true>(s1[q], c1[q], s2[q], c2[q], ah, 0ull, bx, by, blx, bly);
                    } else if (ACC == LM_DW_C) {
                        lm_step<false, false>(s1[q], c1[q], s2[q], c2[q], ah, 0ull, bx, by, 0ull,
                                              0ull);
                    } else {
                        s1[q] = fma_f32x2(ah, bx, s1[q]);
                        s2[q] = fma_f32x2(ah, by, s2[q]);
                    }
                }
            }
            __syncthreads();  // the stage is refilled two slabs later
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = i0 + 4 * w + q;
            if (i < M && j < N) epi(i, j, s1[q], c1[q], s2[q], c2[q]);
        }
    }
    __syncthreads();
}


// The four products of a refinement step (n x n):
//   Y = H X (H double-word), S = X^H Y (Y double-word), G = X^H X, and
//   X2 = X + X E (FP32, E in SR with its diagonal).
// S and G skip tiles with no entry on or above the diagonal; S_ij (i < j)
// -> SR[i][j], S_ii -> sd; R_ij = -G_ij (i < j) -> SR[j][i], R_ii = 1 - G_ii
// -> rd.
enum { LM_HX = 0, LM_S = 1, LM_G = 2, LM_XE = 3 };

template <int MODE>
__device__ void lm_gemm(const LargeMixed &s, const cx<float> *__restrict__ X,
                        cx<float> *__restrict__ X2, const LmVec &v, int n) {
    const float2 *Xf = reinterpret_cast<const float2 *>(X);
    auto noskip = [](int, int) { return false; };
    auto upper = [n](int i0, int j0) { return min(j0 + 31, n - 1) < i0; };
    auto dw_init = [&](int i, int j, u64 &s1, u64 &c1, u64 &s2, u64 &c2, float bound) {
        (void)i;
        (void)j;
        s1 = s2 = lm_anchor(bound);
        c1 = c2 = 0ull;
    };
    if (MODE == LM_HX) {
        auto bound = [&](int i, int j) { return v.rn[min(i, n - 1)] * v.cn[min(j, n - 1)]; };
        lm_tiles<LM_DW_ALO, false>(
            n, n, n, s.H, n, Xf, n, v, noskip,
            [&](int i, int j, u64 &s1, u64 &c1, u64 &s2, u64 &c2) {
                dw_init(i, j, s1, c1, s2, c2, bound(i, j));
            },
            [&](int i, int j, u64 s1, u64 c1, u64 s2, u64 c2) {
                const u64 K = lm_anchor(bound(i, j));
                s.Y[(size_t)i * n + j] = lm_dw<false>(s1, c1, s2, c2, K);
            });
    } else if (MODE == LM_S) {
        auto bound = [&](int i, int j) { return v.cn[min(i, n - 1)] * v.yn[min(j, n - 1)]; };
        lm_tiles<LM_DW_CBLO, true>(
            n, n, n, Xf, n, s.Y, n, v, upper,
            [&](int i, int j, u64 &s1, u64 &c1, u64 &s2, u64 &c2) {
                dw_init(i, j, s1, c1, s2, c2, bound(i, j));
            },
            [&](int i, int j, u64 s1, u64 c1, u64 s2, u64 c2) {
                const u64 K = lm_anchor(bound(i, j));
                const float4 r = lm_dw<true>(s1, c1, s2, c2, K);
                if (i == j)
                    v.sd[i] = make_float2(r.x, r.z);
                else if (i < j)
                    s.SR[(size_t)i * n + j] = mk<float>(r.x + r.z, r.y + r.w);
            });
    } else if (MODE == LM_G) {
        auto bound = [&](int i, int j) { return v.cn[min(i, n - 1)] * v.cn[min(j, n - 1)]; };
        lm_tiles<LM_DW_C, true>(
            n, n, n, Xf, n, Xf, n, v, upper,
            [&](int i, int j, u64 &s1, u64 &c1, u64 &s2, u64 &c2) {
                dw_init(i, j, s1, c1, s2, c2, bound(i, j));
            },
            [&](int i, int j, u64 s1, u64 c1, u64 s2, u64 c2) {
                const u64 K = lm_anchor(bound(i, j));
                const float4 r = lm_dw<true>(s1, c1, s2, c2, K);
                if (i == j)
                    v.gd[i] = make_float2(r.x - 1.0f, r.z);  // r.x - 1 exact
                else if (i < j)
                    s.SR[(size_t)j * n + i] = mk<float>(-(r.x + r.z), -(r.y + r.w));
            });
    } else {
        lm_tiles<LM_PLAIN, false>(
            n, n, n, Xf, n, reinterpret_cast<const float2 *>(s.SR), n, v, noskip,
            [&](int i, int j, u64 &s1, u64 &, u64 &, u64 &) {
                const cx<float> x = i < n && j < n ? X[(size_t)i * n + j] : mk<float>(0.f, 0.f);
                s1 = f32x2(x.re, x.im);
            },
            [&](int i, int j, u64 s1, u64, u64 s2, u64) {
                X2[(size_t)i * n + j] = lm_plain<false>(s1, s2);
            });
    }
}

// Blocked back-transformation U = Q Z for the FP32 solver (the compact WY
// form of LAPACK zlarft, forward, columnwise): reflectors kb .. kb + nb - 1
// (nb <= LM_KT) act together as P = I - V T V^H on rows kb + 1 .. n - 1 of
// U, with V (m x nb, unit lower trapezoidal) copied out of the reflector
// storage, T upper triangular from tau and the Gram matrix V^H V:
//   T_ii = tau_i,  T[0:i, i] = T[0:i, 0:i] (-tau_i (V^H V)[0:i, i]);
// then W = V^H U_b, W2 = -T W, U_b += V W2 -- three tiled products that read
// U twice per block instead of twice per reflector.  Blocks run last to
// first (U = H_0 H_1 ... H_{n-2} Z).  Scratch: SR (free during the solve)
// holds V, W and W2; the refinement vectors' shared memory holds V^H V and T.
__device__ void lm_back(const LargeMixed &s, const LmVec &v, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    cx<float> *U = s.X;
    for (size_t x = tid; x < (size_t)n * n; x += nt) {
        const int i = (int)(x / n), j = (int)(x - (size_t)i * n);
        U[x] = mk<float>(s.sol.Zt[(size_t)j * n + i], 0.f);
    }
    float2 *Vb = reinterpret_cast<float2 *>(s.SR);  // m x LM_KT
    float2 *W = Vb + (size_t)n * LM_KT;            // LM_KT x n
    float2 *W2 = W + (size_t)n * LM_KT;            // LM_KT x n
    cx<float> *Gs = reinterpret_cast<cx<float> *>(v.lam);  // LM_KT x LM_KT
    cx<float> *Ts = Gs + LM_KT * LM_KT;
    const cx<float> *A = s.sol.A;
    const int nref = n - 1;
    auto noskip = [](int, int) { return false; };
    auto zero = [](int, int, u64 &s1, u64 &, u64 &, u64 &) { s1 = 0ull; };
    __syncthreads();
    for (int kb = ((nref - 1) / LM_KT) * LM_KT; kb >= 0; kb -= LM_KT) {
        const int nb = min(LM_KT, nref - kb), m = n - kb - 1;
        for (int e = tid; e < m * LM_KT; e += nt) {
            const int r = e / LM_KT, c = e % LM_KT;
            cx<float> val = mk<float>(0.f, 0.f);
            if (c < nb && r >= c)
                val = r == c ? mk<float>(1.f, 0.f) : A[(size_t)(kb + 1 + r) * n + kb + c];
            Vb[e] = make_float2(val.re, val.im);
        }
        __syncthreads();
        // V^H V
        lm_tiles<LM_PLAIN_C, true>(nb, nb, m, Vb, LM_KT, Vb, LM_KT, v, noskip, zero,
                                   [&](int i, int j, u64 s1, u64, u64 s2, u64) {
                                       Gs[i * LM_KT + j] = lm_plain<true>(s1, s2);
                                   });
        // T, one column at a time (nb <= 16 threads per column)
        for (int i = 0; i < nb; ++i) {
            const cx<float> taui = s.sol.tau[kb + i];
            if (tid < i) {
                // t_c = -tau_i G[c][i], then T[c][i] = sum_{c' >= c} T[c][c'] t_c'
                cx<float> acc = mk<float>(0.f, 0.f);
                for (int c2 = tid; c2 < i; ++c2) {
                    const cx<float> t = cmul(taui, Gs[c2 * LM_KT + i]);
                    acc = cadd(acc, cmul(Ts[tid * LM_KT + c2], mk<float>(-t.re, -t.im)));
                }
                Ts[tid * LM_KT + i] = acc;
            }
            if (tid == 0) {
                Ts[i * LM_KT + i] = taui;
                for (int r = i + 1; r < LM_KT; ++r) Ts[r * LM_KT + i] = mk<float>(0.f, 0.f);
            }
            __syncthreads();
        }
        // W = V^H U_b
        cx<float> *Ub = U + (size_t)(kb + 1) * n;
        lm_tiles<LM_PLAIN_C, true>(nb, n, m, Vb, LM_KT, reinterpret_cast<const float2 *>(Ub), n, v,
                                   noskip, zero, [&](int i, int j, u64 s1, u64, u64 s2, u64) {
                                       const cx<float> r = lm_plain<true>(s1, s2);
                                       W[(size_t)i * n + j] = make_float2(r.re, r.im);
                                   });
        // W2 = -T W
        for (int e = tid; e < nb * n; e += nt) {
            const int c = e / n, j = e - c * n;
            cx<float> acc = mk<float>(0.f, 0.f);
            for (int c2 = c; c2 < nb; ++c2) {
                const float2 wv = W[(size_t)c2 * n + j];
                acc = cadd(acc, cmul(Ts[c * LM_KT + c2], mk<float>(wv.x, wv.y)));
            }
            W2[(size_t)c * n + j] = make_float2(-acc.re, -acc.im);
        }
        __syncthreads();
        // U_b += V W2
        lm_tiles<LM_PLAIN, false>(
            m, n, nb, Vb, LM_KT, W2, n, v, noskip,
            [&](int i, int j, u64 &s1, u64 &, u64 &, u64 &) {
                const cx<float> u = i < m && j < n ? Ub[(size_t)i * n + j] : mk<float>(0.f, 0.f);
                s1 = f32x2(u.re, u.im);
            },
            [&](int i, int j, u64 s1, u64, u64 s2, u64) {
                Ub[(size_t)i * n + j] = lm_plain<false>(s1, s2);
            });
    }
}

// Column 2-norms of an n x n matrix of (re, im) pairs with element stride
// `stride` floats (X: 2, the hi part of Y: 4).
__device__ __forceinline__ void lm_colnorms(const float *M, int stride, int n, float *out) {
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        float acc = 0.f;
        for (int k = 0; k < n; ++k) {
            const float *e = M + ((size_t)k * n + j) * stride;
            acc = fmaf(e[0], e[0], fmaf(e[1], e[1], acc));
        }
        out[j] = sqrtf(acc);
    }
}

// One refinement step of the eigenvector columns X into X2 and of the
// eigenvalues v.lam, clusters resolved as in the n <= 64 refinement
// (msp_cluster.cuh; T in the Y buffer, free once S is formed).  Returns the
// step's largest correction.
__device__ float lm_refine(const LargeMixed &s, const cx<float> *__restrict__ X,
                           cx<float> *__restrict__ X2, const LmVec &v, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    cx<float> *__restrict__ SR = s.SR;
    lm_colnorms(reinterpret_cast<const float *>(X), 2, n, v.cn);
    if (tid < 4) v.step[tid] = 0;  // step, max|l|, amax (float bits)
    __syncthreads();
    lm_gemm<LM_HX>(s, X, X2, v, n);
    lm_colnorms(reinterpret_cast<const float *>(s.Y), 4, n, v.yn);
    __syncthreads();
    lm_gemm<LM_S>(s, X, X2, v, n);
    lm_gemm<LM_G>(s, X, X2, v, n);
    float lmax = 0.f;
    for (int i = tid; i < n; i += nt) {
        const float2 l = dw_rayleigh(v.sd[i], v.gd[i]);
        v.lam[i] = l;
        v.lamf[i] = l.x;
        v.corr[i] = 0.f;
        lmax = fmaxf(lmax, fabsf(l.x));
    }
    atomicMax(&v.step[1], __float_as_int(lmax));  // non-negative: int order = float order
    __syncthreads();
    OaCluster cl;
    cl.rank = v.rank;
    cl.order = v.order;
    cl.cstart = v.cstart;
    cl.scal = v.step + 2;
    cl.T = reinterpret_cast<cx<float> *>(s.Y);
    cl.ldt = n;
    oa_clusters(SR, n, v.lam, v.lamf, n, cl);
    float emax = 0.f;
    const int nup = n * (n - 1) / 2;
    for (int e = tid; e < nup; e += nt) {
        int i, j;
        oa_pair_of(e, i, j);
        oa_pair_correction(SR, n, v.lam, v.lamf, cl, v.corr, i, j, emax);
    }
    __syncthreads();
    oa_cluster_diagonal(v.lam, v.corr, n, cl);
    for (int j = tid; j < n; j += nt)  // E_jj = R_jj / 2
        SR[(size_t)j * n + j] = mk<float>(-0.5f * (v.gd[j].x + v.gd[j].y), 0.f);
    __syncthreads();
    lm_gemm<LM_XE>(s, X, X2, v, n);
    emax = fmaxf(emax, oa_resolve_clusters(X2, n, n, v.lam, v.corr, n, cl,
                                           __int_as_float(v.step[1])));
    atomicMax(v.step, __float_as_int(emax));  // non-negative: int order = float order
    __syncthreads();
    const float step = __int_as_float(*v.step);
    __syncthreads();
    return step;
}

// Blocked tridiagonalisation for the FP32 solver (the panel scheme of
// LAPACK zlatrd / zhetrd, lower form, full storage): columns are reduced
// LM_KT at a time.  Within a panel the trailing matrix stays as it was at
// the panel start ("stale"); reflector j of the panel keeps v_j and w_j in
// VW (rows: V in columns 0..15, W in 16..31), so that the true trailing
// matrix is the stale one minus V W^H + W V^H:
//   1. column k (rows k..) is brought up to date from the panel's V, W;
//   2. its reflector (as in the unblocked form; d_k, e_k, tau_k);
//   3. p = A22 v over the stale matrix, in the same column-parallel pass
//      as y = VW^H v (32 extra "columns" read from VW);
//   4. p -= V (W^H v) + W (V^H v), p *= tau, alpha = -tau (p^H v) / 2,
//      w = p + alpha v;
// and after the panel one rank-2 LM_KT update of the trailing matrix,
// A22 += [V W] [-W^H; -V^H], through the tile engine.  The trailing matrix
// is read about 1.2 times per column instead of three times.  Leaves d, e
// in the solver's shared memory, the reflectors in A (below the
// subdiagonal) and their scalars in tau.  Scratch: SR (free during the
// solve) holds VW (n x 32) and the update's right operand (32 x n).
__device__ void lm_tridiag(const LargeMixed &s, const LmVec &vv, char *smem, int n) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int RW = nt < 64 ? nt : 64, G = nt / RW, pr = tid % RW, pg = tid / RW;
    const LargeSm<float> sm = large_sm<float>(smem, n, nt);
    cx<float> *A = s.sol.A;
    cx<float> *VW = s.SR;                   // n x 32
    cx<float> *Bt = s.SR + (size_t)n * 32;  // 32 x n
    cx<float> *v = sm.v, *p = sm.p, *part = sm.part, *y = sm.y;
    const size_t pst = (size_t)n + 32;  // stride of the partial sums
    auto noskip = [](int, int) { return false; };
    for (int k0 = 0; k0 + 1 < n; k0 += LM_KT) {
        const int nbp = min(LM_KT, n - 1 - k0);
        for (size_t x = (size_t)k0 * 32 + tid; x < (size_t)n * 32; x += nt)
            VW[x] = mk<float>(0.f, 0.f);
        __syncthreads();
        for (int j = 0; j < nbp; ++j) {
            const int k = k0 + j, m = n - k - 1;
            // 1. column k, rows k.., minus the panel's V W^H + W V^H
            if (j > 0) {
                const cx<float> *vk = VW + (size_t)k * 32;
                for (int r = k + tid; r < n; r += nt) {
                    const cx<float> *vr = VW + (size_t)r * 32;
                    cx<float> a = A[(size_t)r * n + k];
                    for (int c = 0; c < j; ++c) {
                        const cx<float> t1 = cmul(vr[c], conj(vk[16 + c]));
                        const cx<float> t2 = cmul(vr[16 + c], conj(vk[c]));
                        a = mk<float>(a.re - t1.re - t2.re, a.im - t1.im - t2.im);
                    }
                    A[(size_t)r * n + k] = a;
                }
                __syncthreads();
            }
            // 2. reflector of A[k+1.., k]
            float xn2 = 0.f;
            for (int i = 1 + tid; i < m; i += nt) xn2 += cabs2(A[(size_t)(k + 1 + i) * n + k]);
            xn2 = block_sum(xn2, sm.red);
            const cx<float> alpha = A[(size_t)(k + 1) * n + k];
            cx<float> tau = mk<float>(0.f, 0.f);
            float beta = alpha.re;
            const bool reflect = !(xn2 == 0.f && alpha.im == 0.f);
            if (reflect) {
                beta = -copysignf(sqrtf(alpha.re * alpha.re + alpha.im * alpha.im + xn2), alpha.re);
                tau = mk<float>((beta - alpha.re) / beta, -alpha.im / beta);
                const cx<float> den = mk<float>(alpha.re - beta, alpha.im);
                const float dd = 1.f / cabs2(den);
                const cx<float> sc = mk<float>(den.re * dd, -den.im * dd);
                for (int i = tid; i < m; i += nt)
                    v[i] = i == 0 ? mk<float>(1.f, 0.f) : cmul(A[(size_t)(k + 1 + i) * n + k], sc);
            } else {
                for (int i = tid; i < m; i += nt) v[i] = mk<float>(0.f, 0.f);  // V and W columns stay 0
            }
            if (tid == 0) {
                sm.d[k] = A[(size_t)k * n + k].re;
                sm.e[k] = beta;
                s.sol.tau[k] = tau;
            }
            __syncthreads();
            // 3. p = A22 v (stale A22, Hermitian: p_i = sum_l conj(A22_li) v_l) and
            //    y = VW^H v in extra columns i = m .. m + 31
            if (pg < G) {
                const int lb = (int)((long long)m * pg / G), le = (int)((long long)m * (pg + 1) / G);
                for (int i = pr; i < m + 32; i += RW) {
                    const cx<float> *col = i < m ? A + (size_t)(k + 1) * n + (k + 1 + i)
                                                 : VW + (size_t)(k + 1) * 32 + (i - m);
                    const size_t ld = i < m ? (size_t)n : 32;
                    float r0 = 0.f, i0 = 0.f, r1 = 0.f, i1 = 0.f;
                    int l = lb;
#pragma unroll 4
                    for (; l + 1 < le; l += 2) {
                        const cx<float> a0 = col[(size_t)l * ld], a1 = col[(size_t)(l + 1) * ld];
                        const cx<float> x0 = v[l], x1 = v[l + 1];
                        r0 += a0.re * x0.re + a0.im * x0.im;
                        i0 += a0.re * x0.im - a0.im * x0.re;
                        r1 += a1.re * x1.re + a1.im * x1.im;
                        i1 += a1.re * x1.im - a1.im * x1.re;
                    }
                    if (l < le) {
                        const cx<float> a0 = col[(size_t)l * ld], x0 = v[l];
                        r0 += a0.re * x0.re + a0.im * x0.im;
                        i0 += a0.re * x0.im - a0.im * x0.re;
                    }
                    part[(size_t)pg * pst + i] = mk<float>(r0 + r1, i0 + i1);
                }
            }
            __syncthreads();
            for (int i = tid; i < m + 32; i += nt) {
                float sr = 0.f, si = 0.f;
                for (int g = 0; g < G; ++g) {
                    sr += part[(size_t)g * pst + i].re;
                    si += part[(size_t)g * pst + i].im;
                }
                if (i < m)
                    p[i] = mk<float>(sr, si);
                else
                    y[i - m] = mk<float>(sr, si);  // V^H v in 0..15, W^H v in 16..31
            }
            __syncthreads();
            // 4. p = tau (p - V (W^H v) - W (V^H v)); w = p + alpha v
            float hr = 0.f, hi = 0.f;
            for (int i = tid; i < m; i += nt) {
                cx<float> acc = p[i];
                const cx<float> *vr = VW + (size_t)(k + 1 + i) * 32;
                for (int c = 0; c < j; ++c) {
                    const cx<float> t1 = cmul(vr[c], y[16 + c]), t2 = cmul(vr[16 + c], y[c]);
                    acc = mk<float>(acc.re - t1.re - t2.re, acc.im - t1.im - t2.im);
                }
                acc = cmul(tau, acc);
                p[i] = acc;
                const cx<float> c = cmulc(acc, v[i]);  // conj(p_i) v_i
                hr += c.re;
                hi += c.im;
            }
            hr = block_sum(hr, sm.red);
            hi = block_sum(hi, sm.red);
            const cx<float> a2 = cscale(-0.5f, cmul(tau, mk<float>(hr, hi)));
            for (int i = tid; i < m; i += nt) {
                const cx<float> vi = v[i];
                VW[(size_t)(k + 1 + i) * 32 + j] = vi;
                VW[(size_t)(k + 1 + i) * 32 + 16 + j] = cadd(p[i], cmul(a2, vi));
                if (i > 0 && reflect) A[(size_t)(k + 1 + i) * n + k] = vi;  // for the back-transformation
            }
            __syncthreads();
        }
        // rank-2 LM_KT update of the trailing matrix (rows and columns k1..)
        const int k1 = k0 + nbp, mt = n - k1;
        if (mt > 0) {
            for (int x = tid; x < 32 * mt; x += nt) {
                const int kk = x / mt, jj = x - kk * mt;
                const cx<float> w = VW[(size_t)(k1 + jj) * 32 + (kk < 16 ? 16 + kk : kk - 16)];
                Bt[(size_t)kk * n + jj] = mk<float>(-w.re, w.im);  // -conj
            }
            __syncthreads();
            cx<float> *At = A + (size_t)k1 * n + k1;
            lm_tiles<LM_PLAIN, false>(
                mt, mt, 32, reinterpret_cast<const float2 *>(VW + (size_t)k1 * 32), 32,
                reinterpret_cast<const float2 *>(Bt), n, vv, noskip,
                [&](int i, int j, u64 &s1, u64 &, u64 &, u64 &) {
                    const cx<float> a = i < mt && j < mt ? At[(size_t)i * n + j] : mk<float>(0.f, 0.f);
                    s1 = f32x2(a.re, a.im);
                },
                [&](int i, int j, u64 s1, u64, u64 s2, u64) {
                    At[(size_t)i * n + j] = lm_plain<false>(s1, s2);
                });
        }
    }
    if (tid == 0) {
        sm.d[n - 1] = A[(size_t)(n - 1) * n + (n - 1)].re;
        sm.e[n - 1] = 0.f;
    }
    __syncthreads();
}

// The fast path for n > 64 in MIXED precision: H = Hsys + b . Z in FP64,
// split into hi + lo; the FP32 solver on hi; refinement steps until the
// correction drops below 2e-4 (at most four; one step leaves an error of
// order E^2); M = U^H (sigma_p (x) 1_d) U in FP32; pair records with FP64
// frequencies from the refined eigenvalues.
// Pair record of the mixed kernel: FP32 coefficient and, from the level gap
// d (double-word), the double-word phases on a uniform grid or the FP64
// frequency otherwise.
__device__ __forceinline__ void lm_store_pair(const SnapArgs &a, size_t o, float cA, float2 d) {
    reinterpret_cast<float2 *>(a.pair_coef)[o] = make_float2(cA, 0.f);
    if (a.pair_phase) {
        const float2 psi = dw_phase_mod2pi(d, a.c_dt);
        const float2 ph0 = a.t0_zero ? make_float2(0.f, 0.f) : dw_phase_mod2pi(d, a.c_t0);
        a.pair_phase[o] = make_float4(psi.x, psi.y, ph0.x, ph0.y);
    } else {
        a.pair_omega[o] = 6.283185307179586476925 * dw_to_double(d);
    }
}

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
        // the blocked reduction pays from n ~ 128 (measured: 20% faster at
        // n = 192, 20% slower at n = 96)
        int st;
        if (n >= 128) {
            lm_tridiag(s, v, smem, n);
            st = large_eigh<float, false, false>(s.sol, n, smem);
        } else {
            st = large_eigh<float, false, true>(s.sol, n, smem);
        }
        lm_back(s, v, n);
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
        const int max_refine = a.max_refine > 0 ? a.max_refine : 4;
        st |= MSP_ITEM_REFINE_LIMIT;
        for (int it = 0; it < max_refine; ++it) {
            const float step = lm_refine(s, X, X2, v, n);
            cx<float> *t = X;
            X = X2;
            X2 = t;
            if (step <= 2e-4f) {
                st &= ~MSP_ITEM_REFINE_LIMIT;
                break;
            }
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
        const float scale_f = (float)scale;
        double diag = 0.0;
        // G = X^H W (tiles with an entry j >= k only); A_jk = |G_jk|^2
        lm_tiles<LM_PLAIN_C, true>(
            n, n, n, reinterpret_cast<const float2 *>(X), n, reinterpret_cast<const float2 *>(X2),
            n, v, [](int i0, int j0) { return i0 + 4 * (int)(blockDim.x >> 5) - 1 < j0; },
            [](int, int, u64 &, u64 &, u64 &, u64 &) {},
            [&](int j, int k, u64 s1, u64, u64 s2, u64) {
                if (j < k) return;
                const cx<float> G = lm_plain<true>(s1, s2);
                const float Am = G.re * G.re + G.im * G.im;
                if (j == k)
                    diag += (double)Am;
                else
                    lm_store_pair(a, (size_t)sn * P + (size_t)j * (j - 1) / 2 + k, scale_f * Am,
                                  dw_sub(v.lam[j], v.lam[k]));
            });
        diag = block_sum(diag, red);
        if (tid == 0) {
            a.snap_const[sn] = scale * 0.5 * diag;
            a.status[g] = st;
        }
        __syncthreads();
    }
}

size_t large_mixed_scratch_per_cta(int n) { return lm_scratch_bytes(n); }

// Resident CTAs per SM of the mixed kernel with `threads` threads (by
// occupancy: registers and shared memory).
int large_mixed_occupancy(int n, int threads) {
    int occ = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_large_fast_mixed_kernel, threads,
                                                      lm_smem_bytes(n, threads)) !=
            cudaSuccess ||
        occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    return occ;
}

cudaError_t launch_large_fast_mixed(const SnapArgs &a, double *scratch, int grid,
                                    cudaStream_t st, int threads) {
    if (threads > 256) return cudaErrorInvalidValue;
    const size_t smem = lm_smem_bytes(a.n, threads);
    cudaError_t e = cudaFuncSetAttribute(msp_large_fast_mixed_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    msp_large_fast_mixed_kernel<<<grid, threads, smem, st>>>(a, reinterpret_cast<char *>(scratch));
    return cudaGetLastError();
}

}  // namespace msp
