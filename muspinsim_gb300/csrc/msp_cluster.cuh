// Cluster handling of the Ogita-Aishima refinement step (T. Ogita and
// K. Aishima, "Iterative refinement for symmetric eigenvalue decomposition
// II: clustered eigenvalues", Japan J. Indust. Appl. Math. 36 (2019) 435),
// shared by the n <= 64 and n > 64 mixed-precision refinements.  Part of
// the replacement of np.linalg.eigh in Hermitian.diag
// (muspinsim/spinop.py:51-82).
//
// One refinement step has, from the FP32 eigenvector matrix X and the
// Hermitian H, the double-word products S = X^H H X and R = I - X^H X and
// the Rayleigh quotients l_i = S_ii / (1 - R_ii).  For a pair of levels the
// first-order correction E_ij = (S_ij + l_j R_ij) / (l_j - l_i) is accurate
// only while it is small.  Here:
//   * a = S_ij + l_i R_ij, b = S_ij + l_j R_ij; amax = the largest
//     component of any a or b;
//   * levels sorted by l form clusters: runs whose consecutive gaps are at
//     most gamma = 100 amax.  Two levels in different clusters are more
//     than gamma apart, so their first-order |E| stays below 1e-2;
//   * pairs in different clusters get the first-order E and the
//     second-order eigenvalue term; pairs in one cluster are only
//     orthonormalised (E_ij = R_ij / 2);
//   * each cluster of k >= 2 levels is then resolved exactly: the k x k
//     Hermitian block T (off-diagonal c_ij = S_ij + (l_i + l_j) / 2 R_ij,
//     diagonal l_i - l_ref plus the level's second-order term) is
//     diagonalised by cyclic Jacobi in FP32, one warp per cluster, and each
//     rotation is applied to the two columns of X + X E it acts on.  The
//     cluster's eigenvalues are l_ref + diag(T).
// Couplings at or below the double-word noise floor (4 n 2^-44 max|l|) are
// not rotated: inside an exactly degenerate multiplet any orthonormal basis
// is exact.  The step's size (which decides whether another step follows)
// counts the first-order |E| and the |s| of rotations whose coupling is
// more than 16 times that floor.
//
// T lives in sorted coordinates (row and column = sorted position), so
// the clusters are disjoint diagonal blocks of one n x n buffer.
#pragma once

#include "msp_dw.cuh"
#include "msp_jacobi.cuh"

namespace msp {

// Strict upper pair e -> (i, j), i < j, e = j (j - 1) / 2 + i.
__device__ __forceinline__ void oa_pair_of(int e, int &i, int &j) {
    j = (int)((sqrtf(8.0f * (float)e + 1.0f) + 1.0f) * 0.5f);
    while (j * (j - 1) / 2 > e) --j;
    while ((j + 1) * j / 2 <= e) ++j;
    i = e - j * (j - 1) / 2;
}

struct OaCluster {
    int *rank;    // level -> sorted position
    int *order;   // sorted position -> level
    int *cstart;  // sorted position -> first sorted position of its cluster
    int *scal;    // [0]: amax (float bits)
    cx<float> *T; // cluster blocks, row stride ldt (sorted coordinates)
    int ldt;
};

// Whether sorted position r belongs to a cluster of two or more levels.
__device__ __forceinline__ bool oa_in_cluster(const int *cstart, int n, int r) {
    return (r > 0 && cstart[r - 1] == cstart[r]) || (r + 1 < n && cstart[r + 1] == cstart[r]);
}

// Clusters of the refinement step: amax, the sort, the cluster starts and
// the off-diagonal entries of T.  SR holds S_ij (i < j) at [i][j] and R_ij
// at [j][i] (row stride ld); lam / lamf are the Rayleigh quotients (lam as
// double-words, msp_dw.cuh; lamf their high words).
// c.scal[0] must be zero on entry (made visible by a barrier).  All threads
// of the CTA call it; it ends with a barrier.
static __device__ void oa_clusters(const cx<float> *SR, int ld, const float2 *lam,
                                   const float *lamf, int n, const OaCluster &c) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int nup = n * (n - 1) / 2;
    float amax = 0.f;
    for (int e = tid; e < nup; e += nt) {
        int i, j;
        oa_pair_of(e, i, j);
        const cx<float> S = SR[(size_t)i * ld + j], R = SR[(size_t)j * ld + i];
        const float ar = S.re + lamf[i] * R.re, ai = S.im + lamf[i] * R.im;
        const float br = S.re + lamf[j] * R.re, bi = S.im + lamf[j] * R.im;
        amax = fmaxf(amax, fmaxf(fmaxf(fabsf(ar), fabsf(ai)), fmaxf(fabsf(br), fabsf(bi))));
    }
    atomicMax(&c.scal[0], __float_as_int(amax));  // non-negative: int order = float order
    // ascending order, ties by index
    for (int i = tid; i < n; i += nt) {
        const float2 li = lam[i];
        int r = 0;
        for (int k = 0; k < n; ++k) {
            const float2 lk = lam[k];
            r += dw_less(lk, li) || (dw_equal(lk, li) && k < i);
        }
        c.rank[i] = r;
        c.order[r] = i;
    }
    __syncthreads();
    const float gamma = 100.0f * __int_as_float(c.scal[0]);
    if (tid < 32) {
        // cluster start of every sorted position: an inclusive max-scan of
        // the break positions, in contiguous chunks of `per` positions
        const int lane = tid, per = (n + 31) >> 5;
        const int q0 = lane * per, q1 = min(q0 + per, n);
        int run = -1;
        for (int q = q0; q < q1; ++q) {
            const bool brk = q == 0 || dw_sub_f(lam[c.order[q]], lam[c.order[q - 1]]) > gamma;
            if (brk) run = q;
            c.cstart[q] = run;  // -1: continues a run from an earlier chunk
        }
        int carry = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, carry, o);
            if (lane >= o) carry = max(carry, v);
        }
        int before = __shfl_up_sync(0xffffffffu, carry, 1);
        if (lane == 0) before = 0;
        for (int q = q0; q < q1; ++q)
            if (c.cstart[q] < 0) c.cstart[q] = before;
    }
    __syncthreads();
    for (int e = tid; e < nup; e += nt) {
        int i, j;
        oa_pair_of(e, i, j);
        const int ri = c.rank[i], rj = c.rank[j];
        if (c.cstart[ri] != c.cstart[rj]) continue;
        const cx<float> S = SR[(size_t)i * ld + j], R = SR[(size_t)j * ld + i];
        const float h = 0.5f * (lamf[i] + lamf[j]);
        const cx<float> v = mk<float>(S.re + h * R.re, S.im + h * R.im);
        c.T[(size_t)ri * c.ldt + rj] = v;
        c.T[(size_t)rj * c.ldt + ri] = conj(v);
    }
    __syncthreads();
}

// E for the pair (i < j) in place of S_ij / R_ij, with the second-order
// eigenvalue terms (cross-cluster pairs) and the step size.
__device__ __forceinline__ void oa_pair_correction(cx<float> *SR, int ld, const float2 *lam,
                                                   const float *lamf, const OaCluster &c,
                                                   float *corr, int i, int j, float &emax) {
    const cx<float> S = SR[(size_t)i * ld + j], R = SR[(size_t)j * ld + i];
    cx<float> Eij, Eji;
    if (c.cstart[c.rank[i]] == c.cstart[c.rank[j]]) {
        Eij = mk<float>(0.5f * R.re, 0.5f * R.im);
        Eji = mk<float>(0.5f * R.re, -0.5f * R.im);
    } else {
        // only the gap needs the double-words (a difference of nearly equal
        // large numbers)
        const float dl = dw_sub_f(lam[j], lam[i]);
        const float br = S.re + lamf[j] * R.re, bi = S.im + lamf[j] * R.im;  // S_ij + l_j R_ij
        const float ar = S.re + lamf[i] * R.re, ai = S.im + lamf[i] * R.im;  // S_ij + l_i R_ij
        const float inv = 1.0f / dl;
        Eij = mk<float>(br * inv, bi * inv);
        Eji = mk<float>(-ar * inv, ai * inv);
        atomicAdd(&corr[i], -(ar * ar + ai * ai) * inv);
        atomicAdd(&corr[j], (br * br + bi * bi) * inv);
        emax = fmaxf(emax, fmaxf(fmaxf(fabsf(Eij.re), fabsf(Eij.im)),
                                 fmaxf(fabsf(Eji.re), fabsf(Eji.im))));
    }
    SR[(size_t)i * ld + j] = Eij;
    SR[(size_t)j * ld + i] = Eji;
}

// Diagonal of T (after the pair corrections, so the second-order terms are
// in corr).  Ends with a barrier.
static __device__ void oa_cluster_diagonal(const float2 *lam, const float *corr, int n,
                                           const OaCluster &c) {
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        if (!oa_in_cluster(c.cstart, n, r)) continue;
        const int i = c.order[r];
        const float2 lref = lam[c.order[c.cstart[r]]];
        c.T[(size_t)r * c.ldt + r] = mk<float>(dw_sub_f(lam[i], lref) + corr[i], 0.f);
    }
    __syncthreads();
}

// Resolves every cluster of two or more levels (one warp per cluster) on
// the corrected eigenvector matrix X (nrows x n, row stride ldx), and sets
// the clusters' eigenvalues; the other levels get l_i + corr_i.  Returns
// this thread's share of the step size.  Ends with a barrier.
static __device__ float oa_resolve_clusters(cx<float> *X, int ldx, int nrows, float2 *lam,
                                     const float *corr, int n, const OaCluster &c,
                                     float lscale) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    const float noise = 4.0f * (float)n * 5.684341886080802e-14f * lscale;  // 4 n 2^-44 max|l|
    const float big2 = 256.0f * noise * noise;
    float emax = 0.f;
    for (int q0 = warp; q0 < n; q0 += nwarps) {
        if (c.cstart[q0] != q0 || q0 + 1 >= n || c.cstart[q0 + 1] != q0) continue;
        int k = 2;
        while (q0 + k < n && c.cstart[q0 + k] == q0) ++k;
        const float2 lref = lam[c.order[q0]];
        cx<float> *T = c.T + (size_t)q0 * c.ldt + q0;
        const int ldt = c.ldt;
        for (int sweep = 0; sweep < 16; ++sweep) {
            int nrot = 0;
            for (int p = 0; p < k - 1; ++p) {
                for (int q = p + 1; q < k; ++q) {
                    const cx<float> apq = T[(size_t)p * ldt + q];
                    const float mag2 = cabs2(apq);
                    if (!(mag2 > noise * noise)) continue;
                    JRot<float> R;
                    float na, nb;
                    jacobi_rotation<float>(T[(size_t)p * ldt + p].re, T[(size_t)q * ldt + q].re,
                                           apq, noise, p, q, R, na, nb);
                    ++nrot;
                    if (mag2 > big2) emax = fmaxf(emax, fmaxf(fabsf(R.sr), fabsf(R.si)));
                    const cx<float> s = mk<float>(R.sr, R.si);
                    // rows p and q of G^H T (columns other than p, q), mirrored
                    for (int col = lane; col < k; col += 32) {
                        if (col == p || col == q) continue;
                        const cx<float> tp = T[(size_t)p * ldt + col], tq = T[(size_t)q * ldt + col];
                        const cx<float> np = cadd(cscale(R.c, tp), cscale(-1.0f, cmul(s, tq)));
                        const cx<float> nq = cadd(cmulc(s, tp), cscale(R.c, tq));
                        T[(size_t)p * ldt + col] = np;
                        T[(size_t)q * ldt + col] = nq;
                        T[(size_t)col * ldt + p] = conj(np);
                        T[(size_t)col * ldt + q] = conj(nq);
                    }
                    // X <- X G on the two levels' columns
                    const int i = c.order[q0 + p], j = c.order[q0 + q];
                    for (int r = lane; r < nrows; r += 32) {
                        const cx<float> x = X[(size_t)r * ldx + i], y = X[(size_t)r * ldx + j];
                        X[(size_t)r * ldx + i] = cadd(cscale(R.c, x), cscale(-1.0f, cmulc(s, y)));
                        X[(size_t)r * ldx + j] = cadd(cmul(s, x), cscale(R.c, y));
                    }
                    __syncwarp();
                    if (lane == 0) {
                        T[(size_t)p * ldt + p] = mk<float>(na, 0.f);
                        T[(size_t)q * ldt + q] = mk<float>(nb, 0.f);
                        T[(size_t)p * ldt + q] = mk<float>(0.f, 0.f);
                        T[(size_t)q * ldt + p] = mk<float>(0.f, 0.f);
                    }
                    __syncwarp();
                }
            }
            if (nrot == 0) break;
        }
        for (int p = lane; p < k; p += 32)
            lam[c.order[q0 + p]] = dw_add_f(lref, T[(size_t)p * ldt + p].re);
        __syncwarp();
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x)
        if (!oa_in_cluster(c.cstart, n, r))
            lam[c.order[r]] = dw_add_f(lam[c.order[r]], corr[c.order[r]]);
    __syncthreads();
    return emax;
}

}  // namespace msp
