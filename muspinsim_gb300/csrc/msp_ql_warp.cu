// FP32 Householder + implicit-shift QL eigensolver for batches of n <= 32
// Hamiltonians: the first stage of the MIXED snapshot pipeline (the
// alternative to msp_jacobi_warp.cu's cyclic Jacobi), replacing the FP32
// part of Hermitian.diag's eigensolve (muspinsim/spinop.py:51-82) for the
// batched snapshots of ExperimentRunner (muspinsim/experiment.py:332-341,
// 434-498).  The second stage (msp_snap.cu, PRE variants) refines the
// eigenvectors this kernel leaves in scratch, exactly as it refines the
// Jacobi's.
//
// The algorithm is msp_large.cuh's (LAPACK zhetd2 tridiagonalisation of the
// lower triangle, EISPACK tql2 QL with the rotations accumulated into a real
// Z, back-transformation U = Q Z).  A warp takes G matrices at a time:
//   1. two matrices at a time, one warp, their steps interleaved
//      instruction by instruction (each step is a chain of warp reductions
//      and shared-memory round trips; two independent chains fill each
//      other's latency: 0.54 -> 0.52 ms on the headline): A (full
//      Hermitian, row-major, row stride NM + 1 float2 so that column and
//      row walks are both free of bank conflicts) in shared memory, both
//      matrices side by side in the region the Z matrices later take.
//      Step k: lane i holds x_i = A[k+1+i][k]; the reflector v_k (v_0 = 1)
//      replaces column k of A, zero outside rows k+1 .. n-1, and is parked
//      as row k of the snapshot's eigenvector scratch; p = tau A22 v and the
//      rank-2 update A22 -= v w^H + w v^H are column-parallel (lane i owns
//      column k+1+i; v_j, w_j are warp broadcasts).  d, e and tau stay in
//      shared memory.
//   2. the G QL runs side by side, 32 / G lanes per matrix: a QL step's
//      shift and rotation chain are serial, so each lane group computes its
//      own matrix's chain (its lanes redundantly) and applies every rotation
//      to its rows of Z (column-major in shared memory, aliasing A).  The
//      groups advance one QL step per round; a round waits for the longest
//      chain, which on the 24 x 24 powder Hamiltonians (513 .. 613 rotations
//      in 45 .. 49 steps) costs under 10% over the groups' own work.  The
//      reciprocal square root of each rotation is the hardware
//      approximation plus one Newton step.
//   3. per matrix, one warp: lane j holds column j of U = Q Z in registers
//      and applies the parked reflectors last to first, s = v^H u,
//      u -= v (tau s), skipping the four-row groups where v is zero; U
//      overwrites the reflectors in the scratch.
// The FP32 eigenvectors only have to be orthonormal to FP32 rounding; the
// refinement stage restores full accuracy and resolves clusters.
#include "msp_internal.cuh"
#include "msp_large.cuh"

namespace msp {

namespace {

constexpr int QW_WARPS = 2;  // warps per CTA

// Per-warp shared memory for a batch of G matrices up to NM x NM (NM a
// multiple of 8): region R holds the two working matrices A (NM x (NM + 1)
// float2 each) while matrices are tridiagonalised and the G matrices Z_g
// (NM x (NM + 1) floats each) from the QL on; then per matrix d, e (NM
// floats each) and tau (NM float2); then the two v/w pair buffers (NM
// float4 each).
template <int NM, int G>
struct QwShape {
    static constexpr int LDA = NM + 1;  // float2
    static constexpr int LDZ = NM + 1;  // float
    static constexpr int A_BYTES = 8 * NM * LDA;
    static constexpr int Z_FLOATS = NM * LDZ;  // one matrix
    static constexpr int A_F2 = NM * LDA;  // float2 of one working matrix
    static constexpr int R_BYTES =
        (2 * A_BYTES > 4 * G * Z_FLOATS ? 2 * A_BYTES : 4 * G * Z_FLOATS + 15) / 16 * 16;
    static constexpr int DEV_BYTES = 16 * NM;  // d, e, tau of one matrix
    static constexpr int BYTES = R_BYTES + G * DEV_BYTES + 32 * NM;
    static constexpr int LPM = 32 / G;              // lanes per matrix in the QL
    static constexpr int RPL = (NM + LPM - 1) / LPM;  // rows of Z per lane
    // CTAs per SM that the shared memory allows (1 KB reserved per CTA),
    // capped where registers would fall below ~96 a thread
    static constexpr int CTAS = (227 * 1024) / (QW_WARPS * BYTES + 1024);
    static constexpr int REG_CTAS = 65536 / (QW_WARPS * 32 * 96);
    static constexpr int MINB = CTAS < 1 ? 1 : (CTAS > REG_CTAS ? REG_CTAS : CTAS);
    static_assert(NM % 8 == 0 && NM <= 32, "NM: a multiple of 8 up to 32");
    static_assert(G == 1 || G == 2 || G == 4 || G == 8, "G divides 32");
    static_assert(A_BYTES % 16 == 0 && BYTES % 16 == 0, "alignment");
};

}  // namespace

template <int NM, int G>
__global__ void __launch_bounds__(QW_WARPS * 32, QwShape<NM, G>::MINB)
    msp_ql_warp_kernel(SnapArgs a) {
    using S = QwShape<NM, G>;
    constexpr int LDA = S::LDA, LDZ = S::LDZ, LPM = S::LPM, RPL = S::RPL;
    extern __shared__ __align__(16) char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    char *mine = smem + (size_t)warp * S::BYTES;
    float2 *const A = reinterpret_cast<float2 *>(mine);  // phase 1
    float *const Zb = reinterpret_cast<float *>(mine);   // phases 2, 3
    char *const devb = mine + S::R_BYTES;
    float4 *const vw = reinterpret_cast<float4 *>(devb + G * S::DEV_BYTES);
    auto dptr = [&](int q) { return reinterpret_cast<float *>(devb + q * S::DEV_BYTES); };

    const int n = a.n;
    const int nn = n * n;
    float2 *evec = reinterpret_cast<float2 *>(a.evec);
    const int ntask = (a.num_snap + G - 1) / G;
    for (int task = blockIdx.x * QW_WARPS + warp; task < ntask; task += gridDim.x * QW_WARPS) {
        const int sn0 = task * G;
        const int cnt = min(G, a.num_snap - sn0);

        // ---- 1. two matrices at a time (their steps interleaved instruction
        // by instruction): H, tridiagonalisation.  A missing second matrix
        // (odd count) is zero: no reflections, nothing stored for it.
        for (int q0 = 0; q0 < cnt; q0 += 2) {
            const bool has1 = q0 + 1 < cnt;
            float2 *Ap[2] = {A, A + S::A_F2};
            float4 *vwp[2] = {vw, vw + NM};
            float *dsp[2], *esp[2];
            float2 *tp[2], *Vtp[2];
            SnapSource src[2];
            double bx[2], by[2], bz[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int q = q0 + u;
                dsp[u] = dptr(q);
                esp[u] = dsp[u] + NM;
                tp[u] = reinterpret_cast<float2 *>(esp[u] + NM);
                const int sn = (u == 0 || has1) ? sn0 + q : sn0 + q0;
                Vtp[u] = evec + (size_t)sn * nn;
                src[u] = snap_source(a, sn);
                bx[u] = a.field[3 * (size_t)src[u].g];
                by[u] = a.field[3 * (size_t)src[u].g + 1];
                bz[u] = a.field[3 * (size_t)src[u].g + 2];
            }
            // H = Hsys + b . Z in FP32 (from the double-word high parts when
            // the caller pre-split the matrices, else from FP64), upper
            // triangle mirrored; rows and columns n .. NM-1 zero
            for (int e = lane; e < NM * (NM + 1) / 2; e += 32) {
                int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);  // e = i (i + 1) / 2 + j
                while ((i + 1) * (i + 2) / 2 <= e) ++i;
                while (i * (i + 1) / 2 > e) --i;
                const int j = e - i * (i + 1) / 2;  // j <= i: element (j, i)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    float hr = 0.f, hi = 0.f;
                    if (i < n && (u == 0 || has1)) {
                        const size_t o = (size_t)j * n + i;
                        if (src[u].Hdw != nullptr) {
                            const float bxf = (float)bx[u], byf = (float)by[u], bzf = (float)bz[u];
                            const float4 hs = src[u].Hdw[o], z0 = src[u].Zdw[o],
                                         z1 = src[u].Zdw[nn + o], z2 = src[u].Zdw[2 * (size_t)nn + o];
                            hr = fmaf(bzf, z2.x, fmaf(byf, z1.x, fmaf(bxf, z0.x, hs.x)));
                            hi = fmaf(bzf, z2.y, fmaf(byf, z1.y, fmaf(bxf, z0.y, hs.y)));
                        } else {
                            const cx<double> hs = src[u].Hsys[o], z0 = src[u].Z[o],
                                             z1 = src[u].Z[nn + o], z2 = src[u].Z[2 * (size_t)nn + o];
                            hr = (float)(hs.re + bx[u] * z0.re + by[u] * z1.re + bz[u] * z2.re);
                            hi = (float)(hs.im + bx[u] * z0.im + by[u] * z1.im + bz[u] * z2.im);
                        }
                    }
                    if (i == j) {
                        Ap[u][i * LDA + i] = make_float2(hr, 0.f);
                    } else {
                        Ap[u][j * LDA + i] = make_float2(hr, hi);
                        Ap[u][i * LDA + j] = make_float2(hr, -hi);
                    }
                }
            }
            __syncwarp();

            // d, e, tau; reflector k into column k of A and row k of the
            // eigenvector scratch.  A step without a reflection (tau = 0)
            // runs the updates too: they add exact zeros.
            for (int k = 0; k + 1 < n; ++k) {
                const int m = n - k - 1;  // length of x
                float2 xi[2];
                float dk[2], xn2[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    xi[u] = lane < m ? Ap[u][(k + 1 + lane) * LDA + k] : make_float2(0.f, 0.f);
                    dk[u] = Ap[u][k * LDA + k].x;
                    xn2[u] = lane >= 1 ? xi[u].x * xi[u].x + xi[u].y * xi[u].y : 0.f;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                    for (int u = 0; u < 2; ++u) xn2[u] += __shfl_xor_sync(0xffffffffu, xn2[u], o);
                }
                float beta[2];
                cx<float> tau[2], vi[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float2 alpha = make_float2(__shfl_sync(0xffffffffu, xi[u].x, 0),
                                                     __shfl_sync(0xffffffffu, xi[u].y, 0));
                    const bool reflect = !(xn2[u] == 0.f && alpha.y == 0.f);
                    const float br =
                        -copysignf(sqrtf(alpha.x * alpha.x + alpha.y * alpha.y + xn2[u]), alpha.x);
                    const cx<float> tr = mk<float>((br - alpha.x) / br, -alpha.y / br);
                    // v = x / (alpha - beta), v_0 = 1
                    const float dr = alpha.x - br, di = alpha.y;
                    const float dd = 1.f / (dr * dr + di * di);
                    const cx<float> vr = cmul(mk<float>(xi[u].x, xi[u].y), mk<float>(dr * dd, -di * dd));
                    beta[u] = reflect ? br : alpha.x;
                    tau[u] = reflect ? tr : mk<float>(0.f, 0.f);
                    vi[u] = lane == 0 ? mk<float>(1.f, 0.f)
                                      : (reflect ? vr : mk<float>(0.f, 0.f));
                }
                __syncwarp();  // column k (x, A[k][k]) read by every lane
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    // column k <- v, zero outside rows k+1 .. n-1
                    const int src_lane = (lane - k - 1) & 31;
                    const float vr = __shfl_sync(0xffffffffu, vi[u].re, src_lane);
                    const float vim = __shfl_sync(0xffffffffu, vi[u].im, src_lane);
                    const float2 vv =
                        (lane > k && lane < n) ? make_float2(vr, vim) : make_float2(0.f, 0.f);
                    if (lane < NM) Ap[u][lane * LDA + k] = vv;
                    if (lane < n && (u == 0 || has1)) Vtp[u][(size_t)k * n + lane] = vv;
                    if (lane == 0) {
                        dsp[u][k] = dk[u];
                        esp[u][k] = beta[u];
                        tp[u][k] = make_float2(tau[u].re, tau[u].im);
                    }
                }
                __syncwarp();
                // p_i = tau sum_j conj(A22[j][i]) v_j (A22 Hermitian), lane i
                // owns column k+1+i
                cx<float> pi[2] = {mk<float>(0.f, 0.f), mk<float>(0.f, 0.f)};
                if (lane < m) {
                    float r0[2] = {0.f, 0.f}, i0[2] = {0.f, 0.f}, r1[2] = {0.f, 0.f},
                          i1[2] = {0.f, 0.f};
                    int j = 0;
                    for (; j + 1 < m; j += 2) {
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const float2 *col = Ap[u] + (k + 1) * LDA + (k + 1 + lane);
                            const float2 *vk = Ap[u] + (k + 1) * LDA + k;
                            const float2 a0 = col[j * LDA], a1 = col[(j + 1) * LDA];
                            const float2 v0 = vk[j * LDA], v1 = vk[(j + 1) * LDA];
                            r0[u] += a0.x * v0.x + a0.y * v0.y;
                            i0[u] += a0.x * v0.y - a0.y * v0.x;
                            r1[u] += a1.x * v1.x + a1.y * v1.y;
                            i1[u] += a1.x * v1.y - a1.y * v1.x;
                        }
                    }
                    if (j < m) {
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const float2 a0 = Ap[u][(k + 1 + j) * LDA + (k + 1 + lane)];
                            const float2 v0 = Ap[u][(k + 1 + j) * LDA + k];
                            r0[u] += a0.x * v0.x + a0.y * v0.y;
                            i0[u] += a0.x * v0.y - a0.y * v0.x;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 2; ++u)
                        pi[u] = cmul(tau[u], mk<float>(r0[u] + r1[u], i0[u] + i1[u]));
                }
                // alpha2 = -1/2 tau (p^H v); w = p + alpha2 v
                float hr[2], hi[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const cx<float> pv = lane < m ? cmulc(pi[u], vi[u]) : mk<float>(0.f, 0.f);
                    hr[u] = pv.re;
                    hi[u] = pv.im;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        hr[u] += __shfl_xor_sync(0xffffffffu, hr[u], o);
                        hi[u] += __shfl_xor_sync(0xffffffffu, hi[u], o);
                    }
                }
                cx<float> wi[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const cx<float> a2 = cscale(-0.5f, cmul(tau[u], mk<float>(hr[u], hi[u])));
                    wi[u] = cadd(pi[u], cmul(a2, vi[u]));
                    if (lane < m) vwp[u][lane] = make_float4(vi[u].re, vi[u].im, wi[u].re, wi[u].im);
                }
                __syncwarp();
                // A22[j][i] -= v_j conj(w_i) + w_j conj(v_i), lane i owns column i
                if (lane < m) {
                    for (int j = 0; j < m; ++j) {
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            float2 *cp = Ap[u] + (k + 1 + j) * LDA + (k + 1 + lane);
                            const float4 qv = vwp[u][j];
                            const float2 x = *cp;
                            const float tr = qv.x * wi[u].re + qv.y * wi[u].im + qv.z * vi[u].re +
                                             qv.w * vi[u].im;
                            const float ti = qv.y * wi[u].re - qv.x * wi[u].im + qv.w * vi[u].re -
                                             qv.z * vi[u].im;
                            *cp = make_float2(x.x - tr, x.y - ti);
                        }
                    }
                }
                __syncwarp();
            }
            if (lane == 0) {
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    dsp[u][n - 1] = Ap[u][(n - 1) * LDA + (n - 1)].x;
                    esp[u][n - 1] = 0.f;
                }
            }
            __syncwarp();  // A is reused by the next pair, then by Z
        }

        // ---- 2. QL with implicit shifts (tql2) on the G matrices side by
        // side: lane group g (LPM lanes) runs matrix g; Z_g = I
        for (int e = lane; e < G * S::Z_FLOATS; e += 32) Zb[e] = 0.f;
        __syncwarp();
        for (int e = lane; e < G * NM; e += 32) {
            const int q = e / NM, i = e - q * NM;
            if (i < n) Zb[q * S::Z_FLOATS + i * LDZ + i] = 1.f;
        }
        __syncwarp();
        const int g = lane / LPM, sub = lane - g * LPM;
        const unsigned gmask = LPM == 32 ? 0xffffffffu : (((1u << (LPM & 31)) - 1u) << (g * LPM));
        int status = MSP_ITEM_OK;
        {
            float *const ds = dptr(g);
            float *const es = ds + NM;
            float *const Zg = Zb + g * S::Z_FLOATS;
            const float eps = 1.1920928955078125e-7f;  // 2^-23
            bool done = g >= cnt;
            int l = 0, iter = 0;
            float f = 0.f, tst = 0.f;
            for (;;) {
                // deflate converged levels; m: the first index >= l whose
                // coupling is negligible (n - 1 at the latest)
                int m = l;
                if (!done) {
                    for (;;) {
                        if (iter == 0) tst = fmaxf(tst, fabsf(ds[l]) + fabsf(es[l]));
                        m = l;
                        while (m < n - 1 && fabsf(es[m]) > eps * tst) ++m;
                        if (m != l && iter < 60) break;
                        if (m != l) status = MSP_ITEM_NOT_CONVERGED;
                        __syncwarp(gmask);
                        if (sub == 0) {
                            ds[l] += f;
                            es[l] = 0.f;
                        }
                        __syncwarp(gmask);
                        iter = 0;
                        if (++l >= n) {
                            done = true;
                            break;
                        }
                    }
                }
                if (__all_sync(0xffffffffu, done)) break;
                if (!done) {
                    ++iter;
                    const float g0 = ds[l], el = es[l], el1 = es[l + 1];
                    const float qs = (ds[l + 1] - g0) / (2.f * el);
                    const float r0 = hypotf(qs, 1.f);
                    const float t1 = qs + copysignf(r0, qs);
                    const float dl = el / t1, dl1 = el * t1;
                    const float h = g0 - dl;
                    f += h;
                    __syncwarp(gmask);  // every lane of the group has read d and e
                    if (sub == 0) {
                        ds[l] = dl;
                        ds[l + 1] = dl1;
                    }
                    for (int i = l + 2 + sub; i < n; i += LPM) ds[i] -= h;
                    __syncwarp(gmask);
                    float pp = ds[m];
                    float c = 1.f, c2 = 1.f, c3 = 1.f, s = 0.f, s2 = 0.f;
                    // this lane's rows of Z: r = sub + LPM t
                    float hc[RPL], zi[RPL];
#pragma unroll
                    for (int t = 0; t < RPL; ++t) {
                        const int r = sub + LPM * t;
                        hc[t] = r < n ? Zg[m * LDZ + r] : 0.f;
                        zi[t] = r < n ? Zg[(m - 1) * LDZ + r] : 0.f;
                    }
                    float ei = es[m - 1], di = ds[m - 1];
                    for (int i = m - 1; i >= l; --i) {
                        // operands of the next rotation: written by this chain
                        // only after they are read
                        const int ip = max(i - 1, l);
                        const float ein = es[ip], din = ds[ip];
                        float zin[RPL];
#pragma unroll
                        for (int t = 0; t < RPL; ++t) {
                            const int r = sub + LPM * t;
                            zin[t] = r < n ? Zg[ip * LDZ + r] : 0.f;
                        }
                        c3 = c2;
                        c2 = c;
                        s2 = s;
                        const float gq = c * ei, hh = c * pp;
                        const float x2 = fmaf(pp, pp, ei * ei);
                        float r, cn, sn;
                        if (x2 > 1e-36f && x2 < 1e36f) {
                            const float y = rsqrt_newton<float>(x2);
                            r = x2 * y;
                            sn = ei * y;
                            cn = pp * y;
                        } else {
                            r = hypotf(pp, ei);
                            sn = ei / r;
                            cn = pp / r;
                        }
                        es[i + 1] = s * r;
                        s = sn;
                        c = cn;
                        pp = c * di - s * gq;
                        ds[i + 1] = hh + s * (c * gq + s * di);
#pragma unroll
                        for (int t = 0; t < RPL; ++t) {
                            const int rr = sub + LPM * t;
                            if (rr < n) Zg[(i + 1) * LDZ + rr] = s * zi[t] + c * hc[t];
                            hc[t] = c * zi[t] - s * hc[t];
                            zi[t] = zin[t];
                        }
                        ei = ein;
                        di = din;
                    }
#pragma unroll
                    for (int t = 0; t < RPL; ++t) {
                        const int r = sub + LPM * t;
                        if (r < n) Zg[l * LDZ + r] = hc[t];
                    }
                    pp = -s * s2 * c3 * el1 * el / dl1;
                    __syncwarp(gmask);
                    if (sub == 0) {
                        es[l] = s * pp;
                        ds[l] = c * pp;
                    }
                    __syncwarp(gmask);
                }
                __syncwarp();
            }
        }

        // ---- 3. per matrix: U = Q Z, lane j holds column j of U
        for (int q = 0; q < cnt; ++q) {
            const int sn = sn0 + q;
            const int status_q = __shfl_sync(0xffffffffu, status, q * LPM);
            const float *Zq = Zb + q * S::Z_FLOATS;
            const float2 *taus = reinterpret_cast<const float2 *>(dptr(q) + 2 * NM);
            float2 *const Vt = evec + (size_t)sn * nn;
            cx<float> u[NM];
#pragma unroll
            for (int i = 0; i < NM; ++i)
                u[i] = mk<float>(lane < n && i < n ? Zq[lane * LDZ + i] : 0.f, 0.f);
            for (int k = n - 2; k >= 0; --k) {
                const float2 tk = taus[k];
                if (tk.x == 0.f && tk.y == 0.f) continue;  // the same in every lane
                const float2 *vk = Vt + (size_t)k * n;
                // s = v^H u over the four-row groups that hold part of v
                // (rows k+1 .. n-1)
                float sr0 = 0.f, si0 = 0.f, sr1 = 0.f, si1 = 0.f;
#pragma unroll
                for (int gq = 0; gq < NM / 4; ++gq) {
                    if (4 * gq + 3 > k && 4 * gq < n) {
#pragma unroll
                        for (int t = 0; t < 4; t += 2) {
                            const int i = 4 * gq + t;
                            const float2 v0 = i < n ? vk[i] : make_float2(0.f, 0.f);
                            const float2 v1 = i + 1 < n ? vk[i + 1] : make_float2(0.f, 0.f);
                            sr0 += v0.x * u[i].re + v0.y * u[i].im;
                            si0 += v0.x * u[i].im - v0.y * u[i].re;
                            sr1 += v1.x * u[i + 1].re + v1.y * u[i + 1].im;
                            si1 += v1.x * u[i + 1].im - v1.y * u[i + 1].re;
                        }
                    }
                }
                const cx<float> ts = cmul(mk<float>(tk.x, tk.y), mk<float>(sr0 + sr1, si0 + si1));
#pragma unroll
                for (int gq = 0; gq < NM / 4; ++gq) {
                    if (4 * gq + 3 > k && 4 * gq < n) {
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            const int i = 4 * gq + t;
                            const float2 v = i < n ? vk[i] : make_float2(0.f, 0.f);
                            u[i].re -= v.x * ts.re - v.y * ts.im;
                            u[i].im -= v.x * ts.im + v.y * ts.re;
                        }
                    }
                }
            }
            __syncwarp();  // every lane has read the reflectors
            // eigenvectors (columns of U) to scratch, row-major
            if (lane < n) {
#pragma unroll
                for (int i = 0; i < NM; ++i)
                    if (i < n) Vt[(size_t)i * n + lane] = make_float2(u[i].re, u[i].im);
            }
            if (lane == 0) a.status[snap_source(a, sn).g] = status_q;
        }
        __syncwarp();  // R and the per-matrix tables are reused by the next batch
    }
}

template <int NM, int G>
static cudaError_t qw_launch(const SnapArgs &a, cudaStream_t st) {
    using S = QwShape<NM, G>;
    const size_t smem = (size_t)QW_WARPS * S::BYTES;
    cudaError_t e = cudaFuncSetAttribute(msp_ql_warp_kernel<NM, G>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0, sms = 0, dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_ql_warp_kernel<NM, G>,
                                                          QW_WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    const long long tasks = (a.num_snap + G - 1) / G;
    long long grid = (tasks + QW_WARPS - 1) / QW_WARPS;
    const long long cap = (long long)sms * (occ > 0 ? occ : 1);
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    msp_ql_warp_kernel<NM, G><<<(int)grid, QW_WARPS * 32, smem, st>>>(a);
    return cudaGetLastError();
}

bool ql_warp_supported(int n) { return n >= 2 && n <= 32; }

#ifndef QW_G24
#define QW_G24 4
#endif
#ifndef QW_G32
#define QW_G32 4
#endif
cudaError_t launch_ql_warp(const SnapArgs &a, cudaStream_t st) {
    if (a.num_snap <= 0) return cudaSuccess;
    if (a.n <= 8) return qw_launch<8, 8>(a, st);
    if (a.n <= 16) return qw_launch<16, 8>(a, st);
    if (a.n <= 24) return qw_launch<24, QW_G24>(a, st);
    if (a.n <= 32) return qw_launch<32, QW_G32>(a, st);
    return cudaErrorInvalidValue;
}

}  // namespace msp
