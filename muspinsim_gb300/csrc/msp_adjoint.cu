// Adjoint of the fast-path powder average (K6): dL/dHsys and dL/dB_lab for
// an upstream gradient g(t) = dL/dP(t).  The reference has no gradient (its
// fitting differentiates muspinsim/fitting.py:67-179 by re-running the
// simulation); this is the analytic derivative of the quantity computed by
// Hamiltonian.fast_evolve (muspinsim/hamiltonian.py:166-217) per snapshot.
//
// Per snapshot, with S = (p . sigma) (x) 1_d, H = U diag(l) U^H,
// M = U^H S U and E_a(t) = e^{2 pi i l_a t}:
//   P(t) = kappa Tr(S V S V^H),  V = e^{2 pi i H t},  kappa = wscale / (4 d),
//   dL = 2 kappa Re sum_bc dH'_bc K_bc,  dH' = U^H dH U,
//   K_bc = sum_a M_ca M_ab D_abc,
//   D_abc = sum_t g(t) (E_b - E_c) E_a^* / (l_b - l_c)
//         = (G(l_b - l_a) - G(l_c - l_a)) / (l_b - l_c),
// where G(nu) = sum_t g(t) e^{2 pi i nu t}; for (near-)equal l_b, l_c the
// divided difference becomes the mean of G'(nu) = sum_t g(t) 2 pi i t
// e^{2 pi i nu t} at the two arguments (the Frechet derivative of the
// exponential: finite at degeneracies).  The Hermitian gradient is
//   dL/dH = U [kappa (conj(K) + K^T)] U^H,  dL/db_a = Re Tr(dL/dH^H Z_a).
#include <math_constants.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "msp_internal.cuh"

namespace msp {

int record_error(int code, const char *msg);

static size_t adj_align(size_t x) { return (x + 255) & ~(size_t)255; }

struct AdjointLayout {
    size_t H, evecs, evals, Gh, Gd, total;
};

static AdjointLayout adjoint_layout(int n, int S) {
    AdjointLayout L;
    const size_t mat = adj_align((size_t)S * n * n * 16);
    size_t off = 0;
    L.H = off;  // assembled H; later the per-snapshot gradients
    off += mat;
    L.evecs = off;
    off += mat;
    L.evals = off;
    off += adj_align((size_t)S * n * 8);
    L.Gh = off;
    off += mat;
    L.Gd = off;
    off += mat;
    L.total = off;
    return L;
}

// G(nu) and G'(nu) for nu = l_b - l_a, a <= b, of every snapshot; one warp
// per (snapshot, a, b), lanes over time samples.  Uniform grids use the
// recurrence e^{i phi_{k+32}} = e^{i phi_k} e^{i 2 pi nu 32 dt}, restarted
// from sincos every 16 steps; arbitrary grids take sincos per sample.
// Fills the full n x n tables: G(-nu) = conj(G(nu)), G'(-nu) = -conj(G'(nu)).
__global__ void msp_adjoint_transform_kernel(const double *__restrict__ evals, int n, int S,
                                             const int *__restrict__ slot,
                                             const double *__restrict__ g, int T, int uniform,
                                             double t0, double dt,
                                             const double *__restrict__ times,
                                             cx<double> *__restrict__ Gh,
                                             cx<double> *__restrict__ Gd) {
    const int lane = threadIdx.x & 31;
    const int warps = (blockDim.x >> 5) * gridDim.x;
    const int ntri = n * (n + 1) / 2;
    const long long items = (long long)S * ntri;
    const double twopi = 6.283185307179586476925;
    for (long long it = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < items;
         it += warps) {
        const int s = (int)(it / ntri);
        const int e = (int)(it - (long long)s * ntri);
        // e -> (b, a), b >= a, e = b (b + 1) / 2 + a
        int b = (int)((sqrt(8.0 * e + 1.0) - 1.0) * 0.5);
        while ((b + 1) * (b + 2) / 2 <= e) ++b;
        while (b * (b + 1) / 2 > e) --b;
        const int a = e - b * (b + 1) / 2;
        const double nu = evals[(size_t)s * n + b] - evals[(size_t)s * n + a];
        const double *gs = g + (size_t)slot[s] * T;
        double hr = 0.0, hi = 0.0, dr = 0.0, di = 0.0;
        if (uniform) {
            double sr, cr;
            sincos(twopi * nu * 32.0 * dt, &sr, &cr);
            int step = 0;
            double er = 1.0, ei = 0.0;
            for (int k = lane; k < T; k += 32, ++step) {
                const double t = t0 + (double)k * dt;
                if ((step & 15) == 0) sincos(twopi * nu * t, &ei, &er);
                const double gv = gs[k];
                hr += gv * er;
                hi += gv * ei;
                dr += gv * t * er;
                di += gv * t * ei;
                const double nr = er * cr - ei * sr;
                ei = er * sr + ei * cr;
                er = nr;
            }
        } else {
            for (int k = lane; k < T; k += 32) {
                const double t = times[k];
                double si, co;
                sincos(twopi * nu * t, &si, &co);
                const double gv = gs[k];
                hr += gv * co;
                hi += gv * si;
                dr += gv * t * co;
                di += gv * t * si;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            hr += __shfl_xor_sync(0xffffffffu, hr, o);
            hi += __shfl_xor_sync(0xffffffffu, hi, o);
            dr += __shfl_xor_sync(0xffffffffu, dr, o);
            di += __shfl_xor_sync(0xffffffffu, di, o);
        }
        if (lane == 0) {
            // G'(nu) = 2 pi i sum t g e^{i ...}
            const cx<double> h = mk<double>(hr, hi);
            const cx<double> d = mk<double>(-twopi * di, twopi * dr);
            const size_t base = (size_t)s * n * n;
            Gh[base + (size_t)a * n + b] = h;
            Gd[base + (size_t)a * n + b] = d;
            if (a != b) {
                Gh[base + (size_t)b * n + a] = conj(h);
                Gd[base + (size_t)b * n + a] = mk<double>(-d.re, d.im);
            }
        }
    }
}

// One CTA per snapshot: M = U^H S U, K, the Hermitian gradient in the
// eigenbasis, back to the lab basis, and its contraction with Z.  Shared
// memory: U, M, W (n x n complex each) and the eigenvalues.
__global__ void msp_adjoint_snap_kernel(int n, int S, const double *__restrict__ evals,
                                        const cx<double> *__restrict__ evecs,
                                        const double *__restrict__ pol,
                                        const double *__restrict__ wscale,
                                        const cx<double> *__restrict__ Gh,
                                        const cx<double> *__restrict__ Gd, double tmax,
                                        const cx<double> *__restrict__ Z,
                                        cx<double> *__restrict__ Gs,
                                        double *__restrict__ grad_field) {
    extern __shared__ __align__(16) char smem[];
    cx<double> *sU = reinterpret_cast<cx<double> *>(smem);
    cx<double> *sM = sU + n * n;
    cx<double> *sW = sM + n * n;
    double *sl = reinterpret_cast<double *>(sW + n * n);
    __shared__ double red[3][33];
    const int tid = threadIdx.x, nt = blockDim.x, d = n / 2;
    const double twopi = 6.283185307179586476925;
    const FastDiv fdn(n);
    for (int s = blockIdx.x; s < S; s += gridDim.x) {
        const cx<double> *Ub = evecs + (size_t)s * n * n;
        for (int e = tid; e < n * n; e += nt) sU[e] = Ub[e];
        for (int i = tid; i < n; i += nt) sl[i] = evals[(size_t)s * n + i];
        __syncthreads();
        // W = S U (Pauli p . sigma on the muon, the slowest digit)
        const double px = pol[3 * (size_t)s], py = pol[3 * (size_t)s + 1],
                     pz = pol[3 * (size_t)s + 2];
        for (int e = tid; e < n * n; e += nt) {
            const int i = fdn.div(e), k = e - i * n;
            cx<double> v;
            if (i < d) {
                const cx<double> x = sU[i * n + k], y = sU[(i + d) * n + k];
                v = mk<double>(pz * x.re + px * y.re + py * y.im, pz * x.im + px * y.im - py * y.re);
            } else {
                const cx<double> x = sU[(i - d) * n + k], y = sU[i * n + k];
                v = mk<double>(px * x.re - py * x.im - pz * y.re, px * x.im + py * x.re - pz * y.im);
            }
            sW[e] = v;
        }
        __syncthreads();
        // M = U^H W
        for (int e = tid; e < n * n; e += nt) {
            const int j = fdn.div(e), k = e - j * n;
            double mr = 0.0, mi = 0.0;
            for (int i = 0; i < n; ++i) {
                const cx<double> u = sU[i * n + j], w = sW[i * n + k];
                mr += u.re * w.re + u.im * w.im;
                mi += u.re * w.im - u.im * w.re;
            }
            sM[e] = mk<double>(mr, mi);
        }
        __syncthreads();
        // K_bc = sum_a M_ca M_ab D_abc; W <- kappa (conj(K) + K^T) needs K_bc
        // and K_cb: compute K into W first
        const cx<double> *gh = Gh + (size_t)s * n * n, *gd = Gd + (size_t)s * n * n;
        for (int e = tid; e < n * n; e += nt) {
            const int b = fdn.div(e), c = e - b * n;
            const double gap = sl[b] - sl[c];
            const bool dd = fabs(twopi * tmax * gap) > 1e-5;
            const double inv = dd ? 1.0 / gap : 0.0;
            double kr = 0.0, ki = 0.0;
            for (int a = 0; a < n; ++a) {
                cx<double> D;
                if (dd) {
                    const cx<double> x = gh[a * n + b], y = gh[a * n + c];
                    D = mk<double>((x.re - y.re) * inv, (x.im - y.im) * inv);
                } else {
                    const cx<double> x = gd[a * n + b], y = gd[a * n + c];
                    D = mk<double>(0.5 * (x.re + y.re), 0.5 * (x.im + y.im));
                }
                const cx<double> p = cmul(sM[c * n + a], sM[a * n + b]);
                kr += p.re * D.re - p.im * D.im;
                ki += p.re * D.im + p.im * D.re;
            }
            sW[e] = mk<double>(kr, ki);
        }
        __syncthreads();
        const double kappa = wscale[s] / (4.0 * d);
        // G' = kappa (conj(K) + K^T) into M (M no longer needed)
        for (int e = tid; e < n * n; e += nt) {
            const int b = fdn.div(e), c = e - b * n;
            const cx<double> k1 = sW[b * n + c], k2 = sW[c * n + b];
            sM[e] = mk<double>(kappa * (k1.re + k2.re), kappa * (k2.im - k1.im));
        }
        __syncthreads();
        // W = G' U^H
        for (int e = tid; e < n * n; e += nt) {
            const int b = fdn.div(e), j = e - b * n;
            double wr = 0.0, wi = 0.0;
            for (int c = 0; c < n; ++c) {
                const cx<double> gv = sM[b * n + c], u = sU[j * n + c];  // (U^H)_cj = conj(U_jc)
                wr += gv.re * u.re + gv.im * u.im;
                wi += gv.im * u.re - gv.re * u.im;
            }
            sW[e] = mk<double>(wr, wi);
        }
        __syncthreads();
        // G = U W -> global; contraction with Z
        double z0 = 0.0, z1 = 0.0, z2 = 0.0;
        cx<double> *Go = Gs + (size_t)s * n * n;
        const size_t nn = (size_t)n * n;
        for (int e = tid; e < n * n; e += nt) {
            const int i = fdn.div(e), j = e - i * n;
            double gr = 0.0, gi = 0.0;
            for (int b = 0; b < n; ++b) {
                const cx<double> u = sU[i * n + b], w = sW[b * n + j];
                gr += u.re * w.re - u.im * w.im;
                gi += u.re * w.im + u.im * w.re;
            }
            Go[e] = mk<double>(gr, gi);
            const cx<double> za = Z[e], zb = Z[nn + e], zc = Z[2 * nn + e];
            z0 += gr * za.re + gi * za.im;
            z1 += gr * zb.re + gi * zb.im;
            z2 += gr * zc.re + gi * zc.im;
        }
        if (grad_field) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                z0 += __shfl_xor_sync(0xffffffffu, z0, o);
                z1 += __shfl_xor_sync(0xffffffffu, z1, o);
                z2 += __shfl_xor_sync(0xffffffffu, z2, o);
            }
            if ((tid & 31) == 0) {
                red[0][tid >> 5] = z0;
                red[1][tid >> 5] = z1;
                red[2][tid >> 5] = z2;
            }
            __syncthreads();
            if (tid < 3) {
                double v = 0.0;
                for (int w = 0; w < (nt >> 5); ++w) v += red[tid][w];
                grad_field[3 * (size_t)s + tid] = v;
            }
        }
        __syncthreads();
    }
}

// grad[e] = sum_s Gs[s][e] in snapshot order per warp, then warp order.
#define MSP_ADJ_SUM_WARPS 8
__global__ void __launch_bounds__(32 * MSP_ADJ_SUM_WARPS)
    msp_adjoint_sum_kernel(const double *__restrict__ Gs, int S, int len,
                           double *__restrict__ out) {
    __shared__ double red[MSP_ADJ_SUM_WARPS][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int e = blockIdx.x * 32 + lane;
    double v = 0.0;
    if (e < len)
        for (int s = warp; s < S; s += MSP_ADJ_SUM_WARPS) v += Gs[(size_t)s * len + e];
    red[warp][lane] = v;
    __syncthreads();
    if (warp == 0 && e < len) {
        double t = 0.0;
        for (int w = 0; w < MSP_ADJ_SUM_WARPS; ++w) t += red[w][lane];
        out[e] = t;
    }
}

}  // namespace msp

using namespace msp;

static int adj_fail(int code, const char *msg) { return record_error(code, msg); }

static int adj_check(const msp_adjoint_args *a) {
    if (a == NULL) return adj_fail(MSP_ERR_ARG, "msp_adjoint: args is NULL");
    if (a->n < 2 || (a->n & 1)) return adj_fail(MSP_ERR_ARG, "msp_adjoint: n must be even and >= 2");
    if (a->n > MSP_MAX_DIM) return adj_fail(MSP_ERR_UNSUPPORTED, "msp_adjoint: n exceeds MSP_MAX_DIM");
    if (a->num_snap < 0 || a->num_slots < 1)
        return adj_fail(MSP_ERR_ARG, "msp_adjoint: num_snap < 0 or num_slots < 1");
    if (a->num_times < 1) return adj_fail(MSP_ERR_ARG, "msp_adjoint: num_times < 1");
    if (!a->uniform && a->times == NULL)
        return adj_fail(MSP_ERR_ARG, "msp_adjoint: times is NULL on a non-uniform grid");
    return MSP_OK;
}

static int adj_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return MSP_OK;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return adj_fail(MSP_ERR_CUDA, buf);
}

extern "C" {

int msp_adjoint_workspace(const msp_adjoint_args *a, size_t *bytes) {
    const int rc = adj_check(a);
    if (rc != MSP_OK) return rc;
    if (bytes == NULL) return adj_fail(MSP_ERR_ARG, "msp_adjoint_workspace: bytes is NULL");
    *bytes = adjoint_layout(a->n, a->num_snap).total;
    return MSP_OK;
}

int msp_adjoint_fast(const msp_adjoint_args *a) {
    int rc = adj_check(a);
    if (rc != MSP_OK) return rc;
    if (a->grad_hsys == NULL) return adj_fail(MSP_ERR_ARG, "msp_adjoint: grad_hsys is NULL");
    const int n = a->n, S = a->num_snap;
    cudaStream_t st = (cudaStream_t)a->stream;
    if (S == 0) return adj_cuda(cudaMemsetAsync(a->grad_hsys, 0, (size_t)n * n * 16, st),
                                "msp_adjoint");
    if (!a->Hsys || !a->Z || !a->field || !a->pol || !a->wscale || !a->slot || !a->grad_out ||
        !a->status)
        return adj_fail(MSP_ERR_ARG, "msp_adjoint: a required pointer is NULL");
    const AdjointLayout L = adjoint_layout(n, S);
    if (a->workspace == NULL || a->workspace_bytes < L.total)
        return adj_fail(MSP_ERR_WORKSPACE, "msp_adjoint: workspace too small");
    if (reinterpret_cast<uintptr_t>(a->workspace) & 255)
        return adj_fail(MSP_ERR_ARG, "msp_adjoint: workspace not 256-byte aligned");
    char *ws = reinterpret_cast<char *>(a->workspace);
    double *H = reinterpret_cast<double *>(ws + L.H);
    double *V = reinterpret_cast<double *>(ws + L.evecs);
    double *lam = reinterpret_cast<double *>(ws + L.evals);
    cx<double> *Gh = reinterpret_cast<cx<double> *>(ws + L.Gh);
    cx<double> *Gd = reinterpret_cast<cx<double> *>(ws + L.Gd);

    rc = adj_cuda(launch_assemble(a->Hsys, a->Z, a->field, n, S, H, st), "msp_adjoint assemble");
    if (rc != MSP_OK) return rc;
    rc = adj_cuda(launch_eigh(H, n, S, MSP_PREC_FP64, a->max_sweeps > 0 ? a->max_sweeps : 40, lam,
                              V, a->status, st),
                  "msp_adjoint eigh");
    if (rc != MSP_OK) return rc;

    // largest |t| of the grid (the divided-difference switch)
    double tmax = 0.0;
    if (a->uniform) {
        tmax = fmax(fabs(a->t0), fabs(a->t0 + (a->num_times - 1) * a->dt));
    } else {
        tmax = 0.0;  // filled from the host copy below
        double *th = (double *)malloc((size_t)a->num_times * sizeof(double));
        if (th == NULL) return adj_fail(MSP_ERR_ARG, "msp_adjoint: host allocation failed");
        cudaError_t e = cudaMemcpyAsync(th, a->times, (size_t)a->num_times * 8,
                                        cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            free(th);
            return adj_cuda(e, "msp_adjoint times");
        }
        for (int k = 0; k < a->num_times; ++k) tmax = fmax(tmax, fabs(th[k]));
        free(th);
    }

    {
        const long long items = (long long)S * (n * (n + 1) / 2);
        long long blocks = (items + 7) / 8;
        if (blocks > 152 * 16) blocks = 152 * 16;
        msp_adjoint_transform_kernel<<<(int)blocks, 256, 0, st>>>(
            lam, n, S, a->slot, a->grad_out, a->num_times, a->uniform, a->t0, a->dt, a->times, Gh,
            Gd);
        rc = adj_cuda(cudaGetLastError(), "msp_adjoint_transform");
        if (rc != MSP_OK) return rc;
    }
    cx<double> *Gs = reinterpret_cast<cx<double> *>(H);  // H is consumed
    {
        const size_t smem = (size_t)3 * n * n * 16 + (size_t)n * 8;
        rc = adj_cuda(cudaFuncSetAttribute(msp_adjoint_snap_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "msp_adjoint_snap attribute");
        if (rc != MSP_OK) return rc;
        const int grid = S < 152 * 8 ? S : 152 * 8;
        msp_adjoint_snap_kernel<<<grid, n <= 16 ? 64 : 128, smem, st>>>(
            n, S, lam, reinterpret_cast<const cx<double> *>(V), a->pol, a->wscale, Gh, Gd, tmax,
            reinterpret_cast<const cx<double> *>(a->Z), Gs, a->grad_field);
        rc = adj_cuda(cudaGetLastError(), "msp_adjoint_snap");
        if (rc != MSP_OK) return rc;
    }
    {
        const int len = 2 * n * n;
        msp_adjoint_sum_kernel<<<(len + 31) / 32, 32 * MSP_ADJ_SUM_WARPS, 0, st>>>(
            reinterpret_cast<const double *>(Gs), S, len, a->grad_hsys);
        rc = adj_cuda(cudaGetLastError(), "msp_adjoint_sum");
    }
    return rc;
}

}  // extern "C"
