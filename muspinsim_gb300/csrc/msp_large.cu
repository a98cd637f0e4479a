// The large-n kernels (64 < n <= MSP_MAX_DIM_LARGE) on the FP64 solver of
// msp_large.cuh -- the eigensolver API, the fast path and the general path
// (EVOLVE / INTEGRAL) -- and the host side of every large-n launch (the
// MIXED fast path's kernel is in msp_large_mixed.cu).
#include "msp_large.cuh"
#include "msp_rho.cuh"

namespace msp {

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

// ------------------------------------------------------------------ general path

// The general path for n > 64 (EVOLVE / INTEGRAL), FP64 in both
// precisions: the large-n counterpart of msp_snap_rho_kernel
// (muspinsim/hamiltonian.py:40-164 with rho0 of muspinsim/experiment.py:
// 170-236).  Per snapshot: rho0's Kronecker factors (shared memory, after
// the solver's), H = Hsys + b . Z, the FP64 solver, rho0 U factor by factor
// (n^2 sum_i d_i), rho'_jk = (U^dag rho0 U)_jk for j >= k, O U on the muon
// digit (O = p . S_mu), O'_kj, then the pair coefficients C_jk =
// rho'_jk O'_kj with their frequencies (EVOLVE) or the decaying integral
// (INTEGRAL).  Scratch: the solver's working set plus two n x n complex
// matrices (ping-pong for rho0 U, and rho').
__host__ __device__ inline size_t large_rho_scratch_doubles(int n) {
    return large_scratch_doubles(n) + (size_t)4 * n * n;
}

__host__ __device__ inline size_t large_rho_fac_offset(int n, int threads) {
    return (large_smem_bytes(n, threads) + 15) & ~size_t(15);
}

// Y = (1 (x) F (x) 1) X on the digit of the given stride and size (n x n,
// row-major, complex)
__device__ void large_apply_digit(const cx<double> *F, int dim, int stride,
                                  const cx<double> *__restrict__ X, cx<double> *__restrict__ Y,
                                  int n) {
    for (size_t e = threadIdx.x; e < (size_t)n * n; e += blockDim.x) {
        const int i = (int)(e / n), k = (int)(e - (size_t)i * n);
        const int di = (i / stride) % dim, base = i - di * stride;
        double yr = 0, yi = 0;
        for (int l = 0; l < dim; ++l) {
            const cx<double> f = F[di * dim + l], x = X[(size_t)(base + l * stride) * n + k];
            yr += f.re * x.re - f.im * x.im;
            yi += f.re * x.im + f.im * x.re;
        }
        Y[e] = mk<double>(yr, yi);
    }
    __syncthreads();
}

template <bool INTEGRAL>
__global__ void msp_large_rho_kernel(SnapArgs a, double *__restrict__ scratch) {
    extern __shared__ __align__(16) char smem[];
    const int n = a.n, P = n * (n - 1) / 2;
    const size_t nn = (size_t)n * n;
    double *base = scratch + (size_t)blockIdx.x * large_rho_scratch_doubles(n);
    LargeScratch s = large_carve(base, n);
    cx<double> *B = reinterpret_cast<cx<double> *>(base + large_scratch_doubles(n));
    cx<double> *R = B + nn;
    cx<double> *fac = reinterpret_cast<cx<double> *>(smem + large_rho_fac_offset(n, blockDim.x));
    const int tid = threadIdx.x, nt = blockDim.x;
    __shared__ double red[32];
    const double twopi = 6.283185307179586476925;
    const size_t ntri = (size_t)n * (n + 1) / 2;
    for (int sn = blockIdx.x; sn < a.num_snap; sn += gridDim.x) {
        if (a.rho_fac) {
            for (int e = tid; e < a.fac_len; e += nt)
                fac[e] = a.rho_fac[(size_t)sn * a.fac_len + e];
        } else {
            build_rho_factors(a, sn, fac);
        }
        const double bx = a.field[3 * (size_t)sn], by = a.field[3 * (size_t)sn + 1],
                     bz = a.field[3 * (size_t)sn + 2];
        for (size_t x = tid; x < nn; x += nt) {
            const cx<double> hs = a.Hsys[x], z0 = a.Z[x], z1 = a.Z[nn + x], z2 = a.Z[2 * nn + x];
            s.A[x] = mk<double>(hs.re + bx * z0.re + by * z1.re + bz * z2.re,
                                hs.im + bx * z0.im + by * z1.im + bz * z2.im);
        }
        __syncthreads();
        const int st = large_eigh(s, n, smem);
        const cx<double> *U = s.U;
        // rho0 U by Kronecker factors: X ping-pongs between A (free now) and B
        const cx<double> *X = U;
        cx<double> *Y = s.A;
        {
            int off = 0;
            for (int sp = 0; sp < a.num_spins; ++sp) {
                const int dim = a.dims[sp];
                large_apply_digit(fac + off, dim, a.strides[sp], X, Y, n);
                off += dim * dim;
                X = Y;
                Y = (Y == s.A) ? B : s.A;
            }
        }
        // rho'_jk = sum_i conj(U_ij) (rho0 U)_ik, j >= k, into R
        for (size_t e = tid; e < ntri; e += nt) {
            int j = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
            while ((size_t)(j + 1) * (j + 2) / 2 <= e) ++j;
            while ((size_t)j * (j + 1) / 2 > e) --j;
            const int k = (int)(e - (size_t)j * (j + 1) / 2);
            double gr = 0, gi = 0;
            for (int i = 0; i < n; ++i) {
                const cx<double> u = U[(size_t)i * n + j], x = X[(size_t)i * n + k];
                gr += u.re * x.re + u.im * x.im;
                gi += u.re * x.im - u.im * x.re;
            }
            R[(size_t)j * n + k] = mk<double>(gr, gi);
        }
        __syncthreads();
        // O U into Y (free): O = sum_a p_a S^a on the muon digit
        cx<double> *OU = Y;
        {
            const double px = a.pol[3 * (size_t)sn], py = a.pol[3 * (size_t)sn + 1],
                         pz = a.pol[3 * (size_t)sn + 2];
            const int stride = a.strides[a.mu_index];
            const cx<double> o00 = mk<double>(0.5 * pz, 0.0), o01 = mk<double>(0.5 * px, -0.5 * py);
            const cx<double> o10 = mk<double>(0.5 * px, 0.5 * py), o11 = mk<double>(-0.5 * pz, 0.0);
            for (size_t e = tid; e < nn; e += nt) {
                const int i = (int)(e / n), k = (int)(e - (size_t)i * n);
                const int di = (i / stride) & 1, b0 = i - di * stride;
                const cx<double> x0 = U[(size_t)b0 * n + k], x1 = U[(size_t)(b0 + stride) * n + k];
                OU[e] = di == 0 ? cadd(cmul(o00, x0), cmul(o01, x1))
                                : cadd(cmul(o10, x0), cmul(o11, x1));
            }
        }
        __syncthreads();
        const double scale = a.wscale[sn];
        double local = 0.0;
        for (size_t e = tid; e < ntri; e += nt) {
            int j = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
            while ((size_t)(j + 1) * (j + 2) / 2 <= e) ++j;
            while ((size_t)j * (j + 1) / 2 > e) --j;
            const int k = (int)(e - (size_t)j * (j + 1) / 2);
            // O'_kj = sum_i conj(U_ik) (O U)_ij
            double orr = 0, oii = 0;
            for (int i = 0; i < n; ++i) {
                const cx<double> u = U[(size_t)i * n + k], x = OU[(size_t)i * n + j];
                orr += u.re * x.re + u.im * x.im;
                oii += u.re * x.im - u.im * x.re;
            }
            const cx<double> r = R[(size_t)j * n + k];
            // C_jk = rho'_jk O'_kj
            const double cr = r.re * orr - r.im * oii, ci = r.re * oii + r.im * orr;
            if (INTEGRAL) {
                // term = -C_jk / (2 pi i (l_k - l_j) - 1/tau); pairs count twice
                const double inv_tau = 1.0 / a.tau;
                if (j == k) {
                    local += cr * a.tau;
                } else {
                    const double x = twopi * (s.lam[k] - s.lam[j]);
                    const double den = inv_tau * inv_tau + x * x;
                    local += 2.0 * (cr * inv_tau - ci * x) / den;
                }
            } else {
                if (j == k)
                    local += cr;
                else
                    large_store_pair(a, (size_t)sn * P + (size_t)j * (j - 1) / 2 + k,
                                     2.0 * scale * cr, twopi * (s.lam[j] - s.lam[k]),
                                     2.0 * scale * ci);
            }
        }
        local = block_sum(local, red);
        if (tid == 0) {
            a.snap_const[sn] = INTEGRAL ? scale * local / a.tau : scale * local;
            a.status[sn] = st;
        }
        __syncthreads();
    }
}

size_t large_rho_smem_bytes(int n, int threads, int fac_len) {
    return large_rho_fac_offset(n, threads) + (size_t)fac_len * sizeof(cx<double>);
}

size_t large_rho_scratch_bytes(int n, int grid) {
    return large_rho_scratch_doubles(n) * 8 * (size_t)grid;
}

// Persistent grid of the general path: resident CTAs per SM by occupancy,
// all CTAs' scratch within about 2 GB, at most one CTA per snapshot.
int large_rho_grid(int batch, int n, int fac_len) {
    const int threads = large_threads(n);
    int occ = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_large_rho_kernel<false>, threads,
                                                      large_rho_smem_bytes(n, threads, fac_len)) !=
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
    const size_t per = large_rho_scratch_doubles(n) * 8, budget = (size_t)2 << 30;
    while (occ > 1 && (size_t)occ * sms * per > budget) --occ;
    const int g = sms * occ;
    return batch < g ? (batch > 0 ? batch : 1) : g;
}

cudaError_t launch_large_rho(const SnapArgs &a, double *scratch, int grid, cudaStream_t st,
                             int integral) {
    const int threads = large_threads(a.n);
    const size_t smem = large_rho_smem_bytes(a.n, threads, a.fac_len);
    const void *fn = integral ? reinterpret_cast<const void *>(msp_large_rho_kernel<true>)
                              : reinterpret_cast<const void *>(msp_large_rho_kernel<false>);
    cudaError_t e =
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (integral)
        msp_large_rho_kernel<true><<<grid, threads, smem, st>>>(a, scratch);
    else
        msp_large_rho_kernel<false><<<grid, threads, smem, st>>>(a, scratch);
    return cudaGetLastError();
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
    if (threads & 31) return cudaErrorInvalidValue;
    if (precision == MSP_PREC_MIXED) return launch_large_fast_mixed(a, scratch, grid, st, threads);
    const size_t smem = large_smem_bytes(a.n, threads);
    cudaError_t e = cudaFuncSetAttribute(msp_large_fast_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    msp_large_fast_kernel<<<grid, threads, smem, st>>>(a, scratch);
    return cudaGetLastError();
}

size_t large_scratch_bytes(int n, int grid, int precision) {
    const size_t per = precision == MSP_PREC_MIXED ? large_mixed_scratch_per_cta(n)
                                                   : large_scratch_doubles(n) * 8;
    return per * (size_t)grid;
}

// Resident CTAs of the large-n kernels per SM with large_threads(n)
// threads, cut so that all CTAs' scratch stays within about 2 GB (large n
// keeps one CTA per SM).
int large_ctas_per_sm(int n, int precision) {
    const int threads = large_threads(n);
    int occ = 1;
    if (precision == MSP_PREC_MIXED) {
        occ = large_mixed_occupancy(n, threads);
    } else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_large_fast_kernel, threads,
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
// one per matrix.  (Spreading the matrices evenly over fewer CTAs to avoid
// a short last round was measured slower: a snapshot's time is set by
// latency, not by how many CTAs share the SM, so more resident matrices
// win.)
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
