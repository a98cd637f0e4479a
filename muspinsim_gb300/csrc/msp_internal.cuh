// Internal declarations shared by the translation units of libmspgpu.
#pragma once

#include "msp_common.cuh"
#include "msp_dw.cuh"

namespace msp {

template <typename T>
struct PairCoef;
template <>
struct PairCoef<double> {
    typedef double2 type;
    __device__ static __forceinline__ double2 make(double a, double b) {
        return make_double2(a, b);
    }
};
template <>
struct PairCoef<float> {
    typedef float2 type;
    __device__ static __forceinline__ float2 make(double a, double b) {
        return make_float2((float)a, (float)b);
    }
};

// Everything a per-snapshot kernel reads and writes.
struct SnapArgs {
    int n;
    int num_snap;
    int max_sweeps;
    int max_refine;  // MIXED refinement step cap
    const cx<double> *Hsys;
    const cx<double> *Z;
    // MIXED (optional): Hsys and Z pre-split into double-words, one float4
    // (re_hi, im_hi, re_lo, im_lo) per entry, same indexing; NULL: the
    // kernels split the FP64 matrices themselves
    const float4 *Hsys_dw;
    const float4 *Z_dw;
    const double *field;
    const double *pol;
    const double *wscale;
    // general path (EVOLVE / INTEGRAL)
    int num_spins;
    int mu_index;
    int dims[MSP_MAX_SPINS];
    int strides[MSP_MAX_SPINS];
    const cx<double> *rho_fac;  // optional host-built factors
    const double *temperature;  // NULL = T inf
    double gammas[MSP_MAX_SPINS];
    int fac_len;
    double tau;
    // time grid (uniform grids: t_k = t0 + k dt); c_dt, c_t0 = 2 pi dt and
    // 2 pi t0 as double-words (hi, lo) for the mixed path's phase records,
    // and t0_zero = (t0 == 0)
    double t0, dt;
    float2 c_dt, c_t0;
    int t0_zero;
    // outputs
    void *pair_coef;     // num_snap * P of float2 / double2: (a_c, a_s)
    double *pair_omega;  // num_snap * P angular frequencies (FP64 path, arbitrary grids)
    float4 *pair_phase;  // mixed path on a uniform grid instead of pair_omega:
                         // (psi_hi, psi_lo, phi0_hi, phi0_lo), psi = w dt and
                         // phi0 = w t0 reduced modulo 2 pi, as double-word floats
    double *snap_const;  // num_snap
    int *status;         // num_snap
    int coef_f32;        // n > 64 kernels: pair_coef holds float2 (MIXED) instead of double2
    void *evec;          // MIXED, n <= 32: num_snap * n * n FP32 complex eigenvectors
                         // (row-major) from the warp Jacobi stage; NULL runs the
                         // single-kernel form
    // Heterogeneous batches (msp_multi_*): when num_seg > 0 the launch's
    // snapshots form num_seg segments; snapshot sn of segment j
    // (seg_first[j] <= sn < seg_first[j + 1]) reads its field, polarisation
    // and weight, and writes its status, at global snapshot
    // seg_g0[j] + sn - seg_first[j], and its system's Hsys / Z start
    // seg_hoff[j] / 3 seg_hoff[j] complex entries into Hsys / Z.  Pair
    // records and snap_const stay indexed by sn.
    int num_seg;
    const int *seg_first;
    const int *seg_g0;
    const long long *seg_hoff;
};

// Sets c_dt, c_t0 and t0_zero from t0 and dt.
inline void snap_time_constants(SnapArgs &a) {
    a.c_dt = dw_of(6.283185307179586476925 * a.dt);
    a.c_t0 = dw_of(6.283185307179586476925 * a.t0);
    a.t0_zero = a.t0 == 0.0;
}

// Global snapshot index and system matrices of launch-local snapshot sn.
struct SnapSource {
    int g;
    const cx<double> *Hsys, *Z;
    const float4 *Hdw, *Zdw;
};

__device__ __forceinline__ SnapSource snap_source(const SnapArgs &a, int sn) {
    SnapSource r;
    r.g = sn;
    r.Hsys = a.Hsys;
    r.Z = a.Z;
    r.Hdw = a.Hsys_dw;
    r.Zdw = a.Z_dw;
    if (a.num_seg > 0) {
        int lo = 0, hi = a.num_seg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.seg_first[mid] <= sn)
                lo = mid;
            else
                hi = mid - 1;
        }
        r.g = a.seg_g0[lo] + (sn - a.seg_first[lo]);
        const long long o = a.seg_hoff[lo];
        r.Hsys = a.Hsys + o;
        r.Z = a.Z + 3 * o;
        if (a.Hsys_dw) {
            r.Hdw = a.Hsys_dw + o;
            r.Zdw = a.Z_dw + 3 * o;
        }
    }
    return r;
}

// Everything the phase-sum and reduction kernels read and write.
struct PhaseArgs {
    const void *pair_coef;
    const double *pair_omega;
    const float4 *pair_phase;  // see SnapArgs::pair_phase
    int P;             // pairs per snapshot
    int IP;            // pairs per work item (a work item never straddles two slots)
    const int *slot_first;
    const int *item_first;
    int num_slots;
    double t0, dt;
    int num_times;
    const double *times;  // NULL for uniform grids
    double *partial;      // max_items * num_times
    float *partial_f32;   // mixed path on a uniform grid: FP32 partials instead
    const int *slot_row;  // reduce: output row of each slot (NULL: row = slot)
    int accumulate;       // reduce: out += sum instead of out = sum
};

size_t snap_smem_bytes(int n, int mode, int precision, int fac_len);
// Hsys (nh entries) and Z (nz entries) split into double-words into dst
// (nh + nz float4: Hsys first), for SnapArgs::Hsys_dw / Z_dw.
cudaError_t launch_split_dw(const double *Hsys, size_t nh, const double *Z, size_t nz,
                            float4 *dst, cudaStream_t st);
// Two-stage MIXED snapshots (n <= 32): the warp-per-matrix FP32 Jacobi
// (msp_jacobi_warp.cu) writes eigenvectors to SnapArgs::evec; the snapshot
// kernels refine them.  Bytes of that scratch for num_snap snapshots (0 when
// the form does not apply).
bool jacobi_warp_supported(int n);
size_t snap_evec_bytes(int n, long long num_snap, int precision);
cudaError_t launch_jacobi_warp(const SnapArgs &a, cudaStream_t st);
// Householder + QL alternative to the warp Jacobi (msp_ql_warp.cu), same
// inputs and eigenvector scratch
bool ql_warp_supported(int n);
cudaError_t launch_ql_warp(const SnapArgs &a, cudaStream_t st);
cudaError_t launch_snapshots_refine(const SnapArgs &a, int mode, cudaStream_t st, int threads = 0,
                                    int grid = 0);
cudaError_t launch_snapshots(const SnapArgs &a, int mode, int precision, cudaStream_t st,
                             int threads = 0, int grid = 0);
// Threads per CTA of the snapshot kernels when the caller gives none.
int snap_default_threads(int n);
// CTAs of one snapshot kernel that fit on one SM with `threads` threads.
int snap_occupancy(int n, int mode, int precision, int threads);
cudaError_t launch_eigh(const double *H, int n, int batch, int precision, int max_sweeps,
                        double *evals, double *evecs, int *status, cudaStream_t st);
cudaError_t launch_assemble(const double *Hsys, const double *Z, const double *fields, int n,
                            int batch, double *H, cudaStream_t st);
cudaError_t launch_basis_change(const double *U, long long u_stride, const double *M,
                                long long m_stride, int n, int batch, int adjoint, double *out,
                                cudaStream_t st);

cudaError_t launch_schedule(const int *slot, int num_snap, int num_slots, int P, int IP,
                            int count_items, int *slot_first, int *item_first, int *status,
                            cudaStream_t st);
cudaError_t launch_phase(const PhaseArgs &a, int precision, int max_items, int uniform,
                         cudaStream_t st);
cudaError_t launch_reduce(const PhaseArgs &a, const double *snap_const, double *out,
                          int num_times, cudaStream_t st);

cudaError_t launch_fast_cos_sum(const double *times, int num_times, int d, const double *A,
                                const double *W, int n, double *out, cudaStream_t st);
cudaError_t launch_fast_amplitudes(const double *evals, const double *evecs,
                                   const double *sigma, int n, int d, double *A, double *W,
                                   cudaStream_t st);
cudaError_t launch_evolve_expect(const double *evals, const double *rho, const double *ops,
                                 int n, int num_ops, const double *times, int num_times,
                                 double *out, cudaStream_t st);
cudaError_t launch_evolve_phases(const double *evals, const double *rho, int n,
                                 const double *times, int num_times, double *out,
                                 cudaStream_t st);
cudaError_t launch_integrate(const double *evals, const double *rho, const double *ops, int n,
                             int num_ops, double tau, double *out, cudaStream_t st);

// n > 64 (msp_large.cu): Householder + QL eigensolver, one CTA per matrix
// with `grid` CTAs, each owning large_scratch_bytes(n, 1, precision) of
// scratch.  The eigensolver API (launch_eigh_large) is FP64; the fast path
// runs FP64 or MIXED (FP32 solve, double-word refinement).
cudaError_t launch_eigh_large(const double *H, int n, int batch, double *evals, double *evecs,
                              int *status, double *scratch, int grid, cudaStream_t st);
cudaError_t launch_large_fast(const SnapArgs &a, double *scratch, int grid, cudaStream_t st,
                              int threads = 0, int precision = MSP_PREC_FP64);
int large_threads(int n);
size_t large_scratch_bytes(int n, int grid, int precision = MSP_PREC_FP64);
int large_ctas_per_sm(int n, int precision = MSP_PREC_FP64);
int large_grid(int batch, int n, int precision = MSP_PREC_FP64);
// The MIXED fast path's kernel (msp_large_mixed.cu).
cudaError_t launch_large_fast_mixed(const SnapArgs &a, double *scratch, int grid,
                                    cudaStream_t st, int threads);
size_t large_mixed_scratch_per_cta(int n);
int large_mixed_occupancy(int n, int threads);
// General path for n > 64 (EVOLVE / INTEGRAL, FP64 in both precisions).
cudaError_t launch_large_rho(const SnapArgs &a, double *scratch, int grid, cudaStream_t st,
                             int integral);
size_t large_rho_scratch_bytes(int n, int grid);
int large_rho_grid(int batch, int n, int fac_len);

// Work decomposition of the phase sum (host side).  A work item sums at
// most MSP_F32_ITEM_PAIRS pairs in FP32 (mixed precision): longer FP32
// running sums lose ~1e-6 of P(t) to rounding at n ~ 100.
#define MSP_F32_ITEM_PAIRS 1024
bool phase_use_tensor_cores();
int phase_snaps_per_item(int num_snap, int P, int precision);
int phase_pairs_per_item(int num_snap, int P, int precision);
int phase_max_items(int num_snap, int num_slots, int P, int IP);

}  // namespace msp
