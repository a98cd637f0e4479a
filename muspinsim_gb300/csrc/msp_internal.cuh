// Internal declarations shared by the translation units of libmspgpu.
#pragma once

#include "msp_common.cuh"

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
    const cx<double> *Hsys;
    const cx<double> *Z;
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
    // time grid (uniform grids: t_k = t0 + k dt)
    double t0, dt;
    // outputs
    void *pair_coef;     // num_snap * P of float2 / double2: (a_c, a_s)
    double *pair_omega;  // num_snap * P angular frequencies (FP64 path, arbitrary grids)
    float4 *pair_phase;  // mixed path on a uniform grid instead of pair_omega:
                         // (psi_hi, psi_lo, phi0_hi, phi0_lo), psi = w dt and
                         // phi0 = w t0 reduced modulo 2 pi, as double-word floats
    double *snap_const;  // num_snap
    int *status;         // num_snap
    int coef_f32;        // n > 64 kernels: pair_coef holds float2 (MIXED) instead of double2
};

// Everything the phase-sum and reduction kernels read and write.
struct PhaseArgs {
    const void *pair_coef;
    const double *pair_omega;
    const float4 *pair_phase;  // see SnapArgs::pair_phase
    int P;             // pairs per snapshot
    int SB;            // snapshots per work item
    const int *slot_first;
    const int *item_first;
    int num_slots;
    double t0, dt;
    int num_times;
    const double *times;  // NULL for uniform grids
    double *partial;      // max_items * num_times
    float *partial_f32;   // mixed path on a uniform grid: FP32 partials instead
};

size_t snap_smem_bytes(int n, int mode, int precision, int fac_len);
cudaError_t launch_snapshots(const SnapArgs &a, int mode, int precision, cudaStream_t st);
cudaError_t launch_eigh(const double *H, int n, int batch, int precision, int max_sweeps,
                        double *evals, double *evecs, int *status, cudaStream_t st);
cudaError_t launch_assemble(const double *Hsys, const double *Z, const double *fields, int n,
                            int batch, double *H, cudaStream_t st);
cudaError_t launch_basis_change(const double *U, long long u_stride, const double *M,
                                long long m_stride, int n, int batch, int adjoint, double *out,
                                cudaStream_t st);

cudaError_t launch_schedule(const int *slot, int num_snap, int num_slots, int SB,
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

// n > 64 (msp_large.cu): FP64 Householder + QL eigensolver, one CTA per
// matrix with `grid` CTAs, each owning large_scratch_bytes(n, 1) of scratch.
cudaError_t launch_eigh_large(const double *H, int n, int batch, double *evals, double *evecs,
                              int *status, double *scratch, int grid, cudaStream_t st);
cudaError_t launch_large_fast(const SnapArgs &a, double *scratch, int grid, cudaStream_t st);
size_t large_scratch_bytes(int n, int grid);
int large_grid(int batch);

// Work decomposition of the phase sum (host side).
int phase_snaps_per_item(int num_snap, int P, int precision);
int phase_max_items(int num_snap, int num_slots, int SB);

}  // namespace msp
