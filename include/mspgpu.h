/*
 * mspgpu.h -- C ABI of the GB300 muon-polarisation library (libmspgpu.so).
 *
 * Drop-in replacement for the numerical core of MuSpinSim's polarisation
 * path.  Every entry point:
 *   - takes DEVICE pointers (CUDA global memory) unless stated otherwise;
 *   - stores complex numbers as interleaved (re, im) doubles, matrices
 *     row-major, batches back to back;
 *   - runs asynchronously on the given CUDA stream (NULL = legacy default
 *     stream) and allocates nothing: scratch memory comes from the caller,
 *     sized by the matching *_workspace query;
 *   - returns an msp status code; MSP_OK means the work was enqueued.
 *     Data-dependent outcomes (an eigensolve that hit its sweep cap, an
 *     out-of-range slot index) are written to the caller's per-item
 *     `status` array, read after the stream has been synchronised.
 *
 * Units follow the reference: Hamiltonians in MHz, fields in T, times in
 * microseconds, phases 2 pi * MHz * us.
 */
#ifndef MSPGPU_H
#define MSPGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define MSP_OK 0
#define MSP_ERR_ARG 1         /* invalid argument (see msp_last_error) */
#define MSP_ERR_CUDA 2        /* a CUDA runtime call or launch failed */
#define MSP_ERR_WORKSPACE 3   /* caller workspace too small */
#define MSP_ERR_UNSUPPORTED 4 /* size outside the supported range */

/* per-item status values written by the kernels */
#define MSP_ITEM_OK 0
#define MSP_ITEM_NOT_CONVERGED 1 /* Jacobi reached max_sweeps, or QL 60 steps on a level */
#define MSP_ITEM_BAD_SLOT 2      /* slot index out of range / not sorted */
#define MSP_ITEM_REFINE_LIMIT 4  /* MIXED: the last eigenvector refinement step
                                    allowed (max_refine) still corrected by more
                                    than 2e-4; the snapshot may miss the 1e-6
                                    accuracy of the mixed form */

/* precision of the eigensolve and phase sum */
#define MSP_PREC_FP64 0  /* all-FP64: bit-faithful drop-in (max|dP| <= 1e-10) */
#define MSP_PREC_MIXED 1 /* FP32 Jacobi + FP64 Rayleigh-quotient eigenvalues,
                            FP32 phase sum with FP64 phase reduction and
                            FP64 cross-block accumulation */

/* evolution algorithm of a snapshot batch */
#define MSP_MODE_FAST 0     /* muon-first, T = inf cosine sum */
#define MSP_MODE_EVOLVE 1   /* general <O>(t) from rho0 */
#define MSP_MODE_INTEGRAL 2 /* exponentially weighted time integral */

#define MSP_MAX_DIM 64   /* largest Hilbert dimension of the Jacobi kernels */
#define MSP_MAX_DIM_LARGE 1024 /* largest n of the Householder + QL path */
#define MSP_MAX_SPINS 16

/* ---- library information ---------------------------------------------- */
int msp_version(void);
/* Copies the message of the last MSP_ERR_* in this thread into buf. */
int msp_last_error(char *buf, size_t len);

/* ---- building blocks ---------------------------------------------------- */

/* H[b] = Hsys + sum_a fields[b][a] * Z[a]  (n x n complex128, batch b).
 * Replaces ExperimentRunner.Hz / Htot (muspinsim/experiment.py:239-250,
 * 332-341).  fields: batch*3 doubles. */
int msp_assemble(const double *Hsys, const double *Z, const double *fields, int n,
                 int batch, double *H, void *stream);

/* Hamiltonians of rotated copies of a spin system (the tensor-rotation
 * formulation of SpinSystem.rotate + .hamiltonian, muspinsim/spinsys.py:
 * 103-110, 128-135, 594-626): for each rotation R_s (batch x 9 doubles,
 * row-major)
 *   H_s = sum_t sum_ab (R_s T_t R_s^T)_ab B[9 t + 3 a + b]
 *       + sum_u (R_s v_u)_a B[9 num_double + 3 u + a].
 * tensors: num_double 3x3 tensors T_t (9 doubles each); vectors: num_single
 * 3-vectors v_u; basis: (9 num_double + 3 num_single) n x n complex128 --
 * the Kronecker-embedded S^a_i S^b_j of each bilinear term (the product
 * S^a_i S^b_i for a same-spin term) and S^a_i of each single term.  At most
 * 64 terms of each kind.  H: batch x n x n complex128.  ExperimentRunner
 * rotates the field instead (muspinsim/experiment.py:405-406); both give
 * unitarily equivalent Hamiltonians. */
int msp_assemble_rotated(const double *rot, int batch, const double *tensors, int num_double,
                         const double *vectors, int num_single, const double *basis, int n,
                         double *H, void *stream);

/* Batched Hermitian eigensolve, 1 <= n <= MSP_MAX_DIM: cyclic Jacobi, one CTA
 * per matrix.  evals: batch*n ascending; evecs: batch*n*n complex128 with the
 * eigenvectors as COLUMNS (numpy.linalg.eigh layout); status: batch ints.
 * precision MSP_PREC_MIXED runs the sweeps in FP32 and refines the eigenvalues
 * with FP64 Rayleigh quotients.  Replaces Hermitian.diag / numpy.linalg.eigh
 * (muspinsim/spinop.py:51-82). */
int msp_eigh_batched(const double *H, int n, int batch, int precision, int max_sweeps,
                     double *evals, double *evecs, int *status, void *stream);

/* Scratch bytes msp_eigh_batched_ws needs for (n, batch): 0 for
 * n <= MSP_MAX_DIM, else one working set per CTA of the large-n solver. */
int msp_eigh_workspace(int n, int batch, size_t *bytes);

/* msp_eigh_batched for 1 <= n <= MSP_MAX_DIM_LARGE.  n <= MSP_MAX_DIM runs
 * the Jacobi kernels (workspace unused); larger n runs, in FP64 for both
 * precisions, Householder tridiagonalisation + implicit-shift QL with
 * eigenvector accumulation + back-transformation, one CTA per matrix with
 * its working matrices in `workspace` (>= msp_eigh_workspace bytes,
 * 256-byte aligned).  Same outputs and replaced reference code as
 * msp_eigh_batched. */
int msp_eigh_batched_ws(const double *H, int n, int batch, int precision, int max_sweeps,
                        double *evals, double *evecs, int *status, void *workspace,
                        size_t workspace_bytes, void *stream);

/* out[b] = U[b]^dag M[b] U[b]  (adjoint = 0)  or  U[b] M[b] U[b]^dag
 * (adjoint = 1), 1 <= n <= MSP_MAX_DIM_LARGE.  m_stride = complex elements
 * between consecutive M matrices (0 broadcasts one M), u_stride likewise
 * for U.  Replaces Operator.basis_change (muspinsim/spinop.py:330-355). */
int msp_basis_change(const double *U, long long u_stride, const double *M,
                     long long m_stride, int n, int batch, int adjoint, double *out,
                     void *stream);

/* out[i] = (1/d) sum_j [ 0.5 A[j,j] + sum_{k<j} A[j,k] cos(W[j,k] t_i) ]
 * A, W: n x n doubles.  Same arithmetic as parallel_fast_time_evolve
 * (muspinsim/cython/parallel.pyx:16-69). */
int msp_fast_cos_sum(const double *times, int num_times, int other_dimension,
                     const double *A, const double *W, int n, double *out, void *stream);

/* A = |U^dag (sigma (x) 1_d) U|^2, W = 2 pi (l_j - l_k); sigma: 2x2
 * complex128 (muon first), n <= MSP_MAX_DIM_LARGE.  Replaces
 * muspinsim/hamiltonian.py:204-211. */
int msp_fast_amplitudes(const double *evals, const double *evecs, const double *sigma,
                        int n, int other_dimension, double *A, double *W, void *stream);

/* out[t][o] = sum_ij rho[i][j] op_o[j][i] exp(-2 pi i (l_i - l_j) t_t), with
 * rho and ops already in the eigenbasis; out: num_times*num_ops complex128.
 * Replaces the time loop of Hamiltonian.evolve (muspinsim/hamiltonian.py:86-107). */
int msp_evolve_expect(const double *evals, const double *rho, const double *ops, int n,
                      int num_ops, const double *times, int num_times, double *out,
                      void *stream);

/* out[t] = exp(-2 pi i (l_i - l_j) t) * rho[i][j] for every time: the
 * eigenbasis density matrices of Hamiltonian.evolve without operators
 * (muspinsim/hamiltonian.py:89-90, 108-116); out: num_times*n*n complex128. */
int msp_evolve_phases(const double *evals, const double *rho, int n, const double *times,
                      int num_times, double *out, void *stream);

/* out[o] = sum_ij rho[i][j] * (-op_o[j][i] / (2 pi i (l_j - l_i) - 1/tau)),
 * rho and ops in the eigenbasis; out: num_ops complex128.  Replaces
 * Hamiltonian.integrate_decaying (muspinsim/hamiltonian.py:150-164). */
int msp_integrate_decaying(const double *evals, const double *rho, const double *ops,
                           int n, int num_ops, double tau, double *out, void *stream);

/* Lab-frame vectors of the snapshots of an orientation grid: for each row
 * the stored conjugate quaternion q* of MuSpinConfig._validate_orient
 * (muspinsim/simconfig.py:596-613; polar rows (theta, phi) as Euler
 * (phi, theta, phi) 'zyz', muspinsim/utils.py:53-68) rotates the field and
 * the polarisation as ExperimentRunner.load_config does
 * (muspinsim/experiment.py:405-411): field = q*(B) + B_intr, pol = q*(p).
 * rows: num_rows x row_len doubles (device); row_len 2 = (theta, phi),
 * 3 = (a, b, c), 4 = (a, b, c, w); euler_mode 0 = 'zyz', 1 = 'zxz'.
 * B, p, B_intr (may be NULL): HOST 3-vectors.  field, pol: num_rows*3
 * outputs.  weight (may be NULL): num_rows outputs w_k * weight_norm, w_k
 * the row weight (4-column rows, more than one row) or 1 -- weight_norm =
 * 1 / sum(w) gives the normalised weights of muspinsim/simconfig.py:152-159
 * divided by the averaged count. */
int msp_orient_snapshots(const double *rows, int num_rows, int row_len, int euler_mode,
                         const double *B, const double *p, const double *B_intr,
                         double weight_norm, double *field, double *pol, double *weight,
                         void *stream);

/* Orientation grids generated on the device (the input keywords
 * `orientation zcw(N)` / `eulrange(N)`: muspinsim/utils.py:34-50,
 * muspinsim/input/keyword.py:38), expanded as the Cartesian product of a
 * field list and the grid (MuSpinConfig's snapshot product,
 * muspinsim/simconfig.py:299-321, for a field axis or file range with
 * averaged orientations).  Snapshot s = f * num_orient + o gets the
 * lab-frame field R_o fields[f] + B_intr, polarisation R_o p, weight
 * w_o * weight_norm (w_o = 1 for ZCW, sin(beta) for eulrange; 1 when the
 * grid has one point) and, when slot is not NULL, output row f.  ZCW point
 * j of N: polar angles theta = arccos(c1 (c2 j / N - 1)), phi = 2 pi
 * frac(j g / N) (c = (1, 2) sphere, (-1, 1) hemisphere; g = zcw_generator,
 * coprime with N), rotated like a (theta, phi) row; eulrange: N^3 ZYZ (or
 * ZXZ, euler_mode 1) angles a, c = linspace(0, 2 pi, N), b = interior of
 * linspace(0, pi, N + 2), in the reference's meshgrid order.  fields is a
 * DEVICE array of num_fields x 3; p and B_intr are host 3-vectors; the
 * outputs are device arrays of num_fields * num_orient snapshots. */
#define MSP_GRID_ZCW_SPHERE 0
#define MSP_GRID_ZCW_HEMISPHERE 1
#define MSP_GRID_EULRANGE 2
int msp_orient_grid_snapshots(int grid_kind, int grid_n, int zcw_generator, int euler_mode,
                              const double *fields, int num_fields, const double *p,
                              const double *B_intr, double weight_norm, double *field,
                              double *pol, double *weight, int *slot, void *stream);

/* ---- stage timer ---------------------------------------------------------- */

/* Opaque set of CUDA events that msp_powder_run records around its stages
 * when msp_powder_args.timer is set: eigensolve (the warp-per-matrix FP32
 * Jacobi of the two-stage MIXED form, n <= 32; empty otherwise), snapshots
 * (assembly, eigensolve or refinement, eigenbasis amplitudes), schedule,
 * phase sum, reduction.  No counterpart in
 * the reference, which has no timing beyond wall-clock logging
 * (muspinsim/__main__.py:124, 163-165). */
typedef struct msp_timer msp_timer;
#define MSP_TIMER_STAGES 5
#define MSP_TIMER_CAPACITY 512 /* runs recorded between two reads */

int msp_timer_create(msp_timer **timer);
int msp_timer_destroy(msp_timer *timer);
/* Waits for the recorded runs, writes the summed milliseconds of each stage
 * into ms[MSP_TIMER_STAGES] and the number of runs into *runs, and empties
 * the timer. */
int msp_timer_read(msp_timer *timer, double *ms, int *runs);

/* ---- fused powder pipeline ---------------------------------------------- */

/* One batch of configuration snapshots of one spin system, reduced on the
 * device into output rows ("slots"): the loop of ExperimentRunner.run /
 * run_single plus MuSpinConfig.store_time_slice (muspinsim/experiment.py:
 * 358-382, 434-498; muspinsim/simconfig.py:347-368).  All pointers are
 * device pointers except where noted. */
typedef struct msp_powder_args {
    int n;                    /* Hilbert dimension, 2 .. MSP_MAX_DIM_LARGE; above
                                 MSP_MAX_DIM the Householder + QL kernels run
                                 (FAST: FP64, or FP32 + double-word refinement
                                 for MIXED; EVOLVE / INTEGRAL: FP64) */
    int num_spins;            /* spins in the system, <= MSP_MAX_SPINS */
    int mu_index;             /* position of the muon in the spin order */
    int dims[MSP_MAX_SPINS];  /* per-spin multiplicity 2I+1 (host values) */
    const double *Hsys;       /* n*n complex128, field-independent part (MHz) */
    const double *Z;          /* 3*n*n complex128, Z_a = sum_i gamma_i S^a_i */
    int num_snap;             /* snapshots in the batch */
    const double *field;      /* num_snap*3 lab-frame field incl. intrinsic (T) */
    const double *pol;        /* num_snap*3 lab-frame muon polarisation */
    const double *wscale;     /* num_snap: orientation weight / averaged count */
    const int *slot;          /* num_snap output rows, non-decreasing, < num_slots */
    const double *temperature;/* EVOLVE/INTEGRAL: num_snap temperatures (K) of the
                                 initial state; NULL means T = inf for all */
    double gammas[MSP_MAX_SPINS]; /* per-spin gyromagnetic ratio, MHz/T (host) */
    const double *rho_fac;    /* EVOLVE/INTEGRAL, optional: per snapshot, the
                                 Kronecker factors of rho0 (dims[s]^2 complex128
                                 per spin, spin order), back to back.  NULL:
                                 the kernel builds them from field, pol,
                                 temperature and gammas: muon pure along pol,
                                 other spins thermal in their own Zeeman
                                 field (muspinsim/experiment.py:170-236) */
    int num_slots;            /* output rows */
    const double *times;      /* num_times (ignored when uniform = 1) */
    int num_times;            /* FAST/EVOLVE time samples; 1 for INTEGRAL */
    int uniform;              /* 1: t_k = t0 + k dt */
    double t0, dt;
    double tau;               /* INTEGRAL: decay time (us) */
    int mode;                 /* MSP_MODE_* */
    int precision;            /* MSP_PREC_* */
    int max_sweeps;           /* Jacobi sweep cap, <= 0 selects 40 (the QL eigensolvers cap
                                 their steps at 60 per level instead) */
    double *out;              /* num_slots*num_times (FAST/EVOLVE) or num_slots */
    int *status;              /* num_snap per-snapshot status (MSP_ITEM_*) */
    void *workspace;          /* caller scratch, >= msp_powder_workspace bytes,
                                 256-byte aligned */
    size_t workspace_bytes;
    void *stream;             /* cudaStream_t */
    msp_timer *timer;         /* optional stage timer (NULL: none) */
    int max_refine;           /* MIXED: eigenvector refinement step cap, <= 0
                                 selects 4 (MSP_ITEM_REFINE_LIMIT when used up) */
} msp_powder_args;

/* Scratch bytes msp_powder_run needs for these arguments (no pointer is
 * dereferenced). */
int msp_powder_workspace(const msp_powder_args *args, size_t *bytes);

/* Runs the batch: Hamiltonian assembly, batched eigensolve, eigenbasis
 * amplitudes, phase sum over time, weighted reduction into args->out
 * (overwritten).  Kernels launched: msp_snap_* (one CTA per snapshot),
 * msp_schedule, msp_phase_* (time tiles x pair chunks), msp_reduce. */
int msp_powder_run(const msp_powder_args *args);

/* Bytes of scratch built into the library for msp_powder_run_static. */
#define MSP_STATIC_SCRATCH_BYTES (32u << 20)

/* msp_powder_run for callers that cannot allocate device memory (a host
 * whose GPU memory belongs to another runtime, a binding with no route to
 * cudaMalloc, a loop that must not let an allocation synchronise the
 * device).  No counterpart in the reference.  args->workspace and
 * args->workspace_bytes are ignored: the scratch is a file-scope device
 * array of MSP_STATIC_SCRATCH_BYTES that every GPU loading the library keeps
 * until exit, and a batch needing more returns MSP_ERR_WORKSPACE with the
 * sizes in msp_last_error.  Nothing is allocated.  The first call on each
 * device (with it current) looks up the array's device address; make that
 * call before any stream capture.  That address is not valid across
 * cudaDeviceReset: do not call this entry point on a device after resetting
 * it.  All calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller.  Same
 * results as msp_powder_run. */
int msp_powder_run_static(const msp_powder_args *args);

/* ---- heterogeneous batch: many spin systems of uneven dimension ----------
 * The loop of ExperimentRunner.run / run_single with store_time_slice
 * (muspinsim/experiment.py:358-498, muspinsim/simconfig.py:347-368) run for
 * many spin systems at once, each reduced into its own output row, on the
 * muon-first T = inf path (Hamiltonian.fast_evolve, muspinsim/hamiltonian.py:
 * 166-217).  The reference runs one ExperimentRunner per system.
 *
 * Systems are grouped into size buckets (one per distinct n).  A bucket is
 * one persistent snapshot launch over all its snapshots, the phase sum and a
 * reduction; buckets run concurrently on plan-owned streams forked from and
 * joined to the caller's stream.  n <= MSP_MAX_DIM runs the Jacobi kernels
 * (both precisions), larger n the FP64 Householder + QL kernel. */

/* Launch parameters for the systems of one dimension (e.g. an autotuner's
 * choice).  Zero fields keep the library's default. */
typedef struct msp_multi_tuning {
    int n;              /* Hilbert dimension the entry applies to */
    int snap_threads;   /* threads per snapshot CTA: multiple of 32, <= 512 */
    int ctas_per_sm;    /* resident snapshot CTAs per SM of the persistent grid
                           (capped by occupancy; n > 64: scratch per CTA) */
    int snaps_per_item; /* snapshots per phase-sum work item (the FP32 partial
                           sums still hold at most 1024 pairs) */
} msp_multi_tuning;

/* Sizes of a heterogeneous batch; all pointers are HOST pointers, read only
 * during msp_multi_plan_create. */
typedef struct msp_multi_desc {
    int num_systems;
    const int *sys_n;          /* num_systems Hilbert dimensions: even (muon first),
                                  2 .. MSP_MAX_DIM_LARGE */
    const int *sys_snap_first; /* num_systems + 1: system k owns snapshots
                                  [sys_snap_first[k], sys_snap_first[k + 1]) */
    int num_times;
    int uniform;               /* 1: t_k = t0 + k dt */
    double t0, dt;
    int precision;             /* MSP_PREC_* */
    int max_sweeps;            /* Jacobi sweep cap, <= 0 selects 40 (the QL eigensolvers cap
                                  their steps at 60 per level instead) */
    long long max_pairs_per_chunk; /* pair records a bucket holds at once; larger
                                      buckets run in chunks (0: 2^26) */
    const msp_multi_tuning *tuning;
    int num_tuning;
} msp_multi_desc;

/* Device buffers of one run. */
typedef struct msp_multi_io {
    const double *Hsys_all;  /* every system's Hsys back to back, system order:
                                n_k^2 complex128 each */
    const double *Z_all;     /* every system's Z_x, Z_y, Z_z back to back: 3 n_k^2
                                complex128 each */
    const double *field;     /* num_snap*3 lab-frame field incl. intrinsic (T) */
    const double *pol;       /* num_snap*3 lab-frame muon polarisation */
    const double *wscale;    /* num_snap: orientation weight / averaged count */
    const double *times;     /* num_times (ignored when uniform = 1) */
    double *out;             /* num_systems*num_times: row k = system k (overwritten) */
    int *status;             /* num_snap per-snapshot status (MSP_ITEM_*) */
    void *workspace;         /* >= msp_multi_workspace bytes, 256-byte aligned; holds
                                the plan's tables and scratch during a run */
    size_t workspace_bytes;
} msp_multi_io;

typedef struct msp_multi_plan msp_multi_plan;

/* One size bucket of a plan (msp_multi_plan_info). */
typedef struct msp_multi_bucket_info {
    int n, num_systems;
    long long num_snap;
    int num_chunks;
    int snap_threads;
    int grid;            /* persistent snapshot CTAs (0 until the first run for n <= 64) */
    int pairs_per_item;
    int max_items;
    size_t scratch_bytes;
} msp_multi_bucket_info;

/* Plans a batch: buckets, chunks, work tables and the workspace size.  Host
 * work only; streams, events and a pinned copy of the tables are made by
 * the first run, on the device current then (every later run must have the
 * same device current). */
int msp_multi_plan_create(const msp_multi_desc *desc, msp_multi_plan **plan);
int msp_multi_plan_destroy(msp_multi_plan *plan);
int msp_multi_workspace(const msp_multi_plan *plan, size_t *bytes);
/* Buckets in launch order; writes at most `capacity` entries of info. */
int msp_multi_plan_info(const msp_multi_plan *plan, int *num_buckets,
                        msp_multi_bucket_info *info, int capacity);
/* Enqueues the batch on `stream`: table upload, output clear, per bucket
 * msp_snap_fast / msp_large_fast (persistent), msp_phase_*, msp_reduce.
 * Runs of one plan must not overlap (they share its streams). */
int msp_multi_run(msp_multi_plan *plan, const msp_multi_io *io, void *stream);
/* msp_multi_run through a CUDA graph: the first call (and any call whose io
 * pointers differ from the captured ones) captures the launch sequence on a
 * plan-owned stream and instantiates it; every call launches the graph on
 * `stream`. */
int msp_multi_run_graph(msp_multi_plan *plan, const msp_multi_io *io, void *stream);

/* ---- dissipation: Lindblad superoperators -------------------------------
 * The reference switches to a Lindbladian when the configuration has
 * dissipation terms (muspinsim/experiment.py:272-341) and diagonalises the
 * n^2 x n^2 superoperator L with a dense non-Hermitian eig
 * (muspinsim/lindbladian.py:43-173).  Here the same quantities come from
 * exp(2 pi L dt) (scaling and squaring, FP64) and from a pivoted LU solve
 * of (1/tau - 2 pi L): rho(t) = exp(2 pi L t) rho0 and
 * int_0^inf <O>(t) e^{-t/tau} dt = vec(O^T) . (1/tau - 2 pi L)^-1 rho0.
 * Superoperators act on row-major vec(rho); n <= 32. */

/* Scratch bytes of msp_superop_evolve / _integrate for an n-level system. */
int msp_superop_workspace(int n, int num_ops, size_t *bytes);

/* <O_op>(t_k) = Tr(O_op rho(t_k)), rho(t) = exp(2 pi L t) rho0: the
 * expectation series of Lindbladian.evolve (muspinsim/lindbladian.py:43-111).
 * L: n^2 x n^2 complex128; rho0: n x n; ops: num_ops x n x n; out:
 * num_times x num_ops complex128, or with num_ops = 0 the density matrices
 * (num_times x n x n).  uniform = 1: t_k = t0 + k dt (times unused). */
int msp_superop_evolve(const double *L, int n, const double *rho0, const double *ops,
                       int num_ops, const double *times, int num_times, int uniform, double t0,
                       double dt, double *out, void *workspace, size_t workspace_bytes,
                       void *stream);

/* int_0^inf <O_op>(t) e^{-t/tau} dt for each operator: Lindbladian.
 * integrate_decaying (muspinsim/lindbladian.py:113-173); out: num_ops
 * complex128. */
int msp_superop_integrate(const double *L, int n, const double *rho0, const double *ops,
                          int num_ops, double tau, double *out, void *workspace,
                          size_t workspace_bytes, void *stream);

/* A batch of dissipative snapshots of one spin system, reduced into output
 * rows: run_single's Lindbladian branch plus store_time_slice
 * (muspinsim/experiment.py:434-498, 272-341; muspinsim/simconfig.py:
 * 347-368).  Per snapshot the kernel builds H = Hsys + b.Z, rho0 (muon along
 * p, other spins thermal), the dissipators S+/- of every dissipative spin
 * about the field direction with rates a Zu / (pi (1 + Zu)) and
 * a / (pi (1 + Zu)), Zu = exp(-h gamma |B| 1e6 / (k T)), and L; then the
 * time series (MSP_MODE_EVOLVE) or the decaying integral divided by tau
 * (MSP_MODE_INTEGRAL), real part times wscale. */
typedef struct msp_lindblad_args {
    int n;                         /* Hilbert dimension, 2 .. 32 */
    int num_spins;
    int mu_index;
    int dims[MSP_MAX_SPINS];       /* 2I+1 per spin (host), <= 10 */
    double gammas[MSP_MAX_SPINS];  /* MHz/T (host) */
    const double *Hsys;            /* n*n complex128 */
    const double *Z;               /* 3*n*n complex128 */
    const double *spin_ops;        /* num_spins x 3 x n x n complex128: S^x,y,z of
                                      each spin, Kronecker-embedded */
    int num_dissipative;
    int dissipative_spin[MSP_MAX_SPINS];    /* host: spin indices */
    double dissipative_rate[MSP_MAX_SPINS]; /* host: rates (MHz) */
    int num_snap;
    const double *field;           /* num_snap*3 (T) */
    const double *pol;             /* num_snap*3 */
    const double *wscale;          /* num_snap */
    const int *slot;               /* num_snap, non-decreasing, < num_slots */
    const double *temperature;     /* num_snap (K), NULL = inf */
    int num_slots;
    const double *times;           /* num_times (ignored when uniform = 1) */
    int num_times;
    int uniform;
    double t0, dt;
    double tau;                    /* INTEGRAL: decay time (us) */
    int mode;                      /* MSP_MODE_EVOLVE or MSP_MODE_INTEGRAL */
    double *out;                   /* num_slots*num_times (EVOLVE) or num_slots */
    int *status;                   /* num_snap */
    void *workspace;               /* >= msp_lindblad_workspace bytes, 256-byte aligned */
    size_t workspace_bytes;
    void *stream;
    int precision;                 /* MSP_PREC_FP64, or MSP_PREC_MIXED: for EVOLVE on a
                                      uniform grid with n^2 <= 64, propagators and states
                                      in double-word FP32 (hi + lo) on the FP32 pipe */
} msp_lindblad_args;

int msp_lindblad_workspace(const msp_lindblad_args *args, size_t *bytes);
int msp_lindblad_run(const msp_lindblad_args *args);

/* ---------------------------------------------------------------- adjoint
 * Gradient of a scalar loss L through the fast-path powder average
 * (K6).  The reference has no gradient: its fitting
 * (muspinsim/fitting.py:67-179) re-runs ExperimentRunner per objective
 * evaluation and differentiates by finite differences; this entry point
 * returns dL/dHsys and dL/dB_lab for one upstream gradient dL/dP(t) of
 * the msp_powder_run output (MSP_MODE_FAST arguments: muon first, T = inf).
 *
 * Per snapshot, P_s(t) = kappa_s Tr(S e^{2 pi i H t} S e^{-2 pi i H t}) with
 * S = (p . sigma) (x) 1_d and kappa_s = wscale_s / (4 d).  Its derivative
 * uses the Frechet derivative of the matrix exponential in the FP64
 * eigenbasis (divided differences of e^{2 pi i lambda t}, their derivative
 * for (near-)degenerate levels), so degenerate spectra need no special
 * handling by the caller.  Gradients use the convention
 * dL = Re sum_ij conj(G_ij) dH_ij (the PyTorch complex-gradient convention). */
typedef struct msp_adjoint_args {
    int n;                    /* Hilbert dimension, even, 2 .. MSP_MAX_DIM */
    const double *Hsys;       /* n*n complex128 (MHz) */
    const double *Z;          /* 3*n*n complex128 */
    int num_snap;
    const double *field;      /* num_snap*3 lab-frame field (T) */
    const double *pol;        /* num_snap*3 lab-frame muon polarisation */
    const double *wscale;     /* num_snap weights, as msp_powder_args */
    const int *slot;          /* num_snap rows of grad_out, non-decreasing */
    int num_slots;
    const double *times;      /* num_times (ignored when uniform = 1) */
    int num_times;
    int uniform;              /* 1: t_k = t0 + k dt */
    double t0, dt;
    const double *grad_out;   /* num_slots*num_times: dL/dP */
    double *grad_hsys;        /* out: n*n complex128, sum over snapshots of dL/dH_s */
    double *grad_field;       /* out, optional (NULL): num_snap*3 dL/dfield */
    int *status;              /* num_snap per-snapshot eigensolve status */
    int max_sweeps;           /* Jacobi sweep cap, <= 0 selects 40 (the QL eigensolvers cap
                                 their steps at 60 per level instead) */
    void *workspace;          /* >= msp_adjoint_workspace bytes, 256-byte aligned */
    size_t workspace_bytes;
    void *stream;             /* cudaStream_t */
} msp_adjoint_args;

/* Scratch bytes msp_adjoint_fast needs (no pointer is dereferenced). */
int msp_adjoint_workspace(const msp_adjoint_args *args, size_t *bytes);

/* Kernels: msp_assemble, msp_eigh (FP64), msp_adjoint_transform (per level
 * pair: sum_t g(t) e^{2 pi i nu t} and its t-weighted form, FP64),
 * msp_adjoint_snap (one CTA per snapshot: dL/dH_s, dL/db_s),
 * msp_adjoint_sum (deterministic sum over snapshots). */
int msp_adjoint_fast(const msp_adjoint_args *args);

/* ---------------------------------------------------------------- Celio's method
 * Trotter evolution without diagonalisation: CelioHamiltonian.evolve and
 * .fast_evolve (muspinsim/celio.py:210-476) and the reference's native
 * module behind the latter (muspinsim/cpp/celio.cpp:23-64,
 * muspinsim/cpp/parallel.cpp:126-262: celio_evolve, fast_measure_h,
 * fast_evolve).  A state is a tensor of `num_digits` digits (spin
 * multiplicities, digit 0 slowest).  One Trotter pass applies every factor
 * in order -- factor f multiplies the D_f-element groups of its one or two
 * digits (given in the factor's own order, the reference's spin_order) by
 * the D_f x D_f complex matrix at factor_mat[f] in the snapshot's block --
 * and one time step is trotter_k passes.  Per time sample, first measure,
 * then step.
 *   MSP_CELIO_PURE:    num_digits = spins, muon first (digit 0 of dimension
 *                      2); states_per_snapshot random initial states
 *                      mu_psi (x) exp(2 pi i r) / sqrt(d) per snapshot, r
 *                      from `phases` ([S][A][d], uniform in [0,1)) or, when
 *                      phases is NULL, from a counter-based generator keyed
 *                      by `seed`; series[s][a][t] = Re <psi|(sigma_s (x) 1)|psi>.
 *   MSP_CELIO_DENSITY: num_digits = 2 x spins (row digits, then column
 *                      digits of rho); pass the factors as (U^dagger on the
 *                      row digits, U^T on the column digits) so that a pass
 *                      maps rho to U^dagger rho U as the reference's
 *                      T^dag rho0 T does; series[s][t][j] = sum rho .* meas_j
 *                      (meas_j = O_j^T, complex).
 * rows_out[r][t] (optional) = sum over the snapshots row_start[r] ..
 * row_start[r+1]-1 of wscale[s] * (PURE: 0.5 / A sum_a series, DENSITY:
 * Re series of operator 0) -- the averaged, weighted result of
 * ExperimentRunner.run_single.  FP64 by default; MSP_PREC_MIXED keeps states
 * and factors as double-word FP32 (see `precision`).  States that fit in one
 * CTA's shared memory run there from start to end; larger ones run from
 * global memory (path: 0 automatic, 1 shared memory, 2 global memory). */
#define MSP_CELIO_PURE 0
#define MSP_CELIO_DENSITY 1

typedef struct msp_celio_args {
    int mode;                     /* MSP_CELIO_* */
    int num_digits;               /* 1..32 */
    const int *digit_dims;        /* host [num_digits] */
    int num_factors;              /* 0..1024 factor applications per Trotter pass */
    const int *factor_digits;     /* host [num_factors][2]; second digit -1 for one */
    const long long *factor_mat;  /* host [num_factors]: matrix offset (complex entries) */
    const double *mats;           /* device complex [num_snapshots or 1][mats_len] */
    long long mats_len;
    int mats_per_snapshot;        /* 1: one block per snapshot; 0: one shared block */
    int num_snapshots;
    int states_per_snapshot;      /* PURE: averages; DENSITY: 1 */
    int trotter_k;                /* >= 1 */
    int num_times;
    const double *mu_psi;         /* PURE: device complex [S][2] */
    const double *sigma;          /* PURE: device complex [S][2][2], Hermitian */
    const double *phases;         /* PURE: device [S][A][d] or NULL */
    unsigned long long seed;
    const double *rho0;           /* DENSITY: device complex [S][N][N] */
    const double *meas;           /* DENSITY: device complex [S or 1][num_ops][N][N] */
    int num_ops;
    int meas_per_snapshot;
    void *series;                 /* device: PURE double [S][A][T]; DENSITY complex
                                     [S][T][num_ops]; NULL = in the workspace */
    const double *wscale;         /* device [S] or NULL (1) */
    const int *row_start;         /* device [num_rows + 1], for rows_out */
    int num_rows;
    double *rows_out;             /* device [num_rows][T] or NULL */
    int path;                     /* 0 automatic, 1 shared memory, 2 global memory */
    int precision;                /* MSP_PREC_FP64, or MSP_PREC_MIXED: double-word FP32
                                     (hi + lo, ~2^-40 per factor application) on the FP32
                                     pipe, either memory path */
} msp_celio_args;

int msp_celio_workspace(const msp_celio_args *args, size_t *bytes);
int msp_celio_run(const msp_celio_args *args, void *workspace, size_t workspace_bytes,
                  void *stream);

/* Trotter factors that depend on the field, per snapshot: U = exp(-2 pi i
 * tau (H0_f + sum_a B[s][a] G_f[a])) for each field-dependent factor f
 * (a spin's Zeeman term, alone or merged with other one-spin terms:
 * muspinsim/celio.py:145-160, muspinsim/experiment.py:251-267), tau =
 * dt / k; written into each snapshot's block of `mats` as U, U^dagger and /
 * or U^T at out_offsets[f][0..2] (-1 skips).  dims (host, 1..16 each) and
 * out_offsets (host) describe up to 64 factors; H0 (device) holds their
 * D_f x D_f complex matrices back to back and G (device) three per factor
 * (x, y, z); fields (device) [S][3] in T. */
int msp_celio_expm(int num_snapshots, int num_factors, const int *dims, const double *H0,
                   const double *G, const double *fields, double tau,
                   const long long *out_offsets, double *mats, long long mats_len,
                   void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MSPGPU_H */
