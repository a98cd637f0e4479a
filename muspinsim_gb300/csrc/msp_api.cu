// extern "C" entry points of libmspgpu.so (declared in include/mspgpu.h):
// argument checks, workspace carving and kernel launch order.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "msp_internal.cuh"

using namespace msp;

static thread_local char g_last_error[512] = "";

static int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

static int cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        return fail(MSP_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return MSP_OK;
}

namespace msp {
// Records an error message for msp_last_error from another translation unit.
int record_error(int code, const char *msg) { return fail(code, "%s", msg); }
}  // namespace msp

#define MSP_CHECK_PTR(p)                                    \
    do {                                                    \
        if ((p) == NULL) return fail(MSP_ERR_ARG, "%s is NULL", #p); \
    } while (0)

extern "C" {

int msp_version(void) { return 10000; }

int msp_last_error(char *buf, size_t len) {
    if (buf == NULL || len == 0) return MSP_ERR_ARG;
    strncpy(buf, g_last_error, len - 1);
    buf[len - 1] = '\0';
    return MSP_OK;
}

int msp_assemble(const double *Hsys, const double *Z, const double *fields, int n, int batch,
                 double *H, void *stream) {
    if (n < 1 || batch < 0) return fail(MSP_ERR_ARG, "msp_assemble: n=%d batch=%d", n, batch);
    if (batch == 0) return MSP_OK;
    MSP_CHECK_PTR(Hsys);
    MSP_CHECK_PTR(Z);
    MSP_CHECK_PTR(fields);
    MSP_CHECK_PTR(H);
    return cuda_check(launch_assemble(Hsys, Z, fields, n, batch, H, (cudaStream_t)stream),
                      "msp_assemble");
}

int msp_eigh_batched(const double *H, int n, int batch, int precision, int max_sweeps,
                     double *evals, double *evecs, int *status, void *stream) {
    if (n < 1 || batch < 0)
        return fail(MSP_ERR_ARG, "msp_eigh_batched: n=%d batch=%d", n, batch);
    if (n > MSP_MAX_DIM)
        return fail(MSP_ERR_UNSUPPORTED, "msp_eigh_batched: n=%d exceeds %d", n, MSP_MAX_DIM);
    if (precision != MSP_PREC_FP64 && precision != MSP_PREC_MIXED)
        return fail(MSP_ERR_ARG, "msp_eigh_batched: precision=%d", precision);
    if (batch == 0) return MSP_OK;
    MSP_CHECK_PTR(H);
    MSP_CHECK_PTR(evals);
    MSP_CHECK_PTR(evecs);
    MSP_CHECK_PTR(status);
    if (max_sweeps <= 0) max_sweeps = 40;
    return cuda_check(launch_eigh(H, n, batch, precision, max_sweeps, evals, evecs, status,
                                  (cudaStream_t)stream),
                      "msp_eigh_batched");
}

int msp_eigh_workspace(int n, int batch, size_t *bytes) {
    if (n < 1 || batch < 0 || bytes == NULL)
        return fail(MSP_ERR_ARG, "msp_eigh_workspace: n=%d batch=%d", n, batch);
    if (n > MSP_MAX_DIM_LARGE)
        return fail(MSP_ERR_UNSUPPORTED, "msp_eigh_workspace: n=%d exceeds %d", n,
                    MSP_MAX_DIM_LARGE);
    *bytes = n <= MSP_MAX_DIM ? 0 : large_scratch_bytes(n, large_grid(batch, n));
    return MSP_OK;
}

int msp_eigh_batched_ws(const double *H, int n, int batch, int precision, int max_sweeps,
                        double *evals, double *evecs, int *status, void *workspace,
                        size_t workspace_bytes, void *stream) {
    if (n <= MSP_MAX_DIM)
        return msp_eigh_batched(H, n, batch, precision, max_sweeps, evals, evecs, status, stream);
    if (n > MSP_MAX_DIM_LARGE || batch < 0)
        return fail(n > MSP_MAX_DIM_LARGE ? MSP_ERR_UNSUPPORTED : MSP_ERR_ARG,
                    "msp_eigh_batched_ws: n=%d batch=%d", n, batch);
    if (precision != MSP_PREC_FP64 && precision != MSP_PREC_MIXED)
        return fail(MSP_ERR_ARG, "msp_eigh_batched_ws: precision=%d", precision);
    if (batch == 0) return MSP_OK;
    MSP_CHECK_PTR(H);
    MSP_CHECK_PTR(evals);
    MSP_CHECK_PTR(evecs);
    MSP_CHECK_PTR(status);
    const int grid = large_grid(batch, n);
    const size_t need = large_scratch_bytes(n, grid);
    if (workspace == NULL || workspace_bytes < need)
        return fail(MSP_ERR_WORKSPACE, "msp_eigh_batched_ws: workspace %zu < %zu bytes",
                    workspace_bytes, need);
    if (reinterpret_cast<uintptr_t>(workspace) & 255)
        return fail(MSP_ERR_ARG, "msp_eigh_batched_ws: workspace not 256-byte aligned");
    return cuda_check(launch_eigh_large(H, n, batch, evals, evecs, status,
                                        reinterpret_cast<double *>(workspace), grid,
                                        (cudaStream_t)stream),
                      "msp_eigh_batched_ws");
}

int msp_basis_change(const double *U, long long u_stride, const double *M, long long m_stride,
                     int n, int batch, int adjoint, double *out, void *stream) {
    if (n < 1 || batch < 0 || u_stride < 0 || m_stride < 0)
        return fail(MSP_ERR_ARG, "msp_basis_change: n=%d batch=%d", n, batch);
    if (n > MSP_MAX_DIM_LARGE)
        return fail(MSP_ERR_UNSUPPORTED, "msp_basis_change: n=%d exceeds %d", n,
                    MSP_MAX_DIM_LARGE);
    if (batch == 0) return MSP_OK;
    MSP_CHECK_PTR(U);
    MSP_CHECK_PTR(M);
    MSP_CHECK_PTR(out);
    return cuda_check(launch_basis_change(U, u_stride, M, m_stride, n, batch, adjoint ? 1 : 0,
                                          out, (cudaStream_t)stream),
                      "msp_basis_change");
}

int msp_fast_cos_sum(const double *times, int num_times, int other_dimension, const double *A,
                     const double *W, int n, double *out, void *stream) {
    if (num_times < 0 || n < 1 || other_dimension < 1)
        return fail(MSP_ERR_ARG, "msp_fast_cos_sum: num_times=%d n=%d d=%d", num_times, n,
                    other_dimension);
    if (num_times == 0) return MSP_OK;
    MSP_CHECK_PTR(times);
    MSP_CHECK_PTR(A);
    MSP_CHECK_PTR(W);
    MSP_CHECK_PTR(out);
    return cuda_check(launch_fast_cos_sum(times, num_times, other_dimension, A, W, n, out,
                                          (cudaStream_t)stream),
                      "msp_fast_cos_sum");
}

int msp_fast_amplitudes(const double *evals, const double *evecs, const double *sigma, int n,
                        int other_dimension, double *A, double *W, void *stream) {
    if (n < 2 || other_dimension < 1 || 2 * other_dimension != n)
        return fail(MSP_ERR_ARG, "msp_fast_amplitudes: n=%d d=%d (need n = 2 d)", n,
                    other_dimension);
    if (n > MSP_MAX_DIM_LARGE)
        return fail(MSP_ERR_UNSUPPORTED, "msp_fast_amplitudes: n=%d exceeds %d", n,
                    MSP_MAX_DIM_LARGE);
    MSP_CHECK_PTR(evals);
    MSP_CHECK_PTR(evecs);
    MSP_CHECK_PTR(sigma);
    MSP_CHECK_PTR(A);
    MSP_CHECK_PTR(W);
    return cuda_check(launch_fast_amplitudes(evals, evecs, sigma, n, other_dimension, A, W,
                                             (cudaStream_t)stream),
                      "msp_fast_amplitudes");
}

int msp_evolve_expect(const double *evals, const double *rho, const double *ops, int n,
                      int num_ops, const double *times, int num_times, double *out,
                      void *stream) {
    if (n < 1 || num_ops < 0 || num_times < 0)
        return fail(MSP_ERR_ARG, "msp_evolve_expect: n=%d ops=%d times=%d", n, num_ops,
                    num_times);
    if (num_ops == 0 || num_times == 0) return MSP_OK;
    MSP_CHECK_PTR(evals);
    MSP_CHECK_PTR(rho);
    MSP_CHECK_PTR(ops);
    MSP_CHECK_PTR(times);
    MSP_CHECK_PTR(out);
    return cuda_check(launch_evolve_expect(evals, rho, ops, n, num_ops, times, num_times, out,
                                           (cudaStream_t)stream),
                      "msp_evolve_expect");
}

int msp_evolve_phases(const double *evals, const double *rho, int n, const double *times,
                      int num_times, double *out, void *stream) {
    if (n < 1 || num_times < 0)
        return fail(MSP_ERR_ARG, "msp_evolve_phases: n=%d times=%d", n, num_times);
    if (num_times == 0) return MSP_OK;
    MSP_CHECK_PTR(evals);
    MSP_CHECK_PTR(rho);
    MSP_CHECK_PTR(times);
    MSP_CHECK_PTR(out);
    return cuda_check(
        launch_evolve_phases(evals, rho, n, times, num_times, out, (cudaStream_t)stream),
        "msp_evolve_phases");
}

int msp_integrate_decaying(const double *evals, const double *rho, const double *ops, int n,
                           int num_ops, double tau, double *out, void *stream) {
    if (n < 1 || num_ops < 0) return fail(MSP_ERR_ARG, "msp_integrate_decaying: n=%d", n);
    if (!(tau > 0.0)) return fail(MSP_ERR_ARG, "msp_integrate_decaying: tau must be > 0");
    if (num_ops == 0) return MSP_OK;
    MSP_CHECK_PTR(evals);
    MSP_CHECK_PTR(rho);
    MSP_CHECK_PTR(ops);
    MSP_CHECK_PTR(out);
    return cuda_check(
        launch_integrate(evals, rho, ops, n, num_ops, tau, out, (cudaStream_t)stream),
        "msp_integrate_decaying");
}

// ---------------------------------------------------------------- stage timer

struct msp_timer {
    cudaEvent_t ev[MSP_TIMER_CAPACITY][MSP_TIMER_STAGES + 1];
    int used;
};

int msp_timer_create(msp_timer **timer) {
    if (timer == NULL) return fail(MSP_ERR_ARG, "msp_timer_create: timer is NULL");
    msp_timer *t = new (std::nothrow) msp_timer;
    if (t == NULL) return fail(MSP_ERR_ARG, "msp_timer_create: out of host memory");
    t->used = 0;
    for (int r = 0; r < MSP_TIMER_CAPACITY; ++r)
        for (int k = 0; k <= MSP_TIMER_STAGES; ++k) {
            cudaError_t e = cudaEventCreate(&t->ev[r][k]);
            if (e != cudaSuccess) {
                for (int r2 = 0; r2 <= r; ++r2)
                    for (int k2 = 0; k2 <= MSP_TIMER_STAGES; ++k2)
                        if (r2 < r || k2 < k) cudaEventDestroy(t->ev[r2][k2]);
                delete t;
                return cuda_check(e, "msp_timer_create");
            }
        }
    *timer = t;
    return MSP_OK;
}

int msp_timer_destroy(msp_timer *t) {
    if (t == NULL) return MSP_OK;
    for (int r = 0; r < MSP_TIMER_CAPACITY; ++r)
        for (int k = 0; k <= MSP_TIMER_STAGES; ++k) cudaEventDestroy(t->ev[r][k]);
    delete t;
    return MSP_OK;
}

int msp_timer_read(msp_timer *t, double *ms, int *runs) {
    if (t == NULL || ms == NULL) return fail(MSP_ERR_ARG, "msp_timer_read: NULL argument");
    for (int k = 0; k < MSP_TIMER_STAGES; ++k) ms[k] = 0.0;
    for (int r = 0; r < t->used; ++r) {
        int rc = cuda_check(cudaEventSynchronize(t->ev[r][MSP_TIMER_STAGES]), "msp_timer_read");
        if (rc != MSP_OK) return rc;
        for (int k = 0; k < MSP_TIMER_STAGES; ++k) {
            float v = 0.f;
            rc = cuda_check(cudaEventElapsedTime(&v, t->ev[r][k], t->ev[r][k + 1]),
                            "msp_timer_read");
            if (rc != MSP_OK) return rc;
            ms[k] += v;
        }
    }
    if (runs) *runs = t->used;
    t->used = 0;
    return MSP_OK;
}

static cudaEvent_t *timer_slot(msp_timer *t) {
    if (t == NULL || t->used >= MSP_TIMER_CAPACITY) return NULL;
    return t->ev[t->used++];
}

// ---------------------------------------------------------------- powder pipeline

struct Layout {
    size_t coef, omega, snap_const, slot_first, item_first, partial, large, evec, hdw, total;
    int P, IP, max_items, T;
    bool phase_records;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Complex entries of rho0's Kronecker factors (sum of dims^2).
static int powder_fac_len(const msp_powder_args *a) {
    int fac = 0;
    for (int s = 0; s < a->num_spins; ++s) fac += a->dims[s] * a->dims[s];
    return fac;
}

static int check_powder(const msp_powder_args *a) {
    if (a == NULL) return fail(MSP_ERR_ARG, "msp_powder: args is NULL");
    if (a->n < 2) return fail(MSP_ERR_ARG, "msp_powder: n=%d", a->n);
    if (a->n > MSP_MAX_DIM_LARGE)
        return fail(MSP_ERR_UNSUPPORTED, "msp_powder: n=%d exceeds %d", a->n, MSP_MAX_DIM_LARGE);
    if (a->num_snap < 0 || a->num_slots < 1)
        return fail(MSP_ERR_ARG, "msp_powder: num_snap=%d num_slots=%d", a->num_snap,
                    a->num_slots);
    if (a->num_slots > 65535)
        return fail(MSP_ERR_UNSUPPORTED, "msp_powder: num_slots=%d exceeds 65535", a->num_slots);
    if (a->mode != MSP_MODE_FAST && a->mode != MSP_MODE_EVOLVE && a->mode != MSP_MODE_INTEGRAL)
        return fail(MSP_ERR_ARG, "msp_powder: mode=%d", a->mode);
    if (a->precision != MSP_PREC_FP64 && a->precision != MSP_PREC_MIXED)
        return fail(MSP_ERR_ARG, "msp_powder: precision=%d", a->precision);
    if (a->mode == MSP_MODE_INTEGRAL) {
        if (!(a->tau > 0.0)) return fail(MSP_ERR_ARG, "msp_powder: tau must be > 0");
    } else {
        if (a->num_times < 1) return fail(MSP_ERR_ARG, "msp_powder: num_times=%d", a->num_times);
        if (!a->uniform && a->times == NULL)
            return fail(MSP_ERR_ARG, "msp_powder: times is NULL on a non-uniform grid");
    }
    if (a->mode == MSP_MODE_FAST && (a->n & 1))
        return fail(MSP_ERR_ARG, "msp_powder: the fast path needs the muon first (n even)");
    if (a->mode != MSP_MODE_FAST) {
        if (a->num_spins < 1 || a->num_spins > MSP_MAX_SPINS)
            return fail(MSP_ERR_ARG, "msp_powder: num_spins=%d", a->num_spins);
        long long prod = 1;
        for (int s = 0; s < a->num_spins; ++s) {
            if (a->dims[s] < 1) return fail(MSP_ERR_ARG, "msp_powder: dims[%d]=%d", s, a->dims[s]);
            prod *= a->dims[s];
        }
        if (prod != a->n)
            return fail(MSP_ERR_ARG, "msp_powder: product of dims %lld != n %d", prod, a->n);
        if (a->mu_index < 0 || a->mu_index >= a->num_spins || a->dims[a->mu_index] != 2)
            return fail(MSP_ERR_ARG, "msp_powder: mu_index=%d", a->mu_index);
        if (a->rho_fac == NULL)
            for (int s = 0; s < a->num_spins; ++s)
                if (a->dims[s] > 10)
                    return fail(MSP_ERR_UNSUPPORTED,
                                "msp_powder: spin %d has 2I+1=%d > 10; pass rho_fac", s,
                                a->dims[s]);
    }
    return MSP_OK;
}

static Layout powder_layout(const msp_powder_args *a) {
    Layout L;
    const size_t S = (size_t)a->num_snap;
    L.T = a->mode == MSP_MODE_INTEGRAL ? 1 : a->num_times;
    L.P = a->n * (a->n - 1) / 2;
    const int has_pairs = a->mode != MSP_MODE_INTEGRAL;
    L.IP = phase_pairs_per_item(a->num_snap, L.P, a->precision);
    L.max_items = has_pairs ? phase_max_items(a->num_snap, a->num_slots, L.P, L.IP) : 0;
    const size_t ce = a->precision == MSP_PREC_MIXED ? 8 : 16;
    size_t off = 0;
    L.coef = off;
    off += align256(has_pairs ? S * L.P * ce : 0);
    L.omega = off;
    // mixed precision on a uniform grid stores double-word phases (16 B)
    // instead of FP64 frequencies (8 B)
    L.phase_records = has_pairs && a->precision == MSP_PREC_MIXED && a->uniform;
    off += align256(has_pairs ? S * L.P * (L.phase_records ? 16 : 8) : 0);
    L.snap_const = off;
    off += align256(S * 8);
    L.slot_first = off;
    off += align256((size_t)(a->num_slots + 1) * 4);
    L.item_first = off;
    off += align256((size_t)(a->num_slots + 1) * 4);
    L.partial = off;
    off += align256((size_t)L.max_items * L.T * (L.phase_records ? 4 : 8));
    L.evec = off;
    off += align256(snap_evec_bytes(a->n, a->num_snap, a->precision));
    // MIXED, n <= MSP_MAX_DIM: Hsys and Z as double-words (no FP64 in the
    // snapshot kernels)
    L.hdw = off;
    if (a->precision == MSP_PREC_MIXED && a->n <= MSP_MAX_DIM && a->num_snap > 0)
        off += align256((size_t)4 * a->n * a->n * 16);
    L.large = off;
    if (a->n > MSP_MAX_DIM) {
        if (a->mode == MSP_MODE_FAST)
            off += align256(large_scratch_bytes(
                a->n, large_grid(a->num_snap, a->n, a->precision), a->precision));
        else
            off += align256(large_rho_scratch_bytes(
                a->n, large_rho_grid(a->num_snap, a->n, powder_fac_len(a))));
    }
    L.total = off;
    return L;
}

int msp_powder_workspace(const msp_powder_args *args, size_t *bytes) {
    int rc = check_powder(args);
    if (rc != MSP_OK) return rc;
    if (bytes == NULL) return fail(MSP_ERR_ARG, "msp_powder_workspace: bytes is NULL");
    *bytes = powder_layout(args).total;
    return MSP_OK;
}

int msp_powder_run(const msp_powder_args *a) {
    int rc = check_powder(a);
    if (rc != MSP_OK) return rc;
    MSP_CHECK_PTR(a->out);
    if (a->num_snap > 0) {
        MSP_CHECK_PTR(a->Hsys);
        MSP_CHECK_PTR(a->Z);
        MSP_CHECK_PTR(a->field);
        MSP_CHECK_PTR(a->pol);
        MSP_CHECK_PTR(a->wscale);
        MSP_CHECK_PTR(a->slot);
        MSP_CHECK_PTR(a->status);
    }
    const Layout L = powder_layout(a);
    if (L.total > 0) {
        if (a->workspace == NULL || a->workspace_bytes < L.total)
            return fail(MSP_ERR_WORKSPACE, "msp_powder_run: workspace %zu < %zu bytes",
                        a->workspace_bytes, L.total);
        if (reinterpret_cast<uintptr_t>(a->workspace) & 255)
            return fail(MSP_ERR_ARG, "msp_powder_run: workspace not 256-byte aligned");
    }
    cudaStream_t st = (cudaStream_t)a->stream;
    char *ws = reinterpret_cast<char *>(a->workspace);

    SnapArgs sa;
    memset(&sa, 0, sizeof(sa));
    sa.n = a->n;
    sa.num_snap = a->num_snap;
    sa.max_sweeps = a->max_sweeps > 0 ? a->max_sweeps : 40;
    sa.max_refine = a->max_refine > 0 ? a->max_refine : 4;
    sa.Hsys = reinterpret_cast<const cx<double> *>(a->Hsys);
    sa.Z = reinterpret_cast<const cx<double> *>(a->Z);
    sa.field = a->field;
    sa.pol = a->pol;
    sa.wscale = a->wscale;
    sa.tau = a->tau;
    if (a->mode != MSP_MODE_FAST) {
        sa.num_spins = a->num_spins;
        sa.mu_index = a->mu_index;
        int stride = 1, fac = 0;
        for (int s = a->num_spins - 1; s >= 0; --s) {
            sa.dims[s] = a->dims[s];
            sa.strides[s] = stride;
            stride *= a->dims[s];
            fac += a->dims[s] * a->dims[s];
        }
        sa.rho_fac = reinterpret_cast<const cx<double> *>(a->rho_fac);
        sa.temperature = a->temperature;
        for (int s = 0; s < a->num_spins; ++s) sa.gammas[s] = a->gammas[s];
        sa.fac_len = fac;
    }
    sa.pair_coef = ws + L.coef;
    sa.pair_omega = L.phase_records ? NULL : reinterpret_cast<double *>(ws + L.omega);
    sa.pair_phase = L.phase_records ? reinterpret_cast<float4 *>(ws + L.omega) : NULL;
    sa.t0 = a->t0;
    sa.dt = a->dt;
    snap_time_constants(sa);
    sa.snap_const = reinterpret_cast<double *>(ws + L.snap_const);
    sa.status = a->status;
    sa.coef_f32 = a->precision == MSP_PREC_MIXED;
    sa.evec = snap_evec_bytes(a->n, a->num_snap, a->precision) > 0 ? ws + L.evec : NULL;

    const bool large = a->n > MSP_MAX_DIM;
    if (!large) {
        const size_t smem = snap_smem_bytes(a->n, a->mode, a->precision, sa.fac_len);
        if (smem > 227 * 1024)
            return fail(MSP_ERR_UNSUPPORTED, "msp_powder_run: %zu bytes of shared memory needed",
                        smem);
    }

    cudaEvent_t *ev = timer_slot(a->timer);
    if (ev) cudaEventRecord(ev[0], st);
    if (a->precision == MSP_PREC_MIXED && !large && a->num_snap > 0) {
        const size_t nn = (size_t)a->n * a->n;
        float4 *hdw = reinterpret_cast<float4 *>(ws + L.hdw);
        rc = cuda_check(launch_split_dw(a->Hsys, nn, a->Z, 3 * nn, hdw, st), "msp_split_dw");
        if (rc != MSP_OK) return rc;
        sa.Hsys_dw = hdw;
        sa.Z_dw = hdw + nn;
    }
    // two-stage MIXED snapshots (n <= 32): the warp Jacobi is its own stage
    const bool two_stage = !large && sa.evec != NULL && a->num_snap > 0;
    if (two_stage) {
        rc = cuda_check(launch_jacobi_warp(sa, st), "msp_jacobi_warp");
        if (rc != MSP_OK) return rc;
    }
    if (ev) cudaEventRecord(ev[1], st);
    if (two_stage)
        rc = cuda_check(launch_snapshots_refine(sa, a->mode, st), "msp_snap");
    else if (large && a->num_snap > 0 && a->mode == MSP_MODE_FAST)
        rc = cuda_check(launch_large_fast(sa, reinterpret_cast<double *>(ws + L.large),
                                          large_grid(a->num_snap, a->n, a->precision), st, 0,
                                          a->precision),
                        "msp_large_fast");
    else if (large && a->num_snap > 0)
        rc = cuda_check(launch_large_rho(sa, reinterpret_cast<double *>(ws + L.large),
                                         large_rho_grid(a->num_snap, a->n, sa.fac_len), st,
                                         a->mode == MSP_MODE_INTEGRAL),
                        "msp_large_rho");
    else
        rc = cuda_check(launch_snapshots(sa, a->mode, a->precision, st), "msp_snap");
    if (rc != MSP_OK) return rc;
    if (ev) cudaEventRecord(ev[2], st);

    PhaseArgs pa;
    memset(&pa, 0, sizeof(pa));
    pa.pair_coef = ws + L.coef;
    pa.pair_omega = L.phase_records ? NULL : reinterpret_cast<const double *>(ws + L.omega);
    pa.pair_phase = L.phase_records ? reinterpret_cast<const float4 *>(ws + L.omega) : NULL;
    pa.P = L.P;
    pa.IP = L.IP;
    pa.slot_first = reinterpret_cast<int *>(ws + L.slot_first);
    pa.item_first = reinterpret_cast<int *>(ws + L.item_first);
    pa.num_slots = a->num_slots;
    pa.t0 = a->t0;
    pa.dt = a->dt;
    pa.num_times = L.T;
    pa.times = a->times;
    pa.partial = L.phase_records ? NULL : reinterpret_cast<double *>(ws + L.partial);
    pa.partial_f32 = L.phase_records ? reinterpret_cast<float *>(ws + L.partial) : NULL;

    rc = cuda_check(launch_schedule(a->slot, a->num_snap, a->num_slots, L.P, L.IP,
                                    a->mode != MSP_MODE_INTEGRAL,
                                    reinterpret_cast<int *>(ws + L.slot_first),
                                    reinterpret_cast<int *>(ws + L.item_first), a->status, st),
                    "msp_schedule");
    if (rc != MSP_OK) return rc;
    if (ev) cudaEventRecord(ev[3], st);
    if (a->mode != MSP_MODE_INTEGRAL) {
        rc = cuda_check(launch_phase(pa, a->precision, L.max_items, a->uniform, st), "msp_phase");
        if (rc != MSP_OK) return rc;
    }
    if (ev) cudaEventRecord(ev[4], st);
    rc = cuda_check(launch_reduce(pa, sa.snap_const, a->out, L.T, st), "msp_reduce");
    if (rc != MSP_OK) return rc;
    if (ev) cudaEventRecord(ev[5], st);
    return MSP_OK;
}

}  // extern "C"
