/*
 * CPU oracle -- test infrastructure only, never part of the product path.
 *
 * Plain-C restatement of the reference's cosine phase-sum kernel
 * (muspinsim/cython/parallel.pyx:16-69, called from
 * muspinsim/hamiltonian.py:213):
 *
 *   out[i] = (1/d) * sum_j [ 0.5*A[j,j] + sum_{k<j} A[j,k]*cos(W[j,k]*t_i) ]
 *
 * The summation order per time (j ascending, the diagonal term first, then
 * k = 0..j-1) is the reference's, so with the same libm the results match the
 * compiled reference bit for bit.  OpenMP splits the times across threads the
 * way the reference's prange does.
 */
#include <math.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void oracle_fast_cos_sum(const double *times, long num_times, long other_dimension,
                         const double *A, const double *W, long mat_dim,
                         double *out, int nthreads)
{
    const double one_over_d = 1.0 / (double)other_dimension;
    long i;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (i = 0; i < num_times; ++i) {
        double acc = 0.0;
        const double t = times[i];
        for (long j = 0; j < mat_dim; ++j) {
            acc += 0.5 * A[j * mat_dim + j];
            for (long k = 0; k < j; ++k)
                acc += A[j * mat_dim + k] * cos(W[j * mat_dim + k] * t);
        }
        out[i] = acc * one_over_d;
    }
}

/*
 * Powder sum of many fast-path snapshots: out[i] += sum_s wscale[s] *
 * P_s(t_i), where snapshot s has amplitude/frequency matrices A_s, W_s
 * (n x n, row-major, packed back to back).  Used to time the reference
 * algorithm's CPU cost on whole orientation batches.
 */
void oracle_fast_cos_powder(const double *times, long num_times, long other_dimension,
                            const double *A, const double *W, long mat_dim,
                            long num_snap, const double *wscale, double *out,
                            int nthreads)
{
    const double one_over_d = 1.0 / (double)other_dimension;
    const long nn = mat_dim * mat_dim;
    long i;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (i = 0; i < num_times; ++i) {
        const double t = times[i];
        double total = 0.0;
        for (long s = 0; s < num_snap; ++s) {
            const double *As = A + s * nn;
            const double *Ws = W + s * nn;
            double acc = 0.0;
            for (long j = 0; j < mat_dim; ++j) {
                acc += 0.5 * As[j * mat_dim + j];
                for (long k = 0; k < j; ++k)
                    acc += As[j * mat_dim + k] * cos(Ws[j * mat_dim + k] * t);
            }
            total += wscale[s] * (acc * one_over_d);
        }
        out[i] += total;
    }
}
