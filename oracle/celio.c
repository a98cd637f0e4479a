/* Celio's method on the CPU -- TEST INFRASTRUCTURE ONLY (the timed CPU
 * baseline of the Celio workload and a second checker of the GPU path).
 *
 * Plain-C restatement of the reference's native kernels:
 *   - oracle_celio_apply   : (M (x) 1_d) V through an index map, in place
 *                            (muspinsim/cpp/parallel.cpp:236-262), OpenMP
 *                            over the d groups as the reference does;
 *   - oracle_celio_measure : Re V^dag (M (x) 1_d) V for Hermitian M using the
 *                            upper triangle twice
 *                            (muspinsim/cpp/parallel.cpp:126-160);
 *   - oracle_celio_evolve  : per time, measure then k passes over the
 *                            factors (muspinsim/cpp/celio.cpp:23-64), adding
 *                            into results.
 * Complex numbers are interleaved (re, im) doubles. */
#include <complex.h>
#include <stdlib.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

void oracle_celio_apply(cplx* V, const cplx* M, long D, long d, const unsigned long* idx) {
#pragma omp parallel
    {
        cplx tmp[256];
#pragma omp for
        for (long k = 0; k < d; ++k) {
            for (long i = 0; i < D; ++i) {
                cplx acc = 0.0;
                for (long j = 0; j < D; ++j) acc += M[i * D + j] * V[idx[j * d + k]];
                tmp[i] = acc;
            }
            for (long i = 0; i < D; ++i) V[idx[i * d + k]] = tmp[i];
        }
    }
}

double oracle_celio_measure(const cplx* V, const cplx* M, long D, long d) {
    double result = 0.0;
#pragma omp parallel for reduction(+ : result)
    for (long k = 0; k < d; ++k) {
        for (long i = 0; i < D; ++i) {
            cplx term = M[i * D + i] * V[i * d + k];
            for (long j = i + 1; j < D; ++j) term += M[i * D + j] * V[j * d + k] * 2.0;
            result += creal(conj(V[i * d + k]) * term);
        }
    }
    return result;
}

/* mats: the factors back to back (D_f^2 each); dims_f[f] = D_f;
 * other_f[f] = d_f; idx: num_factors index maps of N entries each. */
void oracle_celio_evolve(int num_times, cplx* psi, const cplx* sigma, long half_dim, int k,
                         int num_factors, const cplx* mats, const long* dims_f,
                         const long* other_f, const unsigned long* idx, long N,
                         double* results, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int i = 0; i < num_times; ++i) {
        results[i] += oracle_celio_measure(psi, sigma, 2, half_dim);
        for (int r = 0; r < k; ++r) {
            const cplx* m = mats;
            for (int f = 0; f < num_factors; ++f) {
                oracle_celio_apply(psi, m, dims_f[f], other_f[f], idx + (long)f * N);
                m += dims_f[f] * dims_f[f];
            }
        }
    }
}
