// Initial density matrix of a configuration snapshot as Kronecker factors,
// shared by the snapshot kernels and the Lindblad kernels.
#pragma once

#include <math_constants.h>

#include "msp_internal.cuh"

namespace msp {

#define MSP_FACTOR_MAXD 10

// Kronecker factors of rho0 for snapshot s (muspinsim/experiment.py:170-236):
// the muon in the pure +1/2 state along its polarisation, every other spin
// thermal in its own Zeeman field gamma_i B (uniform at T = inf, ground
// state at T <= 0).  Each factor is sum_k w_k P_k with P_k the spectral
// projectors of n.S, written exactly by Lagrange interpolation over the
// eigenvalues m = I .. -I -- the reference's 2x2/3x3 eigh in closed form.
// One thread per spin; spins up to I = 9/2.
__device__ __forceinline__ void build_rho_factors(const SnapArgs &a, int s, cx<double> *fac) {
    const int i = threadIdx.x;
    if (i >= a.num_spins) return;
    int off = 0;
    for (int k = 0; k < i; ++k) off += a.dims[k] * a.dims[k];
    const int d = a.dims[i];
    cx<double> *R = fac + off;
    for (int e = 0; e < d * d; ++e) R[e] = mk<double>(0.0, 0.0);
    if (d > MSP_FACTOR_MAXD) return;  // rejected on the host
    const double I = 0.5 * (d - 1);
    const bool is_mu = i == a.mu_index;
    const double *v = is_mu ? a.pol + 3 * (size_t)s : a.field + 3 * (size_t)s;
    const double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double nx = 0.0, ny = 0.0, nz = 1.0;
    if (vn > 0.0) {
        nx = v[0] / vn;
        ny = v[1] / vn;
        nz = v[2] / vn;
    }
    double w[MSP_FACTOR_MAXD];
    if (is_mu) {
        for (int k = 0; k < d; ++k) w[k] = k == 0 ? 1.0 : 0.0;
    } else {
        const double T = a.temperature ? a.temperature[s] : CUDART_INF;
        const double h = 6.62607015e-34, kB = 1.380649e-23;
        double E[MSP_FACTOR_MAXD];
        for (int k = 0; k < d; ++k) E[k] = (I - k) * vn * 1e6 * a.gammas[i];
        double sum = 0.0;
        if (T > 0.0) {
            double xmax = -CUDART_INF;
            for (int k = 0; k < d; ++k) {
                w[k] = -h * E[k] / (kB * T);
                xmax = fmax(xmax, w[k]);
            }
            for (int k = 0; k < d; ++k) {
                w[k] = exp(w[k] - xmax);
                sum += w[k];
            }
        } else {
            double emin = E[0];
            for (int k = 1; k < d; ++k) emin = fmin(emin, E[k]);
            for (int k = 0; k < d; ++k) {
                w[k] = E[k] == emin ? 1.0 : 0.0;
                sum += w[k];
            }
        }
        for (int k = 0; k < d; ++k) w[k] = sum > 0.0 ? w[k] / sum : 1.0 / d;
    }
    // n.S: diagonal n_z m_k, off-diagonal (n_x -/+ i n_y)/2 c_k,
    // c_k = sqrt((k+1)(2I-k)) = <m+1|S+|m>
    cx<double> nS[MSP_FACTOR_MAXD * MSP_FACTOR_MAXD];
    for (int e = 0; e < d * d; ++e) nS[e] = mk<double>(0.0, 0.0);
    for (int k = 0; k < d; ++k) nS[k * d + k] = mk<double>(nz * (I - k), 0.0);
    for (int k = 0; k + 1 < d; ++k) {
        const double c = sqrt((double)(k + 1) * (2.0 * I - k));
        nS[k * d + k + 1] = mk<double>(0.5 * nx * c, -0.5 * ny * c);
        nS[(k + 1) * d + k] = mk<double>(0.5 * nx * c, 0.5 * ny * c);
    }
    cx<double> P[MSP_FACTOR_MAXD * MSP_FACTOR_MAXD], Tm[MSP_FACTOR_MAXD * MSP_FACTOR_MAXD];
    for (int k = 0; k < d; ++k) {
        if (w[k] == 0.0) continue;
        const double mk_ = I - k;
        for (int e = 0; e < d * d; ++e) P[e] = mk<double>((e / d) == (e % d) ? 1.0 : 0.0, 0.0);
        for (int k2 = 0; k2 < d; ++k2) {
            if (k2 == k) continue;
            const double m2 = I - k2, inv = 1.0 / (mk_ - m2);
            // Tm = P (nS - m2) / (mk - m2)
            for (int r = 0; r < d; ++r)
                for (int c = 0; c < d; ++c) {
                    double tr = 0.0, ti = 0.0;
                    for (int l = 0; l < d; ++l) {
                        cx<double> x = nS[l * d + c];
                        if (l == c) x.re -= m2;
                        const cx<double> p = P[r * d + l];
                        tr += p.re * x.re - p.im * x.im;
                        ti += p.re * x.im + p.im * x.re;
                    }
                    Tm[r * d + c] = mk<double>(tr * inv, ti * inv);
                }
            for (int e = 0; e < d * d; ++e) P[e] = Tm[e];
        }
        for (int e = 0; e < d * d; ++e) {
            R[e].re += w[k] * P[e].re;
            R[e].im += w[k] * P[e].im;
        }
    }
    double tr = 0.0;
    for (int k = 0; k < d; ++k) tr += R[k * d + k].re;
    for (int e = 0; e < d * d; ++e) {
        R[e].re /= tr;
        R[e].im /= tr;
    }
}


}  // namespace msp
