// Tensor-rotation formulation of the Hamiltonian assembly, batched: the
// Hamiltonian of each rotated copy of a spin system, as SpinSystem.rotate
// followed by SpinSystem.hamiltonian computes it (muspinsim/spinsys.py:
// 103-110 SingleTerm.rotate v R^T, 128-135 DoubleTerm.rotate R M R^T,
// 594-626 the rotated system and its term sum).  With the term operators
// expanded in a fixed basis -- per bilinear term the nine Kronecker-embedded
// products S^a_i S^b_j (the matrix product S^a_i S^b_i for a same-spin
// term, muspinsim/spinsys.py:45-53), per single term the three S^a_i --
//   H_s = sum_t sum_ab (R_s T_t R_s^T)_ab B_t,ab + sum_u (R_s v_u)_a B_u,a,
// a contraction of per-snapshot coefficients with basis matrices that stay
// in L2 for the whole batch.
//
// ExperimentRunner does not use this formulation (it rotates the field and
// the polarisation instead, muspinsim/experiment.py:405-406); it is the
// building block for callers that rotate the couplings themselves.  Both
// give unitarily equivalent Hamiltonians (same spectra, same P(t)).
#include "msp_internal.cuh"

namespace msp {
int record_error(int code, const char *msg);

#define MSP_ROT_MAX_TERMS 64
#define MSP_ROT_CHUNK 1024  // complex elements of H per CTA

__global__ void __launch_bounds__(256) msp_assemble_rotated_kernel(
    const double *__restrict__ rot, const double *__restrict__ tensors, int num_double,
    const double *__restrict__ vectors, int num_single, const cx<double> *__restrict__ basis,
    int n, cx<double> *__restrict__ H) {
    __shared__ double coef[9 * MSP_ROT_MAX_TERMS + 3 * MSP_ROT_MAX_TERMS];
    __shared__ double R[9];
    const int s = blockIdx.x, tid = threadIdx.x;
    if (tid < 9) R[tid] = rot[9 * (size_t)s + tid];
    __syncthreads();
    const int Kd = 9 * num_double, K = Kd + 3 * num_single;
    for (int k = tid; k < K; k += blockDim.x) {
        double c = 0.0;
        if (k < Kd) {  // (R T R^T)_ab = sum_cd R_ac T_cd R_bd
            const int t = k / 9, a = (k % 9) / 3, b = k % 3;
            const double *T = tensors + 9 * (size_t)t;
            for (int cc = 0; cc < 3; ++cc)
                for (int d = 0; d < 3; ++d) c += R[3 * a + cc] * T[3 * cc + d] * R[3 * b + d];
        } else {  // (R v)_a
            const int u = (k - Kd) / 3, a = (k - Kd) % 3;
            const double *v = vectors + 3 * (size_t)u;
            c = R[3 * a] * v[0] + R[3 * a + 1] * v[1] + R[3 * a + 2] * v[2];
        }
        coef[k] = c;
    }
    __syncthreads();
    const size_t nn = (size_t)n * n;
    const size_t e0 = (size_t)blockIdx.y * MSP_ROT_CHUNK;
    for (size_t e = e0 + tid; e < nn && e < e0 + MSP_ROT_CHUNK; e += blockDim.x) {
        double hr = 0.0, hi = 0.0;
        for (int k = 0; k < K; ++k) {
            const cx<double> b = basis[(size_t)k * nn + e];
            hr = fma(coef[k], b.re, hr);
            hi = fma(coef[k], b.im, hi);
        }
        H[(size_t)s * nn + e] = mk<double>(hr, hi);
    }
}

}  // namespace msp

using namespace msp;

extern "C" int msp_assemble_rotated(const double *rot, int batch, const double *tensors,
                                    int num_double, const double *vectors, int num_single,
                                    const double *basis, int n, double *H, void *stream) {
    if (batch < 0 || n < 1 || num_double < 0 || num_single < 0)
        return record_error(MSP_ERR_ARG, "msp_assemble_rotated: negative size or n < 1");
    if (num_double > MSP_ROT_MAX_TERMS || num_single > MSP_ROT_MAX_TERMS)
        return record_error(MSP_ERR_UNSUPPORTED,
                            "msp_assemble_rotated: more than 64 double or 64 single terms");
    if (batch == 0) return MSP_OK;
    if (rot == NULL || basis == NULL || H == NULL || (num_double && tensors == NULL) ||
        (num_single && vectors == NULL))
        return record_error(MSP_ERR_ARG, "msp_assemble_rotated: a required pointer is NULL");
    if (num_double + num_single == 0) {
        const cudaError_t e = cudaMemsetAsync(H, 0, sizeof(double) * 2 * (size_t)n * n * batch,
                                              (cudaStream_t)stream);
        return e == cudaSuccess ? MSP_OK : record_error(MSP_ERR_CUDA, cudaGetErrorString(e));
    }
    const size_t nn = (size_t)n * n;
    dim3 grid(batch, (unsigned)((nn + MSP_ROT_CHUNK - 1) / MSP_ROT_CHUNK));
    msp_assemble_rotated_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
        rot, tensors, num_double, vectors, num_single, reinterpret_cast<const cx<double> *>(basis),
        n, reinterpret_cast<cx<double> *>(H));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MSP_OK : record_error(MSP_ERR_CUDA, cudaGetErrorString(e));
}
