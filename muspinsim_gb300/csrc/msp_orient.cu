// Orientation rows -> lab-frame vectors of each configuration snapshot, on
// the device.  Replaces, per row, MuSpinConfig._validate_orient (the stored
// CONJUGATE quaternion of the Euler / polar angles, muspinsim/simconfig.py:
// 596-613; polar rows through quat_from_polar, muspinsim/utils.py:53-68) and
// the rotation of the field and the muon polarisation in
// ExperimentRunner.load_config (muspinsim/experiment.py:405-411), plus the
// orientation weight normalisation (muspinsim/simconfig.py:152-159).
//
// Quaternions are [w, x, y, z] with the Hamilton product; Euler angles
// (a, b, c) give q_z(c) q_b(b) q_z(a) with b about y ('zyz') or x ('zxz');
// the stored q* rotates a vector v to q* v q.
#include "msp_internal.cuh"

namespace msp {

struct Quat {
    double w, x, y, z;
};

__device__ __forceinline__ Quat qmul(const Quat &a, const Quat &b) {
    Quat r;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x;
    r.z = a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w;
    return r;
}

// rotation by `angle` about a coordinate axis (0 = x, 1 = y, 2 = z)
__device__ __forceinline__ Quat qaxis(int axis, double angle) {
    double s, c;
    sincos(0.5 * angle, &s, &c);
    Quat q = {c, 0.0, 0.0, 0.0};
    if (axis == 0) q.x = s;
    else if (axis == 1) q.y = s;
    else q.z = s;
    return q;
}

// q v q^-1 for a unit quaternion (v as the pure quaternion [0, v])
__device__ __forceinline__ void qrotate(const Quat &q, const double *v, double *out) {
    const Quat pv = {0.0, v[0], v[1], v[2]};
    const Quat qc = {q.w, -q.x, -q.y, -q.z};
    const Quat r = qmul(qmul(q, pv), qc);
    out[0] = r.x;
    out[1] = r.y;
    out[2] = r.z;
}

struct OrientArgs {
    const double *rows;
    int num_rows, row_len, euler_axis;  // euler_axis: 1 'zyz', 0 'zxz'
    double B[3], p[3], Bi[3];
    double wnorm;
    double *field, *pol, *weight;
};

__global__ void msp_orient_kernel(OrientArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.num_rows) return;
    const double *r = a.rows + (size_t)k * a.row_len;
    double ea, eb, ec;
    int bax = a.euler_axis;
    if (a.row_len == 2) {  // (theta, phi): Euler (phi, theta, phi) in 'zyz'
        ea = r[1];
        eb = r[0];
        ec = r[1];
        bax = 1;
    } else {
        ea = r[0];
        eb = r[1];
        ec = r[2];
    }
    const Quat q = qmul(qmul(qaxis(2, ec), qaxis(bax, eb)), qaxis(2, ea));
    const Quat qs = {q.w, -q.x, -q.y, -q.z};  // the stored conjugate
    double b[3], p[3];
    qrotate(qs, a.B, b);
    qrotate(qs, a.p, p);
    a.field[3 * (size_t)k] = b[0] + a.Bi[0];
    a.field[3 * (size_t)k + 1] = b[1] + a.Bi[1];
    a.field[3 * (size_t)k + 2] = b[2] + a.Bi[2];
    a.pol[3 * (size_t)k] = p[0];
    a.pol[3 * (size_t)k + 1] = p[1];
    a.pol[3 * (size_t)k + 2] = p[2];
    if (a.weight) {
        const double w = (a.row_len == 4 && a.num_rows > 1) ? r[3] : 1.0;
        a.weight[k] = w * a.wnorm;
    }
}

}  // namespace msp

using namespace msp;

namespace msp {
int record_error(int code, const char *msg);
}

extern "C" int msp_orient_snapshots(const double *rows, int num_rows, int row_len,
                                    int euler_mode, const double *B, const double *p,
                                    const double *B_intr, double weight_norm, double *field,
                                    double *pol, double *weight, void *stream) {
    if (num_rows < 0 || row_len < 2 || row_len > 4 || (euler_mode != 0 && euler_mode != 1))
        return record_error(MSP_ERR_ARG,
                            "msp_orient_snapshots: num_rows < 0, row_len outside 2..4 or "
                            "euler_mode not 0 ('zyz') / 1 ('zxz')");
    if (num_rows == 0) return MSP_OK;
    if (rows == NULL || B == NULL || p == NULL || field == NULL || pol == NULL)
        return record_error(MSP_ERR_ARG, "msp_orient_snapshots: a required pointer is NULL");
    OrientArgs a;
    a.rows = rows;
    a.num_rows = num_rows;
    a.row_len = row_len;
    a.euler_axis = euler_mode == 0 ? 1 : 0;
    for (int i = 0; i < 3; ++i) {
        a.B[i] = B[i];
        a.p[i] = p[i];
        a.Bi[i] = B_intr ? B_intr[i] : 0.0;
    }
    a.wnorm = weight_norm;
    a.field = field;
    a.pol = pol;
    a.weight = weight;
    msp_orient_kernel<<<(num_rows + 255) / 256, 256, 0, (cudaStream_t)stream>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(MSP_ERR_CUDA, cudaGetErrorString(e));
    return MSP_OK;
}
