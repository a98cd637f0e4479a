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

// Generated grids times a field list: snapshot s = f * num_orient + o.
struct GridArgs {
    int kind, n, gen, euler_axis;  // kind: MSP_GRID_*; gen: ZCW generator g
    int num_orient, num_fields;
    const double *B;               // num_fields x 3 (device)
    double p[3], Bi[3];
    double wnorm;
    double *field, *pol, *weight;
    int *slot;
};

// Euler angles (a, b, c) in the grid's convention and the row weight of
// grid point o: ZCW (theta, phi) rows as polar angles (Euler (phi, theta,
// phi), 'zyz'), eulrange (a, b, c, sin b).
__device__ __forceinline__ void grid_point(const GridArgs &g, int o, double &ea, double &eb,
                                           double &ec, double &w, int &bax) {
    const double twopi = 6.283185307179586476925;
    if (g.kind == MSP_GRID_EULRANGE) {
        const int N = g.n;
        const int k = o % N, j = (o / N) % N, i = o / (N * N);
        const double da = N > 1 ? twopi / (double)(N - 1) : 0.0;
        ea = j == N - 1 && N > 1 ? twopi : (double)j * da;
        eb = (double)(i + 1) * (3.14159265358979323846 / (double)(N + 1));
        ec = k == N - 1 && N > 1 ? twopi : (double)k * da;
        w = sin(eb);
        bax = g.euler_axis;
    } else {
        // beta = arccos(c1 (c2 j / N - 1)), alpha = 2 pi frac(j g / N)
        const double c1 = g.kind == MSP_GRID_ZCW_HEMISPHERE ? -1.0 : 1.0;
        const double c2 = g.kind == MSP_GRID_ZCW_HEMISPHERE ? 1.0 : 2.0;
        double x = c1 * (c2 * ((double)o / (double)g.n) - 1.0);
        x = fmin(1.0, fmax(-1.0, x));
        const double theta = acos(x);
        const long long jg = ((long long)o * (long long)g.gen) % (long long)g.n;
        const double phi = twopi * ((double)jg / (double)g.n);
        ea = phi;
        eb = theta;
        ec = phi;
        w = 1.0;
        bax = 1;
    }
}

__global__ void msp_orient_grid_kernel(GridArgs g) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)g.num_orient * g.num_fields;
    if (s >= total) return;
    const int f = (int)(s / g.num_orient), o = (int)(s - (long long)f * g.num_orient);
    double ea, eb, ec, w;
    int bax;
    grid_point(g, o, ea, eb, ec, w, bax);
    const Quat q = qmul(qmul(qaxis(2, ec), qaxis(bax, eb)), qaxis(2, ea));
    const Quat qs = {q.w, -q.x, -q.y, -q.z};  // the stored conjugate
    double b[3], p[3];
    qrotate(qs, g.B + 3 * (size_t)f, b);
    qrotate(qs, g.p, p);
    for (int i = 0; i < 3; ++i) {
        g.field[3 * s + i] = b[i] + g.Bi[i];
        g.pol[3 * s + i] = p[i];
    }
    g.weight[s] = (g.num_orient > 1 ? w : 1.0) * g.wnorm;
    if (g.slot) g.slot[s] = f;
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

extern "C" int msp_orient_grid_snapshots(int grid_kind, int grid_n, int zcw_generator,
                                         int euler_mode, const double *fields, int num_fields,
                                         const double *p, const double *B_intr,
                                         double weight_norm, double *field, double *pol,
                                         double *weight, int *slot, void *stream) {
    if (grid_kind < MSP_GRID_ZCW_SPHERE || grid_kind > MSP_GRID_EULRANGE || grid_n < 1 ||
        num_fields < 0 || (euler_mode != 0 && euler_mode != 1))
        return record_error(MSP_ERR_ARG,
                            "msp_orient_grid_snapshots: unknown grid kind, grid_n < 1, "
                            "num_fields < 0 or euler_mode not 0 / 1");
    long long num_orient = grid_kind == MSP_GRID_EULRANGE
                               ? (long long)grid_n * grid_n * grid_n : (long long)grid_n;
    if (grid_kind != MSP_GRID_EULRANGE &&
        (zcw_generator < 1 || (grid_n > 1 && zcw_generator >= grid_n)))
        return record_error(MSP_ERR_ARG,
                            "msp_orient_grid_snapshots: ZCW generator outside 1 .. grid_n - 1");
    if (num_orient * (long long)num_fields > (1LL << 31) - 1)
        return record_error(MSP_ERR_UNSUPPORTED,
                            "msp_orient_grid_snapshots: more than 2^31 - 1 snapshots");
    if (num_fields == 0) return MSP_OK;
    if (fields == NULL || p == NULL || field == NULL || pol == NULL || weight == NULL)
        return record_error(MSP_ERR_ARG, "msp_orient_grid_snapshots: a required pointer is NULL");
    GridArgs g;
    g.kind = grid_kind;
    g.n = grid_n;
    g.gen = zcw_generator;
    g.euler_axis = euler_mode == 0 ? 1 : 0;
    g.num_orient = (int)num_orient;
    g.num_fields = num_fields;
    g.B = fields;
    for (int i = 0; i < 3; ++i) {
        g.p[i] = p[i];
        g.Bi[i] = B_intr ? B_intr[i] : 0.0;
    }
    g.wnorm = weight_norm;
    g.field = field;
    g.pol = pol;
    g.weight = weight;
    g.slot = slot;
    const long long total = num_orient * num_fields;
    msp_orient_grid_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(g);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(MSP_ERR_CUDA, cudaGetErrorString(e));
    return MSP_OK;
}
