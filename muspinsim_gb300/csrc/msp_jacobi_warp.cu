// FP32 cyclic Jacobi with one warp per Hamiltonian (n <= 32), the first
// stage of the MIXED snapshot pipeline for batches under 4,096 snapshots
// (larger ones take msp_ql_warp.cu's Householder + QL): replaces the FP32
// sweeps of Hermitian.diag's eigensolve (muspinsim/spinop.py:51-82) for the
// batched snapshots of ExperimentRunner (muspinsim/experiment.py:332-341,
// 434-498).
// The second stage (msp_snap.cu, PRE variants) refines the eigenvectors
// this kernel leaves in scratch.
//
// Why a warp per matrix: with one CTA per matrix, every Jacobi step of a
// 24 x 24 matrix ended in a CTA-wide barrier, the top stall of that kernel.
// A warp needs only __syncwarp, and several matrices share an SM.
//
// Layout.  m = n rounded up to even, h = m / 2 pairs.  The rotation pairs
// of every step are the positions (2k, 2k+1); between steps the positions
// are permuted by the round-robin ("circle") schedule: position 0 stays,
// the others move one place along the ring
//   t_1 -> t_2 -> ... -> t_{h-1} -> b_{h-1} -> b_{h-2} -> ... -> b_0 -> t_1
// (t_k = 2k, b_k = 2k+1), so every pair of indices meets once in m - 1
// steps and a full sweep returns every index to its own position.  The
// permutation is folded into where each updated element is stored.
//   * H, upper triangle, as h (h + 1) / 2 blocks of 2 x 2 complex (block
//     (X, Y), X <= Y, holds rows 2X..2X+1 and columns 2Y..2Y+1; first rows
//     and second rows in two separate arrays, jw_slot); a diagonal
//     block keeps only its coupling (2X, 2X+1), the diagonal entries are
//     tracked separately.  Double-buffered: step s reads one buffer and
//     writes the permuted result into the other.
//   * The eigenvector matrix U (U <- U G): lane r keeps row r in registers;
//     the rotations of a step act on register pairs (2k, 2k+1), then the
//     row is permuted like the positions.
// A step: each lane updates whole off-diagonal 2 x 2 blocks,
// B' = G_k1^H B G_k2, and stores every element at its permuted place
// (conjugated when it lands in the lower triangle: a store code is the
// element's byte offset with the conjugation in bit 31, so a store is a
// mask, an add and a sign-bit xor); the elements that
// become next-step couplings land in the diagonal blocks.  After a
// __syncwarp, lane X computes next-step pair X's rotation from its coupling
// and the two diagonal entries (this step's rotated diagonal, moved), and
// stores the zero left by this step's pair X at its new place.  The
// rotation arithmetic uses the hardware reciprocal and reciprocal square
// root: a rotation only has to stay unitary to FP32 rounding, and the
// refinement stage restores full accuracy.  Convergence test and tolerances are those of
// msp_jacobi.cuh (FP32: off-diagonal norm <= 4e-7 of the total, or a
// rounding floor of 2e-5 that a sweep no longer shrinks).
#include "msp_internal.cuh"
#include "msp_jacobi.cuh"

namespace msp {

namespace {

constexpr int JW_WARPS = 4;  // matrices per CTA

// Next position of the element at position p (h pairs).
__host__ __device__ constexpr int jw_next(int p, int h) {
    return p == 0 ? 0
                  : ((p & 1) ? ((p >> 1) == 0 ? 2 : p - 2)
                             : ((p >> 1) == h - 1 ? p + 1 : p + 2));
}

// Previous position of the element now at position p (the inverse of
// jw_next).
__host__ __device__ constexpr int jw_prev(int p, int h) {
    return p == 0 ? 0
                  : (p == 2 ? 1
                            : ((p & 1) == 0 ? p - 2 : (p == 2 * h - 1 ? p - 1 : p + 2)));
}

// Storage index of block (X, Y), X <= Y: diagonal blocks first.
__host__ __device__ constexpr int jw_blk(int X, int Y, int h) {
    return X == Y ? X : h + X * (2 * h - X - 1) / 2 + (Y - X - 1);
}

// float2 index of slot s (row-in-pair * 2 + column-in-pair) of block b:
// slots 0, 1 of every block in one array and slots 2, 3 in another, so that
// a lane reads its block's two rows with two conflict-free 16-byte loads.
__host__ __device__ constexpr int jw_slot(int b, int s, int h) {
    return (s >> 1) * (h * (h + 1)) + 2 * b + (s & 1);
}

// Route code of one updated element: destination float2 index (15 bits)
// and a conjugate flag (bit 15) when the element lands in the lower
// triangle.  A next-step coupling (both positions in pair X) goes to slot 1
// of diagonal block X as element (2X, 2X+1).
__device__ __forceinline__ unsigned jw_route(int x0, int y0, int h) {
    const int x = jw_next(x0, h), y = jw_next(y0, h);
    const int X = x >> 1, Y = y >> 1;
    if (X < Y) return (unsigned)jw_slot(jw_blk(X, Y, h), (x & 1) * 2 + (y & 1), h);
    if (X > Y) return (unsigned)jw_slot(jw_blk(Y, X, h), (y & 1) * 2 + (x & 1), h) | (1u << 15);
    return (unsigned)jw_slot(X, 1, h) | ((unsigned)(x & 1) << 15);
}

// Rotation [[c, s], [-conj(s), c]] zeroing apq (diagonal app, aqq) and the
// new diagonal entries, couplings at or below `skip` left alone; float4
// (c, s.re, s.im, 0).
__device__ __forceinline__ float4 jw_rotation(float app, float aqq, float2 apq, float skip,
                                              float &na, float &nb) {
    const float mag2 = fmaf(apq.x, apq.x, apq.y * apq.y);
    na = app;
    nb = aqq;
    if (!(mag2 > skip * skip)) return make_float4(1.f, 0.f, 0.f, 0.f);
    const float rinv = rsqrtf(mag2), mag = mag2 * rinv;
    const float zeta = 0.5f * (aqq - app) * rinv;
    // t = sign(zeta) / (|zeta| + sqrt(zeta^2 + 1)) from the hardware
    // reciprocal and reciprocal square root: a rotated coupling above `skip`
    // bounds |zeta| by ~5e7 (zeta^2 + 1 stays far from overflow), and an
    // approximate t still gives an exactly-normalised rotation below
    const float q1 = fmaf(zeta, zeta, 1.f);
    const float t = copysignf(__fdividef(1.f, fabsf(zeta) + q1 * rsqrtf(q1)), zeta);
    const float c = rsqrtf(fmaf(t, t, 1.f));
    const float f = t * c * rinv;
    na = app - t * mag;
    nb = aqq + t * mag;
    return make_float4(c, f * apq.x, f * apq.y, 0.f);
}

template <int M>
struct JwShape {
    static constexpr int H = M / 2;
    static constexpr int NB = H * (H + 1) / 2;  // blocks
    static constexpr int NOFF = NB - H;         // off-diagonal blocks
};

// Per-warp shared memory (floats): two H buffers, two rotation tables, two
// diagonal tables.
template <int M>
__host__ __device__ constexpr int jw_warp_floats() {
    return 2 * JwShape<M>::NB * 4 * 2 + 2 * (M / 2) * 4 + 2 * M;
}

template <int M>
__host__ __device__ constexpr size_t jw_smem_bytes() {
    // route table (four 32-bit store codes + packed k1 | k2 << 8 per
    // off-diagonal block, one 16-bit code per diagonal block), then the
    // warps' areas
    return (size_t)JwShape<M>::NOFF * 20 + (size_t)JwShape<M>::H * 4 + 16 +
           (size_t)JW_WARPS * jw_warp_floats<M>() * 4;
}

__device__ __forceinline__ void jw_rotate(float4 R, cx<float> &x, cx<float> &y) {
    // (x, y) <- (c x - conj(s) y, s x + c y)
    const float c = R.x, sr = R.y, si = R.z;
    const cx<float> nx = mk<float>(c * x.re - (sr * y.re + si * y.im),
                                   c * x.im - (sr * y.im - si * y.re));
    const cx<float> ny = mk<float>(sr * x.re - si * x.im + c * y.re,
                                   sr * x.im + si * x.re + c * y.im);
    x = nx;
    y = ny;
}

}  // namespace

template <int M>
__global__ void __launch_bounds__(JW_WARPS * 32, M <= 24 ? 5 : 4) msp_jacobi_warp_kernel(SnapArgs a) {
    using S = JwShape<M>;
    constexpr int H = S::H, NB = S::NB, NOFF = S::NOFF;
    extern __shared__ __align__(16) char smem[];
    // store codes of an off-diagonal block's four elements: byte offset in
    // the H buffer, bit 31 set when the element lands conjugated
    uint4 *route = reinterpret_cast<uint4 *>(smem);                  // NOFF codes
    unsigned *kk = reinterpret_cast<unsigned *>(route + NOFF);        // NOFF k1 | k2 << 8
    unsigned *zroute = kk + NOFF;                                     // H codes
    float *wbase = reinterpret_cast<float *>(
        smem + (((size_t)NOFF * 20 + (size_t)H * 4 + 15) & ~(size_t)15));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *mine = wbase + (size_t)warp * jw_warp_floats<M>();
    // buffer b of each double-buffered table: base + b * stride
    float2 *const Hb0 = reinterpret_cast<float2 *>(mine);
    float4 *const rot0 = reinterpret_cast<float4 *>(mine + 2 * NB * 8);
    float *const dia0 = mine + 2 * NB * 8 + 2 * H * 4;
    auto Hbuf = [&](int b) { return Hb0 + b * (NB * 4); };
    auto rbuf = [&](int b) { return rot0 + b * H; };
    auto dbuf = [&](int b) { return dia0 + b * M; };

    // route tables
    for (int o = threadIdx.x; o < NOFF; o += blockDim.x) {
        int k1 = 0, rem = o;
        while (rem >= H - 1 - k1) {
            rem -= H - 1 - k1;
            ++k1;
        }
        const int k2 = k1 + 1 + rem;  // o = jw_blk(k1, k2) - H
        unsigned c[4];
        for (int r = 0; r < 2; ++r)
            for (int q = 0; q < 2; ++q) c[r * 2 + q] = jw_route(2 * k1 + r, 2 * k2 + q, H);
        unsigned b4[4];
        for (int q = 0; q < 4; ++q) b4[q] = ((c[q] & 0x7fffu) * 8u) | ((c[q] & 0x8000u) << 16);
        route[o] = make_uint4(b4[0], b4[1], b4[2], b4[3]);
        kk[o] = (unsigned)k1 | ((unsigned)k2 << 8);
    }
    for (int k = threadIdx.x; k < H; k += blockDim.x) zroute[k] = jw_route(2 * k, 2 * k + 1, H);
    __syncthreads();

    const int n = a.n;
    const int nn = n * n;
    float2 *evec = reinterpret_cast<float2 *>(a.evec);
    const float tol = JacobiConst<float>::tol, ftol = JacobiConst<float>::floor_tol;
    for (int sn = blockIdx.x * JW_WARPS + warp; sn < a.num_snap; sn += gridDim.x * JW_WARPS) {
        const SnapSource src = snap_source(a, sn);
        const double bx = a.field[3 * (size_t)src.g], by = a.field[3 * (size_t)src.g + 1],
                     bz = a.field[3 * (size_t)src.g + 2];
        const float bxf = (float)bx, byf = (float)by, bzf = (float)bz;
        // H = Hsys + b . Z (FP32 from the double-word high parts when the
        // caller pre-split the matrices, else FP64) into the blocks of
        // buffer 0, diagonal into dia[1] (free until step 0's producers
        // write it)
        float fro = 0.f;
        for (int e = lane; e < M * (M + 1) / 2; e += 32) {
            int i = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);  // e = i (i + 1) / 2 + j
            while ((i + 1) * (i + 2) / 2 <= e) ++i;
            while (i * (i + 1) / 2 > e) --i;
            const int j = e - i * (i + 1) / 2;  // j <= i: element (j, i) of the upper triangle
            float hr = 0.f, hi = 0.f;
            if (i < n) {
                const size_t o = (size_t)j * n + i;
                if (src.Hdw != nullptr) {
                    const float4 hs = src.Hdw[o], z0 = src.Zdw[o], z1 = src.Zdw[nn + o],
                                 z2 = src.Zdw[2 * (size_t)nn + o];
                    hr = fmaf(bzf, z2.x, fmaf(byf, z1.x, fmaf(bxf, z0.x, hs.x)));
                    hi = fmaf(bzf, z2.y, fmaf(byf, z1.y, fmaf(bxf, z0.y, hs.y)));
                } else {
                    const cx<double> hs = src.Hsys[o], z0 = src.Z[o], z1 = src.Z[nn + o],
                                     z2 = src.Z[2 * (size_t)nn + o];
                    hr = (float)(hs.re + bx * z0.re + by * z1.re + bz * z2.re);
                    hi = (float)(hs.im + bx * z0.im + by * z1.im + bz * z2.im);
                }
            }
            if (i == j) {
                dbuf(1)[i] = hr;
                fro += hr * hr;
            } else {
                const int X = j >> 1, Y = i >> 1;
                Hbuf(0)[jw_slot(jw_blk(X, Y, H), (j & 1) * 2 + (i & 1), H)] = make_float2(hr, hi);
                fro += 2.f * (hr * hr + hi * hi);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
        __syncwarp();
        const float skip = tol * sqrtf(fro) / (float)M;
        // rotations of step 0
        if (lane < H) {
            float na, nb;
            rbuf(0)[lane] = jw_rotation(dbuf(1)[2 * lane], dbuf(1)[2 * lane + 1],
                                        Hbuf(0)[jw_slot(lane, 1, H)], skip, na, nb);
            dbuf(0)[2 * lane] = na;
            dbuf(0)[2 * lane + 1] = nb;
        }
        // U = I: lane r holds row r
        cx<float> u[M];
#pragma unroll
        for (int p = 0; p < M; ++p) u[p] = mk<float>(p == lane ? 1.f : 0.f, 0.f);
        __syncwarp();

        int cur = 0;
        int status = MSP_ITEM_NOT_CONVERGED;
        float prev_off = -1.f;
        for (int sweep = 0;; ++sweep) {
            // off-diagonal norm (both triangles) of buffer cur
            float off = 0.f;
            for (int t = lane; t < NB; t += 32) {
                if (t < H) {
                    const float2 v = Hbuf(cur)[jw_slot(t, 1, H)];
                    off += 2.f * (v.x * v.x + v.y * v.y);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float2 v = Hbuf(cur)[jw_slot(t, q, H)];
                        off += 2.f * (v.x * v.x + v.y * v.y);
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
            if (off <= tol * tol * fro) {
                status = MSP_ITEM_OK;
                break;
            }
            if (prev_off >= 0.f && off > 0.25f * prev_off && off <= ftol * ftol * fro) {
                status = MSP_ITEM_OK;
                break;
            }
            if (sweep >= a.max_sweeps) break;
            prev_off = off;
            for (int step = 0; step < M - 1; ++step) {
                const int nxt = cur ^ 1;
                const float4 *rc = rbuf(cur);
                const float *dc = dbuf(cur);
                float2 *Hn = Hbuf(nxt);
                // eigenvector row: rotate the register pairs, then permute
                if (lane < M) {
#pragma unroll
                    for (int k = 0; k < H; ++k) jw_rotate(rc[k], u[2 * k], u[2 * k + 1]);
                    cx<float> w[M];
#pragma unroll
                    for (int p = 0; p < M; ++p) w[jw_next(p, H)] = u[p];
#pragma unroll
                    for (int p = 0; p < M; ++p) u[p] = w[p];
                }
                // full rounds of whole blocks; a short last round (at most 8
                // blocks, m = 24: 2 of 66) is split into single elements over
                // four lanes per block instead of leaving 30 lanes idle
                constexpr int FULL = (NOFF / 32) * 32, LEFT = NOFF - FULL;
                constexpr bool SPLIT = LEFT > 0 && 4 * LEFT <= 32;
                for (int o = lane; o < (SPLIT ? FULL : NOFF); o += 32) {
                    const unsigned k12 = kk[o];
                    const int k1 = (int)(k12 & 255u), k2 = (int)(k12 >> 8);
                    const float2 *B = Hbuf(cur);
                    const float4 bA = *reinterpret_cast<const float4 *>(B + jw_slot(H + o, 0, H));
                    const float4 bB = *reinterpret_cast<const float4 *>(B + jw_slot(H + o, 2, H));
                    const cx<float> b00 = mk<float>(bA.x, bA.y), b01 = mk<float>(bA.z, bA.w);
                    const cx<float> b10 = mk<float>(bB.x, bB.y), b11 = mk<float>(bB.z, bB.w);
                    const float4 R1 = rc[k1], R2 = rc[k2];
                    const float c1 = R1.x, c2 = R2.x;
                    const cx<float> s1 = mk<float>(R1.y, R1.z), s2 = mk<float>(R2.y, R2.z);
                    // T = G1^H B
                    const cx<float> t00 = cadd(cscale(c1, b00), cscale(-1.f, cmul(s1, b10)));
                    const cx<float> t01 = cadd(cscale(c1, b01), cscale(-1.f, cmul(s1, b11)));
                    const cx<float> t10 = cadd(cmulc(s1, b00), cscale(c1, b10));
                    const cx<float> t11 = cadd(cmulc(s1, b01), cscale(c1, b11));
                    // B' = T G2
                    cx<float> nv[4];
                    nv[0] = cadd(cscale(c2, t00), cscale(-1.f, cmulc(s2, t01)));
                    nv[1] = cadd(cmul(s2, t00), cscale(c2, t01));
                    nv[2] = cadd(cscale(c2, t10), cscale(-1.f, cmulc(s2, t11)));
                    nv[3] = cadd(cmul(s2, t10), cscale(c2, t11));
                    const uint4 rt = route[o];
                    const unsigned cq[4] = {rt.x, rt.y, rt.z, rt.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        *reinterpret_cast<float2 *>(reinterpret_cast<char *>(Hn) +
                                                    (cq[q] & 0x7fffffffu)) =
                            make_float2(nv[q].re, __uint_as_float(__float_as_uint(nv[q].im) ^
                                                                  (cq[q] & 0x80000000u)));
                }
                if (SPLIT && lane < 4 * LEFT) {
                    // element (r, cc) of B' = G1^H B G2 for block FULL + lane / 4
                    const int o = FULL + (lane >> 2), q = lane & 3, r = q >> 1, cc = q & 1;
                    const unsigned k12 = kk[o];
                    const int k1 = (int)(k12 & 255u), k2 = (int)(k12 >> 8);
                    const float2 *B = Hbuf(cur);
                    const float4 bA = *reinterpret_cast<const float4 *>(B + jw_slot(H + o, 0, H));
                    const float4 bB = *reinterpret_cast<const float4 *>(B + jw_slot(H + o, 2, H));
                    const cx<float> b00 = mk<float>(bA.x, bA.y), b01 = mk<float>(bA.z, bA.w);
                    const cx<float> b10 = mk<float>(bB.x, bB.y), b11 = mk<float>(bB.z, bB.w);
                    const float4 R1 = rc[k1], R2 = rc[k2];
                    const float c1 = R1.x, c2 = R2.x;
                    const cx<float> s1 = mk<float>(R1.y, R1.z), s2 = mk<float>(R2.y, R2.z);
                    // row r of T = G1^H B
                    const cx<float> t0 = r == 0 ? cadd(cscale(c1, b00), cscale(-1.f, cmul(s1, b10)))
                                                : cadd(cmulc(s1, b00), cscale(c1, b10));
                    const cx<float> t1 = r == 0 ? cadd(cscale(c1, b01), cscale(-1.f, cmul(s1, b11)))
                                                : cadd(cmulc(s1, b01), cscale(c1, b11));
                    const cx<float> v = cc == 0 ? cadd(cscale(c2, t0), cscale(-1.f, cmulc(s2, t1)))
                                                : cadd(cmul(s2, t0), cscale(c2, t1));
                    const unsigned cq = reinterpret_cast<const unsigned *>(route + o)[q];
                    *reinterpret_cast<float2 *>(reinterpret_cast<char *>(Hn) + (cq & 0x7fffffffu)) =
                        make_float2(v.re, __uint_as_float(__float_as_uint(v.im) ^ (cq & 0x80000000u)));
                }
                __syncwarp();
                // next-step rotations; this step's zeroed couplings moved
                if (lane < H) {
                    Hn[zroute[lane] & 0x7fffu] = make_float2(0.f, 0.f);
                    float na, nb;
                    rbuf(nxt)[lane] = jw_rotation(dc[jw_prev(2 * lane, H)],
                                                  dc[jw_prev(2 * lane + 1, H)],
                                                  Hn[jw_slot(lane, 1, H)], skip, na, nb);
                    dbuf(nxt)[2 * lane] = na;
                    dbuf(nxt)[2 * lane + 1] = nb;
                }
                __syncwarp();
                cur = nxt;
            }
        }
        // eigenvectors (columns of U) to scratch: row r of U is lane r
        if (lane < n) {
            float2 *dst = evec + (size_t)sn * nn + (size_t)lane * n;
#pragma unroll
            for (int p = 0; p < M; ++p)
                if (p < n) dst[p] = make_float2(u[p].re, u[p].im);
        }
        if (lane == 0) a.status[src.g] = status;
        __syncwarp();
    }
}

template <int M>
static cudaError_t jw_launch(const SnapArgs &a, cudaStream_t st) {
    const size_t smem = jw_smem_bytes<M>();
    cudaError_t e = cudaFuncSetAttribute(msp_jacobi_warp_kernel<M>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0, sms = 0, dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msp_jacobi_warp_kernel<M>,
                                                          JW_WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    long long grid = (a.num_snap + JW_WARPS - 1) / JW_WARPS;
    const long long cap = (long long)sms * (occ > 0 ? occ : 1);
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    msp_jacobi_warp_kernel<M><<<(int)grid, JW_WARPS * 32, smem, st>>>(a);
    return cudaGetLastError();
}

bool jacobi_warp_supported(int n) {
    const int m = n + (n & 1);
    return m >= 4 && m <= 32;
}

// First stage of the two-stage MIXED snapshots.  Batches of 4,096 snapshots
// or more take the Householder + QL form (msp_ql_warp.cu: at 10,000
// snapshots of dimension 24 it takes 0.55 ms against the Jacobi's 0.86 ms,
// and 20% less at dimension 32); smaller batches fill the GPU with too few
// of its four-matrix warp tasks and keep the Jacobi (at 4,000 snapshots the
// two tie).  MSP_EIGH_WARP = 0 or 2 pins one form.
#ifndef MSP_EIGH_WARP
#define MSP_EIGH_WARP 1
#endif
cudaError_t launch_jacobi_warp(const SnapArgs &a, cudaStream_t st) {
    if (MSP_EIGH_WARP == 2 && ql_warp_supported(a.n)) return launch_ql_warp(a, st);
    if (MSP_EIGH_WARP == 1 && ql_warp_supported(a.n) && a.num_snap >= 4096)
        return launch_ql_warp(a, st);
    if (a.num_snap <= 0) return cudaSuccess;
    switch (a.n + (a.n & 1)) {
        case 4: return jw_launch<4>(a, st);
        case 6: return jw_launch<6>(a, st);
        case 8: return jw_launch<8>(a, st);
        case 10: return jw_launch<10>(a, st);
        case 12: return jw_launch<12>(a, st);
        case 14: return jw_launch<14>(a, st);
        case 16: return jw_launch<16>(a, st);
        case 18: return jw_launch<18>(a, st);
        case 20: return jw_launch<20>(a, st);
        case 22: return jw_launch<22>(a, st);
        case 24: return jw_launch<24>(a, st);
        case 26: return jw_launch<26>(a, st);
        case 28: return jw_launch<28>(a, st);
        case 30: return jw_launch<30>(a, st);
        case 32: return jw_launch<32>(a, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace msp
