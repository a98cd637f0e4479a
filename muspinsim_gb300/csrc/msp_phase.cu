// Time-domain kernels: the phase sum over eigenvalue pairs, its work
// schedule and its deterministic reduction into output rows, plus the small
// single-Hamiltonian building blocks of the C ABI.
//
// The phase sum replaces the per-snapshot time loops of the reference --
// the Cython cosine sum (muspinsim/cython/parallel.pyx:59-67) and the
// evolve loop (muspinsim/hamiltonian.py:95-107) -- and the accumulation of
// MuSpinConfig.store_time_slice (muspinsim/simconfig.py:347-368): all pairs
// of all snapshots that feed one output row are summed on the device.
//
// Uniform grids t_k = t0 + k dt use a blocked form.  A time tile of
// 64 x 64 samples, k = 64 k1 + k0, factorises every term:
//   Re[(a_c - i a_s) e^{i w t_k}] = Re[X_m(k1) Y_m(k0)],
//   X_m(k1) = (a_c - i a_s) e^{i w (t_tile + 64 k1 dt)},  Y_m(k0) = e^{i w k0 dt},
// so each tile is a sum of outer products -- 2 FMAs per (pair, sample) in
// register tiles, with no per-sample sin/cos.  X and Y come from a phase
// recurrence: five exactly reduced phases per pair (w dt, 8 w dt, 64 w dt,
// 512 w dt, w t_tile, reduced modulo 2 pi in FP64), their sin/cos, then
// products of short power tables -- at most 16 rounding steps from an exact
// value, which is the periodic resync.
#include <stdlib.h>

#include "msp_dw.cuh"
#include "msp_internal.cuh"

namespace msp {

template <typename T>
struct PhaseCfg;
template <>
struct PhaseCfg<float> {
    enum { TM = 8, TN = 8, PS = 32 };
};
template <>
struct PhaseCfg<double> {
    enum { TM = 4, TN = 8, PS = 16 };
};

__device__ __forceinline__ void sincos_t(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, float *s, float *c) {
    sincosf((float)x, s, c);
}

// Pair range [begin, end) of work item `item`; begin = -1 when the item does
// not exist.  item_first / slot_first are num_slots + 1 prefix arrays; the
// items of a slot cover its pairs in runs of IP.
__device__ __forceinline__ void item_range(const PhaseArgs &a, int item, int *b, int *e) {
    const int total = a.item_first[a.num_slots];
    if (item >= total) {
        *b = -1;
        *e = -1;
        return;
    }
    int lo = 0, hi = a.num_slots - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.item_first[mid] <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int pb = a.slot_first[lo] * a.P + (item - a.item_first[lo]) * a.IP;
    const int slot_end = a.slot_first[lo + 1] * a.P;
    const int pe = pb + a.IP;
    *b = pb;
    *e = pe < slot_end ? pe : slot_end;
}

template <typename T>
__global__ void __launch_bounds__(128) msp_phase_uniform_kernel(PhaseArgs a) {
    constexpr int K = 64, TM = PhaseCfg<T>::TM, TN = PhaseCfg<T>::TN, PS = PhaseCfg<T>::PS;
    constexpr int TY = K / TM, TX = K / TN, TPG = TY * TX, GROUPS = 128 / TPG;
    typedef typename PairCoef<T>::type coef_t;
    typedef cx<T> C;
    __shared__ __align__(16) C Xs[PS][K];
    __shared__ __align__(16) C Ys[PS][K];
    // power tables, pair index last with a padded stride: the chain writes
    // (consecutive pairs) and the table-fill reads (8 powers of one pair)
    // both hit distinct banks
    __shared__ __align__(16) C pw[4][8][PS + 1];
    __shared__ __align__(16) C pc[PS];  // (a_c - i a_s) e^{i w t_tile}
    __shared__ int s_range[2];

    const int tid = threadIdx.x;
    if (tid == 0) item_range(a, blockIdx.x, &s_range[0], &s_range[1]);
    __syncthreads();
    const int pbeg = s_range[0], pend = s_range[1];
    if (pbeg < 0) return;

    const int g = tid / TPG, lt = tid - (tid / TPG) * TPG;
    const int ty = lt / TX, tx = lt - (lt / TX) * TX;
    const double dt = a.dt;
    const long long tile_base = (long long)blockIdx.y * (K * K);
    const double tb = a.t0 + (double)tile_base * dt;
    const coef_t *coef = reinterpret_cast<const coef_t *>(a.pair_coef);

    T acc[TM][TN];
#pragma unroll
    for (int r = 0; r < TM; ++r)
#pragma unroll
        for (int c = 0; c < TN; ++c) acc[r][c] = T(0);

    for (int pb = pbeg; pb < pend; pb += PS) {
        const int np = (pend - pb) < PS ? (pend - pb) : PS;
        // setup, spread over the CTA: thread (chain c, pair i) reduces the
        // phase 8^c w dt exactly in FP64 and builds that chain's 8 powers;
        // chain 0 also forms the tile-start coefficient
        for (int e = tid; e < 4 * PS; e += 128) {
            const int c = e / PS, i = e - (e / PS) * PS;
            if (i < np) {
                const double w = a.pair_omega[pb + i];
                double ph = reduce_2pi(w * dt);
                for (int q = 0; q < c; ++q) ph = reduce_2pi(8.0 * ph);
                C base;
                sincos_t(ph, &base.im, &base.re);
                C p = mk<T>(T(1), T(0));
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    pw[c][r][i] = p;
                    p = cmul(p, base);
                }
                if (c == 0) {
                    const coef_t cf = coef[pb + i];
                    C e0;
                    sincos_t(reduce_2pi(w * tb), &e0.im, &e0.re);
                    pc[i] = cmul(mk<T>((T)cf.x, (T)(-cf.y)), e0);
                }
            }
        }
        __syncthreads();
        // Y[k0] = e^{i w dt k0}, X[k1] = coef e^{i w (t_tile + 64 dt k1)}
        for (int e = tid; e < np * 2 * K; e += 128) {
            const int i = e / (2 * K), k = e - (e / (2 * K)) * (2 * K);
            if (k < K) {
                Ys[i][k] = cmul(pw[1][k >> 3][i], pw[0][k & 7][i]);
            } else {
                const int kk = k - K;
                Xs[i][kk] = cmul(pc[i], cmul(pw[3][kk >> 3][i], pw[2][kk & 7][i]));
            }
        }
        __syncthreads();
        for (int i = g; i < np; i += GROUPS) {
            C xv[TM], yv[TN];
#pragma unroll
            for (int r = 0; r < TM; ++r) xv[r] = Xs[i][ty + TY * r];
#pragma unroll
            for (int c = 0; c < TN; ++c) yv[c] = Ys[i][tx + TX * c];
#pragma unroll
            for (int r = 0; r < TM; ++r)
#pragma unroll
                for (int c = 0; c < TN; ++c) {
                    acc[r][c] = fma(xv[r].re, yv[c].re, acc[r][c]);
                    acc[r][c] = fma(-xv[r].im, yv[c].im, acc[r][c]);
                }
        }
        __syncthreads();
    }

    // combine the groups (they summed disjoint pairs of the same tile)
    T *red = reinterpret_cast<T *>(&Xs[0][0]);  // K*K values fit in Xs+Ys
    if (GROUPS > 1) {
        for (int gg = 1; gg < GROUPS; ++gg) {
            if (g == gg) {
#pragma unroll
                for (int r = 0; r < TM; ++r)
#pragma unroll
                    for (int c = 0; c < TN; ++c) {
                        const int k = (ty + TY * r) * K + tx + TX * c;
                        red[k] = (gg == 1) ? acc[r][c] : red[k] + acc[r][c];
                    }
            }
            __syncthreads();
        }
    }
    if (g == 0) {
        double *out = a.partial + (size_t)blockIdx.x * a.num_times;
#pragma unroll
        for (int r = 0; r < TM; ++r)
#pragma unroll
            for (int c = 0; c < TN; ++c) {
                const int k = (ty + TY * r) * K + tx + TX * c;
                const long long t = tile_base + k;
                double v = (double)acc[r][c];
                if (GROUPS > 1) v += (double)red[k];
                if (t < a.num_times) out[t] = v;
            }
    }
}

// ---------------------------------------------------------------- FP32 path
//
// Mixed precision on a uniform grid.  Same tiling as above, two changes:
//  * no FP64 on the GPU's slow FP64 pipe: the snapshot kernel stored each
//    pair's phases psi = w dt and phi0 = w t0 already reduced modulo 2 pi as
//    double-word floats (hi + lo); the chain phases 8^c psi are exact float
//    scalings, reduced again in double-word arithmetic, then evaluated as
//    sincosf(hi) turned by the small angle lo;
//  * the outer products use the packed FP32x2 FMA of sm_100-class GPUs
//    (fma.rn.f32x2): two accumulators of adjacent time columns per
//    instruction, half the issue slots of scalar FMAs.

// MSP_TWOPI_HI / _LO, dw_reduce_2pi and dw_add: msp_dw.cuh.

// e^{i (h + l)} for |l| <~ 1e-3: sincosf(h) turned by l, second order in l.
__device__ __forceinline__ cx<float> dw_expi(float h, float l) {
    float s, c;
    sincosf(h, &s, &c);
    const float cl = 1.0f - 0.5f * l * l;
    return mk<float>(c * cl - s * l, s * cl + c * l);
}

__device__ __forceinline__ unsigned long long pk2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ void ffma2(unsigned long long &acc, unsigned long long a,
                                      unsigned long long b) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}

__global__ void __launch_bounds__(128, 4) msp_phase_uniform_f32_kernel(PhaseArgs a) {
    constexpr int K = 64, PS = 32;
    __shared__ __align__(16) cx<float> Xs[PS][K];  // (x_re, -x_im)
    __shared__ __align__(16) float Yr[PS][K];
    __shared__ __align__(16) float Yi[PS][K];
    __shared__ __align__(16) cx<float> pw[4][8][PS + 1];
    __shared__ int s_range[2];

    const int tid = threadIdx.x;
    if (tid == 0) item_range(a, blockIdx.x, &s_range[0], &s_range[1]);
    __syncthreads();
    const int pbeg = s_range[0], pend = s_range[1];
    if (pbeg < 0) return;

    const int g = tid >> 6, lt = tid & 63;
    const int ty = lt >> 3, tx = lt & 7;
    const long long tile_base = (long long)blockIdx.y * (K * K);
    const float tile_steps = (float)tile_base;  // exact: < 2^24
    const float2 *coef = reinterpret_cast<const float2 *>(a.pair_coef);

    unsigned long long acc[8][4];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[r][j] = 0ull;

    for (int pb = pbeg; pb < pend; pb += PS) {
        const int np = (pend - pb) < PS ? (pend - pb) : PS;
        {
            // thread (chain c, pair i): e^{i 8^c psi} and its powers 0..7;
            // chain 3 starts from the tile-start coefficient
            // (a_c - i a_s) e^{i (phi0 + tile_base psi)}, so that X needs one
            // product per entry
            const int c = tid >> 5, i = tid & 31;
            if (i < np) {
                const float4 rec = a.pair_phase[pb + i];
                const float sc = c == 0 ? 1.f : c == 1 ? 8.f : c == 2 ? 64.f : 512.f;
                float h = rec.x * sc, l = rec.y * sc;  // exact power-of-two scaling
                dw_reduce_2pi(h, l);
                const cx<float> base = dw_expi(h, l);
                cx<float> p = mk<float>(1.f, 0.f);
                if (c == 3) {
                    float th = rec.z, tl = rec.w;
                    if (tile_base > 0) {
                        const float ph = rec.x * tile_steps;
                        float bh = ph, bl = fmaf(rec.x, tile_steps, -ph) + rec.y * tile_steps;
                        dw_reduce_2pi(bh, bl);
                        dw_add(th, tl, bh, bl);
                        dw_reduce_2pi(th, tl);
                    }
                    const float2 cf = coef[pb + i];
                    p = mk<float>(cf.x, -cf.y);
                    if (th != 0.f || tl != 0.f) p = cmul(p, dw_expi(th, tl));
                }
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    pw[c][r][i] = p;
                    p = cmul(p, base);
                }
            }
        }
        __syncthreads();
        for (int e = tid; e < np * 2 * K; e += 128) {
            const int i = e >> 7, k = e & 127;
            if (k < K) {
                const cx<float> y = cmul(pw[1][k >> 3][i], pw[0][k & 7][i]);
                Yr[i][k] = y.re;
                Yi[i][k] = y.im;
            } else {
                const int kk = k - K;
                const cx<float> x = cmul(pw[3][kk >> 3][i], pw[2][kk & 7][i]);
                Xs[i][kk] = mk<float>(x.re, -x.im);
            }
        }
        __syncthreads();
        for (int i = g; i < np; i += 2) {
            unsigned long long yr[4], yi[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                yr[j] = *reinterpret_cast<const unsigned long long *>(&Yr[i][2 * tx + 16 * j]);
                yi[j] = *reinterpret_cast<const unsigned long long *>(&Yi[i][2 * tx + 16 * j]);
            }
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const cx<float> x = Xs[i][ty + 8 * r];
                const unsigned long long xr = pk2(x.re, x.re), xi = pk2(x.im, x.im);
                // real-part products for the four column pairs first, so that
                // no FMA waits on the one just issued
#pragma unroll
                for (int j = 0; j < 4; ++j) ffma2(acc[r][j], xr, yr[j]);
#pragma unroll
                for (int j = 0; j < 4; ++j) ffma2(acc[r][j], xi, yi[j]);
            }
        }
        __syncthreads();
    }

    // combine the two groups, then write FP32 partials (msp_reduce_kernel
    // sums them across items as double-words)
    float *red = reinterpret_cast<float *>(&Xs[0][0]);  // K*K floats
    if (g == 1) {
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float v0, v1;
                asm("mov.b64 {%0, %1}, %2;" : "=f"(v0), "=f"(v1) : "l"(acc[r][j]));
                const int k = (ty + 8 * r) * K + 2 * tx + 16 * j;
                red[k] = v0;
                red[k + 1] = v1;
            }
    }
    __syncthreads();
    if (g == 0) {
        float *out = a.partial_f32 + (size_t)blockIdx.x * a.num_times;
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float v0, v1;
                asm("mov.b64 {%0, %1}, %2;" : "=f"(v0), "=f"(v1) : "l"(acc[r][j]));
                const int k = (ty + 8 * r) * K + 2 * tx + 16 * j;
                const long long t = tile_base + k;
                if (t < a.num_times) out[t] = v0 + red[k];
                if (t + 1 < a.num_times) out[t + 1] = v1 + red[k + 1];
            }
    }
}

// ---------------------------------------------------------------- tensor-core path
//
// Mixed precision on a uniform grid, on the 5th-generation tensor cores.
// A time tile of 128 x N samples (k = N k1 + k0) is the GEMM
//   D[k1][k0] = sum_m A[k1][m] B[k0][m],  m = 2 p + {0: re, 1: im},
//   A[k1][2p] = Re X_p(k1),  A[k1][2p+1] = -Im X_p(k1),
//   B[k0][2p] = Re Y_p(k0),  B[k0][2p+1] =  Im Y_p(k0),
// with X and Y the factors of the SIMT kernel above (D = sum_p Re X_p Y_p).
// Operands are FP32 values split as x = hi + lo, hi = tf32(x), lo =
// tf32(x - hi) (round to nearest), and D accumulates hi.hi + hi.lo + lo.hi
// (3xTF32: ~2^-22 relative per product) in FP32 in tensor memory.
//
// Per CTA (128 threads, one work item, one time tile):
//   * stages of 16 pairs (K = 32 per stage, 4 MMAs of K = 8 per product),
//     double-buffered in shared memory; all threads build a stage's power
//     tables and operands (K-major, no swizzle: 8-row x 16-byte core
//     matrices, the K-direction stride in the descriptor's leading byte
//     offset, the 8-row-group stride in its stride byte offset) while the
//     tensor core runs the previous stage;
//   * one thread issues the stage's 12 tcgen05.mma (cta_group::1,
//     kind::tf32, M = 128) and commits them to the buffer's mbarrier, which
//     the thread building the stage after next waits on before overwriting
//     the buffer;
//   * the epilogue reads the 128 x N accumulator with tcgen05.ld (warp w owns
//     TMEM lanes 32w .. 32w + 31 = rows k1), transposes it through shared
//     memory and writes the item's FP32 partials coalesced.
// Every wait is bounded; a wait that runs out marks the tile's partials NaN
// (the powder average then reads NaN) and the CTA still releases its tensor
// memory.

#define MSP_TC_PS 16          // pairs per stage
#define MSP_TC_WAIT (1 << 24)  // polls before a wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor: K-major, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version (bits 46-48 = 0b001)
    return d;
}

__device__ __forceinline__ float tf32_rn(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    uint32_t done = 0;
    for (int it = 0; it < MSP_TC_WAIT && !done; ++it)
        asm volatile(
            "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;"
            " selp.b32 %0, 1, 0, p;}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
    return done != 0;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc,
                                       uint32_t acc) {
    asm volatile(
        "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

template <int N>
struct TcLayout {
    static constexpr int CA = 16 * 128;          // bytes of one A K-chunk (128 rows x 16 B)
    static constexpr int CB = (N / 8) * 128;     // bytes of one B K-chunk
    static constexpr int A_BYTES = 8 * CA;       // 8 K-chunks per stage (K = 32)
    static constexpr int B_BYTES = 8 * CB;
    static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;  // hi and lo of A and B
    static constexpr int SMEM = 2 * STAGE;       // two stages
};

// Reads the 32-lane x N-column block (N = 32, 16 or 8) of tensor memory at
// taddr (this warp's lanes) into r[0..N).
template <int N>
__device__ __forceinline__ void tmem_load(uint32_t taddr, uint32_t (&r)[32]) {
    if (N == 32) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
            "%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31},"
            " [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
              "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
              "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
              "=r"(r[31])
            : "r"(taddr));
    } else if (N == 16) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
            "%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
    } else {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7])
            : "r"(taddr));
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Accumulation: the tensor core's own FP32 accumulation over hundreds of
// MMAs loses ~1e-6 of a single crystallite's P(t), so every stage
// accumulates into one of two tensor-memory blocks (alternating, 32 columns
// each) that the threads drain into round-to-nearest FP32 registers once the
// stage's MMAs have completed -- while the next stage's MMAs run into the
// other block.
//
// 256 threads: warps w and w + 4 own the same 32 TMEM lanes (rows k1) and
// drain the two column halves; operand generation is spread over all
// threads (A: 4 K-chunks of one row each, B: one K-chunk each); the power
// tables are five chains of at most 8 products (the 16-entry X chain is
// split in two, its second half started from its own exactly reduced
// phase).
#define MSP_TC_THREADS 256

// Power tables of the 16 pairs of one stage, thread (chain c, pair i) for
// c < 5: Y e^{i psi b} (b < 8), e^{i 8 psi a} (a < N/8); X e^{i N psi b}
// (b < 8) and c e^{i (phi0 + psi (tile + 8 N a))} for a < 8 (c = 3) and
// 8 <= a < 16 (c = 4, started from its own exactly reduced phase).
template <int N>
struct TcTables {
    cx<float> ylo[8][MSP_TC_PS + 1], yhi[N / 8][MSP_TC_PS + 1], xlo[8][MSP_TC_PS + 1],
        xhi[16][MSP_TC_PS + 1];
};

// rec / cf: the stage's first pair record and coefficient (global or
// shared memory); np <= MSP_TC_PS of them are valid.
template <int N>
__device__ __forceinline__ void tc_build_tables(const float4 *rec_p, const float2 *cf_p,
                                                TcTables<N> &tb, int np, float tile_steps,
                                                int tid) {
    constexpr int PS = MSP_TC_PS, YH = N / 8;
    if (tid >= 5 * PS) return;
    const int c = tid / PS, i = tid - c * PS;
    const int len = c == 1 ? YH : 8;
    cx<float> *dst = c == 0 ? &tb.ylo[0][i] : c == 1 ? &tb.yhi[0][i] : c == 2 ? &tb.xlo[0][i]
                                                : c == 3 ? &tb.xhi[0][i] : &tb.xhi[8][i];
    cx<float> p = mk<float>(c >= 3 ? 0.f : 1.f, 0.f), base = mk<float>(1.f, 0.f);
    if (i < np) {
        const float4 rec = rec_p[i];
        const float sc = c == 0 ? 1.f : c == 1 ? 8.f : c == 2 ? (float)N : 8.f * N;
        float h = rec.x * sc, l = rec.y * sc;  // exact power-of-two scaling
        dw_reduce_2pi(h, l);
        base = dw_expi(h, l);
        if (c >= 3) {
            float th = rec.z, tl = rec.w;
            const float steps = tile_steps + (c == 4 ? 64.f * N : 0.f);  // exact
            if (steps > 0.f) {
                const float ph = rec.x * steps;
                float bh = ph, bl = fmaf(rec.x, steps, -ph) + rec.y * steps;
                dw_reduce_2pi(bh, bl);
                dw_add(th, tl, bh, bl);
                dw_reduce_2pi(th, tl);
            }
            const float2 cf = cf_p[i];
            p = mk<float>(cf.x, -cf.y);
            if (th != 0.f || tl != 0.f) p = cmul(p, dw_expi(th, tl));
        }
    }
    for (int q = 0; q < len; ++q) {
        dst[q * (PS + 1)] = p;
        p = cmul(p, base);
    }
}

// Seeds of one pair's power tables (the bases and starting values of
// tc_build_tables' five chains), for the warp-specialised kernel, which
// computes them for a whole work item at once: e^{i psi}, e^{i 8 psi},
// e^{i N psi}, e^{i 8 N psi}, and c e^{i (phi0 + psi tile)},
// c e^{i (phi0 + psi (tile + 64 N))} -- the same operations as
// tc_build_tables, so the tables are identical.
struct TcSeed {
    cx<float> e1, e8, eN, e8N, p3, p4;
};

template <int N>
__device__ __forceinline__ TcSeed tc_seed(float4 rec, float2 cf, float tile_steps) {
    TcSeed sd;
    const float sc[4] = {1.f, 8.f, (float)N, 8.f * N};
    cx<float> e[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float h = rec.x * sc[c], l = rec.y * sc[c];  // exact power-of-two scaling
        dw_reduce_2pi(h, l);
        e[c] = dw_expi(h, l);
    }
    sd.e1 = e[0];
    sd.e8 = e[1];
    sd.eN = e[2];
    sd.e8N = e[3];
#pragma unroll
    for (int c = 3; c < 5; ++c) {
        float th = rec.z, tl = rec.w;
        const float steps = tile_steps + (c == 4 ? 64.f * N : 0.f);  // exact
        if (steps > 0.f) {
            const float ph = rec.x * steps;
            float bh = ph, bl = fmaf(rec.x, steps, -ph) + rec.y * steps;
            dw_reduce_2pi(bh, bl);
            dw_add(th, tl, bh, bl);
            dw_reduce_2pi(th, tl);
        }
        cx<float> p = mk<float>(cf.x, -cf.y);
        if (th != 0.f || tl != 0.f) p = cmul(p, dw_expi(th, tl));
        if (c == 3)
            sd.p3 = p;
        else
            sd.p4 = p;
    }
    return sd;
}

// The power tables of one stage from its pairs' seeds (np of them valid).
template <int N>
__device__ __forceinline__ void tc_chain_tables(const TcSeed *seed, TcTables<N> &tb, int np,
                                                int tid) {
    constexpr int PS = MSP_TC_PS, YH = N / 8;
    if (tid >= 5 * PS) return;
    const int c = tid / PS, i = tid - c * PS;
    const int len = c == 1 ? YH : 8;
    cx<float> *dst = c == 0 ? &tb.ylo[0][i] : c == 1 ? &tb.yhi[0][i] : c == 2 ? &tb.xlo[0][i]
                                                : c == 3 ? &tb.xhi[0][i] : &tb.xhi[8][i];
    cx<float> p = mk<float>(c >= 3 ? 0.f : 1.f, 0.f), base = mk<float>(1.f, 0.f);
    if (i < np) {
        const TcSeed &sd = seed[i];
        base = c == 0 ? sd.e1 : c == 1 ? sd.e8 : c == 2 ? sd.eN : sd.e8N;
        if (c == 3) p = sd.p3;
        if (c == 4) p = sd.p4;
    }
    for (int q = 0; q < len; ++q) {
        dst[q * (PS + 1)] = p;
        p = cmul(p, base);
    }
}


// 256 threads: warps w and w + 4 own the same 32 TMEM lanes (rows k1) and
// drain the two column halves; operand generation is spread over all
// threads (A: 4 K-chunks of one row each, B: one K-chunk each).  One
// barrier per stage: every thread polls the stage mbarrier itself, and the
// tables of stage s + 1 (double-buffered) are built after the operands of
// stage s, so their latency overlaps the other warps' operand work.
template <int N>
__global__ void __launch_bounds__(MSP_TC_THREADS) msp_phase_tc_kernel(PhaseArgs a) {
    typedef TcLayout<N> L;
    constexpr int PS = MSP_TC_PS, NH = N / 2;
    extern __shared__ __align__(1024) char tsm[];
    __shared__ __align__(16) TcTables<N> tabs[2];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t s_tmem;
    __shared__ int s_range[2];

    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        item_range(a, blockIdx.x, &s_range[0], &s_range[1]);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    __syncthreads();
    const int pbeg = s_range[0], pend = s_range[1];
    if (pbeg < 0) return;
    const long long tile_base = (long long)blockIdx.y * (128 * N);
    const float tile_steps = (float)tile_base;  // exact: < 2^24
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(
            smem_u32(&s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    const float2 *coef = reinterpret_cast<const float2 *>(a.pair_coef);
    tc_build_tables<N>(a.pair_phase + pbeg, coef + pbeg, tabs[0],
                       (pend - pbeg) < PS ? (pend - pbeg) : PS, tile_steps, tid);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;
    // this warp's TMEM lanes and column half
    const int half = warp >> 2;
    const uint32_t my_tmem = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(half * NH);

    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
                           ((uint32_t)(128 >> 4) << 24);
    const int nstage = (pend - pbeg + PS - 1) / PS;
    int issued = 0;   // stages whose MMAs were committed (uniform across the CTA)
    int drained = 0;  // stages added into acc (uniform)
    int fail = 0;     // uniform: set from the barrier's OR
    float acc[NH];
#pragma unroll
    for (int j = 0; j < NH; ++j) acc[j] = 0.f;
    uint32_t r[32];

    for (int s = 0; s < nstage; ++s) {
        const int buf = s & 1;
        char *A_hi = tsm + buf * L::STAGE;
        char *A_lo = A_hi + L::A_BYTES;
        char *B_hi = A_lo + L::A_BYTES;
        char *B_lo = B_hi + L::B_BYTES;
        const TcTables<N> &tb = tabs[buf];
        int my_fail = 0;
        if (s >= 2) {
            // stage s - 2 (same operand buffer, same accumulator block) done:
            // drain its block before stage s overwrites it
            if (mbar_wait(smem_u32(&mbar[buf]), ((s >> 1) - 1) & 1)) {
                asm volatile("tcgen05.fence::after_thread_sync;");
                tmem_load<NH>(my_tmem + 32u * buf, r);
#pragma unroll
                for (int j = 0; j < NH; ++j) acc[j] += __uint_as_float(r[j]);
            } else {
                my_fail = 1;
            }
            drained = s - 1;
        }
        // A: thread = (row k1, half h): K-chunks g = h, h + 2, h + 4, h + 6
        {
            const int k1 = tid & 127, h0 = tid >> 7;
            const int off = (k1 >> 3) * 128 + (k1 & 7) * 16;
#pragma unroll 2
            for (int gi = 0; gi < PS / 4; ++gi) {
                const int g = h0 + 2 * gi;
                const cx<float> x0 = cmul(tb.xhi[k1 >> 3][2 * g], tb.xlo[k1 & 7][2 * g]);
                const cx<float> x1 = cmul(tb.xhi[k1 >> 3][2 * g + 1], tb.xlo[k1 & 7][2 * g + 1]);
                const float4 v = make_float4(x0.re, -x0.im, x1.re, -x1.im);
                const float4 hh = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
                // the tensor core reads lo as tf32 (truncated): |lo| <= 2^-11 |x|
                const float4 lo = make_float4(v.x - hh.x, v.y - hh.y, v.z - hh.z, v.w - hh.w);
                *reinterpret_cast<float4 *>(A_hi + g * L::CA + off) = hh;
                *reinterpret_cast<float4 *>(A_lo + g * L::CA + off) = lo;
            }
        }
        // B: task = (row k0, K-chunk g)
        for (int e = tid; e < N * (PS / 2); e += MSP_TC_THREADS) {
            const int k0 = e % N, g = e / N;
            const cx<float> y0 = cmul(tb.yhi[k0 >> 3][2 * g], tb.ylo[k0 & 7][2 * g]);
            const cx<float> y1 = cmul(tb.yhi[k0 >> 3][2 * g + 1], tb.ylo[k0 & 7][2 * g + 1]);
            const float4 v = make_float4(y0.re, y0.im, y1.re, y1.im);
            const float4 hh = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
            const float4 lo = make_float4(v.x - hh.x, v.y - hh.y, v.z - hh.z, v.w - hh.w);
            const int off = g * L::CB + (k0 >> 3) * 128 + (k0 & 7) * 16;
            *reinterpret_cast<float4 *>(B_hi + off) = hh;
            *reinterpret_cast<float4 *>(B_lo + off) = lo;
        }
        // tables of the next stage (the buffer last read by stage s - 1)
        if (s + 1 < nstage) {
            const int pb1 = pbeg + (s + 1) * PS;
            tc_build_tables<N>(a.pair_phase + pb1, coef + pb1, tabs[buf ^ 1],
                               (pend - pb1) < PS ? (pend - pb1) : PS,
                               tile_steps, tid);
        }
        // operands written by the generic proxy, read by the tensor core;
        // this thread's tensor-memory reads ordered before the next MMAs
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        fail = __syncthreads_or(my_fail);
        if (fail) break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t ah = smem_u32(A_hi), al = smem_u32(A_lo);
            const uint32_t bh = smem_u32(B_hi), bl = smem_u32(B_lo);
            const uint32_t d = tmem + 32u * buf;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const uint32_t ao = ks * 2 * L::CA, bo = ks * 2 * L::CB;
                const uint64_t dah = tc_desc(ah + ao, L::CA, 128), dal = tc_desc(al + ao, L::CA, 128);
                const uint64_t dbh = tc_desc(bh + bo, L::CB, 128), dbl = tc_desc(bl + bo, L::CB, 128);
                // the small products first, the block restarts at each stage
                tc_mma(d, dal, dbh, idesc, ks > 0 ? 1u : 0u);
                tc_mma(d, dah, dbl, idesc, 1u);
                tc_mma(d, dah, dbh, idesc, 1u);
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&mbar[buf]))
                : "memory");
        }
        issued = s + 1;
    }
    // epilogue: wait for the last commit (it covers every MMA issued before
    // it; waited for, bounded, even after a failed wait, so that no MMA still
    // reads shared or tensor memory when the CTA releases them), then drain
    // the blocks of the stages not yet added
    const int last = issued - 1;
    int my_fail = 0;
    if (last >= 0 && !mbar_wait(smem_u32(&mbar[last & 1]), (last >> 1) & 1)) my_fail = 1;
    fail = __syncthreads_or(my_fail | fail);
    asm volatile("tcgen05.fence::after_thread_sync;");
    const bool ok = !fail;
    if (ok) {
        for (int st = drained; st < issued; ++st) {  // at most two stages
            tmem_load<NH>(my_tmem + 32u * (st & 1), r);
#pragma unroll
            for (int j = 0; j < NH; ++j) acc[j] += __uint_as_float(r[j]);
        }
    }
    float *tile = reinterpret_cast<float *>(tsm);  // operand buffers are free now
    {
        const int k1 = 32 * (warp & 3) + (tid & 31);  // this thread's TMEM lane
#pragma unroll
        for (int j = 0; j < NH; ++j)
            tile[k1 * (N + 1) + half * NH + j] = ok ? acc[j] : __int_as_float(0x7fc00000);
    }
    __syncthreads();
    float *out = a.partial_f32 + (size_t)blockIdx.x * a.num_times;
    for (int e = tid; e < 128 * N; e += MSP_TC_THREADS) {
        const long long t = tile_base + e;
        if (t < a.num_times) out[t] = tile[(e / N) * (N + 1) + (e % N)];
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

// ---------------------------------------------------------------- warp-specialised form
//
// The same GEMM and numerics as msp_phase_tc_kernel, with the per-stage
// CTA barrier replaced by mbarriers so that table building, operand
// building, MMA issue and accumulator draining overlap:
//   * warps 0..7 (producers): drain the accumulator block of stage s - 2
//     (when its MMAs have completed), build stage s's operands from its
//     tables, then arrive on op_full[b] and tab_empty[t];
//   * warps 8..10 (tables): build the power tables of stage s into one of
//     three table buffers once tab_empty says the stage that used it is
//     built, then arrive on tab_full[t];
//   * warp 11, one lane (MMA): waits on op_full[b], issues the stage's 12
//     MMAs into accumulator block b and commits them to mma_done[b].
// Producers and table warps arrive once per warp (lane 0, after a
// __syncwarp that orders the other lanes' work before it): 8 + 8 + 3
// arrivals a stage rather than one per thread.  Their waits and failure
// checks are warp-uniform (__all_sync / __any_sync), so a warp never
// splits around a __syncwarp or a tcgen05 instruction.
// Every wait polls a bounded number of times and also gives up when another
// thread has recorded a failure (s_fail), so a failure ends every loop
// quickly; the tile's partials are then NaN and the tensor memory is
// released only after the last committed MMAs have completed (waited for,
// bounded).
//
// The A operands live in tensor memory rather than shared memory: each
// producer thread stores its row's 16 K-columns of A hi and A lo with
// tcgen05.st (row k1 = TMEM lane k1, K index = column, one tf32 per
// column), and the MMAs read A from there.  Only B (N rows) is staged in
// shared memory (a stage moves ~20 KB through it instead of ~100 KB), which
// leaves room for the work item's table seeds (TcSeed, 48 B for each of at
// most MSP_F32_ITEM_PAIRS pairs): all threads compute them at the start, so
// a stage's tables are only short multiplication chains.  Built per stage
// from the pair records, the tables' latency (~2000 cycles a stage, with
// the loads and the sincosf calls) paced the pipeline; the MMAs of a stage
// take ~300 cycles and the producers ~900.
// Tensor memory per CTA (256 columns): accumulator blocks at columns 0 and
// 32, A buffer b (hi, lo) at columns 64 + 64 b and 96 + 64 b.  The dynamic
// shared memory is padded so that two CTAs share an SM (2 x 256 = 512
// columns): a third would wait in tcgen05.alloc.
#define MSP_TCW_PRODUCERS 256
#define MSP_TCW_TABLE_THREADS 96
#define MSP_TCW_THREADS (MSP_TCW_PRODUCERS + MSP_TCW_TABLE_THREADS + 32)
#define MSP_TCW_TABLES 3
#define MSP_TCW_TMEM_COLS 256
#define MSP_TCW_A_COL 64u

template <int N>
struct TcwLayout {
    static constexpr int CB = (N / 8) * 128;  // bytes of one B K-chunk
    static constexpr int B_BYTES = 8 * CB;    // 8 K-chunks per stage (K = 32)
    static constexpr int STAGE = 2 * B_BYTES; // hi and lo of B
    static constexpr int REC = 16 * 1024;     // the item's table seeds (48 B per pair)
    static constexpr int SMEM = 80 * 1024;    // padded: two CTAs per SM
    // the epilogue's 128 x (N + 1) tile may overlap the seeds (dead by then)
    static_assert(2 * STAGE <= REC && 128 * (N + 1) * 4 <= SMEM &&
                      REC + 48 * MSP_F32_ITEM_PAIRS <= SMEM,
                  "TcwLayout");
};

// Stores r[0..16) into 16 consecutive columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_store16(uint32_t taddr, const uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
        "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
        "r"(r[15])
        : "memory");
}

// One MMA with A read from tensor memory (address a_tmem), B from shared
// memory (descriptor bd).
__device__ __forceinline__ void tc_mma_ta(uint32_t tmem, uint32_t a_tmem, uint64_t bd,
                                          uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{.reg .pred p; setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;}" ::"r"(tmem),
        "r"(a_tmem), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Bounded wait that also stops when *fail is set (checked every 256 polls).
// (A suspend-time hint on try_wait cut the polls from ~8 to ~1 a wait but
// did not make the kernel faster.)
__device__ __forceinline__ bool mbar_wait_or_fail(uint32_t bar, uint32_t parity,
                                                  volatile int *fail) {
    for (int it = 0; it < MSP_TC_WAIT; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;"
            " selp.b32 %0, 1, 0, p;}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255) == 255 && *fail) return false;
    }
    *fail = 1;
    return false;
}

template <int N>
__global__ void __launch_bounds__(MSP_TCW_THREADS, 2) msp_phase_tcw_kernel(PhaseArgs a) {
    typedef TcwLayout<N> L;
    constexpr int PS = MSP_TC_PS, NH = N / 2;
    extern __shared__ __align__(1024) char tsm[];
    __shared__ __align__(16) TcTables<N> tabs[MSP_TCW_TABLES];
    __shared__ __align__(8) uint64_t tab_full[MSP_TCW_TABLES], tab_empty[MSP_TCW_TABLES];
    __shared__ __align__(8) uint64_t op_full[2], mma_done[2];
    __shared__ uint32_t s_tmem;
    __shared__ int s_range[2];
    __shared__ int s_issued;
    __shared__ volatile int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        item_range(a, blockIdx.x, &s_range[0], &s_range[1]);
        for (int t = 0; t < MSP_TCW_TABLES; ++t) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tab_full[t])),
                         "r"(MSP_TCW_TABLE_THREADS / 32));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tab_empty[t])),
                         "r"(MSP_TCW_PRODUCERS / 32));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&op_full[b])),
                         "r"(MSP_TCW_PRODUCERS / 32));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mma_done[b])));
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_issued = 0;
        s_fail = 0;
    }
    __syncthreads();
    const int pbeg = s_range[0], pend = s_range[1];
    if (pbeg < 0) return;
    const long long tile_base = (long long)blockIdx.y * (128 * N);
    const float tile_steps = (float)tile_base;  // exact: < 2^24
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s_tmem)),
                     "n"(MSP_TCW_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = s_tmem;
    const int nstage = (pend - pbeg + PS - 1) / PS;
    // every pair's table seeds, by all threads at once (the per-stage table
    // work is then short multiplication chains)
    TcSeed *seeds = reinterpret_cast<TcSeed *>(tsm + L::REC);
    {
        const float2 *coef = reinterpret_cast<const float2 *>(a.pair_coef);
        for (int e = tid; e < pend - pbeg; e += MSP_TCW_THREADS)
            seeds[e] = tc_seed<N>(a.pair_phase[pbeg + e], coef[pbeg + e], tile_steps);
    }
    __syncthreads();

    float acc[NH];
#pragma unroll
    for (int j = 0; j < NH; ++j) acc[j] = 0.f;

    if (tid < MSP_TCW_PRODUCERS) {
        // ------------------------------------------------------------ producers
        const int half = warp >> 2;
        const uint32_t my_tmem =
            tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(half * NH);
        uint32_t r[32];
        // waits decided warp-uniformly: tcgen05.ld is a whole-warp instruction
        for (int s = 0; s < nstage; ++s) {
            if (__any_sync(0xffffffffu, s_fail)) break;
            const int b = s & 1, t = s % MSP_TCW_TABLES;
            if (!__all_sync(0xffffffffu, mbar_wait_or_fail(smem_u32(&tab_full[t]),
                                                            (s / MSP_TCW_TABLES) & 1, &s_fail)))
                break;
            if (s >= 2) {
                if (!__all_sync(0xffffffffu, mbar_wait_or_fail(smem_u32(&mma_done[b]),
                                                                ((s >> 1) - 1) & 1, &s_fail)))
                    break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                tmem_load<NH>(my_tmem + 32u * b, r);
#pragma unroll
                for (int j = 0; j < NH; ++j) acc[j] += __uint_as_float(r[j]);
            }
            char *B_hi = tsm + b * L::STAGE;
            char *B_lo = B_hi + L::B_BYTES;
            const TcTables<N> &tb = tabs[t];
            {
                // A row k1, K-columns 16 h0 .. 16 h0 + 15 (pairs 8 h0 .. 8 h0 + 7)
                const int k1 = tid & 127, h0 = tid >> 7;
                uint32_t rh[16], rl[16];
#pragma unroll
                for (int gi = 0; gi < 4; ++gi) {
                    const int g = 4 * h0 + gi;
                    const cx<float> x0 = cmul(tb.xhi[k1 >> 3][2 * g], tb.xlo[k1 & 7][2 * g]);
                    const cx<float> x1 =
                        cmul(tb.xhi[k1 >> 3][2 * g + 1], tb.xlo[k1 & 7][2 * g + 1]);
                    const float v[4] = {x0.re, -x0.im, x1.re, -x1.im};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float hh = tf32_rn(v[q]);
                        // the tensor core reads lo as tf32 (truncated): |lo| <= 2^-11 |x|
                        rh[4 * gi + q] = __float_as_uint(hh);
                        rl[4 * gi + q] = __float_as_uint(v[q] - hh);
                    }
                }
                const uint32_t ta = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + MSP_TCW_A_COL +
                                    64u * b + 16u * h0;
                tmem_store16(ta, rh);
                tmem_store16(ta + 32u, rl);
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            }
            for (int e = tid; e < N * (PS / 2); e += MSP_TCW_PRODUCERS) {
                const int k0 = e % N, g = e / N;
                const cx<float> y0 = cmul(tb.yhi[k0 >> 3][2 * g], tb.ylo[k0 & 7][2 * g]);
                const cx<float> y1 = cmul(tb.yhi[k0 >> 3][2 * g + 1], tb.ylo[k0 & 7][2 * g + 1]);
                const float4 v = make_float4(y0.re, y0.im, y1.re, y1.im);
                const float4 hh =
                    make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
                const float4 lo = make_float4(v.x - hh.x, v.y - hh.y, v.z - hh.z, v.w - hh.w);
                const int off = g * L::CB + (k0 >> 3) * 128 + (k0 & 7) * 16;
                *reinterpret_cast<float4 *>(B_hi + off) = hh;
                *reinterpret_cast<float4 *>(B_lo + off) = lo;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&tab_empty[t]));
            // B written by the generic proxy, read by the tensor core; this
            // thread's tensor-memory loads and stores ordered before the MMAs
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&op_full[b]));
        }
        // the blocks of the last two stages
        for (int st = nstage >= 2 ? nstage - 2 : 0; st < nstage; ++st) {
            if (__any_sync(0xffffffffu, s_fail)) break;
            if (!__all_sync(0xffffffffu, mbar_wait_or_fail(smem_u32(&mma_done[st & 1]),
                                                            (st >> 1) & 1, &s_fail)))
                break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            tmem_load<NH>(my_tmem + 32u * (st & 1), r);
#pragma unroll
            for (int j = 0; j < NH; ++j) acc[j] += __uint_as_float(r[j]);
        }
    } else if (tid < MSP_TCW_PRODUCERS + MSP_TCW_TABLE_THREADS) {
        // ------------------------------------------------------------ tables
        const int tt = tid - MSP_TCW_PRODUCERS;
        for (int s = 0; s < nstage; ++s) {
            if (__any_sync(0xffffffffu, s_fail)) break;
            const int t = s % MSP_TCW_TABLES;
            if (s >= MSP_TCW_TABLES &&
                !__all_sync(0xffffffffu,
                            mbar_wait_or_fail(smem_u32(&tab_empty[t]),
                                              ((s / MSP_TCW_TABLES) - 1) & 1, &s_fail)))
                break;
            const int pb = pbeg + s * PS;
            tc_chain_tables<N>(seeds + (pb - pbeg), tabs[t], (pend - pb) < PS ? (pend - pb) : PS,
                               tt);
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&tab_full[t]));
        }
    } else if (lane == 0) {
        // ------------------------------------------------------------ MMA issue
        const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) |
                               ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
        int issued = 0;
        for (int s = 0; s < nstage && !s_fail; ++s) {
            const int b = s & 1;
            if (!mbar_wait_or_fail(smem_u32(&op_full[b]), (s >> 1) & 1, &s_fail)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t bh = smem_u32(tsm + b * L::STAGE), bl = bh + L::B_BYTES;
            const uint32_t ah = tmem + MSP_TCW_A_COL + 64u * b, al = ah + 32u;
            const uint32_t d = tmem + 32u * b;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const uint32_t bo = ks * 2 * L::CB;
                const uint64_t dbh = tc_desc(bh + bo, L::CB, 128), dbl = tc_desc(bl + bo, L::CB, 128);
                // the small products first, the block restarts at each stage
                tc_mma_ta(d, al + 8u * ks, dbh, idesc, ks > 0 ? 1u : 0u);
                tc_mma_ta(d, ah + 8u * ks, dbl, idesc, 1u);
                tc_mma_ta(d, ah + 8u * ks, dbh, idesc, 1u);
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&mma_done[b]))
                : "memory");
            issued = s + 1;
        }
        s_issued = issued;
    }
    // epilogue: every MMA committed has completed before the tensor memory
    // goes (waited for, bounded, even after a failure)
    __syncthreads();
    const int issued = s_issued;
    if (tid == 0 && issued > 0) {
        const int last = issued - 1;
        volatile int never = 0;
        if (!mbar_wait_or_fail(smem_u32(&mma_done[last & 1]), (last >> 1) & 1, &never))
            s_fail = 1;
    }
    if (tid == 0 && issued < nstage) s_fail = 1;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const bool ok = !s_fail;
    float *tile = reinterpret_cast<float *>(tsm);  // operand buffers are free now
    if (tid < MSP_TCW_PRODUCERS) {
        const int half = warp >> 2;
        const int k1 = 32 * (warp & 3) + lane;  // this thread's TMEM lane
#pragma unroll
        for (int j = 0; j < NH; ++j)
            tile[k1 * (N + 1) + half * NH + j] = ok ? acc[j] : __int_as_float(0x7fc00000);
    }
    __syncthreads();
    float *out = a.partial_f32 + (size_t)blockIdx.x * a.num_times;
    for (int e = tid; e < 128 * N; e += MSP_TCW_THREADS) {
        const long long t = tile_base + e;
        if (t < a.num_times) out[t] = tile[(e / N) * (N + 1) + (e % N)];
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "n"(MSP_TCW_TMEM_COLS));
}

// Arbitrary time grids: one thread per sample, every pair's phase reduced in
// FP64 and evaluated with sincos.
template <typename T>
__global__ void __launch_bounds__(256) msp_phase_direct_kernel(PhaseArgs a) {
    typedef typename PairCoef<T>::type coef_t;
    __shared__ coef_t sc[256];
    __shared__ double sw[256];
    __shared__ int s_range[2];
    const int tid = threadIdx.x;
    if (tid == 0) item_range(a, blockIdx.x, &s_range[0], &s_range[1]);
    __syncthreads();
    const int pbeg = s_range[0], pend = s_range[1];
    if (pbeg < 0) return;
    const coef_t *coef = reinterpret_cast<const coef_t *>(a.pair_coef);
    const int t = blockIdx.y * 256 + tid;
    const bool valid = t < a.num_times;
    const double tt = valid ? a.times[t] : 0.0;
    double acc = 0.0;
    for (int pb = pbeg; pb < pend; pb += 256) {
        const int np = (pend - pb) < 256 ? (pend - pb) : 256;
        if (tid < np) {
            sc[tid] = coef[pb + tid];
            sw[tid] = a.pair_omega[pb + tid];
        }
        __syncthreads();
        T part = T(0);
        for (int i = 0; i < np; ++i) {
            T s, c;
            sincos_t(reduce_2pi(sw[i] * tt), &s, &c);
            part = fma((T)sc[i].x, c, part);
            part = fma((T)sc[i].y, s, part);
        }
        acc += (double)part;
        __syncthreads();
    }
    if (valid) a.partial[(size_t)blockIdx.x * a.num_times + t] = acc;
}

// Slot bookkeeping: first snapshot of every output row, and the prefix of
// work items (runs of IP pairs, never straddling two rows).  A slot
// index out of range or out of order marks the snapshot MSP_ITEM_BAD_SLOT
// and empties the whole schedule.
__global__ void msp_schedule_kernel(const int *__restrict__ slot, int S, int num_slots, int P,
                                    int IP, int count_items, int *__restrict__ slot_first,
                                    int *__restrict__ item_first, int *__restrict__ status) {
    __shared__ int bad;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) bad = 0;
    __syncthreads();
    for (int s = tid; s < S; s += nt) {
        const int sl = slot[s];
        const bool ok = sl >= 0 && sl < num_slots && (s == 0 || sl >= slot[s - 1]);
        if (!ok) {
            status[s] |= MSP_ITEM_BAD_SLOT;
            atomicOr(&bad, 1);
        }
    }
    __syncthreads();
    if (bad) {
        for (int x = tid; x <= num_slots; x += nt) {
            slot_first[x] = 0;
            item_first[x] = 0;
        }
        return;
    }
    for (int s = tid; s < S; s += nt) {
        const int sl = slot[s];
        const int prev = s == 0 ? -1 : slot[s - 1];
        for (int x = prev + 1; x <= sl; ++x) slot_first[x] = s;
    }
    const int last = S > 0 ? slot[S - 1] : -1;
    for (int x = last + 1 + tid; x <= num_slots; x += nt) slot_first[x] = S;
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int x = 0; x < num_slots; ++x) {
            item_first[x] = acc;
            if (count_items) {
                const long long pairs = (long long)(slot_first[x + 1] - slot_first[x]) * P;
                acc += (int)((pairs + IP - 1) / IP);
            }
        }
        item_first[num_slots] = acc;
    }
}

// out[slot][t] = sum of the slot's snapshot constants + its items' partials,
// in a fixed order (deterministic); heterogeneous batches map slots to
// output rows (slot_row) and add to the row (accumulate) when a system's
// snapshots are split over several launches.  A block covers 8 times of
// one slot (so that a 4096-time row gives 512 blocks: the slot's partials
// are tens of MB that only many outstanding loads stream at HBM rate): lane
// (g, tt) of warp w reads time tt of items 4 w + g, 4 w + g + 64, ...
// (32-byte sectors of 4 items per load), summing FP32 partials as a
// double-word (FP64 partials in FP64); the 64 stream sums are then added in
// stream order in FP64.
#define MSP_REDUCE_WARPS 16
#define MSP_REDUCE_T 8
#define MSP_REDUCE_STREAMS (MSP_REDUCE_WARPS * 32 / MSP_REDUCE_T)
__global__ void __launch_bounds__(32 * MSP_REDUCE_WARPS)
    msp_reduce_kernel(PhaseArgs a, const double *__restrict__ snap_const,
                      double *__restrict__ out, int T) {
    __shared__ double red[MSP_REDUCE_STREAMS][MSP_REDUCE_T + 1];
    __shared__ double cred[MSP_REDUCE_WARPS];
    const int sl = blockIdx.y;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int s0 = a.slot_first[sl], s1 = a.slot_first[sl + 1];
    double c = 0.0;
    for (int s = s0 + tid; s < s1; s += blockDim.x) c += snap_const[s];
    // block reduction of the constants (fixed tree: deterministic)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cred[warp] = c;
    const int tt = lane & (MSP_REDUCE_T - 1), stream = warp * (32 / MSP_REDUCE_T) +
                                                      lane / MSP_REDUCE_T;
    const int t = blockIdx.x * MSP_REDUCE_T + tt;
    double v = 0.0;
    if (t < T) {
        const int i0 = a.item_first[sl], i1 = a.item_first[sl + 1];
        if (a.partial_f32) {
            const float *p = a.partial_f32 + t;
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll 8
            for (int it = i0 + stream; it < i1; it += MSP_REDUCE_STREAMS)
                acc = dw_add_f(acc, p[(size_t)it * T]);
            v = dw_to_double(acc);
        } else {
            const double *p = a.partial + t;
#pragma unroll 8
            for (int it = i0 + stream; it < i1; it += MSP_REDUCE_STREAMS) v += p[(size_t)it * T];
        }
    }
    red[stream][tt] = v;
    __syncthreads();
    if (tid < MSP_REDUCE_T && t < T) {
        double s = 0.0;
        for (int w = 0; w < MSP_REDUCE_WARPS; ++w) s += cred[w];
        for (int q = 0; q < MSP_REDUCE_STREAMS; ++q) s += red[q][tid];
        const size_t o = (size_t)(a.slot_row ? a.slot_row[sl] : sl) * T + t;
        if (a.accumulate)
            out[o] += s;
        else
            out[o] = s;
    }
}

// The mixed-precision uniform-grid phase sum runs on the tensor cores
// unless MSP_PHASE_SIMT=1 is set in the environment (read at each launch),
// which selects the FP32 SIMT kernel -- the two give the same sums to FP32
// rounding; the parity tests compare them.
bool phase_use_tensor_cores() {
    const char *v = getenv("MSP_PHASE_SIMT");
    return !(v != NULL && v[0] == '1');
}

// The tensor-core phase sum runs in its warp-specialised form unless
// MSP_PHASE_TC_BARRIER=1 selects the one-barrier-per-stage form.
static bool phase_tc_warp_specialised() {
    const char *v = getenv("MSP_PHASE_TC_BARRIER");
    return !(v != NULL && v[0] == '1');
}

template <int N>
static cudaError_t launch_tc(const PhaseArgs &a, int max_items, cudaStream_t st) {
    const dim3 grid(max_items, (a.num_times + 128 * N - 1) / (128 * N));
    if (phase_tc_warp_specialised()) {
        const int smem = TcwLayout<N>::SMEM;
        cudaError_t e = cudaFuncSetAttribute(msp_phase_tcw_kernel<N>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        msp_phase_tcw_kernel<N><<<grid, MSP_TCW_THREADS, smem, st>>>(a);
    } else {
        const int smem = TcLayout<N>::SMEM;
        cudaError_t e = cudaFuncSetAttribute(msp_phase_tc_kernel<N>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        msp_phase_tc_kernel<N><<<grid, MSP_TC_THREADS, smem, st>>>(a);
    }
    return cudaGetLastError();
}

int phase_snaps_per_item(int num_snap, int P, int precision) {
    if (P <= 0) return 1;
    // about 1500 items for load balance; FP32 accumulates at most
    // MSP_F32_ITEM_PAIRS pairs
    const int cap = (precision == MSP_PREC_MIXED ? MSP_F32_ITEM_PAIRS : 65536) / P;
    int sb = (num_snap + 1499) / 1500;
    if (sb > cap) sb = cap;
    if (sb < 1) sb = 1;
    return sb;
}

int phase_pairs_per_item(int num_snap, int P, int precision) {
    const long long ip = (long long)phase_snaps_per_item(num_snap, P, precision) * P;
    const long long cap = precision == MSP_PREC_MIXED ? MSP_F32_ITEM_PAIRS : (1LL << 30);
    return (int)(ip > cap ? cap : (ip < 1 ? 1 : ip));
}

int phase_max_items(int num_snap, int num_slots, int P, int IP) {
    return (int)(((long long)num_snap * P + IP - 1) / IP) + num_slots;
}

cudaError_t launch_schedule(const int *slot, int num_snap, int num_slots, int P, int IP,
                            int count_items, int *slot_first, int *item_first, int *status,
                            cudaStream_t st) {
    msp_schedule_kernel<<<1, 1024, 0, st>>>(slot, num_snap, num_slots, P, IP, count_items,
                                            slot_first, item_first, status);
    return cudaGetLastError();
}

cudaError_t launch_phase(const PhaseArgs &a, int precision, int max_items, int uniform,
                         cudaStream_t st) {
    if (max_items <= 0 || a.num_times <= 0) return cudaSuccess;
    if (uniform && precision == MSP_PREC_MIXED && phase_use_tensor_cores()) {
        return a.num_times > 2048 ? launch_tc<32>(a, max_items, st)
                                  : launch_tc<16>(a, max_items, st);
    } else if (uniform) {
        dim3 grid(max_items, (a.num_times + 4095) / 4096);
        if (precision == MSP_PREC_MIXED)
            msp_phase_uniform_f32_kernel<<<grid, 128, 0, st>>>(a);
        else
            msp_phase_uniform_kernel<double><<<grid, 128, 0, st>>>(a);
    } else {
        dim3 grid(max_items, (a.num_times + 255) / 256);
        if (precision == MSP_PREC_MIXED)
            msp_phase_direct_kernel<float><<<grid, 256, 0, st>>>(a);
        else
            msp_phase_direct_kernel<double><<<grid, 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_reduce(const PhaseArgs &a, const double *snap_const, double *out,
                          int num_times, cudaStream_t st) {
    if (a.num_slots <= 0) return cudaSuccess;
    dim3 grid((num_times + MSP_REDUCE_T - 1) / MSP_REDUCE_T, a.num_slots);
    msp_reduce_kernel<<<grid, 32 * MSP_REDUCE_WARPS, 0, st>>>(a, snap_const, out, num_times);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ building blocks

// The reference's cosine sum, same summation order per time
// (muspinsim/cython/parallel.pyx:59-67).
__global__ void msp_fast_cos_sum_kernel(const double *__restrict__ times, int T, int d,
                                        const double *__restrict__ A,
                                        const double *__restrict__ W, int n,
                                        double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    const double t = times[i];
    double acc = 0.0;
    for (int j = 0; j < n; ++j) {
        acc += 0.5 * A[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) acc += A[(size_t)j * n + k] * cos(W[(size_t)j * n + k] * t);
    }
    out[i] = acc * (1.0 / (double)d);
}

cudaError_t launch_fast_cos_sum(const double *times, int num_times, int d, const double *A,
                                const double *W, int n, double *out, cudaStream_t st) {
    if (num_times <= 0) return cudaSuccess;
    msp_fast_cos_sum_kernel<<<(num_times + 127) / 128, 128, 0, st>>>(times, num_times, d, A, W,
                                                                      n, out);
    return cudaGetLastError();
}

// A = |U^dag (sigma (x) 1_d) U|^2, W = 2 pi (l_j - l_k) (muspinsim/hamiltonian.py:204-211)
__global__ void msp_fast_amplitudes_kernel(const double *__restrict__ evals,
                                           const cx<double> *__restrict__ U,
                                           const cx<double> *__restrict__ sig, int n, int d,
                                           double *__restrict__ A, double *__restrict__ W) {
    extern __shared__ __align__(16) char smem[];
    cx<double> *sU = reinterpret_cast<cx<double> *>(smem);
    cx<double> *sM = sU + n * n;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < n * n; e += nt) sU[e] = U[e];
    __syncthreads();
    const cx<double> s00 = sig[0], s01 = sig[1], s10 = sig[2], s11 = sig[3];
    for (int e = tid; e < n * n; e += nt) {
        const int i = e / n, k = e - (e / n) * n;
        cx<double> v;
        if (i < d)
            v = cadd(cmul(s00, sU[i * n + k]), cmul(s01, sU[(i + d) * n + k]));
        else
            v = cadd(cmul(s10, sU[(i - d) * n + k]), cmul(s11, sU[i * n + k]));
        sM[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {
        const int j = e / n, k = e - (e / n) * n;
        double gr = 0, gi = 0;
        for (int i = 0; i < n; ++i) {
            const cx<double> u = sU[i * n + j], mm = sM[i * n + k];
            gr += u.re * mm.re + u.im * mm.im;
            gi += u.re * mm.im - u.im * mm.re;
        }
        A[e] = gr * gr + gi * gi;
        W[e] = 6.283185307179586476925 * (evals[j] - evals[k]);
    }
}

// n > 64: one CTA per column k from global memory: (sigma (x) 1_d) U[:, k]
// staged in shared memory, then A_jk, W_jk for every j.
__global__ void msp_fast_amplitudes_col_kernel(const double *__restrict__ evals,
                                               const cx<double> *__restrict__ U,
                                               const cx<double> *__restrict__ sig, int n, int d,
                                               double *__restrict__ A, double *__restrict__ W) {
    extern __shared__ __align__(16) char smem[];
    cx<double> *uc = reinterpret_cast<cx<double> *>(smem);
    cx<double> *wc = uc + n;
    const int k = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < n; i += nt) uc[i] = U[(size_t)i * n + k];
    __syncthreads();
    const cx<double> s00 = sig[0], s01 = sig[1], s10 = sig[2], s11 = sig[3];
    for (int i = tid; i < n; i += nt)
        wc[i] = i < d ? cadd(cmul(s00, uc[i]), cmul(s01, uc[i + d]))
                      : cadd(cmul(s10, uc[i - d]), cmul(s11, uc[i]));
    __syncthreads();
    for (int j = tid; j < n; j += nt) {
        double gr = 0, gi = 0;
        for (int i = 0; i < n; ++i) {
            const cx<double> u = U[(size_t)i * n + j], mm = wc[i];
            gr += u.re * mm.re + u.im * mm.im;
            gi += u.re * mm.im - u.im * mm.re;
        }
        A[(size_t)j * n + k] = gr * gr + gi * gi;
        W[(size_t)j * n + k] = 6.283185307179586476925 * (evals[j] - evals[k]);
    }
}

cudaError_t launch_fast_amplitudes(const double *evals, const double *evecs,
                                   const double *sigma, int n, int d, double *A, double *W,
                                   cudaStream_t st) {
    if (n > MSP_MAX_DIM) {
        msp_fast_amplitudes_col_kernel<<<n, 256, (size_t)2 * n * sizeof(cx<double>), st>>>(
            evals, reinterpret_cast<const cx<double> *>(evecs),
            reinterpret_cast<const cx<double> *>(sigma), n, d, A, W);
        return cudaGetLastError();
    }
    const size_t smem = (size_t)2 * n * n * sizeof(cx<double>);
    cudaError_t e = cudaFuncSetAttribute(msp_fast_amplitudes_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    msp_fast_amplitudes_kernel<<<1, 256, smem, st>>>(
        evals, reinterpret_cast<const cx<double> *>(evecs),
        reinterpret_cast<const cx<double> *>(sigma), n, d, A, W);
    return cudaGetLastError();
}

// out[t][o] = sum_ij rho_ij op_o[j][i] exp(-i w_ij t), w_ij = 2 pi (l_i - l_j):
// the general (not necessarily Hermitian operator) expectation series of
// Hamiltonian.evolve (muspinsim/hamiltonian.py:86-107).  One thread per time.
__global__ void __launch_bounds__(256) msp_evolve_expect_kernel(
    const double *__restrict__ evals, const cx<double> *__restrict__ rho,
    const cx<double> *__restrict__ ops, int n, int num_ops, const double *__restrict__ times,
    int T, cx<double> *__restrict__ out) {
    __shared__ cx<double> sc[256];
    __shared__ double sw[256];
    const int o = blockIdx.y;
    const cx<double> *op = ops + (size_t)o * n * n;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = t < T;
    const double tt = valid ? times[t] : 0.0;
    double ar = 0.0, ai = 0.0;
    const int nn = n * n;
    for (int b = 0; b < nn; b += 256) {
        const int e = b + threadIdx.x;
        if (e < nn) {
            const int i = e / n, j = e - (e / n) * n;
            sc[threadIdx.x] = cmul(rho[(size_t)i * n + j], op[(size_t)j * n + i]);
            sw[threadIdx.x] = 6.283185307179586476925 * (evals[i] - evals[j]);
        }
        __syncthreads();
        const int cnt = (nn - b) < 256 ? (nn - b) : 256;
        for (int q = 0; q < cnt; ++q) {
            double s, c;
            sincos(reduce_2pi(sw[q] * tt), &s, &c);
            // C (cos - i sin)
            ar += sc[q].re * c + sc[q].im * s;
            ai += sc[q].im * c - sc[q].re * s;
        }
        __syncthreads();
    }
    if (valid) out[(size_t)t * num_ops + o] = mk<double>(ar, ai);
}

cudaError_t launch_evolve_expect(const double *evals, const double *rho, const double *ops,
                                 int n, int num_ops, const double *times, int num_times,
                                 double *out, cudaStream_t st) {
    if (num_times <= 0 || num_ops <= 0) return cudaSuccess;
    dim3 grid((num_times + 255) / 256, num_ops);
    msp_evolve_expect_kernel<<<grid, 256, 0, st>>>(
        evals, reinterpret_cast<const cx<double> *>(rho),
        reinterpret_cast<const cx<double> *>(ops), n, num_ops, times, num_times,
        reinterpret_cast<cx<double> *>(out));
    return cudaGetLastError();
}

__global__ void msp_evolve_phases_kernel(const double *__restrict__ evals,
                                         const cx<double> *__restrict__ rho, int n,
                                         const double *__restrict__ times, int T,
                                         cx<double> *__restrict__ out) {
    const size_t nn = (size_t)n * n, total = nn * T;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t t = e / nn, o = e - t * nn;
        const int i = (int)(o / n), j = (int)(o - (o / n) * n);
        double s, c;
        sincos(reduce_2pi(6.283185307179586476925 * (evals[i] - evals[j]) * times[t]), &s, &c);
        // exp(-i w t) * rho_ij
        out[e] = cmul(mk<double>(c, -s), rho[o]);
    }
}

cudaError_t launch_evolve_phases(const double *evals, const double *rho, int n,
                                 const double *times, int num_times, double *out,
                                 cudaStream_t st) {
    const size_t total = (size_t)n * n * num_times;
    if (total == 0) return cudaSuccess;
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 16) grid = 152 * 16;
    msp_evolve_phases_kernel<<<grid, 256, 0, st>>>(evals,
                                                   reinterpret_cast<const cx<double> *>(rho), n,
                                                   times, num_times,
                                                   reinterpret_cast<cx<double> *>(out));
    return cudaGetLastError();
}

// out[o] = sum_ij rho_ij (-op_o[j][i]) / (2 pi i (l_j - l_i) - 1/tau)
// (muspinsim/hamiltonian.py:155-164).  One CTA per operator.
__global__ void __launch_bounds__(256) msp_integrate_kernel(const double *__restrict__ evals,
                                                            const cx<double> *__restrict__ rho,
                                                            const cx<double> *__restrict__ ops,
                                                            int n, double tau,
                                                            cx<double> *__restrict__ out) {
    __shared__ double red[16];
    const int o = blockIdx.x;
    const cx<double> *op = ops + (size_t)o * n * n;
    double ar = 0.0, ai = 0.0;
    const double inv_tau = 1.0 / tau;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - (e / n) * n;
        const cx<double> c = cmul(rho[(size_t)i * n + j], op[(size_t)j * n + i]);
        const double x = 6.283185307179586476925 * (evals[j] - evals[i]);
        // -c / (-1/tau + i x) = c (1/tau + i x) / (1/tau^2 + x^2)
        const double den = inv_tau * inv_tau + x * x;
        ar += (c.re * inv_tau - c.im * x) / den;
        ai += (c.im * inv_tau + c.re * x) / den;
    }
    block_sum2(ar, ai, red);
    if (threadIdx.x == 0) out[o] = mk<double>(ar, ai);
}

cudaError_t launch_integrate(const double *evals, const double *rho, const double *ops, int n,
                             int num_ops, double tau, double *out, cudaStream_t st) {
    if (num_ops <= 0) return cudaSuccess;
    msp_integrate_kernel<<<num_ops, 256, 0, st>>>(evals, reinterpret_cast<const cx<double> *>(rho),
                                                  reinterpret_cast<const cx<double> *>(ops), n,
                                                  tau, reinterpret_cast<cx<double> *>(out));
    return cudaGetLastError();
}

}  // namespace msp
