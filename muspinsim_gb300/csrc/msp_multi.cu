// Heterogeneous batches: many spin systems of uneven Hilbert dimension in one
// pipeline (msp_multi_*).  The reference evaluates one system per
// ExperimentRunner and one configuration snapshot at a time
// (muspinsim/experiment.py:358-498, muspinsim/simconfig.py:347-368); a study
// of many candidate muon sites or isotopologues therefore runs that loop once
// per system.  Here every system of the batch is evaluated together:
//
//  * systems are grouped into size buckets (one bucket per distinct n); each
//    bucket runs the fast-path snapshot kernel as one persistent launch over
//    all snapshots of all its systems -- a CTA finds the system of a
//    snapshot through a segment table (msp_internal.cuh: snap_source) -- then
//    the phase sum and a reduction into the systems' output rows;
//  * buckets run concurrently on their own streams, forked from and joined
//    back to the caller's stream; the whole launch sequence can be captured
//    once into a CUDA graph and replayed (msp_multi_run_graph);
//  * a bucket whose pair records would exceed max_pairs_per_chunk is run in
//    chunks that reuse its scratch; the reductions accumulate into the
//    zeroed output rows, so a system split across chunks is summed exactly
//    once per snapshot, in a fixed order.
//
// Every table the kernels read (segments, work items, output rows) depends
// only on the plan's sizes, so it is computed on the host when the plan is
// made and copied into the caller's workspace at the start of each run.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "msp_internal.cuh"

namespace msp {
int record_error(int code, const char *msg);
}

using namespace msp;

static int mfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return record_error(code, buf);
}

static int mcuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess)
        return mfail(MSP_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return MSP_OK;
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

namespace {

// Segment tables of one chunk, as byte offsets into the table block.
struct MultiChunk {
    int snap_begin, snap_end;  // bucket-local snapshot range
    int num_seg;
    int num_items;
    size_t seg_first, seg_g0, slot_row, item_first, seg_hoff;
};

struct MultiBucket {
    int n, P;
    bool large;
    int threads;      // snapshot-kernel CTA size
    int ctas_per_sm;  // persistent CTAs per SM (0: occupancy limit, set at first run)
    int grid;         // persistent grid of the snapshot kernel (set at first run for n <= 64)
    int ip;           // pairs per phase-sum work item
    int cap_snap;     // snapshots per chunk
    long long num_snap;
    std::vector<int> systems;  // global system ids, ascending
    std::vector<MultiChunk> chunks;
    int max_items;
    size_t off_coef, off_phase, off_const, off_partial, off_evec, off_large, bytes;
    cudaStream_t stream;
    cudaEvent_t done;
};

}  // namespace

struct msp_multi_plan {
    int num_systems, num_snap, num_times, uniform, precision, max_sweeps;
    double t0, dt;
    int sms;
    std::vector<int> sys_n;
    std::vector<long long> h_off;
    std::vector<int> snap_first;
    std::vector<MultiBucket> buckets;  // in launch order (most work first)
    std::vector<char> tab;            // host copy of the tables
    size_t tab_bytes;
    size_t ws_bytes;
    // created at the first run on the plan's device
    bool ready;
    int device;
    char *tab_pinned;
    cudaStream_t origin;
    cudaEvent_t fork;
    // graph of the last captured run
    cudaGraphExec_t exec;
    msp_multi_io graph_io;
};

static const msp_multi_tuning *find_tuning(const msp_multi_desc *d, int n) {
    if (d->tuning == NULL) return NULL;
    for (int i = 0; i < d->num_tuning; ++i)
        if (d->tuning[i].n == n) return &d->tuning[i];
    return NULL;
}

static int device_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0) {
        cudaGetLastError();
        return 152;  // GB300
    }
    return sms;
}

// Builds buckets, chunks, tables and the workspace layout (host only).
static int plan_layout(msp_multi_plan *p, const msp_multi_desc *d) {
    const int ns = d->num_systems;
    const bool mixed = d->precision == MSP_PREC_MIXED;
    const long long max_pairs = d->max_pairs_per_chunk > 0 ? d->max_pairs_per_chunk : (1LL << 26);
    // bucket per distinct n
    std::vector<int> dims(p->sys_n);
    std::sort(dims.begin(), dims.end());
    dims.erase(std::unique(dims.begin(), dims.end()), dims.end());
    p->buckets.clear();
    for (int n : dims) {
        MultiBucket b;
        b.n = n;
        b.P = n * (n - 1) / 2;
        b.large = n > MSP_MAX_DIM;
        b.num_snap = 0;
        for (int k = 0; k < ns; ++k)
            if (p->sys_n[k] == n) {
                b.systems.push_back(k);
                b.num_snap += p->snap_first[k + 1] - p->snap_first[k];
            }
        const msp_multi_tuning *t = find_tuning(d, n);
        b.threads = t && t->snap_threads > 0 ? t->snap_threads
                                             : (b.large ? large_threads(n) : snap_default_threads(n));
        b.ctas_per_sm = t && t->ctas_per_sm > 0 ? t->ctas_per_sm
                                                : (b.large ? large_ctas_per_sm(n, d->precision) : 0);
        long long cap = max_pairs / (b.P > 0 ? b.P : 1);
        if (cap < 1) cap = 1;
        if (cap > b.num_snap) cap = b.num_snap > 0 ? b.num_snap : 1;
        if (cap > (1LL << 30) / (b.P > 0 ? b.P : 1)) cap = (1LL << 30) / (b.P > 0 ? b.P : 1);
        b.cap_snap = (int)(cap > 0 ? cap : 1);
        long long ip = t && t->snaps_per_item > 0
                           ? (long long)t->snaps_per_item * b.P
                           : (long long)phase_pairs_per_item(b.cap_snap, b.P, d->precision);
        if (mixed && ip > MSP_F32_ITEM_PAIRS) ip = MSP_F32_ITEM_PAIRS;  // FP32 running-sum length
        if (ip > (1LL << 30)) ip = 1LL << 30;
        if (ip < 1) ip = 1;
        b.ip = (int)ip;
        b.grid = 0;
        b.stream = NULL;
        b.done = NULL;
        p->buckets.push_back(b);
    }
    // launch order: most pair work first (largest n breaks ties)
    std::stable_sort(p->buckets.begin(), p->buckets.end(),
                     [](const MultiBucket &a, const MultiBucket &b) {
                         const double wa = (double)a.num_snap * a.n * a.n * (a.n + 64.0);
                         const double wb = (double)b.num_snap * b.n * b.n * (b.n + 64.0);
                         return wa > wb;
                     });
    // chunks and tables
    size_t toff = 0;
    for (MultiBucket &b : p->buckets) {
        b.chunks.clear();
        b.max_items = 0;
        // bucket-local snapshot index of each system's first snapshot
        std::vector<long long> local_first(b.systems.size() + 1, 0);
        for (size_t j = 0; j < b.systems.size(); ++j) {
            const int k = b.systems[j];
            local_first[j + 1] = local_first[j] + (p->snap_first[k + 1] - p->snap_first[k]);
        }
        long long s0 = 0;
        do {
            const long long s1 = std::min<long long>(s0 + b.cap_snap, b.num_snap);
            MultiChunk c;
            c.snap_begin = (int)s0;
            c.snap_end = (int)s1;
            // segments: the systems with snapshots in [s0, s1); an empty
            // system keeps the zero its output row was cleared to
            std::vector<int> sf, g0, row, itf;
            std::vector<long long> ho;
            int items = 0;
            for (size_t j = 0; j < b.systems.size(); ++j) {
                const long long a0 = std::max(local_first[j], s0);
                const long long a1 = std::min(local_first[j + 1], s1);
                if (a1 <= a0) continue;
                const int k = b.systems[j];
                sf.push_back((int)(a0 - s0));
                g0.push_back((int)(p->snap_first[k] + (a0 - local_first[j])));
                row.push_back(k);
                ho.push_back(p->h_off[k]);
                itf.push_back(items);
                const long long pairs = (a1 - a0) * (long long)b.P;
                items += (int)((pairs + b.ip - 1) / b.ip);
            }
            sf.push_back((int)(s1 - s0));
            itf.push_back(items);
            c.num_seg = (int)row.size();
            c.num_items = items;
            b.max_items = std::max(b.max_items, items);
            const size_t nsg = (size_t)c.num_seg;
            c.seg_first = toff;
            toff = al256(toff + (nsg + 1) * 4);
            c.seg_g0 = toff;
            toff = al256(toff + nsg * 4 + 4);
            c.slot_row = toff;
            toff = al256(toff + nsg * 4 + 4);
            c.item_first = toff;
            toff = al256(toff + (nsg + 1) * 4);
            c.seg_hoff = toff;
            toff = al256(toff + nsg * 8 + 8);
            p->tab.resize(toff);
            memcpy(&p->tab[c.seg_first], sf.data(), sf.size() * 4);
            if (nsg) {
                memcpy(&p->tab[c.seg_g0], g0.data(), nsg * 4);
                memcpy(&p->tab[c.slot_row], row.data(), nsg * 4);
                memcpy(&p->tab[c.seg_hoff], ho.data(), nsg * 8);
            }
            memcpy(&p->tab[c.item_first], itf.data(), itf.size() * 4);
            b.chunks.push_back(c);
            s0 = s1;
        } while (s0 < b.num_snap);
    }
    p->tab_bytes = al256(toff);
    p->tab.resize(p->tab_bytes > 0 ? p->tab_bytes : 256);
    // workspace: tables, then each bucket's scratch (buckets run concurrently)
    size_t off = p->tab_bytes;
    const int T = p->num_times;
    const bool records = mixed && p->uniform;
    for (MultiBucket &b : p->buckets) {
        const size_t S = (size_t)b.cap_snap, P = (size_t)b.P;
        const size_t start = off;
        b.off_coef = off;
        off += al256(S * P * (mixed ? 8 : 16));
        b.off_phase = off;
        off += al256(S * P * (records ? 16 : 8));
        b.off_const = off;
        off += al256(S * 8);
        b.off_partial = off;
        off += al256((size_t)b.max_items * T * (records ? 4 : 8));
        b.off_evec = off;
        off += al256(b.large ? 0 : snap_evec_bytes(b.n, (long long)S, p->precision));
        b.off_large = off;
        if (b.large) {
            int g = p->sms * b.ctas_per_sm;
            if (g > b.cap_snap) g = b.cap_snap;
            if (g < 1) g = 1;
            b.grid = g;
            off += al256(large_scratch_bytes(b.n, g, p->precision));
        }
        b.bytes = off - start;
    }
    p->ws_bytes = off;
    return MSP_OK;
}

static void plan_release(msp_multi_plan *p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    p->exec = NULL;
    if (p->ready) {
        for (MultiBucket &b : p->buckets) {
            if (b.stream) cudaStreamDestroy(b.stream);
            if (b.done) cudaEventDestroy(b.done);
            b.stream = NULL;
            b.done = NULL;
        }
        if (p->origin) cudaStreamDestroy(p->origin);
        if (p->fork) cudaEventDestroy(p->fork);
        if (p->tab_pinned) cudaFreeHost(p->tab_pinned);
        p->origin = NULL;
        p->fork = NULL;
        p->tab_pinned = NULL;
        p->ready = false;
    }
}

// Streams, events, the pinned table copy, function attributes and the
// persistent grids, made once on the device current at the first run.
static int plan_prepare(msp_multi_plan *p) {
    int dev = 0;
    int rc = mcuda(cudaGetDevice(&dev), "msp_multi_run: cudaGetDevice");
    if (rc != MSP_OK) return rc;
    if (p->ready) {
        if (dev != p->device)
            return mfail(MSP_ERR_ARG, "msp_multi_run: plan prepared on device %d, current is %d",
                         p->device, dev);
        return MSP_OK;
    }
    p->device = dev;
    p->ready = true;  // plan_release cleans up a partial set-up
    rc = mcuda(cudaStreamCreateWithFlags(&p->origin, cudaStreamNonBlocking), "msp_multi_run");
    if (rc == MSP_OK) rc = mcuda(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming), "msp_multi_run");
    if (rc == MSP_OK)
        rc = mcuda(cudaMallocHost(&p->tab_pinned, p->tab_bytes > 0 ? p->tab_bytes : 256),
                   "msp_multi_run: pinned table copy");
    if (rc == MSP_OK) memcpy(p->tab_pinned, p->tab.data(), p->tab_bytes);
    // bucket streams by priority in launch order (most work first): the
    // long large-n kernel gets the SMs first and the small buckets fill in
    // around it, in eager runs and in the graph (node priorities)
    int prio_least = 0, prio_greatest = 0;
    if (rc == MSP_OK)
        rc = mcuda(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest),
                   "msp_multi_run: stream priorities");
    int rank = 0;
    for (MultiBucket &b : p->buckets) {
        if (rc != MSP_OK) break;
        int prio = prio_greatest + rank++;
        if (prio > prio_least) prio = prio_least;
        rc = mcuda(cudaStreamCreateWithPriority(&b.stream, cudaStreamNonBlocking, prio),
                   "msp_multi_run");
        if (rc == MSP_OK)
            rc = mcuda(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming), "msp_multi_run");
        if (rc == MSP_OK && !b.large) {
            int cps = b.ctas_per_sm;
            const int occ = snap_occupancy(b.n, MSP_MODE_FAST, p->precision, b.threads);
            if (cps <= 0 || cps > occ) cps = occ;
            int g = p->sms * cps;
            if (g > b.cap_snap) g = b.cap_snap;
            b.grid = g > 0 ? g : 1;
        }
    }
    if (rc != MSP_OK) plan_release(p);
    return rc;
}

static int check_io(const msp_multi_plan *p, const msp_multi_io *io) {
    if (io == NULL) return mfail(MSP_ERR_ARG, "msp_multi_run: io is NULL");
    if (io->out == NULL) return mfail(MSP_ERR_ARG, "msp_multi_run: out is NULL");
    if (p->num_snap > 0) {
        if (!io->Hsys_all || !io->Z_all || !io->field || !io->pol || !io->wscale || !io->status)
            return mfail(MSP_ERR_ARG, "msp_multi_run: a snapshot input or status pointer is NULL");
    }
    if (!p->uniform && io->times == NULL)
        return mfail(MSP_ERR_ARG, "msp_multi_run: times is NULL on a non-uniform grid");
    if (io->workspace == NULL || io->workspace_bytes < p->ws_bytes)
        return mfail(MSP_ERR_WORKSPACE, "msp_multi_run: workspace %zu < %zu bytes",
                     io->workspace_bytes, p->ws_bytes);
    if (reinterpret_cast<uintptr_t>(io->workspace) & 255)
        return mfail(MSP_ERR_ARG, "msp_multi_run: workspace not 256-byte aligned");
    return MSP_OK;
}

// The launch sequence of one run on `st` (also what a graph captures).
static int plan_enqueue(msp_multi_plan *p, const msp_multi_io *io, cudaStream_t st) {
    char *ws = reinterpret_cast<char *>(io->workspace);
    const int T = p->num_times;
    const bool mixed = p->precision == MSP_PREC_MIXED;
    const bool records = mixed && p->uniform;
    int rc = mcuda(cudaMemcpyAsync(ws, p->tab_pinned, p->tab_bytes, cudaMemcpyHostToDevice, st),
                   "msp_multi_run: tables");
    if (rc == MSP_OK)
        rc = mcuda(cudaMemsetAsync(io->out, 0, sizeof(double) * (size_t)p->num_systems * T, st),
                   "msp_multi_run: clear output");
    if (rc == MSP_OK) rc = mcuda(cudaEventRecord(p->fork, st), "msp_multi_run: fork");
    if (rc != MSP_OK) return rc;
    for (MultiBucket &b : p->buckets) {
        rc = mcuda(cudaStreamWaitEvent(b.stream, p->fork, 0), "msp_multi_run: fork");
        if (rc != MSP_OK) return rc;
        for (const MultiChunk &c : b.chunks) {
            const int cs = c.snap_end - c.snap_begin;
            SnapArgs sa;
            memset(&sa, 0, sizeof(sa));
            sa.n = b.n;
            sa.num_snap = cs;
            sa.max_sweeps = p->max_sweeps > 0 ? p->max_sweeps : 40;
            sa.max_refine = 4;
            sa.Hsys = reinterpret_cast<const cx<double> *>(io->Hsys_all);
            sa.Z = reinterpret_cast<const cx<double> *>(io->Z_all);
            sa.field = io->field;
            sa.pol = io->pol;
            sa.wscale = io->wscale;
            sa.t0 = p->t0;
            sa.dt = p->dt;
            snap_time_constants(sa);
            sa.pair_coef = ws + b.off_coef;
            sa.pair_omega = records ? NULL : reinterpret_cast<double *>(ws + b.off_phase);
            sa.pair_phase = records ? reinterpret_cast<float4 *>(ws + b.off_phase) : NULL;
            sa.snap_const = reinterpret_cast<double *>(ws + b.off_const);
            sa.status = io->status;
            sa.coef_f32 = mixed;
            sa.evec = (!b.large && snap_evec_bytes(b.n, 1, p->precision) > 0) ? ws + b.off_evec
                                                                               : NULL;
            sa.num_seg = c.num_seg;
            sa.seg_first = reinterpret_cast<const int *>(ws + c.seg_first);
            sa.seg_g0 = reinterpret_cast<const int *>(ws + c.seg_g0);
            sa.seg_hoff = reinterpret_cast<const long long *>(ws + c.seg_hoff);
            if (cs > 0) {
                if (b.large)
                    rc = mcuda(launch_large_fast(sa, reinterpret_cast<double *>(ws + b.off_large),
                                                 std::min(b.grid, cs), b.stream, b.threads,
                                                 p->precision),
                               "msp_multi_run: large-n snapshots");
                else
                    rc = mcuda(launch_snapshots(sa, MSP_MODE_FAST, p->precision, b.stream,
                                                b.threads, std::min(b.grid, cs)),
                               "msp_multi_run: snapshots");
                if (rc != MSP_OK) return rc;
            }
            PhaseArgs pa;
            memset(&pa, 0, sizeof(pa));
            pa.pair_coef = ws + b.off_coef;
            pa.pair_omega = sa.pair_omega;
            pa.pair_phase = sa.pair_phase;
            pa.P = b.P;
            pa.IP = b.ip;
            pa.slot_first = sa.seg_first;
            pa.item_first = reinterpret_cast<const int *>(ws + c.item_first);
            pa.num_slots = c.num_seg;
            pa.t0 = p->t0;
            pa.dt = p->dt;
            pa.num_times = T;
            pa.times = io->times;
            pa.partial = records ? NULL : reinterpret_cast<double *>(ws + b.off_partial);
            pa.partial_f32 = records ? reinterpret_cast<float *>(ws + b.off_partial) : NULL;
            pa.slot_row = reinterpret_cast<const int *>(ws + c.slot_row);
            pa.accumulate = 1;
            if (c.num_items > 0) {
                rc = mcuda(launch_phase(pa, p->precision, c.num_items, p->uniform, b.stream),
                           "msp_multi_run: phase sum");
                if (rc != MSP_OK) return rc;
            }
            if (c.num_seg > 0) {
                rc = mcuda(launch_reduce(pa, sa.snap_const, io->out, T, b.stream),
                           "msp_multi_run: reduction");
                if (rc != MSP_OK) return rc;
            }
        }
        rc = mcuda(cudaEventRecord(b.done, b.stream), "msp_multi_run: join");
        if (rc == MSP_OK) rc = mcuda(cudaStreamWaitEvent(st, b.done, 0), "msp_multi_run: join");
        if (rc != MSP_OK) return rc;
    }
    return MSP_OK;
}

extern "C" {

int msp_multi_plan_create(const msp_multi_desc *d, msp_multi_plan **out) {
    if (out == NULL) return mfail(MSP_ERR_ARG, "msp_multi_plan_create: plan is NULL");
    *out = NULL;
    if (d == NULL) return mfail(MSP_ERR_ARG, "msp_multi_plan_create: desc is NULL");
    if (d->num_systems < 1 || d->sys_n == NULL || d->sys_snap_first == NULL)
        return mfail(MSP_ERR_ARG, "msp_multi_plan_create: num_systems=%d or a NULL table",
                     d->num_systems);
    if (d->num_times < 1) return mfail(MSP_ERR_ARG, "msp_multi_plan_create: num_times=%d", d->num_times);
    if (d->precision != MSP_PREC_FP64 && d->precision != MSP_PREC_MIXED)
        return mfail(MSP_ERR_ARG, "msp_multi_plan_create: precision=%d", d->precision);
    if (d->num_tuning < 0 || (d->num_tuning > 0 && d->tuning == NULL))
        return mfail(MSP_ERR_ARG, "msp_multi_plan_create: num_tuning=%d", d->num_tuning);
    for (int i = 0; i < d->num_tuning; ++i) {
        const msp_multi_tuning &t = d->tuning[i];
        if (t.snap_threads < 0 || t.snap_threads > 512 || (t.snap_threads & 31) ||
            t.ctas_per_sm < 0 || t.ctas_per_sm > 32 || t.snaps_per_item < 0)
            return mfail(MSP_ERR_ARG,
                         "msp_multi_plan_create: tuning[%d] (threads %d: multiple of 32 up to 512; "
                         "ctas_per_sm %d: 0..32; snaps_per_item %d >= 0)",
                         i, t.snap_threads, t.ctas_per_sm, t.snaps_per_item);
    }
    if (d->sys_snap_first[0] != 0)
        return mfail(MSP_ERR_ARG, "msp_multi_plan_create: sys_snap_first[0] must be 0");
    long long hoff = 0;
    for (int k = 0; k < d->num_systems; ++k) {
        const int n = d->sys_n[k];
        if (n < 2 || (n & 1))
            return mfail(MSP_ERR_ARG,
                         "msp_multi_plan_create: system %d has n=%d (the fast path needs the "
                         "muon first: n even, >= 2)",
                         k, n);
        if (n > MSP_MAX_DIM_LARGE)
            return mfail(MSP_ERR_UNSUPPORTED, "msp_multi_plan_create: system %d has n=%d > %d", k,
                         n, MSP_MAX_DIM_LARGE);
        if (d->sys_snap_first[k + 1] < d->sys_snap_first[k])
            return mfail(MSP_ERR_ARG, "msp_multi_plan_create: sys_snap_first decreases at %d", k);
        hoff += (long long)n * n;
    }
    msp_multi_plan *p = new (std::nothrow) msp_multi_plan();
    if (p == NULL) return mfail(MSP_ERR_ARG, "msp_multi_plan_create: out of host memory");
    p->num_systems = d->num_systems;
    p->num_snap = d->sys_snap_first[d->num_systems];
    p->num_times = d->num_times;
    p->uniform = d->uniform ? 1 : 0;
    p->t0 = d->t0;
    p->dt = d->dt;
    p->precision = d->precision;
    p->max_sweeps = d->max_sweeps;
    p->sms = device_sms();
    p->sys_n.assign(d->sys_n, d->sys_n + d->num_systems);
    p->snap_first.assign(d->sys_snap_first, d->sys_snap_first + d->num_systems + 1);
    p->h_off.resize(d->num_systems);
    hoff = 0;
    for (int k = 0; k < d->num_systems; ++k) {
        p->h_off[k] = hoff;
        hoff += (long long)p->sys_n[k] * p->sys_n[k];
    }
    p->ready = false;
    p->tab_pinned = NULL;
    p->origin = NULL;
    p->fork = NULL;
    p->exec = NULL;
    int rc = plan_layout(p, d);
    if (rc != MSP_OK) {
        delete p;
        return rc;
    }
    *out = p;
    return MSP_OK;
}

int msp_multi_plan_destroy(msp_multi_plan *p) {
    if (p == NULL) return MSP_OK;
    plan_release(p);
    delete p;
    return MSP_OK;
}

int msp_multi_workspace(const msp_multi_plan *p, size_t *bytes) {
    if (p == NULL || bytes == NULL) return mfail(MSP_ERR_ARG, "msp_multi_workspace: NULL argument");
    *bytes = p->ws_bytes;
    return MSP_OK;
}

int msp_multi_plan_info(const msp_multi_plan *p, int *num_buckets, msp_multi_bucket_info *info,
                        int capacity) {
    if (p == NULL || num_buckets == NULL)
        return mfail(MSP_ERR_ARG, "msp_multi_plan_info: NULL argument");
    *num_buckets = (int)p->buckets.size();
    for (int i = 0; i < *num_buckets && i < capacity && info != NULL; ++i) {
        const MultiBucket &b = p->buckets[i];
        msp_multi_bucket_info &o = info[i];
        o.n = b.n;
        o.num_systems = (int)b.systems.size();
        o.num_snap = b.num_snap;
        o.num_chunks = (int)b.chunks.size();
        o.snap_threads = b.threads;
        o.grid = b.grid;
        o.pairs_per_item = b.ip;
        o.max_items = b.max_items;
        o.scratch_bytes = b.bytes;
    }
    return MSP_OK;
}

int msp_multi_run(msp_multi_plan *p, const msp_multi_io *io, void *stream) {
    if (p == NULL) return mfail(MSP_ERR_ARG, "msp_multi_run: plan is NULL");
    int rc = check_io(p, io);
    if (rc == MSP_OK) rc = plan_prepare(p);
    if (rc != MSP_OK) return rc;
    return plan_enqueue(p, io, (cudaStream_t)stream);
}

int msp_multi_run_graph(msp_multi_plan *p, const msp_multi_io *io, void *stream) {
    if (p == NULL) return mfail(MSP_ERR_ARG, "msp_multi_run_graph: plan is NULL");
    int rc = check_io(p, io);
    if (rc == MSP_OK) rc = plan_prepare(p);
    if (rc != MSP_OK) return rc;
    const msp_multi_io &g = p->graph_io;
    const bool same = p->exec != NULL && g.Hsys_all == io->Hsys_all && g.Z_all == io->Z_all &&
                      g.field == io->field && g.pol == io->pol && g.wscale == io->wscale &&
                      g.times == io->times && g.out == io->out && g.status == io->status &&
                      g.workspace == io->workspace;
    if (!same) {
        if (p->exec) {
            cudaGraphExecDestroy(p->exec);
            p->exec = NULL;
        }
        rc = mcuda(cudaStreamBeginCapture(p->origin, cudaStreamCaptureModeRelaxed),
                   "msp_multi_run_graph: begin capture");
        if (rc != MSP_OK) return rc;
        const int rc_enq = plan_enqueue(p, io, p->origin);
        cudaGraph_t graph = NULL;
        const cudaError_t e = cudaStreamEndCapture(p->origin, &graph);
        if (rc_enq != MSP_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc_enq;
        }
        rc = mcuda(e, "msp_multi_run_graph: end capture");
        if (rc == MSP_OK)
            rc = mcuda(cudaGraphInstantiate(&p->exec, graph, cudaGraphInstantiateFlagUseNodePriority),
                       "msp_multi_run_graph: instantiate");
        if (graph) cudaGraphDestroy(graph);
        if (rc != MSP_OK) {
            p->exec = NULL;
            return rc;
        }
        p->graph_io = *io;
    }
    return mcuda(cudaGraphLaunch(p->exec, (cudaStream_t)stream), "msp_multi_run_graph: launch");
}

}  // extern "C"
