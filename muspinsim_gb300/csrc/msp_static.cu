// msp_powder_run_static: the powder pipeline for callers that cannot
// allocate GPU memory.
//
// msp_powder_run needs a scratch buffer (eigenvalue-pair lists, per-item
// partial sums, schedule tables) that its caller allocates.  Some callers
// cannot do that: a host whose device memory is owned by another runtime
// and must not be allocated behind its back, a binding language with no
// way to reach cudaMalloc, or a latency-critical loop where a cudaMalloc
// (which can synchronise the whole device) is not acceptable.  This entry
// point takes its scratch from a fixed array compiled into the library
// instead, so the caller passes only the inputs and outputs and nothing is
// allocated at any call.
//
// The array is a file-scope __device__ variable of MSP_STATIC_SCRATCH_BYTES;
// every GPU that loads the library holds it until the process exits.  Host
// code cannot use the array's name as a device address, so the first call
// on each device -- with that device current -- looks the address up with
// cudaGetSymbolAddress and caches it; make that first call before any
// stream capture.  The cached address belongs to the device's primary
// context: cudaDeviceReset destroys that context (and the array with it),
// after which the cached address is stale, so a process that resets a
// device must not call this entry point on it again.  Every call shares the one array and finds the previous
// call's contents in it: the pipeline writes every scratch byte before
// reading it, so nothing has to be cleared, but two calls that overlap on
// the GPU (different streams, or different host threads) race on the array
// and must be serialised by the caller.
#include <stdio.h>

#include <mutex>

#include "msp_internal.cuh"

namespace msp {
int record_error(int code, const char *msg);
}

static __device__ __align__(256) unsigned char g_msp_static_scratch[MSP_STATIC_SCRATCH_BYTES];

#define MSP_STATIC_MAX_DEVICES 64
static std::mutex g_static_mu;
static void *g_static_addr[MSP_STATIC_MAX_DEVICES];

// Device address of the scratch array on the current device (looked up once
// per device), or NULL with the error recorded.
static void *static_scratch_address(int *rc) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *rc = msp::record_error(MSP_ERR_CUDA, "msp_powder_run_static: cudaGetDevice failed");
        return NULL;
    }
    if (dev < 0 || dev >= MSP_STATIC_MAX_DEVICES) {
        *rc = msp::record_error(MSP_ERR_UNSUPPORTED,
                                "msp_powder_run_static: device ordinal beyond 64");
        return NULL;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (g_static_addr[dev] == NULL) {
        void *p = NULL;
        e = cudaGetSymbolAddress(&p, g_msp_static_scratch);
        if (e != cudaSuccess || p == NULL) {
            *rc = msp::record_error(MSP_ERR_CUDA,
                                    "msp_powder_run_static: cudaGetSymbolAddress failed");
            return NULL;
        }
        g_static_addr[dev] = p;
    }
    *rc = MSP_OK;
    return g_static_addr[dev];
}

extern "C" int msp_powder_run_static(const msp_powder_args *args) {
    size_t need = 0;
    int rc = msp_powder_workspace(args, &need);
    if (rc != MSP_OK) return rc;
    if (need > (size_t)MSP_STATIC_SCRATCH_BYTES) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "msp_powder_run_static: this batch needs %zu bytes of scratch but the built-in "
                 "scratch holds %u; split the batch (fewer snapshots or times) or use "
                 "msp_powder_run with a caller workspace",
                 need, (unsigned)MSP_STATIC_SCRATCH_BYTES);
        return msp::record_error(MSP_ERR_WORKSPACE, msg);
    }
    void *scratch = static_scratch_address(&rc);
    if (scratch == NULL) return rc;
    msp_powder_args a = *args;
    a.workspace = scratch;
    a.workspace_bytes = MSP_STATIC_SCRATCH_BYTES;
    return msp_powder_run(&a);
}
