// noalloc.cu — the grid sort for callers that must not allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc or any allocating routine
// at the point where they sort particles:
//   * hosts that run under a fixed device-memory budget enforced by their own
//     pool allocator, where a raw cudaMalloc would either fail or escape the
//     budget accounting;
//   * real-time loops that may not pay cudaMalloc/cudaFree's implicit device
//     synchronisation or their latency.
// gsph_grid_sort_dev already lets the caller pass its own scratch buffer; this
// variant goes further and needs no scratch from the caller at all. Its
// scratch is one file-scope __device__ array of fixed size, so the only memory
// it uses is the caller's inputs and outputs plus that array. The array is part
// of the library's device image: every GPU on which the library is loaded
// holds it (GSPH_NOALLOC_SCRATCH_BYTES) until the process exits.
//
// This entry point has no counterpart in the reference.
#include <mutex>

#include <cuda.h>

#include "gsph_internal.h"

namespace gsph {
namespace {

constexpr int kMaxDevices = 64;

// Sized for GSPH_NOALLOC_MAX_PARTICLES particles and GSPH_NOALLOC_MAX_CELLS
// cells (the layout gsph_grid_sort_dev carves out of a scratch buffer).
static __device__ __align__(256) unsigned char
    g_sort_scratch[GSPH_NOALLOC_SCRATCH_BYTES];

std::mutex g_scratch_mutex;
// Per device: the address of g_sort_scratch and the unique ID of the CUDA
// context it was looked up in. A context ID is never reused within a process,
// so a cudaDeviceReset (which unloads the module with its context) or a
// different current context (a non-primary driver context) forces a new
// look-up instead of reusing an address of another context.
struct ScratchCache {
    unsigned long long ctx_id;
    void *addr;
};
ScratchCache g_scratch[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// Unique ID of the current context, or 0 where none is current or the driver
// does not report one (then every call looks the address up again).
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        resolved = true;
        void *fa = nullptr, *fb = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fa, 12000,
                                             cudaEnableDefault, &qa) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &fb, 12000,
                                             cudaEnableDefault, &qb) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(fa);
            get_id = reinterpret_cast<CtxGetIdFn>(fb);
        }
        cudaGetLastError();
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_sort_scratch in the current context. In host code the
// array's name is only a host-side stand-in, so the address is looked up with
// the device current — once per device and context: the first call on a
// device (and the first after a device reset) does this set-up.
gsph_status scratch_address(int device, void **out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    ScratchCache &c = g_scratch[device];
    const unsigned long long id = current_context_id();
    if (id != 0 && c.addr && c.ctx_id == id) {
        *out = c.addr;
        return GSPH_OK;
    }
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        set_error("gsph_grid_sort_dev_noalloc: cudaGetSymbolAddress failed "
                  "on device %d: %s",
                  device, cudaGetErrorString(e));
        return GSPH_ERR_CUDA;
    }
    // the look-up made the context current if it was not yet
    c.ctx_id = id != 0 ? id : current_context_id();
    c.addr = p;
    *out = p;
    return GSPH_OK;
}

}  // namespace
}  // namespace gsph

using namespace gsph;

extern "C" gsph_status gsph_grid_sort_dev_noalloc(
    const gsph_params *p, uint32_t n, const float *pos_in, const float *vel_in,
    const float *ev_in, float *pos_out, float *vel_out, float *ev_out,
    uint32_t *key_out, int32_t *perm_out, int32_t *cell_start_out,
    void *stream) {
    if (!p) {
        set_error("gsph_grid_sort_dev_noalloc: null parameters");
        return GSPH_ERR_INVALID_ARG;
    }
    long long numc = 0;
    {
        const gsph_status gs = check_grid(*p, "gsph_grid_sort_dev_noalloc", &numc);
        if (gs) return gs;
    }
    if (n > GSPH_NOALLOC_MAX_PARTICLES || numc > GSPH_NOALLOC_MAX_CELLS) {
        set_error("gsph_grid_sort_dev_noalloc: %u particles and %lld cells "
                  "exceed the fixed scratch (at most %u particles and %u "
                  "cells); use gsph_grid_sort_dev with caller scratch",
                  n, numc, GSPH_NOALLOC_MAX_PARTICLES, GSPH_NOALLOC_MAX_CELLS);
        return GSPH_ERR_CAPACITY;
    }
    const size_t need = gsph_grid_sort_scratch_bytes(n, uint32_t(numc));
    if (need > GSPH_NOALLOC_SCRATCH_BYTES) {
        set_error("gsph_grid_sort_dev_noalloc: %zu scratch bytes needed, %u "
                  "available",
                  need, GSPH_NOALLOC_SCRATCH_BYTES);
        return GSPH_ERR_CAPACITY;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess || device < 0 || device >= kMaxDevices) {
        set_error("gsph_grid_sort_dev_noalloc: no usable current device (%s)",
                  cudaGetErrorString(e));
        return GSPH_ERR_NO_DEVICE;
    }
    void *scratch = nullptr;
    gsph_status st = scratch_address(device, &scratch);
    if (st) return st;
    // The sort clears the counters it accumulates into (cell counts, frame
    // counters) at the start of every call, so contents left by the previous
    // call do not matter; calls that overlap on the GPU share the array and
    // race.
    return gsph_grid_sort_dev(p, n, pos_in, vel_in, ev_in, pos_out, vel_out,
                              ev_out, key_out, perm_out, cell_start_out,
                              scratch, GSPH_NOALLOC_SCRATCH_BYTES, stream);
}
