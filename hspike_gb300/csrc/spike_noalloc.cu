// spike_noalloc.cu -- the fixed device workspace behind
// spike_dsolve_device_noalloc (see spike_gb300.h).
//
// Some callers must not allocate device memory at solve time: code that runs
// while a stream is being captured into a CUDA graph (cudaMalloc is not a
// capturable operation), latency-critical loops that cannot afford the device
// synchronisation cudaMalloc/cudaFree imply, and hosts that hand the whole
// device heap to their own pool allocator.  For them the library reserves one
// file-scope device array, sized once and for all, that the no-allocation
// solve carves its workspace from.  Every GPU that loads the library holds
// these bytes until the process exits.
#include <cuda_runtime.h>

#include "spike_internal.h"

#define SPK_NOALLOC_MAX_DEVICES 64

// The workspace itself.  Host code must not take its address directly (in host
// code the name is a host-side shadow, not a device address); it asks
// spk_noalloc_scratch() below, which resolves the device address per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SPK_NOALLOC_SCRATCH_BYTES];

static void *g_noalloc_ptr[SPK_NOALLOC_MAX_DEVICES];

// Device address of the workspace on the current device.  The first call on a
// device resolves it with cudaGetSymbolAddress (this is the set-up; it loads
// the module on that device and must not happen during stream capture) and
// caches it; later calls only read the cache.  Returns SPK_OK or SPK_ECUDA.
extern "C" int spk_noalloc_scratch(void **ptr, size_t *bytes)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SPK_NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return SPK_ECUDA;
    }
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return SPK_ECUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *ptr = g_noalloc_ptr[dev];
    *bytes = (size_t)SPK_NOALLOC_SCRATCH_BYTES;
    return SPK_OK;
}
