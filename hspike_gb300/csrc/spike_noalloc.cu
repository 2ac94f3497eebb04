// spike_noalloc.cu -- the fixed device workspace behind
// spike_dsolve_device_noalloc (declared in spike_gb300.h).
//
// Some callers cannot allocate device memory when they solve: programs whose
// own pool allocator has taken the device heap (a cudaMalloc from a library
// would fail or fragment it), latency-critical loops that cannot absorb the
// device-wide synchronisation that cudaFree implies, and plugin hosts that do
// not let a library allocate on their behalf.  For them the library keeps one
// file-scope device array of a fixed size, and the no-allocation solve carves
// every temporary from it.  Every GPU that loads the library holds these bytes
// until the process exits.
#include <cuda_runtime.h>

#include "spike_gb300.h"
#include "spike_internal.h"

static_assert(SPK_NOALLOC_SCRATCH_BYTES == SPIKE_NOALLOC_WORKSPACE_BYTES,
              "the workspace the header announces is the array's size");

// The workspace itself.  In host code this name is a host-side stand-in, not
// a device address: a kernel handed it would fault, or silently use the wrong
// memory where the GPU can reach host memory.  Host code asks
// spk_noalloc_scratch() below for the device address instead.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SPK_NOALLOC_SCRATCH_BYTES];

// Device address of the workspace on the current device, resolved with
// cudaGetSymbolAddress on every call (not a stream operation, and cheap once
// the module is loaded on the device, so nothing is cached that a device
// reset could make stale).  Returns SPK_OK or SPK_ECUDA.
extern "C" int spk_noalloc_scratch(void **ptr, size_t *bytes)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return SPK_ECUDA;
    }
    *ptr = p;
    *bytes = (size_t)SPK_NOALLOC_SCRATCH_BYTES;
    return SPK_OK;
}
