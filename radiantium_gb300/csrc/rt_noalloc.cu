/*
 * rt_noalloc.cu - the fixed device scratch of rt_render_device_noalloc.
 *
 * Some hosts cannot let a library allocate device memory while they render:
 * an engine that hands all of the GPU's memory to its own pool allocator at
 * start-up, or a frame loop that cannot afford the device-wide
 * synchronisation cudaFree brings with it.  For them the megakernel render
 * (k_render + k_accumulate + k_finalize in rt_kernels.cu) runs out of this one
 * array.  It lives in its own translation unit.  Under lazy module loading
 * (CUDA_MODULE_LOADING=LAZY, the default of CUDA 12.2 and later) its module -
 * and the RT_NOALLOC_SCRATCH_BYTES the runtime reserves for it - is loaded
 * only by the first lookup below, never by the other entry points; with
 * CUDA_MODULE_LOADING=EAGER every process that loads the library reserves the
 * array when its context is created, whether it renders this way or not.
 * The layout is set by
 * render_noalloc in rt_host.cpp: status word, counters, film sums, then one
 * chunk of per-sample radiance.
 */
#include <cuda_runtime.h>
#include <mutex>
#include "rt_launch.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[RT_NOALLOC_SCRATCH_BYTES];

cudaError_t rt_noalloc_scratch(int device, void** ptr) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static void* cached[kMaxDevices] = {};
    if (!ptr || device < 0 || device >= kMaxDevices) return cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lock(mu);
    if (!cached[device]) {
        int cur = -1;
        cudaError_t e = cudaGetDevice(&cur);
        if (e != cudaSuccess) return e;
        if (cur != device) return cudaErrorInvalidDevice;
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        cached[device] = p;
    }
    *ptr = cached[device];
    return cudaSuccess;
}
