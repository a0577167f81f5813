// dtrt_gb300 — dtrt_render_fwd_noalloc: a forward-mode render that allocates nothing.
//
// Callers that cannot call cudaMalloc during a render (a runtime that owns every device
// allocation, a fixed memory budget set at start-up, a thread that must not take the
// allocator's locks) get every work buffer of the render from the array below instead:
// FP64 accumulators, task queues, counters and the staging copy of a host output.
//
// The array is a file-scope __device__ variable, so each GPU that loads this library holds
// DTRT_NOALLOC_SCRATCH_BYTES until the process exits. Host code cannot use the array's
// name as a device address (in host code it names a host-side shadow), so the first call
// on each device asks the runtime for the real address with cudaGetSymbolAddress and
// caches it; make that first call before any stream capture. Every call shares the array
// and leaves the previous call's contents behind; the render zeroes what must start at
// zero (accumulators, queue counters, error flags). Calls that overlap on the GPU race on
// the array and must be serialised by the caller. The cached address belongs to the
// device's primary context: it is not looked up again after a device reset, and a
// caller that renders under a context of its own creation is not supported.
#include <mutex>

#include "dt_host.h"

namespace dt {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[DTRT_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once per device).
int noalloc_scratch(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return DTRT_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_error("dtrt_render_fwd_noalloc: device index out of range");
        return DTRT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_last_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            return DTRT_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = (unsigned char *)p;
    }
    *out = g_noalloc_ptr[dev];
    return DTRT_OK;
}

}  // namespace
}  // namespace dt

extern "C" int dtrt_render_fwd_noalloc(dtrt_scene *scene, const dtrt_render_options *opts, float *out,
                                       int out_on_device, void *stream) {
    if (!scene || !opts || !out) {
        dt::set_last_error("null argument");
        return DTRT_ERR_INVALID;
    }
    if (opts->spp < 0 || opts->sppse < 0) {
        dt::set_last_error("spp and sppse must be >= 0");
        return DTRT_ERR_INVALID;
    }
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != scene->device) {
        cudaGetLastError();
        dt::set_last_error("dtrt_render_fwd_noalloc: the current device is not the scene's device");
        return DTRT_ERR_INVALID;
    }
    unsigned char *scratch = nullptr;
    int st = dt::noalloc_scratch(&scratch);
    if (st != DTRT_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t bytes = DTRT_NOALLOC_SCRATCH_BYTES;
    switch (scene->nder) {
        case 1: return dt::render_n_noalloc<1>(scene, opts, out, out_on_device, s, scratch, bytes);
        case 3: return dt::render_n_noalloc<3>(scene, opts, out, out_on_device, s, scratch, bytes);
        case 4: return dt::render_n_noalloc<4>(scene, opts, out, out_on_device, s, scratch, bytes);
        case 8: return dt::render_n_noalloc<8>(scene, opts, out, out_on_device, s, scratch, bytes);
    }
    dt::set_last_error("unsupported nder");
    return DTRT_ERR_UNSUPPORTED;
}
