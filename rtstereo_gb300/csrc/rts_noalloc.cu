// rts_noalloc.cu -- winner-takes-all for callers that cannot allocate device memory.
//
// rts_WTA (rts_modules.cpp) takes its scratch (the per-pixel winners and the
// per-row summaries of the carry pass) from the context arena, which grows
// with cudaMalloc.  Some hosts cannot allow that: an application that fixes
// its device memory at start-up and owns every allocation itself, or a frame
// loop where the implicit device-wide synchronisation of cudaMalloc/cudaFree
// would stall its other streams.  rts_WTA_noalloc gives them the same result
// with no allocation at all: its scratch is the file-scope device array below,
// created with the module when the library is loaded and held by every GPU
// that loads it until the process exits.
//
// Limits: at most kNoAllocMaxPixels pixels (rdim*cdim) and kNoAllocMaxRows rows.
// Every call shares the one array, so calls whose kernels overlap on the GPU
// (concurrent streams, or threads) race on it and must be serialised by the
// caller.
#include <mutex>

#include "rts_common.cuh"

namespace rts {

constexpr long kNoAllocMaxPixels = 1L << 21;  // 2,097,152 pixels: 1920x1080 fits
constexpr int kNoAllocMaxRows = 8192;

// winners (u16 per pixel) followed by the row summaries (int per row)
static __device__ __align__(256) unsigned char g_wta_scratch[kNoAllocMaxPixels * 2 + kNoAllocMaxRows * 4];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices];  // device address of g_wta_scratch on each device, set up once
}  // namespace

// Looks up (once per device, with that device current) the device address of
// the scratch array.  The host-side name g_wta_scratch is not a device address.
static cudaError_t noalloc_scratch(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_wta_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace rts

using namespace rts;

extern "C" rts_status rts_WTA_noalloc(const float *cost, uint8_t *winners, int rdim, int cdim, int dispRange,
                                      void *cuda_stream) {
    if (!cost || !winners) return RTS_ERR_INVALID_ARG;
    if (rdim <= 0 || cdim <= 0 || dispRange <= 0 || dispRange > kMaxDisp) return RTS_ERR_INVALID_ARG;
    if ((long)rdim * cdim > kNoAllocMaxPixels || rdim > kNoAllocMaxRows) return RTS_ERR_INVALID_ARG;
    // an error left by earlier work on this thread is reported before any work of
    // this call, so that the status after the launches is this call's own
    if (cudaGetLastError() != cudaSuccess) return RTS_ERR_CUDA;
    void *base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) return e == cudaErrorNoDevice ? RTS_ERR_UNSUPPORTED : RTS_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    uint16_t *raw = (uint16_t *)base;
    int *row_last = (int *)((unsigned char *)base + kNoAllocMaxPixels * 2);
    // the row summaries must start at -1 on every call (the array keeps the last call's contents)
    if (cudaMemsetAsync(row_last, 0xff, (size_t)rdim * sizeof(int), s) != cudaSuccess) return RTS_ERR_CUDA;
    launch_wta_local(s, cost, raw, row_last, rdim, cdim, dispRange, 0);
    if (cudaGetLastError() != cudaSuccess) return RTS_ERR_CUDA;
    launch_wta_fill(s, raw, row_last, winners, rdim, cdim, 0);
    return cudaGetLastError() == cudaSuccess ? RTS_OK : RTS_ERR_CUDA;
}
