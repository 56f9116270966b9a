// Σ cell volumes over device-resident results without allocating anything.
//
// Who needs this: callers that already hold the per-cell volumes on the device
// (vgpu_device_results) and run where a device allocation is not acceptable —
// a serving process that has handed its whole device memory budget to its own
// pool, or a latency-critical loop in which the first-call cudaMalloc of
// vgpu_sum_cell_volumes (its partial-sum buffer) would synchronise the device.
// This entry point takes the caller's pointers and stream, keeps its partial
// sums in a fixed static device array, and never calls cudaMalloc/cudaFree or
// any allocating library.
//
// Scratch: g_partials, kMaxPartials doubles (64 KB), one partial per tile of
// kTile cells, so n is limited to kTile * kMaxPartials = 33,554,432 cells;
// larger n is rejected with VGPU_ERR_ARG.  Nothing in the scratch has to
// start at zero: every call writes each partial it later reads.
//
// Set-up: the first call on each device (with that device current) looks up
// the scratch's device address with cudaGetSymbolAddress, which can also load
// this library's device code onto that device; make that first call before any
// stream capture.  Later calls reuse the cached address, so the entry point
// must not be used after a cudaDeviceReset (or any other teardown of the
// device's primary context) in the same process: the module, and with it the
// scratch, may then live at another address.
//
// Device: every call runs on the current device, which must own dev_vol,
// dev_out and the stream; the pointers are checked (cudaPointerGetAttributes,
// which allocates nothing) and a pointer of another device or of host memory
// is rejected with VGPU_ERR_ARG before anything is launched.
//
// Concurrency: there is one scratch array per device.  Two calls that overlap
// on one device (different streams, or different host threads) race on it and
// corrupt each other's partials; serialise them (one stream, or events).
#include <mutex>

#include "../../include/vorogpu.h"
#include "vgpu_internal.cuh"

namespace vgpu {

namespace {

constexpr int kTile = 4096;          // cells per partial
constexpr int kMaxPartials = 8192;   // 8192 doubles = 64 KB
constexpr long long kMaxCells = (long long)kTile * kMaxPartials;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_partials[kMaxPartials];

std::mutex g_setup_mutex;
double *g_scratch[kMaxDevices];   // device address of g_partials per device (nullptr: not set up)

__device__ __forceinline__ double block_sum(double s, double *red) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(0xffffffffu, t, d);
    }
    return t;   // valid in thread 0
}

// One CTA per tile of kTile cells; fixed summation order (deterministic).
__global__ void __launch_bounds__(kThreads) tile_sums_kernel(const double *vol, long long n, double *partials) {
    __shared__ double red[kThreads / 32];
    const long long base = (long long)blockIdx.x * kTile;
    double s = 0.0;
    for (int i = threadIdx.x; i < kTile; i += kThreads) {
        const long long k = base + i;
        if (k < n) s += vol[k];
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// One CTA folds the tiles' partials in a fixed order and writes the total.
__global__ void __launch_bounds__(kThreads) total_kernel(const double *partials, int ntiles, double *out) {
    __shared__ double red[kThreads / 32];
    double s = 0.0;
    for (int i = threadIdx.x; i < ntiles; i += kThreads) s += partials[i];
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) *out = t;
}

// VGPU_OK if p is device (or managed) memory of device dev.
int check_on_device(const void *p, int dev, const char *what) {
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();   // clear it: the caller's pointer is what is wrong
        return report_error(VGPU_ERR_ARG, "%s: not a CUDA pointer (%s)", what, cudaGetErrorString(e));
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
        return report_error(VGPU_ERR_ARG, "%s is not device memory", what);
    if (a.device != dev)
        return report_error(VGPU_ERR_ARG, "%s lives on device %d but device %d is current", what, a.device, dev);
    return VGPU_OK;
}

int scratch_for_current_device(double **out, int *dev_out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return report_error(VGPU_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return report_error(VGPU_ERR_ARG, "device ordinal %d out of range", dev);
    *dev_out = dev;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess || !p)
            return report_error(VGPU_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_scratch[dev] = static_cast<double *>(p);
    }
    *out = g_scratch[dev];
    return VGPU_OK;
}

}  // namespace

}  // namespace vgpu

extern "C" int vgpu_sum_volumes_noalloc(const double *dev_vol, int64_t n, double *dev_out, void *stream) {
    using namespace vgpu;
    if (!dev_out) return report_error(VGPU_ERR_ARG, "null output pointer");
    if (n < 0) return report_error(VGPU_ERR_ARG, "negative cell count %lld", (long long)n);
    if (n > kMaxCells)
        return report_error(VGPU_ERR_ARG,
                            "%lld cells exceed the no-alloc scratch capacity of %lld cells (%d partials of %d)",
                            (long long)n, kMaxCells, kMaxPartials, kTile);
    if (n > 0 && !dev_vol) return report_error(VGPU_ERR_ARG, "null volume pointer");
    double *scratch = nullptr;
    int dev = -1;
    int rc = scratch_for_current_device(&scratch, &dev);
    if (rc != VGPU_OK) return rc;
    if (n > 0 && (rc = check_on_device(dev_vol, dev, "dev_vol")) != VGPU_OK) return rc;
    if ((rc = check_on_device(dev_out, dev, "dev_out")) != VGPU_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int ntiles = (int)((n + kTile - 1) / kTile);
    if (ntiles > 0) {
        tile_sums_kernel<<<ntiles, kThreads, 0, s>>>(dev_vol, (long long)n, scratch);
        note_launch();
    }
    total_kernel<<<1, kThreads, 0, s>>>(scratch, ntiles, dev_out);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return report_error(VGPU_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
    return VGPU_OK;
}
