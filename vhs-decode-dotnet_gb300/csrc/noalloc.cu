// Sync-pulse edge scan that allocates no device memory.
//
// Some callers cannot allocate while they decode: a host thread that is
// capturing the decode into a CUDA graph (cudaMalloc is not a capturable
// operation and cudaFree synchronises the device), a real-time capture loop
// that must not stall on the allocator, or an application whose memory
// budget is fixed up front.  For them this entry point runs the same two-pass
// pulse edge scan as the session path, but its per-slice count and offset
// scratch lives in a fixed array of device memory that belongs to the
// library image, so the call only launches kernels on the caller's stream.
//
// Limits and rules of use:
// * at most kNoAllocMaxSamples samples per call; longer inputs are rejected;
// * every call made outside a stream capture (any arguments, n = 0 included)
//   looks up the scratch array's address with the current device; the first
//   call on a device must be such a call, made before any stream capture;
// * the scratch array is shared by every call on a device, so calls must not
//   overlap: issue them on one stream, or order them, never from two streams
//   or threads at once;
// * nothing needs to start at zero: each call writes every count and offset
//   slot it reads before reading it, and writes *total.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "../../include/vhsdecode_gb300.h"
#include "kernels.h"

namespace vhsd {
int32_t set_last_error(int32_t status, const char* msg);
}
using namespace vhsd;

namespace {

constexpr int64_t kNoAllocMaxSamples = int64_t(1) << 24;  // 16,777,216 samples
constexpr int64_t kNoAllocSlots = (kNoAllocMaxSamples + kPulseChunk - 1) / kPulseChunk * 4;

// counts in [0, slots), offsets in [slots, 2 * slots): 256 KiB per device
static __device__ __align__(256) int64_t g_pulse_scratch[2 * kNoAllocSlots];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
int64_t* g_scratch_ptr[kMaxDevices] = {};

// The address is looked up again on every call made outside a stream capture,
// so a context that was torn down and recreated (cudaDeviceReset) gets the
// reloaded module's address; a call inside a capture uses the address of the
// last call made outside one.
int32_t scratch_for_current_device(cudaStream_t stream, int64_t** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0)
        return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no current CUDA device");
    if (dev >= kMaxDevices)
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "device index above 63");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess)
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT,
                              (std::string("stream query: ") + cudaGetErrorString(e)).c_str());
    std::lock_guard<std::mutex> lock(g_mutex);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
        if (cap != cudaStreamCaptureStatusNone)
            return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT,
                                  "first no-allocation call on this device made inside a stream capture");
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_pulse_scratch);
        if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
            return set_last_error(VHSDECODE_GB300_STATUS_CUDA_UNAVAILABLE, "no usable CUDA device");
        if (e != cudaSuccess || !p)
            return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR,
                                  (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
        g_scratch_ptr[dev] = static_cast<int64_t*>(p);
    }
    *out = g_scratch_ptr[dev];
    return VHSDECODE_GB300_STATUS_OK;
}

}  // namespace

extern "C" {

VHSDECODE_GB300_API int32_t VHSDECODE_GB300_CALL vhsdecode_gb300_pulse_events_noalloc(
    const float* sync, int64_t length, double high, int64_t* events, int64_t capacity,
    int64_t* total, void* stream) {
    int64_t* scratch = nullptr;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int32_t st = scratch_for_current_device(s, &scratch);
    if (st != VHSDECODE_GB300_STATUS_OK) return st;
    if (length < 0 || capacity < 0)
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT, "negative length or capacity");
    if (length > kNoAllocMaxSamples)
        return set_last_error(VHSDECODE_GB300_STATUS_INVALID_ARGUMENT,
                              "length above the 16777216-sample limit of the no-allocation pulse scan");
    if (!total || (length && !sync) || (capacity && !events))
        return set_last_error(VHSDECODE_GB300_STATUS_NULL_POINTER, "null argument");
    cudaError_t e = launch_pulse_events<float>(sync, length, high, scratch, scratch + kNoAllocSlots,
                                               events, capacity, total, s);
    if (e != cudaSuccess)
        return set_last_error(VHSDECODE_GB300_STATUS_INTERNAL_ERROR,
                              (std::string("pulse scan launch: ") + cudaGetErrorString(e)).c_str());
    return set_last_error(VHSDECODE_GB300_STATUS_OK, "");
}

}  // extern "C"
