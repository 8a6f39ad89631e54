// Squared error collector for callers that cannot allocate device memory.
//
// Some hosts of this library own all of the device memory through their own
// pool (an in-situ analysis hook inside a simulation whose allocator reserved
// the HBM up front, or a plugin host that forbids allocation inside its
// callbacks): a cudaMalloc there fails once the pool holds the free memory, or
// bypasses the pool's accounting, and cudaMalloc / cudaFree also synchronise
// the device, which a per-timestep hook cannot afford. Such a caller has no
// workspace to hand to prodm_collect_squared either. prodm_collect_squared_noalloc
// computes the same table with its scratch in the fixed device array below.
//
// Scratch: kPartialSlots (608) per-CTA partial tables of up to 65 doubles,
// 316,160 bytes, enough for the largest table (64 bitplanes, fp64). Larger
// num_bitplanes are rejected with PRODM_EINVAL.
//
// Set-up: a call on a stream that is not capturing looks up the array's
// device address (cudaGetSymbolAddress, with the calling thread's current
// device) and remembers it for that device; a call on a capturing stream uses
// the remembered address, so the first call on a device should come before
// any stream capture. Looking the address up again on every uncaptured call
// keeps it right after cudaDeviceReset or a switch of the device's context,
// where the module and its array are loaded anew.
//
// Sharing: every call on every stream of a device uses the same array, which
// keeps the last call's contents. Each call writes every partial entry that it
// reads before reading it, so nothing has to start at zero. Calls that overlap
// on the GPU (two streams, or two host threads with different streams) race on
// the array; calls on one stream run in order.
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

int fail(int status, const std::string& msg);
int cuda_status(cudaError_t e, const char* where);
int check_dtype(int dtype);

namespace {

constexpr int kNoallocMaxBitplanes = 64;
constexpr size_t kNoallocScratchDoubles = (size_t)kPartialSlots * (kNoallocMaxBitplanes + 1);

static __device__ __align__(256) double g_sq_scratch[kNoallocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// the scratch address on the current device: looked up on every call whose
// stream is not capturing, remembered for calls made during a capture
int scratch_on_current_device(cudaStream_t st, double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "prodm_collect_squared_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return fail(PRODM_EUNSUPPORTED, "prodm_collect_squared_noalloc: device index above 63");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return cuda_status(e, "prodm_collect_squared_noalloc: cudaStreamIsCapturing");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sq_scratch);
        if (e != cudaSuccess) return cuda_status(e, "prodm_collect_squared_noalloc: cudaGetSymbolAddress");
        g_scratch_ptr[dev] = (double*)p;
    } else if (!g_scratch_ptr[dev]) {
        return fail(PRODM_EINVAL, "prodm_collect_squared_noalloc: first call on this device made during a stream "
                                  "capture (call it once before capturing)");
    }
    *out = g_scratch_ptr[dev];
    return PRODM_OK;
}

}  // namespace
}  // namespace prodm

using namespace prodm;

extern "C" int prodm_collect_squared_noalloc(int dtype, const void* d, uint64_t n, int B, double maxv, double* out,
                                             void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!d || !out) return fail(PRODM_EINVAL, "prodm_collect_squared_noalloc: NULL pointer");
    const int maxB = dtype == PRODM_F64 ? kNoallocMaxBitplanes : 32;
    if (B < 1 || B > maxB)
        return fail(PRODM_EINVAL, "prodm_collect_squared_noalloc: num_bitplanes must be in [1, " +
                                      std::to_string(maxB) + "] (fixed scratch of " +
                                      std::to_string(kNoallocScratchDoubles * sizeof(double)) + " bytes)");
    cudaStream_t st = (cudaStream_t)stream;
    double* partial = nullptr;
    if ((rc = scratch_on_current_device(st, &partial))) return rc;
    if (dtype == PRODM_F64) return launch_sq_collect<double>((const double*)d, n, B, maxv, partial, out, st);
    return launch_sq_collect<float>((const float*)d, n, B, (float)maxv, partial, out, st);
}
