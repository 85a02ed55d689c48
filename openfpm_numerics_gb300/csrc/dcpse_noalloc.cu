// dcpse_noalloc.cu -- the batched FP32 apply without any device allocation.
//
// Who needs this: code that runs where cudaMalloc is off limits -- inside a
// custom allocator or memory-pool callback, in a real-time loop that must
// never block on the driver's allocator, or in a process whose device memory
// is entirely handed out by another framework.  (A host function enqueued
// with cudaLaunchHostFunc may make no CUDA call at all, so it cannot call
// this either: enqueue the call from ordinary host code on the stream.)
// Such callers already own the neighbour list, the FP32 output weights, the
// field and the output buffers (all device memory); the only extra memory
// the FP32 apply needs is the (hi, lo) split of the field, and that lives
// here in a fixed file-scope device array.
//
// Cost and limit: the array (kNoAllocMaxParticles x 8 bytes = 16 MiB) is
// part of this library's device code, so the CUDA runtime places it on a GPU
// when it loads the library's module there: with lazy module loading (the
// default since CUDA 12) that is the first call on that device, and the
// memory stays until the process exits.  The kernels the call launches are
// loaded the same way, at their first launch.  A call with n = 0 does that
// set-up (the array and every kernel this entry point may launch) and
// nothing else; make it once per device at start-up, before any callback or
// stream capture.  A call accepts at most kNoAllocMaxParticles particles.
// The device address is cached per device: after cudaDeviceReset the cache
// is stale, so this entry point must not be used after a reset.
#include <mutex>

#include "dcpse_internal.h"

static_assert(DCPSE_NOALLOC_MAX_PARTICLES == (1 << 21), "keep the header's limit in step");

namespace {

constexpr int64_t kNoAllocMaxParticles = DCPSE_NOALLOC_MAX_PARTICLES;  // 2,097,152 particles

// The split field of the FP32 apply (overwritten in full by every call, so
// nothing in it needs to start at zero).
__device__ __align__(256) float2 g_noalloc_field[kNoAllocMaxParticles];

constexpr int kMaxDevices = 64;
float2* g_field_ptr[kMaxDevices] = {};
std::mutex g_field_mu;

// Device address of g_noalloc_field on the current device, resolved once per
// device with cudaGetSymbolAddress (in host code the symbol itself is only a
// host-side stand-in and must not be passed to a kernel).
cudaError_t field_scratch(float2** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_field_mu);
    if (!g_field_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_field);
        if (e != cudaSuccess) return e;
        g_field_ptr[dev] = static_cast<float2*>(p);
    }
    *out = g_field_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" {

int dcpse_apply_batched_f32_noalloc(int64_t n, int n_outputs, const int64_t* d_rowptr, const int32_t* d_cols,
                                    const float* d_w, int64_t w_stride, const double* d_f, double* d_out,
                                    void* stream) {
    if (n < 0) return dcpse::set_error(DCPSE_ERR_ARG, "n must be >= 0");
    if (n > kNoAllocMaxParticles)
        return dcpse::set_error(DCPSE_ERR_CAPACITY,
                                "dcpse_apply_batched_f32_noalloc: more particles than its fixed scratch holds "
                                "(DCPSE_NOALLOC_MAX_PARTICLES = 2097152)");
    if (n_outputs < 1 || n_outputs > dcpse::kMaxOutputs) return dcpse::set_error(DCPSE_ERR_ARG, "1..8 outputs");
    // resolve the scratch first, so that an n = 0 call is the warm-up that
    // places the array on this device
    float2* f2 = nullptr;
    cudaError_t e = field_scratch(&f2);
    if (e == cudaSuccess && n == 0) e = dcpse::preload_apply_f32_direct();
    if (e != cudaSuccess) return dcpse::set_error(DCPSE_ERR_CUDA, cudaGetErrorString(e));
    if (n == 0) return DCPSE_OK;
    if (!d_rowptr || !d_cols || !d_w || !d_f || !d_out || w_stride < 0) return dcpse::set_error(DCPSE_ERR_ARG, "NULL array");
    if (n_outputs > 1 && w_stride == 0)
        return dcpse::set_error(DCPSE_ERR_ARG, "w_stride must be >= rowptr[n] with more than one output");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    e = dcpse::split_f64(d_f, n, f2, s);
    if (e == cudaSuccess) e = dcpse::apply_batched_f32(n, n_outputs, d_rowptr, d_cols, d_w, w_stride, f2, d_out, s);
    if (e != cudaSuccess) return dcpse::set_error(DCPSE_ERR_CUDA, cudaGetErrorString(e));
    return DCPSE_OK;
}

}  // extern "C"
