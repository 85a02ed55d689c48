// dcpse_calibrate.cu -- measured FP64 fused multiply-add throughput of the
// current GPU, the ceiling against which the FP64 assembly is reported.
//
// Every thread runs 8 independent FMA chains (enough to cover the pipe
// latency) for a fixed number of iterations; the result is written out so
// the work cannot be removed.  Timed with CUDA events on the given stream.
#include "dcpse_internal.h"

namespace {

__global__ void __launch_bounds__(256) fp64_fma_kernel(double seed, int iters, double* out) {
    double a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = seed + 1e-3 * (threadIdx.x + i);
    const double m = 0.999999, c = 1e-7;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = fma(a[i], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == -1.0) out[blockIdx.x] = s;  // never true; keeps the chains alive
}

}  // namespace

extern "C" int dcpse_measure_fp64_peak(void* stream, double* tflops) {
    if (!tflops) return dcpse::set_error(DCPSE_ERR_ARG, "NULL output");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int blocks = dcpse::num_sms() * 8, threads = 256, iters = 4096;
    double* out = nullptr;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) return dcpse::set_error(DCPSE_ERR_CUDA, cudaGetErrorString(e));
    fp64_fma_kernel<<<blocks, threads, 0, s>>>(1.0, iters / 8, out);  // warm-up
    cudaEventRecord(e0, s);
    fp64_fma_kernel<<<blocks, threads, 0, s>>>(1.0, iters, out);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return dcpse::set_error(DCPSE_ERR_CUDA, cudaGetErrorString(e));
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return DCPSE_OK;
}
