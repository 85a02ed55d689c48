// dcpse_apply.cu -- DC-PSE operator application on the device.
//
// Replaces Dcpse::computeDifferentialOperator (src/DCPSE/Dcpse.hpp:467-499,
// 560-603) and the host loop that evaluates `getV<j>(parts) = Op(getV<i>())`
// particle by particle (src/Operators/Vector/cuda/vector_dist_operators_cuda.cuh
// :444-461; the reference evaluates DC-PSE nodes on the host only).
//
//  * apply_term_f64: one reference Dcpse object, FP64, in the reference's
//    order  Df_p = (sum_q (f_q + s f_p) K_pq) * eps_p^-|alpha|.  Compiled with
//    -fmad=false, so it matches the CPU oracle bit for bit.
//  * apply_batched_{f32,f64}: every output of a plan in one pass over the
//    neighbour list, with eps^-|alpha| folded into the weights and the
//    difference form  Df_p = sum_q w_pq (f_q - f_p)  (equal to the reference
//    formula because the kernels of even |alpha| annihilate constants by
//    construction and those of odd |alpha| sum to zero by the moment
//    condition on the constant monomial).  G lanes share a row; each lane
//    streams G-strided neighbour entries, the G partial sums are combined by
//    shuffles.  The FP32 path reads f as an exact (hi, lo) float pair so that
//    f_q - f_p keeps full FP32 relative accuracy.
#include "dcpse_internal.h"

namespace dcpse {
namespace {

__global__ void __launch_bounds__(256) apply_term_f64_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                             const int32_t* __restrict__ cols,
                                                             const double* __restrict__ K,
                                                             const double* __restrict__ eip, double sign,
                                                             const double* __restrict__ f, double* __restrict__ out,
                                                             int accumulate) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const double fxp = sign * f[p];
        double D = 0.0;
        const int64_t e = rowptr[p + 1];
        for (int64_t j = rowptr[p]; j < e; ++j) D = D + (f[cols[j]] + fxp) * K[j];
        D = D * eip[p];
        out[p] = accumulate ? out[p] + D : D;
    }
}

__global__ void split_kernel(const double* __restrict__ f, int64_t n, float2* __restrict__ f2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = f[i];
        float hi = (float)v;
        float lo = (float)(v - (double)hi);
        f2[i] = make_float2(hi, lo);
    }
}

template <int G, int NO>
__global__ void __launch_bounds__(256) apply_f32_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ cols,
                                                        const float* __restrict__ w, int64_t nnz,
                                                        const float2* __restrict__ f2, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int sub = lane & (G - 1);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / G;
    // every lane of a warp runs the same number of passes (shuffles below)
    const int64_t first = (tid - lane) / G;
    for (int64_t base = first; base < n; base += rows_per_pass) {
        const int64_t row = base + lane / G;
        float acc[NO];
#pragma unroll
        for (int o = 0; o < NO; ++o) acc[o] = 0.0f;
        if (row < n) {
            const float2 fp = f2[row];
            const int64_t e = rowptr[row + 1];
            for (int64_t j = rowptr[row] + sub; j < e; j += G) {
                const float2 fq = f2[cols[j]];
                const float d = (fq.x - fp.x) + (fq.y - fp.y);
#pragma unroll
                for (int o = 0; o < NO; ++o) acc[o] = fmaf(w[(int64_t)o * nnz + j], d, acc[o]);
            }
        }
#pragma unroll
        for (int o = 0; o < NO; ++o) {
#pragma unroll
            for (int s = G / 2; s > 0; s >>= 1) acc[o] += __shfl_xor_sync(0xffffffffu, acc[o], s);
        }
        if (row < n) {
#pragma unroll
            for (int o = 0; o < NO; ++o)
                if (sub == (o & (G - 1))) out[(int64_t)o * n + row] = (double)acc[o];
        }
    }
}

template <int G, int NO>
__global__ void __launch_bounds__(256) apply_f64_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ cols,
                                                        const double* __restrict__ w, int64_t nnz,
                                                        const double* __restrict__ f, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int sub = lane & (G - 1);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / G;
    const int64_t first = (tid - lane) / G;
    for (int64_t base = first; base < n; base += rows_per_pass) {
        const int64_t row = base + lane / G;
        double acc[NO];
#pragma unroll
        for (int o = 0; o < NO; ++o) acc[o] = 0.0;
        if (row < n) {
            const double fp = f[row];
            const int64_t e = rowptr[row + 1];
            for (int64_t j = rowptr[row] + sub; j < e; j += G) {
                const double d = f[cols[j]] - fp;
#pragma unroll
                for (int o = 0; o < NO; ++o) acc[o] = fma(w[(int64_t)o * nnz + j], d, acc[o]);
            }
        }
#pragma unroll
        for (int o = 0; o < NO; ++o) {
#pragma unroll
            for (int s = G / 2; s > 0; s >>= 1) acc[o] += __shfl_xor_sync(0xffffffffu, acc[o], s);
        }
        if (row < n) {
#pragma unroll
            for (int o = 0; o < NO; ++o)
                if (sub == (o & (G - 1))) out[(int64_t)o * n + row] = acc[o];
        }
    }
}

int grid_rows(int64_t rows, int rows_per_block) {
    int64_t g = (rows + rows_per_block - 1) / rows_per_block;
    int64_t cap = (int64_t)num_sms() * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

template <int G, typename W, typename F>
cudaError_t launch_batched(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const W* w, int64_t nnz,
                           const F* f, double* out, cudaStream_t s) {
    const int grid = grid_rows(n, 256 / G);
#define DCPSE_CASE(NO)                                                                        \
    case NO:                                                                                  \
        if constexpr (sizeof(W) == 4)                                                         \
            apply_f32_kernel<G, NO><<<grid, 256, 0, s>>>(n, rowptr, cols, (const float*)w, nnz, \
                                                         (const float2*)f, out);              \
        else                                                                                  \
            apply_f64_kernel<G, NO><<<grid, 256, 0, s>>>(n, rowptr, cols, (const double*)w, nnz, \
                                                         (const double*)f, out);              \
        break;
    switch (nout) {
        DCPSE_CASE(1)
        DCPSE_CASE(2)
        DCPSE_CASE(3)
        DCPSE_CASE(4)
        DCPSE_CASE(5)
        DCPSE_CASE(6)
        DCPSE_CASE(7)
        DCPSE_CASE(8)
        default:
            return cudaErrorInvalidValue;
    }
#undef DCPSE_CASE
    return cudaGetLastError();
}

int lanes_for(int64_t n, int64_t nnz) {
    double avg = n > 0 ? (double)nnz / (double)n : 0.0;
    if (avg <= 24.0) return 8;
    if (avg <= 96.0) return 16;
    return 32;
}

}  // namespace

cudaError_t apply_term_f64(int64_t n, const int64_t* rowptr, const int32_t* cols, const double* K, const double* eip,
                           unsigned ord, const double* f, double* out, int accumulate, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const double sign = (ord % 2 == 0) ? -1.0 : 1.0;
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)num_sms() * 8;
    apply_term_f64_kernel<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(n, rowptr, cols, K, eip, sign, f, out,
                                                                         accumulate);
    return cudaGetLastError();
}

cudaError_t split_f64(const double* f, int64_t n, float2* f2, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)num_sms() * 8;
    split_kernel<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(f, n, f2);
    return cudaGetLastError();
}

cudaError_t apply_batched_f32(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const float* w,
                              int64_t nnz, const float2* f2, double* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    switch (lanes_for(n, nnz)) {
        case 8: return launch_batched<8>(n, nout, rowptr, cols, w, nnz, f2, out, s);
        case 16: return launch_batched<16>(n, nout, rowptr, cols, w, nnz, f2, out, s);
        default: return launch_batched<32>(n, nout, rowptr, cols, w, nnz, f2, out, s);
    }
}

cudaError_t apply_batched_f64(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const double* w,
                              int64_t nnz, const double* f, double* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    switch (lanes_for(n, nnz)) {
        case 8: return launch_batched<8>(n, nout, rowptr, cols, w, nnz, f, out, s);
        case 16: return launch_batched<16>(n, nout, rowptr, cols, w, nnz, f, out, s);
        default: return launch_batched<32>(n, nout, rowptr, cols, w, nnz, f, out, s);
    }
}

}  // namespace dcpse
