// dcpse_surface.cu -- surface DC-PSE: normal extension of the support set and
// accumulation of the virtual particles' kernels onto the surface particles.
//
// Replaces SurfaceDcpse::createNormalParticles (src/DCPSE/Dcpse.hpp:855-876,
// positions appended to the support set on the host) and
// SurfaceDcpse::accumulateAndDeleteNormalParticles (Dcpse.hpp:947-1015, a
// host loop with a hash map per particle).  The assembly in between is the
// ordinary one, run on the extended support.
//
// Extended support: the nb base particles, then for every base particle p
// and i = 1..n_count the two virtual particles x_p + (i s_p) n_p and
// x_p - (i s_p) n_p, so virtual particle v belongs to base particle
// (v - nb) / (2 n_count).
//
// Accumulation: one thread per domain row walks the row in list order; a
// base particle met for the first time opens the next slot of the new row
// with the entry's value, later entries of the same base particle are added
// to that slot in list order (the reference's map lookup + "+=").
#include <cuda_bf16.h>

#include "dcpse_internal.h"

namespace dcpse {
namespace {

__global__ void extend_kernel(int dim, const double* __restrict__ base, const double* __restrict__ normals, int64_t nb,
                              int n_count, double spacing, const double* __restrict__ spacings,
                              double* __restrict__ out) {
    const int64_t total = nb * n_count;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t / n_count;
        const int i = (int)(t - p * n_count) + 1;
        const double s = spacings ? spacings[p] : spacing;
        const double is = (double)i * s;
        const int64_t v = nb + p * 2 * n_count + 2 * (i - 1);
        for (int j = 0; j < dim; ++j) {
            const double x = base[p * dim + j];
            const double d = is * normals[p * dim + j];
            out[v * dim + j] = x + d;
            out[(v + 1) * dim + j] = x - d;
        }
    }
}

__device__ __forceinline__ int64_t base_of(int64_t q, int64_t nb, int n_count) {
    return q < nb ? q : (q - nb) / (2 * (int64_t)n_count);
}

__global__ void acc_count_kernel(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ cols, int64_t n,
                                 int64_t nb, int n_count, int32_t* __restrict__ counts) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = rowptr[p], e = rowptr[p + 1];
        int32_t c = 0;
        for (int64_t j = b; j < e; ++j) {
            const int64_t r = base_of(cols[j], nb, n_count);
            bool first = true;
            for (int64_t i = b; i < j && first; ++i) first = base_of(cols[i], nb, n_count) != r;
            c += first ? 1 : 0;
        }
        counts[p] = c;
    }
}

__global__ void acc_fill_kernel(SurfAcc a) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.n; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = a.rowptr[p], e = a.rowptr[p + 1];
        const int64_t o = a.out_rowptr[p];
        int64_t used = 0;
        for (int64_t j = b; j < e; ++j) {
            const int32_t r = (int32_t)base_of(a.cols[j], a.nb, a.n_count);
            int64_t slot = -1;
            for (int64_t s = 0; s < used && slot < 0; ++s)
                if (a.out_cols[o + s] == r) slot = s;
            if (slot < 0) {
                slot = used++;
                a.out_cols[o + slot] = r;
                for (int t = 0; t < a.nst; ++t) a.out[t][o + slot] = a.in[t][j];
            } else {
                for (int t = 0; t < a.nst; ++t) a.out[t][o + slot] = a.out[t][o + slot] + a.in[t][j];
            }
        }
    }
}

__global__ void narrow_kernel(const double* __restrict__ w64, int64_t m, float* __restrict__ w32, void* r16,
                              float* __restrict__ r32) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const double w = w64[i];
        const float f = (float)w;
        w32[i] = f;
        if (r16) reinterpret_cast<__nv_bfloat16*>(r16)[i] = __float2bfloat16_rn((float)(w - (double)f));
        if (r32) r32[i] = (float)(w - (double)f);
    }
}

int grid_of(int64_t n) {
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

cudaError_t surface_extend(int dim, const double* base, const double* normals, int64_t nb, int n_count, double spacing,
                           const double* spacings, double* out, cudaStream_t s) {
    if (nb == 0) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(out, base, sizeof(double) * nb * dim, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess || n_count < 1) return e;
    extend_kernel<<<grid_of(nb * n_count), 256, 0, s>>>(dim, base, normals, nb, n_count, spacing, spacings, out);
    return cudaGetLastError();
}

cudaError_t surface_count(const int64_t* rowptr, const int32_t* cols, int64_t n, int64_t nb, int n_count,
                          int32_t* counts, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    acc_count_kernel<<<grid_of(n), 256, 0, s>>>(rowptr, cols, n, nb, n_count, counts);
    return cudaGetLastError();
}

cudaError_t surface_fill(const SurfAcc& a, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    acc_fill_kernel<<<grid_of(a.n), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t narrow_weights(const double* w64, int64_t m, float* w32, void* r16, cudaStream_t s, float* r32) {
    if (m == 0) return cudaSuccess;
    narrow_kernel<<<grid_of(m), 256, 0, s>>>(w64, m, w32, r16, r32);
    return cudaGetLastError();
}

}  // namespace dcpse
