// dcpse_rk4.cu -- classic RK4 for two-species reaction-diffusion with a
// DC-PSE Laplacian (the Gray-Scott system), forward and adjoint stages.
//
// Replaces the reference's pattern of boost::numeric::odeint::runge_kutta4
// over openfpm state types with the DC-PSE Laplacian evaluated on the host
// every stage (src/OdeIntegrators/tests/OdeIntegratores_base_tests.cpp:33-72,
// 478-577; GPU algebra for_each*_ker in vector_algebra_ofp_gpu.hpp:13-190).
// Here one kernel per stage does the two Laplacian gathers (one weight
// stream, both species), the reaction terms and the RK4 stage update:
//   du = Du L u - u v^2 + F (1 - u),   dv = Dv L v + u v^2 - (F + k) v
//   Y1 = y; Y2 = y + dt/2 k1; Y3 = y + dt/2 k2; Y4 = y + dt k3;
//   y' = y + dt/6 (k1 + 2 k2 + 2 k3 + k4).
// The adjoint stage computes J(Y)^T kbar with L^T through the transposed
// neighbour list:
//   ubar = Du L^T kbar_u - (v^2 + F) kbar_u + v^2 kbar_v
//   vbar = Dv L^T kbar_v - 2 u v kbar_u + (2 u v - F - k) kbar_v
// and the reverse RK4 recursion
//   kbar4 = dt/6 ybar; Ybar4 = J4^T kbar4; kbar3 = dt/3 ybar + dt Ybar4;
//   Ybar3 = J3^T kbar3; kbar2 = dt/3 ybar + dt/2 Ybar3; Ybar2 = J2^T kbar2;
//   kbar1 = dt/6 ybar + dt/2 Ybar2; Ybar1 = J1^T kbar1;
//   ybar_n = ybar + Ybar1 + Ybar2 + Ybar3 + Ybar4.
#include <type_traits>

#include "dcpse_internal.h"

namespace dcpse {
namespace {

template <typename T>
__device__ __forceinline__ T tfma(T a, T b, T c);
template <>
__device__ __forceinline__ float tfma<float>(float a, float b, float c) {
    return fmaf(a, b, c);
}
template <>
__device__ __forceinline__ double tfma<double>(double a, double b, double c) {
    return fma(a, b, c);
}

// the two species of the stage input side by side, so a neighbour's pair
// is one 8-byte (FP32) or 16-byte (FP64) gather instead of two
template <typename T>
struct Pair;
template <>
struct Pair<float> {
    typedef float2 type;
};
template <>
struct Pair<double> {
    typedef double2 type;
};

template <typename T>
__global__ void pack_kernel(const T* __restrict__ u, const T* __restrict__ v, int64_t n,
                            typename Pair<T>::type* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        typename Pair<T>::type p;
        p.x = u[i];
        p.y = v[i];
        out[i] = p;
    }
}

// reaction terms and the RK4 stage combination of one row, given its
// Laplacian sums lu, lv and its stage input (up, vp)
template <typename T>
__device__ __forceinline__ void stage_update(const RkArgs<T>& a, int64_t row, T up, T vp, T lu, T lv) {
    const T uvv = up * vp * vp;
    const T ku = (T)a.Du * lu - uvv + (T)a.F * ((T)1 - up);
    const T kv = (T)a.Dv * lv + uvv - ((T)a.F + (T)a.K) * vp;
    const T dt = (T)a.dt;
    const T y0u = a.y0u[row], y0v = a.y0v[row];
    switch (a.stage) {
        case 0:
            a.accu[row] = ku;
            a.accv[row] = kv;
            a.outu[row] = y0u + (dt / (T)2) * ku;
            a.outv[row] = y0v + (dt / (T)2) * kv;
            break;
        case 1:
            a.accu[row] += (T)2 * ku;
            a.accv[row] += (T)2 * kv;
            a.outu[row] = y0u + (dt / (T)2) * ku;
            a.outv[row] = y0v + (dt / (T)2) * kv;
            break;
        case 2:
            a.accu[row] += (T)2 * ku;
            a.accv[row] += (T)2 * kv;
            a.outu[row] = y0u + dt * ku;
            a.outv[row] = y0v + dt * kv;
            break;
        default:
            a.outu[row] = y0u + (dt / (T)6) * (a.accu[row] + ku);
            a.outv[row] = y0v + (dt / (T)6) * (a.accv[row] + kv);
            break;
    }
}

template <typename T, int G>
__global__ void __launch_bounds__(256) gs_stage_kernel(RkArgs<T> a) {
    typedef typename Pair<T>::type P2;
    const P2* __restrict__ Y2 = static_cast<const P2*>(a.pack);
    const int lane = threadIdx.x & 31;
    const int sub = lane & (G - 1);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / G;
    const int64_t first = (tid - lane) / G;
    for (int64_t base = first; base < a.n; base += rows_per_pass) {
        const int64_t row = base + lane / G;
        T lu = 0, lv = 0;
        T up = 0, vp = 0;
        if (row < a.n) {
            up = a.Yu[row];
            vp = a.Yv[row];
            const int64_t rb = a.rowptr[row];
            const int k = (int)(a.rowptr[row + 1] - rb);
            const int32_t* __restrict__ c = a.cols + rb;
            const T* __restrict__ w = a.w + rb;
            // U entries per lane in flight: every load of a batch is issued
            // before its arithmetic; entries past the row end gather the row's
            // own values with weight 0
            constexpr int U = 4;
            for (int j0 = sub; j0 < k; j0 += G * U) {
                int32_t q[U];
                T wq[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = j0 + u * G;
                    q[u] = j < k ? c[j] : (int32_t)row;
                    wq[u] = j < k ? w[j] : (T)0;
                }
                P2 y[U];
#pragma unroll
                for (int u = 0; u < U; ++u) y[u] = Y2[q[u]];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    lu = tfma<T>(wq[u], y[u].x - up, lu);
                    lv = tfma<T>(wq[u], y[u].y - vp, lv);
                }
            }
        }
#pragma unroll
        for (int m = G / 2; m > 0; m >>= 1) {
            lu += __shfl_xor_sync(0xffffffffu, lu, m);
            lv += __shfl_xor_sync(0xffffffffu, lv, m);
        }
        if (row < a.n && sub == 0) stage_update(a, row, up, vp, lu, lv);
    }
}

// FP32 stage on the sliced ELL layout of the weights (slices of 32 rows
// stored entry-major, rows sorted by length within windows of 256): a row per
// thread, 8 gathers of (u, v) pairs in flight; entries past the slice end
// take the row's own pair with weight 0 (an exact zero)
__global__ void __launch_bounds__(256) gs_stage_sell_kernel(RkArgs<float> a, int64_t nwin) {
    const float2* __restrict__ Y2 = static_cast<const float2*>(a.pack);
    const int lane = threadIdx.x & 31;
    constexpr int U = 8;
    for (int64_t win = blockIdx.x; win < nwin; win += gridDim.x) {
        const int64_t s = win * 8 + (threadIdx.x >> 5);
        const int32_t row = a.srow[s * 32 + lane];
        if (row < 0) continue;
        const int64_t b = a.soff[s];
        const int L = (int)((a.soff[s + 1] - b) / 32);
        const float2 yp = Y2[row];
        const int32_t* __restrict__ c = a.scols + b + lane;
        const float* __restrict__ w = a.sw + b + lane;
        float lu = 0.f, lv = 0.f;
        // the column stream runs one chunk ahead of the gathers
        int32_t qn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) qn[u] = u < L ? c[(int64_t)u * 32] : 0;
        for (int j0 = 0; j0 < L; j0 += U) {
            float2 y[U];
#pragma unroll
            for (int u = 0; u < U; ++u) y[u] = j0 + u < L ? Y2[qn[u]] : yp;
            float wq[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + u;
                qn[u] = j + U < L ? c[(int64_t)(j + U) * 32] : 0;
                wq[u] = j < L ? w[(int64_t)j * 32] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                lu = fmaf(wq[u], y[u].x - yp.x, lu);
                lv = fmaf(wq[u], y[u].y - yp.y, lv);
            }
        }
        stage_update(a, row, yp.x, yp.y, lu, lv);
    }
}

// the end of an adjoint stage for row p, from the gathered lu = (W^T kbar_u)_p
// and lv: Ybar of the stage, the accumulator, and the next stage's kbar
template <typename T>
__device__ __forceinline__ void adj_finish(const RkAdjArgs<T>& a, int64_t p, T lu, T lv) {
    typedef typename Pair<T>::type P2;
    T kbu, kbv;
    if (a.kb_packed) {
        const P2 kb = static_cast<const P2*>(a.pack)[p];
        kbu = kb.x;
        kbv = kb.y;
    } else {
        kbu = a.kbu[p];
        kbv = a.kbv[p];
    }
    lu = lu - a.rs[p] * kbu;
    lv = lv - a.rs[p] * kbv;
    const T u = a.Yu[p], v = a.Yv[p];
    const T Ybu = (T)a.Du * lu - (v * v + (T)a.F) * kbu + v * v * kbv;
    const T Ybv = (T)a.Dv * lv - (T)2 * u * v * kbu + ((T)2 * u * v - (T)a.F - (T)a.K) * kbv;
    if (a.acc_mode == 2) {
        a.yb_out_u[p] = a.accu[p] + Ybu;
        a.yb_out_v[p] = a.accv[p] + Ybv;
    } else if (a.acc_mode == 1) {
        a.accu[p] = a.ybu[p] + Ybu;
        a.accv[p] = a.ybv[p] + Ybv;
    } else {
        a.accu[p] += Ybu;
        a.accv[p] += Ybv;
    }
    if (a.pack_out) {
        P2 nx;
        nx.x = (T)a.cy * a.ybu[p] + (T)a.cY * Ybu;
        nx.y = (T)a.cy * a.ybv[p] + (T)a.cY * Ybv;
        static_cast<P2*>(a.pack_out)[p] = nx;
    } else if (a.next_u) {
        a.next_u[p] = (T)a.cy * a.ybu[p] + (T)a.cY * Ybu;
        a.next_v[p] = (T)a.cy * a.ybv[p] + (T)a.cY * Ybv;
    }
}

// adjoint stage: G lanes per particle over its transposed row, kbar of the
// stage gathered as packed (u, v) pairs in 4-deep batches
template <typename T, int G>
__global__ void __launch_bounds__(256) gs_adjoint_kernel(RkAdjArgs<T> a) {
    typedef typename Pair<T>::type P2;
    const P2* __restrict__ KB = static_cast<const P2*>(a.pack);
    const int lane = threadIdx.x & 31;
    const int sub = lane & (G - 1);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / G;
    const int64_t first = (tid - lane) / G;
    for (int64_t base = first; base < a.n; base += rows_per_pass) {
        const int64_t row = base + lane / G;
        T lu = 0, lv = 0;
        if (row < a.n) {
            const int64_t rb = a.trow[row];
            const int k = (int)(a.trow[row + 1] - rb);
            const int32_t* __restrict__ c = a.tsrc + rb;
            const T* __restrict__ w = a.wT + rb;
            constexpr int U = 4;
            for (int j0 = sub; j0 < k; j0 += G * U) {
                int32_t q[U];
                T wq[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = j0 + u * G;
                    q[u] = j < k ? c[j] : (int32_t)row;
                    wq[u] = j < k ? w[j] : (T)0;
                }
                P2 y[U];
#pragma unroll
                for (int u = 0; u < U; ++u) y[u] = KB[q[u]];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    lu = tfma<T>(wq[u], y[u].x, lu);
                    lv = tfma<T>(wq[u], y[u].y, lv);
                }
            }
        }
#pragma unroll
        for (int m = G / 2; m > 0; m >>= 1) {
            lu += __shfl_xor_sync(0xffffffffu, lu, m);
            lv += __shfl_xor_sync(0xffffffffu, lv, m);
        }
        if (row < a.n && sub == 0) adj_finish<T>(a, row, lu, lv);
    }
}

// FP32 adjoint stage on the sliced ELL layout of the transposed weights: a
// row per thread, 8 gathers of (kbar_u, kbar_v) pairs in flight; entries past
// the slice end add the row's own pair with weight 0 (an exact zero)
__global__ void __launch_bounds__(256) gs_adjoint_sell_kernel(RkAdjArgs<float> a, int64_t nwin) {
    const float2* __restrict__ KB = static_cast<const float2*>(a.pack);
    const int lane = threadIdx.x & 31;
    constexpr int U = 8;
    for (int64_t win = blockIdx.x; win < nwin; win += gridDim.x) {
        const int64_t s = win * 8 + (threadIdx.x >> 5);
        const int32_t p = a.srow[s * 32 + lane];
        if (p < 0) continue;
        const int64_t b = a.soff[s];
        const int L = (int)((a.soff[s + 1] - b) / 32);
        const int32_t* __restrict__ c = a.scols + b + lane;
        const float* __restrict__ w = a.sw + b + lane;
        float lu = 0.f, lv = 0.f;
        // the column stream runs one chunk ahead of the gathers
        int32_t qn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) qn[u] = u < L ? c[(int64_t)u * 32] : p;
        for (int j0 = 0; j0 < L; j0 += U) {
            float2 y[U];
#pragma unroll
            for (int u = 0; u < U; ++u) y[u] = KB[qn[u]];
            float wq[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = j0 + u;
                qn[u] = j + U < L ? c[(int64_t)(j + U) * 32] : p;
                wq[u] = j < L ? w[(int64_t)j * 32] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                lu = fmaf(wq[u], y[u].x, lu);
                lv = fmaf(wq[u], y[u].y, lv);
            }
        }
        adj_finish<float>(a, p, lu, lv);
    }
}

template <typename T>
__global__ void gather_kernel(const int64_t* __restrict__ tidx, int64_t nnz, const T* __restrict__ w,
                              T* __restrict__ wT) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz; t += (int64_t)gridDim.x * blockDim.x)
        wT[t] = w[tidx[t]];
}

template <typename T>
__global__ void rowsum_t_kernel(const int64_t* __restrict__ rowptr, int64_t n, const T* __restrict__ w,
                                T* __restrict__ rs) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        T s = 0;
        for (int64_t j = rowptr[p]; j < rowptr[p + 1]; ++j) s += w[j];
        rs[p] = s;
    }
}

int grid_n(int64_t items, int per_block) {
    int64_t g = (items + per_block - 1) / per_block, cap = (int64_t)num_sms() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

template <typename T>
cudaError_t rk_stage(const RkArgs<T>& a, int lanes, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    pack_kernel<T><<<grid_n(a.n, 256), 256, 0, s>>>(a.Yu, a.Yv, a.n, static_cast<typename Pair<T>::type*>(a.pack));
    if constexpr (std::is_same<T, float>::value) {
        if (a.srow) {
            const int64_t nwin = (a.n + 255) / 256;
            gs_stage_sell_kernel<<<(unsigned)nwin, 256, 0, s>>>(a, nwin);
            return cudaGetLastError();
        }
    }
    switch (lanes) {
        case 4: gs_stage_kernel<T, 4><<<grid_n(a.n, 64), 256, 0, s>>>(a); break;
        case 8: gs_stage_kernel<T, 8><<<grid_n(a.n, 32), 256, 0, s>>>(a); break;
        case 16: gs_stage_kernel<T, 16><<<grid_n(a.n, 16), 256, 0, s>>>(a); break;
        default: gs_stage_kernel<T, 32><<<grid_n(a.n, 8), 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

template <typename T>
__global__ void pack_scaled_kernel(const T* __restrict__ u, const T* __restrict__ v, int64_t n, T scale,
                                   typename Pair<T>::type* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        typename Pair<T>::type p;
        p.x = u[i] * scale;
        p.y = v[i] * scale;
        out[i] = p;
    }
}

template <typename T>
cudaError_t rk_pack_scaled(const T* ybu, const T* ybv, int64_t n, double scale, void* pack, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    pack_scaled_kernel<T><<<grid_n(n, 256), 256, 0, s>>>(ybu, ybv, n, (T)scale,
                                                          static_cast<typename Pair<T>::type*>(pack));
    return cudaGetLastError();
}

template <typename T>
cudaError_t rk_adjoint_stage(const RkAdjArgs<T>& a, int lanes, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    // the stage's kbar as pairs (already so in a fused reverse step)
    if (!a.kb_packed)
        pack_kernel<T><<<grid_n(a.n, 256), 256, 0, s>>>(a.kbu, a.kbv, a.n, static_cast<typename Pair<T>::type*>(a.pack));
    if constexpr (std::is_same<T, float>::value) {
        if (a.srow) {
            const int64_t nwin = (a.n + 255) / 256;
            gs_adjoint_sell_kernel<<<(unsigned)nwin, 256, 0, s>>>(a, nwin);
            return cudaGetLastError();
        }
    }
    switch (lanes) {
        case 4: gs_adjoint_kernel<T, 4><<<grid_n(a.n, 64), 256, 0, s>>>(a); break;
        case 8: gs_adjoint_kernel<T, 8><<<grid_n(a.n, 32), 256, 0, s>>>(a); break;
        case 16: gs_adjoint_kernel<T, 16><<<grid_n(a.n, 16), 256, 0, s>>>(a); break;
        default: gs_adjoint_kernel<T, 32><<<grid_n(a.n, 8), 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t rk_transpose_weights(const int64_t* rowptr, const int64_t* tidx, int64_t n, int64_t nnz, const T* w,
                                 T* wT, T* rs, cudaStream_t s) {
    if (nnz > 0) gather_kernel<T><<<grid_n(nnz, 256), 256, 0, s>>>(tidx, nnz, w, wT);
    if (n > 0) rowsum_t_kernel<T><<<grid_n(n, 256), 256, 0, s>>>(rowptr, n, w, rs);
    return cudaGetLastError();
}

template cudaError_t rk_stage<float>(const RkArgs<float>&, int, cudaStream_t);
template cudaError_t rk_stage<double>(const RkArgs<double>&, int, cudaStream_t);
template cudaError_t rk_adjoint_stage<float>(const RkAdjArgs<float>&, int, cudaStream_t);
template cudaError_t rk_adjoint_stage<double>(const RkAdjArgs<double>&, int, cudaStream_t);
template cudaError_t rk_pack_scaled<float>(const float*, const float*, int64_t, double, void*, cudaStream_t);
template cudaError_t rk_pack_scaled<double>(const double*, const double*, int64_t, double, void*, cudaStream_t);
template cudaError_t rk_transpose_weights<float>(const int64_t*, const int64_t*, int64_t, int64_t, const float*,
                                                 float*, float*, cudaStream_t);
template cudaError_t rk_transpose_weights<double>(const int64_t*, const int64_t*, int64_t, int64_t, const double*,
                                                  double*, double*, cudaStream_t);

}  // namespace dcpse
