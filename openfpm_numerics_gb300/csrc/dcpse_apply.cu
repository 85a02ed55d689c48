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
//  * batched applies: every output of a plan in one pass over the neighbour
//    list, eps^-|alpha| folded into the weights, difference form
//    Df_p = sum_q w_pq (f_q - f_p)  (equal to the reference formula: kernels
//    of even |alpha| annihilate constants by construction, those of odd
//    |alpha| sum to zero by the moment condition on the constant monomial).
//    G lanes share a row; lane l takes entries l, l+G, l+2G, ...; the G
//    partial sums are combined by a shuffle tree.
//
// FP32 arithmetic of the batched apply: the field is an exact (hi, lo) float
// pair; f_q - f_p is formed exactly as dh + dl with TwoSum (Knuth); each
// product w*dh enters a compensated sum (TwoSum of the running sum and the
// product, plus the product's exact error from fmaf), so the result carries
// the FP32 weight rounding and little else.  An optional bf16 residual of
// every weight (w64 - w32) restores the weights to ~2^-33 relative.
//
// Two kernels implement it with the same per-lane order (identical results):
//  * apply_f32_kernel reads the CSR streams straight from global memory;
//  * apply_f32_tma_kernel stages each tile of rows' columns and weight
//    streams into shared memory with cp.async.bulk (TMA bulk copies)
//    completing on an mbarrier, several tiles in flight per CTA.
#include <cuda_bf16.h>

#include "dcpse_internal.h"
#include "dcpse_f32_row.cuh"

namespace dcpse {
namespace {

// ------------------------------------------------------------ FP64 term ---
// The thread-per-row FP64 kernels below are bound by the FP64 pipe, where a
// warp instruction costs the same with idle lanes: a warp whose rows differ
// in length runs every lane to its longest row.  Each block therefore takes
// a window of 256 consecutive rows (neighbourhoods that overlap, so gathers
// stay in L1) and hands them to its threads longest first: the 32 rows of a
// warp then have nearly equal lengths.  Which thread sums a row does not
// change the row's sum.  blockDim.x must be 256.
__device__ __forceinline__ int64_t row_by_length(int64_t base, int64_t n, const int64_t* __restrict__ rowptr,
                                                 int* s_len, int* s_row) {
    const int t = threadIdx.x;
    const int64_t p0 = base + t;
    const int len = p0 < n ? (int)(rowptr[p0 + 1] - rowptr[p0]) : -1;
    s_len[t] = len;
    __syncthreads();
    int rank = 0;  // longer rows first, ties in row order
    for (int j = 0; j < 256; ++j) {
        const int lj = s_len[j];
        rank += (lj > len) | ((lj == len) & (j < t));
    }
    s_row[rank] = t;
    __syncthreads();
    const int64_t p = base + s_row[t];
    __syncthreads();  // the next window rewrites s_len and s_row
    return p;         // >= n: no row for this thread
}

__global__ void __launch_bounds__(256) apply_term_f64_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                             const int32_t* __restrict__ cols,
                                                             const double* __restrict__ K,
                                                             const double* __restrict__ eip, double sign,
                                                             const double* __restrict__ f, double* __restrict__ out,
                                                             int accumulate) {
    __shared__ int s_len[256], s_row[256];
    for (int64_t base = (int64_t)blockIdx.x * 256; base < n; base += (int64_t)gridDim.x * 256) {
        const int64_t p = row_by_length(base, n, rowptr, s_len, s_row);
        if (p >= n) continue;
        const double fxp = sign * f[p];
        double D = 0.0;
        const int64_t e = rowptr[p + 1];
        int64_t j = rowptr[p];
        // 4 entries in flight: all loads of a batch are issued first, the
        // sum then takes them in row order
        for (; j + 4 <= e; j += 4) {
            int32_t q[4];
            double k[4], fq[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                q[u] = cols[j + u];
                k[u] = K[j + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) fq[u] = f[q[u]];
#pragma unroll
            for (int u = 0; u < 4; ++u) D = D + (fq[u] + fxp) * k[u];
        }
        for (; j < e; ++j) D = D + (f[cols[j]] + fxp) * K[j];
        D = D * eip[p];
        out[p] = accumulate ? out[p] + D : D;
    }
}

// Dcpse::p2p (Dcpse.hpp:198-297): Df_p = epsInvPow_p * (sum_q f_q K_pq) per
// component, f on the support set ([n_sup][ncomp]), out on the domain set.
__global__ void __launch_bounds__(256) p2p_f64_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ cols, const double* __restrict__ K,
                                                      const double* __restrict__ eip, int ncomp,
                                                      const double* __restrict__ f, double* __restrict__ out) {
    __shared__ int s_len[256], s_row[256];
    for (int64_t base = (int64_t)blockIdx.x * 256; base < n; base += (int64_t)gridDim.x * 256) {
        const int64_t p = row_by_length(base, n, rowptr, s_len, s_row);
        if (p >= n) continue;
        const int64_t b = rowptr[p], e = rowptr[p + 1];
        for (int c = 0; c < ncomp; ++c) {
            double D = 0.0;
            int64_t j = b;
            // 4 entries in flight, summed in row order
            for (; j + 4 <= e; j += 4) {
                int32_t q[4];
                double k[4], fq[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    q[u] = cols[j + u];
                    k[u] = K[j + u];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) fq[u] = f[(int64_t)q[u] * ncomp + c];
#pragma unroll
                for (int u = 0; u < 4; ++u) D = D + fq[u] * k[u];
            }
            for (; j < e; ++j) D = D + f[(int64_t)cols[j] * ncomp + c] * K[j];
            out[p * ncomp + c] = eip[p] * D;
        }
    }
}

__global__ void split_kernel(const double* __restrict__ f, int64_t n, int64_t stride, float2* __restrict__ f2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = f[i * stride];
        float hi = (float)v;
        float lo = (float)(v - (double)hi);
        f2[i] = make_float2(hi, lo);
    }
}

struct F32Args {
    int64_t n;
    const int64_t* rowptr;
    const int32_t* cols;
    const float* w;                 // [NO][ws]
    const __nv_bfloat16* r;         // [NO][ws] or null
    int64_t ws;                     // weight stream stride (elements)
    const float2* f2;
    double* out;                    // output o of row r at out[o * oos + r * ors]
    int64_t oos, ors;
    int64_t row0;                   // rows [row0, n) (direct kernel)
    uint32_t comp;                  // outputs that take the compensated sum
    int no_self;                    // interpolation: no f_p term, f2 indexed by the support set
};

// Neighbour entries of one lane, U at a time: all loads of a batch are issued
// before any arithmetic (memory-level parallelism), then the entries are
// accumulated in ascending order.  Entries past the row end read the row's
// own particle with zero weights, which adds exactly nothing.
template <int G, int NO, bool RESID, int U, typename ColF, typename WF, typename RF>
__device__ __forceinline__ void row_entries(RowAcc<NO, RESID>& acc, int k, int sub, int32_t self, float2 fp,
                                            const float2* __restrict__ f2, uint32_t comp, ColF col, WF wgt, RF res) {
    // batches of U entries per lane; entry order within the lane ascending
    // for every U (the accumulation order does not depend on U)
    for (int j0 = sub; j0 < k; j0 += G * U) {
        int32_t q[U];
        float w[U][NO], r[U][NO];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = j0 + u * G;
            const bool ok = j < k;
            q[u] = ok ? col(j) : self;
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                w[u][o] = ok ? wgt(o, j) : 0.0f;
                r[u][o] = (RESID && ok) ? res(o, j) : 0.0f;
            }
        }
        float2 fq[U];
#pragma unroll
        for (int u = 0; u < U; ++u) fq[u] = f2[q[u]];
#pragma unroll
        for (int u = 0; u < U; ++u) acc.add(w[u], r[u], fq[u], fp, comp);
    }
}

template <int G, int NO, bool RESID, int U>
__global__ void __launch_bounds__(256) apply_f32_kernel(F32Args a) {
    const int lane = threadIdx.x & 31;
    const int sub = lane & (G - 1);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rows_per_pass = ((int64_t)gridDim.x * blockDim.x) / G;
    const int64_t first = (tid - lane) / G;
    for (int64_t base = a.row0 + first; base < a.n; base += rows_per_pass) {
        const int64_t row = base + lane / G;
        RowAcc<NO, RESID> acc;
        acc.init();
        if (row < a.n) {
            const float2 fp = a.no_self ? make_float2(0.f, 0.f) : a.f2[row];
            const int64_t rb = a.rowptr[row];
            const int k = (int)(a.rowptr[row + 1] - rb);
            const int32_t* c = a.cols + rb;
            const float* w0 = a.w + rb;
            const __nv_bfloat16* r0 = RESID ? a.r + rb : nullptr;
            const int64_t ws = a.ws;
            row_entries<G, NO, RESID, U>(
                acc, k, sub, a.no_self ? 0 : (int32_t)row, fp, a.f2, a.comp, [&](int j) { return c[j]; },
                [&](int o, int j) { return w0[o * ws + j]; },
                [&](int o, int j) { return __bfloat162float(r0[o * ws + j]); });
        }
        acc.template reduce<G>();
        if (row < a.n) {
#pragma unroll
            for (int o = 0; o < NO; ++o)
                if (sub == (o & (G - 1))) a.out[(int64_t)o * a.oos + row * a.ors] = acc.value(o);
        }
    }
}

// ------------------------------------------------------- TMA bulk staging --
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: returns false after ~2^22 polls (each try_wait itself blocks
// for a while), so a copy that never lands cannot hang the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < (1u << 22); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

struct TmaCfg {
    int stages;
    int ecap;        // entries per stage buffer (multiple of 8)
    int stage_bytes; // bytes of one stage (16-byte multiple)
    int64_t ntiles;
    int64_t nnz;     // stride of the weight streams (element offset o*nnz)
};

// 16-byte aligned window [a0, a1) of a 4-byte stream covering [b, e)
__device__ __forceinline__ int64_t win_lo4(int64_t b) { return b & ~int64_t(3); }
__device__ __forceinline__ int64_t win_hi4(int64_t e) { return (e + 3) & ~int64_t(3); }
__device__ __forceinline__ int64_t win_lo8(int64_t b) { return b & ~int64_t(7); }
__device__ __forceinline__ int64_t win_hi8(int64_t e) { return (e + 7) & ~int64_t(7); }

// Layout of one stage: cols[ecap] i32 | w[NO][ecap] f32 | r[NO][ecap] bf16
template <int NO, bool RESID>
__device__ __forceinline__ void issue_tile(const F32Args& a, const TmaCfg& c, int64_t tile, int R, unsigned char* stage,
                                           uint32_t bar) {
    const int64_t r0 = tile * R;
    const int64_t r1 = min(r0 + R, a.n);
    const int64_t e0 = a.rowptr[r0], e1 = a.rowptr[r1];
    uint32_t total = 0;
    const int64_t c0 = win_lo4(e0), c1 = win_hi4(e1);
    total += (uint32_t)((c1 - c0) * 4);
#pragma unroll
    for (int o = 0; o < NO; ++o) {
        const int64_t b = (int64_t)o * a.ws + e0, e = (int64_t)o * a.ws + e1;
        total += (uint32_t)((win_hi4(e) - win_lo4(b)) * 4);
        if (RESID) total += (uint32_t)((win_hi8(e) - win_lo8(b)) * 2);
    }
    mbar_expect_tx(bar, total);
    unsigned char* p = stage;
    if (c1 > c0) bulk_g2s(smem_u32(p), a.cols + c0, (uint32_t)((c1 - c0) * 4), bar);
    p += (size_t)c.ecap * 4;
#pragma unroll
    for (int o = 0; o < NO; ++o) {
        const int64_t b = (int64_t)o * a.ws + e0, e = (int64_t)o * a.ws + e1;
        if (win_hi4(e) > win_lo4(b))
            bulk_g2s(smem_u32(p + (size_t)o * c.ecap * 4), a.w + win_lo4(b), (uint32_t)((win_hi4(e) - win_lo4(b)) * 4),
                     bar);
    }
    if (RESID) {
        p += (size_t)NO * c.ecap * 4;
#pragma unroll
        for (int o = 0; o < NO; ++o) {
            const int64_t b = (int64_t)o * a.ws + e0, e = (int64_t)o * a.ws + e1;
            if (win_hi8(e) > win_lo8(b))
                bulk_g2s(smem_u32(p + (size_t)o * c.ecap * 2), a.r + win_lo8(b),
                         (uint32_t)((win_hi8(e) - win_lo8(b)) * 2), bar);
        }
    }
}

template <int G, int NO, bool RESID>
__global__ void __launch_bounds__(256) apply_f32_tma_kernel(F32Args a, TmaCfg c, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int R = 256 / G;  // rows per tile: one G-lane group per row
    __shared__ __align__(8) unsigned long long bars[16];
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int sub = lane & (G - 1);
    const int grp = tid / G;
    const int S = c.stages;
    if (tid == 0) {
        for (int s = 0; s < S; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            int64_t t = blockIdx.x + (int64_t)s * gridDim.x;
            if (t < c.ntiles) issue_tile<NO, RESID>(a, c, t, R, smem + (size_t)s * c.stage_bytes, smem_u32(&bars[s]));
        }
    }
    for (int64_t i = 0;; ++i) {
        const int64_t t = blockIdx.x + i * gridDim.x;
        if (t >= c.ntiles) break;
        const int s = (int)(i % S);
        const uint32_t parity = (uint32_t)((i / S) & 1);
        if (tid == 0) s_ok = mbar_wait_bounded(smem_u32(&bars[s]), parity) ? 1 : 0;
        __syncthreads();
        if (!s_ok) {
            if (tid == 0) {
                atomicExch(err, 1);
                // let copies already issued for later stages land (bounded)
                for (int64_t k = 1; k < S; ++k) {
                    const int64_t ii = i + k;
                    if (blockIdx.x + ii * gridDim.x >= c.ntiles) break;
                    mbar_wait_bounded(smem_u32(&bars[ii % S]), (uint32_t)((ii / S) & 1));
                }
            }
            return;
        }
        const unsigned char* stage = smem + (size_t)s * c.stage_bytes;
        const int64_t r0 = t * R;
        const int64_t e0 = a.rowptr[r0];
        const int32_t* scols = reinterpret_cast<const int32_t*>(stage);
        const float* sw = reinterpret_cast<const float*>(stage + (size_t)c.ecap * 4);
        const __nv_bfloat16* sr = reinterpret_cast<const __nv_bfloat16*>(stage + (size_t)c.ecap * 4 * (1 + NO));
        const int64_t row = r0 + grp;
        RowAcc<NO, RESID> acc;
        acc.init();
        if (row < a.n) {
            const float2 fp = a.no_self ? make_float2(0.f, 0.f) : a.f2[row];
            const int64_t rb = a.rowptr[row], re = a.rowptr[row + 1];
            const int32_t* cptr = scols + (rb - win_lo4(e0));
            const float* wp[NO];
            const __nv_bfloat16* rpp[NO];
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                wp[o] = sw + (size_t)o * c.ecap + ((int64_t)o * a.ws + rb - win_lo4((int64_t)o * a.ws + e0));
                rpp[o] = sr + (size_t)o * c.ecap + ((int64_t)o * a.ws + rb - win_lo8((int64_t)o * a.ws + e0));
            }
            row_entries<G, NO, RESID, 4>(
                acc, (int)(re - rb), sub, a.no_self ? 0 : (int32_t)row, fp, a.f2, a.comp, [&](int j) { return cptr[j]; },
                [&](int o, int j) { return wp[o][j]; },
                [&](int o, int j) { return __bfloat162float(rpp[o][j]); });
        }
        acc.template reduce<G>();
        if (row < a.n) {
#pragma unroll
            for (int o = 0; o < NO; ++o)
                if (sub == (o & (G - 1))) a.out[(int64_t)o * a.oos + row * a.ors] = acc.value(o);
        }
        __syncthreads();  // every thread is done with stage s
        if (tid == 0) {
            const int64_t t2 = t + (int64_t)S * gridDim.x;
            if (t2 < c.ntiles) {
                fence_proxy_async();
                issue_tile<NO, RESID>(a, c, t2, R, smem + (size_t)s * c.stage_bytes, smem_u32(&bars[s]));
            }
        }
    }
}

template <int G, int NO, int U>
__global__ void __launch_bounds__(256) apply_f64_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ cols,
                                                        const double* __restrict__ w, int64_t nnz,
                                                        const double* __restrict__ f, double* __restrict__ out,
                                                        int no_self, int64_t oos, int64_t ors, int64_t fs) {
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
            const double fp = no_self ? 0.0 : f[row * fs];
            const int64_t e = rowptr[row + 1];
            int64_t j = rowptr[row] + sub;
            // U entries per lane in flight: columns, then the gathered field
            // values and the weights, then the FMAs
            for (; j + (U - 1) * G < e; j += U * G) {
                int32_t q[U];
                double fq[U], wv[U][NO];
#pragma unroll
                for (int u = 0; u < U; ++u) q[u] = cols[j + u * G];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    fq[u] = f[(int64_t)q[u] * fs];
#pragma unroll
                    for (int o = 0; o < NO; ++o) wv[u][o] = w[(int64_t)o * nnz + j + u * G];
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const double d = fq[u] - fp;
#pragma unroll
                    for (int o = 0; o < NO; ++o) acc[o] = fma(wv[u][o], d, acc[o]);
                }
            }
            for (; j < e; j += G) {
                const double d = f[(int64_t)cols[j] * fs] - fp;
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
                if (sub == (o & (G - 1))) out[(int64_t)o * oos + row * ors] = acc[o];
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

// FP64 batched apply (4-deep load batches up to 4 outputs, 2-deep above):
// 8 to 16 entries per lane, as for the FP32 apply
int lanes_for(int64_t n, int64_t nnz) {
    const double avg = n > 0 ? (double)nnz / (double)n : 0.0;
    int g = 4;
    while (g < 32 && avg / (2 * g) >= 8.0) g *= 2;
    return g;
}

// FP32 batched apply (4-deep load batches): 8 to 16 entries per lane, the
// best of the sweeps on GB300 (128^3 cloud, 84 entries per row: 8 lanes
// 0.727 ms, 4 lanes 0.763 ms, 16 lanes 0.998 ms)
int lanes_for_f32(int64_t n, int64_t nnz) {
    const double avg = n > 0 ? (double)nnz / (double)n : 0.0;
    int g = 4;
    while (g < 32 && avg / (2 * g) >= 8.0) g *= 2;
    return g;
}

template <int G, int NO, bool RESID, int U>
cudaError_t launch_f32_direct(const F32Args& a, cudaStream_t s) {
    apply_f32_kernel<G, NO, RESID, U><<<grid_rows(a.n - a.row0, 256 / G), 256, 0, s>>>(a);
    return cudaGetLastError();
}

template <int G, int NO, bool RESID>
cudaError_t launch_f32_tma(const F32Args& a, int maxk, int* err, cudaStream_t s, bool* used) {
    *used = false;
    constexpr int R = 256 / G;
    TmaCfg c{};
    c.ecap = ((R * maxk + 16) + 7) & ~7;
    size_t per = (size_t)c.ecap * (4 + 4 * NO + (RESID ? 2 * NO : 0));
    per = (per + 127) & ~size_t(127);
    c.stage_bytes = (int)per;
    c.ntiles = (a.n + R - 1) / R;
    c.nnz = a.ws;
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // two CTAs per SM, as many stages as fit (2..8)
    int stages = (int)((smem_max / 2 - 1024) / per);
    if (stages > 8) stages = 8;
    if (stages < 2) return cudaSuccess;  // rows too long for staging: caller uses the direct kernel
    c.stages = stages;
    size_t bytes = per * stages;
    auto kern = apply_f32_tma_kernel<G, NO, RESID>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, bytes);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaSuccess;
    int64_t grid = (int64_t)num_sms() * per_sm;
    if (grid > c.ntiles) grid = c.ntiles;
    kern<<<(unsigned)grid, 256, bytes, s>>>(a, c, err);
    *used = true;
    return cudaGetLastError();
}

template <int G, bool RESID>
cudaError_t dispatch_f32(const F32Args& a, int nout, int maxk, int* err, int mode, cudaStream_t s) {
#define DCPSE_F32_CASE(NO)                                                            \
    case NO: {                                                                        \
        if (mode == 0 || mode == 2) {                                                 \
            bool used = false;                                                        \
            cudaError_t e = launch_f32_tma<G, NO, RESID>(a, maxk, err, s, &used);     \
            if (e != cudaSuccess || used) return e;                                   \
            if (mode == 2) return cudaErrorInvalidConfiguration; /* tiles too big */  \
        }                                                                             \
        if (mode == 3 && !RESID && G <= 8) return launch_f32_direct<G, NO, RESID, 8>(a, s); \
        return launch_f32_direct<G, NO, RESID, 4>(a, s);                              \
    }
    switch (nout) {
        DCPSE_F32_CASE(1)
        DCPSE_F32_CASE(2)
        DCPSE_F32_CASE(3)
        DCPSE_F32_CASE(4)
        DCPSE_F32_CASE(5)
        DCPSE_F32_CASE(6)
        DCPSE_F32_CASE(7)
        DCPSE_F32_CASE(8)
        default:
            return cudaErrorInvalidValue;
    }
#undef DCPSE_F32_CASE
}

template <int G>
cudaError_t launch_f64(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const double* w, int64_t nnz,
                       const double* f, double* out, int no_self, int64_t oos, int64_t ors, int64_t fs,
                       cudaStream_t s) {
    const int grid = grid_rows(n, 256 / G);
#define DCPSE_F64_CASE(NO)                                                                                     \
    case NO:                                                                                                   \
        apply_f64_kernel<G, NO, (NO <= 4 ? 4 : 2)>                                                             \
            <<<grid, 256, 0, s>>>(n, rowptr, cols, w, nnz, f, out, no_self, oos, ors, fs);                     \
        break;
    switch (nout) {
        DCPSE_F64_CASE(1)
        DCPSE_F64_CASE(2)
        DCPSE_F64_CASE(3)
        DCPSE_F64_CASE(4)
        DCPSE_F64_CASE(5)
        DCPSE_F64_CASE(6)
        DCPSE_F64_CASE(7)
        DCPSE_F64_CASE(8)
        default:
            return cudaErrorInvalidValue;
    }
#undef DCPSE_F64_CASE
    return cudaGetLastError();
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

cudaError_t split_f64(const double* f, int64_t n, float2* f2, cudaStream_t s, int64_t stride) {
    if (n == 0) return cudaSuccess;
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)num_sms() * 8;
    split_kernel<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(f, n, stride, f2);
    return cudaGetLastError();
}

cudaError_t p2p_f64(int64_t n, const int64_t* rowptr, const int32_t* cols, const double* K, const double* eip,
                    int ncomp, const double* f, double* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)num_sms() * 8;
    p2p_f64_kernel<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(n, rowptr, cols, K, eip, ncomp, f, out);
    return cudaGetLastError();
}

// Loads the split kernel and every direct FP32 kernel apply_batched_f32 may
// launch (4-deep batches, no residuals, 4..32 lanes, 1..8 outputs) onto the
// current device.  Under lazy module loading a kernel's code is placed on
// the GPU at its first launch; cudaFuncGetAttributes does that up front.
cudaError_t preload_apply_f32_direct() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, split_kernel);
#define DCPSE_PRELOAD_NO(GG, NO) \
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, apply_f32_kernel<GG, NO, false, 4>);
#define DCPSE_PRELOAD_G(GG)                                                                     \
    DCPSE_PRELOAD_NO(GG, 1) DCPSE_PRELOAD_NO(GG, 2) DCPSE_PRELOAD_NO(GG, 3) DCPSE_PRELOAD_NO(GG, 4) \
    DCPSE_PRELOAD_NO(GG, 5) DCPSE_PRELOAD_NO(GG, 6) DCPSE_PRELOAD_NO(GG, 7) DCPSE_PRELOAD_NO(GG, 8)
    DCPSE_PRELOAD_G(4)
    DCPSE_PRELOAD_G(8)
    DCPSE_PRELOAD_G(16)
    DCPSE_PRELOAD_G(32)
#undef DCPSE_PRELOAD_G
#undef DCPSE_PRELOAD_NO
    return e;
}

int64_t f32_rows_per_wave(int64_t n, int64_t nnz, int lanes) {
    const int G = lanes ? lanes : lanes_for_f32(n, nnz);
    return (int64_t)num_sms() * 8 * (256 / G);
}

cudaError_t apply_batched_f32x(const ApplyF32& p, cudaStream_t s) {
    if (p.n == 0) return cudaSuccess;
    F32Args a{};
    a.n = p.row1 ? p.row1 : p.n;
    a.row0 = p.row0;
    if (a.row0 >= a.n) return cudaSuccess;
    // the staged kernel tiles whole lists: row ranges take the direct kernel
    if ((a.row0 != 0 || a.n != p.n) && p.mode == 2) return cudaErrorInvalidValue;
    a.rowptr = p.rowptr;
    a.cols = p.cols;
    a.w = p.w;
    a.r = reinterpret_cast<const __nv_bfloat16*>(p.resid);
    a.ws = p.ws;
    a.f2 = p.f2;
    a.out = p.out;
    a.oos = p.oos ? p.oos : p.n;
    a.ors = p.ors ? p.ors : 1;
    a.comp = p.comp;
    a.no_self = p.no_self;
    const int G = p.lanes ? p.lanes : lanes_for_f32(p.n, p.nnz);
    const bool resid = p.resid != nullptr;
    // 0 auto = direct loads (the staged kernel was slower at every size
    // measured on GB300), 1 direct, 2 staged, 3 direct x8
    const int mode = p.mode == 0 ? 1 : p.mode;
#define DCPSE_G(GG)                                                                                  \
    case GG:                                                                                         \
        return resid ? dispatch_f32<GG, true>(a, p.nout, p.maxk, p.err, mode, s)                     \
                     : dispatch_f32<GG, false>(a, p.nout, p.maxk, p.err, mode, s);
    switch (G) {
        DCPSE_G(4)
        DCPSE_G(8)
        DCPSE_G(16)
        DCPSE_G(32)
        default:
            return cudaErrorInvalidValue;
    }
#undef DCPSE_G
}

cudaError_t apply_batched_f32(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const float* w,
                              int64_t nnz, const float2* f2, double* out, cudaStream_t s) {
    ApplyF32 p{};
    p.n = n;
    p.nout = nout;
    p.rowptr = rowptr;
    p.cols = cols;
    p.w = w;
    p.ws = nnz;
    p.nnz = -1;
    p.f2 = f2;
    p.out = out;
    p.mode = 1;  // caller-owned arrays: no over-read of padded windows
    p.comp = 0xffffffffu;  // every output compensated
    // lanes from the mean row length (needs nnz; read from rowptr[n] is a
    // host sync, so the caller's stride stands in when it equals nnz)
    p.lanes = 0;
    p.nnz = nnz;
    return apply_batched_f32x(p, s);
}

cudaError_t apply_batched_f64(int64_t n, int nout, const int64_t* rowptr, const int32_t* cols, const double* w,
                              int64_t nnz, const double* f, double* out, cudaStream_t s, int no_self, int64_t oos,
                              int64_t ors, int64_t fs) {
    if (n == 0) return cudaSuccess;
    if (oos == 0) oos = n;
    if (ors == 0) ors = 1;
    if (fs == 0) fs = 1;
    switch (lanes_for(n, nnz)) {
        case 4: return launch_f64<4>(n, nout, rowptr, cols, w, nnz, f, out, no_self, oos, ors, fs, s);
        case 8: return launch_f64<8>(n, nout, rowptr, cols, w, nnz, f, out, no_self, oos, ors, fs, s);
        case 16: return launch_f64<16>(n, nout, rowptr, cols, w, nnz, f, out, no_self, oos, ors, fs, s);
        default: return launch_f64<32>(n, nout, rowptr, cols, w, nnz, f, out, no_self, oos, ors, fs, s);
    }
}

}  // namespace dcpse
