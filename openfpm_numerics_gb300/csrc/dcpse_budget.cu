// dcpse_budget.cu -- the FP64 residual correction of the FP32 batched apply,
// applied where an error budget asks for it.
//
// The FP32 apply (field as an exact float pair, exact differences,
// compensated sums) is exact up to the rounding of its weights: with
// w32 = RN(w64), |w64 - w32| <= 2^-24 |w32| (1 + 2^-23), so the error of
// output o at row p is at most 2^-24 (1 + 2^-23) B_o,p with
//     B_o,p = sum_q |w32_o,pq| |f_q - f_p|,
// which the sliced FP32 kernel accumulates beside the output.  With the bf16
// residual streams r16 = RN_bf16(RN32(w64 - w32)) added (8-bit significands,
// unit roundoff 2^-8) the weight error is at most 2^-32 (1 + 2^-23) |w32|,
// so the same B bounds it with the factor 2^-32.  The compensated sums' own
// rounding (O(k 2^-48) B for k entries) and that of B itself (a sum of at
// most a few hundred FP32 terms) stay inside a margin of 2^-8.
// A call with relative budget eps must end with
//     max_p |out_o,p - out64_o,p| <= eps max_p |out64_o,p|     (each output o).
// A row is corrected when its bound exceeds half the budget against the
// call's own largest |output| M_o (the FP32 outputs: M_o overestimates the
// FP64 maximum by at most the largest FP32 error, which the factor 1/2 and
// the corrected rows themselves cover).  The correction adds
//     sum_q (r_o,pq - r16_o,pq) (f_q - f_p),   r = RN32(w64 - w32)
// (r16 = 0 without the bf16 streams; r - r16 is exact in FP32 since r16 is
// within a factor 2 of r; |w64 - w32 - r| <= 2^-24 |w64 - w32|, so the
// corrected row is exact up to 2^-48 B_o,p).  The correction is summed with
// the FP32 apply's own arithmetic (the field's float pair, exact
// differences, compensated sums): it needs only FP32 relative accuracy,
// being 2^-24 of the output's terms.
//
// Two kernels.  The first tests every row against the thresholds (one lane
// per row, reading the bounds coalesced) and appends the flagged rows, with
// their output masks, to a list (one atomic per warp).  The second walks the
// list with a warp per row (control flow stays uniform within the warp):
// the row's columns and residual streams are contiguous in the CSR layout;
// the lanes' sums are reduced by shuffles in a fixed order and the
// corrections added in place, so the results do not depend on the list's
// order.  Without bounds (flag_all) every row is
// corrected: the path for applies whose FP32 kernel does not compute them.
#include <cuda_bf16.h>

#include "dcpse_internal.h"
#include "dcpse_f32_row.cuh"

namespace dcpse {
namespace {

template <int NO>
__global__ void __launch_bounds__(256) budget_flag_kernel(BudgetArgs a) {
    __shared__ float thr[NO];
    if (threadIdx.x < NO) {
        // scale (1 + 2^-8) B > eps M / 2  <=>  B > thr
        const float m = a.flag_all ? 0.0f : __uint_as_float(a.maxabs[threadIdx.x]);
        thr[threadIdx.x] = (float)((double)m * a.budget * 0.5 / (a.bound_scale * (1.0 + 1.0 / 256.0)));
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < a.n; base += stride) {
        const int64_t p = base + lane;
        unsigned mask = 0;
        if (p < a.n) {
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                // a NaN bound or threshold flags the row (its FP64 sum decides)
                const bool flag = a.flag_all || !(a.bnd[(int64_t)o * a.n + p] <= thr[o]);
                mask |= flag ? (1u << o) : 0u;
            }
        }
        const unsigned rows = __ballot_sync(0xffffffffu, mask != 0);
        if (!rows) continue;
        const unsigned npairs = __reduce_add_sync(0xffffffffu, (unsigned)__popc(mask));
        unsigned slot0 = 0;
        if (lane == 0) {
            slot0 = atomicAdd(a.list_len, (unsigned)__popc(rows));
            if (a.count) atomicAdd(a.count, (unsigned long long)npairs);
        }
        slot0 = __shfl_sync(0xffffffffu, slot0, 0);
        if (mask) {
            const unsigned rank = __popc(rows & ((1u << lane) - 1u));
            a.list[slot0 + rank] = make_uint2((unsigned)p, mask);
        }
    }
}

template <int NO, bool R16>
__global__ void __launch_bounds__(256) budget_apply_kernel(BudgetArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t len = *a.list_len;
    const int64_t stride = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < len; e += stride) {
        const uint2 item = a.list[e];
        const int64_t row = item.x;
        const unsigned pm = item.y;
        const int64_t beg = a.rowptr[row], end = a.rowptr[row + 1];
        const float2 fp = a.f2[a.inv ? (int64_t)a.inv[row] : row];
        // the FP32 apply's exact differences and compensated sums: the
        // residuals are 2^-24 of the weights, so the correction needs only
        // FP32 relative accuracy (GB300's FP64 pipe is narrow)
        RowAcc<NO, false> acc;
        acc.init();
        float rz[NO];
#pragma unroll
        for (int o = 0; o < NO; ++o) rz[o] = 0.0f;
        for (int64_t j = beg + lane; j < end; j += 32) {
            const int32_t q = a.cols[j];
            const float2 fq = a.f2[a.inv ? a.inv[q] : q];
            float r[NO];
#pragma unroll
            for (int o = 0; o < NO; ++o) {
                r[o] = 0.0f;
                if (pm & (1u << o)) {
                    r[o] = a.r32[(int64_t)o * a.ws + j];
                    if (R16)
                        r[o] -= __bfloat162float(static_cast<const __nv_bfloat16*>(a.r16)[(int64_t)o * a.ws + j]);
                }
            }
            acc.add(r, rz, fq, fp, 0xffffffffu);
        }
        acc.template reduce<32>();
        if (lane < NO && (pm & (1u << lane))) {
#pragma unroll
            for (int o = 0; o < NO; ++o)
                if (o == lane) {
                    double* dst = a.out + (int64_t)o * a.oos + row * a.ors;
                    *dst = *dst + acc.value(o);
                }
        }
    }
}

}  // namespace

cudaError_t budget_correct(const BudgetArgs& a, int nout, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    if (a.n > 0xffffffffll) return cudaErrorInvalidValue;  // rows are listed as 32-bit indices
    const int64_t cap = (int64_t)num_sms() * 8;
    const int64_t gflag = std::min<int64_t>((a.n + 255) / 256, cap);
    // the list length is read on the device: a full wave of warps
    const int64_t gapply = cap;
    switch (nout) {
#define DCPSE_BUDGET_CASE(NO)                                                          \
    case NO:                                                                           \
        budget_flag_kernel<NO><<<(unsigned)gflag, 256, 0, s>>>(a);                     \
        if (a.r16)                                                                     \
            budget_apply_kernel<NO, true><<<(unsigned)gapply, 256, 0, s>>>(a);         \
        else                                                                           \
            budget_apply_kernel<NO, false><<<(unsigned)gapply, 256, 0, s>>>(a);        \
        break;
        DCPSE_BUDGET_CASE(1)
        DCPSE_BUDGET_CASE(2)
        DCPSE_BUDGET_CASE(3)
        DCPSE_BUDGET_CASE(4)
        DCPSE_BUDGET_CASE(5)
        DCPSE_BUDGET_CASE(6)
        DCPSE_BUDGET_CASE(7)
        DCPSE_BUDGET_CASE(8)
#undef DCPSE_BUDGET_CASE
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace dcpse
