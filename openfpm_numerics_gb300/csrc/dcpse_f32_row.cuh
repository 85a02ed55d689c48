// dcpse_f32_row.cuh -- per-entry arithmetic of the batched FP32 applies
// (CSR and sliced ELL kernels): the field as an exact (hi, lo) float pair,
// f_q - f_p formed exactly as dh + dl with TwoSum (Knuth), every product
// w * dh entering a compensated sum (TwoSum of the running sum and the
// product, the rounding errors collected in a second float) for the outputs
// selected in comp, a plain fused multiply-add for the others.
#pragma once

#include <cuda_runtime.h>

namespace dcpse {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <int NO, bool RESID>
struct RowAcc {
    float s[NO], c[NO];
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int o = 0; o < NO; ++o) s[o] = c[o] = 0.0f;
    }
    // one neighbour: weights w[o] (and residuals r[o]), field pair fq, fp.
    // Outputs whose bit is set in comp take the compensated sum (derivatives
    // of order >= 2, whose first-order contributions cancel); the others a
    // plain fused multiply-add into (s, c).
    __device__ __forceinline__ void add(const float (&w)[NO], const float (&r)[NO], float2 fq, float2 fp,
                                        uint32_t comp) {
        float dh, e0;
        two_sum(fq.x, -fp.x, dh, e0);
        const float dl = e0 + (fq.y - fp.y);
#pragma unroll
        for (int o = 0; o < NO; ++o) {
            if (comp & (1u << o)) {
                const float p = w[o] * dh;
                float ns, e;
                two_sum(s[o], p, ns, e);
                s[o] = ns;
                float t = fmaf(w[o], dh, -p) + e;
                t = fmaf(w[o], dl, t);
                if (RESID) t = fmaf(r[o], dh, t);
                c[o] = c[o] + t;
            } else {
                s[o] = fmaf(w[o], dh, s[o]);
                float t = fmaf(w[o], dl, c[o]);
                if (RESID) t = fmaf(r[o], dh, t);
                c[o] = t;
            }
        }
    }
    template <int G>
    __device__ __forceinline__ void reduce() {
#pragma unroll
        for (int o = 0; o < NO; ++o) {
#pragma unroll
            for (int m = G / 2; m > 0; m >>= 1) {
                float os = __shfl_xor_sync(0xffffffffu, s[o], m);
                float oc = __shfl_xor_sync(0xffffffffu, c[o], m);
                float ns, e;
                two_sum(s[o], os, ns, e);
                s[o] = ns;
                c[o] = (c[o] + oc) + e;
            }
        }
    }
    __device__ __forceinline__ double value(int o) const { return (double)s[o] + (double)c[o]; }
};

}  // namespace dcpse
