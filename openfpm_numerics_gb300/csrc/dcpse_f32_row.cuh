// dcpse_f32_row.cuh -- per-entry arithmetic of the batched FP32 applies
// (CSR and sliced ELL kernels): the field as an exact (hi, lo) float pair,
// f_q - f_p formed exactly as dh + dl with TwoSum (Knuth), every product
// w * dh entering a compensated sum (TwoSum of the running sum and the
// product, the rounding errors collected in a second float) for the outputs
// selected in comp, a plain fused multiply-add for the others.  The weight
// pairs' apply reads the field in fixed point instead (int64, one power-of-two
// scale per call): f_q - f_p is then exact in int64 and enters as a float pair.
#pragma once

#include <cuda_runtime.h>

namespace dcpse {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// d 2^-64 (|d| < 2^63) as a float pair dh + dl, |d 2^-64 - dh - dl| <=
// 2^-47 |d| 2^-64 (the scale keeps products with large weights inside the
// FP32 range).  d 2^-64 = x + y + z exactly with x = (d >> 42) 2^-22, y =
// bits 21-41 of d times 2^-43, z = bits 0-20 times 2^-64, each formed exactly
// by placing the integer in the mantissa of a float whose unit in the last
// place is that power of two and subtracting that float's value (3.0: unit
// 2^-22; 2^-20: unit 2^-43; 2^-41: unit 2^-64).  Then Fast2Sum (Dekker) of x
// and y (|x| >= |y| unless x = 0), the error term plus z rounded once (exact
// unless |x + y| >= 2^-19, where it is a 2^-48 relative error), and Fast2Sum
// again to normalise the pair.
__device__ __forceinline__ void fixed_pair(long long d, float& dh, float& dl) {
    const int a = (int)(d >> 42);  // [-2^21, 2^21)
    const unsigned b = (unsigned)(d >> 21) & 0x1fffffu;
    const unsigned c = (unsigned)d & 0x1fffffu;
    const float x = __int_as_float(0x40400000 + a) - 3.0f;
    const float y = __uint_as_float(0x35800000u | b) - 0x1p-20f;
    const float z = __uint_as_float(0x2B000000u | c) - 0x1p-41f;
    const float s = x + y;
    const float t = (y - (s - x)) + z;
    dh = s + t;
    dl = t - (dh - s);
}

// LOW2: the low sum c is itself compensated (TwoSum, its errors collected in
// cc), for the weight pairs, whose results are held to the FP64 apply's
// accuracy: with plain FP32 low sums, rows whose terms cancel ~1e3-fold lost
// ~1e-12 normwise there
template <int NO, bool RESID, bool LOW2 = false>
struct RowAcc {
    float s[NO], c[NO];
    float cc[LOW2 ? NO : 1];
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int o = 0; o < NO; ++o) s[o] = c[o] = 0.0f;
        if constexpr (LOW2) {
#pragma unroll
            for (int o = 0; o < NO; ++o) cc[o] = 0.0f;
        }
    }
    // one neighbour: weights w[o] (and residuals r[o]), field pair fq, fp.
    // Outputs whose bit is set in comp take the compensated sum (derivatives
    // of order >= 2, whose first-order contributions cancel); the others a
    // plain fused multiply-add into (s, c).
    __device__ __forceinline__ void add(const float (&w)[NO], const float (&r)[NO], float2 fq, float2 fp,
                                        uint32_t comp) {
        float dh, e0;
        two_sum(fq.x, -fp.x, dh, e0);
        add_diff(w, r, dh, e0 + (fq.y - fp.y), comp);
    }
    // the field in fixed point: the difference in int64, then as a float pair
    // (the sum is then in units of 2^64 times the field's quantum)
    __device__ __forceinline__ void add(const float (&w)[NO], const float (&r)[NO], long long fq, long long fp,
                                        uint32_t comp) {
        float dh, dl;
        fixed_pair(fq - fp, dh, dl);
        add_diff(w, r, dh, dl, comp);
    }
    // one neighbour's difference f_q - f_p = dh + dl
    __device__ __forceinline__ void add_diff(const float (&w)[NO], const float (&r)[NO], float dh, float dl,
                                             uint32_t comp) {
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
                if constexpr (LOW2) {
                    float nc, e2;
                    two_sum(c[o], t, nc, e2);
                    c[o] = nc;
                    cc[o] = cc[o] + e2;
                } else {
                    c[o] = c[o] + t;
                }
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
    __device__ __forceinline__ double value(int o) const {
        if constexpr (LOW2) return (double)s[o] + ((double)c[o] + (double)cc[o]);
        return (double)s[o] + (double)c[o];
    }
};

}  // namespace dcpse
