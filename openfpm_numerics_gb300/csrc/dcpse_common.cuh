// dcpse_common.cuh -- shared device helpers of the GB300 DC-PSE path.
//
// The FP64 helpers here fix the operation sequence (and so the rounding) of
// every step that feeds the moment matrices and kernels.  Translation units
// that use them for assembly are compiled with -fmad=false; fused
// multiply-adds are written out as fma().
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace dcpse {

constexpr int kMaxDim = 3;

// ---------------------------------------------------------------- exp -----
// Cody & Waite (1980) argument reduction, x = k ln2 + r with |r| <= ln2/2,
// then the degree-13 Taylor polynomial of exp(r) by Horner's rule and a
// scaling by 2^k.  Max error about 1 ulp; the same sequence of correctly
// rounded operations on every platform, so results are reproducible bit for
// bit.  LN2_HI has 32 significant bits (k*LN2_HI exact for |k| < 2^21).
__host__ __device__ __forceinline__ double pow2i(int k) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)(k + 1023) << 52);
#else
    union { uint64_t u; double d; } c;
    c.u = (uint64_t)(k + 1023) << 52;
    return c.d;
#endif
}

__host__ __device__ __forceinline__ double cw_exp(double x) {
    const double LN2_HI = 0x1.62e42ff000000p-1;
    const double LN2_LO = -0x1.718432a1b0e26p-35;
    const double INV_LN2 = 0x1.71547652b82fep+0;
    if (x != x) return x;
    if (x > 709.0) return INFINITY;
    if (x < -745.0) return 0.0;
    double kd = rint(x * INV_LN2);
    double r = fma(-kd, LN2_HI, x);
    r = fma(-kd, LN2_LO, r);
    double p = 0x1.6124613a86d09p-33;      // 1/13!
    p = fma(p, r, 0x1.1eed8eff8d898p-29);  // 1/12!
    p = fma(p, r, 0x1.ae64567f544e4p-26);  // 1/11!
    p = fma(p, r, 0x1.27e4fb7789f5cp-22);  // 1/10!
    p = fma(p, r, 0x1.71de3a556c734p-19);  // 1/9!
    p = fma(p, r, 0x1.a01a01a01a01ap-16);  // 1/8!
    p = fma(p, r, 0x1.a01a01a01a01ap-13);  // 1/7!
    p = fma(p, r, 0x1.6c16c16c16c17p-10);  // 1/6!
    p = fma(p, r, 0x1.1111111111111p-7);   // 1/5!
    p = fma(p, r, 0x1.5555555555555p-5);   // 1/4!
    p = fma(p, r, 0x1.5555555555555p-3);   // 1/3!
    p = fma(p, r, 0x1.0000000000000p-1);   // 1/2!
    p = fma(p, r, 1.0);
    p = fma(p, r, 1.0);
    int k = (int)kd;
    if (k < -1022) {
        p = p * pow2i(-1022);
        k = k + 1022;
    }
    return p * pow2i(k);
}

// Exponentiation by squaring (the role of openfpm::math::intpowlog in
// src/DCPSE/Monomial.hpp:153 and Dcpse.hpp:743).
__host__ __device__ __forceinline__ double ipow(double x, unsigned e) {
    double r = 1.0;
    if (e == 0) return r;
    // iterative form of: h = ipow(x, e/2); r = h*h; if (e odd) r *= x;
    // processes the exponent bits from the most significant one down, which
    // performs exactly the multiplications of the recursive definition.
    int top = 0;
    while ((e >> (top + 1)) != 0u) ++top;
    r = x;
    for (int b = top - 1; b >= 0; --b) {
        r = r * r;
        if ((e >> b) & 1u) r = r * x;
    }
    return r;
}

// x_p - x_q with the minimum image along periodic axes.
struct Geom {
    double L[kMaxDim];
    double half[kMaxDim];
    int per[kMaxDim];
};

__host__ __device__ __forceinline__ double offset1(const Geom& g, int d, double a, double b) {
    double o = a - b;
    if (g.per[d]) {
        double L = g.L[d];
        double h = g.half[d];
        if (o > h)
            o = o - L;
        else if (o < -h)
            o = o + L;
    }
    return o;
}

template <int DIM>
__host__ __device__ __forceinline__ double norm2(const double* x) {
    double s = x[0] * x[0];
#pragma unroll
    for (int d = 1; d < DIM; ++d) s = s + x[d] * x[d];
    return s;
}

enum PartStatus { ST_OK = 0, ST_TOO_FEW = 1, ST_BAD_EPS = 2, ST_SINGULAR = 3, ST_NONFINITE = 4 };

}  // namespace dcpse
