// The engine's exponential, one implementation for the GPU and for host code.
//
// Acceptance probabilities and Rosenbluth weights are products and ratios of
// exponentials; when a move regrows a configuration whose weight equals the
// old one's, the ratio is 1 up to rounding, and whether it rounds to exactly 1
// decides whether the acceptance test draws a random number at all.  The
// outcome then depends on the last bit of every exponential, which differs
// between math libraries.  This function gives the same bits on the device and
// on the host, so that a host restatement of the moves follows the kernels
// draw for draw.
//
// Method: Cody and Waite's argument reduction (W. J. Cody and W. Waite,
// "Software Manual for the Elementary Functions", Prentice-Hall, 1980),
// x = k ln 2 + r with |r| <= ln 2 / 2, then the Taylor series of e^r to the
// r^13 term by Horner's rule, and the exact scaling by 2^k.  Every product
// that meets a sum is an explicit fused multiply-add and every other operation
// is a single correctly rounded IEEE operation, so no compiler can contract
// them differently on either side.  Error below one unit in the last place.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define LDO_MATH_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define LDO_MATH_HD inline
#endif

namespace ldo_math {

LDO_MATH_HD double fma_(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
LDO_MATH_HD double mul_(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    volatile double p = a * b;
    return p;
#endif
}
LDO_MATH_HD double rint_(double x) {
#if defined(__CUDA_ARCH__)
    return rint(x);
#else
    return std::nearbyint(x);
#endif
}
LDO_MATH_HD double pow2i(int k) {   // 2^k for -1022 <= k <= 1023; 1024 gives +infinity
    uint64_t b = (uint64_t)(k + 1023) << 52;
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
}

LDO_MATH_HD double exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return pow2i(1024);   // +infinity
    if (x < -745.2) return 0.0;
    // ln 2 = LN2_HI + LN2_LO, LN2_HI the double nearest ln 2
    const double LN2_HI = 0x1.62e42fefa39efp-1;
    const double LN2_LO = 0x1.abc9e3b39803fp-56;
    const double INV_LN2 = 0x1.71547652b82fep0;
    double k = rint_(mul_(x, INV_LN2));
    double r = fma_(-k, LN2_HI, x);
    r = fma_(-k, LN2_LO, r);
    // 1 / n! for n = 13 .. 2, rounded to nearest
    double p = 0x1.6124613a86d09p-33;
    p = fma_(p, r, 0x1.1eed8eff8d898p-29);
    p = fma_(p, r, 0x1.ae64567f544e4p-26);
    p = fma_(p, r, 0x1.27e4fb7789f5cp-22);
    p = fma_(p, r, 0x1.71de3a556c734p-19);
    p = fma_(p, r, 0x1.a01a01a01a01ap-16);
    p = fma_(p, r, 0x1.a01a01a01a01ap-13);
    p = fma_(p, r, 0x1.6c16c16c16c17p-10);
    p = fma_(p, r, 0x1.1111111111111p-7);
    p = fma_(p, r, 0x1.5555555555555p-5);
    p = fma_(p, r, 0x1.5555555555555p-3);
    p = fma_(p, r, 0.5);
    p = fma_(p, r, 1.0);
    p = fma_(p, r, 1.0);
    int ki = (int)k;
    if (ki > 1023) return mul_(mul_(p, pow2i(1023)), pow2i(ki - 1023));
    if (ki < -1022) return mul_(mul_(p, pow2i(ki + 600)), pow2i(-600));
    return mul_(p, pow2i(ki));
}

} // namespace ldo_math
