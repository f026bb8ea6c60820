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
// Method: P. T. P. Tang, "Table-driven implementation of the exponential
// function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, with 32
// table entries: x = (32 m + j) ln2/32 + r, |r| <= ln2/64, and
// e^x = 2^m 2^(j/32) (1 + p(r)) with p the Taylor polynomial of e^r - 1 to the
// r^6 term; 2^(j/32) is held as a sum of two doubles.  Every product that
// meets a sum is an explicit fused multiply-add and every other operation a
// single correctly rounded IEEE operation, so no compiler can contract them
// differently on either side.  Error about half a unit in the last place.
// Twelve FP64 operations: the GB300's FP64 rate is low, and the MC kernel
// calls this several times per move.
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

// 2^(j/32) = EXP2_TAB[2j] + EXP2_TAB[2j+1], j = 0..31
#define LDO_EXP2_TAB \
    0x1.0000000000000p+0, 0x0.0p+0, \
    0x1.059b0d3158574p+0, 0x1.d73e2a475b465p-55, \
    0x1.0b5586cf9890fp+0, 0x1.8a62e4adc610bp-54, \
    0x1.11301d0125b51p+0, -0x1.6c51039449b3ap-54, \
    0x1.172b83c7d517bp+0, -0x1.19041b9d78a76p-55, \
    0x1.1d4873168b9aap+0, 0x1.e016e00a2643cp-54, \
    0x1.2387a6e756238p+0, 0x1.9b07eb6c70573p-54, \
    0x1.29e9df51fdee1p+0, 0x1.612e8afad1255p-55, \
    0x1.306fe0a31b715p+0, 0x1.6f46ad23182e4p-55, \
    0x1.371a7373aa9cbp+0, -0x1.63aeabf42eae2p-54, \
    0x1.3dea64c123422p+0, 0x1.ada0911f09ebcp-55, \
    0x1.44e086061892dp+0, 0x1.89b7a04ef80d0p-59, \
    0x1.4bfdad5362a27p+0, 0x1.d4397afec42e2p-56, \
    0x1.5342b569d4f82p+0, -0x1.07abe1db13cadp-55, \
    0x1.5ab07dd485429p+0, 0x1.6324c054647adp-54, \
    0x1.6247eb03a5585p+0, -0x1.383c17e40b497p-54, \
    0x1.6a09e667f3bcdp+0, -0x1.bdd3413b26456p-54, \
    0x1.71f75e8ec5f74p+0, -0x1.16e4786887a99p-55, \
    0x1.7a11473eb0187p+0, -0x1.41577ee04992fp-55, \
    0x1.82589994cce13p+0, -0x1.d4c1dd41532d8p-54, \
    0x1.8ace5422aa0dbp+0, 0x1.6e9f156864b27p-54, \
    0x1.93737b0cdc5e5p+0, -0x1.75fc781b57ebcp-57, \
    0x1.9c49182a3f090p+0, 0x1.c7c46b071f2bep-56, \
    0x1.a5503b23e255dp+0, -0x1.d2f6edb8d41e1p-54, \
    0x1.ae89f995ad3adp+0, 0x1.7a1cd345dcc81p-54, \
    0x1.b7f76f2fb5e47p+0, -0x1.5584f7e54ac3bp-56, \
    0x1.c199bdd85529cp+0, 0x1.11065895048ddp-55, \
    0x1.cb720dcef9069p+0, 0x1.503cbd1e949dbp-56, \
    0x1.d5818dcfba487p+0, 0x1.2ed02d75b3707p-55, \
    0x1.dfc97337b9b5fp+0, -0x1.1a5cd4f184b5cp-54, \
    0x1.ea4afa2a490dap+0, -0x1.e9c23179c2893p-54, \
    0x1.f50765b6e4540p+0, 0x1.9d3e12dd8a18bp-54
#if defined(__CUDACC__)
static __constant__ const double kExp2TabDev[64] = {LDO_EXP2_TAB};
#endif
static const double kExp2TabHost[64] = {LDO_EXP2_TAB};

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
LDO_MATH_HD double add_(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    volatile double q = a + b;
    return q;
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
    // ln2/32 = L_HI + L_LO
    const double L_HI = 0x1.62e42fefa39efp-6;
    const double L_LO = 0x1.abc9e3b39803fp-61;
    const double INV_L = 0x1.71547652b82fep+5;
    double n = rint_(mul_(x, INV_L));
    double r = fma_(-n, L_HI, x);
    r = fma_(-n, L_LO, r);
    // p = e^r - 1 = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720)
    double p = 0x1.6c16c16c16c17p-10;
    p = fma_(p, r, 0x1.1111111111111p-7);
    p = fma_(p, r, 0x1.5555555555555p-5);
    p = fma_(p, r, 0x1.5555555555555p-3);
    p = fma_(p, r, 0.5);
    p = fma_(p, mul_(r, r), r);
    int ni = (int)n;
    int j = ni & 31;
    int m = (ni - j) >> 5;
#if defined(__CUDA_ARCH__)
    double t_hi = kExp2TabDev[2 * j], t_lo = kExp2TabDev[2 * j + 1];
#else
    double t_hi = kExp2TabHost[2 * j], t_lo = kExp2TabHost[2 * j + 1];
#endif
    // 2^(j/32) (1 + p) = t_hi + (t_lo + t_hi p)
    double y = add_(t_hi, fma_(t_hi, p, t_lo));
    if (m > 1023) return mul_(mul_(y, pow2i(1023)), pow2i(m - 1023));
    if (m < -1022) return mul_(mul_(y, pow2i(m + 600)), pow2i(-600));
    return mul_(y, pow2i(m));
}

} // namespace ldo_math
