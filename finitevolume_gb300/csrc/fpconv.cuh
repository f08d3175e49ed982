// float <-> double conversions on the integer pipe.
//
// On GB300 a hardware double<->float conversion issues on the FP64 pipe,
// which runs at about 1.6 thread-operations per SM-clock; in the FP32-flux
// kernels those conversions, not the FP32 work, set the run time.  These
// routines produce the IEEE 754 results bit for bit (float -> double is
// exact; double -> float rounds to nearest, ties to even, with float
// subnormals, signed zeros, overflow to infinity and NaN handled) using
// only integer shifts, adds and selects, straight from the binary32 /
// binary64 encodings:
//   binary32: sign 1 | exponent 8 (bias 127)  | fraction 23
//   binary64: sign 1 | exponent 11 (bias 1023) | fraction 52
// so a normal value keeps its fraction bits (shifted by 29) and has its
// exponent re-biased by 1023 - 127 = 896.
//
// rcp_nr3 (an FP64 reciprocal with three FP64-pipe instructions) uses the
// same encodings to seed its iteration from the FP32 reciprocal.
#pragma once

#include <cstdint>

namespace fvconv {

__device__ __forceinline__ double f2d(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint32_t a = b & 0x7fffffffu;
    const uint32_t ef = a >> 23;
    uint64_t r;
    if (ef - 1u < 254u) {
        // normal: re-bias the exponent, widen the fraction
        r = ((uint64_t)a << 29) + ((uint64_t)896 << 52);
    } else if (ef == 255u) {
        // infinity / NaN: all-ones exponent, fraction kept (quiet bit stays)
        r = 0x7ff0000000000000ull | ((uint64_t)(a & 0x7fffffu) << 29);
    } else if (a == 0u) {
        r = 0;
    } else {
        // subnormal float: value = m * 2^-149 with m < 2^23; normalise so the
        // leading one (bit p) becomes the implicit bit of a normal double
        const int p = 31 - __clz((int)a);
        r = ((uint64_t)(p + 874) << 52) | (((uint64_t)a << (52 - p)) & 0x000fffffffffffffull);
    }
    return __longlong_as_double((long long)(sign | r));
}

__device__ __forceinline__ float d2f(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint64_t a = b & 0x7fffffffffffffffull;
    const uint32_t ed = (uint32_t)(a >> 52);
    uint32_t r;
    if (ed - 897u < 254u) {
        // normal float range: drop 29 fraction bits, round to nearest even;
        // a carry out of the fraction bumps the exponent (to infinity past
        // the largest float), as IEEE rounding requires
        const uint64_t t = a - ((uint64_t)896 << 52);
        const uint32_t q = (uint32_t)(t >> 29);
        const uint32_t rem = (uint32_t)t & 0x1fffffffu;
        r = q + ((rem > 0x10000000u) | ((rem == 0x10000000u) & (q & 1u)));
    } else if (ed >= 1151u) {
        // overflow -> infinity; NaN stays NaN (quiet, payload top bits kept)
        r = a > 0x7ff0000000000000ull ? (0x7fc00000u | (uint32_t)((a >> 29) & 0x3fffffu)) : 0x7f800000u;
    } else if (ed < 871u) {
        // below half the smallest float subnormal (2^-150): rounds to zero
        r = 0;
    } else {
        // float subnormal result: m = round(x * 2^149); with the implicit bit,
        // x * 2^149 = full * 2^(ed - 926), a right shift by s = 926 - ed
        // (30 <= s <= 55).  m may round up to 2^23 = the smallest normal.
        const uint64_t full = (a & 0x000fffffffffffffull) | 0x0010000000000000ull;
        const int s = 926 - (int)ed;
        const uint64_t q = full >> s;
        const uint64_t rem = full & ((1ull << s) - 1ull);
        const uint64_t half = 1ull << (s - 1);
        r = (uint32_t)(q + ((rem > half) | ((rem == half) & (q & 1ull))));
    }
    return __uint_as_float(sign | r);
}

// FP64 reciprocal with three DFMA: the FP32 approximate reciprocal of x
// (x truncated to float on the integer pipe, rcp.approx.f32, widened on
// the integer pipe) is a seed y with relative error e <= 2^-22, i.e.
// r = 1 - x y = e; one step of the third-order Newton-Raphson iteration for
// 1/x (the Taylor series 1/x = y (1 + r + r^2 + ...) truncated after r^2)
// leaves x y' = 1 - e^3 ~ 1 - 2^-66, so the single rounding of the final
// FMA gives 1/x to within about half an ulp.  Values outside the float
// normal range (and 0, inf, NaN) take the IEEE division.
__device__ __forceinline__ double rcp_nr3(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    if (e - 898u > 250u) return 1.0 / x;  // |x| outside [2^-125, 2^126)
    const unsigned fb = ((unsigned)(b >> 32) & 0x80000000u) | ((e - 896u) << 23) | ((unsigned)(b >> 29) & 0x7fffffu);
    float s;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(__uint_as_float(fb)));
    const double y = f2d(s);
    const double r = fma(-x, y, 1.0);
    return fma(y, fma(r, r, r), y);
}

// x^k for x near 1 with a short chain of dependent FP64 operations (for
// boundary states on a critical path; the library pow is a much longer
// chain).  ln x = 2 atanh z with z = (x - 1) / (x + 1) (x - 1 is exact for
// x in [1/2, 2]), then e^y with y = k ln x:
//   |x - 1| <= 1/64 (|z| <= 1/127): atanh z = z (1 + z^2/3 + ... + z^8/9)
//     (the first omitted term is below 2^-70 of the sum) and, for
//     |y| <= 1/12, e^y = (e^(y/2))^2 with e^t - 1 = t (1 + t/2 + ... +
//     t^7/8!) (|t| <= 1/24, remainder below 2^-64), both polynomials by
//     Estrin's scheme (half the dependent depth of Horner's);
//   |x - 1| <= 1/8 (|z| <= 1/15): the atanh series to z^14/15 (below 2^-58)
//     and, for |y| <= 3/4, e^y = (e^(y/8))^8 with e^t - 1 to degree 10
//     (|t| <= 3/32, below 2^-62), by Horner;
//   otherwise the library pow.
// e^t - 1 is carried through the squarings ((1 + u)^2 - 1 = u (u + 2)) so
// that the small part keeps its relative accuracy until the final 1 + u.
// The rounding of y (a few ulps, times |y|) dominates: the result is within
// 8 ulps of x^k (5 measured against the library pow on 2^26 bases).
__device__ __forceinline__ double pow_near1(double x, double k) {
    const double xm = x - 1.0;
    const double axm = fabs(xm);
    if (!(axm <= 0.125)) return pow(x, k);
    const double z = xm * rcp_nr3(x + 1.0);
    const double z2 = z * z;
    if (axm <= 1.0 / 64.0) {
        const double z4 = z2 * z2;
        const double inner = fma(z4, 1.0 / 9.0, fma(z2, 1.0 / 7.0, 1.0 / 5.0));
        const double q = fma(z4, inner, fma(z2, 1.0 / 3.0, 1.0));
        const double y = (2.0 * k) * (z * q);
        if (fabs(y) <= 1.0 / 12.0) {
            const double t = 0.5 * y;
            const double t2 = t * t, t4 = t2 * t2;
            const double p01 = fma(t, 0.5, 1.0), p23 = fma(t, 1.0 / 24.0, 1.0 / 6.0);
            const double p45 = fma(t, 1.0 / 720.0, 1.0 / 120.0), p67 = fma(t, 1.0 / 40320.0, 1.0 / 5040.0);
            const double lo = fma(t2, p23, p01), hi = fma(t2, p67, p45);
            double u = t * fma(t4, hi, lo);
            u = fma(u, u, u + u);
            return 1.0 + u;
        }
    }
    double q = 1.0 / 15.0;
    q = fma(q, z2, 1.0 / 13.0);
    q = fma(q, z2, 1.0 / 11.0);
    q = fma(q, z2, 1.0 / 9.0);
    q = fma(q, z2, 1.0 / 7.0);
    q = fma(q, z2, 1.0 / 5.0);
    q = fma(q, z2, 1.0 / 3.0);
    q = fma(q, z2, 1.0);
    const double y = (2.0 * k) * (z * q);
    if (!(fabs(y) <= 0.75)) return pow(x, k);
    const double t = 0.125 * y;
    double u = 1.0 / 3628800.0;  // 1/10!
    u = fma(u, t, 1.0 / 362880.0);
    u = fma(u, t, 1.0 / 40320.0);
    u = fma(u, t, 1.0 / 5040.0);
    u = fma(u, t, 1.0 / 720.0);
    u = fma(u, t, 1.0 / 120.0);
    u = fma(u, t, 1.0 / 24.0);
    u = fma(u, t, 1.0 / 6.0);
    u = fma(u, t, 0.5);
    u = fma(u, t, 1.0);
    u = u * t;
    u = fma(u, u, u + u);
    u = fma(u, u, u + u);
    u = fma(u, u, u + u);
    return 1.0 + u;
}

}  // namespace fvconv
