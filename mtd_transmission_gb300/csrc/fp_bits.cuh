// IEEE 754 binary32 <-> binary64 conversions done with integer operations.
//
// The GB300 FP64 pipe runs at a small fraction of the FP32 rate and the
// hardware conversions between float and double issue on it.  The cap
// accumulation adds in FP64 but its inputs and outputs are FP32, so it
// widens every hit and narrows every cell; doing both on the integer pipe
// leaves the FP64 pipe to the additions.  Both functions give the exact IEEE
// results: widening is exact, narrowing rounds to nearest, ties to even, with
// subnormal results, overflow to infinity and NaN handled as the standard
// says.  The header also compiles as plain C++ for the host-side check.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define TDM_FP_HD __host__ __device__ __forceinline__
#else
#define TDM_FP_HD inline
#endif

namespace tdm {

TDM_FP_HD uint64_t fp_bits(double d) {
    uint64_t b;
    std::memcpy(&b, &d, sizeof b);
    return b;
}
TDM_FP_HD double fp_double(uint64_t b) {
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
}
TDM_FP_HD uint32_t fp_bits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, sizeof b);
    return b;
}
TDM_FP_HD float fp_float(uint32_t b) {
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
}
TDM_FP_HD int fp_clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __clz((int)x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

// Exact float -> double.  Normal inputs take the short path; zero,
// subnormals, infinities and NaN the general one.
TDM_FP_HD double widen_any(float f) {
    const uint32_t u = fp_bits(f);
    const uint32_t ex = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    uint64_t body;
    if (ex != 0u) {
        // normal (biased exponent + 1023 - 127), or infinity / quiet NaN
        const uint32_t mq = (ex == 0xFFu && m) ? (m | 0x400000u) : m;
        body = ((uint64_t)(ex == 0xFFu ? 0x7FFu : ex + 896u) << 52) | ((uint64_t)mq << 29);
    } else if (m != 0u) {
        // subnormal m * 2^-149: leading bit p becomes the implicit one
        const int p = 31 - fp_clz32(m);
        body = ((uint64_t)(p + 874) << 52) | (((uint64_t)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
    } else {
        body = 0;
    }
    return fp_double(sign | body);
}

TDM_FP_HD double widen(float f) {
    const uint32_t u = fp_bits(f);
    if ((u & 0x7F800000u) - 0x00800000u < 0x7F000000u) {  // exponent field in [1, 254]
        const uint32_t hi = (u & 0x80000000u) | (((u & 0x7FFFFFFFu) >> 3) + (896u << 20));
        return fp_double(((uint64_t)hi << 32) | (uint64_t)(u << 29));
    }
    return widen_any(f);
}

// double -> float, round to nearest, ties to even.  narrow() takes the short
// path when the result is a normal float before rounding, narrow_any() covers
// every input.
TDM_FP_HD float narrow_any(double d) {
    const uint64_t b = fp_bits(d);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7FF);
    const uint64_t m = b & 0xFFFFFFFFFFFFFull;
    if (ex == 0x7FF) return fp_float(sign | 0x7F800000u | (m ? 0x400000u | (uint32_t)(m >> 29) : 0u));
    const int fe = ex - 896;  // float biased exponent
    if (fe >= 0xFF) return fp_float(sign | 0x7F800000u);
    uint64_t rem, half;
    uint32_t q;
    if (fe > 0) {
        q = ((uint32_t)fe << 23) | (uint32_t)(m >> 29);
        rem = m & 0x1FFFFFFFull;
        half = 0x10000000ull;
    } else {
        // subnormal or zero result: significand with its implicit bit, in
        // units of 2^-149 after a right shift by 30 - fe (>= 30)
        if (ex == 0 || fe < -30) return fp_float(sign);
        const uint64_t sig = m | (1ull << 52);
        const int sh = 30 - fe;
        q = (uint32_t)(sig >> sh);
        rem = sig & ((1ull << sh) - 1);
        half = 1ull << (sh - 1);
    }
    q += (rem > half || (rem == half && (q & 1u))) ? 1u : 0u;  // a carry into the exponent is correct
    return fp_float(sign | q);
}

TDM_FP_HD float narrow(double d) {
    const uint64_t b = fp_bits(d);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    if ((hi & 0x7FF00000u) - (897u << 20) < (254u << 20)) {  // double exponent in [897, 1150]
        uint32_t q = (((hi & 0x7FFFFFFFu) - (896u << 20)) << 3) | (lo >> 29);
        q += ((lo & 0x1FFFFFFFu) + (q & 1u)) > 0x10000000u ? 1u : 0u;  // ties to even
        return fp_float((hi & 0x80000000u) | q);
    }
    return narrow_any(d);
}

}  // namespace tdm
