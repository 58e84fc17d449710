// Host-side check of the cap accumulation's integer float <-> double
// conversions (short and general paths) against the host's IEEE conversions:
// every float for the widening; for the narrowing, doubles at and around
// every rounding boundary of every float exponent (ties, subnormal results,
// overflow) plus random bit patterns.  Prints "ok" or the first mismatch.
// Built and run by test_fp_bits.py.
#include <cmath>
#include <cstdio>
#include <random>

#include "fp_bits.cuh"

using namespace tdm;

static bool same(float a, float b) { return (std::isnan(a) && std::isnan(b)) || fp_bits(a) == fp_bits(b); }
static bool same(double a, double b) { return (std::isnan(a) && std::isnan(b)) || fp_bits(a) == fp_bits(b); }

static int check_narrow(uint64_t bits) {
    const double d = fp_double(bits);
    if (!same(narrow(d), (float)d) || !same(narrow_any(d), (float)d)) {
        std::printf("narrow mismatch: %016llx -> %08x, host %08x\n", (unsigned long long)bits,
                    fp_bits(narrow(d)), fp_bits((float)d));
        return 1;
    }
    return 0;
}

int main() {
    for (uint64_t u = 0; u <= 0xFFFFFFFFull; ++u) {
        const float f = fp_float((uint32_t)u);
        if (!same(widen(f), (double)f) || !same(widen_any(f), (double)f)) {
            std::printf("widen mismatch: %08x\n", (unsigned)u);
            return 1;
        }
    }
    // around every float boundary: for each float x (strided through all
    // exponents), x's double image and the midpoints to its neighbours, +-0..2 ulp
    for (uint64_t u = 0; u < 0x7F800000ull; u += 97) {
        for (int s = 0; s < 2; ++s) {
            const uint64_t db = fp_bits(widen(fp_float((uint32_t)u))) | ((uint64_t)s << 63);
            const uint64_t mid = db + (1ull << 28);  // halfway to the next float (normal range)
            for (int k = -2; k <= 2; ++k)
                if (check_narrow(db + k) || check_narrow(mid + k)) return 1;
        }
    }
    // subnormal results, the overflow boundary, tiny and huge doubles
    for (int ex = 0; ex < 2048; ++ex)
        for (uint64_t m : {0ull, 1ull, 0x8000000000000ull, 0x10000000ull, 0x10000001ull, 0xFFFFFFFFFFFFFull,
                           0x0FFFFFFFull, 0x30000000ull, 0x20000000ull, 0x7FFFFFFFFFFFFull})
            for (uint64_t s = 0; s < 2; ++s)
                if (check_narrow((s << 63) | ((uint64_t)ex << 52) | m)) return 1;
    for (int ex = 860; ex <= 900; ++ex)  // every tie of the subnormal range
        for (int sh = 0; sh < 53; ++sh)
            for (int k = -1; k <= 1; ++k)
                if (check_narrow(((uint64_t)ex << 52) | (((1ull << sh) + k) & 0xFFFFFFFFFFFFFull))) return 1;
    std::mt19937_64 rng(7);
    for (int i = 0; i < 20000000; ++i)
        if (check_narrow(rng())) return 1;
    std::printf("ok\n");
    return 0;
}
