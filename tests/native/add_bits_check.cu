// Host-side checks of the ray walk's integer-pipe arithmetic
// (opensss_gb300/csrc/trace.cuh):
//  * sss::add_nonneg_bits against the host's IEEE binary64 addition (round
//    to nearest even) on seeded random operands of every kind the walk can
//    meet -- equal and distant exponents, near-equal values, subnormals, and
//    running sums of walk-like steps;
//  * sss::ceil_clear (the ceiling of a voxel quotient from a product with
//    the reciprocal) against ceil of the host's division, on coordinates in
//    and around grids of several voxel sizes, voxel faces included;
//  * sss::div_bits against the host's IEEE binary64 division: operands of
//    random exponents and signs, one binade, near-equal significands,
//    divisors with trailing zero bits, exact quotients and zero dividends.
// Prints the number of cases and of mismatches; exits non-zero on any.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "trace.cuh"

static uint64_t bits_of(double x)
{
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}

static double double_of(uint64_t u)
{
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

int main(int argc, char** argv)
{
    const long cases = argc > 1 ? std::atol(argv[1]) : 4000000;
    std::mt19937_64 rng(20261204);
    constexpr uint64_t kPos = 0x7FFFFFFFFFFFFFFFull, kFrac = 0x000FFFFFFFFFFFFFull;
    long checked = 0, bad = 0;
    auto check = [&](uint64_t x, uint64_t y) {
        if ((x >> 52) == 0x7FF || (y >> 52) == 0x7FF) return;
        const double s = double_of(x) + double_of(y);
        if (!(s < 8.98846567431158e307)) return;  // the walk keeps sums below 2^1023
        const uint64_t got = sss::add_nonneg_bits(x, y);
        ++checked;
        if (got != bits_of(s)) {
            if (bad < 8)
                std::printf("mismatch %016llx + %016llx: %016llx, IEEE %016llx\n", (unsigned long long)x,
                            (unsigned long long)y, (unsigned long long)got, (unsigned long long)bits_of(s));
            ++bad;
        }
    };
    for (long i = 0; i < cases; ++i) {
        uint64_t x = rng() & kPos, y = rng() & kPos;
        switch (i % 6) {
        case 1:  // same exponent
            y = (x & ~kFrac) | (rng() & kFrac);
            break;
        case 2:  // within a few ulps
            y = (x + (rng() % 64) - 32) & kPos;
            break;
        case 3: {  // exponent difference below 60
            const uint64_t e = x >> 52, e2 = e > 60 ? e - rng() % 60 : e;
            y = (e2 << 52) | (rng() & kFrac);
            break;
        }
        case 4:  // subnormal operands and sums crossing into the normal range
            x &= kFrac;
            y &= 0x001FFFFFFFFFFFFFull;
            break;
        case 5:  // parameters near 1 plus voxel steps
            x = (x & 0x3FFFFFFFFFFFFFFFull) | 0x3000000000000000ull;
            y = (y & kFrac) | ((uint64_t)(0x3FF - rng() % 70) << 52);
            break;
        default:
            break;
        }
        check(x, y);
    }
    // running sums as a walk forms them: a start near 0 plus a fixed step
    std::uniform_real_distribution<double> start(0.0, 1e-3), step(1e-4, 0.2);
    for (int r = 0; r < 4000; ++r) {
        double t = start(rng);
        const double d = step(rng);
        for (int k = 0; k < 300; ++k) {
            check(bits_of(t), bits_of(d));
            t = t + d;
        }
    }
    // voxel quotients: ceil((c - lo) / vs) for coordinates on and around the
    // voxel faces of grids with awkward voxel sizes
    long long deferred = 0, ceils = 0;
    const double sizes[] = {0.6, 0.4, 1.0, 2.0 / 3.0, 40.0 / 37.0, 0.15625, 3.1, 51.0 / 17.0};
    std::uniform_int_distribution<int> face(-3, 140);
    std::uniform_real_distribution<double> jitter(-1e-9, 1e-9), any(-60.0, 60.0);
    for (double vs : sizes) {
        const double lo = -vs * 64.0, inv = 1.0 / vs;
        for (int i = 0; i < 400000; ++i) {
            double c;
            switch (i % 4) {
            case 0: c = lo + face(rng) * vs; break;                              // on a face
            case 1: c = (face(rng) + 1) * 2 * (vs * 32.0) / 64.0 - vs * 32.0; break; // scatter-point form
            case 2: c = lo + face(rng) * vs + jitter(rng); break;                // next to a face
            default: c = any(rng); break;
            }
            const double num = c - lo;
            long long k = 0;
            ++ceils;
            if (!sss::ceil_clear(num * inv, k)) {
                ++deferred;
                continue;
            }
            if ((double)k != std::ceil(num / vs)) {
                if (bad < 8) std::printf("ceil mismatch vs=%.17g c=%.17g: %lld, division %.17g\n", vs, c, k,
                                         std::ceil(num / vs));
                ++bad;
            }
        }
    }
    std::printf("ceilings %lld, deferred to the division %lld\n", ceils, deferred);
    // divisions
    long long divs = 0, div_deferred = 0;
    auto check_div = [&](double x, double y) {
        uint64_t q = 0;
        if (!sss::div_bits(bits_of(x), bits_of(y), q)) {
            ++div_deferred;
            return;
        }
        ++divs;
        if (q != bits_of(x / y)) {
            if (bad < 8) std::printf("div mismatch %.17g / %.17g: %.17g, IEEE %.17g\n", x, y, double_of(q), x / y);
            ++bad;
        }
    };
    std::uniform_real_distribution<double> wide(-100.0, 100.0), unit(0.1, 10.0);
    for (long i = 0; i < cases; ++i) {
        uint64_t x = rng(), y = rng();
        switch (i % 5) {
        case 0:  // exponents over a wide range, any signs
            x = (x & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(900 + rng() % 300) << 52);
            y = (y & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(900 + rng() % 300) << 52);
            break;
        case 1:  // one binade
            x = (x & 0x800FFFFFFFFFFFFFull) | (1023ull << 52);
            y = (y & 0x800FFFFFFFFFFFFFull) | (1023ull << 52);
            break;
        case 2:  // near-equal significands
            y = (y & 0x800FFFFFFFFFFFFFull) | (1023ull << 52);
            x = ((y & kFrac) + rng() % 7 - 3) | (1023ull << 52);
            break;
        case 3: {  // set-up-like operands
            const double a = wide(rng), b = wide(rng);
            check_div(a, b);
            check_div(1.0, b);
            check_div(0.6, b);
            continue;
        }
        default:  // divisors with trailing zero bits
            y = ((y & kFrac) | (1023ull << 52)) & ~((1ull << (rng() % 50)) - 1);
            x = (x & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1000 + rng() % 40) << 52);
            break;
        }
        check_div(double_of(x), double_of(y));
    }
    for (int i = 0; i < 200000; ++i) {  // exact quotients and zero dividends
        const double y = unit(rng), k = (double)(rng() % 1000);
        check_div(k * y, y);
        check_div(0.0, y);
        check_div(-0.0, y);
    }
    std::printf("divisions %lld, deferred to FP64 %lld\n", divs, div_deferred);
    std::printf("checked %ld, mismatches %ld\n", checked, bad);
    return bad != 0;
}
