// Host harness for tests/test_softfp64.py: the integer-pipe FP64 operations of
// csrc/kernels/softfp64.cuh, compiled for the host, against the host FPU
// (IEEE binary64, round-to-nearest-even; compiled with -ffp-contract=off).
#include <cstdint>

#include "../dvm-snapshot-r6603-fork_gb300/csrc/kernels/softfp64.cuh"

static uint64_t mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void pair(uint64_t seed, uint64_t i, double &a, double &b) {
    uint64_t r0 = mix(seed + 4 * i + 1), r1 = mix(seed + 4 * i + 2), r2 = mix(seed + 4 * i + 3);
    uint64_t A = r0, B = r1;
    switch (r2 & 7) {
        case 0: break;
        case 1: B = ((A & 0xFFF0000000000000ull) ^ ((r2 >> 8) & 0x0030000000000000ull)) | (r1 & sf::MANT); break;
        case 2: B = (A ^ sf::SIGN) ^ (r1 & ((1ull << ((r2 >> 8) % 53)) - 1)); break;
        case 3:
            A = sf::bits((double)(r0 >> 11) * (1.0 / 9007199254740992.0));
            B = sf::bits((double)(r1 >> 11) * (1.0 / 9007199254740992.0) * (double)((r2 >> 8) & 15));
            break;
        case 4: B = (A & 0x800FFFFFFFFFFFFFull) | ((((A >> 52) & 0x7FF) - ((r2 >> 8) % 70)) & 0x7FF) << 52; break;
        case 5: A |= 0x000FFFFFFFFFFF00ull; B = (A & 0xFFF0000000000000ull) | (r1 & 0xFFull); break;
        case 6:
            A = (A & 0x800FFFFFFFFFFFFFull) | ((r2 >> 8) % 4 + 1) << 52;
            B = (B & 0x800FFFFFFFFFFFFFull) | (0x7FEull - (r2 >> 16) % 3) << 52;
            break;
        default: B = (A & 0x8000000000000000ull) | ((((A >> 52) & 0x7FF) - 53) & 0x7FF) << 52; break;
    }
    a = sf::from(A);
    b = sf::from(B);
}

static bool same(double x, double y) {
    uint64_t X = sf::bits(x), Y = sf::bits(y);
    return X == Y || ((X & ~sf::SIGN) > sf::EXPINF && (Y & ~sf::SIGN) > sf::EXPINF);
}

extern "C" void softfp64_check(long n, uint64_t seed, long bad[4]) {
    volatile double six = 6.0;  // a real division, not a constant-folded one
    for (int k = 0; k < 4; k++) bad[k] = 0;
    for (long i = 0; i < n; i++) {
        double a, b;
        pair(seed, (uint64_t)i, a, b);
        bad[0] += !same(sf::add(a, b), a + b);
        bad[1] += !same(sf::sub(a, b), a - b);
        bad[2] += !same(sf::mul(a, b), a * b);
        bad[3] += !same(sf::div3p2(a, 1), a / six);
    }
}
