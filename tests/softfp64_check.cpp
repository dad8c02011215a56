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

// add_pos over pos_ok operands: exponent gaps 0..60 (beyond the far limit),
// zeros, half-way patterns, carries into the next binade, values near 2^1022.
static void posPair(uint64_t seed, uint64_t i, double &a, double &b) {
    uint64_t r0 = mix(seed + 4 * i + 1), r1 = mix(seed + 4 * i + 2), r2 = mix(seed + 4 * i + 3);
    uint64_t ea = 1 + (r2 & 0x3FF) % 0x7FC, gap = (r2 >> 12) % 61;
    uint64_t eb = ea > gap ? ea - gap : 1;
    uint64_t A = (ea << 52) | (r0 & sf::MANT), B = (eb << 52) | (r1 & sf::MANT);
    switch ((r2 >> 20) & 7) {
        case 0: B = 0; break;                                            // x + 0
        case 1: B = (eb << 52) | (r1 & 0x000FFFFFFFF00000ull); break;   // few low bits: exact or tie
        case 2: A |= 0x000FFFFFFFFFFFF0ull; break;                       // carry out of the significand
        case 3: B = (eb << 52) | (1ull << ((r2 >> 24) % 52)); break;     // single bit: half-way cases
        case 4: A = (0x7FDull << 52) | (r0 & sf::MANT); B = (0x7FDull << 52) | (r1 & sf::MANT); break;
        case 5: A = sf::bits((double)(r0 >> 11) * (1.0 / 9007199254740992.0)); B = sf::bits((double)(r1 >> 11) * (1.0 / 9007199254740992.0)); break;
        default: break;
    }
    a = sf::from(A);
    b = sf::from(B);
    if ((r2 >> 40) & 1) { double t = a; a = b; b = t; }
}

extern "C" long softfp64_check_pos(long n, uint64_t seed) {
    long bad = 0;
    for (long i = 0; i < n; i++) {
        double a, b;
        posPair(seed, (uint64_t)i, a, b);
        if (!sf::pos_ok(a) || !sf::pos_ok(b)) { bad++; continue; }
        bad += !same(sf::add_pos(a, b), a + b);
    }
    // chains of additions of [0,1) values: the stencil's use
    for (long i = 0; i < n / 16; i++) {
        double s = 0.0, t = 0.0;
        for (int q = 0; q < 6; q++) {
            double v = (double)(mix(seed ^ (uint64_t)(i * 8 + q)) >> 11) * (1.0 / 9007199254740992.0);
            s = sf::add_pos(s, v);
            t = t + v;
        }
        bad += !same(s, t);
    }
    return bad;
}

// scale_up(x, 2) == x * 4.0 wherever scale_up_ok(x, 2); pos_small implies pos_ok
extern "C" long softfp64_check_scale(long n, uint64_t seed) {
    long bad = 0;
    for (long i = 0; i < n; i++) {
        uint64_t r = mix(seed + 2 * i + 1), q = mix(seed + 2 * i + 2);
        uint64_t X = r;
        switch (q & 7) {
            case 0: X &= sf::SIGN; break;                                          // +-0
            case 1: X = (X & 0x800FFFFFFFFFFFFFull); break;                         // subnormal
            case 2: X = (X & 0x800FFFFFFFFFFFFFull) | (0x7FCull << 52); break;      // largest that scales
            case 3: X = (X & 0x800FFFFFFFFFFFFFull) | (0x7FDull << 52); break;      // would overflow
            case 4: X |= 0x7FF0000000000000ull; break;                              // inf / nan
            default: break;
        }
        double x = sf::from(X);
        if (sf::scale_up_ok(x, 2)) bad += !same(sf::scale_up(x, 2), x * 4.0);
        if ((q & 7) == 1 && (X & ~sf::SIGN) != 0) bad += sf::scale_up_ok(x, 2);  // subnormals must be refused
        if ((q & 7) == 3) bad += sf::scale_up_ok(x, 2);
        if (sf::pos_small(x)) bad += !sf::pos_ok(x) || x < 0.0 || x >= 0x1p1009;
    }
    return bad;
}

// q61 chains: ((((a + b) + c) + d) + e) + f, then / 6, for q61_ok operands
// (exponent fields 1014..1022 or +0, mantissas with random, sparse or
// all-ones low bits so that ties and carries into the next binade occur)
static double q61Operand(uint64_t r, uint64_t q) {
    if ((q & 15) == 0) return 0.0;
    uint64_t e = 1014 + (q >> 4) % 9, m = r & sf::MANT;
    switch ((q >> 12) & 3) {
        case 0: m &= ~((1ull << ((q >> 16) % 53)) - 1); break;  // few significant low bits
        case 1: m |= (1ull << ((q >> 16) % 52)) - 1; break;     // runs of ones
        default: break;
    }
    return sf::from((e << 52) | m);
}

extern "C" long softfp64_check_q61(long n, uint64_t seed) {
    volatile double six = 6.0;
    volatile uint32_t one = 1, two = 2;
    sf::Q61Round tab[sf::Q61_ROUND_ENTRIES];
    for (int e = 0; e < sf::Q61_ROUND_ENTRIES; e++) tab[e] = sf::q61_round_entry(e);
    long bad = 0;
    for (long i = 0; i < n; i++) {
        double v[6];
        for (int k = 0; k < 6; k++) v[k] = q61Operand(mix(seed + 12 * i + 2 * k), mix(seed + 12 * i + 2 * k + 1));
        double t = v[0];
        uint64_t s = sf::q61(v[0]), st = s;
        for (int k = 0; k < 6; k++) {
            if (!sf::q61_ok(v[k]) || sf::q61_to(sf::q61(v[k])) != v[k]) bad++;
            if (k == 0) continue;
            t = t + v[k];
            s = sf::q61_add(s, sf::q61(v[k]));
            st = sf::q61_add_t(st, sf::q61(v[k]), tab, one, two);
            bad += !same(sf::q61_to(s), t) + (st != s);
        }
        bad += !same(sf::q61_div6(s), t / six) + !same(sf::div6_fma(sf::q61_to(s)), t / six);
    }
    // the range test refuses everything outside [2^-9, 1) and +0
    const double outside[] = {-0.0, -0.5, 1.0, 1.5, 0x1p-10, 0x1.fffffffffffffp-10, 5e-324, 1e300};
    for (double x : outside) bad += sf::q61_ok(x);
    const double inside[] = {0.0, 0x1p-9, 0x1.fffffffffffffp-1, 0.5, 0.1};
    for (double x : inside) bad += !sf::q61_ok(x);
    return bad;
}

// RN(x / 6) by div6_fma against the host FPU's division: q61 stencil sums
// (six operands of q61Operand, summed left to right), and normal doubles with
// random significands and exponents in (-1000, 1000), both signs
extern "C" long softfp64_check_div6_fma(long n, uint64_t seed) {
    volatile double six = 6.0;
    long bad = 0;
    for (long i = 0; i < n; i++) {
        double t = q61Operand(mix(seed + 14 * i), mix(seed + 14 * i + 1));
        for (int k = 1; k < 6; k++) t = t + q61Operand(mix(seed + 14 * i + 2 * k), mix(seed + 14 * i + 2 * k + 1));
        bad += !same(sf::div6_fma(t), t / six);
        const uint64_t r = mix(seed + 14 * i + 12), q = mix(seed + 14 * i + 13);
        const double x = sf::from(((q & 1) << 63) | ((uint64_t)(1023 - 999 + (q >> 1) % 1998) << 52) | (r & sf::MANT));
        bad += !same(sf::div6_fma(x), x / six);
    }
    const double edge[] = {0.0, 0x1p-9, 0x1.fffffffffffffp-1, 6.0 - 0x1p-50, 3.0, 6.0, 0x1.5555555555555p-3, 0x1p-999,
                           0x1.fffffffffffffp999};
    for (double x : edge) bad += !same(sf::div6_fma(x), x / six);
    return bad;
}
