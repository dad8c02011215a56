// IEEE-754 binary64 arithmetic on the integer pipe, bit-exact with the FP64
// unit in round-to-nearest-even.
//
// Why: a GB300 SM executes 2 FP64 thread-operations per clock but 128
// integer/FP32 thread-operations per clock.  An FP64 stencil therefore runs
// out of FP64 issue long before it runs out of HBM bandwidth.  Moving part of
// the FP64 operations of a cell onto the integer pipe -- with results
// identical bit for bit -- lets both pipes work at once.
//
// Method (standard binary floating-point arithmetic, e.g. Goldberg 1991,
// "What every computer scientist should know about floating-point arithmetic";
// Muller et al., Handbook of Floating-Point Arithmetic, ch. 7-8): unpack the
// 53-bit significands, align with a sticky bit, add/multiply exactly in
// 64/128-bit integers, normalise, round to nearest even on the guard bit and
// the sticky OR of the rest, repack.  Only the common case is emulated: both
// operands and the result normal and finite.  Zeros, subnormals, infinities,
// NaNs and results that would overflow or underflow take the native FP64
// instruction, so the edge semantics are the hardware's by construction.
//
// sf_div3p2(x, k) = RN(x / (3 * 2^k)) (k >= 0): the exact quotient
// floor(m * 2^11 / 3) of the significand by the multiply-high reciprocal
// identity floor(n / 3) = floor(mulhi(n, 0xAAAAAAAAAAAAAAAB) / 2) for 64-bit n,
// the remainder for the sticky bit, then rounding.  A quotient by 3 is never
// exactly half-way between two doubles (the denominator is odd), so ties do
// not arise; the rounding code still implements ties-to-even.
//
// The same source compiles for the host (the self-tests check it against the
// host FPU) and for the device.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SF_HD __host__ __device__ __forceinline__
#else
#define SF_HD static inline
#endif

namespace sf {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t MANT = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t HID = 0x0010000000000000ull;
constexpr uint64_t EXPINF = 0x7FF0000000000000ull;

SF_HD uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

SF_HD double from(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

SF_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

SF_HD uint64_t mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// The FP64 unit's own operations, as volatile inline PTX: the compiler may not
// execute them speculatively, so an emulated operation never also issues the
// native instruction it replaces.
SF_HD double nadd(double a, double b) {
#ifdef __CUDA_ARCH__
    double r;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
#else
    return a + b;
#endif
}
SF_HD double nmul(double a, double b) {
#ifdef __CUDA_ARCH__
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
#else
    return a * b;
#endif
}
SF_HD double ndiv(double a, double b) {
#ifdef __CUDA_ARCH__
    double r;
    asm volatile("div.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
#else
    return a / b;
#endif
}

// RN(a + b)
SF_HD double add(double a, double b) {
    uint64_t A = bits(a), B = bits(b);
    uint64_t ea = (A >> 52) & 0x7FF, eb = (B >> 52) & 0x7FF;
    if (ea - 1 >= 0x7FE || eb - 1 >= 0x7FE) return nadd(a, b);  // zero, subnormal, inf, nan
    uint64_t absA = A & ~SIGN, absB = B & ~SIGN;
    if (absA < absB) {
        uint64_t t = A; A = B; B = t;
        t = ea; ea = eb; eb = t;
    }
    uint64_t d = ea - eb;
    if (d > 63) return from(A);  // |b| < ulp(a)/2^10: RN(a+b) = a
    uint64_t ma = ((A & MANT) | HID) << 8;  // leading one at bit 60
    uint64_t mb = ((B & MANT) | HID) << 8;
    if (d) {
        uint64_t lost = mb << (64 - d);
        mb = (mb >> d) | (uint64_t)(lost != 0);
    }
    uint64_t s = ((A ^ B) & SIGN) ? ma - mb : ma + mb;
    if (s == 0) return 0.0;  // x + (-x) = +0 in round-to-nearest
    int lz = clz64(s);
    int64_t e = (int64_t)ea;
    if (lz == 2) {
        s = (s >> 1) | (s & 1);
        e += 1;
    } else if (lz > 3) {
        // exact: either no bit was lost (d <= 1) or the shift is one place and
        // the sticky bit stays below the guard bit
        s <<= (lz - 3);
        e -= (lz - 3);
    }
    if (e <= 0) return nadd(a, b);  // subnormal result
    uint64_t m = s >> 8;
    uint32_t rem = (uint32_t)(s & 0xFF);
    m += (uint64_t)((rem > 0x80) | ((rem == 0x80) & (uint32_t)(m & 1)));
    if (m >> 53) {
        m >>= 1;
        e += 1;
    }
    if (e >= 0x7FF) return nadd(a, b);  // overflow
    return from((A & SIGN) | ((uint64_t)e << 52) | (m & MANT));
}

SF_HD double sub(double a, double b) { return add(a, from(bits(b) ^ SIGN)); }

// RN(a * b)
SF_HD double mul(double a, double b) {
    uint64_t A = bits(a), B = bits(b);
    uint64_t ea = (A >> 52) & 0x7FF, eb = (B >> 52) & 0x7FF;
    if (ea - 1 >= 0x7FE || eb - 1 >= 0x7FE) return nmul(a, b);
    uint64_t ma = (A & MANT) | HID, mb = (B & MANT) | HID;
    uint64_t lo = ma * mb, hi = mulhi(ma, mb);  // product in [2^104, 2^106)
    int64_t e = (int64_t)ea + (int64_t)eb - 1023;
    uint64_t m, guard, sticky;
    if (hi >> 41) {  // bit 105 set
        m = (hi << 11) | (lo >> 53);
        guard = (lo >> 52) & 1;
        sticky = lo & ((1ull << 52) - 1);
        e += 1;
    } else {
        m = (hi << 12) | (lo >> 52);
        guard = (lo >> 51) & 1;
        sticky = lo & ((1ull << 51) - 1);
    }
    if (e <= 0) return nmul(a, b);  // subnormal or zero result: rounded at a coarser position
    m += guard & (uint64_t)((sticky != 0) | (m & 1));
    if (m >> 53) {
        m >>= 1;
        e += 1;
    }
    if (e >= 0x7FF) return nmul(a, b);  // overflow
    return from(((A ^ B) & SIGN) | ((uint64_t)e << 52) | (m & MANT));
}

// RN(x / (3 * 2^k)), k >= 0
SF_HD double div3p2(double x, int k) {
    uint64_t X = bits(x);
    uint64_t ex = (X >> 52) & 0x7FF;
    if (ex - 1 >= 0x7FE) return ndiv(x, 3.0 * (double)(1ull << k));
    uint64_t n = ((X & MANT) | HID) << 11;  // in [2^63, 2^64)
    uint64_t q = mulhi(n, 0xAAAAAAAAAAAAAAABull) >> 1;
    uint64_t r = n - 3 * q;
    int64_t e;
    uint64_t m, guard, sticky;
    if (q >> 62) {
        m = q >> 10;
        guard = (q >> 9) & 1;
        sticky = (q & 0x1FF) | r;
        e = (int64_t)ex - 1;
    } else {
        m = q >> 9;
        guard = (q >> 8) & 1;
        sticky = (q & 0xFF) | r;
        e = (int64_t)ex - 2;
    }
    e -= k;
    if (e <= 0) return ndiv(x, 3.0 * (double)(1ull << k));  // subnormal result
    m += guard & (uint64_t)((sticky != 0) | (m & 1));
    if (m >> 53) {
        m >>= 1;
        e += 1;
    }
    return from((X & SIGN) | ((uint64_t)e << 52) | (m & MANT));
}

// RN(x * 2^-k) for 0 < k < 64: exact exponent decrement while the result stays
// normal (x / 4.0 and x * 0.25 are the same correctly rounded value)
SF_HD double scale_down(double x, int k) {
    uint64_t X = bits(x);
    uint64_t ex = (X >> 52) & 0x7FF;
    if (ex <= (uint64_t)k || ex == 0x7FF) return nmul(x, from((uint64_t)(1023 - k) << 52));
    return from(X - ((uint64_t)k << 52));
}

// ---------------------------------------------------------------- branch-free fast paths
//
// add_fast / div3p2_fast / scale_down_fast compute the result with integer
// operations only and never issue an FP64 instruction, including for a zero
// operand (x + 0 = x) and far-apart exponents.  They OR `special` with true
// when the result may be wrong: a subnormal, infinite or NaN operand, a sum of
// two zeros, a subnormal or overflowing result.  The caller then recomputes
// that element with the native operations in a warp-uniform branch (rare), so
// the FP64 unit sees no predicated-off instruction in the common path.

SF_HD uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }

SF_HD double add_fast(double a, double b, bool &special) {
    uint64_t A = bits(a), B = bits(b);
    uint64_t absA = A & ~SIGN, absB = B & ~SIGN;
    bool swp = absA < absB;
    uint64_t X = swp ? B : A, Y = swp ? A : B;  // |X| >= |Y|
    uint32_t ex = (hi32(X) >> 20) & 0x7FF, ey = (hi32(Y) >> 20) & 0x7FF;
    bool yzero = (Y & ~SIGN) == 0;
    // Y may be a zero (X + 0 = X); any other subnormal, inf or nan is special
    special |= (ex - 1 >= 0x7FE) | ((ey - 1 >= 0x7FE) & !yzero);
    uint32_t d = ex - ey;
    bool far = yzero | (d > 63);  // RN(x + y) = x
    uint32_t dd = far ? 0 : d;
    uint64_t mx = ((X & MANT) | HID) << 8, my = ((Y & MANT) | HID) << 8;
    uint64_t lost = dd ? (my << (64 - dd)) : 0;
    my = (my >> dd) | (uint64_t)(lost != 0);
    bool subtr = ((X ^ Y) & SIGN) != 0;
    uint64_t s = subtr ? mx - my : mx + my;
    int lz = clz64(s);
    bool carry = lz == 2;
    int sh = carry ? 0 : lz - 3;
    uint64_t sn = carry ? ((s >> 1) | (s & 1)) : (s << (sh & 63));
    int e = (int)ex + (carry ? 1 : -sh);
    uint64_t m = sn >> 8;
    uint32_t rem = (uint32_t)sn & 0xFF;
    m += (uint64_t)((rem > 0x80) | ((rem == 0x80) & (uint32_t)(m & 1)));
    uint32_t c = (uint32_t)(m >> 53);
    m >>= c;
    e += (int)c;
    bool zero = s == 0;  // exact cancellation: +0 in round-to-nearest
    special |= !far & !zero & ((e <= 0) | (e >= 0x7FF));
    special |= yzero & ((X & ~SIGN) == 0);  // both zero: sign rules
    uint64_t r = (X & SIGN) | ((uint64_t)(uint32_t)e << 52) | (m & MANT);
    r = zero ? 0 : r;
    return from(far ? X : r);
}

SF_HD double sub_fast(double a, double b, bool &special) { return add_fast(a, from(bits(b) ^ SIGN), special); }

SF_HD double div3p2_fast(double x, int k, bool &special) {
    uint64_t X = bits(x);
    uint32_t ex = (hi32(X) >> 20) & 0x7FF;
    bool zero = (X & ~SIGN) == 0;
    uint64_t n = ((X & MANT) | HID) << 11;
    uint64_t q = mulhi(n, 0xAAAAAAAAAAAAAAABull) >> 1;
    uint64_t r = n - 3 * q;
    bool top = (q >> 62) != 0;
    int sh = top ? 10 : 9;
    uint64_t m = q >> sh;
    uint64_t guard = (q >> (sh - 1)) & 1;
    uint64_t sticky = (q & ((1ull << (sh - 1)) - 1)) | r;
    int e = (int)ex - (top ? 1 : 2) - k;
    special |= !zero & ((ex - 1 >= 0x7FE) | (e <= 0));
    m += guard & (uint64_t)((sticky != 0) | (m & 1));
    uint32_t c = (uint32_t)(m >> 53);
    m >>= c;
    e += (int)c;
    uint64_t res = (X & SIGN) | ((uint64_t)(uint32_t)e << 52) | (m & MANT);
    return from(zero ? X : res);
}

SF_HD double scale_down_fast(double x, int k, bool &special) {
    uint64_t X = bits(x);
    uint32_t ex = (hi32(X) >> 20) & 0x7FF;
    bool zero = (X & ~SIGN) == 0;
    special |= !zero & ((ex <= (uint32_t)k) | (ex == 0x7FF));
    return from(zero ? X : X - ((uint64_t)k << 52));
}

// ---------------------------------------------------------------- non-negative operands
//
// add_pos(x, y) = RN(x + y) for x, y each +0 or a positive normal double below
// 2^1022 ("pos_ok" below) -- the caller checks its inputs once (a tile of a
// stencil whose values are all non-negative), so the addition needs no sign,
// cancellation, subnormal or overflow handling: align the smaller significand
// with a sticky bit, add, renormalise by at most one bit, round to nearest
// even, repack (the significand's hidden bit carries into the exponent field,
// which also covers a rounding overflow to the next binade).  The sum of two
// pos_ok values is pos_ok again or 2^1022 <= s < 2^1023 (normal), so chains of
// additions stay exact as long as the partial sums stay below 2^1022.
SF_HD bool pos_ok(double x) {
    uint32_t h = hi32(bits(x));
    return (h >> 20) - 1 < 0x7FDu || bits(x) == 0;  // exponent 1..0x7FD and sign clear, or +0
}

SF_HD double add_pos(double a, double b) {
    uint64_t A = bits(a), B = bits(b);
    bool ab = A >= B;                          // integer order = value order here
    uint64_t X = ab ? A : B, Y = ab ? B : A;   // X >= Y
    uint32_t ex = hi32(X) >> 20, ey = hi32(Y) >> 20;
    uint32_t d = ex - ey;
    bool far = (ey == 0) | (d >= 54);          // y = 0, or y < ulp(x) / 2: RN(x + y) = x
    uint32_t dd = far ? 0 : d;
    uint64_t mx = ((X & MANT) | HID) << 10, my = ((Y & MANT) | HID) << 10;
    uint64_t lost = dd ? my << (64 - dd) : 0;  // the bits shifted out (sticky)
    uint64_t s = mx + ((my >> dd) | (uint64_t)(lost != 0));
    uint32_t carry = (uint32_t)(s >> 63);
    s = carry ? ((s >> 1) | (s & 1)) : s;      // top bit at 62, sticky kept in bit 0
    uint32_t g = (uint32_t)s & 0x7FF;          // bit 10: result lsb, bits 9..0: rounding bits
    uint64_t m = (s >> 10) + (uint64_t)(((g & 0x3FF) > 0x200) | (((g & 0x3FF) == 0x200) & (g >> 10)));
    uint64_t r = ((uint64_t)(ex + carry - 1) << 52) + m;
    return from(far ? X : r);
}

// pos_small: +0 or a positive normal below 2^1009 -- sums of up to 2^13 such
// values stay below 2^1022, so chains of add_pos over them stay exact.
SF_HD bool pos_small(double x) {
    uint32_t h = hi32(bits(x));
    return (h >> 20) - 1 < 0x7EFu || bits(x) == 0;  // exponent field 1..0x7EF: below 2^1009
}

// x * 2^k exactly for x = +-0 or a normal x whose exponent field is at most
// 0x7FE - k (scale_up_ok); the exponent field is incremented by k.
SF_HD bool scale_up_ok(double x, int k) {
    uint32_t e = (hi32(bits(x)) >> 20) & 0x7FF;
    return (e - 1 < (uint32_t)(0x7FE - k)) || (bits(x) & ~SIGN) == 0;
}
SF_HD double scale_up(double x, int k) {
    uint64_t X = bits(x);
    return (X & ~SIGN) == 0 ? x : from(X + ((uint64_t)k << 52));
}

// x * 2^64 as an exact 64-bit integer for x = +0 or 2^-12 <= x < 1 (such x are
// multiples of 2^-64 below 1); ok is cleared for any other x (result 0).
SF_HD uint64_t q64(double x, bool &ok) {
    uint64_t X = bits(x);
    uint32_t e = hi32(X) >> 20;  // the sign bit makes a negative x out of range
    bool in = e - 1011u <= 11u;
    ok &= in | (X == 0);
    return in ? ((X & MANT) | HID) << (e - 1011u) : 0;
}

// ---------------------------------------------------------------- 61-bit fixed point (stencil sums)
//
// A double x = +0 or 2^-9 <= x < 1 is an integer multiple of 2^-61 below 2^61
// (its last significand bit weighs at least 2^-9 * 2^-52), so q61(x) = x * 2^61
// is exact in a uint64.  Sums of up to six such values stay below 6 * 2^61 <
// 2^64.  In this form an FP64 addition of two q61-representable values is an
// integer addition (exact) followed by a rounding of the sum to 53
// significant bits, to nearest even: the bits below the sum's 53-bit
// significand are at most 11 (the sum is below 2^64), so the rounding touches
// the low 32-bit word and a carry.  RN(a + b) of the FP64 unit and
// q61_add(q61(a), q61(b)) are the same number, and the rounded sum is again a
// multiple of 2^-61, so chains of additions stay exact in this form.  The
// division by 6 of the stencil rounds the q61 sum straight to a double.
// (The rounding is the textbook round-to-nearest-even on a guard position:
// Goldberg 1991; Muller et al., Handbook of Floating-Point Arithmetic, ch. 2.)

SF_HD bool q61_ok(double x) {
    uint32_t h = hi32(bits(x));
    return (h >> 20) - 1014u <= 8u || bits(x) == 0;  // exponent field 1014..1022 and sign clear, or +0
}

// the high word of (hi:lo) << sh and the low word of (hi:lo) >> sh, sh < 32
SF_HD uint32_t fshl(uint32_t lo, uint32_t hi, uint32_t sh) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, sh);
#else
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << sh) >> 32);
#endif
}
SF_HD uint32_t fshr(uint32_t lo, uint32_t hi, uint32_t sh) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, sh);
#else
    return (uint32_t)((((uint64_t)hi << 32) | lo) >> sh);
#endif
}

// x * 2^61 for a q61_ok x (an arbitrary value for any other x): the
// significand shifted left by the exponent field - 1014 (0..8)
SF_HD uint64_t q61(double x) {
    const uint64_t X = bits(x);
    const uint32_t h = hi32(X), l = (uint32_t)X;
    const uint32_t sh = ((h >> 20) - 1014u) & 31u;
    const uint32_t mh = (h & 0xFFFFFu) | 0x100000u;  // the significand's high word with the hidden bit
    const uint64_t m = ((uint64_t)fshl(l, mh, sh) << 32) | (uint32_t)(l << sh);
    return X == 0 ? 0 : m;
}

// the index of the most significant set bit of a 32-bit word, -1 for 0
SF_HD int msb32(uint32_t x) {
#ifdef __CUDA_ARCH__
    int r;
    asm("bfind.u32 %0, %1;" : "=r"(r) : "r"(x));
    return r;
#else
    return x ? 31 - __builtin_clz(x) : -1;
#endif
}

// RN(s + t) for q61 operands whose exact sum is below 2^64
SF_HD uint64_t q61_add(uint64_t s, uint64_t t) {
    uint64_t u = s + t;
    int r = msb32((uint32_t)(u >> 32)) - 20;  // significant bits beyond 53 (msb index - 52)
    r = r < 0 ? 0 : r;
    const uint32_t lo = (uint32_t)u, m1 = 1u << r, mask = m1 - 1u;
    // half - 1 + lsb: carries into the kept bits iff the dropped part is above
    // half, or exactly half with an odd lsb; masked to 0 when nothing is dropped
    const uint32_t inc = ((m1 >> 1) - 1u + ((lo >> r) & 1u)) & mask;
    u += inc;
    return u & ~(uint64_t)mask;
}

// The same addition in the form the TMA-staged stencil uses.  There the
// q61 sums keep the integer ALU pipe busy (shifts, masks, compares) while the
// multiply-add pipe idles, so: the 64-bit additions are 32 x 32 + 64-bit
// multiply-adds by a `one` the compiler cannot see (they go to the
// multiply-add pipe), and the rounding constants come from a 33-entry table
// indexed by the position of the sum's leading bit (a shared-memory load).
// Rounding to nearest even by adding half: v = u + half carries into the kept
// bits iff the dropped part is at least half; it was exactly half iff v's
// dropped bits are then 0, and the tie goes to even by clearing v's last kept
// bit as well (it is already 0 when u's was 1, the carry having cleared it).
struct Q61Round {
    uint32_t half, mask;  // half of the last kept bit's weight (0: nothing dropped), the dropped bits
};
constexpr int Q61_ROUND_ENTRIES = 33;
// entry idx = msb(high word of the sum) + 1, 0 for a zero high word
SF_HD Q61Round q61_round_entry(int idx) {
    const int r = idx - 21 < 0 ? 0 : idx - 21;  // bits beyond 53 (msb index - 52)
    return Q61Round{r ? 1u << (r - 1) : 0u, (1u << r) - 1u};
}

// a * one + c in 64 bits (one == 1)
SF_HD uint64_t madw(uint32_t a, uint32_t one, uint64_t c) {
#ifdef __CUDA_ARCH__
    uint64_t d;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(one), "l"(c));
    return d;
#else
    return (uint64_t)a * one + c;
#endif
}
// a * b + c in 32 bits
SF_HD uint32_t mad32(uint32_t a, uint32_t b, uint32_t c) {
#ifdef __CUDA_ARCH__
    uint32_t d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
#else
    return a * b + c;
#endif
}

// q61_add(s, t); tab = the Q61_ROUND_ENTRIES entries q61_round_entry(0..32),
// one == 1, two == 2
SF_HD uint64_t q61_add_t(uint64_t s, uint64_t t, const Q61Round *tab, uint32_t one, uint32_t two) {
    const uint64_t u0 = madw((uint32_t)s, one, t);
    const uint32_t uh = mad32(hi32(s), one, hi32(u0));
    const uint64_t u = ((uint64_t)uh << 32) | (uint32_t)u0;
    const Q61Round e = tab[msb32(uh) + 1];
    const uint64_t v = madw(e.half, one, u);
    const uint32_t lo = (uint32_t)v;
    const uint32_t clr = (lo & e.mask) == 0 ? mad32(e.half, two, e.mask) : e.mask;  // tie: the last kept bit too
    return ((uint64_t)hi32(v) << 32) | (lo & ~clr);
}

// RN((s * 2^-61) / 6) for a q61 value s with at most 53 significant bits
// that is 0 or at least 2^32 -- every sum of q61 values is: a nonzero q61
// value is at least 2^52 (2^-9 * 2^61).  The quotient's significand comes
// from floor(n / 3) of s normalised to bit 63 (the multiply-high reciprocal
// identity), its rounding from the bits below and the remainder.
SF_HD double q61_div6(uint64_t s) {
    const uint32_t sh_ = hi32(s), sl = (uint32_t)s;
    const int c = 31 - msb32(sh_);  // leading zeros of s (32 for s == 0, handled at the end)
    const uint32_t cc = (uint32_t)c & 31u;
    const uint64_t n = ((uint64_t)fshl(sl, sh_, cc) << 32) | (uint32_t)(sl << cc);  // leading one at bit 63
    const uint64_t q = mulhi(n, 0xAAAAAAAAAAAAAAABull) >> 1;  // floor(n / 3), in [2^61, 2^63)
    const uint32_t r = (uint32_t)n - 3u * (uint32_t)q;         // n - 3q, in {0, 1, 2}
    const uint32_t qh = hi32(q), ql = (uint32_t)q;
    const uint32_t top = qh >> 30;  // q >= 2^62: the significand is q's bits 62..10, else 61..9
    const uint32_t sh = 9u + top;
    const uint32_t mh = qh >> sh, ml = fshr(ql, qh, sh);
    const uint32_t guard = (ql >> (sh - 1u)) & 1u;
    const uint32_t sticky = (ql & ((1u << (sh - 1u)) - 1u)) | r;
    const uint32_t inc = guard & (uint32_t)((sticky != 0) | (ml & 1u));
    const uint64_t m = (((uint64_t)mh << 32) | ml) + inc;
    const uint32_t e = (top ? 1023u : 1022u) - (uint32_t)c;  // exponent field of the quotient
    // the significand's leading one adds 1 to the exponent field; a rounding
    // carry to 2^53 adds 2, which is the next binade with a zero significand
    const uint64_t res = ((uint64_t)(e - 1u) << 52) + m;
    return from(s == 0 ? 0 : res);
}

// the double s * 2^-61 for a q61 value with at most 53 significant bits
SF_HD double q61_to(uint64_t s) {
    if (s == 0) return 0.0;
    const int c = clz64(s);
    const int p = 63 - c;  // msb index
    const uint64_t m = p >= 52 ? s >> (p - 52) : s << (52 - p);
    return from(((uint64_t)(p - 61 + 1023 - 1) << 52) + m);
}

// RN(x / 6) on the FP64 unit by one multiply and two fused multiply-adds:
// q = RN(x z) with z = RN(1/6) is within an ulp of x / 6, the residual
// r = x - 6 q is exact in an FMA, and RN(q + r z) is the correctly rounded
// quotient (Markstein's correction theorem: P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990; Muller et al., Handbook of Floating-Point Arithmetic,
// 2nd ed., sec. 4.7).  For x = +0 or a normal x with 2^-1000 < |x| < 2^1000
// (no underflow of r, no overflow); the stencil uses it for sums in [2^-9, 6)
// and +0.  Three FP64-unit operations instead of the integer pipe's ~40.
SF_HD double div6_fma(double x) {
    const double z = 0x1.5555555555555p-3;  // RN(1/6)
#ifdef __CUDA_ARCH__
    const double q = __dmul_rn(x, z);
    const double r = __fma_rn(-q, 6.0, x);
    return __fma_rn(r, z, q);
#else
    const double q = x * z;
    const double r = std::fma(-q, 6.0, x);
    return std::fma(r, z, q);
#endif
}

// Max(|t|, m) on bit patterns: for non-negative doubles the IEEE order is the
// unsigned integer order.  A NaN t leaves m unchanged, as (t > m ? t : m) does.
SF_HD uint64_t absmax_bits(double t, uint64_t m) {
    uint64_t b = bits(t) & ~SIGN;
    return (b <= EXPINF && b > m) ? b : m;
}

}  // namespace sf
