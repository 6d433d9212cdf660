// bgk_softfp64.h -- IEEE-754 binary64 addition and multiplication, round to nearest even, in
// 64-bit integer arithmetic.
//
// GB300 retires about 2 FP64 instructions per clock per SM, against 64 integer and 128 FP32
// lanes.  The exact FP64 collision (DOUBLE and MIXED2 builds) is therefore bound by the FP64
// pipe.  Moving part of its additions and multiplications to the integer pipes, as the
// operations defined here, raises the step rate while every result stays the IEEE result.
//
// Method: the textbook one for a binary floating-point format (IEEE 754-2008 §4.3.1, §5.4.1;
// e.g. Goldberg, "What every computer scientist should know about floating-point arithmetic",
// ACM Computing Surveys 23(1), 1991, on guard and sticky bits).  Significands with their hidden
// bit are held in 64-bit integers with 10 bits below the 53-bit significand for the sum (an
// exponent difference of at most 1 loses no bit; beyond that one sticky bit stands for every bit
// shifted out, which is enough for round-to-nearest-even of both sums and differences), and as the
// exact 106-bit integer product for the multiplication.
//
// Scope: finite operands whose result is a normal number, and zeros.  The functions return
// false, and leave the result to the hardware instruction, for subnormal, infinite or NaN
// operands and for results that overflow or fall below the normal range.  Such values do not
// occur in a running simulation; the callers (soft_add / soft_mul below) take the hardware path
// for them, so the value returned is the IEEE result in every case.
//
// The functions compile for the host as well, so tests/test_softfp64.py checks them against the
// host's IEEE double arithmetic bit for bit; the GPU tests check the device build against the
// GPU's own DADD and DMUL.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define SFP_HD __host__ __device__ __forceinline__
#else
#define SFP_HD static inline
#endif

namespace bgk {
namespace sfp {

constexpr uint64_t SIGN = 0x8000000000000000ull;
constexpr uint64_t FRAC = 0x000fffffffffffffull;
constexpr uint64_t HIDDEN = 0x0010000000000000ull;

SFP_HD int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// high 64 bits of the 128-bit product
SFP_HD uint64_t mulhi64(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Both operations are written without data-dependent branches (selects only), so that the lanes
// of a warp stay together whatever their operands; `ok` is false only for the cases left to the
// hardware.

// s: significand with its leading one at bit 62 and 10 bits below the 53-bit significand (the
// lowest of them sticky), biased exponent e.  Rounds to nearest even and packs the magnitude;
// clears ok when e is below the normal range (subnormal rounding is left to the hardware) or the
// rounded result overflows.
SFP_HD uint64_t round_pack(uint64_t s, int64_t e, bool &ok)
{
    ok = ok && e > 0;
    uint64_t m = s >> 10;
    const uint64_t rem = s & 0x3ffu;
    m += (rem > 0x200u || (rem == 0x200u && (m & 1u))) ? 1u : 0u;
    const uint64_t carry = m >> 53;  // rounding carried into a new leading bit
    m >>= carry;
    e += (int64_t)carry;
    ok = ok && e < 0x7ff;
    return ((uint64_t)e << 52) | (m & FRAC);
}

// a + b for the bit patterns a, b; true when *r holds the IEEE round-to-nearest-even sum
SFP_HD bool add(uint64_t a, uint64_t b, uint64_t *r)
{
    const uint64_t ma = a & ~SIGN, mb = b & ~SIGN;
    const bool swap = mb > ma;  // larger magnitude first
    const uint64_t hi = swap ? b : a, lo = swap ? a : b;
    const uint64_t mhi = swap ? mb : ma, mlo = swap ? ma : mb;
    const int64_t eh = (int64_t)(mhi >> 52), el = (int64_t)(mlo >> 52);
    // zero operands: x + 0 = x; two zeros give -0 only when both are -0
    const bool lo_zero = mlo == 0;
    bool ok = eh != 0x7ff && (el != 0 || lo_zero);  // no inf/nan, no subnormal operand
    const uint64_t sh = ((hi & FRAC) | HIDDEN) << 10;  // leading one at bit 62
    const uint64_t l0 = ((lo & FRAC) | HIDDEN) << 10;
    const int64_t d = eh - el < 63 ? eh - el : 63;   // beyond 63 only the sticky bit is left
    const uint64_t lost = l0 & ((1ull << d) - 1u);
    const uint64_t sl = (l0 >> d) | (lost != 0 ? 1u : 0u);
    const bool sub = ((a ^ b) & SIGN) != 0;
    uint64_t s = sub ? sh - sl : sh + sl;  // sum < 2^64; difference > 0 or exactly 0
    const bool exact_zero = s == 0;
    // leading one back to bit 62: one place right after a carry out of a sum, or left after a
    // difference lost leading bits
    const bool over = (s >> 63) != 0;
    const int lz = exact_zero ? 0 : clz64(s) - 1;
    s = over ? ((s >> 1) | (s & 1u)) : (s << (lz > 0 ? lz : 0));
    const int64_t e = over ? eh + 1 : eh - (lz > 0 ? lz : 0);
    const uint64_t m = round_pack(s, e, ok);
    uint64_t out = (hi & SIGN) | m;
    out = exact_zero ? 0u : out;                      // x + (-x) = +0
    out = lo_zero ? (mhi == 0 ? (a & b) : hi) : out;
    ok = ok || (lo_zero && eh != 0x7ff);
    *r = out;
    return ok;
}

// a * b for the bit patterns a, b; true when *r holds the IEEE round-to-nearest-even product
SFP_HD bool mul(uint64_t a, uint64_t b, uint64_t *r)
{
    const uint64_t sign = (a ^ b) & SIGN;
    const int64_t ea = (int64_t)((a >> 52) & 0x7ffu), eb = (int64_t)((b >> 52) & 0x7ffu);
    const bool zero = (a & ~SIGN) == 0 || (b & ~SIGN) == 0;  // zero times finite: a signed zero
    bool ok = ea != 0x7ff && eb != 0x7ff && ((ea != 0 && eb != 0) || zero);
    const uint64_t pa = (a & FRAC) | HIDDEN, pb = (b & FRAC) | HIDDEN;
    // exact product in [2^104, 2^106): hi:lo
    const uint64_t lo = pa * pb, hi = mulhi64(pa, pb);
    const int top = (int)(hi >> 41) & 1;  // bit 105 set: one more leading bit
    const int64_t e = ea + eb - 1023 + top;
    // the 63 leading bits with the leading one at bit 62, i.e. hi:lo >> (42 + top), and a sticky
    // bit for the rest
    const int shr = 42 + top;
    uint64_t s = (hi << (64 - shr)) | (lo >> shr);
    s |= (lo & ((1ull << shr) - 1u)) != 0 ? 1u : 0u;
    bool okr = true;
    const uint64_t m = round_pack(s, e, okr);
    *r = zero ? sign : (sign | m);
    return ok && (zero || okr);
}

}  // namespace sfp
}  // namespace bgk
