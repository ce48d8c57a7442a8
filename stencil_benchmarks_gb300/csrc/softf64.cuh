// Binary64 addition, subtraction, multiplication and reciprocal in integer
// arithmetic, correctly rounded to nearest-even: bit-identical to the
// hardware's __dadd_rn / __dsub_rn / __dmul_rn / __drcp_rn (and to numpy) for
// every input the fast paths accept.
//
// Why: GB300 executes fp64 arithmetic at 0.52 Tops/s, 1/57 of its 32-bit
// integer rate, so the exact fp64 stencils are bound by the fp64 pipe while
// the integer pipe idles.  Routing part of a kernel's operations through
// these functions lets both pipes work.
//
// Method: the textbook software implementation of IEEE 754 binary
// floating-point operators (J.-M. Muller et al., Handbook of Floating-Point
// Arithmetic, 2nd ed. 2018, ch. 8 "Algorithms for the basic operations" and
// ch. 10 on software implementations; D. Goldberg, "What every computer
// scientist should know about floating-point arithmetic", 1991, on guard
// and sticky bits):
//   * unpack the significands (implicit bit for normal numbers; zero and
//     subnormal operands carry exponent 1 and no implicit bit);
//   * addition: order the operands by magnitude, align the smaller one
//     with a right shift whose lost bits are ORed into the lowest bit
//     ("sticky" jamming), add or subtract, normalise with a count of
//     leading zeros;
//   * multiplication: the 106-bit product of the significands, its low half
//     ORed into the lowest bit of the high half, normalised by at most one
//     bit;
//   * round to nearest, ties to even, at the 53rd significant bit, and
//     assemble sign | (exponent - 1) << 52 + significand (the significand's
//     implicit bit increments the exponent field; a rounding carry out of
//     the significand does the same, which also yields infinity exactly at
//     overflow).
// The working significands carry 10 (addition) or 11 (multiplication) bits
// below the rounding position, so after the sticky jamming the computed
// value is odd in its lowest bit and lies within one unit of the exact
// value: no rounding boundary (a multiple of 2^7 units or more) can
// separate them, and the rounding is correct.
//
// Each fast path returns false for the cases it leaves to the hardware
// instruction (a NaN or infinite operand, a subnormal or overflowing
// result before rounding); the caller then evaluates the operation in fp64.
// The functions are host-callable too, so the host test harness checks
// them against the host's IEEE arithmetic.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SB_SF_HD __host__ __device__ __forceinline__
#else
#define SB_SF_HD inline
#endif

namespace sb {
namespace sf {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kAbs = 0x7fffffffffffffffull;
constexpr uint64_t kMant = 0x000fffffffffffffull;
constexpr uint64_t kImplicit = 0x0010000000000000ull;

SB_SF_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

SB_SF_HD double from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

SB_SF_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

SB_SF_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Round a normalised working significand w (bit 63 set, `low` bits below the
// 53-bit result) to nearest-even and assemble the result with biased
// exponent e + 1 (0 <= e <= 2045) and sign bit `sign`.
template <int LOW>
SB_SF_HD uint64_t round_pack(uint64_t sign, uint32_t e, uint64_t w) {
    const uint64_t m = w >> LOW;
    const uint32_t rest = (uint32_t)w & ((1u << LOW) - 1u);
    const uint64_t up = (rest + ((uint32_t)m & 1u)) > (1u << (LOW - 1));
    return sign | (((uint64_t)e << 52) + m + up);
}

// a + b (the bit patterns of two doubles).  Returns false where the hardware
// must compute it: a NaN or infinite operand, or a result below the normal
// range (subnormal) or at or above 2^1024 before rounding.
SB_SF_HD bool add(uint64_t a, uint64_t b, uint64_t& r) {
    uint64_t ma = a & kAbs, mb = b & kAbs;
    if (ma < mb) {
        const uint64_t t = a, tm = ma;
        a = b;
        ma = mb;
        b = t;
        mb = tm;
    }
    const uint32_t ea = (uint32_t)(ma >> 52), eb = (uint32_t)(mb >> 52);
    if (ea == 0x7ffu) return false;
    const uint64_t fa = (ma & kMant) | ((uint64_t)(ea != 0u) << 52);
    const uint64_t fb = (mb & kMant) | ((uint64_t)(eb != 0u) << 52);
    const uint32_t ea1 = ea + (ea == 0u), eb1 = eb + (eb == 0u);
    uint32_t d = ea1 - eb1;
    d = d > 63u ? 63u : d;
    const uint64_t xa = fa << 10, xb = fb << 10;
    uint64_t yb = xb >> d;
    yb |= (uint64_t)((yb << d) != xb);
    const bool sub = (int64_t)(a ^ b) < 0;
    uint64_t s = sub ? xa - yb : xa + yb;
    if (s == 0) {
        r = sub ? 0ull : (a & kSign);  // exact cancellation gives +0; equal-signed zeros keep the sign
        return true;
    }
    const int lz = clz64(s);
    const int e = (int)ea1 - lz;
    if ((unsigned)e > 2045u) return false;
    r = round_pack<11>(a & kSign, (uint32_t)e, s << lz);
    return true;
}

SB_SF_HD bool sub(uint64_t a, uint64_t b, uint64_t& r) { return add(a, b ^ kSign, r); }

// a * b.  Returns false where the hardware must compute it: a NaN,
// infinite or subnormal operand, or a result below the normal range or at
// or above 2^1024 before rounding.  A zero operand gives the signed zero.
SB_SF_HD bool mul(uint64_t a, uint64_t b, uint64_t& r) {
    const uint64_t sign = (a ^ b) & kSign;
    const uint32_t ea = (uint32_t)(a >> 52) & 0x7ffu, eb = (uint32_t)(b >> 52) & 0x7ffu;
    if (ea - 1u >= 2046u || eb - 1u >= 2046u) {
        // zero times a finite number: the signed zero; everything else special
        if (((a & kAbs) == 0 && eb != 0x7ffu) || ((b & kAbs) == 0 && ea != 0x7ffu)) {
            r = sign;
            return true;
        }
        return false;
    }
    // significands with the implicit bit, shifted to the top: a << 11 moves the
    // exponent out except its lowest bit, which lands on bit 63, where the
    // implicit bit belongs (normal operands only, checked above)
    const uint64_t xa = (a << 11) | kSign, xb = (b << 11) | kSign;
    uint64_t hi = mulhi64(xa, xb);
    hi |= (uint64_t)((xa * xb) != 0);  // sticky: the low half
    const int n = (int)(~hi >> 63);     // 1 when the product is below 2^127
    const int e = (int)(ea + eb) - 1023 - n;
    if ((unsigned)e > 2045u) return false;
    r = round_pack<11>(sign, (uint32_t)e, hi << n);
    return true;
}

#if !defined(__CUDA_ARCH__)
// Host builds: ulps added to the seed reciprocal (a test knob that stands in
// for the device's approximate reciprocal instruction; 0 by default).
inline int& rcp_seed_perturb() {
    static int ulps = 0;
    return ulps;
}
#endif

// float approximation of 1 / x for x in [2^23, 2^24): the device's
// rcp.approx (relative error below 2^-22); on the host the correctly rounded
// quotient, moved by rcp_seed_perturb() ulps.
SB_SF_HD float rcp_seed(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    float r = 1.0f / x;
    uint32_t b;
    std::memcpy(&b, &r, sizeof b);
    b = (uint32_t)((int32_t)b + rcp_seed_perturb());
    std::memcpy(&r, &b, sizeof r);
    return r;
#endif
}

// One Newton step towards u = 2^126 / d (d in (2^63, 2^64)) from y ~ u:
// y + y * E / 2^126, with E = 2^126 - d*y computed exactly in 128 bits and
// shifted right by SE bits so that it fits a signed 64-bit word e; then
// y * E / 2^126 = mulhi(y, e) / 2^(62 - SE).
template <int SE>
SB_SF_HD uint64_t rcp_step(uint64_t d, uint64_t y) {
    constexpr int SC = 62 - SE;
    const uint64_t plo = d * y, phi = mulhi64(d, y);
    const uint64_t elo = 0ull - plo;
    const uint64_t ehi = (1ull << 62) - phi - (uint64_t)(plo != 0);
    const int64_t e = (int64_t)((ehi << (64 - SE)) | (elo >> SE));
    const uint64_t mag = e < 0 ? 0ull - (uint64_t)e : (uint64_t)e;
    const uint64_t c = mulhi64(y, mag) >> SC;
    return e < 0 ? y - c : y + c;
}

// 1 / a, correctly rounded to nearest (bit-identical to __drcp_rn and to
// numpy's 1.0 / a).  Returns false where the hardware must compute it: a
// zero, subnormal, NaN or infinite operand, or |a| >= 2^1022 (a result at or
// below the bottom of the normal range).
//
// Method (restated from the Newton-Raphson reciprocal iteration with an exact
// remainder correction; Muller et al., Handbook of Floating-Point Arithmetic,
// 2nd ed., sec. 4.7 and ch. 8 on division):  with the significand M in
// (2^52, 2^53) (a power of two is exact), the rounded significand of 1/a is
// S = round(2^105 / M) = (floor(2^106 / M) + 1) >> 1 (2^105 / M is never a
// tie).  With d = M << 11, floor(2^106 / M) = floor(2^117 / d) =
// floor(u / 2^9), u = 2^126 / d in (2^62, 2^63):
//   * seed: the float reciprocal of d's top 32 bits (relative error below
//     2^-20);
//   * a Newton step y <- y (2 - dh y) in 32 x 32-bit products on those top
//     bits (relative error below 2^-30, set by the dropped low bits of d),
//     then one on the full d in 64-bit products, y <- y (2 - d y / 2^126),
//     which squares it: |y2 - u| <= 4;
//   * q = y2 >> 9 is floor(2^117 / d) or one off; the exact remainder
//     2^117 - q d (128-bit) decides the +-1 correction.
SB_SF_HD bool rcp(uint64_t a, uint64_t& r) {
    const uint32_t ea = (uint32_t)(a >> 52) & 0x7ffu;
    if (ea - 1u >= 2044u) return false;  // zero / subnormal (0), exponent >= 2045, inf / NaN
    const uint64_t sign = a & kSign;
    const uint64_t frac = a & kMant;
    if (frac == 0) {
        r = sign | ((uint64_t)(2046u - ea) << 52);
        return true;
    }
    const uint64_t d = (a << 11) | kSign;  // the significand at the top (as in mul)
    // first step on d's top 32 bits: y0 ~ 2^62 / dh (31 bits), E = 2^62 - dh y0
    // (|E| < 2^43), y1 = y0 2^32 + y0 E / 2^30 ~ 2^94 / dh = u (1 + eta),
    // |eta| < 2^-30 (the truncation of d dominates the squared seed error)
    const uint32_t dh = (uint32_t)(d >> 32);
    const uint32_t y0 = (uint32_t)(rcp_seed((float)dh) * 0x1p62f);
    const int64_t e0 = (int64_t)((1ull << 62) - (uint64_t)dh * y0);
    const uint64_t c0 = ((uint64_t)y0 * ((e0 < 0 ? 0ull - (uint64_t)e0 : (uint64_t)e0) >> 10)) >> 20;
    const uint64_t y1 = e0 < 0 ? ((uint64_t)y0 << 32) - c0 : ((uint64_t)y0 << 32) + c0;
    const uint64_t y2 = rcp_step<34>(d, y1);  // |E| < 2^96: e = E >> 34 fits
    uint64_t q = y2 >> 9;
    const uint64_t plo = q * d, phi = mulhi64(q, d);
    const uint64_t rlo = 0ull - plo;
    const int64_t rhi = (int64_t)((1ull << 53) - phi - (uint64_t)(plo != 0));
    if (rhi < 0) {
        q -= 1;
    } else if (rhi > 0 || rlo >= d) {
        q += 1;
    }
    r = sign | (((uint64_t)(2044u - ea) << 52) + ((q + 1) >> 1));
    return true;
}

}  // namespace sf
}  // namespace sb
