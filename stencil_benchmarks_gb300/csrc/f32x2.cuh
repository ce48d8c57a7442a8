// Float-pair ("double-float") arithmetic: a value is hi + lo with two
// float32 numbers, |lo| <= ulp(hi)/2, about 48 significant bits.  On GB300
// the fp64 pipe runs at 1/73 of the fp32 rate (measured: 0.52 vs 38 Tops/s),
// and f64 <-> f32 conversions run on the slow pipe too, so this file builds
// float64 storage values into pairs and back with integer operations only and
// does all arithmetic on the fp32 pipe.
//
// Algorithms (error-free transformations and double-word arithmetic):
//   TwoSum (Knuth), Fast2Sum (Dekker), TwoProd via FMA;
//   add: "sloppy" double-word addition, mul: double-word times double-word
//   with FMA, reciprocal: one Newton step on a correctly rounded float
//   reciprocal -- M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous
//   error bounds for basic building blocks of double-word arithmetic",
//   ACM TOMS 44(2), 2017.  Relative error of add/mul/rcp is a few 2^-48
//   (addition: absolute, a few 2^-48 of the larger operand).
//
// Range: float64 values with magnitudes in [2^-126, 2^128) convert with 48+
// significant bits; smaller magnitudes keep the precision of float32
// (subnormals flush gradually), larger ones become +-inf; inf and nan pass
// through.  Everything here compiles for the host as well (same IEEE float32
// operations, rounded to nearest even), so it is unit-tested on the CPU.
#pragma once

#include <stdint.h>

#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define SB_HD __host__ __device__ __forceinline__
// rare paths that run on the fp64 pipe: out of line, so the compiler cannot
// evaluate them speculatively on every element of the common path
#define SB_HD_COLD static __host__ __device__ __noinline__
#else
#define SB_HD inline
#define SB_HD_COLD static inline
#endif

namespace sb {

struct alignas(8) f32x2 {
    float hi, lo;
    f32x2() = default;
    SB_HD constexpr f32x2(float h, float l) : hi(h), lo(l) {}
    SB_HD explicit constexpr f32x2(int zero) : hi((float)zero), lo(0.0f) {}
};

namespace fx {

SB_HD uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
SB_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}
SB_HD uint64_t d2u(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
#endif
}
SB_HD double u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    std::memcpy(&x, &u, 8);
    return x;
#endif
}
SB_HD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
SB_HD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
SB_HD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
SB_HD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
SB_HD float rcp(float a) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(a);
#else
    return 1.0f / a;
#endif
}
SB_HD float i2f(int32_t v) {
#if defined(__CUDA_ARCH__)
    return __int2float_rn(v);
#else
    return (float)v;
#endif
}
SB_HD float narrow(double x) {  // rare path only (fp64 pipe on the device)
#if defined(__CUDA_ARCH__)
    return __double2float_rn(x);
#else
    return (float)x;
#endif
}
SB_HD double widen(float x) {  // rare path only
    return (double)x;
}

// ---- error-free transformations
SB_HD f32x2 two_sum(float a, float b) {
    const float s = add(a, b);
    const float bb = sub(s, a);
    const float e = add(sub(a, sub(s, bb)), sub(b, bb));
    return {s, e};
}
SB_HD f32x2 fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
    const float s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
SB_HD f32x2 two_prod(float a, float b) {
    const float p = mul(a, b);
    return {p, fma(a, b, -p)};
}

}  // namespace fx

// ---- conversions --------------------------------------------------------------

SB_HD_COLD f32x2 f32x2_from_double_rare(double x) { return {fx::narrow(x), 0.0f}; }
SB_HD_COLD double f32x2_to_double_rare(float hi, float lo) { return fx::widen(hi) + fx::widen(lo); }

// float64 -> pair, integer operations only on the common path.  With the
// 53-bit significand M (implicit bit included) of |x| = M * 2^(E-1075):
// hi = round(M / 2^29) * 2^(E-1046) (the rounding carry moves into the
// exponent field), lo = (M - round(M / 2^29) * 2^29) * 2^(E-1075), whose
// integer factor has at most 28 bits and is rounded once to float32.
SB_HD f32x2 f32x2_from_double(double x) {
    const uint64_t b = fx::d2u(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    const int ef = e - 1023 + 127;  // float biased exponent of hi
    if (ef >= 1 && ef <= 253) {
        const uint64_t m = b & ((1ull << 52) - 1);
        const uint64_t hm = (m + (1ull << 28)) >> 29;  // rounded top bits (0 .. 2^23)
        const float hi = fx::u2f(sign | (((uint32_t)ef << 23) + (uint32_t)hm));
        const int32_t r = (int32_t)(int64_t)(m - (hm << 29));  // in [-2^28, 2^28)
        // scale 2^(e-1075) = 2^(ef-179): float exponent field ef-52 (two steps below 1)
        float lo = fx::i2f(r);
        if (ef > 52) {
            lo = fx::mul(lo, fx::u2f((uint32_t)(ef - 52) << 23));
        } else {
            lo = fx::mul(fx::mul(lo, fx::u2f((uint32_t)(ef + 12) << 23)), 0x1p-64f);
        }
        return {hi, fx::u2f(fx::f2u(lo) ^ sign)};
    }
    return f32x2_from_double_rare(x);  // zero, subnormal, tiny, huge, inf, nan
}

// pair -> float64 (hi + lo, within one unit in the last place of float64),
// integer operations only when hi is a normal float and lo is normal or zero.
SB_HD double f32x2_to_double(f32x2 a) {
    const uint32_t hb = fx::f2u(a.hi), lb = fx::f2u(a.lo);
    const int eh = (int)((hb >> 23) & 0xff), el = (int)((lb >> 23) & 0xff);
    if (eh >= 1 && eh <= 254 && (el >= 1 || (lb << 1) == 0) && el <= 254) {
        // hi = (2^23 + mh) * 2^(eh-150) = H * 2^(eh-179) with H = (2^23 + mh) << 29
        int64_t H = (int64_t)((1u << 23) | (hb & 0x7fffffu)) << 29;
        if ((lb << 1) != 0) {
            // lo = (2^23 + ml) * 2^(el-150) in units of 2^(eh-179): shift by el - eh + 29
            const int64_t L = (int64_t)((1u << 23) | (lb & 0x7fffffu));
            const int s = el - eh + 29;
            int64_t Ls;
            if (s >= 0) {
                Ls = s < 40 ? (L << s) : 0;  // s <= 5 for a normalised pair
            } else if (s > -40) {
                Ls = (L + ((int64_t)1 << (-s - 1))) >> (-s);
            } else {
                Ls = 0;
            }
            H += ((hb ^ lb) >> 31) ? -Ls : Ls;
        }
        int exp = eh + 896;  // value H * 2^(eh-179); H in [2^52, 2^53) has double exponent eh + 896
        // |lo| <= ulp(hi)/2 moves H by less than 2^29 from [2^52, 2^53): one shift normalises it
        if (H >= ((int64_t)1 << 53)) {
            H = (H + 1) >> 1;
            ++exp;
        } else if (H < ((int64_t)1 << 52)) {
            H <<= 1;
            --exp;
        }
        if (H >= ((int64_t)1 << 52) && H < ((int64_t)1 << 53) && exp >= 1 && exp <= 2046) {
            return fx::u2d(((uint64_t)(hb & 0x80000000u) << 32) | ((uint64_t)exp << 52) |
                           ((uint64_t)H & ((1ull << 52) - 1)));
        }
    }
    return f32x2_to_double_rare(a.hi, a.lo);  // zero, subnormal, inf, nan
}

SB_HD f32x2 f32x2_from_float(float x) { return {x, 0.0f}; }

// ---- arithmetic ---------------------------------------------------------------
SB_HD f32x2 neg(f32x2 a) { return {-a.hi, -a.lo}; }
SB_HD f32x2 operator-(f32x2 a) { return neg(a); }

SB_HD f32x2 add(f32x2 x, f32x2 y) {
    const f32x2 s = fx::two_sum(x.hi, y.hi);
    const float v = fx::add(x.lo, y.lo);
    const float w = fx::add(s.lo, v);
    return fx::fast_two_sum(s.hi, w);
}
SB_HD f32x2 sub(f32x2 x, f32x2 y) { return add(x, neg(y)); }

SB_HD f32x2 mul(f32x2 x, f32x2 y) {
    const f32x2 p = fx::two_prod(x.hi, y.hi);
    const float t = fx::fma(x.lo, y.hi, fx::mul(x.hi, y.lo));
    return fx::fast_two_sum(p.hi, fx::add(p.lo, t));
}

// exact multiplication by 2^E (no overflow / underflow in the operands' range)
template <int E>
SB_HD f32x2 scale2(f32x2 x) {
    constexpr float f = E >= 0 ? (float)(1u << (E >= 0 ? E : 0)) : 1.0f / (float)(1u << (E >= 0 ? 0 : -E));
    return {fx::mul(x.hi, f), fx::mul(x.lo, f)};
}

SB_HD f32x2 rcp(f32x2 y) {
    const float t = fx::rcp(y.hi);
    float r = fx::fma(-y.hi, t, 1.0f);  // 1 - yh*t, exact
    r = fx::fma(-y.lo, t, r);
    return fx::fast_two_sum(t, fx::mul(t, r));
}
SB_HD f32x2 div(f32x2 x, f32x2 y) { return mul(x, rcp(y)); }

// sign of x - y for two pairs: -1, 0, +1 (normalised pairs compare by hi, then lo)
SB_HD int cmp(f32x2 x, f32x2 y) {
    if (x.hi != y.hi) return x.hi > y.hi ? 1 : -1;
    if (x.lo != y.lo) return x.lo > y.lo ? 1 : -1;
    return 0;
}

}  // namespace sb
