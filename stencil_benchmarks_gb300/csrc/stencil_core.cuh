// Per-warp / per-thread stencil bodies shared by the per-domain kernels
// (hdiff.cu, vadv.cu) and the persistent batched kernel (batch.cu).
#pragma once

#include <type_traits>

#include "common.cuh"

namespace sb {

// ---------------------------------------------------------------------------
// horizontal diffusion, one warp, one k-plane strip of 32 columns
// ---------------------------------------------------------------------------
// Lane L owns column i = i_lane (caller passes i0 - 2 + L); lanes 2..29 write
// rows [j0, j1) of the output (28 columns), lanes 0-1 and 30-31 supply the
// i-halo.  Arithmetic and order as stencil_benchmarks/benchmarks_collection/
// stencils/base.py:284-311; inp(i+-1), lap(i+1), flx(i-1) by shuffles; U rows
// of loads issued together.  All 32 lanes must call this (full-mask shuffles).
constexpr int kJscanOut = 28;

template <class S, class C, int U, class IDX>
__device__ __forceinline__ void hdiff_jscan_strip(const S* __restrict__ inp, const S* __restrict__ coeff,
                                                  S* __restrict__ out, int ni, int nj, IDX si, IDX sj, IDX sk,
                                                  int i, int lane, int j0, int j1, int k) {
    using A = Ar<C>;
    const bool col_in = i <= ni + 1;  // inside the halo'd array (i >= -2 always)
    const bool writer = lane >= 2 && lane < 2 + kJscanOut && i < ni;
    const int rmax = nj + 1;  // last row inside the halo'd array
    const IDX obase = (IDX)k * sk + (IDX)i * si;
    auto load_row = [&](int r) -> C {
        return (col_in && r <= rmax) ? ld<C, S>(inp + (obase + (IDX)r * sj)) : C(0);
    };
    auto lap_of = [&](C below, C center, C above) -> C {
        const C left = shfl_up(center, 1);
        const C right = shfl_down(center, 1);
        return A::sub(A::template scale2<2>(center), A::add(A::add(A::add(right, left), above), below));
    };
    // preamble: rows j0-2 .. j0+1
    const C am2 = load_row(j0 - 2);
    C a0 = load_row(j0 - 1);
    C a1 = load_row(j0);
    C a2 = load_row(j0 + 1);
    const C lap_m1 = lap_of(am2, a0, a1);               // lap(j0-1)
    C lap0 = lap_of(a0, a1, a2);                        // lap(j0)
    C fly_m1 = A::limit(A::sub(lap0, lap_m1), a1, a0);  // fly(j0-1)
    C right0 = shfl_down(a1, 1);    // inp(i+1, j0)
    // state for output row j: a0 = inp(j), a1 = inp(j+1), lap0 = lap(j)
    a0 = a1;
    a1 = a2;
    for (int jb = j0; jb < j1; jb += U) {
        C nxt[U], cf[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = jb + u;
            nxt[u] = load_row(j + 2);
            cf[u] = (writer && j < j1) ? ld<C, S>(coeff + (obase + (IDX)j * sj)) : C(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = jb + u;
            if (j >= j1) break;  // warp-uniform
            const C a2n = nxt[u];
            const C left1 = shfl_up(a1, 1);
            const C right1 = shfl_down(a1, 1);
            const C lap1 = A::sub(A::template scale2<2>(a1), A::add(A::add(A::add(right1, left1), a2n), a0));
            const C fly0 = A::limit(A::sub(lap1, lap0), a1, a0);      // fly(i, j)
            const C lapR = shfl_down(lap0, 1);    // lap(i+1, j)
            const C flx0 = A::limit(A::sub(lapR, lap0), right0, a0);  // flx(i, j)
            const C flxL = shfl_up(flx0, 1);      // flx(i-1, j)
            if (writer) {
                const C d = A::sub(A::add(A::sub(flx0, flxL), fly0), fly_m1);
                st<S, C>(out + (obase + (IDX)j * sj), A::sub(a0, A::mul(cf[u], d)));
            }
            a0 = a1;
            a1 = a2n;
            lap0 = lap1;
            fly_m1 = fly0;
            right0 = right1;
        }
    }
}

// ---------------------------------------------------------------------------
// horizontal diffusion, one warp, one k-plane strip of 32*V columns
// ---------------------------------------------------------------------------
// The JSCAN march with V columns per lane: lane L holds columns
// c = cs + V*L + q (q < V) of each row, moved as one aligned vector of
// V*sizeof(S) bytes (the caller picks cs so that column cs starts a vector).
// Neighbours inside a lane's group are registers; across lanes four shuffles
// per row serve V points (inp left/right, lap right, flx left).  Outputs are
// the columns [cs+2, cs+2+step) within [0, ni).  A vector is loaded when it
// holds at least one column of the halo'd row [-2, ni+2); its other columns
// lie in the same aligned V*sizeof(S)-byte block of the caller's memory and
// only feed points that are not stored.  Same arithmetic and order as
// hdiff_jscan_strip.  All 32 lanes must call this (full-mask shuffles).
template <class S, class C, int V, int U, class IDX>
__device__ __forceinline__ void hdiff_vscan_strip(const S* __restrict__ inp, const S* __restrict__ coeff,
                                                  S* __restrict__ out, int ni, int nj, IDX sj, IDX sk, int cs,
                                                  int step, int lane, int j0, int j1, int k) {
    using A = Ar<C>;
    const int c0 = cs + V * lane;
    const bool grp_in = c0 + V > -2 && c0 < ni + 2;
    const int wlo = max(cs + 2, 0), whi = min(cs + 2 + step, ni);
    const bool any_w = c0 + V > wlo && c0 < whi;
    const bool all_w = c0 >= wlo && c0 + V <= whi;
    const int rmax = nj + 1;
    const IDX obase = (IDX)k * sk + (IDX)c0;
    auto load_row = [&](int r, C(&o)[V]) {
        if (grp_in && r <= rmax) {
            ld_vec<S, C, V>(inp + (obase + (IDX)r * sj), o);
        } else {
#pragma unroll
            for (int q = 0; q < V; ++q) o[q] = C(0);
        }
    };
    // lap of the centre row c given the rows below (b) and above (a)
    auto lap_row = [&](const C(&b)[V], const C(&c)[V], const C(&a)[V], C(&o)[V], C& right) {
        const C left = shfl_up(c[V - 1], 1);  // column c0 - 1
        right = shfl_down(c[0], 1);           // column c0 + V
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const C l = q == 0 ? left : c[q - 1];
            const C r = q == V - 1 ? right : c[q + 1];
            o[q] = A::sub(A::template scale2<2>(c[q]), A::add(A::add(A::add(r, l), a[q]), b[q]));
        }
    };
    C am2[V], a0[V], a1[V], a2[V], lap_m1[V], lap0[V], fly_m1[V];
    load_row(j0 - 2, am2);
    load_row(j0 - 1, a0);
    load_row(j0, a1);
    load_row(j0 + 1, a2);
    C unused, rnb0;
    lap_row(am2, a0, a1, lap_m1, unused);  // lap(j0-1)
    lap_row(a0, a1, a2, lap0, rnb0);       // lap(j0); rnb0 = inp(c0+V, j0)
#pragma unroll
    for (int q = 0; q < V; ++q) {
        fly_m1[q] = A::limit(A::sub(lap0[q], lap_m1[q]), a1[q], a0[q]);  // fly(j0-1)
        a0[q] = a1[q];
        a1[q] = a2[q];
    }
    // state for output row j: a0 = inp(j), a1 = inp(j+1), lap0 = lap(j), rnb0 = inp(c0+V, j)
    for (int jb = j0; jb < j1; jb += U) {
        C nxt[U][V], cf[U][V];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = jb + u;
            load_row(j + 2, nxt[u]);
            if (any_w && j < j1) {
                ld_vec<S, C, V>(coeff + (obase + (IDX)j * sj), cf[u]);
            } else {
#pragma unroll
                for (int q = 0; q < V; ++q) cf[u][q] = C(0);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = jb + u;
            if (j >= j1) break;  // warp-uniform
            C lap1[V], fly0[V], flx0[V], res[V], rnb1;
            lap_row(a0, a1, nxt[u], lap1, rnb1);
            const C lapR = shfl_down(lap0[0], 1);  // lap(c0+V, j)
#pragma unroll
            for (int q = 0; q < V; ++q) {
                fly0[q] = A::limit(A::sub(lap1[q], lap0[q]), a1[q], a0[q]);
                const C lr = q == V - 1 ? lapR : lap0[q + 1];
                const C ir = q == V - 1 ? rnb0 : a0[q + 1];
                flx0[q] = A::limit(A::sub(lr, lap0[q]), ir, a0[q]);
            }
            const C flxL = shfl_up(flx0[V - 1], 1);  // flx(c0-1, j)
#pragma unroll
            for (int q = 0; q < V; ++q) {
                const C fl = q == 0 ? flxL : flx0[q - 1];
                const C d = A::sub(A::add(A::sub(flx0[q], fl), fly0[q]), fly_m1[q]);
                res[q] = A::sub(a0[q], A::mul(cf[u][q], d));
            }
            S* orow = out + (obase + (IDX)j * sj);
            if (all_w) {
                st_vec<S, C, V>(orow, res);
            } else if (any_w) {
#pragma unroll
                for (int q = 0; q < V; ++q)
                    if (c0 + q >= wlo && c0 + q < whi) st<S, C>(orow + q, res[q]);
            }
#pragma unroll
            for (int q = 0; q < V; ++q) {
                a0[q] = a1[q];
                a1[q] = nxt[u][q];
                lap0[q] = lap1[q];
                fly_m1[q] = fly0[q];
            }
            rnb0 = rnb1;
        }
    }
}

// ---------------------------------------------------------------------------
// horizontal diffusion in 64-bit fixed point (float64 storage), one warp strip
// ---------------------------------------------------------------------------
// lap, flx, fly and their sum S are additions only, so they are exact in
// two's-complement integers once the inputs share a scale.  Per warp strip
// (32 columns x rows j0-2 .. j1+1 of one k-plane) the largest biased
// exponent E of the inputs sets the unit u = 2^(E-1078): |inp| / u < 2^56,
// |lap| < 2^59, |flx| < 2^60, |S| < 2^62.  Inputs below 1/8 of the strip's
// largest binade lose the bits under u (at most 2^-56 of the largest value).
// The limiter's sign of inp(+1) - inp is taken exactly from the float64 bit
// patterns; flx and fly are exact integers.  The result is
//     out = fma(-coeff, S * u, inp)
// with S * u rounded once to float64: one fp64 operation per point, errors
// at float64 rounding level relative to the strip's largest value.  Strips
// with inf/nan, |inp| >= 2^1017, all |inp| < 2^-500 (where fp64 products of
// differences could underflow) or nonzero values spanning more than 2^40
// are computed by the float64 strip instead.
struct fix64 {};  // compute tag: 64-bit fixed point

__device__ __forceinline__ int dsign_diff(unsigned long long b1, unsigned long long b0) {
    if (((b1 | b0) << 1) == 0) return 0;  // +-0 and +-0
    const unsigned long long k1 = (b1 >> 63) ? ~b1 : (b1 | (1ull << 63));
    const unsigned long long k0 = (b0 >> 63) ? ~b0 : (b0 | (1ull << 63));
    return (k1 > k0) - (k1 < k0);
}

// (f * (inp1 - inp0) > 0) ? 0 : f for fixed-point f.  Truncation toward zero
// is monotone, so a nonzero a1 - a0 has the sign of inp1 - inp0; equal fixed
// values (rare) compare the float64 bit patterns.
__device__ __forceinline__ long long fix_limit(long long f, long long a1, long long a0, unsigned long long b1,
                                               unsigned long long b0) {
    const long long d = a1 - a0;
    if (d == 0) {
        const int s = dsign_diff(b1, b0);
        return ((f > 0 && s > 0) || (f < 0 && s < 0)) ? 0 : f;
    }
    return (f != 0 && (f ^ d) >= 0) ? 0 : f;
}

// float64 bit pattern -> integer multiple of 2^(E-1078), truncated toward
// zero (E >= 523: subnormals and zeros shift out entirely)
__device__ __forceinline__ long long fix_of(unsigned long long b, int E) {
    const unsigned hi = (unsigned)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned long long m = ((unsigned long long)((hi & 0xfffffu) | 0x100000u) << 32) | (unsigned)b;
    const int rs = E - e;  // >= 0: |inp| / u = m * 2^3 / 2^rs
    const unsigned long long mag = rs < 3 ? (m << (3 - rs)) : (rs < 67 ? (m >> (rs - 3)) : 0ull);
    const long long sgn = (long long)b >> 63;  // 0 or -1
    return ((long long)mag ^ sgn) - sgn;
}

// S * 2^Ue rounded to float64 (|S| < 2^62; the scaling is an exponent add)
__device__ __forceinline__ double fix_to_double(long long S, int Ue) {
    const double d = __ll2double_rn(S);
    if (S == 0) return 0.0;
    return __longlong_as_double(__double_as_longlong(d) + ((long long)Ue << 52));
}

template <int U, class IDX>
__device__ __forceinline__ void hdiff_fixed_strip(const double* __restrict__ inp, const double* __restrict__ coeff,
                                                  double* __restrict__ out, int ni, int nj, IDX si, IDX sj, IDX sk,
                                                  int i, int lane, int j0, int j1, int k) {
    const bool col_in = i <= ni + 1;
    const bool writer = lane >= 2 && lane < 2 + kJscanOut && i < ni;
    const int rmax = nj + 1;
    const IDX obase = (IDX)k * sk + (IDX)i * si;
    auto load_bits = [&](int r) -> unsigned long long {
        return (col_in && r <= rmax) ? (unsigned long long)__double_as_longlong(__ldg(inp + (obase + (IDX)r * sj)))
                                     : 0ull;
    };
    // scale of the strip: largest and smallest biased exponent of the values
    // (exponent field 0, i.e. zeros and subnormals, does not count as smallest)
    unsigned emax = 0, emin = 0x7ff00000u;
    for (int r = j0 - 2; r <= j1 + 1; ++r) {
        const unsigned ef = (unsigned)(load_bits(r) >> 32) & 0x7ff00000u;
        emax = max(emax, ef);
        emin = min(emin, ef ? ef : 0x7ff00000u);
    }
    emax = __reduce_max_sync(0xffffffffu, emax) >> 20;
    emin = __reduce_min_sync(0xffffffffu, emin) >> 20;
    if (emax >= 2040u || emax < 523u || emax - emin > 40u) {
        hdiff_jscan_strip<double, double, U, IDX>(inp, coeff, out, ni, nj, si, sj, sk, i, lane, j0, j1, k);
        return;
    }
    const int E = (int)emax, Ue = E - 1078;

    const long long am2 = fix_of(load_bits(j0 - 2), E);
    unsigned long long b0 = load_bits(j0 - 1), b1 = load_bits(j0), b2 = load_bits(j0 + 1);
    long long a0 = fix_of(b0, E), a1 = fix_of(b1, E), a2 = fix_of(b2, E);
    auto lap_of = [&](long long below, long long center, long long above) -> long long {
        return 4 * center - (shfl_down(center, 1) + shfl_up(center, 1) + above + below);
    };
    const long long lap_m1 = lap_of(am2, a0, a1);
    long long lap0 = lap_of(a0, a1, a2);
    long long fly_m1 = fix_limit(lap0 - lap_m1, a1, a0, b1, b0);
    unsigned long long right0 = shfl_down(b1, 1);  // bits of inp(i+1, j0)
    long long rightf0 = shfl_down(a1, 1);          // fixed inp(i+1, j0)
    a0 = a1;
    a1 = a2;
    b0 = b1;
    b1 = b2;
    for (int jb = j0; jb < j1; jb += U) {
        unsigned long long nxt[U];
        double cf[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = jb + u;
            nxt[u] = load_bits(j + 2);
            cf[u] = (writer && j < j1) ? __ldg(coeff + (obase + (IDX)j * sj)) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int j = jb + u;
            if (j >= j1) break;  // warp-uniform
            const unsigned long long b2n = nxt[u];
            const long long a2n = fix_of(b2n, E);
            const long long rightf1 = shfl_down(a1, 1);
            const long long lap1 = 4 * a1 - (rightf1 + shfl_up(a1, 1) + a2n + a0);
            const long long fly0 = fix_limit(lap1 - lap0, a1, a0, b1, b0);           // fly(i, j)
            const long long lapR = shfl_down(lap0, 1);                                // lap(i+1, j)
            const long long flx0 = fix_limit(lapR - lap0, rightf0, a0, right0, b0);   // flx(i, j)
            const long long flxL = shfl_up(flx0, 1);                                  // flx(i-1, j)
            const unsigned long long right1 = shfl_down(b1, 1);
            if (writer) {
                const long long sum = ((flx0 - flxL) + fly0) - fly_m1;
                out[obase + (IDX)j * sj] = __fma_rn(-cf[u], fix_to_double(sum, Ue), __longlong_as_double((long long)b0));
            }
            a0 = a1;
            a1 = a2n;
            b0 = b1;
            b1 = b2n;
            lap0 = lap1;
            fly_m1 = fly0;
            right0 = right1;
            rightf0 = rightf1;
        }
    }
}

// one strip in compute type C (fix64: the fixed-point strip, float64 storage)
template <class S, class C, int U, class IDX>
__device__ __forceinline__ void hdiff_strip(const S* __restrict__ inp, const S* __restrict__ coeff,
                                            S* __restrict__ out, int ni, int nj, IDX si, IDX sj, IDX sk, int i,
                                            int lane, int j0, int j1, int k) {
    if constexpr (std::is_same<C, fix64>::value) {
        hdiff_fixed_strip<U, IDX>(inp, coeff, out, ni, nj, si, sj, sk, i, lane, j0, j1, k);
    } else {
        hdiff_jscan_strip<S, C, U, IDX>(inp, coeff, out, ni, nj, si, sj, sk, i, lane, j0, j1, k);
    }
}

// ---------------------------------------------------------------------------
// vertical advection, one thread, one column
// ---------------------------------------------------------------------------
// Storage of the per-level elimination factors (ccol, dcol):
template <class C>
struct SmemFactors {  // shared memory, level k at c[k * stride]
    C* c;
    C* d;
    int stride;
    static constexpr bool kPrefetch = false;
    __device__ __forceinline__ void put(int k, C cv, C dv) const {
        c[(size_t)k * stride] = cv;
        d[(size_t)k * stride] = dv;
    }
    __device__ __forceinline__ C getc(int k) const { return c[(size_t)k * stride]; }
    __device__ __forceinline__ C getd(int k) const { return d[(size_t)k * stride]; }
};

template <class C>
struct GlobalFactors {  // global memory, level k at c[k * stride] (read back with prefetch)
    C* c;
    C* d;
    int64_t stride;
    static constexpr bool kPrefetch = true;
    __device__ __forceinline__ void put(int k, C cv, C dv) const {
        c[k * stride] = cv;
        d[k * stride] = dv;
    }
    __device__ __forceinline__ C getc(int k) const { return c[k * stride]; }
    __device__ __forceinline__ C getd(int k) const { return d[k * stride]; }
};

// Thomas solve of the column at offset `col`; oracle
// stencil_benchmarks/benchmarks_collection/stencils/base.py:410-473 with the
// exact rewrites documented in vadv.cu.  Inputs of the forward sweep are
// prefetched D levels ahead in a register ring (slot u holds level kb+u);
// pos (and factors kept in global memory) likewise in the backward sweep.
// The new tensstage goes to `out` (may equal tensstage: each level is read
// before it is written, by the same thread).
template <class S, class C, int D, class F>
__device__ __forceinline__ void vadv_column(const S* __restrict__ stage, const S* __restrict__ pos,
                                            const S* __restrict__ tens, const S* tensstage,
                                            const S* __restrict__ wcon, S* out, int64_t col, int nk, int64_t sk,
                                            int64_t wsh, const F& fac) {
    using A = Ar<C>;
    const C dtr = konst<C>(3.0 / 20.0);
    // ---- forward sweep, k = 0
    int64_t o = col;
    C gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + o + sk + wsh), ld<C, S>(wcon + o + sk)));
    C cs = A::template scale2<-1>(gcv);  // gcv * bet_m == gcv * bet_p
    C sprev = ld<C, S>(stage + o);
    C scur = ld<C, S>(stage + o + sk);
    C dup = A::sub(scur, sprev);  // stage[k+1] - stage[k]
    C bcol = A::sub(dtr, cs);
    C corr = A::mul(-cs, dup);
    C dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
    C cp = A::div(cs, bcol);
    C dp = A::div(dv, bcol);
    fac.put(0, cp, dp);

    // ---- forward sweep, 0 < k < nk-1
    C rw1[D], rw0[D], rst[D], rpo[D], rte[D], rts[D];
    auto fetch = [&](C& w1, C& w0, C& s1, C& p0, C& t0, C& ts0, int k) {
        if (k < nk - 1) {
            const int64_t q = col + (int64_t)k * sk;
            w1 = ld<C, S>(wcon + q + sk + wsh);
            w0 = ld<C, S>(wcon + q + sk);
            s1 = ld<C, S>(stage + q + sk);
            p0 = ld<C, S>(pos + q);
            t0 = ld<C, S>(tens + q);
            ts0 = ldc<C, S>(tensstage + q);
        }
    };
#pragma unroll
    for (int u = 0; u < D; ++u) fetch(rw1[u], rw0[u], rst[u], rpo[u], rte[u], rts[u], 1 + u);
    for (int kb = 1; kb < nk - 1; kb += D) {
#pragma unroll
        for (int u = 0; u < D; ++u) {
            const int k = kb + u;
            if (k >= nk - 1) break;                      // uniform: every thread has the same nk
            const C as_ = A::template scale2<-1>(-gcv);  // gav * bet_m == acol, gav = -gcv(k-1)
            gcv = A::template scale2<-2>(A::add(rw1[u], rw0[u]));
            cs = A::template scale2<-1>(gcv);
            const C snext = rst[u];
            const C ddown = A::neg_diff(dup, scur, sprev);  // stage[k-1] - stage[k]
            dup = A::sub(snext, scur);                     // stage[k+1] - stage[k]
            bcol = A::sub(A::sub(dtr, as_), cs);
            corr = A::sub(A::mul(-as_, ddown), A::mul(cs, dup));
            dv = A::add(A::add(A::add(A::mul(dtr, rpo[u]), rte[u]), rts[u]), corr);
            fetch(rw1[u], rw0[u], rst[u], rpo[u], rte[u], rts[u], k + D);
            const C divided = A::rcp(A::sub(bcol, A::mul(cp, as_)));
            cp = A::mul(cs, divided);
            dp = A::mul(A::sub(dv, A::mul(dp, as_)), divided);
            fac.put(k, cp, dp);
            sprev = scur;
            scur = snext;
        }
    }

    // ---- forward sweep, k = nk-1
    {
        const int k = nk - 1;
        o = col + (int64_t)k * sk;
        const C as_ = A::template scale2<-1>(-gcv);
        bcol = A::sub(dtr, as_);
        const C ddown = A::neg_diff(dup, scur, sprev);
        corr = A::mul(-as_, ddown);
        dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
        dp = A::div(A::sub(dv, A::mul(dp, as_)), A::sub(bcol, A::mul(cp, as_)));
    }

    // ---- backward sweep
    C data = dp;
    o = col + (int64_t)(nk - 1) * sk;
    st<S, C>(out + o, A::mul(dtr, A::sub(data, ld<C, S>(pos + o))));
    C bpo[D], bcc[D], bdd[D];
    auto fetch_back = [&](C& p0, C& c0, C& d0, int k) {
        if (k >= 0) {
            p0 = ld<C, S>(pos + col + (int64_t)k * sk);
            if (F::kPrefetch) {
                c0 = fac.getc(k);
                d0 = fac.getd(k);
            }
        }
    };
#pragma unroll
    for (int u = 0; u < D; ++u) fetch_back(bpo[u], bcc[u], bdd[u], nk - 2 - u);
    for (int kb = nk - 2; kb >= 0; kb -= D) {
#pragma unroll
        for (int u = 0; u < D; ++u) {
            const int k = kb - u;
            if (k < 0) break;
            const C cv = F::kPrefetch ? bcc[u] : fac.getc(k);
            const C dvv = F::kPrefetch ? bdd[u] : fac.getd(k);
            const C p0 = bpo[u];
            fetch_back(bpo[u], bcc[u], bdd[u], k - D);
            data = A::sub(dvv, A::mul(cv, data));
            st<S, C>(out + col + (int64_t)k * sk, A::mul(dtr, A::sub(data, p0)));
        }
    }
}

// Precision of the Thomas recurrences: the bulk arithmetic in C, the
// forward-elimination divisor and factors and the back-substitution in P.
// Every form uses P = C; the type split keeps the solve generic.
template <class P, class C>
__device__ __forceinline__ P to_p(C x) {
    if constexpr (std::is_same<P, C>::value) return x;
    else return P(x, 0.0f);
}
template <class C, class P>
__device__ __forceinline__ C from_p(P x) {
    if constexpr (std::is_same<P, C>::value) return x;
    else return x.hi;  // a normalised pair's hi is its value rounded to float
}

// Ring entries of the SMEM-async solve.  Storage of 4 or 8 bytes is staged
// as is.  cp.async copies at least 4 bytes, so 2-byte storage is staged as
// the aligned 4-byte word that holds the element (its neighbour comes along;
// the word never leaves the allocation's aligned 4-byte granule), and the
// element's half is picked with a byte permutation when it is used.  Which
// half holds level k of a field is bit 1 of its address: the level-0 value
// flipped when k * sk is odd.
template <class S>
struct RingOf {
    using T = S;
};
template <>
struct RingOf<bf16> {
    using T = uint32_t;
};

template <class S>
__device__ __forceinline__ const void* ring_src(const S* p) {
    if constexpr (sizeof(S) == 2) return (const void*)((uintptr_t)p & ~(uintptr_t)3);
    else return (const void*)p;
}

// __byte_perm selector moving the addressed half of the staged word to the
// high half (a bfloat16 there is the float32 of the same value)
template <class S>
__device__ __forceinline__ uint32_t half_sel(const S* p) {
    return (((uintptr_t)p >> 1) & 1) ? 0x3244u : 0x1044u;
}

template <class C, class S, class T>
__device__ __forceinline__ C from_ring(T w, uint32_t sel) {
    if constexpr (sizeof(S) == 2) {
        static_assert(sizeof(C) == 4, "2-byte storage is computed in float32");
        return __uint_as_float(__byte_perm(w, 0u, sel));
    } else {
        return cvt<C, S>(w);
    }
}

// SMEM-async column solve (one thread): inputs staged global -> shared with
// cp.async into a ring of R = D+1 slots ([R][6][BT] ring entries, this
// thread's entries at stride BT).  Factors (ccol, dcol of each level):
//   SLAB = false: in shared memory sc/sd ([nk][BT], level stride BT);
//   SLAB = true:  in global memory sc/sd with level stride fs (a compact
//                 per-thread slab, small enough to stay in L2), read back in
//                 the backward sweep through the same cp.async ring (fields
//                 0 and 1 of a slot; needs ring entries of the compute size).
// Every shared-memory address below is a per-thread base plus a
// compile-time offset.
// The nine products of a vadv level (sites 4, 5, 7, 11, 13, 14, 16, 17, 20 of
// vadv_async_column): the placement that pays on the integer pipe.
constexpr uint32_t kVadvProductSites = (1u << 4) | (1u << 5) | (1u << 7) | (1u << 11) | (1u << 13) | (1u << 14) |
                                       (1u << 16) | (1u << 17) | (1u << 20);
// The level's reciprocal (site 21).
constexpr uint32_t kVadvRcpSite = 1u << 21;
// The float64 default: the nine products and the reciprocal in integer
// arithmetic, the additions on the fp64 pipe.
constexpr uint32_t kVadvDefaultIntSites = kVadvProductSites | kVadvRcpSite;

// PL: integer-pipe placement mask over the operation sites 0-21 below (Mix).
template <class S, class C, int BT, int D, class IDX, bool SLAB = false, class P = C, uint32_t PL = 0u>
__device__ __forceinline__ void vadv_async_column(const S* __restrict__ stage, const S* __restrict__ pos,
                                                  const S* __restrict__ tens, const S* tensstage,
                                                  const S* __restrict__ wcon, S* out, IDX col, int nk, IDX sk,
                                                  IDX wsh, P* sc, P* sd, typename RingOf<S>::T* ring,
                                                  int fs = 0) {
    using A = Ar<C>;
    using AP = Ar<P>;
    using X = Mix<C, PL>;
    using XP = Mix<P, PL>;
    using T = typename RingOf<S>::T;
    constexpr int R = D + 1;
    constexpr int B = sizeof(T);
    static_assert(!SLAB || sizeof(T) == sizeof(P), "slab factors are staged in ring entries");
    const int64_t FS = SLAB ? (int64_t)fs : (int64_t)BT;  // level stride of the factors
    const C dtr = konst<C>(3.0 / 20.0);
    // half selectors of level 0 (2-byte storage only; unused otherwise)
    const uint32_t sel_w1 = half_sel(wcon + col + sk + wsh), sel_w0 = half_sel(wcon + col + sk);
    const uint32_t sel_st = half_sel(stage + col + sk), sel_po = half_sel(pos + col);
    const uint32_t sel_te = half_sel(tens + col), sel_ts = half_sel(tensstage + col);
    const uint32_t sk_odd = (uint32_t)sk & 1u;
    auto flip = [&](int k) -> uint32_t { return ((uint32_t)k & sk_odd) ? 0x2200u : 0u; };

    auto issue = [&](int slot, int k) {
        if (k < nk - 1) {
            const IDX q = col + (IDX)k * sk;
            T* d = ring + slot * 6 * BT;
            cp_async<B>(d, ring_src(wcon + q + sk + wsh));
            cp_async<B>(d + BT, ring_src(wcon + q + sk));
            cp_async<B>(d + 2 * BT, ring_src(stage + q + sk));
            cp_async<B>(d + 3 * BT, ring_src(pos + q));
            cp_async<B>(d + 4 * BT, ring_src(tens + q));
            cp_async<B>(d + 5 * BT, ring_src(tensstage + q));
        }
        cp_async_commit();
    };
    // level L is staged in slot (L-1) % R
#pragma unroll
    for (int u = 0; u < D; ++u) issue(u, 1 + u);

    // ---- forward sweep, k = 0 (direct loads)
    C gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + col + sk + wsh), ld<C, S>(wcon + col + sk)));
    C cs = A::template scale2<-1>(gcv);
    C sprev = ld<C, S>(stage + col);
    C scur = ld<C, S>(stage + col + sk);
    C dup = A::sub(scur, sprev);
    C bcol = A::sub(dtr, cs);
    C corr = A::mul(-cs, dup);
    C dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + col)), ld<C, S>(tens + col)), ldc<C, S>(tensstage + col)), corr);
    P cp = AP::div(to_p<P>(cs), to_p<P>(bcol));
    P dp = AP::div(to_p<P>(dv), to_p<P>(bcol));
    sc[0] = cp;
    sd[0] = dp;

    // ---- forward sweep, 0 < k < nk-1
    for (int kb = 1; kb < nk - 1; kb += R) {
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k = kb + u;
            if (k >= nk - 1) break;  // uniform
            cp_async_wait<D - 1>();
            const T* sl = ring + u * 6 * BT;
            const uint32_t f = flip(k);
            const C w1 = from_ring<C, S>(sl[0], sel_w1 ^ f), w0 = from_ring<C, S>(sl[BT], sel_w0 ^ f);
            const C snext = from_ring<C, S>(sl[2 * BT], sel_st ^ f), p0 = from_ring<C, S>(sl[3 * BT], sel_po ^ f);
            const C t0 = from_ring<C, S>(sl[4 * BT], sel_te ^ f), ts0 = from_ring<C, S>(sl[5 * BT], sel_ts ^ f);
            issue((u + D) % R, k + D);  // the slot of level k-1, already consumed
            const C as_ = A::template scale2<-1>(-gcv);
            gcv = A::template scale2<-2>(X::add(w1, w0, site<0>{}));
            cs = A::template scale2<-1>(gcv);
            const C ddown = A::neg_diff(dup, scur, sprev);
            dup = X::sub(snext, scur, site<1>{});
            bcol = X::sub(X::sub(dtr, as_, site<2>{}), cs, site<3>{});
            corr = X::sub(X::mul(-as_, ddown, site<4>{}), X::mul(cs, dup, site<5>{}), site<6>{});
            dv = X::add(X::add(X::add(X::mul(dtr, p0, site<7>{}), t0, site<8>{}), ts0, site<9>{}), corr, site<10>{});
            const P pas = to_p<P>(as_);
            const P divided = XP::rcp(XP::sub(to_p<P>(bcol), XP::mul(cp, pas, site<11>{}), site<12>{}), site<21>{});
            cp = XP::mul(to_p<P>(cs), divided, site<13>{});
            dp = XP::mul(XP::sub(to_p<P>(dv), XP::mul(dp, pas, site<14>{}), site<15>{}), divided, site<16>{});
            sc[k * FS] = cp;
            sd[k * FS] = dp;
            sprev = scur;
            scur = snext;
        }
    }
    cp_async_wait<0>();

    // ---- forward sweep, k = nk-1
    {
        const IDX o = col + (IDX)(nk - 1) * sk;
        const C as_ = A::template scale2<-1>(-gcv);
        bcol = A::sub(dtr, as_);
        const C ddown = A::neg_diff(dup, scur, sprev);
        corr = A::mul(-as_, ddown);
        dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
        const P pas = to_p<P>(as_);
        dp = AP::div(AP::sub(to_p<P>(dv), AP::mul(dp, pas)), AP::sub(to_p<P>(bcol), AP::mul(cp, pas)));
    }

    // ---- backward sweep; pos of level L staged in slot (nk-2-L) % R, field 3
    // (slab factors in fields 0 and 1)
    auto issue_b = [&](int slot, int k) {
        if (k >= 0) {
            cp_async<B>(ring + slot * 6 * BT + 3 * BT, ring_src(pos + (col + (IDX)k * sk)));
            if constexpr (SLAB) {
                cp_async<sizeof(P)>(ring + slot * 6 * BT, sc + k * FS);
                cp_async<sizeof(P)>(ring + slot * 6 * BT + BT, sd + k * FS);
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int u = 0; u < D; ++u) issue_b(u, nk - 2 - u);
    P data = dp;
    {
        const IDX o = col + (IDX)(nk - 1) * sk;
        st<S, C>(out + o, A::mul(dtr, from_p<C>(AP::sub(data, to_p<P>(ld<C, S>(pos + o))))));
    }
    for (int kb = nk - 2; kb >= 0; kb -= R) {
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k = kb - u;
            if (k < 0) break;
            cp_async_wait<D - 1>();
            const C p0 = from_ring<C, S>(ring[u * 6 * BT + 3 * BT], sel_po ^ flip(k));
            P cv, dv_k;
            if constexpr (SLAB) {
                cv = *reinterpret_cast<const P*>(ring + u * 6 * BT);
                dv_k = *reinterpret_cast<const P*>(ring + u * 6 * BT + BT);
            } else {
                cv = sc[k * BT];
                dv_k = sd[k * BT];
            }
            issue_b((u + D) % R, k - D);
            data = XP::sub(dv_k, XP::mul(cv, data, site<17>{}), site<18>{});
            st<S, C>(out + (col + (IDX)k * sk),
                     X::mul(dtr, from_p<C>(XP::sub(data, to_p<P>(p0), site<19>{})), site<20>{}));
        }
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// vertical advection, one warp, 32 consecutive columns, rows staged together
// ---------------------------------------------------------------------------
// With i unit-stride the level-k inputs of a warp's 32 columns are six
// contiguous rows.  The warp copies each row's 16-byte-aligned span with
// 16-byte cp.async chunks and spreads the chunks of all six rows over its
// lanes, so a level costs ceil(6 * CPR / 32) copy instructions per lane
// (2 for float32) instead of six; each lane then waits for its own copies and
// __syncwarp makes the others' visible.  A chunk always contains a byte of
// the row, so it never leaves the row's aligned 16-byte granules.  Factors go
// to the thread's compact slab (level stride fs) and come back through the
// same ring (rows pos, ccol, dcol) in the backward sweep.  All 32 lanes call
// this; lanes at or past `nvalid` compute on stale ring bytes, load their
// direct values from the last valid column and store nothing.
template <class S, class C, int D>
struct WarpRing {
    static constexpr int ES = sizeof(S);
    static constexpr int WB = ES > (int)sizeof(C) ? ES : (int)sizeof(C);
    static constexpr int ROWB = (32 * WB + 16 + 15) / 16 * 16;  // one row's aligned span, at most
    static constexpr int CPR = ROWB / 16;                        // 16-byte chunks per row, at most
    static constexpr int R = D + 1;
    static constexpr int SLOT = 6 * ROWB;
    static constexpr int BYTES = R * SLOT;  // ring bytes per warp
};

template <class S, class C, int D, class IDX>
__device__ __forceinline__ void vadv_warp_column(const S* __restrict__ stage, const S* __restrict__ pos,
                                                 const S* __restrict__ tens, const S* tensstage,
                                                 const S* __restrict__ wcon, S* out, IDX col0, int lane,
                                                 int nvalid, int nk, IDX sk, IDX wsh, C* slab_c0, C* slab_d0,
                                                 int64_t fs, unsigned char* ring) {
    using A = Ar<C>;
    using W = WarpRing<S, C, D>;
    constexpr int R = W::R, ES = W::ES, CPR = W::CPR, ROWB = W::ROWB, SLOT = W::SLOT;
    constexpr int MF = (6 * CPR + 31) / 32;  // forward chunks per lane
    constexpr int MB = (3 * CPR + 31) / 32;  // backward chunks per lane
    const C dtr = konst<C>(3.0 / 20.0);
    const bool valid = lane < nvalid;
    const IDX col = col0 + (IDX)(valid ? lane : nvalid - 1);
    C* sc = slab_c0 + lane;
    C* sd = slab_d0 + lane;
    const int64_t kstep = (int64_t)sk * ES;  // bytes from level k to k+1 in a field
    const int nbytes = nvalid * ES;

    // forward rows at level k: wcon(k+1) shifted, wcon(k+1), stage(k+1), pos(k), tens(k), tensstage(k)
    const unsigned char* const g0 = (const unsigned char*)(wcon + col0 + sk + wsh);
    const unsigned char* const g1 = (const unsigned char*)(wcon + col0 + sk);
    const unsigned char* const g2 = (const unsigned char*)(stage + col0 + sk);
    const unsigned char* const g3 = (const unsigned char*)(pos + col0);
    const unsigned char* const g4 = (const unsigned char*)(tens + col0);
    const unsigned char* const g5 = (const unsigned char*)(tensstage + col0);
    auto gsel = [&](int r) -> const unsigned char* {  // r is per lane: selects, not an indexed array
        return r == 0 ? g0 : r == 1 ? g1 : r == 2 ? g2 : r == 3 ? g3 : r == 4 ? g4 : g5;
    };
    unsigned mis0[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) mis0[f] = (unsigned)((uintptr_t)gsel(f) & 15u);
    // this lane's chunks: slot s = lane + 32 m -> row s / CPR, chunk s % CPR
    const unsigned char* cg[MF];
    int cdst[MF], cidx[MF];
#pragma unroll
    for (int m = 0; m < MF; ++m) {
        const int sidx = lane + 32 * m, r = sidx / CPR;
        cidx[m] = r < 6 ? sidx % CPR : CPR;  // CPR = never issued
        cdst[m] = (r < 6 ? r : 0) * ROWB + (sidx % CPR) * 16;
        cg[m] = gsel(r < 6 ? r : 0);
    }
    auto issue = [&](int slot, int k) {
        if (k < nk - 1) {  // uniform
            const int64_t kb = (int64_t)k * kstep;
#pragma unroll
            for (int m = 0; m < MF; ++m) {
                const uintptr_t a = (uintptr_t)(cg[m] + kb);
                const int n = (int)(((a & 15u) + (unsigned)nbytes + 15u) >> 4);
                if (cidx[m] < n)
                    cp_async<16>(ring + slot * SLOT + cdst[m], (const void*)((a & ~(uintptr_t)15) + 16 * cidx[m]));
            }
        }
        cp_async_commit();
    };
    auto row = [&](int slot, int f, unsigned kmis) -> const S* {
        return (const S*)(ring + slot * SLOT + f * ROWB + ((mis0[f] + kmis) & 15u)) + lane;
    };
    // level L is staged in slot (L-1) % R
#pragma unroll
    for (int u = 0; u < D; ++u) issue(u, 1 + u);

    // ---- forward sweep, k = 0 (direct loads)
    C gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + col + sk + wsh), ld<C, S>(wcon + col + sk)));
    C cs = A::template scale2<-1>(gcv);
    C sprev = ld<C, S>(stage + col);
    C scur = ld<C, S>(stage + col + sk);
    C dup = A::sub(scur, sprev);
    C bcol = A::sub(dtr, cs);
    C corr = A::mul(-cs, dup);
    C dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + col)), ld<C, S>(tens + col)), ldc<C, S>(tensstage + col)), corr);
    C cp = A::div(cs, bcol);
    C dp = A::div(dv, bcol);
    sc[0] = cp;
    sd[0] = dp;

    // ---- forward sweep, 0 < k < nk-1
    for (int kb = 1; kb < nk - 1; kb += R) {
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k = kb + u;
            if (k >= nk - 1) break;  // uniform
            cp_async_wait<D - 1>();
            __syncwarp();
            const unsigned kmis = (unsigned)(((int64_t)k * kstep) & 15);
            const C w1 = cvt<C, S>(*row(u, 0, kmis)), w0 = cvt<C, S>(*row(u, 1, kmis));
            const C snext = cvt<C, S>(*row(u, 2, kmis)), p0 = cvt<C, S>(*row(u, 3, kmis));
            const C t0 = cvt<C, S>(*row(u, 4, kmis)), ts0 = cvt<C, S>(*row(u, 5, kmis));
            issue((u + D) % R, k + D);  // the slot of level k-1: every lane has read it (__syncwarp above)
            const C as_ = A::template scale2<-1>(-gcv);
            gcv = A::template scale2<-2>(A::add(w1, w0));
            cs = A::template scale2<-1>(gcv);
            const C ddown = A::neg_diff(dup, scur, sprev);
            dup = A::sub(snext, scur);
            bcol = A::sub(A::sub(dtr, as_), cs);
            corr = A::sub(A::mul(-as_, ddown), A::mul(cs, dup));
            dv = A::add(A::add(A::add(A::mul(dtr, p0), t0), ts0), corr);
            const C divided = A::rcp(A::sub(bcol, A::mul(cp, as_)));
            cp = A::mul(cs, divided);
            dp = A::mul(A::sub(dv, A::mul(dp, as_)), divided);
            sc[k * fs] = cp;
            sd[k * fs] = dp;
            sprev = scur;
            scur = snext;
        }
    }
    cp_async_wait<0>();
    // every lane's slab stores are read back by other lanes' copies
    __threadfence_block();
    __syncwarp();

    // ---- forward sweep, k = nk-1
    {
        const IDX o = col + (IDX)(nk - 1) * sk;
        const C as_ = A::template scale2<-1>(-gcv);
        bcol = A::sub(dtr, as_);
        const C ddown = A::neg_diff(dup, scur, sprev);
        corr = A::mul(-as_, ddown);
        dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
        dp = A::div(A::sub(dv, A::mul(dp, as_)), A::sub(bcol, A::mul(cp, as_)));
    }

    // ---- backward sweep: rows pos(k), ccol(k), dcol(k) of level k in slot (nk-2-k) % R
    const unsigned char* const gb0 = (const unsigned char*)(pos + col0);
    const unsigned char* const gb1 = (const unsigned char*)slab_c0;
    const unsigned char* const gb2 = (const unsigned char*)slab_d0;
    const int64_t fstep = fs * (int64_t)sizeof(C);  // bytes from level k to k+1 in a slab
    const int fbytes = nvalid * (int)sizeof(C);
    const unsigned char* bg[MB];
    int bdst[MB], bidx[MB], brow[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) {
        const int sidx = lane + 32 * m, r = sidx / CPR;
        bidx[m] = r < 3 ? sidx % CPR : CPR;
        brow[m] = r < 3 ? r : 0;
        bdst[m] = brow[m] * ROWB + (sidx % CPR) * 16;
        bg[m] = brow[m] == 0 ? gb0 : brow[m] == 1 ? gb1 : gb2;
    }
    auto issue_b = [&](int slot, int k) {
        if (k >= 0) {
#pragma unroll
            for (int m = 0; m < MB; ++m) {
                const int64_t st_ = brow[m] == 0 ? kstep : fstep;
                const int nb_ = brow[m] == 0 ? nbytes : fbytes;
                const uintptr_t a = (uintptr_t)(bg[m] + (int64_t)k * st_);
                const int n = (int)(((a & 15u) + (unsigned)nb_ + 15u) >> 4);
                if (bidx[m] < n)
                    cp_async<16>(ring + slot * SLOT + bdst[m], (const void*)((a & ~(uintptr_t)15) + 16 * bidx[m]));
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int u = 0; u < D; ++u) issue_b(u, nk - 2 - u);
    C data = dp;
    if (valid) {
        const IDX o = col + (IDX)(nk - 1) * sk;
        st<S, C>(out + o, A::mul(dtr, A::sub(data, ld<C, S>(pos + o))));
    }
    const unsigned mis_p = (unsigned)((uintptr_t)gb0 & 15u);
    const unsigned mis_c = (unsigned)((uintptr_t)gb1 & 15u), mis_d = (unsigned)((uintptr_t)gb2 & 15u);
    for (int kb = nk - 2; kb >= 0; kb -= R) {
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k = kb - u;
            if (k < 0) break;
            cp_async_wait<D - 1>();
            __syncwarp();
            const unsigned char* sl = ring + u * SLOT;
            const unsigned kp = (unsigned)(((int64_t)k * kstep) & 15), kf = (unsigned)(((int64_t)k * fstep) & 15);
            const C p0 = cvt<C, S>(((const S*)(sl + ((mis_p + kp) & 15u)))[lane]);
            const C cv = ((const C*)(sl + ROWB + ((mis_c + kf) & 15u)))[lane];
            const C dvk = ((const C*)(sl + 2 * ROWB + ((mis_d + kf) & 15u)))[lane];
            issue_b((u + D) % R, k - D);
            data = A::sub(dvk, A::mul(cv, data));
            if (valid) st<S, C>(out + (col + (IDX)k * sk), A::mul(dtr, A::sub(data, p0)));
        }
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// vertical advection, one warp, factors in tensor memory (TMEM)
// ---------------------------------------------------------------------------
// The WSLAB march (rows staged by the warp with 16-byte cp.async chunks) with
// float32 compute, but each thread keeps its column's factors ccol(k),
// dcol(k) in its own TMEM lane instead of a global slab: level k at columns
// 2k, 2k+1 of the warp's column range, written with one tcgen05.st per
// level and read back eight levels at a time with tcgen05.ld ...x16.  Only
// pos rows are staged for the backward sweep.  `tcol` is the TMEM address
// of lane 0 / column 0 of this warp's range (lane field 32 * (warp % 4)); the
// range holds 2 * ceil(nk / 8) * 8 columns.  All 32 lanes must call this.
__device__ __forceinline__ void tmem_st2(uint32_t taddr, float a, float b) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};\n" ::"r"(taddr), "r"(__float_as_uint(a)),
                 "r"(__float_as_uint(b))
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }
// 16 consecutive columns of this thread's lane; returns after the load completed
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&f)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) f[q] = __uint_as_float(r[q]);
}

// Shared-memory accesses by 32-bit shared address (the ring's base converted
// once), so per-level offsets fold into the instructions' immediates.
__device__ __forceinline__ void cp_async16_s(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
template <class S>
__device__ __forceinline__ S lds(uint32_t addr);
template <>
__device__ __forceinline__ float lds<float>(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];\n" : "=f"(v) : "r"(addr) : "memory");
    return v;
}
template <>
__device__ __forceinline__ bf16 lds<bf16>(uint32_t addr) {
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];\n" : "=h"(v) : "r"(addr) : "memory");
    return __ushort_as_bfloat16(v);
}

// KP: how the level stride sk * sizeof(S) sits on 16-byte granules.  KP = 1:
// a multiple of 16 bytes, so every level's rows share level 0's offsets
// within their granules; KP = 2: 8 modulo 16, so even and odd levels each
// share one set of offsets.  Then the copy addresses advance by a constant
// and the staged rows sit at fixed ring offsets (per parity), which takes
// far fewer instructions per level than the general case (KP = 0).
// SA: stage and read the ring through 32-bit shared addresses (cp_async16_s,
// lds) instead of generic pointers.
template <class S, int D, int KP, class IDX, bool SA = false>
__device__ __forceinline__ void vadv_tmem_column(const S* __restrict__ stage, const S* __restrict__ pos,
                                                 const S* __restrict__ tens, const S* tensstage,
                                                 const S* __restrict__ wcon, S* out, IDX col0, int lane, int nvalid,
                                                 int nk, IDX sk, IDX wsh, uint32_t tcol, unsigned char* ring) {
    using C = float;
    using A = Ar<C>;
    using W = WarpRing<S, C, D>;
    constexpr int R = W::R, ES = W::ES, CPR = W::CPR, ROWB = W::ROWB, SLOT = W::SLOT;
    constexpr int MF = (6 * CPR + 31) / 32;  // forward chunks per lane
    constexpr int MB = (CPR + 31) / 32;      // backward chunks per lane (pos only)
    const C dtr = konst<C>(3.0 / 20.0);
    const bool valid = lane < nvalid;
    const IDX col = col0 + (IDX)(valid ? lane : nvalid - 1);
    const int64_t kstep = (int64_t)sk * ES;  // bytes from level k to k+1 in a field
    const int nbytes = nvalid * ES;
    const uint32_t ring_s = (uint32_t)__cvta_generic_to_shared(ring);

    // forward rows at level k: wcon(k+1) shifted, wcon(k+1), stage(k+1), pos(k), tens(k), tensstage(k)
    const unsigned char* const g0 = (const unsigned char*)(wcon + col0 + sk + wsh);
    const unsigned char* const g1 = (const unsigned char*)(wcon + col0 + sk);
    const unsigned char* const g2 = (const unsigned char*)(stage + col0 + sk);
    const unsigned char* const g3 = (const unsigned char*)(pos + col0);
    const unsigned char* const g4 = (const unsigned char*)(tens + col0);
    const unsigned char* const g5 = (const unsigned char*)(tensstage + col0);
    auto gsel = [&](int r) -> const unsigned char* {  // r is per lane: selects, not an indexed array
        return r == 0 ? g0 : r == 1 ? g1 : r == 2 ? g2 : r == 3 ? g3 : r == 4 ? g4 : g5;
    };
    unsigned mis0[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) mis0[f] = (unsigned)((uintptr_t)gsel(f) & 15u);
    // chunk m of this lane: slot s = lane + 32 m -> row s / CPR, chunk s % CPR.  For level
    // parity q (KP > 0): the source of level k is cg[q][m] + k * kstep, and cuse[q][m] says
    // whether the chunk holds a byte of the row.
    const unsigned kph = (unsigned)(kstep & 15);  // granule offset added by one level
    const unsigned char* cg[2][MF];
    int cdst[MF], cidx[MF];
    bool cuse[2][MF];
#pragma unroll
    for (int m = 0; m < MF; ++m) {
        const int sidx = lane + 32 * m, r = sidx / CPR;
        cidx[m] = r < 6 ? sidx % CPR : CPR;  // CPR = never issued
        cdst[m] = (r < 6 ? r : 0) * ROWB + (sidx % CPR) * 16;
        const unsigned char* g = gsel(r < 6 ? r : 0);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const unsigned mq = (unsigned)(((uintptr_t)g + (q ? kph : 0u)) & 15u);
            const int n = (int)((mq + (unsigned)nbytes + 15u) >> 4);
            cuse[q][m] = cidx[m] < n;
            cg[q][m] = KP ? g - mq + 16 * (cuse[q][m] ? cidx[m] : 0) : g;
        }
    }
    auto issue = [&](int slot, int k) {
        if (k < nk - 1) {  // uniform
            const int64_t kb = (int64_t)k * kstep;
#pragma unroll
            for (int m = 0; m < MF; ++m) {
                if constexpr (KP > 0) {
                    const bool odd = KP == 2 && (k & 1);
                    const bool use = odd ? cuse[1][m] : cuse[0][m];
                    if constexpr (SA) {
                        if (use) cp_async16_s(ring_s + slot * SLOT + cdst[m], (const void*)((odd ? cg[1][m] : cg[0][m]) + kb));
                    } else {
                        if (use) cp_async<16>(ring + slot * SLOT + cdst[m], (const void*)((odd ? cg[1][m] : cg[0][m]) + kb));
                    }
                } else {
                    const uintptr_t a = (uintptr_t)(cg[0][m] + kb);
                    const int n = (int)(((a & 15u) + (unsigned)nbytes + 15u) >> 4);
                    if (cidx[m] < n)
                        cp_async<16>(ring + slot * SLOT + cdst[m],
                                     (const void*)((a & ~(uintptr_t)15) + 16 * cidx[m]));
                }
            }
        }
        cp_async_commit();
    };
    // this lane's element of staged row f in slot 0, for even and odd levels (KP > 0)
    const unsigned char* rowb[2][6];
    uint32_t rows_s[2][6];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
        rowb[0][f] = ring + f * ROWB + mis0[f] + lane * ES;
        rowb[1][f] = ring + f * ROWB + ((mis0[f] + kph) & 15u) + lane * ES;
        rows_s[0][f] = ring_s + (uint32_t)(f * ROWB) + mis0[f] + (uint32_t)(lane * ES);
        rows_s[1][f] = ring_s + (uint32_t)(f * ROWB) + ((mis0[f] + kph) & 15u) + (uint32_t)(lane * ES);
    }
    auto rd = [&](int slot, int f, int k) -> C {
        if constexpr (KP > 0 && SA) {
            const bool odd = KP == 2 && (k & 1);
            return cvt<C, S>(lds<S>((odd ? rows_s[1][f] : rows_s[0][f]) + slot * SLOT));
        } else if constexpr (KP > 0) {
            const bool odd = KP == 2 && (k & 1);
            return cvt<C, S>(*(const S*)((odd ? rowb[1][f] : rowb[0][f]) + slot * SLOT));
        } else {
            const unsigned kmis = (unsigned)(((int64_t)k * kstep) & 15);
            return cvt<C, S>(((const S*)(ring + slot * SLOT + f * ROWB + ((mis0[f] + kmis) & 15u)))[lane]);
        }
    };
#pragma unroll
    for (int u = 0; u < D; ++u) issue(u, 1 + u);

    // ---- forward sweep, k = 0 (direct loads)
    C gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + col + sk + wsh), ld<C, S>(wcon + col + sk)));
    C cs = A::template scale2<-1>(gcv);
    C sprev = ld<C, S>(stage + col);
    C scur = ld<C, S>(stage + col + sk);
    C dup = A::sub(scur, sprev);
    C bcol = A::sub(dtr, cs);
    C corr = A::mul(-cs, dup);
    C dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + col)), ld<C, S>(tens + col)), ldc<C, S>(tensstage + col)), corr);
    C cp = A::div(cs, bcol);
    C dp = A::div(dv, bcol);
    tmem_st2(tcol, cp, dp);

    // ---- forward sweep, 0 < k < nk-1
    for (int kb = 1; kb < nk - 1; kb += R) {
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k = kb + u;
            if (k >= nk - 1) break;  // uniform
            cp_async_wait<D - 1>();
            __syncwarp();
            const C w1 = rd(u, 0, k), w0 = rd(u, 1, k);
            const C snext = rd(u, 2, k), p0 = rd(u, 3, k);
            const C t0 = rd(u, 4, k), ts0 = rd(u, 5, k);
            issue((u + D) % R, k + D);  // the slot of level k-1: every lane has read it (__syncwarp above)
            const C as_ = A::template scale2<-1>(-gcv);
            gcv = A::template scale2<-2>(A::add(w1, w0));
            cs = A::template scale2<-1>(gcv);
            const C ddown = A::neg_diff(dup, scur, sprev);
            dup = A::sub(snext, scur);
            bcol = A::sub(A::sub(dtr, as_), cs);
            corr = A::sub(A::mul(-as_, ddown), A::mul(cs, dup));
            dv = A::add(A::add(A::add(A::mul(dtr, p0), t0), ts0), corr);
            const C divided = A::rcp(A::sub(bcol, A::mul(cp, as_)));
            cp = A::mul(cs, divided);
            dp = A::mul(A::sub(dv, A::mul(dp, as_)), divided);
            tmem_st2(tcol + 2u * (uint32_t)k, cp, dp);
            sprev = scur;
            scur = snext;
        }
    }
    cp_async_wait<0>();
    __syncwarp();

    // ---- forward sweep, k = nk-1
    {
        const IDX o = col + (IDX)(nk - 1) * sk;
        const C as_ = A::template scale2<-1>(-gcv);
        bcol = A::sub(dtr, as_);
        const C ddown = A::neg_diff(dup, scur, sprev);
        corr = A::mul(-as_, ddown);
        dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
        dp = A::div(A::sub(dv, A::mul(dp, as_)), A::sub(bcol, A::mul(cp, as_)));
    }
    tmem_wait_st();

    // ---- backward sweep: pos(k) of level k staged in row slot k % 8
    const unsigned char* const gb0 = (const unsigned char*)(pos + col0);
    const unsigned mis_p = (unsigned)((uintptr_t)gb0 & 15u);
    const unsigned char* bg[2][MB];
    int bdst[MB], bidx[MB];
    bool buse[2][MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) {
        const int sidx = lane + 32 * m;
        bidx[m] = sidx < CPR ? sidx : CPR;
        bdst[m] = (sidx < CPR ? sidx : 0) * 16;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const unsigned mq = (unsigned)(((uintptr_t)gb0 + (q ? kph : 0u)) & 15u);
            const int n = (int)((mq + (unsigned)nbytes + 15u) >> 4);
            buse[q][m] = bidx[m] < n;
            bg[q][m] = KP ? gb0 - mq + 16 * (buse[q][m] ? bidx[m] : 0) : gb0;
        }
    }
    // backward ring: 8 row slots of ROWB bytes in the ring's memory, level k in
    // slot k % 8 (so the slot of each level of an 8-level TMEM block is a
    // constant), DB = 7 levels in flight: the slot refilled after reading level
    // k is level k+1's, which every lane has read by the __syncwarp
    constexpr int DB = 7;
    static_assert(8 * ROWB <= R * SLOT, "the backward slots fit in the ring");
    auto issue_b = [&](int bslot, int k) {
        if (k >= 0) {
            const int64_t kb = (int64_t)k * kstep;
#pragma unroll
            for (int m = 0; m < MB; ++m) {
                if constexpr (KP > 0) {
                    const bool odd = KP == 2 && (k & 1);
                    const bool use = odd ? buse[1][m] : buse[0][m];
                    if constexpr (SA) {
                        if (use) cp_async16_s(ring_s + bslot * ROWB + bdst[m], (const void*)((odd ? bg[1][m] : bg[0][m]) + kb));
                    } else {
                        if (use) cp_async<16>(ring + bslot * ROWB + bdst[m], (const void*)((odd ? bg[1][m] : bg[0][m]) + kb));
                    }
                } else {
                    const uintptr_t a = (uintptr_t)(bg[0][m] + kb);
                    const int n = (int)(((a & 15u) + (unsigned)nbytes + 15u) >> 4);
                    if (bidx[m] < n)
                        cp_async<16>(ring + bslot * ROWB + bdst[m],
                                     (const void*)((a & ~(uintptr_t)15) + 16 * bidx[m]));
                }
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int u = 0; u < DB; ++u) issue_b((nk - 2 - u) & 7, nk - 2 - u);
    C data = dp;
    if (valid) {
        const IDX o = col + (IDX)(nk - 1) * sk;
        st<S, C>(out + o, A::mul(dtr, A::sub(data, ld<C, S>(pos + o))));
    }
    const unsigned char* const prow0 = ring + mis_p + lane * ES;  // KP > 0: pos element of slot 0, even levels
    const unsigned char* const prow1 = ring + ((mis_p + kph) & 15u) + lane * ES;  // odd levels
    const uint32_t prow0_s = ring_s + mis_p + (uint32_t)(lane * ES);
    const uint32_t prow1_s = ring_s + ((mis_p + kph) & 15u) + (uint32_t)(lane * ES);
    S* optr = out + col;
    for (int w = (nk - 2) >> 3; w >= 0; --w) {
        float f[16];  // ccol, dcol of levels 8w .. 8w+7
        tmem_ld16(tcol + 16u * (uint32_t)w, f);
#pragma unroll
        for (int q = 7; q >= 0; --q) {
            const int k = 8 * w + q;  // in slot q
            if (k > nk - 2) continue;  // uniform
            cp_async_wait<DB - 1>();
            __syncwarp();
            C p0;
            if constexpr (KP > 0 && SA) {
                const bool odd = KP == 2 && (q & 1);
                p0 = cvt<C, S>(lds<S>((odd ? prow1_s : prow0_s) + (uint32_t)(q * ROWB)));
            } else if constexpr (KP > 0) {
                const bool odd = KP == 2 && (q & 1);
                p0 = cvt<C, S>(*(const S*)((odd ? prow1 : prow0) + q * ROWB));
            } else {
                const unsigned kp = (unsigned)(((int64_t)k * kstep) & 15);
                p0 = cvt<C, S>(((const S*)(ring + q * ROWB + ((mis_p + kp) & 15u)))[lane]);
            }
            issue_b((q + 1) & 7, k - DB);  // (k - 7) % 8: the slot of level k+1
            data = A::sub(f[2 * q + 1], A::mul(f[2 * q], data));
            if (valid) st<S, C>(optr + (IDX)k * sk, A::mul(dtr, A::sub(data, p0)));
        }
    }
    cp_async_wait<0>();
    __syncwarp();
}

}  // namespace sb
