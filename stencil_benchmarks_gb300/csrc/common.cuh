// Shared helpers of the sbgb300 library: error reporting, element types,
// correctly rounded arithmetic, device properties and the timed-launch
// wrapper used by every entry point.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include <type_traits>

#include "../../include/sbgb300.h"
#include "f32x2.cuh"
#include "softf64.cuh"

namespace sb {

// ---------------------------------------------------------------------------
// errors: a per-thread message, read back with sb_last_error()
// ---------------------------------------------------------------------------
int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

#define SB_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t sb_e_ = (call);                                                    \
        if (sb_e_ != cudaSuccess) {                                                    \
            return ::sb::fail(SB_ERR_CUDA, "%s failed: %s", #call,                     \
                              cudaGetErrorString(sb_e_));                              \
        }                                                                              \
    } while (0)

#define SB_CHECK(cond, code, ...)                                                      \
    do {                                                                               \
        if (!(cond)) return ::sb::fail((code), __VA_ARGS__);                           \
    } while (0)

// ---------------------------------------------------------------------------
// device properties (cached per device)
// ---------------------------------------------------------------------------
struct DeviceProps {
    int device;
    int sm_count;
    int max_threads_per_block;
    int max_grid_y, max_grid_z;
    int smem_optin;  // max dynamic shared memory per block after opt-in
    int l2_bytes;
};
int device_props(const DeviceProps** out);

// ---------------------------------------------------------------------------
// bounded device-side waits
// ---------------------------------------------------------------------------
// A kernel whose wait gives up sets a process-wide status word that lives in
// page-locked, device-mapped host memory (allocated on the first call of
// status_word), so the host reads it without synchronising.  take_wait_status
// returns SB_ERR_TIMEOUT (with a message) and clears the word if it was set.
int status_word(int** device_ptr);
int take_wait_status();
// Polls of a first wait before a thread block gives up (default 2^20; the
// drain of copies still in flight after a give-up always uses the default).
constexpr int kDefaultWaitPolls = 1 << 20;
int wait_polls();

// ---------------------------------------------------------------------------
// element types
// ---------------------------------------------------------------------------
using bf16 = __nv_bfloat16;

inline int storage_size(int t) { return t == SB_F64 ? 8 : t == SB_F32 ? 4 : t == SB_BF16 ? 2 : 0; }

// load a storage element as compute type C (read-only path)
template <class C, class S>
__device__ __forceinline__ C ld(const S* p);
template <>
__device__ __forceinline__ double ld<double, double>(const double* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ld<float, float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ double ld<double, float>(const float* p) { return (double)__ldg(p); }
template <>
__device__ __forceinline__ float ld<float, bf16>(const bf16* p) {
    return __bfloat162float(__ldg(p));
}
template <>
__device__ __forceinline__ double ld<double, bf16>(const bf16* p) {
    return (double)__bfloat162float(__ldg(p));
}
template <>
__device__ __forceinline__ f32x2 ld<f32x2, double>(const double* p) {
    return f32x2_from_double(__ldg(p));
}

// load through the coherent path (for fields the same kernel also writes)
template <class C, class S>
__device__ __forceinline__ C ldc(const S* p);
template <>
__device__ __forceinline__ double ldc<double, double>(const double* p) { return *p; }
template <>
__device__ __forceinline__ float ldc<float, float>(const float* p) { return *p; }
template <>
__device__ __forceinline__ double ldc<double, float>(const float* p) { return (double)*p; }
template <>
__device__ __forceinline__ float ldc<float, bf16>(const bf16* p) { return __bfloat162float(*p); }
template <>
__device__ __forceinline__ double ldc<double, bf16>(const bf16* p) {
    return (double)__bfloat162float(*p);
}
template <>
__device__ __forceinline__ f32x2 ldc<f32x2, double>(const double* p) {
    return f32x2_from_double(*p);
}

// store a compute value into storage type S with one rounding
template <class S, class C>
__device__ __forceinline__ void st(S* p, C v);
template <>
__device__ __forceinline__ void st<double, double>(double* p, double v) { *p = v; }
template <>
__device__ __forceinline__ void st<float, float>(float* p, float v) { *p = v; }
template <>
__device__ __forceinline__ void st<float, double>(float* p, double v) { *p = __double2float_rn(v); }
template <>
__device__ __forceinline__ void st<bf16, float>(bf16* p, float v) { *p = __float2bfloat16_rn(v); }
template <>
__device__ __forceinline__ void st<double, f32x2>(double* p, f32x2 v) { *p = f32x2_to_double(v); }

// a compile-time constant in compute type C (the float pair of a double)
template <class C>
__device__ __forceinline__ C konst(double v) {
    return (C)v;
}
template <>
__device__ __forceinline__ f32x2 konst<f32x2>(double v) {
    return f32x2_from_double(v);
}

// whole-warp shuffles of compute values
template <class C>
__device__ __forceinline__ C shfl_up(C v, unsigned d) {
    return __shfl_up_sync(0xffffffffu, v, d);
}
template <class C>
__device__ __forceinline__ C shfl_down(C v, unsigned d) {
    return __shfl_down_sync(0xffffffffu, v, d);
}
template <>
__device__ __forceinline__ f32x2 shfl_up<f32x2>(f32x2 v, unsigned d) {
    return {__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
}
template <>
__device__ __forceinline__ f32x2 shfl_down<f32x2>(f32x2 v, unsigned d) {
    return {__shfl_down_sync(0xffffffffu, v.hi, d), __shfl_down_sync(0xffffffffu, v.lo, d)};
}

// ---------------------------------------------------------------------------
// arithmetic with exactly one IEEE rounding per operation (never contracted
// into FMA), matching numpy's evaluation of the reference's verification.
// ---------------------------------------------------------------------------
template <class C>
struct Ar;

// Rare fp64 paths of Ar<double>, kept out of line: inline, the compiler
// evaluates them under a predicate on every call, and each predicated fp64
// instruction still takes a slot of GB300's narrow fp64 pipe.
static __device__ __noinline__ double fp64_mul_cold(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double fp64_sub_cold(double a, double b) { return __dsub_rn(a, b); }
static __device__ __noinline__ double fp64_limit_cold(double f, double a1, double a0) {
    return (__dmul_rn(f, __dsub_rn(a1, a0)) > 0.0) ? 0.0 : f;
}

template <>
struct Ar<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double rcp(double a) { return __drcp_rn(a); }

    // Exact x * 2^e for small |e|: adjusts the exponent field with integer
    // arithmetic when x and the result are normal numbers, otherwise falls
    // back to a (correctly rounded) multiplication.  Saves an fp64 pipe slot.
    template <int E>
    static __device__ __forceinline__ double scale2(double x) {
        const int hi = __double2hiint(x);
        const int e = (hi >> 20) & 0x7ff;
        const int en = e + E;
        if (e >= 1 && e <= 2046 && en >= 1 && en <= 2046) {
            return __hiloint2double(hi + E * (1 << 20), __double2loint(x));
        }
        return fp64_mul_cold(x, E >= 0 ? (double)(1 << (E >= 0 ? E : 0))
                                       : 1.0 / (double)(1 << (E >= 0 ? 0 : -E)));
    }

    // Exact `(f * (a1 - a0) > 0) ? 0 : f` (the reference's flux limiter).
    // Sign logic on the bit patterns replaces the fp64 subtract, multiply
    // and compare whenever the product provably neither underflows nor
    // involves zero/inf/nan; the rare remaining cases evaluate it literally.
    static __device__ __forceinline__ double limit(double f, double a1, double a0) {
        const int hf = __double2hiint(f);
        const int h1 = __double2hiint(a1);
        const int h0 = __double2hiint(a0);
        const unsigned ef = ((unsigned)hf >> 20) & 0x7ffu;
        const unsigned e1 = ((unsigned)h1 >> 20) & 0x7ffu;
        const unsigned e0 = ((unsigned)h0 >> 20) & 0x7ffu;
        const unsigned emin = e1 < e0 ? e1 : e0;
        const long long b1 = __double_as_longlong(a1);
        const long long b0 = __double_as_longlong(a0);
        // f, a1, a0 finite normal; a1 != a0; |f| * |a1 - a0| >= 2^(ef-1023) * 2^(emin-1075)
        // stays above the underflow threshold 2^-1075 when ef + emin >= 1024.
        if (ef - 1u < 2046u && e1 - 1u < 2046u && e0 - 1u < 2046u && b1 != b0 && ef + emin >= 1024u) {
            // sign(a1 - a0): compare as sign-magnitude integers
            bool gt;
            if ((b1 ^ b0) < 0) {
                gt = b1 >= 0;  // different signs: the non-negative one is larger
            } else {
                gt = (b1 >= 0) ? (b1 > b0) : (b1 < b0);
            }
            const bool fpos = hf >= 0;
            return (fpos == gt) ? 0.0 : f;  // same sign -> product > 0 -> limited
        }
        return fp64_limit_cold(f, a1, a0);
    }

    // -x, except that (a - b) and (b - a) both give +0 when a == b: returns
    // the exact value of (b - a) given x = (a - b).
    static __device__ __forceinline__ double neg_diff(double x, double a, double b) {
        if ((__double_as_longlong(x) << 1) == 0) return fp64_sub_cold(b, a);
        return -x;
    }
};

// ---------------------------------------------------------------------------
// binary64 operations on the integer pipe (softf64.cuh): bit-identical to the
// fp64 instructions; the cases the integer path declines (NaN/inf operands,
// subnormal or overflowing results) take the fp64 instruction out of line.
// ---------------------------------------------------------------------------
static __device__ __noinline__ double fp64_add_cold(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ double iadd(double a, double b) {
    uint64_t r;
    if (sf::add(sf::bits(a), sf::bits(b), r)) return sf::from_bits(r);
    return fp64_add_cold(a, b);
}
__device__ __forceinline__ double isub(double a, double b) {
    uint64_t r;
    if (sf::sub(sf::bits(a), sf::bits(b), r)) return sf::from_bits(r);
    return fp64_sub_cold(a, b);
}
__device__ __forceinline__ double imul(double a, double b) {
    uint64_t r;
    if (sf::mul(sf::bits(a), sf::bits(b), r)) return sf::from_bits(r);
    return fp64_mul_cold(a, b);
}
static __device__ __noinline__ double fp64_rcp_cold(double a) { return __drcp_rn(a); }
__device__ __forceinline__ double ircp(double a) {
    uint64_t r;
    if (sf::rcp(sf::bits(a), r)) return sf::from_bits(r);
    return fp64_rcp_cold(a);
}

// Arithmetic with a per-site choice of pipe.  A kernel numbers its operation
// sites (site<K>); for float64 compute, bit K of the placement mask PL sends
// site K to the integer pipe (iadd / isub / imul / ircp), the others use the fp64
// instructions.  The results are the same bits either way; only the balance
// between the two pipes changes.  Other compute types ignore the mask.
template <int K>
using site = std::integral_constant<int, K>;

template <class C, uint32_t PL>
struct Mix {
    template <int K>
    static __device__ __forceinline__ C add(C a, C b, site<K>) { return Ar<C>::add(a, b); }
    template <int K>
    static __device__ __forceinline__ C sub(C a, C b, site<K>) { return Ar<C>::sub(a, b); }
    template <int K>
    static __device__ __forceinline__ C mul(C a, C b, site<K>) { return Ar<C>::mul(a, b); }
    template <int K>
    static __device__ __forceinline__ C rcp(C a, site<K>) { return Ar<C>::rcp(a); }
};

template <uint32_t PL>
struct Mix<double, PL> {
    template <int K>
    static __device__ __forceinline__ double add(double a, double b, site<K>) {
        if constexpr (((PL >> K) & 1u) != 0u) return iadd(a, b);
        else return __dadd_rn(a, b);
    }
    template <int K>
    static __device__ __forceinline__ double sub(double a, double b, site<K>) {
        if constexpr (((PL >> K) & 1u) != 0u) return isub(a, b);
        else return __dsub_rn(a, b);
    }
    template <int K>
    static __device__ __forceinline__ double mul(double a, double b, site<K>) {
        if constexpr (((PL >> K) & 1u) != 0u) return imul(a, b);
        else return __dmul_rn(a, b);
    }
    template <int K>
    static __device__ __forceinline__ double rcp(double a, site<K>) {
        if constexpr (((PL >> K) & 1u) != 0u) return ircp(a);
        else return __drcp_rn(a);
    }
};

template <>
struct Ar<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float rcp(float a) { return __frcp_rn(a); }
    template <int E>
    static __device__ __forceinline__ float scale2(float x) {
        return __fmul_rn(x, E >= 0 ? (float)(1 << (E >= 0 ? E : 0))
                                   : 1.0f / (float)(1 << (E >= 0 ? 0 : -E)));
    }
    static __device__ __forceinline__ float limit(float f, float a1, float a0) {
        return (__fmul_rn(f, __fsub_rn(a1, a0)) > 0.0f) ? 0.0f : f;
    }
    static __device__ __forceinline__ float neg_diff(float x, float a, float b) {
        return (x == 0.0f) ? __fsub_rn(b, a) : -x;
    }
};

// Float-pair compute (f32x2.cuh): about 48 significant bits on the fp32 pipe,
// within a few 2^-48 of the float64 result per operation instead of
// bit-identical to it.  The limiter compares the pair values exactly.
template <>
struct Ar<f32x2> {
    static __device__ __forceinline__ f32x2 add(f32x2 a, f32x2 b) { return sb::add(a, b); }
    static __device__ __forceinline__ f32x2 sub(f32x2 a, f32x2 b) { return sb::sub(a, b); }
    static __device__ __forceinline__ f32x2 mul(f32x2 a, f32x2 b) { return sb::mul(a, b); }
    static __device__ __forceinline__ f32x2 div(f32x2 a, f32x2 b) { return sb::div(a, b); }
    static __device__ __forceinline__ f32x2 rcp(f32x2 a) { return sb::rcp(a); }
    template <int E>
    static __device__ __forceinline__ f32x2 scale2(f32x2 x) {
        return sb::scale2<E>(x);
    }
    // (f * (a1 - a0) > 0) ? 0 : f, with the sign of a1 - a0 from an exact comparison
    static __device__ __forceinline__ f32x2 limit(f32x2 f, f32x2 a1, f32x2 a0) {
        const int c = cmp(a1, a0);
        const int fs = (f.hi > 0.0f) - (f.hi < 0.0f);
        return (fs != 0 && fs == c) ? f32x2(0) : f;
    }
    static __device__ __forceinline__ f32x2 neg_diff(f32x2 x, f32x2, f32x2) { return sb::neg(x); }
};

// ---------------------------------------------------------------------------
// asynchronous global -> shared copies (cp.async, per thread, 4/8/16 bytes).
// Completion is tracked per thread in commit groups, so a thread can keep
// several levels of loads in flight without tying up registers.
// ---------------------------------------------------------------------------
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gsrc) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem_dst);
    if (BYTES == 4) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gsrc) : "memory");
    } else if (BYTES == 8) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
    } else {
        static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// storage -> compute conversion of a value already in registers/shared memory
template <class C, class S>
__device__ __forceinline__ C cvt(S v);
template <>
__device__ __forceinline__ double cvt<double, double>(double v) { return v; }
template <>
__device__ __forceinline__ float cvt<float, float>(float v) { return v; }
template <>
__device__ __forceinline__ double cvt<double, float>(float v) { return (double)v; }
template <>
__device__ __forceinline__ float cvt<float, bf16>(bf16 v) { return __bfloat162float(v); }
template <>
__device__ __forceinline__ f32x2 cvt<f32x2, double>(double v) { return f32x2_from_double(v); }
template <>
__device__ __forceinline__ f32x2 cvt<f32x2, f32x2>(f32x2 v) { return v; }

// V consecutive storage elements moved as one aligned vector of V*sizeof(S)
// bytes (4, 8 or 16), converted to / rounded from compute type C per element.
template <int B>
struct RawVec;
template <>
struct RawVec<4> {
    using T = unsigned;
};
template <>
struct RawVec<8> {
    using T = uint2;
};
template <>
struct RawVec<16> {
    using T = uint4;
};

template <class S, class C, int V>
__device__ __forceinline__ void ld_vec(const S* p, C (&o)[V]) {
    using R = typename RawVec<(int)sizeof(S) * V>::T;
    const R r = __ldg(reinterpret_cast<const R*>(p));
    S e[V];
    memcpy(e, &r, sizeof(R));
#pragma unroll
    for (int q = 0; q < V; ++q) o[q] = cvt<C, S>(e[q]);
}

template <class S, class C, int V>
__device__ __forceinline__ void st_vec(S* p, const C (&v)[V]) {
    using R = typename RawVec<(int)sizeof(S) * V>::T;
    S e[V];
#pragma unroll
    for (int q = 0; q < V; ++q) st<S, C>(&e[q], v[q]);
    R r;
    memcpy(&r, e, sizeof(R));
    *reinterpret_cast<R*>(p) = r;
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------

// Run `launch()` on `stream`; with `time_s` non-NULL time it with CUDA events
// (reference: stencils/cuda_hip/templates/base.j2:145-190).
template <class F>
int timed(cudaStream_t stream, double* time_s, F&& launch) {
    cudaEvent_t start = nullptr, stop = nullptr;
    if (time_s) {
        SB_CUDA(cudaEventCreate(&start));
        cudaError_t e = cudaEventCreate(&stop);
        if (e != cudaSuccess) {
            cudaEventDestroy(start);
            return fail(SB_ERR_CUDA, "cudaEventCreate failed: %s", cudaGetErrorString(e));
        }
        e = cudaEventRecord(start, stream);
        if (e != cudaSuccess) {
            cudaEventDestroy(start);
            cudaEventDestroy(stop);
            return fail(SB_ERR_CUDA, "cudaEventRecord failed: %s", cudaGetErrorString(e));
        }
    }
    int rc = launch();
    if (rc == SB_OK) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(SB_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    }
    if (time_s) {
        if (rc == SB_OK) {
            cudaError_t e = cudaEventRecord(stop, stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(stop);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, start, stop);
            if (e != cudaSuccess) {
                rc = fail(SB_ERR_CUDA, "timing the launch failed: %s", cudaGetErrorString(e));
            } else {
                *time_s = (double)ms / 1000.0;
            }
        }
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
    }
    return rc;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Shared validation of a 3D field description.
int check_domain(int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk);

}  // namespace sb
