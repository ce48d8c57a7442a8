// Device-side support for serving: seeded field generation and event polling.
//
// sb_fill_batch fills many device fields in one launch with uniform values
// from a counter-based generator, so request fields are created where they
// are used (no host->device copy) and are reproducible on the host.  The
// generator avoids fp64 arithmetic (the fp64 pipe runs at 1/73 of the fp32
// rate here) and spends one 32-bit hash per float32 element, one per two
// bfloat16 elements and two per float64 element.  With H the lowbias32 hash
// (C. Wellons, "Prospecting for hash functions", 2018) and, per field,
//     k0 = H(lo32(seed) ^ 0xA511E9B3) | 1,  k1 = H(hi32(seed) + 0x632BE5AB),
//     k2 = H(k0 ^ k1),  x(n) = lo32(n) * k0 + k1 + hi32(n) * 0x9E3779B9:
//     float32:  v[e] = lo_f + span_f * ((H(x(e)) >> 8) * 2^-24)          (float32)
//     bfloat16: h = H(x(m)) for the pair m = e / 2;  v[2m] from h & 0xFFFF,
//               v[2m+1] from h >> 16, each lo_f + span_f * (bits * 2^-16)
//               in float32, then rounded to bfloat16
//     float64:  h1 = H(x(e)), h2 = H(h1 ^ k2), k = h1 << 21 | h2 >> 11,
//               v[e] = lo + span * (k * 2^-53)                            (double)
// (lo_f = (float)lo, span_f = (float)(hi - lo)); every operation rounded to
// nearest even, no fused multiply-add.  The float64 value is built with
// integer operations when hi - lo is a power of two and lo is 0 or
// -(hi - lo)/2 (the fp64 formula otherwise; both give the same bits).
#include <vector>

#include "common.cuh"

namespace sb {
namespace {

// sb_fill_desc after fill_prepare_kernel has rewritten it in place: the
// per-field constants, computed once instead of by every thread.
struct FillPlan {
    void* ptr;
    uint64_t meta;  // count (bits 0-47) | storage (48-49) | f64 mode (50-51) | e0 + 2048 (52-63)
    uint64_t seed;
    double lo, span;
    float lo_f, span_f;
};
static_assert(sizeof(FillPlan) == sizeof(sb_fill_desc), "FillPlan must fit in place of sb_fill_desc");

constexpr int kF64General = 0;  // fp64 formula
constexpr int kF64FromZero = 1;  // lo = 0, span = 2^P:        v = k * 2^(P-53)
constexpr int kF64Centred = 2;   // lo = -span/2, span = 2^P:  v = (k - 2^52) * 2^(P-53)

__device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

struct FillKeys {
    uint32_t k0, k1, k2;
};

__device__ __forceinline__ FillKeys fill_keys(uint64_t seed) {
    FillKeys k;
    k.k0 = lowbias32((uint32_t)seed ^ 0xA511E9B3u) | 1u;
    k.k1 = lowbias32((uint32_t)(seed >> 32) + 0x632BE5ABu);
    k.k2 = lowbias32(k.k0 ^ k.k1);
    return k;
}

__device__ __forceinline__ uint32_t fill_hash(uint64_t n, const FillKeys& k) {
    return lowbias32((uint32_t)n * k.k0 + k.k1 + (uint32_t)(n >> 32) * 0x9E3779B9u);
}

// lo_f + span_f * (bits * 2^-B) with bits < 2^B (B = 24 or 16): the product
// bits * 2^-B is exact
__device__ __forceinline__ float fill_f32(uint32_t bits, float scale, float lo_f, float span_f) {
    return __fadd_rn(lo_f, __fmul_rn(span_f, __fmul_rn(__uint2float_rn(bits), scale)));
}

__device__ __forceinline__ double fill_f64(uint32_t h1, uint32_t k2, double lo, double span, int mode, int e0) {
    const uint32_t h2 = lowbias32(h1 ^ k2);
    const uint64_t k = ((uint64_t)h1 << 21) | (h2 >> 11);  // 53 bits
    if (mode == kF64General) return __dadd_rn(lo, __dmul_rn(span, __dmul_rn(__ull2double_rn(k), 0x1p-53)));
    // exact: v = x * 2^e0 with x = k - c an integer below 2^53 in magnitude
    const int64_t x = (int64_t)k - (mode == kF64Centred ? (int64_t)1 << 52 : 0);
    if (x == 0) return 0.0;
    const uint64_t sign = x < 0 ? 1ull << 63 : 0;
    const uint64_t a = x < 0 ? (uint64_t)(-x) : (uint64_t)x;
    const int msb = 63 - __clzll((long long)a);  // 0..52
    const uint64_t mant = (a << (52 - msb)) & ((1ull << 52) - 1);
    return __longlong_as_double((long long)(sign | ((uint64_t)(1023 + msb + e0) << 52) | mant));
}

__global__ void fill_prepare_kernel(void* scratch, int n) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    const sb_fill_desc in = ((const sb_fill_desc*)scratch)[d];
    FillPlan out;
    out.ptr = in.ptr;
    out.seed = in.seed;
    out.lo = in.lo;
    out.span = __dsub_rn(in.hi, in.lo);
    out.lo_f = __double2float_rn(in.lo);
    out.span_f = __double2float_rn(out.span);
    int mode = kF64General, e0 = 0;
    const uint64_t b = (uint64_t)__double_as_longlong(out.span);
    const int biased = (int)((b >> 52) & 0x7ff);
    if (in.storage == SB_F64 && (b & ((1ull << 52) - 1)) == 0 && !(b >> 63) && biased >= 1 && biased <= 2046) {
        const int P = biased - 1023;  // span = 2^P
        if (P >= -969) {
            if (in.lo == 0.0) mode = kF64FromZero;
            else if (in.lo == __dmul_rn(-0.5, out.span)) mode = kF64Centred;
            e0 = P - 53;
        }
    }
    out.meta = (uint64_t)in.count | ((uint64_t)in.storage << 48) | ((uint64_t)mode << 50) |
               ((uint64_t)(e0 + 2048) << 52);
    ((FillPlan*)scratch)[d] = out;
}

// One 16-byte store per thread and chunk (V elements); the ragged end and
// fields that are not 16-byte aligned go element by element.
template <int STORAGE>
__device__ __forceinline__ void fill_field(const FillPlan& f, int64_t gtid, int64_t gsize) {
    constexpr int kSize = STORAGE == SB_F64 ? 8 : STORAGE == SB_F32 ? 4 : 2;
    constexpr int V = 16 / kSize;
    const int64_t count = (int64_t)(f.meta & ((1ull << 48) - 1));
    const int mode = (int)((f.meta >> 50) & 3);
    const int e0 = (int)(f.meta >> 52) - 2048;
    const FillKeys keys = fill_keys(f.seed);
    auto value64 = [&](int64_t e) -> uint64_t {
        return (uint64_t)__double_as_longlong(fill_f64(fill_hash((uint64_t)e, keys), keys.k2, f.lo, f.span, mode, e0));
    };
    auto value32 = [&](int64_t e) -> uint32_t {
        return __float_as_uint(fill_f32(fill_hash((uint64_t)e, keys) >> 8, 0x1p-24f, f.lo_f, f.span_f));
    };
    auto bf = [&](uint32_t bits16) -> uint32_t {  // one bfloat16 from 16 random bits
        return __bfloat16_as_ushort(__float2bfloat16_rn(fill_f32(bits16, 0x1p-16f, f.lo_f, f.span_f)));
    };
    char* base = (char*)f.ptr;
    const int64_t chunks = ((uintptr_t)base & 15) == 0 ? count / V : 0;
    for (int64_t c = gtid; c < chunks; c += gsize) {
        uint32_t w[4];
        if constexpr (STORAGE == SB_F64) {
            for (int t = 0; t < 2; ++t) {
                const uint64_t v = value64(c * V + t);
                w[2 * t] = (uint32_t)v;
                w[2 * t + 1] = (uint32_t)(v >> 32);
            }
        } else if constexpr (STORAGE == SB_F32) {
            for (int t = 0; t < 4; ++t) w[t] = value32(c * V + t);
        } else {
            for (int t = 0; t < 4; ++t) {  // elements 2m, 2m+1 with m = c * 4 + t
                const uint32_t h = fill_hash((uint64_t)(c * 4 + t), keys);
                w[t] = bf(h & 0xffffu) | (bf(h >> 16) << 16);
            }
        }
        *(uint4*)(base + c * 16) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    for (int64_t e = chunks * V + gtid; e < count; e += gsize) {
        if constexpr (STORAGE == SB_F64) {
            ((uint64_t*)base)[e] = value64(e);
        } else if constexpr (STORAGE == SB_F32) {
            ((uint32_t*)base)[e] = value32(e);
        } else {
            const uint32_t h = fill_hash((uint64_t)(e >> 1), keys);
            ((uint16_t*)base)[e] = (uint16_t)bf((e & 1) ? (h >> 16) : (h & 0xffffu));
        }
    }
}

__global__ void fill_batch_kernel(const FillPlan* __restrict__ plans, int n) {
    const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int d = 0; d < n; ++d) {
        const FillPlan f = plans[d];
        const int storage = (int)((f.meta >> 48) & 3);
        if (storage == SB_F64) fill_field<SB_F64>(f, gtid, gsize);
        else if (storage == SB_F32) fill_field<SB_F32>(f, gtid, gsize);
        else fill_field<SB_BF16>(f, gtid, gsize);
    }
}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" {

int sb_fill_batch(const sb_fill_desc* descs, int n, void* desc_scratch, void* stream) {
    clear_error();
    SB_CHECK(n >= 0 && (n == 0 || descs), SB_ERR_INVALID, "bad fill descriptors");
    SB_CHECK(n == 0 || desc_scratch, SB_ERR_INVALID, "desc_scratch (device, n descriptors) is NULL");
    if (n == 0) return SB_OK;
    int64_t total = 0;
    for (int d = 0; d < n; ++d) {
        SB_CHECK(descs[d].ptr && descs[d].count >= 0 && descs[d].count < (1ll << 48), SB_ERR_INVALID,
                 "fill descriptor %d is invalid", d);
        SB_CHECK(descs[d].storage >= SB_F64 && descs[d].storage <= SB_BF16, SB_ERR_INVALID,
                 "fill descriptor %d: unknown storage %d", d, descs[d].storage);
        total += descs[d].count;
    }
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SB_CUDA(cudaMemcpyAsync(desc_scratch, descs, sizeof(sb_fill_desc) * n, cudaMemcpyHostToDevice, s));
    fill_prepare_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, s>>>(desc_scratch, n);
    const int64_t want = ceil_div(total, 256 * 4);
    const int blocks = (int)std::min<int64_t>(std::max<int64_t>(want, 1), (int64_t)p->sm_count * 8);
    fill_batch_kernel<<<blocks, 256, 0, s>>>((const FillPlan*)desc_scratch, n);
    SB_CUDA(cudaGetLastError());
    return SB_OK;
}

int sb_stream_wait_event(void* stream, void* event) {
    SB_CUDA(cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)event, 0));
    return SB_OK;
}

int sb_event_query(void* event) {
    const cudaError_t e = cudaEventQuery((cudaEvent_t)event);
    if (e == cudaSuccess) return SB_OK;
    if (e == cudaErrorNotReady) {
        cudaGetLastError();
        return SB_NOT_READY;
    }
    return fail(SB_ERR_CUDA, "cudaEventQuery failed: %s", cudaGetErrorString(e));
}

}  // extern "C"
