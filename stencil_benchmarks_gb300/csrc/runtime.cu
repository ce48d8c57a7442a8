// Library plumbing behind the C ABI: error strings, device queries, memory,
// streams/events, L2 flush and the arithmetic-rate probe.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace sb {

namespace {
thread_local std::string g_error;

std::mutex g_props_mutex;
std::vector<DeviceProps> g_props;  // indexed by device, device == -1 when unset
}  // namespace

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

void clear_error() { g_error.clear(); }

int device_props(const DeviceProps** out) {
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_props_mutex);
    if ((int)g_props.size() <= dev) g_props.resize(dev + 1, DeviceProps{-1, 0, 0, 0, 0, 0, 0});
    DeviceProps& p = g_props[dev];
    if (p.device != dev) {
        cudaDeviceProp prop;
        SB_CUDA(cudaGetDeviceProperties(&prop, dev));
        p.sm_count = prop.multiProcessorCount;
        p.max_threads_per_block = prop.maxThreadsPerBlock;
        p.max_grid_y = prop.maxGridSize[1];
        p.max_grid_z = prop.maxGridSize[2];
        p.smem_optin = (int)prop.sharedMemPerBlockOptin;
        p.l2_bytes = prop.l2CacheSize;
        p.device = dev;
    }
    *out = &p;
    return SB_OK;
}

namespace {
std::once_flag g_status_once;
int* g_status = nullptr;  // host address == device address (unified addressing)
cudaError_t g_status_error = cudaSuccess;
std::atomic<int> g_wait_polls{kDefaultWaitPolls};
}  // namespace

int status_word(int** device_ptr) {
    std::call_once(g_status_once, [] {
        void* p = nullptr;
        g_status_error = cudaHostAlloc(&p, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable);
        if (g_status_error == cudaSuccess) {
            g_status = static_cast<int*>(p);
            __atomic_store_n(g_status, 0, __ATOMIC_RELEASE);
        }
    });
    if (!g_status)
        return fail(SB_ERR_CUDA, "cudaHostAlloc of the wait-status word failed: %s",
                    cudaGetErrorString(g_status_error));
    *device_ptr = g_status;
    return SB_OK;
}

int take_wait_status() {
    if (!g_status || !__atomic_exchange_n(g_status, 0, __ATOMIC_ACQ_REL)) return SB_OK;
    return fail(SB_ERR_TIMEOUT,
                "a thread block of an earlier launch gave up waiting for its tensor copies: that launch's "
                "output is incomplete");
}

int wait_polls() { return g_wait_polls.load(std::memory_order_relaxed); }

int check_domain(int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk) {
    SB_CHECK(ni >= 0 && nj >= 0 && nk >= 0, SB_ERR_INVALID,
             "negative domain size (%lld, %lld, %lld)", (long long)ni, (long long)nj, (long long)nk);
    SB_CHECK(ni < (1LL << 31) && nj < (1LL << 31) && nk < (1LL << 31), SB_ERR_INVALID,
             "domain size exceeds 2^31 along an axis");
    SB_CHECK(si != 0 && sj != 0 && sk != 0, SB_ERR_INVALID, "zero stride");
    return SB_OK;
}

// ---------------------------------------------------------------------------
// L2 flush buffer (one per device, grown on demand)
// ---------------------------------------------------------------------------
namespace {
std::mutex g_flush_mutex;
std::vector<std::pair<void*, size_t>> g_flush;

__global__ void flush_kernel(uint4* buf, size_t n, unsigned salt) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        buf[i] = make_uint4(salt, (unsigned)i, salt ^ 0x5bd1e995u, (unsigned)(i >> 32));
    }
}

// A 64-bit leading-zero count from the exponent of a round-toward-zero
// unsigned-to-float conversion of the upper (or, when it is zero, the lower)
// 32-bit word, exactly floor(log2(w)) (H. S. Warren, Hacker's Delight, 2nd
// ed., sec. 5-3): the rate probe's comparison for the leading-zero
// instruction that the integer add uses.  x must be non-zero.
__device__ __forceinline__ int clz64_by_conversion(uint64_t x) {
    const uint32_t hi = (uint32_t)(x >> 32);
    const uint32_t w = hi ? hi : (uint32_t)x;
    return (hi ? 158 : 190) - (int)(__float_as_uint(__uint2float_rz(w)) >> 23);
}

// Dependent-free arithmetic chains for the rate probe: each thread runs 8
// independent accumulators so the pipe, not latency, is the limit.
template <int KIND>
__global__ void arith_probe_kernel(double* out, int iters, double x) {
    if (KIND == 2) {
        float a[8];
        for (int u = 0; u < 8; ++u) a[u] = (float)x + (float)(threadIdx.x + u);
        const float m = 0.999f, c = 1e-3f;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = __fmaf_rn(a[u], m, c);
        }
        float s = 0.f;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678f) out[0] = s;
    } else if (KIND == 3) {  // f64 -> f32 conversion (the way back is an integer move)
        double a[8];
        for (int u = 0; u < 8; ++u) a[u] = x + (double)(threadIdx.x + u);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u)
                a[u] = __hiloint2double(__float_as_int(__double2float_rn(a[u])) ^ 0x40000000, it);
        }
        double s = 0.0;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678) out[0] = s;
    } else if (KIND == 4) {  // f32 -> f64 conversion (the way back is an integer move)
        float a[8];
        for (int u = 0; u < 8; ++u) a[u] = (float)x + (float)(threadIdx.x + u);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = __int_as_float(__double2hiint((double)a[u]) ^ it);
        }
        float s = 0.f;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678f) out[0] = s;
    } else if (KIND == 5) {  // 32-bit integer shift, xor, multiply (3 operations a step, not foldable)
        unsigned a[8];
        for (int u = 0; u < 8; ++u) a[u] = (unsigned)x + threadIdx.x + u;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = (a[u] ^ (a[u] >> 15)) * 0x2C1B3C6Du;
        }
        unsigned s = 0;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345u) out[0] = s;
    } else if (KIND == 7) {  // s32 -> f32 conversion (the way back is an integer move)
        float a[8];
        for (int u = 0; u < 8; ++u) a[u] = (float)x + (float)(threadIdx.x + u);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = __int2float_rn(__float_as_int(a[u]) ^ it);
        }
        float s = 0.f;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678f) out[0] = s;
    } else if (KIND == 6) {  // u32 -> f32 conversion (the way back is an integer move)
        float a[8];
        for (int u = 0; u < 8; ++u) a[u] = (float)x + (float)(threadIdx.x + u);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = __uint2float_rn(__float_as_uint(a[u]) ^ (unsigned)it);
        }
        float s = 0.f;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678f) out[0] = s;
    } else if (KIND == 10 || KIND == 11) {  // f64 add chains beside 32-bit integer chains (10), or the integer chains alone (11)
        double a[8];
        unsigned b[8];
        for (int u = 0; u < 8; ++u) {
            a[u] = x + (double)(threadIdx.x + u);
            b[u] = (unsigned)x + threadIdx.x + u;
        }
        const double c = 1e-3;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (KIND == 10) a[u] = __dadd_rn(a[u], c);
#pragma unroll
                for (int r = 0; r < 16; ++r) b[u] = (b[u] ^ (b[u] >> 15)) * 0x2C1B3C6Du;
            }
        }
        double s = 0.0;
        unsigned t = 0;
        for (int u = 0; u < 8; ++u) {
            s += a[u];
            t += b[u];
        }
        if (s == 12345.678 || t == 12345u) out[0] = s;
    } else if (KIND == 12 || KIND == 13) {  // binary64 reciprocal: integer pipe (12), __drcp_rn (13)
        double a[8];
        for (int u = 0; u < 8; ++u) a[u] = x + (double)(threadIdx.x + u);
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = KIND == 12 ? ircp(a[u]) : __drcp_rn(a[u]);
        }
        double s = 0.0;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678) out[0] = s;
    } else if (KIND >= 14 && KIND <= 17) {
        // 64-bit leading-zero counts: the instruction (__clzll; 14) or the
        // conversion form (15), each in a chain with a rotate and an add;
        // 16 / 17: the same chains with one f64 add beside each count
        // (counted as adds: the fp64 rate if the two do not compete)
        uint64_t v[8];
        double a[8];
        for (int u = 0; u < 8; ++u) {
            v[u] = 0x9E3779B97F4A7C15ull * (uint64_t)(threadIdx.x + u + 1);
            a[u] = x + (double)(threadIdx.x + u);
        }
        const double c = 1e-3;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int z = (KIND == 14 || KIND == 16) ? __clzll((long long)v[u]) : clz64_by_conversion(v[u]);
                v[u] = (((v[u] << 5) | (v[u] >> 59)) + (uint64_t)z) | 1ull;
                if (KIND >= 16) a[u] = __dadd_rn(a[u], c);
            }
        }
        double s = 0.0;
        uint64_t t = 0;
        for (int u = 0; u < 8; ++u) {
            s += a[u];
            t += v[u];
        }
        if (s == 12345.678 || t == 12345u) out[0] = s;
    } else if (KIND >= 18 && KIND <= 20) {
        // one f64 add per step beside: the integer-arithmetic binary64 add
        // (18), a 64-bit shift by a variable amount (19), or a 64-bit add and
        // a 64-bit compare (20); counted as f64 adds, so each runs at the fp64
        // rate (kind 0) unless the integer work also occupies the fp64 pipe
        double a[8], b[8];
        uint64_t v[8];
        for (int u = 0; u < 8; ++u) {
            a[u] = x + (double)(threadIdx.x + u);
            b[u] = 1.5 + (double)u;
            v[u] = 0x9E3779B97F4A7C15ull * (uint64_t)(threadIdx.x + u + 1);
        }
        const double c = 1e-3;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                a[u] = __dadd_rn(a[u], c);
                if (KIND == 18) {
                    b[u] = iadd(b[u], 1e-7);
                } else if (KIND == 19) {
                    const unsigned s = (unsigned)v[u] & 63u;
                    v[u] = (v[u] << s) ^ (v[u] >> (63u - s)) ^ 0x5bd1e995ull;
                } else {
                    const uint64_t w = v[u] + 0x9E3779B97F4A7C15ull;
                    v[u] = (w < v[u]) ? w ^ 0x2545F4914F6CDD1Dull : w;
                }
            }
        }
        double s = 0.0;
        uint64_t t = 0;
        for (int u = 0; u < 8; ++u) {
            s += a[u] + b[u];
            t += v[u];
        }
        if (s == 12345.678 || t == 12345u) out[0] = s;
    } else if (KIND == 8 || KIND == 9) {  // binary64 add / mul on the integer pipe (softf64.cuh)
        double a[8];
        for (int u = 0; u < 8; ++u) a[u] = x + (double)(threadIdx.x + u);
        const double m = 0.999, c = 1e-3;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = KIND == 8 ? iadd(a[u], c) : imul(a[u], m);
        }
        double s = 0.0;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678) out[0] = s;
    } else {
        double a[8];
        for (int u = 0; u < 8; ++u) a[u] = x + (double)(threadIdx.x + u);
        const double m = 0.999, c = 1e-3;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = KIND == 0 ? __dadd_rn(a[u], c) : __fma_rn(a[u], m, c);
        }
        double s = 0.0;
        for (int u = 0; u < 8; ++u) s += a[u];
        if (s == 12345.678) out[0] = s;
    }
}
// Copy through the SMs (16-byte loads and stores, 4 in flight per thread):
// either side may be page-locked host memory, which the loads or stores then
// reach over the host link; the tail that is not a whole vector goes bytewise.
__global__ void __launch_bounds__(512) sm_copy_kernel(uint4* __restrict__ dst, const uint4* __restrict__ src,
                                                      size_t nvec, unsigned char* __restrict__ dtail,
                                                      const unsigned char* __restrict__ stail, size_t ntail) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < nvec; i += 4 * stride) {
        const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < nvec; i += stride) dst[i] = src[i];
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < ntail; t += stride) dtail[t] = stail[t];
}

// The integer-arithmetic binary64 operations (softf64.cuh) element-wise, for
// checking the device build against the host's IEEE arithmetic.
__global__ void soft_f64_kernel(int op, const double* __restrict__ a, const double* __restrict__ b,
                                double* __restrict__ out, int64_t n) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double x = a[q];
        out[q] = op == 0 ? iadd(x, b[q]) : op == 1 ? isub(x, b[q]) : op == 2 ? imul(x, b[q]) : ircp(x);
    }
}
}  // namespace

}  // namespace sb

using namespace sb;

extern "C" {

const char* sb_last_error(void) { return g_error.c_str(); }

int sb_version(void) { return 10000; }

int sb_device_count(int* count) {
    SB_CHECK(count, SB_ERR_INVALID, "count is NULL");
    *count = 0;
    cudaError_t e = cudaGetDeviceCount(count);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) {
        cudaGetLastError();
        *count = 0;
        return SB_OK;
    }
    SB_CUDA(e);
    return SB_OK;
}

int sb_set_device(int device) {
    SB_CUDA(cudaSetDevice(device));
    return SB_OK;
}

int sb_get_device(int* device) {
    SB_CHECK(device, SB_ERR_INVALID, "device is NULL");
    SB_CUDA(cudaGetDevice(device));
    return SB_OK;
}

int sb_device_info(int device, char* name, int name_len, int* sm_count, int* cc_major,
                   int* cc_minor, size_t* total_mem, int* l2_bytes, int* smem_optin) {
    cudaDeviceProp prop;
    SB_CUDA(cudaGetDeviceProperties(&prop, device));
    if (name && name_len > 0) {
        strncpy(name, prop.name, (size_t)name_len - 1);
        name[name_len - 1] = '\0';
    }
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    if (total_mem) *total_mem = prop.totalGlobalMem;
    if (l2_bytes) *l2_bytes = prop.l2CacheSize;
    if (smem_optin) *smem_optin = (int)prop.sharedMemPerBlockOptin;
    return SB_OK;
}

int sb_synchronize(void) {
    SB_CUDA(cudaDeviceSynchronize());
    return take_wait_status();
}

int sb_kernel_status(void) { return take_wait_status(); }

int sb_debug_wait_limit(int polls) {
    SB_CHECK(polls >= -1, SB_ERR_INVALID, "polls must be >= -1");
    g_wait_polls.store(polls < 0 ? kDefaultWaitPolls : polls, std::memory_order_relaxed);
    return SB_OK;
}

int sb_malloc(void** ptr, size_t bytes) {
    SB_CHECK(ptr, SB_ERR_INVALID, "ptr is NULL");
    *ptr = nullptr;
    if (bytes == 0) return SB_OK;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(SB_ERR_NOMEM, "cudaMalloc of %zu bytes failed: out of device memory", bytes);
    }
    SB_CUDA(e);
    return SB_OK;
}

int sb_free(void* ptr) {
    if (ptr) SB_CUDA(cudaFree(ptr));
    return SB_OK;
}

int sb_malloc_host(void** ptr, size_t bytes) {
    SB_CHECK(ptr, SB_ERR_INVALID, "ptr is NULL");
    *ptr = nullptr;
    if (bytes == 0) return SB_OK;
    cudaError_t e = cudaMallocHost(ptr, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(SB_ERR_NOMEM, "cudaMallocHost of %zu bytes failed", bytes);
    }
    SB_CUDA(e);
    return SB_OK;
}

int sb_free_host(void* ptr) {
    if (ptr) SB_CUDA(cudaFreeHost(ptr));
    return SB_OK;
}

int sb_memcpy(void* dst, const void* src, size_t bytes, int kind) {
    SB_CHECK(kind >= 0 && kind <= 4, SB_ERR_INVALID, "bad memcpy kind %d", kind);
    if (bytes == 0) return SB_OK;
    SB_CUDA(cudaMemcpy(dst, src, bytes, (cudaMemcpyKind)kind));
    return SB_OK;
}

int sb_memcpy_async(void* dst, const void* src, size_t bytes, int kind, void* stream) {
    SB_CHECK(kind >= 0 && kind <= 4, SB_ERR_INVALID, "bad memcpy kind %d", kind);
    if (bytes == 0) return SB_OK;
    SB_CUDA(cudaMemcpyAsync(dst, src, bytes, (cudaMemcpyKind)kind, (cudaStream_t)stream));
    return SB_OK;
}

int sb_memcpy_sm(void* dst, const void* src, size_t bytes, void* stream) {
    clear_error();
    SB_CHECK((dst && src) || bytes == 0, SB_ERR_INVALID, "NULL pointer");
    if (bytes == 0) return SB_OK;
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    const bool vec = ((uintptr_t)dst % 16 == 0) && ((uintptr_t)src % 16 == 0);
    const size_t nvec = vec ? bytes / 16 : 0;
    const int blocks = p->sm_count * 4;
    sm_copy_kernel<<<blocks, 512, 0, (cudaStream_t)stream>>>((uint4*)dst, (const uint4*)src, nvec,
                                                            (unsigned char*)dst + nvec * 16,
                                                            (const unsigned char*)src + nvec * 16,
                                                            bytes - nvec * 16);
    SB_CUDA(cudaGetLastError());
    return SB_OK;
}

int sb_memset(void* dst, int value, size_t bytes) {
    if (bytes == 0) return SB_OK;
    SB_CUDA(cudaMemset(dst, value, bytes));
    return SB_OK;
}

int sb_mem_info(size_t* free_bytes, size_t* total_bytes) {
    size_t f = 0, t = 0;
    SB_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return SB_OK;
}

int sb_stream_create(void** stream) {
    SB_CHECK(stream, SB_ERR_INVALID, "stream is NULL");
    cudaStream_t s;
    SB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *stream = (void*)s;
    return SB_OK;
}

int sb_stream_destroy(void* stream) {
    if (stream) SB_CUDA(cudaStreamDestroy((cudaStream_t)stream));
    return SB_OK;
}

int sb_stream_synchronize(void* stream) {
    SB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return take_wait_status();
}

int sb_event_create(void** event) {
    SB_CHECK(event, SB_ERR_INVALID, "event is NULL");
    cudaEvent_t e;
    SB_CUDA(cudaEventCreate(&e));
    *event = (void*)e;
    return SB_OK;
}

int sb_event_destroy(void* event) {
    if (event) SB_CUDA(cudaEventDestroy((cudaEvent_t)event));
    return SB_OK;
}

int sb_event_record(void* event, void* stream) {
    SB_CUDA(cudaEventRecord((cudaEvent_t)event, (cudaStream_t)stream));
    return SB_OK;
}

int sb_event_synchronize(void* event) {
    SB_CUDA(cudaEventSynchronize((cudaEvent_t)event));
    return take_wait_status();
}

int sb_event_elapsed(void* start, void* stop, double* seconds) {
    float ms = 0.f;
    SB_CUDA(cudaEventElapsedTime(&ms, (cudaEvent_t)start, (cudaEvent_t)stop));
    if (seconds) *seconds = ms / 1000.0;
    return SB_OK;
}

int sb_l2_flush(void* stream) {
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    const size_t bytes = (size_t)(p->l2_bytes > 0 ? p->l2_bytes : (128 << 20)) * 2;
    void* buf = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_flush_mutex);
        if ((int)g_flush.size() <= p->device) g_flush.resize(p->device + 1, {nullptr, 0});
        auto& slot = g_flush[p->device];
        if (slot.second < bytes) {
            if (slot.first) cudaFree(slot.first);
            slot = {nullptr, 0};
            void* ptr = nullptr;
            cudaError_t e = cudaMalloc(&ptr, bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(SB_ERR_NOMEM, "L2 flush buffer allocation failed: %s",
                            cudaGetErrorString(e));
            }
            slot = {ptr, bytes};
        }
        buf = slot.first;
    }
    static unsigned salt = 1;
    const size_t n = bytes / sizeof(uint4);
    flush_kernel<<<p->sm_count * 4, 512, 0, (cudaStream_t)stream>>>((uint4*)buf, n, salt++);
    SB_CUDA(cudaGetLastError());
    return SB_OK;
}

int sb_debug_soft_f64(int op, const void* a, const void* b, void* out, int64_t n, void* stream) {
    clear_error();
    SB_CHECK(op >= 0 && op <= 3, SB_ERR_INVALID, "op must be 0 (add), 1 (sub), 2 (mul) or 3 (reciprocal)");
    SB_CHECK(n >= 0 && a && out && (op == 3 || b), SB_ERR_INVALID, "bad arguments");
    if (n == 0) return SB_OK;
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    const int blocks = (int)std::min<int64_t>(ceil_div(n, (int64_t)256), (int64_t)p->sm_count * 16);
    soft_f64_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(op, (const double*)a, (const double*)b, (double*)out, n);
    SB_CUDA(cudaGetLastError());
    return SB_OK;
}

int sb_probe_arith_rate(int kind, double* ops_per_s) {
    SB_CHECK(kind >= 0 && kind <= 20 && ops_per_s, SB_ERR_INVALID, "bad probe arguments");
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    double* out = nullptr;
    SB_CUDA(cudaMalloc(&out, sizeof(double)));
    const int blocks = p->sm_count * 8, threads = 256,
              iters = (kind == 2 || (kind >= 5 && kind <= 9)) ? 8192
                                                                 : (kind >= 12 && kind <= 15 ? 2048 : 512);
    auto launch = [&]() {
        if (kind == 0) arith_probe_kernel<0><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 1) arith_probe_kernel<1><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 2) arith_probe_kernel<2><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 3) arith_probe_kernel<3><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 4) arith_probe_kernel<4><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 5) arith_probe_kernel<5><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 6) arith_probe_kernel<6><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 7) arith_probe_kernel<7><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 8) arith_probe_kernel<8><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 9) arith_probe_kernel<9><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 10) arith_probe_kernel<10><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 11) arith_probe_kernel<11><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 12) arith_probe_kernel<12><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 13) arith_probe_kernel<13><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 14) arith_probe_kernel<14><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 15) arith_probe_kernel<15><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 16) arith_probe_kernel<16><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 17) arith_probe_kernel<17><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 18) arith_probe_kernel<18><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 19) arith_probe_kernel<19><<<blocks, threads>>>(out, iters, 0.5);
        if (kind == 20) arith_probe_kernel<20><<<blocks, threads>>>(out, iters, 0.5);
        return SB_OK;
    };
    double t = 0.0;
    rc = timed(nullptr, nullptr, launch);  // warm-up
    if (rc == SB_OK) rc = timed(nullptr, &t, launch);
    cudaFree(out);
    if (rc) return rc;
    *ops_per_s = (double)blocks * threads * iters * 8.0 * (kind == 5 ? 3.0 : 1.0) / t;
    return SB_OK;
}

}  // extern "C"
