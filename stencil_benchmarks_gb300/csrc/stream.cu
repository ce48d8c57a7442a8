// STREAM copy / scale / add / triad (+ init) on sm_103a.
//
// Semantics follow the reference's GPU STREAM
// (stencil_benchmarks/benchmarks_collection/stream/cuda_hip.j2:132-173):
//   init  a = 1, b = 2, c = 0      copy  c = a      scale  b = s * c
//   add   c = a + b                triad a = b + s * c   (one fused multiply-add,
//                                  as nvcc contracts the reference's kernel)
// Design: 16-byte vector accesses (double2 / float4), several independent
// vectors in flight per thread, a grid of a few CTAs per SM that strides over
// the arrays, optional evict-first stores for data that is not re-read.
#include "common.cuh"

namespace sb {
namespace {

template <class T>
struct Vec16;
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int width = 2;
};
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int width = 4;
};

template <int OP, class T>
__device__ __forceinline__ T elem(T x, T y, T s) {
    if (OP == SB_STREAM_COPY) return x;
    if (OP == SB_STREAM_SCALE) return s * x;
    if (OP == SB_STREAM_ADD) return x + y;
    return fma(s, y, x);  // triad: x + s*y
}

template <int OP>
__device__ __forceinline__ double2 vop(double2 x, double2 y, double s) {
    return make_double2(elem<OP>(x.x, y.x, s), elem<OP>(x.y, y.y, s));
}
template <int OP>
__device__ __forceinline__ float4 vop(float4 x, float4 y, float s) {
    return make_float4(elem<OP>(x.x, y.x, s), elem<OP>(x.y, y.y, s), elem<OP>(x.z, y.z, s),
                       elem<OP>(x.w, y.w, s));
}

template <class V>
__device__ __forceinline__ void vstore(V* p, V v, bool streaming) {
    if (streaming)
        __stcs(p, v);
    else
        *p = v;
}

// dst = OP(x, y) over nvec 16-byte vectors; `UNROLL` vectors per thread per
// trip keep UNROLL * 16 (or 32) bytes of loads in flight per thread.
template <int OP, class T, int UNROLL>
__global__ void __launch_bounds__(512) stream_vec_kernel(typename Vec16<T>::type* __restrict__ dst,
                                                         const typename Vec16<T>::type* __restrict__ x,
                                                         const typename Vec16<T>::type* __restrict__ y,
                                                         T s, int64_t nvec, bool streaming) {
    using V = typename Vec16<T>::type;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (UNROLL - 1) * stride < nvec; i += UNROLL * stride) {
        V vx[UNROLL], vy[UNROLL];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            vx[u] = __ldg(x + i + u * stride);
            vy[u] = (OP == SB_STREAM_ADD || OP == SB_STREAM_TRIAD) ? __ldg(y + i + u * stride) : vx[u];
        }
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) vstore(dst + i + u * stride, vop<OP>(vx[u], vy[u], s), streaming);
    }
    for (; i < nvec; i += stride) {
        const V vx1 = __ldg(x + i);
        const V vy1 = (OP == SB_STREAM_ADD || OP == SB_STREAM_TRIAD) ? __ldg(y + i) : vx1;
        vstore(dst + i, vop<OP>(vx1, vy1, s), streaming);
    }
}

// dst = OP(x, y) with one block per `blockDim.x * UNROLL` vectors (no stride
// loop): thread t of block b handles vectors b * blockDim.x * UNROLL + t +
// u * blockDim.x, u < UNROLL, so each block streams one contiguous chunk and
// the hardware block scheduler balances the SMs.
template <int OP, class T, int UNROLL>
__global__ void __launch_bounds__(1024) stream_chunk_kernel(typename Vec16<T>::type* __restrict__ dst,
                                                            const typename Vec16<T>::type* __restrict__ x,
                                                            const typename Vec16<T>::type* __restrict__ y,
                                                            T s, int64_t nvec, bool streaming) {
    using V = typename Vec16<T>::type;
    const int64_t base = (int64_t)blockIdx.x * blockDim.x * UNROLL + threadIdx.x;
    V vx[UNROLL], vy[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
        const int64_t i = base + (int64_t)u * blockDim.x;
        if (i < nvec) {
            vx[u] = __ldg(x + i);
            vy[u] = (OP == SB_STREAM_ADD || OP == SB_STREAM_TRIAD) ? __ldg(y + i) : vx[u];
        }
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
        const int64_t i = base + (int64_t)u * blockDim.x;
        if (i < nvec) vstore(dst + i, vop<OP>(vx[u], vy[u], s), streaming);
    }
}

// scalar kernel for the tail and for pointers that are not 16-byte aligned
template <int OP, class T>
__global__ void stream_scalar_kernel(T* __restrict__ dst, const T* __restrict__ x,
                                     const T* __restrict__ y, T s, int64_t begin, int64_t n) {
    for (int64_t i = begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        T yv = (OP == SB_STREAM_ADD || OP == SB_STREAM_TRIAD) ? y[i] : T(0);
        dst[i] = elem<OP>(x[i], yv, s);
    }
}

template <class T>
__global__ void stream_init_kernel(T* __restrict__ a, T* __restrict__ b, T* __restrict__ c, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        a[i] = T(1);
        b[i] = T(2);
        c[i] = T(0);
    }
}

// grid shape when the tune gives none, and the chunk shape's defaults
constexpr int kStreamDefaultGrid = SB_STREAM_GRID_CHUNK;
constexpr int kStreamChunkThreads = 1024;
constexpr int kStreamChunkUnroll = 2;

template <int OP, class T>
int launch_op(T* dst, const T* x, const T* y, T s, int64_t n, const sb_tune* tune,
              cudaStream_t stream, const DeviceProps* p) {
    using V = typename Vec16<T>::type;
    constexpr int W = Vec16<T>::width;
    const bool streaming = tune && (tune->flags & 1);
    const int grid_mode = (tune && tune->variant > 0) ? tune->variant : kStreamDefaultGrid;
    SB_CHECK(grid_mode == SB_STREAM_GRID_STRIDE || grid_mode == SB_STREAM_GRID_CHUNK, SB_ERR_INVALID,
             "STREAM grid mode must be %d (stride) or %d (chunks)", SB_STREAM_GRID_STRIDE, SB_STREAM_GRID_CHUNK);
    const bool chunks = grid_mode == SB_STREAM_GRID_CHUNK;
    const int threads = (tune && tune->block_x > 0) ? tune->block_x : (chunks ? kStreamChunkThreads : 512);
    const int unroll = (tune && tune->unroll > 0) ? tune->unroll : (chunks ? kStreamChunkUnroll : 4);
    if (threads > (chunks ? 1024 : 512) || threads % 32)
        return fail(SB_ERR_INVALID, "STREAM block size must be a multiple of 32 <= %d", chunks ? 1024 : 512);
    const bool aligned = ((uintptr_t)dst % 16 == 0) && ((uintptr_t)x % 16 == 0) &&
                         (y == nullptr || (uintptr_t)y % 16 == 0);
    int64_t done = 0;
    if (aligned && chunks) {
        const int64_t nvec = n / W;
        if (nvec > 0) {
            const int64_t blocks = ceil_div(nvec, (int64_t)threads * unroll);
            SB_CHECK(blocks < (1LL << 31), SB_ERR_INVALID, "STREAM array too large for one chunk per block");
            switch (unroll) {
                case 1:
                    stream_chunk_kernel<OP, T, 1><<<(unsigned)blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                case 2:
                    stream_chunk_kernel<OP, T, 2><<<(unsigned)blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                case 4:
                    stream_chunk_kernel<OP, T, 4><<<(unsigned)blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                case 8:
                    stream_chunk_kernel<OP, T, 8><<<(unsigned)blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                default:
                    return fail(SB_ERR_INVALID, "STREAM unroll must be 1, 2, 4 or 8 (got %d)", unroll);
            }
            done = nvec * W;
        }
    } else if (aligned) {
        const int64_t nvec = n / W;
        if (nvec > 0) {
            const int64_t want = ceil_div(nvec, (int64_t)threads * unroll);
            const int64_t cap = (int64_t)p->sm_count * (2048 / threads) * 2;
            const int blocks = (int)(want < cap ? want : cap);
            switch (unroll) {
                case 1:
                    stream_vec_kernel<OP, T, 1><<<blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                case 2:
                    stream_vec_kernel<OP, T, 2><<<blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                case 4:
                    stream_vec_kernel<OP, T, 4><<<blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                case 8:
                    stream_vec_kernel<OP, T, 8><<<blocks, threads, 0, stream>>>((V*)dst, (const V*)x, (const V*)y, s, nvec, streaming);
                    break;
                default:
                    return fail(SB_ERR_INVALID, "STREAM unroll must be 1, 2, 4 or 8 (got %d)", unroll);
            }
            done = nvec * W;
        }
    }
    if (done < n) {
        const int64_t rest = n - done;
        const int64_t want = ceil_div(rest, 256);
        const int blocks = (int)(want < (int64_t)p->sm_count * 8 ? want : (int64_t)p->sm_count * 8);
        stream_scalar_kernel<OP, T><<<blocks, 256, 0, stream>>>(dst, x, y, s, done, n);
    }
    return SB_OK;
}

template <class T>
int dispatch(int op, T* a, T* b, T* c, T s, int64_t n, const sb_tune* tune, cudaStream_t stream,
             const DeviceProps* p) {
    switch (op) {
        case SB_STREAM_INIT: {
            const int64_t want = ceil_div(n, 512);
            const int blocks = (int)(want < (int64_t)p->sm_count * 8 ? want : (int64_t)p->sm_count * 8);
            stream_init_kernel<T><<<blocks, 512, 0, stream>>>(a, b, c, n);
            return SB_OK;
        }
        case SB_STREAM_COPY: return launch_op<SB_STREAM_COPY, T>(c, a, nullptr, s, n, tune, stream, p);
        case SB_STREAM_SCALE: return launch_op<SB_STREAM_SCALE, T>(b, c, nullptr, s, n, tune, stream, p);
        case SB_STREAM_ADD: return launch_op<SB_STREAM_ADD, T>(c, a, b, s, n, tune, stream, p);
        case SB_STREAM_TRIAD: return launch_op<SB_STREAM_TRIAD, T>(a, b, c, s, n, tune, stream, p);
    }
    return fail(SB_ERR_INVALID, "unknown STREAM op %d", op);
}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" int sb_stream_op(int op, int dtype, void* a, void* b, void* c, double scalar, int64_t n,
                            const sb_tune* tune, void* stream, double* time_s) {
    clear_error();
    SB_CHECK(n >= 0, SB_ERR_INVALID, "negative array size");
    SB_CHECK(dtype == SB_F64 || dtype == SB_F32, SB_ERR_UNSUPPORTED, "STREAM supports f64 and f32 only");
    SB_CHECK(op >= SB_STREAM_INIT && op <= SB_STREAM_TRIAD, SB_ERR_INVALID, "unknown STREAM op %d", op);
    const bool need_a = op != SB_STREAM_SCALE;
    const bool need_b = op != SB_STREAM_COPY;
    SB_CHECK((!need_a || a) && (!need_b || b) && c, SB_ERR_INVALID, "NULL array pointer");
    if (n == 0) {
        if (time_s) *time_s = 0.0;
        return SB_OK;
    }
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    return timed((cudaStream_t)stream, time_s, [&]() {
        if (dtype == SB_F64)
            return dispatch<double>(op, (double*)a, (double*)b, (double*)c, scalar, n, tune, (cudaStream_t)stream, p);
        return dispatch<float>(op, (float*)a, (float*)b, (float*)c, (float)scalar, n, tune, (cudaStream_t)stream, p);
    });
}
