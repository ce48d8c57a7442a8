// Basic stencils: copy, Laplacian along chosen axes, one-sided and symmetric
// averages.  Oracles: stencil_benchmarks/benchmarks_collection/stencils/base.py
// 180-254; the arithmetic below evaluates exactly the same operations in the
// same order, one rounding each.
//
// Layout: threads run along i (the unit-stride axis of the default layout)
// so warps read and write contiguous rows; each thread handles PK points
// along k with all loads issued before the stores, so a warp keeps PK
// independent 128/256-byte requests in flight.
#include "common.cuh"

namespace sb {
namespace {

constexpr int kBasicPK = 4;

enum BasicOp { OP_COPY = 0, OP_LAP = 1, OP_AVG1 = 2, OP_AVG2 = 3 };

// 0 + t evaluated exactly (only changes -0 into +0)
template <class C>
__device__ __forceinline__ C plus_zero(C t);
template <>
__device__ __forceinline__ double plus_zero<double>(double t) {
    return ((__double_as_longlong(t) << 1) == 0) ? 0.0 : t;
}
template <>
__device__ __forceinline__ float plus_zero<float>(float t) {
    return __fadd_rn(0.0f, t);
}

template <int OP, class S, class C>
__device__ __forceinline__ C basic_point(const S* __restrict__ p, int64_t si, int64_t sj,
                                         int64_t sk, int mask, int64_t ds) {
    using A = Ar<C>;
    if (OP == OP_COPY) return ld<C, S>(p);
    if (OP == OP_AVG1) return A::template scale2<-1>(A::add(ld<C, S>(p + ds), ld<C, S>(p)));
    if (OP == OP_AVG2) return A::template scale2<-1>(A::add(ld<C, S>(p + ds), ld<C, S>(p - ds)));
    // Laplacian: result = 0; result += (2*inp - inp[+1]) - inp[-1] per axis x, y, z
    const C two_x = A::template scale2<1>(ld<C, S>(p));
    C acc = C(0);
    bool first = true;
    const int64_t strides[3] = {si, sj, sk};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        if (mask & (1 << ax)) {
            const C t = A::sub(A::sub(two_x, ld<C, S>(p + strides[ax])), ld<C, S>(p - strides[ax]));
            acc = first ? plus_zero<C>(t) : A::add(acc, t);
            first = false;
        }
    }
    return acc;
}

template <int OP, class S, class C>
__global__ void __launch_bounds__(256) basic_kernel(const S* __restrict__ inp, S* __restrict__ out,
                                                    int ni, int nj, int nk, int64_t si, int64_t sj,
                                                    int64_t sk, int mask, int64_t ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k0 = blockIdx.z * kBasicPK;
    if (i >= ni || j >= nj) return;
    const int64_t base = (int64_t)i * si + (int64_t)j * sj;
    C r[kBasicPK];
#pragma unroll
    for (int q = 0; q < kBasicPK; ++q) {
        const int k = k0 + q;
        if (k < nk) r[q] = basic_point<OP, S, C>(inp + base + (int64_t)k * sk, si, sj, sk, mask, ds);
    }
#pragma unroll
    for (int q = 0; q < kBasicPK; ++q) {
        const int k = k0 + q;
        if (k < nk) st<S, C>(out + base + (int64_t)k * sk, r[q]);
    }
}

template <int OP, class S, class C>
int launch_basic(const void* inp, void* out, int64_t ni, int64_t nj, int64_t nk, int64_t si,
                 int64_t sj, int64_t sk, int mask, int64_t ds, const sb_tune* tune,
                 cudaStream_t stream) {
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    int bx = (tune && tune->block_x > 0) ? tune->block_x : 128;
    int by = (tune && tune->block_y > 0) ? tune->block_y : 2;
    SB_CHECK(bx * by <= 256 && bx % 32 == 0, SB_ERR_INVALID,
             "block (%d, %d): need a multiple of 32 along i and at most 256 threads", bx, by);
    const int64_t gx = ceil_div(ni, bx), gy = ceil_div(nj, by), gz = ceil_div(nk, kBasicPK);
    SB_CHECK(gy <= p->max_grid_y && gz <= p->max_grid_z, SB_ERR_INVALID,
             "domain too large for the launch grid (%lld, %lld, %lld)", (long long)gx,
             (long long)gy, (long long)gz);
    basic_kernel<OP, S, C><<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), dim3(bx, by), 0, stream>>>(
        (const S*)inp, (S*)out, (int)ni, (int)nj, (int)nk, si, sj, sk, mask, ds);
    return SB_OK;
}

template <int OP>
int dispatch_basic(int storage, int compute, const void* inp, void* out, int64_t ni, int64_t nj,
                   int64_t nk, int64_t si, int64_t sj, int64_t sk, int mask, int64_t ds,
                   const sb_tune* tune, cudaStream_t stream) {
    if (storage == SB_F64 && compute == SB_F64)
        return launch_basic<OP, double, double>(inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, stream);
    if (storage == SB_F32 && compute == SB_F32)
        return launch_basic<OP, float, float>(inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, stream);
    if (storage == SB_F32 && compute == SB_F64)
        return launch_basic<OP, float, double>(inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, stream);
    if (storage == SB_BF16 && compute == SB_F32)
        return launch_basic<OP, bf16, float>(inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, stream);
    return fail(SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
}

int basic_entry(int op, int storage, int compute, const void* inp, void* out, int64_t ni,
                int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, int mask, int64_t ds,
                const sb_tune* tune, void* stream, double* time_s) {
    clear_error();
    int rc = check_domain(ni, nj, nk, si, sj, sk);
    if (rc) return rc;
    SB_CHECK(inp && out, SB_ERR_INVALID, "NULL field pointer");
    if (ni == 0 || nj == 0 || nk == 0) {
        if (time_s) *time_s = 0.0;
        return SB_OK;
    }
    return timed((cudaStream_t)stream, time_s, [&]() {
        switch (op) {
            case OP_COPY:
                return dispatch_basic<OP_COPY>(storage, compute, inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, (cudaStream_t)stream);
            case OP_LAP:
                return dispatch_basic<OP_LAP>(storage, compute, inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, (cudaStream_t)stream);
            case OP_AVG1:
                return dispatch_basic<OP_AVG1>(storage, compute, inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, (cudaStream_t)stream);
            default:
                return dispatch_basic<OP_AVG2>(storage, compute, inp, out, ni, nj, nk, si, sj, sk, mask, ds, tune, (cudaStream_t)stream);
        }
    });
}

// Empty: the reference's launch-overhead probe (its generated kernel body is
// empty): the grid of the basic stencils over the domain, touching no memory.
__global__ void __launch_bounds__(256) empty_kernel() {}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" {

int sb_empty(int64_t ni, int64_t nj, int64_t nk, const sb_tune* tune, void* stream, double* time_s) {
    clear_error();
    SB_CHECK(ni >= 0 && nj >= 0 && nk >= 0, SB_ERR_INVALID, "negative domain size");
    if (ni == 0 || nj == 0 || nk == 0) {
        if (time_s) *time_s = 0.0;
        return SB_OK;
    }
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    const int bx = (tune && tune->block_x > 0) ? tune->block_x : 128;
    const int by = (tune && tune->block_y > 0) ? tune->block_y : 2;
    SB_CHECK(bx * by <= 256 && bx % 32 == 0, SB_ERR_INVALID,
             "block (%d, %d): need a multiple of 32 along i and at most 256 threads", bx, by);
    const int64_t gx = ceil_div(ni, bx), gy = ceil_div(nj, by), gz = ceil_div(nk, kBasicPK);
    SB_CHECK(gx < (1LL << 31) && gy <= p->max_grid_y && gz <= p->max_grid_z, SB_ERR_INVALID,
             "domain too large for the launch grid");
    return timed((cudaStream_t)stream, time_s, [&]() {
        empty_kernel<<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), dim3(bx, by), 0, (cudaStream_t)stream>>>();
        SB_CUDA(cudaGetLastError());
        return SB_OK;
    });
}

int sb_copy(int storage, const void* inp, void* out, int64_t ni, int64_t nj, int64_t nk, int64_t si,
            int64_t sj, int64_t sk, const sb_tune* tune, void* stream, double* time_s) {
    const int compute = storage == SB_F64 ? SB_F64 : SB_F32;
    return basic_entry(OP_COPY, storage, compute, inp, out, ni, nj, nk, si, sj, sk, 0, 0, tune, stream, time_s);
}

int sb_laplacian(int storage, int compute, const void* inp, void* out, int64_t ni, int64_t nj,
                 int64_t nk, int64_t si, int64_t sj, int64_t sk, int along_mask,
                 const sb_tune* tune, void* stream, double* time_s) {
    SB_CHECK(along_mask >= 0 && along_mask <= 7, SB_ERR_INVALID, "along_mask must be in [0, 7]");
    return basic_entry(OP_LAP, storage, compute, inp, out, ni, nj, nk, si, sj, sk, along_mask, 0, tune,
                       stream, time_s);
}

int sb_average(int storage, int compute, const void* inp, void* out, int64_t ni, int64_t nj,
               int64_t nk, int64_t si, int64_t sj, int64_t sk, int axis, int symmetric,
               const sb_tune* tune, void* stream, double* time_s) {
    SB_CHECK(axis >= 0 && axis <= 2, SB_ERR_INVALID, "axis must be 0, 1 or 2");
    const int64_t ds = axis == 0 ? si : axis == 1 ? sj : sk;
    return basic_entry(symmetric ? OP_AVG2 : OP_AVG1, storage, compute, inp, out, ni, nj, nk, si, sj,
                       sk, 0, ds, tune, stream, time_s);
}

}  // extern "C"
