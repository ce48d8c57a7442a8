// Device-side support for serving: seeded field generation and event polling.
//
// sb_fill_batch fills many device fields in one launch with uniform values
// from a counter-based generator, so request fields are created where they
// are used (no host->device copy) and are reproducible on the host: element e
// of a field with seed s gets
//     u = (splitmix64(s + (e + 1) * golden) >> 11) * 2^-53      (in [0, 1))
//     v = lo + (hi - lo) * u                                     (in double)
// rounded once to float32 storage, or to float32 and then to bfloat16.
// splitmix64 is the published 64-bit finaliser of Steele, Lea and Flood's
// SplitMix generator (increment 0x9E3779B97F4A7C15, shifts 30/27/31).
#include <vector>

#include "common.cuh"

namespace sb {
namespace {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__global__ void fill_batch_kernel(const sb_fill_desc* __restrict__ descs, int n) {
    const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int d = 0; d < n; ++d) {
        const sb_fill_desc& f = descs[d];
        const double span = f.hi - f.lo;
        for (int64_t e = gtid; e < f.count; e += gsize) {
            const unsigned long long z = splitmix64(f.seed + (unsigned long long)(e + 1) * 0x9E3779B97F4A7C15ULL);
            const double u = (double)(z >> 11) * 0x1.0p-53;
            const double v = f.lo + span * u;
            if (f.storage == SB_F64) {
                ((double*)f.ptr)[e] = v;
            } else if (f.storage == SB_F32) {
                ((float*)f.ptr)[e] = __double2float_rn(v);
            } else {
                ((bf16*)f.ptr)[e] = __float2bfloat16_rn(__double2float_rn(v));
            }
        }
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
        SB_CHECK(descs[d].ptr && descs[d].count >= 0, SB_ERR_INVALID, "fill descriptor %d is invalid", d);
        SB_CHECK(descs[d].storage >= SB_F64 && descs[d].storage <= SB_BF16, SB_ERR_INVALID,
                 "fill descriptor %d: unknown storage %d", d, descs[d].storage);
        total += descs[d].count;
    }
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SB_CUDA(cudaMemcpyAsync(desc_scratch, descs, sizeof(sb_fill_desc) * n, cudaMemcpyHostToDevice, s));
    const int64_t want = ceil_div(total, 256);
    const int blocks = (int)std::min<int64_t>(std::max<int64_t>(want, 1), (int64_t)p->sm_count * 8);
    fill_batch_kernel<<<blocks, 256, 0, s>>>((const sb_fill_desc*)desc_scratch, n);
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
