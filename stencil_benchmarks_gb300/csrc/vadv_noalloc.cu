// sb_vadv_noalloc: vertical advection for callers that cannot allocate
// device memory.
//
// The GLOBAL form of vertical advection keeps the forward-elimination factors
// (ccol, dcol) of every column in global memory.  sb_vadv takes that scratch
// from the caller; this entry point instead uses one fixed array compiled
// into the library, so a call performs no cudaMalloc/cudaFree and calls no
// allocating library routine.  It serves code that runs inside a host
// framework which owns every device allocation (fixed memory pools, or paths
// that must not trigger the device-wide synchronisation cudaMalloc and
// cudaFree can cause).
//
// Scratch: g_vadv_scratch, SB_VADV_NOALLOC_SCRATCH_BYTES (32 MiB) per device
// that loads the library, held until the process exits.  The kernel walks
// the columns with a grid-stride loop; each thread slot owns 2 * nk factors
// ([level][slot], coalesced across threads), so the number of slots is what
// fits in the array.  Every factor is written before it is read, so nothing
// has to start at zero and nothing is cleared.  All calls share the array:
// calls that overlap on the GPU (different streams, or different host
// threads) race on it and must be serialised by the caller.
//
// The host side needs the array's device address: the array's name in host
// code is only a host-side stand-in, which a kernel must never receive.  The
// first call on each device looks the address up with cudaGetSymbolAddress
// (with that device current) and caches it; make that first call before any
// stream capture on that device.
//
// Arithmetic: the same operations in the same order as sb_vadv
// (stencil_benchmarks/benchmarks_collection/stencils/base.py:410-473), so the
// results are bit-identical to sb_vadv's.
#include <mutex>
#include <vector>

#include "common.cuh"

namespace sb {
namespace {

static __device__ __align__(256) unsigned char g_vadv_scratch[SB_VADV_NOALLOC_SCRATCH_BYTES];

std::mutex g_scratch_mutex;
std::vector<void*> g_scratch_addr;  // per device; nullptr until looked up

int scratch_address(void** out) {
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if ((int)g_scratch_addr.size() <= dev) g_scratch_addr.resize(dev + 1, nullptr);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_vadv_scratch);
        if (e != cudaSuccess || ptr == nullptr) {
            return fail(SB_ERR_CUDA, "cudaGetSymbolAddress of the vadv scratch array failed: %s",
                        cudaGetErrorString(e));
        }
        g_scratch_addr[dev] = ptr;
    }
    *out = g_scratch_addr[dev];
    return SB_OK;
}

constexpr int kNoallocBlock = 64;

template <class S, class C>
__global__ void __launch_bounds__(kNoallocBlock)
    vadv_noalloc_kernel(const S* __restrict__ stage, const S* __restrict__ pos, const S* __restrict__ tens,
                        const S* tensstage, const S* __restrict__ wcon, S* out, C* __restrict__ scratch,
                        int ni, int nj, int nk, int64_t si, int64_t sj, int64_t sk, int64_t wsh, int nslots) {
    using A = Ar<C>;
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= nslots) return;
    C* fc = scratch + slot;                        // ccol of level k at fc[k * nslots]
    C* fd = scratch + (size_t)nk * nslots + slot;  // dcol of level k at fd[k * nslots]
    const C dtr = (C)(3.0 / 20.0);
    const int64_t ncols = (int64_t)ni * nj;
    for (int64_t c = slot; c < ncols; c += nslots) {
        const int i = (int)(c % ni);
        const int j = (int)(c / ni);
        const int64_t col = (int64_t)i * si + (int64_t)j * sj;

        // forward sweep, k = 0
        int64_t o = col;
        C gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + o + sk + wsh), ld<C, S>(wcon + o + sk)));
        C cs = A::template scale2<-1>(gcv);
        C sprev = ld<C, S>(stage + o);
        C scur = ld<C, S>(stage + o + sk);
        C dup = A::sub(scur, sprev);
        C bcol = A::sub(dtr, cs);
        C corr = A::mul(-cs, dup);
        C dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
        C cp = A::div(cs, bcol);
        C dp = A::div(dv, bcol);
        fc[0] = cp;
        fd[0] = dp;
        // forward sweep, 0 < k < nk-1
        for (int k = 1; k < nk - 1; ++k) {
            o = col + (int64_t)k * sk;
            const C as_ = A::template scale2<-1>(-gcv);
            gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + o + sk + wsh), ld<C, S>(wcon + o + sk)));
            cs = A::template scale2<-1>(gcv);
            const C snext = ld<C, S>(stage + o + sk);
            const C ddown = A::neg_diff(dup, scur, sprev);
            dup = A::sub(snext, scur);
            bcol = A::sub(A::sub(dtr, as_), cs);
            corr = A::sub(A::mul(-as_, ddown), A::mul(cs, dup));
            dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
            const C divided = A::rcp(A::sub(bcol, A::mul(cp, as_)));
            cp = A::mul(cs, divided);
            dp = A::mul(A::sub(dv, A::mul(dp, as_)), divided);
            fc[(size_t)k * nslots] = cp;
            fd[(size_t)k * nslots] = dp;
            sprev = scur;
            scur = snext;
        }
        // forward sweep, k = nk-1
        {
            o = col + (int64_t)(nk - 1) * sk;
            const C as_ = A::template scale2<-1>(-gcv);
            bcol = A::sub(dtr, as_);
            const C ddown = A::neg_diff(dup, scur, sprev);
            corr = A::mul(-as_, ddown);
            dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
            dp = A::div(A::sub(dv, A::mul(dp, as_)), A::sub(bcol, A::mul(cp, as_)));
        }
        // backward sweep
        C data = dp;
        o = col + (int64_t)(nk - 1) * sk;
        st<S, C>(out + o, A::mul(dtr, A::sub(data, ld<C, S>(pos + o))));
        for (int k = nk - 2; k >= 0; --k) {
            o = col + (int64_t)k * sk;
            data = A::sub(fd[(size_t)k * nslots], A::mul(fc[(size_t)k * nslots], data));
            st<S, C>(out + o, A::mul(dtr, A::sub(data, ld<C, S>(pos + o))));
        }
    }
}

template <class S, class C>
int launch_noalloc(const void* stage, const void* pos, const void* tens, const void* tensstage, const void* wcon,
                   void* out, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
                   int64_t wsh, cudaStream_t stream) {
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    const size_t per_slot = 2 * sizeof(C) * (size_t)nk;
    const int64_t fit = (int64_t)(SB_VADV_NOALLOC_SCRATCH_BYTES / per_slot) / kNoallocBlock * kNoallocBlock;
    SB_CHECK(fit >= kNoallocBlock, SB_ERR_BUDGET,
             "sb_vadv_noalloc: nk = %lld needs %zu bytes of scratch per block of %d columns, more than the "
             "%u-byte static scratch array holds",
             (long long)nk, per_slot * kNoallocBlock, kNoallocBlock, (unsigned)SB_VADV_NOALLOC_SCRATCH_BYTES);
    const int64_t ncols = ni * nj;
    const int64_t want = ceil_div(ncols, kNoallocBlock) * kNoallocBlock;
    const int64_t resident = (int64_t)p->sm_count * 2048;
    int64_t nslots = fit;
    if (nslots > want) nslots = want;
    if (nslots > resident) nslots = resident / kNoallocBlock * kNoallocBlock;
    void* scratch = nullptr;
    rc = scratch_address(&scratch);
    if (rc) return rc;
    vadv_noalloc_kernel<S, C><<<(unsigned)(nslots / kNoallocBlock), kNoallocBlock, 0, stream>>>(
        (const S*)stage, (const S*)pos, (const S*)tens, (const S*)tensstage, (const S*)wcon, (S*)out, (C*)scratch,
        (int)ni, (int)nj, (int)nk, si, sj, sk, wsh, (int)nslots);
    return SB_OK;
}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" int sb_vadv_noalloc(int storage, int compute, const void* stage, const void* pos, const void* tens,
                               const void* tensstage, const void* wcon, void* out, int64_t ni, int64_t nj,
                               int64_t nk, int64_t si, int64_t sj, int64_t sk, int wshift_i, int wshift_j,
                               void* stream, double* time_s) {
    clear_error();
    int rc = check_domain(ni, nj, nk, si, sj, sk);
    if (rc) return rc;
    SB_CHECK(stage && pos && tens && tensstage && wcon && out, SB_ERR_INVALID, "NULL field pointer");
    SB_CHECK(wshift_i >= 0 && wshift_i <= 1 && wshift_j >= 0 && wshift_j <= 1 && wshift_i + wshift_j <= 1,
             SB_ERR_INVALID, "wcon shift must be (1,0), (0,1) or (0,0)");
    if (ni == 0 || nj == 0 || nk == 0) {
        if (time_s) *time_s = 0.0;
        return SB_OK;
    }
    SB_CHECK(nk >= 2, SB_ERR_INVALID, "vertical advection needs at least 2 levels (nk = %lld)", (long long)nk);
    const int64_t wsh = (int64_t)wshift_i * si + (int64_t)wshift_j * sj;
    cudaStream_t s = (cudaStream_t)stream;
    return timed(s, time_s, [&]() {
        if (storage == SB_F64 && compute == SB_F64)
            return launch_noalloc<double, double>(stage, pos, tens, tensstage, wcon, out, ni, nj, nk, si, sj, sk, wsh, s);
        if (storage == SB_F32 && compute == SB_F32)
            return launch_noalloc<float, float>(stage, pos, tens, tensstage, wcon, out, ni, nj, nk, si, sj, sk, wsh, s);
        if (storage == SB_F32 && compute == SB_F64)
            return launch_noalloc<float, double>(stage, pos, tens, tensstage, wcon, out, ni, nj, nk, si, sj, sk, wsh, s);
        if (storage == SB_BF16 && compute == SB_F32)
            return launch_noalloc<bf16, float>(stage, pos, tens, tensstage, wcon, out, ni, nj, nk, si, sj, sk, wsh, s);
        return fail(SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
    });
}
