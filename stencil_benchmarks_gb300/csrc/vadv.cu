// Vertical advection (vadv): per-column implicit tridiagonal (Thomas) solve.
//
// Oracle: stencil_benchmarks/benchmarks_collection/stencils/base.py:410-473
// (forward_sweep / backward_sweep with dtr_stage = 3/20, beta_v = 0, so
// bet_m = bet_p = 0.5).  The arithmetic below performs the same operations
// in the same order with one IEEE rounding each (1.0/x is the correctly
// rounded reciprocal, the two true divisions at k = 0 and k = nk-1 are IEEE
// divisions), so fp64 results are bit-identical to the reference.
//
// Exact rewrites used to save fp64 pipe slots (all are identities in IEEE
// arithmetic, not approximations):
//   gav(k) = -gcv(k-1)                 both are +-0.25 * (wcon_shift[k] + wcon[k])
//   as_ = acol, cs = ccol_raw          bet_m == bet_p == 0.5
//   x * 0.5, x * 0.25                  exponent decrements (Ar::scale2)
//   stage[k-1] - stage[k]              negation of the previous stage[k] - stage[k-1]
//                                      (recomputed when it is zero, to keep the sign of 0)
//
// The result goes to `out`, which is either tensstage itself (the reference's
// in-place update; each thread reads its own column's tensstage in the
// forward sweep before writing it in the backward sweep, through the
// coherent load path) or a separate field.
//
// One thread owns one (i, j) column; threads run along i so every k-level
// access of a warp is one contiguous row segment.  The forward sweep keeps
// the stage window, gcv and the previous (ccol, dcol) in registers and
// spills the per-level (ccol, dcol) pairs to
//   SMEM   : shared memory, [level][thread] (bank-conflict free), or
//   GLOBAL : the caller's ccol/dcol fields (the reference's arguments of the
//            same names), for columns too tall for shared memory.
// The backward sweep reads them back in reverse order.
#include "common.cuh"

namespace sb {
namespace {

template <class S, class C, bool GLOBAL>
__global__ void __launch_bounds__(256)
    vadv_kernel(const S* __restrict__ stage, const S* __restrict__ pos, const S* __restrict__ tens,
                const S* tensstage, const S* __restrict__ wcon, S* out, C* __restrict__ gccol,
                C* __restrict__ gdcol, int ni, int nj, int nk, int64_t si, int64_t sj, int64_t sk,
                int64_t wsh) {
    using A = Ar<C>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nthr = blockDim.x * blockDim.y;
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    C* sc = reinterpret_cast<C*>(smem_raw);
    C* sd = sc + (size_t)nk * nthr;

    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= ni || j >= nj) return;  // no block-wide barrier below

    const C dtr = (C)(3.0 / 20.0);
    const int64_t col = (int64_t)i * si + (int64_t)j * sj;

    auto put = [&](int k, C cv, C dv) {
        if (GLOBAL) {
            gccol[col + (int64_t)k * sk] = cv;
            gdcol[col + (int64_t)k * sk] = dv;
        } else {
            sc[(size_t)k * nthr + t] = cv;
            sd[(size_t)k * nthr + t] = dv;
        }
    };
    auto get_c = [&](int k) -> C { return GLOBAL ? gccol[col + (int64_t)k * sk] : sc[(size_t)k * nthr + t]; };
    auto get_d = [&](int k) -> C { return GLOBAL ? gdcol[col + (int64_t)k * sk] : sd[(size_t)k * nthr + t]; };

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
    put(0, cp, dp);

    // ---- forward sweep, 0 < k < nk-1
#pragma unroll 2
    for (int k = 1; k < nk - 1; ++k) {
        o = col + (int64_t)k * sk;
        const C as_ = A::template scale2<-1>(-gcv);  // gav * bet_m == acol, gav = -gcv(k-1)
        gcv = A::template scale2<-2>(A::add(ld<C, S>(wcon + o + sk + wsh), ld<C, S>(wcon + o + sk)));
        cs = A::template scale2<-1>(gcv);
        const C snext = ld<C, S>(stage + o + sk);
        const C ddown = A::neg_diff(dup, scur, sprev);  // stage[k-1] - stage[k]
        dup = A::sub(snext, scur);                     // stage[k+1] - stage[k]
        bcol = A::sub(A::sub(dtr, as_), cs);
        corr = A::sub(A::mul(-as_, ddown), A::mul(cs, dup));
        dv = A::add(A::add(A::add(A::mul(dtr, ld<C, S>(pos + o)), ld<C, S>(tens + o)), ldc<C, S>(tensstage + o)), corr);
        const C divided = A::rcp(A::sub(bcol, A::mul(cp, as_)));
        cp = A::mul(cs, divided);
        dp = A::mul(A::sub(dv, A::mul(dp, as_)), divided);
        put(k, cp, dp);
        sprev = scur;
        scur = snext;
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
#pragma unroll 2
    for (int k = nk - 2; k >= 0; --k) {
        o = col + (int64_t)k * sk;
        data = A::sub(get_d(k), A::mul(get_c(k), data));
        st<S, C>(out + o, A::mul(dtr, A::sub(data, ld<C, S>(pos + o))));
    }
}

template <class S, class C>
int launch_typed(const void* stage, const void* pos, const void* tens, const void* tensstage,
                 const void* wcon, void* out, void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk,
                 int64_t si, int64_t sj, int64_t sk, int64_t wsh, const sb_tune* tune,
                 cudaStream_t stream) {
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    int variant = tune ? tune->variant : SB_VARIANT_AUTO;
    int bx = (tune && tune->block_x > 0) ? tune->block_x : 32;
    int by = (tune && tune->block_y > 0) ? tune->block_y : 1;
    SB_CHECK(bx * by <= 256 && bx >= 1 && by >= 1, SB_ERR_INVALID, "vadv block (%d, %d) exceeds 256 threads", bx, by);
    const size_t smem = 2 * sizeof(C) * (size_t)nk * (size_t)(bx * by);
    const bool can_global = ccol && dcol && sizeof(S) == sizeof(C);
    if (variant == SB_VARIANT_AUTO) variant = ((int64_t)smem <= p->smem_optin) ? SB_VADV_SMEM : SB_VADV_GLOBAL;
    SB_CHECK(variant == SB_VADV_SMEM || variant == SB_VADV_GLOBAL, SB_ERR_UNSUPPORTED, "vadv variant %d is not available", variant);
    const int64_t gx = ceil_div(ni, bx), gy = ceil_div(nj, by);
    SB_CHECK(gy <= p->max_grid_y, SB_ERR_INVALID, "vadv grid too large");
    const dim3 grid((unsigned)gx, (unsigned)gy), block(bx, by);
    if (variant == SB_VADV_SMEM) {
        SB_CHECK((int64_t)smem <= p->smem_optin, SB_ERR_INVALID,
                 "vadv: %lld levels x %d columns need %zu bytes of shared memory (limit %d); "
                 "use fewer threads per block or the GLOBAL variant with ccol/dcol scratch",
                 (long long)nk, bx * by, smem, p->smem_optin);
        auto kernel = vadv_kernel<S, C, false>;
        if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<grid, block, smem, stream>>>((const S*)stage, (const S*)pos, (const S*)tens, (const S*)tensstage,
                                              (const S*)wcon, (S*)out, nullptr, nullptr, (int)ni, (int)nj, (int)nk,
                                              si, sj, sk, wsh);
    } else {
        SB_CHECK(can_global, SB_ERR_INVALID,
                 "vadv GLOBAL variant needs ccol/dcol scratch fields of the compute type");
        vadv_kernel<S, C, true><<<grid, block, 0, stream>>>((const S*)stage, (const S*)pos, (const S*)tens,
                                                          (const S*)tensstage, (const S*)wcon, (S*)out,
                                                          (C*)ccol, (C*)dcol,
                                                          (int)ni, (int)nj, (int)nk, si, sj, sk, wsh);
    }
    return SB_OK;
}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" int sb_vadv(int storage, int compute, const void* stage, const void* pos, const void* tens,
                       const void* tensstage, const void* wcon, void* out, void* ccol, void* dcol,
                       int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
                       int wshift_i, int wshift_j, const sb_tune* tune, void* stream, double* time_s) {
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
            return launch_typed<double, double>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        if (storage == SB_F32 && compute == SB_F32)
            return launch_typed<float, float>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        if (storage == SB_F32 && compute == SB_F64)
            return launch_typed<float, double>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        if (storage == SB_BF16 && compute == SB_F32)
            return launch_typed<bf16, float>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        return fail(SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
    });
}
