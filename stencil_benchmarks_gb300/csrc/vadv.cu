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
#include <algorithm>
#include <initializer_list>
#include <type_traits>

#include "stencil_core.cuh"

namespace sb {
namespace {

template <class S, class C, bool GLOBAL, int D>
__global__ void __launch_bounds__(256)
    vadv_kernel(const S* __restrict__ stage, const S* __restrict__ pos, const S* __restrict__ tens,
                const S* tensstage, const S* __restrict__ wcon, S* out, C* __restrict__ gccol,
                C* __restrict__ gdcol, int ni, int nj, int nk, int64_t si, int64_t sj, int64_t sk,
                int64_t wsh) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nthr = blockDim.x * blockDim.y;
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= ni || j >= nj) return;  // no block-wide barrier below
    const int64_t col = (int64_t)i * si + (int64_t)j * sj;
    if (GLOBAL) {
        const GlobalFactors<C> fac{gccol + col, gdcol + col, sk};
        vadv_column<S, C, D>(stage, pos, tens, tensstage, wcon, out, col, nk, sk, wsh, fac);
    } else {
        C* sc = reinterpret_cast<C*>(smem_raw);
        const SmemFactors<C> fac{sc + t, sc + (size_t)nk * nthr + t, nthr};
        vadv_column<S, C, D>(stage, pos, tens, tensstage, wcon, out, col, nk, sk, wsh, fac);
    }
}

// Integer-pipe placements of float64 vadv's operation sites (bit K = site K
// of vadv_async_column: 0 the wcon sum, 1 the stage difference, 2-3 bcol,
// 4-6 the correction, 7-10 the right-hand side, 11-12 the pivot, 13 ccol,
// 14-16 dcol, 17-18 the back substitution, 19-20 the output, 21 the pivot's
// reciprocal).  sb_tune.flags
// bits 4-7 pick one for the SLAB form: 0 the default, 1 every site on the
// fp64 pipe, 2.. the mixes below; SLAB shapes other than 32 threads x depth 1
// and the SMEM-async form use the default.
constexpr uint32_t vadv_sites(std::initializer_list<int> ks) {
    uint32_t m = 0;
    for (int k : ks) m |= 1u << k;
    return m;
}
constexpr uint32_t kVadvMuls = kVadvProductSites;
static_assert(kVadvMuls == vadv_sites({4, 5, 7, 11, 13, 14, 16, 17, 20}), "the nine products");
constexpr uint32_t kVadvPlacements[] = {
    0u,
    0u,
    kVadvMuls,
    vadv_sites({7, 14, 17, 20}) | kVadvRcpSite,
    vadv_sites({5, 14, 17, 20}) | kVadvRcpSite,
    vadv_sites({5, 7, 17, 20}) | kVadvRcpSite,
    vadv_sites({5, 7, 14, 17}) | kVadvRcpSite,
    vadv_sites({5, 7, 14, 20}) | kVadvRcpSite,
    vadv_sites({14, 17, 20}) | kVadvRcpSite,
    kVadvDefaultIntSites,
    kVadvRcpSite,
    vadv_sites({4, 5, 7, 14, 17, 20}) | kVadvRcpSite,
    vadv_sites({4, 5, 7, 14, 17}) | kVadvRcpSite,
    vadv_sites({4, 5, 7, 17, 20}) | kVadvRcpSite,
    vadv_sites({4, 5, 7, 14, 16, 17, 20}) | kVadvRcpSite,
    vadv_sites({5, 7, 14, 17, 20}) | kVadvRcpSite,
};
static_assert(kVadvDefaultIntSites == (kVadvMuls | kVadvRcpSite), "the default split");
// Measured at 512x512x80 (32-thread SLAB blocks): every site on the fp64
// pipe 1171-1201 us whatever the blocks per SM or ring depth.  Depth 4, 24
// blocks per SM: the nine products on the integer pipe (preset 2) 980-989 us
// (1019 with 16 blocks per SM, 1189 with 8: the integer sequences need more
// warps in flight); the pivot's reciprocal alone (preset 10) 991 us; the
// reciprocal with five or six products 859-892 us, with all nine 940 us.
// Depth 2 (a smaller ring, fewer copies in flight, more blocks fit): preset 2
// 912 us, five products + reciprocal 817 us, all nine + reciprocal (preset 9,
// the default) 798 us at 24 blocks per SM and 776 us at 28, where 8192
// column groups over 4256 blocks leave no block a third group.  Additions on
// the integer pipe cost more than they save (a binary64 add in integer
// arithmetic runs at 0.31 Tops/s against 0.52 for the fp64 instruction, a
// multiply at 0.56, a reciprocal at 0.22 against 0.12 for the fp64
// sequence).  Depth 1 (the next level's inputs in flight while one is
// solved) is faster again: 742 us against 779 at depth 2, same bits.  The
// default float64 SLAB form: depth 1, up to 28 blocks per SM, the grid
// balanced so that every block takes the same number of groups.
constexpr int kVadvPlacementDefault = 9;
constexpr int kVadvSlabBlocksPerSm = 28;
constexpr int kVadvPlacementCount = (int)(sizeof(kVadvPlacements) / sizeof(kVadvPlacements[0]));
template <class C>
constexpr uint32_t kVadvDefaultPlacement = std::is_same<C, double>::value ? kVadvPlacements[kVadvPlacementDefault] : 0u;

// SMEM variant with asynchronous staging: the six
// per-level inputs of the forward sweep (wcon at k+1 in both columns, stage
// at k+1, pos/tens/tensstage at k) are copied global -> shared with cp.async
// into a ring of R = D+1 slots, D levels ahead of the recurrence; the
// backward sweep streams pos the same way.  Slots are compile-time indices
// (the level loops are unrolled by R) and BT threads per block is a template
// parameter, so every shared-memory address is a register + immediate.
// Layout of dynamic shared memory: ccol[nk][BT], dcol[nk][BT] (compute type),
// then ring[R][6][BT] (RingOf<storage>), 16-byte aligned.
template <class S, class C, int BT, int D, class P = C>
__global__ void __launch_bounds__(BT)
    vadv_async_kernel(const S* __restrict__ stage, const S* __restrict__ pos, const S* __restrict__ tens,
                      const S* tensstage, const S* __restrict__ wcon, S* out, int ni, int nj, int nk,
                      int si, int sj, int sk, int wsh, int ring_offset) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int t = threadIdx.x;
    P* sc = reinterpret_cast<P*>(smem_raw) + t;
    auto* ring = reinterpret_cast<typename RingOf<S>::T*>(smem_raw + ring_offset) + t;
    const int i = blockIdx.x * BT + t;
    const int j = blockIdx.y;
    if (i >= ni) return;  // no block-wide barrier below
    vadv_async_column<S, C, BT, D, int, false, P>(stage, pos, tens, tensstage, wcon, out, i * si + j * sj, nk, sk,
                                                  wsh, sc, sc + nk * BT, ring);
}

// SLAB variant: a persistent grid of BT-thread blocks walks the (i-block, j)
// column groups; each thread keeps its forward-sweep factors in a compact
// slab of the caller's ccol/dcol memory (level k of slot q at [k * nslots +
// q]) instead of at its column's own position, so the factor working set is
// nslots * nk * 2 elements -- sized to stay in L2 -- rather than the whole
// field.  Inputs and read-back factors are staged with cp.async
// (vadv_async_column<..., SLAB = true>); the shared memory is the ring only.
template <class S, class C, int BT, int D, uint32_t PL>
__global__ void __launch_bounds__(BT)
    vadv_slab_kernel(const S* __restrict__ stage, const S* __restrict__ pos, const S* __restrict__ tens,
                     const S* tensstage, const S* __restrict__ wcon, S* out, C* __restrict__ slab_c,
                     C* __restrict__ slab_d, int ni, int nj, int nk, int si, int sj, int sk, int wsh) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int t = threadIdx.x;
    auto* ring = reinterpret_cast<typename RingOf<S>::T*>(smem_raw) + t;
    const int nslots = gridDim.x * BT;
    const int slot = blockIdx.x * BT + t;
    const int gx = (ni + BT - 1) / BT;
    const int64_t ngroups = (int64_t)gx * nj;
    for (int64_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int i = (int)(g % gx) * BT + t;
        const int j = (int)(g / gx);
        if (i < ni) {
            vadv_async_column<S, C, BT, D, int, true, C, PL>(stage, pos, tens, tensstage, wcon, out, i * si + j * sj,
                                                             nk, sk, wsh, slab_c + slot, slab_d + slot, ring, nslots);
        }
    }
}

// WSLAB variant: the SLAB scheme with the rows of each warp's 32 columns
// staged together (vadv_warp_column): fewer, wider copies per level.  Needs
// i unit-stride.  Each block's warps take 32-column pieces of one
// BT-column group.
template <class S, class C, int W, int D>
__global__ void __launch_bounds__(32 * W)
    vadv_wslab_kernel(const S* __restrict__ stage, const S* __restrict__ pos, const S* __restrict__ tens,
                      const S* tensstage, const S* __restrict__ wcon, S* out, C* __restrict__ slab_c,
                      C* __restrict__ slab_d, int ni, int nj, int nk, int sj, int sk, int wsh) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int BT = 32 * W;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* ring = smem_raw + warp * WarpRing<S, C, D>::BYTES;
    const int64_t nslots = (int64_t)gridDim.x * BT;
    const int64_t slot0 = (int64_t)blockIdx.x * BT + warp * 32;
    const int gx = (ni + BT - 1) / BT;
    const int64_t ngroups = (int64_t)gx * nj;
    for (int64_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
        const int i0 = (int)(g % gx) * BT + warp * 32;
        const int j = (int)(g / gx);
        const int nvalid = min(32, ni - i0);
        if (nvalid <= 0) continue;  // warp-uniform
        vadv_warp_column<S, C, D, int>(stage, pos, tens, tensstage, wcon, out, i0 + j * sj, lane, nvalid, nk, sk, wsh,
                                       slab_c + slot0, slab_d + slot0, nslots, ring);
    }
}

template <class S, class C, bool GLOBAL, int D>
int launch_one(dim3 grid, dim3 block, size_t smem, cudaStream_t stream, const void* stage, const void* pos,
               const void* tens, const void* tensstage, const void* wcon, void* out, void* ccol, void* dcol,
               int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, int64_t wsh) {
    auto kernel = vadv_kernel<S, C, GLOBAL, D>;
    if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<grid, block, smem, stream>>>((const S*)stage, (const S*)pos, (const S*)tens, (const S*)tensstage,
                                          (const S*)wcon, (S*)out, (C*)ccol, (C*)dcol, (int)ni, (int)nj, (int)nk,
                                          si, sj, sk, wsh);
    return SB_OK;
}

template <class S, class C, bool GLOBAL>
int launch_depth(int depth, dim3 grid, dim3 block, size_t smem, cudaStream_t stream, const void* stage,
                 const void* pos, const void* tens, const void* tensstage, const void* wcon, void* out,
                 void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj,
                 int64_t sk, int64_t wsh) {
    switch (depth) {
        case 1: return launch_one<S, C, GLOBAL, 1>(grid, block, smem, stream, stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
        case 2: return launch_one<S, C, GLOBAL, 2>(grid, block, smem, stream, stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
        case 4: return launch_one<S, C, GLOBAL, 4>(grid, block, smem, stream, stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
        case 8: return launch_one<S, C, GLOBAL, 8>(grid, block, smem, stream, stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
    }
    return fail(SB_ERR_INVALID, "vadv prefetch depth (unroll) must be 1, 2, 4 or 8 (got %d)", depth);
}

// Shared memory of the asynchronous SMEM kernel for BT threads and depth D
// (factors in the recurrence type P).
template <class S, class P>
size_t async_smem(int64_t nk, int bt, int depth, int* ring_offset) {
    const size_t scratch = ((2 * sizeof(P) * (size_t)nk * (size_t)bt) + 15) / 16 * 16;
    if (ring_offset) *ring_offset = (int)scratch;
    return scratch + (size_t)(depth + 1) * 6 * (size_t)bt * sizeof(typename RingOf<S>::T);
}

template <class S, class C, int BT, int D, class P>
int launch_async_one(dim3 grid, size_t smem, int ring_offset, cudaStream_t stream, const void* stage,
                     const void* pos, const void* tens, const void* tensstage, const void* wcon, void* out,
                     int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, int64_t wsh) {
    auto kernel = vadv_async_kernel<S, C, BT, D, P>;
    if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<grid, BT, smem, stream>>>((const S*)stage, (const S*)pos, (const S*)tens, (const S*)tensstage,
                                       (const S*)wcon, (S*)out, (int)ni, (int)nj, (int)nk, (int)si, (int)sj,
                                       (int)sk, (int)wsh, ring_offset);
    return SB_OK;
}

// Asynchronous SMEM kernel if this launch qualifies (one
// row of 32 or 64 columns per block, all offsets within 32 bits); returns
// SB_ERR_UNSUPPORTED (without error text) when it does not.
template <class S, class C, class P = C>
int launch_async(int bx, int by, int depth, const DeviceProps* p, cudaStream_t stream, const void* stage,
                 const void* pos, const void* tens, const void* tensstage, const void* wcon, void* out,
                 int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, int64_t wsh) {
    if constexpr (sizeof(S) == 2 && sizeof(C) != 4) {
        return SB_ERR_UNSUPPORTED;
    } else {
    if (by != 1 || (bx != 32 && bx != 64) || (depth != 4 && depth != 8)) return SB_ERR_UNSUPPORTED;
    if (si <= 0 || sj <= 0 || sk <= 0 || nj > p->max_grid_y) return SB_ERR_UNSUPPORTED;
    const int64_t span = (ni + 1) * si + nj * sj + (nk + 1) * sk;
    if (span >= (1LL << 31)) return SB_ERR_UNSUPPORTED;
    int ring_offset = 0;
    const size_t smem = async_smem<S, P>(nk, bx, depth, &ring_offset);
    if ((int64_t)smem > p->smem_optin) return SB_ERR_UNSUPPORTED;
    const dim3 grid((unsigned)ceil_div(ni, bx), (unsigned)nj);
#define SB_VADV_ASYNC(BTV, DV)                                                                              \
    if (bx == BTV && depth == DV)                                                                           \
        return launch_async_one<S, C, BTV, DV, P>(grid, smem, ring_offset, stream, stage, pos, tens, tensstage, \
                                               wcon, out, ni, nj, nk, si, sj, sk, wsh);
    SB_VADV_ASYNC(32, 4)
    SB_VADV_ASYNC(32, 8)
    SB_VADV_ASYNC(64, 4)
    SB_VADV_ASYNC(64, 8)
#undef SB_VADV_ASYNC
    return SB_ERR_UNSUPPORTED;
    }
}

template <class S, class C, int BT, int D, uint32_t PL>
int launch_slab_one(int blocks_per_sm, const DeviceProps* p, cudaStream_t stream, const void* stage,
                    const void* pos, const void* tens, const void* tensstage, const void* wcon, void* out,
                    void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
                    int64_t wsh) {
    auto kernel = vadv_slab_kernel<S, C, BT, D, PL>;
    const size_t smem = (size_t)(D + 1) * 6 * BT * sizeof(typename RingOf<S>::T);
    if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int fit = 0;
    SB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kernel, BT, smem));
    int per_sm = std::max(1, fit);
    if (blocks_per_sm > 0) {
        per_sm = std::min(per_sm, blocks_per_sm);
    } else if (PL != 0u) {
        // integer-pipe products: more warps in flight beat an L2-resident slab
        per_sm = std::min(per_sm, kVadvSlabBlocksPerSm);
    } else {
        // keep the factor slabs (2 * nk elements per thread) within half of L2
        const int64_t per_block = 2 * nk * (int64_t)sizeof(C) * BT * p->sm_count;
        const int64_t budget = (int64_t)(p->l2_bytes > 0 ? p->l2_bytes : (128 << 20)) / 2;
        per_sm = (int)std::max<int64_t>(1, std::min<int64_t>(per_sm, budget / std::max<int64_t>(1, per_block)));
    }
    const int64_t ngroups = ceil_div(ni, BT) * nj;
    // the slabs use ccol/dcol as raw memory: nslots * nk elements must lie
    // inside the fields' interior span
    const int64_t span = (ni - 1) * si + (nj - 1) * sj + (nk - 1) * sk + 1;
    int64_t grid = std::min<int64_t>((int64_t)per_sm * p->sm_count, ngroups);
    grid = std::min<int64_t>(grid, span / (nk * BT));
    if (grid < 1) return SB_ERR_UNSUPPORTED;
    // balance: the fewest blocks that still take every group in the same
    // number of rounds, so that no block runs an extra round alone -- where
    // that keeps at least 90% of the blocks (fewer warps in flight cost more:
    // 512x512x80 at 24 blocks per SM, balanced to 18, 798 -> 850 us; at 28,
    // balanced to 27, 798 -> 777 us)
    const int64_t balanced = ceil_div(ngroups, ceil_div(ngroups, grid));
    if (balanced * 10 >= grid * 9) grid = balanced;
    kernel<<<(unsigned)grid, BT, smem, stream>>>((const S*)stage, (const S*)pos, (const S*)tens, (const S*)tensstage,
                                                 (const S*)wcon, (S*)out, (C*)ccol, (C*)dcol, (int)ni, (int)nj,
                                                 (int)nk, (int)si, (int)sj, (int)sk, (int)wsh);
    return SB_OK;
}

// SLAB variant if this launch qualifies (ccol/dcol given, ring entries of the
// compute size, positive strides, 32-bit offsets); SB_ERR_UNSUPPORTED (without
// error text) otherwise.
template <class S, class C>
int launch_slab(int bx, int depth, int blocks_per_sm, int placement, const DeviceProps* p, cudaStream_t stream,
                const void* stage, const void* pos, const void* tens, const void* tensstage, const void* wcon,
                void* out, void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj,
                int64_t sk, int64_t wsh) {
    if constexpr (sizeof(typename RingOf<S>::T) != sizeof(C)) {
        return SB_ERR_UNSUPPORTED;
    } else {
        if (!ccol || !dcol || si <= 0 || sj <= 0 || sk <= 0) return SB_ERR_UNSUPPORTED;
        const int64_t span = (ni + 1) * si + nj * sj + (nk + 1) * sk;
        if (span >= (1LL << 31) || (int64_t)ni * nj * nk >= (1LL << 31)) return SB_ERR_UNSUPPORTED;
        SB_CHECK(placement >= 0 && placement < kVadvPlacementCount, SB_ERR_INVALID,
                 "vadv SLAB: placement preset %d out of range [0, %d)", placement, kVadvPlacementCount);
        if constexpr (std::is_same<C, double>::value) {
            if (bx == 32 && depth == 1 && placement != 0) {
#define SB_VADV_SLAB_PL(Q)                                                                                         \
    if (placement == Q)                                                                                            \
        return launch_slab_one<S, C, 32, 1, kVadvPlacements[Q]>(blocks_per_sm, p, stream, stage, pos, tens,        \
                                                                tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, \
                                                                sj, sk, wsh);
                SB_VADV_SLAB_PL(1)
                SB_VADV_SLAB_PL(2)
                SB_VADV_SLAB_PL(3)
                SB_VADV_SLAB_PL(4)
                SB_VADV_SLAB_PL(5)
                SB_VADV_SLAB_PL(6)
                SB_VADV_SLAB_PL(7)
                SB_VADV_SLAB_PL(8)
                SB_VADV_SLAB_PL(9)
                SB_VADV_SLAB_PL(10)
                SB_VADV_SLAB_PL(11)
                SB_VADV_SLAB_PL(12)
                SB_VADV_SLAB_PL(13)
                SB_VADV_SLAB_PL(14)
                SB_VADV_SLAB_PL(15)
#undef SB_VADV_SLAB_PL
            }
        }
#define SB_VADV_SLAB_CASE(BTV, DV)                                                                                 \
    if (bx == BTV && depth == DV)                                                                                  \
        return launch_slab_one<S, C, BTV, DV, kVadvDefaultPlacement<C>>(blocks_per_sm, p, stream, stage, pos,   \
                                                                           tens, tensstage, wcon, out, ccol, dcol, \
                                                                           ni, nj, nk, si, sj, sk, wsh);
        SB_VADV_SLAB_CASE(32, 1)
        SB_VADV_SLAB_CASE(32, 2)
        SB_VADV_SLAB_CASE(32, 4)
        SB_VADV_SLAB_CASE(32, 8)
        SB_VADV_SLAB_CASE(64, 2)
        SB_VADV_SLAB_CASE(64, 4)
        SB_VADV_SLAB_CASE(64, 8)
#undef SB_VADV_SLAB_CASE
        return SB_ERR_UNSUPPORTED;
    }
}

template <class S, class C, int W, int D>
int launch_wslab_one(int blocks_per_sm, const DeviceProps* p, cudaStream_t stream, const void* stage,
                     const void* pos, const void* tens, const void* tensstage, const void* wcon, void* out,
                     void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
                     int64_t wsh) {
    constexpr int BT = 32 * W;
    auto kernel = vadv_wslab_kernel<S, C, W, D>;
    const size_t smem = (size_t)W * WarpRing<S, C, D>::BYTES;
    if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int fit = 0;
    SB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kernel, BT, smem));
    int per_sm = std::max(1, fit);
    if (blocks_per_sm > 0) {
        per_sm = std::min(per_sm, blocks_per_sm);
    } else {
        const int64_t per_block = 2 * nk * (int64_t)sizeof(C) * BT * p->sm_count;
        const int64_t budget = (int64_t)(p->l2_bytes > 0 ? p->l2_bytes : (128 << 20)) / 2;
        per_sm = (int)std::max<int64_t>(1, std::min<int64_t>(per_sm, budget / std::max<int64_t>(1, per_block)));
    }
    const int64_t ngroups = ceil_div(ni, BT) * nj;
    const int64_t span = (ni - 1) * si + (nj - 1) * sj + (nk - 1) * sk + 1;
    int64_t grid = std::min<int64_t>((int64_t)per_sm * p->sm_count, ngroups);
    grid = std::min<int64_t>(grid, span / (nk * BT));
    if (grid < 1) return SB_ERR_UNSUPPORTED;
    kernel<<<(unsigned)grid, BT, smem, stream>>>((const S*)stage, (const S*)pos, (const S*)tens, (const S*)tensstage,
                                                 (const S*)wcon, (S*)out, (C*)ccol, (C*)dcol, (int)ni, (int)nj,
                                                 (int)nk, (int)sj, (int)sk, (int)wsh);
    return SB_OK;
}

// WSLAB variant if this launch qualifies (ccol/dcol given, i unit-stride,
// positive strides, 32-bit offsets); SB_ERR_UNSUPPORTED otherwise.
template <class S, class C>
int launch_wslab(int bx, int depth, int blocks_per_sm, const DeviceProps* p, cudaStream_t stream,
                 const void* stage, const void* pos, const void* tens, const void* tensstage, const void* wcon,
                 void* out, void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj,
                 int64_t sk, int64_t wsh) {
    if (!ccol || !dcol || si != 1 || sj <= 0 || sk <= 0) return SB_ERR_UNSUPPORTED;
    const int64_t span = (ni + 1) * si + nj * sj + (nk + 1) * sk;
    if (span >= (1LL << 31) || (int64_t)ni * nj * nk >= (1LL << 31)) return SB_ERR_UNSUPPORTED;
#define SB_VADV_WSLAB_CASE(WV, DV)                                                                               \
    if (bx == 32 * WV && depth == DV)                                                                            \
        return launch_wslab_one<S, C, WV, DV>(blocks_per_sm, p, stream, stage, pos, tens, tensstage, wcon, out, \
                                              ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
    SB_VADV_WSLAB_CASE(1, 2)
    SB_VADV_WSLAB_CASE(1, 4)
    SB_VADV_WSLAB_CASE(1, 8)
    SB_VADV_WSLAB_CASE(2, 2)
    SB_VADV_WSLAB_CASE(2, 4)
    SB_VADV_WSLAB_CASE(2, 8)
#undef SB_VADV_WSLAB_CASE
    return SB_ERR_UNSUPPORTED;
}

// ---------------------------------------------------------------------------
// TMEM variant (float32 compute): one persistent block of 4*G warps per SM.
// Warp w solves 32-column groups with vadv_tmem_column and keeps its
// columns' factors in TMEM lanes 32*(w%4) .. +31 (the lanes warp w may
// access), columns (w/4)*cpw .. +cpw-1 of the block's 512-column allocation.
// The block allocates all 512 columns and asks for enough shared memory that
// no second block shares its SM, so the allocation never waits.
// ---------------------------------------------------------------------------
// The fields of up to three components on one wcon (u, v, w of the
// reference's all_components: wcon shifted by wsh[c] elements), all with the
// same layout; nc components are solved for each column group in turn, so a
// group's wcon rows come from HBM once and from L2 for the others.
template <class S>
struct TmemComponents {
    const S* stage[3];
    const S* pos[3];
    const S* tens[3];
    const S* tensstage[3];
    S* out[3];
    int wsh[3];
    int nc;
};

template <class S, int D, int KP, bool SA>
__global__ void __launch_bounds__(512, 1)
    vadv_tmem_kernel(const TmemComponents<S> f, const S* __restrict__ wcon, int ni, int nj, int nk, int sj, int sk,
                     int cpw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(smem_raw);
    unsigned char* ring = smem_raw + 16 + warp * WarpRing<S, float, D>::BYTES;
    if (warp == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(s_taddr), ncols = 512u;
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(dst), "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tbase = *reinterpret_cast<volatile uint32_t*>(s_taddr);
    const uint32_t tcol = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)((warp >> 2) * cpw);
    const int gx = (ni + 31) / 32;
    const int64_t ngroups = (int64_t)gx * nj;
    for (int64_t g = (int64_t)blockIdx.x * nwarps + warp; g < ngroups; g += (int64_t)gridDim.x * nwarps) {
        const int i0 = (int)(g % gx) * 32;
        const int j = (int)(g / gx);
        const int nvalid = min(32, ni - i0);
        for (int c = 0; c < f.nc; ++c)
            vadv_tmem_column<S, D, KP, int, SA>(f.stage[c], f.pos[c], f.tens[c], f.tensstage[c], wcon, f.out[c],
                                                i0 + j * sj, lane, nvalid, nk, sk, f.wsh[c], tcol, ring);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0) {
        const uint32_t ncols = 512u;
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(ncols) : "memory");
    }
}

// TMEM staging through 32-bit shared addresses (sb_tune.flags bit 10) or
// generic pointers (bit 11); neither bit: the default below (512x512x80:
// float32 135 vs 136 us, bfloat16 120 vs 125 us at ring depth 8).
constexpr bool kTmemSharedAddr = true;

template <class S, int D>
int launch_tmem_one(int g4, int cpw, bool sa, const DeviceProps* p, cudaStream_t stream,
                    const TmemComponents<S>& comps, const void* wcon, int64_t ni, int64_t nj, int64_t nk, int64_t sj,
                    int64_t sk) {
    const int64_t kmod = ((int64_t)sk * (int64_t)sizeof(S)) % 16;
    auto kernel = kmod == 0 ? (sa ? vadv_tmem_kernel<S, D, 1, true> : vadv_tmem_kernel<S, D, 1, false>)
                  : kmod == 8 ? (sa ? vadv_tmem_kernel<S, D, 2, true> : vadv_tmem_kernel<S, D, 2, false>)
                              : vadv_tmem_kernel<S, D, 0, false>;
    // fewer warps per lane quarter when their rings do not fit
    g4 = std::min<int64_t>(g4, (p->smem_optin - 16) / (4 * (int64_t)WarpRing<S, float, D>::BYTES));
    if (g4 < 1) return SB_ERR_UNSUPPORTED;
    const int nwarps = 4 * g4;
    // at least 120 KB: one block per SM, so the 512-column allocation is free
    const size_t smem = std::max<size_t>(16 + (size_t)nwarps * WarpRing<S, float, D>::BYTES, 120 * 1024);
    if ((int64_t)smem > p->smem_optin) return SB_ERR_UNSUPPORTED;
    SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t ngroups = ceil_div(ni, (int64_t)32) * nj;
    const int64_t grid = std::min<int64_t>(p->sm_count, ceil_div(ngroups, (int64_t)nwarps));
    kernel<<<(unsigned)grid, 32 * nwarps, smem, stream>>>(comps, (const S*)wcon, (int)ni, (int)nj, (int)nk,
                                                          (int)sj, (int)sk, cpw);
    return SB_OK;
}

// TMEM variant if this launch qualifies (float32 compute, i unit-stride,
// positive strides, 32-bit offsets, 2 <= nk <= 256); SB_ERR_UNSUPPORTED
// otherwise.  depth 0 = the deepest ring that fits.
template <class S, class C>
int launch_tmem_comps(int depth, bool sa, const DeviceProps* p, cudaStream_t stream, const TmemComponents<S>& comps,
                      const void* wcon, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk) {
    if constexpr (!std::is_same<C, float>::value) {
        return SB_ERR_UNSUPPORTED;
    } else {
        if (si != 1 || sj <= 0 || sk <= 0 || nk < 2 || nk > 256) return SB_ERR_UNSUPPORTED;
        const int64_t span = (ni + 1) * si + nj * sj + (nk + 1) * sk;
        if (span >= (1LL << 31) || (int64_t)ni * nj * nk >= (1LL << 31)) return SB_ERR_UNSUPPORTED;
        const int cpw = 16 * (int)ceil_div(nk, (int64_t)8);  // ccol, dcol of ceil8(nk) levels
        const int g4 = std::min(4, 512 / cpw);             // warps per TMEM lane quarter
        int rc = SB_ERR_UNSUPPORTED;
        if ((depth == 0 || depth == 16) && rc == SB_ERR_UNSUPPORTED)
            rc = launch_tmem_one<S, 16>(g4, cpw, sa, p, stream, comps, wcon, ni, nj, nk, sj, sk);
        if ((depth == 0 || depth == 8) && rc == SB_ERR_UNSUPPORTED)
            rc = launch_tmem_one<S, 8>(g4, cpw, sa, p, stream, comps, wcon, ni, nj, nk, sj, sk);
        if (depth == 4 && rc == SB_ERR_UNSUPPORTED)
            rc = launch_tmem_one<S, 4>(g4, cpw, sa, p, stream, comps, wcon, ni, nj, nk, sj, sk);
        return rc;
    }
}

// one component
template <class S, class C>
int launch_tmem(int depth, bool sa, const DeviceProps* p, cudaStream_t stream, const void* stage, const void* pos,
                const void* tens, const void* tensstage, const void* wcon, void* out, int64_t ni, int64_t nj,
                int64_t nk, int64_t si, int64_t sj, int64_t sk, int64_t wsh) {
    TmemComponents<S> comps{};
    comps.stage[0] = (const S*)stage;
    comps.pos[0] = (const S*)pos;
    comps.tens[0] = (const S*)tens;
    comps.tensstage[0] = (const S*)tensstage;
    comps.out[0] = (S*)out;
    comps.wsh[0] = (int)wsh;
    comps.nc = 1;
    return launch_tmem_comps<S, C>(depth, sa, p, stream, comps, wcon, ni, nj, nk, si, sj, sk);
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
    const int placement = tune ? (tune->flags >> 4) & 15 : 0;
    int bx = (tune && tune->block_x > 0) ? tune->block_x : 32;
    int by = (tune && tune->block_y > 0) ? tune->block_y : 1;
    SB_CHECK(bx * by <= 256 && bx >= 1 && by >= 1, SB_ERR_INVALID, "vadv block (%d, %d) exceeds 256 threads", bx, by);
    const size_t smem = 2 * sizeof(C) * (size_t)nk * (size_t)(bx * by);
    const bool can_global = ccol && dcol && sizeof(S) == sizeof(C);
    // float32 compute, no explicit shape: factors in tensor memory (512x512x80
    // float32 137 us against 171 us for WSLAB and 180 us for SMEM async;
    // bfloat16 113 us when the level stride is a multiple of 16 bytes, else
    // the staging address arithmetic makes it no faster than WSLAB / SMEM).
    // Below 2048 column groups of 32 (256 x 256) the one-block-per-SM launch
    // is not filled and SMEM async is as fast or faster (22 vs 27 us at 64^2).
    if constexpr (std::is_same<C, float>::value) {
        if (variant == SB_VARIANT_AUTO && !(tune && (tune->block_x || tune->block_y || tune->unroll)) &&
            ceil_div(ni, (int64_t)32) * nj >= 2048 && (sizeof(S) == 4 || (sk * (int64_t)sizeof(S)) % 8 == 0)) {
            const int arc = launch_tmem<S, C>(8, kTmemSharedAddr, p, stream, stage, pos, tens, tensstage, wcon, out,
                                              ni, nj, nk, si, sj, sk, wsh);
            if (arc != SB_ERR_UNSUPPORTED) return arc;
        }
    }
    if (variant == SB_VARIANT_AUTO && ccol && dcol && !(tune && (tune->block_x || tune->block_y || tune->unroll))) {
        // scratch fields given and no explicit shape: the persistent slab forms
        // (row-staged for 2- and 4-byte storage), falling back below if the
        // layout does not qualify
        const int arc = sizeof(S) <= 4
                            ? launch_wslab<S, C>(32, 4, 0, p, stream, stage, pos, tens, tensstage, wcon, out, ccol,
                                                 dcol, ni, nj, nk, si, sj, sk, wsh)
                            : (std::is_same<C, double>::value
                                   ? launch_slab<S, C>(32, 1, kVadvSlabBlocksPerSm, placement, p, stream, stage, pos,
                                                       tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj,
                                                       sk, wsh)
                                   : launch_slab<S, C>(64, 2, 32, placement, p, stream, stage, pos, tens, tensstage,
                                                       wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh));
        if (arc != SB_ERR_UNSUPPORTED) return arc;
    }
    if (variant == SB_VARIANT_AUTO) variant = ((int64_t)smem <= p->smem_optin) ? SB_VADV_SMEM : SB_VADV_GLOBAL;
    SB_CHECK(variant == SB_VADV_SMEM || variant == SB_VADV_GLOBAL || variant == SB_VADV_SLAB ||
                 variant == SB_VADV_WSLAB || variant == SB_VADV_TMEM,
             SB_ERR_UNSUPPORTED, "vadv variant %d is not available", variant);
    if (variant == SB_VADV_TMEM) {
        const int d = (tune && tune->unroll > 0) ? tune->unroll : 0;
        SB_CHECK(d == 0 || d == 4 || d == 8 || d == 16, SB_ERR_INVALID, "vadv TMEM ring depth must be 4, 8 or 16");
        const bool sa = tune && (tune->flags & 0x400) ? true : (tune && (tune->flags & 0x800) ? false : kTmemSharedAddr);
        const int rc2 = launch_tmem<S, C>(d, sa, p, stream, stage, pos, tens, tensstage, wcon, out, ni, nj, nk, si, sj,
                                          sk, wsh);
        SB_CHECK(rc2 != SB_ERR_UNSUPPORTED, SB_ERR_UNSUPPORTED,
                 "vadv TMEM variant: needs float32 compute, i unit-stride, positive strides, 32-bit offsets and "
                 "2 <= nk <= 256");
        return rc2;
    }
    if (variant == SB_VADV_WSLAB) {
        SB_CHECK(ccol && dcol, SB_ERR_INVALID, "vadv WSLAB variant needs ccol/dcol scratch fields");
        const int d = (tune && tune->unroll > 0) ? tune->unroll : 4;
        const int bpsm = tune ? tune->k_per_cta : 0;
        const int rc2 = launch_wslab<S, C>(bx, d, bpsm, p, stream, stage, pos, tens, tensstage, wcon, out, ccol, dcol,
                                           ni, nj, nk, si, sj, sk, wsh);
        SB_CHECK(rc2 != SB_ERR_UNSUPPORTED, SB_ERR_UNSUPPORTED,
                 "vadv WSLAB variant: needs blocks of 32 or 64 threads, depth 2, 4 or 8, i unit-stride, positive "
                 "strides and 32-bit offsets");
        return rc2;
    }
    if (variant == SB_VADV_SLAB) {
        SB_CHECK(ccol && dcol, SB_ERR_INVALID, "vadv SLAB variant needs ccol/dcol scratch fields");
        const int d = (tune && tune->unroll > 0) ? tune->unroll : 4;
        const int bpsm = tune ? tune->k_per_cta : 0;
        const int rc2 = launch_slab<S, C>(bx, d, bpsm, placement, p, stream, stage, pos, tens, tensstage, wcon, out,
                                          ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
        SB_CHECK(rc2 != SB_ERR_UNSUPPORTED, SB_ERR_UNSUPPORTED,
                 "vadv SLAB variant: needs blocks of 32 or 64 threads, depth 1 (32 threads), 2, 4 or 8, positive strides, "
                 "32-bit offsets and a compute type as wide as the storage ring entries");
        return rc2;
    }
    const int64_t gx = ceil_div(ni, bx), gy = ceil_div(nj, by);
    SB_CHECK(gy <= p->max_grid_y, SB_ERR_INVALID, "vadv grid too large");
    const dim3 grid((unsigned)gx, (unsigned)gy), block(bx, by);
    const int depth = (tune && tune->unroll > 0) ? tune->unroll : (sizeof(C) == 8 ? 4 : 8);
    if (variant == SB_VADV_SMEM) {
        const int arc = launch_async<S, C>(bx, by, depth, p, stream, stage, pos, tens, tensstage, wcon, out, ni, nj,
                                           nk, si, sj, sk, wsh);
        if (arc != SB_ERR_UNSUPPORTED) return arc;
        SB_CHECK((int64_t)smem <= p->smem_optin, SB_ERR_INVALID,
                 "vadv: %lld levels x %d columns need %zu bytes of shared memory (limit %d); "
                 "use fewer threads per block or the GLOBAL variant with ccol/dcol scratch",
                 (long long)nk, bx * by, smem, p->smem_optin);
        return launch_depth<S, C, false>(depth, grid, block, smem, stream, stage, pos, tens, tensstage, wcon, out,
                                         nullptr, nullptr, ni, nj, nk, si, sj, sk, wsh);
    }
    SB_CHECK(can_global, SB_ERR_INVALID, "vadv GLOBAL variant needs ccol/dcol scratch fields of the compute type");
    return launch_depth<S, C, true>(depth, grid, block, 0, stream, stage, pos, tens, tensstage, wcon, out,
                                    ccol, dcol, ni, nj, nk, si, sj, sk, wsh);
}

// All three components (the reference's all_components,
// stencils/base.py:475-483; its fused kernel: cuda_hip/templates/
// vertical_advection_localmemmerged.j2): with float32 compute on a layout the
// tensor-memory form takes, one launch solves u, v and w of each column group
// in turn (wcon read from HBM once); otherwise one launch per component.
template <class S, class C>
int launch_typed3(const void* const* stage, const void* const* pos, const void* const* tens,
                  const void* const* tensstage, const void* wcon, void* const* out, void* ccol, void* dcol,
                  int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, const sb_tune* tune,
                  cudaStream_t stream) {
    const int64_t wsh[3] = {si, sj, 0};  // u: wcon at (i+1, j); v: (i, j+1); w: (i, j)
    const int variant = tune ? tune->variant : SB_VARIANT_AUTO;
    if constexpr (std::is_same<C, float>::value) {
        const bool auto_fused = variant == SB_VARIANT_AUTO &&
                                !(tune && (tune->block_x || tune->block_y || tune->unroll)) &&
                                ceil_div(ni, (int64_t)32) * nj >= 2048 &&
                                (sizeof(S) == 4 || (sk * (int64_t)sizeof(S)) % 8 == 0);
        if (auto_fused || variant == SB_VADV_TMEM) {
            const DeviceProps* p;
            int rc = device_props(&p);
            if (rc) return rc;
            TmemComponents<S> comps{};
            for (int c = 0; c < 3; ++c) {
                comps.stage[c] = (const S*)stage[c];
                comps.pos[c] = (const S*)pos[c];
                comps.tens[c] = (const S*)tens[c];
                comps.tensstage[c] = (const S*)tensstage[c];
                comps.out[c] = (S*)out[c];
                comps.wsh[c] = (int)wsh[c];
            }
            comps.nc = 3;
            const int d = (tune && tune->unroll > 0) ? tune->unroll : (variant == SB_VADV_TMEM ? 0 : 8);
            SB_CHECK(d == 0 || d == 4 || d == 8 || d == 16, SB_ERR_INVALID, "vadv TMEM ring depth must be 4, 8 or 16");
            const bool sa =
                tune && (tune->flags & 0x400) ? true : (tune && (tune->flags & 0x800) ? false : kTmemSharedAddr);
            const int arc = launch_tmem_comps<S, C>(d, sa, p, stream, comps, wcon, ni, nj, nk, si, sj, sk);
            if (arc != SB_ERR_UNSUPPORTED) return arc;
            SB_CHECK(variant != SB_VADV_TMEM, SB_ERR_UNSUPPORTED,
                     "vadv TMEM variant: needs float32 compute, i unit-stride, positive strides, 32-bit offsets and "
                     "2 <= nk <= 256");
        }
    }
    for (int c = 0; c < 3; ++c) {
        const int rc = launch_typed<S, C>(stage[c], pos[c], tens[c], tensstage[c], wcon, out[c], ccol, dcol, ni, nj,
                                          nk, si, sj, sk, wsh[c], tune, stream);
        if (rc) return rc;
    }
    return SB_OK;
}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" int sb_vadv3(int storage, int compute, const void* const* stage, const void* const* pos,
                        const void* const* tens, const void* const* tensstage, const void* wcon, void* const* out,
                        void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj,
                        int64_t sk, const sb_tune* tune, void* stream, double* time_s) {
    clear_error();
    int rc = check_domain(ni, nj, nk, si, sj, sk);
    if (rc) return rc;
    SB_CHECK(stage && pos && tens && tensstage && out && wcon, SB_ERR_INVALID, "NULL field array");
    for (int c = 0; c < 3; ++c)
        SB_CHECK(stage[c] && pos[c] && tens[c] && tensstage[c] && out[c], SB_ERR_INVALID,
                 "NULL field pointer (component %d)", c);
    SB_CHECK((storage == SB_F64 && (compute == SB_F64 || compute == SB_F32X2)) ||
                 (storage == SB_F32 && (compute == SB_F32 || compute == SB_F64)) ||
                 (storage == SB_BF16 && compute == SB_F32),
             SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
    if (ni == 0 || nj == 0 || nk == 0) {
        if (time_s) *time_s = 0.0;
        return SB_OK;
    }
    SB_CHECK(nk >= 2, SB_ERR_INVALID, "vertical advection needs at least 2 levels (nk = %lld)", (long long)nk);
    cudaStream_t s = (cudaStream_t)stream;
    return timed(s, time_s, [&]() {
        if (storage == SB_F64 && compute == SB_F64)
            return launch_typed3<double, double>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F64 && compute == SB_F32X2)
            return launch_typed3<double, f32x2>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F32 && compute == SB_F32)
            return launch_typed3<float, float>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F32 && compute == SB_F64)
            return launch_typed3<float, double>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, tune, s);
        return launch_typed3<bf16, float>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, tune, s);
    });
}

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
    SB_CHECK((storage == SB_F64 && (compute == SB_F64 || compute == SB_F32X2)) ||
                 (storage == SB_F32 && (compute == SB_F32 || compute == SB_F64)) ||
                 (storage == SB_BF16 && compute == SB_F32),
             SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
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
        if (storage == SB_F64 && compute == SB_F32X2)
            return launch_typed<double, f32x2>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        if (storage == SB_F32 && compute == SB_F32)
            return launch_typed<float, float>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        if (storage == SB_F32 && compute == SB_F64)
            return launch_typed<float, double>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        if (storage == SB_BF16 && compute == SB_F32)
            return launch_typed<bf16, float>(stage, pos, tens, tensstage, wcon, out, ccol, dcol, ni, nj, nk, si, sj, sk, wsh, tune, s);
        return fail(SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
    });
}
