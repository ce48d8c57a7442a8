// Horizontal diffusion (hdiff) on sm_103a.
//
// Oracle: stencil_benchmarks/benchmarks_collection/stencils/base.py:276-311
//   lap = 4*inp - (((inp[i+1] + inp[i-1]) + inp[j+1]) + inp[j-1])
//   flx = lap[i+1] - lap[i];  flx = 0 where flx * (inp[i+1] - inp[i]) > 0
//   fly = lap[j+1] - lap[j];  fly = 0 where fly * (inp[j+1] - inp[j]) > 0
//   out = inp - coeff * (((flx[i] - flx[i-1]) + fly[j]) - fly[j-1])
// Every operation is rounded once, in this order, so fp64 results are
// bit-identical to the reference's numpy verification.
//
// TILE variant: a CTA owns a TX x TY tile of (i, j) and walks KPER k-planes.
// Per plane it stages inp with its 2-point halo in shared memory, then
// computes lap on (TX+2) x (TY+2), flx on (TX+1) x TY and fly on TX x (TY+1)
// -- each value once per tile, not five times per point -- and finally the
// output, reading coeff and writing out straight from/to HBM with coalesced
// accesses along i.  On GB300 the fp64 pipe (1/64 of the fp32 rate) is the
// binding resource for the fp64 form, so the kernel minimises fp64
// instructions: 4*inp is an exponent increment and the limiter's sign test
// runs on integer bit patterns (Ar<double>::scale2 / ::limit).
//
// Caller contract: inp is readable on [-2, ni+1] x [-2, nj+1] x [0, nk)
// relative to the interior pointer (a halo of at least 2 in i and j).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <mutex>
#include <type_traits>

#include "stencil_core.cuh"

namespace sb {
namespace {

template <class C>
struct HdiffSmem {
    static size_t bytes(int tx, int ty) {
        return sizeof(C) * (size_t)((ty + 4) * (tx + 4) + (ty + 2) * (tx + 2) + ty * (tx + 1) + (ty + 1) * tx);
    }
};

template <class S, class C, int TX, int NTY>
__global__ void __launch_bounds__(TX* NTY)
    hdiff_tile_kernel(const S* __restrict__ inp, const S* __restrict__ coeff, S* __restrict__ out,
                      int ni, int nj, int nk, int64_t si, int64_t sj, int64_t sk, int TY, int kper) {
    using A = Ar<C>;
    constexpr int WI = TX + 4, WL = TX + 2, WF = TX + 1, WY = TX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s_in = reinterpret_cast<C*>(smem_raw);  // (TY+4) x WI
    C* s_lap = s_in + (TY + 4) * WI;            // (TY+2) x WL
    C* s_flx = s_lap + (TY + 2) * WL;           // TY x WF
    C* s_fly = s_flx + TY * WF;                 // (TY+1) x WY

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * kper;
    const int k1 = min(nk, k0 + kper);
    const int ilim = ni + 1 - (i0 - 2);  // staged column ii is inside the halo'd array iff ii <= ilim
    const int jlim = nj + 1 - (j0 - 2);

    for (int k = k0; k < k1; ++k) {
        const S* in_k = inp + (int64_t)k * sk + (int64_t)(i0 - 2) * si + (int64_t)(j0 - 2) * sj;
        for (int jj = ty; jj < TY + 4; jj += NTY) {
            for (int ii = tx; ii < WI; ii += TX) {
                C v = C(0);
                if (ii <= ilim && jj <= jlim) v = ld<C, S>(in_k + (int64_t)ii * si + (int64_t)jj * sj);
                s_in[jj * WI + ii] = v;
            }
        }
        __syncthreads();

        // lap at local (ii, jj) <-> global (i0-1+ii, j0-1+jj)
        for (int jj = ty; jj < TY + 2; jj += NTY) {
            for (int ii = tx; ii < WL; ii += TX) {
                const C* c = s_in + (jj + 1) * WI + ii + 1;
                const C sum = A::add(A::add(A::add(c[1], c[-1]), c[WI]), c[-WI]);
                s_lap[jj * WL + ii] = A::sub(A::template scale2<2>(c[0]), sum);
            }
        }
        __syncthreads();

        // flx at local (ii, jj) <-> global (i0-1+ii, j0+jj)
        for (int jj = ty; jj < TY; jj += NTY) {
            for (int ii = tx; ii < WF; ii += TX) {
                const C* l = s_lap + (jj + 1) * WL + ii;
                const C* x = s_in + (jj + 2) * WI + ii + 1;
                s_flx[jj * WF + ii] = A::limit(A::sub(l[1], l[0]), x[1], x[0]);
            }
        }
        // fly at local (ii, jj) <-> global (i0+ii, j0-1+jj)
        for (int jj = ty; jj < TY + 1; jj += NTY) {
            for (int ii = tx; ii < WY; ii += TX) {
                const C* l = s_lap + jj * WL + ii + 1;
                const C* x = s_in + (jj + 1) * WI + ii + 2;
                s_fly[jj * WY + ii] = A::limit(A::sub(l[WL], l[0]), x[WI], x[0]);
            }
        }
        __syncthreads();

        // out at local (tx, jj) <-> global (i0+tx, j0+jj)
        const int gi = i0 + tx;
        for (int jj = ty; jj < TY; jj += NTY) {
            const int gj = j0 + jj;
            if (gi < ni && gj < nj) {
                const C fx1 = s_flx[jj * WF + tx + 1], fx0 = s_flx[jj * WF + tx];
                const C fy1 = s_fly[(jj + 1) * WY + tx], fy0 = s_fly[jj * WY + tx];
                const C x = s_in[(jj + 2) * WI + tx + 2];
                const int64_t o = (int64_t)k * sk + (int64_t)gi * si + (int64_t)gj * sj;
                const C cf = ld<C, S>(coeff + o);
                st<S, C>(out + o, A::sub(x, A::mul(cf, A::sub(A::add(A::sub(fx1, fx0), fy1), fy0))));
            }
        }
        __syncthreads();
    }
}

// JSCAN variant: one warp owns 32 consecutive i-columns (lanes) and marches
// along j; lanes 2..29 produce outputs (28 per warp), lanes 0-1 and 30-31
// only supply the i-halo.  Per row step a lane loads one inp value and one
// coeff value; inp(i+-1), lap(i+1) and flx(i-1) come from warp shuffles and
// inp/lap/fly of the previous rows stay in registers, so every lap, flx and
// fly of the strip is computed exactly once.  Rows are loaded U at a time
// (all loads of a chunk issued before its arithmetic) to keep U row
// requests per warp in flight.  Block = (32, NW) warps side by side in i;
// grid = (strips of 28*NW columns, j-segments of TY rows, k-chunks of KPER).
template <class S, class C, int U, class IDX>
__global__ void __launch_bounds__(256)
    hdiff_jscan_kernel(const S* __restrict__ inp, const S* __restrict__ coeff, S* __restrict__ out,
                       int ni, int nj, int nk, IDX si, IDX sj, IDX sk, int TY, int kper) {
    const int lane = threadIdx.x;
    const int i = (blockIdx.x * blockDim.y + threadIdx.y) * kJscanOut - 2 + lane;  // column of this lane
    const int j0 = blockIdx.y * TY;
    const int j1 = min(nj, j0 + TY);  // output rows [j0, j1)
    const int k0 = blockIdx.z * kper;
    const int k1 = min(nk, k0 + kper);
    for (int k = k0; k < k1; ++k) hdiff_strip<S, C, U, IDX>(inp, coeff, out, ni, nj, si, sj, sk, i, lane, j0, j1, k);
}

template <class S, class C, class IDX>
int launch_jscan_idx(dim3 grid, dim3 block, cudaStream_t stream, const void* inp, const void* coeff, void* out,
                     int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, int ty, int kper,
                     int unroll) {
#define SB_JSCAN(UV)                                                                                        \
    hdiff_jscan_kernel<S, C, UV, IDX><<<grid, block, 0, stream>>>((const S*)inp, (const S*)coeff, (S*)out,    \
                                                                  (int)ni, (int)nj, (int)nk, (IDX)si,       \
                                                                  (IDX)sj, (IDX)sk, ty, kper)
    switch (unroll) {
        case 1: SB_JSCAN(1); break;
        case 2: SB_JSCAN(2); break;
        case 4: SB_JSCAN(4); break;
        case 8: SB_JSCAN(8); break;
        default: return fail(SB_ERR_INVALID, "jscan unroll must be 1, 2, 4 or 8 (got %d)", unroll);
    }
#undef SB_JSCAN
    return SB_OK;
}

template <class S, class C>
int launch_jscan(const void* inp, const void* coeff, void* out, int64_t ni, int64_t nj, int64_t nk,
                 int64_t si, int64_t sj, int64_t sk, int nw, int ty, int kper, int unroll,
                 cudaStream_t stream, const DeviceProps* p) {
    SB_CHECK(nw >= 1 && nw <= 8, SB_ERR_INVALID, "jscan: 1..8 warps per block");
    const int64_t gx = ceil_div(ni, (int64_t)kJscanOut * nw), gy = ceil_div(nj, ty), gz = ceil_div(nk, kper);
    SB_CHECK(gy <= p->max_grid_y && gz <= p->max_grid_z, SB_ERR_INVALID, "hdiff grid too large");
    const dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)gz), block(32, nw);
    // 32-bit offsets when every address of the halo'd fields fits (the common case)
    const int64_t lo = -2 * (std::abs(si) + std::abs(sj));
    const int64_t hi = (ni + 2 + 32) * std::abs(si) + (nj + 2) * std::abs(sj) + nk * std::abs(sk);
    if (lo > -(1LL << 31) && hi < (1LL << 31))
        return launch_jscan_idx<S, C, int>(grid, block, stream, inp, coeff, out, ni, nj, nk, si, sj, sk, ty, kper, unroll);
    return launch_jscan_idx<S, C, int64_t>(grid, block, stream, inp, coeff, out, ni, nj, nk, si, sj, sk, ty, kper, unroll);
}

// VSCAN: warp strips of 32*V columns (hdiff_vscan_strip), strip s = blockIdx.x
// starting at column cs0 + s*step; the warps of a block take consecutive
// TY-row tiles of that strip (few strips per domain, so no idle warps).
template <class S, class C, int V, int U, class IDX>
__global__ void __launch_bounds__(256)
    hdiff_vscan_kernel(const S* __restrict__ inp, const S* __restrict__ coeff, S* __restrict__ out, int ni, int nj,
                       int nk, IDX sj, IDX sk, int cs0, int step, int TY, int kper) {
    const int strip = blockIdx.x;
    const int j0 = (blockIdx.y * blockDim.y + threadIdx.y) * TY;
    if (j0 >= nj) return;  // whole warp
    const int j1 = min(nj, j0 + TY);
    const int k0 = blockIdx.z * kper;
    const int k1 = min(nk, k0 + kper);
    for (int k = k0; k < k1; ++k)
        hdiff_vscan_strip<S, C, V, U, IDX>(inp, coeff, out, ni, nj, sj, sk, cs0 + strip * step, step, threadIdx.x,
                                           j0, j1, k);
}

// VSCAN launch if the layout qualifies: i unit-stride, j/k strides multiples
// of the vector size, and inp / coeff / out at the same offset from a vector
// boundary (then one column grid is vector-aligned in all three fields);
// SB_ERR_UNSUPPORTED (no error text) if not.
template <class S, class C, int V>
int launch_vscan(const void* inp, const void* coeff, void* out, int64_t ni, int64_t nj, int64_t nk, int64_t si,
                 int64_t sj, int64_t sk, int nw, int ty, int kper, int unroll, cudaStream_t stream,
                 const DeviceProps* p) {
    constexpr int ES = (int)sizeof(S), VB = V * ES;
    if (si != 1 || sj <= 0 || sk <= 0 || (sj * ES) % VB || (sk * ES) % VB) return SB_ERR_UNSUPPORTED;
    const uintptr_t a = (uintptr_t)inp;
    if (a % ES || (uintptr_t)coeff % VB != a % VB || (uintptr_t)out % VB != a % VB) return SB_ERR_UNSUPPORTED;
    SB_CHECK(nw >= 1 && nw <= 8, SB_ERR_INVALID, "vscan: 1..8 warps per block");
    SB_CHECK(ty >= 1 && kper >= 1, SB_ERR_INVALID, "vscan: tile_y and k_per_cta must be positive");
    const int off = (int)((a % VB) / ES);
    const int cs0 = -2 - (((off - 2) % V) + V) % V;  // <= -2, (off + cs0) % V == 0
    const int step = 32 * V - V * ((4 + V - 1) / V);
    const int64_t nstrips = ceil_div(ni - (cs0 + 2), (int64_t)step);
    const int64_t gx = nstrips, gy = ceil_div(ceil_div(nj, ty), (int64_t)nw), gz = ceil_div(nk, kper);
    SB_CHECK(gy <= p->max_grid_y && gz <= p->max_grid_z, SB_ERR_INVALID, "hdiff grid too large");
    const dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)gz), block(32, nw);
    const int64_t lo = -(2 + V) - 2 * sj;
    const int64_t hi = ni + 2 + 32 * V + (nj + 2) * sj + nk * sk;
    const bool small = lo > -(1LL << 31) && hi < (1LL << 31);
#define SB_VSCAN(UV, IDXT)                                                                                   \
    hdiff_vscan_kernel<S, C, V, UV, IDXT><<<grid, block, 0, stream>>>(                                        \
        (const S*)inp, (const S*)coeff, (S*)out, (int)ni, (int)nj, (int)nk, (IDXT)sj, (IDXT)sk, cs0, step,    \
        ty, kper)
#define SB_VSCAN_U(IDXT)                                                                                     \
    switch (unroll) {                                                                                         \
        case 1: SB_VSCAN(1, IDXT); break;                                                                     \
        case 2: SB_VSCAN(2, IDXT); break;                                                                     \
        case 4: SB_VSCAN(4, IDXT); break;                                                                     \
        case 8: SB_VSCAN(8, IDXT); break;                                                                     \
        default: return fail(SB_ERR_INVALID, "vscan unroll must be 1, 2, 4 or 8 (got %d)", unroll);           \
    }
    if (small) {
        SB_VSCAN_U(int)
    } else {
        SB_VSCAN_U(int64_t)
    }
#undef SB_VSCAN_U
#undef SB_VSCAN
    return SB_OK;
}

template <class S, class C, int TX, int NTY>
int launch_tile(const void* inp, const void* coeff, void* out, int64_t ni, int64_t nj, int64_t nk,
                int64_t si, int64_t sj, int64_t sk, int ty, int kper, cudaStream_t stream,
                const DeviceProps* p) {
    const size_t smem = HdiffSmem<C>::bytes(TX, ty);
    SB_CHECK((int64_t)smem <= p->smem_optin, SB_ERR_INVALID,
             "hdiff tile %dx%d needs %zu bytes of shared memory (device limit %d)", TX, ty, smem,
             p->smem_optin);
    auto kernel = hdiff_tile_kernel<S, C, TX, NTY>;
    if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t gx = ceil_div(ni, TX), gy = ceil_div(nj, ty), gz = ceil_div(nk, kper);
    SB_CHECK(gy <= p->max_grid_y && gz <= p->max_grid_z, SB_ERR_INVALID, "hdiff grid too large");
    kernel<<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), dim3(TX, NTY), smem, stream>>>(
        (const S*)inp, (const S*)coeff, (S*)out, (int)ni, (int)nj, (int)nk, si, sj, sk, ty, kper);
    return SB_OK;
}

// ---------------------------------------------------------------------------
// TMA variant: the TILE computation with inp staged by the tensor memory
// accelerator.  A CTA owns a TX x TY tile and walks KPER k-planes; plane k's
// box of inp arrives by one cp.async.bulk.tensor into one of two
// shared-memory stages, signalled by the stage's mbarrier, while the CTA
// computes the previous plane.  The tensor map starts at the 16-byte boundary
// at or below the halo corner inp(-2, -2, 0), `off` elements before it, so a
// box for the tile at i0 starts at x = i0 (a multiple of TX elements, hence of
// 16 bytes) and holds global i = i0 - 2 - off + c in column c; the box is
// TX + PADX columns wide (PADX >= 4 + the largest off) and TY + 4 rows high.
// Boxes reaching past the array are zero-filled by the hardware; those
// columns and rows only feed points that are not stored.  Waits are bounded
// (`polls` tries).  The give-up decision is taken by the whole CTA at the
// barrier after the lap phase (__syncthreads_or of the threads' results), so
// all threads leave together and none stores an output of that plane; before
// leaving, the leader waits (with the default bound) for the copies the CTA
// still has in flight and sets the status word, which the next status check
// of the library reports as SB_ERR_TIMEOUT.  Only if such a copy does not
// land within the default bound either can the CTA exit with it pending.
thread_local bool t_tma_used = false;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, int polls) {
    for (int it = 0; it < polls; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_plane(const CUtensorMap* map, uint32_t dst, uint32_t bar, int x, int y,
                                               int z, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

template <class S, class C>
struct TmaSmem {
    static constexpr int PADX = sizeof(S) == 2 ? 16 : 8;
    static __host__ __device__ size_t stage_bytes(int tx, int ty) {
        return ((size_t)(tx + PADX) * (ty + 4) * sizeof(S) + 127) / 128 * 128;
    }
    // Narrower storage than compute: each landed plane is widened once into a
    // compute-typed copy (a float -> double conversion per use would cost more
    // than the extra shared-memory pass).
    static constexpr bool CONV = !std::is_same<S, C>::value;
    static __host__ __device__ size_t conv_bytes(int tx, int ty) {
        return CONV ? ((size_t)(tx + PADX) * (ty + 4) * sizeof(C) + 127) / 128 * 128 : 0;
    }
    static size_t bytes(int tx, int ty) {
        return 2 * stage_bytes(tx, ty) + conv_bytes(tx, ty) +
               sizeof(C) * (size_t)((ty + 2) * (tx + 2) + ty * (tx + 1) + (ty + 1) * tx) + 16 + 16;
    }
};

template <class S, class C, int TX, int NTY, uint32_t PL>
__global__ void __launch_bounds__(TX* NTY)
    hdiff_tma_kernel(const __grid_constant__ CUtensorMap tmap, const S* __restrict__ coeff, S* __restrict__ out,
                     int ni, int nj, int nk, int64_t sj, int64_t sk, int TY, int kper, int off, int polls,
                     int* status) {
    using A = Ar<C>;
    using X = Mix<C, PL>;  // sites 0-10 below
    using M = TmaSmem<S, C>;
    using T = typename std::conditional<M::CONV, C, S>::type;  // element type the stencil reads
    constexpr int BX = TX + M::PADX, WL = TX + 2, WF = TX + 1, WY = TX;
    extern __shared__ __align__(128) unsigned char smem_tma[];
    const size_t stage = M::stage_bytes(TX, TY);
    C* s_conv = reinterpret_cast<C*>(smem_tma + 2 * stage);  // (TY+4) x BX, CONV only
    C* s_lap = reinterpret_cast<C*>(smem_tma + 2 * stage + M::conv_bytes(TX, TY));  // (TY+2) x WL
    C* s_flx = s_lap + (TY + 2) * WL;                        // TY x WF
    C* s_fly = s_flx + TY * WF;                              // (TY+1) x WY
    uint64_t* bars = reinterpret_cast<uint64_t*>(
        (reinterpret_cast<uintptr_t>(s_fly + (TY + 1) * WY) + 15) & ~(uintptr_t)15);
    const uint32_t stage0 = smem_addr(smem_tma), bar0 = smem_addr(bars);
    const uint32_t box_bytes = (uint32_t)(BX * (TY + 4) * sizeof(S));

    const int tx = threadIdx.x, ty = threadIdx.y;
    const bool leader = tx == 0 && ty == 0;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * kper;
    const int k1 = min(nk, k0 + kper);
    if (leader) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (leader) {
        for (int q = 0; q < 2 && k0 + q < k1; ++q)
            tma_load_plane(&tmap, stage0 + q * (uint32_t)stage, bar0 + 8 * q, i0, j0, k0 + q, box_bytes);
    }
    uint32_t phases = 0u;  // bit q: parity to wait for on stage q
    for (int k = k0; k < k1; ++k) {
        const int sidx = (k - k0) & 1;
        const bool landed = mbar_wait(bar0 + 8 * sidx, (phases >> sidx) & 1u, polls);
        // a CTA that gives up: drain its copies in flight, flag, leave together
        auto give_up = [&]() {
            if (leader) {
                mbar_wait(bar0 + 8 * sidx, (phases >> sidx) & 1u, kDefaultWaitPolls);
                if (k + 1 < k1) mbar_wait(bar0 + 8 * (sidx ^ 1), (phases >> (sidx ^ 1)) & 1u, kDefaultWaitPolls);
                *(volatile int*)status = 1;
                __threadfence_system();
            }
            __syncthreads();
        };
        phases ^= 1u << sidx;
        // s_in(r, c) <-> global (i0 - 2 + c, j0 - 2 + r)
        const S* s_land = reinterpret_cast<const S*>(smem_tma + sidx * stage) + off;
        const T* s_in;
        if constexpr (M::CONV) {
            for (int r = ty; r < TY + 4; r += NTY)
                for (int c = tx; c < TX + 4; c += TX) s_conv[r * BX + c] = cvt<C, S>(s_land[r * BX + c]);
            if (__syncthreads_or(!landed)) {
                phases ^= 1u << sidx;  // the drain waits on the phase not yet seen
                give_up();
                return;
            }
            s_in = s_conv;
        } else {
            s_in = s_land;
        }

        // lap at local (ii, jj) <-> global (i0-1+ii, j0-1+jj)
        for (int jj = ty; jj < TY + 2; jj += NTY) {
            for (int ii = tx; ii < WL; ii += TX) {
                const T* c = s_in + (jj + 1) * BX + ii + 1;
                const C sum = X::add(X::add(X::add(cvt<C, T>(c[1]), cvt<C, T>(c[-1]), site<0>{}), cvt<C, T>(c[BX]),
                                            site<1>{}),
                                     cvt<C, T>(c[-BX]), site<2>{});
                s_lap[jj * WL + ii] = X::sub(A::template scale2<2>(cvt<C, T>(c[0])), sum, site<3>{});
            }
        }
        if constexpr (M::CONV) {
            __syncthreads();
        } else if (__syncthreads_or(!landed)) {
            phases ^= 1u << sidx;  // the drain waits on the phase not yet seen
            give_up();
            return;
        }
        for (int jj = ty; jj < TY; jj += NTY) {
            for (int ii = tx; ii < WF; ii += TX) {
                const C* l = s_lap + (jj + 1) * WL + ii;
                const T* x = s_in + (jj + 2) * BX + ii + 1;
                s_flx[jj * WF + ii] = A::limit(X::sub(l[1], l[0], site<4>{}), cvt<C, T>(x[1]), cvt<C, T>(x[0]));
            }
        }
        for (int jj = ty; jj < TY + 1; jj += NTY) {
            for (int ii = tx; ii < WY; ii += TX) {
                const C* l = s_lap + jj * WL + ii + 1;
                const T* x = s_in + (jj + 1) * BX + ii + 2;
                s_fly[jj * WY + ii] = A::limit(X::sub(l[WL], l[0], site<5>{}), cvt<C, T>(x[BX]), cvt<C, T>(x[0]));
            }
        }
        __syncthreads();
        const int gi = i0 + tx;
        for (int jj = ty; jj < TY; jj += NTY) {
            const int gj = j0 + jj;
            if (gi < ni && gj < nj) {
                const C fx1 = s_flx[jj * WF + tx + 1], fx0 = s_flx[jj * WF + tx];
                const C fy1 = s_fly[(jj + 1) * WY + tx], fy0 = s_fly[jj * WY + tx];
                const C x = cvt<C, T>(s_in[(jj + 2) * BX + tx + 2]);
                const int64_t o = (int64_t)k * sk + (int64_t)gi + (int64_t)gj * sj;
                const C cf = ld<C, S>(coeff + o);
                const C div = X::sub(X::add(X::sub(fx1, fx0, site<6>{}), fy1, site<7>{}), fy0, site<8>{});
                st<S, C>(out + o, X::sub(x, X::mul(cf, div, site<9>{}), site<10>{}));
            }
        }
        __syncthreads();  // stage sidx and the lap/flux buffers are free again
        if (leader && k + 2 < k1) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            tma_load_plane(&tmap, stage0 + sidx * (uint32_t)stage, bar0 + 8 * sidx, i0, j0, k + 2, box_bytes);
        }
    }
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        cudaGetLastError();
    });
    return fn;
}

template <class S>
CUtensorMapDataType tma_type() {
    if constexpr (sizeof(S) == 8) return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    else if constexpr (sizeof(S) == 4) return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    else return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
}

// TMA launch if the layout qualifies (i unit-stride, j/k strides multiples
// of 16 bytes, tile rows within the 256-row box limit); SB_ERR_UNSUPPORTED
// (no error text) if not.
template <class S, class C, int TX, int NTY, uint32_t PL>
int launch_tma(const void* inp, const void* coeff, void* out, int64_t ni, int64_t nj, int64_t nk, int64_t si,
               int64_t sj, int64_t sk, int ty, int kper, cudaStream_t stream, const DeviceProps* p) {
    constexpr int ES = (int)sizeof(S), PADX = TmaSmem<S, C>::PADX;
    static_assert(((TX + PADX) * ES) % 16 == 0 && (TX * ES) % 16 == 0 && PADX >= 4 + 16 / ES - 1,
                  "TMA box rows and x offsets must be 16-byte multiples covering the halo at any offset");
    if (si != 1 || sj <= 0 || sk <= 0 || (sj * ES) % 16 || (sk * ES) % 16) return SB_ERR_UNSUPPORTED;
    if (ty < NTY || ty + 4 > 256 || ni + 4 + 16 > (1LL << 31) || nj + 4 > (1LL << 31)) return SB_ERR_UNSUPPORTED;
    // The 16-byte boundary at or below the halo corner: the bytes between it
    // and the corner share the corner's 16-byte block, so reading them is safe.
    const uintptr_t corner = (uintptr_t)((const S*)inp - 2 - 2 * sj);
    if (corner % ES) return SB_ERR_UNSUPPORTED;
    const int off = (int)((corner & 15) / ES);
    const void* base = (const void*)(corner - (corner & 15));
    auto encode = tensor_map_encoder();
    if (!encode) return SB_ERR_UNSUPPORTED;
    CUtensorMap tmap;
    const cuuint64_t dims[3] = {(cuuint64_t)(ni + 4 + off), (cuuint64_t)(nj + 4), (cuuint64_t)nk};
    const cuuint64_t strides[2] = {(cuuint64_t)(sj * ES), (cuuint64_t)(sk * ES)};
    const cuuint32_t box[3] = {(cuuint32_t)(TX + PADX), (cuuint32_t)(ty + 4), 1};
    const cuuint32_t estride[3] = {1, 1, 1};
    const CUresult cr = encode(&tmap, tma_type<S>(), 3, const_cast<void*>(base), dims, strides, box, estride,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return SB_ERR_UNSUPPORTED;
    const size_t smem = TmaSmem<S, C>::bytes(TX, ty);
    SB_CHECK((int64_t)smem <= p->smem_optin, SB_ERR_INVALID, "hdiff TMA tile %dx%d needs %zu bytes of shared memory",
             TX, ty, smem);
    auto kernel = hdiff_tma_kernel<S, C, TX, NTY, PL>;
    if (smem > 48 * 1024) SB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t gx = ceil_div(ni, TX), gy = ceil_div(nj, ty), gz = ceil_div(nk, kper);
    SB_CHECK(gy <= p->max_grid_y && gz <= p->max_grid_z, SB_ERR_INVALID, "hdiff grid too large");
    int* status = nullptr;
    const int rc = status_word(&status);
    if (rc) return rc;
    t_tma_used = true;
    kernel<<<dim3((unsigned)gx, (unsigned)gy, (unsigned)gz), dim3(TX, NTY), smem, stream>>>(
        tmap, (const S*)coeff, (S*)out, (int)ni, (int)nj, (int)nk, sj, sk, ty, kper, off, wait_polls(), status);
    return SB_OK;
}

// Integer-pipe placements of the float64 TMA tile's operation sites (bit K =
// site K of hdiff_tma_kernel: 0-2 the Laplacian's neighbour sum, 3 its
// 4*inp - sum, 4/5 the flux differences, 6-8 the flux divergence, 9 the
// coefficient product, 10 the update).  sb_tune.flags bits 4-7 pick one:
// 0 the default, 1 every site on the fp64 pipe, 2.. the mixes below; shapes
// other than the 128 x 4 tile always use the default.
constexpr uint32_t kTmaPlacements[] = {
    0u,
    0u,
    1u << 9,
    (1u << 9) | (1u << 6) | (1u << 7) | (1u << 8),
    (1u << 9) | (1u << 6) | (1u << 7) | (1u << 8) | (1u << 10),
    (1u << 9) | (1u << 0) | (1u << 1) | (1u << 2) | (1u << 3),
    (1u << 9) | (1u << 0) | (1u << 1) | (1u << 6) | (1u << 7),
    (1u << 9) | (1u << 0) | (1u << 1) | (1u << 2) | (1u << 6) | (1u << 7) | (1u << 8),
    (1u << 9) | (1u << 0) | (1u << 1) | (1u << 2) | (1u << 3) | (1u << 6) | (1u << 7) | (1u << 8) | (1u << 10),
};
// Measured at 512x512x80 fp64: 561 us with every site on the fp64 pipe;
// every mix above is slower (600-1269 us): the tile's phases are separated by
// block barriers and each point's operations form one dependent chain, so the
// long integer sequences do not overlap the fp64 work.  The default keeps
// every site on the fp64 pipe.
constexpr int kTmaPlacementDefault = 1;
constexpr int kTmaPlacementCount = (int)(sizeof(kTmaPlacements) / sizeof(kTmaPlacements[0]));

template <class S, class C, int TX, int NTY>
int launch_tma_placed(int placement, const void* inp, const void* coeff, void* out, int64_t ni, int64_t nj,
                      int64_t nk, int64_t si, int64_t sj, int64_t sk, int ty, int kper, cudaStream_t stream,
                      const DeviceProps* p) {
    SB_CHECK(placement >= 0 && placement < kTmaPlacementCount, SB_ERR_INVALID,
             "hdiff TMA: placement preset %d out of range [0, %d)", placement, kTmaPlacementCount);
    constexpr uint32_t kDefault = kTmaPlacements[kTmaPlacementDefault];
    if constexpr (std::is_same<C, double>::value && TX == 128 && NTY == 4) {
#define SB_TMA_PL(Q)                                                                                          \
    if (placement == Q)                                                                                       \
        return launch_tma<S, C, TX, NTY, kTmaPlacements[Q]>(inp, coeff, out, ni, nj, nk, si, sj, sk, ty, kper,   \
                                                           stream, p);
        SB_TMA_PL(1)
        SB_TMA_PL(2)
        SB_TMA_PL(3)
        SB_TMA_PL(4)
        SB_TMA_PL(5)
        SB_TMA_PL(6)
        SB_TMA_PL(7)
        SB_TMA_PL(8)
#undef SB_TMA_PL
    }
    return launch_tma<S, C, TX, NTY, std::is_same<C, double>::value ? kDefault : 0u>(
        inp, coeff, out, ni, nj, nk, si, sj, sk, ty, kper, stream, p);
}

template <class S, class C>
int launch_typed(const void* inp, const void* coeff, void* out, int64_t ni, int64_t nj, int64_t nk,
                 int64_t si, int64_t sj, int64_t sk, const sb_tune* tune, cudaStream_t stream) {
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    int variant = tune ? tune->variant : SB_VARIANT_AUTO;
    const int placement = tune ? (tune->flags >> 4) & 15 : 0;
    // fp64 compute is bound by the fp64 pipe: TILE computes every lap/flx/fly
    // once per tile (fewest fp64 operations); fp32 and float-pair compute are
    // bound by instruction issue: JSCAN (shuffles, no block barriers) is faster.
    // With float64 storage too, the TMA-staged tile is faster still (its
    // loads leave the issue slots to the fp64 arithmetic and overlap the
    // previous plane's compute); it needs TMA-describable strides, else TILE.
    // 128 x 4 threads, 16-row tiles, one k-plane per block at 512x512x80:
    // 550 us, 560 with 2 planes, 566 with 4; 8- and 12-row tiles 552-582,
    // 24 and 32 rows 652-716 (two blocks per SM no longer fit).
    const bool auto_tile = variant == SB_VARIANT_AUTO && std::is_same<C, double>::value;
    if constexpr (std::is_same<S, double>::value && std::is_same<C, double>::value) {
        if (variant == SB_VARIANT_AUTO) {
            const int rc_tma =
                launch_tma_placed<S, C, 128, 4>(placement, inp, coeff, out, ni, nj, nk, si, sj, sk, 16, 1, stream, p);
            if (rc_tma != SB_ERR_UNSUPPORTED) return rc_tma;
        }
    }
    // bfloat16 storage, float-pair and float32 compute: vector strips (V
    // columns per lane) issue fewer instructions per point than JSCAN (56 vs
    // 62 us, 271 vs 313 us and, with V = 2, 51 vs 53 us at 512x512x80).
    if constexpr (std::is_same<S, bf16>::value || std::is_same<C, f32x2>::value) {
        if (variant == SB_VARIANT_AUTO) {
            constexpr int V = sizeof(S) == 8 ? 2 : 4;
            const int rc_v = launch_vscan<S, C, V>(inp, coeff, out, ni, nj, nk, si, sj, sk, 1, 16, 1, 1, stream, p);
            if (rc_v != SB_ERR_UNSUPPORTED) return rc_v;
        }
    }
    if constexpr (std::is_same<S, float>::value && std::is_same<C, float>::value) {
        if (variant == SB_VARIANT_AUTO) {
            const int rc_v = launch_vscan<S, C, 2>(inp, coeff, out, ni, nj, nk, si, sj, sk, 2, 16, 1, 4, stream, p);
            if (rc_v != SB_ERR_UNSUPPORTED) return rc_v;
        }
    }
    if (variant == SB_VARIANT_AUTO) variant = auto_tile ? SB_HDIFF_TILE : SB_HDIFF_JSCAN;
    if constexpr (std::is_same<C, fix64>::value) {
        SB_CHECK(variant == SB_HDIFF_JSCAN, SB_ERR_UNSUPPORTED, "fixed-point hdiff runs as JSCAN strips only");
    }
    SB_CHECK(variant == SB_HDIFF_TILE || variant == SB_HDIFF_JSCAN || variant == SB_HDIFF_TMA ||
                 variant == SB_HDIFF_VSCAN,
             SB_ERR_UNSUPPORTED, "hdiff variant %d is not available", variant);
    if (variant == SB_HDIFF_TMA) {
        if constexpr (std::is_same<C, fix64>::value) {
            return fail(SB_ERR_UNSUPPORTED, "fixed-point hdiff runs as JSCAN strips only");
        } else {
            const int bx = (tune && tune->block_x > 0) ? tune->block_x : 64;
            const int by = (tune && tune->block_y > 0) ? tune->block_y : 4;
            const int ty = (tune && tune->tile_y > 0) ? tune->tile_y : 16;
            const int kper = (tune && tune->k_per_cta > 0) ? tune->k_per_cta : 8;
            int rc2 = SB_ERR_UNSUPPORTED;
#define SB_TMA_CASE(TXV, NTYV)                                                                               \
    if (bx == TXV && by == NTYV)                                                                              \
        rc2 = launch_tma_placed<S, C, TXV, NTYV>(placement, inp, coeff, out, ni, nj, nk, si, sj, sk, ty, kper, stream, p);
            SB_TMA_CASE(32, 8)
            SB_TMA_CASE(64, 4)
            SB_TMA_CASE(64, 8)
            SB_TMA_CASE(128, 2)
            SB_TMA_CASE(128, 4)
#undef SB_TMA_CASE
            SB_CHECK(rc2 != SB_ERR_UNSUPPORTED, SB_ERR_UNSUPPORTED,
                     "hdiff TMA: needs blocks 32x8, 64x{4,8} or 128x{2,4}, i unit-stride, 16-byte aligned j/k "
                     "strides and halo corner, tile rows in [block_y, 252]");
            return rc2;
        }
    }
    if (variant == SB_HDIFF_VSCAN) {
        if constexpr (std::is_same<C, fix64>::value) {
            return fail(SB_ERR_UNSUPPORTED, "fixed-point hdiff runs as JSCAN strips only");
        } else {
            const int nw = (tune && tune->block_y > 0) ? tune->block_y : 4;
            const int ty = (tune && tune->tile_y > 0) ? tune->tile_y : 32;
            const int kper = (tune && tune->k_per_cta > 0) ? tune->k_per_cta : 1;
            const int unroll = (tune && tune->unroll > 0) ? tune->unroll : 4;
            constexpr int VDEF = (int)(16 / sizeof(S)) > 4 ? 4 : (int)(16 / sizeof(S));
            const int width = (tune && tune->block_x > 0) ? tune->block_x : 32 * VDEF;
            int rc2 = SB_ERR_UNSUPPORTED;
            bool shape_ok = false;
            if constexpr (sizeof(S) == 8) {
                if (width == 64) {
                    shape_ok = true;
                    rc2 = launch_vscan<S, C, 2>(inp, coeff, out, ni, nj, nk, si, sj, sk, nw, ty, kper, unroll, stream, p);
                }
            } else if constexpr (sizeof(S) == 4) {
                if (width == 64 || width == 128) shape_ok = true;
                if (width == 64)
                    rc2 = launch_vscan<S, C, 2>(inp, coeff, out, ni, nj, nk, si, sj, sk, nw, ty, kper, unroll, stream, p);
                if (width == 128)
                    rc2 = launch_vscan<S, C, 4>(inp, coeff, out, ni, nj, nk, si, sj, sk, nw, ty, kper, unroll, stream, p);
            } else {
                if (width == 128 || width == 256) shape_ok = true;
                if (width == 128)
                    rc2 = launch_vscan<S, C, 4>(inp, coeff, out, ni, nj, nk, si, sj, sk, nw, ty, kper, unroll, stream, p);
                if (width == 256)
                    rc2 = launch_vscan<S, C, 8>(inp, coeff, out, ni, nj, nk, si, sj, sk, nw, ty, kper, unroll, stream, p);
            }
            SB_CHECK(shape_ok, SB_ERR_INVALID,
                     "hdiff vscan strip width (block_x) must be 64 for 8-byte, 64 or 128 for 4-byte and 128 or 256 "
                     "for 2-byte storage (got %d)", width);
            SB_CHECK(rc2 != SB_ERR_UNSUPPORTED, SB_ERR_UNSUPPORTED,
                     "hdiff VSCAN: needs i unit-stride, j/k strides that are multiples of the %d-column vector and "
                     "inp/coeff/out at the same offset from a vector boundary", width / 32);
            return rc2;
        }
    }
    if (variant == SB_HDIFF_JSCAN) {
        // fixed-point strips: one warp per block (512x512x80: 176 us, 191 us with 4)
        const int nw = (tune && tune->block_y > 0) ? tune->block_y : (std::is_same<C, fix64>::value ? 1 : 4);
        const int ty = (tune && tune->tile_y > 0) ? tune->tile_y : 32;
        const int kper = (tune && tune->k_per_cta > 0) ? tune->k_per_cta : 1;
        const int unroll = (tune && tune->unroll > 0) ? tune->unroll : 4;
        SB_CHECK(!tune || tune->block_x == 0 || tune->block_x == 32, SB_ERR_INVALID,
                 "hdiff jscan uses one warp (block_x = 32) per strip");
        return launch_jscan<S, C>(inp, coeff, out, ni, nj, nk, si, sj, sk, nw, ty, kper, unroll, stream, p);
    }
    if constexpr (std::is_same<C, fix64>::value) {
        return SB_ERR_UNSUPPORTED;
    } else {
    const int bx = (tune && tune->block_x > 0) ? tune->block_x : (auto_tile ? 128 : 64);
    const int by = (tune && tune->block_y > 0) ? tune->block_y : 4;
    int ty = (tune && tune->tile_y > 0) ? tune->tile_y : 16;
    int kper = (tune && tune->k_per_cta > 0) ? tune->k_per_cta : 4;
    SB_CHECK(ty >= by && ty <= 256, SB_ERR_INVALID, "tile_y must be in [block_y, 256]");
#define SB_HDIFF_CASE(TXV, NTYV)                                                            \
    if (bx == TXV && by == NTYV)                                                            \
        return launch_tile<S, C, TXV, NTYV>(inp, coeff, out, ni, nj, nk, si, sj, sk, ty, kper, stream, p);
    SB_HDIFF_CASE(32, 4)
    SB_HDIFF_CASE(32, 8)
    SB_HDIFF_CASE(64, 2)
    SB_HDIFF_CASE(64, 4)
    SB_HDIFF_CASE(64, 8)
    SB_HDIFF_CASE(128, 2)
    SB_HDIFF_CASE(128, 4)
#undef SB_HDIFF_CASE
    return fail(SB_ERR_UNSUPPORTED,
                "hdiff block (%d, %d) not instantiated; use 32x{4,8}, 64x{2,4,8} or 128x{2,4}", bx, by);
    }
}

}  // namespace
}  // namespace sb

using namespace sb;

extern "C" int sb_hdiff(int storage, int compute, const void* inp, const void* coeff, void* out,
                        int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
                        const sb_tune* tune, void* stream, double* time_s) {
    clear_error();
    int rc = check_domain(ni, nj, nk, si, sj, sk);
    if (rc) return rc;
    SB_CHECK(inp && coeff && out, SB_ERR_INVALID, "NULL field pointer");
    SB_CHECK((storage == SB_F64 && (compute == SB_F64 || compute == SB_F32X2 || compute == SB_FIX64)) ||
                 (storage == SB_F32 && (compute == SB_F32 || compute == SB_F64)) ||
                 (storage == SB_BF16 && compute == SB_F32),
             SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
    if (ni == 0 || nj == 0 || nk == 0) {
        if (time_s) *time_s = 0.0;
        return SB_OK;
    }
    // a give-up of an earlier launch is reported before anything new runs
    rc = take_wait_status();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    t_tma_used = false;
    rc = timed(s, time_s, [&]() {
        if (storage == SB_F64 && compute == SB_F64)
            return launch_typed<double, double>(inp, coeff, out, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F64 && compute == SB_F32X2)
            return launch_typed<double, f32x2>(inp, coeff, out, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F64 && compute == SB_FIX64)
            return launch_typed<double, fix64>(inp, coeff, out, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F32 && compute == SB_F32)
            return launch_typed<float, float>(inp, coeff, out, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_F32 && compute == SB_F64)
            return launch_typed<float, double>(inp, coeff, out, ni, nj, nk, si, sj, sk, tune, s);
        if (storage == SB_BF16 && compute == SB_F32)
            return launch_typed<bf16, float>(inp, coeff, out, ni, nj, nk, si, sj, sk, tune, s);
        return fail(SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
    });
    if (rc == SB_OK && time_s && t_tma_used) rc = take_wait_status();
    return rc;
}
