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
// Laplacian march defaults: rows per strip, warps per block, k-planes per thread
constexpr int kLapRows = 4;
constexpr int kLapWarps = 4;
constexpr int kLapPlanes = 2;
// which Laplacian kernel runs when the tune names none
constexpr int kLapDefaultVariant = SB_BASIC_MARCH;

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

// Laplacian by row strips: lanes along i, warps of a block along k; each
// thread takes a strip of R rows of j for PK k-planes, loads the strip's rows
// (and, along j, the row before and after it) into registers at once so that
// all its loads are in flight together, then computes the R rows.  Each input
// row is read once per strip plus the two rows beyond it; the i-neighbours are
// loads of rows already fetched (L1 hits).  Same operations in the same order
// as basic_point; PL places the float64 subtractions/additions (sites 0-7) on
// the integer pipe.
template <int MASK, class S, class C, int R, int PK, uint32_t PL>
__global__ void __launch_bounds__(256) lap_march_kernel(const S* __restrict__ inp, S* __restrict__ out, int ni,
                                                        int nj, int nk, int64_t si, int64_t sj, int64_t sk) {
    constexpr bool JN = (MASK & 2) != 0;
    using A = Ar<C>;
    using X = Mix<C, PL>;
    constexpr int NR = JN ? R + 2 : R;  // rows held: j0-1 .. j0+R along j, else j0 .. j0+R-1
    constexpr int R0 = JN ? 1 : 0;      // index of row j0 in v[]
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j0 = blockIdx.y * R;
    const int kb = (blockIdx.z * blockDim.y + threadIdx.y) * PK;
    if (i >= ni || kb >= nk) return;
    const int nrow = min(R, nj - j0);  // rows of this strip inside the domain
    const S* col = inp + (int64_t)i * si + (int64_t)kb * sk + (int64_t)j0 * sj;
    S* ocol = out + (int64_t)i * si + (int64_t)kb * sk + (int64_t)j0 * sj;
    C v[PK][NR];
#pragma unroll
    for (int q = 0; q < PK; ++q) {
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            // rows j0 - R0 + r up to j0 + nrow (the row after the strip, halo at the edge)
            v[q][r] = (kb + q < nk && r - R0 <= nrow - (JN ? 0 : 1))
                          ? ld<C, S>(col + (int64_t)(r - R0) * sj + (int64_t)q * sk)
                          : C(0);
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if (r < nrow) {
#pragma unroll
            for (int q = 0; q < PK; ++q) {
                if (kb + q < nk) {
                    const S* p = col + (int64_t)r * sj + (int64_t)q * sk;
                    const C two_x = A::template scale2<1>(v[q][r + R0]);
                    C acc = C(0);
                    bool first = true;
                    if (MASK & 1) {
                        const C t = X::sub(X::sub(two_x, ld<C, S>(p + si), site<0>{}), ld<C, S>(p - si), site<1>{});
                        acc = plus_zero<C>(t);
                        first = false;
                    }
                    if (MASK & 2) {
                        const C t = X::sub(X::sub(two_x, v[q][r + 2], site<2>{}), v[q][r], site<3>{});
                        acc = first ? plus_zero<C>(t) : X::add(acc, t, site<4>{});
                        first = false;
                    }
                    if (MASK & 4) {
                        const C t = X::sub(X::sub(two_x, ld<C, S>(p + sk), site<5>{}), ld<C, S>(p - sk), site<6>{});
                        acc = first ? plus_zero<C>(t) : X::add(acc, t, site<7>{});
                    }
                    st<S, C>(ocol + (int64_t)r * sj + (int64_t)q * sk, acc);
                }
            }
        }
    }
}

// float64 placements of the along-x-and-y strips (sites 0-4), by preset: 1 all
// fp64, 2 the closing addition, 3 the second subtraction of each axis, 4 both
// of those and the addition (0 selects the default preset)
constexpr uint32_t kLapPlacements[] = {0u, 0u, 0x10u, 0x0Au, 0x1Au};
constexpr int kLapPlacementDefault = 1;

template <int MASK, class S, class C, int R, int PK>
int launch_lap_march_pl(int placement, const S* inp, S* out, int64_t ni, int64_t nj, int64_t nk, int64_t si,
                        int64_t sj, int64_t sk, int warps, cudaStream_t stream) {
    const dim3 block(32, warps);
    const int64_t gz = ceil_div(nk, (int64_t)warps * PK);
    const dim3 grid((unsigned)ceil_div(ni, (int64_t)32), (unsigned)ceil_div(nj, (int64_t)R), (unsigned)gz);
    auto go = [&](auto kernel) {
        kernel<<<grid, block, 0, stream>>>(inp, out, (int)ni, (int)nj, (int)nk, si, sj, sk);
        return SB_OK;
    };
    if constexpr (MASK == 3 && std::is_same<C, double>::value) {
        switch (placement) {
            case 2: return go(lap_march_kernel<MASK, S, C, R, PK, kLapPlacements[2]>);
            case 3: return go(lap_march_kernel<MASK, S, C, R, PK, kLapPlacements[3]>);
            case 4: return go(lap_march_kernel<MASK, S, C, R, PK, kLapPlacements[4]>);
            default: break;
        }
    }
    return go(lap_march_kernel<MASK, S, C, R, PK, 0u>);
}

template <int MASK, class S, class C>
int launch_lap_march_shape(int rows, int pk, int placement, const S* inp, S* out, int64_t ni, int64_t nj,
                           int64_t nk, int64_t si, int64_t sj, int64_t sk, int warps, cudaStream_t stream) {
    if (pk == 2 && rows == 4)
        return launch_lap_march_pl<MASK, S, C, 4, 2>(placement, inp, out, ni, nj, nk, si, sj, sk, warps, stream);
    if (pk == 2 && rows == 8)
        return launch_lap_march_pl<MASK, S, C, 8, 2>(placement, inp, out, ni, nj, nk, si, sj, sk, warps, stream);
    return fail(SB_ERR_INVALID, "Laplacian strips: 4 or 8 rows x 2 k-planes per thread (got %d x %d)", rows, pk);
}

template <class S, class C>
int launch_lap_march(const void* inp, void* out, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj,
                     int64_t sk, int mask, const sb_tune* tune, cudaStream_t stream) {
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    const int rows = (tune && tune->tile_y > 0) ? tune->tile_y : kLapRows;
    const int warps = (tune && tune->block_y > 0) ? tune->block_y : kLapWarps;
    const int pk = (tune && tune->k_per_cta > 0) ? tune->k_per_cta : kLapPlanes;
    const int placement = tune ? ((tune->flags >> 4) & 15) : 0;
    SB_CHECK(warps >= 1 && warps <= 8, SB_ERR_INVALID, "Laplacian strips: 1 to 8 warps per block (got %d)", warps);
    SB_CHECK(placement >= 0 && placement < (int)(sizeof(kLapPlacements) / sizeof(kLapPlacements[0])),
             SB_ERR_INVALID, "Laplacian placement preset %d out of range", placement);
    SB_CHECK(ceil_div(nj, (int64_t)rows) <= p->max_grid_y &&
                 ceil_div(nk, (int64_t)warps * pk) <= p->max_grid_z,
             SB_ERR_INVALID, "domain too large for the Laplacian strip grid");
    const S* in = (const S*)inp;
    S* o = (S*)out;
    const int pl = placement == 0 ? kLapPlacementDefault : placement;
    switch (mask) {
#define SB_LAP_MASK(M) \
    case M: return launch_lap_march_shape<M, S, C>(rows, pk, pl, in, o, ni, nj, nk, si, sj, sk, warps, stream);
        SB_LAP_MASK(1)
        SB_LAP_MASK(2)
        SB_LAP_MASK(3)
        SB_LAP_MASK(4)
        SB_LAP_MASK(5)
        SB_LAP_MASK(6)
        SB_LAP_MASK(7)
#undef SB_LAP_MASK
    }
    return fail(SB_ERR_INVALID, "along_mask must be in [1, 7] for the Laplacian strips");
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
    if constexpr (OP == OP_LAP) {
        const int variant = (tune && tune->variant > 0) ? tune->variant : kLapDefaultVariant;
        SB_CHECK(variant == SB_BASIC_POINT || variant == SB_BASIC_MARCH, SB_ERR_INVALID,
                 "Laplacian variant must be %d (point) or %d (row march)", SB_BASIC_POINT, SB_BASIC_MARCH);
        if (variant == SB_BASIC_MARCH && mask != 0) {
            if (storage == SB_F64 && compute == SB_F64)
                return launch_lap_march<double, double>(inp, out, ni, nj, nk, si, sj, sk, mask, tune, stream);
            if (storage == SB_F32 && compute == SB_F32)
                return launch_lap_march<float, float>(inp, out, ni, nj, nk, si, sj, sk, mask, tune, stream);
            if (storage == SB_F32 && compute == SB_F64)
                return launch_lap_march<float, double>(inp, out, ni, nj, nk, si, sj, sk, mask, tune, stream);
            if (storage == SB_BF16 && compute == SB_F32)
                return launch_lap_march<bf16, float>(inp, out, ni, nj, nk, si, sj, sk, mask, tune, stream);
            return fail(SB_ERR_UNSUPPORTED, "unsupported storage/compute combination (%d, %d)", storage, compute);
        }
    }
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
