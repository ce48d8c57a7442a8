// Batched execution: many hdiff / vadv domains of uneven size in one graph
// launch of persistent kernels that pull work from device-side queues.
//
// One graph (captured on the first launch, replayed afterwards):
//     copy the domain table from pinned host memory -> zero the queue counters
//       -> fork:  hdiff kernel            (queue 0)
//                 vadv kernel, nk bucket 0 (queue 1)
//                 ...                      (one per bucket)
//       -> join
// Kernels of different branches run concurrently on the GPU, so the long
// serial vadv columns overlap the bandwidth-bound hdiff strips.
//
// hdiff: persistent warps; an item is a strip of 28 output columns x `rows`
//   rows x `planes` k-planes of one domain (stencil_core.cuh:
//   hdiff_jscan_strip).  A warp takes the next item with one atomicAdd and
//   finds its domain by binary search over first-item offsets staged in
//   shared memory.
// vadv: persistent blocks of BT threads; an item is BT consecutive columns of
//   one j-row of one domain, one column per thread (stencil_core.cuh:
//   vadv_async_column: cp.async-staged inputs).  Factors live in shared memory
//   for float32 storage and arithmetic, otherwise in a slab workspace per
//   bucket (per thread slot, level stride = the bucket's thread count), which
//   frees shared memory for more blocks per SM.  Domains are grouped into 8 nk
//   buckets (caps max_nk/8, 2*max_nk/8, ...) and each bucket's kernel and slab
//   are sized for its cap, so short columns do not pay for the tallest one.
// No kernel waits on another warp or kernel: every queue is one atomic counter.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "stencil_core.cuh"

namespace sb {
namespace {

constexpr int kMaxBatchDomains = 1024;
constexpr int kBuckets = 8;
constexpr int kVadvDepth = 4;

struct DevDomain {
    int32_t op;  // SB_OP_HDIFF / SB_OP_VADV
    int32_t ni, nj, nk;
    int64_t si, sj, sk, wsh;
    const void* f[5];
    void* out;
    int64_t item_begin;  // first item of this domain in its queue
    int32_t items_i, items_j;
    int32_t kp;  // vadv: level stride 0 (1) or 8 (2) modulo 16 bytes, else 0 (TMEM staging shortcuts)
    int32_t pad;
};

struct DevTable {
    int32_t ndomains, n_hdiff;
    int32_t rows, planes;
    int64_t hdiff_items;
    int32_t bucket_first[kBuckets + 1];  // vadv bucket b: domains [bucket_first[b], bucket_first[b+1])
    int32_t pad;
    int64_t bucket_items[kBuckets];
    DevDomain dom[1];  // ndomains entries: hdiff first, then vadv by bucket
};

size_t table_bytes(int n) { return offsetof(DevTable, dom) + sizeof(DevDomain) * (size_t)(n > 0 ? n : 1); }

template <class S, class C, int U, class IDX>
__global__ void __launch_bounds__(256)
    batch_hdiff_kernel(const DevTable* __restrict__ tab, unsigned long long* __restrict__ counter) {
    __shared__ int64_t s_begin[kMaxBatchDomains + 1];
    const int nd = tab->n_hdiff;
    const int64_t total = tab->hdiff_items;
    if (total == 0) return;
    const int rows = tab->rows, planes = tab->planes;
    for (int d = threadIdx.x; d < nd; d += blockDim.x) s_begin[d] = tab->dom[d].item_begin;
    if (threadIdx.x == 0) s_begin[nd] = total;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(counter, 1ULL);
        item = __shfl_sync(0xffffffffu, item, 0);
        if ((int64_t)item >= total) break;
        int lo = 0, hi = nd - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_begin[mid] <= (int64_t)item) lo = mid; else hi = mid - 1;
        }
        const DevDomain& dm = tab->dom[lo];
        const int64_t local = (int64_t)item - s_begin[lo];
        const int strip = (int)(local % dm.items_i);
        const int64_t rest = local / dm.items_i;
        const int jb = (int)(rest % dm.items_j);
        const int k0 = (int)(rest / dm.items_j) * planes;
        const int k1 = min(dm.nk, k0 + planes);
        const int i = strip * kJscanOut - 2 + lane;
        const int j0 = jb * rows;
        const int j1 = min(dm.nj, j0 + rows);
        for (int k = k0; k < k1; ++k) {
            hdiff_strip<S, C, U, IDX>((const S*)dm.f[0], (const S*)dm.f[1], (S*)dm.out, dm.ni, dm.nj,
                                            (IDX)dm.si, (IDX)dm.sj, (IDX)dm.sk, i, lane, j0, j1, k);
        }
    }
}

// Dynamic shared memory: ccol[cap][BT], dcol[cap][BT] (compute type), then the
// staging ring [D+1][6][BT] (RingOf<storage>) at ring_offset.  With SLAB the
// factors live in the bucket's slab workspace instead (level k of thread slot
// q at slab[k * nslots + q], dcol after cap * nslots ccol entries) and the
// shared memory is the ring only, so many more blocks fit per SM.
template <class S, class C, int BT, int D, class IDX, class P = C, bool SLAB = false, uint32_t PL = 0u>
__global__ void __launch_bounds__(BT)
    batch_vadv_kernel(const DevTable* __restrict__ tab, unsigned long long* __restrict__ counter, int bucket,
                      int cap, int ring_offset, P* __restrict__ slab) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_dom;
    __shared__ int64_t s_local;
    const int first = tab->bucket_first[bucket], last = tab->bucket_first[bucket + 1];
    const int64_t total = tab->bucket_items[bucket];
    if (total == 0) return;
    const int t = threadIdx.x;
    const int64_t nslots = (int64_t)gridDim.x * BT;
    P* sc = SLAB ? slab + (int64_t)blockIdx.x * BT + t : reinterpret_cast<P*>(smem_raw) + t;
    auto* ring = reinterpret_cast<typename RingOf<S>::T*>(smem_raw + ring_offset) + t;
    for (;;) {
        if (t == 0) {
            const int64_t item = (int64_t)atomicAdd(counter, 1ULL);
            int d = -1;
            if (item < total) {
                int lo = first, hi = last - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (tab->dom[mid].item_begin <= item) lo = mid; else hi = mid - 1;
                }
                d = lo;
                s_local = item - tab->dom[lo].item_begin;
            }
            s_dom = d;
        }
        __syncthreads();
        const int d = s_dom;
        if (d < 0) break;
        const DevDomain& dm = tab->dom[d];
        const int group = (int)(s_local % dm.items_i);
        const int j = (int)(s_local / dm.items_i);
        const int i = group * BT + t;
        if (i < dm.ni) {
            const IDX col = (IDX)i * (IDX)dm.si + (IDX)j * (IDX)dm.sj;
            if constexpr (SLAB) {
                vadv_async_column<S, C, BT, D, IDX, true, P, PL>((const S*)dm.f[0], (const S*)dm.f[1],
                                                             (const S*)dm.f[2], (const S*)dm.f[3],
                                                             (const S*)dm.f[4], (S*)dm.out, col, dm.nk,
                                                             (IDX)dm.sk, (IDX)dm.wsh, sc, sc + (int64_t)cap * nslots,
                                                             ring, (int)nslots);
            } else {
                vadv_async_column<S, C, BT, D, IDX, false, P>((const S*)dm.f[0], (const S*)dm.f[1],
                                                              (const S*)dm.f[2], (const S*)dm.f[3],
                                                              (const S*)dm.f[4], (S*)dm.out, col, dm.nk,
                                                              (IDX)dm.sk, (IDX)dm.wsh, sc, sc + dm.nk * BT, ring);
            }
        }
        __syncthreads();  // s_dom / s_local are rewritten by the next grab
    }
}

// float32-compute vadv with the factors in tensor memory (vadv_tmem_column):
// one persistent block of 4*G warps per SM and bucket; each warp takes
// 32-column items of the bucket's domains from the bucket queue.  Columns of
// TMEM per warp: cpw = 16 * ceil(cap / 8) for the bucket's largest nk.  The
// block allocates all 512 columns and the launch asks for enough shared
// memory that no other TMEM block shares its SM.
template <class S, int D>
__global__ void __launch_bounds__(512, 1)
    batch_vadv_tmem_kernel(const DevTable* __restrict__ tab, unsigned long long* __restrict__ counter, int bucket,
                           int cpw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int first = tab->bucket_first[bucket], last = tab->bucket_first[bucket + 1];
    const int64_t total = tab->bucket_items[bucket];
    if (total == 0) return;  // whole block, before any TMEM allocation
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
    for (;;) {
        unsigned long long item = 0;
        if (lane == 0) item = atomicAdd(counter, 1ULL);
        item = __shfl_sync(0xffffffffu, item, 0);
        if ((int64_t)item >= total) break;  // whole warp
        int lo = first, hi = last - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tab->dom[mid].item_begin <= (int64_t)item) lo = mid; else hi = mid - 1;
        }
        const DevDomain& dm = tab->dom[lo];
        const int64_t local = (int64_t)item - dm.item_begin;
        const int i0 = (int)(local % dm.items_i) * 32;
        const int j = (int)(local / dm.items_i);
        const int nvalid = min(32, dm.ni - i0);
        const int col0 = i0 + j * (int)dm.sj;
        if (dm.kp == 1)
            vadv_tmem_column<S, D, 1, int, true>((const S*)dm.f[0], (const S*)dm.f[1], (const S*)dm.f[2],
                                           (const S*)dm.f[3], (const S*)dm.f[4], (S*)dm.out, col0, lane, nvalid,
                                           dm.nk, (int)dm.sk, (int)dm.wsh, tcol, ring);
        else if (dm.kp == 2)
            vadv_tmem_column<S, D, 2, int, true>((const S*)dm.f[0], (const S*)dm.f[1], (const S*)dm.f[2],
                                           (const S*)dm.f[3], (const S*)dm.f[4], (S*)dm.out, col0, lane, nvalid,
                                           dm.nk, (int)dm.sk, (int)dm.wsh, tcol, ring);
        else
            vadv_tmem_column<S, D, 0, int>((const S*)dm.f[0], (const S*)dm.f[1], (const S*)dm.f[2],
                                           (const S*)dm.f[3], (const S*)dm.f[4], (S*)dm.out, col0, lane, nvalid,
                                           dm.nk, (int)dm.sk, (int)dm.wsh, tcol, ring);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0) {
        const uint32_t ncols = 512u;
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(ncols) : "memory");
    }
}
constexpr int kTmemDepth = 8;

struct Kinds {
    void (*hdiff)(dim3, dim3, cudaStream_t, const DevTable*, unsigned long long*);
    void (*vadv32)(dim3, dim3, size_t, cudaStream_t, const DevTable*, unsigned long long*, int, int, int, void*);
    void (*vadv64)(dim3, dim3, size_t, cudaStream_t, const DevTable*, unsigned long long*, int, int, int, void*);
    bool slab;  // vadv keeps its factors in a slab workspace
    const void* vadv32_fn;
    const void* vadv64_fn;
    int storage_bytes, compute_bytes;
    bool int_products;  // float64 slab buckets run their products in integer arithmetic
    int vadv_depth;     // levels of inputs the vadv ring keeps in flight
    // float32 vadv with factors in tensor memory (nullptr for other compute types)
    void (*vadv_tmem)(dim3, dim3, size_t, cudaStream_t, const DevTable*, unsigned long long*, int, int);
    const void* vadv_tmem_fn;
    int tmem_ring_bytes;  // staging ring per warp
};

template <class S, class C, int U, class IDX>
void run_hdiff(dim3 g, dim3 b, cudaStream_t s, const DevTable* t, unsigned long long* c) {
    batch_hdiff_kernel<S, C, U, IDX><<<g, b, 0, s>>>(t, c);
}
// ring depth of a bucket kernel: 1 for the float64 slabs with the integer
// split (as the single-domain kernel), kVadvDepth otherwise
template <uint32_t PL>
constexpr int kBucketDepth = PL != 0u ? 1 : kVadvDepth;

template <class S, class C, int BT, class IDX, class P, bool SLAB, uint32_t PL>
void run_vadv(dim3 g, dim3 b, size_t smem, cudaStream_t s, const DevTable* t, unsigned long long* c, int bucket,
              int cap, int ring_offset, void* slab) {
    batch_vadv_kernel<S, C, BT, kBucketDepth<PL>, IDX, P, SLAB, PL><<<g, b, smem, s>>>(t, c, bucket, cap,
                                                                                       ring_offset, (P*)slab);
}

template <class S>
void run_vadv_tmem(dim3 g, dim3 b, size_t smem, cudaStream_t s, const DevTable* t, unsigned long long* c,
                   int bucket, int cpw) {
    batch_vadv_tmem_kernel<S, kTmemDepth><<<g, b, smem, s>>>(t, c, bucket, cpw);
}

// hdiff computes in HC, vadv in VC with its recurrences in P
template <class S, class HC, class VC, int U, class IDX, class P = VC>
Kinds kinds_for() {
    Kinds k;
    // slab factors need ring entries of the factor size; for float32 storage
    // and arithmetic the shared-memory factors measured faster in batches
    constexpr bool SLAB = sizeof(typename RingOf<S>::T) == sizeof(P) &&
                          !(std::is_same<S, float>::value && std::is_same<P, float>::value);
    k.slab = SLAB;
    k.hdiff = &run_hdiff<S, HC, U, IDX>;
    // float64 slab buckets: the single-domain kernel's split between the fp64
    // and integer pipes (more blocks per SM, below)
    constexpr uint32_t PL = SLAB && std::is_same<P, double>::value && std::is_same<VC, double>::value
                                ? kVadvDefaultIntSites
                                : 0u;
    k.int_products = PL != 0u;
    k.vadv_depth = kBucketDepth<PL>;
    k.vadv32 = &run_vadv<S, VC, 32, IDX, P, SLAB, PL>;
    k.vadv64 = &run_vadv<S, VC, 64, IDX, P, SLAB, PL>;
    k.vadv32_fn = (const void*)&batch_vadv_kernel<S, VC, 32, kBucketDepth<PL>, IDX, P, SLAB, PL>;
    k.vadv64_fn = (const void*)&batch_vadv_kernel<S, VC, 64, kBucketDepth<PL>, IDX, P, SLAB, PL>;
    k.storage_bytes = sizeof(typename RingOf<S>::T);  // ring entry
    k.compute_bytes = sizeof(P);                      // factor entry
    if constexpr (std::is_same<VC, float>::value && std::is_same<P, float>::value && std::is_same<IDX, int>::value) {
        k.vadv_tmem = &run_vadv_tmem<S>;
        k.vadv_tmem_fn = (const void*)&batch_vadv_tmem_kernel<S, kTmemDepth>;
        k.tmem_ring_bytes = WarpRing<S, float, kTmemDepth>::BYTES;
    } else {
        k.vadv_tmem = nullptr;
        k.vadv_tmem_fn = nullptr;
        k.tmem_ring_bytes = 0;
    }
    return k;
}

bool pick_kinds(int storage, int compute, bool idx64, Kinds* out) {
#define SB_PICK(SC, CC, S, HC, VC, U, P)                                                            \
    if (storage == SC && compute == CC) {                                                           \
        *out = idx64 ? kinds_for<S, HC, VC, U, int64_t, P>() : kinds_for<S, HC, VC, U, int, P>();   \
        return true;                                                                                \
    }
    SB_PICK(SB_F64, SB_F64, double, double, double, 2, double)
    SB_PICK(SB_F64, SB_F32X2, double, f32x2, f32x2, 2, f32x2)
    SB_PICK(SB_F64, SB_FIX64, double, fix64, f32x2, 2, f32x2)  // fixed-point hdiff, float-pair vadv
    SB_PICK(SB_F32, SB_F32, float, float, float, 4, float)
    SB_PICK(SB_F32, SB_F64, float, double, double, 2, double)
    SB_PICK(SB_BF16, SB_F32, bf16, float, float, 4, float)
#undef SB_PICK
    return false;
}

}  // namespace
}  // namespace sb

using namespace sb;

struct sb_batch {
    int device = 0;
    int storage = 0, compute = 0;
    int max_domains = 0;
    int64_t max_nk = 0;
    sb_batch_tune tune{};
    int hdiff_grid = 0, hdiff_block = 0;
    int vadv_block = 32;
    int cap[kBuckets] = {};
    int vadv_grid[kBuckets] = {};
    size_t vadv_smem[kBuckets] = {};
    int ring_offset[kBuckets] = {};
    void* slab[kBuckets] = {};  // per-bucket factor slabs (inside slab_mem)
    void* slab_mem = nullptr;
    size_t slab_bytes = 0;
    bool idx64 = false;
    DevTable* host_table = nullptr;  // pinned
    DevTable* dev_table = nullptr;
    unsigned long long* counters = nullptr;  // [1 + kBuckets]
    cudaStream_t streams[1 + 1 + kBuckets] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t joins[1 + kBuckets] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_idx64 = false;
    int64_t total_items = 0;
    // float32 vadv in tensor memory: possible for this batch's form and tune,
    // used by the current domain set, used by the captured graph
    bool tmem_capable = false, use_tmem = false, graph_tmem = false;
    int tmem_block[kBuckets] = {}, tmem_cpw[kBuckets] = {};
    int vadv_tmem_grid = 0;
    size_t tmem_smem = 0;
};

namespace {

void release(sb_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto& s : b->streams)
        if (s) cudaStreamDestroy(s);
    if (b->fork) cudaEventDestroy(b->fork);
    for (auto& e : b->joins)
        if (e) cudaEventDestroy(e);
    if (b->counters) cudaFree(b->counters);
    if (b->slab_mem) cudaFree(b->slab_mem);
    if (b->dev_table) cudaFree(b->dev_table);
    if (b->host_table) cudaFreeHost(b->host_table);
    delete b;
}

size_t vadv_smem_bytes(int cap, int bt, int cbytes, int sbytes, int depth, int* ring_offset) {
    const size_t fac = ((2 * (size_t)cbytes * cap * bt) + 15) / 16 * 16;
    if (ring_offset) *ring_offset = (int)fac;
    return fac + (size_t)(depth + 1) * 6 * bt * sbytes;
}

int capture_graph(sb_batch* b) {
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    Kinds k;
    SB_CHECK(pick_kinds(b->storage, b->compute, b->idx64, &k), SB_ERR_UNSUPPORTED, "unsupported form");
    auto vadv_run = b->vadv_block == 64 ? k.vadv64 : k.vadv32;
    const void* vadv_fn = b->vadv_block == 64 ? k.vadv64_fn : k.vadv32_fn;
    for (int q = 0; q < kBuckets; ++q) {
        if (b->vadv_smem[q] > 48 * 1024)
            SB_CUDA(cudaFuncSetAttribute(vadv_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->vadv_smem[q]));
    }
    if (b->use_tmem)
        SB_CUDA(cudaFuncSetAttribute(k.vadv_tmem_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->tmem_smem));
    cudaStream_t s0 = b->streams[0];
    SB_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
    cudaMemcpyAsync(b->dev_table, b->host_table, table_bytes(b->max_domains), cudaMemcpyHostToDevice, s0);
    cudaMemsetAsync(b->counters, 0, sizeof(unsigned long long) * (1 + kBuckets), s0);
    cudaEventRecord(b->fork, s0);
    // order 0: hdiff first, then the vadv buckets; order 1: the vadv buckets
    // first (tallest first), so their blocks are resident before the hdiff
    // blocks take the remaining room of each SM
    const bool vadv_first = b->tune.order == 1;
    auto launch_hdiff = [&]() {
        cudaStreamWaitEvent(b->streams[1], b->fork, 0);
        k.hdiff(dim3(b->hdiff_grid), dim3(b->hdiff_block), b->streams[1], b->dev_table, b->counters);
        cudaEventRecord(b->joins[0], b->streams[1]);
    };
    if (!vadv_first) launch_hdiff();
    for (int qq = 0; qq < kBuckets; ++qq) {
        const int q = vadv_first ? kBuckets - 1 - qq : qq;
        cudaStreamWaitEvent(b->streams[2 + q], b->fork, 0);
        if (b->use_tmem)
            k.vadv_tmem(dim3(b->vadv_tmem_grid), dim3(b->tmem_block[q]), b->tmem_smem, b->streams[2 + q],
                        b->dev_table, b->counters + 1 + q, q, b->tmem_cpw[q]);
        else
            vadv_run(dim3(b->vadv_grid[q]), dim3(b->vadv_block), b->vadv_smem[q], b->streams[2 + q], b->dev_table,
                     b->counters + 1 + q, q, b->cap[q], b->ring_offset[q], b->slab[q]);
        cudaEventRecord(b->joins[1 + q], b->streams[2 + q]);
    }
    if (vadv_first) launch_hdiff();
    for (int q = 0; q < 1 + kBuckets; ++q) cudaStreamWaitEvent(s0, b->joins[q], 0);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s0, &graph);
    if (ec != cudaSuccess) {
        cudaGetLastError();
        return fail(SB_ERR_CUDA, "capturing the batch graph failed: %s", cudaGetErrorString(ec));
    }
    b->graph = graph;
    SB_CUDA(cudaGraphInstantiate(&b->exec, graph, 0));
    b->graph_idx64 = b->idx64;
    b->graph_tmem = b->use_tmem;
    return SB_OK;
}

}  // namespace

extern "C" {

int sb_batch_create(sb_batch** out, int storage, int compute, int max_domains, int64_t max_nk,
                    const sb_batch_tune* tune) {
    clear_error();
    SB_CHECK(out, SB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    Kinds k;
    SB_CHECK(pick_kinds(storage, compute, false, &k), SB_ERR_UNSUPPORTED,
             "unsupported storage/compute combination (%d, %d)", storage, compute);
    SB_CHECK(max_domains >= 1 && max_domains <= kMaxBatchDomains, SB_ERR_INVALID,
             "max_domains must be in [1, %d]", kMaxBatchDomains);
    SB_CHECK(max_nk >= 2 && max_nk <= (1 << 20), SB_ERR_INVALID, "max_nk must be in [2, 2^20]");
    const DeviceProps* p;
    int rc = device_props(&p);
    if (rc) return rc;
    sb_batch* b = new sb_batch();
    b->device = p->device;
    b->storage = storage;
    b->compute = compute;
    b->max_domains = max_domains;
    b->max_nk = max_nk;
    if (tune) b->tune = *tune;
    b->hdiff_block = b->tune.block > 0 ? b->tune.block : 128;
    const int per_sm = b->tune.blocks_per_sm > 0 ? b->tune.blocks_per_sm : 4;
    b->vadv_block = b->tune.vadv_block > 0 ? b->tune.vadv_block : 32;
    if (b->hdiff_block % 32 || b->hdiff_block > 256 || per_sm > 32 || (b->vadv_block != 32 && b->vadv_block != 64)) {
        release(b);
        return fail(SB_ERR_INVALID,
                    "batch: hdiff block must be a multiple of 32 <= 256, blocks_per_sm <= 32, vadv block 32 or 64");
    }
    if (b->tune.hdiff_rows <= 0) b->tune.hdiff_rows = 32;
    if (b->tune.hdiff_planes <= 0) b->tune.hdiff_planes = 1;
    b->hdiff_grid = p->sm_count * per_sm;
    for (int q = 0; q < kBuckets; ++q) {
        b->cap[q] = (int)std::max<int64_t>(2, ceil_div(max_nk * (q + 1), kBuckets));
        // slab mode: shared memory holds the ring only (cap 0 factor levels)
        b->vadv_smem[q] = vadv_smem_bytes(k.slab ? 0 : b->cap[q], b->vadv_block, k.compute_bytes, k.storage_bytes,
                                          k.vadv_depth,
                                          &b->ring_offset[q]);
        if ((int64_t)b->vadv_smem[q] > p->smem_optin) {
            const size_t need = b->vadv_smem[q];
            release(b);
            return fail(SB_ERR_INVALID,
                        "batch: columns of %lld levels need %zu bytes of shared memory per block (limit %d); "
                        "use a smaller max_nk or vadv block",
                        (long long)max_nk, need, p->smem_optin);
        }
        const int fit = (int)std::min<int64_t>(k.int_products ? 28 : 16,
                                               (p->smem_optin + 1024) / (int64_t)(b->vadv_smem[q] + 1024));
        // slab mode: 8 blocks per SM by default (the slabs grow with the grid);
        // 24 with the float64 integer split, which needs more warps in flight
        // (64 domains of 512x512x80 with the products in integer arithmetic:
        // 17.46 ms at 24, 17.69 at 16, 18.40 at 8)
        const int vdef = k.slab ? std::min(fit, k.int_products ? 24 : 8) : fit;
        const int vper = b->tune.vadv_blocks_per_sm > 0 ? std::min(b->tune.vadv_blocks_per_sm, fit) : vdef;
        b->vadv_grid[q] = p->sm_count * std::max(1, vper);
    }
    if (k.vadv_tmem && b->vadv_block == 32 && max_nk <= 256) {
        // per bucket: TMEM columns per warp for its cap, warps per block as the
        // 512 columns and the shared memory allow; >= 120 KB of shared memory
        // keeps every other TMEM block off the SM
        const int fit4 = (int)((p->smem_optin - 16) / (4 * (int64_t)k.tmem_ring_bytes));
        b->tmem_capable = fit4 >= 1;
        size_t smem = 120 * 1024;
        for (int q = 0; q < kBuckets && b->tmem_capable; ++q) {
            b->tmem_cpw[q] = 16 * (int)ceil_div((int64_t)b->cap[q], (int64_t)8);
            const int g4 = std::max(1, std::min({4, 512 / b->tmem_cpw[q], fit4}));
            b->tmem_block[q] = 128 * g4;
            smem = std::max(smem, 16 + (size_t)(4 * g4) * k.tmem_ring_bytes);
        }
        b->tmem_smem = smem;
        b->vadv_tmem_grid = p->sm_count;
    }
    size_t slab_total = 0;
    size_t slab_off[kBuckets] = {};
    if (k.slab) {
        for (int q = 0; q < kBuckets; ++q) {
            slab_off[q] = slab_total;
            slab_total += (2 * (size_t)b->cap[q] * b->vadv_grid[q] * b->vadv_block * k.compute_bytes + 255) / 256 * 256;
        }
    }
    cudaError_t e = cudaMallocHost((void**)&b->host_table, table_bytes(max_domains));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->dev_table, table_bytes(max_domains));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->counters, sizeof(unsigned long long) * (1 + kBuckets));
    if (e == cudaSuccess && slab_total) {
        e = cudaMalloc(&b->slab_mem, slab_total);
        if (e == cudaSuccess) {
            b->slab_bytes = slab_total;
            for (int q = 0; q < kBuckets; ++q) b->slab[q] = (char*)b->slab_mem + slab_off[q];
        }
    }
    for (auto& s : b->streams)
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (auto& ev : b->joins)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release(b);
        return fail(e == cudaErrorMemoryAllocation ? SB_ERR_NOMEM : SB_ERR_CUDA, "batch allocation failed: %s",
                    cudaGetErrorString(e));
    }
    memset(b->host_table, 0, table_bytes(max_domains));
    b->host_table->rows = b->tune.hdiff_rows;
    b->host_table->planes = b->tune.hdiff_planes;
    *out = b;
    return SB_OK;
}

int sb_batch_destroy(sb_batch* b) {
    if (b) {
        for (auto& s : b->streams)
            if (s) cudaStreamSynchronize(s);
        release(b);
    }
    return SB_OK;
}

int sb_batch_set(sb_batch* b, const sb_domain* domains, int n) {
    clear_error();
    SB_CHECK(b, SB_ERR_INVALID, "batch is NULL");
    SB_CHECK(n >= 0 && n <= b->max_domains, SB_ERR_INVALID, "%d domains exceed the batch capacity %d", n,
             b->max_domains);
    SB_CHECK(n == 0 || domains, SB_ERR_INVALID, "domains is NULL");
    // validate; classify: hdiff (in given order), vadv by bucket (decreasing nk within a bucket)
    std::vector<int> hd, vd[kBuckets];
    for (int q = 0; q < n; ++q) {
        const sb_domain& s = domains[q];
        int rc = check_domain(s.ni, s.nj, s.nk, s.si, s.sj, s.sk);
        if (rc) return rc;
        SB_CHECK(s.op == SB_OP_HDIFF || s.op == SB_OP_VADV, SB_ERR_INVALID, "domain %d: unknown op %d", q, s.op);
        const int nin = s.op == SB_OP_HDIFF ? 2 : 5;
        for (int f = 0; f < nin; ++f) SB_CHECK(s.f[f], SB_ERR_INVALID, "domain %d: NULL field %d", q, f);
        SB_CHECK(s.out, SB_ERR_INVALID, "domain %d: NULL output", q);
        if (s.op == SB_OP_HDIFF) {
            hd.push_back(q);
        } else {
            SB_CHECK(s.nk >= 2 || s.ni == 0 || s.nj == 0, SB_ERR_INVALID,
                     "domain %d: vertical advection needs nk >= 2", q);
            SB_CHECK(s.nk <= b->max_nk, SB_ERR_INVALID, "domain %d: nk = %lld exceeds the batch's max_nk %lld", q,
                     (long long)s.nk, (long long)b->max_nk);
            SB_CHECK(s.wshift_i >= 0 && s.wshift_i <= 1 && s.wshift_j >= 0 && s.wshift_j <= 1 &&
                         s.wshift_i + s.wshift_j <= 1,
                     SB_ERR_INVALID, "domain %d: bad wcon shift", q);
            int bucket = 0;
            while (bucket < kBuckets - 1 && s.nk > b->cap[bucket]) ++bucket;
            vd[bucket].push_back(q);
        }
    }
    for (auto& v : vd)
        std::stable_sort(v.begin(), v.end(), [&](int x, int y) { return domains[x].nk > domains[y].nk; });
    bool idx64 = false;
    bool tmem_ok = b->tmem_capable;
    const int es = storage_size(b->storage);
    DevTable* t = b->host_table;
    int slot = 0;
    auto fill = [&](int q, int64_t& items) {
        const sb_domain& s = domains[q];
        DevDomain& d = t->dom[slot++];
        memset(&d, 0, sizeof(d));
        d.op = s.op;
        d.ni = (int32_t)s.ni;
        d.nj = (int32_t)s.nj;
        d.nk = (int32_t)s.nk;
        d.si = s.si;
        d.sj = s.sj;
        d.sk = s.sk;
        for (int f = 0; f < 5; ++f) d.f[f] = s.f[f];
        d.out = s.out;
        d.item_begin = items;
        const int64_t span = (s.ni + 33) * std::abs(s.si) + (s.nj + 2) * std::abs(s.sj) + (s.nk + 1) * std::abs(s.sk);
        if (span >= (1LL << 31)) idx64 = true;
        if (s.ni == 0 || s.nj == 0 || s.nk == 0) return;
        if (s.op == SB_OP_HDIFF) {
            d.items_i = (int32_t)ceil_div(s.ni, kJscanOut);
            d.items_j = (int32_t)ceil_div(s.nj, b->tune.hdiff_rows);
            items += (int64_t)d.items_i * d.items_j * ceil_div(s.nk, b->tune.hdiff_planes);
        } else {
            d.wsh = (int64_t)s.wshift_i * s.si + (int64_t)s.wshift_j * s.sj;
            d.kp = (s.sk * es) % 16 == 0 ? 1 : (s.sk * es) % 16 == 8 ? 2 : 0;
            if (s.si != 1 || s.sj <= 0 || s.sk <= 0) tmem_ok = false;
            d.items_i = (int32_t)ceil_div(s.ni, b->vadv_block);
            d.items_j = (int32_t)s.nj;
            items += (int64_t)d.items_i * d.items_j;
        }
    };
    int64_t hitems = 0;
    for (int q : hd) fill(q, hitems);
    t->n_hdiff = (int32_t)hd.size();
    t->hdiff_items = hitems;
    int64_t total = hitems;
    for (int bk = 0; bk < kBuckets; ++bk) {
        t->bucket_first[bk] = slot;
        int64_t items = 0;
        for (int q : vd[bk]) fill(q, items);
        t->bucket_items[bk] = items;
        total += items;
    }
    t->bucket_first[kBuckets] = slot;
    t->ndomains = n;
    b->total_items = total;
    b->idx64 = idx64;
    b->use_tmem = tmem_ok && !idx64;
    return SB_OK;
}

int sb_batch_launch(sb_batch* b, void* stream, double* time_s) {
    clear_error();
    SB_CHECK(b, SB_ERR_INVALID, "batch is NULL");
    int dev = 0;
    SB_CUDA(cudaGetDevice(&dev));
    SB_CHECK(dev == b->device, SB_ERR_INVALID, "batch was created on device %d, current device is %d", b->device,
             dev);
    if (!b->exec || b->graph_idx64 != b->idx64 || b->graph_tmem != b->use_tmem) {
        int rc = capture_graph(b);
        if (rc) return rc;
    }
    return timed((cudaStream_t)stream, time_s, [&]() {
        SB_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
        return SB_OK;
    });
}

int sb_batch_info(sb_batch* b, int64_t* total_items, size_t* workspace_bytes, int* grid, int* block) {
    SB_CHECK(b, SB_ERR_INVALID, "batch is NULL");
    if (total_items) *total_items = b->total_items;
    if (workspace_bytes) *workspace_bytes = b->slab_bytes;
    if (grid) *grid = b->hdiff_grid;
    if (block) *block = b->hdiff_block;
    return SB_OK;
}

}  // extern "C"
