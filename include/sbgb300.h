/*
 * sbgb300 -- C ABI of the GB300 (sm_103a) structured-grid stencil backend.
 *
 * Every entry point takes plain pointers, sizes and integer codes; none takes
 * or returns a C++ or PyTorch type.  All return an int status: SB_OK (0) on
 * success, a non-zero SB_ERR_* code otherwise, with a description available
 * from sb_last_error() on the calling thread.  This mirrors the reference's
 * generated launcher, which returns 0 or 1 and prints the CUDA error
 * (stencil_benchmarks/benchmarks_collection/stencils/cuda_hip/templates/base.j2:48-55),
 * and which the reference's ctypes wrapper turns into ExecutionError
 * (stencil_benchmarks/tools/compilation.py:176-193).
 *
 * Field convention (same as the reference): a field is a 3D array with a halo;
 * the pointer passed is the address of the FIRST INTERIOR POINT (reference:
 * compilation.data_ptr(array, halo), tools/compilation.py:273-282) and
 * (si, sj, sk) are its strides in ELEMENTS.  All fields of one call share
 * the same strides, because the reference allocates them identically
 * (stencils/base.py:87-101).  Unlike the reference, which compiles domain and
 * strides into each generated kernel (stencils/cuda_hip/mixin.py:113-123),
 * every size here is a run-time argument: one prebuilt library serves all
 * shapes.
 *
 * Timing convention: when `time_s` is non-NULL, the call records CUDA events
 * on `stream` around the kernel launch, waits for the end event and stores
 * the elapsed seconds (reference: base.j2:145-190, "gpu" timers).  When it is
 * NULL the launch is asynchronous on `stream` (NULL = legacy default stream).
 */
#ifndef SBGB300_H
#define SBGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define SB_OK 0
#define SB_ERR_INVALID 1     /* invalid argument: shape, stride, type, alignment */
#define SB_ERR_CUDA 2        /* a CUDA runtime call failed                         */
#define SB_ERR_UNSUPPORTED 3 /* valid request the library does not implement       */
#define SB_ERR_NOMEM 4       /* device or host allocation failed                   */
#define SB_ERR_TIMEOUT 5     /* a bounded device-side wait gave up                 */
#define SB_ERR_BUDGET 6      /* request exceeds a configured memory budget         */

/* ---- element types (storage and compute) -------------------------------- */
#define SB_F64 0
#define SB_F32 1
#define SB_BF16 2 /* storage only; computed in f32 (or f64) */
#define SB_F32X2 3 /* compute only, with f64 storage: float pair ("double-float"),
                    * ~48-bit significand on the fp32 pipe; results within a few
                    * 2^-48 (relative to the operands) of the f64 ones, not
                    * bit-identical */
#define SB_FIX64 4 /* compute only, hdiff with f64 storage: lap/flx/fly sums exact
                    * in 64-bit fixed point on a per-strip scale, one f64 FMA per
                    * point; errors at f64 rounding level, not bit-identical */

/* ---- memcpy kinds (same values as cudaMemcpyKind) ------------------------ */
#define SB_H2H 0
#define SB_H2D 1
#define SB_D2H 2
#define SB_D2D 3
#define SB_DEFAULT 4

/* ---- kernel variants ------------------------------------------------------ */
#define SB_VARIANT_AUTO 0  /* the library's choice, where the layout qualifies:
                            * hdiff: TMA for float64, VSCAN for float32, bfloat16
                            * and float pairs, JSCAN otherwise (and for fixed64);
                            * vadv: TMEM for float32 compute on >= 2048 column
                            * groups (bfloat16: level stride a multiple of 8 bytes),
                            * else SLAB / WSLAB when ccol/dcol are given, else SMEM */
#define SB_HDIFF_TILE 1   /* smem-staged k-plane tiles, lap/flx/fly once per point */
#define SB_HDIFF_JSCAN 2  /* register j-march, i-neighbours by warp shuffles       */
#define SB_HDIFF_TMA 3    /* TILE with inp k-planes staged by TMA (cp.async.bulk.tensor)
                           * into two shared-memory stages (i unit-stride, 16-byte
                           * aligned j/k strides and halo corner)                   */
#define SB_HDIFF_VSCAN 4  /* JSCAN with V columns per lane moved as one aligned
                           * vector (block_x = strip width 32*V: 64 for 8-byte,
                           * 64 or 128 for 4-byte, 128 or 256 for 2-byte storage); i
                           * unit-stride, j/k strides multiples of the vector,
                           * inp/coeff/out at one offset from a vector boundary */
#define SB_VADV_SMEM 1    /* one thread per column, ccol/dcol in shared memory     */
#define SB_VADV_GLOBAL 2  /* one thread per column, ccol/dcol in caller scratch    */
#define SB_VADV_SLAB 3    /* persistent threads, factors in compact per-thread slabs of
                           * the caller's ccol/dcol (L2-resident), cp.async staging;
                           * tune: block_x 32/64, unroll = depth 1 (32-thread
                           * blocks) / 2 / 4 / 8, k_per_cta = blocks per SM (0:
                           * 28 with the float64 integer split, the grid balanced
                           * so that every block takes as many column groups;
                           * otherwise as many as fit with slabs <= L2/2)        */
#define SB_VADV_WSLAB 4   /* SLAB with each warp's 32-column rows staged together in
                           * 16-byte copies (needs i unit-stride); same tune fields.
                           * SB_VARIANT_AUTO with ccol/dcol given and no block/unroll
                           * in the tune picks WSLAB for 2/4-byte storage and SLAB
                           * for 8-byte storage when the layout qualifies and TMEM
                           * does not apply */
#define SB_VADV_TMEM 5    /* float32 compute: WSLAB row staging, factors in tensor
                           * memory (tcgen05.st / tcgen05.ld) instead of a slab; one
                           * persistent block per SM; no scratch; needs i unit-stride
                           * and 2 <= nk <= 256; unroll = ring depth 4, 8 or 16
                           * (0: deepest that fits) */

/*
 * Launch tuning.  Zero in any field means "choose the default".  The
 * reference exposes the same knobs as benchmark Parameters (block_size,
 * unroll_factor; stencils/cuda_hip/horizontal_diffusion.py:41,
 * vertical_advection.py:40-46) baked into generated code; here they are
 * run-time values validated against the device limits (base.j2:92-135).
 */
typedef struct sb_tune {
    int32_t variant;   /* SB_HDIFF_* / SB_VADV_* or SB_VARIANT_AUTO            */
    int32_t block_x;   /* threads along i                                       */
    int32_t block_y;   /* threads along j                                       */
    int32_t tile_y;    /* hdiff: rows of j per CTA                              */
    int32_t k_per_cta; /* hdiff: k-planes per CTA                               */
    int32_t unroll;    /* STREAM: vectors per thread per iteration             */
    int32_t flags;     /* STREAM: bit0 streaming (evict-first) stores;
                        * vadv TMEM: bit 10 / 11 stage through 32-bit shared
                        * addresses / generic pointers (neither: the default);
                        * float64 hdiff TMA / vadv SLAB / Laplacian strips:
                        * bits 4-7 pick which operations run as integer
                        * arithmetic instead of fp64 instructions (same bits
                        * either way; 0: the library's default split, 1: all
                        * on the fp64 pipe, 2-8 (hdiff), 2-15 (vadv), 2-4
                        * (Laplacian): other splits)                          */
    int32_t reserved;
} sb_tune;

/* ---- library / device ---------------------------------------------------- */
const char* sb_last_error(void);
int sb_version(void);
int sb_device_count(int* count);
int sb_set_device(int device);
int sb_get_device(int* device); /* the calling thread's current device */
int sb_device_info(int device, char* name, int name_len, int* sm_count, int* cc_major,
                   int* cc_minor, size_t* total_mem, int* l2_bytes, int* smem_optin);
int sb_synchronize(void);

/* Bounded waits.  The only kernels that wait on the device are the hdiff
 * TMA tiles (SB_HDIFF_TMA), which wait on an mbarrier for each plane's tensor
 * copy.  A wait gives up after a bounded number of polls; the whole thread
 * block then stops before storing that plane, waits (bounded) for the copies
 * it still has in flight and sets a process-wide status word held in
 * page-locked, device-mapped host memory (allocated by the first TMA launch:
 * make the first sb_hdiff call before any stream capture).  The give-up is
 * reported as SB_ERR_TIMEOUT, and the word cleared, by the first of: a timed
 * sb_hdiff call (after its launch), the next sb_hdiff call (before it
 * launches anything), sb_synchronize, sb_stream_synchronize,
 * sb_event_synchronize, or sb_kernel_status.  No reference counterpart (its
 * kernels do not wait on the device).
 * sb_kernel_status: SB_ERR_TIMEOUT if a launch has given up since the last
 * report, else SB_OK; does not synchronise.
 * sb_debug_wait_limit: testing aid, the polls of each first wait (0: give up
 * at once; -1: the default, 2^20); the drain of copies in flight always uses
 * the default.                                                              */
int sb_kernel_status(void);
int sb_debug_wait_limit(int polls);

/* ---- memory (reference: stencils/cuda_hip/api.py:54-94 via libcudart) ---- */
int sb_malloc(void** ptr, size_t bytes);
int sb_free(void* ptr);
int sb_malloc_host(void** ptr, size_t bytes); /* page-locked host memory */
int sb_free_host(void* ptr);
int sb_memcpy(void* dst, const void* src, size_t bytes, int kind);
int sb_memcpy_async(void* dst, const void* src, size_t bytes, int kind, void* stream);
/* The same copy done by the SMs instead of a copy engine (asynchronous on
 * `stream`): any mix of device and page-locked host memory (sb_malloc_host),
 * 16-byte vectors where both pointers are 16-byte aligned. */
int sb_memcpy_sm(void* dst, const void* src, size_t bytes, void* stream);
int sb_memset(void* dst, int value, size_t bytes);
int sb_mem_info(size_t* free_bytes, size_t* total_bytes);

/* ---- streams and events --------------------------------------------------- */
int sb_stream_create(void** stream);
int sb_stream_destroy(void* stream);
int sb_stream_synchronize(void* stream);
int sb_event_create(void** event);
int sb_event_destroy(void* event);
int sb_event_record(void* event, void* stream);
int sb_event_elapsed(void* start, void* stop, double* seconds);
int sb_event_synchronize(void* event);

/* Overwrite an internal device buffer larger than L2 on `stream` so that the
 * next kernel starts cold (the reference cycles `data_sets` for the same
 * purpose, stencils/base.py:47-51,152). */
int sb_l2_flush(void* stream);

/* ---- STREAM (reference: stream/cuda_hip.j2:132-173, run() 179-288) --------
 * op: 0 init (a=1, b=2, c=0), 1 copy (c=a), 2 scale (b=s*c), 3 add (c=a+b),
 *     4 triad (a=b+s*c).  dtype SB_F64 or SB_F32; n elements per array.      */
#define SB_STREAM_INIT 0
#define SB_STREAM_COPY 1
#define SB_STREAM_SCALE 2
#define SB_STREAM_ADD 3
#define SB_STREAM_TRIAD 4
/* tune->variant picks the grid: SB_STREAM_GRID_STRIDE, a few blocks per SM
 * striding over the arrays (block_x <= 512, default 512 threads x 4 vectors);
 * SB_STREAM_GRID_CHUNK, one block per block_x * unroll 16-byte vectors
 * (block_x <= 1024, default 1024 x 2); 0: the library's choice (chunks;
 * 2^29-element float64 arrays: 7.2-7.3 TB/s against 6.8-6.9 striding).  tune->flags
 * bit0: streaming (evict-first) stores.                                    */
#define SB_STREAM_GRID_STRIDE 1
#define SB_STREAM_GRID_CHUNK 2
int sb_stream_op(int op, int dtype, void* a, void* b, void* c, double scalar, int64_t n,
                 const sb_tune* tune, void* stream, double* time_s);

/* ---- basic stencils (reference: stencils/cuda_hip/basic.py:115-132 bodies,
 *      oracles stencils/base.py:180-254) -------------------------------------- */
int sb_copy(int storage, const void* inp, void* out, int64_t ni, int64_t nj, int64_t nk,
            int64_t si, int64_t sj, int64_t sk, const sb_tune* tune, void* stream,
            double* time_s);
/* along_mask: bit0 x, bit1 y, bit2 z (LaplacianStencil along_x/y/z).
 * tune->variant: SB_BASIC_POINT, one thread per point and 4 k-planes
 * (block_x x block_y threads, default 128 x 2); SB_BASIC_MARCH, lanes along i,
 * each thread holding a strip of tile_y rows of j for k_per_cta k-planes in
 * registers (4 or 8 rows x 2 planes; default 4 x 2) with block_y warps per
 * block (default 4); float64 along x and y: flags bits 4-7 pick which
 * subtractions run as integer arithmetic (0: the library's default, 1: all
 * fp64, 2-4: other splits); variant 0: the library's choice (the strips;
 * along_mask 0 always runs the point kernel).  Same bits from every variant. */
#define SB_BASIC_POINT 1
#define SB_BASIC_MARCH 2
int sb_laplacian(int storage, int compute, const void* inp, void* out, int64_t ni, int64_t nj,
                 int64_t nk, int64_t si, int64_t sj, int64_t sk, int along_mask,
                 const sb_tune* tune, void* stream, double* time_s);
/* Empty (reference: the generated kernel with an empty body, stencils/cuda_hip/
 * basic.py:101-103): the basic stencils' grid over the domain, no memory access */
int sb_empty(int64_t ni, int64_t nj, int64_t nk, const sb_tune* tune, void* stream, double* time_s);
/* symmetric 0: (inp[+1] + inp) / 2; symmetric 1: (inp[+1] + inp[-1]) / 2 */
int sb_average(int storage, int compute, const void* inp, void* out, int64_t ni, int64_t nj,
               int64_t nk, int64_t si, int64_t sj, int64_t sk, int axis, int symmetric,
               const sb_tune* tune, void* stream, double* time_s);

/* ---- horizontal diffusion (reference: stencils/cuda_hip/horizontal_diffusion.py,
 *      oracle stencils/base.py:276-311).  Needs a halo of >= 2 in i and j.    */
int sb_hdiff(int storage, int compute, const void* inp, const void* coeff, void* out,
             int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
             const sb_tune* tune, void* stream, double* time_s);

/* ---- vertical advection, one velocity component (reference:
 *      stencils/cuda_hip/vertical_advection.py, oracle stencils/base.py:410-473).
 * The new tensstage is written to `out`; pass out == tensstage for the
 * reference's in-place update (any other overlap is not allowed).  wcon is
 * read at the column shifted by (wshift_i, wshift_j): (1,0) for u, (0,1)
 * for v, (0,0) for w.  ccol/dcol may be NULL; they are only used as scratch
 * (the reference's fields of the same names, compute-type sized elements) by
 * SB_VADV_GLOBAL, SB_VADV_SLAB, SB_VADV_WSLAB, and by SB_VARIANT_AUTO, which
 * picks a slab form when they are given and the tensor-memory form does not
 * apply.  Needs nk >= 2.                                                       */
int sb_vadv(int storage, int compute, const void* stage, const void* pos, const void* tens,
            const void* tensstage, const void* wcon, void* out, void* ccol, void* dcol, int64_t ni,
            int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk, int wshift_i, int wshift_j,
            const sb_tune* tune, void* stream, double* time_s);
/* All three components of vertical advection on one wcon field (reference:
 * all_components=True, stencils/base.py:475-483, and its fused kernel
 * cuda_hip/templates/vertical_advection_localmemmerged.j2): stage, pos, tens,
 * tensstage and out are arrays of three pointers (u, v, w), every field with
 * the same layout; u reads wcon at (i+1, j), v at (i, j+1), w at (i, j).
 * With float32 compute on a layout the tensor-memory form takes (variant
 * AUTO with no explicit shape and at least 2048 column groups of 32, or
 * SB_VADV_TMEM) one launch solves the three components of each column group
 * in turn, so wcon comes from HBM once; otherwise one sb_vadv launch per
 * component.  Same bits either way. */
int sb_vadv3(int storage, int compute, const void* const* stage, const void* const* pos,
             const void* const* tens, const void* const* tensstage, const void* wcon, void* const* out,
             void* ccol, void* dcol, int64_t ni, int64_t nj, int64_t nk, int64_t si, int64_t sj, int64_t sk,
             const sb_tune* tune, void* stream, double* time_s);

/* ---- batched execution: many domains, one persistent launch ----------------
 * No single counterpart in the reference, which launches one generated kernel
 * per domain (stencils/cuda_hip/templates/base.j2:68-193); this batches the
 * same hdiff / vadv computations.  A batch holds up to max_domains domains of
 * one (storage, compute) form; sb_batch_launch runs all of them in one graph
 * launch (captured on the first launch) of persistent kernels -- one for the
 * hdiff domains, one per nk bucket for the vadv domains, running side by side
 * -- that pull work items from device-side queues.  Results
 * are bit-identical to sb_hdiff / sb_vadv on the same domain.  The domain
 * table lives in pinned host memory and is copied by each launch: do not
 * call sb_batch_set while a launch of the same batch may still be pending
 * (synchronise its stream first).  Distinct batches are independent.  Except
 * for float32/float32 the vadv kernels keep their factors in a device
 * workspace owned by the batch (sb_batch_info reports its size).            */
#define SB_OP_HDIFF 0
#define SB_OP_VADV 1
typedef struct sb_domain {
    int32_t op;                 /* SB_OP_HDIFF or SB_OP_VADV                        */
    int32_t wshift_i, wshift_j; /* vadv: wcon column shift (1,0) u, (0,1) v, (0,0) w */
    int32_t reserved;
    int64_t ni, nj, nk, si, sj, sk; /* interior size, element strides              */
    const void* f[5];           /* hdiff: inp, coeff; vadv: stage, pos, tens, tensstage, wcon */
    void* out;                  /* hdiff: out; vadv: new tensstage (may be tensstage) */
} sb_domain;
typedef struct sb_batch_tune {
    int32_t block;         /* threads per block, multiple of 32, <= 256 (0: 128)   */
    int32_t blocks_per_sm; /* persistent blocks per SM (0: 4)                      */
    int32_t hdiff_rows;    /* rows of j per hdiff item (0: 32)                     */
    int32_t hdiff_planes;  /* k-planes per hdiff item (0: 1)                       */
    int32_t order;         /* 0: the hdiff kernel enters the graph first; 1: the vadv
                            * bucket kernels first (tallest bucket first), so their
                            * blocks are resident before hdiff fills the SMs    */
    int32_t vadv_block;    /* threads (= columns) per vadv block: 32 or 64 (0: 32)   */
    int32_t vadv_blocks_per_sm; /* persistent vadv blocks per SM (0: as many as fit;
                                 * with a factor workspace at most 8, or 24 when the
                                 * float64 products run in integer arithmetic; at
                                 * most 28 when given)                             */
    int32_t reserved;
} sb_batch_tune;
typedef struct sb_batch sb_batch;
int sb_batch_create(sb_batch** batch, int storage, int compute, int max_domains, int64_t max_nk,
                    const sb_batch_tune* tune);
int sb_batch_set(sb_batch* batch, const sb_domain* domains, int n);
int sb_batch_launch(sb_batch* batch, void* stream, double* time_s);
int sb_batch_info(sb_batch* batch, int64_t* total_items, size_t* workspace_bytes, int* grid, int* block);
int sb_batch_destroy(sb_batch* batch);

/* ---- serving support --------------------------------------------------------
 * No counterpart in the reference (it runs one benchmark at a time).
 * sb_fill_batch: fill n device fields in one launch with seeded uniform values
 * in [lo, hi), generated without fp64 arithmetic on the device.  With H the
 * 32-bit lowbias32 hash and, per field, k0 = H(lo32(seed) ^ 0xA511E9B3) | 1,
 * k1 = H(hi32(seed) + 0x632BE5AB), k2 = H(k0 ^ k1),
 * x(n) = lo32(n) * k0 + k1 + hi32(n) * 0x9E3779B9 (32-bit arithmetic):
 *   float32:  v[e] = lo_f + span_f * ((H(x(e)) >> 8) * 2^-24)  in float32
 *             (lo_f = (float)lo, span_f = (float)(hi - lo));
 *   bfloat16: h = H(x(e / 2)); v[e] = lo_f + span_f * (b * 2^-16) in float32
 *             with b = h & 0xFFFF for even e, h >> 16 for odd e, then
 *             rounded to bfloat16;
 *   float64:  h1 = H(x(e)), h2 = H(h1 ^ k2), k = h1 << 21 | h2 >> 11,
 *             v[e] = lo + (hi - lo) * (k * 2^-53)  in double;
 * each operation rounded to nearest even, no fused multiply-add.  The
 * descriptors are copied (asynchronously on
 * `stream`, from the caller's host memory, which must stay valid until the
 * stream reaches the copy) into `desc_scratch`, a device buffer of at least n
 * descriptors owned by the caller.  From page-locked host memory the copy is
 * queued; from pageable memory CUDA first waits for `stream` to drain.
 * sb_event_query: SB_OK if the event has completed, SB_NOT_READY if not.      */
#define SB_NOT_READY 7
typedef struct sb_fill_desc {
    void* ptr;     /* device field (whole span, halo included)  */
    int64_t count; /* elements                                   */
    uint64_t seed;
    double lo, hi;
    int32_t storage; /* SB_F64, SB_F32, SB_BF16 */
    int32_t reserved;
} sb_fill_desc;
int sb_fill_batch(const sb_fill_desc* descs, int n, void* desc_scratch, void* stream);
int sb_event_query(void* event);
int sb_stream_wait_event(void* stream, void* event); /* later work on stream waits for event */

/* ---- device-memory arena (serving) -------------------------------------------
 * Best-fit allocator with coalescing over a caller-provided address range
 * [base, base + bytes) (normally one cudaMalloc); pure host bookkeeping, no
 * CUDA call, thread-safe.  sb_arena_alloc returns SB_ERR_BUDGET when no free
 * block is large enough.                                                     */
typedef struct sb_arena sb_arena;
int sb_arena_create(sb_arena** arena, uint64_t base, uint64_t bytes, uint64_t align);
int sb_arena_alloc(sb_arena* arena, uint64_t bytes, uint64_t* address);
int sb_arena_free(sb_arena* arena, uint64_t address);
int sb_arena_stats(sb_arena* arena, uint64_t* in_use, uint64_t* peak, uint64_t* largest_free,
                   uint64_t* free_blocks);
int sb_arena_destroy(sb_arena* arena);

/* ---- request server (continuous batching) -----------------------------------
 * No counterpart in the reference (it runs one benchmark at a time).  A
 * request is one hdiff or vadv (u component) solve on its own domain, with
 * float64, float32 or bfloat16 storage (float32 compute for the latter two;
 * float64 requests in float64, or with float64_compute = SB_FIX64 in the fast
 * forms: fixed-point hdiff, float-pair vadv).  The server owns one device
 * region of budget_bytes (allocated by sb_server_create), carves request
 * fields from it, generates the inputs on the device (sb_fill_batch, seeds
 * derived from the request seed) and runs requests as batched graph replays
 * (mode 0) or one kernel launch each (mode 1), with slots_per_form batches of
 * each precision in flight.  sb_server_step(now) polls completions, admits
 * waiting requests in arrival order as the budget allows, and dispatches;
 * `now` (any clock, seconds) stamps what happens in the step.  Completed
 * requests are reported by sb_server_take_completed; with keep bit 0 (outputs)
 * or bit 1 (inputs) set their fields stay allocated (sb_server_field gives
 * the address of field q: hdiff inp, coeff, out; vadv stage, pos, tens,
 * tensstage, wcon, out; i unit-stride, j stride ni + 2h, k stride
 * (ni + 2h)(nj + 2h), halo h = 2 for hdiff, 1 for vadv) until
 * sb_server_release; sb_server_query reports the times of a request the
 * server still holds.  simulate = 1 makes no CUDA call (scheduling tests;
 * sb_server_debug_complete finishes the in-flight slots, sb_server_debug_launches
 * lists the launches as (storage, requests)).  One thread per server.        */
typedef struct sb_server sb_server;
typedef struct sb_server_config {
    uint64_t budget_bytes;
    int32_t max_batch;       /* requests per batch (0: 64)                       */
    int32_t max_nk;          /* largest vadv nk accepted (0: 137)                */
    int32_t slots_per_form;  /* batches in flight per precision (0: 3)           */
    int32_t float64_compute; /* SB_F64 (0 also) or SB_FIX64                      */
    int32_t mode;            /* 0 batched graph replays, 1 one launch per request */
    int32_t keep;            /* bit 0 outputs, bit 1 inputs: kept until released */
    int32_t fill_capacity;   /* fill descriptors per step (0: 4096)              */
    int32_t simulate;
    sb_batch_tune tune;      /* batch launch shape (zeros: defaults)             */
} sb_server_config;
typedef struct sb_request {
    int64_t id;              /* unique among the requests the server holds       */
    int32_t op;              /* SB_OP_HDIFF or SB_OP_VADV                        */
    int32_t storage;         /* SB_F64, SB_F32 or SB_BF16                        */
    int64_t ni, nj, nk;
    uint64_t seed;
    double arrival;          /* caller's clock, copied into the completion       */
} sb_request;
typedef struct sb_completion {
    int64_t id;
    double arrival, admitted, launched, completed;
} sb_completion;
typedef struct sb_server_state {
    uint64_t budget_bytes, in_use_bytes, peak_bytes;
    int64_t waiting, ready, inflight, max_waiting, busy_slots;
    double work_seconds;     /* host time in steps that retired, admitted or launched */
} sb_server_state;
typedef struct sb_server_launch {
    int32_t storage, requests;
} sb_server_launch;
int sb_server_create(sb_server** server, const sb_server_config* config);
int sb_server_destroy(sb_server* server);
int sb_server_submit(sb_server* server, const sb_request* request);
int sb_server_step(sb_server* server, double now, int* busy);
int sb_server_take_completed(sb_server* server, sb_completion* out, int capacity, int* n);
int sb_server_field(sb_server* server, int64_t id, int field, void** ptr);
/* times of a request the server still holds (-1: not yet) */
int sb_server_query(sb_server* server, int64_t id, sb_completion* record);
int sb_server_release(sb_server* server, int64_t id);
int sb_server_stats(sb_server* server, sb_server_state* stats);
int sb_server_debug_complete(sb_server* server);
int sb_server_debug_launches(sb_server* server, sb_server_launch* out, int capacity, int* n);

/* ---- vertical advection without device allocation -------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * code embedded in a host framework that owns every device allocation (fixed
 * memory pools), or paths that must not trigger the device-wide
 * synchronisation that cudaMalloc/cudaFree can cause.  Computes exactly what
 * sb_vadv computes (bit-identical results) with the factors of the
 * elimination kept in global memory, but that scratch is one fixed array of
 * SB_VADV_NOALLOC_SCRATCH_BYTES compiled into the library (held by every
 * device that loads the library until the process exits) instead of
 * caller-provided ccol/dcol fields; the call allocates nothing.  The caller
 * still passes all input and output fields.  Columns are processed in a
 * grid-stride loop over as many thread slots as the array holds (2 * nk
 * factors per slot); a call whose nk leaves room for fewer than one block of
 * 64 slots fails with SB_ERR_BUDGET before launching.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and
 * caches it: make that first call before any stream capture on the device.
 * The cached address does not survive cudaDeviceReset: a process that resets
 * a device must not call this entry point on that device afterwards.
 * Every call shares the array, so calls that overlap on the GPU race and
 * must be serialised by the caller; every factor is written before it is
 * read, so no state carries over between calls.                             */
#define SB_VADV_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int sb_vadv_noalloc(int storage, int compute, const void* stage, const void* pos, const void* tens,
                    const void* tensstage, const void* wcon, void* out, int64_t ni, int64_t nj, int64_t nk,
                    int64_t si, int64_t sj, int64_t sk, int wshift_i, int wshift_j, void* stream,
                    double* time_s);

/* ---- measurement helpers ---------------------------------------------------- */
/* Throughput of dependent-free arithmetic on this device, in operations per
 * second (kind 0: f64 add, 1: f64 fma, 2: f32 fma, 3: f64->f32 conversion,
 * 4: f32->f64 conversion, 5: 32-bit integer shift/xor/multiply, 6: u32->f32
 * conversion, 7: s32->f32 conversion, 8: f64 add and 9: f64 multiply in
 * integer arithmetic, bit-identical to the fp64 instructions; 10: f64 adds
 * with independent 32-bit integer work beside them, 48 integer operations per
 * add, counted as adds; 11: that integer work alone, counted the same way --
 * 10 runs at the rate of 0 if the two pipes overlap, and at
 * 1 / (1/rate(0) + 1/rate(11)) if they do not; 12: f64 reciprocal in integer
 * arithmetic, 13: the f64 reciprocal instruction sequence, __drcp_rn; 14:
 * the 64-bit leading-zero instruction (the integer add's normalisation),
 * 15: a leading-zero count from an int-to-float conversion, for comparison;
 * 16 / 17: 14 / 15 with one f64 add beside each count, counted as adds;
 * 18 / 19 / 20: f64 adds beside one integer binary64 add, one 64-bit
 * variable shift, or one 64-bit add and compare each, counted as adds). */
int sb_probe_arith_rate(int kind, double* ops_per_s);
/* The binary64 operations the kernels can run in integer arithmetic, applied
 * element-wise on the device to n doubles (op 0: a + b, 1: a - b, 2: a * b,
 * 3: 1 / a, b unused), asynchronously on `stream`: for checking them against
 * IEEE arithmetic.  Operands the integer path declines take the fp64
 * instruction, as in the kernels. */
int sb_debug_soft_f64(int op, const void* a, const void* b, void* out, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SBGB300_H */
