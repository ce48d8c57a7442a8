// Continuous-batching request server, native: admission by memory budget,
// device-side field generation, dispatch into batched graph replays (or one
// launch per request), retirement -- all without a Python call per request.
//
// One sb_server_step(now):
//   1. poll: every slot whose completion event has fired retires its requests
//      (completed = now) and returns their fields to the arena, except the
//      kept ones;
//   2. admit: waiting requests, in arrival order, get their fields from the
//      budget-capped arena (one device region allocated at creation, carved
//      by sb_arena: no cudaMalloc per request); the inputs of everything
//      admitted in this step are generated on the device by one
//      sb_fill_batch launch on the fill stream;
//   3. dispatch: for every precision form with admitted requests and a free
//      slot, up to max_batch of them are packed into that slot's sb_batch and
//      launched (one graph replay) on the slot's stream after the fill, or,
//      in plain mode, launched one sb_hdiff / sb_vadv each.
// Several slots per form are in flight at once: requests that arrive while
// others run are admitted as memory frees up and overlap on the device.
//
// A request's field q has seed (seed * 0x9E3779B97F4A7C15 + (q + 1) *
// 0xD1B54A32D192ED03) mod 2^64 and the layout of the reference's fields with
// i unit-stride and no padding: shape (ni + 2 hi, nj + 2 hj, nk), halo (2, 2,
// 0) for hdiff and (1, 1, 0) for vadv.  Fields: hdiff inp, coeff U[0, 1),
// out; vadv stage, pos, tens, tensstage U[-1, 1), wcon U[-0.5, 0.5), out.
//
// With `simulate` set the server makes no CUDA call at all (a fake region,
// no fills or launches; a slot's work completes when sb_server_debug_complete
// is called): the scheduling logic can be tested without a GPU.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace sb {
namespace {

constexpr uint64_t kAlign = 256;
constexpr int kFillDepth = 8;
constexpr int kForms = 3;  // float64, float32, bfloat16 storage

struct FieldSpec {
    const char* name;
    double lo, hi;
    bool input;
};
constexpr FieldSpec kHdiffFields[] = {{"inp", 0.0, 1.0, true}, {"coeff", 0.0, 1.0, true}, {"out", 0, 0, false}};
constexpr FieldSpec kVadvFields[] = {{"stage", -1.0, 1.0, true}, {"pos", -1.0, 1.0, true},
                                     {"tens", -1.0, 1.0, true},  {"tensstage", -1.0, 1.0, true},
                                     {"wcon", -0.5, 0.5, true},  {"out", 0, 0, false}};

int form_of(int storage) { return storage == SB_F64 ? 0 : storage == SB_F32 ? 1 : storage == SB_BF16 ? 2 : -1; }

struct Req {
    sb_request r;
    double admitted = -1.0, launched = -1.0, completed = -1.0;
    uint64_t field[6] = {};
    int nfields = 0;
    bool kept = false;

    int64_t hi() const { return r.op == SB_OP_HDIFF ? 2 : 1; }
    int64_t sx() const { return r.ni + 2 * hi(); }
    int64_t sy() const { return r.nj + 2 * hi(); }
    int64_t count() const { return sx() * sy() * r.nk; }
    int64_t interior_offset() const { return hi() + hi() * sx(); }  // elements
};

uint64_t field_seed(uint64_t seed, int q) {
    return seed * 0x9E3779B97F4A7C15ull + (uint64_t)(q + 1) * 0xD1B54A32D192ED03ull;
}

struct Slot {
    sb_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<Req*> reqs;
    bool busy = false;
    bool sim_done = false;
};

}  // namespace
}  // namespace sb

using namespace sb;

struct sb_server {
    sb_server_config cfg{};
    int device = 0;
    void* region = nullptr;
    sb_arena* arena = nullptr;
    std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
    std::deque<Req*> waiting;
    std::deque<Req*> ready[kForms];
    std::vector<Slot> slots[kForms];
    std::vector<sb_completion> completed;
    // fills
    cudaStream_t fill_stream = nullptr;
    void* fill_scratch = nullptr;
    sb_fill_desc* fill_staging = nullptr;  // pinned, kFillDepth * fill_capacity descriptors
    cudaEvent_t fill_events[kFillDepth] = {};
    bool fill_used[kFillDepth] = {};
    int fill_next = 0;
    int fill_last = -1;  // staging slot of the latest fill (-1: none yet)
    std::vector<sb_fill_desc> descs;
    std::vector<sb_domain> doms;
    std::vector<sb_server_launch> launch_log;  // simulate only
    int64_t max_waiting = 0;
    int64_t inflight = 0;
    double work_seconds = 0.0;  // in steps that retired, admitted or launched something

    bool sim() const { return cfg.simulate != 0; }
    int compute_of(int form, int op) const {
        if (form == 0) {
            if (cfg.float64_compute == SB_FIX64) return op == SB_OP_HDIFF ? SB_FIX64 : SB_F32X2;
            return SB_F64;
        }
        return SB_F32;
    }
    int storage_of(int form) const { return form == 0 ? SB_F64 : form == 1 ? SB_F32 : SB_BF16; }

    ~sb_server() {
        if (!sim()) {
            for (auto& forms : slots)
                for (auto& s : forms) {
                    if (s.batch) sb_batch_destroy(s.batch);
                    if (s.stream) cudaStreamDestroy(s.stream);
                    if (s.done) cudaEventDestroy(s.done);
                }
            for (auto& e : fill_events)
                if (e) cudaEventDestroy(e);
            if (fill_stream) cudaStreamDestroy(fill_stream);
            if (fill_scratch) cudaFree(fill_scratch);
            if (fill_staging) cudaFreeHost(fill_staging);
            if (region) cudaFree(region);
        }
        if (arena) sb_arena_destroy(arena);
    }

    int release_fields(Req* q, bool keep_out, bool keep_in) {
        const FieldSpec* specs = q->r.op == SB_OP_HDIFF ? kHdiffFields : kVadvFields;
        bool any_kept = false;
        for (int f = 0; f < q->nfields; ++f) {
            if (!q->field[f]) continue;
            if (specs[f].input ? keep_in : keep_out) {
                any_kept = true;
                continue;
            }
            const int rc = sb_arena_free(arena, q->field[f]);
            if (rc) return rc;
            q->field[f] = 0;
        }
        q->kept = any_kept;
        return SB_OK;
    }

    int poll(double now) {
        for (int form = 0; form < kForms; ++form) {
            for (auto& s : slots[form]) {
                if (!s.busy) continue;
                if (sim()) {
                    if (!s.sim_done) continue;
                } else {
                    const cudaError_t e = cudaEventQuery(s.done);
                    if (e == cudaErrorNotReady) continue;
                    if (e != cudaSuccess) return fail(SB_ERR_CUDA, "server: %s", cudaGetErrorString(e));
                }
                for (Req* q : s.reqs) {
                    q->completed = now;
                    const int rc = release_fields(q, cfg.keep & 1, cfg.keep & 2);
                    if (rc) return rc;
                    completed.push_back(sb_completion{q->r.id, q->r.arrival, q->admitted, q->launched, q->completed});
                    if (!q->kept) reqs.erase(q->r.id);
                }
                inflight -= (int64_t)s.reqs.size();
                s.reqs.clear();
                s.busy = false;
                s.sim_done = false;
            }
        }
        return SB_OK;
    }

    int admit(double now) {
        descs.clear();
        const int cap = cfg.fill_capacity;
        while (!waiting.empty() && (int)descs.size() + 6 <= cap) {
            Req* q = waiting.front();
            const int nf = q->r.op == SB_OP_HDIFF ? 3 : 6;
            const FieldSpec* specs = q->r.op == SB_OP_HDIFF ? kHdiffFields : kVadvFields;
            const uint64_t bytes = (uint64_t)q->count() * (uint64_t)storage_size(q->r.storage);
            int got = 0;
            for (; got < nf; ++got) {
                uint64_t addr = 0;
                const int rc = sb_arena_alloc(arena, bytes, &addr);
                if (rc == SB_ERR_BUDGET) break;
                if (rc) return rc;
                q->field[got] = addr;
            }
            if (got < nf) {  // budget exhausted: wait for completions (arrival order kept)
                for (int f = 0; f < got; ++f) {
                    sb_arena_free(arena, q->field[f]);
                    q->field[f] = 0;
                }
                break;
            }
            waiting.pop_front();
            q->nfields = nf;
            for (int f = 0; f < nf; ++f) {
                if (!specs[f].input) continue;
                sb_fill_desc d{};
                d.ptr = (void*)q->field[f];
                d.count = q->count();
                d.seed = field_seed(q->r.seed, f);
                d.lo = specs[f].lo;
                d.hi = specs[f].hi;
                d.storage = q->r.storage;
                descs.push_back(d);
            }
            q->admitted = now;
            ready[form_of(q->r.storage)].push_back(q);
        }
        if (descs.empty() || sim()) return SB_OK;
        const int k = fill_next;
        fill_next = (k + 1) % kFillDepth;
        if (fill_used[k]) SB_CUDA(cudaEventSynchronize(fill_events[k]));  // normally long done
        sb_fill_desc* staging = fill_staging + (size_t)k * cap;
        std::memcpy(staging, descs.data(), descs.size() * sizeof(sb_fill_desc));
        const int rc = sb_fill_batch(staging, (int)descs.size(), fill_scratch, fill_stream);
        if (rc) return rc;
        SB_CUDA(cudaEventRecord(fill_events[k], fill_stream));
        fill_used[k] = true;
        fill_last = k;
        return SB_OK;
    }

    sb_domain domain_of(const Req* q) const {
        sb_domain d{};
        const int64_t es = storage_size(q->r.storage);
        const uint64_t off = (uint64_t)(q->interior_offset() * es);
        d.op = q->r.op;
        d.wshift_i = 1;
        d.wshift_j = 0;
        d.ni = q->r.ni;
        d.nj = q->r.nj;
        d.nk = q->r.nk;
        d.si = 1;
        d.sj = q->sx();
        d.sk = q->sx() * q->sy();
        const int nin = q->r.op == SB_OP_HDIFF ? 2 : 5;
        for (int f = 0; f < nin; ++f) d.f[f] = (const void*)(q->field[f] + off);
        d.out = (void*)(q->field[nin] + off);
        return d;
    }

    int launch_one(const Req* q, int form, cudaStream_t stream) {
        const sb_domain d = domain_of(q);
        const int compute = compute_of(form, q->r.op);
        if (q->r.op == SB_OP_HDIFF)
            return sb_hdiff(q->r.storage, compute, d.f[0], d.f[1], d.out, d.ni, d.nj, d.nk, d.si, d.sj, d.sk, nullptr,
                            stream, nullptr);
        return sb_vadv(q->r.storage, compute, d.f[0], d.f[1], d.f[2], d.f[3], d.f[4], d.out, nullptr, nullptr, d.ni,
                       d.nj, d.nk, d.si, d.sj, d.sk, 1, 0, nullptr, stream, nullptr);
    }

    int dispatch(double now) {
        for (int form = 0; form < kForms; ++form) {
            auto& queue = ready[form];
            while (!queue.empty()) {
                Slot* slot = nullptr;
                for (auto& s : slots[form])
                    if (!s.busy) {
                        slot = &s;
                        break;
                    }
                if (!slot) break;
                const int n = (int)std::min<size_t>((size_t)cfg.max_batch, queue.size());
                slot->reqs.assign(queue.begin(), queue.begin() + n);
                queue.erase(queue.begin(), queue.begin() + n);
                if (sim()) {
                    launch_log.push_back(sb_server_launch{storage_of(form), n});
                } else {
                    if (fill_last >= 0) SB_CUDA(cudaStreamWaitEvent(slot->stream, fill_events[fill_last], 0));
                    if (cfg.mode == 0) {
                        doms.clear();
                        for (const Req* q : slot->reqs) doms.push_back(domain_of(q));
                        int rc = sb_batch_set(slot->batch, doms.data(), n);
                        if (rc == SB_OK) rc = sb_batch_launch(slot->batch, slot->stream, nullptr);
                        if (rc) return rc;
                    } else {
                        for (const Req* q : slot->reqs) {
                            const int rc = launch_one(q, form, slot->stream);
                            if (rc) return rc;
                        }
                    }
                    SB_CUDA(cudaEventRecord(slot->done, slot->stream));
                }
                for (Req* q : slot->reqs) q->launched = now;
                inflight += n;
                slot->busy = true;
            }
        }
        return SB_OK;
    }
};

extern "C" {

int sb_server_create(sb_server** out, const sb_server_config* cfg_in) {
    clear_error();
    SB_CHECK(out && cfg_in, SB_ERR_INVALID, "NULL argument");
    *out = nullptr;
    sb_server_config cfg = *cfg_in;
    if (cfg.max_batch <= 0) cfg.max_batch = 64;
    if (cfg.max_nk <= 0) cfg.max_nk = 137;
    if (cfg.slots_per_form <= 0) cfg.slots_per_form = 3;
    if (cfg.fill_capacity <= 0) cfg.fill_capacity = 4096;
    if (cfg.float64_compute == 0) cfg.float64_compute = SB_F64;
    SB_CHECK(cfg.float64_compute == SB_F64 || cfg.float64_compute == SB_FIX64, SB_ERR_INVALID,
             "float64_compute must be SB_F64 or SB_FIX64");
    SB_CHECK(cfg.mode == 0 || cfg.mode == 1, SB_ERR_INVALID, "mode must be 0 (batched) or 1 (plain)");
    SB_CHECK(cfg.fill_capacity >= 6, SB_ERR_INVALID, "fill_capacity must hold one request's fields (6)");
    SB_CHECK(cfg.max_batch <= 1024, SB_ERR_INVALID, "max_batch must be at most 1024");
    const uint64_t budget = cfg.budget_bytes / kAlign * kAlign;
    SB_CHECK(budget >= kAlign, SB_ERR_INVALID, "budget_bytes must be at least %llu", (unsigned long long)kAlign);
    cfg.budget_bytes = budget;
    auto s = std::make_unique<sb_server>();
    s->cfg = cfg;
    uint64_t base = 1ull << 40;  // simulate: an address range nothing dereferences
    if (!s->sim()) {
        SB_CUDA(cudaGetDevice(&s->device));
        SB_CUDA(cudaMalloc(&s->region, budget));
        base = (uint64_t)(uintptr_t)s->region;
        SB_CUDA(cudaStreamCreateWithFlags(&s->fill_stream, cudaStreamNonBlocking));
        SB_CUDA(cudaMalloc(&s->fill_scratch, sizeof(sb_fill_desc) * (size_t)cfg.fill_capacity));
        SB_CUDA(cudaMallocHost((void**)&s->fill_staging, sizeof(sb_fill_desc) * (size_t)cfg.fill_capacity * kFillDepth));
        for (auto& e : s->fill_events) SB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    int rc = sb_arena_create(&s->arena, base, budget, kAlign);
    if (rc) return rc;
    for (int form = 0; form < kForms; ++form) {
        s->slots[form].resize(cfg.slots_per_form);
        if (s->sim()) continue;
        for (auto& slot : s->slots[form]) {
            SB_CUDA(cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking));
            SB_CUDA(cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming));
            if (cfg.mode == 0) {
                const int storage = s->storage_of(form);
                const int compute = form == 0 ? cfg.float64_compute : SB_F32;
                rc = sb_batch_create(&slot.batch, storage, compute, cfg.max_batch, cfg.max_nk, &cfg.tune);
                if (rc) return rc;
            }
        }
    }
    *out = s.release();
    return SB_OK;
}

int sb_server_destroy(sb_server* s) {
    if (s && !s->sim()) cudaDeviceSynchronize();
    delete s;
    return SB_OK;
}

int sb_server_submit(sb_server* s, const sb_request* r) {
    clear_error();
    SB_CHECK(s && r, SB_ERR_INVALID, "NULL argument");
    SB_CHECK(r->op == SB_OP_HDIFF || r->op == SB_OP_VADV, SB_ERR_INVALID, "unknown op %d", r->op);
    SB_CHECK(form_of(r->storage) >= 0, SB_ERR_INVALID, "unknown storage %d", r->storage);
    SB_CHECK(r->ni > 0 && r->nj > 0 && r->nk > 0, SB_ERR_INVALID, "empty domain");
    SB_CHECK(r->op == SB_OP_HDIFF || (r->nk >= 2 && r->nk <= s->cfg.max_nk), SB_ERR_INVALID,
             "vadv nk = %lld outside [2, max_nk = %d]", (long long)r->nk, s->cfg.max_nk);
    SB_CHECK(s->reqs.find(r->id) == s->reqs.end(), SB_ERR_INVALID, "request id %lld is in use", (long long)r->id);
    auto q = std::make_unique<Req>();
    q->r = *r;
    const int nf = r->op == SB_OP_HDIFF ? 3 : 6;
    const uint64_t one = ((uint64_t)q->count() * (uint64_t)storage_size(r->storage) + kAlign - 1) / kAlign * kAlign;
    SB_CHECK(one * (uint64_t)nf <= s->cfg.budget_bytes, SB_ERR_INVALID,
             "request %lld needs %llu bytes, more than the whole budget", (long long)r->id,
             (unsigned long long)(one * nf));
    SB_CHECK(q->count() < (1LL << 31), SB_ERR_INVALID, "request field exceeds 2^31 elements");
    Req* p = q.get();
    s->reqs.emplace(r->id, std::move(q));
    s->waiting.push_back(p);
    s->max_waiting = std::max<int64_t>(s->max_waiting, (int64_t)s->waiting.size());
    return SB_OK;
}

int sb_server_step(sb_server* s, double now, int* busy) {
    clear_error();
    SB_CHECK(s, SB_ERR_INVALID, "NULL server");
    const auto t0 = std::chrono::steady_clock::now();
    if (!s->sim()) SB_CUDA(cudaSetDevice(s->device));
    const size_t done0 = s->completed.size();
    const int64_t inflight0 = s->inflight, waiting0 = (int64_t)s->waiting.size();
    int rc = s->poll(now);
    if (rc == SB_OK) rc = s->admit(now);
    if (rc == SB_OK) rc = s->dispatch(now);
    if (s->completed.size() != done0 || s->inflight != inflight0 || (int64_t)s->waiting.size() != waiting0)
        s->work_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (busy) {
        bool any = !s->waiting.empty() || s->inflight > 0;
        for (auto& q : s->ready) any = any || !q.empty();
        *busy = any ? 1 : 0;
    }
    return rc;
}

int sb_server_take_completed(sb_server* s, sb_completion* out, int capacity, int* n) {
    SB_CHECK(s && n && (out || capacity == 0), SB_ERR_INVALID, "NULL argument");
    const int m = (int)std::min<size_t>((size_t)std::max(capacity, 0), s->completed.size());
    if (m) std::memcpy(out, s->completed.data(), sizeof(sb_completion) * (size_t)m);
    s->completed.erase(s->completed.begin(), s->completed.begin() + m);
    *n = m;
    return SB_OK;
}

int sb_server_field(sb_server* s, int64_t id, int field, void** ptr) {
    clear_error();
    SB_CHECK(s && ptr, SB_ERR_INVALID, "NULL argument");
    auto it = s->reqs.find(id);
    SB_CHECK(it != s->reqs.end(), SB_ERR_INVALID, "request %lld not held by the server", (long long)id);
    const Req* q = it->second.get();
    SB_CHECK(field >= 0 && field < q->nfields && q->field[field], SB_ERR_INVALID,
             "request %lld has no field %d (not admitted, or released)", (long long)id, field);
    *ptr = (void*)q->field[field];
    return SB_OK;
}

int sb_server_query(sb_server* s, int64_t id, sb_completion* rec) {
    clear_error();
    SB_CHECK(s && rec, SB_ERR_INVALID, "NULL argument");
    auto it = s->reqs.find(id);
    SB_CHECK(it != s->reqs.end(), SB_ERR_INVALID, "request %lld not held by the server", (long long)id);
    const Req* q = it->second.get();
    *rec = sb_completion{q->r.id, q->r.arrival, q->admitted, q->launched, q->completed};
    return SB_OK;
}

int sb_server_release(sb_server* s, int64_t id) {
    clear_error();
    SB_CHECK(s, SB_ERR_INVALID, "NULL server");
    auto it = s->reqs.find(id);
    SB_CHECK(it != s->reqs.end() && it->second->completed >= 0.0, SB_ERR_INVALID,
             "request %lld is not a completed request with kept fields", (long long)id);
    int rc = s->release_fields(it->second.get(), false, false);
    if (rc) return rc;
    s->reqs.erase(it);
    return SB_OK;
}

int sb_server_stats(sb_server* s, sb_server_state* st) {
    SB_CHECK(s && st, SB_ERR_INVALID, "NULL argument");
    uint64_t in_use = 0, peak = 0, largest = 0, blocks = 0;
    const int rc = sb_arena_stats(s->arena, &in_use, &peak, &largest, &blocks);
    if (rc) return rc;
    st->budget_bytes = s->cfg.budget_bytes;
    st->in_use_bytes = in_use;
    st->peak_bytes = peak;
    st->waiting = (int64_t)s->waiting.size();
    st->ready = 0;
    for (auto& q : s->ready) st->ready += (int64_t)q.size();
    st->inflight = s->inflight;
    st->max_waiting = s->max_waiting;
    st->work_seconds = s->work_seconds;
    st->busy_slots = 0;
    for (auto& forms : s->slots)
        for (auto& slot : forms) st->busy_slots += slot.busy ? 1 : 0;
    return SB_OK;
}

int sb_server_debug_complete(sb_server* s) {
    SB_CHECK(s && s->sim(), SB_ERR_INVALID, "only a simulating server completes work on request");
    for (auto& forms : s->slots)
        for (auto& slot : forms)
            if (slot.busy) slot.sim_done = true;
    return SB_OK;
}

int sb_server_debug_launches(sb_server* s, sb_server_launch* out, int capacity, int* n) {
    SB_CHECK(s && n && (out || capacity == 0), SB_ERR_INVALID, "NULL argument");
    const int m = (int)std::min<size_t>((size_t)std::max(capacity, 0), s->launch_log.size());
    if (m) std::memcpy(out, s->launch_log.data(), sizeof(sb_server_launch) * (size_t)m);
    *n = (int)s->launch_log.size();
    return SB_OK;
}

}  // extern "C"
