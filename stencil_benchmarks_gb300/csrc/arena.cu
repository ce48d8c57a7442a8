// Device-memory arena for the serving path: one caller-provided region (one
// cudaMalloc up front), carved into blocks by a host-side best-fit allocator
// with coalescing.  Allocating and freeing request fields then costs no CUDA
// call -- cudaMalloc/cudaFree synchronise the whole device, which would
// serialise every batch in flight.  The arena only does address arithmetic:
// it never touches the memory, so it can be exercised without a GPU.
#include <cstdint>
#include <map>
#include <mutex>
#include <unordered_map>

#include "common.cuh"

struct sb_arena {
    uint64_t base = 0, bytes = 0, align = 256;
    std::map<uint64_t, uint64_t> free_by_addr;        // address -> size
    std::multimap<uint64_t, uint64_t> free_by_size;   // size -> address
    std::unordered_map<uint64_t, uint64_t> used;      // address -> size
    uint64_t in_use = 0, peak = 0;
    std::mutex mutex;

    void insert_free(uint64_t addr, uint64_t size) {
        free_by_addr[addr] = size;
        free_by_size.emplace(size, addr);
    }
    void erase_free(std::map<uint64_t, uint64_t>::iterator it) {
        auto range = free_by_size.equal_range(it->second);
        for (auto s = range.first; s != range.second; ++s) {
            if (s->second == it->first) {
                free_by_size.erase(s);
                break;
            }
        }
        free_by_addr.erase(it);
    }
};

using namespace sb;

extern "C" {

int sb_arena_create(sb_arena** arena, uint64_t base, uint64_t bytes, uint64_t align) {
    clear_error();
    SB_CHECK(arena, SB_ERR_INVALID, "arena is NULL");
    SB_CHECK(align >= 1 && (align & (align - 1)) == 0, SB_ERR_INVALID, "alignment must be a power of two");
    SB_CHECK(base % align == 0, SB_ERR_INVALID, "base is not aligned to %llu", (unsigned long long)align);
    sb_arena* a = new sb_arena();
    a->base = base;
    a->bytes = bytes / align * align;
    a->align = align;
    if (a->bytes) a->insert_free(base, a->bytes);
    *arena = a;
    return SB_OK;
}

int sb_arena_destroy(sb_arena* arena) {
    delete arena;
    return SB_OK;
}

int sb_arena_alloc(sb_arena* arena, uint64_t bytes, uint64_t* address) {
    SB_CHECK(arena && address, SB_ERR_INVALID, "NULL argument");
    const uint64_t size = bytes == 0 ? arena->align : (bytes + arena->align - 1) / arena->align * arena->align;
    std::lock_guard<std::mutex> lock(arena->mutex);
    auto it = arena->free_by_size.lower_bound(size);  // best fit: smallest block that is large enough
    if (it == arena->free_by_size.end()) {
        return fail(SB_ERR_BUDGET, "arena: no free block of %llu bytes (%llu of %llu in use)",
                    (unsigned long long)size, (unsigned long long)arena->in_use, (unsigned long long)arena->bytes);
    }
    const uint64_t addr = it->second, have = it->first;
    arena->erase_free(arena->free_by_addr.find(addr));
    if (have > size) arena->insert_free(addr + size, have - size);
    arena->used[addr] = size;
    arena->in_use += size;
    if (arena->in_use > arena->peak) arena->peak = arena->in_use;
    *address = addr;
    return SB_OK;
}

int sb_arena_free(sb_arena* arena, uint64_t address) {
    SB_CHECK(arena, SB_ERR_INVALID, "arena is NULL");
    std::lock_guard<std::mutex> lock(arena->mutex);
    auto u = arena->used.find(address);
    SB_CHECK(u != arena->used.end(), SB_ERR_INVALID, "arena: %#llx is not an allocated block",
             (unsigned long long)address);
    uint64_t addr = address, size = u->second;
    arena->used.erase(u);
    arena->in_use -= size;
    auto next = arena->free_by_addr.find(addr + size);
    if (next != arena->free_by_addr.end()) {  // merge with the following free block
        size += next->second;
        arena->erase_free(next);
    }
    auto prev = arena->free_by_addr.lower_bound(addr);
    if (prev != arena->free_by_addr.begin()) {  // merge with the preceding free block
        --prev;
        if (prev->first + prev->second == addr) {
            addr = prev->first;
            size += prev->second;
            arena->erase_free(prev);
        }
    }
    arena->insert_free(addr, size);
    return SB_OK;
}

int sb_arena_stats(sb_arena* arena, uint64_t* in_use, uint64_t* peak, uint64_t* largest_free, uint64_t* free_blocks) {
    SB_CHECK(arena, SB_ERR_INVALID, "arena is NULL");
    std::lock_guard<std::mutex> lock(arena->mutex);
    if (in_use) *in_use = arena->in_use;
    if (peak) *peak = arena->peak;
    if (largest_free) *largest_free = arena->free_by_size.empty() ? 0 : arena->free_by_size.rbegin()->first;
    if (free_blocks) *free_blocks = arena->free_by_addr.size();
    return SB_OK;
}

}  // extern "C"
