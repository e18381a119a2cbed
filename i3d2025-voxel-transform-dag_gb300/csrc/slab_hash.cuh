// slab_hash.cuh — warp-cooperative slab hash table over a bitmap slab allocator, for the global
// content tables of the streamed scene build (the GPU hash-DAG deduplication that merges chunk after
// chunk into one DAG).
//
// Design precedent: the renderer's GPU hash DAG (renderer/src/dags/my_gpu_dags/my_gpu_hash_dag/
// hash_tables/gpu_hash_table_base.h:172-219; dynamic_slab_alloc.h:61-125): buckets of 32-word slabs
// that a warp reads in one step, chains grown by slabs taken from bitmap super-blocks. This is a
// restatement of that design, not of its code, with two differences the reference lacks: every loop is
// bounded (a full pool or an over-long chain sets TDAG_ERR_ALLOC / TDAG_ERR_TABLE_FULL in the status
// word and returns; the reference's allocator retries forever, dynamic_slab_alloc.h:74-115), and the
// host regrows the pool and resumes instead.
//
// Layout: slab s is 32 u64 words. Words 0..30 hold entries (tag << 32 | id, tag = the top 32 bits of the
// key's fingerprint, id = the item's index in the table's item array), all ones when empty; word 31
// holds the index of the next slab, all ones for none. Slabs 0..numBuckets-1 are the bucket heads;
// the others are allocated through a bitmap (bit i of word j: slab numBuckets + 32 j + i in use), 32
// words (1024 slabs) per super-block. Entries of a slab fill from word 0 upwards and are never
// removed, so a slab with an empty word ends its chain's entries, and a slab is linked to a successor
// only once it is full.
#pragma once
#include "common.cuh"

namespace tdag {

constexpr uint64_t kSlabEmpty = ~0ull;
constexpr uint32_t kSlabNone = 0xFFFFFFFFu;
constexpr uint32_t kSlabEntries = 31;
constexpr uint32_t kSlabMaxChain = 1u << 16; // slabs walked before a chain counts as full
constexpr uint32_t kSlabAllocAttempts = 64; // super-blocks tried per allocation

struct SlabPoolView {
    unsigned long long* slabs; // numSlabs x 32
    uint32_t numBuckets;
    uint32_t numSlabs; // heads + allocatable
    uint32_t* bitmap; // ceil((numSlabs - numBuckets) / 32) words, bits past the end preset to 1
    uint32_t bitmapWords;
};

__device__ __forceinline__ uint64_t slabLoad(const unsigned long long* p) { return *reinterpret_cast<const volatile unsigned long long*>(p); }

// Warp-wide (all 32 lanes): a free slab, or kSlabNone with TDAG_ERR_ALLOC recorded.
__device__ uint32_t slabAlloc(const SlabPoolView& p, uint32_t seed, uint32_t* status)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t superBlocks = (p.bitmapWords + 31) / 32;
    for (uint32_t attempt = 0; attempt < kSlabAllocAttempts && superBlocks; ++attempt) {
        const uint32_t sb = (uint32_t)(mix64((uint64_t)seed * 0x9E3779B97F4A7C15ull + attempt) % superBlocks);
        const uint32_t w = sb * 32 + lane;
        uint32_t freeBits = w < p.bitmapWords ? ~*reinterpret_cast<volatile uint32_t*>(&p.bitmap[w]) : 0u;
        // every round either takes a slab or clears at least one bit of one lane's free set
        for (uint32_t round = 0; round < 32 * 33; ++round) {
            const unsigned withFree = __ballot_sync(0xffffffffu, freeBits != 0);
            if (!withFree)
                break;
            const int src = __ffs(withFree) - 1;
            uint32_t got = kSlabNone;
            if ((int)lane == src) {
                const uint32_t bit = (uint32_t)(__ffs(freeBits) - 1);
                const uint32_t old = atomicOr(&p.bitmap[w], 1u << bit);
                if (!(old & (1u << bit)))
                    got = p.numBuckets + 32 * w + bit;
                freeBits = ~(old | (1u << bit));
            }
            got = __shfl_sync(0xffffffffu, got, src);
            if (got != kSlabNone)
                return got;
        }
    }
    if (lane == 0)
        setDeviceError(status, TDAG_ERR_ALLOC, 420);
    return kSlabNone;
}

__device__ __forceinline__ void slabFree(const SlabPoolView& p, uint32_t slab)
{
    const uint32_t i = slab - p.numBuckets;
    atomicAnd(&p.bitmap[i / 32], ~(1u << (i % 32)));
}

// Warp-wide lookup of a W-word key (lane k < W holds word k in `myWord`) in its bucket's chain; the
// item array holds W words per id. Returns the id, or kSlabNone when absent. Read-only phase: no
// insertion runs concurrently.
template <int W>
__device__ uint32_t slabFind(const SlabPoolView& p, uint32_t bucket, uint32_t tag, uint64_t myWord, const uint64_t* __restrict__ items,
    uint32_t* status)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t slab = bucket;
    for (uint32_t step = 0; step < kSlabMaxChain; ++step) {
        const uint64_t e = __ldcg(&p.slabs[(uint64_t)slab * 32 + lane]);
        unsigned cand = __ballot_sync(0xffffffffu, lane < kSlabEntries && e != kSlabEmpty && (uint32_t)(e >> 32) == tag);
        while (cand) {
            const int src = __ffs(cand) - 1;
            const uint32_t id = (uint32_t)__shfl_sync(0xffffffffu, e, src);
            const bool eq = lane >= (uint32_t)W || items[(uint64_t)id * W + lane] == myWord;
            if (__all_sync(0xffffffffu, eq))
                return id;
            cand &= cand - 1;
        }
        if (__ballot_sync(0xffffffffu, lane < kSlabEntries && e == kSlabEmpty))
            return kSlabNone;
        const uint64_t next = __shfl_sync(0xffffffffu, e, 31);
        if (next == kSlabEmpty)
            return kSlabNone;
        slab = (uint32_t)next;
    }
    if (lane == 0)
        setDeviceError(status, TDAG_ERR_TABLE_FULL, 421);
    return kSlabNone;
}

// Warp-wide insertion of an entry whose key is not in the table and is inserted by no other warp.
// Returns false when the pool ran out (TDAG_ERR_ALLOC) or the chain is over-long (TDAG_ERR_TABLE_FULL);
// the caller can retry after the host has grown the pool.
__device__ bool slabInsert(const SlabPoolView& p, uint32_t bucket, uint64_t entry, uint32_t seed, uint32_t* status)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t slab = bucket;
    for (uint32_t step = 0; step < kSlabMaxChain; ++step) {
        unsigned long long* row = p.slabs + (uint64_t)slab * 32;
        const uint64_t e = slabLoad(&row[lane]);
        const unsigned empty = __ballot_sync(0xffffffffu, lane < kSlabEntries && e == kSlabEmpty);
        if (empty) {
            const int src = __ffs(empty) - 1;
            int ok = 0;
            if ((int)lane == src)
                ok = atomicCAS(&row[src], kSlabEmpty, (unsigned long long)entry) == kSlabEmpty;
            if (__shfl_sync(0xffffffffu, ok, src))
                return true;
            continue; // another warp took that word: read the slab again
        }
        const uint64_t next = __shfl_sync(0xffffffffu, e, 31);
        if (next != kSlabEmpty) {
            slab = (uint32_t)next;
            continue;
        }
        const uint32_t fresh = slabAlloc(p, seed + step, status);
        if (fresh == kSlabNone)
            return false;
        p.slabs[(uint64_t)fresh * 32 + lane] = kSlabEmpty;
        __threadfence();
        unsigned long long old = 0;
        if (lane == 31)
            old = atomicCAS(&row[31], kSlabEmpty, (unsigned long long)fresh);
        old = __shfl_sync(0xffffffffu, old, 31);
        if (old != kSlabEmpty) { // another warp linked first: return ours, follow theirs
            if (lane == 0)
                slabFree(p, fresh);
            slab = (uint32_t)old;
        } else {
            slab = fresh;
        }
    }
    if (lane == 0)
        setDeviceError(status, TDAG_ERR_TABLE_FULL, 422);
    return false;
}

} // namespace tdag
