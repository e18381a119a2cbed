// internal.cuh — library-internal types shared by the .cu translation units of libtdag.so.
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "common.cuh"

namespace tdag {

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    TransformTables* tables = nullptr; // device copy
    uint32_t* status = nullptr; // device status words [4]
    uint32_t* hostStatus = nullptr; // pinned mirror
    tdag_tuning tuning {};
    int numSMs = 0;
    cudaEvent_t ev[8] {};

    // Synchronise the stream, read the device status word, throw on a recorded error.
    void checkStatus(const std::string& where);
};

// Device-resident view of an EditStructure<void, uint32_t>.
struct DeviceSvdag {
    uint32_t resolution = 0, rootLevel = 0;
    const uint32_t* nodes[TDAG_MAX_LEVELS] {};
    uint64_t nodeCounts[TDAG_MAX_LEVELS] {};
    const uint64_t* leaves = nullptr;
    uint64_t leafCount = 0;
};

struct HierOutput {
    std::vector<DevBuf<uint64_t>> levels; // per level: unique nodes x 8 TransformPointers
    DevBuf<uint64_t> leaves; // unique leaves
    DevBuf<uint32_t> midInv; // new -> old index at the mid level
};

struct MatchOutput {
    DevBuf<uint64_t> mapping; // per item: TransformPointer into the unique list
    DevBuf<uint32_t> uniques; // item positions kept (ascending)
    uint32_t numUnique = 0;
};

inline uint64_t allowedMask(const tdag_config& c)
{
    uint64_t m = 0;
    for (uint32_t t = 0; t < 48; ++t) {
        if (!c.axis_permutation && (t >> 3) != 0)
            continue;
        if (!c.symmetry && (t & 7) != 0)
            continue;
        m |= 1ull << t;
    }
    return m;
}

void fillU64(uint64_t* p, uint64_t v, size_t n, cudaStream_t s);
void fillU32(uint32_t* p, uint32_t v, size_t n, cudaStream_t s);

HierOutput runHierarchical(Context& ctx, const DeviceSvdag& in, const tdag_config& cfg, uint32_t midLevel, tdag_stats* stats);

// findDuplicatesAmongFlattenedItems on n dense grids of level `level` (device pointer, n x W words).
MatchOutput runMatcher(Context& ctx, uint32_t level, const uint64_t* grids, uint32_t n, const tdag_config& cfg, tdag_level_stats* stats);

} // namespace tdag
