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
    void* stage = nullptr; // pinned staging buffer of host-bound results (grown on demand)
    size_t stageBytes = 0;
    int pageableAccess = -1; // cudaDevAttrPageableMemoryAccess of the device (-1: not queried yet)

    uint32_t tableRegrows = 0; // class-table doublings of the current build
    unsigned char* noAllocScratch = nullptr; // device address of the no-allocation matcher's array
    std::shared_ptr<StreamState> streamState; // owns `stream` together with the buffers allocated on it

    // Synchronise the stream, read the device status word, throw on a recorded error.
    void checkStatus(const std::string& where);
    // Synchronise, read and clear the device status word; returns its error code (0: none).
    uint32_t takeStatus(uint32_t* aux = nullptr);
    // Slots of a class table for n items at the tuned load (power of two, at least n / load + 16).
    uint64_t classTableCapacity(uint64_t n) const;
    uint32_t tableRegrowLimit() const { return tuning.table_regrow_limit ? tuning.table_regrow_limit : 4u; }
};

// Runs attempt(capacity) — a class-table insert and the kernels that read the table — and then
// checks the device status. A table whose bounded probes ran out (TDAG_ERR_TABLE_FULL) is doubled
// and the attempt rerun, up to the context's regrow limit; each doubling is counted in
// ctx.tableRegrows. Any other device error, or a table still full at the limit, throws. The table
// capacity changes no result: class membership and class minima do not depend on slot positions.
template <typename F>
void withClassTable(Context& ctx, uint64_t n, const std::string& where, F&& attempt)
{
    uint64_t cap = ctx.classTableCapacity(n);
    for (uint32_t regrows = 0;; ++regrows) {
        attempt(cap);
        uint32_t aux = 0;
        const uint32_t code = ctx.takeStatus(&aux);
        if (code == 0)
            return;
        if (code == TDAG_ERR_TABLE_FULL && regrows < ctx.tableRegrowLimit()) {
            cap *= 2;
            ++ctx.tableRegrows;
            continue;
        }
        throw Error((int)code, where + ": device reported error " + std::to_string(code) + " (aux " + std::to_string(aux) + ")" +
                (code == TDAG_ERR_TABLE_FULL ? " after " + std::to_string(regrows) + " table regrows" : std::string()));
    }
}

// Device-resident view of an EditStructure<void, uint32_t>, or of a batch of them concatenated level
// by level in grid order (child indices then address the concatenated level below). For a batch,
// segOff[l] holds each grid's first item at level l (size numGrids + 1; level 2 = leaves) and
// gridOf[l] the grid of every item. A single structure is the batch of one (numGrids == 1, no
// segment arrays).
struct DeviceSvdag {
    uint32_t resolution = 0, rootLevel = 0;
    const uint32_t* nodes[TDAG_MAX_LEVELS] {};
    uint64_t nodeCounts[TDAG_MAX_LEVELS] {};
    const uint64_t* leaves = nullptr;
    uint64_t leafCount = 0;
    uint32_t numGrids = 1;
    std::vector<uint64_t> segOff[TDAG_MAX_LEVELS];
    const uint32_t* gridOf[TDAG_MAX_LEVELS] {};
    // StaticStructure input (constructStaticTransformDAG): the hierarchical pass groups nodes by a
    // hash of their children's word offsets in the packed levels instead of their indices.
    bool staticOffsets = false;
};

// Grid segmentation of a list of items (host offsets + device per-item grid ids and offsets).
struct Segments {
    uint32_t numGrids = 1;
    std::vector<uint64_t> off; // size numGrids + 1
    const uint32_t* gridOf = nullptr; // device, per item; null for a single grid
    const uint32_t* offDev = nullptr; // device copy of off (u32); null for a single grid
    bool batched() const { return numGrids > 1; }
};

struct HierOutput {
    std::vector<DevBuf<uint64_t>> levels; // per level: unique nodes x 8 TransformPointers (grid-local child handles)
    DevBuf<uint64_t> leaves; // unique leaves
    DevBuf<uint32_t> midInv; // new -> old index at the mid level
    std::vector<std::vector<uint64_t>> handleOff; // per level: first output item of each grid (numGrids + 1)
};

struct MatchOutput {
    DevBuf<uint64_t> mapping; // per item: TransformPointer into its grid's unique list
    DevBuf<uint32_t> uniques; // item positions kept (ascending)
    uint32_t numUnique = 0;
    std::vector<uint64_t> uniqueOff; // first kept item of each grid in `uniques` (numGrids + 1)
};

// Per-grid salt folded into corner-hash keys of batched builds (grid 0: no salt, so a single grid's
// table is exactly the unsalted one).
__host__ __device__ __forceinline__ uint64_t gridSalt(uint32_t g) { return g ? mix64(0x632BE59BD9B4E019ull + g) : 0ull; }

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
void preloadFillKernels(); // loads the fill kernels' code now (primitives or hierarchical TU)
void prepareNoAlloc(Context& ctx); // matcher.cu; called by tdag_ctx_create

HierOutput runHierarchical(Context& ctx, const DeviceSvdag& in, const tdag_config& cfg, uint32_t midLevel, tdag_stats* stats);

// findDuplicatesAmongFlattenedItems on n dense grids of level `level` (device pointer, n x W words).
// seg (optional) splits the items into independent grids of a batch. sources (optional, device, a
// single grid only) restricts the searching sources to numSources item indices: every item is still
// a target and its own candidate, but only the listed items probe (the learned-proposal mode).
MatchOutput runMatcher(Context& ctx, uint32_t level, const uint64_t* grids, uint32_t n, const tdag_config& cfg, tdag_level_stats* stats,
    const Segments* seg = nullptr, const uint32_t* sources = nullptr, uint32_t numSources = 0);

// Throws TDAG_ERR_ARG unless the context's device can dereference p: device memory of that device,
// managed memory, mapped pinned host memory, or pageable host memory on systems where the GPU reads
// it directly (cudaDevAttrPageableMemoryAccess). Null passes (callers check counts). (build.cu)
void requireDeviceAccessible(Context& c, const void* p, const char* what);
void requireDeviceView(Context& c, const tdag_svdag_view& v);

// Device -> host copies of several arrays through the context's pinned staging buffer; complete on
// return (build.cu).
struct Download {
    void* dst;
    const void* src;
    size_t bytes;
};
void downloadStaged(Context& c, const std::vector<Download>& items);

// Segment helpers: per-item grid ids from offsets, per-grid counts of a grid-id list.
void segmentIds(const uint32_t* offDev, uint32_t numGrids, uint64_t n, uint32_t* out, cudaStream_t s);
std::vector<uint64_t> countPerGrid(const uint32_t* gridIds, const uint32_t* idx, uint64_t n, uint32_t numGrids, cudaStream_t s);

} // namespace tdag
