// encode16.cu — the .tdag16 encoder on the device: constructTransformDAG16(EditStructure<void,
// TransformPointer>, ...) (tools/svdag_encoding/src/transform_dag_encoding.cpp:240-497) and the
// TransformDAG16 file layout (:1023-1030).
//
// Two passes over the levels of a transform DAG:
//   1. top-down, sortByReferenceCount (pointer_encoding.h:27-72): every level below the root is
//      reordered by how often the (already reordered) level above references each item, descending,
//      with unreferenced items dropped and the parents' child indices remapped;
//   2. bottom-up, per node level: child indices become u16 offsets into the encoded child level; the
//      distinct child pointers are counted and ordered by count (descending); each gets its encoded
//      form (Huffman-coded pointer type or the plain layout) and is stored inline in the node or in
//      the level's pointer table; nodes are written as a u16 child mask followed by 1-3 u16 per child.
//
// How items with equal counts are ordered decides the file bytes (not the voxels, sizes or Huffman
// tables). The reference leaves it to std::sort (pass 1, pointer_encoding.h:49) and to the iteration
// order of a std::unordered_map followed by std::sort (pass 2, transform_dag_encoding.cpp:276-295).
//  * TDAG16_TIES_REFERENCE (default): those two steps run on the host, with libstdc++'s std::sort and
//    std::unordered_map, the reference's hash of a TransformPointer and the reference's insertion
//    sequence; everything else stays on the device. The bytes equal the reference's as built with
//    GCC and the serial parallel-algorithm backend (a TBB build may order ties differently).
//  * TDAG16_TIES_CANONICAL: ties by ascending item index (pass 1) and ascending 64-bit pointer value
//    (pass 2), both from stable radix sorts on the device, with no host step.
//
// Everything else is integer work on small arrays (a few bytes per node) dominated by radix sorts;
// the other host step per level is the 384-symbol length-limited Huffman code (package-merge), which
// is tiny and fixed-size.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <memory_resource>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "internal.cuh"
#include "tdag16.h"

namespace tdag {
namespace {

constexpr uint32_t kMaxTypes = 384; // 8 mirrors x 6 permutations x 8 translation-axis sets
constexpr uint32_t kMaxCodeLen = 16; // createLengthLimitedHuffmanCodeTable(..., 16)
constexpr uint32_t kSmallTable = 0xFFFF; // pointer tables up to this size take 16-bit indices

struct PointerCode {
    uint64_t code;
    uint32_t bits;
    uint32_t pad;
};

// ------------------------------------------------------------------------------------------------
// Host: length-limited Huffman code by package-merge (huffman.cpp:100-170; Moffat 2019, alg. 3).
// Items of a level are kept in the reference's total order (frequency, leaves before packages,
// leaves by symbol, packages by their two members in that same order), the 2n-2 smallest of the top
// level are chosen, and chosen packages select the 2k smallest of the level below. A package's
// members are named by their positions in the sorted level below, so comparing members is comparing
// positions. Code words are assigned canonically in order of increasing length (huffman.cpp:78-98;
// std::sort, like the reference, so that the order of equal lengths is the same) and bit-reversed
// for LSB-first decoding (huffman.cpp:172-182).
// ------------------------------------------------------------------------------------------------
struct Pm {
    uint64_t freq;
    int32_t symbol; // -1: package of the items at positions (a, b) of the sorted level below
    int32_t a, b;
};
inline bool pmLess(const Pm& x, const Pm& y)
{
    if (x.freq != y.freq)
        return x.freq < y.freq;
    const bool xl = x.symbol >= 0, yl = y.symbol >= 0;
    if (xl != yl)
        return xl;
    if (xl)
        return x.symbol < y.symbol;
    return x.a != y.a ? x.a < y.a : x.b < y.b;
}
std::vector<PointerCode> huffmanCodes(const std::vector<uint64_t>& freq, uint32_t maxCodeLen = kMaxCodeLen, bool lsbFirst = true)
{
    const uint32_t n = (uint32_t)freq.size();
    TDAG_CHECK(n >= 1 && maxCodeLen >= 1 && maxCodeLen <= 32, TDAG_ERR_ARG, "Huffman code: empty alphabet or length limit outside 1..32");
    struct {
        std::vector<std::vector<Pm>> lv;
    } pm;
    pm.lv.resize(maxCodeLen);
    // The leaves, sorted once, start every level. The packages of a level pair up consecutive items of
    // the sorted level below, so they are already in order (non-decreasing sums, increasing positions),
    // and each level is the merge of the two sorted lists in the same total order.
    std::vector<Pm> leaves(n);
    for (uint32_t s = 0; s < n; ++s)
        leaves[s] = { freq[s], (int32_t)s, -1, -1 };
    std::sort(leaves.begin(), leaves.end(), pmLess);
    pm.lv[0] = leaves;
    std::vector<Pm> packs;
    for (uint32_t l = 1; l < maxCodeLen; ++l) {
        const auto& below = pm.lv[l - 1];
        packs.clear();
        for (size_t i = 0; i + 1 < below.size(); i += 2)
            packs.push_back({ below[i].freq + below[i + 1].freq, -1, (int32_t)i, (int32_t)(i + 1) });
        auto& cur = pm.lv[l];
        cur.resize(packs.size() + leaves.size());
        std::merge(leaves.begin(), leaves.end(), packs.begin(), packs.end(), cur.begin(), pmLess);
    }
    std::vector<uint32_t> len(n, 0);
    size_t take = 2 * (size_t)n - 2;
    for (int l = (int)maxCodeLen - 1; l >= 0 && take > 0; --l) {
        const auto& items = pm.lv[l];
        TDAG_CHECK(take <= items.size(), TDAG_ERR_ARG, "Huffman code length limit too small");
        size_t packages = 0;
        for (size_t i = 0; i < take; ++i) {
            if (items[i].symbol >= 0)
                ++len[items[i].symbol];
            else
                ++packages;
        }
        take = 2 * packages;
    }
    uint64_t kraft = 0;
    for (uint32_t l : len)
        kraft += 1ull << (32 - l);
    TDAG_CHECK(kraft <= (1ull << 32), TDAG_ERR_ARG, "Huffman code lengths violate the Kraft inequality");
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [&](uint32_t l, uint32_t r) { return len[l] < len[r]; });
    const uint32_t maxLen = *std::max_element(len.begin(), len.end());
    std::vector<PointerCode> codes(n);
    uint64_t next = 0;
    for (uint32_t s : order) {
        const uint64_t msb = next >> (maxLen - len[s]);
        uint64_t lsb = 0;
        for (uint32_t i = 0; i < len[s]; ++i)
            lsb |= ((msb >> i) & 1) << (len[s] - 1 - i);
        codes[s] = { lsbFirst ? lsb : msb, len[s], 0 };
        next += 1ull << (maxLen - len[s]);
    }
    return codes;
}

// ------------------------------------------------------------------------------------------------
// Host: the reference's order of equal counts (TDAG16_TIES_REFERENCE).
// ------------------------------------------------------------------------------------------------
// std::hash<TransformPointer> (transform_dag.h:412-433): hash_combine (hash.h:10-15) over ptr, the
// three mirror flags, the three permutation entries and the three translations, each through the
// identity std::hash of its type; the int translations sign-extend to size_t. The call is not
// noexcept, like the reference's, so libstdc++ caches the hash codes in the nodes as it does there.
struct ReferencePointerHash {
    size_t operator()(uint64_t tp) const
    {
        uint64_t seed = hashCombine(0, tpPtr(tp));
        for (int k = 0; k < 3; ++k)
            seed = hashCombine(seed, (tp >> (37 + k)) & 1);
        for (int k = 0; k < 3; ++k)
            seed = hashCombine(seed, (tp >> (40 + 2 * k)) & 3);
        for (int k = 0; k < 3; ++k)
            seed = hashCombine(seed, (uint64_t)(int64_t)tpT(tp, k));
        return (size_t)seed;
    }
};

// sortByReferenceCount's order (pointer_encoding.h:46-49): the indices 0..n-1 under std::sort by
// count, descending. Unreferenced items (count 0) come last; the caller keeps the first `kept`.
uint32_t referenceCountOrder(const std::vector<uint32_t>& counts, std::vector<uint32_t>& order)
{
    order.resize(counts.size());
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [&](uint32_t l, uint32_t r) { return counts[l] > counts[r]; });
    uint32_t kept = 0;
    while (kept < order.size() && counts[order[kept]] != 0)
        ++kept;
    return kept;
}

// The distinct child pointers of a level in the reference's order (transform_dag_encoding.cpp:276-295):
// counted in a std::unordered_map in node order, children 0..7, then iterated and std::sort-ed by
// count, descending. The map's iteration order depends only on which keys it holds when, i.e. on the
// sequence of first occurrences and their hash codes: a repeated key changes nothing but its count.
// So the device hands over the distinct pointers in first-occurrence order (values, counts, run ids)
// and the host inserts each once, into the same container with the same hash, and sorts the same
// way; std::sort's moves depend only on its comparisons, so sorting (count, run id) pairs permutes
// exactly as the reference's (count, pointer) pairs. Node storage comes from an arena: the iteration
// order does not depend on the allocator. Returns the run ids in the reference's order.
std::vector<uint32_t> referencePointerOrder(const std::vector<uint64_t>& firstValues, const std::vector<uint32_t>& firstRuns,
    const std::vector<uint32_t>& runCount)
{
    std::pmr::monotonic_buffer_resource arena(firstValues.size() * 48 + 4096);
    std::pmr::unordered_map<uint64_t, uint32_t, ReferencePointerHash> runOf(&arena);
    for (size_t k = 0; k < firstValues.size(); ++k)
        runOf[firstValues[k]] = firstRuns[k];
    std::vector<std::pair<uint32_t, uint32_t>> byCount; // (count, run)
    byCount.reserve(runOf.size());
    for (const auto& [tp, run] : runOf)
        byCount.push_back({ runCount[run], run });
    std::sort(byCount.begin(), byCount.end(), [](const auto& l, const auto& r) { return l.first > r.first; });
    std::vector<uint32_t> out(byCount.size());
    for (size_t i = 0; i < byCount.size(); ++i)
        out[i] = byCount[i].second;
    return out;
}

// ------------------------------------------------------------------------------------------------
// Device helpers.
// ------------------------------------------------------------------------------------------------
struct EncodeParams {
    uint32_t childLevel;
    uint32_t sym, perm, trans, maxTransLevel;
    uint32_t pointerTables, huffman;
};

__device__ __forceinline__ uint32_t tpPermCode(uint64_t v) // encodeAxisPermutation: 2*p0 + (p2 < p1)
{
    const uint32_t p0 = (uint32_t)(v >> 40) & 3, p1 = (uint32_t)(v >> 42) & 3, p2 = (uint32_t)(v >> 44) & 3;
    return 2 * p0 + (p2 < p1 ? 1u : 0u);
}
__device__ __forceinline__ bool tpHasTransform(uint64_t v) // transform_dag.h:115-130
{
    return tpSym(v) != 0 || ((v >> 40) & 63) != (0u | 1u << 2 | 2u << 4) || tpT(v, 0) != 0 || tpT(v, 1) != 0 || tpT(v, 2) != 0;
}
// Pointer type: [perm code][mirror bits][non-zero translation axes] (transform_dag_encoding.cpp:124-140).
__device__ __forceinline__ uint32_t pointerType(uint64_t v, const EncodeParams& p)
{
    uint32_t out = 0;
    if (p.perm)
        out = tpPermCode(v);
    if (p.sym)
        out = (out << 3) | tpSym(v);
    if (p.trans && p.childLevel <= p.maxTransLevel)
        out = (out << 3) | (tpT(v, 0) != 0 ? 1u : 0u) | (tpT(v, 1) != 0 ? 2u : 0u) | (tpT(v, 2) != 0 ? 4u : 0u);
    return out;
}
// Encoded pointer (transform_dag_encoding.cpp:320-380).
__device__ __forceinline__ uint64_t encodePointer(uint64_t v, const EncodeParams& p, const PointerCode* codes)
{
    const uint32_t tb = p.childLevel + 1;
    const int bias = 1 << p.childLevel;
    uint64_t e = tpPtr(v);
    if (p.huffman) {
        const PointerCode c = codes[pointerType(v, p)];
        for (int k = 0; k < 3; ++k)
            if (tpT(v, k) != 0)
                e = (e << tb) | (uint64_t)(unsigned)(tpT(v, k) + bias);
        return (e << c.bits) | c.code;
    }
    const bool has = tpHasTransform(v);
    if (p.perm && has)
        e = (e << 3) | tpPermCode(v);
    if (p.sym && has)
        e = (e << 3) | tpSym(v);
    if (p.trans && p.childLevel <= p.maxTransLevel && has)
        for (int k = 2; k >= 0; --k)
            e = (e << tb) | (uint64_t)(unsigned)(tpT(v, k) + bias);
    if (p.perm || p.sym || p.trans)
        e = (e << 1) | (has ? 1u : 0u);
    return e;
}
__device__ __forceinline__ uint32_t u16Words(uint64_t v) { return (uint32_t)((64 - __clzll((long long)v) + 15) / 16); }

// ------------------------------------------------------------------------------------------------
// Pass 1 kernels: reference counts, order, pruning, remap.
// ------------------------------------------------------------------------------------------------
__global__ void countRefsKernel(const uint64_t* __restrict__ parents, uint64_t slots, uint32_t* __restrict__ counts, uint64_t items,
    uint32_t* __restrict__ status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots)
        return;
    const uint64_t v = parents[i];
    if (v == tpSentinel())
        return;
    const uint32_t idx = (uint32_t)v;
    if (idx >= items) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 16);
        return;
    }
    atomicAdd(&counts[idx], 1u);
}
// key = maxCount - count: an ascending stable sort orders by count descending, ties by index.
__global__ void refKeysKernel(const uint32_t* __restrict__ counts, uint64_t n, uint32_t maxCount, uint64_t* __restrict__ keys,
    uint32_t* __restrict__ vals, uint32_t* __restrict__ kept)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t live = 0;
    if (i < n) {
        const uint32_t c = counts[i];
        keys[i] = maxCount - c;
        vals[i] = (uint32_t)i;
        live = c != 0;
    }
    live = __syncthreads_count(live);
    if (threadIdx.x == 0 && live)
        atomicAdd(kept, live);
}
template <int W>
__global__ void gatherKeptKernel(const uint64_t* __restrict__ in, const uint32_t* __restrict__ order, uint32_t kept, uint64_t* __restrict__ out,
    uint32_t* __restrict__ mapping)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)kept * W)
        return;
    const uint32_t p = (uint32_t)(i / W), k = (uint32_t)(i % W);
    const uint32_t src = order[p];
    out[i] = in[(uint64_t)src * W + k];
    if (k == 0)
        mapping[src] = p;
}
__global__ void remapChildrenKernel(uint64_t* __restrict__ parents, uint64_t slots, const uint32_t* __restrict__ mapping)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots)
        return;
    const uint64_t v = parents[i];
    if (v != tpSentinel())
        parents[i] = tpWithPtr(v, mapping[(uint32_t)v]);
}

// ------------------------------------------------------------------------------------------------
// Pass 2 kernels: distinct child pointers, encoding, node streams.
// ------------------------------------------------------------------------------------------------
// Child indices -> u16 offsets of the encoded child level (prevOff == null: leaves, identity).
__global__ void childSlotsKernel(uint64_t* __restrict__ nodes, uint64_t slots, const uint32_t* __restrict__ prevOff, uint64_t prevCount,
    uint32_t* __restrict__ flags, uint32_t* __restrict__ status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots)
        return;
    uint64_t v = nodes[i];
    if (v == tpSentinel()) {
        flags[i] = 0;
        return;
    }
    const uint64_t c = tpPtr(v);
    const uint32_t p0 = (uint32_t)(v >> 40) & 3, p1 = (uint32_t)(v >> 42) & 3, p2 = (uint32_t)(v >> 44) & 3;
    const bool permOk = p0 < 3 && p1 < 3 && p2 < 3 && p0 != p1 && p1 != p2 && p0 != p2; // keeps pointer types < 384
    if (c >= prevCount || !permOk) {
        setDeviceError(status, TDAG_ERR_CORRUPT, c >= prevCount ? 17 : 19);
        flags[i] = 0;
        return;
    }
    if (prevOff) {
        v = tpWithPtr(v, prevOff[c]);
        nodes[i] = v;
    }
    flags[i] = 1;
}
__global__ void instanceKeysKernel(const uint64_t* __restrict__ nodes, const uint32_t* __restrict__ slots, uint32_t m, uint64_t* __restrict__ keys,
    uint32_t* __restrict__ vals)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m)
        return;
    const uint32_t s = slots[j];
    keys[j] = nodes[s];
    vals[j] = s;
}
__global__ void runFlagsKernel(const uint64_t* __restrict__ keys, uint32_t m, uint32_t* __restrict__ flags)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m)
        flags[j] = (j == 0 || keys[j] != keys[j - 1]) ? 1u : 0u;
}
__global__ void runCollectKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, const uint32_t* __restrict__ flags,
    const uint32_t* __restrict__ scan, uint32_t m, uint64_t* __restrict__ runVal, uint32_t* __restrict__ runStart, uint32_t* __restrict__ slotRun)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m)
        return;
    const uint32_t r = scan[j] + flags[j] - 1;
    slotRun[vals[j]] = r;
    if (flags[j]) {
        runVal[r] = keys[j];
        runStart[r] = j;
    }
}
__global__ void runCountKeysKernel(const uint32_t* __restrict__ runStart, uint32_t u, uint32_t m, uint32_t maxCount, uint32_t* __restrict__ runCount,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= u)
        return;
    const uint32_t c = (r + 1 < u ? runStart[r + 1] : m) - runStart[r];
    runCount[r] = c;
    keys[r] = maxCount - c;
    vals[r] = r;
}
__global__ void typeHistogramKernel(const uint64_t* __restrict__ runVal, uint32_t u, EncodeParams p, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[kMaxTypes];
    for (uint32_t t = threadIdx.x; t < kMaxTypes; t += blockDim.x)
        h[t] = 0;
    __syncthreads();
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < u; r += gridDim.x * blockDim.x)
        atomicAdd(&h[pointerType(runVal[r], p)], 1u);
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < kMaxTypes; t += blockDim.x)
        if (h[t])
            atomicAdd(&hist[t], h[t]);
}
// Per distinct pointer in count order: its encoded form and, with pointer tables, whether the table
// is cheaper while the table still takes 16-bit indices (transform_dag_encoding.cpp:386-425).
__global__ void encodeEntriesKernel(const uint64_t* __restrict__ runVal, const uint32_t* __restrict__ runCount, const uint32_t* __restrict__ byCount,
    uint32_t u, EncodeParams p, const PointerCode* __restrict__ codes, uint64_t* __restrict__ enc, uint32_t* __restrict__ tableSmall)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= u)
        return;
    const uint32_t r = byCount[k];
    const uint64_t e = encodePointer(runVal[r], p, codes);
    enc[k] = e;
    if (p.pointerTables) {
        const uint32_t cnt = runCount[r];
        const uint32_t inlSize = max(2u, u16Words(e << 1));
        const uint32_t inlineCost = inlSize > 3 ? 0xFFFFFFFFu : cnt * inlSize;
        tableSmall[k] = (cnt * 1u + 4u < inlineCost) ? 1u : 0u;
    }
}
// The first position whose table prefix count reaches 65536: from there on table indices take 32 bits.
__global__ void regimeSwitchKernel(const uint32_t* __restrict__ scan, uint32_t u, uint32_t* __restrict__ jstar)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < u && scan[k] > kSmallTable && (k == 0 || scan[k - 1] <= kSmallTable))
        *jstar = k;
}
__global__ void tableLargeKernel(const uint64_t* __restrict__ enc, const uint32_t* __restrict__ runCount, const uint32_t* __restrict__ byCount, uint32_t u,
    const uint32_t* __restrict__ jstar, uint32_t* __restrict__ tableLarge)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= u)
        return;
    uint32_t d = 0;
    if (k >= *jstar) {
        const uint32_t cnt = runCount[byCount[k]];
        const uint32_t inlSize = max(2u, u16Words(enc[k] << 1));
        const uint32_t inlineCost = inlSize > 3 ? 0xFFFFFFFFu : cnt * inlSize;
        d = (cnt * 2u + 4u < inlineCost) ? 1u : 0u;
    }
    tableLarge[k] = d;
}
// Final entry of every distinct pointer: (value, size in u16) as the node stores it; table entries.
// stats: [0..2] table pointers of 1/2/3 u16, [3..5] direct pointers of 1/2/3 u16.
__global__ void entriesKernel(const uint64_t* __restrict__ enc, uint32_t u, uint32_t pointerTables, const uint32_t* __restrict__ tableSmall,
    const uint32_t* __restrict__ scanSmall, const uint32_t* __restrict__ tableLarge, const uint32_t* __restrict__ scanLarge,
    const uint32_t* __restrict__ jstar, uint64_t* __restrict__ entryVal, uint8_t* __restrict__ entrySize, uint64_t* __restrict__ table,
    unsigned long long* __restrict__ stats, uint32_t* __restrict__ status)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= u)
        return;
    const uint64_t e = enc[k];
    uint64_t val;
    uint32_t size, cls;
    if (pointerTables) {
        const bool large = k >= *jstar;
        const bool inTable = large ? tableLarge[k] != 0 : tableSmall[k] != 0;
        if (inTable) {
            const uint64_t idx = large ? (uint64_t)kSmallTable + 1 + scanLarge[k] : scanSmall[k];
            table[idx] = e;
            val = large ? (idx << 1) | 1 : idx;
            size = large ? 2 : 1;
            cls = size - 1;
        } else {
            val = e << 1;
            size = max(2u, u16Words(val));
            cls = 3 + size - 1;
        }
    } else {
        val = e;
        size = max(1u, u16Words(e));
        cls = 3 + size - 1;
    }
    if (size > 3) {
        setDeviceError(status, TDAG_ERR_ARG, 18); // a pointer wider than 48 bits needs pointer tables
        size = 3;
        cls = 5;
    }
    entryVal[k] = val;
    entrySize[k] = (uint8_t)size;
    atomicAdd(&stats[cls], 1ull);
}
__global__ void nodeSizesKernel(const uint64_t* __restrict__ nodes, uint32_t n, const uint32_t* __restrict__ slotRun, const uint32_t* __restrict__ rankOfRun,
    const uint8_t* __restrict__ entrySize, uint32_t* __restrict__ sizes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t s = 1;
    for (uint32_t c = 0; c < 8; ++c) {
        const uint64_t slot = (uint64_t)i * 8 + c;
        if (nodes[slot] != tpSentinel())
            s += entrySize[rankOfRun[slotRun[slot]]];
    }
    sizes[i] = s;
}
__global__ void nodeWriteKernel(const uint64_t* __restrict__ nodes, uint32_t n, const uint32_t* __restrict__ slotRun, const uint32_t* __restrict__ rankOfRun,
    const uint64_t* __restrict__ entryVal, const uint8_t* __restrict__ entrySize, const uint32_t* __restrict__ off, uint16_t* __restrict__ stream)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t at = off[i] + 1;
    uint32_t mask = 0;
    for (uint32_t c = 0; c < 8; ++c) {
        const uint64_t slot = (uint64_t)i * 8 + c;
        if (nodes[slot] == tpSentinel())
            continue;
        const uint32_t k = rankOfRun[slotRun[slot]];
        const uint32_t size = entrySize[k];
        const uint64_t v = entryVal[k];
        for (uint32_t w = 0; w < size; ++w)
            stream[at + w] = (uint16_t)(v >> (16 * w));
        at += size;
        mask |= size << (2 * c);
    }
    stream[off[i]] = (uint16_t)mask;
}

// Per run (distinct pointer, runs in ascending value): the slot of its first occurrence as a sort key
// (the stable value sort keeps equal values in slot order) and the run id as the value.
__global__ void firstOccurrenceKeysKernel(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ runStart, uint32_t u, uint64_t* __restrict__ keys,
    uint32_t* __restrict__ runIds)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= u)
        return;
    keys[r] = vals[runStart[r]];
    runIds[r] = r;
}
__global__ void gatherValuesKernel(const uint64_t* __restrict__ runVal, const uint32_t* __restrict__ runIds, uint32_t u, uint64_t* __restrict__ out)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < u)
        out[k] = runVal[runIds[k]];
}

__global__ void scatterRankKernel(const uint32_t* __restrict__ byCount, uint32_t u, uint32_t* __restrict__ rankOfRun)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < u)
        rankOfRun[byCount[k]] = k;
}

inline uint32_t bitWidth(uint64_t v)
{
    uint32_t b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

constexpr unsigned kBlock = 256;

// Reorders items (W u64 each) by reference count from `parents`, drops unreferenced ones and remaps
// the parents' child indices (sortByReferenceCount with prune = true).
template <int W>
DevBuf<uint64_t> sortByReferenceCount(Context& c, const DevBuf<uint64_t>& items, uint64_t count, DevBuf<uint64_t>& parents, uint64_t parentCount,
    bool referenceTies, uint64_t& keptOut)
{
    cudaStream_t s = c.stream;
    const uint64_t slots = parentCount * 8;
    TDAG_CHECK(count < 0xFFFFFFFFull && slots < 0xFFFFFFFFull, TDAG_ERR_ARG, "level too large for the encoder");
    DevBuf<uint32_t> counts(std::max<uint64_t>(count, 1), s), vals(std::max<uint64_t>(count, 1), s), kept(1, s);
    DevBuf<uint64_t> keys(std::max<uint64_t>(count, 1), s);
    TDAG_CUDA(cudaMemsetAsync(counts.get(), 0, count * 4, s));
    TDAG_CUDA(cudaMemsetAsync(kept.get(), 0, 4, s));
    if (slots) {
        countRefsKernel<<<gridFor(slots, kBlock), kBlock, 0, s>>>(parents.get(), slots, counts.get(), count, c.status);
        TDAG_LAUNCHED();
    }
    const uint32_t maxCount = (uint32_t)std::min<uint64_t>(slots, 0xFFFFFFFFull);
    uint32_t k = 0;
    if (referenceTies) {
        std::vector<uint32_t> hostCounts(count), order;
        if (count)
            downloadStaged(c, { { hostCounts.data(), counts.get(), (size_t)count * 4 } });
        c.checkStatus("encode16: reference counts");
        k = referenceCountOrder(hostCounts, order);
        if (k) {
            TDAG_CUDA(cudaMemcpyAsync(vals.get(), order.data(), (uint64_t)k * 4, cudaMemcpyHostToDevice, s));
            TDAG_CUDA(cudaStreamSynchronize(s)); // `order` is pageable host memory released on return
        }
    } else {
        if (count) {
            refKeysKernel<<<gridFor(count, kBlock), kBlock, 0, s>>>(counts.get(), count, maxCount, keys.get(), vals.get(), kept.get());
            TDAG_LAUNCHED();
            radixSortPairs(keys.get(), vals.get(), count, 0, std::max(1u, bitWidth(maxCount)), s, c.status);
        }
        TDAG_CUDA(cudaMemcpyAsync(&k, kept.get(), 4, cudaMemcpyDeviceToHost, s));
        c.checkStatus("encode16: reference counts");
    }
    DevBuf<uint64_t> out(std::max<uint64_t>((uint64_t)k * W, 1), s);
    DevBuf<uint32_t> mapping(std::max<uint64_t>(count, 1), s);
    if (k) {
        gatherKeptKernel<W><<<gridFor((uint64_t)k * W, kBlock), kBlock, 0, s>>>(items.get(), vals.get(), k, out.get(), mapping.get());
        TDAG_LAUNCHED();
    }
    if (slots) {
        remapChildrenKernel<<<gridFor(slots, kBlock), kBlock, 0, s>>>(parents.get(), slots, mapping.get());
        TDAG_LAUNCHED();
    }
    keptOut = k;
    return out;
}

struct EncodedLevel {
    DevBuf<uint16_t> stream;
    uint64_t length = 0; // u16 words
    DevBuf<uint64_t> table;
    uint64_t tableSize = 0;
    std::vector<PointerCode> codes;
};

} // namespace

// The whole encoder; see the file comment. `dag` arrays may be host or device memory.
void encodeTdag16(Context& c, const tdag_result& dag, const tdag_config& cfg, const tdag_encoding_config& enc, tdag16_result& out)
{
    cudaStream_t s = c.stream;
    const uint32_t root = dag.root_level;
    TDAG_CHECK(root >= 3 && root < TDAG_MAX_LEVELS, TDAG_ERR_ARG, "the encoder needs a root level of 3 or more");
    TDAG_CHECK(enc.tie_order == TDAG16_TIES_REFERENCE || enc.tie_order == TDAG16_TIES_CANONICAL, TDAG_ERR_ARG,
        "tie_order must be TDAG16_TIES_REFERENCE or TDAG16_TIES_CANONICAL");
    const bool referenceTies = enc.tie_order == TDAG16_TIES_REFERENCE;
    const uint64_t launches0 = g_kernelLaunches.load();
    TDAG_CUDA(cudaEventRecord(c.ev[5], s));

    // Working copies of the levels (the caller's result stays unchanged).
    const cudaMemcpyKind kind = dag.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    std::vector<DevBuf<uint64_t>> nodes(root + 1);
    std::vector<uint64_t> counts(root + 1, 0);
    for (uint32_t l = 3; l <= root; ++l) {
        counts[l] = dag.node_counts[l];
        nodes[l] = DevBuf<uint64_t>(std::max<uint64_t>(counts[l] * 8, 1), s);
        if (counts[l])
            TDAG_CUDA(cudaMemcpyAsync(nodes[l].get(), dag.nodes[l], counts[l] * 64, kind, s));
    }
    counts[2] = dag.leaf_count;
    DevBuf<uint64_t> leaves(std::max<uint64_t>(counts[2], 1), s);
    if (counts[2])
        TDAG_CUDA(cudaMemcpyAsync(leaves.get(), dag.leaves, counts[2] * 8, kind, s));

    // Pass 1: top-down reference-count order (pointer_encoding.h:27-72; transform_dag_encoding.cpp:246-253).
    for (uint32_t l = root - 1; l > 2; --l) {
        uint64_t kept = 0;
        nodes[l] = sortByReferenceCount<8>(c, nodes[l], counts[l], nodes[l + 1], counts[l + 1], referenceTies, kept);
        counts[l] = kept;
    }
    {
        uint64_t kept = 0;
        leaves = sortByReferenceCount<1>(c, leaves, counts[2], nodes[3], counts[3], referenceTies, kept);
        counts[2] = kept;
    }

    // Pass 2: bottom-up encoding (transform_dag_encoding.cpp:273-478).
    std::vector<EncodedLevel> levels(root + 1);
    DevBuf<uint32_t> prevOff;
    uint64_t prevCount = counts[2];
    DevBuf<unsigned long long> stats(6, s);
    DevBuf<uint32_t> jstarDev(1, s);
    DevBuf<PointerCode> codesDev(kMaxTypes, s);
    DevBuf<uint32_t> histDev(kMaxTypes, s);
    const uint32_t numTypes = (cfg.symmetry ? 8u : 1u) * (cfg.axis_permutation ? 6u : 1u) * (cfg.translation ? 8u : 1u);
    std::memset(out.levels, 0, sizeof(out.levels));
    out.levels[2].num_nodes = counts[2];
    out.levels[2].memory_in_bytes = counts[2] * 8;
    for (uint32_t l = 3; l <= root; ++l) {
        const uint32_t childLevel = l - 1;
        const uint64_t n = counts[l];
        const uint64_t slots = n * 8;
        TDAG_CHECK(slots < 0xFFFFFFFFull, TDAG_ERR_ARG, "level too large for the encoder");
        EncodeParams p { childLevel, (uint32_t)(cfg.symmetry != 0), (uint32_t)(cfg.axis_permutation != 0), (uint32_t)(cfg.translation != 0),
            cfg.max_translation_level, (uint32_t)(enc.pointer_tables != 0), (uint32_t)(enc.huffman_code != 0) };
        tdag16_level_stats& ls = out.levels[l];
        ls.num_nodes = n;

        // distinct child pointers with their reference counts
        DevBuf<uint32_t> flags(std::max<uint64_t>(slots, 1), s), instSlots(std::max<uint64_t>(slots, 1), s);
        uint32_t m = 0;
        if (slots) {
            childSlotsKernel<<<gridFor(slots, kBlock), kBlock, 0, s>>>(nodes[l].get(), slots, childLevel > 2 ? prevOff.get() : nullptr, prevCount,
                flags.get(), c.status);
            TDAG_LAUNCHED();
            m = compactFlags(flags.get(), instSlots.get(), slots, s);
        }
        c.checkStatus("encode16: child pointers");
        DevBuf<uint64_t> keys(std::max<uint32_t>(m, 1), s);
        DevBuf<uint32_t> vals(std::max<uint32_t>(m, 1), s), runFlag(std::max<uint32_t>(m, 1), s), runScan(std::max<uint32_t>(m, 1), s);
        DevBuf<uint32_t> slotRun(std::max<uint64_t>(slots, 1), s);
        uint32_t u = 0;
        if (m) {
            instanceKeysKernel<<<gridFor(m, kBlock), kBlock, 0, s>>>(nodes[l].get(), instSlots.get(), m, keys.get(), vals.get());
            TDAG_LAUNCHED();
            radixSortPairs(keys.get(), vals.get(), m, 0, 64, s, c.status);
            runFlagsKernel<<<gridFor(m, kBlock), kBlock, 0, s>>>(keys.get(), m, runFlag.get());
            TDAG_LAUNCHED();
            u = (uint32_t)exclusiveScanU32Total(runFlag.get(), runScan.get(), m, s);
        }
        DevBuf<uint64_t> runVal(std::max<uint32_t>(u, 1), s), countKeys(std::max<uint32_t>(u, 1), s);
        DevBuf<uint32_t> runStart(std::max<uint32_t>(u, 1), s), runCount(std::max<uint32_t>(u, 1), s), byCount(std::max<uint32_t>(u, 1), s),
            rankOfRun(std::max<uint32_t>(u, 1), s);
        if (m) {
            runCollectKernel<<<gridFor(m, kBlock), kBlock, 0, s>>>(keys.get(), vals.get(), runFlag.get(), runScan.get(), m, runVal.get(), runStart.get(),
                slotRun.get());
            TDAG_LAUNCHED();
            runCountKeysKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(runStart.get(), u, m, m, runCount.get(), countKeys.get(), byCount.get());
            TDAG_LAUNCHED();
            if (referenceTies) {
                // the distinct pointers in first-occurrence order (runs are numbered by ascending value)
                firstOccurrenceKeysKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(vals.get(), runStart.get(), u, countKeys.get(), byCount.get());
                TDAG_LAUNCHED();
                radixSortPairs(countKeys.get(), byCount.get(), u, 0, std::max(1u, bitWidth(slots)), s, c.status);
                gatherValuesKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(runVal.get(), byCount.get(), u, countKeys.get());
                TDAG_LAUNCHED();
                std::vector<uint64_t> firstValues(u);
                std::vector<uint32_t> firstRuns(u), counts(u);
                downloadStaged(c, { { firstValues.data(), countKeys.get(), (size_t)u * 8 }, { firstRuns.data(), byCount.get(), (size_t)u * 4 },
                                      { counts.data(), runCount.get(), (size_t)u * 4 } });
                c.checkStatus("encode16: distinct pointers");
                const std::vector<uint32_t> runOrder = referencePointerOrder(firstValues, firstRuns, counts);
                TDAG_CHECK(runOrder.size() == u, TDAG_ERR_CUDA, "encode16: distinct pointer counts disagree");
                TDAG_CUDA(cudaMemcpyAsync(byCount.get(), runOrder.data(), (uint64_t)u * 4, cudaMemcpyHostToDevice, s));
                TDAG_CUDA(cudaStreamSynchronize(s)); // `runOrder` is released at the end of this scope
            } else {
                radixSortPairs(countKeys.get(), byCount.get(), u, 0, std::max(1u, bitWidth(m)), s, c.status);
            }
            scatterRankKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(byCount.get(), u, rankOfRun.get());
            TDAG_LAUNCHED();
        }
        ls.unique_pointers = u;

        // Huffman code of the pointer types (over distinct pointers, not references)
        EncodedLevel& el = levels[childLevel];
        if (enc.huffman_code) {
            TDAG_CUDA(cudaMemsetAsync(histDev.get(), 0, kMaxTypes * 4, s));
            if (u) {
                typeHistogramKernel<<<std::min<unsigned>(gridFor(u, kBlock), (unsigned)c.numSMs * 4), kBlock, 0, s>>>(runVal.get(), u, p, histDev.get());
                TDAG_LAUNCHED();
            }
            std::vector<uint32_t> hist(kMaxTypes);
            TDAG_CUDA(cudaMemcpyAsync(hist.data(), histDev.get(), kMaxTypes * 4, cudaMemcpyDeviceToHost, s));
            TDAG_CUDA(cudaStreamSynchronize(s));
            el.codes = huffmanCodes(std::vector<uint64_t>(hist.begin(), hist.begin() + numTypes));
            std::vector<PointerCode> padded(kMaxTypes, PointerCode { 0, 0, 0 });
            std::copy(el.codes.begin(), el.codes.end(), padded.begin());
            TDAG_CUDA(cudaMemcpyAsync(codesDev.get(), padded.data(), kMaxTypes * sizeof(PointerCode), cudaMemcpyHostToDevice, s));
            // the host vector must outlive the copy
            TDAG_CUDA(cudaStreamSynchronize(s));
        }

        // encoded pointers, inline-or-table decisions, entries
        DevBuf<uint64_t> encv(std::max<uint32_t>(u, 1), s), entryVal(std::max<uint32_t>(u, 1), s);
        DevBuf<uint32_t> tSmall(std::max<uint32_t>(u, 1), s), sSmall(std::max<uint32_t>(u, 1), s), tLarge(std::max<uint32_t>(u, 1), s),
            sLarge(std::max<uint32_t>(u, 1), s);
        DevBuf<uint8_t> entrySize(std::max<uint32_t>(u, 1), s);
        TDAG_CUDA(cudaMemsetAsync(stats.get(), 0, 6 * 8, s));
        TDAG_CUDA(cudaMemcpyAsync(jstarDev.get(), &u, 4, cudaMemcpyHostToDevice, s));
        uint64_t tableSize = 0;
        if (u) {
            encodeEntriesKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(runVal.get(), runCount.get(), byCount.get(), u, p, codesDev.get(), encv.get(),
                tSmall.get());
            TDAG_LAUNCHED();
            if (enc.pointer_tables) {
                const uint64_t smallTotal = exclusiveScanU32Total(tSmall.get(), sSmall.get(), u, s);
                tableSize = smallTotal;
                if (smallTotal > kSmallTable) {
                    regimeSwitchKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(sSmall.get(), u, jstarDev.get());
                    TDAG_LAUNCHED();
                    tableLargeKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(encv.get(), runCount.get(), byCount.get(), u, jstarDev.get(), tLarge.get());
                    TDAG_LAUNCHED();
                    uint32_t jstar = u;
                    TDAG_CUDA(cudaMemcpyAsync(&jstar, jstarDev.get(), 4, cudaMemcpyDeviceToHost, s));
                    const uint64_t largeTotal = exclusiveScanU32Total(tLarge.get(), sLarge.get(), u, s); // synchronises
                    if (jstar < u)
                        tableSize = (uint64_t)kSmallTable + 1 + largeTotal;
                }
            }
            el.table = DevBuf<uint64_t>(std::max<uint64_t>(tableSize, 1), s);
            el.tableSize = tableSize;
            entriesKernel<<<gridFor(u, kBlock), kBlock, 0, s>>>(encv.get(), u, p.pointerTables, tSmall.get(), sSmall.get(), tLarge.get(), sLarge.get(),
                jstarDev.get(), entryVal.get(), entrySize.get(), el.table.get(), stats.get(), c.status);
            TDAG_LAUNCHED();
        }
        unsigned long long st[6] = { 0, 0, 0, 0, 0, 0 };
        TDAG_CUDA(cudaMemcpyAsync(st, stats.get(), sizeof(st), cudaMemcpyDeviceToHost, s));
        c.checkStatus("encode16: pointer entries");
        for (int k = 0; k < 3; ++k) {
            ls.table_pointers[k] = st[k];
            ls.direct_pointers[k] = st[3 + k];
        }
        ls.table_size = tableSize;

        // node streams
        DevBuf<uint32_t> sizes(std::max<uint64_t>(n, 1), s), off(std::max<uint64_t>(n, 1), s);
        uint64_t length = 0;
        if (n) {
            nodeSizesKernel<<<gridFor(n, kBlock), kBlock, 0, s>>>(nodes[l].get(), (uint32_t)n, slotRun.get(), rankOfRun.get(), entrySize.get(), sizes.get());
            TDAG_LAUNCHED();
            length = exclusiveScanU32Total(sizes.get(), off.get(), n, s);
            TDAG_CHECK(length < 0xFFFFFFFFull, TDAG_ERR_ARG, "encoded level exceeds 2^32 u16 words");
        }
        EncodedLevel& nl = levels[l];
        nl.stream = DevBuf<uint16_t>(std::max<uint64_t>(length, 1), s);
        nl.length = length;
        if (n) {
            nodeWriteKernel<<<gridFor(n, kBlock), kBlock, 0, s>>>(nodes[l].get(), (uint32_t)n, slotRun.get(), rankOfRun.get(), entryVal.get(),
                entrySize.get(), off.get(), nl.stream.get());
            TDAG_LAUNCHED();
        }
        ls.memory_in_bytes = length * 2;
        prevOff = std::move(off);
        prevCount = n;
    }
    TDAG_CUDA(cudaEventRecord(c.ev[7], s));
    c.checkStatus("encode16");
    TDAG_CUDA(cudaEventElapsedTime(&out.encode_ms, c.ev[5], c.ev[7]));

    // TransformDAG16::writeTo: config (8 B, padding byte zero), encoding config (2 B), nodesPerLevel,
    // subGrids, resolution, rootLevel, pointerTables, huffmanDecoders (each LUT writes its code list;
    // a Code is 16 bytes of which the last 4 are padding, written as zero).
    const uint64_t nl = root + 1;
    uint64_t size = 8 + 2 + 8;
    for (uint32_t l = 0; l <= root; ++l)
        size += 8 + (l >= 3 ? levels[l].length * 2 : 0);
    size += 8 + counts[2] * 8 + 4 + 4 + 8;
    for (uint32_t l = 0; l <= root; ++l)
        size += 8 + levels[l].tableSize * 8;
    size += 8;
    if (enc.huffman_code)
        for (uint32_t l = 0; l <= root; ++l)
            size += 8 + levels[l].codes.size() * 16;
    uint8_t* bytes = (uint8_t*)std::malloc(size);
    TDAG_CHECK(bytes != nullptr, TDAG_ERR_OOM, "host allocation of the .tdag16 buffer failed");
    std::unique_ptr<uint8_t, decltype(&std::free)> hold(bytes, &std::free);
    std::memset(bytes, 0, size);
    std::vector<Download> dl;
    uint64_t at = 0;
    auto put = [&](const void* src, size_t n) {
        std::memcpy(bytes + at, src, n);
        at += n;
    };
    auto putU64 = [&](uint64_t v) { put(&v, 8); };
    const uint8_t cfgBytes[8] = { (uint8_t)(cfg.symmetry != 0), (uint8_t)(cfg.axis_permutation != 0), (uint8_t)(cfg.translation != 0), 0,
        (uint8_t)cfg.max_translation_level, (uint8_t)(cfg.max_translation_level >> 8), (uint8_t)(cfg.max_translation_level >> 16),
        (uint8_t)(cfg.max_translation_level >> 24) };
    put(cfgBytes, 8);
    const uint8_t encBytes[2] = { (uint8_t)(enc.pointer_tables != 0), (uint8_t)(enc.huffman_code != 0) };
    put(encBytes, 2);
    putU64(nl);
    for (uint32_t l = 0; l <= root; ++l) {
        const uint64_t len = l >= 3 ? levels[l].length : 0;
        putU64(len);
        if (len)
            dl.push_back({ bytes + at, levels[l].stream.get(), len * 2 });
        at += len * 2;
    }
    putU64(counts[2]);
    if (counts[2])
        dl.push_back({ bytes + at, leaves.get(), counts[2] * 8 });
    at += counts[2] * 8;
    put(&dag.resolution, 4);
    put(&dag.root_level, 4);
    putU64(nl);
    for (uint32_t l = 0; l <= root; ++l) {
        putU64(levels[l].tableSize);
        if (levels[l].tableSize)
            dl.push_back({ bytes + at, levels[l].table.get(), levels[l].tableSize * 8 });
        at += levels[l].tableSize * 8;
    }
    putU64(enc.huffman_code ? nl : 0);
    if (enc.huffman_code)
        for (uint32_t l = 0; l <= root; ++l) {
            putU64(levels[l].codes.size());
            for (const PointerCode& pc : levels[l].codes) {
                put(&pc.code, 8);
                put(&pc.bits, 4);
                at += 4;
            }
        }
    TDAG_CHECK(at == size, TDAG_ERR_ARG, "internal: .tdag16 size mismatch");
    downloadStaged(c, dl);
    out.bytes = hold.release();
    out.size = size;
    out.root_level = root;
    out.kernel_launches = g_kernelLaunches.load() - launches0;
}

} // namespace tdag

struct tdag_ctx;
tdag::Context& ctxOf(tdag_ctx* c); // build.cu
int guardedCall(const std::function<void()>& f); // build.cu
int failWith(int code, const char* msg); // build.cu

extern "C" int tdag_encode16(tdag_ctx* ctx, const tdag_result* dag, const tdag_config* config, const tdag_encoding_config* encoding,
    tdag16_result** out)
{
    using namespace tdag;
    if (!ctx || !dag || !config || !encoding || !out)
        return failWith(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        std::unique_ptr<tdag16_result> r(new tdag16_result {});
        const auto t0 = std::chrono::steady_clock::now();
        encodeTdag16(c, *dag, *config, *encoding, *r);
        r->wall_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        *out = r.release();
    });
}

extern "C" int tdag16_huffman_code_table(const uint64_t* frequencies, uint32_t n, uint32_t max_code_length, int lsb_first,
    uint64_t* out_codes, uint32_t* out_bits)
{
    using namespace tdag;
    if (!frequencies || !out_codes || !out_bits)
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        const auto codes = huffmanCodes(std::vector<uint64_t>(frequencies, frequencies + n), max_code_length, lsb_first != 0);
        for (uint32_t i = 0; i < n; ++i) {
            out_codes[i] = codes[i].code;
            out_bits[i] = codes[i].bits;
        }
    });
}

extern "C" int tdag16_result_free(tdag16_result* r)
{
    if (r) {
        std::free(r->bytes);
        delete r;
    }
    return TDAG_OK;
}
