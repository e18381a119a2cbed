// matcher.cu — GPU sub-grid matching under translation + the 48 mirror/permutation transforms.
//
// Restates findDuplicatesAmongFlattenedItems_cpp2<Level> (tools/lib/src/voxel/find_translation.cpp:616-1000):
//   * items are visited as sources in stable popcount-descending order (:631-643); the encoded parent
//     pointer stores the source's position in that order (:781, :837) and is decoded back (:923-937);
//   * a directional box hash of every grid is read at each of its 8 corners (:672-720) and indexed by
//     hash value (:721-760);
//   * every source, for each of the 8 directions and 6 axis orders, hashes the box seen from every voxel
//     (:481-495, :202-264), looks the non-zero values up, and each candidate (target, corner) gives
//     the transform (mirror = direction ^ corner, translation from the anchor, :835-837);
//   * candidates are filtered by the config (:840-845), skipped when they cannot lower the target's
//     parent (:830-850), verified by an exact grid comparison (:857-862) and merged with a 64-bit
//     atomic minimum (:864);
//   * sources run in batches of increasing popcount order; after a batch the table drops every
//     target whose parent no later source can lower (:887-915);
//   * the isUnique pass keeps every item that is nobody's child or somebody's parent (:953-961) and
//     numbers the kept items in their original order (:982-997).
// The result is the minimum encoded pointer over all verified candidates, which does not depend on
// thread order or batching, so the GPU output equals the CPU output bit for bit.
//
// Search kernel layout (one team of R*R threads per source grid, one thread per grid line):
//   pass 1 (6 per source) folds the occupancy bits along axis a0 into G1, pass 2 (24 per source)
//   folds G1 along a1 into G2, pass 3 (48 per source) folds G2 along a2 in place — the thread keeps
//   its original line in registers so both a2 directions come from one G2. Passes 1 and 2 are shared
//   by the permutations that start with the same axes (78 passes instead of 144). Every non-zero hash
//   is tested against a one-bit membership filter (global, L2-resident), the survivors are queued in
//   shared memory, looked up in the table (16-byte slots: key + range) and each hit's candidate range
//   is spread across the warp.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <functional>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "internal.cuh"

namespace tdag {

namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------- bulk copies (TMA)
// A 1-D bulk copy (cp.async.bulk, the TMA unit's untiled form) from this GPU's global memory into the
// CTA's shared memory, completed on an mbarrier: both addresses 16-byte aligned, the size a multiple
// of 16. No multicast. Every wait is bounded.
__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}
// Orders this thread's earlier shared-memory accesses (and barrier inits) before later async-proxy ones.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulkCopyToShared(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smemAddr(dst)), "l"(src),
        "r"(bytes), "r"(smemAddr(bar))
        : "memory");
}
// L2 eviction-priority hints (per instruction; no cache state outlives the kernel). The level-4
// probe marks its membership-filter loads evict-last and its streamed stores (survivor records and
// the sources' line orientations, hundreds of MB per build) evict-first, so that they do not push
// the filter out of L2.
__device__ __forceinline__ uint64_t l2PolicyEvictLast()
{
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint64_t l2PolicyEvictFirst()
{
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint32_t ldL2Hint(const uint32_t* p, uint64_t pol)
{
    uint32_t v;
    asm volatile("ld.global.cg.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void stL2Hint(ulonglong2* p, ulonglong2 v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.v2.u64 [%0], {%1, %2}, %3;" ::"l"(p), "l"(v.x), "l"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void stL2Hint(uint16_t* p, uint16_t v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.u16 [%0], %1, %2;" ::"l"(p), "h"(v), "l"(pol) : "memory");
}

// Waits until the barrier's phase with the given parity has completed; false after the bound.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity)
{
    const uint32_t a = smemAddr(bar);
    for (uint32_t i = 0; i < (1u << 20); ++i) {
        uint32_t done = 0;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}

// The directional box hash. The reference folds every axis with hash_combine and clamps to 1 once
// started (find_translation.cpp:210-218). Which hash is used does not change the result: a probe only
// proposes (source, target, transform) candidates, every candidate is verified exactly, and
// verification passes precisely when the two boxes agree after leading empty elements are stripped
// on every axis -- which makes any hash of that stripped form equal. The requirements are (a) leading
// empty elements leave the state at zero and (b) a non-empty box never hashes to zero (it would not
// be probed). Here:
//  - pass 1 (along the first fold axis) is exact: the window of the line from the anchor to v, read
//    as a base-2 number with the element at v as its lowest digit (leading empties add nothing), then
//    doubled plus one if non-empty, so a non-empty window is odd;
//  - passes 2 and 3 are a polynomial hash mod 2^64 with an odd base per pass, and bit 0 carries
//    "started": 0 stays 0, a non-empty box stays odd. Three integer multiply-adds and a logic op.
// Pass-1 code of `line` (bit c = element c) for the window ending at v; fromHigh: the anchor is R-1.
__device__ __forceinline__ uint32_t lineCode(uint32_t line, int v, bool fromHigh)
{
    const uint32_t c = fromHigh ? (line >> v) : (__brev(line) >> (31 - v));
    return (c << 1) | (c != 0u ? 1u : 0u);
}
template <int P>
__device__ __forceinline__ uint64_t boxFold(uint64_t acc, uint64_t v)
{
    constexpr uint64_t K = P == 1 ? 0xC2B2AE3D27D4EB4Full : 0x165667B19E3779F9ull;
    static_assert(P == 1 || P == 2, "passes 2 and 3 fold; pass 1 is lineCode");
    return (acc * K + v) | (acc & 1u);
}

// Table slot and membership-filter indices (32-bit multiply-xorshift hashes of the 64-bit key).
__host__ __device__ __forceinline__ uint32_t slotHash(uint64_t k)
{
    uint32_t h = (uint32_t)k * 0xCC9E2D51u ^ (uint32_t)(k >> 32) * 0x1B873593u;
    h ^= h >> 15;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    return h;
}
// Membership filter: a blocked Bloom filter, two bits of one 32-bit word per key (filterShift =
// 32 - log2(filter bits), so the word index is the top log2(bits) - 5 bits of a multiplicative hash).
__host__ __device__ __forceinline__ uint32_t filterFold(uint64_t k) { return (uint32_t)k ^ (uint32_t)(k >> 32); }
__host__ __device__ __forceinline__ uint32_t filterWordIndex(uint32_t x, uint32_t filterShift) { return (x * 0x9E3779B1u) >> (filterShift + 5); }
__host__ __device__ __forceinline__ uint32_t filterBits(uint32_t x) { return (1u << (x & 31u)) | (1u << ((x >> 5) & 31u)); }

// Table key of a corner view in the split search: the (salted) hash times an odd constant -- a
// bijection that spreads the small hashes of boxes whose content starts at their far end (leading
// empties add nothing to the fold) over the high bits -- cut to its top 40 bits, with bit 0 set so it
// is never the empty slot 0. A probe looks its box hash up reduced the same way. Matching on 40 bits
// can only add candidates, which verification rejects; the view sort needs 5 radix digits instead of
// 8, and the top bits serve as the home slot.
constexpr uint64_t kViewKeyMask = ~((1ull << 24) - 1);
constexpr uint32_t kViewKeyLowBit = 24; // the view sort starts at this bit
__host__ __device__ __forceinline__ uint64_t viewKey(uint64_t h) { return ((h * 0x9E3779B97F4A7C15ull) & kViewKeyMask) | 1ull; }

// Per-grid salt of the box hashes of a batch member: even, so a salted non-empty box hash stays odd
// and never collides with the empty-slot key 0; 0 for a single grid, leaving the key unchanged.
__host__ __device__ __forceinline__ uint64_t boxSalt(uint32_t g) { return gridSalt(g) & ~1ull; }

// ---------------------------------------------------------------------------- popcount order
// Sort key: grid id above (R^3 - popcount), so a batch sorts grid by grid, popcount descending.
template <int W>
__global__ void popcountKeyKernel(const uint64_t* __restrict__ grids, uint32_t n, uint32_t maxCount, uint64_t* __restrict__ key, uint32_t* __restrict__ val,
    const uint32_t* __restrict__ gridOf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t c = 0;
#pragma unroll 8
    for (int k = 0; k < W; ++k)
        c += __popcll(grids[(size_t)i * W + k]);
    key[i] = (gridOf ? ((uint64_t)gridOf[i] << 13) : 0ull) | (maxCount - c); // ascending key == descending popcount; stable sort keeps index order
    val[i] = i;
}

// ---------------------------------------------------------------------------- corner hashes
// Warp per (item, direction). The value at the anchor corner is a nested fold: x-lines, then the
// anchor x-plane along y, then the anchor column along z (computeGridHashInPlace<R, +x, +y, +z>).
template <int R>
__global__ void cornerHashKernel(const uint64_t* __restrict__ grids, uint32_t n, uint64_t* __restrict__ keys, uint32_t* __restrict__ payload,
    const uint32_t* __restrict__ gridOf)
{
    constexpr int W = R * R * R / 64;
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    __shared__ uint64_t xres[kThreads / 32][R * R];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (uint64_t)n * 8)
        return;
    const uint32_t item = (uint32_t)(gw >> 3), d = (uint32_t)(gw & 7);
    const bool px = d & 1, py = d & 2, pz = d & 4;
    const uint64_t* g = grids + (size_t)item * W;
    for (int line = lane; line < R * R; line += 32) { // line = y + R z
        const uint32_t bitOff = (uint32_t)line * R;
        const uint32_t row = (uint32_t)(g[bitOff >> 6] >> (bitOff & 63)) & rowMask;
        xres[warp][line] = lineCode(row, px ? 0 : R - 1, px); // the whole row, ending at the far side
    }
    __syncwarp();
    uint64_t yv = 0;
    if (lane < R) { // column along y at the anchor x, for z = lane
        uint64_t acc = 0;
        for (int k = 0; k < R; ++k) {
            const int y = py ? R - 1 - k : k;
            acc = boxFold<1>(acc, xres[warp][y + R * lane]);
        }
        yv = acc;
    }
    uint64_t acc = 0;
    for (int k = 0; k < R; ++k) {
        const int z = pz ? R - 1 - k : k;
        const uint64_t v = __shfl_sync(0xffffffffu, yv, z);
        acc = boxFold<2>(acc, v);
    }
    if (lane == 0) {
        keys[gw] = gridOf ? acc ^ boxSalt(gridOf[item]) : acc; // a grid is never empty: acc is odd
        payload[gw] = item * 8 + d;
    }
}

// The two axes other than a, in increasing order.
__device__ __forceinline__ int otherLo(int a) { return a == 0 ? 1 : 0; }
__device__ __forceinline__ int otherHi(int a) { return a == 2 ? 1 : 2; }

// ---------------------------------------------------------------------------- permuted corner views
// The reference search folds every source in all six axis orders (a0, a1, a2) and eight directions
// and looks the box hashes up among the targets' eight corner views (find_translation.cpp:780-870).
// Permuting axes commutes with cropping and turns shifts and mirrors into shifts and mirrors, so
// t = crop(shift_T(mirror_S(perm_a(s)))) holds exactly when b(t) = crop(shift_T'(mirror_S'(s))) with
// b = a^-1 and S', T' the mirror bits and translation re-indexed by b. The split search therefore
// folds each source in the identity order only (8 directions instead of 48 orientations) and looks
// its box hashes up among 48 views per target: for each axis order b (pidB = 2 b0 + (b2 < b1)) and
// corner c' (bit i: pass i folds down from R-1), the whole grid folded along b0, then b1, then b2.
// Every (source, target, transform) the reference finds is found once, and the lookup maps it back
// to the reference's (perm, sym, translation). payload = item << 6 | pidB << 3 | c'.
template <int R>
__global__ void __launch_bounds__(kThreads) cornerViewsKernel(const uint64_t* __restrict__ grids, uint32_t n, uint32_t perms, uint64_t* __restrict__ keys,
    uint32_t* __restrict__ payload, const uint32_t* __restrict__ gridOf)
{
    constexpr int W = R * R * R / 64;
    constexpr int WARPS = kThreads / 32;
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    __shared__ uint64_t sGrid[WARPS][W];
    __shared__ uint16_t sLines[WARPS][3 * R * R]; // [a][u_lo + R u_hi]
    __shared__ uint64_t sG2[WARPS][6 * 4 * R]; // [(pidB * 4 + c0 + 2 c1) * R + w2]
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t item = blockIdx.x * WARPS + warp;
    if (item >= n) // warp-uniform
        return;
    const uint64_t* g = grids + (size_t)item * W;
    for (int k = lane; k < W; k += 32)
        sGrid[warp][k] = g[k];
    __syncwarp();
    for (int t = lane; t < R * R; t += 32) {
        const int tA = t % R, tB = t / R;
        const uint32_t off = (uint32_t)R * (tA + R * tB); // x-line at (y, z) = (tA, tB)
        uint32_t ly = 0, lz = 0;
        for (int j = 0; j < R; ++j) {
            const uint32_t iy = tA + R * j + R * R * tB; // (x=tA, y=j, z=tB)
            const uint32_t iz = tA + R * tB + R * R * j; // (x=tA, y=tB, z=j)
            ly |= (uint32_t)((sGrid[warp][iy >> 6] >> (iy & 63)) & 1) << j;
            lz |= (uint32_t)((sGrid[warp][iz >> 6] >> (iz & 63)) & 1) << j;
        }
        sLines[warp][t] = (uint16_t)((uint32_t)(sGrid[warp][off >> 6] >> (off & 63)) & rowMask);
        sLines[warp][R * R + t] = (uint16_t)ly;
        sLines[warp][2 * R * R + t] = (uint16_t)lz;
    }
    __syncwarp();
    // pass 2: for every axis order, pass-1 and pass-2 direction and coordinate w2 along b2, the fold
    // along b1 of the pass-1 codes of the whole lines along b0
    for (int ch = lane; ch < (int)perms * 4 * R; ch += 32) {
        const int w2 = ch % R, c01 = (ch / R) & 3, pb = ch / (4 * R);
        const int b0 = pb >> 1, lo = otherLo(b0), hi = otherHi(b0);
        const int b1 = (pb & 1) ? hi : lo, b2 = (pb & 1) ? lo : hi;
        const int c0 = c01 & 1, c1 = c01 >> 1;
        const uint16_t* La = sLines[warp] + b0 * R * R;
        const int sj = b1 < b2 ? 1 : R, bw = b1 < b2 ? R * w2 : w2; // line index with u[b1] = j, u[b2] = w2
        uint64_t acc = 0;
        for (int k = 0; k < R; ++k) {
            const int j = c1 ? R - 1 - k : k;
            acc = boxFold<1>(acc, lineCode(La[bw + j * sj], c0 ? 0 : R - 1, c0));
        }
        sG2[warp][ch] = acc;
    }
    __syncwarp();
    // pass 3 along b2: one view per (pidB, c')
    const uint32_t views = perms * 8;
    const uint64_t salt = gridOf ? boxSalt(gridOf[item]) : 0ull;
    for (uint32_t v = lane; v < views; v += 32) {
        const uint32_t pb = v >> 3, cp = v & 7;
        const uint64_t* G = sG2[warp] + (pb * 4 + (cp & 3)) * R;
        uint64_t acc = 0;
        for (int k = 0; k < R; ++k)
            acc = boxFold<2>(acc, G[(cp >> 2) ? R - 1 - k : k]);
        const size_t e = (size_t)item * views + v;
        keys[e] = viewKey(acc ^ salt);
        payload[e] = (item << 6) | (pb << 3) | cp;
    }
}

// ---------------------------------------------------------------------------- corner-hash table
// slots: (key, start | count << 32) pairs; entries: payload (item * 8 + corner) grouped by key.
__global__ void tableInsertKernel(const uint64_t* __restrict__ ekeys, size_t m, ulonglong2* __restrict__ slots, uint32_t* __restrict__ tcount,
    uint32_t* __restrict__ slotOfEntry, uint32_t capMask, uint32_t* __restrict__ numDistinct, uint32_t* status)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m)
        return;
    const uint64_t key = ekeys[e];
    if (key == 0) { // an empty grid has no corner view (find_translation.cpp:722)
        slotOfEntry[e] = 0xFFFFFFFFu;
        return;
    }
    uint32_t slot = slotHash(key) & capMask;
    for (uint32_t probe = 0; probe <= capMask; ++probe) {
        unsigned long long cur = slots[slot].x;
        if (cur == 0) {
            cur = atomicCAS(&slots[slot].x, 0ull, (unsigned long long)key);
            if (cur == 0) {
                atomicAdd(numDistinct, 1u);
                cur = key;
            }
        }
        if (cur == key) {
            atomicAdd(&tcount[slot], 1u);
            slotOfEntry[e] = slot;
            return;
        }
        slot = (slot + 1) & capMask;
    }
    slotOfEntry[e] = 0xFFFFFFFFu;
    setDeviceError(status, TDAG_ERR_TABLE_FULL, 200);
}

__global__ void tableScatterKernel(const uint32_t* __restrict__ epayload, const uint32_t* __restrict__ slotOfEntry, size_t m, const uint32_t* __restrict__ tstart,
    uint32_t* __restrict__ tfill, uint32_t* __restrict__ entries)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m)
        return;
    const uint32_t slot = slotOfEntry[e];
    if (slot == 0xFFFFFFFFu)
        return;
    const uint32_t p = tstart[slot] + atomicAdd(&tfill[slot], 1u);
    entries[p] = epayload[e];
}

__global__ void tableRangesKernel(ulonglong2* __restrict__ slots, const uint32_t* __restrict__ tstart, const uint32_t* __restrict__ tcount, uint32_t cap,
    uint32_t* __restrict__ filter, uint32_t filterShift)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cap)
        return;
    const uint64_t key = slots[s].x;
    slots[s].y = (uint64_t)tstart[s] | ((uint64_t)tcount[s] << 32);
    if (key != 0) {
        const uint32_t x = filterFold(key);
        atomicOr(&filter[filterWordIndex(x, filterShift)], filterBits(x));
    }
}

// Runs of equal keys in a key-sorted entry array: flags[i] = 1 where a run starts.
__global__ void markRunsKernel(const uint64_t* __restrict__ keys, size_t m, uint32_t* __restrict__ flags)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m)
        flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// starts[run] = first entry of the run; starts[runs] = m.
__global__ void runStartsKernel(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ runIdx, size_t m, uint32_t* __restrict__ starts, uint32_t runs)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m && flags[i])
        starts[runIdx[i]] = (uint32_t)i;
    if (i == 0)
        starts[runs] = (uint32_t)m;
}

// Slot placement for runs sorted by key. A run's home slot is the top log2(cap) bits of its key, so
// the homes are non-decreasing in run order, and linear probing places run d at
//   pos_d = max(home_d, pos_{d-1} + 1) = d + max over j <= d of (home_j - j),
// an inclusive max-scan: no atomics, and the slots are written in increasing order. The slot array
// ends past max(cap - 1, pos of the last run) with an empty slot, so probes never wrap.
constexpr int kPlaceThreads = 256;
constexpr int kPlaceItems = 16;
constexpr int kPlaceTile = kPlaceThreads * kPlaceItems;

__device__ __forceinline__ long long runHomeMinusIndex(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ starts, uint32_t d, uint32_t homeShift)
{
    return (long long)(keys[starts[d]] >> homeShift) - (long long)d;
}

// Block-wide inclusive max-scan of one value per thread (kPlaceThreads threads); returns the
// exclusive prefix (LLONG_MIN for thread 0) and the block maximum.
__device__ __forceinline__ long long blockExclusiveMax(long long v, long long* sm, long long& total)
{
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if ((int)lane >= o)
            inc = max(inc, t);
    }
    if (lane == 31)
        sm[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        constexpr int NW = kPlaceThreads / 32;
        long long w = lane < NW ? sm[lane] : LLONG_MIN;
        long long wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, wi, o);
            if ((int)lane >= o)
                wi = max(wi, t);
        }
        const long long wex = __shfl_up_sync(0xffffffffu, wi, 1);
        if (lane < NW)
            sm[lane] = lane == 0 ? LLONG_MIN : wex;
        if (lane == NW - 1)
            sm[NW] = wi;
    }
    __syncthreads();
    const long long ex = __shfl_up_sync(0xffffffffu, inc, 1);
    const long long res = max(sm[warp], lane == 0 ? LLONG_MIN : ex);
    total = sm[kPlaceThreads / 32];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kPlaceThreads) runPlaceReduceKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ starts, uint32_t runs,
    uint32_t homeShift, long long* __restrict__ tileMax)
{
    __shared__ long long sm[kPlaceThreads / 32 + 1];
    long long m = LLONG_MIN;
    const uint32_t base = blockIdx.x * kPlaceTile;
#pragma unroll 4
    for (int k = 0; k < kPlaceItems; ++k) {
        const uint32_t d = base + k * kPlaceThreads + threadIdx.x;
        if (d < runs)
            m = max(m, runHomeMinusIndex(keys, starts, d, homeShift));
    }
    long long total;
    blockExclusiveMax(m, sm, total);
    if (threadIdx.x == 0)
        tileMax[blockIdx.x] = total;
}

// One block: tileMax becomes its exclusive max-scan; *total = the maximum over all tiles.
__global__ void __launch_bounds__(kPlaceThreads) tileMaxScanKernel(long long* __restrict__ tileMax, uint32_t numTiles, long long* __restrict__ total)
{
    __shared__ long long sm[kPlaceThreads / 32 + 1];
    long long carry = LLONG_MIN;
    for (uint32_t b = 0; b < numTiles; b += kPlaceThreads) {
        const uint32_t i = b + threadIdx.x;
        const long long v = i < numTiles ? tileMax[i] : LLONG_MIN;
        long long blockMax;
        const long long ex = blockExclusiveMax(v, sm, blockMax);
        if (i < numTiles)
            tileMax[i] = max(carry, ex);
        carry = max(carry, blockMax);
    }
    if (threadIdx.x == 0)
        *total = carry;
}

// Places every run of the tile: slots[pos] = (key, first entry | count << 32), and sets its filter
// bits. Warp w owns the tile's runs [w * 512, (w + 1) * 512), 32 consecutive runs per step (coalesced):
// a first sweep gives the warps' maxima, a second scans with a carried prefix and writes.
__global__ void __launch_bounds__(kPlaceThreads) runPlaceKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ starts, uint32_t runs,
    uint32_t homeShift, const long long* __restrict__ tilePrefix, ulonglong2* __restrict__ slots, uint32_t* __restrict__ filter, uint32_t filterShift)
{
    constexpr int WARPS = kPlaceThreads / 32, STEPS = kPlaceTile / kPlaceThreads; // 512 runs per warp
    __shared__ long long warpMax[WARPS];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t segBase = blockIdx.x * kPlaceTile + warp * (32 * STEPS);
    long long m = LLONG_MIN;
    for (int it = 0; it < STEPS; ++it) {
        const uint32_t d = segBase + it * 32 + lane;
        if (d < runs)
            m = max(m, runHomeMinusIndex(keys, starts, d, homeShift));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0)
        warpMax[warp] = m;
    __syncthreads();
    long long carry = tilePrefix[blockIdx.x];
    for (uint32_t w = 0; w < warp; ++w)
        carry = max(carry, warpMax[w]);
    for (int it = 0; it < STEPS; ++it) {
        const uint32_t d = segBase + it * 32 + lane;
        const bool valid = d < runs;
        uint32_t start = 0, cnt = 0;
        uint64_t key = 0;
        long long v = LLONG_MIN;
        if (valid) {
            start = starts[d];
            cnt = starts[d + 1] - start;
            key = keys[start];
            v = (long long)(key >> homeShift) - (long long)d;
        }
        long long inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, inc, o);
            if ((int)lane >= o)
                inc = max(inc, t);
        }
        if (valid) {
            const long long run = max(carry, inc);
            slots[(uint64_t)((long long)d + run)] = make_ulonglong2(key, (uint64_t)start | ((uint64_t)cnt << 32));
            const uint32_t x = filterFold(key);
            atomicOr(&filter[filterWordIndex(x, filterShift)], filterBits(x));
        }
        carry = max(carry, __shfl_sync(0xffffffffu, inc, 31));
    }
}

// rank[order[p]] = p: every item's position in popcount order.
__global__ void sortedPositionKernel(const uint32_t* __restrict__ order, uint32_t n, uint32_t* __restrict__ rank)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n)
        rank[order[p]] = p;
}

// The listed sources' sorted positions, as keys and values of an ascending sort; an index past the
// level's items records an argument error (and sorts last).
__global__ void gatherPositionsKernel(const uint32_t* __restrict__ sources, uint32_t m, const uint32_t* __restrict__ rank, uint32_t n,
    uint64_t* __restrict__ key, uint32_t* __restrict__ val, uint32_t* status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const uint32_t src = sources[i];
    if (src >= n) {
        setDeviceError(status, TDAG_ERR_ARG, 301);
        key[i] = 0xFFFFFFFFull;
        val[i] = 0;
        return;
    }
    key[i] = rank[src];
    val[i] = rank[src];
}

// Targets that a source at or after the next batch could still give a lower parent: live[t] = 1 when
// parent[t] > the next batch's minimum key.
__global__ void targetLiveKernel(const unsigned long long* __restrict__ parents, uint32_t n, unsigned long long minKeyNext, const uint32_t* __restrict__ gridOf,
    const unsigned long long* __restrict__ minKeyOfGrid, uint8_t* __restrict__ live)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n)
        live[t] = parents[t] > (gridOf ? minKeyOfGrid[gridOf[t]] : minKeyNext) ? 1 : 0;
}

// flags[e] = 1 for the entries of live targets (payload of a permuted corner view: item << 6 | view);
// *count = the live entries.
// Grid-stride over a fixed grid, one atomic per block (a per-warp atomic on one counter serialises).
__global__ void __launch_bounds__(256) entryLiveKernel(const uint32_t* __restrict__ pays, size_t m, const uint8_t* __restrict__ live,
    uint32_t* __restrict__ flags, uint32_t* __restrict__ count)
{
    __shared__ uint32_t warpCounts[8];
    uint32_t c = 0;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (size_t)gridDim.x * blockDim.x) {
        const uint32_t l = live[pays[e] >> 6];
        flags[e] = l;
        c += l;
    }
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0)
        warpCounts[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; ++w)
            t += warpCounts[w];
        if (t)
            atomicAdd(count, t);
    }
}

// Membership filter over the keys of the flagged entries only: a pruning round that keeps the table
// refreshes just the filter. A key is inserted by the first flagged entry of each flagged stretch
// (repeats are harmless: insertion is idempotent).
__global__ void liveFilterKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ flags, size_t m, uint32_t* __restrict__ filter,
    uint32_t filterShift)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m || !flags[e])
        return;
    const uint64_t k = keys[e];
    if (e > 0 && flags[e - 1] && keys[e - 1] == k)
        return;
    const uint32_t x = filterFold(k);
    atomicOr(&filter[filterWordIndex(x, filterShift)], filterBits(x));
}

// Stable compaction of the flagged entries to their exclusive-scan offsets (keeps the key order).
__global__ void compactEntriesKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ pays, const uint32_t* __restrict__ flags,
    const uint32_t* __restrict__ offs, size_t m, uint64_t* __restrict__ keysOut, uint32_t* __restrict__ paysOut)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m && flags[e]) {
        keysOut[offs[e]] = keys[e];
        paysOut[offs[e]] = pays[e];
    }
}

// ---------------------------------------------------------------------------- search
struct SearchParams {
    const uint64_t* grids; // n x W, original order
    const uint32_t* order; // sorted position -> original position
    uint32_t begin, end; // sorted positions of this batch
    const ulonglong2* slots;
    uint32_t capMask;
    const uint32_t* entries;
    const uint32_t* filter;
    uint32_t filterShift;
    unsigned long long* parents; // encoded parent per original position
    uint32_t* workCounter;
    unsigned long long* counters; // probes, filterPass, hits, candidates, verifications, verified
    uint32_t allowSym, allowPerm, allowTrans;
    // batched builds (null for a single grid): grid of every item, first sorted position of every
    // grid, and the batch's list of sorted source positions (indices begin..end of it)
    const uint32_t* gridOf;
    const uint32_t* segOff;
    const uint32_t* workList;
};

template <int R>
struct SearchShape {
    static constexpr int TEAM = R * R; // one thread per line
    static constexpr int TEAMS = kThreads / TEAM;
    static constexpr int W = R * R * R / 64;
    static constexpr int SY = R + 1;
    static constexpr int SZ = (R + 1) * R;
    static constexpr int GRID = (R + 1) * R * R; // padded u64 hash grid
    static constexpr int N = R * R * R;
    // per team: G1, G2, G3 (u64), srcW (u64), lines[3][R*R] (u16), queue[N] (u16), queue count (u32),
    // source info (u32 x 5: local position, first and end target of its grid, salt low/high)
    static constexpr size_t TEAM_BYTES = (size_t)(3 * GRID + W) * 8 + 3 * R * R * 2 + N * 2 + 32;
    static constexpr size_t SMEM = TEAM_BYTES * TEAMS + 16;
};

__device__ __forceinline__ int smemStride(int a, int SY, int SZ) { return a == 0 ? 1 : (a == 1 ? SY : SZ); }

// One row of the exact verification target == translate(mirror(permute(source, P), S), T)
// (find_translation.cpp:857-862): the target's row along x at (w1, w2) against the source line that
// the transform moves there. L = lines[a0]; lines[a][u_lo + R u_hi] holds the source's voxels along
// axis a (bit j = coordinate j).
template <int R>
__device__ __forceinline__ bool verifyRow(const uint64_t* __restrict__ tgrid, const uint16_t* L, int lo, int hi, int a1, uint32_t S, int T0, int T1, int T2, int w1,
    int w2)
{
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    const uint32_t bitOff = (uint32_t)(R * (w1 + R * w2));
    const uint32_t trow = (uint32_t)(tgrid[bitOff >> 6] >> (bitOff & 63)) & rowMask;
    int y1 = w1 - T1, y2 = w2 - T2;
    uint32_t zrow = 0;
    if (y1 >= 0 && y1 < R && y2 >= 0 && y2 < R) {
        if (S & 2)
            y1 = R - 1 - y1;
        if (S & 4)
            y2 = R - 1 - y2;
        // u[a1] = y1, u[a2] = y2; line index = u[lo] + R u[hi]
        const int ulo = (lo == a1) ? y1 : y2;
        const int uhi = (hi == a1) ? y1 : y2;
        uint32_t line = L[ulo + R * uhi];
        if (S & 1)
            line = __brev(line) >> (32 - R);
        zrow = (T0 >= 0) ? ((line << T0) & rowMask) : (line >> (-T0));
    }
    return zrow == trow;
}

// Exact verification by one thread, row by row.
template <int R>
__device__ __noinline__ bool verifyCandidate(const uint64_t* __restrict__ tgrid, const uint16_t* lines, int a0, int a1, int a2, uint32_t S, int T0, int T1, int T2)
{
    const uint16_t* L = lines + a0 * R * R;
    const int lo = otherLo(a0), hi = otherHi(a0);
    for (int w2 = 0; w2 < R; ++w2)
        for (int w1 = 0; w1 < R; ++w1)
            if (!verifyRow<R>(tgrid, L, lo, hi, a1, S, T0, T1, T2, w1, w2))
                return false;
    return true;
}

// The same verification by a whole warp: lane l checks rows l, l + 32, ... of the R * R rows, 32 rows
// per step, and the warp stops at the first step with a mismatch. Every lane of the warp calls it with
// the same arguments.
template <int R>
__device__ __noinline__ bool verifyCandidateWarp(const uint64_t* __restrict__ tgrid, const uint16_t* lines, int a0, int a1, uint32_t S, int T0, int T1, int T2,
    uint32_t lane)
{
    constexpr int ROWS = R * R;
    constexpr int STEPS = (ROWS + 31) / 32;
    const uint16_t* L = lines + a0 * R * R;
    const int lo = otherLo(a0), hi = otherHi(a0);
    // every row's loads are issued before the first compare (one memory latency per verification
    // instead of one per step): most verified candidates pass, so stopping early would save little
    bool ok = true;
#pragma unroll
    for (int k = 0; k < STEPS; ++k) {
        const int r = k * 32 + (int)lane;
        ok &= r >= ROWS || verifyRow<R>(tgrid, L, lo, hi, a1, S, T0, T1, T2, r % R, r / R);
    }
    return __all_sync(0xffffffffu, ok);
}

// This lane's share of a verification by a group of V lanes (V < 32): rows sub, sub + V, ... of the
// R * R rows. Short shares issue every row's loads before the first compare, like the warp version;
// long ones stop at the first mismatch.
template <int R, int V>
__device__ __forceinline__ bool verifyRowsOfLane(const uint64_t* __restrict__ tgrid, const uint16_t* lines, int a0, int a1, uint32_t S, int T0, int T1, int T2,
    uint32_t sub)
{
    constexpr int ROWS = R * R;
    constexpr int STEPS = (ROWS + V - 1) / V;
    const uint16_t* L = lines + a0 * R * R;
    const int lo = otherLo(a0), hi = otherHi(a0);
    bool ok = true;
    if constexpr (STEPS <= 8) {
#pragma unroll
        for (int k = 0; k < STEPS; ++k) {
            const int r = k * V + (int)sub;
            ok &= r >= ROWS || verifyRow<R>(tgrid, L, lo, hi, a1, S, T0, T1, T2, r % R, r / R);
        }
    } else {
        for (int k = 0; k < STEPS && ok; ++k) {
            const int r = k * V + (int)sub;
            if (r < ROWS)
                ok = verifyRow<R>(tgrid, L, lo, hi, a1, S, T0, T1, T2, r % R, r / R);
        }
    }
    return ok;
}

template <int R, int L>
__global__ void __launch_bounds__(kThreads, 2) searchKernel(SearchParams p)
{
    using Sh = SearchShape<R>;
    constexpr int TEAM = Sh::TEAM, TEAMS = Sh::TEAMS, W = Sh::W, SY = Sh::SY, SZ = Sh::SZ, N = Sh::N;
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    extern __shared__ __align__(16) uint8_t smem[];
    const int team = threadIdx.x / TEAM;
    const int tl = threadIdx.x % TEAM;
    const uint32_t lane = threadIdx.x & 31;
    uint8_t* tb = smem + (size_t)team * Sh::TEAM_BYTES;
    uint64_t* G1 = reinterpret_cast<uint64_t*>(tb);
    uint64_t* G2 = G1 + Sh::GRID;
    uint64_t* G3 = G2 + Sh::GRID;
    uint64_t* srcW = G3 + Sh::GRID;
    uint16_t* lines = reinterpret_cast<uint16_t*>(srcW + W);
    uint16_t* queue = lines + 3 * R * R;
    uint32_t* qcount = reinterpret_cast<uint32_t*>(queue + N);
    uint32_t* srcInfo = qcount + 1;
    uint32_t* shBase = reinterpret_cast<uint32_t*>(smem + Sh::TEAM_BYTES * TEAMS);
    const int c1 = tl % R, c2 = tl / R;

    unsigned long long cProbe = 0, cFilter = 0, cHit = 0, cCand = 0, cVer = 0, cOk = 0;

    for (;;) {
        if (threadIdx.x == 0)
            *shBase = p.begin + atomicAdd(p.workCounter, (uint32_t)TEAMS);
        __syncthreads();
        const uint32_t base = *shBase;
        __syncthreads();
        if (base >= p.end)
            break;
        const uint32_t wi = base + team;
        const bool valid = wi < p.end;
        const uint32_t r = valid ? (p.workList ? p.workList[wi] : wi) : 0u;
        uint64_t salt = 0;
        // ---- load the source grid and its three line orientations
        if (valid) {
            const uint32_t orig = p.order[r];
            const uint64_t* g = p.grids + (size_t)orig * W;
            for (int k = tl; k < W; k += TEAM)
                srcW[k] = g[k];
            const uint32_t sg = p.gridOf ? p.gridOf[orig] : 0u;
            salt = boxSalt(sg);
            if (tl == 0) {
                srcInfo[0] = p.segOff ? r - p.segOff[sg] : r;
                srcInfo[1] = p.segOff ? p.segOff[sg] : 0u;
                srcInfo[2] = p.segOff ? p.segOff[sg + 1] : 0xFFFFFFFFu;
            }
        }
        if (tl == 0)
            *qcount = 0;
        __syncthreads();
        if (valid) {
            const uint32_t off = (uint32_t)R * (c1 + R * c2); // x-line at (y, z) = (c1, c2)
            lines[tl] = (uint16_t)((srcW[off >> 6] >> (off & 63)) & rowMask);
            uint32_t ly = 0, lz = 0;
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const uint32_t iy = c1 + R * j + R * R * c2; // (x=c1, y=j, z=c2)
                const uint32_t iz = c1 + R * c2 + R * R * j; // (x=c1, y=c2, z=j)
                ly |= (uint32_t)((srcW[iy >> 6] >> (iy & 63)) & 1) << j;
                lz |= (uint32_t)((srcW[iz >> 6] >> (iz & 63)) & 1) << j;
            }
            lines[R * R + tl] = (uint16_t)ly; // index x + R z
            lines[2 * R * R + tl] = (uint16_t)lz; // index x + R y
        }
        __syncthreads();

        for (int a0 = 0; a0 < 3; ++a0) {
            for (int d0 = 1; d0 >= 0; --d0) {
                // ---- pass 1 along a0 from the occupancy bits
                if (valid) {
                    const int lo = otherLo(a0), hi = otherHi(a0);
                    const int ss = smemStride(a0, SY, SZ);
                    const int sbase = c1 * smemStride(lo, SY, SZ) + c2 * smemStride(hi, SY, SZ);
                    const uint32_t ln = lines[a0 * R * R + tl]; // this thread's line along a0
#pragma unroll 4
                    for (int c = 0; c < R; ++c)
                        G1[sbase + c * ss] = lineCode(ln, c, d0);
                }
                __syncthreads();
                for (int a1i = 0; a1i < 2; ++a1i) {
                    const int a1 = (a0 + 1 + a1i) % 3;
                    const int a2 = 3 - a0 - a1;
                    const uint32_t pid = 2 * a0 + (a2 < a1 ? 1 : 0);
                    for (int d1 = 1; d1 >= 0; --d1) {
                        // ---- pass 2 along a1
                        if (valid) {
                            const int lo = otherLo(a1), hi = otherHi(a1);
                            const int ss = smemStride(a1, SY, SZ);
                            const int sbase = c1 * smemStride(lo, SY, SZ) + c2 * smemStride(hi, SY, SZ);
                            uint64_t acc = 0;
#pragma unroll 4
                            for (int k = 0; k < R; ++k) {
                                const int c = d1 ? R - 1 - k : k;
                                acc = boxFold<1>(acc, G1[sbase + c * ss]);
                                G2[sbase + c * ss] = acc;
                            }
                        }
                        __syncthreads();
                        // ---- pass 3 along a2 into G3, fused with the membership filter; survivors queued
                        const int lo3 = otherLo(a2), hi3 = otherHi(a2);
                        const int ss3 = smemStride(a2, SY, SZ);
                        const int sbase3 = c1 * smemStride(lo3, SY, SZ) + c2 * smemStride(hi3, SY, SZ);
                        const int ls3 = a2 == 0 ? 1 : (a2 == 1 ? R : R * R); // logical stride along a2
                        const int lbase3 = c1 * (lo3 == 0 ? 1 : (lo3 == 1 ? R : R * R)) + c2 * (hi3 == 1 ? R : R * R);
#pragma unroll
                        for (int d2 = 1; d2 >= 0; --d2) {
                            uint32_t pass = 0;
                            if (valid) {
                                // fold the whole line first, then issue every filter load of the line
                                // before the first one is consumed
                                uint64_t acc = 0;
                                uint32_t started = 0;
                                uint32_t fx[R];
#pragma unroll
                                for (int k = 0; k < R; ++k) {
                                    const int c = d2 ? R - 1 - k : k;
                                    acc = boxFold<2>(acc, G2[sbase3 + c * ss3]);
                                    G3[sbase3 + c * ss3] = acc;
                                    started |= (uint32_t)(acc & 1u) << c;
                                    fx[k] = filterFold(acc ^ salt);
                                }
                                uint32_t word[R];
#pragma unroll
                                for (int k = 0; k < R; ++k) {
                                    const int c = d2 ? R - 1 - k : k;
                                    word[k] = ((started >> c) & 1u) ? __ldg(&p.filter[filterWordIndex(fx[k], p.filterShift)]) : 0u;
                                }
#pragma unroll
                                for (int k = 0; k < R; ++k) {
                                    const int c = d2 ? R - 1 - k : k;
                                    const uint32_t bits = filterBits(fx[k]);
                                    pass |= ((word[k] & bits) == bits ? 1u : 0u) << c;
                                }
                                cProbe += __popc(started);
                            }
                            // warp-aggregated enqueue of the surviving voxels (logical index x + R y + R^2 z)
                            {
                                const uint32_t np = __popc(pass);
                                cFilter += np;
                                uint32_t incl = np;
#pragma unroll
                                for (int o = 1; o < 32; o <<= 1) {
                                    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                                    if ((int)lane >= o)
                                        incl += t;
                                }
                                // teams smaller than a warp keep separate counters: restrict the scan to the team
                                uint32_t excl = incl - np;
                                if (TEAM < 32) {
                                    const uint32_t teamFirst = lane & ~(uint32_t)(TEAM - 1);
                                    // every lane takes part in the shuffle; lane 0's exclusive prefix is 0
                                    const uint32_t before = __shfl_sync(0xffffffffu, incl - np, teamFirst);
                                    excl -= before;
                                    const uint32_t teamTotal = __shfl_sync(0xffffffffu, incl, teamFirst + TEAM - 1) - before;
                                    uint32_t off = 0;
                                    if (tl == 0 && teamTotal)
                                        off = atomicAdd(qcount, teamTotal);
                                    off = __shfl_sync(0xffffffffu, off, teamFirst);
                                    excl += off;
                                } else {
                                    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                                    uint32_t off = 0;
                                    if (lane == 0 && total)
                                        off = atomicAdd(qcount, total);
                                    excl += __shfl_sync(0xffffffffu, off, 0);
                                }
                                while (pass) {
                                    const int c = __ffs(pass) - 1;
                                    pass &= pass - 1;
                                    queue[excl++] = (uint16_t)(lbase3 + c * ls3);
                                }
                            }
                            __syncthreads();
                            // ---- table lookups and candidates (warp-uniform trip count)
                            const uint32_t qn = valid ? *qcount : 0u;
                            const uint32_t qmax = __reduce_max_sync(0xffffffffu, qn);
                            const uint32_t dir = (uint32_t)d0 | ((uint32_t)d1 << 1) | ((uint32_t)d2 << 2);
                            for (uint32_t qb = 0; qb < qmax; qb += TEAM) {
                                const uint32_t q = qb + tl;
                                uint32_t start = 0, cnt = 0, vidx = 0;
                                if (q < qn) {
                                    vidx = queue[q];
                                    const int x = vidx % R, y = (vidx / R) % R, z = vidx / (R * R);
                                    const uint64_t h = G3[x + SY * y + SZ * z] ^ salt;
                                    uint32_t slot = slotHash(h) & p.capMask;
                                    for (uint32_t probe = 0; probe <= p.capMask; ++probe) {
                                        const ulonglong2 sv = p.slots[slot];
                                        if (sv.x == h) {
                                            start = (uint32_t)sv.y;
                                            cnt = (uint32_t)(sv.y >> 32);
                                            break;
                                        }
                                        if (sv.x == 0)
                                            break;
                                        slot = (slot + 1) & p.capMask;
                                    }
                                    cHit += cnt ? 1 : 0;
                                }
                                const int an0 = d0 ? 0 : R - 1, an1 = d1 ? 0 : R - 1, an2 = d2 ? 0 : R - 1;
                                // One candidate (target, corner) of a hit at permuted voxel (v0, v1, v2) of the
                                // source of team srcTeam (find_translation.cpp:820-864).
                                auto candidate = [&](uint32_t pay, int v0, int v1, int v2, uint32_t srcTeam, uint32_t rSrc, uint32_t tLo, uint32_t tHi) {
                                    const uint32_t tgt = pay >> 3;
                                    const uint32_t S = dir ^ (pay & 7);
                                    ++cCand;
                                    if (tgt < tLo || tgt >= tHi) // another grid of the batch
                                        return;
                                    const int T0 = (S & 1) ? v0 - an0 : an0 - v0;
                                    const int T1 = (S & 2) ? v1 - an1 : an1 - v1;
                                    const int T2 = (S & 4) ? v2 - an2 : an2 - v2;
                                    if (!p.allowPerm && pid != 0)
                                        return;
                                    if (!p.allowSym && S != 0)
                                        return;
                                    if (!p.allowTrans && (T0 | T1 | T2) != 0)
                                        return;
                                    const uint64_t key = encodeFixed64(rSrc, pid, S, T0, T1, T2, L);
                                    const unsigned long long cur = *((volatile unsigned long long*)&p.parents[tgt]);
                                    if (key >= cur)
                                        return;
                                    ++cVer;
                                    const uint16_t* srcLines = reinterpret_cast<const uint16_t*>(
                                        reinterpret_cast<const uint64_t*>(smem + (size_t)srcTeam * Sh::TEAM_BYTES) + 3 * Sh::GRID + W);
                                    if (!verifyCandidate<R>(p.grids + (size_t)tgt * W, srcLines, a0, a1, a2, S, T0, T1, T2))
                                        return;
                                    ++cOk;
                                    atomicMin(&p.parents[tgt], (unsigned long long)key);
                                };
                                auto teamInfo = [&](uint32_t t) {
                                    return reinterpret_cast<const uint32_t*>(smem + (size_t)t * Sh::TEAM_BYTES + (size_t)(3 * Sh::GRID + W) * 8 + 3 * R * R * 2 + N * 2) + 1;
                                };
                                auto permutedVoxel = [&](uint32_t v, int& v0, int& v1, int& v2) {
                                    const int ux = v % R, uy = (v / R) % R, uz = v / (R * R);
                                    v0 = a0 == 0 ? ux : (a0 == 1 ? uy : uz);
                                    v1 = a1 == 0 ? ux : (a1 == 1 ? uy : uz);
                                    v2 = a2 == 0 ? ux : (a2 == 1 ? uy : uz);
                                };
                                // short ranges: every lane walks its own hit's candidates
                                constexpr uint32_t kSerialMax = 8;
                                if (cnt != 0 && cnt <= kSerialMax) {
                                    const uint32_t myTeam = threadIdx.x / TEAM;
                                    const uint32_t* info = teamInfo(myTeam);
                                    int v0, v1, v2;
                                    permutedVoxel(vidx, v0, v1, v2);
                                    for (uint32_t e = 0; e < cnt; ++e)
                                        candidate(__ldg(&p.entries[start + e]), v0, v1, v2, myTeam, info[0], info[1], info[2]);
                                }
                                // long ranges: the warp walks one range at a time
                                uint32_t hitMask = __ballot_sync(0xffffffffu, cnt > kSerialMax);
                                while (hitMask) {
                                    const int src = __ffs(hitMask) - 1;
                                    hitMask &= hitMask - 1;
                                    const uint32_t bs = __shfl_sync(0xffffffffu, start, src);
                                    const uint32_t bc = __shfl_sync(0xffffffffu, cnt, src);
                                    const uint32_t bv = __shfl_sync(0xffffffffu, vidx, src);
                                    const uint32_t srcTeam = ((threadIdx.x & ~31u) + src) / TEAM;
                                    const uint32_t* info = teamInfo(srcTeam);
                                    int v0, v1, v2;
                                    permutedVoxel(bv, v0, v1, v2);
                                    for (uint32_t e = lane; e < bc; e += 32)
                                        candidate(__ldg(&p.entries[bs + e]), v0, v1, v2, srcTeam, info[0], info[1], info[2]);
                                }
                            }
                            if (tl == 0)
                                *qcount = 0;
                            __syncthreads();
                        }
                    }
                }
            }
        }
    }
    // ---- counters
    unsigned long long vals[6] = { cProbe, cFilter, cHit, cCand, cVer, cOk };
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        unsigned long long v = vals[k];
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v)
            atomicAdd(&p.counters[k], v);
    }
}

// ---------------------------------------------------------------------------- split search
// The same search as searchKernel in two stages, so that neither waits on the other's latencies:
//  1. probeKernel folds the box hashes of every (source, orientation, voxel) in shared memory, tests
//     them against the membership filter and appends the survivors to a record list in device
//     memory (per-warp staging in shared memory, one atomic per flush);
//  2. lookupKernel takes one record per thread: table probe, then the candidates of a hit.
// Record: x = box hash (salted), y = w | vidx << 32 | pid << 44 | dir << 47, with w the source's
// index in the probed range, vidx = x + R y + R^2 z of the voxel in source coordinates, pid the axis
// permutation 2 a0 + (a2 < a1) and dir the fold direction bits d0 | d1 << 1 | d2 << 2.
struct ProbeParams {
    const uint64_t* grids;
    const uint32_t* order;
    const uint32_t* workList; // null: the range is sorted positions
    uint32_t begin, end; // probed range (of sorted positions or of workList)
    const uint32_t* filter;
    uint32_t filterShift;
    const uint32_t* gridOf;
    ulonglong2* recs;
    unsigned long long* recCount; // records produced; past recCap they are counted but not stored
    unsigned long long recCap;
    uint16_t* srcLines; // [end - begin][3][R * R]: every source's lines, for verification
    uint32_t* workCounter;
    unsigned long long* counters; // [0] probes, [1] filter passes
    uint32_t* status;
    uint32_t bulkCopy; // level 4: source grids arrive by a bulk copy one source ahead (ProbeShape::TMA)
};

template <int R>
struct ProbeShape {
    static constexpr int TEAM = R * R; // pass 2: thread per (v0, w2); pass 3: thread per (v0, v1)
    static constexpr int TEAMS = kThreads / TEAM;
    static constexpr int W = R * R * R / 64;
    // G2[x + R y + PS z]: both passes read or write runs of consecutive x per team row; for R < 16 the
    // plane stride is padded so that the team rows of one warp fall into different banks
    static constexpr int PS = R * R + (R < 16 ? R : 0);
    static constexpr int CHUNK = 4; // pass-3 elements whose filter loads are in flight together
    static constexpr int STAGE = 96; // staged records per warp (four CTAs of R = 16 fit an SM)
    static constexpr int FLUSH = STAGE / 2; // a warp flushes once this many are staged
    // per team: G2 (u64), srcW (u64), x-lines[R*R] (u16)
    static constexpr size_t LINES_OFF = (size_t)(PS * R + W) * 8;
    static constexpr size_t TEAM_BYTES = (LINES_OFF + R * R * 2 + 15) & ~(size_t)15;
    static constexpr size_t STAGE_OFF = TEAM_BYTES * TEAMS;
    static constexpr size_t COUNT_OFF = STAGE_OFF + (size_t)(kThreads / 32) * STAGE * 16; // per-warp stage counts
    static constexpr size_t BOX_OFF = COUNT_OFF + (kThreads / 32) * 4; // per team: lo x y z, hi + 1 x y z
    static constexpr size_t BASE_OFF = BOX_OFF + TEAMS * 24; // work base (+ 12 spare bytes)
    // Level 4 (one team per CTA): two 512-byte source-grid buffers filled by bulk copies, and their
    // two mbarriers, after the work base.
    static constexpr bool TMA = R == 16;
    static constexpr size_t PREF_OFF = (BASE_OFF + 16 + 127) & ~(size_t)127;
    static constexpr size_t MBAR_OFF = PREF_OFF + 2 * W * 8;
    static constexpr size_t SMEM = TMA ? MBAR_OFF + 16 : BASE_OFF + 16;
    static_assert(STAGE_OFF % 16 == 0 && TEAM_BYTES % 16 == 0, "alignment");
    static_assert(R == 4 || LINES_OFF % 16 == 0, "pass-2 rows are read as 16-byte vectors");
    static_assert(R % CHUNK == 0, "chunks tile a line");
};

// The R line codes of one pass-2 row (R consecutive u16, 8-byte aligned for R = 4, else 16-byte),
// two per word.
template <int R>
__device__ __forceinline__ void loadRow(const uint16_t* row, uint32_t (&lv)[R / 2])
{
    if constexpr (R == 4) {
        const uint2 v = *reinterpret_cast<const uint2*>(row);
        lv[0] = v.x;
        lv[1] = v.y;
    } else {
#pragma unroll
        for (int q = 0; q < R / 8; ++q) {
            const uint4 v = reinterpret_cast<const uint4*>(row)[q];
            lv[4 * q] = v.x;
            lv[4 * q + 1] = v.y;
            lv[4 * q + 2] = v.z;
            lv[4 * q + 3] = v.w;
        }
    }
}

// Every source is folded in the identity axis order (x, then y, then z) in its eight directions; the
// other five axis orders are covered by the targets' permuted corner views (cornerViewsKernel).
// Only boxes that hold a voxel are probed. With the source's bounding box [lo, hi] per axis, the box
// from the anchor to v is empty unless v is past the box's start on every axis (v >= lo when folding
// up from 0, v <= hi when folding down from R-1). A team therefore runs pass 2 on the (x, z) pairs
// with x past the start and z in [lo, hi], and pass 3 on the (x, y) pairs past the start along x and
// y, folding each z line from its first plane that can be non-empty (rounded down to a chunk; the
// skipped elements hash to 0, exactly as if they had been folded). Planes outside [lo, hi] along z are
// empty and read as 0. SALTED: batch members' keys carry their grid salt.
template <int R, bool SALTED>
__global__ void __launch_bounds__(kThreads, 4) probeKernel(ProbeParams p)
{
    using Sh = ProbeShape<R>;
    constexpr int TEAM = Sh::TEAM, TEAMS = Sh::TEAMS, W = Sh::W, PS = Sh::PS, STAGE = Sh::STAGE, C = Sh::CHUNK;
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    extern __shared__ __align__(16) uint8_t smem[];
    const int team = threadIdx.x / TEAM;
    const int tl = threadIdx.x % TEAM;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint8_t* tb = smem + (size_t)team * Sh::TEAM_BYTES;
    uint64_t* G2 = reinterpret_cast<uint64_t*>(tb);
    uint64_t* srcW = G2 + PS * R;
    uint16_t* xLines = reinterpret_cast<uint16_t*>(tb + Sh::LINES_OFF); // [y + R z]
    ulonglong2* stage = reinterpret_cast<ulonglong2*>(smem + Sh::STAGE_OFF) + warp * STAGE;
    uint32_t* stageCnt = reinterpret_cast<uint32_t*>(smem + Sh::COUNT_OFF) + warp;
    uint32_t* box = reinterpret_cast<uint32_t*>(smem + Sh::BOX_OFF) + team * 6;
    uint32_t* shBase = reinterpret_cast<uint32_t*>(smem + Sh::BASE_OFF);
    // bulk-copy prefetch (level 4): buffer it & 1 holds the source of iteration `it`
    uint64_t* pref = reinterpret_cast<uint64_t*>(smem + (Sh::TMA ? Sh::PREF_OFF : 0));
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + (Sh::TMA ? Sh::MBAR_OFF : 0));
    const bool bulk = Sh::TMA && p.bulkCopy;
    auto sourceGrid = [&](uint32_t wi) {
        const uint32_t r = p.workList ? p.workList[wi] : wi;
        return p.grids + (size_t)p.order[r] * W;
    };
    // lanes of this thread's team within its warp (teams of 16 share a warp)
    const unsigned teamMask = TEAM >= 32 ? 0xffffffffu : (((1u << TEAM) - 1u) << (lane & ~(uint32_t)(TEAM - 1)));
    uint32_t cProbe = 0, cFilter = 0;
    if (lane == 0)
        *stageCnt = 0;
    __syncwarp();
    uint64_t polLast = 0, polFirst = 0; // L2 hints of level 4
    if constexpr (R == 16) {
        polLast = l2PolicyEvictLast();
        polFirst = l2PolicyEvictFirst();
    }

    // Warp-uniform: copy the staged records (at most STAGE; reservations past it were written
    // directly by their lanes) to the record list.
    auto flushStage = [&](uint32_t minCount) {
        __syncwarp();
        const uint32_t cnt = *reinterpret_cast<volatile uint32_t*>(stageCnt);
        if (cnt < minCount || cnt == 0)
            return;
        const uint32_t nrec = cnt < (uint32_t)STAGE ? cnt : (uint32_t)STAGE;
        unsigned long long g = 0;
        if (lane == 0)
            g = atomicAdd(p.recCount, (unsigned long long)nrec);
        g = __shfl_sync(0xffffffffu, g, 0);
        for (uint32_t i = lane; i < nrec; i += 32)
            if (g + i < p.recCap)
                if constexpr (R == 16)
                    stL2Hint(&p.recs[g + i], stage[i], polFirst);
                else
                    p.recs[g + i] = stage[i];
        __syncwarp();
        if (lane == 0)
            *stageCnt = 0;
        __syncwarp();
    };

    if (bulk) {
        if (threadIdx.x == 0) {
            mbarInit(&mbar[0], 1);
            mbarInit(&mbar[1], 1);
            fenceProxyAsync();
            const uint32_t first = p.begin + atomicAdd(p.workCounter, 1u);
            *shBase = first;
            if (first < p.end)
                bulkCopyToShared(pref, sourceGrid(first), W * 8, &mbar[0]);
        }
        __syncthreads();
    }
    for (uint32_t it = 0;; ++it) {
        if (!bulk && threadIdx.x == 0)
            *shBase = p.begin + atomicAdd(p.workCounter, (uint32_t)TEAMS);
        __syncthreads();
        const uint32_t base = *shBase;
        __syncthreads();
        if (base >= p.end)
            break;
        const uint32_t wi = base + team;
        bool valid = wi < p.end;
        const uint32_t wIdx = wi - p.begin;
        uint64_t salt = 0;
        if (bulk) {
            // claim the next source and start its copy into the other buffer (read last iteration,
            // before the barriers above), then wait for this source's copy
            const int b = (int)(it & 1u);
            bool issued = false;
            if (threadIdx.x == 0) {
                const uint32_t next = p.begin + atomicAdd(p.workCounter, 1u);
                *shBase = next;
                if (next < p.end) {
                    fenceProxyAsync();
                    bulkCopyToShared(pref + (b ^ 1) * W, sourceGrid(next), W * 8, &mbar[b ^ 1]);
                    issued = true;
                }
            }
            const bool arrived = mbarWait(&mbar[b], (it >> 1) & 1u);
            if (__syncthreads_or(!arrived)) {
                // a copy never completed: record it, let the copy just issued land (bounded), stop
                if (threadIdx.x == 0) {
                    setDeviceError(p.status, TDAG_ERR_CUDA, 430);
                    if (issued)
                        mbarWait(&mbar[b ^ 1], ((it + 1) >> 1) & 1u);
                }
                break;
            }
            srcW = pref + b * W;
            if (SALTED)
                salt = boxSalt(p.gridOf[p.order[p.workList ? p.workList[wi] : wi]]);
        } else if (valid) {
            const uint32_t r = p.workList ? p.workList[wi] : wi;
            const uint32_t orig = p.order[r];
            const uint64_t* g = p.grids + (size_t)orig * W;
            for (int k = tl; k < W; k += TEAM)
                srcW[k] = g[k];
            if (SALTED)
                salt = boxSalt(p.gridOf[orig]);
        }
        if (tl == 0) {
            box[0] = box[1] = box[2] = R;
            box[3] = box[4] = box[5] = 0;
        }
        __syncthreads();
        if (valid) { // lines[a][u_lo + R u_hi]: the source's voxels along axis a, bit j = coordinate j
            const int tA = tl % R, tB = tl / R;
            const uint32_t off = (uint32_t)R * (tA + R * tB); // x-line at (y, z) = (tA, tB)
            const uint32_t lx = (uint32_t)(srcW[off >> 6] >> (off & 63)) & rowMask;
            uint32_t ly = 0, lz = 0;
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const uint32_t iy = tA + R * j + R * R * tB; // (x=tA, y=j, z=tB)
                const uint32_t iz = tA + R * tB + R * R * j; // (x=tA, y=tB, z=j)
                ly |= (uint32_t)((srcW[iy >> 6] >> (iy & 63)) & 1) << j;
                lz |= (uint32_t)((srcW[iz >> 6] >> (iz & 63)) & 1) << j;
            }
            xLines[tl] = (uint16_t)lx;
            uint16_t* dst = p.srcLines + (size_t)wIdx * 3 * R * R; // all three orientations, for verification
            if constexpr (R == 16) { // read back only for the sources that reach a verification
                stL2Hint(&dst[tl], (uint16_t)lx, polFirst);
                stL2Hint(&dst[R * R + tl], (uint16_t)ly, polFirst);
                stL2Hint(&dst[2 * R * R + tl], (uint16_t)lz, polFirst);
            } else {
                dst[tl] = (uint16_t)lx;
                dst[R * R + tl] = (uint16_t)ly;
                dst[2 * R * R + tl] = (uint16_t)lz;
            }
            // bounding box: lowest set coordinate and highest + 1 along every axis
            const uint32_t l3[3] = { lx, ly, lz };
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const uint32_t lo = __reduce_min_sync(teamMask, l3[a] ? (uint32_t)(__ffs(l3[a]) - 1) : (uint32_t)R);
                const uint32_t hi = __reduce_max_sync(teamMask, l3[a] ? (uint32_t)(32 - __clz(l3[a])) : 0u);
                if ((lane & (uint32_t)(TEAM >= 32 ? 31 : TEAM - 1)) == 0) {
                    atomicMin(&box[a], lo);
                    atomicMax(&box[3 + a], hi);
                }
            }
        }
        __syncthreads();
        const int loX = (int)box[0], loY = (int)box[1], loZ = (int)box[2];
        const int hiX = (int)box[3] - 1, hiY = (int)box[4] - 1, hiZ = (int)box[5] - 1;

        for (int d0 = 1; d0 >= 0; --d0) {
            // active x: the window along x ending at x holds a voxel
            const int v0s = d0 ? 0 : loX;
            const int n0 = d0 ? hiX + 1 : R - loX;
            const int r0 = n0 > 0 ? tl % n0 : 0, q0 = n0 > 0 ? tl / n0 : R;
            const int v0 = v0s + r0;
            for (int d1 = 1; d1 >= 0; --d1) {
                // ---- pass 2 along y from the exact x-line codes, thread (x, z = loZ + q0)
                if (valid && q0 <= hiZ - loZ) {
                    const int w2 = loZ + q0;
                    uint32_t lv[R / 2];
                    loadRow<R>(xLines + R * w2, lv);
                    uint64_t acc = 0;
#pragma unroll
                    for (int k = 0; k < R; ++k) {
                        const int j = d1 ? R - 1 - k : k;
                        const uint32_t ln = (lv[j >> 1] >> ((j & 1) * 16)) & 0xFFFFu;
                        acc = boxFold<1>(acc, lineCode(ln, v0, d0));
                        G2[v0 + R * j + PS * w2] = acc;
                    }
                }
                __syncthreads();
                // ---- pass 3 along z, both directions, thread (x, y = v1s + q0)
                const int v1s = d1 ? 0 : loY;
                const int n1 = d1 ? hiY + 1 : R - loY;
                const bool act3 = valid && q0 < n1;
                const int v1 = v1s + q0;
                const uint64_t* line3 = G2 + v0 + R * v1;
#pragma unroll
                for (int d2 = 1; d2 >= 0; --d2) {
                    if (act3) {
                        const uint64_t meta = (uint64_t)wIdx | ((uint64_t)((uint32_t)d0 | ((uint32_t)d1 << 1) | ((uint32_t)d2 << 2)) << 47);
                        const int k0 = d2 ? R - 1 - hiZ : loZ; // fold index of the first plane that can hold a voxel
                        uint64_t acc = 0;
#pragma unroll 1
                        for (int kq = k0 & ~(C - 1); kq < R; kq += C) {
                            uint64_t key[C];
                            uint32_t word[C], bits[C], nonEmpty = 0;
#pragma unroll
                            for (int c = 0; c < C; ++c) {
                                const int w = d2 ? R - 1 - (kq + c) : kq + c;
                                const uint64_t gv = line3[PS * w];
                                acc = boxFold<2>(acc, (w >= loZ && w <= hiZ) ? gv : 0ull);
                                nonEmpty |= (uint32_t)(acc & 1u) << c;
                                key[c] = viewKey(SALTED ? acc ^ salt : acc);
                            }
                            cProbe += __popc(nonEmpty);
#pragma unroll
                            for (int c = 0; c < C; ++c) {
                                const uint32_t x = filterFold(key[c]);
                                bits[c] = filterBits(x);
                                // level 4: box contents rarely repeat, so filter words bypass L1; the small
                                // boxes of levels 2-3 repeat often enough to hit in it
                                const uint32_t* fw = &p.filter[filterWordIndex(x, p.filterShift)];
                                word[c] = ((nonEmpty >> c) & 1u) ? (R == 16 ? ldL2Hint(fw, polLast) : __ldg(fw)) : 0u;
                            }
                            uint32_t hit = 0;
#pragma unroll
                            for (int c = 0; c < C; ++c)
                                hit |= ((word[c] & bits[c]) == bits[c] ? 1u : 0u) << c;
                            if (hit) {
                                const uint32_t k = __popc(hit);
                                cFilter += k;
                                uint32_t o = atomicAdd(stageCnt, k);
                                const uint32_t over = o + k > (uint32_t)STAGE ? o + k - max(o, (uint32_t)STAGE) : 0u;
                                unsigned long long g = 0;
                                if (over) // the stage is full: these go straight to the record list
                                    g = atomicAdd(p.recCount, (unsigned long long)over);
#pragma unroll
                                for (int c = 0; c < C; ++c) {
                                    if ((hit >> c) & 1u) {
                                        const int w = d2 ? R - 1 - (kq + c) : kq + c;
                                        const uint32_t vidx = (uint32_t)(v0 + R * v1 + R * R * w);
                                        const ulonglong2 rec = make_ulonglong2(key[c], meta | ((uint64_t)vidx << 32));
                                        if (o < (uint32_t)STAGE)
                                            stage[o] = rec;
                                        else if (g < p.recCap)
                                        {
                                            if constexpr (R == 16)
                                                stL2Hint(&p.recs[g], rec, polFirst);
                                            else
                                                p.recs[g] = rec;
                                            ++g;
                                        }
                                        else
                                            ++g;
                                        ++o;
                                    }
                                }
                            }
                        }
                    }
                    flushStage((uint32_t)Sh::FLUSH);
                }
                __syncthreads(); // the next pass 2 rewrites G2
            }
        }
    }
    flushStage(1);
    const uint32_t vals[2] = { cProbe, cFilter };
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        unsigned long long v = vals[k];
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v)
            atomicAdd(&p.counters[k], v);
    }
}

struct LookupParams {
    const ulonglong2* recs;
    const unsigned long long* countDev; // records the probe produced (device): past recCap the launch does nothing
    unsigned long long recCap;
    unsigned long long dynamicBelow; // fewer records than this: warps claim them from `cursor`
    const ulonglong2* slots; // run table: home slot = key >> homeShift, slotCount slots
    uint32_t homeShift;
    unsigned long long slotCount;
    const uint32_t* entries;
    const uint64_t* grids;
    const uint32_t* order;
    const uint32_t* workList;
    uint32_t begin; // the probed range's first position
    const uint16_t* srcLines;
    unsigned long long* parents;
    const uint32_t* gridOf;
    const uint32_t* segOff;
    uint32_t allowSym, allowPerm, allowTrans;
    unsigned long long* counters; // [2] hits, [3] candidates, [4] verifications, [5] verified, [6] longest run
    unsigned long long* cursor; // warps claim `tile` records at a time from it when dynamic (zeroed before the launch)
    uint32_t tile; // records per claim (a multiple of 32)
};

// V: lanes per candidate verification (32: the whole warp verifies one candidate at a time; 1, 4 or
// 8: the warp's 32 / V groups verify as many candidates side by side). The parent keys and so the
// result do not depend on V: a target keeps the smallest verified key whatever the order.
template <int R, int L, int V>
__global__ void __launch_bounds__(kThreads) lookupKernel(LookupParams p)
{
    static_assert(V == 1 || V == 4 || V == 8 || V == 32, "lanes per verification");
    const uint32_t lane = threadIdx.x & 31;
    uint32_t cHit = 0, cCand = 0, cVer = 0, cOk = 0, cMaxRun = 0;

    // every candidate (target, corner view) of the hit recorded in `m` (find_translation.cpp:820-864)
    struct Src {
        uint32_t rSrc, tLo, tHi, dir;
        int ux, uy, uz;
    };
    auto source = [&](uint64_t m) {
        Src s;
        const uint32_t w = (uint32_t)m;
        const uint32_t vidx = (uint32_t)(m >> 32) & 0xFFFu;
        s.dir = (uint32_t)(m >> 47) & 7u; // fold directions along x, y, z
        const uint32_t r = p.workList ? p.workList[p.begin + w] : p.begin + w;
        const uint32_t g = p.gridOf ? p.gridOf[p.order[r]] : 0u;
        s.rSrc = p.segOff ? r - p.segOff[g] : r;
        s.tLo = p.segOff ? p.segOff[g] : 0u;
        s.tHi = p.segOff ? p.segOff[g + 1] : 0xFFFFFFFFu;
        s.ux = (int)(vidx % R);
        s.uy = (int)((vidx / R) % R);
        s.uz = (int)(vidx / (R * R));
        return s;
    };
    // The view folded the target along b0, b1, b2 (pidB) from corner c'; the source was folded along
    // x, y, z in directions dir. In the reference's terms the source orientation is a = b^-1 (source
    // axis a_i lies along target axis i) with fold directions d_i = dir[a_i], the target corner is
    // c_i = c'[a_i], and S = d ^ c, v_i = u[a_i].
    // Prepares the candidate (target, corner view) `pay` of the hit recorded in `m`; true when it needs
    // verification, with the target, its key and the transform (a0 | a1 << 2 | S << 4 | T + 32 in
    // three 6-bit fields from bit 8) in `geo`.
    auto prepare = [&](uint32_t pay, uint64_t m, uint32_t& tgt, uint64_t& key, uint32_t& geo) -> bool {
        const Src s = source(m);
        tgt = pay >> 6;
        const uint32_t pb = (pay >> 3) & 7u, cp = pay & 7u;
        ++cCand;
        if (tgt < s.tLo || tgt >= s.tHi) // another grid of the batch
            return false;
        const int b0 = (int)(pb >> 1), blo = otherLo(b0), bhi = otherHi(b0);
        const int b1 = (pb & 1) ? bhi : blo;
        const int a0 = b0 == 0 ? 0 : (b1 == 0 ? 1 : 2);
        const int a1 = b0 == 1 ? 0 : (b1 == 1 ? 1 : 2);
        const int a2 = 3 - a0 - a1;
        const uint32_t pid = 2 * (uint32_t)a0 + (a2 < a1 ? 1u : 0u);
        const uint32_t xs = s.dir ^ cp;
        const uint32_t S = ((xs >> a0) & 1u) | (((xs >> a1) & 1u) << 1) | (((xs >> a2) & 1u) << 2);
        auto coord = [&](int a) { return a == 0 ? s.ux : (a == 1 ? s.uy : s.uz); };
        const int v0 = coord(a0), v1 = coord(a1), v2 = coord(a2);
        const int an0 = ((s.dir >> a0) & 1u) ? 0 : R - 1;
        const int an1 = ((s.dir >> a1) & 1u) ? 0 : R - 1;
        const int an2 = ((s.dir >> a2) & 1u) ? 0 : R - 1;
        const int T0 = (S & 1) ? v0 - an0 : an0 - v0;
        const int T1 = (S & 2) ? v1 - an1 : an1 - v1;
        const int T2 = (S & 4) ? v2 - an2 : an2 - v2;
        if (!p.allowPerm && pid != 0)
            return false;
        if (!p.allowSym && S != 0)
            return false;
        if (!p.allowTrans && (T0 | T1 | T2) != 0)
            return false;
        key = encodeFixed64(s.rSrc, pid, S, T0, T1, T2, L);
        const unsigned long long cur = *((volatile unsigned long long*)&p.parents[tgt]);
        if (key >= cur)
            return false;
        geo = (uint32_t)a0 | ((uint32_t)a1 << 2) | (S << 4) | ((uint32_t)(T0 + 32) << 8) | ((uint32_t)(T1 + 32) << 14) | ((uint32_t)(T2 + 32) << 20);
        return true;
    };
    // persistent warps, 32 consecutive records per step: with a cursor each warp claims its next 32
    // (balances the few-record batches whose records differ most in verification work; one counter
    // would serialise the claims of the large batches, which take records by a fixed stride)
    // the range's record count, read on the device: a range whose records overflowed their buffer
    // is probed again by the host with a larger one, so this launch leaves it alone
    const unsigned long long count = *p.countDev;
    if (count > p.recCap)
        return;
    const bool dynamic = count < p.dynamicBelow;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
    uint64_t claimEnd = 0;
    if (dynamic) {
        unsigned long long c = 0;
        if (lane == 0)
            c = atomicAdd(p.cursor, (unsigned long long)p.tile);
        i0 = __shfl_sync(0xffffffffu, c, 0);
        claimEnd = i0 + p.tile;
    }
    for (; i0 < count;) {
        const uint64_t i = i0 + lane;
        uint32_t start = 0, cnt = 0;
        uint64_t meta = 0;
        if (i < count) {
            const ulonglong2 rec = p.recs[i];
            meta = rec.y;
            // from the home slot up to the key or an empty slot (the array ends with one)
            for (uint64_t slot = rec.x >> p.homeShift; slot < p.slotCount; ++slot) {
                const ulonglong2 sv = p.slots[slot];
                if (sv.x == rec.x) {
                    start = (uint32_t)sv.y;
                    cnt = (uint32_t)(sv.y >> 32);
                    break;
                }
                if (sv.x == 0)
                    break;
            }
        }
        cHit += cnt ? 1u : 0u;
        cMaxRun = max(cMaxRun, cnt);
        // The warp's candidates, all hits' ranges end to end, dealt 32 at a time over the lanes: lane
        // j's hit is the first lane whose inclusive prefix of counts exceeds j (binary search by shuffles).
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o)
                incl += t;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t excl = incl - cnt;
        for (uint32_t jb = 0; jb < total; jb += 32) {
            const uint32_t j = jb + lane;
            uint32_t h = 0;
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, incl, h + step - 1) <= j)
                    h += step;
            h = min(h, 31u); // lanes past the total search to 32
            const uint32_t hs = __shfl_sync(0xffffffffu, start, h);
            const uint32_t hx = __shfl_sync(0xffffffffu, excl, h);
            const uint64_t hm = __shfl_sync(0xffffffffu, meta, h);
            uint32_t tgt = 0, geo = 0;
            uint64_t key = 0;
            const bool need = j < total && prepare(__ldg(&p.entries[hs + (j - hx)]), hm, tgt, key, geo);
            if constexpr (V < 32) {
                // The verifications of this step, 32 / V at a time: group g of V lanes takes the
                // g-th pending candidate of each round.
                constexpr uint32_t G = 32 / V;
                const uint32_t grp = lane / V, sub = lane % V;
                const uint32_t gmask = ((V == 32) ? 0xFFFFFFFFu : ((1u << V) - 1u)) << (grp * V);
                for (unsigned pending = __ballot_sync(0xffffffffu, need); pending;) {
                    unsigned mine = pending;
                    for (uint32_t k = 0; k < grp && mine; ++k)
                        mine &= mine - 1;
                    const bool have = mine != 0;
                    const int src = have ? __ffs(mine) - 1 : (int)lane;
                    for (uint32_t k = 0; k < G && pending; ++k)
                        pending &= pending - 1;
                    const uint32_t vt = __shfl_sync(0xffffffffu, tgt, src);
                    const uint64_t vk = __shfl_sync(0xffffffffu, key, src);
                    const uint32_t vg = __shfl_sync(0xffffffffu, geo, src);
                    const uint32_t vw = (uint32_t)__shfl_sync(0xffffffffu, hm, src);
                    unsigned long long cur = 0;
                    if (have && sub == 0)
                        cur = *((volatile unsigned long long*)&p.parents[vt]);
                    cur = __shfl_sync(0xffffffffu, cur, (int)(grp * V));
                    const bool go = have && vk < cur;
                    if (go && sub == 0)
                        ++cVer;
                    bool rowsOk = true;
                    if (go) {
                        const int T0 = (int)((vg >> 8) & 63u) - 32, T1 = (int)((vg >> 14) & 63u) - 32, T2 = (int)((vg >> 20) & 63u) - 32;
                        rowsOk = verifyRowsOfLane<R, V>(p.grids + (size_t)vt * (R * R * R / 64), p.srcLines + (size_t)vw * 3 * R * R, (int)(vg & 3u),
                            (int)((vg >> 2) & 3u), (vg >> 4) & 7u, T0, T1, T2, sub);
                    }
                    const uint32_t okMask = __ballot_sync(0xffffffffu, rowsOk);
                    if (go && sub == 0 && (okMask & gmask) == gmask) {
                        ++cOk;
                        atomicMin(&p.parents[vt], (unsigned long long)vk);
                    }
                }
            } else {
            // The verifications of this step, one candidate at a time by the whole warp (a lane alone
            // would run all R * R rows while the rest of the warp waits).
            for (unsigned pending = __ballot_sync(0xffffffffu, need); pending; pending &= pending - 1) {
                const int src = __ffs(pending) - 1;
                const uint32_t vt = __shfl_sync(0xffffffffu, tgt, src);
                const uint64_t vk = __shfl_sync(0xffffffffu, key, src);
                const uint32_t vg = __shfl_sync(0xffffffffu, geo, src);
                const uint32_t vw = (uint32_t)__shfl_sync(0xffffffffu, hm, src); // source index in the range
                // a verification earlier in this step may have lowered the target's parent already
                unsigned long long cur = 0;
                if ((int)lane == src)
                    cur = *((volatile unsigned long long*)&p.parents[vt]);
                cur = __shfl_sync(0xffffffffu, cur, src);
                if (vk >= cur)
                    continue;
                if ((int)lane == src)
                    ++cVer;
                const int T0 = (int)((vg >> 8) & 63u) - 32, T1 = (int)((vg >> 14) & 63u) - 32, T2 = (int)((vg >> 20) & 63u) - 32;
                const bool ok = verifyCandidateWarp<R>(p.grids + (size_t)vt * (R * R * R / 64), p.srcLines + (size_t)vw * 3 * R * R, (int)(vg & 3u),
                    (int)((vg >> 2) & 3u), (vg >> 4) & 7u, T0, T1, T2, lane);
                if (ok && (int)lane == src) {
                    ++cOk;
                    atomicMin(&p.parents[vt], (unsigned long long)vk);
                }
            }
            }
        }
        if (dynamic) {
            i0 += 32;
            if (i0 >= claimEnd) {
                unsigned long long c = 0;
                if (lane == 0)
                    c = atomicAdd(p.cursor, (unsigned long long)p.tile);
                i0 = __shfl_sync(0xffffffffu, c, 0);
                claimEnd = i0 + p.tile;
            }
        } else {
            i0 += stride;
        }
    }
    const uint32_t vals[4] = { cHit, cCand, cVer, cOk };
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        unsigned long long v = vals[k];
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v)
            atomicAdd(&p.counters[2 + k], v);
    }
    cMaxRun = __reduce_max_sync(0xffffffffu, cMaxRun);
    if (lane == 0 && cMaxRun)
        atomicMax(&p.counters[6], (unsigned long long)cMaxRun); // the longest run a record met (diagnostics)
}

// ---------------------------------------------------------------------------- resolve
__global__ void decodeParentsKernel(const unsigned long long* __restrict__ parents, uint32_t n, const uint32_t* __restrict__ order, uint64_t sentinelKey,
    uint32_t level, uint64_t* __restrict__ parentTP, uint32_t* __restrict__ isUnique, const uint32_t* __restrict__ gridOf = nullptr,
    const uint32_t* __restrict__ segOff = nullptr)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint64_t e = parents[i];
    if (e == sentinelKey) {
        parentTP[i] = tpSentinel();
        isUnique[i] = 1;
    } else {
        uint64_t v = decodeFixed64(e, level);
        const uint32_t src = order[tpPtr(v) + (gridOf ? segOff[gridOf[i]] : 0u)]; // parent's sorted position is local to the grid
        parentTP[i] = tpWithPtr(v, src);
        isUnique[src] = 1;
    }
}

__global__ void finalMappingKernel(const uint64_t* __restrict__ parentTP, const uint32_t* __restrict__ isUnique, const uint32_t* __restrict__ newIdx, uint32_t n,
    uint64_t* __restrict__ mapping, const uint32_t* __restrict__ gridOf = nullptr, const uint32_t* __restrict__ segOff = nullptr)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t base = gridOf ? newIdx[segOff[gridOf[i]]] : 0u; // kept items of earlier grids
    if (isUnique[i]) {
        mapping[i] = tpCreate(newIdx[i] - base, 0, 0);
    } else {
        const uint64_t pt = parentTP[i];
        mapping[i] = tpWithPtr(pt, newIdx[tpPtr(pt)] - base);
    }
}

uint64_t pow2AtLeast(uint64_t v)
{
    uint64_t p = 1;
    while (p < v)
        p <<= 1;
    return p;
}

// Corner-view table over entries sorted by key: one slot (key, first entry | count << 32) per run of
// equal keys, the entries being the sorted payload array itself (not owned), and the membership
// filter over the distinct keys.
struct Table {
    DevBuf<ulonglong2> slots;
    DevBuf<uint32_t> filter;
    const uint32_t* entries = nullptr;
    uint32_t homeShift = 58, filterShift = 31; // home slot = key >> homeShift
    uint64_t slotCount = 0, numEntries = 0, distinct = 0;
};

void buildRunTable(Context& ctx, const uint64_t* keys, const uint32_t* pays, size_t m, Table& t)
{
    cudaStream_t s = ctx.stream;
    TDAG_CHECK(m < (1ull << 32), TDAG_ERR_ARG, "corner-view table too large");
    DevBuf<uint32_t> flags(std::max<size_t>(m, 1), s), runIdx(std::max<size_t>(m, 1), s);
    uint64_t runs = 0;
    if (m) {
        markRunsKernel<<<gridFor(m, 256), 256, 0, s>>>(keys, m, flags.get());
        TDAG_LAUNCHED();
        runs = exclusiveScanU32Total(flags.get(), runIdx.get(), m, s);
    }
    DevBuf<uint32_t> starts(runs + 1, s);
    if (m) {
        runStartsKernel<<<gridFor(m, 256), 256, 0, s>>>(flags.get(), runIdx.get(), m, starts.get(), (uint32_t)runs);
        TDAG_LAUNCHED();
    }
    const uint32_t loadPct = ctx.tuning.table_load_percent ? std::min(85u, std::max(25u, ctx.tuning.table_load_percent)) : 50u;
    const uint64_t cap = pow2AtLeast(std::max<uint64_t>(64, runs * 100 / loadPct + 1));
    TDAG_CHECK(cap <= (1ull << 31), TDAG_ERR_ARG, "corner-view table too large");
    uint32_t log2Cap = 0;
    while ((1ull << log2Cap) < cap)
        ++log2Cap;
    t.homeShift = 64 - log2Cap;
    // Filter density: 32 bits per key unless the filter would then exceed 32 MB; past that a share of
    // the probes misses L2 (126 MB over two dies, each SM's die caching the lines it reads, shared with
    // the batch's grids and records), and halving the density (down to 8 bits per key) costs less in
    // extra false-positive lookups than the misses cost. 2048^3 grid, level-4 probe: 20.2 ms with a
    // 64 MB filter, 17.8 ms with 32 MB (8.0 GB of DRAM reads per build with 64 MB); 8192^3 grid: 337 ->
    // 273 ms per build at 8 bits per key.
    uint32_t bitsPerKey = ctx.tuning.filter_bits_per_key;
    if (!bitsPerKey) {
        bitsPerKey = 32;
        while (bitsPerKey > 8 && pow2AtLeast(std::max<uint64_t>(1024, runs * bitsPerKey)) > (1ull << 28))
            bitsPerKey /= 2;
    }
    const uint64_t filterBits = pow2AtLeast(std::max<uint64_t>(1024, runs * bitsPerKey));
    uint32_t log2F = 0;
    while ((1ull << log2F) < filterBits)
        ++log2F;
    t.filterShift = 32 - log2F;
    t.filter = DevBuf<uint32_t>(filterBits / 32, s);
    TDAG_CUDA(cudaMemsetAsync(t.filter.get(), 0, filterBits / 8, s));
    // slot positions: max-scan of home - index over the runs
    const uint32_t tiles = (uint32_t)std::max<uint64_t>(1, (runs + kPlaceTile - 1) / kPlaceTile);
    DevBuf<long long> tileMax(tiles, s), maxAll(1, s);
    long long maxHomeMinusIndex = 0;
    if (runs) {
        runPlaceReduceKernel<<<tiles, kPlaceThreads, 0, s>>>(keys, starts.get(), (uint32_t)runs, t.homeShift, tileMax.get());
        TDAG_LAUNCHED();
        tileMaxScanKernel<<<1, kPlaceThreads, 0, s>>>(tileMax.get(), tiles, maxAll.get());
        TDAG_LAUNCHED();
        uint64_t* h = pinnedScratch();
        readToHost({ { h, maxAll.get(), 8 } }, s);
        maxHomeMinusIndex = (long long)h[0];
    }
    // last run at runs - 1 + max(home - index); probes start at homes up to cap - 1; one empty slot after both
    const uint64_t slotCount = std::max<uint64_t>(cap, runs ? (uint64_t)((long long)runs + maxHomeMinusIndex) : 0) + 1;
    t.slots = DevBuf<ulonglong2>(slotCount, s);
    t.slotCount = slotCount;
    TDAG_CUDA(cudaMemsetAsync(t.slots.get(), 0, slotCount * sizeof(ulonglong2), s));
    if (runs) {
        runPlaceKernel<<<tiles, kPlaceThreads, 0, s>>>(keys, starts.get(), (uint32_t)runs, t.homeShift, tileMax.get(), t.slots.get(), t.filter.get(), t.filterShift);
        TDAG_LAUNCHED();
    }
    t.entries = pays;
    t.numEntries = m;
    t.distinct = runs;
    // no device-side error can arise while placing runs; the level's final status check covers the
    // launches, and the probe can be queued behind the placement without a host round trip
}

template <int L>
MatchOutput runMatcherL(Context& ctx, const uint64_t* grids, uint32_t n, const tdag_config& cfg, tdag_level_stats* stats, const Segments* seg,
    const uint32_t* sources, uint32_t numSources)
{
    constexpr int R = 1 << L;
    constexpr int W = R * R * R / 64;
    cudaStream_t s = ctx.stream;
    MatchOutput out;
    const bool batched = seg && seg->batched();
    const uint32_t numGrids = batched ? seg->numGrids : 1u;
    if (n == 0) {
        out.uniqueOff.assign(numGrids + 1, 0);
        return out;
    }
    TDAG_CHECK(n < (1u << 29), TDAG_ERR_ARG, "too many items for one matcher level");
    TDAG_CHECK(!sources || !batched, TDAG_ERR_ARG, "a source subset applies to a single grid");
    TDAG_CHECK(!sources || !replaying(), TDAG_ERR_ARG, "a source subset cannot be captured in a batch graph");
    const uint32_t* gridOf = batched ? seg->gridOf : nullptr;
    const uint32_t* segOff = batched ? seg->offDev : nullptr;

    // per-stage diagnostics on stderr (TDAG_TRACE)
    const bool trace = std::getenv("TDAG_TRACE") != nullptr && !replaying();
    // probe and batch timing (not while a batch graph captures the build: its events would not complete)
    const bool timed = !replaying();
    std::vector<std::pair<const char*, cudaEvent_t>> marks;
    auto mark = [&](const char* name) {
        if (!trace)
            return;
        cudaEvent_t e;
        TDAG_CUDA(cudaEventCreate(&e));
        TDAG_CUDA(cudaEventRecord(e, s));
        marks.emplace_back(name, e);
    };
    mark("start");

    // popcount order (grid by grid in a batch)
    DevBuf<uint32_t> order(n, s);
    {
        DevBuf<uint64_t> key(n, s);
        popcountKeyKernel<W><<<gridFor(n, 256), 256, 0, s>>>(grids, n, R * R * R, key.get(), order.get(), gridOf);
        TDAG_LAUNCHED();
        uint32_t bits = 16;
        while (batched && (1ull << (bits - 13)) < numGrids)
            bits += 8;
        radixSortPairs(key.get(), order.get(), n, 0, bits, s, ctx.status);
    }

    // learned-proposal mode: the sorted positions of the listed sources, ascending, as the work list
    std::vector<uint32_t> subsetHost;
    DevBuf<uint32_t> subsetDev;
    if (sources) {
        DevBuf<uint32_t> rank(n, s);
        sortedPositionKernel<<<gridFor(n, 256), 256, 0, s>>>(order.get(), n, rank.get());
        TDAG_LAUNCHED();
        DevBuf<uint64_t> sk(std::max<uint32_t>(numSources, 1), s);
        subsetDev = DevBuf<uint32_t>(std::max<uint32_t>(numSources, 1), s);
        if (numSources) {
            gatherPositionsKernel<<<gridFor(numSources, 256), 256, 0, s>>>(sources, numSources, rank.get(), n, sk.get(), subsetDev.get(), ctx.status);
            TDAG_LAUNCHED();
            radixSortPairs(sk.get(), subsetDev.get(), numSources, 0, 32, s, ctx.status);
            subsetHost.resize(numSources);
            TDAG_CUDA(cudaMemcpyAsync(subsetHost.data(), subsetDev.get(), (size_t)numSources * 4, cudaMemcpyDeviceToHost, s));
        }
        ctx.checkStatus("proposed sources");
    }

    // permuted corner views: 48 per item (8 when axis permutation is off: only the identity order)
    TDAG_CHECK(n < (1u << 26), TDAG_ERR_ARG, "too many items for one matcher level (corner-view payloads hold 26-bit item indices)");
    const uint32_t perms = cfg.axis_permutation ? 6u : 1u;
    const size_t m = (size_t)n * perms * 8;
    DevBuf<uint64_t> ekeys(m, s);
    DevBuf<uint32_t> epay(m, s);
    mark("order");
    cornerViewsKernel<R><<<gridFor(n, kThreads / 32), kThreads, 0, s>>>(grids, n, perms, ekeys.get(), epay.get(), gridOf);
    TDAG_LAUNCHED();
    mark("views");

    const uint64_t sentinelKey = encodeFixed64(0xFFFFFFFFull, 0, 0, 0, 0, 0, L);
    DevBuf<unsigned long long> parents(n, s);
    fillU64(reinterpret_cast<uint64_t*>(parents.get()), sentinelKey, n, s);
    DevBuf<uint32_t> work(1, s);
    DevBuf<unsigned long long> lookupCursor(1, s);
    DevBuf<unsigned long long> counters(8, s);
    TDAG_CUDA(cudaMemsetAsync(counters.get(), 0, 64, s));

    const size_t smem = ProbeShape<R>::SMEM;
    auto probe = batched ? probeKernel<R, true> : probeKernel<R, false>;
    TDAG_CUDA(cudaFuncSetAttribute(probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int perSM = 0;
    TDAG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, probe, kThreads, smem));
    if (ctx.tuning.search_ctas_per_sm)
        perSM = std::min<int>(perSM, (int)ctx.tuning.search_ctas_per_sm);
    perSM = std::max(perSM, 1);
    const uint32_t maxBlocks = (uint32_t)ctx.numSMs * perSM;
    // survivor records: at most a quarter of the free device memory per probed range
    const uint64_t freeBytes = deviceFreeBytes();
    const uint64_t maxRecords = std::max<uint64_t>(1u << 20, freeBytes / 4 / sizeof(ulonglong2));
    int lookupPerSM = 0;
    // lanes per candidate verification (tuning.verify_lanes: 1, 4, 8 or 32 (default)) and records per
    // dynamic claim (tuning.lookup_tile: 32 (default) .. 1024)
    const uint32_t vLanes = ctx.tuning.verify_lanes ? ctx.tuning.verify_lanes : 32u;
    TDAG_CHECK(vLanes == 1 || vLanes == 4 || vLanes == 8 || vLanes == 32, TDAG_ERR_ARG, "verify_lanes must be 1, 4, 8 or 32");
    auto lookup = vLanes == 1 ? lookupKernel<R, L, 1> : (vLanes == 4 ? lookupKernel<R, L, 4> : (vLanes == 8 ? lookupKernel<R, L, 8> : lookupKernel<R, L, 32>));
    const uint32_t lookupTile = ctx.tuning.lookup_tile ? ctx.tuning.lookup_tile : 32u;
    TDAG_CHECK(lookupTile >= 32 && lookupTile <= 1024 && lookupTile % 32 == 0, TDAG_ERR_ARG, "lookup_tile must be a multiple of 32 in 32..1024");
    TDAG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lookupPerSM, lookup, kThreads, 0));
    const uint32_t lookupBlocks = (uint32_t)ctx.numSMs * (uint32_t)std::max(lookupPerSM, 1);

    // Source batches. Single grid: ranges of sorted positions growing by the factor below (every batch
    // costs a pruning round, so a few large batches beat many small ones) after a first batch of one
    // team per SM, starting at eight teams per SM (fixed, so that the schedule does not move with the
    // probe kernel's occupancy). Batch: the same
    // fractions of every grid (1/512, 1/64, 1/8, 1), as a list of sorted positions per batch, with
    // each grid's own next-batch start for the pruning keys.
    std::vector<uint32_t> bounds { 0 };
    std::vector<uint32_t> workList;
    std::vector<std::vector<unsigned long long>> minKeys; // per batch, per grid
    // (the positions batched over: sorted positions, or indices into the subset's work list)
    const uint32_t nSrc = sources ? numSources : n;
    if (!batched) {
        const uint32_t minBatch = std::max<uint32_t>((uint32_t)ctx.numSMs * 8 * ProbeShape<R>::TEAMS, nSrc / 256);
        // Growth per batch. Every batch ends in a pruning round (liveness pass, filter refresh or table
        // rebuild); smaller grids probe faster, so their rounds weigh more: 16x at levels 2-3. At level
        // 4, up to 384 Ki sources 32x (2048^3 bench grid, 272 K sources: 49.2 -> 47.7 ms per build),
        // above that 8x, where the lookups the rounds save outweigh them (4096^3, 492 K sources: 91.4 ms
        // at 8x, 92.6 ms at 32x; 8192^3: 186.1 against 194.5 ms).
        const uint64_t growth = R == 16 ? (nSrc <= (384u << 10) ? 32 : 8) : 16;
        // A first batch of one team per SM: the largest sources give most targets that many sources
        // match (small, common boxes) their parent, and the pruning after it drops them, so that the
        // next batch's sources do not enumerate their table runs again.
        bounds.push_back(std::min<uint32_t>(nSrc, (uint32_t)ctx.numSMs * ProbeShape<R>::TEAMS));
        while (bounds.back() < nSrc) {
            const uint32_t b = bounds.back();
            bounds.push_back((uint32_t)std::min<uint64_t>(nSrc, std::max<uint64_t>((uint64_t)b + minBatch, growth * b)));
        }
    } else {
        constexpr int kBatches = 4; // fractions 1/512, 1/64, 1/8, 1: eightfold growth, as for a single grid
        auto frac = [](uint64_t cnt, int k) { return k == 0 ? 0ull : (k >= kBatches ? cnt : (cnt >> (3 * (kBatches - k)))); };
        workList.reserve(n);
        for (int k = 0; k < kBatches; ++k) {
            std::vector<unsigned long long> mk(numGrids);
            for (uint32_t g = 0; g < numGrids; ++g) {
                const uint64_t cnt = seg->off[g + 1] - seg->off[g];
                const uint64_t lo = frac(cnt, k), hi = frac(cnt, k + 1);
                for (uint64_t q = lo; q < hi; ++q)
                    workList.push_back((uint32_t)(seg->off[g] + q));
                mk[g] = encodeFixed64(lo, 0, 0, 1 - R, 1 - R, 1 - R, L);
            }
            minKeys.push_back(std::move(mk));
            bounds.push_back((uint32_t)workList.size());
        }
    }
    DevBuf<uint32_t> workListDev(workList.size(), s);
    DevBuf<unsigned long long> minKeyDev(numGrids, s);
    if (!workList.empty())
        uploadToDevice(workListDev.get(), workList.data(), workList.size() * 4, s);

    // equal view keys side by side (the sort is stable: a run keeps item order)
    radixSortPairs(ekeys.get(), epay.get(), m, kViewKeyLowBit, 64, s, ctx.status);
    mark("view sort");
    Table table;
    buildRunTable(ctx, ekeys.get(), epay.get(), m, table);
    mark("table");
    const uint64_t entriesInitial = table.numEntries;
    float searchMs = 0, probeMs = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> batchEv;
    struct EventPairs {
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>>& v;
        ~EventPairs()
        {
            for (auto& e : v) {
                if (e.first)
                    cudaEventDestroy(e.first);
                if (e.second)
                    cudaEventDestroy(e.second);
            }
        }
    } batchEvGuard { batchEv };
    DevBuf<uint32_t> flags(m, s), liveIdx(m, s);
    DevBuf<uint64_t> k2(m, s);
    DevBuf<uint32_t> p2(m, s);
    // the live entries, still sorted by key (pruning compacts them stably), and the spare pair
    uint64_t* curKeys = ekeys.get();
    uint32_t* curPays = epay.get();
    uint64_t* spareKeys = k2.get();
    uint32_t* sparePays = p2.get();
    size_t mCur = m;
    DevBuf<uint8_t> targetLive(n, s);
    DevBuf<uint32_t> liveCount(1, s); // live entries
    uint32_t maxBatch = 1;
    for (size_t bi = 0; bi + 1 < bounds.size(); ++bi)
        maxBatch = std::max(maxBatch, bounds[bi + 1] - bounds[bi]);
    DevBuf<uint16_t> srcLines((size_t)maxBatch * 3 * R * R, s);
    DevBuf<ulonglong2> recs;
    DevBuf<unsigned long long> recCount(1, s);
    double recsPerSource = 2.0 * R * R * R; // first estimate (the first batch's big sources pass the filter most); then a running average
    unsigned long long probeCounts[2] = { 0, 0 }; // probes and filter passes before the current range
    // per-batch diagnostics on stderr (TDAG_TRACE): probe and lookup time, records
    cudaEvent_t traceEv[2] = { nullptr, nullptr };
    if (trace)
        for (auto& e : traceEv)
            TDAG_CUDA(cudaEventCreate(&e));
    float traceProbeMs = 0, traceLookupMs = 0;
    unsigned long long traceRecords = 0;
    for (size_t bi = 0; bi + 1 < bounds.size(); ++bi) {
        const uint32_t b0 = bounds[bi], b1 = bounds[bi + 1];
        if (b0 == b1)
            continue;
        if (bi > 0) {
            // drop targets whose parent no source at or after this batch can lower
            const unsigned long long minKeyNext = encodeFixed64(sources ? subsetHost[b0] : b0, 0, 0, 1 - R, 1 - R, 1 - R, L);
            if (batched) {
                uploadToDevice(minKeyDev.get(), minKeys[bi].data(), (size_t)numGrids * 8, s);
                syncHost(s);
            }
            TDAG_CUDA(cudaMemsetAsync(liveCount.get(), 0, 4, s));
            targetLiveKernel<<<gridFor(n, 256), 256, 0, s>>>(parents.get(), n, minKeyNext, gridOf, batched ? minKeyDev.get() : nullptr, targetLive.get());
            TDAG_LAUNCHED();
            entryLiveKernel<<<(unsigned)std::min<uint64_t>(gridFor(mCur, 256), (uint64_t)ctx.numSMs * 8), 256, 0, s>>>(curPays, mCur, targetLive.get(),
                flags.get(), liveCount.get());
            TDAG_LAUNCHED();
            // the live entries' count decides between a filter refresh (no scan needed) and a compaction
            uint64_t* hp = pinnedScratch();
            readToHost({ { hp, liveCount.get(), 4 } }, s);
            const uint64_t live = hp[0] & 0xFFFFFFFFull;
            if (trace)
                std::fprintf(stderr, "[tdag] L%d before batch %zu: %llu of %llu entries live\n", L, bi, (unsigned long long)live, (unsigned long long)mCur);
            if (live == 0)
                break;
            if (2 * live >= mCur && mCur <= (1ull << 25)) {
                // Most entries live in a table of up to 2^25 entries: keep it and refresh only the
                // filter from the live keys. Dead entries left in a run cost a parent read in the
                // lookup, where their key (no smaller than minKeyNext) already fails the `key < parent`
                // test. Larger tables are compacted and rebuilt: there the dead entries' lookup work
                // outweighs a rebuild (2048^3: 67.7 -> 64.8 ms kept; 16384^3: 874 -> 1000 ms kept).
                TDAG_CUDA(cudaMemsetAsync(table.filter.get(), 0, table.filter.bytes(), s));
                liveFilterKernel<<<gridFor(mCur, 256), 256, 0, s>>>(curKeys, flags.get(), mCur, table.filter.get(), table.filterShift);
                TDAG_LAUNCHED();
            } else {
                exclusiveScanU32(flags.get(), liveIdx.get(), mCur, s);
                compactEntriesKernel<<<gridFor(mCur, 256), 256, 0, s>>>(curKeys, curPays, flags.get(), liveIdx.get(), mCur, spareKeys, sparePays);
                TDAG_LAUNCHED();
                std::swap(curKeys, spareKeys);
                std::swap(curPays, sparePays);
                mCur = live;
                buildRunTable(ctx, curKeys, curPays, mCur, table);
            }
        }
        ProbeParams pp {};
        pp.grids = grids;
        pp.order = order.get();
        pp.workList = batched ? workListDev.get() : (sources ? subsetDev.get() : nullptr);
        pp.filter = table.filter.get();
        pp.filterShift = table.filterShift;
        pp.gridOf = gridOf;
        pp.recCount = recCount.get();
        pp.workCounter = work.get();
        pp.counters = counters.get();
        pp.status = ctx.status;
        // 1: on, 0 (default) or 2: off; a bulk copy needs a 16-byte aligned source (caller-owned grids may not be)
        pp.bulkCopy = (ctx.tuning.probe_bulk_copy == 1 && ((uintptr_t)grids & 15u) == 0) ? 1u : 0u;
        LookupParams lp {};
        lp.slots = table.slots.get();
        lp.homeShift = table.homeShift;
        lp.slotCount = table.slotCount;
        lp.entries = table.entries;
        lp.grids = grids;
        lp.order = order.get();
        lp.workList = pp.workList;
        lp.parents = parents.get();
        lp.gridOf = gridOf;
        lp.segOff = segOff;
        lp.allowSym = cfg.symmetry ? 1 : 0;
        lp.allowPerm = cfg.axis_permutation ? 1 : 0;
        lp.allowTrans = cfg.translation ? 1 : 0;
        lp.counters = counters.get();
        // batch timing events, read once the level has finished (no round trip per batch)
        if (timed) {
            batchEv.emplace_back();
            TDAG_CUDA(cudaEventCreate(&batchEv.back().first));
            TDAG_CUDA(cudaEventCreate(&batchEv.back().second));
            TDAG_CUDA(cudaEventRecord(batchEv.back().first, s));
        }
        // Probe ranges of the batch sized so that their records fit; a range whose records overflow
        // the buffer is probed again after the buffer grew to the exact count (or, past the memory
        // limit, as two halves).
        for (uint32_t pos = b0; pos < b1;) {
            uint32_t cs = (uint32_t)std::min<uint64_t>(b1 - pos, std::max<uint64_t>(1, (uint64_t)((double)maxRecords / (recsPerSource * 1.25 + 1.0))));
            unsigned long long produced = 0;
            for (;;) {
                const uint64_t want = std::min<uint64_t>(maxRecords, (uint64_t)((double)cs * recsPerSource * 1.25) + 4096);
                if (recs.n < want)
                    recs = DevBuf<ulonglong2>(want, s);
                pp.recs = recs.get();
                pp.recCap = recs.n;
                pp.begin = pos;
                pp.end = pos + cs;
                pp.srcLines = srcLines.get();
                TDAG_CUDA(cudaMemsetAsync(work.get(), 0, 4, s));
                TDAG_CUDA(cudaMemsetAsync(recCount.get(), 0, 8, s));
                const uint64_t groups = ((uint64_t)cs + ProbeShape<R>::TEAMS - 1) / ProbeShape<R>::TEAMS;
                const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(maxBlocks, groups));
                if (timed)
                    TDAG_CUDA(cudaEventRecord(ctx.ev[5], s)); // ev[2..4] time the build's stages
                probe<<<blocks, kThreads, smem, s>>>(pp);
                TDAG_LAUNCHED();
                if (timed)
                    TDAG_CUDA(cudaEventRecord(ctx.ev[6], s));
                // The range's lookup follows at once, with no round trip: it reads the record count
                // on the device and returns without work if the records overflowed their buffer.
                lp.recs = recs.get();
                lp.countDev = recCount.get();
                lp.recCap = recs.n;
                lp.dynamicBelow = 1ull << 20; // few records: balance them dynamically
                lp.begin = pos;
                lp.srcLines = srcLines.get();
                lp.cursor = lookupCursor.get();
                lp.tile = lookupTile;
                TDAG_CUDA(cudaMemsetAsync(lp.cursor, 0, 8, s));
                if (trace)
                    TDAG_CUDA(cudaEventRecord(traceEv[0], s));
                lookup<<<lookupBlocks, kThreads, 0, s>>>(lp);
                TDAG_LAUNCHED();
                if (trace)
                    TDAG_CUDA(cudaEventRecord(traceEv[1], s));
                uint64_t* hp = pinnedScratch();
                readToHost({ { hp, recCount.get(), 8 } }, s);
                produced = hp[0];
                if (timed) {
                    float pm = 0; // the stream was synchronised for the record count
                    TDAG_CUDA(cudaEventElapsedTime(&pm, ctx.ev[5], ctx.ev[6]));
                    probeMs += pm;
                    traceProbeMs += pm;
                }
                if (trace) {
                    float lm = 0;
                    TDAG_CUDA(cudaEventElapsedTime(&lm, traceEv[0], traceEv[1]));
                    traceLookupMs += lm;
                }
                if (produced <= pp.recCap)
                    break;
                // the discarded run's probe and filter counts (diagnostics) are rolled back
                if (timed)
                    TDAG_CUDA(cudaMemcpyAsync(counters.get(), probeCounts, 16, cudaMemcpyHostToDevice, s));
                if (produced <= maxRecords) {
                    recsPerSource = std::max(recsPerSource, (double)produced / cs);
                    recs = DevBuf<ulonglong2>(produced, s);
                } else {
                    TDAG_CHECK(cs > 1, TDAG_ERR_OOM, "one source produced more probe records than fit in device memory");
                    cs = (cs + 1) / 2;
                }
            }
            if (timed)
                TDAG_CUDA(cudaMemcpyAsync(probeCounts, counters.get(), 16, cudaMemcpyDeviceToHost, s));
            recsPerSource = 0.5 * recsPerSource + 0.5 * ((double)produced / cs);
            traceRecords += produced;
            pos += cs;
        }
        if (timed)
            TDAG_CUDA(cudaEventRecord(batchEv.back().second, s));
        if (trace) {
            TDAG_CUDA(cudaEventSynchronize(batchEv.back().second));
            float ms = 0;
            TDAG_CUDA(cudaEventElapsedTime(&ms, batchEv.back().first, batchEv.back().second));
            unsigned long long c[8];
            TDAG_CUDA(cudaMemcpy(c, counters.get(), 64, cudaMemcpyDeviceToHost));
            std::fprintf(stderr, "[tdag] L%d batch %zu sources %u table %llu ms %.3f (probe %.3f lookup %.3f records %llu) | cumulative probes %llu filter %llu hits %llu cand %llu ver %llu longest run %llu\n",
                L, bi, b1 - b0, (unsigned long long)table.numEntries, ms, traceProbeMs, traceLookupMs, traceRecords, c[0], c[1], c[2], c[3], c[4], c[6]);
            traceProbeMs = traceLookupMs = 0;
            traceRecords = 0;
        }
    }
    for (auto e : traceEv)
        if (e)
            cudaEventDestroy(e);
    table = Table();
    flags.release();
    liveIdx.release();
    k2.release();
    p2.release();

    mark("batches");
    // resolve
    DevBuf<uint64_t> parentTP(n, s);
    DevBuf<uint32_t> isUnique(n, s), newIdx(n, s);
    TDAG_CUDA(cudaMemsetAsync(isUnique.get(), 0, (size_t)n * 4, s));
    decodeParentsKernel<<<gridFor(n, 256), 256, 0, s>>>(parents.get(), n, order.get(), sentinelKey, L, parentTP.get(), isUnique.get(), gridOf, segOff);
    TDAG_LAUNCHED();
    out.uniques = DevBuf<uint32_t>(n, s);
    out.numUnique = compactFlags(isUnique.get(), out.uniques.get(), n, s);
    exclusiveScanU32(isUnique.get(), newIdx.get(), n, s);
    out.mapping = DevBuf<uint64_t>(n, s);
    finalMappingKernel<<<gridFor(n, 256), 256, 0, s>>>(parentTP.get(), isUnique.get(), newIdx.get(), n, out.mapping.get(), gridOf, segOff);
    TDAG_LAUNCHED();
    out.uniqueOff = batched ? countPerGrid(gridOf, out.uniques.get(), out.numUnique, numGrids, s) : std::vector<uint64_t> { 0, out.numUnique };

    syncHost(s);
    for (auto& e : batchEv) {
        float ms = 0;
        TDAG_CUDA(cudaEventElapsedTime(&ms, e.first, e.second));
        searchMs += ms;
    }
    if (stats && timed) {
        unsigned long long c[8];
        TDAG_CUDA(cudaMemcpyAsync(c, counters.get(), 64, cudaMemcpyDeviceToHost, s));
        TDAG_CUDA(cudaStreamSynchronize(s));
        stats->items += n;
        stats->unique += out.numUnique;
        stats->probes += c[0];
        stats->filter_pass += c[1];
        stats->hits += c[2];
        stats->candidates += c[3];
        stats->verifications += c[4];
        stats->verified += c[5];
        stats->table_entries += entriesInitial;
        stats->search_ms += searchMs;
        stats->probe_ms += probeMs;
    }
    mark("resolve");
    if (trace) {
        TDAG_CUDA(cudaStreamSynchronize(s));
        std::string line = "[tdag] L" + std::to_string(L) + " stages ms:";
        for (size_t k = 1; k < marks.size(); ++k) {
            float ms = 0;
            TDAG_CUDA(cudaEventElapsedTime(&ms, marks[k - 1].second, marks[k].second));
            char buf[64];
            std::snprintf(buf, sizeof buf, " %s %.3f", marks[k].first, ms);
            line += buf;
        }
        std::fprintf(stderr, "%s (search %.3f)\n", line.c_str(), searchMs);
        for (auto& mk : marks)
            cudaEventDestroy(mk.second);
    }
    ctx.checkStatus("matcher level " + std::to_string(L));
    return out;
}

} // namespace

// ================================================================================================
// Matcher entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs inside a host application which owns every
// byte of device memory (a game engine's or renderer's fixed arena, a per-frame budget) or a
// memory-capped service where an allocation could fail or stall at an arbitrary point. For them,
// tdag_find_duplicates_level_noalloc runs one matcher level with all of its scratch (popcount
// order, corner-hash table and entries, membership filter, parents, resolve arrays) in one
// file-scope __device__ array of kNoAllocScratchBytes. The caller passes device pointers for the
// grids and the outputs; the function calls no cudaMalloc, cudaFree or allocating routine.
//
// Limits: at most kNoAllocMaxItems items per call (levels 2..4). The array is part of the module:
// every GPU that loads libtdag.so holds it until the process exits. All calls share it, so calls
// that overlap on the GPU (two contexts, or two threads on one context) race and must be
// serialised by the caller. tdag_ctx_create resolves the array's device address with
// cudaGetSymbolAddress (with the context's device current) and keeps it in the context, and it
// loads the kernels of this path, so that the driver's lazy module loading places the array and
// the code at context creation rather than inside the first call. The call is synchronous on the
// context's stream: it reads the device status word before it returns.
// ================================================================================================
namespace {

constexpr uint32_t kNoAllocMaxItems = 4096;
constexpr size_t kNoAllocScratchBytes = 4u << 20;
static __device__ __align__(256) unsigned char g_noAllocScratch[kNoAllocScratchBytes];

// Stable rank by popcount (descending) for n <= kNoAllocMaxItems: O(n^2) comparisons, no sort temp.
template <int W>
__global__ void noAllocRankKernel(const uint64_t* __restrict__ grids, uint32_t n, uint32_t* __restrict__ pc, uint32_t* __restrict__ order)
{
    __shared__ uint32_t cnt[kNoAllocMaxItems];
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t c = 0;
        for (int k = 0; k < W; ++k)
            c += __popcll(grids[(size_t)i * W + k]);
        cnt[i] = c;
        pc[i] = c;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint32_t rank = 0;
        const uint32_t ci = cnt[i];
        for (uint32_t j = 0; j < n; ++j)
            rank += (cnt[j] > ci) || (cnt[j] == ci && j < i);
        order[rank] = i;
    }
}

// Single-block exclusive scan (in < 2^32 total); writes the total to *total.
__global__ void noAllocScanKernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n, uint32_t* __restrict__ total)
{
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < n ? in[i] : 0;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o)
                incl += t;
        }
        if (lane == 31)
            warpSums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = lane < nw ? warpSums[lane] : 0;
            uint32_t wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
                if ((int)lane >= o)
                    wi += t;
            }
            if (lane < nw)
                warpSums[lane] = wi - w;
        }
        __syncthreads();
        const uint32_t c = carry;
        if (i < n)
            out[i] = c + warpSums[warp] + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1)
            carry = c + warpSums[warp] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *total = carry;
}

// Kept items -> compacted positions (the scan gives their new indices).
__global__ void noAllocUniquesKernel(const uint32_t* __restrict__ isUnique, const uint32_t* __restrict__ newIdx, uint32_t n, uint32_t* __restrict__ outUnique)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && isUnique[i])
        outUnique[newIdx[i]] = i;
}

struct NoAllocLayout {
    uint32_t *pc, *order, *epay, *slotOfEntry, *tcount, *tstart, *tfill, *entries, *filter, *isUnique, *newIdx, *misc;
    uint64_t *ekeys, *parentTP;
    unsigned long long *parents, *counters;
    ulonglong2* slots;
    uint32_t capMask, filterShift;
    size_t bytes;
};

// Carve the scratch array; cap and filter sized for n items.
NoAllocLayout noAllocCarve(unsigned char* base, uint32_t n)
{
    NoAllocLayout L {};
    const uint64_t m = (uint64_t)n * 8;
    const uint64_t cap = pow2AtLeast(std::max<uint64_t>(64, m * 2));
    const uint64_t filterBits = pow2AtLeast(std::max<uint64_t>(1024, m * 32));
    uint32_t log2F = 0;
    while ((1ull << log2F) < filterBits)
        ++log2F;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += (bytes + 255) & ~(size_t)255;
        return p;
    };
    L.slots = reinterpret_cast<ulonglong2*>(take(cap * 16));
    L.ekeys = reinterpret_cast<uint64_t*>(take(m * 8));
    L.parents = reinterpret_cast<unsigned long long*>(take((size_t)n * 8));
    L.parentTP = reinterpret_cast<uint64_t*>(take((size_t)n * 8));
    L.counters = reinterpret_cast<unsigned long long*>(take(64));
    L.pc = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
    L.order = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
    L.epay = reinterpret_cast<uint32_t*>(take(m * 4));
    L.slotOfEntry = reinterpret_cast<uint32_t*>(take(m * 4));
    L.tcount = reinterpret_cast<uint32_t*>(take(cap * 4));
    L.tstart = reinterpret_cast<uint32_t*>(take(cap * 4));
    L.tfill = reinterpret_cast<uint32_t*>(take(cap * 4));
    L.entries = reinterpret_cast<uint32_t*>(take(m * 4));
    L.filter = reinterpret_cast<uint32_t*>(take(filterBits / 8));
    L.isUnique = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
    L.newIdx = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
    L.misc = reinterpret_cast<uint32_t*>(take(64)); // [0] work counter, [1] distinct keys, [2] entries, [3] kept
    L.capMask = (uint32_t)(cap - 1);
    L.filterShift = 32 - log2F;
    L.bytes = off;
    return L;
}

template <int LV>
void runMatcherNoAlloc(Context& ctx, unsigned char* scratch, const uint64_t* grids, uint32_t n, const tdag_config& cfg, uint64_t* outMapping,
    uint32_t* outUnique, uint32_t* outCount)
{
    constexpr int R = 1 << LV;
    constexpr int W = R * R * R / 64;
    cudaStream_t s = ctx.stream;
    NoAllocLayout A = noAllocCarve(scratch, n);
    TDAG_CHECK(A.bytes <= kNoAllocScratchBytes, TDAG_ERR_ARG, "no-alloc scratch too small for this level and item count");
    const uint64_t m = (uint64_t)n * 8;
    const uint64_t cap = (uint64_t)A.capMask + 1;
    // everything that must start at zero (the array keeps the previous call's contents)
    TDAG_CUDA(cudaMemsetAsync(A.slots, 0, cap * 16, s));
    TDAG_CUDA(cudaMemsetAsync(A.tcount, 0, cap * 4, s));
    TDAG_CUDA(cudaMemsetAsync(A.tfill, 0, cap * 4, s));
    TDAG_CUDA(cudaMemsetAsync(A.filter, 0, (size_t)1 << (32 - A.filterShift) >> 3, s));
    TDAG_CUDA(cudaMemsetAsync(A.isUnique, 0, (size_t)n * 4, s));
    TDAG_CUDA(cudaMemsetAsync(A.counters, 0, 64, s));
    TDAG_CUDA(cudaMemsetAsync(A.misc, 0, 64, s));

    noAllocRankKernel<W><<<1, 1024, 0, s>>>(grids, n, A.pc, A.order);
    TDAG_LAUNCHED();
    cornerHashKernel<R><<<gridFor(m * 32, kThreads), kThreads, 0, s>>>(grids, n, A.ekeys, A.epay, nullptr);
    TDAG_LAUNCHED();
    tableInsertKernel<<<gridFor(m, 256), 256, 0, s>>>(A.ekeys, m, A.slots, A.tcount, A.slotOfEntry, A.capMask, A.misc + 1, ctx.status);
    TDAG_LAUNCHED();
    noAllocScanKernel<<<1, 1024, 0, s>>>(A.tcount, A.tstart, (uint32_t)cap, A.misc + 2);
    TDAG_LAUNCHED();
    tableScatterKernel<<<gridFor(m, 256), 256, 0, s>>>(A.epay, A.slotOfEntry, m, A.tstart, A.tfill, A.entries);
    TDAG_LAUNCHED();
    tableRangesKernel<<<gridFor(cap, 256), 256, 0, s>>>(A.slots, A.tstart, A.tcount, (uint32_t)cap, A.filter, A.filterShift);
    TDAG_LAUNCHED();
    const uint64_t sentinelKey = encodeFixed64(0xFFFFFFFFull, 0, 0, 0, 0, 0, LV);
    fillU64(reinterpret_cast<uint64_t*>(A.parents), sentinelKey, n, s);

    SearchParams sp {};
    sp.grids = grids;
    sp.order = A.order;
    sp.begin = 0;
    sp.end = n;
    sp.slots = A.slots;
    sp.capMask = A.capMask;
    sp.entries = A.entries;
    sp.filter = A.filter;
    sp.filterShift = A.filterShift;
    sp.parents = A.parents;
    sp.workCounter = A.misc;
    sp.counters = A.counters;
    sp.allowSym = cfg.symmetry ? 1 : 0;
    sp.allowPerm = cfg.axis_permutation ? 1 : 0;
    sp.allowTrans = cfg.translation ? 1 : 0;
    const size_t smem = SearchShape<R>::SMEM;
    TDAG_CUDA(cudaFuncSetAttribute(searchKernel<R, LV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned blocks = (unsigned)std::max<uint32_t>(1, std::min<uint32_t>((uint32_t)ctx.numSMs * 2, (n + SearchShape<R>::TEAMS - 1) / SearchShape<R>::TEAMS));
    searchKernel<R, LV><<<blocks, kThreads, smem, s>>>(sp);
    TDAG_LAUNCHED();

    decodeParentsKernel<<<gridFor(n, 256), 256, 0, s>>>(A.parents, n, A.order, sentinelKey, LV, A.parentTP, A.isUnique);
    TDAG_LAUNCHED();
    noAllocScanKernel<<<1, 1024, 0, s>>>(A.isUnique, A.newIdx, n, outCount);
    TDAG_LAUNCHED();
    noAllocUniquesKernel<<<gridFor(n, 256), 256, 0, s>>>(A.isUnique, A.newIdx, n, outUnique);
    TDAG_LAUNCHED();
    finalMappingKernel<<<gridFor(n, 256), 256, 0, s>>>(A.parentTP, A.isUnique, A.newIdx, n, outMapping);
    TDAG_LAUNCHED();
    ctx.checkStatus("no-alloc matcher level " + std::to_string(LV));
}

template <typename K>
void loadKernel(K* kernel)
{
    cudaFuncAttributes fa;
    TDAG_CUDA(cudaFuncGetAttributes(&fa, kernel));
}

} // namespace

// Called by tdag_ctx_create with the context's device current: the scratch array's device address
// (kept in the context, so that it always belongs to the current primary context of the device) and
// every kernel the no-allocation path launches, loaded now instead of lazily inside its first call.
void prepareNoAlloc(Context& ctx)
{
    void* p = nullptr;
    TDAG_CUDA(cudaGetSymbolAddress(&p, g_noAllocScratch));
    ctx.noAllocScratch = static_cast<unsigned char*>(p);
    loadKernel(noAllocRankKernel<1>);
    loadKernel(noAllocRankKernel<8>);
    loadKernel(noAllocRankKernel<64>);
    loadKernel(cornerHashKernel<4>);
    loadKernel(cornerHashKernel<8>);
    loadKernel(cornerHashKernel<16>);
    loadKernel(searchKernel<4, 2>);
    loadKernel(searchKernel<8, 3>);
    loadKernel(searchKernel<16, 4>);
    loadKernel(tableInsertKernel);
    loadKernel(noAllocScanKernel);
    loadKernel(tableScatterKernel);
    loadKernel(tableRangesKernel);
    loadKernel(decodeParentsKernel);
    loadKernel(noAllocUniquesKernel);
    loadKernel(finalMappingKernel);
    preloadFillKernels();
}

MatchOutput runMatcher(Context& ctx, uint32_t level, const uint64_t* grids, uint32_t n, const tdag_config& cfg, tdag_level_stats* stats, const Segments* seg,
    const uint32_t* sources, uint32_t numSources)
{
    switch (level) {
    case 2:
        return runMatcherL<2>(ctx, grids, n, cfg, stats, seg, sources, numSources);
    case 3:
        return runMatcherL<3>(ctx, grids, n, cfg, stats, seg, sources, numSources);
    case 4:
        return runMatcherL<4>(ctx, grids, n, cfg, stats, seg, sources, numSources);
    default:
        throw Error(TDAG_ERR_ARG, "translation matching supports levels 2..4");
    }
}

} // namespace tdag

// ================================================================================================
// C ABI of the no-allocation matcher entry point
// ================================================================================================
struct tdag_ctx;
tdag::Context& ctxOf(tdag_ctx* c); // build.cu
int guardedCall(const std::function<void()>& f); // build.cu
int failWith(int code, const char* msg); // build.cu

extern "C" int tdag_find_duplicates_level_noalloc(tdag_ctx* ctx, uint32_t level, const uint64_t* d_grids, uint32_t n, const tdag_config* cfg,
    uint64_t* d_out_mapping, uint32_t* d_out_unique, uint32_t* d_n_unique)
{
    using namespace tdag;
    if (!ctx || !cfg || !d_n_unique || (n && (!d_grids || !d_out_mapping || !d_out_unique)))
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        TDAG_CHECK(level >= 2 && level <= 4, TDAG_ERR_ARG, "level must be 2..4");
        TDAG_CHECK(n <= kNoAllocMaxItems, TDAG_ERR_ARG, "tdag_find_duplicates_level_noalloc accepts at most 4096 items per call");
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        requireDeviceAccessible(c, d_n_unique, "d_n_unique");
        if (n) {
            requireDeviceAccessible(c, d_grids, "d_grids");
            requireDeviceAccessible(c, d_out_mapping, "d_out_mapping");
            requireDeviceAccessible(c, d_out_unique, "d_out_unique");
        }
        if (n == 0) {
            TDAG_CUDA(cudaMemsetAsync(d_n_unique, 0, 4, c.stream));
            TDAG_CUDA(cudaStreamSynchronize(c.stream));
            return;
        }
        unsigned char* scratch = c.noAllocScratch;
        TDAG_CHECK(scratch != nullptr, TDAG_ERR_NO_DEVICE, "the context has no no-allocation scratch array");
        if (level == 2)
            runMatcherNoAlloc<2>(c, scratch, d_grids, n, *cfg, d_out_mapping, d_out_unique, d_n_unique);
        else if (level == 3)
            runMatcherNoAlloc<3>(c, scratch, d_grids, n, *cfg, d_out_mapping, d_out_unique, d_n_unique);
        else
            runMatcherNoAlloc<4>(c, scratch, d_grids, n, *cfg, d_out_mapping, d_out_unique, d_n_unique);
    });
}
