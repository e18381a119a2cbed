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
//   * the isUnique pass keeps every item that is nobody's child or somebody's parent (:953-961) and
//     numbers the kept items in their original order (:982-997).
// The result is the minimum encoded pointer over all verified candidates, which does not depend on
// thread order, so the GPU output equals the CPU output bit for bit.
#include <algorithm>

#include "common.cuh"
#include "internal.cuh"

namespace tdag {

namespace {

constexpr int kThreads = 256;

// One step of the directional box hash (find_translation.cpp:210-218).
__device__ __forceinline__ uint64_t foldStep(uint64_t acc, uint64_t v)
{
    const bool started = (v | acc) != 0;
    uint64_t c = hashCombine(acc, v);
    c = c < 1 ? 1 : c;
    return started ? c : 0;
}

// ---------------------------------------------------------------------------- popcount order
template <int W>
__global__ void popcountKeyKernel(const uint64_t* __restrict__ grids, uint32_t n, uint32_t maxCount, uint64_t* __restrict__ key, uint32_t* __restrict__ val)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t c = 0;
#pragma unroll 8
    for (int k = 0; k < W; ++k)
        c += __popcll(grids[(size_t)i * W + k]);
    key[i] = maxCount - c; // ascending key == descending popcount; stable sort keeps index order
    val[i] = i;
}

__global__ void invertOrderKernel(const uint32_t* __restrict__ order, uint32_t n, uint32_t* __restrict__ posOf)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n)
        posOf[order[r]] = r;
}

// ---------------------------------------------------------------------------- corner hashes
// Warp per (item, direction). The value at the anchor corner is a nested fold: x-lines, then the
// anchor x-plane along y, then the anchor column along z (computeGridHashInPlace<R, +x, +y, +z>).
template <int R>
__global__ void cornerHashKernel(const uint64_t* __restrict__ grids, uint32_t n, uint64_t* __restrict__ keys, uint32_t* __restrict__ payload)
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
        uint64_t acc = 0;
        for (int k = 0; k < R; ++k) {
            const int x = px ? R - 1 - k : k;
            acc = foldStep(acc, (row >> x) & 1);
        }
        xres[warp][line] = acc;
    }
    __syncwarp();
    uint64_t yv = 0;
    if (lane < R) { // column along y at the anchor x, for z = lane
        uint64_t acc = 0;
        for (int k = 0; k < R; ++k) {
            const int y = py ? R - 1 - k : k;
            acc = foldStep(acc, xres[warp][y + R * lane]);
        }
        yv = acc;
    }
    uint64_t acc = 0;
    for (int k = 0; k < R; ++k) {
        const int z = pz ? R - 1 - k : k;
        const uint64_t v = __shfl_sync(0xffffffffu, yv, z);
        acc = foldStep(acc, v);
    }
    if (lane == 0) {
        keys[gw] = acc;
        payload[gw] = item * 8 + d;
    }
}

// ---------------------------------------------------------------------------- corner-hash table
__device__ __forceinline__ uint64_t slotHash(uint64_t key) { return mix64(key ^ 0x2545F4914F6CDD1Dull); }

__global__ void tableInsertKernel(const uint64_t* __restrict__ ekeys, size_t m, uint64_t* __restrict__ tkeys, uint32_t* __restrict__ tcount,
    uint32_t* __restrict__ slotOfEntry, uint64_t capMask, uint32_t* __restrict__ numDistinct, uint32_t* status)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m)
        return;
    const uint64_t key = ekeys[e];
    if (key == 0) {
        slotOfEntry[e] = 0xFFFFFFFFu;
        return;
    }
    uint64_t slot = slotHash(key) & capMask;
    for (uint64_t probe = 0; probe <= capMask; ++probe) {
        uint64_t cur = tkeys[slot];
        if (cur == 0) {
            cur = atomicCAS((unsigned long long*)&tkeys[slot], 0ull, (unsigned long long)key);
            if (cur == 0) {
                atomicAdd(numDistinct, 1u);
                cur = key;
            }
        }
        if (cur == key) {
            atomicAdd(&tcount[slot], 1u);
            slotOfEntry[e] = (uint32_t)slot;
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

__global__ void tableRangesKernel(const uint64_t* __restrict__ tkeys, const uint32_t* __restrict__ tstart, const uint32_t* __restrict__ tcount, uint64_t cap,
    uint64_t* __restrict__ ranges, uint32_t* __restrict__ filter, uint64_t filterMask)
{
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cap)
        return;
    const uint64_t key = tkeys[s];
    ranges[s] = (uint64_t)tstart[s] | ((uint64_t)tcount[s] << 32);
    if (key != 0) {
        const uint64_t fb = (slotHash(key) >> 20) & filterMask;
        atomicOr(&filter[fb >> 5], 1u << (fb & 31));
    }
}

// ---------------------------------------------------------------------------- search
struct SearchParams {
    const uint64_t* grids; // n x W, original order
    const uint32_t* order; // sorted position -> original position
    uint32_t n;
    const uint64_t* tkeys;
    const uint64_t* tranges;
    uint64_t capMask;
    const uint32_t* entries;
    const uint32_t* filter;
    uint64_t filterMask;
    unsigned long long* parents; // encoded parent per original position
    uint32_t* workCounter;
    unsigned long long* counters; // probes, filterPass, hits, candidates, verifications, verified
    uint32_t allowSym, allowPerm, allowTrans;
};

template <int R>
struct SearchShape {
    static constexpr int TEAM = R * R; // one thread per line
    static constexpr int TEAMS = (kThreads / TEAM) > 0 ? (kThreads / TEAM) : 1;
    static constexpr int W = R * R * R / 64;
    static constexpr int SY = R + 1;
    static constexpr int SZ = (R + 1) * R;
    static constexpr int GRID = (R + 1) * R * R; // padded u64 hash grid
    // per team: G1, G2 (u64), srcW (u64), lines[3][R*R] (u16)
    static constexpr size_t TEAM_BYTES = (size_t)(2 * GRID + W) * 8 + 3 * R * R * 2;
    static constexpr size_t SMEM = TEAM_BYTES * TEAMS + 16;
};

template <int R>
__device__ __forceinline__ int sidx(int x, int y, int z) { return x + SearchShape<R>::SY * y + SearchShape<R>::SZ * z; }

// Exact verification: target == translate(mirror(permute(source, P), S), T) (find_translation.cpp:857-862),
// row by row. lines[a][u_lo + R u_hi] holds the source's voxels along axis a (bit j = coordinate j).
template <int R>
__device__ bool verifyCandidate(const uint64_t* __restrict__ tgrid, const uint16_t* lines, int a0, int a1, int a2, uint32_t S, int T0, int T1, int T2)
{
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    const uint16_t* L = lines + a0 * R * R;
    const int lo = (a0 == 0) ? 1 : 0; // other axes of a0 in increasing order
    const int hi = (a0 == 2) ? 1 : 2;
    for (int w2 = 0; w2 < R; ++w2) {
        for (int w1 = 0; w1 < R; ++w1) {
            const uint32_t bitOff = (uint32_t)(R * (w1 + R * w2));
            const uint32_t trow = (uint32_t)(tgrid[bitOff >> 6] >> (bitOff & 63)) & rowMask;
            int y1 = w1 - T1, y2 = w2 - T2;
            uint32_t zrow = 0;
            if (y1 >= 0 && y1 < R && y2 >= 0 && y2 < R) {
                if (S & 2)
                    y1 = R - 1 - y1;
                if (S & 4)
                    y2 = R - 1 - y2;
                int u[3];
                u[a1] = y1;
                u[a2] = y2;
                uint32_t line = L[u[lo] + R * u[hi]];
                if (S & 1)
                    line = __brev(line) >> (32 - R);
                zrow = (T0 >= 0) ? ((line << T0) & rowMask) : (line >> (-T0));
            }
            if (zrow != trow)
                return false;
        }
    }
    return true;
}

template <int R, int L>
__global__ void __launch_bounds__(kThreads) searchKernel(SearchParams p)
{
    using Sh = SearchShape<R>;
    constexpr int TEAM = Sh::TEAM, TEAMS = Sh::TEAMS, W = Sh::W;
    constexpr uint32_t rowMask = (R == 16) ? 0xFFFFu : ((1u << R) - 1u);
    extern __shared__ __align__(16) uint8_t smem[];
    const int team = threadIdx.x / TEAM;
    const int tl = threadIdx.x % TEAM;
    const bool active = team < TEAMS;
    uint8_t* tb = smem + (size_t)(active ? team : 0) * Sh::TEAM_BYTES;
    uint64_t* G1 = reinterpret_cast<uint64_t*>(tb);
    uint64_t* G2 = G1 + Sh::GRID;
    uint64_t* srcW = G2 + Sh::GRID;
    uint16_t* lines = reinterpret_cast<uint16_t*>(srcW + W);
    uint32_t* shBase = reinterpret_cast<uint32_t*>(smem + Sh::TEAM_BYTES * TEAMS);

    unsigned long long cProbe = 0, cFilter = 0, cHit = 0, cCand = 0, cVer = 0, cOk = 0;

    for (;;) {
        if (threadIdx.x == 0)
            *shBase = atomicAdd(p.workCounter, (uint32_t)TEAMS);
        __syncthreads();
        const uint32_t base = *shBase;
        __syncthreads();
        if (base >= p.n)
            break;
        const uint32_t r = base + team;
        const bool valid = active && r < p.n;
        // ---- load the source grid and its three line orientations
        if (valid) {
            const uint64_t* g = p.grids + (size_t)p.order[r] * W;
            for (int k = tl; k < W; k += TEAM)
                srcW[k] = g[k];
        }
        __syncthreads();
        if (valid) {
            const int c1 = tl % R, c2 = tl / R;
            // x-lines: (y, z) = (c1, c2)
            {
                const uint32_t off = (uint32_t)R * (c1 + R * c2);
                lines[0 * R * R + tl] = (uint16_t)((srcW[off >> 6] >> (off & 63)) & rowMask);
            }
            uint32_t ly = 0, lz = 0;
            for (int j = 0; j < R; ++j) {
                const uint32_t iy = c1 + R * j + R * R * c2; // (x=c1, y=j, z=c2)
                const uint32_t iz = c1 + R * c2 + R * R * j; // (x=c1, y=c2, z=j)
                ly |= (uint32_t)((srcW[iy >> 6] >> (iy & 63)) & 1) << j;
                lz |= (uint32_t)((srcW[iz >> 6] >> (iz & 63)) & 1) << j;
            }
            lines[1 * R * R + tl] = (uint16_t)ly; // index x + R z
            lines[2 * R * R + tl] = (uint16_t)lz; // index x + R y
        }
        __syncthreads();

        const uint64_t srcPos = r;
        for (int a0 = 0; a0 < 3; ++a0) {
            for (int d0 = 1; d0 >= 0; --d0) {
                // ---- pass 1 along a0 from the occupancy bits
                if (valid) {
                    const int b = (a0 == 0) ? 1 : 0, c = (a0 == 2) ? 1 : 2;
                    int u[3];
                    u[b] = tl % R;
                    u[c] = tl / R;
                    uint64_t acc = 0;
                    for (int k = 0; k < R; ++k) {
                        u[a0] = d0 ? R - 1 - k : k;
                        const uint32_t bi = u[0] + R * u[1] + R * R * u[2];
                        acc = foldStep(acc, (srcW[bi >> 6] >> (bi & 63)) & 1);
                        G1[sidx<R>(u[0], u[1], u[2])] = acc;
                    }
                }
                __syncthreads();
                for (int a1i = 0; a1i < 2; ++a1i) {
                    const int a1 = (a0 + 1 + a1i) % 3;
                    const int a2 = 3 - a0 - a1;
                    const uint32_t pid = 2 * a0 + (a2 < a1 ? 1 : 0);
                    for (int d1 = 1; d1 >= 0; --d1) {
                        // ---- pass 2 along a1
                        if (valid) {
                            const int b = (a1 == 0) ? 1 : 0, c = (a1 == 2) ? 1 : 2;
                            int u[3];
                            u[b] = tl % R;
                            u[c] = tl / R;
                            uint64_t acc = 0;
                            for (int k = 0; k < R; ++k) {
                                u[a1] = d1 ? R - 1 - k : k;
                                const int si = sidx<R>(u[0], u[1], u[2]);
                                acc = foldStep(acc, G1[si]);
                                G2[si] = acc;
                            }
                        }
                        __syncthreads();
                        // ---- pass 3 along a2, consumed in place
                        if (valid) {
                            const int b = (a2 == 0) ? 1 : 0, c = (a2 == 2) ? 1 : 2;
                            int u[3];
                            u[b] = tl % R;
                            u[c] = tl / R;
                            for (int d2 = 1; d2 >= 0; --d2) {
                                const uint32_t dir = (uint32_t)d0 | ((uint32_t)d1 << 1) | ((uint32_t)d2 << 2);
                                const int anchor0 = d0 ? 0 : R - 1, anchor1 = d1 ? 0 : R - 1, anchor2 = d2 ? 0 : R - 1;
                                uint64_t acc = 0;
                                for (int k = 0; k < R; ++k) {
                                    u[a2] = d2 ? R - 1 - k : k;
                                    acc = foldStep(acc, G2[sidx<R>(u[0], u[1], u[2])]);
                                    if (acc == 0)
                                        continue;
                                    ++cProbe;
                                    const uint64_t h = slotHash(acc);
                                    const uint64_t fb = (h >> 20) & p.filterMask;
                                    if (!((__ldg(&p.filter[fb >> 5]) >> (fb & 31)) & 1))
                                        continue;
                                    ++cFilter;
                                    uint64_t slot = h & p.capMask;
                                    uint64_t range = 0;
                                    bool hit = false;
                                    for (uint64_t probe = 0; probe <= p.capMask; ++probe) {
                                        const uint64_t tk = __ldg(&p.tkeys[slot]);
                                        if (tk == acc) {
                                            range = __ldg(&p.tranges[slot]);
                                            hit = true;
                                            break;
                                        }
                                        if (tk == 0)
                                            break;
                                        slot = (slot + 1) & p.capMask;
                                    }
                                    if (!hit)
                                        continue;
                                    ++cHit;
                                    // permuted voxel = (u[a0], u[a1], u[a2])
                                    const int v0 = u[a0], v1 = u[a1], v2 = u[a2];
                                    const uint32_t start = (uint32_t)range, cnt = (uint32_t)(range >> 32);
                                    for (uint32_t e = 0; e < cnt; ++e) {
                                        const uint32_t pay = __ldg(&p.entries[start + e]);
                                        const uint32_t tgt = pay >> 3;
                                        const uint32_t S = dir ^ (pay & 7);
                                        ++cCand;
                                        const int T0 = (S & 1) ? v0 - anchor0 : anchor0 - v0;
                                        const int T1 = (S & 2) ? v1 - anchor1 : anchor1 - v1;
                                        const int T2 = (S & 4) ? v2 - anchor2 : anchor2 - v2;
                                        if (!p.allowPerm && pid != 0)
                                            continue;
                                        if (!p.allowSym && S != 0)
                                            continue;
                                        if (!p.allowTrans && (T0 | T1 | T2) != 0)
                                            continue;
                                        const uint64_t key = encodeFixed64(srcPos, pid, S, T0, T1, T2, L);
                                        const unsigned long long cur = *((volatile unsigned long long*)&p.parents[tgt]);
                                        if (key >= cur)
                                            continue;
                                        ++cVer;
                                        if (!verifyCandidate<R>(p.grids + (size_t)tgt * W, lines, a0, a1, a2, S, T0, T1, T2))
                                            continue;
                                        ++cOk;
                                        atomicMin(&p.parents[tgt], (unsigned long long)key);
                                    }
                                }
                            }
                        }
                        __syncthreads();
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
        if ((threadIdx.x & 31) == 0 && v)
            atomicAdd(&p.counters[k], v);
    }
}

// ---------------------------------------------------------------------------- resolve
__global__ void decodeParentsKernel(const unsigned long long* __restrict__ parents, uint32_t n, const uint32_t* __restrict__ order, uint64_t sentinelKey,
    uint32_t level, uint64_t* __restrict__ parentTP, uint32_t* __restrict__ isUnique)
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
        const uint32_t src = order[tpPtr(v)];
        parentTP[i] = tpWithPtr(v, src);
        isUnique[src] = 1;
    }
}

__global__ void finalMappingKernel(const uint64_t* __restrict__ parentTP, const uint32_t* __restrict__ isUnique, const uint32_t* __restrict__ newIdx, uint32_t n,
    uint64_t* __restrict__ mapping)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    if (isUnique[i]) {
        mapping[i] = tpCreate(newIdx[i], 0, 0);
    } else {
        const uint64_t pt = parentTP[i];
        mapping[i] = tpWithPtr(pt, newIdx[tpPtr(pt)]);
    }
}

uint64_t pow2AtLeast(uint64_t v)
{
    uint64_t p = 1;
    while (p < v)
        p <<= 1;
    return p;
}

template <int L>
MatchOutput runMatcherL(Context& ctx, const uint64_t* grids, uint32_t n, const tdag_config& cfg, tdag_level_stats* stats)
{
    constexpr int R = 1 << L;
    constexpr int W = R * R * R / 64;
    cudaStream_t s = ctx.stream;
    MatchOutput out;
    if (n == 0)
        return out;
    TDAG_CHECK(n < (1u << 29), TDAG_ERR_ARG, "too many items for one matcher level");

    // popcount order
    DevBuf<uint32_t> order(n, s), posOf(n, s);
    {
        DevBuf<uint64_t> key(n, s);
        popcountKeyKernel<W><<<gridFor(n, 256), 256, 0, s>>>(grids, n, R * R * R, key.get(), order.get());
        TDAG_LAUNCHED();
        radixSortPairs(key.get(), order.get(), n, 0, 16, s);
        invertOrderKernel<<<gridFor(n, 256), 256, 0, s>>>(order.get(), n, posOf.get());
        TDAG_LAUNCHED();
    }

    // corner hashes + table
    const size_t m = (size_t)n * 8;
    DevBuf<uint64_t> ekeys(m, s);
    DevBuf<uint32_t> epay(m, s);
    cornerHashKernel<R><<<gridFor(m * 32, kThreads), kThreads, 0, s>>>(grids, n, ekeys.get(), epay.get());
    TDAG_LAUNCHED();
    const uint32_t loadPct = ctx.tuning.table_load_percent ? std::min(85u, std::max(25u, ctx.tuning.table_load_percent)) : 50u;
    const uint64_t cap = pow2AtLeast(m * 100 / loadPct + 16);
    DevBuf<uint64_t> tkeys(cap, s), tranges(cap, s);
    DevBuf<uint32_t> tcount(cap, s), tstart(cap, s), slotOfEntry(m, s), numDistinct(1, s);
    TDAG_CUDA(cudaMemsetAsync(tkeys.get(), 0, cap * 8, s));
    TDAG_CUDA(cudaMemsetAsync(tcount.get(), 0, cap * 4, s));
    TDAG_CUDA(cudaMemsetAsync(numDistinct.get(), 0, 4, s));
    tableInsertKernel<<<gridFor(m, 256), 256, 0, s>>>(ekeys.get(), m, tkeys.get(), tcount.get(), slotOfEntry.get(), cap - 1, numDistinct.get(), ctx.status);
    TDAG_LAUNCHED();
    const uint64_t numEntries = exclusiveScanU32Total(tcount.get(), tstart.get(), cap, s);
    uint32_t distinct = 0;
    TDAG_CUDA(cudaMemcpyAsync(&distinct, numDistinct.get(), 4, cudaMemcpyDeviceToHost, s));
    ctx.checkStatus("corner-hash table");
    DevBuf<uint32_t> entries(numEntries ? numEntries : 1, s);
    {
        DevBuf<uint32_t> tfill(cap, s);
        TDAG_CUDA(cudaMemsetAsync(tfill.get(), 0, cap * 4, s));
        tableScatterKernel<<<gridFor(m, 256), 256, 0, s>>>(epay.get(), slotOfEntry.get(), m, tstart.get(), tfill.get(), entries.get());
        TDAG_LAUNCHED();
    }
    const uint32_t bitsPerKey = ctx.tuning.filter_bits_per_key ? ctx.tuning.filter_bits_per_key : 32u;
    const uint64_t filterBits = pow2AtLeast(std::max<uint64_t>(1024, (uint64_t)distinct * bitsPerKey));
    DevBuf<uint32_t> filter(filterBits / 32, s);
    TDAG_CUDA(cudaMemsetAsync(filter.get(), 0, filterBits / 8, s));
    tableRangesKernel<<<gridFor(cap, 256), 256, 0, s>>>(tkeys.get(), tstart.get(), tcount.get(), cap, tranges.get(), filter.get(), filterBits - 1);
    TDAG_LAUNCHED();
    ekeys.release();
    epay.release();
    slotOfEntry.release();
    tcount.release();
    tstart.release();

    // search
    const uint64_t sentinelKey = encodeFixed64(0xFFFFFFFFull, 0, 0, 0, 0, 0, L);
    DevBuf<unsigned long long> parents(n, s);
    fillU64(reinterpret_cast<uint64_t*>(parents.get()), sentinelKey, n, s);
    DevBuf<uint32_t> work(1, s);
    DevBuf<unsigned long long> counters(8, s);
    TDAG_CUDA(cudaMemsetAsync(work.get(), 0, 4, s));
    TDAG_CUDA(cudaMemsetAsync(counters.get(), 0, 64, s));
    SearchParams sp;
    sp.grids = grids;
    sp.order = order.get();
    sp.n = n;
    sp.tkeys = tkeys.get();
    sp.tranges = tranges.get();
    sp.capMask = cap - 1;
    sp.entries = entries.get();
    sp.filter = filter.get();
    sp.filterMask = filterBits - 1;
    sp.parents = parents.get();
    sp.workCounter = work.get();
    sp.counters = counters.get();
    sp.allowSym = cfg.symmetry ? 1 : 0;
    sp.allowPerm = cfg.axis_permutation ? 1 : 0;
    sp.allowTrans = cfg.translation ? 1 : 0;
    const size_t smem = SearchShape<R>::SMEM;
    TDAG_CUDA(cudaFuncSetAttribute(searchKernel<R, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int perSM = 0;
    TDAG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, searchKernel<R, L>, kThreads, smem));
    if (ctx.tuning.search_ctas_per_sm)
        perSM = std::min<int>(perSM, (int)ctx.tuning.search_ctas_per_sm);
    perSM = std::max(perSM, 1);
    const uint64_t groups = (n + SearchShape<R>::TEAMS - 1) / SearchShape<R>::TEAMS;
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)ctx.numSMs * perSM, groups));
    TDAG_CUDA(cudaEventRecord(ctx.ev[0], s));
    searchKernel<R, L><<<blocks, kThreads, smem, s>>>(sp);
    TDAG_LAUNCHED();
    TDAG_CUDA(cudaEventRecord(ctx.ev[1], s));

    // resolve
    DevBuf<uint64_t> parentTP(n, s);
    DevBuf<uint32_t> isUnique(n, s), newIdx(n, s);
    TDAG_CUDA(cudaMemsetAsync(isUnique.get(), 0, (size_t)n * 4, s));
    decodeParentsKernel<<<gridFor(n, 256), 256, 0, s>>>(parents.get(), n, order.get(), sentinelKey, L, parentTP.get(), isUnique.get());
    TDAG_LAUNCHED();
    out.uniques = DevBuf<uint32_t>(n, s);
    out.numUnique = compactFlags(isUnique.get(), out.uniques.get(), n, s);
    exclusiveScanU32(isUnique.get(), newIdx.get(), n, s);
    out.mapping = DevBuf<uint64_t>(n, s);
    finalMappingKernel<<<gridFor(n, 256), 256, 0, s>>>(parentTP.get(), isUnique.get(), newIdx.get(), n, out.mapping.get());
    TDAG_LAUNCHED();

    if (stats) {
        unsigned long long c[8];
        TDAG_CUDA(cudaMemcpyAsync(c, counters.get(), 64, cudaMemcpyDeviceToHost, s));
        TDAG_CUDA(cudaStreamSynchronize(s));
        float ms = 0;
        TDAG_CUDA(cudaEventElapsedTime(&ms, ctx.ev[0], ctx.ev[1]));
        stats->items = n;
        stats->unique = out.numUnique;
        stats->probes = c[0];
        stats->filter_pass = c[1];
        stats->hits = c[2];
        stats->candidates = c[3];
        stats->verifications = c[4];
        stats->verified = c[5];
        stats->table_entries = numEntries;
        stats->search_ms = ms;
    }
    ctx.checkStatus("matcher level " + std::to_string(L));
    return out;
}

} // namespace

MatchOutput runMatcher(Context& ctx, uint32_t level, const uint64_t* grids, uint32_t n, const tdag_config& cfg, tdag_level_stats* stats)
{
    switch (level) {
    case 2:
        return runMatcherL<2>(ctx, grids, n, cfg, stats);
    case 3:
        return runMatcherL<3>(ctx, grids, n, cfg, stats);
    case 4:
        return runMatcherL<4>(ctx, grids, n, cfg, stats);
    default:
        throw Error(TDAG_ERR_ARG, "translation matching supports levels 2..4");
    }
}

} // namespace tdag
