// query16.cu — queries on an encoded .tdag16 in device memory: voxel lookups (TransformDAG16::get,
// tools/svdag_encoding/src/transform_dag_encoding.cpp:699-745, with getChildPointer :519-562 and the
// pointer decoders :142-224) and a lossless check of a .tdag16 against the SVDAG it was built from
// (the role of verifyComplexTransformDAG, transform_dag_encoding.h:81-117).
//
// Child pointer semantics: the content of a child = translate(mirror(permute(C, P), S), T), so a
// lookup maps coordinates into each child's canonical frame: subtract T, mirror the flagged axes,
// then u[P[k]] = w[k]. Every index read from the file is bounds-checked; a bad one sets
// TDAG_ERR_CORRUPT in the context's status word and the lookup answers "empty".
//
// The check walks the source SVDAG and the .tdag16 together, level by level from the root:
//   * above the boundary level B (the highest level whose incoming pointers may carry a
//     translation, or the leaf level without translation) octants align, so each (source node,
//     .tdag16 node, accumulated mirror/permutation) pair compares which of its 8 children exist and
//     queues the pairs of existing children (the pointer's mirror/permutation composed into the map);
//   * at level B every voxel of each pair's 2^B box is compared, the .tdag16 side through the
//     pair's pending pointer (with its translation) and the same lookup as the point queries.
// Empty regions are checked too: a child that exists on one side only is a mismatch.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "common.cuh"
#include "internal.cuh"
#include "tdag16.h"

namespace tdag {
namespace {

constexpr int kLevels = 24; // root levels up to 23 (resolution 2^23)

struct D16 {
    uint32_t root, resolution;
    uint32_t sym, perm, trans, maxTL, pointerTables, huffman;
    const uint16_t* nodes[kLevels];
    uint64_t nodeLen[kLevels];
    const uint64_t* tables[kLevels];
    uint64_t tableLen[kLevels];
    const uint2* lut[kLevels]; // Huffman decode table: (symbol, code length)
    uint32_t lutMask[kLevels];
    const uint64_t* leaves;
    uint64_t leafCount;
};

struct Ptr16 {
    uint64_t index;
    uint32_t sym, perm; // mirror bits, permutation id (0..5, order 012 021 102 120 201 210)
    int t[3];
};

__device__ __forceinline__ uint32_t permAxis(uint32_t perm, int k) { return (permBitsOf(perm) >> (2 * k)) & 3; }

// Child pointer `ci` of the node at u16 offset `at` of `level` (getChildPointer + decoders).
__device__ bool decodeChild(const D16& d, uint32_t level, uint64_t at, uint32_t ci, Ptr16& out, uint32_t* status)
{
    if (at >= d.nodeLen[level]) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 40);
        return false;
    }
    const uint16_t* s = d.nodes[level];
    const uint32_t mask = s[at];
    const uint32_t bits = (mask >> (2 * ci)) & 3;
    if (!bits)
        return false;
    uint64_t p = at + 1;
    for (uint32_t i = 0; i < ci; ++i)
        p += (mask >> (2 * i)) & 3;
    if (p + bits > d.nodeLen[level]) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 41);
        return false;
    }
    uint64_t e = 0;
    for (uint32_t w = 0; w < bits; ++w)
        e |= (uint64_t)s[p + w] << (16 * w);
    const uint32_t cl = level - 1;
    if (d.pointerTables) {
        if (bits == 1 || (e & 1)) {
            const uint64_t idx = bits == 1 ? e : e >> 1;
            if (idx >= d.tableLen[cl]) {
                setDeviceError(status, TDAG_ERR_CORRUPT, 42);
                return false;
            }
            e = d.tables[cl][idx];
        } else {
            e >>= 1;
        }
    }
    const uint32_t tb = cl + 1;
    const uint64_t tm = (1ull << tb) - 1;
    const int bias = 1 << cl;
    out.sym = 0;
    out.perm = 0;
    out.t[0] = out.t[1] = out.t[2] = 0;
    const bool transHere = d.trans && cl <= d.maxTL;
    if (d.huffman) {
        if (!d.lut[cl]) {
            setDeviceError(status, TDAG_ERR_CORRUPT, 43);
            return false;
        }
        const uint2 sl = d.lut[cl][(uint32_t)e & d.lutMask[cl]];
        uint32_t type = sl.x;
        e >>= sl.y;
        uint32_t axes = 0;
        if (transHere) {
            axes = type & 7;
            type >>= 3;
        }
        for (int k = 2; k >= 0; --k)
            if (axes & (1u << k)) {
                out.t[k] = (int)(e & tm) - bias;
                e >>= tb;
            }
        if (d.sym) {
            out.sym = type & 7;
            type >>= 3;
        }
        if (d.perm)
            out.perm = type & 7;
    } else {
        bool has = false;
        if (d.perm || d.sym || d.trans) {
            has = e & 1;
            e >>= 1;
        }
        if (has) {
            if (transHere)
                for (int k = 0; k < 3; ++k) {
                    out.t[k] = (int)(e & tm) - bias;
                    e >>= tb;
                }
            if (d.sym) {
                out.sym = e & 7;
                e >>= 3;
            }
            if (d.perm) {
                out.perm = e & 7;
                e >>= 3;
            }
        }
    }
    if (out.perm >= 6) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 44);
        return false;
    }
    out.index = e;
    return true;
}

// Into the pointer's canonical frame at scale `size`: w = v - T (outside the box: empty), mirror,
// u[P[k]] = w[k]. Returns false for coordinates that fall outside.
__device__ __forceinline__ bool applyPointer(const Ptr16& p, int size, int v[3])
{
    int w[3];
    for (int k = 0; k < 3; ++k) {
        w[k] = v[k] - p.t[k];
        if (w[k] < 0 || w[k] >= size)
            return false;
        if ((p.sym >> k) & 1)
            w[k] = size - 1 - w[k];
    }
    for (int k = 0; k < 3; ++k)
        v[permAxis(p.perm, k)] = w[k];
    return true;
}

// Lookup from node `at` of `level` with coordinates v in that node's canonical frame.
__device__ bool lookupFrom(const D16& d, uint32_t level, uint64_t at, int v[3], uint32_t* status)
{
    for (; level > 2; --level) {
        const int half = 1 << (level - 1);
        const uint32_t ci = (v[0] >= half ? 1u : 0u) | (v[1] >= half ? 2u : 0u) | (v[2] >= half ? 4u : 0u);
        Ptr16 p;
        if (!decodeChild(d, level, at, ci, p, status))
            return false;
        for (int k = 0; k < 3; ++k)
            v[k] &= half - 1;
        if (!applyPointer(p, half, v))
            return false;
        at = p.index;
    }
    if (at >= d.leafCount) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 45);
        return false;
    }
    return (d.leaves[at] >> morton3((uint32_t)v[0], (uint32_t)v[1], (uint32_t)v[2])) & 1;
}

__global__ void getKernel(D16 d, const uint32_t* __restrict__ xyz, uint64_t n, uint8_t* __restrict__ out, uint32_t* status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    uint8_t r = 0;
    if (x < d.resolution && y < d.resolution && z < d.resolution && d.nodeLen[d.root] > 0) {
        int v[3] = { (int)x, (int)y, (int)z };
        r = lookupFrom(d, d.root, 0, v, status) ? 1 : 0;
    }
    out[i] = r;
}

// ---- ray queries ------------------------------------------------------------------------------
// Voxel probe for the traversal: solid, or an empty world-aligned box containing the voxel. Above the
// translation levels pointers only mirror and permute, which keeps child boxes aligned, so a missing
// child is an empty aligned box of the child's size. Once a translated pointer has been followed (a
// box of 2^maxTranslationLevel voxels or less) the empty box is the voxel itself.
__device__ bool probeVoxel(const D16& d, const int w[3], int emptyLo[3], int& emptySize, uint32_t* status)
{
    int v[3] = { w[0], w[1], w[2] };
    uint64_t at = 0;
    bool aligned = true;
    for (uint32_t level = d.root; level > 2; --level) {
        const int half = 1 << (level - 1);
        const uint32_t ci = (v[0] >= half ? 1u : 0u) | (v[1] >= half ? 2u : 0u) | (v[2] >= half ? 4u : 0u);
        Ptr16 p;
        const bool has = decodeChild(d, level, at, ci, p, status);
        bool inside = has;
        if (has) {
            for (int k = 0; k < 3; ++k)
                v[k] &= half - 1;
            if (p.t[0] | p.t[1] | p.t[2])
                aligned = false;
            inside = applyPointer(p, half, v);
        }
        if (!inside) {
            emptySize = aligned ? half : 1;
            for (int k = 0; k < 3; ++k)
                emptyLo[k] = w[k] & ~(emptySize - 1);
            return false;
        }
        at = p.index;
    }
    if (at >= d.leafCount) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 45);
        emptySize = 1;
        for (int k = 0; k < 3; ++k)
            emptyLo[k] = w[k];
        return false;
    }
    if ((d.leaves[at] >> morton3((uint32_t)v[0], (uint32_t)v[1], (uint32_t)v[2])) & 1)
        return true;
    emptySize = 1;
    for (int k = 0; k < 3; ++k)
        emptyLo[k] = w[k];
    return false;
}

// First solid voxel along each ray (restart traversal, double precision). The ray enters the grid
// box [0, res)^3, and from each empty box it moves to the neighbouring cell across the face it
// leaves through (ties: the lowest axis); t is the entry parameter of the hit voxel.
__global__ void raycastKernel(D16 d, const tdag16_ray* __restrict__ rays, uint64_t n, tdag16_hit* __restrict__ hits, uint32_t maxSteps, uint32_t* status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const tdag16_ray r = rays[i];
    tdag16_hit h {};
    h.t = r.tmax;
    const double R = (double)d.resolution;
    double o[3], dir[3], inv[3];
    for (int k = 0; k < 3; ++k) {
        o[k] = r.origin[k];
        dir[k] = r.direction[k];
        inv[k] = dir[k] != 0.0 ? 1.0 / dir[k] : 0.0;
    }
    // entry into the grid box
    double t0 = r.tmin, t1 = r.tmax;
    int entryAxis = -1;
    for (int k = 0; k < 3; ++k) {
        if (dir[k] == 0.0) {
            if (o[k] < 0.0 || o[k] >= R)
                t0 = t1 + 1.0;
            continue;
        }
        double a = (0.0 - o[k]) * inv[k], b = (R - o[k]) * inv[k];
        if (a > b) {
            const double tmp = a;
            a = b;
            b = tmp;
        }
        if (a > t0) {
            t0 = a;
            entryAxis = k;
        }
        if (b < t1)
            t1 = b;
    }
    if (d.nodeLen[d.root] == 0 || !(t0 < t1)) {
        hits[i] = h;
        return;
    }
    int c[3];
    for (int k = 0; k < 3; ++k) {
        double x = o[k] + t0 * dir[k];
        int ck = (int)floor(x);
        if (k == entryAxis)
            ck = dir[k] > 0 ? 0 : (int)d.resolution - 1;
        c[k] = min(max(ck, 0), (int)d.resolution - 1);
    }
    double t = t0;
    uint32_t steps = 0;
    for (; steps < maxSteps; ++steps) {
        int lo[3], size;
        if (probeVoxel(d, c, lo, size, status)) {
            h.hit = 1;
            h.t = (float)t;
            h.voxel[0] = (uint32_t)c[0];
            h.voxel[1] = (uint32_t)c[1];
            h.voxel[2] = (uint32_t)c[2];
            break;
        }
        // leave the empty box
        double tk[3];
        for (int k = 0; k < 3; ++k)
            tk[k] = dir[k] > 0.0 ? ((double)(lo[k] + size) - o[k]) * inv[k] : dir[k] < 0.0 ? ((double)lo[k] - o[k]) * inv[k] : 1e300;
        int ax = 0;
        if (tk[1] < tk[ax])
            ax = 1;
        if (tk[2] < tk[ax])
            ax = 2;
        const double tn = tk[ax] > t ? tk[ax] : t;
        if (tn >= t1)
            break;
        for (int k = 0; k < 3; ++k) {
            if (k == ax) {
                c[k] = dir[k] > 0.0 ? lo[k] + size : lo[k] - 1;
            } else {
                const int ck = (int)floor(o[k] + tn * dir[k]);
                c[k] = min(max(ck, lo[k]), lo[k] + size - 1);
            }
        }
        if (c[ax] < 0 || c[ax] >= (int)d.resolution)
            break;
        t = tn;
    }
    h.steps = steps;
    hits[i] = h;
}

// ---- lossless check ---------------------------------------------------------------------------
// A pair: a source node and the .tdag16 state covering the same box. map = (mirror | perm << 3)
// maps box-local world coordinates w into the frame the pending pointer applies to:
// v[P[k]] = S_k ? size-1-w[k] : w[k]. Above level B the pointer is folded into the map (it has no
// translation there), so `ptr` only carries the node index; at level B it keeps its transform.
struct Pair {
    uint32_t src;
    uint32_t map;
    uint64_t index;
    uint32_t psym, pperm;
    int pt[3];
};

struct SourceView {
    const uint32_t* nodes[kLevels];
    uint64_t counts[kLevels];
    const uint64_t* leaves;
    uint64_t leafCount;
};

struct VerifyCounters {
    unsigned long long existence; // children present on one side only
    unsigned long long voxels; // voxels that differ inside compared boxes
    unsigned long long boxes; // boxes compared voxel by voxel
    unsigned long long pairs; // pairs walked above the boundary level
};

__device__ __forceinline__ void mapApply(uint32_t map, int size, const int w[3], int v[3])
{
    for (int k = 0; k < 3; ++k) {
        const int x = ((map >> k) & 1) ? size - 1 - w[k] : w[k];
        v[permAxis(map >> 3, k)] = x;
    }
}
// map followed by a translation-free pointer (mirror psym, permutation pperm):
// P'[k] = Pp[P[k]], S'_k = S_k ^ Sp[P[k]].
__device__ __forceinline__ uint32_t mapCompose(uint32_t map, uint32_t psym, uint32_t pperm)
{
    uint32_t s = 0, pb = 0;
    for (int k = 0; k < 3; ++k) {
        const uint32_t pk = permAxis(map >> 3, k);
        s |= (((map >> k) & 1) ^ ((psym >> pk) & 1)) << k;
        pb |= permAxis(pperm, (int)pk) << (2 * k);
    }
    return s | (permIdOfBits(pb) << 3);
}

// One thread per (pair, world octant) above level B.
__global__ void expandKernel(D16 d, SourceView src, uint32_t level, const Pair* __restrict__ in, uint32_t n, Pair* __restrict__ out,
    uint32_t* __restrict__ outCount, uint32_t capacity, uint32_t boundary, VerifyCounters* counters, uint32_t* status)
{
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)n * 8)
        return;
    const Pair p = in[t >> 3];
    const uint32_t o = (uint32_t)(t & 7);
    if (p.src >= src.counts[level]) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 46);
        return;
    }
    const uint32_t sc = src.nodes[level][(uint64_t)p.src * 8 + o];
    // the .tdag16 child covering world octant o: its octant in the node's canonical frame
    uint32_t c = 0;
    for (int k = 0; k < 3; ++k)
        c |= (((o >> k) & 1) ^ ((p.map >> k) & 1)) << permAxis(p.map >> 3, k);
    Ptr16 q;
    const bool has16 = decodeChild(d, level, p.index, c, q, status);
    const bool hasSrc = sc != kEmpty32;
    if (has16 != hasSrc) {
        atomicAdd(&counters->existence, 1ull);
        return;
    }
    if (!hasSrc)
        return;
    const uint32_t slot = atomicAdd(outCount, 1u);
    if (slot >= capacity) {
        setDeviceError(status, TDAG_ERR_ALLOC, 47);
        return;
    }
    Pair r;
    r.src = sc;
    if (level - 1 > boundary) {
        if (q.t[0] | q.t[1] | q.t[2]) {
            setDeviceError(status, TDAG_ERR_CORRUPT, 48); // translations only up to the boundary level
            return;
        }
        r.map = mapCompose(p.map, q.sym, q.perm);
        r.psym = 0;
        r.pperm = 0;
        r.pt[0] = r.pt[1] = r.pt[2] = 0;
    } else {
        r.map = p.map;
        r.psym = q.sym;
        r.pperm = q.perm;
        r.pt[0] = q.t[0];
        r.pt[1] = q.t[1];
        r.pt[2] = q.t[2];
    }
    r.index = q.index;
    out[slot] = r;
}

__device__ bool sourceVoxel(const SourceView& s, uint32_t level, uint32_t node, uint32_t x, uint32_t y, uint32_t z, uint32_t* status)
{
    for (; level > 2; --level) {
        const uint32_t cl = level - 1;
        const uint32_t c = ((x >> cl) & 1) | (((y >> cl) & 1) << 1) | (((z >> cl) & 1) << 2);
        if (node >= s.counts[level]) {
            setDeviceError(status, TDAG_ERR_CORRUPT, 49);
            return false;
        }
        node = s.nodes[level][(uint64_t)node * 8 + c];
        if (node == kEmpty32)
            return false;
    }
    if (node >= s.leafCount) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 50);
        return false;
    }
    return (s.leaves[node] >> morton3(x & 3, y & 3, z & 3)) & 1;
}

// One block per pair at the boundary level: every voxel of the 2^B box.
constexpr int kBoxThreads = 128;
__global__ void __launch_bounds__(kBoxThreads) compareBoxKernel(D16 d, SourceView src, uint32_t level, const Pair* __restrict__ pairs, uint32_t n,
    VerifyCounters* counters, uint32_t* status)
{
    __shared__ unsigned long long bad;
    const int size = 1 << level;
    const uint32_t voxels = (uint32_t)size * size * size;
    for (uint32_t b = blockIdx.x; b < n; b += gridDim.x) {
        if (threadIdx.x == 0)
            bad = 0;
        __syncthreads();
        const Pair p = pairs[b];
        Ptr16 q;
        q.index = p.index;
        q.sym = p.psym;
        q.perm = p.pperm;
        q.t[0] = p.pt[0];
        q.t[1] = p.pt[1];
        q.t[2] = p.pt[2];
        uint32_t local = 0;
        for (uint32_t i = threadIdx.x; i < voxels; i += kBoxThreads) {
            const int w[3] = { (int)(i & (size - 1)), (int)((i >> level) & (size - 1)), (int)(i >> (2 * level)) };
            const bool a = sourceVoxel(src, level, p.src, (uint32_t)w[0], (uint32_t)w[1], (uint32_t)w[2], status);
            int v[3];
            mapApply(p.map, size, w, v);
            bool e = false;
            if (applyPointer(q, size, v))
                e = lookupFrom(d, level, p.index, v, status);
            local += a != e;
        }
        if (local)
            atomicAdd(&bad, (unsigned long long)local);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (bad)
                atomicAdd(&counters->voxels, bad);
            atomicAdd(&counters->boxes, 1ull);
        }
        __syncthreads();
    }
}

} // namespace

// Device copy of a .tdag16 file (aligned arrays), built from its bytes.
struct Tdag16Device {
    cudaStream_t stream = nullptr;
    D16 d {};
    std::vector<DevBuf<uint16_t>> nodes;
    std::vector<DevBuf<uint64_t>> tables;
    std::vector<DevBuf<uint2>> luts;
    DevBuf<uint64_t> leaves;
};

namespace {
struct ByteReader {
    const uint8_t* p;
    uint64_t n, off = 0;
    template <typename T>
    T pod()
    {
        TDAG_CHECK(off + sizeof(T) <= n, TDAG_ERR_CORRUPT, ".tdag16: truncated");
        T v;
        std::memcpy(&v, p + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
    const uint8_t* span(uint64_t bytes)
    {
        TDAG_CHECK(bytes <= n - off, TDAG_ERR_CORRUPT, ".tdag16: truncated array");
        const uint8_t* r = p + off;
        off += bytes;
        return r;
    }
};
} // namespace

// Parses TransformDAG16::writeTo bytes (transform_dag_encoding.cpp:1023-1030) into device arrays.
std::unique_ptr<Tdag16Device> uploadTdag16(Context& c, const uint8_t* bytes, uint64_t size)
{
    cudaStream_t s = c.stream;
    auto h = std::make_unique<Tdag16Device>();
    h->stream = s;
    D16& d = h->d;
    ByteReader r { bytes, size };
    const uint8_t* cfg = r.span(8);
    d.sym = cfg[0] != 0;
    d.perm = cfg[1] != 0;
    d.trans = cfg[2] != 0;
    std::memcpy(&d.maxTL, cfg + 4, 4);
    d.pointerTables = r.pod<uint8_t>() != 0;
    d.huffman = r.pod<uint8_t>() != 0;
    const uint64_t nl = r.pod<uint64_t>();
    TDAG_CHECK(nl >= 4 && nl <= (uint64_t)kLevels, TDAG_ERR_CORRUPT, ".tdag16: level count outside 4..24");
    h->nodes.resize(nl);
    for (uint64_t l = 0; l < nl; ++l) {
        const uint64_t len = r.pod<uint64_t>();
        const uint8_t* src = r.span(len * 2);
        TDAG_CHECK(len < (1ull << 40), TDAG_ERR_CORRUPT, ".tdag16: level too large");
        h->nodes[l] = DevBuf<uint16_t>(std::max<uint64_t>(len, 1), s);
        if (len)
            TDAG_CUDA(cudaMemcpyAsync(h->nodes[l].get(), src, len * 2, cudaMemcpyHostToDevice, s));
        d.nodes[l] = h->nodes[l].get();
        d.nodeLen[l] = len;
    }
    const uint64_t nLeaves = r.pod<uint64_t>();
    TDAG_CHECK(nLeaves < (1ull << 40), TDAG_ERR_CORRUPT, ".tdag16: leaf count too large");
    const uint8_t* leafSrc = r.span(nLeaves * 8);
    h->leaves = DevBuf<uint64_t>(std::max<uint64_t>(nLeaves, 1), s);
    if (nLeaves)
        TDAG_CUDA(cudaMemcpyAsync(h->leaves.get(), leafSrc, nLeaves * 8, cudaMemcpyHostToDevice, s));
    d.leaves = h->leaves.get();
    d.leafCount = nLeaves;
    d.resolution = r.pod<uint32_t>();
    d.root = r.pod<uint32_t>();
    TDAG_CHECK(d.root + 1 == nl && d.root >= 3, TDAG_ERR_CORRUPT, ".tdag16: root level does not match the level count");
    TDAG_CHECK(d.resolution == (1u << d.root), TDAG_ERR_CORRUPT, ".tdag16: resolution is not 2^rootLevel");
    const uint64_t nt = r.pod<uint64_t>();
    TDAG_CHECK(nt <= (uint64_t)kLevels, TDAG_ERR_CORRUPT, ".tdag16: pointer table count");
    h->tables.resize(nt);
    for (uint64_t l = 0; l < nt; ++l) {
        const uint64_t len = r.pod<uint64_t>();
        TDAG_CHECK(len < (1ull << 40), TDAG_ERR_CORRUPT, ".tdag16: pointer table too large");
        const uint8_t* src = r.span(len * 8);
        h->tables[l] = DevBuf<uint64_t>(std::max<uint64_t>(len, 1), s);
        if (len)
            TDAG_CUDA(cudaMemcpyAsync(h->tables[l].get(), src, len * 8, cudaMemcpyHostToDevice, s));
        d.tables[l] = h->tables[l].get();
        d.tableLen[l] = len;
    }
    const uint64_t nh = r.pod<uint64_t>();
    TDAG_CHECK(nh <= (uint64_t)kLevels, TDAG_ERR_CORRUPT, ".tdag16: Huffman table count");
    TDAG_CHECK(!d.huffman || nh == nl, TDAG_ERR_CORRUPT, ".tdag16: Huffman tables missing");
    h->luts.resize(nh);
    // HuffmanDecodeLUT::initFromInputCodes (huffman.cpp:184-201): every key whose low bits equal a
    // code maps to (symbol, code length).
    std::vector<std::vector<uint2>> hostLuts(nh);
    for (uint64_t l = 0; l < nh; ++l) {
        const uint64_t cnt = r.pod<uint64_t>();
        TDAG_CHECK(cnt <= 4096, TDAG_ERR_CORRUPT, ".tdag16: Huffman table too large");
        std::vector<std::pair<uint64_t, uint32_t>> codes(cnt);
        uint32_t maxLen = 0;
        for (auto& cd : codes) {
            cd.first = r.pod<uint64_t>();
            cd.second = r.pod<uint32_t>();
            (void)r.pod<uint32_t>();
            TDAG_CHECK(cd.second <= 16, TDAG_ERR_CORRUPT, ".tdag16: Huffman code longer than 16 bits");
            maxLen = std::max(maxLen, cd.second);
        }
        if (!cnt)
            continue;
        auto& lut = hostLuts[l];
        lut.assign(1ull << maxLen, make_uint2(0, 0));
        for (uint32_t k = 0; k < cnt; ++k) {
            const uint32_t b = codes[k].second;
            TDAG_CHECK(codes[k].first < (1ull << b) || b == 0, TDAG_ERR_CORRUPT, ".tdag16: Huffman code wider than its length");
            for (uint64_t suffix = 0; suffix < (1ull << (maxLen - b)); ++suffix)
                lut[(suffix << b) | codes[k].first] = make_uint2(k, b);
        }
        h->luts[l] = DevBuf<uint2>(lut.size(), s);
        TDAG_CUDA(cudaMemcpyAsync(h->luts[l].get(), lut.data(), lut.size() * sizeof(uint2), cudaMemcpyHostToDevice, s));
        d.lut[l] = h->luts[l].get();
        d.lutMask[l] = (uint32_t)(lut.size() - 1);
    }
    TDAG_CHECK(r.off == size, TDAG_ERR_CORRUPT, ".tdag16: trailing bytes");
    TDAG_CUDA(cudaStreamSynchronize(s)); // the host LUTs and the caller's bytes may go now
    return h;
}

void tdag16Get(Context& c, const Tdag16Device& h, const uint32_t* dXyz, uint64_t n, uint8_t* dOut)
{
    if (n) {
        getKernel<<<gridFor(n, 256), 256, 0, c.stream>>>(h.d, dXyz, n, dOut, c.status);
        TDAG_LAUNCHED();
    }
    c.checkStatus("tdag16_get");
}

void tdag16Raycast(Context& c, const Tdag16Device& h, const tdag16_ray* dRays, uint64_t n, tdag16_hit* dHits)
{
    if (n) {
        const uint32_t maxSteps = 8u * h.d.resolution + 64u; // each step leaves a box; a ray crosses at most 3 * res voxels
        raycastKernel<<<gridFor(n, 128), 128, 0, c.stream>>>(h.d, dRays, n, dHits, maxSteps, c.status);
        TDAG_LAUNCHED();
    }
    c.checkStatus("tdag16_raycast");
}

void tdag16Verify(Context& c, const Tdag16Device& h, const tdag_svdag_view& in, tdag16_verify_stats& out)
{
    cudaStream_t s = c.stream;
    const D16& d = h.d;
    TDAG_CHECK(in.root_level == d.root && in.resolution == d.resolution, TDAG_ERR_ARG, "source and .tdag16 differ in size");
    SourceView sv {};
    for (uint32_t l = 3; l <= in.root_level; ++l) {
        sv.nodes[l] = in.nodes[l];
        sv.counts[l] = in.node_counts[l];
    }
    sv.leaves = in.leaves;
    sv.leafCount = in.leaf_count;
    const uint32_t boundary = std::min(d.root, d.trans ? std::max<uint32_t>(d.maxTL, 2) : 2u);
    TDAG_CHECK(boundary <= 6, TDAG_ERR_ARG, "translation levels above 6 are not supported by the check");
    DevBuf<VerifyCounters> counters(1, s);
    TDAG_CUDA(cudaMemsetAsync(counters.get(), 0, sizeof(VerifyCounters), s));
    DevBuf<uint32_t> count(1, s);
    // root pair: identity map, pending identity pointer to node 0
    Pair root {};
    std::vector<Pair> hostRoot(1, root);
    DevBuf<Pair> cur(1, s);
    TDAG_CUDA(cudaMemcpyAsync(cur.get(), hostRoot.data(), sizeof(Pair), cudaMemcpyHostToDevice, s));
    uint32_t n = (in.node_counts[in.root_level] > 0 && d.nodeLen[d.root] > 0) ? 1 : 0;
    const bool emptySrc = in.node_counts[in.root_level] == 0, empty16 = d.nodeLen[d.root] == 0;
    uint64_t pairsWalked = 0;
    for (uint32_t level = d.root; level > boundary && n; --level) {
        const uint64_t cap = (uint64_t)n * 8;
        TDAG_CHECK(cap < 0xFFFFFFFFull, TDAG_ERR_ARG, "verification frontier too large");
        DevBuf<Pair> next(cap, s);
        TDAG_CUDA(cudaMemsetAsync(count.get(), 0, 4, s));
        expandKernel<<<gridFor(cap, 256), 256, 0, s>>>(d, sv, level, cur.get(), n, next.get(), count.get(), (uint32_t)cap, boundary, counters.get(),
            c.status);
        TDAG_LAUNCHED();
        pairsWalked += n;
        TDAG_CUDA(cudaMemcpyAsync(&n, count.get(), 4, cudaMemcpyDeviceToHost, s));
        c.checkStatus("tdag16_verify: walk");
        cur = std::move(next);
    }
    if (n) {
        const unsigned blocks = (unsigned)std::min<uint64_t>(n, (uint64_t)c.numSMs * 16);
        compareBoxKernel<<<blocks, kBoxThreads, 0, s>>>(d, sv, boundary, cur.get(), n, counters.get(), c.status);
        TDAG_LAUNCHED();
    }
    VerifyCounters vc {};
    TDAG_CUDA(cudaMemcpyAsync(&vc, counters.get(), sizeof(vc), cudaMemcpyDeviceToHost, s));
    c.checkStatus("tdag16_verify: compare");
    out.existence_mismatches = vc.existence + (emptySrc != empty16 ? 1 : 0);
    out.voxel_mismatches = vc.voxels;
    out.boxes_compared = vc.boxes;
    out.box_level = boundary;
    out.pairs_walked = pairsWalked;
}

} // namespace tdag

struct tdag16_device {
    std::unique_ptr<tdag::Tdag16Device> h;
};

struct tdag_ctx;
tdag::Context& ctxOf(tdag_ctx* c); // build.cu
int guardedCall(const std::function<void()>& f); // build.cu
int failWith(int code, const char* msg); // build.cu

extern "C" int tdag16_upload(tdag_ctx* ctx, const uint8_t* bytes, uint64_t size, tdag16_device** out)
{
    using namespace tdag;
    if (!ctx || !bytes || !out)
        return failWith(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        auto r = std::make_unique<tdag16_device>();
        r->h = uploadTdag16(c, bytes, size);
        *out = r.release();
    });
}

extern "C" int tdag16_device_free(tdag16_device* dev)
{
    delete dev;
    return TDAG_OK;
}

extern "C" int tdag16_get(tdag_ctx* ctx, const tdag16_device* dev, const uint32_t* d_xyz, uint64_t n, uint8_t* d_out)
{
    using namespace tdag;
    if (!ctx || !dev || (n && (!d_xyz || !d_out)))
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        if (n) {
            requireDeviceAccessible(c, d_xyz, "d_xyz");
            requireDeviceAccessible(c, d_out, "d_out");
        }
        tdag16Get(c, *dev->h, d_xyz, n, d_out);
    });
}

extern "C" int tdag16_raycast(tdag_ctx* ctx, const tdag16_device* dev, const tdag16_ray* d_rays, uint64_t n, tdag16_hit* d_hits)
{
    using namespace tdag;
    if (!ctx || !dev || (n && (!d_rays || !d_hits)))
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        if (n) {
            requireDeviceAccessible(c, d_rays, "d_rays");
            requireDeviceAccessible(c, d_hits, "d_hits");
        }
        tdag16Raycast(c, *dev->h, d_rays, n, d_hits);
    });
}

extern "C" int tdag16_verify(tdag_ctx* ctx, const tdag16_device* dev, const tdag_svdag_view* source_device, tdag16_verify_stats* out)
{
    using namespace tdag;
    if (!ctx || !dev || !source_device || !out)
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        requireDeviceView(c, *source_device);
        *out = tdag16_verify_stats {};
        tdag16Verify(c, *dev->h, *source_device, *out);
    });
}
