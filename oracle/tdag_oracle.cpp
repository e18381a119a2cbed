// tdag_oracle.cpp — CPU ORACLE (test infrastructure only).
//
// This file is the checker for the GB300 Transform-DAG construction library. It is a from-scratch
// CPU restatement of the reference algorithm (mathijs727/i3d2025-voxel-transform-dag, default CPU
// path, USE_GPU = 0). It is NOT part of the product: only tests/, __graft_entry__.smoke() and
// bench.py's cpu_baseline leg / reference arm may load it. Every function cites the reference
// file:line whose behaviour it restates. The reference itself cannot be compiled here (glm,
// libmorton, robin_hood, TBB, spdlog ... are absent), so parity of the translation/hierarchical
// stages rests on this restatement plus the reference's own structure/round-trip test cases.
//
// Interface: bytes in / bytes out in the reference's own on-disk formats (.svo, .tdag), plus the
// inner per-level seam (findDuplicatesAmongFlattenedItems_cpp2) on dense grids.
//
// Parallelism: OpenMP only where the reference uses std::execution::par* on order-independent
// loops (hash-key computation, per-range search, the translation search over source items).

#include <algorithm>
#include <array>
#include <atomic>
#include <bit>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <optional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>
#include <omp.h>

namespace orc {

// ------------------------------------------------------------------------------------------------
// Errors: the reference uses assert_always (throws std::runtime_error on the host,
// tools/lib/include/voxcom/utility/error_handling.h:34-44). The C API turns throws into status codes.
// ------------------------------------------------------------------------------------------------
static void check(bool ok, const char* what)
{
    if (!ok)
        throw std::runtime_error(what);
}

// ------------------------------------------------------------------------------------------------
// Morton (libmorton morton3D_32 semantics: x in bit 0), used via tools/lib/include/voxcom/voxel/morton.h:12-13,26
// ------------------------------------------------------------------------------------------------
static inline uint32_t part1by2(uint32_t v)
{
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}
static inline uint32_t compact1by2(uint32_t v)
{
    v &= 0x09249249;
    v = (v ^ (v >> 2)) & 0x030C30C3;
    v = (v ^ (v >> 4)) & 0x0300F00F;
    v = (v ^ (v >> 8)) & 0x030000FF;
    v = (v ^ (v >> 16)) & 0x000003FF;
    return v;
}
static inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) { return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2); }
static inline void demorton3(uint32_t m, uint32_t& x, uint32_t& y, uint32_t& z)
{
    x = compact1by2(m);
    y = compact1by2(m >> 1);
    z = compact1by2(m >> 2);
}

// ------------------------------------------------------------------------------------------------
// hash_combine (tools/lib/include/voxcom/utility/hash.h:10-20). std::hash on integers is the
// identity in libstdc++; 0x9e3779b9 is an unsigned int promoted to 64 bit; size_t arithmetic wraps.
// ------------------------------------------------------------------------------------------------
static inline void hash_combine(uint64_t& seed, uint64_t key)
{
    seed ^= key + 0x9e3779b9ull + (seed << 6) + (seed >> 2);
}

// ------------------------------------------------------------------------------------------------
// Transforms: 48 = 8 mirror (symmetry) × 6 axis permutations.
// Transform ID = symmetryID | permutationID << 3 (transform_dag_hierarchical.cpp:23-46); the
// symmetry ID is the Morton code of (sx, sy, sz) = sx | sy<<1 | sz<<2; permutation IDs follow
// TransformPointer::decodeAxisPermutation (transform_dag.h:136-147). A transform maps a position v to
// P(v) ^ S where P(v) = (v[p0], v[p1], v[p2]) (applyAxisPermutation, transform_dag.h:181-189).
// ------------------------------------------------------------------------------------------------
static const uint8_t kPerm[6][3] = { { 0, 1, 2 }, { 0, 2, 1 }, { 1, 0, 2 }, { 1, 2, 0 }, { 2, 0, 1 }, { 2, 1, 0 } };

static inline uint32_t permCode(const uint8_t p[3]) { return 2u * p[0] + (p[2] < p[1] ? 1u : 0u); } // transform_dag.h:326-331
static inline uint32_t applyPermBits(uint32_t bits3, const uint8_t p[3])
{
    return ((bits3 >> p[0]) & 1u) | (((bits3 >> p[1]) & 1u) << 1) | (((bits3 >> p[2]) & 1u) << 2);
}
struct TransformTables {
    uint8_t compose[48][48]; // compose[a][b] = a ∘ b
    uint8_t inverse[48];
    uint8_t pos[48][8]; // image of 2x2x2 child index
    TransformTables()
    {
        for (uint32_t a = 0; a < 48; ++a) {
            const uint32_t sa = a & 7;
            const uint8_t* pa = kPerm[a >> 3];
            for (uint32_t i = 0; i < 8; ++i)
                pos[a][i] = (uint8_t)(applyPermBits(i, pa) ^ sa);
            for (uint32_t b = 0; b < 48; ++b) {
                const uint32_t sb = b & 7;
                const uint8_t* pb = kPerm[b >> 3];
                // (a∘b)(v) = Pa(Pb(v) ^ Sb) ^ Sa = (Pa∘Pb)(v) ^ (Pa(Sb) ^ Sa); (Pa∘Pb)[i] = pb[pa[i]]
                uint8_t pc[3] = { pb[pa[0]], pb[pa[1]], pb[pa[2]] };
                const uint32_t sc = applyPermBits(sb, pa) ^ sa;
                compose[a][b] = (uint8_t)(sc | (permCode(pc) << 3));
            }
        }
        for (uint32_t a = 0; a < 48; ++a)
            for (uint32_t b = 0; b < 48; ++b)
                if (compose[a][b] == 0)
                    inverse[a] = (uint8_t)b;
    }
};
static const TransformTables& tt()
{
    static const TransformTables t;
    return t;
}

struct Config {
    bool symmetry = true, axisPermutation = true, translation = true;
    uint32_t maxTranslationLevel = 4;
};
static inline bool allowedTransform(uint32_t t, const Config& c)
{
    if (!c.axisPermutation && (t >> 3) != 0)
        return false;
    if (!c.symmetry && (t & 7) != 0)
        return false;
    return true;
}

// ------------------------------------------------------------------------------------------------
// TransformPointer, COMPACT layout (transform_dag.h:19-33): ptr:37 | sx sy sz | p0:2 p1:2 p2:2 |
// tx:6 ty:6 tz:6 (biased by +32). GCC allocates bit-fields from the least significant bit.
// ------------------------------------------------------------------------------------------------
namespace tp {
    static constexpr uint64_t kPtrMask = (1ull << 37) - 1;
    static inline uint64_t create(uint64_t ptr, uint32_t sym = 0, uint32_t permId = 0, int tx = 0, int ty = 0, int tz = 0)
    {
        const uint8_t* p = kPerm[permId];
        uint64_t v = ptr & kPtrMask;
        v |= (uint64_t)(sym & 7) << 37;
        v |= (uint64_t)p[0] << 40 | (uint64_t)p[1] << 42 | (uint64_t)p[2] << 44;
        v |= (uint64_t)((unsigned)(tx + 32) & 63) << 46;
        v |= (uint64_t)((unsigned)(ty + 32) & 63) << 52;
        v |= (uint64_t)((unsigned)(tz + 32) & 63) << 58;
        return v;
    }
    static inline uint64_t createT(uint64_t ptr, uint32_t transformId) { return create(ptr, transformId & 7, transformId >> 3); }
    static inline uint64_t ptr(uint64_t v) { return v & kPtrMask; }
    static inline uint32_t sym(uint64_t v) { return (uint32_t)(v >> 37) & 7; }
    static inline void perm(uint64_t v, uint8_t p[3])
    {
        p[0] = (v >> 40) & 3;
        p[1] = (v >> 42) & 3;
        p[2] = (v >> 44) & 3;
    }
    static inline int tx(uint64_t v) { return (int)((v >> 46) & 63) - 32; }
    static inline int ty(uint64_t v) { return (int)((v >> 52) & 63) - 32; }
    static inline int tz(uint64_t v) { return (int)((v >> 58) & 63) - 32; }
    static inline uint64_t sentinel() { return create(0xFFFFFFFFull); } // transform_dag.h:344-347
    static inline bool hasTransform(uint64_t v) // transform_dag.h:115-130
    {
        uint8_t p[3];
        perm(v, p);
        return sym(v) != 0 || !(p[0] == 0 && p[1] == 1 && p[2] == 2) || tx(v) != 0 || ty(v) != 0 || tz(v) != 0;
    }
    // encodeFixed64 (transform_dag.h:375-397)
    static inline uint64_t encodeFixed64(uint64_t v, uint32_t level)
    {
        uint8_t p[3];
        perm(v, p);
        uint64_t out = ptr(v);
        out <<= 3;
        out |= permCode(p);
        out <<= 3;
        out |= sym(v);
        if (level != 0) {
            const uint32_t sb = level + 1;
            const int bias = 1 << level;
            out <<= sb;
            out |= (uint64_t)(unsigned)(tz(v) + bias);
            out <<= sb;
            out |= (uint64_t)(unsigned)(ty(v) + bias);
            out <<= sb;
            out |= (uint64_t)(unsigned)(tx(v) + bias);
        }
        return out;
    }
    // decodeFixed64 (transform_dag.h:349-373)
    static inline uint64_t decodeFixed64(uint64_t e, uint32_t level)
    {
        int t[3] = { 0, 0, 0 };
        if (level != 0) {
            const uint32_t sb = level + 1;
            const uint64_t m = (1ull << sb) - 1;
            for (int a = 0; a < 3; ++a) {
                t[a] = (int)(e & m) - (1 << level);
                e >>= sb;
            }
        }
        const uint32_t s = (uint32_t)(e & 7);
        e >>= 3;
        const uint32_t pc = (uint32_t)(e & 7);
        e >>= 3;
        return create(e, s, pc, t[0], t[1], t[2]);
    }
}

// ------------------------------------------------------------------------------------------------
// Structures (structure.h:44-211) and their binary format (binary_writer.h:48-78; structure.h:493-501;
// export_import_structure.cpp:12-24).
// ------------------------------------------------------------------------------------------------
static constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;
template <typename C>
struct Structure {
    std::vector<std::vector<std::array<C, 8>>> nodes; // per level, size rootLevel+1
    std::vector<uint64_t> leaves; // EditSubGrid<void>::bitmask, Morton bit order
    uint32_t resolution = 0, rootLevel = 0, structureType = 0; // 0 = Tree, 1 = DAG
};
using Structure32 = Structure<uint32_t>;
using StructureTP = Structure<uint64_t>;

struct Writer {
    std::vector<uint8_t> buf;
    template <typename T>
    void pod(const T& v)
    {
        const auto* p = reinterpret_cast<const uint8_t*>(&v);
        buf.insert(buf.end(), p, p + sizeof(T));
    }
    template <typename T>
    void vec(const std::vector<T>& v)
    {
        pod<uint64_t>(v.size());
        const auto* p = reinterpret_cast<const uint8_t*>(v.data());
        buf.insert(buf.end(), p, p + v.size() * sizeof(T));
    }
};
struct Reader {
    const uint8_t* p;
    size_t n, off = 0;
    template <typename T>
    T pod()
    {
        check(off + sizeof(T) <= n, "truncated input");
        T v;
        std::memcpy(&v, p + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
    template <typename T>
    std::vector<T> vec()
    {
        const uint64_t cnt = pod<uint64_t>();
        check(cnt <= (n - off) / sizeof(T), "truncated vector");
        std::vector<T> v(cnt);
        std::memcpy(v.data(), p + off, cnt * sizeof(T));
        off += cnt * sizeof(T);
        return v;
    }
};
template <typename C>
static void writeStructure(Writer& w, const Structure<C>& s)
{
    w.pod<uint64_t>(s.nodes.size());
    for (const auto& lvl : s.nodes)
        w.vec(lvl);
    w.vec(s.leaves);
    w.pod(s.resolution);
    w.pod(s.rootLevel);
    w.pod(s.structureType);
}
template <typename C>
static Structure<C> readStructure(Reader& r)
{
    Structure<C> s;
    const uint64_t nl = r.pod<uint64_t>();
    check(nl <= 64, "corrupt level count");
    s.nodes.resize(nl);
    for (auto& lvl : s.nodes)
        lvl = r.vec<std::array<C, 8>>();
    s.leaves = r.vec<uint64_t>();
    s.resolution = r.pod<uint32_t>();
    s.rootLevel = r.pod<uint32_t>();
    s.structureType = r.pod<uint32_t>();
    check(s.rootLevel + 1 == nl, "rootLevel does not match level count");
    return s;
}
static constexpr uint32_t kSvoMagic = 72198382, kSvoVersion = 2; // export_import_structure.cpp:12-13

// ------------------------------------------------------------------------------------------------
// A1: EditStructure(VoxelGrid) (structure.h:407-429, 658-701). Dense input: uint8 per voxel,
// index x + res*y + res*res*z.
// ------------------------------------------------------------------------------------------------
static uint32_t buildRec(Structure32& s, const uint8_t* dense, uint32_t res, int level, uint32_t x, uint32_t y, uint32_t z)
{
    if (level == 2) {
        uint64_t mask = 0;
        for (uint32_t i = 0; i < 64; ++i) {
            uint32_t ox, oy, oz;
            demorton3(i, ox, oy, oz);
            if (dense[(size_t)(x + ox) + (size_t)res * (y + oy) + (size_t)res * res * (z + oz)])
                mask |= 1ull << i;
        }
        if (!mask)
            return kEmpty32;
        s.leaves.push_back(mask);
        return (uint32_t)s.leaves.size() - 1;
    }
    const uint32_t half = 1u << (level - 1);
    std::array<uint32_t, 8> node;
    bool allEmpty = true;
    for (uint32_t i = 0; i < 8; ++i) {
        uint32_t ox, oy, oz;
        demorton3(i, ox, oy, oz);
        node[i] = buildRec(s, dense, res, level - 1, x + ox * half, y + oy * half, z + oz * half);
        allEmpty &= (node[i] == kEmpty32);
    }
    if (allEmpty)
        return kEmpty32;
    s.nodes[level].push_back(node);
    return (uint32_t)s.nodes[level].size() - 1;
}
static Structure32 svoFromDense(const uint8_t* dense, uint32_t res)
{
    check(res >= 4 && std::popcount(res) == 1, "resolution must be a power of two >= 4");
    Structure32 s;
    s.resolution = res;
    const uint32_t numLevels = (uint32_t)std::bit_width(res - 1) + 1;
    s.nodes.resize(numLevels);
    s.rootLevel = numLevels - 1;
    buildRec(s, dense, res, (int)s.rootLevel, 0, 0, 0);
    s.structureType = 0;
    return s;
}

// ------------------------------------------------------------------------------------------------
// A2: toDAG, first-occurrence dedup per level, bottom-up (structure.h:703-763).
// ------------------------------------------------------------------------------------------------
struct ArrHash {
    size_t operator()(const std::array<uint32_t, 8>& a) const
    {
        uint64_t h = 0;
        for (uint32_t v : a)
            hash_combine(h, v);
        return (size_t)h;
    }
};
static void toDAG(Structure32& s)
{
    std::vector<uint32_t> mapping;
    {
        std::unordered_map<uint64_t, uint32_t> lut;
        lut.reserve(s.leaves.size());
        std::vector<uint64_t> out;
        for (uint64_t m : s.leaves) {
            auto it = lut.find(m);
            if (it != lut.end()) {
                mapping.push_back(it->second);
            } else {
                const uint32_t h = (uint32_t)out.size();
                out.push_back(m);
                lut.emplace(m, h);
                mapping.push_back(h);
            }
        }
        s.leaves = std::move(out);
    }
    for (uint32_t level = 3; level <= s.rootLevel; ++level) {
        auto& in = s.nodes[level];
        for (auto& node : in)
            for (auto& c : node)
                if (c != kEmpty32)
                    c = mapping[c];
        mapping.clear();
        std::unordered_map<std::array<uint32_t, 8>, uint32_t, ArrHash> lut;
        lut.reserve(in.size());
        std::vector<std::array<uint32_t, 8>> out;
        for (const auto& node : in) {
            auto it = lut.find(node);
            if (it != lut.end()) {
                mapping.push_back(it->second);
            } else {
                const uint32_t h = (uint32_t)out.size();
                out.push_back(node);
                lut.emplace(node, h);
                mapping.push_back(h);
            }
        }
        in = std::move(out);
    }
    s.structureType = 1;
}

// ------------------------------------------------------------------------------------------------
// A3-A5: hierarchical symmetry + axis-permutation canonicalisation
// (transform_dag_hierarchical.cpp:48-123, 158-262, 293-523).
// ------------------------------------------------------------------------------------------------
struct Tagged {
    uint64_t ptr; // TransformPointer::ptr
    uint32_t t; // transform ID of the pointer (symmetry | perm << 3); translation is always 0 here
    uint64_t inv; // invariance bit mask of the canonical item `ptr`
};
static inline bool taggedEq(const Tagged& a, const Tagged& b) // TaggedPointer::operator== (:79-122)
{
    if (a.ptr != b.ptr)
        return false;
    // Equal pointers carry the same canonical's invariance mask (asserted at :84 in the reference).
    const uint32_t req = tt().compose[tt().inverse[a.t]][b.t];
    return (a.inv >> req) & 1;
}
static inline Tagged taggedSentinel() { return Tagged { 0xFFFFFFFFull, 0, ~0ull }; }
static inline bool isTaggedSentinel(const Tagged& a) { return a.ptr == 0xFFFFFFFFull && a.t == 0 && a.inv == ~0ull; }

struct TNode {
    std::array<Tagged, 8> c;
    TNode transform(uint32_t t) const // TransformNode::transform (:233-259)
    {
        TNode out;
        for (uint32_t i = 0; i < 8; ++i) {
            const Tagged& in = c[i];
            out.c[tt().pos[t][i]] = Tagged { in.ptr, tt().compose[t][in.t], in.inv };
        }
        return out;
    }
    bool operator==(const TNode& o) const
    {
        for (uint32_t i = 0; i < 8; ++i)
            if (!taggedEq(c[i], o.c[i]))
                return false;
        return true;
    }
};
struct TNodeHash { // TransformNodeHash (:293-302)
    size_t operator()(const TNode& n) const
    {
        uint64_t h = 0;
        for (const auto& x : n.c)
            hash_combine(h, x.ptr);
        return (size_t)h;
    }
};

static inline uint32_t transformByte(uint32_t b, uint32_t t) // applyTransformToBitMask2x2x2 (:48-60)
{
    uint32_t out = 0;
    for (uint32_t i = 0; i < 8; ++i)
        if ((b >> i) & 1)
            out |= 1u << tt().pos[t][i];
    return out;
}
static std::array<Tagged, 256> canonicalLeafTable(const Config& cfg) // (:158-203)
{
    std::array<uint64_t, 256> invMasks {};
    std::array<Tagged, 256> out;
    for (auto& o : out)
        o = Tagged { 0xFFFF, 0, 0 };
    for (uint32_t c = 0; c < 256; ++c) {
        for (uint32_t t = 0; t < 48; ++t) {
            const uint32_t b = transformByte(c, t);
            if (!allowedTransform(t, cfg))
                continue;
            if (c < out[b].ptr)
                out[b] = Tagged { c, t, 0 };
            if (b == c)
                invMasks[c] |= 1ull << t;
        }
    }
    for (auto& o : out)
        o.inv = invMasks[o.ptr];
    return out;
}

struct HierResult {
    StructureTP out;
    std::vector<uint32_t> midInvMapping;
};

// processLevel (:359-448): group by hash of sorted child ptrs, canonical search in (hash, index) order.
// outHandles receives, for each emitted (canonical) node, its input index in emission order.
// ptrValue (optional): the value hashed for a child pointer ptr, ptrValue[ptr] (the static variant
// hashes the child's word offset in its packed level, transform_dag_hierarchical.cpp:597-606, 696-703).
static void processLevel(const std::vector<TNode>& nodes, std::vector<Tagged>& mapping, std::vector<uint32_t>& emitted, const Config& cfg,
    const std::vector<uint64_t>* ptrValue = nullptr)
{
    const size_t n = nodes.size();
    mapping.assign(n, Tagged {});
    emitted.clear();
    if (n == 0)
        return;
    std::vector<std::pair<uint64_t, uint32_t>> keys(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        std::array<uint64_t, 8> p;
        for (int k = 0; k < 8; ++k) {
            const uint64_t c = nodes[i].c[k].ptr;
            p[k] = (ptrValue && c != 0xFFFFFFFFull) ? (*ptrValue)[c] : c;
        }
        std::sort(p.begin(), p.end());
        uint64_t seed = 0;
        for (uint64_t v : p)
            hash_combine(seed, v);
        keys[i] = { seed, (uint32_t)i };
    }
    std::sort(keys.begin(), keys.end());
    std::vector<std::pair<uint32_t, uint32_t>> ranges;
    {
        uint64_t prev = keys[0].first;
        uint32_t start = 0;
        for (uint32_t i = 0; i < n; ++i) {
            if (keys[i].first != prev) {
                ranges.push_back({ start, i });
                start = i;
                prev = keys[i].first;
            }
        }
        ranges.push_back({ start, (uint32_t)n });
    }
    std::vector<Tagged> found(n);
    std::vector<uint64_t> invMasks(n);
    std::vector<uint8_t> isNew(n, 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t r = 0; r < (int64_t)ranges.size(); ++r) {
        std::unordered_map<TNode, std::pair<uint32_t, uint64_t>, TNodeHash> lut;
        const auto [b, e] = ranges[r];
        lut.reserve(e - b);
        for (uint32_t j = b; j < e; ++j) {
            const uint32_t index = keys[j].second;
            const TNode& node = nodes[index];
            // findTransformNode (:326-357)
            uint64_t invMask = 0;
            bool hit = false;
            for (uint32_t t = 0; t < 48; ++t) {
                if (!allowedTransform(t, cfg))
                    continue;
                const TNode tn = node.transform(t);
                auto it = lut.find(tn);
                if (it != lut.end()) {
                    // store canonical -> node: inverse of t (:343-344)
                    found[index] = Tagged { it->second.first, tt().inverse[t], it->second.second };
                    invMask = it->second.second;
                    hit = true;
                    break;
                }
                if (tn == node)
                    invMask |= 1ull << t;
            }
            if (!hit) {
                lut.emplace(node, std::pair<uint32_t, uint64_t> { index, invMask });
                isNew[index] = 1;
            }
            invMasks[index] = invMask;
        }
    }
    for (const auto& kv : keys) {
        const uint32_t index = kv.second;
        if (!isNew[index]) {
            Tagged tg = found[index];
            tg.ptr = mapping[tg.ptr].ptr; // canonical already emitted earlier in this order
            mapping[index] = tg;
        } else {
            const uint32_t handle = (uint32_t)emitted.size();
            emitted.push_back(index);
            mapping[index] = Tagged { handle, 0, invMasks[index] };
        }
    }
}

// staticOffsets: the StaticStructure variant (constructStaticTransformDAGHierarchical,
// transform_dag_hierarchical.cpp:531-743). It makes the same decisions, but a child pointer's value is
// the word offset of the child in its packed level (header + one word per child), so the grouping hash,
// and with it the emission order, differs from levels 4 up.
static HierResult constructHierarchical(const Structure32& in, uint32_t midLevel, const Config& cfg, bool staticOffsets = false)
{
    HierResult res;
    StructureTP& out = res.out;
    out.resolution = in.resolution;
    out.rootLevel = in.rootLevel;
    out.structureType = 0; // default-constructed EditStructure (:307-309)
    const auto storeMid = [&](size_t numOut, const std::vector<Tagged>& mapping) { // (:312-320)
        res.midInvMapping.assign(numOut, 0);
        for (uint32_t old = 0; old < mapping.size(); ++old) {
            if (mapping[old].t != 0)
                continue;
            res.midInvMapping[mapping[old].ptr] = old;
        }
    };
    std::vector<Tagged> mapping;
    {
        const auto canon = canonicalLeafTable(cfg);
        for (uint32_t b = 0; b < 256; ++b) // reconstruction assert (:216-217)
            check(transformByte((uint32_t)canon[b].ptr, canon[b].t) == b, "leaf canonical reconstruction");
        std::vector<TNode> nodes(in.leaves.size());
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)in.leaves.size(); ++i) {
            for (uint32_t k = 0; k < 8; ++k) {
                const uint32_t b = (uint32_t)(in.leaves[i] >> (8 * k)) & 0xFF;
                nodes[i].c[k] = canon[b];
            }
        }
        std::vector<uint32_t> emitted;
        processLevel(nodes, mapping, emitted, cfg);
        out.leaves.resize(emitted.size());
        for (size_t i = 0; i < emitted.size(); ++i)
            out.leaves[i] = in.leaves[emitted[i]];
        if (midLevel == 2)
            storeMid(out.leaves.size(), mapping);
    }
    out.nodes.resize(in.nodes.size());
    std::vector<uint64_t> prevOffsets; // word offsets of the previous level's emitted nodes (static variant)
    for (uint32_t level = 3; level <= in.rootLevel; ++level) {
        const auto& inNodes = in.nodes[level];
        std::vector<TNode> nodes(inNodes.size());
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)inNodes.size(); ++i)
            for (uint32_t k = 0; k < 8; ++k)
                nodes[i].c[k] = (inNodes[i][k] == kEmpty32) ? taggedSentinel() : mapping[inNodes[i][k]];
        std::vector<uint32_t> emitted;
        std::vector<Tagged> newMapping;
        processLevel(nodes, newMapping, emitted, cfg, (staticOffsets && level >= 4) ? &prevOffsets : nullptr);
        auto& outNodes = out.nodes[level];
        outNodes.resize(emitted.size());
        for (size_t i = 0; i < emitted.size(); ++i)
            for (uint32_t k = 0; k < 8; ++k) {
                const Tagged& c = nodes[emitted[i]].c[k];
                outNodes[i][k] = tp::createT(c.ptr, c.t);
            }
        if (staticOffsets) {
            prevOffsets.assign(outNodes.size(), 0);
            uint64_t off = 0;
            for (size_t i = 0; i < outNodes.size(); ++i) {
                prevOffsets[i] = off;
                off += 1;
                for (uint64_t c : outNodes[i])
                    off += c != tp::sentinel() ? 1 : 0;
            }
        }
        mapping = std::move(newMapping);
        if (level == midLevel)
            storeMid(outNodes.size(), mapping);
    }
    return res;
}

// ------------------------------------------------------------------------------------------------
// A7: dense flattening of a level-L treelet (transform_dag.cpp:44-116); LargeSubGrid bit order
// x + R*y + R*R*z (large_sub_grid.h:80-97).
// ------------------------------------------------------------------------------------------------
template <typename C>
static void flattenRec(const Structure<C>& s, uint32_t level, uint32_t idx, uint32_t R, uint32_t bx, uint32_t by, uint32_t bz, uint64_t* out)
{
    if (level == 2) {
        const uint64_t m = s.leaves[idx];
        for (uint32_t i = 0; i < 64; ++i) {
            if (!((m >> i) & 1))
                continue;
            uint32_t x, y, z;
            demorton3(i, x, y, z);
            const uint32_t li = (bx + x) + R * (by + y) + R * R * (bz + z);
            out[li >> 6] |= 1ull << (li & 63);
        }
        return;
    }
    const uint32_t half = 1u << (level - 1);
    for (uint32_t c = 0; c < 8; ++c) {
        const uint64_t child = (uint64_t)s.nodes[level][idx][c];
        if ((uint32_t)child == kEmpty32)
            continue;
        uint32_t x, y, z;
        demorton3(c, x, y, z);
        flattenRec(s, level - 1, (uint32_t)child, R, bx + x * half, by + y * half, bz + z * half, out);
    }
}

// ------------------------------------------------------------------------------------------------
// A8-A12: translation + symmetry + permutation matching (find_translation.cpp:66-125, 202-264,
// 466-495, 616-1000).
// ------------------------------------------------------------------------------------------------
struct MatchStats {
    uint64_t items = 0, probes = 0, hits = 0, candidates = 0, verifications = 0, verified = 0, tableEntries = 0, unique = 0;
};

template <uint32_t R>
struct Grid {
    static constexpr uint32_t N = R * R * R;
    static constexpr uint32_t W = (N + 63) / 64;
    std::array<uint64_t, W> w {};
    bool get(uint32_t x, uint32_t y, uint32_t z) const
    {
        const uint32_t i = x + R * y + R * R * z;
        return (w[i >> 6] >> (i & 63)) & 1;
    }
    void set(uint32_t x, uint32_t y, uint32_t z)
    {
        const uint32_t i = x + R * y + R * R * z;
        w[i >> 6] |= 1ull << (i & 63);
    }
    bool operator==(const Grid& o) const { return w == o.w; }
};

// computeGridHashInPlace{X,Y,Z} (:202-264): one pass along `axis`, from the far end towards the anchor.
template <uint32_t R>
static void hashPass(std::vector<uint64_t>& h, uint32_t axis, bool positive)
{
    const uint32_t stride[3] = { 1, R, R * R };
    const uint32_t sa = stride[axis], s1 = stride[(axis + 1) % 3], s2 = stride[(axis + 2) % 3];
    for (uint32_t a = 0; a < R; ++a)
        for (uint32_t b = 0; b < R; ++b) {
            uint64_t combined = 0;
            for (uint32_t k = 0; k < R; ++k) {
                const uint32_t c = positive ? (R - 1 - k) : k;
                uint64_t& cell = h[c * sa + a * s1 + b * s2];
                const uint64_t v = cell;
                const uint64_t started = ((v | combined) == 0) ? 0 : ~0ull;
                hash_combine(combined, v);
                combined = std::max<uint64_t>(combined, 1);
                combined &= started;
                cell = combined;
            }
        }
}

template <uint32_t R>
static Grid<R> permuteGrid(const Grid<R>& g, const uint8_t p[3]) // (:109-125)
{
    Grid<R> out;
    for (uint32_t z = 0; z < R; ++z)
        for (uint32_t y = 0; y < R; ++y)
            for (uint32_t x = 0; x < R; ++x)
                if (g.get(x, y, z)) {
                    const uint32_t v[3] = { x, y, z };
                    out.set(v[p[0]], v[p[1]], v[p[2]]);
                }
    return out;
}
template <uint32_t R>
static Grid<R> mirrorGrid(const Grid<R>& g, uint32_t s) // (:85-107)
{
    Grid<R> out;
    for (uint32_t z = 0; z < R; ++z)
        for (uint32_t y = 0; y < R; ++y)
            for (uint32_t x = 0; x < R; ++x)
                if (g.get(x, y, z))
                    out.set((s & 1) ? R - 1 - x : x, (s & 2) ? R - 1 - y : y, (s & 4) ? R - 1 - z : z);
    return out;
}
template <uint32_t R>
static Grid<R> translateGrid(const Grid<R>& g, int tx, int ty, int tz) // (:66-84)
{
    Grid<R> out;
    for (int z = 0; z < (int)R; ++z)
        for (int y = 0; y < (int)R; ++y)
            for (int x = 0; x < (int)R; ++x) {
                const int ix = x - tx, iy = y - ty, iz = z - tz;
                if (ix < 0 || iy < 0 || iz < 0 || ix >= (int)R || iy >= (int)R || iz >= (int)R)
                    continue;
                if (g.get(ix, iy, iz))
                    out.set(x, y, z);
            }
    return out;
}

static inline void atomicMin64(std::atomic<uint64_t>& a, uint64_t v) // (:543-548)
{
    uint64_t e = a.load(std::memory_order_relaxed);
    while (v < e && !a.compare_exchange_weak(e, v, std::memory_order_relaxed, std::memory_order_relaxed))
        ;
}

// findDuplicatesAmongFlattenedItems_cpp2<Level> (:616-1000). grids: n items × W words (original order).
// Returns the list of unique item positions (in original order); outMapping[i] = TransformPointer.
template <uint32_t L>
static std::vector<uint32_t> findDuplicates(const std::vector<Grid<1u << L>>& grids, std::vector<uint64_t>& outMapping, const Config& cfg, MatchStats& st)
{
    constexpr uint32_t R = 1u << L;
    constexpr uint32_t N = R * R * R;
    const size_t n = grids.size();
    st.items += n;
    outMapping.assign(n, tp::sentinel());
    if (n == 0)
        return {};

    // Popcount order, stable, descending (:631-643).
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    {
        std::vector<uint16_t> counts(n);
        for (size_t i = 0; i < n; ++i) {
            uint32_t c = 0;
            for (uint64_t w : grids[i].w)
                c += (uint32_t)std::popcount(w);
            counts[i] = (uint16_t)c;
        }
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return counts[a] > counts[b]; });
    }

    const uint64_t encodedSentinel = tp::encodeFixed64(tp::sentinel(), L);
    std::vector<std::atomic<uint64_t>> parents(n);
    for (auto& p : parents)
        p.store(encodedSentinel, std::memory_order_relaxed);

    // Corner hashes (:672-720): TransformPointer::create(item, direction) with the ORIGINAL index.
    std::vector<std::pair<uint64_t, uint64_t>> hp(8 * n);
    for (uint32_t d = 0; d < 8; ++d) {
        const bool px = d & 1, py = d & 2, pz = d & 4;
        const uint32_t ax = px ? 0 : R - 1, ay = py ? 0 : R - 1, az = pz ? 0 : R - 1;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            std::vector<uint64_t> h(N);
            for (uint32_t v = 0; v < N; ++v)
                h[v] = (grids[i].w[v >> 6] >> (v & 63)) & 1;
            hashPass<R>(h, 0, px);
            hashPass<R>(h, 1, py);
            hashPass<R>(h, 2, pz);
            hp[d * n + i] = { h[ax + R * ay + R * R * az], tp::create((uint64_t)i, d) };
        }
    }
    std::erase_if(hp, [](const auto& e) { return e.first == 0; });
    std::sort(hp.begin(), hp.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    st.tableEntries += hp.size();
    std::vector<uint64_t> pointers(hp.size());
    std::unordered_map<uint64_t, std::pair<uint32_t, uint32_t>> lut;
    {
        size_t start = 0;
        for (size_t i = 0; i <= hp.size(); ++i) {
            if (i == hp.size() || hp[i].first != hp[start].first) {
                if (i > start)
                    lut.emplace(hp[start].first, std::pair<uint32_t, uint32_t> { (uint32_t)start, (uint32_t)i });
                start = i;
            }
        }
        for (size_t i = 0; i < hp.size(); ++i)
            pointers[i] = hp[i].second;
    }

    // Search (:769-877). The batch-wise range pruning (:887-915) only removes candidates that cannot
    // lower a parent; the result is the minimum over verified candidates either way.
    uint64_t sProbes = 0, sHits = 0, sCand = 0, sVer = 0, sOk = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : sProbes, sHits, sCand, sVer, sOk)
    for (int64_t r = 0; r < (int64_t)n; ++r) {
        const uint32_t itemIdx = (uint32_t)r; // position in popcount order
        const uint64_t minKey = tp::encodeFixed64(tp::create(itemIdx, 0, 0, 1 - (int)R, 1 - (int)R, 1 - (int)R), L);
        const Grid<R>& grid = grids[order[r]];
        std::vector<uint64_t> init(N), h(N);
        for (uint32_t v = 0; v < N; ++v)
            init[v] = (grid.w[v >> 6] >> (v & 63)) & 1;
        for (uint32_t d = 0; d < 8; ++d) {
            const bool dir[3] = { (d & 1) != 0, (d & 2) != 0, (d & 4) != 0 };
            const int anchor[3] = { dir[0] ? 0 : (int)R - 1, dir[1] ? 0 : (int)R - 1, dir[2] ? 0 : (int)R - 1 };
            for (uint32_t pid = 0; pid < 6; ++pid) {
                const uint8_t* P = kPerm[pid];
                h = init;
                // computePermutedGridHashInPlace_AVX2 (:481-495): pass k runs along axis P[k] with direction dir[k]
                hashPass<R>(h, P[0], dir[0]);
                hashPass<R>(h, P[1], dir[1]);
                hashPass<R>(h, P[2], dir[2]);
                for (uint32_t v = 0; v < N; ++v) {
                    const uint64_t hash = h[v];
                    if (hash == 0)
                        continue;
                    ++sProbes;
                    auto it = lut.find(hash);
                    if (it == lut.end())
                        continue;
                    ++sHits;
                    const int hv[3] = { (int)(v % R), (int)((v / R) % R), (int)(v / (R * R)) };
                    const int voxel[3] = { hv[P[0]], hv[P[1]], hv[P[2]] };
                    for (uint32_t gi = it->second.first; gi < it->second.second; ++gi) {
                        const uint64_t cand = pointers[gi];
                        const uint32_t target = (uint32_t)tp::ptr(cand);
                        ++sCand;
                        const uint64_t cur = parents[target].load(std::memory_order_relaxed);
                        if (minKey >= cur)
                            continue;
                        const uint32_t S = d ^ tp::sym(cand);
                        int T[3];
                        for (int k = 0; k < 3; ++k)
                            T[k] = ((S >> k) & 1) ? voxel[k] - anchor[k] : anchor[k] - voxel[k];
                        const uint64_t sp = tp::create(itemIdx, S, pid, T[0], T[1], T[2]);
                        if (!cfg.axisPermutation && pid != 0)
                            continue;
                        if (!cfg.symmetry && S != 0)
                            continue;
                        if (!cfg.translation && (T[0] != 0 || T[1] != 0 || T[2] != 0))
                            continue;
                        const uint64_t key = tp::encodeFixed64(sp, L);
                        if (key >= cur)
                            continue;
                        ++sVer;
                        const Grid<R> g2 = translateGrid<R>(mirrorGrid<R>(permuteGrid<R>(grid, P), S), T[0], T[1], T[2]);
                        if (!(grids[target] == g2))
                            continue;
                        ++sOk;
                        atomicMin64(parents[target], key);
                    }
                }
            }
        }
    }
    st.probes += sProbes;
    st.hits += sHits;
    st.candidates += sCand;
    st.verifications += sVer;
    st.verified += sOk;

    // Decode (:923-937) and resolve (:943-999).
    std::vector<uint64_t> par(n);
    for (size_t i = 0; i < n; ++i) {
        const uint64_t e = parents[i].load();
        if (e == encodedSentinel) {
            par[i] = tp::sentinel();
        } else {
            uint64_t v = tp::decodeFixed64(e, L);
            v = (v & ~tp::kPtrMask) | order[tp::ptr(v)];
            par[i] = v;
        }
    }
    std::vector<uint8_t> isUnique(n, 0);
    for (size_t i = 0; i < n; ++i) {
        if (par[i] == tp::sentinel())
            isUnique[i] = 1;
        else
            isUnique[tp::ptr(par[i])] = 1;
    }
    std::vector<uint32_t> uniques;
    for (size_t i = 0; i < n; ++i)
        if (isUnique[i]) {
            outMapping[i] = tp::create(uniques.size());
            uniques.push_back((uint32_t)i);
        }
    for (size_t i = 0; i < n; ++i)
        if (!isUnique[i]) {
            uint64_t p = par[i];
            p = (p & ~tp::kPtrMask) | tp::ptr(outMapping[tp::ptr(p)]);
            outMapping[i] = p;
        }
    st.unique += uniques.size();
    return uniques;
}

static std::array<uint64_t, 8> toTransformNode(const std::array<uint32_t, 8>& n) // transform_dag.cpp:123-135
{
    std::array<uint64_t, 8> o;
    for (int k = 0; k < 8; ++k)
        o[k] = (n[k] == kEmpty32) ? tp::sentinel() : tp::create(n[k]);
    return o;
}

template <uint32_t L>
static void translationLevel(const Structure32& in, StructureTP& out, const Config& cfg, MatchStats& st)
{
    constexpr uint32_t R = 1u << L;
    const size_t numItems = (L == 2) ? in.leaves.size() : in.nodes[L].size();
    std::vector<uint8_t> referenced(numItems, 0);
    auto& parentNodes = out.nodes[L + 1];
    for (const auto& node : parentNodes)
        for (uint64_t c : node)
            if (c != tp::sentinel())
                referenced[tp::ptr(c)] = 1;
    std::vector<uint32_t> indices;
    for (uint32_t i = 0; i < numItems; ++i)
        if (referenced[i])
            indices.push_back(i);
    std::vector<Grid<R>> grids(indices.size());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)indices.size(); ++i)
        flattenRec(in, L, indices[i], R, 0, 0, 0, grids[i].w.data());
    std::vector<uint64_t> mapping;
    const auto remaining = findDuplicates<L>(grids, mapping, cfg, st);
    if (L == 2) {
        out.leaves.resize(remaining.size());
        for (size_t i = 0; i < remaining.size(); ++i)
            out.leaves[i] = in.leaves[indices[remaining[i]]];
    } else {
        out.nodes[L].resize(remaining.size());
        for (size_t i = 0; i < remaining.size(); ++i)
            out.nodes[L][i] = toTransformNode(in.nodes[L][indices[remaining[i]]]);
    }
    for (auto& node : parentNodes)
        for (uint64_t& c : node) {
            if (c == tp::sentinel())
                continue;
            auto it = std::lower_bound(indices.begin(), indices.end(), (uint32_t)tp::ptr(c));
            check(it != indices.end() && *it == tp::ptr(c), "parent pointer not referenced");
            c = mapping[it - indices.begin()];
        }
}

// A6: constructTransformDAG (transform_dag.cpp:138-240).
static StructureTP constructTransformDAG(const Structure32& in, const Config& cfg, MatchStats& st, std::vector<uint64_t>* levelTimes = nullptr,
    bool staticOffsets = false)
{
    if (!staticOffsets) // the static variant does not check (transform_dag.cpp:244)
        check(in.structureType == 1, "input structure must be a DAG");
    const double t0 = omp_get_wtime();
    HierResult h = constructHierarchical(in, cfg.maxTranslationLevel + 1, cfg, staticOffsets);
    const double t1 = omp_get_wtime();
    if (levelTimes)
        levelTimes->push_back((uint64_t)((t1 - t0) * 1e9));
    if (!cfg.translation)
        return std::move(h.out);
    StructureTP& out = h.out;
    check(cfg.maxTranslationLevel >= 2 && cfg.maxTranslationLevel <= 4, "maxTranslationLevel must be in [2, 4]");
    check(in.rootLevel >= cfg.maxTranslationLevel + 1, "rootLevel must exceed maxTranslationLevel");
    out.leaves.clear();
    for (uint32_t level = 3; level <= cfg.maxTranslationLevel; ++level)
        out.nodes[level].clear();
    auto& mid = out.nodes[cfg.maxTranslationLevel + 1];
    check(mid.size() == h.midInvMapping.size(), "mid level size mismatch");
    for (size_t i = 0; i < mid.size(); ++i)
        mid[i] = toTransformNode(in.nodes[cfg.maxTranslationLevel + 1][h.midInvMapping[i]]);
    for (uint32_t level = cfg.maxTranslationLevel; level >= 2; --level) {
        const double ta = omp_get_wtime();
        if (level == 4)
            translationLevel<4>(in, out, cfg, st);
        else if (level == 3)
            translationLevel<3>(in, out, cfg, st);
        else
            translationLevel<2>(in, out, cfg, st);
        if (levelTimes)
            levelTimes->push_back((uint64_t)((omp_get_wtime() - ta) * 1e9));
    }
    return std::move(out);
}

// ------------------------------------------------------------------------------------------------
// Lossless decode of a transform DAG (semantics of TransformPointer as applied by the hierarchical
// and translation stages: content = translate(mirror(permute(C, P), S), T)).
// ------------------------------------------------------------------------------------------------
static bool tdagGet(const StructureTP& s, uint32_t x, uint32_t y, uint32_t z)
{
    if (s.nodes[s.rootLevel].empty())
        return false;
    uint64_t ptr = tp::create(0);
    int v[3] = { (int)x, (int)y, (int)z };
    for (uint32_t level = s.rootLevel;; --level) {
        const int R = 1 << level;
        // undo the pointer's transform: world -> canonical local coordinates
        int w[3] = { v[0] - tp::tx(ptr), v[1] - tp::ty(ptr), v[2] - tp::tz(ptr) };
        for (int k = 0; k < 3; ++k)
            if (w[k] < 0 || w[k] >= R)
                return false;
        const uint32_t S = tp::sym(ptr);
        for (int k = 0; k < 3; ++k)
            if ((S >> k) & 1)
                w[k] = R - 1 - w[k];
        uint8_t P[3];
        tp::perm(ptr, P);
        int u[3];
        for (int k = 0; k < 3; ++k)
            u[P[k]] = w[k];
        const uint64_t idx = tp::ptr(ptr);
        if (level == 2) {
            const uint32_t bit = morton3((uint32_t)u[0], (uint32_t)u[1], (uint32_t)u[2]);
            return (s.leaves[idx] >> bit) & 1;
        }
        const int half = R / 2;
        const uint32_t c = morton3(u[0] >= half, u[1] >= half, u[2] >= half);
        const uint64_t child = s.nodes[level][idx][c];
        if (child == tp::sentinel())
            return false;
        for (int k = 0; k < 3; ++k)
            v[k] = u[k] % half;
        ptr = child;
    }
}

// ------------------------------------------------------------------------------------------------
// StaticStructure (structure.h:298-320, 765-798, 859-895): per level a packed word stream, each node a
// header word (child mask, bit i = child i) followed by one word per present child in child order;
// child words are word offsets into the level below (level 3: leaf indices). Words are uint32_t for
// EditNode<uint32_t> inputs and the 64-bit TransformPointer for transform DAGs.
// ------------------------------------------------------------------------------------------------
template <typename W>
struct StaticS {
    std::vector<std::vector<W>> words;
    std::vector<uint64_t> leaves;
    uint32_t resolution = 0, rootLevel = 0, structureType = 0;
};
template <typename W, typename C>
static StaticS<W> toStatic(const Structure<C>& s, C empty) // StaticStructure(const EditStructure&) (:765-798)
{
    StaticS<W> out;
    out.resolution = s.resolution;
    out.rootLevel = s.rootLevel;
    out.structureType = s.structureType;
    out.leaves = s.leaves;
    out.words.resize(s.nodes.size());
    std::vector<uint64_t> prev(s.leaves.size());
    std::iota(prev.begin(), prev.end(), 0ull);
    for (uint32_t level = 3; level <= s.rootLevel; ++level) {
        std::vector<uint64_t> cur(s.nodes[level].size());
        auto& w = out.words[level];
        for (size_t i = 0; i < s.nodes[level].size(); ++i) {
            cur[i] = w.size();
            const size_t head = w.size();
            w.push_back(0);
            for (uint32_t k = 0; k < 8; ++k) {
                const C c = s.nodes[level][i][k];
                if (c == empty)
                    continue;
                if constexpr (sizeof(C) == 8)
                    w.push_back((W)((c & ~tp::kPtrMask) | (prev[tp::ptr(c)] & tp::kPtrMask)));
                else
                    w.push_back((W)prev[c]);
                w[head] |= (W)1 << k;
            }
        }
        prev = std::move(cur);
    }
    return out;
}
// The inverse: node starts by a sequential walk (getLevelNodeStarts, :859-876), offsets -> indices.
template <typename W, typename C>
static Structure<C> fromStatic(const StaticS<W>& s, C empty)
{
    Structure<C> out;
    out.resolution = s.resolution;
    out.rootLevel = s.rootLevel;
    out.structureType = s.structureType;
    out.leaves = s.leaves;
    out.nodes.resize(s.words.size());
    std::unordered_map<uint64_t, uint64_t> prev; // child word offset -> index (level 3: identity)
    for (uint32_t level = 3; level <= s.rootLevel; ++level) {
        const auto& w = s.words[level];
        std::unordered_map<uint64_t, uint64_t> cur;
        for (size_t at = 0; at < w.size();) {
            const uint32_t mask = (uint32_t)w[at] & 0xFF;
            check(((uint64_t)w[at] >> 8) == 0 || sizeof(W) == 8, "static header word has bits above the child mask");
            cur[at] = out.nodes[level].size();
            std::array<C, 8> node;
            node.fill(empty);
            size_t c = at + 1;
            for (uint32_t k = 0; k < 8; ++k) {
                if (!((mask >> k) & 1))
                    continue;
                check(c < w.size(), "static node runs past its level");
                const uint64_t v = w[c++];
                const uint64_t off = sizeof(C) == 8 ? tp::ptr(v) : v;
                uint64_t idx = off;
                if (level > 3) {
                    auto it = prev.find(off);
                    check(it != prev.end(), "static child pointer is not a node start");
                    idx = it->second;
                } else {
                    check(idx < s.leaves.size(), "static leaf pointer out of range");
                }
                if constexpr (sizeof(C) == 8)
                    node[k] = (C)((v & ~tp::kPtrMask) | (idx & tp::kPtrMask));
                else
                    node[k] = (C)idx;
            }
            out.nodes[level].push_back(node);
            at = c;
        }
        prev = std::move(cur);
    }
    return out;
}
template <typename W>
static void writeStatic(Writer& wr, const StaticS<W>& s) // StaticStructure::writeTo (:888-895)
{
    wr.pod<uint64_t>(s.words.size());
    for (const auto& l : s.words)
        wr.vec(l);
    wr.vec(s.leaves);
    wr.pod(s.resolution);
    wr.pod(s.rootLevel);
    wr.pod(s.structureType);
}
template <typename W>
static StaticS<W> readStatic(Reader& r)
{
    StaticS<W> s;
    const uint64_t nl = r.pod<uint64_t>();
    check(nl >= 4 && nl <= 32, "corrupt static level count");
    s.words.resize(nl);
    for (auto& l : s.words)
        l = r.vec<W>();
    s.leaves = r.vec<uint64_t>();
    s.resolution = r.pod<uint32_t>();
    s.rootLevel = r.pod<uint32_t>();
    s.structureType = r.pod<uint32_t>();
    check(s.rootLevel + 1 == nl, "rootLevel does not match level count");
    return s;
}

} // namespace orc

// ================================================================================================
// C API (ctypes). All functions return 0 on success, non-zero on error (message via orc_last_error).
// ================================================================================================
static thread_local std::string g_err;
static int fail(const std::exception& e)
{
    g_err = e.what();
    return 1;
}
static uint8_t* dupBuf(const std::vector<uint8_t>& b, uint64_t* outLen)
{
    uint8_t* p = (uint8_t*)std::malloc(b.size() ? b.size() : 1);
    if (!b.empty())
        std::memcpy(p, b.data(), b.size());
    *outLen = b.size();
    return p;
}
static orc::Structure32 readSvo(const uint8_t* buf, uint64_t len)
{
    orc::Reader r { buf, len };
    orc::check(r.pod<uint32_t>() == orc::kSvoMagic, "bad .svo magic");
    orc::check(r.pod<uint32_t>() == orc::kSvoVersion, "bad .svo version");
    auto s = orc::readStructure<uint32_t>(r);
    orc::check(r.off == len, "trailing bytes in .svo");
    return s;
}
static std::vector<uint8_t> writeSvo(const orc::Structure32& s)
{
    orc::Writer w;
    w.pod(orc::kSvoMagic);
    w.pod(orc::kSvoVersion);
    orc::writeStructure(w, s);
    return std::move(w.buf);
}
static orc::Config mkCfg(int sym, int axis, int trans, uint32_t maxL)
{
    orc::Config c;
    c.symmetry = sym != 0;
    c.axisPermutation = axis != 0;
    c.translation = trans != 0;
    c.maxTranslationLevel = maxL;
    return c;
}

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }
void orc_free(void* p) { std::free(p); }
void orc_set_threads(int n)
{
    if (n > 0)
        omp_set_num_threads(n);
}
int orc_max_threads() { return omp_get_max_threads(); }

int orc_svo_from_dense(const uint8_t* dense, uint32_t res, uint8_t** out, uint64_t* outLen)
{
    try {
        *out = dupBuf(writeSvo(orc::svoFromDense(dense, res)), outLen);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int orc_to_dag(const uint8_t* svo, uint64_t len, uint8_t** out, uint64_t* outLen)
{
    try {
        auto s = readSvo(svo, len);
        orc::toDAG(s);
        *out = dupBuf(writeSvo(s), outLen);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// .tdag = EditStructure<void,TransformPointer>::writeTo followed by the raw 8-byte TransformDAGConfig
// (voxelizer/src/main.cpp:144-151); the config's padding byte (offset 3) is written as zero.
// stats (may be null): [items, probes, hits, candidates, verifications, verified, tableEntries, unique]
// times_ns (may be null, 4 entries): hierarchical, level 4, level 3, level 2.
int orc_construct_tdag(const uint8_t* svo, uint64_t len, int sym, int axis, int trans, uint32_t maxL, uint8_t** out, uint64_t* outLen, uint64_t* stats, uint64_t* timesNs)
{
    try {
        auto in = readSvo(svo, len);
        const orc::Config cfg = mkCfg(sym, axis, trans, maxL);
        orc::MatchStats st;
        std::vector<uint64_t> times;
        auto res = orc::constructTransformDAG(in, cfg, st, &times);
        orc::Writer w;
        orc::writeStructure(w, res);
        const uint8_t cfgBytes[8] = { (uint8_t)cfg.symmetry, (uint8_t)cfg.axisPermutation, (uint8_t)cfg.translation, 0,
            (uint8_t)(maxL & 0xFF), (uint8_t)((maxL >> 8) & 0xFF), (uint8_t)((maxL >> 16) & 0xFF), (uint8_t)(maxL >> 24) };
        w.buf.insert(w.buf.end(), cfgBytes, cfgBytes + 8);
        *out = dupBuf(w.buf, outLen);
        if (stats) {
            const uint64_t s[8] = { st.items, st.probes, st.hits, st.candidates, st.verifications, st.verified, st.tableEntries, st.unique };
            std::memcpy(stats, s, sizeof(s));
        }
        if (timesNs)
            for (size_t i = 0; i < 4; ++i)
                timesNs[i] = i < times.size() ? times[i] : 0;
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// Inner seam: findDuplicatesAmongFlattenedItems_cpp2<level> on dense grids (W = R^3/64 words per item,
// bit i = x + R*y + R*R*z). outMapping: n TransformPointers; outUnique: item positions of the unique items.
int orc_find_duplicates(uint32_t level, const uint64_t* grids, uint32_t n, int sym, int axis, int trans, uint64_t* outMapping, uint32_t* outUnique, uint32_t* nUnique, uint64_t* stats)
{
    try {
        const orc::Config cfg = mkCfg(sym, axis, trans, 4);
        orc::MatchStats st;
        std::vector<uint64_t> mapping;
        std::vector<uint32_t> uniq;
        const auto run = [&]<uint32_t L>() {
            constexpr uint32_t W = orc::Grid<(1u << L)>::W;
            std::vector<orc::Grid<(1u << L)>> g(n);
            for (uint32_t i = 0; i < n; ++i)
                std::memcpy(g[i].w.data(), grids + (size_t)i * W, W * 8);
            uniq = orc::findDuplicates<L>(g, mapping, cfg, st);
        };
        if (level == 2)
            run.template operator()<2>();
        else if (level == 3)
            run.template operator()<3>();
        else if (level == 4)
            run.template operator()<4>();
        else
            throw std::runtime_error("level must be 2, 3 or 4");
        std::memcpy(outMapping, mapping.data(), n * 8);
        std::memcpy(outUnique, uniq.data(), uniq.size() * 4);
        *nUnique = (uint32_t)uniq.size();
        if (stats) {
            const uint64_t s[8] = { st.items, st.probes, st.hits, st.candidates, st.verifications, st.verified, st.tableEntries, st.unique };
            std::memcpy(stats, s, sizeof(s));
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// Hierarchical pass alone (constructTransformDAGHierarchical without translation), as .tdag bytes
// without the trailing config.
int orc_hierarchical(const uint8_t* svo, uint64_t len, int sym, int axis, uint8_t** out, uint64_t* outLen)
{
    try {
        auto in = readSvo(svo, len);
        orc::Config cfg = mkCfg(sym, axis, 0, 0);
        auto h = orc::constructHierarchical(in, ~0u, cfg);
        orc::Writer w;
        orc::writeStructure(w, h.out);
        *out = dupBuf(w.buf, outLen);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// Decode a .tdag (structure part; trailing config optional) into a dense res^3 byte grid.
int orc_tdag_decode(const uint8_t* tdag, uint64_t len, uint8_t* dense, uint32_t res)
{
    try {
        orc::Reader r { tdag, len };
        auto s = orc::readStructure<uint64_t>(r);
        orc::check(s.resolution == res, "resolution mismatch");
#pragma omp parallel for schedule(static)
        for (int64_t z = 0; z < (int64_t)res; ++z)
            for (uint32_t y = 0; y < res; ++y)
                for (uint32_t x = 0; x < res; ++x)
                    dense[(size_t)x + (size_t)res * y + (size_t)res * res * z] = orc::tdagGet(s, x, y, (uint32_t)z) ? 1 : 0;
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// .svo (EditStructure<void, uint32_t>) -> StaticStructure<void, uint32_t>::writeTo bytes.
int orc_to_static(const uint8_t* svo, uint64_t len, uint8_t** out, uint64_t* outLen)
{
    try {
        const auto s = readSvo(svo, len);
        orc::Writer w;
        orc::writeStatic(w, orc::toStatic<uint32_t, uint32_t>(s, orc::kEmpty32));
        *out = dupBuf(w.buf, outLen);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// constructStaticTransformDAG (transform_dag.cpp:242-390) on StaticStructure<void, uint32_t> bytes:
// the same construction as orc_construct_tdag with the static variant's grouping hash, returned as
// StaticStructure<void, TransformPointer>::writeTo bytes.
int orc_construct_static_tdag(const uint8_t* in, uint64_t len, int sym, int axis, int trans, uint32_t maxL, uint8_t** out, uint64_t* outLen)
{
    try {
        orc::Reader r { in, len };
        const auto st32 = orc::readStatic<uint32_t>(r);
        const auto edit = orc::fromStatic<uint32_t, uint32_t>(st32, orc::kEmpty32);
        orc::MatchStats ms;
        const auto res = orc::constructTransformDAG(edit, mkCfg(sym, axis, trans, maxL), ms, nullptr, true);
        orc::Writer w;
        orc::writeStatic(w, orc::toStatic<uint64_t, uint64_t>(res, orc::tp::sentinel()));
        *out = dupBuf(w.buf, outLen);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// Every voxel of a StaticStructure<void, TransformPointer> (dense[x + res*y + res*res*z]).
int orc_static_tdag_decode(const uint8_t* in, uint64_t len, uint8_t* dense, uint32_t res)
{
    try {
        orc::Reader r { in, len };
        const auto s = orc::fromStatic<uint64_t, uint64_t>(orc::readStatic<uint64_t>(r), orc::tp::sentinel());
        orc::check(s.resolution == res, "resolution mismatch");
#pragma omp parallel for schedule(static)
        for (int64_t z = 0; z < (int64_t)res; ++z)
            for (uint32_t y = 0; y < res; ++y)
                for (uint32_t x = 0; x < res; ++x)
                    dense[(size_t)x + (size_t)res * y + (size_t)res * res * z] = orc::tdagGet(s, x, y, (uint32_t)z) ? 1 : 0;
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// Transform tables for cross-checking the library's own tables.
int orc_transform_tables(uint8_t* compose48x48, uint8_t* inverse48, uint8_t* pos48x8)
{
    const auto& t = orc::tt();
    std::memcpy(compose48x48, t.compose, sizeof(t.compose));
    std::memcpy(inverse48, t.inverse, sizeof(t.inverse));
    std::memcpy(pos48x8, t.pos, sizeof(t.pos));
    return 0;
}

uint64_t orc_encode_fixed64(uint64_t tpRaw, uint32_t level) { return orc::tp::encodeFixed64(tpRaw, level); }
uint64_t orc_decode_fixed64(uint64_t e, uint32_t level) { return orc::tp::decodeFixed64(e, level); }

} // extern "C"
