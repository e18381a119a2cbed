// tdag16_oracle.cpp — CPU ORACLE (test infrastructure only): the .tdag16 encoding of a transform DAG.
//
// A from-scratch CPU restatement of the reference's TransformDAG16 encoder and decoder
// (tools/svdag_encoding/src/transform_dag_encoding.cpp:240-497, 519-562, 1023-1040;
// pointer_encoding.h:27-72, 159-177; huffman.cpp:27-236). It is NOT part of the product: only tests/,
// __graft_entry__.smoke() and bench.py's CPU legs may load it (through oracle.py).
//
// Tie order. Two steps of the reference order equal-count items through libstdc++ internals:
//   * sortByReferenceCount (pointer_encoding.h:49) orders items by reference count with std::sort,
//     whose placement of equal counts is the introsort's;
//   * the per-level unique child pointers come from iterating std::unordered_map<TransformPointer,...>
//     (transform_dag_encoding.cpp:276-295) and are then sorted by count with std::sort(par), whose tie
//     placement also depends on the parallel backend the reference was built with.
// The file bytes depend on these orders (item indices and pointer-table slots); the decoded voxels and
// the Huffman tables do not. kTieLibstdcxx reproduces the reference as compiled with libstdc++ and a
// serial parallel-algorithms backend: the real std::sort / std::unordered_map with the reference's
// hash functor (transform_dag.h:412-433). kTieCanonical breaks every tie by a stated key — items by
// ascending index (a stable sort), unique pointers by ascending 64-bit value — which a GPU can produce
// with stable radix sorts; the library's encoder is bit-exact with this mode.

#include <algorithm>
#include <cmath>
#include <array>
#include <bit>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>
#include <omp.h>

namespace orc16 {

static void check(bool ok, const char* what)
{
    if (!ok)
        throw std::runtime_error(what);
}

enum TieMode : int { kTieCanonical = 0, kTieLibstdcxx = 1 };

// ------------------------------------------------------------------------------------------------
// TransformPointer, compact layout (transform_dag.h:19-33): ptr:37 | sx sy sz | p0:2 p1:2 p2:2 |
// tx:6 ty:6 tz:6 (translations biased by 32). Permutation code 2*p0 + (p2 < p1) (transform_dag.h:326-331).
// ------------------------------------------------------------------------------------------------
static constexpr uint64_t kPtrMask = (1ull << 37) - 1;
static const uint8_t kPerm[6][3] = { { 0, 1, 2 }, { 0, 2, 1 }, { 1, 0, 2 }, { 1, 2, 0 }, { 2, 0, 1 }, { 2, 1, 0 } };
static inline uint64_t tpPtr(uint64_t v) { return v & kPtrMask; }
static inline uint64_t tpWithPtr(uint64_t v, uint64_t p) { return (v & ~kPtrMask) | (p & kPtrMask); }
static inline uint32_t tpSym(uint64_t v) { return (uint32_t)(v >> 37) & 7; }
static inline uint32_t tpP(uint64_t v, int k) { return (uint32_t)(v >> (40 + 2 * k)) & 3; }
static inline uint32_t tpPermCode(uint64_t v) { return 2 * tpP(v, 0) + (tpP(v, 2) < tpP(v, 1) ? 1 : 0); }
static inline int tpT(uint64_t v, int axis) { return (int)((v >> (46 + 6 * axis)) & 63) - 32; }
static inline uint64_t tpSentinel() { return 0xFFFFFFFFull | (0ull << 40) | (1ull << 42) | (2ull << 44) | (32ull << 46) | (32ull << 52) | (32ull << 58); }
static inline bool tpHasTransform(uint64_t v) // transform_dag.h:115-130
{
    return tpSym(v) != 0 || !(tpP(v, 0) == 0 && tpP(v, 1) == 1 && tpP(v, 2) == 2) || tpT(v, 0) != 0 || tpT(v, 1) != 0 || tpT(v, 2) != 0;
}

struct DagConfig {
    bool symmetry = true, axisPermutation = true, translation = true;
    uint32_t maxTranslationLevel = 4;
};
struct EncConfig {
    bool pointerTables = false, huffmanCode = false;
};

// ------------------------------------------------------------------------------------------------
// Huffman codes (huffman.cpp). Code = {u64 code; u32 bits} is written raw: 16 bytes, of which the last
// 4 are struct padding (written as zero here; the reference writes whatever the padding holds).
// ------------------------------------------------------------------------------------------------
struct Code {
    uint64_t code = 0;
    uint32_t bits = 0;
};

// Length-limited code lengths by package-merge, restating createLengthLimitedHuffmanCodeLengths
// (huffman.cpp:100-163; Moffat, "Huffman Coding", ACM CSUR 2019, algorithm 3). Each level keeps its
// items in the reference's total order: by frequency, then leaves before packages, leaves by symbol,
// packages lexicographically by their two members (the std::set<Node> order of huffman.cpp:115-125).
struct PmItem {
    uint64_t freq;
    int32_t symbol; // >= 0: leaf; -1: package of (a, b) in the previous level's arena
    int32_t a, b;
    uint32_t level;
};
struct PackageMerge {
    std::vector<std::vector<PmItem>> levels; // sorted items per level
    bool less(const PmItem& x, const PmItem& y) const
    {
        if (x.freq != y.freq)
            return x.freq < y.freq;
        const bool xl = x.symbol >= 0, yl = y.symbol >= 0;
        if (xl != yl)
            return xl; // variant index: leaf (0) before package (1)
        if (xl)
            return x.symbol < y.symbol;
        const auto& prev = levels[x.level - 1];
        if (less(prev[x.a], prev[y.a]))
            return true;
        if (less(prev[y.a], prev[x.a]))
            return false;
        return less(prev[x.b], prev[y.b]);
    }
};
static std::vector<uint32_t> lengthLimitedCodeLengths(const std::vector<uint64_t>& freq, uint32_t maxLen)
{
    const uint32_t n = (uint32_t)freq.size();
    check(n >= 1 && maxLen >= 1, "huffman: empty alphabet");
    PackageMerge pm;
    pm.levels.resize(maxLen);
    auto sortLevel = [&](uint32_t l) {
        auto& v = pm.levels[l];
        std::sort(v.begin(), v.end(), [&](const PmItem& x, const PmItem& y) { return pm.less(x, y); });
        for (size_t i = 1; i < v.size(); ++i)
            check(pm.less(v[i - 1], v[i]), "huffman: equal package-merge items");
    };
    for (uint32_t s = 0; s < n; ++s)
        pm.levels[0].push_back({ freq[s], (int32_t)s, -1, -1, 0 });
    sortLevel(0);
    for (uint32_t l = 1; l < maxLen; ++l) {
        const auto& prev = pm.levels[l - 1];
        auto& cur = pm.levels[l];
        for (size_t i = 0; i + 1 < prev.size(); i += 2)
            cur.push_back({ prev[i].freq + prev[i + 1].freq, -1, (int32_t)i, (int32_t)(i + 1), l });
        for (uint32_t s = 0; s < n; ++s)
            cur.push_back({ freq[s], (int32_t)s, -1, -1, l });
        sortLevel(l);
    }
    // The 2n-2 smallest items of the top level are chosen; going down, each chosen package selects
    // the 2 * (chosen packages) smallest items of the level below. A symbol's length is the number of
    // chosen leaves carrying it.
    std::vector<uint32_t> lengths(n, 0);
    size_t take = 2 * (size_t)n - 2;
    for (int l = (int)maxLen - 1; l >= 0 && take > 0; --l) {
        const auto& items = pm.levels[l];
        check(take <= items.size(), "huffman: code length limit too small for the alphabet");
        size_t packages = 0;
        for (size_t i = 0; i < take; ++i) {
            if (items[i].symbol >= 0)
                ++lengths[items[i].symbol];
            else
                ++packages;
        }
        take = 2 * packages;
    }
    return lengths;
}

// Canonical code words (huffman.cpp:78-98): symbols in order of increasing length — ordered by
// std::sort, as the reference does, so equal lengths take the same order — get consecutive codes.
static std::vector<Code> assignCodeWords(const std::vector<uint32_t>& lengths)
{
    std::vector<uint32_t> symbols(lengths.size());
    std::iota(symbols.begin(), symbols.end(), 0u);
    std::sort(symbols.begin(), symbols.end(), [&](uint32_t l, uint32_t r) { return lengths[l] < lengths[r]; });
    const uint32_t maxLen = *std::max_element(lengths.begin(), lengths.end());
    uint32_t next = 0;
    std::vector<Code> codes(lengths.size());
    for (uint32_t s : symbols) {
        const uint32_t bits = lengths[s];
        codes[s] = Code { (uint64_t)(next >> (maxLen - bits)), bits };
        next += 1u << (maxLen - bits);
    }
    return codes;
}
static void codesToLsb(std::vector<Code>& codes) // huffman.cpp:172-182: bit-reverse each code
{
    for (Code& c : codes) {
        uint64_t r = 0;
        for (uint32_t i = 0; i < c.bits; ++i)
            r |= ((c.code >> i) & 1) << (c.bits - 1 - i);
        c.code = r;
    }
}
static bool kraftOk(const std::vector<uint32_t>& lengths) // exact form of kraftSum(...) <= 1
{
    uint64_t s = 0;
    for (uint32_t l : lengths)
        s += 1ull << (32 - l);
    return s <= (1ull << 32);
}
static std::vector<Code> lengthLimitedCodeTable(const std::vector<uint64_t>& freq, uint32_t maxLen) // huffman.cpp:165-170
{
    const auto lengths = lengthLimitedCodeLengths(freq, maxLen);
    check(kraftOk(lengths), "huffman: Kraft sum above 1");
    return assignCodeWords(lengths);
}
// Decode table (huffman.cpp:184-201): every key whose low `bits` bits equal a code maps to it.
struct DecodeLut {
    std::vector<std::pair<uint32_t, uint32_t>> table;
    uint32_t mask = 0;
    explicit DecodeLut(const std::vector<Code>& codes)
    {
        uint32_t maxLen = 0;
        for (const Code& c : codes)
            maxLen = std::max(maxLen, c.bits);
        mask = (1u << maxLen) - 1u;
        table.assign(1ull << maxLen, { 0u, 0u });
        for (uint32_t k = 0; k < codes.size(); ++k)
            for (uint32_t suffix = 0; suffix < (1u << (maxLen - codes[k].bits)); ++suffix)
                table[(suffix << codes[k].bits) | (uint32_t)codes[k].code] = { k, codes[k].bits };
    }
    std::pair<uint32_t, uint32_t> decode(uint32_t key) const { return table[key & mask]; }
};

// ------------------------------------------------------------------------------------------------
// Input: EditStructure<void, TransformPointer> as written to .tdag (structure + 8-byte config).
// ------------------------------------------------------------------------------------------------
struct Dag {
    std::vector<std::vector<std::array<uint64_t, 8>>> nodes; // per level
    std::vector<uint64_t> leaves;
    uint32_t resolution = 0, rootLevel = 0;
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
        if (cnt)
            std::memcpy(v.data(), p + off, cnt * sizeof(T));
        off += cnt * sizeof(T);
        return v;
    }
};
static void readTdag(const uint8_t* buf, size_t len, Dag& dag, DagConfig& cfg)
{
    Reader r { buf, len };
    const uint64_t nl = r.pod<uint64_t>();
    check(nl >= 4 && nl <= 32, "tdag16 needs root level 3..31");
    dag.nodes.resize(nl);
    for (auto& l : dag.nodes)
        l = r.vec<std::array<uint64_t, 8>>();
    dag.leaves = r.vec<uint64_t>();
    dag.resolution = r.pod<uint32_t>();
    dag.rootLevel = r.pod<uint32_t>();
    (void)r.pod<uint32_t>(); // structureType
    check(dag.rootLevel + 1 == nl, "rootLevel does not match level count");
    uint8_t c[8];
    for (auto& b : c)
        b = r.pod<uint8_t>();
    cfg.symmetry = c[0];
    cfg.axisPermutation = c[1];
    cfg.translation = c[2];
    std::memcpy(&cfg.maxTranslationLevel, c + 4, 4);
}

// ------------------------------------------------------------------------------------------------
// sortByReferenceCount (pointer_encoding.h:27-72) with pruning: items ordered by how often the parent
// level references them (descending), unreferenced items dropped, parents' child indices remapped
// (only the index: TransformPointer::operator=(uint32_t), transform_dag.h:333-337).
// ------------------------------------------------------------------------------------------------
template <typename T>
static std::vector<T> sortByReferenceCount(const std::vector<T>& items, std::vector<std::array<uint64_t, 8>>& parents, TieMode mode)
{
    const uint64_t sentinel = tpSentinel();
    std::vector<uint32_t> refs(items.size(), 0);
    std::vector<uint8_t> referenced(items.size(), 0);
    for (const auto& p : parents)
        for (uint64_t c : p)
            if (c != sentinel) {
                const uint32_t idx = (uint32_t)c;
                check(idx < items.size(), "dangling child pointer");
                referenced[idx] = 1;
                ++refs[idx];
            }
    std::vector<uint32_t> order(items.size());
    std::iota(order.begin(), order.end(), 0u);
    auto byCount = [&](uint32_t l, uint32_t r) { return refs[l] > refs[r]; };
    if (mode == kTieLibstdcxx)
        std::sort(order.begin(), order.end(), byCount);
    else
        std::stable_sort(order.begin(), order.end(), byCount);
    std::vector<T> out;
    out.reserve(items.size());
    std::vector<uint32_t> mapping(items.size(), 0);
    for (uint32_t i : order) {
        if (!referenced[i])
            continue;
        mapping[i] = (uint32_t)out.size();
        out.push_back(items[i]);
    }
    for (auto& p : parents)
        for (uint64_t& c : p)
            if (c != sentinel)
                c = tpWithPtr(c, mapping[(uint32_t)c]);
    return out;
}

// std::hash<TransformPointer> (transform_dag.h:412-433): hash_combine over ptr, the symmetry flags,
// the permutation and the translation, each through the identity std::hash of its type (ints are
// sign-extended to size_t). Only kTieLibstdcxx iterates a map keyed with it.
struct RefHash {
    static void combine(uint64_t& seed, uint64_t v) { seed ^= v + 0x9e3779b9ull + (seed << 6) + (seed >> 2); }
    size_t operator()(uint64_t tp) const
    {
        uint64_t s = 0;
        combine(s, tpPtr(tp));
        for (int k = 0; k < 3; ++k)
            combine(s, (tpSym(tp) >> k) & 1);
        for (int k = 0; k < 3; ++k)
            combine(s, tpP(tp, k));
        for (int k = 0; k < 3; ++k)
            combine(s, (uint64_t)(int64_t)tpT(tp, k));
        return (size_t)s;
    }
};

// Pointer type (transform_dag_encoding.cpp:124-140): [perm code][sym bits][non-zero translation axes].
static uint32_t pointerType(uint64_t tp, uint32_t childLevel, const DagConfig& cfg)
{
    uint32_t out = 0;
    if (cfg.axisPermutation)
        out |= tpPermCode(tp);
    if (cfg.symmetry)
        out = (out << 3) | tpSym(tp);
    if (cfg.translation && childLevel <= cfg.maxTranslationLevel)
        out = (out << 3) | (tpT(tp, 0) != 0 ? 1u : 0u) | (tpT(tp, 1) != 0 ? 2u : 0u) | (tpT(tp, 2) != 0 ? 4u : 0u);
    return out;
}
static uint32_t numPointerTypes(const DagConfig& cfg) // transform_dag_encoding.cpp:303-310
{
    return (cfg.symmetry ? 8u : 1u) * (cfg.axisPermutation ? 6u : 1u) * (cfg.translation ? 8u : 1u);
}

// Encoded pointer (transform_dag_encoding.cpp:320-380).
static uint64_t encodePointer(uint64_t tp, uint32_t childLevel, const DagConfig& cfg, const EncConfig& enc, const std::vector<Code>& codes)
{
    const uint32_t tb = childLevel + 1;
    const int bias = 1 << childLevel;
    if (enc.huffmanCode) {
        const Code& c = codes[pointerType(tp, childLevel, cfg)];
        uint64_t e = tpPtr(tp);
        for (int k = 0; k < 3; ++k)
            if (tpT(tp, k) != 0)
                e = (e << tb) | (uint64_t)(unsigned)(tpT(tp, k) + bias);
        return (e << c.bits) | c.code;
    }
    const bool has = tpHasTransform(tp);
    uint64_t e = tpPtr(tp);
    if (cfg.axisPermutation && has)
        e = (e << 3) | tpPermCode(tp);
    if (cfg.symmetry && has)
        e = (e << 3) | tpSym(tp);
    if (cfg.translation && childLevel <= cfg.maxTranslationLevel && has)
        for (int k = 2; k >= 0; --k)
            e = (e << tb) | (uint64_t)(unsigned)(tpT(tp, k) + bias);
    if (cfg.axisPermutation || cfg.symmetry || cfg.translation)
        e = (e << 1) | (has ? 1 : 0);
    return e;
}

static inline uint32_t u16Words(uint64_t bits) { return (uint32_t)((bits + 15) / 16); }

struct LevelStats {
    uint64_t numNodes = 0, memoryInBytes = 0, tableSize = 0, uniquePointers = 0;
    uint64_t table[3] = { 0, 0, 0 }, direct[3] = { 0, 0, 0 };
};

struct Tdag16 {
    DagConfig cfg;
    EncConfig enc;
    std::vector<std::vector<uint16_t>> nodes;
    std::vector<uint64_t> leaves;
    uint32_t resolution = 0, rootLevel = 0;
    std::vector<std::vector<uint64_t>> pointerTables;
    std::vector<std::vector<Code>> huffman; // per level; empty entries are default LUTs
    bool hasHuffman = false;
};

// constructTransformDAG16(EditStructure<void, TransformPointer>, ...) (transform_dag_encoding.cpp:240-497).
static Tdag16 encode(Dag dag, const DagConfig& cfg, const EncConfig& enc, TieMode mode, std::vector<LevelStats>& stats)
{
    const uint32_t root = dag.rootLevel, subGridLevel = 2;
    const uint64_t sentinel = tpSentinel();
    stats.assign(root + 1, LevelStats {});
    for (uint32_t level = root - 1; level > subGridLevel; --level)
        dag.nodes[level] = sortByReferenceCount(dag.nodes[level], dag.nodes[level + 1], mode);
    dag.leaves = sortByReferenceCount(dag.leaves, dag.nodes[subGridLevel + 1], mode);

    Tdag16 out;
    out.cfg = cfg;
    out.enc = enc;
    out.leaves = dag.leaves;
    out.resolution = dag.resolution;
    out.rootLevel = root;
    out.nodes.resize(root + 1);
    out.pointerTables.resize(root + 1);
    out.hasHuffman = enc.huffmanCode;
    if (enc.huffmanCode)
        out.huffman.resize(root + 1);
    stats[subGridLevel].numNodes = out.leaves.size();
    stats[subGridLevel].memoryInBytes = out.leaves.size() * 8;

    std::vector<uint64_t> prevMap(out.leaves.size());
    std::iota(prevMap.begin(), prevMap.end(), 0ull);
    for (uint32_t level = subGridLevel + 1; level <= root; ++level) {
        const uint32_t childLevel = level - 1;
        auto& in = dag.nodes[level];
        auto& st = stats[level];
        // Child pointers now address the encoded child level; count each distinct pointer.
        std::vector<std::pair<uint32_t, uint64_t>> unique; // (reference count, pointer)
        if (mode == kTieLibstdcxx) {
            std::unordered_map<uint64_t, uint32_t, RefHash> counts;
            for (auto& node : in)
                for (uint64_t& c : node)
                    if (c != sentinel) {
                        c = tpWithPtr(c, prevMap[tpPtr(c)]);
                        counts[c]++;
                    }
            for (const auto& [tp, cnt] : counts)
                unique.push_back({ cnt, tp });
            std::sort(unique.begin(), unique.end(), [](const auto& l, const auto& r) { return l.first > r.first; });
        } else {
            std::map<uint64_t, uint32_t> counts; // ascending pointer value
            for (auto& node : in)
                for (uint64_t& c : node)
                    if (c != sentinel) {
                        c = tpWithPtr(c, prevMap[tpPtr(c)]);
                        counts[c]++;
                    }
            for (const auto& [tp, cnt] : counts)
                unique.push_back({ cnt, tp });
            std::stable_sort(unique.begin(), unique.end(), [](const auto& l, const auto& r) { return l.first > r.first; });
        }
        st.uniquePointers = unique.size();

        std::vector<Code> codes;
        if (enc.huffmanCode) {
            std::vector<uint64_t> hist(numPointerTypes(cfg), 0);
            for (const auto& u : unique)
                hist[pointerType(u.second, childLevel, cfg)]++;
            codes = lengthLimitedCodeTable(hist, 16);
            codesToLsb(codes);
            out.huffman[childLevel] = codes;
        }

        // Inline or table pointer for every distinct pointer, in reference-count order
        // (transform_dag_encoding.cpp:382-433).
        std::unordered_map<uint64_t, std::pair<uint64_t, uint32_t>> lut;
        auto& table = out.pointerTables[childLevel];
        for (const auto& [cnt, tp] : unique) {
            const uint64_t e = encodePointer(tp, childLevel, cfg, enc, codes);
            if (enc.pointerTables) {
                const uint64_t inl = e << 1;
                const uint32_t inlSize = std::max(2u, u16Words(std::bit_width(inl)));
                uint32_t inlineCost = cnt * inlSize;
                if (inlSize > 3)
                    inlineCost = UINT32_MAX;
                uint64_t tab;
                uint32_t tabSize;
                if (table.size() <= 0xFFFF) {
                    tab = table.size();
                    tabSize = 1;
                } else {
                    tab = ((uint64_t)table.size() << 1) | 1;
                    tabSize = u16Words(std::bit_width((uint64_t)table.size()));
                }
                const uint32_t tableCost = cnt * tabSize + 4;
                if (tableCost < inlineCost) {
                    table.push_back(e);
                    st.table[tabSize - 1]++;
                    lut[tp] = { tab, tabSize };
                } else {
                    st.direct[inlSize - 1]++;
                    lut[tp] = { inl, inlSize };
                }
            } else {
                const uint32_t size = std::max(1u, u16Words(std::bit_width(e)));
                check(size <= 3, "pointer wider than 48 bits without pointer tables");
                lut[tp] = { e, size };
                st.direct[size - 1]++;
            }
        }
        st.tableSize = table.size();

        // Nodes: u16 child mask (2 bits per child: pointer size in u16s), then the pointers.
        auto& os = out.nodes[level];
        prevMap.clear();
        for (const auto& node : in) {
            prevMap.push_back(os.size());
            const size_t maskAt = os.size();
            os.push_back(0);
            uint16_t mask = 0;
            for (uint32_t ci = 0; ci < 8; ++ci) {
                if (node[ci] == sentinel)
                    continue;
                const auto [v, size] = lut.find(node[ci])->second;
                for (uint32_t w = 0; w < size; ++w)
                    os.push_back((uint16_t)(v >> (16 * w)));
                mask |= (uint16_t)(size << (2 * ci));
            }
            os[maskAt] = mask;
        }
        st.numNodes = in.size();
        st.memoryInBytes = os.size() * 2;
    }
    return out;
}

// TransformDAG16::writeTo (transform_dag_encoding.cpp:1023-1030; TransformBaseDAG::writeTo,
// transform_dag_encoding.h:62-69; HuffmanDecodeLUT::writeTo, huffman.cpp:212-215).
static std::vector<uint8_t> serialize(const Tdag16& t)
{
    std::vector<uint8_t> b;
    auto pod = [&](const auto& v) {
        const auto* p = reinterpret_cast<const uint8_t*>(&v);
        b.insert(b.end(), p, p + sizeof(v));
    };
    auto raw = [&](const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); };
    const uint8_t cfgBytes[8] = { (uint8_t)t.cfg.symmetry, (uint8_t)t.cfg.axisPermutation, (uint8_t)t.cfg.translation, 0,
        (uint8_t)t.cfg.maxTranslationLevel, (uint8_t)(t.cfg.maxTranslationLevel >> 8), (uint8_t)(t.cfg.maxTranslationLevel >> 16),
        (uint8_t)(t.cfg.maxTranslationLevel >> 24) };
    raw(cfgBytes, 8);
    pod((uint8_t)t.enc.pointerTables);
    pod((uint8_t)t.enc.huffmanCode);
    pod((uint64_t)t.nodes.size());
    for (const auto& l : t.nodes) {
        pod((uint64_t)l.size());
        raw(l.data(), l.size() * 2);
    }
    pod((uint64_t)t.leaves.size());
    raw(t.leaves.data(), t.leaves.size() * 8);
    pod(t.resolution);
    pod(t.rootLevel);
    pod((uint64_t)t.pointerTables.size());
    for (const auto& l : t.pointerTables) {
        pod((uint64_t)l.size());
        raw(l.data(), l.size() * 8);
    }
    pod((uint64_t)(t.hasHuffman ? t.huffman.size() : 0));
    if (t.hasHuffman)
        for (const auto& l : t.huffman) {
            pod((uint64_t)l.size());
            for (const Code& c : l) {
                pod(c.code);
                pod(c.bits);
                pod((uint32_t)0); // padding of the 16-byte Code
            }
        }
    return b;
}

static Tdag16 deserialize(const uint8_t* buf, size_t len)
{
    Reader r { buf, len };
    Tdag16 t;
    uint8_t c[8];
    for (auto& x : c)
        x = r.pod<uint8_t>();
    t.cfg.symmetry = c[0];
    t.cfg.axisPermutation = c[1];
    t.cfg.translation = c[2];
    std::memcpy(&t.cfg.maxTranslationLevel, c + 4, 4);
    t.enc.pointerTables = r.pod<uint8_t>();
    t.enc.huffmanCode = r.pod<uint8_t>();
    const uint64_t nl = r.pod<uint64_t>();
    check(nl >= 4 && nl <= 32, "corrupt level count");
    t.nodes.resize(nl);
    for (auto& l : t.nodes)
        l = r.vec<uint16_t>();
    t.leaves = r.vec<uint64_t>();
    t.resolution = r.pod<uint32_t>();
    t.rootLevel = r.pod<uint32_t>();
    check(t.rootLevel + 1 == nl, "rootLevel does not match level count");
    const uint64_t np = r.pod<uint64_t>();
    check(np <= 32, "corrupt pointer table count");
    t.pointerTables.resize(np);
    for (auto& l : t.pointerTables)
        l = r.vec<uint64_t>();
    const uint64_t nh = r.pod<uint64_t>();
    check(nh <= 32, "corrupt Huffman table count");
    t.hasHuffman = t.enc.huffmanCode;
    t.huffman.resize(nh);
    for (auto& l : t.huffman) {
        const uint64_t n = r.pod<uint64_t>();
        check(n <= 4096, "corrupt Huffman table");
        l.resize(n);
        for (auto& code : l) {
            code.code = r.pod<uint64_t>();
            code.bits = r.pod<uint32_t>();
            (void)r.pod<uint32_t>();
        }
    }
    check(r.off == len, "trailing bytes");
    return t;
}

// ------------------------------------------------------------------------------------------------
// Decoder: TransformDAG16::getChildPointer (transform_dag_encoding.cpp:519-562) with the Huffman and
// plain pointer decoders (:142-224), and a voxel query whose traversal maps world coordinates into
// each child's canonical frame: content(child) = translate(mirror(permute(C, P), S), T).
// ------------------------------------------------------------------------------------------------
struct Decoded {
    uint64_t index;
    uint32_t sym, permCode;
    int t[3];
};
struct Decoder {
    const Tdag16& t;
    std::vector<DecodeLut> luts;
    explicit Decoder(const Tdag16& dag)
        : t(dag)
    {
        if (t.enc.huffmanCode)
            for (const auto& codes : t.huffman)
                luts.emplace_back(codes.empty() ? std::vector<Code> { Code {} } : codes);
    }
    bool child(uint32_t level, uint64_t nodeAt, uint32_t ci, Decoded& out) const
    {
        const auto& s = t.nodes[level];
        check(nodeAt < s.size(), "node offset out of range");
        const uint16_t mask = s[nodeAt];
        const uint32_t bits = (mask >> (2 * ci)) & 3;
        if (!bits)
            return false;
        uint64_t at = nodeAt + 1;
        for (uint32_t i = 0; i < ci; ++i)
            at += (mask >> (2 * i)) & 3;
        uint64_t e = 0;
        for (uint32_t w = 0; w < bits; ++w) {
            check(at + w < s.size(), "pointer past the level's stream");
            e |= (uint64_t)s[at + w] << (16 * w);
        }
        const uint32_t childLevel = level - 1;
        if (t.enc.pointerTables) {
            if (bits == 1 || (e & 1)) {
                const uint64_t idx = bits == 1 ? e : e >> 1;
                check(idx < t.pointerTables[childLevel].size(), "pointer table index out of range");
                e = t.pointerTables[childLevel][idx];
            } else {
                e >>= 1;
            }
        }
        const DagConfig& cfg = t.cfg;
        const uint32_t tb = childLevel + 1;
        const uint64_t tm = (1ull << tb) - 1;
        const int bias = 1 << childLevel;
        out = Decoded { 0, 0, 0, { 0, 0, 0 } };
        if (t.enc.huffmanCode) {
            auto [type, len] = luts[childLevel].decode((uint32_t)e);
            e >>= len;
            uint32_t axes = 0;
            if (cfg.translation && childLevel <= cfg.maxTranslationLevel) {
                axes = type & 7;
                type >>= 3;
            }
            for (int k = 2; k >= 0; --k)
                if (axes & (1u << k)) {
                    out.t[k] = (int)(e & tm) - bias;
                    e >>= tb;
                }
            if (cfg.symmetry) {
                out.sym = type & 7;
                type >>= 3;
            }
            if (cfg.axisPermutation)
                out.permCode = type & 7;
        } else {
            bool has = false;
            if (cfg.axisPermutation || cfg.symmetry || cfg.translation) {
                has = e & 1;
                e >>= 1;
            }
            if (has) {
                if (cfg.translation && childLevel <= cfg.maxTranslationLevel)
                    for (int k = 0; k < 3; ++k) {
                        out.t[k] = (int)(e & tm) - bias;
                        e >>= tb;
                    }
                if (cfg.symmetry) {
                    out.sym = e & 7;
                    e >>= 3;
                }
                if (cfg.axisPermutation) {
                    out.permCode = e & 7;
                    e >>= 3;
                }
            }
        }
        check(out.permCode < 6, "corrupt permutation code");
        out.index = e;
        return true;
    }
    bool get(uint32_t x, uint32_t y, uint32_t z) const
    {
        int v[3] = { (int)x, (int)y, (int)z };
        uint64_t at = 0;
        if (t.nodes[t.rootLevel].empty())
            return false;
        for (uint32_t level = t.rootLevel; level > 2; --level) {
            const int half = 1 << (level - 1);
            const uint32_t ci = (v[0] >= half ? 1u : 0u) | (v[1] >= half ? 2u : 0u) | (v[2] >= half ? 4u : 0u);
            Decoded d;
            if (!child(level, at, ci, d))
                return false;
            int w[3];
            for (int k = 0; k < 3; ++k) {
                w[k] = v[k] % half - d.t[k];
                if (w[k] < 0 || w[k] >= half)
                    return false;
                if ((d.sym >> k) & 1)
                    w[k] = half - 1 - w[k];
            }
            const uint8_t* p = kPerm[d.permCode];
            for (int k = 0; k < 3; ++k)
                v[p[k]] = w[k];
            at = d.index;
        }
        check(at < t.leaves.size(), "leaf index out of range");
        const uint32_t bit = [&] {
            uint32_t m = 0;
            for (int b = 0; b < 2; ++b)
                m |= (((uint32_t)v[0] >> b) & 1) << (3 * b) | (((uint32_t)v[1] >> b) & 1) << (3 * b + 1) | (((uint32_t)v[2] >> b) & 1) << (3 * b + 2);
            return m;
        }();
        return (t.leaves[at] >> bit) & 1;
    }
};

// First solid voxel along a ray by voxel-by-voxel DDA (Amanatides and Woo 1987) over Decoder::get, in
// double precision. Entry into [0, res)^3 by slabs; the crossing parameter of each cell face is
// recomputed from the cell index, and ties go to the lowest axis. t is where the ray enters the hit voxel.
struct RayHit {
    bool hit = false;
    double t = 0;
    uint32_t voxel[3] = { 0, 0, 0 };
};
static RayHit castRay(const Decoder& dec, uint32_t res, const double o[3], const double dir[3], double tmin, double tmax)
{
    RayHit h;
    h.t = tmax;
    const double R = res;
    double inv[3];
    for (int k = 0; k < 3; ++k)
        inv[k] = dir[k] != 0.0 ? 1.0 / dir[k] : 0.0;
    double t0 = tmin, t1 = tmax;
    int entryAxis = -1;
    for (int k = 0; k < 3; ++k) {
        if (dir[k] == 0.0) {
            if (o[k] < 0.0 || o[k] >= R)
                t0 = t1 + 1.0;
            continue;
        }
        double a = (0.0 - o[k]) * inv[k], b = (R - o[k]) * inv[k];
        if (a > b)
            std::swap(a, b);
        if (a > t0) {
            t0 = a;
            entryAxis = k;
        }
        if (b < t1)
            t1 = b;
    }
    if (dec.t.nodes[dec.t.rootLevel].empty() || !(t0 < t1))
        return h;
    int c[3];
    for (int k = 0; k < 3; ++k) {
        int ck = (int)std::floor(o[k] + t0 * dir[k]);
        if (k == entryAxis)
            ck = dir[k] > 0 ? 0 : (int)res - 1;
        c[k] = std::min(std::max(ck, 0), (int)res - 1);
    }
    double t = t0;
    for (uint64_t steps = 0; steps < 8ull * res + 64; ++steps) {
        if (dec.get((uint32_t)c[0], (uint32_t)c[1], (uint32_t)c[2])) {
            h.hit = true;
            h.t = t;
            for (int k = 0; k < 3; ++k)
                h.voxel[k] = (uint32_t)c[k];
            return h;
        }
        double tk[3];
        for (int k = 0; k < 3; ++k)
            tk[k] = dir[k] > 0.0 ? ((double)(c[k] + 1) - o[k]) * inv[k] : dir[k] < 0.0 ? ((double)c[k] - o[k]) * inv[k] : 1e300;
        int ax = 0;
        if (tk[1] < tk[ax])
            ax = 1;
        if (tk[2] < tk[ax])
            ax = 2;
        const double tn = std::max(tk[ax], t);
        if (tn >= t1)
            return h;
        c[ax] += dir[ax] > 0.0 ? 1 : -1;
        if (c[ax] < 0 || c[ax] >= (int)res)
            return h;
        t = tn;
    }
    return h;
}

} // namespace orc16

// ================================================================================================
// C API (ctypes), alongside tdag_oracle.cpp's. 0 = success; the message goes to orc16_last_error().
// ================================================================================================
static thread_local std::string g_err16;
static int fail16(const std::exception& e)
{
    g_err16 = e.what();
    return 1;
}

extern "C" {

const char* orc16_last_error() { return g_err16.c_str(); }

// Code lengths of the length-limited Huffman code (createLengthLimitedHuffmanCodeLengths).
int orc16_huffman_lengths(const uint64_t* freq, uint32_t n, uint32_t maxLen, uint32_t* outLengths)
{
    try {
        const auto l = orc16::lengthLimitedCodeLengths(std::vector<uint64_t>(freq, freq + n), maxLen);
        std::copy(l.begin(), l.end(), outLengths);
        return 0;
    } catch (const std::exception& e) {
        return fail16(e);
    }
}
// assignCodeWords, then (lsb != 0) convertHuffmanToLSB.
int orc16_huffman_codes(const uint32_t* lengths, uint32_t n, int lsb, uint64_t* outCodes, uint32_t* outBits)
{
    try {
        auto c = orc16::assignCodeWords(std::vector<uint32_t>(lengths, lengths + n));
        if (lsb)
            orc16::codesToLsb(c);
        for (uint32_t i = 0; i < n; ++i) {
            outCodes[i] = c[i].code;
            outBits[i] = c[i].bits;
        }
        return 0;
    } catch (const std::exception& e) {
        return fail16(e);
    }
}
// HuffmanDecodeLUT::decode for the given (LSB) code table.
int orc16_huffman_decode(const uint64_t* codes, const uint32_t* bits, uint32_t n, uint32_t key, uint32_t* outSymbol, uint32_t* outBits)
{
    try {
        std::vector<orc16::Code> c(n);
        for (uint32_t i = 0; i < n; ++i)
            c[i] = { codes[i], bits[i] };
        const orc16::DecodeLut lut(c);
        const auto [s, b] = lut.decode(key);
        *outSymbol = s;
        *outBits = b;
        return 0;
    } catch (const std::exception& e) {
        return fail16(e);
    }
}

// .tdag bytes (structure + config) -> .tdag16 bytes. levelStats (may be null): (root+1) x 10 u64 =
// numNodes, memoryInBytes, tableSize, uniquePointers, table[3], direct[3].
int orc16_encode(const uint8_t* tdag, uint64_t len, int pointerTables, int huffman, int tieMode, uint8_t** out, uint64_t* outLen,
    uint64_t* levelStats, uint32_t statsCapacity)
{
    try {
        orc16::Dag dag;
        orc16::DagConfig cfg;
        orc16::readTdag(tdag, len, dag, cfg);
        std::vector<orc16::LevelStats> st;
        const auto t = orc16::encode(std::move(dag), cfg, orc16::EncConfig { pointerTables != 0, huffman != 0 },
            tieMode == 1 ? orc16::kTieLibstdcxx : orc16::kTieCanonical, st);
        const auto bytes = orc16::serialize(t);
        *out = (uint8_t*)std::malloc(std::max<size_t>(bytes.size(), 1));
        orc16::check(*out != nullptr, "out of memory");
        std::memcpy(*out, bytes.data(), bytes.size());
        *outLen = bytes.size();
        if (levelStats)
            for (uint32_t l = 0; l < st.size() && l < statsCapacity; ++l) {
                const auto& s = st[l];
                const uint64_t row[10] = { s.numNodes, s.memoryInBytes, s.tableSize, s.uniquePointers, s.table[0], s.table[1], s.table[2],
                    s.direct[0], s.direct[1], s.direct[2] };
                std::memcpy(levelStats + 10 * l, row, sizeof(row));
            }
        return 0;
    } catch (const std::exception& e) {
        return fail16(e);
    }
}

// rays: n x 8 floats (origin xyz, direction xyz, tmin, tmax). outT: entry parameter of the hit voxel
// (tmax on a miss), outVoxel: n x 3, outHit: n.
int orc16_raycast(const uint8_t* buf, uint64_t len, const float* rays, uint64_t n, float* outT, uint32_t* outVoxel, uint8_t* outHit)
{
    try {
        const auto t = orc16::deserialize(buf, len);
        const orc16::Decoder d(t);
        std::string err;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            try {
                const float* r = rays + 8 * i;
                const double o[3] = { r[0], r[1], r[2] }, dir[3] = { r[3], r[4], r[5] };
                const auto h = orc16::castRay(d, t.resolution, o, dir, r[6], r[7]);
                outT[i] = (float)h.t;
                outHit[i] = h.hit ? 1 : 0;
                for (int k = 0; k < 3; ++k)
                    outVoxel[3 * i + k] = h.voxel[k];
            } catch (const std::exception& e) {
#pragma omp critical
                err = e.what();
            }
        }
        if (!err.empty())
            throw std::runtime_error(err);
        return 0;
    } catch (const std::exception& e) {
        return fail16(e);
    }
}

// Decode every voxel of a .tdag16 into dense[x + res*y + res*res*z] (res = the file's resolution).
int orc16_decode_dense(const uint8_t* buf, uint64_t len, uint8_t* dense, uint32_t res)
{
    try {
        const auto t = orc16::deserialize(buf, len);
        orc16::check(t.resolution == res, "resolution mismatch");
        const orc16::Decoder d(t);
        std::string err;
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t z = 0; z < (int64_t)res; ++z) {
            try {
                for (uint32_t y = 0; y < res; ++y)
                    for (uint32_t x = 0; x < res; ++x)
                        dense[x + (uint64_t)res * (y + (uint64_t)res * (uint64_t)z)] = d.get(x, y, (uint32_t)z) ? 1 : 0;
            } catch (const std::exception& e) {
#pragma omp critical
                err = e.what();
            }
        }
        if (!err.empty())
            throw std::runtime_error(err);
        return 0;
    } catch (const std::exception& e) {
        return fail16(e);
    }
}

} // extern "C"
