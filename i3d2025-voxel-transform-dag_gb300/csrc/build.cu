// build.cu — constructTransformDAG driver and the C ABI of libtdag.so.
//
// Driver restates constructTransformDAG (tools/lib/src/voxel/transform_dag.cpp:138-240):
//   1. hierarchical symmetry/permutation pass with midLevel = maxTranslationLevel + 1 (:144);
//   2. if translation is on: drop levels 2..maxTranslationLevel, re-seed the mid level with the
//      original nodes of its canonical entries (:147-160);
//   3. for level = maxTranslationLevel .. 2 (:165-238): collect the items referenced by the level
//      above in ascending order (:177-192), flatten them into dense grids (FlatGridGenerator,
//      transform_dag.cpp:44-116, 417-441), run the matcher, keep the unique items (:208-221) and
//      rewrite the parents' child pointers through the mapping (:224-233; the lower_bound lookup is
//      a rank array here).
#include <array>
#include <chrono>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "internal.cuh"

namespace tdag {

std::atomic<uint64_t> g_kernelLaunches { 0 };

// ------------------------------------------------------------------------------------------------
// Transform tables
// ------------------------------------------------------------------------------------------------
const TransformTables& hostTables()
{
    static TransformTables t = [] {
        TransformTables tt {};
        auto perm = [](uint32_t id, int k) { return (permBitsOf(id) >> (2 * k)) & 3; };
        auto applyPerm = [&](uint32_t bits3, uint32_t id) {
            uint32_t o = 0;
            for (int k = 0; k < 3; ++k)
                o |= ((bits3 >> perm(id, k)) & 1u) << k;
            return o;
        };
        for (uint32_t a = 0; a < 48; ++a) {
            const uint32_t sa = a & 7, pa = a >> 3;
            for (uint32_t i = 0; i < 8; ++i)
                tt.pos[a][i] = (uint8_t)(applyPerm(i, pa) ^ sa);
            for (uint32_t i = 0; i < 8; ++i)
                tt.invPos[a][tt.pos[a][i]] = (uint8_t)i;
            for (uint32_t b = 0; b < 48; ++b) {
                const uint32_t sb = b & 7, pb = b >> 3;
                // (a∘b)(v) = Pa(Pb(v)) ^ Pa(Sb) ^ Sa ; (Pa∘Pb)[k] = pb[pa[k]]
                uint32_t pc = 0;
                for (int k = 0; k < 3; ++k)
                    pc |= perm(pb, (int)perm(pa, k)) << (2 * k);
                const uint32_t sc = applyPerm(sb, pa) ^ sa;
                tt.compose[a][b] = (uint8_t)(sc | (permIdOfBits(pc) << 3));
            }
            for (uint32_t byte = 0; byte < 256; ++byte) {
                uint32_t o = 0;
                for (uint32_t i = 0; i < 8; ++i)
                    if ((byte >> i) & 1)
                        o |= 1u << tt.pos[a][i];
                tt.byteMap[a][byte] = (uint8_t)o;
            }
        }
        for (uint32_t a = 0; a < 48; ++a)
            for (uint32_t b = 0; b < 48; ++b)
                if (tt.compose[a][b] == 0)
                    tt.inverse[a] = (uint8_t)b;
        return tt;
    }();
    return t;
}

uint32_t Context::takeStatus(uint32_t* aux)
{
    readToHost({ { hostStatus, status, 16 } }, stream);
    const uint32_t code = hostStatus[0];
    if (aux)
        *aux = hostStatus[1];
    if (code != 0) {
        TDAG_CUDA(cudaMemsetAsync(status, 0, 16, stream));
        syncHost(stream);
    }
    return code;
}

void Context::checkStatus(const std::string& where)
{
    uint32_t aux = 0;
    const uint32_t code = takeStatus(&aux);
    if (code != 0)
        throw Error((int)code, where + ": device reported error " + std::to_string(code) + " (aux " + std::to_string(aux) + ")");
}

uint64_t Context::classTableCapacity(uint64_t n) const
{
    const uint64_t load = tuning.class_table_load_percent ? tuning.class_table_load_percent : 50;
    uint64_t cap = 1;
    const uint64_t want = n * 100 / load + 16;
    while (cap < want)
        cap <<= 1;
    return cap;
}

namespace {
std::mutex g_streamMutex;
std::unordered_map<cudaStream_t, std::weak_ptr<StreamState>> g_streams;
}

StreamState::~StreamState()
{
    if (stream)
        cudaStreamDestroy(stream);
}

std::shared_ptr<StreamState> streamStateOf(cudaStream_t stream)
{
    // one cached entry per host thread spares the lock on the hot path (many buffers per build)
    thread_local cudaStream_t lastStream = nullptr;
    thread_local std::weak_ptr<StreamState> lastState;
    if (stream && stream == lastStream)
        if (auto st = lastState.lock())
            return st;
    std::lock_guard<std::mutex> lock(g_streamMutex);
    const auto it = g_streams.find(stream);
    if (it == g_streams.end())
        return nullptr;
    auto st = it->second.lock();
    lastStream = stream;
    lastState = st;
    return st;
}

std::shared_ptr<StreamState> registerStream(cudaStream_t stream, uint64_t limit)
{
    auto st = std::make_shared<StreamState>();
    st->stream = stream;
    st->limit = limit;
    std::lock_guard<std::mutex> lock(g_streamMutex);
    g_streams[stream] = st;
    return st;
}

void unregisterStream(cudaStream_t stream)
{
    std::lock_guard<std::mutex> lock(g_streamMutex);
    g_streams.erase(stream);
}

void chargeBudget(StreamState& b, uint64_t bytes)
{
    const uint64_t before = b.used.fetch_add(bytes);
    if (before + bytes > b.limit) {
        b.used -= bytes;
        throw Error(TDAG_ERR_OOM, "device memory limit of the context reached: " + std::to_string(before) + " B held, " + std::to_string(bytes) +
                " B requested, limit " + std::to_string(b.limit) + " B");
    }
}

namespace {

// ------------------------------------------------------------------------------------------------
// Kernels of the driver
// ------------------------------------------------------------------------------------------------
struct LevelPtrs {
    const uint32_t* nodes[6]; // levels 0..5 (3..5 used)
    const uint64_t* leaves;
};

// Dense grid of a level-L item: thread per output word; 16 x-runs of 4 voxels per word.
template <int L>
__global__ void flattenKernel(LevelPtrs lp, const uint32_t* __restrict__ indices, uint32_t n, uint64_t* __restrict__ grids, uint32_t* status)
{
    constexpr int R = 1 << L;
    constexpr int W = R * R * R / 64;
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)n * W)
        return;
    const uint32_t item = (uint32_t)(gid / W), w = (uint32_t)(gid % W);
    const uint32_t orig = indices[item];
    // A word's 64 bits touch at most four 4^3 leaves (R = 16: the four x-blocks of four rows; R = 8:
    // 2 x 2 blocks in x and y; R = 4: one). Each is fetched once, and the walks are independent, so
    // their loads overlap.
    auto slotOf = [](uint32_t x, uint32_t y) -> uint32_t { return R == 16 ? (x >> 2) & 3u : (R == 8 ? ((x >> 2) & 1u) | (((y >> 2) & 1u) << 1) : 0u); };
    uint64_t leaf[4] = { 0, 0, 0, 0 };
#pragma unroll
    for (uint32_t q = 0; q < 4; ++q) {
        // the first bit group of the word that falls into slot q
        uint32_t g0 = 16;
#pragma unroll
        for (uint32_t g = 0; g < 16; ++g) {
            const uint32_t b = 64 * w + 4 * g;
            if (g0 == 16 && slotOf(b % R, (b / R) % R) == q)
                g0 = g;
        }
        if (g0 == 16)
            continue;
        const uint32_t b = 64 * w + 4 * g0;
        const uint32_t x = b % R, y = (b / R) % R, z = b / (R * R);
        uint32_t idx = orig;
        bool empty = false;
        for (int lvl = L; lvl > 2; --lvl) {
            const uint32_t c = ((x >> (lvl - 1)) & 1) | (((y >> (lvl - 1)) & 1) << 1) | (((z >> (lvl - 1)) & 1) << 2);
            idx = lp.nodes[lvl][(size_t)idx * 8 + c];
            if (idx == kEmpty32) {
                empty = true;
                break;
            }
        }
        leaf[q] = empty ? 0 : lp.leaves[idx];
    }
    uint64_t word = 0;
#pragma unroll
    for (uint32_t g = 0; g < 16; ++g) {
        const uint32_t b = 64 * w + 4 * g;
        const uint32_t x = b % R, y = (b / R) % R, z = b / (R * R);
        const uint32_t ly = y & 3, lz = z & 3;
        const uint32_t base = ((ly & 1) << 1) | ((lz & 1) << 2) | ((ly >> 1) << 4) | ((lz >> 1) << 5);
        const uint64_t m = leaf[slotOf(x, y)];
        const uint64_t row = ((m >> base) & 1) | (((m >> (base + 1)) & 1) << 1) | (((m >> (base + 8)) & 1) << 2) | (((m >> (base + 9)) & 1) << 3);
        word |= row << (4 * g);
    }
    grids[gid] = word;
}

__global__ void markReferencedKernel(const uint64_t* __restrict__ parents, uint64_t count8, uint32_t* __restrict__ ref, uint64_t numItems, uint32_t* status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count8)
        return;
    const uint64_t c = parents[i];
    if (c == tpSentinel())
        return;
    const uint64_t p = tpPtr(c);
    if (p >= numItems) {
        setDeviceError(status, TDAG_ERR_CORRUPT, 300);
        return;
    }
    ref[p] = 1;
}

__global__ void rankKernel(const uint32_t* __restrict__ indices, uint32_t n, uint32_t* __restrict__ rankOf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        rankOf[indices[i]] = i;
}

__global__ void remapParentsKernel(uint64_t* __restrict__ parents, uint64_t count8, const uint32_t* __restrict__ rankOf, const uint64_t* __restrict__ mapping)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count8)
        return;
    const uint64_t c = parents[i];
    if (c == tpSentinel())
        return;
    parents[i] = mapping[rankOf[tpPtr(c)]];
}

// Output nodes of a translation level: original nodes of the kept items, children as TransformPointers.
__global__ void emitOriginalNodesKernel(const uint32_t* __restrict__ nodes, const uint32_t* __restrict__ indices, const uint32_t* __restrict__ kept, uint32_t u,
    uint64_t* __restrict__ out)
{
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)u * 8)
        return;
    const uint32_t h = (uint32_t)(gid >> 3), k = (uint32_t)(gid & 7);
    const uint32_t orig = kept ? indices[kept[h]] : indices[h];
    const uint32_t c = nodes[(size_t)orig * 8 + k];
    out[gid] = (c == kEmpty32) ? tpSentinel() : tpCreate(c, 0, 0);
}

__global__ void emitOriginalLeavesKernel(const uint64_t* __restrict__ leaves, const uint32_t* __restrict__ indices, const uint32_t* __restrict__ kept, uint32_t u,
    uint64_t* __restrict__ out)
{
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < u)
        out[h] = leaves[indices[kept[h]]];
}

__global__ void validateChildrenKernel(const uint32_t* __restrict__ nodes, uint64_t count8, uint64_t childCount, uint32_t level, uint32_t* status)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count8)
        return;
    const uint32_t c = nodes[i];
    if (c != kEmpty32 && c >= childCount)
        setDeviceError(status, TDAG_ERR_CORRUPT, level);
}

__global__ void gatherU32Kernel(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx, uint32_t n, uint32_t* __restrict__ dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        dst[i] = src[idx[i]];
}

struct DeviceResult {
    std::vector<DevBuf<uint64_t>> levels;
    DevBuf<uint64_t> leaves;
    std::vector<std::vector<uint64_t>> off; // per level (2 = leaves): first output item of each grid
};

static DevBuf<uint32_t> uploadU32(const std::vector<uint64_t>& v, cudaStream_t s)
{
    std::vector<uint32_t> h(v.begin(), v.end());
    DevBuf<uint32_t> d(h.size(), s);
    uploadToDevice(d.get(), h.data(), h.size() * 4, s);
    syncHost(s);
    return d;
}

// Learned-proposal hook of a build (tdag_build_device_proposed): picks each level's searching sources.
struct ProposalHook {
    tdag_proposal_fn fn = nullptr;
    void* user = nullptr;
};

template <int L>
static void translationLevel(Context& ctx, const DeviceSvdag& in, DeviceResult& out, const tdag_config& cfg, tdag_stats* stats, const ProposalHook& hook)
{
    cudaStream_t s = ctx.stream;
    const uint64_t numItems = (L == 2) ? in.leafCount : in.nodeCounts[L];
    DevBuf<uint64_t>& parents = out.levels[L + 1];
    const uint64_t count8 = parents.n;
    DevBuf<uint32_t> ref(numItems, s);
    if (numItems)
        TDAG_CUDA(cudaMemsetAsync(ref.get(), 0, numItems * 4, s));
    if (count8) {
        markReferencedKernel<<<gridFor(count8, 256), 256, 0, s>>>(parents.get(), count8, ref.get(), numItems, ctx.status);
        TDAG_LAUNCHED();
    }
    DevBuf<uint32_t> indices(numItems, s);
    const uint32_t m = compactFlags(ref.get(), indices.get(), numItems, s);
    ref.release();
    ctx.checkStatus("referenced items");
    constexpr int R = 1 << L;
    constexpr int W = R * R * R / 64;
    DevBuf<uint64_t> grids((size_t)m * W, s);
    LevelPtrs lp {};
    for (int l = 3; l <= 5 && l <= (int)in.rootLevel; ++l)
        lp.nodes[l] = in.nodes[l];
    lp.leaves = in.leaves;
    if (m) {
        flattenKernel<L><<<gridFor((size_t)m * W, 256), 256, 0, s>>>(lp, indices.get(), m, grids.get(), ctx.status);
        TDAG_LAUNCHED();
    }
    // batch: grid of every matched item (items stay grid-contiguous: indices are ascending)
    Segments sg;
    DevBuf<uint32_t> gridOfM, offM;
    if (in.numGrids > 1) {
        sg.numGrids = in.numGrids;
        gridOfM = DevBuf<uint32_t>(m, s);
        if (m) {
            gatherU32Kernel<<<gridFor(m, 256), 256, 0, s>>>(in.gridOf[L], indices.get(), m, gridOfM.get());
            TDAG_LAUNCHED();
        }
        sg.off = countPerGrid(in.gridOf[L], indices.get(), m, in.numGrids, s);
        offM = uploadU32(sg.off, s);
        sg.gridOf = gridOfM.get();
        sg.offDev = offM.get();
    }
    tdag_level_stats* ls = stats ? &stats->translation[L] : nullptr;
    DevBuf<uint32_t> proposed;
    uint32_t numProposed = 0;
    if (hook.fn && m) {
        TDAG_CHECK(in.numGrids == 1, TDAG_ERR_ARG, "proposal hooks apply to single-grid builds");
        proposed = DevBuf<uint32_t>(m, s);
        TDAG_CUDA(cudaStreamSynchronize(s)); // the hook reads the grids from its own stream
        const int rc = hook.fn(hook.user, L, grids.get(), m, proposed.get(), &numProposed);
        TDAG_CHECK(rc == 0, TDAG_ERR_ARG, "proposal function failed");
        TDAG_CHECK(numProposed <= m, TDAG_ERR_ARG, "proposal function returned more sources than items");
    }
    MatchOutput mo = runMatcher(ctx, L, grids.get(), m, cfg, ls, &sg, hook.fn ? proposed.get() : nullptr, numProposed);
    grids.release();
    out.off[L] = mo.uniqueOff.empty() ? std::vector<uint64_t>(in.numGrids + 1, 0) : mo.uniqueOff;
    const uint32_t u = mo.numUnique;
    if (L == 2) {
        out.leaves = DevBuf<uint64_t>(u, s);
        if (u) {
            emitOriginalLeavesKernel<<<gridFor(u, 256), 256, 0, s>>>(in.leaves, indices.get(), mo.uniques.get(), u, out.leaves.get());
            TDAG_LAUNCHED();
        }
    } else {
        out.levels[L] = DevBuf<uint64_t>((size_t)u * 8, s);
        if (u) {
            emitOriginalNodesKernel<<<gridFor((size_t)u * 8, 256), 256, 0, s>>>(in.nodes[L], indices.get(), mo.uniques.get(), u, out.levels[L].get());
            TDAG_LAUNCHED();
        }
    }
    if (count8 && m) {
        DevBuf<uint32_t> rankOf(numItems, s);
        rankKernel<<<gridFor(m, 256), 256, 0, s>>>(indices.get(), m, rankOf.get());
        TDAG_LAUNCHED();
        remapParentsKernel<<<gridFor(count8, 256), 256, 0, s>>>(parents.get(), count8, rankOf.get(), mo.mapping.get());
        TDAG_LAUNCHED();
    }
}

static void validateInput(Context& ctx, const DeviceSvdag& in)
{
    cudaStream_t s = ctx.stream;
    for (uint32_t level = 3; level <= in.rootLevel; ++level) {
        const uint64_t childCount = (level == 3) ? in.leafCount : in.nodeCounts[level - 1];
        const uint64_t count8 = in.nodeCounts[level] * 8;
        if (count8) {
            validateChildrenKernel<<<gridFor(count8, 256), 256, 0, s>>>(in.nodes[level], count8, childCount, level, ctx.status);
            TDAG_LAUNCHED();
        }
    }
    ctx.checkStatus("input validation");
}

static DeviceResult buildDevice(Context& ctx, const DeviceSvdag& in, const tdag_config& cfg, tdag_stats* stats, const ProposalHook& hook = ProposalHook {})
{
    TDAG_CHECK(in.rootLevel >= 2 && in.rootLevel < TDAG_MAX_LEVELS, TDAG_ERR_ARG, "root_level out of range");
    TDAG_CHECK(in.numGrids > 1 || in.resolution == (1u << in.rootLevel), TDAG_ERR_ARG, "resolution must equal 1 << root_level");
    if (cfg.translation) {
        TDAG_CHECK(cfg.max_translation_level >= 2 && cfg.max_translation_level <= 4, TDAG_ERR_ARG, "max_translation_level must be 2..4 when translation is on");
        TDAG_CHECK(in.rootLevel >= cfg.max_translation_level + 1, TDAG_ERR_ARG, "root_level must exceed max_translation_level");
    }
    for (uint32_t l = 3; l <= in.rootLevel; ++l)
        TDAG_CHECK(in.nodeCounts[l] < (1ull << 31), TDAG_ERR_ARG, "level too large");
    TDAG_CHECK(in.leafCount < (1ull << 31), TDAG_ERR_ARG, "too many leaves");
    validateInput(ctx, in);
    cudaStream_t s = ctx.stream;
    ctx.tableRegrows = 0;
    const uint64_t launches0 = g_kernelLaunches.load();
    // stage timing (not while a batch graph captures the build: its events would not complete)
    const bool timed = !replaying();
    if (timed)
        TDAG_CUDA(cudaEventRecord(ctx.ev[2], s));
    const uint32_t midLevel = cfg.max_translation_level + 1;
    HierOutput h = runHierarchical(ctx, in, cfg, cfg.translation ? midLevel : 0xFFFFFFFFu, stats);
    if (timed)
        TDAG_CUDA(cudaEventRecord(ctx.ev[3], s));
    DeviceResult out;
    out.levels.resize(in.rootLevel + 1);
    out.off = h.handleOff;
    for (uint32_t l = 3; l <= in.rootLevel; ++l)
        out.levels[l] = std::move(h.levels[l]);
    out.leaves = std::move(h.leaves);
    if (cfg.translation) {
        out.leaves.release();
        for (uint32_t l = 3; l <= cfg.max_translation_level; ++l)
            out.levels[l].release();
        const uint32_t u = (uint32_t)(out.levels[midLevel].n / 8);
        TDAG_CHECK(h.midInv.n == u, TDAG_ERR_CORRUPT, "mid level size mismatch");
        if (u) {
            emitOriginalNodesKernel<<<gridFor((size_t)u * 8, 256), 256, 0, s>>>(in.nodes[midLevel], h.midInv.get(), nullptr, u, out.levels[midLevel].get());
            TDAG_LAUNCHED();
        }
        h.midInv.release();
        for (int L = (int)cfg.max_translation_level; L >= 2; --L) {
            if (L == 4)
                translationLevel<4>(ctx, in, out, cfg, stats, hook);
            else if (L == 3)
                translationLevel<3>(ctx, in, out, cfg, stats, hook);
            else
                translationLevel<2>(ctx, in, out, cfg, stats, hook);
        }
    }
    if (timed)
        TDAG_CUDA(cudaEventRecord(ctx.ev[4], s));
    ctx.checkStatus("build");
    if (stats && timed) {
        TDAG_CUDA(cudaEventElapsedTime(&stats->hierarchical_ms, ctx.ev[2], ctx.ev[3]));
        TDAG_CUDA(cudaEventElapsedTime(&stats->translation_ms, ctx.ev[3], ctx.ev[4]));
        TDAG_CUDA(cudaEventElapsedTime(&stats->total_ms, ctx.ev[2], ctx.ev[4]));
        stats->kernel_launches = g_kernelLaunches.load() - launches0;
        stats->table_regrows = ctx.tableRegrows;
    }
    return out;
}

// Child indices of a concatenated level: add the grid's first index at the level below.
__global__ void offsetChildrenKernel(uint32_t* __restrict__ nodes, uint64_t count8, const uint32_t* __restrict__ gridOf, const uint32_t* __restrict__ childOff)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count8)
        return;
    const uint32_t c = nodes[i];
    if (c != kEmpty32)
        nodes[i] = c + childOff[gridOf[i >> 3]];
}

// Device storage of a batch of SVDAGs concatenated level by level.
struct BatchInput {
    std::vector<DevBuf<uint32_t>> nodes, gridOf, offDev;
    DevBuf<uint64_t> leaves;
    DeviceSvdag view;
};

static void concatBatch(Context& ctx, const tdag_svdag_view* v, uint32_t count, bool hostInput, BatchInput& b)
{
    cudaStream_t s = ctx.stream;
    const cudaMemcpyKind kind = hostInput ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    uint32_t maxRoot = 0;
    for (uint32_t g = 0; g < count; ++g)
        maxRoot = std::max(maxRoot, v[g].root_level);
    DeviceSvdag& d = b.view;
    d.numGrids = count;
    d.rootLevel = maxRoot;
    d.resolution = 1u << maxRoot;
    b.nodes.resize(maxRoot + 1);
    b.gridOf.resize(maxRoot + 1);
    b.offDev.resize(maxRoot + 1);
    // offsets
    for (uint32_t l = 2; l <= maxRoot; ++l) {
        auto& off = d.segOff[l];
        off.assign(count + 1, 0);
        for (uint32_t g = 0; g < count; ++g) {
            const uint64_t c = (l == 2) ? v[g].leaf_count : (l <= v[g].root_level ? v[g].node_counts[l] : 0);
            off[g + 1] = off[g] + c;
        }
        TDAG_CHECK(off[count] < (1ull << 31), TDAG_ERR_ARG, "batch level too large");
        b.offDev[l] = uploadU32(off, s);
        b.gridOf[l] = DevBuf<uint32_t>(off[count], s);
        segmentIds(b.offDev[l].get(), count, off[count], b.gridOf[l].get(), s);
        d.gridOf[l] = b.gridOf[l].get();
    }
    // leaves
    b.leaves = DevBuf<uint64_t>(d.segOff[2][count], s);
    for (uint32_t g = 0; g < count; ++g)
        if (v[g].leaf_count)
            TDAG_CUDA(cudaMemcpyAsync(b.leaves.get() + d.segOff[2][g], v[g].leaves, v[g].leaf_count * 8, kind, s));
    d.leaves = b.leaves.get();
    d.leafCount = d.segOff[2][count];
    // nodes, children rebased onto the concatenated level below
    for (uint32_t l = 3; l <= maxRoot; ++l) {
        const uint64_t total = d.segOff[l][count];
        b.nodes[l] = DevBuf<uint32_t>(total * 8, s);
        for (uint32_t g = 0; g < count; ++g) {
            const uint64_t c = d.segOff[l][g + 1] - d.segOff[l][g];
            if (c)
                TDAG_CUDA(cudaMemcpyAsync(b.nodes[l].get() + d.segOff[l][g] * 8, v[g].nodes[l], c * 32, kind, s));
        }
        if (total) {
            offsetChildrenKernel<<<gridFor(total * 8, 256), 256, 0, s>>>(b.nodes[l].get(), total * 8, b.gridOf[l].get(), b.offDev[l - 1].get());
            TDAG_LAUNCHED();
        }
        d.nodes[l] = b.nodes[l].get();
        d.nodeCounts[l] = total;
    }
}

} // namespace
} // namespace tdag

// ================================================================================================
// C ABI
// ================================================================================================
using namespace tdag;

struct tdag_ctx {
    Context c;
};

namespace {
thread_local std::string g_lastError;

int fail(int code, const std::string& msg)
{
    g_lastError = msg;
    return code;
}

template <typename F>
int guarded(F&& f)
{
    try {
        f();
        return TDAG_OK;
    } catch (const Error& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(TDAG_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(TDAG_ERR_ARG, e.what());
    }
}

struct Upload {
    std::vector<DevBuf<uint32_t>> nodes;
    DevBuf<uint64_t> leaves;
};

DeviceSvdag viewToDevice(const tdag_svdag_view* v)
{
    DeviceSvdag d;
    d.resolution = v->resolution;
    d.rootLevel = v->root_level;
    for (uint32_t l = 0; l < TDAG_MAX_LEVELS; ++l) {
        d.nodes[l] = v->nodes[l];
        d.nodeCounts[l] = v->node_counts[l];
    }
    d.leaves = v->leaves;
    d.leafCount = v->leaf_count;
    return d;
}

void checkView(const tdag_svdag_view* v)
{
    TDAG_CHECK(v != nullptr, TDAG_ERR_ARG, "null input view");
    TDAG_CHECK(v->root_level >= 2 && v->root_level < TDAG_MAX_LEVELS, TDAG_ERR_ARG, "root_level out of range");
    TDAG_CHECK(v->structure_type == 1, TDAG_ERR_ARG, "constructTransformDAG requires a DAG (structure_type == 1)");
    for (uint32_t l = 3; l <= v->root_level; ++l)
        TDAG_CHECK(v->node_counts[l] == 0 || v->nodes[l] != nullptr, TDAG_ERR_ARG, "null node array with non-zero count");
    TDAG_CHECK(v->leaf_count == 0 || v->leaves != nullptr, TDAG_ERR_ARG, "null leaf array with non-zero count");
    TDAG_CHECK(v->node_counts[v->root_level] <= 1, TDAG_ERR_ARG, "root level must hold at most one node");
}

tdag_result* newResult(uint32_t res, uint32_t root, bool onDevice)
{
    auto* r = new tdag_result;
    std::memset(r, 0, sizeof(*r));
    r->resolution = res;
    r->root_level = root;
    r->structure_type = 0;
    r->on_device = onDevice ? 1u : 0u;
    return r;
}

} // namespace

// Shared with the other C-ABI translation units.
Context& ctxOf(tdag_ctx* c) { return c->c; }
int guardedCall(const std::function<void()>& f) { return guarded(f); }
int failWith(int code, const char* msg) { return fail(code, msg); }

extern "C" {

const char* tdag_version(void) { return "tdag-gb300 0.1 (sm_103a)"; }
const char* tdag_last_error_message(void) { return g_lastError.c_str(); }

int tdag_ctx_create(int device, const tdag_tuning* tuning, tdag_ctx** out)
{
    if (!out)
        return fail(TDAG_ERR_ARG, "null out pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(TDAG_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count)
        return fail(TDAG_ERR_ARG, "device index out of range");
    auto holder = std::make_unique<tdag_ctx>();
    const int rc = guarded([&] {
        Context& c = holder->c;
        c.device = device;
        TDAG_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop;
        TDAG_CUDA(cudaGetDeviceProperties(&prop, device));
        c.numSMs = prop.multiProcessorCount;
        if (tuning)
            c.tuning = *tuning;
        TDAG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        c.streamState = registerStream(c.stream, c.tuning.device_memory_limit);
        cudaMemPool_t pool;
        TDAG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
        uint64_t threshold = ~0ull;
        TDAG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold));
        TDAG_CUDA(cudaMalloc(&c.tables, sizeof(TransformTables)));
        TDAG_CUDA(cudaMemcpy(c.tables, &hostTables(), sizeof(TransformTables), cudaMemcpyHostToDevice));
        TDAG_CUDA(cudaMalloc(&c.status, 16));
        TDAG_CUDA(cudaMemset(c.status, 0, 16));
        TDAG_CUDA(cudaMallocHost(&c.hostStatus, 16));
        for (auto& e : c.ev)
            TDAG_CUDA(cudaEventCreate(&e));
        // Probe that the kernels load on this device (fails loudly on a non-sm_103 GPU).
        cudaFuncAttributes fa;
        TDAG_CUDA(cudaFuncGetAttributes(&fa, flattenKernel<2>));
        prepareNoAlloc(c);
    });
    if (rc != TDAG_OK) {
        tdag_ctx_destroy(holder.release());
        return rc;
    }
    *out = holder.release();
    return TDAG_OK;
}

int tdag_ctx_destroy(tdag_ctx* ctx)
{
    if (!ctx)
        return TDAG_OK;
    Context& c = ctx->c;
    cudaSetDevice(c.device);
    if (c.stream)
        cudaStreamSynchronize(c.stream);
    for (auto& e : c.ev)
        if (e)
            cudaEventDestroy(e);
    if (c.tables)
        cudaFree(c.tables);
    if (c.status)
        cudaFree(c.status);
    if (c.hostStatus)
        cudaFreeHost(c.hostStatus);
    if (c.stage)
        cudaFreeHost(c.stage);
    if (c.stream) {
        // the stream goes with the last buffer allocated on it (results may outlive the context)
        unregisterStream(c.stream);
        if (!c.streamState)
            cudaStreamDestroy(c.stream);
        c.streamState.reset();
    }
    delete ctx;
    return TDAG_OK;
}

int tdag_ctx_stream(tdag_ctx* ctx, void** out)
{
    if (!ctx || !out)
        return fail(TDAG_ERR_ARG, "null argument");
    *out = (void*)ctx->c.stream;
    return TDAG_OK;
}

} // extern "C"

namespace tdag {
void requireDeviceAccessible(Context& c, const void* p, const char* what)
{
    if (!p)
        return;
    cudaPointerAttributes a {};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        throw Error(TDAG_ERR_ARG, std::string(what) + ": not a pointer the device can use");
    }
    bool ok = false;
    switch (a.type) {
    case cudaMemoryTypeDevice:
        ok = a.device == c.device;
        break;
    case cudaMemoryTypeManaged:
        ok = true;
        break;
    case cudaMemoryTypeHost:
        ok = a.devicePointer == p;
        break;
    default: // unregistered (pageable) host memory
        if (c.pageableAccess < 0) {
            int v = 0;
            TDAG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, c.device));
            c.pageableAccess = v;
        }
        ok = c.pageableAccess == 1;
        break;
    }
    TDAG_CHECK(ok, TDAG_ERR_ARG, std::string(what) + ": expected memory the context's device can read (a device pointer)");
}

void requireDeviceView(Context& c, const tdag_svdag_view& v)
{
    for (uint32_t l = 3; l <= v.root_level && l < TDAG_MAX_LEVELS; ++l)
        if (v.node_counts[l])
            requireDeviceAccessible(c, v.nodes[l], "tdag_svdag_view.nodes");
    if (v.leaf_count)
        requireDeviceAccessible(c, v.leaves, "tdag_svdag_view.leaves");
}

// Copies device arrays into host (pageable) arrays through the context's pinned staging buffer. A
// D2H copy into pinned memory runs at link speed; one straight into freshly allocated pageable pages
// goes page by page through the driver and took ~20 ms for a 32 MB result. The host copies out of
// the stage run on a few threads for large results.
// Pinned host blocks for the arrays of host results (tdag_build): the device writes them directly,
// with no staging copy, and tdag_result_free returns them here. Blocks are powers of two from 64 KiB;
// freed ones are kept for reuse up to 2 GiB in all (past that they are released). Process-wide, as
// results outlive their contexts; deliberately never destroyed (results may be freed at exit).
namespace {
struct HostPool {
    std::mutex m;
    std::unordered_map<void*, size_t> owned; // block -> capacity, for every block of the pool
    std::unordered_multimap<size_t, void*> spare; // capacity -> cached free block
    size_t spareBytes = 0;
    static constexpr size_t kSpareLimit = size_t(2) << 30;
};
HostPool& hostPool()
{
    static HostPool* pool = new HostPool;
    return *pool;
}
} // namespace

void* hostResultAlloc(size_t bytes)
{
    if (bytes == 0)
        return std::malloc(1);
    size_t cap = size_t(64) << 10;
    while (cap < bytes)
        cap <<= 1;
    HostPool& P = hostPool();
    {
        std::lock_guard<std::mutex> lk(P.m);
        auto it = P.spare.find(cap);
        if (it != P.spare.end()) {
            void* p = it->second;
            P.spare.erase(it);
            P.spareBytes -= cap;
            return p;
        }
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, cap, cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        throw Error(TDAG_ERR_OOM, "pinned host allocation failed");
    }
    std::lock_guard<std::mutex> lk(P.m);
    P.owned[p] = cap;
    return p;
}

void hostResultFree(void* p)
{
    if (!p)
        return;
    HostPool& P = hostPool();
    {
        std::lock_guard<std::mutex> lk(P.m);
        auto it = P.owned.find(p);
        if (it == P.owned.end()) {
            std::free(p); // a plain allocation (empty arrays)
            return;
        }
        if (P.spareBytes + it->second <= HostPool::kSpareLimit) {
            P.spare.emplace(it->second, p);
            P.spareBytes += it->second;
            return;
        }
        P.owned.erase(it);
    }
    cudaFreeHost(p);
}

void downloadStaged(Context& c, const std::vector<Download>& items)
{
    size_t total = 0;
    for (const auto& d : items)
        total += (d.bytes + 255) & ~(size_t)255;
    if (total == 0)
        return;
    if (total > c.stageBytes) {
        if (c.stage)
            TDAG_CUDA(cudaFreeHost(c.stage));
        c.stage = nullptr;
        c.stageBytes = 0;
        const size_t want = total + total / 4;
        TDAG_CUDA(cudaMallocHost(&c.stage, want));
        c.stageBytes = want;
    }
    size_t off = 0;
    for (const auto& d : items) {
        if (d.bytes)
            TDAG_CUDA(cudaMemcpyAsync(static_cast<char*>(c.stage) + off, d.src, d.bytes, cudaMemcpyDeviceToHost, c.stream));
        off += (d.bytes + 255) & ~(size_t)255;
    }
    TDAG_CUDA(cudaStreamSynchronize(c.stream));
    // host copies, split into chunks over up to 8 threads
    struct Piece {
        char* dst;
        const char* src;
        size_t bytes;
    };
    std::vector<Piece> pieces;
    constexpr size_t kChunk = 4u << 20;
    off = 0;
    for (const auto& d : items) {
        for (size_t o = 0; o < d.bytes; o += kChunk)
            pieces.push_back({ static_cast<char*>(d.dst) + o, static_cast<const char*>(c.stage) + off + o, std::min(kChunk, d.bytes - o) });
        off += (d.bytes + 255) & ~(size_t)255;
    }
    const unsigned workers = (unsigned)std::min<size_t>({ pieces.size(), (size_t)8, (size_t)std::max(1u, std::thread::hardware_concurrency()) });
    auto work = [&](unsigned w) {
        for (size_t i = w; i < pieces.size(); i += workers)
            std::memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes);
    };
    std::vector<std::thread> threads;
    for (unsigned w = 1; w < workers; ++w)
        threads.emplace_back(work, w);
    work(0);
    for (auto& t : threads)
        t.join();
}
} // namespace tdag

extern "C" {

int tdag_build_device(tdag_ctx* ctx, const tdag_svdag_view* in, const tdag_config* cfg, tdag_result** out)
{
    if (!ctx || !cfg || !out)
        return fail(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guarded([&] {
        checkView(in);
        Context& c = ctx->c;
        TDAG_CUDA(cudaSetDevice(c.device));
        requireDeviceView(c, *in);
        std::unique_ptr<tdag_result> r(newResult(in->resolution, in->root_level, true));
        DeviceResult dr = buildDevice(c, viewToDevice(in), *cfg, &r->stats);
        // hand ownership of the device buffers to the result (freed by tdag_result_free)
        TDAG_CUDA(cudaStreamSynchronize(c.stream));
        for (uint32_t l = 3; l <= in->root_level; ++l) {
            r->node_counts[l] = dr.levels[l].n / 8;
            r->nodes[l] = dr.levels[l].p;
            dr.levels[l].p = nullptr;
        }
        r->leaf_count = dr.leaves.n;
        r->leaves = dr.leaves.p;
        dr.leaves.p = nullptr;
        *out = r.release();
    });
}

int tdag_build_device_proposed(tdag_ctx* ctx, const tdag_svdag_view* in, const tdag_config* cfg, tdag_proposal_fn fn, void* user, tdag_result** out)
{
    if (!ctx || !cfg || !out || !fn)
        return fail(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guarded([&] {
        checkView(in);
        Context& c = ctx->c;
        TDAG_CUDA(cudaSetDevice(c.device));
        requireDeviceView(c, *in);
        std::unique_ptr<tdag_result> r(newResult(in->resolution, in->root_level, true));
        DeviceResult dr = buildDevice(c, viewToDevice(in), *cfg, &r->stats, ProposalHook { fn, user });
        TDAG_CUDA(cudaStreamSynchronize(c.stream));
        for (uint32_t l = 3; l <= in->root_level; ++l) {
            r->node_counts[l] = dr.levels[l].n / 8;
            r->nodes[l] = dr.levels[l].p;
            dr.levels[l].p = nullptr;
        }
        r->leaf_count = dr.leaves.n;
        r->leaves = dr.leaves.p;
        dr.leaves.p = nullptr;
        *out = r.release();
    });
}

int tdag_build(tdag_ctx* ctx, const tdag_svdag_view* in, const tdag_config* cfg, tdag_result** out)
{
    if (!ctx || !cfg || !out)
        return fail(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guarded([&] {
        checkView(in);
        Context& c = ctx->c;
        cudaStream_t s = c.stream;
        TDAG_CUDA(cudaSetDevice(c.device));
        const bool trace = std::getenv("TDAG_TRACE") != nullptr;
        const auto t0 = std::chrono::steady_clock::now();
        Upload up;
        up.nodes.resize(in->root_level + 1);
        tdag_svdag_view dv = *in;
        for (uint32_t l = 3; l <= in->root_level; ++l) {
            const uint64_t cnt = in->node_counts[l];
            up.nodes[l] = DevBuf<uint32_t>(cnt * 8, s);
            if (cnt)
                TDAG_CUDA(cudaMemcpyAsync(up.nodes[l].get(), in->nodes[l], cnt * 32, cudaMemcpyHostToDevice, s));
            dv.nodes[l] = up.nodes[l].get();
        }
        up.leaves = DevBuf<uint64_t>(in->leaf_count, s);
        if (in->leaf_count)
            TDAG_CUDA(cudaMemcpyAsync(up.leaves.get(), in->leaves, in->leaf_count * 8, cudaMemcpyHostToDevice, s));
        dv.leaves = up.leaves.get();
        std::unique_ptr<tdag_result> r(newResult(in->resolution, in->root_level, false));
        const auto t1 = std::chrono::steady_clock::now();
        DeviceResult dr = buildDevice(c, viewToDevice(&dv), *cfg, &r->stats);
        const auto t2 = std::chrono::steady_clock::now();
        // the result arrays are pinned blocks of the host pool: the device writes them directly
        for (uint32_t l = 3; l <= in->root_level; ++l) {
            const size_t cnt = dr.levels[l].n / 8;
            r->node_counts[l] = cnt;
            r->nodes[l] = (uint64_t*)hostResultAlloc(cnt * 64);
            TDAG_CHECK(r->nodes[l] != nullptr, TDAG_ERR_OOM, "host allocation failed");
            if (cnt)
                TDAG_CUDA(cudaMemcpyAsync(r->nodes[l], dr.levels[l].get(), cnt * 64, cudaMemcpyDeviceToHost, s));
        }
        r->leaf_count = dr.leaves.n;
        r->leaves = (uint64_t*)hostResultAlloc(dr.leaves.n * 8);
        TDAG_CHECK(r->leaves != nullptr, TDAG_ERR_OOM, "host allocation failed");
        if (dr.leaves.n)
            TDAG_CUDA(cudaMemcpyAsync(r->leaves, dr.leaves.get(), dr.leaves.n * 8, cudaMemcpyDeviceToHost, s));
        TDAG_CUDA(cudaStreamSynchronize(s));
        if (trace) { // host-side phases: upload enqueue, build (to its return), download
            const auto t3 = std::chrono::steady_clock::now();
            auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
            std::fprintf(stderr, "[tdag] tdag_build host ms: upload %.3f build %.3f download %.3f (device total %.3f)\n", ms(t0, t1), ms(t1, t2), ms(t2, t3),
                r->stats.total_ms);
        }
        *out = r.release();
    });
}

static int buildBatched(tdag_ctx* ctx, const tdag_svdag_view* in, uint32_t count, const tdag_config* cfg, tdag_result** out, tdag_stats* batchStats, bool host)
{
    if (!ctx || !cfg || !out || (count && !in))
        return fail(TDAG_ERR_ARG, "null argument");
    for (uint32_t g = 0; g < count; ++g)
        out[g] = nullptr;
    return guarded([&] {
        for (uint32_t g = 0; g < count; ++g) {
            checkView(&in[g]);
            TDAG_CHECK(in[g].resolution == (1u << in[g].root_level), TDAG_ERR_ARG, "resolution must equal 1 << root_level");
            if (cfg->translation)
                TDAG_CHECK(in[g].root_level >= cfg->max_translation_level + 1, TDAG_ERR_ARG, "root_level must exceed max_translation_level");
        }
        if (count == 0)
            return;
        Context& c = ctx->c;
        cudaStream_t s = c.stream;
        TDAG_CUDA(cudaSetDevice(c.device));
        if (!host)
            for (uint32_t g = 0; g < count; ++g)
                requireDeviceView(c, in[g]);
        BatchInput b;
        concatBatch(c, in, count, host, b);
        tdag_stats st;
        std::memset(&st, 0, sizeof(st));
        DeviceResult dr = buildDevice(c, b.view, *cfg, &st);
        std::vector<std::unique_ptr<tdag_result>> res(count);
        std::vector<Download> dl;
        for (uint32_t g = 0; g < count; ++g) {
            res[g].reset(newResult(in[g].resolution, in[g].root_level, !host));
            res[g]->stats = st;
            for (uint32_t l = 2; l <= in[g].root_level; ++l) {
                const auto& off = dr.off[l];
                const uint64_t first = off.empty() ? 0 : off[g], cnt = off.empty() ? 0 : off[g + 1] - off[g];
                const uint64_t words = (l == 2) ? 1 : 8;
                const uint64_t* src = (l == 2) ? dr.leaves.get() : dr.levels[l].get();
                uint64_t* dst = nullptr;
                const size_t bytes = cnt * words * 8;
                if (host) {
                    dst = (uint64_t*)std::malloc(bytes ? bytes : 1);
                    TDAG_CHECK(dst != nullptr, TDAG_ERR_OOM, "host allocation failed");
                } else {
                    TDAG_CUDA(cudaMalloc(&dst, bytes ? bytes : 8));
                }
                if (l == 2) {
                    res[g]->leaves = dst;
                    res[g]->leaf_count = cnt;
                } else {
                    res[g]->nodes[l] = dst;
                    res[g]->node_counts[l] = cnt;
                }
                if (host)
                    dl.push_back({ dst, src + first * words, bytes });
                else if (bytes)
                    TDAG_CUDA(cudaMemcpyAsync(dst, src + first * words, bytes, cudaMemcpyDeviceToDevice, s));
            }
        }
        if (host)
            downloadStaged(c, dl);
        TDAG_CUDA(cudaStreamSynchronize(s));
        for (uint32_t g = 0; g < count; ++g)
            out[g] = res[g].release();
        if (batchStats)
            *batchStats = st;
    });
}

int tdag_build_batched(tdag_ctx* ctx, const tdag_svdag_view* in, uint32_t count, const tdag_config* cfg, tdag_result** out, tdag_stats* batchStats)
{
    return buildBatched(ctx, in, count, cfg, out, batchStats, true);
}

int tdag_build_batched_device(tdag_ctx* ctx, const tdag_svdag_view* in, uint32_t count, const tdag_config* cfg, tdag_result** out, tdag_stats* batchStats)
{
    return buildBatched(ctx, in, count, cfg, out, batchStats, false);
}

} // extern "C"

// ------------------------------------------------------------------------------------------------
// Batch graph: the batched build recorded once, then captured into one CUDA graph and replayed.
// ------------------------------------------------------------------------------------------------
namespace tdag {
namespace {

// One input array of the batch: the caller's device pointer and its place in the snapshot.
struct InputSpan {
    const uint32_t* src;
    uint64_t off; // in 32-bit words, into the snapshot
    uint64_t words;
};

constexpr uint32_t kSpanBlocks = 64; // blocks per input array in the comparison

// Counts the words of every input array that differ from the snapshot (block b: array b / 64).
__global__ void compareSpansKernel(const InputSpan* __restrict__ spans, const uint32_t* __restrict__ snap, unsigned long long* __restrict__ diff)
{
    const InputSpan sp = spans[blockIdx.x / kSpanBlocks];
    const uint64_t stride = (uint64_t)kSpanBlocks * blockDim.x;
    uint32_t d = 0;
    for (uint64_t i = (uint64_t)(blockIdx.x % kSpanBlocks) * blockDim.x + threadIdx.x; i < sp.words; i += stride)
        d += sp.src[i] != snap[sp.off + i];
    d = __reduce_add_sync(0xffffffffu, d);
    if ((threadIdx.x & 31) == 0 && d)
        atomicAdd(diff, (unsigned long long)d);
}

struct TapeScope {
    explicit TapeScope(ControlTape* t) { setActiveTape(t); }
    ~TapeScope() { setActiveTape(nullptr); }
};

// Offsets and counts of every grid's levels in a build's concatenated output, and the copies that
// place them contiguously (each level 256-byte aligned) in an arena.
struct OutputLayout {
    std::vector<std::array<uint64_t, TDAG_MAX_LEVELS>> off, count; // per grid; off in bytes into the arena
    uint64_t bytes = 0;
};

OutputLayout layoutOf(const DeviceResult& dr, const tdag_svdag_view* in, uint32_t count)
{
    OutputLayout L;
    L.off.resize(count);
    L.count.resize(count);
    for (uint32_t g = 0; g < count; ++g) {
        L.off[g].fill(0);
        L.count[g].fill(0);
        for (uint32_t l = 2; l <= in[g].root_level; ++l) {
            const auto& off = dr.off[l];
            const uint64_t cnt = off.empty() ? 0 : off[g + 1] - off[g];
            L.off[g][l] = L.bytes;
            L.count[g][l] = cnt;
            L.bytes += (cnt * (l == 2 ? 1 : 8) * 8 + 255) & ~255ull;
        }
    }
    return L;
}

void copyToArena(const DeviceResult& dr, const tdag_svdag_view* in, uint32_t count, const OutputLayout& L, unsigned char* arena, cudaStream_t s)
{
    for (uint32_t g = 0; g < count; ++g)
        for (uint32_t l = 2; l <= in[g].root_level; ++l) {
            const uint64_t words = (l == 2) ? 1 : 8, cnt = L.count[g][l];
            if (!cnt)
                continue;
            const uint64_t* src = ((l == 2) ? dr.leaves.get() : dr.levels[l].get()) + dr.off[l][g] * words;
            TDAG_CUDA(cudaMemcpyAsync(arena + L.off[g][l], src, cnt * words * 8, cudaMemcpyDeviceToDevice, s));
        }
}

} // namespace
} // namespace tdag

struct tdag_batch_graph {
    tdag_ctx* ctx = nullptr; // launches run on its stream; the context must outlive them
    int device = 0;
    std::shared_ptr<StreamState> stream; // keeps the stream alive for the destructor
    tdag_config cfg {};
    std::vector<tdag_svdag_view> views;
    std::vector<InputSpan> spans;
    uint32_t* snap = nullptr; // device copy of every input array at creation
    InputSpan* spansDev = nullptr;
    unsigned long long* diff = nullptr; // differing input words (device)
    ControlTape tape;
    unsigned char* uploadsDev = nullptr;
    uint32_t* mismatch = nullptr;
    OutputLayout layout;
    unsigned char* arena = nullptr; // the graph's output, grid by grid
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernelNodes = 0;

    ~tdag_batch_graph()
    {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream->stream);
        }
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        for (void* p : { (void*)snap, (void*)spansDev, (void*)diff, (void*)uploadsDev, (void*)mismatch, (void*)arena })
            if (p)
                cudaFree(p);
        if (stream)
            cudaDeviceGraphMemTrim(device);
    }
};

extern "C" {

int tdag_batch_graph_create(tdag_ctx* ctx, const tdag_svdag_view* in, uint32_t count, const tdag_config* cfg, tdag_batch_graph** out)
{
    if (!ctx || !cfg || !out || !in || count == 0)
        return fail(TDAG_ERR_ARG, "null argument or empty batch");
    *out = nullptr;
    auto G = std::make_unique<tdag_batch_graph>();
    const int rc = guarded([&] {
        for (uint32_t g = 0; g < count; ++g) {
            checkView(&in[g]);
            TDAG_CHECK(in[g].resolution == (1u << in[g].root_level), TDAG_ERR_ARG, "resolution must equal 1 << root_level");
            if (cfg->translation)
                TDAG_CHECK(in[g].root_level >= cfg->max_translation_level + 1, TDAG_ERR_ARG, "root_level must exceed max_translation_level");
        }
        Context& c = ctx->c;
        cudaStream_t s = c.stream;
        TDAG_CUDA(cudaSetDevice(c.device));
        for (uint32_t g = 0; g < count; ++g)
            requireDeviceView(c, in[g]);
        G->ctx = ctx;
        G->device = c.device;
        G->stream = c.streamState;
        G->cfg = *cfg;
        G->views.assign(in, in + count);

        // snapshot of the inputs, compared with the caller's arrays before every launch
        uint64_t words = 0;
        for (uint32_t g = 0; g < count; ++g) {
            auto add = [&](const void* p, uint64_t bytes) {
                if (!bytes)
                    return;
                G->spans.push_back({ static_cast<const uint32_t*>(p), words, bytes / 4 });
                words += (bytes / 4 + 63) & ~63ull;
            };
            add(in[g].leaves, in[g].leaf_count * 8);
            for (uint32_t l = 3; l <= in[g].root_level; ++l)
                add(in[g].nodes[l], in[g].node_counts[l] * 32);
        }
        TDAG_CUDA(cudaMalloc(&G->snap, std::max<uint64_t>(words, 1) * 4));
        for (const InputSpan& sp : G->spans)
            TDAG_CUDA(cudaMemcpyAsync(G->snap + sp.off, sp.src, sp.words * 4, cudaMemcpyDeviceToDevice, s));
        TDAG_CUDA(cudaMalloc(&G->spansDev, std::max<size_t>(G->spans.size(), 1) * sizeof(InputSpan)));
        if (!G->spans.empty())
            TDAG_CUDA(cudaMemcpyAsync(G->spansDev, G->spans.data(), G->spans.size() * sizeof(InputSpan), cudaMemcpyHostToDevice, s));
        TDAG_CUDA(cudaMalloc(&G->diff, 8));
        TDAG_CUDA(cudaStreamSynchronize(s));

        // 1. the plan: an ordinary build that records every host read and upload
        ControlTape& t = G->tape;
        {
            TapeScope scope(&t);
            BatchInput b;
            concatBatch(c, in, count, false, b);
            DeviceResult dr = buildDevice(c, b.view, *cfg, nullptr);
            G->layout = layoutOf(dr, in, count);
            syncHost(s);
        }
        TDAG_CUDA(cudaMalloc(&G->uploadsDev, std::max<size_t>(t.uploads.size(), 1)));
        if (!t.uploads.empty())
            TDAG_CUDA(cudaMemcpy(G->uploadsDev, t.uploads.data(), t.uploads.size(), cudaMemcpyHostToDevice));
        TDAG_CUDA(cudaMalloc(&G->mismatch, 4));
        TDAG_CUDA(cudaMemset(G->mismatch, 0, 4));
        TDAG_CUDA(cudaMalloc(&G->arena, std::max<uint64_t>(G->layout.bytes, 256)));
        preloadTapeKernels();
        t.replay = true;
        t.readPos = t.uploadPos = 0;
        t.readIndex = 0;
        t.uploadsDev = G->uploadsDev;
        t.mismatch = G->mismatch;

        // 2. the same build captured: sizes and launch shapes come from the plan
        TDAG_CUDA(cudaStreamSynchronize(s));
        TDAG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        try {
            TapeScope scope(&t);
            BatchInput b;
            concatBatch(c, in, count, false, b);
            DeviceResult dr = buildDevice(c, b.view, *cfg, nullptr);
            copyToArena(dr, in, count, G->layout, G->arena, s);
        } catch (...) {
            cudaGraph_t broken = nullptr;
            cudaStreamEndCapture(s, &broken);
            if (broken)
                cudaGraphDestroy(broken);
            cudaGetLastError();
            throw;
        }
        TDAG_CUDA(cudaStreamEndCapture(s, &G->graph));
        TDAG_CHECK(t.readPos == t.reads.size() && t.uploadPos == t.uploads.size(), TDAG_ERR_CUDA,
            "batch graph: the captured build did not replay its whole plan");
        size_t numNodes = 0;
        TDAG_CUDA(cudaGraphGetNodes(G->graph, nullptr, &numNodes));
        std::vector<cudaGraphNode_t> nodes(numNodes);
        if (numNodes)
            TDAG_CUDA(cudaGraphGetNodes(G->graph, nodes.data(), &numNodes));
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType ty;
            TDAG_CUDA(cudaGraphNodeGetType(nd, &ty));
            G->kernelNodes += ty == cudaGraphNodeTypeKernel;
        }
        TDAG_CUDA(cudaGraphInstantiate(&G->exec, G->graph, 0));
        TDAG_CUDA(cudaGraphUpload(G->exec, s));
        TDAG_CUDA(cudaStreamSynchronize(s));
    });
    if (rc != TDAG_OK)
        return rc;
    *out = G.release();
    return TDAG_OK;
}

int tdag_batch_graph_launch(tdag_batch_graph* G, tdag_result** out, tdag_stats* stats)
{
    if (!G || !out)
        return fail(TDAG_ERR_ARG, "null argument");
    const uint32_t count = (uint32_t)G->views.size();
    for (uint32_t g = 0; g < count; ++g)
        out[g] = nullptr;
    return guarded([&] {
        Context& c = G->ctx->c;
        cudaStream_t s = c.stream;
        TDAG_CUDA(cudaSetDevice(c.device));
        uint64_t* hp = pinnedScratch();
        // the batch must hold the contents the graph was planned on
        if (!G->spans.empty()) {
            TDAG_CUDA(cudaMemsetAsync(G->diff, 0, 8, s));
            compareSpansKernel<<<(unsigned)(G->spans.size() * kSpanBlocks), 256, 0, s>>>(G->spansDev, G->snap, G->diff);
            TDAG_LAUNCHED();
            readToHost({ { hp, G->diff, 8 } }, s);
            TDAG_CHECK(hp[0] == 0, TDAG_ERR_ARG, "the batch's arrays changed since the graph was created (" + std::to_string(hp[0]) + " words differ)");
        }
        TDAG_CUDA(cudaMemsetAsync(G->mismatch, 0, 4, s));
        TDAG_CUDA(cudaEventRecord(c.ev[2], s));
        TDAG_CUDA(cudaGraphLaunch(G->exec, s));
        TDAG_CUDA(cudaEventRecord(c.ev[3], s));
        readToHost({ { c.hostStatus, c.status, 16 }, { hp, G->mismatch, 4 } }, s);
        const uint32_t code = c.hostStatus[0], aux = c.hostStatus[1];
        const uint32_t mismatch = (uint32_t)hp[0];
        if (code) {
            TDAG_CUDA(cudaMemsetAsync(c.status, 0, 16, s));
            TDAG_CUDA(cudaStreamSynchronize(s));
            throw Error((int)code, "batch graph: device reported error " + std::to_string(code) + " (aux " + std::to_string(aux) + ")");
        }
        TDAG_CHECK(mismatch == 0, TDAG_ERR_CUDA, "batch graph: the replay differed from its plan at host read " + std::to_string(mismatch - 1));
        tdag_stats st;
        std::memset(&st, 0, sizeof(st));
        TDAG_CUDA(cudaEventElapsedTime(&st.total_ms, c.ev[2], c.ev[3]));
        st.kernel_launches = G->kernelNodes;
        std::vector<std::unique_ptr<tdag_result>> res(count);
        for (uint32_t g = 0; g < count; ++g) {
            const tdag_svdag_view& v = G->views[g];
            res[g].reset(newResult(v.resolution, v.root_level, true));
            res[g]->stats = st;
            for (uint32_t l = 2; l <= v.root_level; ++l) {
                const uint64_t cnt = G->layout.count[g][l];
                const size_t bytes = cnt * (l == 2 ? 1 : 8) * 8;
                uint64_t* dst = nullptr;
                TDAG_CUDA(cudaMalloc(&dst, bytes ? bytes : 8));
                if (l == 2) {
                    res[g]->leaves = dst;
                    res[g]->leaf_count = cnt;
                } else {
                    res[g]->nodes[l] = dst;
                    res[g]->node_counts[l] = cnt;
                }
                if (bytes)
                    TDAG_CUDA(cudaMemcpyAsync(dst, G->arena + G->layout.off[g][l], bytes, cudaMemcpyDeviceToDevice, s));
            }
        }
        TDAG_CUDA(cudaStreamSynchronize(s));
        for (uint32_t g = 0; g < count; ++g)
            out[g] = res[g].release();
        if (stats)
            *stats = st;
    });
}

int tdag_batch_graph_free(tdag_batch_graph* G)
{
    delete G;
    return TDAG_OK;
}

int tdag_build_hierarchical(tdag_ctx* ctx, const tdag_svdag_view* in, const tdag_config* cfg, tdag_result** out)
{
    if (!cfg)
        return fail(TDAG_ERR_ARG, "null argument");
    tdag_config c = *cfg;
    c.translation = 0;
    return tdag_build(ctx, in, &c, out);
}

int tdag_result_to_host(tdag_ctx* ctx, const tdag_result* d, tdag_result** out)
{
    if (!ctx || !d || !out)
        return fail(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guarded([&] {
        TDAG_CHECK(d->on_device, TDAG_ERR_ARG, "result is not device-resident");
        Context& c = ctx->c;
        TDAG_CUDA(cudaSetDevice(c.device));
        std::unique_ptr<tdag_result> r(newResult(d->resolution, d->root_level, false));
        r->structure_type = d->structure_type;
        r->stats = d->stats;
        std::vector<Download> dl;
        for (uint32_t l = 3; l <= d->root_level; ++l) {
            const size_t bytes = d->node_counts[l] * 64;
            r->node_counts[l] = d->node_counts[l];
            r->nodes[l] = (uint64_t*)std::malloc(bytes ? bytes : 1);
            TDAG_CHECK(r->nodes[l] != nullptr, TDAG_ERR_OOM, "host allocation failed");
            dl.push_back({ r->nodes[l], d->nodes[l], bytes });
        }
        r->leaf_count = d->leaf_count;
        r->leaves = (uint64_t*)std::malloc(d->leaf_count ? d->leaf_count * 8 : 1);
        TDAG_CHECK(r->leaves != nullptr, TDAG_ERR_OOM, "host allocation failed");
        dl.push_back({ r->leaves, d->leaves, d->leaf_count * 8 });
        downloadStaged(c, dl);
        *out = r.release();
    });
}

int tdag_result_free(tdag_result* r)
{
    if (!r)
        return TDAG_OK;
    // host arrays: pinned pool blocks (tdag_build) or plain allocations (the other host results)
    for (uint32_t l = 0; l < TDAG_MAX_LEVELS; ++l) {
        if (!r->nodes[l])
            continue;
        if (r->on_device)
            cudaFree(r->nodes[l]);
        else
            hostResultFree(r->nodes[l]);
    }
    if (r->leaves) {
        if (r->on_device)
            cudaFree(r->leaves);
        else
            hostResultFree(r->leaves);
    }
    delete r;
    return TDAG_OK;
}

int tdag_find_duplicates_level(tdag_ctx* ctx, uint32_t level, const uint64_t* grids, uint32_t n, const tdag_config* cfg, uint64_t* outMapping,
    uint32_t* outUnique, uint32_t* nUnique, tdag_level_stats* stats)
{
    if (!ctx || !cfg || !nUnique || (n && (!grids || !outMapping || !outUnique)))
        return fail(TDAG_ERR_ARG, "null argument");
    return guarded([&] {
        TDAG_CHECK(level >= 2 && level <= 4, TDAG_ERR_ARG, "level must be 2..4");
        Context& c = ctx->c;
        cudaStream_t s = c.stream;
        TDAG_CUDA(cudaSetDevice(c.device));
        const size_t W = ((size_t)1 << (3 * level)) / 64;
        DevBuf<uint64_t> g(n * W, s);
        if (n)
            TDAG_CUDA(cudaMemcpyAsync(g.get(), grids, n * W * 8, cudaMemcpyHostToDevice, s));
        tdag_level_stats ls {};
        MatchOutput mo = runMatcher(c, level, g.get(), n, *cfg, &ls);
        if (n) {
            TDAG_CUDA(cudaMemcpyAsync(outMapping, mo.mapping.get(), (size_t)n * 8, cudaMemcpyDeviceToHost, s));
            if (mo.numUnique)
                TDAG_CUDA(cudaMemcpyAsync(outUnique, mo.uniques.get(), (size_t)mo.numUnique * 4, cudaMemcpyDeviceToHost, s));
        }
        TDAG_CUDA(cudaStreamSynchronize(s));
        *nUnique = mo.numUnique;
        if (stats)
            *stats = ls;
    });
}

int tdag_device_copy(tdag_ctx* ctx, void* d_dst, const void* d_src, uint64_t bytes)
{
    if (!ctx || (bytes && (!d_dst || !d_src)))
        return fail(TDAG_ERR_ARG, "null argument");
    return guarded([&] {
        Context& c = ctx->c;
        TDAG_CUDA(cudaSetDevice(c.device));
        if (bytes) {
            requireDeviceAccessible(c, d_dst, "d_dst");
            requireDeviceAccessible(c, d_src, "d_src");
            TDAG_CUDA(cudaMemcpyAsync(d_dst, d_src, bytes, cudaMemcpyDeviceToDevice, c.stream));
        }
        TDAG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int tdag_find_duplicates_level_device(tdag_ctx* ctx, uint32_t level, const uint64_t* d_grids, uint32_t n, const tdag_config* cfg, const uint32_t* d_sources,
    uint32_t num_sources, uint64_t* d_out_mapping, uint32_t* d_out_unique, uint32_t* n_unique, tdag_level_stats* stats)
{
    if (!ctx || !cfg || !n_unique || (n && (!d_grids || !d_out_mapping || !d_out_unique)) || (num_sources && !d_sources))
        return fail(TDAG_ERR_ARG, "null argument");
    return guarded([&] {
        TDAG_CHECK(level >= 2 && level <= 4, TDAG_ERR_ARG, "level must be 2..4");
        Context& c = ctx->c;
        cudaStream_t s = c.stream;
        TDAG_CUDA(cudaSetDevice(c.device));
        if (n) {
            requireDeviceAccessible(c, d_grids, "d_grids");
            requireDeviceAccessible(c, d_out_mapping, "d_out_mapping");
            requireDeviceAccessible(c, d_out_unique, "d_out_unique");
        }
        if (num_sources)
            requireDeviceAccessible(c, d_sources, "d_sources");
        tdag_level_stats ls {};
        MatchOutput mo = runMatcher(c, level, d_grids, n, *cfg, &ls, nullptr, d_sources, d_sources ? num_sources : 0);
        if (n) {
            TDAG_CUDA(cudaMemcpyAsync(d_out_mapping, mo.mapping.get(), (size_t)n * 8, cudaMemcpyDeviceToDevice, s));
            if (mo.numUnique)
                TDAG_CUDA(cudaMemcpyAsync(d_out_unique, mo.uniques.get(), (size_t)mo.numUnique * 4, cudaMemcpyDeviceToDevice, s));
        }
        TDAG_CUDA(cudaStreamSynchronize(s));
        *n_unique = mo.numUnique;
        if (stats)
            *stats = ls;
    });
}

} // extern "C"

// ================================================================================================
// constructStaticTransformDAG (transform_dag.cpp:242-390): StaticStructure<void, uint32_t> in,
// StaticStructure<void, TransformPointer> out. A packed level is a word stream: per node a header
// (child mask) and one word per present child, child words being word offsets into the level below
// (leaf indices at level 3). The levels are unpacked on the device (node starts found top-down from
// the parents' child words, then checked to tile each level), built like the EditStructure path
// except that the hierarchical pass hashes child word offsets (transform_dag_hierarchical.cpp:531-743),
// and packed again with 64-bit words.
// ================================================================================================
namespace tdag {
namespace {

__global__ void staticChildCountKernel(const uint32_t* __restrict__ words, uint64_t wordCount, const uint32_t* __restrict__ starts, uint32_t n,
    uint32_t* __restrict__ counts, uint32_t* status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t s = starts[i];
    uint32_t c = 0;
    if (s < wordCount && (words[s] >> 8) == 0 && s + 1 + (uint64_t)__popc(words[s]) <= wordCount)
        c = __popc(words[s]);
    else
        setDeviceError(status, TDAG_ERR_CORRUPT, 60);
    counts[i] = c;
}
__global__ void staticChildWordsKernel(const uint32_t* __restrict__ words, const uint32_t* __restrict__ starts, uint32_t n, const uint32_t* __restrict__ base,
    const uint32_t* __restrict__ counts, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t s = starts[i];
    for (uint32_t j = 0; j < counts[i]; ++j) {
        keys[base[i] + j] = words[s + 1 + j];
        vals[base[i] + j] = 0;
    }
}
__global__ void distinctFlagsKernel(const uint64_t* __restrict__ keys, uint32_t m, uint32_t* __restrict__ flags)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < m)
        flags[j] = (j == 0 || keys[j] != keys[j - 1]) ? 1u : 0u;
}
__global__ void distinctGatherKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ idx, uint32_t u, uint32_t* __restrict__ out)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < u)
        out[j] = (uint32_t)keys[idx[j]];
}
// The starts found from the parents must tile the level: node j ends where node j + 1 starts.
__global__ void staticTileCheckKernel(const uint32_t* __restrict__ words, uint64_t wordCount, const uint32_t* __restrict__ starts, uint32_t n, uint32_t* status)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const uint32_t s = starts[j];
    bool ok = s < wordCount && (j > 0 || s == 0);
    if (ok) {
        const uint32_t h = words[s];
        const uint64_t end = (uint64_t)s + 1 + __popc(h);
        ok = (h >> 8) == 0 && end == (j + 1 < n ? (uint64_t)starts[j + 1] : wordCount);
    }
    if (!ok)
        setDeviceError(status, TDAG_ERR_CORRUPT, 61);
}
// Packed node -> EditNode<uint32_t> (children as indices into the level below).
__global__ void staticUnpackKernel(const uint32_t* __restrict__ words, const uint32_t* __restrict__ starts, uint32_t n, const uint32_t* __restrict__ childStarts,
    uint32_t childCount, bool leavesBelow, uint32_t* __restrict__ nodes, uint32_t* status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t s = starts[i];
    const uint32_t mask = words[s];
    uint32_t w = s + 1;
    for (uint32_t k = 0; k < 8; ++k) {
        uint32_t out = kEmpty32;
        if ((mask >> k) & 1) {
            const uint32_t v = words[w++];
            if (leavesBelow) {
                out = v;
                if (v >= childCount)
                    setDeviceError(status, TDAG_ERR_CORRUPT, 62);
            } else {
                uint32_t lo = 0, hi = childCount; // first start >= v
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (childStarts[mid] < v)
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                if (lo < childCount && childStarts[lo] == v)
                    out = lo;
                else
                    setDeviceError(status, TDAG_ERR_CORRUPT, 63);
            }
        }
        nodes[(size_t)i * 8 + k] = out;
    }
}
__global__ void packSizeKernel(const uint64_t* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ sizes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t w = 1;
    for (int k = 0; k < 8; ++k)
        w += nodes[(size_t)i * 8 + k] != tpSentinel() ? 1u : 0u;
    sizes[i] = w;
}
__global__ void packKernel(const uint64_t* __restrict__ nodes, uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ childOff,
    uint64_t* __restrict__ words)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint64_t at = off[i];
    const uint64_t head = at++;
    uint64_t mask = 0;
    for (int k = 0; k < 8; ++k) {
        const uint64_t c = nodes[(size_t)i * 8 + k];
        if (c == tpSentinel())
            continue;
        mask |= 1ull << k;
        words[at++] = childOff ? tpWithPtr(c, childOff[tpPtr(c)]) : c;
    }
    words[head] = mask;
}

} // namespace

struct StaticOut {
    std::vector<DevBuf<uint64_t>> words;
    std::vector<uint64_t> wordCounts;
    DevBuf<uint64_t> leaves;
    uint64_t leafCount = 0;
};

StaticOut buildStatic(Context& c, const tdag_static_view& in, const tdag_config& cfg, tdag_stats* stats)
{
    cudaStream_t s = c.stream;
    const uint32_t root = in.root_level;
    TDAG_CHECK(root >= 3 && root < TDAG_MAX_LEVELS, TDAG_ERR_ARG, "root_level out of range");
    TDAG_CHECK(in.resolution == (1u << root), TDAG_ERR_ARG, "resolution must equal 1 << root_level");
    TDAG_CHECK(in.leaf_count < (1ull << 31), TDAG_ERR_ARG, "too many leaves");
    // upload the packed levels
    std::vector<DevBuf<uint32_t>> words(root + 1);
    for (uint32_t l = 3; l <= root; ++l) {
        TDAG_CHECK(in.word_counts[l] < 0xFFFFFFFFull, TDAG_ERR_ARG, "a packed level exceeds 2^32 words");
        TDAG_CHECK(in.word_counts[l] == 0 || in.words[l] != nullptr, TDAG_ERR_ARG, "null word array with non-zero count");
        words[l] = DevBuf<uint32_t>(std::max<uint64_t>(in.word_counts[l], 1), s);
        if (in.word_counts[l])
            TDAG_CUDA(cudaMemcpyAsync(words[l].get(), in.words[l], in.word_counts[l] * 4, cudaMemcpyHostToDevice, s));
    }
    DevBuf<uint64_t> leaves(std::max<uint64_t>(in.leaf_count, 1), s);
    if (in.leaf_count)
        TDAG_CUDA(cudaMemcpyAsync(leaves.get(), in.leaves, in.leaf_count * 8, cudaMemcpyHostToDevice, s));
    // node starts, top-down: the root level holds one node at word 0; every other level's starts are
    // the distinct child words of the level above
    std::vector<DevBuf<uint32_t>> starts(root + 1);
    std::vector<uint32_t> count(root + 1, 0);
    count[root] = in.word_counts[root] ? 1 : 0;
    starts[root] = DevBuf<uint32_t>(1, s);
    TDAG_CUDA(cudaMemsetAsync(starts[root].get(), 0, 4, s));
    for (uint32_t l = root; l >= 3; --l) {
        const uint32_t n = count[l];
        if (n) {
            staticTileCheckKernel<<<gridFor(n, 256), 256, 0, s>>>(words[l].get(), in.word_counts[l], starts[l].get(), n, c.status);
            TDAG_LAUNCHED();
        } else {
            TDAG_CHECK(in.word_counts[l] == 0, TDAG_ERR_CORRUPT, "a packed level holds words no parent references");
        }
        c.checkStatus("static input: node starts");
        if (l == 3)
            break;
        DevBuf<uint32_t> cnt(std::max<uint32_t>(n, 1), s), base(std::max<uint32_t>(n, 1), s);
        uint32_t m = 0;
        if (n) {
            staticChildCountKernel<<<gridFor(n, 256), 256, 0, s>>>(words[l].get(), in.word_counts[l], starts[l].get(), n, cnt.get(), c.status);
            TDAG_LAUNCHED();
            m = (uint32_t)exclusiveScanU32Total(cnt.get(), base.get(), n, s);
        }
        DevBuf<uint64_t> keys(std::max<uint32_t>(m, 1), s);
        DevBuf<uint32_t> vals(std::max<uint32_t>(m, 1), s), flags(std::max<uint32_t>(m, 1), s), idx(std::max<uint32_t>(m, 1), s);
        uint32_t u = 0;
        if (m) {
            staticChildWordsKernel<<<gridFor(n, 256), 256, 0, s>>>(words[l].get(), starts[l].get(), n, base.get(), cnt.get(), keys.get(), vals.get());
            TDAG_LAUNCHED();
            radixSortPairs(keys.get(), vals.get(), m, 0, 32, s, c.status);
            distinctFlagsKernel<<<gridFor(m, 256), 256, 0, s>>>(keys.get(), m, flags.get());
            TDAG_LAUNCHED();
            u = compactFlags(flags.get(), idx.get(), m, s);
        }
        starts[l - 1] = DevBuf<uint32_t>(std::max<uint32_t>(u, 1), s);
        if (u) {
            distinctGatherKernel<<<gridFor(u, 256), 256, 0, s>>>(keys.get(), idx.get(), u, starts[l - 1].get());
            TDAG_LAUNCHED();
        }
        count[l - 1] = u;
    }
    // unpack into EditNode<uint32_t> levels
    std::vector<DevBuf<uint32_t>> nodes(root + 1);
    DeviceSvdag dv;
    dv.resolution = in.resolution;
    dv.rootLevel = root;
    dv.staticOffsets = true;
    for (uint32_t l = 3; l <= root; ++l) {
        nodes[l] = DevBuf<uint32_t>(std::max<uint64_t>((uint64_t)count[l] * 8, 1), s);
        if (count[l]) {
            staticUnpackKernel<<<gridFor(count[l], 256), 256, 0, s>>>(words[l].get(), starts[l].get(), count[l], l == 3 ? nullptr : starts[l - 1].get(),
                l == 3 ? (uint32_t)in.leaf_count : count[l - 1], l == 3, nodes[l].get(), c.status);
            TDAG_LAUNCHED();
        }
        dv.nodes[l] = nodes[l].get();
        dv.nodeCounts[l] = count[l];
    }
    dv.leaves = leaves.get();
    dv.leafCount = in.leaf_count;
    c.checkStatus("static input: unpack");
    words.clear();
    starts.clear();
    DeviceResult dr = buildDevice(c, dv, cfg, stats);
    // pack with 64-bit words: child TransformPointers point at word offsets (level 3: leaf indices)
    StaticOut out;
    out.words.resize(root + 1);
    out.wordCounts.assign(root + 1, 0);
    DevBuf<uint32_t> prevOff;
    for (uint32_t l = 3; l <= root; ++l) {
        const uint32_t n = (uint32_t)(dr.levels[l].n / 8);
        DevBuf<uint32_t> sizes(std::max<uint32_t>(n, 1), s), off(std::max<uint32_t>(n, 1), s);
        uint64_t total = 0;
        if (n) {
            packSizeKernel<<<gridFor(n, 256), 256, 0, s>>>(dr.levels[l].get(), n, sizes.get());
            TDAG_LAUNCHED();
            total = exclusiveScanU32Total(sizes.get(), off.get(), n, s);
        }
        out.words[l] = DevBuf<uint64_t>(std::max<uint64_t>(total, 1), s);
        out.wordCounts[l] = total;
        if (n) {
            packKernel<<<gridFor(n, 256), 256, 0, s>>>(dr.levels[l].get(), n, off.get(), l == 3 ? nullptr : prevOff.get(), out.words[l].get());
            TDAG_LAUNCHED();
        }
        prevOff = std::move(off);
    }
    out.leafCount = dr.leaves.n;
    out.leaves = std::move(dr.leaves);
    TDAG_CUDA(cudaStreamSynchronize(s));
    return out;
}

} // namespace tdag

extern "C" {

int tdag_static_result_free(tdag_static_result* r);

int tdag_build_static(tdag_ctx* ctx, const tdag_static_view* in, const tdag_config* cfg, tdag_static_result** out)
{
    if (!ctx || !in || !cfg || !out)
        return fail(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guarded([&] {
        Context& c = ctx->c;
        TDAG_CUDA(cudaSetDevice(c.device));
        std::unique_ptr<tdag_static_result, int (*)(tdag_static_result*)> r(new tdag_static_result, tdag_static_result_free);
        std::memset(r.get(), 0, sizeof(tdag_static_result));
        r->resolution = in->resolution;
        r->root_level = in->root_level;
        r->structure_type = 0;
        StaticOut so = buildStatic(c, *in, *cfg, &r->stats);
        std::vector<Download> dl;
        for (uint32_t l = 3; l <= in->root_level; ++l) {
            r->word_counts[l] = so.wordCounts[l];
            if (so.wordCounts[l]) {
                r->words[l] = static_cast<uint64_t*>(std::malloc(so.wordCounts[l] * 8));
                TDAG_CHECK(r->words[l] != nullptr, TDAG_ERR_OOM, "host allocation failed");
                dl.push_back({ r->words[l], so.words[l].get(), so.wordCounts[l] * 8 });
            }
        }
        r->leaf_count = so.leafCount;
        if (so.leafCount) {
            r->leaves = static_cast<uint64_t*>(std::malloc(so.leafCount * 8));
            TDAG_CHECK(r->leaves != nullptr, TDAG_ERR_OOM, "host allocation failed");
            dl.push_back({ r->leaves, so.leaves.get(), so.leafCount * 8 });
        }
        downloadStaged(c, dl);
        *out = r.release();
    });
}

int tdag_static_result_free(tdag_static_result* r)
{
    if (!r)
        return TDAG_OK;
    for (uint32_t l = 0; l < TDAG_MAX_LEVELS; ++l)
        std::free(r->words[l]);
    std::free(r->leaves);
    delete r;
    return TDAG_OK;
}

} // extern "C"
