// common.cuh — shared device/host definitions for the GB300 Transform-DAG library (libtdag.so).
//
// Integer/bitwise only. Semantics follow the reference's Transform-Aware SVDAG construction:
//   TransformPointer bit layout ............ tools/lib/include/voxcom/voxel/transform_dag.h:19-33
//   encodeFixed64 / decodeFixed64 .......... transform_dag.h:349-397
//   transform IDs (sym | perm << 3) ........ tools/lib/src/voxel/transform_dag_hierarchical.cpp:23-46
//   hash_combine ........................... tools/lib/include/voxcom/utility/hash.h:10-20
#pragma once
#include <cstdint>
#include <atomic>
#include <cstdio>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <cuda_runtime.h>

#include "../../include/tdag.h"

namespace tdag {

// ------------------------------------------------------------------------------------------------
// Errors. Host code throws tdag::Error(code, message); the C-ABI layer converts to a status code.
// Device code never traps: it records the first error in a status word the host reads after the
// stage (TDAG_ERR_TABLE_FULL etc.) and returns.
// ------------------------------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m)
        : std::runtime_error(m)
        , code(c)
    {
    }
};

#define TDAG_CUDA(call)                                                                                         \
    do {                                                                                                        \
        cudaError_t e_ = (call);                                                                                \
        if (e_ != cudaSuccess)                                                                                  \
            throw ::tdag::Error(TDAG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " @" + __FILE__ + ":" + std::to_string(__LINE__)); \
    } while (0)

// Every kernel launch of the library is followed by TDAG_LAUNCHED(): it checks the launch and
// counts it (the count is reported per build as tdag_stats::kernel_launches).
extern std::atomic<uint64_t> g_kernelLaunches;
#define TDAG_LAUNCHED()                                                              \
    do {                                                                             \
        TDAG_CUDA(cudaGetLastError());                                               \
        ::tdag::g_kernelLaunches.fetch_add(1, std::memory_order_relaxed);             \
    } while (0)

#define TDAG_CHECK(cond, code, msg)                \
    do {                                           \
        if (!(cond))                               \
            throw ::tdag::Error((code), (msg));    \
    } while (0)

// Device status word layout: [0] = first error code, [1] = aux (e.g. the level), [2..3] spare.
__device__ __forceinline__ void setDeviceError(uint32_t* status, uint32_t code, uint32_t aux = 0)
{
    if (atomicCAS(status, 0u, code) == 0u)
        status[1] = aux;
}

// ------------------------------------------------------------------------------------------------
// hash_combine with the identity hasher, 64-bit (size_t) wrap-around.
// ------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t hashCombine(uint64_t seed, uint64_t key)
{
    return seed ^ (key + 0x9e3779b9ull + (seed << 6) + (seed >> 2));
}

// A strong 64-bit mixer for table slot selection (splitmix64 finaliser constants are public domain).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

// ------------------------------------------------------------------------------------------------
// Morton codes (x in bit 0), libmorton morton3D_32 semantics.
// ------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t part1by2(uint32_t v)
{
    v &= 0x3ff;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}
__host__ __device__ __forceinline__ uint32_t compact1by2(uint32_t v)
{
    v &= 0x09249249;
    v = (v ^ (v >> 2)) & 0x030C30C3;
    v = (v ^ (v >> 4)) & 0x0300F00F;
    v = (v ^ (v >> 8)) & 0x030000FF;
    v = (v ^ (v >> 16)) & 0x000003FF;
    return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) { return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2); }

// ------------------------------------------------------------------------------------------------
// TransformPointer (compact 64-bit layout): ptr:37 | sx:1 sy:1 sz:1 | p0:2 p1:2 p2:2 | tx:6 ty:6 tz:6,
// translations biased by +32. The 48 rotations/mirrors are numbered sym | permId << 3, where
// permId indexes kPermTable = {012, 021, 102, 120, 201, 210}.
// ------------------------------------------------------------------------------------------------
constexpr uint64_t kPtrMask = (1ull << 37) - 1;
constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;

__host__ __device__ __forceinline__ uint32_t permBitsOf(uint32_t permId)
{
    // packed p0 | p1 << 2 | p2 << 4 for each permutation ID
    constexpr uint32_t packed[6] = { 0 | 1 << 2 | 2 << 4, 0 | 2 << 2 | 1 << 4, 1 | 0 << 2 | 2 << 4, 1 | 2 << 2 | 0 << 4, 2 | 0 << 2 | 1 << 4, 2 | 1 << 2 | 0 << 4 };
    return packed[permId];
}
__host__ __device__ __forceinline__ uint32_t permIdOfBits(uint32_t pbits)
{
    const uint32_t p0 = pbits & 3, p1 = (pbits >> 2) & 3, p2 = (pbits >> 4) & 3;
    return 2 * p0 + (p2 < p1 ? 1 : 0);
}
__host__ __device__ __forceinline__ uint64_t tpCreate(uint64_t ptr, uint32_t sym, uint32_t permId, int tx = 0, int ty = 0, int tz = 0)
{
    uint64_t v = ptr & kPtrMask;
    v |= (uint64_t)(sym & 7) << 37;
    v |= (uint64_t)permBitsOf(permId) << 40;
    v |= (uint64_t)((unsigned)(tx + 32) & 63) << 46;
    v |= (uint64_t)((unsigned)(ty + 32) & 63) << 52;
    v |= (uint64_t)((unsigned)(tz + 32) & 63) << 58;
    return v;
}
__host__ __device__ __forceinline__ uint64_t tpCreateT(uint64_t ptr, uint32_t transformId) { return tpCreate(ptr, transformId & 7, transformId >> 3); }
__host__ __device__ __forceinline__ uint64_t tpSentinel() { return tpCreate(0xFFFFFFFFull, 0, 0); }
__host__ __device__ __forceinline__ uint64_t tpPtr(uint64_t v) { return v & kPtrMask; }
__host__ __device__ __forceinline__ uint32_t tpSym(uint64_t v) { return (uint32_t)(v >> 37) & 7; }
__host__ __device__ __forceinline__ uint32_t tpPermId(uint64_t v) { return permIdOfBits((uint32_t)(v >> 40) & 63); }
__host__ __device__ __forceinline__ uint32_t tpTransformId(uint64_t v) { return tpSym(v) | (tpPermId(v) << 3); }
__host__ __device__ __forceinline__ int tpT(uint64_t v, int axis) { return (int)((v >> (46 + 6 * axis)) & 63) - 32; }
__host__ __device__ __forceinline__ uint64_t tpWithPtr(uint64_t v, uint64_t ptr) { return (v & ~kPtrMask) | (ptr & kPtrMask); }

// encodeFixed64(level): ptr | permCode | sym, then (level+1)-bit z, y, x translations biased by 1 << level.
__host__ __device__ __forceinline__ uint64_t encodeFixed64(uint64_t ptr, uint32_t permId, uint32_t sym, int tx, int ty, int tz, uint32_t level)
{
    uint64_t out = ((ptr << 3 | permId) << 3) | sym;
    const uint32_t sb = level + 1;
    const int bias = 1 << level;
    out = (out << sb) | (uint64_t)(unsigned)(tz + bias);
    out = (out << sb) | (uint64_t)(unsigned)(ty + bias);
    out = (out << sb) | (uint64_t)(unsigned)(tx + bias);
    return out;
}
__host__ __device__ __forceinline__ uint64_t decodeFixed64(uint64_t e, uint32_t level)
{
    const uint32_t sb = level + 1;
    const uint64_t m = (1ull << sb) - 1;
    const int bias = 1 << level;
    const int tx = (int)(e & m) - bias;
    e >>= sb;
    const int ty = (int)(e & m) - bias;
    e >>= sb;
    const int tz = (int)(e & m) - bias;
    e >>= sb;
    const uint32_t sym = (uint32_t)(e & 7);
    e >>= 3;
    const uint32_t pc = (uint32_t)(e & 7);
    e >>= 3;
    return tpCreate(e, sym, pc, tx, ty, tz);
}

// ------------------------------------------------------------------------------------------------
// Transform algebra tables (computed on the host once; copied into shared memory by kernels).
// A transform t maps position v to P(v) ^ S, P(v) = (v[p0], v[p1], v[p2]).
// ------------------------------------------------------------------------------------------------
struct TransformTables {
    uint8_t compose[48][48]; // compose[a][b] = a ∘ b
    uint8_t inverse[48];
    uint8_t pos[48][8]; // image of a 2x2x2 child index
    uint8_t invPos[48][8]; // invPos[t][pos[t][i]] = i
    uint8_t byteMap[48][256]; // image of a 2x2x2 occupancy byte (bit i = child i)
};
const TransformTables& hostTables();

// ------------------------------------------------------------------------------------------------
// Context streams and device-memory budgets. A context's stream is owned by a StreamState that every
// buffer allocated on the stream shares, so buffers and results that outlive their context (and free
// themselves later) still free on a live stream; the stream is destroyed with its last user. A
// context created with tdag_tuning.device_memory_limit also charges every such buffer to its budget
// until the buffer is released; an allocation that would pass the limit throws TDAG_ERR_OOM before
// reaching the driver.
// ------------------------------------------------------------------------------------------------
struct StreamState {
    cudaStream_t stream = nullptr;
    uint64_t limit = 0; // 0: no budget
    std::atomic<uint64_t> used { 0 };
    ~StreamState(); // destroys the stream (its pending work completes first)
};
std::shared_ptr<StreamState> streamStateOf(cudaStream_t stream); // null: a stream no context owns
std::shared_ptr<StreamState> registerStream(cudaStream_t stream, uint64_t limit);
void unregisterStream(cudaStream_t stream);
void chargeBudget(StreamState& st, uint64_t bytes); // throws TDAG_ERR_OOM past the limit

// ------------------------------------------------------------------------------------------------
// Small device-memory helpers (stream-ordered allocations from the context's pool).
// ------------------------------------------------------------------------------------------------
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = 0;
    std::shared_ptr<StreamState> owner; // keeps the stream alive; carries the context's budget
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t stream)
        : n(count)
        , s(stream)
    {
        if (count) {
            owner = streamStateOf(stream);
            if (owner && owner->limit)
                chargeBudget(*owner, count * sizeof(T));
            const cudaError_t e = cudaMallocAsync((void**)&p, count * sizeof(T), stream);
            if (e != cudaSuccess) {
                p = nullptr;
                if (owner && owner->limit)
                    owner->used -= count * sizeof(T);
                owner.reset();
                TDAG_CUDA(e);
            }
        }
    }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
    DevBuf& operator=(DevBuf&& o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            s = o.s;
            owner = std::move(o.owner);
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void release()
    {
        if (p) {
            cudaFreeAsync(p, s);
            if (owner && owner->limit)
                owner->used -= n * sizeof(T);
        }
        owner.reset();
        p = nullptr;
        n = 0;
    }
    T* get() const { return p; }
    size_t bytes() const { return n * sizeof(T); }
};

inline unsigned gridFor(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

// ------------------------------------------------------------------------------------------------
// Primitives (primitives.cu): exclusive scan of u32, stable LSD radix sort of (u64 key, u32 value).
// ------------------------------------------------------------------------------------------------
void exclusiveScanU32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s);
// 64 bytes of pinned host memory owned by the calling host thread, for small device-to-host readbacks.
uint64_t* pinnedScratch();
// Returns total (sum of in) by copying the last element; synchronises the stream.
uint64_t exclusiveScanU32Total(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on bits [beginBit, endBit) of the key. With a status
// word, arrays of more than one tile take the one-sweep path (a look-back wait that gives up records
// TDAG_ERR_CUDA there); without one, the histogram / scan / scatter passes.
void radixSortPairs(uint64_t* keys, uint32_t* vals, size_t n, uint32_t beginBit, uint32_t endBit, cudaStream_t s, uint32_t* status = nullptr);
// Compact indices i in [0, n) with flags[i] != 0 into out (ascending); returns the count.
uint32_t compactFlags(const uint32_t* flags, uint32_t* out, size_t n, cudaStream_t s);
// The same with the device status word read in the same round trip (into hostStatus, 16 bytes):
// returns its error code; only when it is 0 are the indices compacted and *count set.
uint32_t compactFlagsChecked(const uint32_t* flags, uint32_t* out, size_t n, cudaStream_t s, uint32_t* status, uint32_t* hostStatus, uint32_t* count);

// ------------------------------------------------------------------------------------------------
// Host links of a build (primitives.cu). Every value a build reads back to steer itself (counts,
// totals, status words), every stream synchronisation it waits on and every host-to-device upload
// of host-computed data goes through these four calls. With no tape on the calling thread (the
// default) they copy and synchronise as they always did. A batch graph (tdag_batch_graph_create)
// builds once with a recording tape, which keeps every value read, the free device memory queried
// and every uploaded byte, and then captures the same build into a CUDA graph with a replaying
// tape: a read returns the recorded value and enqueues a device check that the replayed build
// computed the same value (a difference sets the tape's mismatch word), a synchronisation is
// dropped, and an upload comes from a device copy of the recorded bytes, so that the graph needs
// no host memory when it runs.
// ------------------------------------------------------------------------------------------------
struct HostRead {
    void* dst; // host
    const void* src; // device
    size_t bytes; // a multiple of 4
};
struct ControlTape {
    bool replay = false;
    std::string reads; // bytes of every read, in order
    size_t readPos = 0;
    std::string uploads; // bytes of every upload, in order
    size_t uploadPos = 0;
    const unsigned char* uploadsDev = nullptr; // device copy of `uploads` (replay)
    uint32_t* mismatch = nullptr; // device word (replay): 1 + the index of the first read that differed
    uint32_t readIndex = 0;
};
ControlTape* activeTape(); // the calling thread's tape, or null
void setActiveTape(ControlTape* tape);
inline bool replaying()
{
    const ControlTape* t = activeTape();
    return t && t->replay;
}
// Copies each item to the host and waits for them (replay: the recorded values, checked on the device).
void readToHost(std::initializer_list<HostRead> items, cudaStream_t s);
// Waits for the stream (replay: nothing; the graph's own order holds).
void syncHost(cudaStream_t s);
// Stream-ordered upload of host bytes (replay: from the device copy of the recorded bytes). Like
// cudaMemcpyAsync from pageable memory, `src` may be reused once the call returns.
void uploadToDevice(void* dst, const void* src, size_t bytes, cudaStream_t s);
// Free device memory (cudaMemGetInfo), recorded and replayed like a read.
uint64_t deviceFreeBytes();
// Loads the replay check's kernel now, so that no module loads while a stream is being captured.
void preloadTapeKernels();

// Statistics accumulated over one build (device counters for the matcher).
struct LevelStats {
    uint64_t items = 0, unique = 0, probes = 0, filterPass = 0, hits = 0, candidates = 0, verifications = 0, verified = 0, tableEntries = 0;
    float searchMs = 0;
};

} // namespace tdag
