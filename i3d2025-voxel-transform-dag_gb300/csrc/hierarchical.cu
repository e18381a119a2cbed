// hierarchical.cu — GPU symmetry + axis-permutation canonicalisation of an SVDAG, bottom-up.
//
// Restates constructTransformDAGHierarchical (tools/lib/src/voxel/transform_dag_hierarchical.cpp:304-523)
// without its sequential per-range search. The reference, per level:
//   1. groups nodes by a hash of their sorted child pointers and sorts (hash, index) (:365-378);
//   2. inside a group, in index order, a node becomes canonical unless some allowed transform, tried
//      in ID order 0..47, maps it onto an earlier canonical (:326-357, :403-414);
//   3. emits canonical nodes in (hash, index) order; a non-canonical node maps to
//      (handle(canonical), inverse(t)) (:343-344, :417-430).
// Equivalence under the allowed transforms is a content equality, so the canonical of a node is the
// smallest index of its equivalence class, and the group hash is a class invariant. This file
// computes an exact class signature per node (the lexicographic minimum of its transformed child
// codes), finds the class minimum with a bounded-probe hash table that compares full signatures,
// then finds the first transform ID that maps each node onto its canonical, exactly as step 2 does.
//
// Child codes: a child pointer (h, tau) with canonical invariance group Inv(h) is represented by
// (h, min ID of the coset tau * Inv(h)), which is equal for two pointers exactly when
// TaggedPointer::operator== (:79-122) says they are equal.
#include <cstdlib>
#include <utility>

#include "common.cuh"
#include "internal.cuh"
#include "class_table.cuh"

namespace tdag {

namespace {

constexpr int kThreads = 256;

struct SmemTables {
    uint8_t compose[48][48];
    uint8_t inverse[48];
    uint8_t pos[48][8];
    uint8_t invPos[48][8];
};

__device__ __forceinline__ void loadTables(SmemTables& s, const TransformTables* g)
{
    const uint8_t* src = &g->compose[0][0];
    uint8_t* dst = &s.compose[0][0];
    for (int i = threadIdx.x; i < 48 * 48; i += blockDim.x)
        dst[i] = src[i];
    for (int i = threadIdx.x; i < 48; i += blockDim.x)
        s.inverse[i] = g->inverse[i];
    for (int i = threadIdx.x; i < 48 * 8; i += blockDim.x) {
        (&s.pos[0][0])[i] = (&g->pos[0][0])[i];
        (&s.invPos[0][0])[i] = (&g->invPos[0][0])[i];
    }
}

// Transform of a 4x4x4 Morton mask: byte k is the 2x2x2 block at child position k; the transform
// moves it to pos[t][k] and maps its content with the 2x2x2 byte map.
__device__ __forceinline__ uint64_t transformLeaf(uint64_t m, uint32_t t, const uint8_t (*byteMap)[256], const uint8_t (*pos)[8])
{
    uint64_t out = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t b = (uint32_t)(m >> (8 * k)) & 0xFF;
        out |= (uint64_t)byteMap[t][b] << (8 * pos[t][k]);
    }
    return out;
}

__device__ __forceinline__ void compareExchange(uint64_t& a, uint64_t& b)
{
    const uint64_t lo = a < b ? a : b;
    b = a < b ? b : a;
    a = lo;
}

__device__ __forceinline__ uint64_t sortedPtrHash(uint64_t p[8])
{
    // sort the 8 child pointers ascending, then hash_combine over them (:365-377); a fixed
    // 19-comparator sorting network keeps the array in registers
    compareExchange(p[0], p[2]); compareExchange(p[1], p[3]); compareExchange(p[4], p[6]); compareExchange(p[5], p[7]);
    compareExchange(p[0], p[4]); compareExchange(p[1], p[5]); compareExchange(p[2], p[6]); compareExchange(p[3], p[7]);
    compareExchange(p[0], p[1]); compareExchange(p[2], p[3]); compareExchange(p[4], p[5]); compareExchange(p[6], p[7]);
    compareExchange(p[2], p[4]); compareExchange(p[3], p[5]);
    compareExchange(p[1], p[4]); compareExchange(p[3], p[6]);
    compareExchange(p[1], p[2]); compareExchange(p[3], p[4]); compareExchange(p[5], p[6]);
    uint64_t seed = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        seed = hashCombine(seed, p[i]);
    return seed;
}

// ---------------------------------------------------------------------------- leaves (level 2)
__global__ void __launch_bounds__(kThreads) leafSigKernel(const uint64_t* __restrict__ leaves, uint32_t n, const TransformTables* __restrict__ tables,
    const uint8_t* __restrict__ canonByte, uint64_t allowed, uint64_t* __restrict__ sig, uint64_t* __restrict__ key, const uint32_t* __restrict__ gridOf)
{
    __shared__ uint8_t byteMap[48][256];
    __shared__ uint8_t pos[48][8];
    __shared__ uint8_t cb[256];
    for (int i = threadIdx.x; i < 48 * 256; i += blockDim.x)
        (&byteMap[0][0])[i] = (&tables->byteMap[0][0])[i];
    for (int i = threadIdx.x; i < 48 * 8; i += blockDim.x)
        (&pos[0][0])[i] = (&tables->pos[0][0])[i];
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        cb[i] = canonByte[i];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint64_t m = leaves[i];
    uint64_t best = m;
    for (uint32_t t = 1; t < 48; ++t) {
        if (!((allowed >> t) & 1))
            continue;
        const uint64_t v = transformLeaf(m, t, byteMap, pos);
        best = v < best ? v : best;
    }
    if (gridOf) { // batched build: the grid id is part of the class key
        sig[2 * (size_t)i] = best;
        sig[2 * (size_t)i + 1] = gridOf[i];
    } else {
        sig[i] = best;
    }
    uint64_t p[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        p[k] = cb[(m >> (8 * k)) & 0xFF];
    key[i] = sortedPtrHash(p);
}

// For each leaf: canonical = class minimum; canonical leaves get their invariance mask, the others
// the first transform ID t with T_t(leaf) == canonical (transform_dag_hierarchical.cpp:329-355).
__global__ void __launch_bounds__(kThreads) leafResolveKernel(const uint64_t* __restrict__ leaves, uint32_t n, const TransformTables* __restrict__ tables,
    uint64_t allowed, const uint32_t* __restrict__ slotOf, const uint32_t* __restrict__ minIdx, uint32_t* __restrict__ canonOf,
    uint8_t* __restrict__ tOf, uint64_t* __restrict__ invOf, uint32_t* __restrict__ isCanon, uint32_t* status)
{
    __shared__ uint8_t byteMap[48][256];
    __shared__ uint8_t pos[48][8];
    for (int i = threadIdx.x; i < 48 * 256; i += blockDim.x)
        (&byteMap[0][0])[i] = (&tables->byteMap[0][0])[i];
    for (int i = threadIdx.x; i < 48 * 8; i += blockDim.x)
        (&pos[0][0])[i] = (&tables->pos[0][0])[i];
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t c = minIdx[slotOf[i]];
    const uint64_t m = leaves[i];
    canonOf[i] = c;
    if (c == i) {
        uint64_t inv = 0;
        for (uint32_t t = 0; t < 48; ++t)
            if (((allowed >> t) & 1) && transformLeaf(m, t, byteMap, pos) == m)
                inv |= 1ull << t;
        invOf[i] = inv;
        tOf[i] = 0;
        isCanon[i] = 1;
    } else {
        const uint64_t mc = leaves[c];
        uint32_t found = 0xFF;
        for (uint32_t t = 0; t < 48; ++t) {
            if (((allowed >> t) & 1) && transformLeaf(m, t, byteMap, pos) == mc) {
                found = t;
                break;
            }
        }
        if (found == 0xFF)
            setDeviceError(status, TDAG_ERR_CORRUPT, 2);
        tOf[i] = (uint8_t)(found == 0xFF ? 0 : found);
        isCanon[i] = 0;
    }
}

// ---------------------------------------------------------------------------- inner nodes
struct Child {
    uint32_t h; // handle at the level below (0xFFFFFFFF: empty)
    uint32_t tau; // transform ID of the child pointer
};

__device__ __forceinline__ Child loadChild(const uint32_t* __restrict__ node, int k, const uint64_t* __restrict__ prevMap)
{
    const uint32_t c = node[k];
    if (c == kEmpty32)
        return Child { kEmpty32, 0 };
    const uint64_t tp = prevMap[c];
    return Child { (uint32_t)tpPtr(tp), tpTransformId(tp) };
}

// Coset representatives of the level's kept nodes: rep[h * 48 + tau] = the smallest transform ID in
// tau ∘ Inv(h), Inv(h) the invariance group of canonical h. Two child pointers (h, tau), (h, tau')
// denote the same child exactly when their cosets agree (transform_dag_hierarchical.cpp:70-123).
__global__ void cosetRepKernel(const uint64_t* __restrict__ inv, uint32_t u, const TransformTables* __restrict__ tables, uint8_t* __restrict__ rep)
{
    __shared__ uint8_t compose[48][48];
    for (int i = threadIdx.x; i < 48 * 48; i += blockDim.x)
        (&compose[0][0])[i] = (&tables->compose[0][0])[i];
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)u * 48)
        return;
    const uint32_t h = (uint32_t)(i / 48), tau = (uint32_t)(i % 48);
    uint64_t bits = inv[h];
    uint32_t r = 63;
    while (bits) {
        const uint32_t g = __ffsll((long long)bits) - 1;
        bits &= bits - 1;
        r = compose[tau][g] < r ? compose[tau][g] : r;
    }
    rep[i] = (uint8_t)r;
}

// code of child (h, t ∘ tau) with coset normalisation
__device__ __forceinline__ uint64_t childCode(const Child& c, uint32_t t, const SmemTables& st, const uint8_t* __restrict__ rep)
{
    if (c.h == kEmpty32)
        return (uint64_t)kEmpty32 << 6;
    return ((uint64_t)c.h << 6) | __ldg(&rep[(size_t)c.h * 48 + st.compose[t][c.tau]]);
}

// A thread's 8 children, kept in shared memory so that they can be gathered by a runtime position
// (a register array indexed at run time would live in local memory).
struct ChildSlots {
    uint32_t h[8][kThreads];
    uint8_t tau[8][kThreads];
    __device__ void put(int k, const Child& c)
    {
        h[k][threadIdx.x] = c.h;
        tau[k][threadIdx.x] = (uint8_t)c.tau;
    }
    __device__ Child get(int k) const { return Child { h[k][threadIdx.x], tau[k][threadIdx.x] }; }
};

// Codes of the 8 children after transform t, in output position order: out[j] is the child that t
// moves to position j.
__device__ __forceinline__ void transformedCodes(const ChildSlots& cs, uint32_t t, const SmemTables& st, const uint8_t* __restrict__ rep, uint64_t out[8])
{
#pragma unroll
    for (int j = 0; j < 8; ++j)
        out[j] = childCode(cs.get(st.invPos[t][j]), t, st, rep);
}

// The identity's codes straight from registers (position j holds child j).
__device__ __forceinline__ void identityCodes(const Child ch[8], const SmemTables& st, const uint8_t* __restrict__ rep, uint64_t out[8])
{
#pragma unroll
    for (int j = 0; j < 8; ++j)
        out[j] = childCode(ch[j], 0, st, rep);
}

__device__ __forceinline__ bool lexLess(const uint64_t a[8], const uint64_t b[8])
{
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (a[k] != b[k])
            return a[k] < b[k];
    }
    return false;
}

// prevValue (optional, static input): the value hashed for a child handle h is prevValue[h], the
// word offset of that node in its packed level (transform_dag_hierarchical.cpp:597-606, 696-703).
__global__ void __launch_bounds__(kThreads) nodeSigKernel(const uint32_t* __restrict__ nodes, uint32_t n, const uint64_t* __restrict__ prevMap,
    const uint8_t* __restrict__ prevRep, const TransformTables* __restrict__ tables, uint64_t allowed, uint64_t* __restrict__ sig, uint64_t* __restrict__ key,
    const uint32_t* __restrict__ gridOf, const uint32_t* __restrict__ prevHandleOff, const uint32_t* __restrict__ prevValue)
{
    __shared__ SmemTables st;
    __shared__ ChildSlots cs;
    loadTables(st, tables);
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t* node = nodes + (size_t)i * 8;
    Child ch[8];
    uint64_t p[8];
    // the grouping key hashes the grid's own handles (a batch numbers handles across grids)
    const uint32_t hbase = gridOf ? prevHandleOff[gridOf[i]] : 0u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        ch[k] = loadChild(node, k, prevMap);
        cs.put(k, ch[k]);
        p[k] = ch[k].h == kEmpty32 ? (uint64_t)kEmpty32 : prevValue ? (uint64_t)prevValue[ch[k].h] : (uint64_t)(ch[k].h - hbase);
    }
    key[i] = sortedPtrHash(p);
    uint64_t best[8], cur[8];
    identityCodes(ch, st, prevRep, best);
    for (uint32_t t = 1; t < 48; ++t) {
        if (!((allowed >> t) & 1))
            continue;
        transformedCodes(cs, t, st, prevRep, cur);
        if (lexLess(cur, best)) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                best[k] = cur[k];
        }
    }
    uint64_t* out = sig + (size_t)i * (gridOf ? 9 : 8);
#pragma unroll
    for (int k = 0; k < 8; ++k)
        out[k] = best[k];
    if (gridOf) // batched build: the grid id is part of the class key
        out[8] = gridOf[i];
}

__global__ void __launch_bounds__(kThreads) nodeResolveKernel(const uint32_t* __restrict__ nodes, uint32_t n, const uint64_t* __restrict__ prevMap,
    const uint8_t* __restrict__ prevRep, const TransformTables* __restrict__ tables, uint64_t allowed, const uint32_t* __restrict__ slotOf,
    const uint32_t* __restrict__ minIdx, uint32_t* __restrict__ canonOf, uint8_t* __restrict__ tOf, uint64_t* __restrict__ invOf,
    uint32_t* __restrict__ isCanon, uint32_t level, uint32_t* status)
{
    __shared__ SmemTables st;
    __shared__ ChildSlots cs;
    loadTables(st, tables);
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t c = minIdx[slotOf[i]];
    canonOf[i] = c;
    Child ch[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        ch[k] = loadChild(nodes + (size_t)i * 8, k, prevMap);
        cs.put(k, ch[k]);
    }
    uint64_t target[8], cur[8];
    if (c == i) {
        identityCodes(ch, st, prevRep, target);
        uint64_t inv = 1; // identity
        for (uint32_t t = 1; t < 48; ++t) {
            if (!((allowed >> t) & 1))
                continue;
            transformedCodes(cs, t, st, prevRep, cur);
            bool eq = true;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                eq &= (cur[k] == target[k]);
            if (eq)
                inv |= 1ull << t;
        }
        invOf[i] = inv;
        tOf[i] = 0;
        isCanon[i] = 1;
    } else {
        Child cc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
            cc[k] = loadChild(nodes + (size_t)c * 8, k, prevMap);
        identityCodes(cc, st, prevRep, target);
        uint32_t found = 0xFF;
        for (uint32_t t = 0; t < 48; ++t) {
            if (!((allowed >> t) & 1))
                continue;
            transformedCodes(cs, t, st, prevRep, cur);
            bool eq = true;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                eq &= (cur[k] == target[k]);
            if (eq) {
                found = t;
                break;
            }
        }
        if (found == 0xFF)
            setDeviceError(status, TDAG_ERR_CORRUPT, level);
        tOf[i] = (uint8_t)(found == 0xFF ? 0 : found);
        isCanon[i] = 0;
    }
}

// ---------------------------------------------------------------------------- emission
__global__ void gatherSortInputKernel(const uint32_t* __restrict__ canonList, uint32_t u, const uint64_t* __restrict__ key, uint64_t* __restrict__ sk, uint32_t* __restrict__ sv)
{
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= u)
        return;
    const uint32_t idx = canonList[h];
    sk[h] = key[idx];
    sv[h] = idx;
}

__global__ void handleKernel(const uint32_t* __restrict__ emitOrder, uint32_t u, const uint64_t* __restrict__ invOf, uint32_t* __restrict__ handleOf, uint64_t* __restrict__ invOut)
{
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= u)
        return;
    const uint32_t idx = emitOrder[h];
    handleOf[idx] = h;
    invOut[h] = invOf[idx];
}

__global__ void mappingKernel(uint32_t n, const uint32_t* __restrict__ canonOf, const uint8_t* __restrict__ tOf, const uint32_t* __restrict__ handleOf,
    const TransformTables* __restrict__ tables, uint64_t* __restrict__ mapOut, uint32_t* __restrict__ midInv)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t c = canonOf[i];
    const uint32_t h = handleOf[c];
    const uint32_t t = (c == i) ? 0u : (uint32_t)tables->inverse[tOf[i]];
    mapOut[i] = tpCreateT(h, t);
    if (midInv && t == 0)
        atomicMax(&midInv[h], i); // storeMidLevelMapping keeps the last identity-mapped index (:312-320)
}

__global__ void emitLeavesKernel(const uint32_t* __restrict__ emitOrder, uint32_t u, const uint64_t* __restrict__ leaves, uint64_t* __restrict__ out)
{
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < u)
        out[h] = leaves[emitOrder[h]];
}

// Children are mapping pointers of the level below; in a batch their handles are made local to the
// node's grid (prevHandleOff = first handle of each grid at the level below).
__global__ void emitNodesKernel(const uint32_t* __restrict__ emitOrder, uint32_t u, const uint32_t* __restrict__ nodes, const uint64_t* __restrict__ prevMap,
    uint64_t* __restrict__ out, const uint32_t* __restrict__ gridOf, const uint32_t* __restrict__ prevHandleOff)
{
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (uint64_t)u * 8)
        return;
    const uint32_t h = (uint32_t)(gid >> 3), k = (uint32_t)(gid & 7);
    const uint32_t node = emitOrder[h];
    const uint32_t c = nodes[(size_t)node * 8 + k];
    if (c == kEmpty32) {
        out[gid] = tpSentinel();
        return;
    }
    uint64_t tp = prevMap[c];
    if (gridOf)
        tp = tpWithPtr(tp, tpPtr(tp) - prevHandleOff[gridOf[node]]);
    out[gid] = tp;
}

__global__ void gatherGridKeysKernel(const uint32_t* __restrict__ emitOrder, uint32_t u, const uint32_t* __restrict__ gridOf, uint64_t* __restrict__ gk)
{
    const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < u)
        gk[h] = gridOf[emitOrder[h]];
}

__global__ void fillU64Kernel(uint64_t* p, uint64_t v, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        p[i] = v;
}
__global__ void fillU32Kernel(uint32_t* p, uint32_t v, size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        p[i] = v;
}

uint64_t pow2AtLeast(uint64_t v)
{
    uint64_t p = 1;
    while (p < v)
        p <<= 1;
    return p;
}

} // namespace

void fillU64(uint64_t* p, uint64_t v, size_t n, cudaStream_t s)
{
    if (!n)
        return;
    fillU64Kernel<<<gridFor(n, 256), 256, 0, s>>>(p, v, n);
    TDAG_LAUNCHED();
}
void fillU32(uint32_t* p, uint32_t v, size_t n, cudaStream_t s)
{
    if (!n)
        return;
    fillU32Kernel<<<gridFor(n, 256), 256, 0, s>>>(p, v, n);
    TDAG_LAUNCHED();
}
void preloadFillKernels()
{
    cudaFuncAttributes fa;
    TDAG_CUDA(cudaFuncGetAttributes(&fa, fillU64Kernel));
    TDAG_CUDA(cudaFuncGetAttributes(&fa, fillU32Kernel));
}

// Shared tail of one level: class table -> canonicals -> emission order -> mapping.
// sigWords = 1 (leaves) or 8 (nodes). Produces mapping (n), inv per handle (u) and the emit order.
static uint32_t canonicaliseLevel(Context& ctx, uint32_t level, uint32_t n, const uint64_t* sig, int sigWords, const uint64_t* key,
    const std::function<void(const uint32_t*, const uint32_t*, uint32_t*, uint8_t*, uint64_t*, uint32_t*)>& resolve, DevBuf<uint64_t>& mapOut,
    DevBuf<uint64_t>& invOut, DevBuf<uint32_t>& emitOrder, DevBuf<uint32_t>* midInv, const uint32_t* gridOf, uint32_t numGrids,
    std::vector<uint64_t>& handleOff)
{
    cudaStream_t s = ctx.stream;
    DevBuf<uint32_t> canonOf(n, s), isCanon(n, s);
    DevBuf<uint8_t> tOf(n, s);
    DevBuf<uint64_t> invOf(n, s);
    // The class table's status and the number of canonical nodes come back in one round trip; a
    // table whose bounded probes ran out is doubled and the attempt rerun, as withClassTable does.
    auto attempt = [&](uint64_t cap) {
        DevBuf<uint64_t> slots(cap, s);
        DevBuf<uint32_t> minIdx(cap, s), slotOf(n, s);
        fillU64(slots.get(), kEmptySlot, cap, s);
        fillU32(minIdx.get(), 0xFFFFFFFFu, cap, s);
        if (sigWords == 1)
            classInsertKernel<1><<<gridFor(n, kThreads), kThreads, 0, s>>>(sig, n, slots.get(), minIdx.get(), slotOf.get(), cap - 1, ctx.status);
        else if (sigWords == 2)
            classInsertKernel<2><<<gridFor(n, kThreads), kThreads, 0, s>>>(sig, n, slots.get(), minIdx.get(), slotOf.get(), cap - 1, ctx.status);
        else if (sigWords == 8)
            classInsertKernel<8><<<gridFor(n, kThreads), kThreads, 0, s>>>(sig, n, slots.get(), minIdx.get(), slotOf.get(), cap - 1, ctx.status);
        else
            classInsertKernel<9><<<gridFor(n, kThreads), kThreads, 0, s>>>(sig, n, slots.get(), minIdx.get(), slotOf.get(), cap - 1, ctx.status);
        TDAG_LAUNCHED();
        slots.release();
        resolve(slotOf.get(), minIdx.get(), canonOf.get(), tOf.get(), invOf.get(), isCanon.get());
    };
    DevBuf<uint32_t> canonList(n, s);
    uint32_t u = 0;
    uint64_t cap = ctx.classTableCapacity(n);
    for (uint32_t regrows = 0;; ++regrows) {
        attempt(cap);
        const uint32_t code = compactFlagsChecked(isCanon.get(), canonList.get(), n, s, ctx.status, ctx.hostStatus, &u);
        if (code == 0)
            break;
        const uint32_t aux = ctx.hostStatus[1];
        TDAG_CUDA(cudaMemsetAsync(ctx.status, 0, 16, s));
        syncHost(s);
        if (code == TDAG_ERR_TABLE_FULL && regrows < ctx.tableRegrowLimit()) {
            cap *= 2;
            ++ctx.tableRegrows;
            continue;
        }
        throw Error((int)code, "hierarchical level " + std::to_string(level) + ": device reported error " + std::to_string(code) + " (aux " + std::to_string(aux) +
                ")" + (code == TDAG_ERR_TABLE_FULL ? " after " + std::to_string(regrows) + " table regrows" : std::string()));
    }
    isCanon.release();
    DevBuf<uint64_t> sk(u, s);
    emitOrder = DevBuf<uint32_t>(u, s);
    gatherSortInputKernel<<<gridFor(u, 256), 256, 0, s>>>(canonList.get(), u, key, sk.get(), emitOrder.get());
    TDAG_LAUNCHED();
    canonList.release();
    radixSortPairs(sk.get(), emitOrder.get(), u, 0, 64, s, ctx.status);
    if (gridOf && numGrids > 1) {
        // batched build: grid-major emission order, (grid, key, index), by a stable pass on the grid id
        gatherGridKeysKernel<<<gridFor(u, 256), 256, 0, s>>>(emitOrder.get(), u, gridOf, sk.get());
        TDAG_LAUNCHED();
        uint32_t bits = 8;
        while ((1ull << bits) < numGrids)
            bits += 8;
        radixSortPairs(sk.get(), emitOrder.get(), u, 0, bits, s, ctx.status);
        handleOff = countPerGrid(gridOf, emitOrder.get(), u, numGrids, s);
    } else {
        handleOff = { 0, u };
    }
    sk.release();

    DevBuf<uint32_t> handleOf(n, s);
    invOut = DevBuf<uint64_t>(u, s);
    handleKernel<<<gridFor(u, 256), 256, 0, s>>>(emitOrder.get(), u, invOf.get(), handleOf.get(), invOut.get());
    TDAG_LAUNCHED();
    mapOut = DevBuf<uint64_t>(n, s);
    uint32_t* mid = nullptr;
    if (midInv) {
        *midInv = DevBuf<uint32_t>(u, s);
        fillU32(midInv->get(), 0, u, s);
        mid = midInv->get();
    }
    mappingKernel<<<gridFor(n, 256), 256, 0, s>>>(n, canonOf.get(), tOf.get(), handleOf.get(), ctx.tables, mapOut.get(), mid);
    TDAG_LAUNCHED();
    return u;
}

namespace {
// Words of a packed node: one header plus one per present child (8 TransformPointers per node in).
__global__ void packedSizeKernel(const uint64_t* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ sizes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t w = 1;
    for (int k = 0; k < 8; ++k)
        w += nodes[(size_t)i * 8 + k] != tpSentinel() ? 1u : 0u;
    sizes[i] = w;
}
} // namespace

HierOutput runHierarchical(Context& ctx, const DeviceSvdag& in, const tdag_config& cfg, uint32_t midLevel, tdag_stats* stats)
{
    cudaStream_t s = ctx.stream;
    const uint64_t allowed = allowedMask(cfg);
    const TransformTables& ht = hostTables();
    // canonical 2x2x2 byte per occupancy byte: the smallest byte of its orbit under the allowed transforms
    uint8_t canonByte[256];
    for (uint32_t b = 0; b < 256; ++b) {
        uint32_t best = b;
        for (uint32_t t = 0; t < 48; ++t)
            if ((allowed >> t) & 1)
                best = ht.byteMap[t][b] < best ? ht.byteMap[t][b] : best;
        canonByte[b] = (uint8_t)best;
    }
    DevBuf<uint8_t> dCanonByte(256, s);
    uploadToDevice(dCanonByte.get(), canonByte, 256, s);

    HierOutput out;
    out.levels.resize(in.rootLevel + 1);
    out.handleOff.resize(in.rootLevel + 1);
    // per-level diagnostics on stderr (TDAG_TRACE): device time, items and kept items
    const bool trace = std::getenv("TDAG_TRACE") != nullptr && !replaying();
    std::vector<cudaEvent_t> traceEv;
    std::vector<std::pair<uint64_t, uint64_t>> traceCounts;
    auto traceMark = [&](uint64_t items, uint64_t kept) {
        if (!trace)
            return;
        cudaEvent_t e;
        TDAG_CUDA(cudaEventCreate(&e));
        TDAG_CUDA(cudaEventRecord(e, s));
        traceEv.push_back(e);
        traceCounts.emplace_back(items, kept);
    };
    traceMark(0, 0);
    DevBuf<uint64_t> prevMap, prevInv;
    DevBuf<uint8_t> prevRep; // coset representatives of the level below's kept nodes
    auto buildRep = [&](uint32_t u) {
        prevRep = DevBuf<uint8_t>((size_t)u * 48, s);
        if (u) {
            cosetRepKernel<<<gridFor((size_t)u * 48, 256), 256, 0, s>>>(prevInv.get(), u, ctx.tables, prevRep.get());
            TDAG_LAUNCHED();
        }
    };
    DevBuf<uint32_t> prevHandleOffDev;
    auto uploadOffsets = [&](const std::vector<uint64_t>& off) {
        DevBuf<uint32_t> d(off.size(), s);
        std::vector<uint32_t> o32(off.begin(), off.end());
        uploadToDevice(d.get(), o32.data(), o32.size() * 4, s);
        syncHost(s);
        return d;
    };
    {
        const uint32_t n = (uint32_t)in.leafCount;
        DevBuf<uint64_t> sig((size_t)n * (in.gridOf[2] ? 2 : 1), s), key(n, s);
        if (n) {
            leafSigKernel<<<gridFor(n, kThreads), kThreads, 0, s>>>(in.leaves, n, ctx.tables, dCanonByte.get(), allowed, sig.get(), key.get(), in.gridOf[2]);
            TDAG_LAUNCHED();
        }
        const uint64_t* leaves = in.leaves;
        auto resolve = [&](const uint32_t* slotOf, const uint32_t* minIdx, uint32_t* canonOf, uint8_t* tOf, uint64_t* invOf, uint32_t* isCanon) {
            leafResolveKernel<<<gridFor(n, kThreads), kThreads, 0, s>>>(leaves, n, ctx.tables, allowed, slotOf, minIdx, canonOf, tOf, invOf, isCanon, ctx.status);
            TDAG_LAUNCHED();
        };
        DevBuf<uint32_t> emitOrder;
        std::vector<uint64_t> hoff { 0, 0 };
        const uint32_t u = n ? canonicaliseLevel(ctx, 2, n, sig.get(), in.gridOf[2] ? 2 : 1, key.get(), resolve, prevMap, prevInv, emitOrder,
                                   midLevel == 2 ? &out.midInv : nullptr, in.gridOf[2], in.numGrids, hoff)
                             : 0;
        out.handleOff[2] = n ? hoff : std::vector<uint64_t>(in.numGrids + 1, 0);
        out.leaves = DevBuf<uint64_t>(u, s);
        if (u) {
            emitLeavesKernel<<<gridFor(u, 256), 256, 0, s>>>(emitOrder.get(), u, in.leaves, out.leaves.get());
            TDAG_LAUNCHED();
        }
        buildRep(u);
        if (stats) {
            stats->hierarchical[2].items = n;
            stats->hierarchical[2].unique = u;
        }
        traceMark(n, u);
    }
    DevBuf<uint32_t> prevWordOff; // static input: word offsets of the previous level's emitted nodes
    for (uint32_t level = 3; level <= in.rootLevel; ++level) {
        const uint32_t n = (uint32_t)in.nodeCounts[level];
        const uint32_t* nodes = in.nodes[level];
        const uint32_t* gridOf = in.gridOf[level];
        const int sw = gridOf ? 9 : 8;
        if (gridOf)
            prevHandleOffDev = uploadOffsets(out.handleOff[level - 1]);
        DevBuf<uint64_t> sig((size_t)n * sw, s), key(n, s);
        if (n) {
            nodeSigKernel<<<gridFor(n, kThreads), kThreads, 0, s>>>(nodes, n, prevMap.get(), prevRep.get(), ctx.tables, allowed, sig.get(), key.get(), gridOf,
                gridOf ? prevHandleOffDev.get() : nullptr, (in.staticOffsets && level >= 4) ? prevWordOff.get() : nullptr);
            TDAG_LAUNCHED();
        }
        const uint64_t* pm = prevMap.get();
        const uint8_t* pr = prevRep.get();
        auto resolve = [&](const uint32_t* slotOf, const uint32_t* minIdx, uint32_t* canonOf, uint8_t* tOf, uint64_t* invOf, uint32_t* isCanon) {
            nodeResolveKernel<<<gridFor(n, kThreads), kThreads, 0, s>>>(nodes, n, pm, pr, ctx.tables, allowed, slotOf, minIdx, canonOf, tOf, invOf, isCanon, level, ctx.status);
            TDAG_LAUNCHED();
        };
        DevBuf<uint64_t> map, inv;
        DevBuf<uint32_t> emitOrder;
        std::vector<uint64_t> hoff { 0, 0 };
        const uint32_t u = n ? canonicaliseLevel(ctx, level, n, sig.get(), sw, key.get(), resolve, map, inv, emitOrder, level == midLevel ? &out.midInv : nullptr,
                                   gridOf, in.numGrids, hoff)
                             : 0;
        out.handleOff[level] = n ? hoff : std::vector<uint64_t>(in.numGrids + 1, 0);
        sig.release();
        key.release();
        auto& lvl = out.levels[level];
        lvl = DevBuf<uint64_t>((size_t)u * 8, s);
        if (u) {
            emitNodesKernel<<<gridFor((size_t)u * 8, 256), 256, 0, s>>>(emitOrder.get(), u, nodes, prevMap.get(), lvl.get(), gridOf,
                gridOf ? prevHandleOffDev.get() : nullptr);
            TDAG_LAUNCHED();
        }
        prevMap = std::move(map);
        prevInv = std::move(inv);
        if (level < in.rootLevel)
            buildRep(u);
        if (in.staticOffsets && level < in.rootLevel) {
            // word offsets of this level's emitted nodes when packed (header + one word per child)
            DevBuf<uint32_t> sizes(std::max<uint32_t>(u, 1), s);
            prevWordOff = DevBuf<uint32_t>(std::max<uint32_t>(u, 1), s);
            if (u) {
                packedSizeKernel<<<gridFor(u, 256), 256, 0, s>>>(lvl.get(), u, sizes.get());
                TDAG_LAUNCHED();
                const uint64_t words = exclusiveScanU32Total(sizes.get(), prevWordOff.get(), u, s);
                TDAG_CHECK(words < 0xFFFFFFFFull, TDAG_ERR_ARG, "a packed level exceeds 2^32 words");
            }
        }
        if (stats) {
            stats->hierarchical[level].items = n;
            stats->hierarchical[level].unique = u;
        }
        traceMark(n, u);
    }
    if (trace) {
        TDAG_CUDA(cudaStreamSynchronize(s));
        std::string line = "[tdag] hierarchical ms (items -> kept):";
        for (size_t k = 1; k < traceEv.size(); ++k) {
            float ms = 0;
            TDAG_CUDA(cudaEventElapsedTime(&ms, traceEv[k - 1], traceEv[k]));
            char buf[96];
            std::snprintf(buf, sizeof buf, " L%zu %.3f (%llu -> %llu)", k + 1, ms, (unsigned long long)traceCounts[k].first,
                (unsigned long long)traceCounts[k].second);
            line += buf;
        }
        std::fprintf(stderr, "%s\n", line.c_str());
        for (auto e : traceEv)
            cudaEventDestroy(e);
    }
    return out;
}

} // namespace tdag
