// nn.cu — kernels of the learned source proposal (tdag_nn.h).
//
// Dense layers, InfoNCE logits and candidate scoring are bf16 GEMMs on the fifth-generation tensor
// cores: operands are staged by the CTA's threads into shared memory in the canonical no-swizzle
// K-major layout (8-row x 16-byte core matrices), one elected thread issues tcgen05.mma (kind::f16,
// M = 128, N <= 256, K = 16 per instruction) into an FP32 accumulator in tensor memory, completion is
// signalled through tcgen05.commit on an mbarrier, and the epilogue reads the accumulator back with
// tcgen05.ld (one TMEM lane per output row). Every wait is bounded; on a timeout the kernel records
// TDAG_ERR_CUDA in the context status, waits once more (bounded) for its MMAs, frees its tensor
// memory and returns.
#include <cuda_bf16.h>
#include <functional>

#include "common.cuh"
#include "internal.cuh"
#include "tdag_nn.h"

namespace tdag {
namespace {

constexpr int kGemmThreads = 128; // four warps: warp w reads TMEM lanes 32w .. 32w + 31
constexpr uint32_t kChunkK = 64;  // K per shared-memory stage: four MMAs of K = 16

// ---------------------------------------------------------------------------- primitives
__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
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
// Orders this thread's generic-proxy shared-memory writes before the tensor cores' (async-proxy) reads.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Tensor memory: allocated and freed by one whole warp.
__device__ __forceinline__ void tmemAlloc(uint32_t* slot, uint32_t cols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(slot)), "r"(cols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemFree(uint32_t taddr, uint32_t cols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: start address, leading-dimension byte offset (between
// core matrices adjacent along K), stride-dimension byte offset (between 8-row groups), version 1.
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t idescBf16(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}
__device__ __forceinline__ void tcMma(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
        "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The mbarrier receives one arrive when every MMA this thread issued before has completed.
__device__ __forceinline__ void tcCommit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar)) : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane (warp-wide; the wait is inside, so the
// registers are valid when the statement ends).
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
                 "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j)
        v[j] = __uint_as_float(r[j]);
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmemLoad32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, "
                 "%19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
                 "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
                 "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                 "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j)
        v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint16_t toBf16(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float fromBf16(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }
__device__ __forceinline__ uint32_t bitPair(uint64_t m, uint32_t k) // elements k, k + 1 of a mask as bf16 1.0 / 0.0
{
    return (((m >> k) & 1u) ? 0x3F80u : 0u) | ((((m >> (k + 1)) & 1u) ? 0x3F80u : 0u) << 16);
}

// ---------------------------------------------------------------------------- operand staging
// Byte offset of the 16-byte group g (elements k = 8g .. 8g + 7 of the stage) of tile row r, for a
// tile of `rows` rows: slab g / 2 holds one MMA's K = 16 (rows x 32 bytes), core matrix (r / 8, g % 2)
// inside it (128 bytes each, 8-row groups 256 bytes apart), row r % 8 inside that.
__device__ __forceinline__ uint32_t tileOffset(uint32_t r, uint32_t g, uint32_t rows)
{
    return (g >> 1) * rows * 32u + (r >> 3) * 256u + (g & 1u) * 128u + (r & 7u) * 16u;
}
constexpr uint32_t kLbo = 128, kSbo = 256;

// Stages rows r0 .. r0 + rows - 1 (zero past `limit`) and K elements k0 .. k0 + 63 (zero past K).
__device__ void stageTile(uint8_t* tile, const tdag_nn_operand& op, uint32_t rows, uint32_t r0, uint32_t limit, uint32_t k0, uint32_t K)
{
    for (uint32_t r = threadIdx.x; r < rows; r += kGemmThreads) {
        const uint32_t gr = r0 + r;
        const bool rowOk = gr < limit;
        uint64_t bits = 0;
        if (op.mode == TDAG_NN_BITS && rowOk)
            bits = static_cast<const uint64_t*>(op.ptr)[gr];
#pragma unroll
        for (uint32_t g = 0; g < kChunkK / 8; ++g) {
            const uint32_t k = k0 + 8 * g;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (rowOk && k < K) { // K is a multiple of 16: k + 8 <= K
                if (op.mode == TDAG_NN_KMAJOR) {
                    v = *reinterpret_cast<const uint4*>(static_cast<const uint16_t*>(op.ptr) + (size_t)gr * op.ld + k);
                } else if (op.mode == TDAG_NN_MNMAJOR) {
                    const uint16_t* p = static_cast<const uint16_t*>(op.ptr) + (size_t)k * op.ld + gr;
                    uint32_t w[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        w[j] = (uint32_t)p[(size_t)(2 * j) * op.ld] | ((uint32_t)p[(size_t)(2 * j + 1) * op.ld] << 16);
                    v = make_uint4(w[0], w[1], w[2], w[3]);
                } else if (op.mode == TDAG_NN_BITS) {
                    v = make_uint4(bitPair(bits, k), bitPair(bits, k + 2), bitPair(bits, k + 4), bitPair(bits, k + 6));
                } else { // TDAG_NN_BITS_T: bit gr of masks k .. k + 7
                    const uint64_t* p = static_cast<const uint64_t*>(op.ptr) + k;
                    uint32_t w[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        w[j] = (((p[2 * j] >> gr) & 1u) ? 0x3F80u : 0u) | ((((p[2 * j + 1] >> gr) & 1u) ? 0x3F80u : 0u) << 16);
                    v = make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
            *reinterpret_cast<uint4*>(tile + tileOffset(r, g, rows)) = v;
        }
    }
}

// Stages a K-major bf16 operand with exactly 32 columns (ld = 32): rows r0 .. r0 + rows - 1, zero
// past `limit`; two MMA slabs.
__device__ void stageTileK32(uint8_t* tile, const uint16_t* src, uint32_t rows, uint32_t r0, uint32_t limit)
{
    for (uint32_t i = threadIdx.x; i < rows * 4; i += kGemmThreads) {
        const uint32_t r = i >> 2, g = i & 3u, gr = r0 + r;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (gr < limit)
            v = *reinterpret_cast<const uint4*>(src + (size_t)gr * 32 + 8 * g);
        *reinterpret_cast<uint4*>(tile + tileOffset(r, g, rows)) = v;
    }
}

// ---------------------------------------------------------------------------- GEMM
struct GemmParams {
    tdag_nn_operand a, b;
    uint32_t M, N, K;
    float alpha;
    const float* bias;
    uint32_t relu;
    const uint16_t* gate;
    uint32_t ldGate;
    void* c;
    uint32_t ldc, cBf16;
    uint32_t* status;
};

template <uint32_t BN>
constexpr uint32_t gemmSmem()
{
    return 2 * (128 * kChunkK * 2 + BN * kChunkK * 2);
}

// One CTA computes the 128 x BN output tile (blockIdx.x = row tile, blockIdx.y = column tile). The two
// shared-memory stages alternate: the threads stage chunk c while the tensor cores run chunk c - 1.
template <uint32_t BN>
__global__ void __launch_bounds__(kGemmThreads) tcGemmKernel(GemmParams p)
{
    static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "tensor-memory columns are a power of two >= 32");
    constexpr uint32_t A_BYTES = 128 * kChunkK * 2, B_BYTES = BN * kChunkK * 2, STAGE = A_BYTES + B_BYTES;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmemSlot;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;

    if (warp == 0)
        tmemAlloc(&tmemSlot, BN);
    if (threadIdx.x == 0) {
        mbarInit(&bar[0], 1);
        mbarInit(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    const uint32_t tmem = tmemSlot;

    // split K (blockIdx.z of gridDim.z): this CTA's chunks are [c0, c0 + chunks); the partial tiles are
    // summed into C by atomic adds
    const uint32_t allChunks = (p.K + kChunkK - 1) / kChunkK;
    const uint32_t per = (allChunks + gridDim.z - 1) / gridDim.z;
    const uint32_t c0 = blockIdx.z * per;
    const uint32_t chunks = c0 < allChunks ? min(per, allChunks - c0) : 0u;
    bool ok = true;
    uint32_t issued = 0; // chunks whose MMAs were committed
    for (uint32_t c = 0; c < chunks; ++c) {
        const uint32_t st = c & 1u;
        uint8_t* tA = smem + st * STAGE;
        uint8_t* tB = tA + A_BYTES;
        if (c >= 2) { // the MMAs of chunk c - 2 read this stage
            const bool w = mbarWait(&bar[st], ((c >> 1) - 1) & 1u);
            if (!__syncthreads_and(w)) {
                ok = false;
                break;
            }
        }
        const uint32_t k0 = (c0 + c) * kChunkK;
        stageTile(tA, p.a, 128, m0, p.M, k0, p.K);
        stageTile(tB, p.b, BN, n0, p.N, k0, p.K);
        fenceProxyAsync();
        __syncthreads();
        if (threadIdx.x == 0) {
            tcFenceAfter();
            const uint32_t steps = min(4u, (p.K - k0) / 16u);
            for (uint32_t s = 0; s < steps; ++s) {
                const uint64_t da = smemDesc(smemAddr(tA) + s * 128u * 32u, kLbo, kSbo);
                const uint64_t db = smemDesc(smemAddr(tB) + s * BN * 32u, kLbo, kSbo);
                tcMma(tmem, da, db, idescBf16(128, BN), (c | s) != 0u);
            }
            tcCommit(&bar[st]);
        }
        issued = c + 1;
    }
    if (ok && chunks) {
        const uint32_t last = chunks - 1;
        ok = __syncthreads_and(mbarWait(&bar[last & 1u], (last >> 1) & 1u));
    }
    tcFenceAfter();
    if (ok && chunks) {
        const uint32_t row = warp * 32 + lane, gm = m0 + row;
        for (uint32_t cc = 0; cc < BN / 16; ++cc) {
            float v[16];
            tmemLoad16(tmem + ((warp * 32u) << 16) + cc * 16u, v);
            if (gm < p.M) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const uint32_t gn = n0 + cc * 16 + j;
                    if (gn >= p.N)
                        break;
                    float x = v[j] * p.alpha;
                    if (p.bias)
                        x += p.bias[gn];
                    if (p.relu)
                        x = fmaxf(x, 0.0f);
                    if (p.gate) {
                        const uint16_t g = p.gate[(size_t)gm * p.ldGate + gn];
                        if ((g & 0x8000u) || !(g & 0x7FFFu))
                            x = 0.0f;
                    }
                    if (gridDim.z > 1)
                        atomicAdd(&static_cast<float*>(p.c)[(size_t)gm * p.ldc + gn], x);
                    else if (p.cBf16)
                        static_cast<uint16_t*>(p.c)[(size_t)gm * p.ldc + gn] = toBf16(x);
                    else
                        static_cast<float*>(p.c)[(size_t)gm * p.ldc + gn] = x;
                }
            }
        }
    } else if (threadIdx.x == 0) {
        setDeviceError(p.status, TDAG_ERR_CUDA, 600);
        if (issued) // the last commit covers every MMA issued: let them land before freeing their memory
            mbarWait(&bar[(issued - 1) & 1u], ((issued - 1) >> 1) & 1u);
    }
    tcFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcFenceAfter();
        tmemFree(tmem, BN);
    }
}

// ---------------------------------------------------------------------------- top-k scoring
// A CTA scores 128 target rows against every earlier source row, 256 sources per MMA tile (K = 32:
// two MMAs), and keeps each row's k best in registers (thread = row = TMEM lane). Source tiles
// alternate between two shared-memory buffers and two 256-column accumulators, so the tensor cores
// score tile t + 1 while the threads scan tile t.
constexpr uint32_t kTopkTile = 256;

template <int KT>
__global__ void __launch_bounds__(kGemmThreads) topkKernel(const uint16_t* __restrict__ emb, uint32_t n, int32_t* __restrict__ outIdx,
    float* __restrict__ outScore, uint32_t* status)
{
    constexpr uint32_t A_BYTES = 128 * 32 * 2, B_BYTES = kTopkTile * 32 * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmemSlot;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t m0 = blockIdx.x * 128;
    uint8_t* tA = smem;
    uint8_t* tB0 = smem + A_BYTES;
    float* mine = reinterpret_cast<float*>(smem + A_BYTES + 2 * B_BYTES) + threadIdx.x * 33; // candidate scores (padded rows)

    if (warp == 0)
        tmemAlloc(&tmemSlot, 512);
    if (threadIdx.x == 0) {
        mbarInit(&bar[0], 1);
        mbarInit(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    const uint32_t tmem = tmemSlot;

    const uint32_t rowEnd = min(n, m0 + 128);
    const uint32_t tiles = (rowEnd - 1 + kTopkTile - 1) / kTopkTile; // sources 0 .. rowEnd - 2 can be chosen
    // stage this CTA's rows (K = 32 fits one stage: the upper half of the stage is never read)
    stageTileK32(tA, emb, 128, m0, n);
    float best[KT];
    int32_t bestIdx[KT];
#pragma unroll
    for (int s = 0; s < KT; ++s) {
        best[s] = -__int_as_float(0x7f800000);
        bestIdx[s] = -1;
    }
    float floorV = -__int_as_float(0x7f800000); // the smallest of best[]
    int floorAt = 0;
    const uint32_t row = warp * 32 + lane, gi = m0 + row;
    bool ok = true;
    auto issue = [&](uint32_t t) { // stage source tile t into buffer t & 1 and start its MMAs
        uint8_t* tB = tB0 + (t & 1u) * B_BYTES;
        stageTileK32(tB, emb, kTopkTile, t * kTopkTile, n);
        fenceProxyAsync();
        __syncthreads();
        if (threadIdx.x == 0) {
            tcFenceAfter();
            const uint32_t d = tmem + (t & 1u) * kTopkTile;
            for (uint32_t s = 0; s < 2; ++s)
                tcMma(d, smemDesc(smemAddr(tA) + s * 128u * 32u, kLbo, kSbo), smemDesc(smemAddr(tB) + s * kTopkTile * 32u, kLbo, kSbo),
                    idescBf16(128, kTopkTile), s);
            tcCommit(&bar[t & 1u]);
        }
    };
    if (tiles > 0)
        issue(0);
    uint32_t failedAt = 0;
    for (uint32_t t = 0; t < tiles; ++t) {
        ok = __syncthreads_and(mbarWait(&bar[t & 1u], (t >> 1) & 1u));
        if (!ok) {
            failedAt = t;
            break;
        }
        tcFenceAfter();
        // Buffer (t + 1) & 1 was read by the MMAs of tile t - 1, complete before tile t's (issued after them).
        if (t + 1 < tiles) {
            tcFenceBefore();
            issue(t + 1);
            tcFenceAfter();
        }
        const uint32_t j0 = t * kTopkTile;
        const bool diagonal = j0 + kTopkTile > m0; // the tile holds sources at or after some of the CTA's targets
        for (uint32_t cc = 0; cc < kTopkTile / 32; ++cc) {
            float v[32];
            tmemLoad32(tmem + ((warp * 32u) << 16) + (t & 1u) * kTopkTile + cc * 32u, v);
            const uint32_t jb = j0 + cc * 32;
            if (diagonal) {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (jb + j >= gi) // sources strictly before the target
                        v[j] = -__int_as_float(0x7f800000);
            }
            float mx = v[0];
#pragma unroll
            for (int j = 1; j < 32; ++j)
                mx = fmaxf(mx, v[j]);
            if (!__any_sync(0xffffffffu, mx > floorV)) // most chunks: no lane has a score above its k-th best
                continue;
            if (mx > floorV) {
                // the rare path, one candidate at a time through shared memory (a register array
                // indexed at run time would live in local memory)
                uint32_t cand = 0;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    mine[j] = v[j];
                    cand |= (v[j] > floorV ? 1u : 0u) << j;
                }
                while (cand) {
                    const int j = __ffs(cand) - 1;
                    cand &= cand - 1u;
                    const float x = mine[j];
                    if (x <= floorV) // the floor rose since the mask was taken
                        continue;
#pragma unroll
                    for (int s = 0; s < KT; ++s)
                        if (s == floorAt) {
                            best[s] = x;
                            bestIdx[s] = (int32_t)(jb + j);
                        }
                    floorV = best[0];
                    floorAt = 0;
#pragma unroll
                    for (int s = 1; s < KT; ++s)
                        if (best[s] < floorV) {
                            floorV = best[s];
                            floorAt = s;
                        }
                }
            }
        }
        tcFenceBefore();
        __syncthreads(); // every thread has read accumulator t & 1 before tile t + 2 overwrites it
    }
    if (!ok) {
        if (threadIdx.x == 0) { // the tile waited on is the last one issued: let its MMAs land before freeing their memory
            setDeviceError(status, TDAG_ERR_CUDA, 601);
            mbarWait(&bar[failedAt & 1u], (failedAt >> 1) & 1u);
        }
    } else if (gi < n) {
#pragma unroll
        for (int s = 0; s < KT; ++s) {
            outIdx[(size_t)gi * KT + s] = bestIdx[s];
            if (outScore)
                outScore[(size_t)gi * KT + s] = best[s];
        }
    }
    tcFenceBefore();
    __syncthreads();
    if (warp == 0) {
        tcFenceAfter();
        tmemFree(tmem, 512);
    }
}

// ---------------------------------------------------------------------------- small kernels
// Block masks of n items (one thread per block): the 4-bit runs along x of a 4^3 block never cross
// a 64-bit word of the item (their offset x + R y + R^2 z is a multiple of 4).
__global__ void blockMasksKernel(const uint64_t* __restrict__ words, uint32_t n, uint32_t level, uint64_t* __restrict__ masks)
{
    const uint32_t R = 1u << level, bs = R / 4, B = bs * bs * bs, W = R * R * R / 64;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)n * B)
        return;
    const uint32_t item = (uint32_t)(t / B), b = (uint32_t)(t % B);
    const uint32_t bx = b % bs, by = (b / bs) % bs, bz = b / (bs * bs);
    const uint64_t* g = words + (size_t)item * W;
    uint64_t m = 0;
    for (uint32_t dz = 0; dz < 4; ++dz)
        for (uint32_t dy = 0; dy < 4; ++dy) {
            const uint32_t off = 4 * bx + R * (4 * by + dy) + R * R * (4 * bz + dz);
            m |= ((g[off >> 6] >> (off & 63u)) & 0xFull) << (4 * dy + 16 * dz);
        }
    masks[t] = m;
}

__device__ __forceinline__ float warpSum(float v)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One warp per item, lane = embedding dimension.
// rowOf (optional) maps block (item, b) to its row of z (the MLP runs once per distinct mask).
__global__ void poolForwardKernel(const float* __restrict__ z, const uint32_t* __restrict__ rowOf, const uint64_t* __restrict__ masks, uint32_t n,
    uint32_t B, float* __restrict__ u, uint16_t* __restrict__ uBf16, float* __restrict__ norm, float* __restrict__ count)
{
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, d = threadIdx.x & 31;
    if (item >= n)
        return;
    float acc = 0.0f, cnt = 0.0f;
    for (uint32_t b = 0; b < B; ++b) {
        const size_t e = (size_t)item * B + b;
        if (masks[e]) {
            acc += z[(size_t)(rowOf ? rowOf[e] : e) * 32 + d];
            cnt += 1.0f;
        }
    }
    cnt = fmaxf(cnt, 1.0f);
    const float e = acc / cnt;
    const float len = fmaxf(sqrtf(warpSum(e * e)), 1e-12f);
    const float x = e / len;
    u[(size_t)item * 32 + d] = x;
    if (uBf16)
        uBf16[(size_t)item * 32 + d] = toBf16(x);
    if (d == 0) {
        norm[item] = len;
        count[item] = cnt;
    }
}

__global__ void poolBackwardKernel(const float* __restrict__ du, const float* __restrict__ u, const float* __restrict__ norm, const float* __restrict__ count,
    const uint64_t* __restrict__ masks, uint32_t n, uint32_t B, uint16_t* __restrict__ dz)
{
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, d = threadIdx.x & 31;
    if (item >= n)
        return;
    const float g = du[(size_t)item * 32 + d], x = u[(size_t)item * 32 + d];
    const float dot = warpSum(g * x);
    const float de = (g - x * dot) / norm[item] / count[item]; // through the normalisation, then the mean
    const uint16_t v = toBf16(de);
    for (uint32_t b = 0; b < B; ++b)
        dz[((size_t)item * B + b) * 32 + d] = masks[(size_t)item * B + b] ? v : (uint16_t)0;
}

// Log-sum-exp of every row (byCol = 0) or column (byCol = 1) of a b x b matrix, one block each.
__global__ void logSumExpKernel(const float* __restrict__ x, uint32_t b, uint32_t byCol, float* __restrict__ out)
{
    __shared__ float red[32];
    const uint32_t line = blockIdx.x;
    auto at = [&](uint32_t i) { return byCol ? x[(size_t)i * b + line] : x[(size_t)line * b + i]; };
    float mx = -__int_as_float(0x7f800000);
    for (uint32_t i = threadIdx.x; i < b; i += blockDim.x)
        mx = fmaxf(mx, at(i));
    for (int o = 16; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = red[0];
    for (uint32_t w = 1; w < blockDim.x / 32; ++w)
        mx = fmaxf(mx, red[w]);
    __syncthreads();
    float s = 0.0f;
    for (uint32_t i = threadIdx.x; i < b; i += blockDim.x)
        s += expf(at(i) - mx);
    s = warpSum(s);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (uint32_t w = 0; w < blockDim.x / 32; ++w)
            t += red[w];
        out[line] = mx + logf(t);
    }
}

// d loss / d logits of the symmetric InfoNCE: (softmax over the row + softmax over the column - 2 I) / (2b).
__global__ void infoNceGradKernel(const float* __restrict__ x, uint32_t b, const float* __restrict__ lseRow, const float* __restrict__ lseCol,
    uint16_t* __restrict__ dx)
{
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)b * b)
        return;
    const uint32_t i = (uint32_t)(t / b), j = (uint32_t)(t % b);
    const float v = x[t];
    const float g = (expf(v - lseRow[i]) + expf(v - lseCol[j]) - (i == j ? 2.0f : 0.0f)) * (0.5f / (float)b);
    dx[t] = toBf16(g);
}

__global__ void infoNceLossKernel(const float* __restrict__ x, uint32_t b, const float* __restrict__ lseRow, const float* __restrict__ lseCol,
    float* __restrict__ loss)
{
    float s = 0.0f;
    for (uint32_t i = threadIdx.x; i < b; i += blockDim.x)
        s += (lseRow[i] - x[(size_t)i * b + i]) + (lseCol[i] - x[(size_t)i * b + i]);
    __shared__ float red[32];
    s = warpSum(s);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (uint32_t w = 0; w < blockDim.x / 32; ++w)
            t += red[w];
        *loss = t * (0.5f / (float)b);
    }
}

// out[n] += sum of x[m][n] over this block's rows (out zeroed before).
constexpr uint32_t kSumRows = 256;
__global__ void columnSumsKernel(const uint16_t* __restrict__ x, uint32_t m, uint32_t n, uint32_t ldx, float* __restrict__ out)
{
    const uint32_t col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= n)
        return;
    const uint32_t r0 = blockIdx.y * kSumRows, r1 = min(m, r0 + kSumRows);
    float s = 0.0f;
    for (uint32_t r = r0; r < r1; ++r)
        s += fromBf16(x[(size_t)r * ldx + col]);
    atomicAdd(&out[col], s);
}

// AdamW (Loshchilov & Hutter): decoupled decay, then the bias-corrected Adam step.
__global__ void adamwKernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2, uint64_t count, float lr,
    float beta1, float beta2, float eps, float decay, float corr1, float corr2Sqrt, uint16_t* __restrict__ wBf16)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    const float gi = g[i];
    float x = w[i] * (1.0f - lr * decay);
    const float a = beta1 * m1[i] + (1.0f - beta1) * gi;
    const float v = beta2 * m2[i] + (1.0f - beta2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    x -= (lr / corr1) * a / (sqrtf(v) / corr2Sqrt + eps);
    w[i] = x;
    if (wBf16)
        wBf16[i] = toBf16(x);
}

// Canonical octant order of an item's eight children: with b the child occupancy byte, the first
// transform t (ID sym | perm << 3) whose image byteMap[t][b] is the smallest; child o goes to slot
// pos[t][o]. One warp per item, lane = embedding dimension.
__device__ __forceinline__ uint32_t canonTransform(const TransformTables* __restrict__ tt, uint32_t b)
{
    uint32_t best = 0, bestByte = 256;
    for (uint32_t t = 0; t < 48; ++t) {
        const uint32_t v = tt->byteMap[t][b];
        if (v < bestByte) {
            bestByte = v;
            best = t;
        }
    }
    return best;
}

// A child row at or past childRows is recorded as TDAG_ERR_ARG and read as an empty child.
__global__ void canonGatherKernel(const float* __restrict__ child, uint32_t childRows, const int32_t* __restrict__ childRow, uint32_t n,
    const TransformTables* __restrict__ tt, uint16_t* __restrict__ x, uint8_t* __restrict__ slotOf, uint32_t* status)
{
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, d = threadIdx.x & 31;
    if (item >= n)
        return;
    int32_t rows[8];
    uint32_t b = 0;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        rows[o] = childRow[(size_t)item * 8 + o];
        if (rows[o] >= 0 && (uint32_t)rows[o] >= childRows) {
            if (d == 0)
                setDeviceError(status, TDAG_ERR_ARG, 700);
            rows[o] = -1;
        }
        b |= (rows[o] >= 0 ? 1u : 0u) << o;
    }
    const uint32_t t = canonTransform(tt, b);
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        const uint32_t slot = tt->pos[t][o];
        const float v = rows[o] >= 0 ? child[(size_t)rows[o] * 32 + d] : 0.0f;
        x[(size_t)item * 256 + 32 * slot + d] = toBf16(v);
        if (d == 0)
            slotOf[(size_t)item * 8 + o] = (uint8_t)slot;
    }
}

__global__ void canonScatterKernel(const void* __restrict__ dx, int dxBf16, const int32_t* __restrict__ childRow, const uint8_t* __restrict__ slotOf,
    uint32_t n, float* __restrict__ dchild, uint32_t childRows, uint32_t* status)
{
    const uint32_t item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, d = threadIdx.x & 31;
    if (item >= n)
        return;
#pragma unroll
    for (int o = 0; o < 8; ++o) {
        const int32_t row = childRow[(size_t)item * 8 + o];
        if (row < 0)
            continue;
        if ((uint32_t)row >= childRows) {
            if (d == 0)
                setDeviceError(status, TDAG_ERR_ARG, 701);
            continue;
        }
        const size_t at = (size_t)item * 256 + 32 * slotOf[(size_t)item * 8 + o] + d;
        const float g = dxBf16 ? __bfloat162float(__ushort_as_bfloat16(static_cast<const uint16_t*>(dx)[at])) : static_cast<const float*>(dx)[at];
        atomicAdd(&dchild[(size_t)row * 32 + d], g);
    }
}

__global__ void toBf16Kernel(const float* __restrict__ x, uint64_t n, uint16_t* __restrict__ out)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = toBf16(x[i]);
}

unsigned gridOf(uint64_t work, unsigned threads) { return (unsigned)std::max<uint64_t>(1, (work + threads - 1) / threads); }

// Few output tiles over a long K (the weight gradients: 256 x 256 outputs, K = the batch's block
// rows) split K across CTAs until about two CTAs run per SM, each split at least 8 chunks long; the
// partial tiles are added into the zeroed FP32 output. Only for a plain FP32 epilogue.
template <uint32_t BN>
void launchGemm(const GemmParams& p, cudaStream_t s, int smCount)
{
    constexpr uint32_t smem = gemmSmem<BN>();
    TDAG_CUDA(cudaFuncSetAttribute(tcGemmKernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const uint32_t tiles = ((p.M + 127) / 128) * ((p.N + BN - 1) / BN);
    const uint32_t chunks = (p.K + kChunkK - 1) / kChunkK;
    uint32_t splits = 1;
    if (!p.cBf16 && !p.bias && !p.relu && !p.gate)
        splits = std::max<uint32_t>(1, std::min<uint32_t>(chunks / 8, (uint32_t)(2 * smCount) / std::max<uint32_t>(1, tiles)));
    if (splits > 1) {
        const uint32_t per = (chunks + splits - 1) / splits;
        splits = (chunks + per - 1) / per; // no empty split
        TDAG_CUDA(cudaMemset2DAsync(p.c, (size_t)p.ldc * 4, 0, (size_t)p.N * 4, p.M, s));
    }
    const dim3 grid((p.M + 127) / 128, (p.N + BN - 1) / BN, splits);
    TDAG_CHECK(grid.y <= 65535u && grid.z <= 65535u, TDAG_ERR_ARG, "tdag_nn_gemm: N too large for one launch");
    tcGemmKernel<BN><<<grid, kGemmThreads, smem, s>>>(p);
    TDAG_LAUNCHED();
}

template <int KT>
void launchTopk(const uint16_t* emb, uint32_t n, int32_t* idx, float* score, uint32_t* status, cudaStream_t s)
{
    // 57 KB are used; asking for 120 KB keeps one CTA per SM, the one whose 512 tensor-memory columns
    // fit (a second CTA would wait in tcgen05.alloc until the first has finished)
    constexpr uint32_t smem = 120 * 1024;
    static_assert(smem >= 128 * 32 * 2 + 2 * kTopkTile * 32 * 2 + kGemmThreads * 33 * 4, "top-k tiles and candidate rows");
    TDAG_CUDA(cudaFuncSetAttribute(topkKernel<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    topkKernel<KT><<<(n + 127) / 128, kGemmThreads, smem, s>>>(emb, n, idx, score, status);
    TDAG_LAUNCHED();
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

void checkOperand(const tdag_nn_operand* o, uint32_t rows, uint32_t k)
{
    TDAG_CHECK(o && o->ptr, TDAG_ERR_ARG, "null GEMM operand");
    switch (o->mode) {
    case TDAG_NN_KMAJOR:
        TDAG_CHECK(aligned16(o->ptr) && o->ld % 8 == 0 && o->ld >= k, TDAG_ERR_ARG, "K-major operand: 16-byte aligned, ld % 8 == 0, ld >= K");
        break;
    case TDAG_NN_MNMAJOR:
        TDAG_CHECK(o->ld >= rows, TDAG_ERR_ARG, "MN-major operand: ld >= rows");
        break;
    case TDAG_NN_BITS:
        TDAG_CHECK(k == 64, TDAG_ERR_ARG, "bit-mask operand: K == 64");
        break;
    case TDAG_NN_BITS_T:
        TDAG_CHECK(rows <= 64, TDAG_ERR_ARG, "transposed bit-mask operand: at most 64 rows");
        break;
    default:
        TDAG_CHECK(false, TDAG_ERR_ARG, "unknown operand mode");
    }
}

} // namespace
} // namespace tdag

struct tdag_ctx;
tdag::Context& ctxOf(tdag_ctx* c); // build.cu
int guardedCall(const std::function<void()>& f); // build.cu
int failWith(int code, const char* msg); // build.cu

extern "C" {

int tdag_nn_gemm(tdag_ctx* ctx, const tdag_nn_operand* a, const tdag_nn_operand* b, uint32_t m, uint32_t n, uint32_t k, float alpha,
    const float* bias, int relu, const uint16_t* gate, uint32_t ld_gate, void* c, uint32_t ldc, int c_bf16)
{
    using namespace tdag;
    if (!ctx || !c || m == 0 || n == 0 || k == 0 || k % 16 != 0 || ldc < n || (gate && ld_gate < n))
        return failWith(TDAG_ERR_ARG, "tdag_nn_gemm: null pointer, empty shape, K not a multiple of 16 or a leading dimension too small");
    return guardedCall([&] {
        checkOperand(a, m, k);
        checkOperand(b, n, k);
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        GemmParams p {};
        p.a = *a;
        p.b = *b;
        p.M = m;
        p.N = n;
        p.K = k;
        p.alpha = alpha;
        p.bias = bias;
        p.relu = relu ? 1u : 0u;
        p.gate = gate;
        p.ldGate = ld_gate;
        p.c = c;
        p.ldc = ldc;
        p.cBf16 = c_bf16 ? 1u : 0u;
        p.status = cx.status;
        int sms = 0;
        TDAG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cx.device));
        if (n <= 32)
            launchGemm<32>(p, cx.stream, sms);
        else if (n <= 64)
            launchGemm<64>(p, cx.stream, sms);
        else if (n <= 128)
            launchGemm<128>(p, cx.stream, sms);
        else
            launchGemm<256>(p, cx.stream, sms);
    });
}

int tdag_nn_block_masks(tdag_ctx* ctx, const uint64_t* words, uint32_t n, uint32_t level, uint64_t* masks)
{
    using namespace tdag;
    if (!ctx || (n && (!words || !masks)) || level < 2 || level > 4)
        return failWith(TDAG_ERR_ARG, "tdag_nn_block_masks: null pointer or level outside 2..4");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        const uint32_t bs = (1u << level) / 4;
        const uint64_t work = (uint64_t)n * bs * bs * bs;
        if (work) {
            blockMasksKernel<<<gridOf(work, 256), 256, 0, cx.stream>>>(words, n, level, masks);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_pool_forward(tdag_ctx* ctx, const float* z, const uint32_t* row_of, const uint64_t* masks, uint32_t n, uint32_t blocks, float* u,
    uint16_t* u_bf16, float* norm, float* count)
{
    using namespace tdag;
    if (!ctx || (n && (!z || !masks || !u || !norm || !count)) || blocks == 0)
        return failWith(TDAG_ERR_ARG, "tdag_nn_pool_forward: null pointer or no blocks");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        if (n) {
            poolForwardKernel<<<gridOf((uint64_t)n * 32, 256), 256, 0, cx.stream>>>(z, row_of, masks, n, blocks, u, u_bf16, norm, count);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_pool_backward(tdag_ctx* ctx, const float* du, const float* u, const float* norm, const float* count, const uint64_t* masks,
    uint32_t n, uint32_t blocks, uint16_t* dz)
{
    using namespace tdag;
    if (!ctx || (n && (!du || !u || !norm || !count || !masks || !dz)) || blocks == 0)
        return failWith(TDAG_ERR_ARG, "tdag_nn_pool_backward: null pointer or no blocks");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        if (n) {
            poolBackwardKernel<<<gridOf((uint64_t)n * 32, 256), 256, 0, cx.stream>>>(du, u, norm, count, masks, n, blocks, dz);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_info_nce(tdag_ctx* ctx, const float* logits, uint32_t b, float* loss_dev, uint16_t* dlogits)
{
    using namespace tdag;
    if (!ctx || !logits || !loss_dev || !dlogits || b == 0)
        return failWith(TDAG_ERR_ARG, "tdag_nn_info_nce: null pointer or empty batch");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        cudaStream_t s = cx.stream;
        DevBuf<float> lse(2 * (size_t)b, s);
        logSumExpKernel<<<b, 256, 0, s>>>(logits, b, 0, lse.get());
        TDAG_LAUNCHED();
        logSumExpKernel<<<b, 256, 0, s>>>(logits, b, 1, lse.get() + b);
        TDAG_LAUNCHED();
        infoNceGradKernel<<<gridOf((uint64_t)b * b, 256), 256, 0, s>>>(logits, b, lse.get(), lse.get() + b, dlogits);
        TDAG_LAUNCHED();
        infoNceLossKernel<<<1, 256, 0, s>>>(logits, b, lse.get(), lse.get() + b, loss_dev);
        TDAG_LAUNCHED();
    });
}

int tdag_nn_column_sums(tdag_ctx* ctx, const uint16_t* x, uint32_t m, uint32_t n, uint32_t ldx, float* out)
{
    using namespace tdag;
    if (!ctx || !out || (m && !x) || n == 0 || ldx < n)
        return failWith(TDAG_ERR_ARG, "tdag_nn_column_sums: null pointer, no columns or ldx < n");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        TDAG_CUDA(cudaMemsetAsync(out, 0, (size_t)n * sizeof(float), cx.stream));
        if (m) {
            const dim3 grid((n + 127) / 128, (m + kSumRows - 1) / kSumRows);
            columnSumsKernel<<<grid, 128, 0, cx.stream>>>(x, m, n, ldx, out);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_adamw(tdag_ctx* ctx, float* w, const float* grad, float* m1, float* m2, uint64_t count, float lr, float beta1, float beta2,
    float eps, float weight_decay, uint32_t step, uint16_t* w_bf16)
{
    using namespace tdag;
    if (!ctx || (count && (!w || !grad || !m1 || !m2)) || step == 0)
        return failWith(TDAG_ERR_ARG, "tdag_nn_adamw: null pointer or step 0");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        const float corr1 = 1.0f - std::pow(beta1, (float)step);
        const float corr2Sqrt = std::sqrt(1.0f - std::pow(beta2, (float)step));
        if (count) {
            adamwKernel<<<gridOf(count, 256), 256, 0, cx.stream>>>(w, grad, m1, m2, count, lr, beta1, beta2, eps, weight_decay, corr1, corr2Sqrt,
                w_bf16);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_topk(tdag_ctx* ctx, const uint16_t* emb, uint32_t n, uint32_t k, int32_t* idx, float* score)
{
    using namespace tdag;
    if (!ctx || (n && (!emb || !idx)) || (k != 8 && k != 16 && k != 32) || (n && !aligned16(emb)))
        return failWith(TDAG_ERR_ARG, "tdag_nn_topk: null or unaligned pointer, or k not 8, 16 or 32");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        if (!n)
            return;
        if (k == 8)
            launchTopk<8>(emb, n, idx, score, cx.status, cx.stream);
        else if (k == 16)
            launchTopk<16>(emb, n, idx, score, cx.status, cx.stream);
        else
            launchTopk<32>(emb, n, idx, score, cx.status, cx.stream);
    });
}

int tdag_nn_to_bf16(tdag_ctx* ctx, const float* x, uint64_t n, uint16_t* out)
{
    using namespace tdag;
    if (!ctx || (n && (!x || !out)))
        return failWith(TDAG_ERR_ARG, "tdag_nn_to_bf16: null pointer");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        if (n) {
            toBf16Kernel<<<gridOf(n, 256), 256, 0, cx.stream>>>(x, n, out);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_canon_gather(tdag_ctx* ctx, const float* child, uint32_t child_rows, const int32_t* child_row, uint32_t n, uint16_t* x, uint8_t* slot_of)
{
    using namespace tdag;
    if (!ctx || (n && (!child_row || !x || !slot_of || (child_rows && !child))))
        return failWith(TDAG_ERR_ARG, "tdag_nn_canon_gather: null pointer");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        if (n) {
            canonGatherKernel<<<gridOf((uint64_t)n * 32, 256), 256, 0, cx.stream>>>(child, child_rows, child_row, n, cx.tables, x, slot_of, cx.status);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_canon_scatter(tdag_ctx* ctx, const void* dx, int dx_bf16, const int32_t* child_row, const uint8_t* slot_of, uint32_t n, float* dchild,
    uint32_t child_rows)
{
    using namespace tdag;
    if (!ctx || (n && (!dx || !child_row || !slot_of || (child_rows && !dchild))))
        return failWith(TDAG_ERR_ARG, "tdag_nn_canon_scatter: null pointer");
    return guardedCall([&] {
        Context& cx = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(cx.device));
        if (n) {
            canonScatterKernel<<<gridOf((uint64_t)n * 32, 256), 256, 0, cx.stream>>>(dx, dx_bf16, child_row, slot_of, n, dchild, child_rows, cx.status);
            TDAG_LAUNCHED();
        }
    });
}

int tdag_nn_sync(tdag_ctx* ctx)
{
    using namespace tdag;
    if (!ctx)
        return failWith(TDAG_ERR_ARG, "tdag_nn_sync: null context");
    return guardedCall([&] { ctxOf(ctx).checkStatus("learned-proposal kernels"); });
}

} // extern "C"
