// diag.cu — the L2 random-load ceiling of the translation probe kernel (tdag_diag.h).
//
// probeKernel tests every non-empty box hash against a membership filter of a few MB to a few tens
// of MB that stays in L2: one independent random 4-byte load per probe. This kernel does only that
// (multiplicative-hash word indices, eight loads in flight per thread, full occupancy), so its rate
// is the ceiling the probe kernel is measured against.
#include <functional>

#include "common.cuh"
#include "internal.cuh"
#include "tdag_diag.h"

namespace tdag {
namespace {

constexpr int kPeakThreads = 256;
constexpr int kPeakInFlight = 8;

__global__ void __launch_bounds__(kPeakThreads) l2ProbePeakKernel(const uint32_t* __restrict__ buf, uint32_t wordShift, uint32_t rounds,
    uint32_t* __restrict__ sink)
{
    uint32_t x = (blockIdx.x * blockDim.x + threadIdx.x) * 0x9E3779B9u + 0x7F4A7C15u;
    uint32_t acc = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint32_t w[kPeakInFlight];
#pragma unroll
        for (int c = 0; c < kPeakInFlight; ++c) {
            x = x * 1664525u + 1013904223u;
            w[c] = __ldg(&buf[(x * 0x9E3779B1u) >> wordShift]);
        }
#pragma unroll
        for (int c = 0; c < kPeakInFlight; ++c)
            acc += w[c];
    }
    if (acc == 0x5BD1E995u) // keeps the loads; practically never true
        sink[0] = acc;
}

} // namespace
} // namespace tdag

struct tdag_ctx;
tdag::Context& ctxOf(tdag_ctx* c); // build.cu
int guardedCall(const std::function<void()>& f); // build.cu
int failWith(int code, const char* msg); // build.cu

extern "C" int tdag_l2_probe_peak(tdag_ctx* ctx, uint64_t buffer_bytes, uint64_t loads, double* loads_per_s)
{
    using namespace tdag;
    if (!ctx || !loads_per_s)
        return failWith(TDAG_ERR_ARG, "null argument");
    if (buffer_bytes < 4096 || buffer_bytes > (1ull << 30) || (buffer_bytes & (buffer_bytes - 1)) || loads == 0)
        return failWith(TDAG_ERR_ARG, "buffer_bytes must be a power of two in 4 KiB .. 1 GiB, loads > 0");
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        cudaStream_t s = c.stream;
        const uint64_t words = buffer_bytes / 4;
        uint32_t log2Words = 0;
        while ((1ull << log2Words) < words)
            ++log2Words;
        DevBuf<uint32_t> buf(words, s), sink(1, s);
        TDAG_CUDA(cudaMemsetAsync(buf.get(), 0x11, buffer_bytes, s));
        int perSM = 0;
        TDAG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, l2ProbePeakKernel, kPeakThreads, 0));
        const uint64_t threads = (uint64_t)c.numSMs * std::max(perSM, 1) * kPeakThreads;
        const uint32_t rounds = (uint32_t)std::max<uint64_t>(1, (loads + threads * kPeakInFlight - 1) / (threads * kPeakInFlight));
        const unsigned blocks = (unsigned)(threads / kPeakThreads);
        l2ProbePeakKernel<<<blocks, kPeakThreads, 0, s>>>(buf.get(), 32 - log2Words, rounds, sink.get()); // warm-up: fills L2
        TDAG_LAUNCHED();
        TDAG_CUDA(cudaEventRecord(c.ev[5], s));
        l2ProbePeakKernel<<<blocks, kPeakThreads, 0, s>>>(buf.get(), 32 - log2Words, rounds, sink.get());
        TDAG_LAUNCHED();
        TDAG_CUDA(cudaEventRecord(c.ev[6], s));
        TDAG_CUDA(cudaEventSynchronize(c.ev[6]));
        float ms = 0;
        TDAG_CUDA(cudaEventElapsedTime(&ms, c.ev[5], c.ev[6]));
        *loads_per_s = (double)threads * rounds * kPeakInFlight / (ms / 1e3);
    });
}

extern "C" int tdag_device_pool_usage(tdag_ctx* ctx, uint64_t* used_bytes, uint64_t* reserved_bytes)
{
    using namespace tdag;
    if (!ctx || !used_bytes || !reserved_bytes)
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        cudaMemPool_t pool;
        TDAG_CUDA(cudaDeviceGetDefaultMemPool(&pool, c.device));
        uint64_t used = 0, reserved = 0; // the attributes are 64-bit values
        TDAG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
        TDAG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved));
        *used_bytes = used;
        *reserved_bytes = reserved;
    });
}
