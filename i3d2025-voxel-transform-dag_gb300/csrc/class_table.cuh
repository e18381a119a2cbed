// class_table.cuh — bounded-probe hash table that assigns every item the smallest index of the
// items with an identical W-word key (first occurrence). Used by the hierarchical pass (keys =
// class signatures) and by toDAG (keys = node / leaf contents).
#pragma once
#include "common.cuh"

namespace tdag {

constexpr uint64_t kEmptySlot = ~0ull;

// Slot = tag << 32 | claimer index. A node belongs to a slot when its full signature equals the
// claimer's. minIdx[slot] collects the class minimum. Probing is bounded by the capacity.
template <int W>
__global__ void __launch_bounds__(256) classInsertKernel(const uint64_t* __restrict__ sig, uint32_t n, uint64_t* __restrict__ slots,
    uint32_t* __restrict__ minIdx, uint32_t* __restrict__ slotOf, uint64_t capMask, uint32_t* status)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint64_t s[W];
    uint64_t fp = 0x5bd1e995ull;
#pragma unroll
    for (int k = 0; k < W; ++k) {
        s[k] = sig[(size_t)i * W + k];
        fp = mix64(fp ^ s[k]);
    }
    const uint32_t tag = (uint32_t)(fp >> 32);
    uint64_t slot = fp & capMask;
    for (uint64_t probe = 0; probe <= capMask; ++probe) {
        uint64_t cur = slots[slot];
        if (cur == kEmptySlot) {
            const uint64_t mine = ((uint64_t)tag << 32) | i;
            cur = atomicCAS((unsigned long long*)&slots[slot], (unsigned long long)kEmptySlot, (unsigned long long)mine);
            if (cur == kEmptySlot) {
                slotOf[i] = (uint32_t)slot;
                atomicMin(&minIdx[slot], i);
                return;
            }
        }
        if ((uint32_t)(cur >> 32) == tag) {
            const uint32_t j = (uint32_t)cur;
            bool eq = true;
#pragma unroll
            for (int k = 0; k < W; ++k)
                eq &= (sig[(size_t)j * W + k] == s[k]);
            if (eq) {
                slotOf[i] = (uint32_t)slot;
                atomicMin(&minIdx[slot], i);
                return;
            }
        }
        slot = (slot + 1) & capMask;
    }
    // Every slot is claimed (the probe visited all of them): name the home slot, whose class minimum
    // is a valid item, so that the kernels reading slotOf before the host sees the status stay in
    // bounds. The pass's results are discarded and it is rerun with a larger table.
    slotOf[i] = (uint32_t)(fp & capMask);
    setDeviceError(status, TDAG_ERR_TABLE_FULL, 100);
}


} // namespace tdag
