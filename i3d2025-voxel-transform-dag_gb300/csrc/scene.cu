// scene.cu — device-side input pipeline: procedural scenes, SVO construction, toDAG.
//
//  * Scenes (no reference counterpart; the reference voxelises meshes, which are not available here):
//    an integer-only fBm value-noise terrain (solid where fbm - z/res > 0) and a seeded union of boxes,
//    spheres and terrain blocks, 30% of them transformed copies of earlier ones, reduced to its
//    1-voxel surface shell. Evaluated per 32^3 brick with a 1-voxel halo; rows of 34 voxels are
//    built analytically for boxes and spheres and per voxel for terrain blocks.
//  * SVO build: restates EditStructure(VoxelGrid) (tools/lib/include/voxcom/voxel/structure.h:423-429,
//    658-701). Its depth-first recursion over Morton child order emits, per level, the non-empty cells
//    in increasing Morton order, so the device build sorts nothing: non-empty leaves are compacted
//    from a Morton-indexed array, and each level is the run-length compaction of the level below.
//  * toDAG: restates EditStructure::toDAG (structure.h:703-763): per level, bottom-up, every item maps
//    to the first occurrence of its content; first occurrences keep their order.
#include <algorithm>
#include <array>
#include <map>
#include <cstring>
#include <memory>
#include <vector>

#include "class_table.cuh"
#include "slab_hash.cuh"
#include "common.cuh"
#include "internal.cuh"

namespace tdag {

// Checkpointing of the streamed scene build (tdag_scene_svdag_checkpointed): the file, a checkpoint
// every `every` finished chunks (0: none), and a stop after `stop_after` chunks of this call (0: none;
// the build then writes its checkpoint and fails with TDAG_ERR_INTERRUPTED).
struct StreamCheckpoint {
    const char* path;
    uint32_t every;
    uint32_t stop_after;
};

struct SvdagOwned {
    uint32_t resolution = 0, rootLevel = 0, structureType = 0;
    std::vector<DevBuf<uint32_t>> nodes;
    DevBuf<uint64_t> leaves;
    uint64_t voxelCount = 0;
};

namespace {

// ------------------------------------------------------------------------------------------------
// fBm value noise, integer only (identical to the CPU statement used by the tests).
// ------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t h)
{
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}
__host__ __device__ __forceinline__ uint32_t latticeValue(int64_t ix, int64_t iy, int64_t iz, uint32_t octave, uint32_t seed)
{
    uint32_t h = seed * 0x9E3779B1u + octave * 0x85EBCA77u;
    h = mix32(h ^ ((uint32_t)ix * 0x27D4EB2Fu));
    h = mix32(h ^ ((uint32_t)iy * 0x165667B1u));
    h = mix32(h ^ ((uint32_t)iz * 0xD3A2646Du));
    return h >> 16;
}
__host__ __device__ __forceinline__ int64_t smoothWeight(int64_t a, int64_t cell)
{
    const int64_t num = 2 * a + 1, den = 2 * cell;
    return (num * num * (3 * den - 2 * num) * 65536) / (den * den * den);
}
__host__ __device__ __forceinline__ int64_t lerpQ16(int64_t a, int64_t b, int64_t w) { return (a * (65536 - w) + b * w) >> 16; }

__host__ __device__ inline int64_t fbmValue(int64_t x, int64_t y, int64_t z, uint32_t seed)
{
    int64_t total = 0;
    for (uint32_t o = 0; o < 5; ++o) {
        const int64_t cell = 64 >> o;
        const int64_t ix = x / cell, iy = y / cell, iz = z / cell;
        const int64_t wx = smoothWeight(x % cell, cell), wy = smoothWeight(y % cell, cell), wz = smoothWeight(z % cell, cell);
        const int64_t x00 = lerpQ16(latticeValue(ix, iy, iz, o, seed), latticeValue(ix + 1, iy, iz, o, seed), wx);
        const int64_t x10 = lerpQ16(latticeValue(ix, iy + 1, iz, o, seed), latticeValue(ix + 1, iy + 1, iz, o, seed), wx);
        const int64_t x01 = lerpQ16(latticeValue(ix, iy, iz + 1, o, seed), latticeValue(ix + 1, iy, iz + 1, o, seed), wx);
        const int64_t x11 = lerpQ16(latticeValue(ix, iy + 1, iz + 1, o, seed), latticeValue(ix + 1, iy + 1, iz + 1, o, seed), wx);
        total += lerpQ16(lerpQ16(x00, x10, wy), lerpQ16(x01, x11, wy), wz) * (16 >> o);
    }
    return total;
}

// ------------------------------------------------------------------------------------------------
// Primitive evaluation
// ------------------------------------------------------------------------------------------------
struct DevPrim {
    int32_t type, perm, mirror, radius;
    int32_t size[3]; // local extent
    int32_t ext[3]; // world extent along each world axis = size[perm[k]]
    int32_t lo[3]; // world offset (minimum corner)
    uint32_t seed, pbits, pad;
};

__device__ __forceinline__ bool terrainInside(const DevPrim& p, int vx, int vy, int vz)
{
    int w[3] = { vx - p.lo[0], vy - p.lo[1], vz - p.lo[2] };
    int u[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if ((p.mirror >> k) & 1)
            w[k] = p.ext[k] - 1 - w[k];
        u[(p.pbits >> (2 * k)) & 3] = w[k];
    }
    return fbmValue(u[0], u[1], u[2], p.seed) * p.size[0] > (int64_t)u[2] * 31 * 65535;
}

// integer square root: largest r with r*r <= v (v >= 0)
__device__ __forceinline__ int isqrt64(int64_t v)
{
    int r = (int)sqrt((double)v);
    while ((int64_t)r * r > v)
        --r;
    while ((int64_t)(r + 1) * (r + 1) <= v)
        ++r;
    return r;
}

constexpr int kBrick = 32;
constexpr int kHalo = kBrick + 2;
constexpr int kMaxList = 1024;

// CTA per 32^3 brick of a chunk of bricksPerAxis^3 bricks whose first brick is (obx, oby, obz).
// Writes the brick's 8^3 leaf masks into the chunk's Morton-indexed leaf array. The primitives
// tested are cand[0..numCand) when cand is given (the chunk's candidates), else all of them.
__global__ void __launch_bounds__(256) sceneBrickKernel(const DevPrim* __restrict__ prims, uint32_t numPrims, const uint32_t* __restrict__ cand,
    uint32_t numCand, uint32_t kind, uint32_t res, uint32_t seed, uint32_t shell, uint32_t bricksPerAxis, uint32_t obx, uint32_t oby, uint32_t obz,
    uint64_t* __restrict__ leafArray, uint32_t* status)
{
    __shared__ uint64_t rows[kHalo * kHalo]; // bit hx (0..33) of row (hy, hz) = voxel (bx0 - 1 + hx, ...)
    __shared__ uint32_t list[kMaxList];
    __shared__ uint32_t listCount;
    const uint32_t b = blockIdx.x;
    const int bx = (int)(b % bricksPerAxis), by = (int)((b / bricksPerAxis) % bricksPerAxis), bz = (int)(b / (bricksPerAxis * bricksPerAxis));
    const int x0 = (int)(obx + bx) * kBrick - 1, y0 = (int)(oby + by) * kBrick - 1, z0 = (int)(obz + bz) * kBrick - 1; // halo origin
    if (threadIdx.x == 0)
        listCount = 0;
    __syncthreads();
    if (kind == TDAG_SCENE_PRIMITIVES) {
        const uint32_t scan = cand ? numCand : numPrims;
        for (uint32_t c = threadIdx.x; c < scan; c += blockDim.x) {
            const uint32_t i = cand ? cand[c] : c;
            const DevPrim& p = prims[i];
            bool hit = true;
            const int lo[3] = { x0, y0, z0 };
#pragma unroll
            for (int k = 0; k < 3; ++k)
                hit &= (p.lo[k] < lo[k] + kHalo) && (p.lo[k] + p.ext[k] > lo[k]);
            if (hit) {
                const uint32_t slot = atomicAdd(&listCount, 1u);
                if (slot < kMaxList)
                    list[slot] = i;
            }
        }
        __syncthreads();
        if (listCount > kMaxList) {
            if (threadIdx.x == 0)
                setDeviceError(status, TDAG_ERR_ALLOC, 400);
            return;
        }
        // A brick whose whole halo box lies inside one box or ball primitive (and inside the grid) is
        // solid throughout: its shell is empty, its solid leaves are full.
        __shared__ int covered;
        if (threadIdx.x == 0)
            covered = 0;
        __syncthreads();
        const bool inGrid = x0 >= 0 && y0 >= 0 && z0 >= 0 && x0 + kHalo <= (int)res && y0 + kHalo <= (int)res && z0 + kHalo <= (int)res;
        if (inGrid)
            for (uint32_t li = threadIdx.x; li < listCount; li += blockDim.x) {
                const DevPrim& p = prims[list[li]];
                const int lo[3] = { x0, y0, z0 };
                bool in = false;
                if (p.type == 0) {
                    in = true;
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        in &= p.lo[k] <= lo[k] && lo[k] + kHalo <= p.lo[k] + p.ext[k];
                } else if (p.type == 1) {
                    in = true; // a ball is convex: all 8 corners inside -> the box inside
                    for (int c = 0; c < 8 && in; ++c) {
                        int64_t d2 = 0;
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const int64_t d = (int64_t)(lo[k] + (((c >> k) & 1) ? kHalo - 1 : 0)) - (p.lo[k] + p.radius);
                            d2 += d * d;
                        }
                        in = d2 <= (int64_t)p.radius * p.radius;
                    }
                }
                if (in)
                    covered = 1;
            }
        __syncthreads();
        if (covered) {
            for (int l = threadIdx.x; l < 512; l += blockDim.x) {
                const uint32_t gx = bx * 8 + (l & 7), gy = by * 8 + ((l >> 3) & 7), gz = bz * 8 + (l >> 6);
                leafArray[(uint64_t)part1by2(gx) | ((uint64_t)part1by2(gy) << 1) | ((uint64_t)part1by2(gz) << 2)] = shell ? 0ull : ~0ull;
            }
            return;
        }
    }
    const uint32_t nList = listCount;
    // ---- inside rows with halo
    for (int r = threadIdx.x; r < kHalo * kHalo; r += blockDim.x) {
        const int hy = r % kHalo, hz = r / kHalo;
        const int y = y0 + hy, z = z0 + hz;
        uint64_t bits = 0;
        if (y >= 0 && z >= 0 && y < (int)res && z < (int)res) {
            if (kind == TDAG_SCENE_TERRAIN) {
                for (int hx = 0; hx < kHalo; ++hx) {
                    const int x = x0 + hx;
                    if (x < 0 || x >= (int)res)
                        continue;
                    if (fbmValue(x, y, z, seed) * (int64_t)res > (int64_t)z * 31 * 65535)
                        bits |= 1ull << hx;
                }
            } else {
                for (uint32_t li = 0; li < nList; ++li) {
                    const DevPrim& p = prims[list[li]];
                    if (y < p.lo[1] || y >= p.lo[1] + p.ext[1] || z < p.lo[2] || z >= p.lo[2] + p.ext[2])
                        continue;
                    int xa = p.lo[0], xb = p.lo[0] + p.ext[0]; // [xa, xb)
                    if (p.type == 0) {
                        // box: the whole x range
                    } else if (p.type == 1) {
                        const int64_t dy = y - (p.lo[1] + p.radius), dz = z - (p.lo[2] + p.radius);
                        const int64_t rem = (int64_t)p.radius * p.radius - dy * dy - dz * dz;
                        if (rem < 0)
                            continue;
                        const int dx = isqrt64(rem);
                        xa = p.lo[0] + p.radius - dx;
                        xb = p.lo[0] + p.radius + dx + 1;
                    } else {
                        const int ha = max(xa, x0), hb = min(xb, x0 + kHalo);
                        for (int x = ha; x < hb; ++x)
                            if (x >= 0 && x < (int)res && !((bits >> (x - x0)) & 1) && terrainInside(p, x, y, z))
                                bits |= 1ull << (x - x0);
                        continue;
                    }
                    const int ha = max(max(xa, x0), 0), hb = min(min(xb, x0 + kHalo), (int)res);
                    if (ha < hb) {
                        const int s = ha - x0, e = hb - x0;
                        bits |= ((e >= 64 ? ~0ull : ((1ull << e) - 1)) & ~((1ull << s) - 1));
                    }
                }
            }
        }
        rows[r] = bits;
    }
    __syncthreads();
    // ---- shell and leaf emission: thread per leaf (8^3 = 512 leaves, 2 per thread)
    for (int l = threadIdx.x; l < 512; l += blockDim.x) {
        const int lx = l & 7, ly = (l >> 3) & 7, lz = l >> 6;
        uint64_t mask = 0;
        for (int vz = 0; vz < 4; ++vz)
            for (int vy = 0; vy < 4; ++vy) {
                const int hy = ly * 4 + vy + 1, hz = lz * 4 + vz + 1;
                const uint64_t c = rows[hy + kHalo * hz];
                uint64_t v = c;
                if (shell) {
                    const uint64_t all = c & (c << 1) & (c >> 1) & rows[hy - 1 + kHalo * hz] & rows[hy + 1 + kHalo * hz] & rows[hy + kHalo * (hz - 1)] & rows[hy + kHalo * (hz + 1)];
                    v = c & ~all;
                }
                const uint32_t four = (uint32_t)(v >> (lx * 4 + 1)) & 0xF;
                for (int vx = 0; vx < 4; ++vx)
                    if ((four >> vx) & 1)
                        mask |= 1ull << morton3(vx, vy, vz);
            }
        const uint32_t gx = bx * 8 + lx, gy = by * 8 + ly, gz = bz * 8 + lz;
        const uint64_t code = (uint64_t)part1by2(gx) | ((uint64_t)part1by2(gy) << 1) | ((uint64_t)part1by2(gz) << 2);
        leafArray[code] = mask;
    }
}

// Dense host grid (uploaded) -> Morton-indexed leaf array.
__global__ void denseLeafKernel(const uint8_t* __restrict__ dense, uint32_t res, uint64_t* __restrict__ leafArray, uint64_t numLeaves)
{
    const uint64_t code = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (code >= numLeaves)
        return;
    const uint32_t lx = compact1by2((uint32_t)code), ly = compact1by2((uint32_t)(code >> 1)), lz = compact1by2((uint32_t)(code >> 2));
    uint64_t mask = 0;
    for (uint32_t i = 0; i < 64; ++i) {
        const uint32_t x = lx * 4 + compact1by2(i), y = ly * 4 + compact1by2(i >> 1), z = lz * 4 + compact1by2(i >> 2);
        if (dense[(size_t)x + (size_t)res * y + (size_t)res * res * z])
            mask |= 1ull << i;
    }
    leafArray[code] = mask;
}

__global__ void nonZeroFlagKernel(const uint64_t* __restrict__ a, uint64_t n, uint32_t* __restrict__ flags, unsigned long long* __restrict__ voxels)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t pc = 0;
    if (i < n) {
        const uint64_t v = a[i];
        flags[i] = v != 0;
        pc = __popcll(v);
    }
    for (int o = 16; o > 0; o >>= 1)
        pc += __shfl_down_sync(0xffffffffu, pc, o);
    if ((threadIdx.x & 31) == 0 && pc)
        atomicAdd(voxels, (unsigned long long)pc);
}

__global__ void gatherLeavesKernel(const uint32_t* __restrict__ codes, uint32_t n, const uint64_t* __restrict__ leafArray, uint64_t* __restrict__ masks,
    uint64_t* __restrict__ codes64)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    masks[i] = leafArray[codes[i]];
    codes64[i] = codes[i];
}

// Level build: parent code = child code >> 3; run heads start new parents.
__global__ void runHeadKernel(const uint64_t* __restrict__ codes, uint32_t n, uint32_t* __restrict__ flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        flags[i] = (i == 0) || ((codes[i] >> 3) != (codes[i - 1] >> 3));
}

__global__ void linkParentsKernel(const uint64_t* __restrict__ codes, uint32_t n, const uint32_t* __restrict__ flags, const uint32_t* __restrict__ offs,
    uint32_t* __restrict__ nodes, uint64_t* __restrict__ parentCodes)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t parent = offs[i] + flags[i] - 1;
    nodes[(size_t)parent * 8 + (codes[i] & 7)] = i;
    if (flags[i])
        parentCodes[parent] = codes[i] >> 3;
}

// toDAG helpers
__global__ void remapChildrenKernel(const uint32_t* __restrict__ in, uint64_t count8, const uint32_t* __restrict__ mapping, uint64_t* __restrict__ keys)
{
    // keys: 4 u64 words per node = the remapped children pairs
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count8 / 2)
        return;
    const uint32_t a = in[2 * i], b = in[2 * i + 1];
    const uint32_t ma = (a == kEmpty32) ? kEmpty32 : mapping[a];
    const uint32_t mb = (b == kEmpty32) ? kEmpty32 : mapping[b];
    keys[i] = (uint64_t)ma | ((uint64_t)mb << 32);
}

__global__ void firstFlagsKernel(const uint32_t* __restrict__ slotOf, const uint32_t* __restrict__ minIdx, uint32_t n, uint32_t* __restrict__ flags,
    uint32_t* __restrict__ canon)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t c = minIdx[slotOf[i]];
    canon[i] = c;
    flags[i] = (c == i);
}

__global__ void dedupMapKernel(const uint32_t* __restrict__ canon, const uint32_t* __restrict__ handleOf, uint32_t n, uint32_t* __restrict__ mapping)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        mapping[i] = handleOf[canon[i]];
}

__global__ void gatherU64Kernel(const uint64_t* __restrict__ src, const uint32_t* __restrict__ idx, uint32_t n, uint32_t words, uint64_t* __restrict__ dst)
{
    const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (uint64_t)n * words)
        return;
    const uint32_t i = (uint32_t)(g / words), w = (uint32_t)(g % words);
    dst[g] = src[(size_t)idx[i] * words + w];
}

uint64_t pow2AtLeast(uint64_t v)
{
    uint64_t p = 1;
    while (p < v)
        p <<= 1;
    return p;
}

// ------------------------------------------------------------------------------------------------
// Host-side primitive list (deterministic, splitmix64-driven)
// ------------------------------------------------------------------------------------------------
struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    uint32_t below(uint32_t n) { return n ? (uint32_t)(next() % n) : 0; }
    int32_t range(int32_t lo, int32_t hi) { return lo + (int32_t)below((uint32_t)(hi - lo + 1)); } // inclusive
};

void placePrimitive(tdag_primitive& p, uint32_t res, Rng& rng)
{
    const uint32_t pbits = permBitsOf(p.xform & 7);
    for (int k = 0; k < 3; ++k) {
        const int32_t ext = p.size[(pbits >> (2 * k)) & 3];
        p.offset[k] = ext >= (int32_t)res ? 0 : (int32_t)rng.below((uint32_t)(res - ext + 1));
    }
}

std::vector<tdag_primitive> scenePrimitives(const tdag_scene& sc)
{
    std::vector<tdag_primitive> out;
    if (sc.kind != TDAG_SCENE_PRIMITIVES)
        return out;
    Rng rng { 0x5EEDull * 1000003ull + sc.seed };
    const int32_t res = (int32_t)sc.resolution;
    auto scaled = [&](int32_t num) { return std::max<int32_t>(1, (int32_t)((int64_t)res * num / 2048)); };
    out.reserve(sc.num_primitives);
    for (uint32_t i = 0; i < sc.num_primitives; ++i) {
        tdag_primitive p {};
        if (i > 0 && rng.below(100) < sc.copy_percent) {
            const uint32_t j = rng.below(i);
            p = out[j];
            p.source = j;
            const uint32_t mode = rng.below(3);
            uint32_t perm = p.xform & 7, mirror = p.xform >> 3;
            if (mode == 0)
                mirror = mirror ^ (1 + rng.below(7)); // a different mirror
            else if (mode == 1)
                perm = (perm + 1 + rng.below(5)) % 6; // a different axis order
            p.xform = perm | (mirror << 3);
            placePrimitive(p, sc.resolution, rng); // mode 2: translation only
        } else {
            const uint32_t r = rng.below(100);
            p.source = i;
            p.seed = (uint32_t)rng.next();
            if (r < 45) {
                p.type = 0;
                for (int k = 0; k < 3; ++k)
                    p.size[k] = rng.range(scaled(8), scaled(256));
            } else if (r < 90) {
                p.type = 1;
                p.radius = rng.range(scaled(4), scaled(128));
                p.size[0] = p.size[1] = p.size[2] = 2 * p.radius + 1;
            } else {
                p.type = 2;
                const int32_t s = rng.range(scaled(32), scaled(256));
                p.size[0] = p.size[1] = p.size[2] = s;
            }
            p.xform = 0;
            placePrimitive(p, sc.resolution, rng);
        }
        out.push_back(p);
    }
    return out;
}

// ------------------------------------------------------------------------------------------------
// Pipeline pieces
// ------------------------------------------------------------------------------------------------
// Morton-indexed leaf array -> SVO tree (levels 2..root) in the reference's order.
void buildTree(Context& ctx, DevBuf<uint64_t>& leafArray, uint64_t numLeafCells, uint32_t res, SvdagOwned& out)
{
    cudaStream_t s = ctx.stream;
    const uint32_t rootLevel = (uint32_t)(31 - __builtin_clz(res));
    out.resolution = res;
    out.rootLevel = rootLevel;
    out.structureType = 0;
    out.nodes.clear();
    out.nodes.resize(rootLevel + 1);
    TDAG_CHECK(numLeafCells < (1ull << 32), TDAG_ERR_ARG, "resolution too large for a single leaf array");
    DevBuf<uint32_t> flags(numLeafCells, s);
    DevBuf<unsigned long long> vox(1, s);
    TDAG_CUDA(cudaMemsetAsync(vox.get(), 0, 8, s));
    nonZeroFlagKernel<<<gridFor(numLeafCells, 256), 256, 0, s>>>(leafArray.get(), numLeafCells, flags.get(), vox.get());
    TDAG_LAUNCHED();
    DevBuf<uint32_t> codes32(numLeafCells, s);
    const uint32_t n = compactFlags(flags.get(), codes32.get(), numLeafCells, s);
    flags.release();
    unsigned long long voxels = 0;
    TDAG_CUDA(cudaMemcpyAsync(&voxels, vox.get(), 8, cudaMemcpyDeviceToHost, s));
    out.leaves = DevBuf<uint64_t>(n, s);
    DevBuf<uint64_t> codes(n, s);
    if (n) {
        gatherLeavesKernel<<<gridFor(n, 256), 256, 0, s>>>(codes32.get(), n, leafArray.get(), out.leaves.get(), codes.get());
        TDAG_LAUNCHED();
    }
    codes32.release();
    leafArray.release();
    uint32_t cur = n;
    for (uint32_t level = 3; level <= rootLevel && cur; ++level) {
        DevBuf<uint32_t> heads(cur, s), offs(cur, s);
        runHeadKernel<<<gridFor(cur, 256), 256, 0, s>>>(codes.get(), cur, heads.get());
        TDAG_LAUNCHED();
        const uint32_t np = (uint32_t)exclusiveScanU32Total(heads.get(), offs.get(), cur, s);
        out.nodes[level] = DevBuf<uint32_t>((size_t)np * 8, s);
        fillU32(out.nodes[level].get(), kEmpty32, (size_t)np * 8, s);
        DevBuf<uint64_t> pcodes(np, s);
        linkParentsKernel<<<gridFor(cur, 256), 256, 0, s>>>(codes.get(), cur, heads.get(), offs.get(), out.nodes[level].get(), pcodes.get());
        TDAG_LAUNCHED();
        codes = std::move(pcodes);
        cur = np;
    }
    TDAG_CUDA(cudaStreamSynchronize(s));
    out.voxelCount = voxels;
}

// First-occurrence dedup of n items with W-word keys; returns the number of unique items, the
// mapping (item -> handle) and the list of first occurrences.
uint32_t dedupLevel(Context& ctx, const uint64_t* keys, int words, uint32_t n, DevBuf<uint32_t>& mapping, DevBuf<uint32_t>& firsts)
{
    cudaStream_t s = ctx.stream;
    DevBuf<uint32_t> flags(n, s), canon(n, s);
    withClassTable(ctx, n, "toDAG", [&](uint64_t cap) {
        DevBuf<uint64_t> slots(cap, s);
        DevBuf<uint32_t> minIdx(cap, s), slotOf(n, s);
        fillU64(slots.get(), kEmptySlot, cap, s);
        fillU32(minIdx.get(), 0xFFFFFFFFu, cap, s);
        if (words == 1)
            classInsertKernel<1><<<gridFor(n, 256), 256, 0, s>>>(keys, n, slots.get(), minIdx.get(), slotOf.get(), cap - 1, ctx.status);
        else
            classInsertKernel<4><<<gridFor(n, 256), 256, 0, s>>>(keys, n, slots.get(), minIdx.get(), slotOf.get(), cap - 1, ctx.status);
        TDAG_LAUNCHED();
        slots.release();
        firstFlagsKernel<<<gridFor(n, 256), 256, 0, s>>>(slotOf.get(), minIdx.get(), n, flags.get(), canon.get());
        TDAG_LAUNCHED();
    });
    firsts = DevBuf<uint32_t>(n, s);
    DevBuf<uint32_t> handleOf(n, s);
    const uint32_t u = compactFlags(flags.get(), firsts.get(), n, s);
    exclusiveScanU32(flags.get(), handleOf.get(), n, s);
    mapping = DevBuf<uint32_t>(n, s);
    dedupMapKernel<<<gridFor(n, 256), 256, 0, s>>>(canon.get(), handleOf.get(), n, mapping.get());
    TDAG_LAUNCHED();
    return u;
}

void toDagDevice(Context& ctx, SvdagOwned& g)
{
    cudaStream_t s = ctx.stream;
    DevBuf<uint32_t> mapping, firsts;
    const uint32_t nl = (uint32_t)g.leaves.n;
    if (nl) {
        const uint32_t u = dedupLevel(ctx, g.leaves.get(), 1, nl, mapping, firsts);
        DevBuf<uint64_t> uniq(u, s);
        gatherU64Kernel<<<gridFor(u, 256), 256, 0, s>>>(g.leaves.get(), firsts.get(), u, 1, uniq.get());
        TDAG_LAUNCHED();
        g.leaves = std::move(uniq);
    }
    for (uint32_t level = 3; level <= g.rootLevel; ++level) {
        const uint32_t n = (uint32_t)(g.nodes[level].n / 8);
        if (!n)
            continue;
        DevBuf<uint64_t> keys((size_t)n * 4, s);
        remapChildrenKernel<<<gridFor((size_t)n * 4, 256), 256, 0, s>>>(g.nodes[level].get(), (uint64_t)n * 8, mapping.get(), keys.get());
        TDAG_LAUNCHED();
        DevBuf<uint32_t> m2, f2;
        const uint32_t u = dedupLevel(ctx, keys.get(), 4, n, m2, f2);
        DevBuf<uint32_t> uniq((size_t)u * 8, s);
        gatherU64Kernel<<<gridFor((size_t)u * 4, 256), 256, 0, s>>>(keys.get(), f2.get(), u, 4, reinterpret_cast<uint64_t*>(uniq.get()));
        TDAG_LAUNCHED();
        g.nodes[level] = std::move(uniq);
        mapping = std::move(m2);
    }
    TDAG_CUDA(cudaStreamSynchronize(s));
    g.structureType = 1;
}

DevPrim toDevPrim(const tdag_primitive& p)
{
    DevPrim d {};
    d.type = (int32_t)p.type;
    d.perm = (int32_t)(p.xform & 7);
    d.mirror = (int32_t)(p.xform >> 3);
    d.radius = p.radius;
    d.pbits = permBitsOf(p.xform & 7);
    for (int k = 0; k < 3; ++k) {
        d.size[k] = p.size[k];
        d.ext[k] = p.size[(d.pbits >> (2 * k)) & 3];
        d.lo[k] = p.offset[k];
    }
    d.seed = p.seed;
    return d;
}

} // namespace

// ------------------------------------------------------------------------------------------------
// Streamed scene build for grids whose leaf array does not fit (16384^3 and other grids above 4096^3): the grid
// is generated in chunks of chunkRes^3 voxels in Morton order of the chunks. Every chunk gets its own
// SVO (levels 2..log2(chunkRes)), is deduplicated within itself (first occurrence), and its unique
// items are merged level by level into global content tables -- slab hash tables whose chains grow by
// slabs from a bitmap allocator (slab_hash.cuh) -- that number items in order of first appearance. The level sequences of the whole tree are the chunks' sequences concatenated in chunk
// Morton order (the depth-first Morton traversal visits chunks in that order), so the global
// numbering is exactly toDAG's first-occurrence numbering of the full tree. Levels above the chunks
// are built from the chunks' root ids on the host (at most (res/chunkRes)^3 entries).
// ------------------------------------------------------------------------------------------------
namespace {

template <int W>
__device__ __forceinline__ uint64_t contentFp(const uint64_t* k)
{
    uint64_t fp = 0x2545F4914F6CDD1Dull;
#pragma unroll
    for (int w = 0; w < W; ++w)
        fp = mix64(fp ^ k[w]);
    return fp;
}
// Global content tables: one slab hash table per level (slab_hash.cuh), warp per key. Lane k < W holds
// word k of the key; the fingerprint decides the bucket (low bits) and the tag (high 32 bits).
constexpr uint32_t kNotFound = 0xFFFFFFFFu;
template <int W>
__device__ __forceinline__ bool warpKey(const uint64_t* __restrict__ keys, uint64_t i, uint64_t& myWord, uint64_t& fp)
{
    const uint32_t lane = threadIdx.x & 31;
    myWord = lane < (uint32_t)W ? keys[i * W + lane] : 0ull;
    uint64_t k[W];
#pragma unroll
    for (int w = 0; w < W; ++w)
        k[w] = __shfl_sync(0xffffffffu, myWord, w);
    fp = contentFp<W>(k);
    return true;
}
// The global id of every key the table already holds, else kNotFound with missing[i] = 1.
template <int W>
__global__ void slabFindKernel(const uint64_t* __restrict__ keys, uint32_t n, SlabPoolView pool, const uint64_t* __restrict__ items,
    uint32_t* __restrict__ outId, uint32_t* __restrict__ missing, uint32_t* status)
{
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n)
        return;
    uint64_t word, fp;
    warpKey<W>(keys, i, word, fp);
    const uint32_t id = slabFind<W>(pool, (uint32_t)fp & (pool.numBuckets - 1), (uint32_t)(fp >> 32), word, items, status);
    if ((threadIdx.x & 31) == 0) {
        outId[i] = id;
        missing[i] = id == kNotFound ? 1u : 0u;
    }
}
// Append the missing keys as ids base + rank (rank = order among the missing ones, so ids follow first
// appearance) and insert them. done[i] records a finished insertion, so that a rerun after the host
// grew the slab pool skips it.
template <int W>
__global__ void slabAppendKernel(const uint64_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ missing, const uint32_t* __restrict__ rank,
    uint64_t base, uint64_t* __restrict__ items, SlabPoolView pool, uint32_t* __restrict__ outId, uint32_t* __restrict__ done, uint32_t* status)
{
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= n || !missing[i] || done[i])
        return;
    const uint32_t lane = threadIdx.x & 31;
    uint64_t word, fp;
    warpKey<W>(keys, i, word, fp);
    const uint64_t id = base + rank[i];
    if (lane < (uint32_t)W)
        items[id * W + lane] = word;
    if (slabInsert(pool, (uint32_t)fp & (pool.numBuckets - 1), (fp >> 32) << 32 | id, (uint32_t)(i * 0x9E3779B9u), status) && lane == 0) {
        outId[i] = (uint32_t)id;
        done[i] = 1;
    }
}
// Reinsert the items [0, count) into a table with more buckets (growth).
template <int W>
__global__ void slabRehashKernel(const uint64_t* __restrict__ items, uint64_t count, SlabPoolView pool, uint32_t* status)
{
    const uint64_t id = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (id >= count)
        return;
    uint64_t word, fp;
    warpKey<W>(items, id, word, fp);
    slabInsert(pool, (uint32_t)fp & (pool.numBuckets - 1), (fp >> 32) << 32 | id, (uint32_t)(id * 0x85EBCA77u), status);
}
__global__ void composeIdsKernel(const uint32_t* __restrict__ mapping, uint32_t n, const uint32_t* __restrict__ uniqueId, uint32_t* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = uniqueId[mapping[i]];
}

// A slab hash table and its pool (slab_hash.cuh).
struct SlabTable {
    DevBuf<unsigned long long> slabs;
    DevBuf<uint32_t> bitmap;
    uint32_t numBuckets = 0, numSlabs = 0, bitmapWords = 0;
    SlabPoolView view() const { return SlabPoolView { slabs.get(), numBuckets, numSlabs, bitmap.get(), bitmapWords }; }

    // A table of `buckets` heads (power of two) and `spare` allocatable slabs, all empty.
    void create(Context& ctx, uint32_t buckets, uint32_t spare)
    {
        cudaStream_t s = ctx.stream;
        numBuckets = buckets;
        numSlabs = buckets + spare;
        bitmapWords = (spare + 31) / 32;
        slabs = DevBuf<unsigned long long>((size_t)numSlabs * 32, s);
        TDAG_CUDA(cudaMemsetAsync(slabs.get(), 0xFF, (size_t)numSlabs * 32 * 8, s));
        bitmap = DevBuf<uint32_t>(std::max<uint32_t>(bitmapWords, 1), s);
        TDAG_CUDA(cudaMemsetAsync(bitmap.get(), 0, (size_t)std::max<uint32_t>(bitmapWords, 1) * 4, s));
        if (spare % 32) { // bits past the pool's end count as taken
            const uint32_t tail = ~((1u << (spare % 32)) - 1u);
            TDAG_CUDA(cudaMemcpyAsync(bitmap.get() + bitmapWords - 1, &tail, 4, cudaMemcpyHostToDevice, s));
            TDAG_CUDA(cudaStreamSynchronize(s));
        }
    }
    // Twice the allocatable slabs, keeping every slab and its index (chains stay valid).
    void growPool(Context& ctx)
    {
        cudaStream_t s = ctx.stream;
        const uint32_t spare = numSlabs - numBuckets;
        TDAG_CHECK((uint64_t)numBuckets + 2ull * std::max<uint32_t>(spare, 32) < 0xFFFFFFF0ull, TDAG_ERR_OOM, "slab pool exceeds 2^32 slabs");
        SlabTable bigger;
        bigger.create(ctx, numBuckets, 2 * std::max<uint32_t>(spare, 32));
        TDAG_CUDA(cudaMemcpyAsync(bigger.slabs.get(), slabs.get(), (size_t)numSlabs * 32 * 8, cudaMemcpyDeviceToDevice, s));
        if (bitmapWords) {
            // the old tail word's padding bits were preset; they are real slabs now
            std::vector<uint32_t> words(bitmapWords);
            TDAG_CUDA(cudaMemcpyAsync(words.data(), bitmap.get(), (size_t)bitmapWords * 4, cudaMemcpyDeviceToHost, s));
            TDAG_CUDA(cudaStreamSynchronize(s));
            if (spare % 32)
                words.back() &= (1u << (spare % 32)) - 1u;
            TDAG_CUDA(cudaMemcpyAsync(bigger.bitmap.get(), words.data(), (size_t)bitmapWords * 4, cudaMemcpyHostToDevice, s));
            TDAG_CUDA(cudaStreamSynchronize(s));
        }
        *this = std::move(bigger);
    }
};

struct GlobalLevel {
    int words = 1;
    DevBuf<uint64_t> items; // count x words
    uint64_t count = 0;
    SlabTable table;
    uint32_t poolGrowths = 0, rehashes = 0;
};

// Buckets for `items` entries: about 8 per bucket (a quarter of a slab), at least 1024.
uint32_t slabBuckets(uint64_t items)
{
    uint64_t b = 1024;
    while (b * 8 < items)
        b <<= 1;
    TDAG_CHECK(b <= (1ull << 31), TDAG_ERR_ARG, "slab table too large");
    return (uint32_t)b;
}

// The slab pool starts at tuning.slab_pool_slabs allocatable slabs when set (tests use a tiny pool to
// exercise the growth path), else at one per bucket.
uint32_t initialSpare(const Context& ctx, uint32_t buckets) { return ctx.tuning.slab_pool_slabs ? ctx.tuning.slab_pool_slabs : buckets; }

template <int W>
void rehashInto(Context& ctx, GlobalLevel& g, uint32_t buckets)
{
    cudaStream_t s = ctx.stream;
    for (uint32_t attempt = 0;; ++attempt) {
        SlabTable t;
        t.create(ctx, buckets, std::max<uint32_t>(initialSpare(ctx, buckets), 32) << attempt);
        if (g.count) {
            slabRehashKernel<W><<<gridFor(g.count * 32, 256), 256, 0, s>>>(g.items.get(), g.count, t.view(), ctx.status);
            TDAG_LAUNCHED();
        }
        uint32_t aux = 0;
        const uint32_t code = ctx.takeStatus(&aux);
        if (code == 0) {
            g.table = std::move(t);
            return;
        }
        TDAG_CHECK(code == TDAG_ERR_ALLOC && attempt < 16, (int)code, "slab table rehash: device reported error " + std::to_string(code));
        ++g.poolGrowths;
    }
}

void reserveGlobal(Context& ctx, GlobalLevel& g, uint64_t incoming)
{
    cudaStream_t s = ctx.stream;
    const uint64_t need = g.count + incoming;
    TDAG_CHECK(need < 0xFFFFFFF0ull, TDAG_ERR_ARG, "a level of the streamed scene exceeds 2^32 unique items");
    if (need * g.words > g.items.n) {
        const uint64_t n = std::max<uint64_t>(need * g.words, g.items.n * 2);
        DevBuf<uint64_t> bigger(n, s);
        if (g.count)
            TDAG_CUDA(cudaMemcpyAsync(bigger.get(), g.items.get(), g.count * g.words * 8, cudaMemcpyDeviceToDevice, s));
        g.items = std::move(bigger);
    }
    // Chains grow by slabs as items arrive; the bucket array is rebuilt only when chains would average
    // four slabs (more than 124 items per bucket).
    if (g.table.numBuckets == 0 || need > (uint64_t)g.table.numBuckets * 124) {
        const uint32_t buckets = slabBuckets(need);
        if (g.table.numBuckets)
            ++g.rehashes;
        if (g.words == 1)
            rehashInto<1>(ctx, g, buckets);
        else
            rehashInto<4>(ctx, g, buckets);
    }
}

// Merge n items of one chunk level (keys: n x words, in tree order) into the global level; returns
// every item's global id.
template <int W>
DevBuf<uint32_t> mergeLevelW(Context& ctx, GlobalLevel& g, const uint64_t* keys, uint32_t n)
{
    cudaStream_t s = ctx.stream;
    DevBuf<uint32_t> mapping, firsts;
    const uint32_t u = dedupLevel(ctx, keys, W, n, mapping, firsts); // first occurrence within the chunk
    DevBuf<uint64_t> ukeys((size_t)u * W, s);
    gatherU64Kernel<<<gridFor((size_t)u * W, 256), 256, 0, s>>>(keys, firsts.get(), u, W, ukeys.get());
    TDAG_LAUNCHED();
    reserveGlobal(ctx, g, u);
    DevBuf<uint32_t> uid(u, s), missing(u, s), rank(u, s), done(u, s);
    TDAG_CUDA(cudaMemsetAsync(done.get(), 0, (size_t)u * 4, s));
    slabFindKernel<W><<<gridFor((uint64_t)u * 32, 256), 256, 0, s>>>(ukeys.get(), u, g.table.view(), g.items.get(), uid.get(), missing.get(), ctx.status);
    TDAG_LAUNCHED();
    const uint64_t added = exclusiveScanU32Total(missing.get(), rank.get(), u, s);
    ctx.checkStatus("scene merge: lookup");
    for (uint32_t attempt = 0;; ++attempt) {
        slabAppendKernel<W><<<gridFor((uint64_t)u * 32, 256), 256, 0, s>>>(ukeys.get(), u, missing.get(), rank.get(), g.count, g.items.get(),
            g.table.view(), uid.get(), done.get(), ctx.status);
        TDAG_LAUNCHED();
        uint32_t aux = 0;
        const uint32_t code = ctx.takeStatus(&aux);
        if (code == 0)
            break;
        // the pool ran out: grow it (chains stay valid) and insert what is left
        TDAG_CHECK(code == TDAG_ERR_ALLOC && attempt < 16, (int)code, "scene merge: device reported error " + std::to_string(code) + " (aux " +
                std::to_string(aux) + ")");
        g.table.growPool(ctx);
        ++g.poolGrowths;
    }
    g.count += added;
    DevBuf<uint32_t> ids(n, s);
    composeIdsKernel<<<gridFor(n, 256), 256, 0, s>>>(mapping.get(), n, uid.get(), ids.get());
    TDAG_LAUNCHED();
    return ids;
}

DevBuf<uint32_t> mergeLevel(Context& ctx, GlobalLevel& g, const uint64_t* keys, uint32_t n)
{
    return g.words == 1 ? mergeLevelW<1>(ctx, g, keys, n) : mergeLevelW<4>(ctx, g, keys, n);
}

inline uint32_t log2u(uint32_t v) { return (uint32_t)(31 - __builtin_clz(v)); }

// ------------------------------------------------------------------------------------------------
// Checkpoints of the streamed build: after a chunk, the state that the rest of the build depends on
// is the global levels' unique items (in first-occurrence order), every finished chunk's root id,
// the voxel count and the next chunk. The slab tables are not stored: they are rebuilt from the
// items on resume, and since a new item's id is its place in that order, the resumed build assigns
// the same ids as an uninterrupted one. Layout (little-endian): "TDAGCKP1", the scene fields and the
// chunk resolution (validated on resume), the next chunk, the voxel count, the number of levels,
// per level (2 .. chunk root) its words per item, item count and items, then every chunk's root id.
// Written to `path`.tmp and renamed over `path`, so a checkpoint on disk is always complete.
// ------------------------------------------------------------------------------------------------
constexpr char kCkptMagic[8] = { 'T', 'D', 'A', 'G', 'C', 'K', 'P', '1' };

struct CkptHeader {
    char magic[8];
    uint32_t kind, resolution, seed, numPrimitives, copyPercent, shell, chunkRes, levels;
    uint64_t nextChunk, voxels, numChunks;
};

bool sameScene(const CkptHeader& h, const tdag_scene& sc, uint32_t chunkRes, uint64_t numChunks, uint32_t levels)
{
    return std::memcmp(h.magic, kCkptMagic, 8) == 0 && h.kind == sc.kind && h.resolution == sc.resolution && h.seed == sc.seed &&
        h.numPrimitives == sc.num_primitives && h.copyPercent == sc.copy_percent && h.shell == sc.shell && h.chunkRes == chunkRes &&
        h.numChunks == numChunks && h.levels == levels;
}

void writeCheckpoint(Context& ctx, const std::string& path, const tdag_scene& sc, uint32_t chunkRes, uint64_t nextChunk, uint64_t voxels,
    const std::vector<GlobalLevel>& glv, const std::vector<uint32_t>& chunkRoot)
{
    CkptHeader h {};
    std::memcpy(h.magic, kCkptMagic, 8);
    h.kind = sc.kind;
    h.resolution = sc.resolution;
    h.seed = sc.seed;
    h.numPrimitives = sc.num_primitives;
    h.copyPercent = sc.copy_percent;
    h.shell = sc.shell;
    h.chunkRes = chunkRes;
    h.levels = (uint32_t)glv.size();
    h.nextChunk = nextChunk;
    h.voxels = voxels;
    h.numChunks = chunkRoot.size();
    const std::string tmp = path + ".tmp";
    std::unique_ptr<FILE, int (*)(FILE*)> file(std::fopen(tmp.c_str(), "wb"), &std::fclose);
    TDAG_CHECK(file != nullptr, TDAG_ERR_ARG, "cannot write the checkpoint " + tmp);
    FILE* f = file.get();
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
    std::vector<uint64_t> host;
    for (uint32_t l = 2; ok && l < glv.size(); ++l) {
        const uint64_t meta[2] = { (uint64_t)glv[l].words, glv[l].count };
        host.resize(glv[l].count * glv[l].words);
        if (!host.empty()) {
            TDAG_CUDA(cudaMemcpyAsync(host.data(), glv[l].items.get(), host.size() * 8, cudaMemcpyDeviceToHost, ctx.stream));
            TDAG_CUDA(cudaStreamSynchronize(ctx.stream));
        }
        ok = std::fwrite(meta, sizeof meta, 1, f) == 1 && (host.empty() || std::fwrite(host.data(), 8, host.size(), f) == host.size());
    }
    ok = ok && std::fwrite(chunkRoot.data(), 4, chunkRoot.size(), f) == chunkRoot.size();
    ok = (std::fclose(file.release()) == 0) && ok;
    TDAG_CHECK(ok, TDAG_ERR_ARG, "writing the checkpoint " + tmp + " failed");
    TDAG_CHECK(std::rename(tmp.c_str(), path.c_str()) == 0, TDAG_ERR_ARG, "cannot move the checkpoint to " + path);
}

// Restores a checkpoint of the same scene into glv / chunkRoot; returns the next chunk (0 when the
// file does not exist). A file of another scene or a damaged one is an error (TDAG_ERR_CORRUPT).
uint64_t readCheckpoint(Context& ctx, const std::string& path, const tdag_scene& sc, uint32_t chunkRes, uint64_t& voxels, std::vector<GlobalLevel>& glv,
    std::vector<uint32_t>& chunkRoot)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f)
        return 0;
    std::unique_ptr<FILE, int (*)(FILE*)> guard(f, &std::fclose);
    CkptHeader h {};
    TDAG_CHECK(std::fread(&h, sizeof h, 1, f) == 1, TDAG_ERR_CORRUPT, "checkpoint " + path + ": truncated header");
    TDAG_CHECK(sameScene(h, sc, chunkRes, chunkRoot.size(), (uint32_t)glv.size()), TDAG_ERR_CORRUPT, "checkpoint " + path + " is of another scene");
    TDAG_CHECK(h.nextChunk <= h.numChunks, TDAG_ERR_CORRUPT, "checkpoint " + path + ": chunk cursor out of range");
    for (uint32_t l = 2; l < glv.size(); ++l) {
        uint64_t meta[2];
        TDAG_CHECK(std::fread(meta, sizeof meta, 1, f) == 1, TDAG_ERR_CORRUPT, "checkpoint " + path + ": truncated level");
        TDAG_CHECK(meta[0] == (uint64_t)glv[l].words && meta[1] < 0xFFFFFFF0ull, TDAG_ERR_CORRUPT, "checkpoint " + path + ": bad level header");
        std::vector<uint64_t> host(meta[1] * meta[0]);
        TDAG_CHECK(host.empty() || std::fread(host.data(), 8, host.size(), f) == host.size(), TDAG_ERR_CORRUPT, "checkpoint " + path + ": truncated items");
        GlobalLevel& g = glv[l];
        g.items = DevBuf<uint64_t>(std::max<size_t>(host.size(), 1), ctx.stream);
        if (!host.empty()) {
            TDAG_CUDA(cudaMemcpyAsync(g.items.get(), host.data(), host.size() * 8, cudaMemcpyHostToDevice, ctx.stream));
            TDAG_CUDA(cudaStreamSynchronize(ctx.stream));
        }
        g.count = meta[1];
        reserveGlobal(ctx, g, 0); // the slab table, rebuilt from the items
    }
    TDAG_CHECK(std::fread(chunkRoot.data(), 4, chunkRoot.size(), f) == chunkRoot.size(), TDAG_ERR_CORRUPT, "checkpoint " + path + ": truncated roots");
    voxels = h.voxels;
    return h.nextChunk;
}

} // namespace

std::unique_ptr<SvdagOwned> sceneSvdagStreamed(Context& ctx, const tdag_scene& sc, uint32_t chunkRes, const StreamCheckpoint* ckpt)
{
    cudaStream_t s = ctx.stream;
    const uint32_t res = sc.resolution, root = log2u(res), lc = log2u(chunkRes);
    TDAG_CHECK(chunkRes >= 64 && chunkRes <= 2048 && (chunkRes & (chunkRes - 1)) == 0 && chunkRes <= res, TDAG_ERR_ARG,
        "chunk resolution must be a power of two in [64, min(2048, resolution)]");
    const uint32_t cpa = res / chunkRes;
    const uint64_t numChunks = (uint64_t)cpa * cpa * cpa;
    auto prims = scenePrimitives(sc);
    std::vector<DevPrim> dp(prims.size());
    for (size_t i = 0; i < prims.size(); ++i)
        dp[i] = toDevPrim(prims[i]);
    DevBuf<DevPrim> dprims(std::max<size_t>(1, dp.size()), s);
    if (!dp.empty())
        TDAG_CUDA(cudaMemcpyAsync(dprims.get(), dp.data(), dp.size() * sizeof(DevPrim), cudaMemcpyHostToDevice, s));
    // candidates per chunk (Morton index): primitives whose box, grown by the 1-voxel shell halo, meets it
    std::vector<std::vector<uint32_t>> perChunk(numChunks);
    if (sc.kind == TDAG_SCENE_PRIMITIVES)
        for (uint32_t i = 0; i < dp.size(); ++i) {
            int lo[3], hi[3];
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::max(0, (dp[i].lo[k] - 1) / (int)chunkRes);
                hi[k] = std::min((int)cpa - 1, (dp[i].lo[k] + dp[i].ext[k]) / (int)chunkRes);
            }
            for (int z = lo[2]; z <= hi[2]; ++z)
                for (int y = lo[1]; y <= hi[1]; ++y)
                    for (int x = lo[0]; x <= hi[0]; ++x)
                        perChunk[morton3((uint32_t)x, (uint32_t)y, (uint32_t)z)].push_back(i);
        }
    std::vector<uint32_t> candOff(numChunks + 1, 0), candIds;
    for (uint64_t m = 0; m < numChunks; ++m) {
        candOff[m + 1] = candOff[m] + (uint32_t)perChunk[m].size();
        candIds.insert(candIds.end(), perChunk[m].begin(), perChunk[m].end());
    }
    DevBuf<uint32_t> dcand(std::max<size_t>(1, candIds.size()), s);
    if (!candIds.empty())
        TDAG_CUDA(cudaMemcpyAsync(dcand.get(), candIds.data(), candIds.size() * 4, cudaMemcpyHostToDevice, s));

    std::vector<GlobalLevel> glv(lc + 1);
    for (uint32_t l = 2; l <= lc; ++l)
        glv[l].words = l == 2 ? 1 : 4;
    std::vector<uint32_t> chunkRoot(numChunks, kEmpty32);
    uint64_t voxels = 0;
    const uint32_t bpa = chunkRes / kBrick;
    const uint64_t cells = (uint64_t)(chunkRes / 4) * (chunkRes / 4) * (chunkRes / 4);
    const bool saving = ckpt && ckpt->path && ckpt->path[0];
    const uint64_t firstChunk = saving ? readCheckpoint(ctx, ckpt->path, sc, chunkRes, voxels, glv, chunkRoot) : 0;
    uint64_t processed = 0; // chunks finished by this call
    auto chunkDone = [&](uint64_t m) {
        ++processed;
        const bool stop = ckpt && ckpt->stop_after && processed == ckpt->stop_after && m + 1 < numChunks;
        if (saving && (stop || (ckpt->every && processed % ckpt->every == 0 && m + 1 < numChunks)))
            writeCheckpoint(ctx, ckpt->path, sc, chunkRes, m + 1, voxels, glv, chunkRoot);
        TDAG_CHECK(!stop, TDAG_ERR_INTERRUPTED, "streamed scene build stopped after " + std::to_string(processed) + " chunks as requested (next chunk " +
                std::to_string(m + 1) + ")");
    };
    for (uint64_t m = firstChunk; m < numChunks; chunkDone(m), ++m) {
        const uint32_t nc = candOff[m + 1] - candOff[m];
        if (sc.kind == TDAG_SCENE_PRIMITIVES && nc == 0)
            continue; // nothing reaches this chunk: empty
        const uint32_t cx = compact1by2((uint32_t)m), cy = compact1by2((uint32_t)(m >> 1)), cz = compact1by2((uint32_t)(m >> 2));
        DevBuf<uint64_t> leafArray(cells, s);
        sceneBrickKernel<<<(unsigned)((uint64_t)bpa * bpa * bpa), 256, 0, s>>>(dprims.get(), (uint32_t)dp.size(),
            sc.kind == TDAG_SCENE_PRIMITIVES ? dcand.get() + candOff[m] : nullptr, nc, sc.kind, res, sc.seed, sc.shell, bpa, cx * bpa, cy * bpa, cz * bpa,
            leafArray.get(), ctx.status);
        TDAG_LAUNCHED();
        ctx.checkStatus("scene generation (chunk)");
        SvdagOwned tree;
        buildTree(ctx, leafArray, cells, chunkRes, tree);
        voxels += tree.voxelCount;
        if (tree.leaves.n == 0)
            continue;
        DevBuf<uint32_t> prevIds = mergeLevel(ctx, glv[2], tree.leaves.get(), (uint32_t)tree.leaves.n);
        for (uint32_t l = 3; l <= lc; ++l) {
            const uint32_t n = (uint32_t)(tree.nodes[l].n / 8);
            DevBuf<uint64_t> keys((size_t)n * 4, s);
            remapChildrenKernel<<<gridFor((size_t)n * 4, 256), 256, 0, s>>>(tree.nodes[l].get(), (uint64_t)n * 8, prevIds.get(), keys.get());
            TDAG_LAUNCHED();
            tree.nodes[l].release();
            prevIds = mergeLevel(ctx, glv[l], keys.get(), n);
        }
        TDAG_CUDA(cudaMemcpyAsync(&chunkRoot[m], prevIds.get(), 4, cudaMemcpyDeviceToHost, s));
        ctx.checkStatus("scene merge (chunk)");
    }

    auto out = std::make_unique<SvdagOwned>();
    out->resolution = res;
    out->rootLevel = root;
    out->structureType = 1;
    out->voxelCount = voxels;
    out->nodes.resize(root + 1);
    out->leaves = DevBuf<uint64_t>(glv[2].count, s);
    if (glv[2].count)
        TDAG_CUDA(cudaMemcpyAsync(out->leaves.get(), glv[2].items.get(), glv[2].count * 8, cudaMemcpyDeviceToDevice, s));
    for (uint32_t l = 3; l <= lc; ++l) {
        out->nodes[l] = DevBuf<uint32_t>(glv[l].count * 8, s);
        if (glv[l].count)
            TDAG_CUDA(cudaMemcpyAsync(out->nodes[l].get(), glv[l].items.get(), glv[l].count * 32, cudaMemcpyDeviceToDevice, s));
    }
    // levels above the chunks: dense Morton arrays of ids, deduplicated by first occurrence
    std::vector<uint32_t> cur = chunkRoot;
    for (uint32_t l = lc + 1; l <= root; ++l) {
        std::vector<uint32_t> next(cur.size() / 8, kEmpty32), nodes;
        std::map<std::array<uint32_t, 8>, uint32_t> seen;
        for (size_t p = 0; p < next.size(); ++p) {
            std::array<uint32_t, 8> c;
            bool any = false;
            for (int k = 0; k < 8; ++k) {
                c[k] = cur[8 * p + k];
                any |= c[k] != kEmpty32;
            }
            if (!any)
                continue;
            auto it = seen.find(c);
            if (it == seen.end()) {
                it = seen.emplace(c, (uint32_t)(nodes.size() / 8)).first;
                nodes.insert(nodes.end(), c.begin(), c.end());
            }
            next[p] = it->second;
        }
        out->nodes[l] = DevBuf<uint32_t>(nodes.size(), s);
        if (!nodes.empty())
            TDAG_CUDA(cudaMemcpyAsync(out->nodes[l].get(), nodes.data(), nodes.size() * 4, cudaMemcpyHostToDevice, s));
        TDAG_CUDA(cudaStreamSynchronize(s)); // `nodes` is reused by the next level
        cur = std::move(next);
    }
    TDAG_CUDA(cudaStreamSynchronize(s));
    return out;
}

std::unique_ptr<SvdagOwned> sceneSvdag(Context& ctx, const tdag_scene& sc, bool toDag, const StreamCheckpoint* ckpt)
{
    TDAG_CHECK(sc.kind == TDAG_SCENE_TERRAIN || sc.kind == TDAG_SCENE_PRIMITIVES, TDAG_ERR_ARG, "unknown scene kind");
    TDAG_CHECK(sc.resolution >= 32 && sc.resolution <= 16384 && (sc.resolution & (sc.resolution - 1)) == 0, TDAG_ERR_ARG,
        "scene resolution must be a power of two in [32, 16384]");
    cudaStream_t s = ctx.stream;
    const uint32_t res = sc.resolution;
    const uint64_t cells = (uint64_t)(res / 4) * (res / 4) * (res / 4);
    const uint32_t chunk = sc.chunk_resolution ? sc.chunk_resolution : (res > 4096 ? 2048u : 0u);
    if (chunk) {
        TDAG_CHECK(toDag, TDAG_ERR_ARG, "a streamed scene build always deduplicates (to_dag = 1)");
        return sceneSvdagStreamed(ctx, sc, chunk, ckpt);
    }
    TDAG_CHECK(!ckpt, TDAG_ERR_ARG, "checkpoints apply to the streamed (chunked) scene build: set chunk_resolution");
    TDAG_CHECK(cells < (1ull << 32), TDAG_ERR_ARG, "scene too large for the single-pass generator");
    auto prims = scenePrimitives(sc);
    std::vector<DevPrim> dp(prims.size());
    for (size_t i = 0; i < prims.size(); ++i)
        dp[i] = toDevPrim(prims[i]);
    DevBuf<DevPrim> dprims(std::max<size_t>(1, dp.size()), s);
    if (!dp.empty())
        TDAG_CUDA(cudaMemcpyAsync(dprims.get(), dp.data(), dp.size() * sizeof(DevPrim), cudaMemcpyHostToDevice, s));
    DevBuf<uint64_t> leafArray(cells, s);
    const uint32_t bpa = res / kBrick;
    const uint64_t bricks = (uint64_t)bpa * bpa * bpa;
    sceneBrickKernel<<<(unsigned)bricks, 256, 0, s>>>(dprims.get(), (uint32_t)dp.size(), nullptr, 0, sc.kind, res, sc.seed, sc.shell, bpa, 0, 0, 0,
        leafArray.get(), ctx.status);
    TDAG_LAUNCHED();
    ctx.checkStatus("scene generation");
    auto out = std::make_unique<SvdagOwned>();
    buildTree(ctx, leafArray, cells, res, *out);
    if (toDag)
        toDagDevice(ctx, *out);
    return out;
}

std::unique_ptr<SvdagOwned> denseSvdag(Context& ctx, const uint8_t* dense, uint32_t res, bool toDag)
{
    TDAG_CHECK(res >= 4 && (res & (res - 1)) == 0 && res <= 2048, TDAG_ERR_ARG, "dense resolution must be a power of two in [4, 2048]");
    cudaStream_t s = ctx.stream;
    const uint64_t nvox = (uint64_t)res * res * res;
    DevBuf<uint8_t> d(nvox, s);
    TDAG_CUDA(cudaMemcpyAsync(d.get(), dense, nvox, cudaMemcpyHostToDevice, s));
    const uint64_t cells = nvox / 64;
    DevBuf<uint64_t> leafArray(cells, s);
    denseLeafKernel<<<gridFor(cells, 256), 256, 0, s>>>(d.get(), res, leafArray.get(), cells);
    TDAG_LAUNCHED();
    d.release();
    auto out = std::make_unique<SvdagOwned>();
    buildTree(ctx, leafArray, cells, res, *out);
    if (toDag)
        toDagDevice(ctx, *out);
    return out;
}

std::vector<tdag_primitive> hostScenePrimitives(const tdag_scene& sc) { return scenePrimitives(sc); }

} // namespace tdag

// ================================================================================================
// C ABI
// ================================================================================================
using namespace tdag;

struct tdag_svdag {
    std::unique_ptr<SvdagOwned> g;
};

Context& ctxOf(tdag_ctx* c); // build.cu
int guardedCall(const std::function<void()>& f); // build.cu
int failWith(int code, const char* msg); // build.cu

extern "C" {

int tdag_scene_primitives(const tdag_scene* scene, tdag_primitive* out, uint32_t capacity, uint32_t* count)
{
    if (!scene || !count)
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        auto p = hostScenePrimitives(*scene);
        *count = (uint32_t)p.size();
        if (out)
            std::memcpy(out, p.data(), std::min<size_t>(capacity, p.size()) * sizeof(tdag_primitive));
    });
}

int tdag_scene_svdag(tdag_ctx* ctx, const tdag_scene* scene, int toDag, tdag_svdag** out)
{
    if (!ctx || !scene || !out)
        return failWith(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        auto h = std::make_unique<tdag_svdag>();
        h->g = sceneSvdag(c, *scene, toDag != 0, nullptr);
        *out = h.release();
    });
}

int tdag_scene_svdag_checkpointed(tdag_ctx* ctx, const tdag_scene* scene, const char* checkpoint_path, uint32_t every_chunks, uint32_t stop_after_chunks,
    tdag_svdag** out)
{
    if (!ctx || !scene || !out || !checkpoint_path || !checkpoint_path[0])
        return failWith(TDAG_ERR_ARG, "null argument or empty checkpoint path");
    *out = nullptr;
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        StreamCheckpoint ck { checkpoint_path, every_chunks, stop_after_chunks };
        auto h = std::make_unique<tdag_svdag>();
        h->g = sceneSvdag(c, *scene, true, &ck);
        *out = h.release();
    });
}

int tdag_svdag_from_dense(tdag_ctx* ctx, const uint8_t* dense, uint32_t res, int toDag, tdag_svdag** out)
{
    if (!ctx || !dense || !out)
        return failWith(TDAG_ERR_ARG, "null argument");
    *out = nullptr;
    return guardedCall([&] {
        Context& c = ctxOf(ctx);
        TDAG_CUDA(cudaSetDevice(c.device));
        auto h = std::make_unique<tdag_svdag>();
        h->g = denseSvdag(c, dense, res, toDag != 0);
        *out = h.release();
    });
}

int tdag_svdag_get_view(const tdag_svdag* sv, tdag_svdag_view* v)
{
    if (!sv || !v)
        return failWith(TDAG_ERR_ARG, "null argument");
    std::memset(v, 0, sizeof(*v));
    const SvdagOwned& g = *sv->g;
    v->resolution = g.resolution;
    v->root_level = g.rootLevel;
    v->structure_type = g.structureType;
    for (uint32_t l = 3; l <= g.rootLevel; ++l) {
        v->nodes[l] = g.nodes[l].get();
        v->node_counts[l] = g.nodes[l].n / 8;
    }
    v->leaves = g.leaves.get();
    v->leaf_count = g.leaves.n;
    return TDAG_OK;
}

int tdag_svdag_voxel_count(const tdag_svdag* sv, uint64_t* out)
{
    if (!sv || !out)
        return failWith(TDAG_ERR_ARG, "null argument");
    *out = sv->g->voxelCount;
    return TDAG_OK;
}

int tdag_svdag_copy_level(tdag_ctx* ctx, const tdag_svdag* sv, uint32_t level, void* dst, uint64_t bytes)
{
    if (!ctx || !sv || (!dst && bytes))
        return failWith(TDAG_ERR_ARG, "null argument");
    return guardedCall([&] {
        const SvdagOwned& g = *sv->g;
        Context& c = ctxOf(ctx);
        TDAG_CHECK(level >= 2 && level <= g.rootLevel, TDAG_ERR_ARG, "level out of range");
        const void* src = level == 2 ? (const void*)g.leaves.get() : (const void*)g.nodes[level].get();
        const uint64_t need = level == 2 ? g.leaves.n * 8 : g.nodes[level].n * 4;
        TDAG_CHECK(bytes >= need, TDAG_ERR_ARG, "destination buffer too small");
        if (need)
            TDAG_CUDA(cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToHost, c.stream));
        TDAG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int tdag_svdag_free(tdag_svdag* sv)
{
    delete sv;
    return TDAG_OK;
}

} // extern "C"
