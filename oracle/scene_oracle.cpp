// CPU statement of the project's procedural primitive scenes (test infrastructure only).
//
// The product generates these grids on the device (libtdag.so: tdag_scene_primitives,
// tdag_scene_svdag). This file is the independent CPU statement of the same integer-only definition,
// in C++ so that the CPU baseline and the reference arm of bench.py can build their inputs, at any
// size and for any sub-box of a grid, without loading the product library. oracle/generator.py is
// the same definition in numpy for small grids; the tests check all three against one another.
//
// Definition (the scene is this project's own; the reference voxelises meshes instead):
//  * primitive list: splitmix64-driven, seeded by 0x5EED * 1000003 + seed. Each primitive is either a
//    transformed copy of an earlier one (copy_percent: a different mirror, a different axis order, or
//    a translation only) or a new box (45 %, sides U[8, 256]), sphere (45 %, radius U[4, 128]) or
//    terrain block (10 %, side U[32, 256]), all scaled by resolution / 2048 and placed uniformly;
//  * a voxel v lies in a primitive when w = v - offset is inside its world extent; mirrored axes map
//    w_k to E_k - 1 - w_k, the local voxel is u[perm[k]] = w_k, and the shape test is: box always;
//    sphere |u - r|^2 <= r^2; terrain fbm(u, seed) * size > u.z * 31 * 65535;
//  * the grid is the union of the primitives, clipped to [0, res)^3, reduced to its 1-voxel shell:
//    a solid voxel stays when one of its 6 neighbours is not solid (outside the grid counts as empty).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

namespace orcscene {

// Field for field the layout of tdag_primitive (include/tdag.h), so the lists compare byte for byte.
struct Primitive {
    uint32_t type; // 0 box, 1 sphere, 2 terrain block
    uint32_t xform; // permutation id | mirror bits << 3
    int32_t size[3];
    int32_t radius;
    int32_t offset[3];
    uint32_t seed;
    uint32_t source;
    uint32_t reserved;
};
static_assert(sizeof(Primitive) == 48, "tdag_primitive layout");

// Axis order per permutation id: p0 | p1 << 2 | p2 << 4 (ids 012 021 102 120 201 210).
inline uint32_t permBits(uint32_t id)
{
    static const uint32_t packed[6] = { 0 | 1 << 2 | 2 << 4, 0 | 2 << 2 | 1 << 4, 1 | 0 << 2 | 2 << 4, 1 | 2 << 2 | 0 << 4, 2 | 0 << 2 | 1 << 4,
        2 | 1 << 2 | 0 << 4 };
    return packed[id];
}

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
    int32_t range(int32_t lo, int32_t hi) { return lo + (int32_t)below((uint32_t)(hi - lo + 1)); }
};

void place(Primitive& p, uint32_t res, Rng& rng)
{
    const uint32_t pb = permBits(p.xform & 7);
    for (int k = 0; k < 3; ++k) {
        const int32_t ext = p.size[(pb >> (2 * k)) & 3];
        p.offset[k] = ext >= (int32_t)res ? 0 : (int32_t)rng.below((uint32_t)(res - ext + 1));
    }
}

std::vector<Primitive> primitives(uint32_t res, uint32_t seed, uint32_t count, uint32_t copyPercent)
{
    std::vector<Primitive> out;
    out.reserve(count);
    Rng rng { 0x5EEDull * 1000003ull + seed };
    auto scaled = [&](int32_t num) { return std::max<int32_t>(1, (int32_t)((int64_t)res * num / 2048)); };
    for (uint32_t i = 0; i < count; ++i) {
        Primitive p {};
        if (i > 0 && rng.below(100) < copyPercent) {
            const uint32_t j = rng.below(i);
            p = out[j];
            p.source = j;
            const uint32_t mode = rng.below(3);
            uint32_t perm = p.xform & 7, mirror = p.xform >> 3;
            if (mode == 0)
                mirror = mirror ^ (1 + rng.below(7));
            else if (mode == 1)
                perm = (perm + 1 + rng.below(5)) % 6;
            p.xform = perm | (mirror << 3);
            place(p, res, rng);
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
            place(p, res, rng);
        }
        out.push_back(p);
    }
    return out;
}

// fBm value noise, integer only: 5 octaves of lattice cells 64 >> o, 16-bit lattice values from a
// 32-bit hash, Q16 smoothstep weights, trilinear interpolation, octave weights 16 >> o.
inline uint32_t mix32(uint32_t h)
{
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}
inline uint32_t lattice(int64_t ix, int64_t iy, int64_t iz, uint32_t octave, uint32_t seed)
{
    uint32_t h = seed * 0x9E3779B1u + octave * 0x85EBCA77u;
    h = mix32(h ^ ((uint32_t)ix * 0x27D4EB2Fu));
    h = mix32(h ^ ((uint32_t)iy * 0x165667B1u));
    h = mix32(h ^ ((uint32_t)iz * 0xD3A2646Du));
    return h >> 16;
}
inline int64_t weight(int64_t a, int64_t cell)
{
    const int64_t num = 2 * a + 1, den = 2 * cell;
    return (num * num * (3 * den - 2 * num) * 65536) / (den * den * den);
}
inline int64_t lerp(int64_t a, int64_t b, int64_t w) { return (a * (65536 - w) + b * w) >> 16; }
int64_t fbm(int64_t x, int64_t y, int64_t z, uint32_t seed)
{
    int64_t total = 0;
    for (uint32_t o = 0; o < 5; ++o) {
        const int64_t cell = 64 >> o;
        const int64_t ix = x / cell, iy = y / cell, iz = z / cell;
        const int64_t wx = weight(x % cell, cell), wy = weight(y % cell, cell), wz = weight(z % cell, cell);
        const int64_t x00 = lerp(lattice(ix, iy, iz, o, seed), lattice(ix + 1, iy, iz, o, seed), wx);
        const int64_t x10 = lerp(lattice(ix, iy + 1, iz, o, seed), lattice(ix + 1, iy + 1, iz, o, seed), wx);
        const int64_t x01 = lerp(lattice(ix, iy, iz + 1, o, seed), lattice(ix + 1, iy, iz + 1, o, seed), wx);
        const int64_t x11 = lerp(lattice(ix, iy + 1, iz + 1, o, seed), lattice(ix + 1, iy + 1, iz + 1, o, seed), wx);
        total += lerp(lerp(x00, x10, wy), lerp(x01, x11, wy), wz) * (16 >> o);
    }
    return total;
}

int64_t isqrt(int64_t v)
{
    int64_t r = (int64_t)std::sqrt((double)v);
    while (r * r > v)
        --r;
    while ((r + 1) * (r + 1) <= v)
        ++r;
    return r;
}

// Solid voxels of the scene in the box [o, o + n) (per axis), written to in[(z * n1 + y) * n0 + x].
void insideBox(const std::vector<Primitive>& prims, uint32_t res, const int64_t o[3], const int64_t n[3], uint8_t* in)
{
    std::memset(in, 0, (size_t)(n[0] * n[1] * n[2]));
    for (const Primitive& p : prims) {
        const uint32_t pb = permBits(p.xform & 7);
        const uint32_t mirror = p.xform >> 3;
        int64_t ext[3], lo[3], hi[3];
        bool empty = false;
        for (int k = 0; k < 3; ++k) {
            ext[k] = p.size[(pb >> (2 * k)) & 3];
            lo[k] = std::max<int64_t>({ (int64_t)p.offset[k], o[k], 0 });
            hi[k] = std::min<int64_t>({ (int64_t)p.offset[k] + ext[k], o[k] + n[k], (int64_t)res });
            empty |= hi[k] <= lo[k];
        }
        if (empty)
            continue;
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t z = lo[2]; z < hi[2]; ++z)
            for (int64_t y = lo[1]; y < hi[1]; ++y) {
                uint8_t* row = in + ((z - o[2]) * n[1] + (y - o[1])) * n[0] - o[0];
                if (p.type == 0) {
                    std::memset(row + lo[0], 1, (size_t)(hi[0] - lo[0]));
                } else if (p.type == 1) {
                    const int64_t dy = y - (p.offset[1] + p.radius), dz = z - (p.offset[2] + p.radius);
                    const int64_t rem = (int64_t)p.radius * p.radius - dy * dy - dz * dz;
                    if (rem < 0)
                        continue;
                    const int64_t dx = isqrt(rem);
                    const int64_t a = std::max<int64_t>(lo[0], p.offset[0] + p.radius - dx);
                    const int64_t b = std::min<int64_t>(hi[0], p.offset[0] + p.radius + dx + 1);
                    if (a < b)
                        std::memset(row + a, 1, (size_t)(b - a));
                } else {
                    for (int64_t x = lo[0]; x < hi[0]; ++x) {
                        if (row[x])
                            continue;
                        int64_t w[3] = { x - p.offset[0], y - p.offset[1], z - p.offset[2] };
                        int64_t u[3];
                        for (int k = 0; k < 3; ++k) {
                            if ((mirror >> k) & 1)
                                w[k] = ext[k] - 1 - w[k];
                            u[(pb >> (2 * k)) & 3] = w[k];
                        }
                        if (fbm(u[0], u[1], u[2], p.seed) * p.size[0] > u[2] * 31 * 65535)
                            row[x] = 1;
                    }
                }
            }
    }
}

} // namespace orcscene

namespace {
thread_local std::string g_sceneError;
}

extern "C" {

const char* orc_scene_last_error() { return g_sceneError.c_str(); }

// The primitive list of a scene (tdag_scene_primitives' definition). out holds capacity entries.
int orc_scene_primitives(uint32_t res, uint32_t seed, uint32_t count, uint32_t copyPercent, void* out, uint32_t capacity, uint32_t* written)
{
    try {
        const auto prims = orcscene::primitives(res, seed, count, copyPercent);
        const uint32_t n = (uint32_t)std::min<size_t>(capacity, prims.size());
        std::memcpy(out, prims.data(), n * sizeof(orcscene::Primitive));
        *written = (uint32_t)prims.size();
        return 0;
    } catch (const std::exception& e) {
        g_sceneError = e.what();
        return 1;
    }
}

// dense[(z * size + y) * size + x] = the scene's voxel (x0 + x, y0 + y, z0 + z), for the sub-box of
// side `size` at (x0, y0, z0); shell != 0 keeps only the 1-voxel surface shell of the whole grid
// (neighbours outside the sub-box are evaluated, so a sub-box is exactly the restriction of the grid).
int orc_scene_dense(uint32_t res, uint32_t seed, uint32_t count, uint32_t copyPercent, int shell, uint32_t x0, uint32_t y0, uint32_t z0,
    uint32_t size, uint8_t* dense)
{
    try {
        if (size == 0 || (uint64_t)x0 + size > res || (uint64_t)y0 + size > res || (uint64_t)z0 + size > res)
            throw std::runtime_error("sub-box outside the grid");
        const auto prims = orcscene::primitives(res, seed, count, copyPercent);
        if (!shell) {
            const int64_t o[3] = { x0, y0, z0 }, n[3] = { size, size, size };
            orcscene::insideBox(prims, res, o, n, dense);
            return 0;
        }
        const int64_t h = (int64_t)size + 2;
        const int64_t o[3] = { (int64_t)x0 - 1, (int64_t)y0 - 1, (int64_t)z0 - 1 }, n[3] = { h, h, h };
        std::vector<uint8_t> in((size_t)(h * h * h));
        orcscene::insideBox(prims, res, o, n, in.data());
        auto at = [&](int64_t x, int64_t y, int64_t z) { return in[(size_t)((z * h + y) * h + x)]; };
#pragma omp parallel for schedule(static)
        for (int64_t z = 0; z < (int64_t)size; ++z)
            for (int64_t y = 0; y < (int64_t)size; ++y)
                for (int64_t x = 0; x < (int64_t)size; ++x) {
                    const int64_t X = x + 1, Y = y + 1, Z = z + 1;
                    const bool solid = at(X, Y, Z);
                    const bool interior = at(X - 1, Y, Z) && at(X + 1, Y, Z) && at(X, Y - 1, Z) && at(X, Y + 1, Z) && at(X, Y, Z - 1) && at(X, Y, Z + 1);
                    dense[(size_t)((z * size + y) * size + x)] = solid && !interior;
                }
        return 0;
    } catch (const std::exception& e) {
        g_sceneError = e.what();
        return 1;
    }
}
}
