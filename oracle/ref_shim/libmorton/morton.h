// Stand-in for libmorton's Morton codes (test infrastructure for oracle/_ref): the standard bit
// interleave, x in bit 0, then y, then z. Plain loops; speed does not matter here.
#pragma once
#include <cstdint>

namespace libmorton {

template <int D, typename M, typename C>
inline M tdag_interleave(const C* c)
{
    M m = 0;
    constexpr int bits = int(sizeof(M) * 8) / D;
    for (int b = 0; b < bits; ++b)
        for (int d = 0; d < D; ++d)
            m |= M((uint64_t(c[d]) >> b) & 1u) << (b * D + d);
    return m;
}
template <int D, typename M, typename C>
inline void tdag_deinterleave(M m, C* c)
{
    constexpr int bits = int(sizeof(M) * 8) / D;
    for (int d = 0; d < D; ++d)
        c[d] = 0;
    for (int b = 0; b < bits; ++b)
        for (int d = 0; d < D; ++d)
            c[d] |= C((uint64_t(m) >> (b * D + d)) & 1u) << b;
}

inline uint_fast32_t morton3D_32_encode(uint_fast16_t x, uint_fast16_t y, uint_fast16_t z)
{
    const uint_fast16_t c[3] = { x, y, z };
    return tdag_interleave<3, uint32_t>(c);
}
inline void morton3D_32_decode(uint_fast32_t m, uint_fast16_t& x, uint_fast16_t& y, uint_fast16_t& z)
{
    uint_fast16_t c[3];
    tdag_deinterleave<3>(uint32_t(m), c);
    x = c[0], y = c[1], z = c[2];
}
inline uint_fast64_t morton3D_64_encode(uint_fast32_t x, uint_fast32_t y, uint_fast32_t z)
{
    const uint_fast32_t c[3] = { x, y, z };
    return tdag_interleave<3, uint64_t>(c);
}
inline void morton3D_64_decode(uint_fast64_t m, uint_fast32_t& x, uint_fast32_t& y, uint_fast32_t& z)
{
    uint_fast32_t c[3];
    tdag_deinterleave<3>(uint64_t(m), c);
    x = c[0], y = c[1], z = c[2];
}
inline uint_fast32_t morton2D_32_encode(uint_fast16_t x, uint_fast16_t y)
{
    const uint_fast16_t c[2] = { x, y };
    return tdag_interleave<2, uint32_t>(c);
}
inline void morton2D_32_decode(uint_fast32_t m, uint_fast16_t& x, uint_fast16_t& y)
{
    uint_fast16_t c[2];
    tdag_deinterleave<2>(uint32_t(m), c);
    x = c[0], y = c[1];
}
inline uint_fast64_t morton2D_64_encode(uint_fast32_t x, uint_fast32_t y)
{
    const uint_fast32_t c[2] = { x, y };
    return tdag_interleave<2, uint64_t>(c);
}
inline void morton2D_64_decode(uint_fast64_t m, uint_fast32_t& x, uint_fast32_t& y)
{
    uint_fast32_t c[2];
    tdag_deinterleave<2>(uint64_t(m), c);
    x = c[0], y = c[1];
}

}
