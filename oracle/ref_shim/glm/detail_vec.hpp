// Stand-in for the parts of the glm vector library that the reference's Transform-DAG path uses
// (test infrastructure: it lets the reference's own sources compile into oracle/_ref, nothing else).
// Written from glm's documented semantics, not from its sources:
//  * vec<L, T> for L = 2, 3, 4 with public members x, y, z, w and their aliases r, g, b, a and
//    s, t, p, q (a structural literal type, so it can be a non-type template parameter as the
//    reference does with glm::u8vec3);
//  * component-wise arithmetic, bitwise and shift operators with vectors and scalars;
//  * relational functions returning bool vectors, any / all, and mix(), where mix(a, b, bvec) picks
//    b in the components where the bool vector is true and mix(a, b, t) interpolates for floats.
// Default construction zero-initialises (glm leaves components undefined; the reference always
// assigns before it reads).
#pragma once
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <type_traits>

namespace glm {

using length_t = int;
enum qualifier { packed_highp, defaultp = packed_highp };

template <length_t L, typename T, qualifier Q = defaultp>
struct vec;

template <typename T, qualifier Q>
struct vec<1, T, Q> {
    T x {};
    constexpr vec() = default;
    constexpr explicit vec(T s) : x(s) {}
    constexpr T& operator[](length_t) { return x; }
    constexpr const T& operator[](length_t) const { return x; }
    static constexpr length_t length() { return 1; }
};

template <typename T, qualifier Q>
struct vec<2, T, Q> {
    union { T x {}; T r; T s; };
    union { T y {}; T g; T t; };
    constexpr vec() = default;
    constexpr explicit vec(T s) : x(s), y(s) {}
    template <typename A, typename B>
    constexpr vec(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    template <typename U, qualifier P>
    constexpr vec(const vec<2, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
    template <typename U, qualifier P>
    constexpr explicit vec(const vec<3, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
    template <typename U, qualifier P>
    constexpr explicit vec(const vec<4, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)) {}
    constexpr T& operator[](length_t i) { return i == 0 ? x : y; }
    constexpr const T& operator[](length_t i) const { return i == 0 ? x : y; }
    static constexpr length_t length() { return 2; }
};

template <typename T, qualifier Q>
struct vec<3, T, Q> {
    union { T x {}; T r; T s; };
    union { T y {}; T g; T t; };
    union { T z {}; T b; T p; };
    constexpr vec() = default;
    constexpr explicit vec(T s) : x(s), y(s), z(s) {}
    template <typename A, typename B, typename C>
    constexpr vec(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U, qualifier P, typename C>
    constexpr vec(const vec<2, U, P>& v, C c) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(c)) {}
    template <typename A, typename U, qualifier P>
    constexpr vec(A a, const vec<2, U, P>& v) : x(static_cast<T>(a)), y(static_cast<T>(v.x)), z(static_cast<T>(v.y)) {}
    template <typename U, qualifier P>
    constexpr vec(const vec<3, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    template <typename U, qualifier P>
    constexpr explicit vec(const vec<4, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)) {}
    constexpr T& operator[](length_t i) { return i == 0 ? x : (i == 1 ? y : z); }
    constexpr const T& operator[](length_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
    static constexpr length_t length() { return 3; }
};

template <typename T, qualifier Q>
struct vec<4, T, Q> {
    union { T x {}; T r; T s; };
    union { T y {}; T g; T t; };
    union { T z {}; T b; T p; };
    union { T w {}; T a; T q; };
    constexpr vec() = default;
    constexpr explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    template <typename A, typename B, typename C, typename D>
    constexpr vec(A a, B b, C c, D d) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
    template <typename U, qualifier P, typename D>
    constexpr vec(const vec<3, U, P>& v, D d) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(d)) {}
    template <typename U, qualifier P>
    constexpr vec(const vec<4, U, P>& v) : x(static_cast<T>(v.x)), y(static_cast<T>(v.y)), z(static_cast<T>(v.z)), w(static_cast<T>(v.w)) {}
    constexpr T& operator[](length_t i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    constexpr const T& operator[](length_t i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    static constexpr length_t length() { return 4; }
};

namespace detail {
    template <length_t L, typename R, typename F>
    constexpr vec<L, R> make(F f)
    {
        vec<L, R> out;
        for (length_t i = 0; i < L; ++i)
            out[i] = static_cast<R>(f(i));
        return out;
    }
    template <typename T>
    using nd = std::type_identity_t<T>;
}

// Component-wise binary operators: vector op vector, vector op scalar, scalar op vector.
#define TDAG_GLM_BINOP(OP)                                                                                 \
    template <length_t L, typename T, qualifier Q>                                                        \
    constexpr vec<L, T, Q> operator OP(const vec<L, T, Q>& a, const vec<L, T, Q>& b)                      \
    {                                                                                                      \
        return detail::make<L, T>([&](length_t i) { return a[i] OP b[i]; });                              \
    }                                                                                                      \
    template <length_t L, typename T, qualifier Q>                                                        \
    constexpr vec<L, T, Q> operator OP(const vec<L, T, Q>& a, detail::nd<T> s)                            \
    {                                                                                                      \
        return detail::make<L, T>([&](length_t i) { return a[i] OP s; });                                 \
    }                                                                                                      \
    template <length_t L, typename T, qualifier Q>                                                        \
    constexpr vec<L, T, Q> operator OP(detail::nd<T> s, const vec<L, T, Q>& b)                            \
    {                                                                                                      \
        return detail::make<L, T>([&](length_t i) { return s OP b[i]; });                                 \
    }                                                                                                      \
    template <length_t L, typename T, qualifier Q>                                                        \
    constexpr vec<L, T, Q>& operator OP##=(vec<L, T, Q>& a, const vec<L, T, Q>& b)                        \
    {                                                                                                      \
        for (length_t i = 0; i < L; ++i)                                                                   \
            a[i] = static_cast<T>(a[i] OP b[i]);                                                          \
        return a;                                                                                          \
    }                                                                                                      \
    template <length_t L, typename T, qualifier Q>                                                        \
    constexpr vec<L, T, Q>& operator OP##=(vec<L, T, Q>& a, detail::nd<T> s)                              \
    {                                                                                                      \
        for (length_t i = 0; i < L; ++i)                                                                   \
            a[i] = static_cast<T>(a[i] OP s);                                                             \
        return a;                                                                                          \
    }
TDAG_GLM_BINOP(+)
TDAG_GLM_BINOP(-)
TDAG_GLM_BINOP(*)
TDAG_GLM_BINOP(/)
TDAG_GLM_BINOP(%)
TDAG_GLM_BINOP(&)
TDAG_GLM_BINOP(|)
TDAG_GLM_BINOP(^)
TDAG_GLM_BINOP(<<)
TDAG_GLM_BINOP(>>)
#undef TDAG_GLM_BINOP

template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> operator-(const vec<L, T, Q>& a)
{
    return detail::make<L, T>([&](length_t i) { return -a[i]; });
}
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> operator+(const vec<L, T, Q>& a) { return a; }
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> operator~(const vec<L, T, Q>& a)
{
    return detail::make<L, T>([&](length_t i) { return ~a[i]; });
}
template <length_t L, typename T, qualifier Q>
constexpr bool operator==(const vec<L, T, Q>& a, const vec<L, T, Q>& b)
{
    for (length_t i = 0; i < L; ++i)
        if (!(a[i] == b[i]))
            return false;
    return true;
}
template <length_t L, typename T, qualifier Q>
constexpr bool operator!=(const vec<L, T, Q>& a, const vec<L, T, Q>& b) { return !(a == b); }
template <length_t L, qualifier Q>
constexpr vec<L, bool, Q> operator&&(const vec<L, bool, Q>& a, const vec<L, bool, Q>& b)
{
    return detail::make<L, bool>([&](length_t i) { return a[i] && b[i]; });
}
template <length_t L, qualifier Q>
constexpr vec<L, bool, Q> operator||(const vec<L, bool, Q>& a, const vec<L, bool, Q>& b)
{
    return detail::make<L, bool>([&](length_t i) { return a[i] || b[i]; });
}

// Relational functions (glm/vector_relational.hpp).
#define TDAG_GLM_REL(NAME, OP)                                                                             \
    template <length_t L, typename T, qualifier Q>                                                        \
    constexpr vec<L, bool, Q> NAME(const vec<L, T, Q>& a, const vec<L, T, Q>& b)                          \
    {                                                                                                      \
        return detail::make<L, bool>([&](length_t i) { return a[i] OP b[i]; });                           \
    }
TDAG_GLM_REL(equal, ==)
TDAG_GLM_REL(notEqual, !=)
TDAG_GLM_REL(lessThan, <)
TDAG_GLM_REL(lessThanEqual, <=)
TDAG_GLM_REL(greaterThan, >)
TDAG_GLM_REL(greaterThanEqual, >=)
#undef TDAG_GLM_REL

template <length_t L, qualifier Q>
constexpr bool any(const vec<L, bool, Q>& v)
{
    for (length_t i = 0; i < L; ++i)
        if (v[i])
            return true;
    return false;
}
template <length_t L, qualifier Q>
constexpr bool all(const vec<L, bool, Q>& v)
{
    for (length_t i = 0; i < L; ++i)
        if (!v[i])
            return false;
    return true;
}
template <length_t L, qualifier Q>
constexpr vec<L, bool, Q> not_(const vec<L, bool, Q>& v)
{
    return detail::make<L, bool>([&](length_t i) { return !v[i]; });
}

// mix(a, b, bvec): b where the selector is true, a elsewhere.
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> mix(const vec<L, T, Q>& a, const vec<L, T, Q>& b, const vec<L, bool, Q>& sel)
{
    return detail::make<L, T>([&](length_t i) { return sel[i] ? b[i] : a[i]; });
}
// mix(a, b, t) for floating point: a + t (b - a).
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> mix(const vec<L, T, Q>& a, const vec<L, T, Q>& b, detail::nd<T> t)
    requires std::is_floating_point_v<T>
{
    return detail::make<L, T>([&](length_t i) { return a[i] * (T(1) - t) + b[i] * t; });
}
template <typename T>
constexpr T mix(T a, T b, T t) requires std::is_floating_point_v<T> { return a * (T(1) - t) + b * t; }
template <typename T>
constexpr T mix(T a, T b, bool sel) { return sel ? b : a; }

template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> min(const vec<L, T, Q>& a, const vec<L, T, Q>& b)
{
    return detail::make<L, T>([&](length_t i) { return b[i] < a[i] ? b[i] : a[i]; });
}
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> max(const vec<L, T, Q>& a, const vec<L, T, Q>& b)
{
    return detail::make<L, T>([&](length_t i) { return a[i] < b[i] ? b[i] : a[i]; });
}
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> min(const vec<L, T, Q>& a, detail::nd<T> s) { return min(a, vec<L, T, Q>(s)); }
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> max(const vec<L, T, Q>& a, detail::nd<T> s) { return max(a, vec<L, T, Q>(s)); }
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> clamp(const vec<L, T, Q>& v, const vec<L, T, Q>& lo, const vec<L, T, Q>& hi) { return min(max(v, lo), hi); }
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> clamp(const vec<L, T, Q>& v, detail::nd<T> lo, detail::nd<T> hi) { return min(max(v, lo), hi); }
template <length_t L, typename T, qualifier Q>
constexpr vec<L, T, Q> abs(const vec<L, T, Q>& v)
{
    return detail::make<L, T>([&](length_t i) { return v[i] < T(0) ? -v[i] : v[i]; });
}
template <length_t L, typename T, qualifier Q>
vec<L, T, Q> floor(const vec<L, T, Q>& v)
{
    return detail::make<L, T>([&](length_t i) { return std::floor(v[i]); });
}
template <length_t L, typename T, qualifier Q>
vec<L, T, Q> fract(const vec<L, T, Q>& v)
{
    return detail::make<L, T>([&](length_t i) { return v[i] - std::floor(v[i]); });
}
template <length_t L, typename T, qualifier Q>
constexpr T compMin(const vec<L, T, Q>& v)
{
    T m = v[0];
    for (length_t i = 1; i < L; ++i)
        m = v[i] < m ? v[i] : m;
    return m;
}
template <length_t L, typename T, qualifier Q>
constexpr T compMax(const vec<L, T, Q>& v)
{
    T m = v[0];
    for (length_t i = 1; i < L; ++i)
        m = m < v[i] ? v[i] : m;
    return m;
}

using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;
using dvec3 = vec<3, double>;
using ivec2 = vec<2, int>;
using ivec3 = vec<3, int>;
using ivec4 = vec<4, int>;
using uvec2 = vec<2, unsigned>;
using uvec3 = vec<3, unsigned>;
using uvec4 = vec<4, unsigned>;
using bvec2 = vec<2, bool>;
using bvec3 = vec<3, bool>;
using bvec4 = vec<4, bool>;
using u8vec2 = vec<2, uint8_t>;
using u8vec3 = vec<3, uint8_t>;
using u8vec4 = vec<4, uint8_t>;
using i8vec3 = vec<3, int8_t>;
using u16vec3 = vec<3, uint16_t>;
using u32vec3 = vec<3, uint32_t>;
using u64vec3 = vec<3, uint64_t>;

// Only the type is needed (bounds.h declares transforms by it).
template <length_t C, length_t R, typename T, qualifier Q = defaultp>
struct mat {
    vec<R, T, Q> cols[C] {};
};
using mat4 = mat<4, 4, float>;
using mat4x4 = mat4;
using mat3 = mat<3, 3, float>;

}
