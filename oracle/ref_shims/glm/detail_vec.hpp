// Test infrastructure (oracle side): a small, project-written stand-in for the
// part of glm 1.0.1's API that torchhull's CUDA sources use, so that those
// sources compile unmodified without the glm package (which the reference's
// CMake build fetches over the network, _C/CMakeLists.txt:26-35).
//
// Only the surface torchhull touches is provided (vec2/3/4 of float,
// i64vec2/3, component access, converting constructors, component-wise
// arithmetic with vectors and scalars, clamp on scalars and epsilonEqual on
// scalars). Semantics follow glm's documented behaviour:
//   * vec<N,T>{a, b, ...} converts each argument with static_cast<T>;
//   * vec<N,T>{s} broadcasts the scalar s to every component;
//   * vec<N,T>{other} converts component-wise from another vector type;
//   * value-initialisation (vec2{}) gives zeros;
//   * clamp(x, lo, hi) = min(max(x, lo), hi);
//   * epsilonEqual(x, y, e) = |x - y| < e.
// Nothing here is called by the product library; it exists only to build the
// reference extension that pins the oracle and serves as the timing point.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define THREF_HD __host__ __device__
#else
#define THREF_HD
#endif

namespace glm
{

template <int N, typename T>
struct vec;

template <typename T>
struct vec<2, T>
{
    using value_type = T;
    T x{}, y{};

    constexpr vec() = default;
    THREF_HD constexpr explicit vec(T s) : x(s), y(s) {}
    template <typename A, typename B>
    THREF_HD constexpr vec(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b))
    {
    }
    template <typename U>
    THREF_HD constexpr explicit vec(const vec<2, U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y))
    {
    }
};

template <typename T>
struct vec<3, T>
{
    using value_type = T;
    T x{}, y{}, z{};

    constexpr vec() = default;
    THREF_HD constexpr explicit vec(T s) : x(s), y(s), z(s) {}
    template <typename A, typename B, typename C>
    THREF_HD constexpr vec(A a, B b, C c) : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c))
    {
    }
    template <typename U>
    THREF_HD constexpr explicit vec(const vec<3, U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z))
    {
    }
};

template <typename T>
struct vec<4, T>
{
    using value_type = T;
    T x{}, y{}, z{}, w{};

    constexpr vec() = default;
    THREF_HD constexpr explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    template <typename A, typename B, typename C, typename D>
    THREF_HD constexpr vec(A a, B b, C c, D d)
        : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d))
    {
    }
    template <typename U>
    THREF_HD constexpr explicit vec(const vec<4, U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)), w(static_cast<T>(o.w))
    {
    }
};

using vec2 = vec<2, float>;
using vec3 = vec<3, float>;
using vec4 = vec<4, float>;
using i64vec2 = vec<2, std::int64_t>;
using i64vec3 = vec<3, std::int64_t>;
using i64vec4 = vec<4, std::int64_t>;

// Component-wise arithmetic: vector with vector, vector with scalar, scalar with vector.
#define THREF_VEC_OP(OP)                                                                                              \
    template <typename T>                                                                                             \
    THREF_HD constexpr vec<2, T> operator OP(const vec<2, T>& a, const vec<2, T>& b)                                  \
    {                                                                                                                 \
        return vec<2, T>(a.x OP b.x, a.y OP b.y);                                                                     \
    }                                                                                                                 \
    template <typename T>                                                                                             \
    THREF_HD constexpr vec<3, T> operator OP(const vec<3, T>& a, const vec<3, T>& b)                                  \
    {                                                                                                                 \
        return vec<3, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                                                         \
    }                                                                                                                 \
    template <typename T>                                                                                             \
    THREF_HD constexpr vec<4, T> operator OP(const vec<4, T>& a, const vec<4, T>& b)                                  \
    {                                                                                                                 \
        return vec<4, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                                             \
    }                                                                                                                 \
    template <int N, typename T>                                                                                      \
    THREF_HD constexpr vec<N, T> operator OP(const vec<N, T>& a, T s)                                                 \
    {                                                                                                                 \
        return a OP vec<N, T>(s);                                                                                     \
    }                                                                                                                 \
    template <int N, typename T>                                                                                      \
    THREF_HD constexpr vec<N, T> operator OP(T s, const vec<N, T>& a)                                                 \
    {                                                                                                                 \
        return vec<N, T>(s) OP a;                                                                                     \
    }

THREF_VEC_OP(+)
THREF_VEC_OP(-)
THREF_VEC_OP(*)
THREF_VEC_OP(/)
#undef THREF_VEC_OP

template <typename T>
THREF_HD constexpr bool operator==(const vec<2, T>& a, const vec<2, T>& b)
{
    return a.x == b.x && a.y == b.y;
}
template <typename T>
THREF_HD constexpr bool operator==(const vec<3, T>& a, const vec<3, T>& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <int N, typename T>
THREF_HD constexpr bool operator!=(const vec<N, T>& a, const vec<N, T>& b)
{
    return !(a == b);
}

// Scalar clamp, as glm::clamp(x, minVal, maxVal) = min(max(x, minVal), maxVal).
template <typename T>
THREF_HD constexpr T clamp(T x, T lo, T hi)
{
    const T m = (x < lo) ? lo : x;
    return (hi < m) ? hi : m;
}

// Scalar epsilonEqual, as glm/gtc/epsilon: |x - y| < epsilon.
template <typename T>
THREF_HD constexpr bool epsilonEqual(const T& x, const T& y, const T& epsilon)
{
    const T d = x - y;
    return ((d < T(0)) ? -d : d) < epsilon;
}

} // namespace glm
