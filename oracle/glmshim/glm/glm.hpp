// Minimal vector-math header written for this project (test infrastructure).
//
// The reference simulator (dkiovics/fluid_simulator, src/Simulator/simulator/**)
// includes <glm/glm.hpp>, which is not installed here.  The reference only uses
// plain component-wise double/int/float 2- and 3-vectors plus dot, length and
// normalize, so this header provides exactly that surface with IEEE semantics:
//   * vec<L,T> for L = 2, 3 (dvec3, ivec3, vec3, dvec2, ivec2, vec2)
//   * constexpr element-wise constructors (with static_cast per element, i.e.
//     truncation toward zero for floating -> int), broadcast constructor,
//     implicit element-type conversion between vectors
//   * + - * / (vec-vec, vec-scalar, scalar-vec), unary minus, compound ops,
//     operator[], == and !=
//   * dot (left-to-right sum of component products), length = sqrt(dot),
//     normalize = v * (1 / sqrt(dot(v, v)))
// It is used only to compile the reference's own sources into the oracle
// library under oracle/_ref; nothing in the product includes it.
#pragma once

#include <cmath>

namespace glm {

typedef int length_t;

template <int L, typename T>
struct vec;

template <typename T>
struct identity_t { typedef T type; };

template <typename T>
struct vec<2, T> {
    T x, y;
    constexpr vec() : x(T(0)), y(T(0)) {}
    constexpr explicit vec(T s) : x(s), y(s) {}
    template <typename A, typename B>
    constexpr vec(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
    template <typename U>
    constexpr vec(const vec<2, U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}
    constexpr vec(const vec& o) = default;
    vec& operator=(const vec& o) = default;

    T& operator[](int i) { return i == 0 ? x : y; }
    constexpr const T& operator[](int i) const { return i == 0 ? x : y; }
    static constexpr length_t length() { return 2; }

    vec& operator+=(const vec& o) { x += o.x; y += o.y; return *this; }
    vec& operator-=(const vec& o) { x -= o.x; y -= o.y; return *this; }
    vec& operator*=(const vec& o) { x *= o.x; y *= o.y; return *this; }
    vec& operator/=(const vec& o) { x /= o.x; y /= o.y; return *this; }
    vec& operator+=(T s) { x += s; y += s; return *this; }
    vec& operator-=(T s) { x -= s; y -= s; return *this; }
    vec& operator*=(T s) { x *= s; y *= s; return *this; }
    vec& operator/=(T s) { x /= s; y /= s; return *this; }
};

template <typename T>
struct vec<3, T> {
    T x, y, z;
    constexpr vec() : x(T(0)), y(T(0)), z(T(0)) {}
    constexpr explicit vec(T s) : x(s), y(s), z(s) {}
    template <typename A, typename B, typename C>
    constexpr vec(A a, B b, C c)
        : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}
    template <typename U>
    constexpr vec(const vec<3, U>& o)
        : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    constexpr vec(const vec& o) = default;
    vec& operator=(const vec& o) = default;

    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    constexpr const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    static constexpr length_t length() { return 3; }

    vec& operator+=(const vec& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec& operator-=(const vec& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec& operator*=(const vec& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    vec& operator/=(const vec& o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
    vec& operator+=(T s) { x += s; y += s; z += s; return *this; }
    vec& operator-=(T s) { x -= s; y -= s; z -= s; return *this; }
    vec& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    vec& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
};

// ---- binary operators (component-wise) ------------------------------------
#define GLMSHIM_BINOP(OP)                                                              \
    template <typename T>                                                              \
    constexpr vec<3, T> operator OP(const vec<3, T>& a, const vec<3, T>& b) {          \
        return vec<3, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                          \
    }                                                                                  \
    template <typename T>                                                              \
    constexpr vec<3, T> operator OP(const vec<3, T>& a, typename identity_t<T>::type s) { \
        return vec<3, T>(a.x OP s, a.y OP s, a.z OP s);                                \
    }                                                                                  \
    template <typename T>                                                              \
    constexpr vec<3, T> operator OP(typename identity_t<T>::type s, const vec<3, T>& a) { \
        return vec<3, T>(s OP a.x, s OP a.y, s OP a.z);                                \
    }                                                                                  \
    template <typename T>                                                              \
    constexpr vec<2, T> operator OP(const vec<2, T>& a, const vec<2, T>& b) {          \
        return vec<2, T>(a.x OP b.x, a.y OP b.y);                                      \
    }                                                                                  \
    template <typename T>                                                              \
    constexpr vec<2, T> operator OP(const vec<2, T>& a, typename identity_t<T>::type s) { \
        return vec<2, T>(a.x OP s, a.y OP s);                                          \
    }                                                                                  \
    template <typename T>                                                              \
    constexpr vec<2, T> operator OP(typename identity_t<T>::type s, const vec<2, T>& a) { \
        return vec<2, T>(s OP a.x, s OP a.y);                                          \
    }

GLMSHIM_BINOP(+)
GLMSHIM_BINOP(-)
GLMSHIM_BINOP(*)
GLMSHIM_BINOP(/)
#undef GLMSHIM_BINOP

template <typename T>
constexpr vec<3, T> operator-(const vec<3, T>& a) { return vec<3, T>(-a.x, -a.y, -a.z); }
template <typename T>
constexpr vec<2, T> operator-(const vec<2, T>& a) { return vec<2, T>(-a.x, -a.y); }
template <typename T>
constexpr vec<3, T> operator+(const vec<3, T>& a) { return a; }

template <typename T>
constexpr bool operator==(const vec<3, T>& a, const vec<3, T>& b) {
    return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <typename T>
constexpr bool operator!=(const vec<3, T>& a, const vec<3, T>& b) { return !(a == b); }
template <typename T>
constexpr bool operator==(const vec<2, T>& a, const vec<2, T>& b) { return a.x == b.x && a.y == b.y; }
template <typename T>
constexpr bool operator!=(const vec<2, T>& a, const vec<2, T>& b) { return !(a == b); }

// ---- geometric functions ----------------------------------------------------
template <typename T>
inline T dot(const vec<3, T>& a, const vec<3, T>& b) {
    vec<3, T> t(a * b);
    return t.x + t.y + t.z;
}
template <typename T>
inline T dot(const vec<2, T>& a, const vec<2, T>& b) {
    vec<2, T> t(a * b);
    return t.x + t.y;
}
template <int L, typename T>
inline T length(const vec<L, T>& v) { return std::sqrt(dot(v, v)); }
template <int L, typename T>
inline vec<L, T> normalize(const vec<L, T>& v) {
    return v * (static_cast<T>(1) / std::sqrt(dot(v, v)));
}

typedef vec<3, double> dvec3;
typedef vec<3, float> vec3;
typedef vec<3, int> ivec3;
typedef vec<2, double> dvec2;
typedef vec<2, float> vec2;
typedef vec<2, int> ivec2;

}  // namespace glm
