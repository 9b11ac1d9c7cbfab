// Minimal vector-math header standing in for the header-only glm library, which is not
// installed here. It is written for this project and only used to compile the reference's
// CPU ray tracer (rt/cpu/bvh2.cpp, libgi/timer.cpp, libgi/rt.cpp) unmodified into
// oracle/_ref/. It is test infrastructure, not part of the product.
//
// Semantics that affect results are those of glm 0.9.9:
//   min(x, y) = (y < x) ? y : x        max(x, y) = (x < y) ? y : x   (component-wise)
//   normalize(v) = v * (1 / sqrt(dot(v, v)))
// Every vector operation is component-wise in plain IEEE float; the recipe compiles with
// -ffp-contract=off so no product is fused into an add.
#pragma once
// glm itself pulls these in; the reference headers rely on that.
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <string>
#include <type_traits>

namespace glm {

typedef int length_t;

template <int L, typename T> struct vec;

template <typename T> struct vec<2, T> {
    T x, y;
    vec() : x(0), y(0) {}
    explicit vec(T s) : x(s), y(s) {}
    vec(T a, T b) : x(a), y(b) {}
    template <typename U> explicit vec(const vec<2, U> &o) : x(T(o.x)), y(T(o.y)) {}
    T &operator[](int i) { return i == 0 ? x : y; }
    const T &operator[](int i) const { return i == 0 ? x : y; }
    static constexpr length_t length() { return 2; }
};

template <typename T> struct vec<3, T> {
    T x, y, z;
    vec() : x(0), y(0), z(0) {}
    vec(T s) : x(s), y(s), z(s) {}
    vec(T a, T b, T c) : x(a), y(b), z(c) {}
    vec(const vec<4, T> &o);
    template <typename U> explicit vec(const vec<3, U> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    static constexpr length_t length() { return 3; }
};

template <typename T> struct vec<4, T> {
    T x, y, z, w;
    vec() : x(0), y(0), z(0), w(0) {}
    explicit vec(T s) : x(s), y(s), z(s), w(s) {}
    vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    vec(const vec<3, T> &v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    template <typename U> explicit vec(const vec<4, U> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    static constexpr length_t length() { return 4; }
};

template <typename T> vec<3, T>::vec(const vec<4, T> &o) : x(o.x), y(o.y), z(o.z) {}

typedef vec<2, float> vec2;
typedef vec<3, float> vec3;
typedef vec<4, float> vec4;
typedef vec<2, int> ivec2;
typedef vec<3, int> ivec3;
typedef vec<4, int> ivec4;
typedef vec<2, unsigned> uvec2;
typedef vec<3, unsigned> uvec3;
typedef vec<4, unsigned> uvec4;

struct mat4 {
    float m[4][4];
    mat4() {
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) m[i][j] = (i == j) ? 1.f : 0.f;
    }
    explicit mat4(float s) {
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) m[i][j] = (i == j) ? s : 0.f;
    }
};

// Right-hand operand of a compound assignment: a scalar of any arithmetic type is first
// converted to the vector's component type (as glm does, e.g. `normal *= -1`); a vector
// passes through unchanged.
template <typename T, typename V, typename std::enable_if<std::is_arithmetic<V>::value, int>::type = 0>
T shim_operand(const V &b) {
    return T(b);
}
template <typename T, typename V, typename std::enable_if<!std::is_arithmetic<V>::value, int>::type = 0>
const V &shim_operand(const V &b) {
    return b;
}

#define GRT_SHIM_BINOP(OP)                                                                          \
    template <typename T> vec<2, T> operator OP(const vec<2, T> &a, const vec<2, T> &b) {            \
        return vec<2, T>(a.x OP b.x, a.y OP b.y);                                                   \
    }                                                                                               \
    template <typename T> vec<3, T> operator OP(const vec<3, T> &a, const vec<3, T> &b) {            \
        return vec<3, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                                       \
    }                                                                                               \
    template <typename T> vec<4, T> operator OP(const vec<4, T> &a, const vec<4, T> &b) {            \
        return vec<4, T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                           \
    }                                                                                               \
    template <typename T> vec<2, T> operator OP(const vec<2, T> &a, T s) {                          \
        return vec<2, T>(a.x OP s, a.y OP s);                                                       \
    }                                                                                               \
    template <typename T> vec<3, T> operator OP(const vec<3, T> &a, T s) {                          \
        return vec<3, T>(a.x OP s, a.y OP s, a.z OP s);                                             \
    }                                                                                               \
    template <typename T> vec<4, T> operator OP(const vec<4, T> &a, T s) {                          \
        return vec<4, T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s);                                   \
    }                                                                                               \
    template <typename T> vec<2, T> operator OP(T s, const vec<2, T> &a) {                          \
        return vec<2, T>(s OP a.x, s OP a.y);                                                       \
    }                                                                                               \
    template <typename T> vec<3, T> operator OP(T s, const vec<3, T> &a) {                          \
        return vec<3, T>(s OP a.x, s OP a.y, s OP a.z);                                             \
    }                                                                                               \
    template <typename T> vec<4, T> operator OP(T s, const vec<4, T> &a) {                          \
        return vec<4, T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w);                                   \
    }                                                                                               \
    template <int L, typename T, typename V> vec<L, T> &operator OP##=(vec<L, T> &a, const V &b) {  \
        a = a OP shim_operand<T>(b);                                                                \
        return a;                                                                                   \
    }

GRT_SHIM_BINOP(+)
GRT_SHIM_BINOP(-)
GRT_SHIM_BINOP(*)
GRT_SHIM_BINOP(/)
#undef GRT_SHIM_BINOP

// double/int scalars mixed with float vectors (e.g. `1.0 - beta` style expressions in the sources)
inline vec3 operator*(double s, const vec3 &a) { return float(s) * a; }
inline vec2 operator*(double s, const vec2 &a) { return float(s) * a; }

template <typename T> vec<2, T> operator-(const vec<2, T> &a) { return vec<2, T>(-a.x, -a.y); }
template <typename T> vec<3, T> operator-(const vec<3, T> &a) { return vec<3, T>(-a.x, -a.y, -a.z); }
template <typename T> vec<4, T> operator-(const vec<4, T> &a) { return vec<4, T>(-a.x, -a.y, -a.z, -a.w); }

template <typename T> bool operator==(const vec<2, T> &a, const vec<2, T> &b) { return a.x == b.x && a.y == b.y; }
template <typename T> bool operator==(const vec<3, T> &a, const vec<3, T> &b) {
    return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <typename T> bool operator==(const vec<4, T> &a, const vec<4, T> &b) {
    return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}
template <int L, typename T> bool operator!=(const vec<L, T> &a, const vec<L, T> &b) { return !(a == b); }

template <typename T> T min(T x, T y) { return (y < x) ? y : x; }
template <typename T> T max(T x, T y) { return (x < y) ? y : x; }
template <typename T> vec<2, T> min(const vec<2, T> &a, const vec<2, T> &b) {
    return vec<2, T>(min(a.x, b.x), min(a.y, b.y));
}
template <typename T> vec<3, T> min(const vec<3, T> &a, const vec<3, T> &b) {
    return vec<3, T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z));
}
template <typename T> vec<2, T> max(const vec<2, T> &a, const vec<2, T> &b) {
    return vec<2, T>(max(a.x, b.x), max(a.y, b.y));
}
template <typename T> vec<3, T> max(const vec<3, T> &a, const vec<3, T> &b) {
    return vec<3, T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z));
}
template <typename T> T clamp(T v, T lo, T hi) { return min(max(v, lo), hi); }

inline float dot(const vec2 &a, const vec2 &b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3 &a, const vec3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4 &a, const vec4 &b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec3 cross(const vec3 &a, const vec3 &b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3 &a) { return std::sqrt(dot(a, a)); }
inline float length(const vec2 &a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3 &a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline vec2 normalize(const vec2 &a) { return a * (1.0f / std::sqrt(dot(a, a))); }
inline vec3 abs(const vec3 &a) { return vec3(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }
inline float abs(float x) { return std::fabs(x); }
inline vec2 floor(const vec2 &a) { return vec2(std::floor(a.x), std::floor(a.y)); }
inline float radians(float d) { return d * float(M_PI / 180.0); }
inline vec3 fract(const vec3 &a) { return vec3(a.x - std::floor(a.x), a.y - std::floor(a.y), a.z - std::floor(a.z)); }
// mix(x, y, a) = x * (1 - a) + y * a
inline vec3 mix(const vec3 &x, const vec3 &y, float a) { return x * (1.0f - a) + y * a; }

template <int L, typename T> std::string to_string(const vec<L, T> &v) {
    std::string s = "vec(";
    for (int i = 0; i < L; ++i) s += (i ? ", " : "") + std::to_string(v[i]);
    return s + ")";
}

}  // namespace glm
