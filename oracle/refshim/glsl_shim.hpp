// glsl_shim.hpp -- just enough GLSL, as C++, to compile the reference's
// BRDF, p-hat and software-traversal shader includes unmodified on the CPU.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle's reference build).
//
// GLSL gives an unsuffixed floating literal type float; C++ gives it type
// double.  The reference's shader code uses such literals (1.0, 0.5, M_PI), so
// compiled as plain C++ it would compute parts of the BRDF in double.  The
// shim therefore maps the GLSL `float` type to `gfloat`, a wrapper whose every
// arithmetic operator first rounds both operands to float and then performs
// one single-precision operation, which is the GLSL rule.  Built-ins carry
// the same meaning as in the oracle and the CUDA kernels:
//   min(x,y) = y<x ? y : x, max(x,y) = x<y ? y : x, clamp = min(max()),
//   mix(x,y,a) = x*(1-a) + y*a, dot = (x0*y0 + x1*y1) + x2*y2,
//   normalize(v) = v / sqrt(dot(v,v)), pow = powf (so pow(r,2.0) == r*r).
#pragma once
#include <cmath>
#include <cstdint>

namespace glsl {

struct gfloat {
    float v;
    gfloat() = default;
    constexpr gfloat(float x) : v(x) {}
    constexpr gfloat(double x) : v(static_cast<float>(x)) {}
    constexpr gfloat(int x) : v(static_cast<float>(x)) {}
    constexpr gfloat(unsigned x) : v(static_cast<float>(x)) {}
    explicit operator float() const { return v; }
    gfloat &operator+=(gfloat o) { v = v + o.v; return *this; }
    gfloat &operator-=(gfloat o) { v = v - o.v; return *this; }
    gfloat &operator*=(gfloat o) { v = v * o.v; return *this; }
    gfloat &operator/=(gfloat o) { v = v / o.v; return *this; }
};
inline gfloat operator+(gfloat a, gfloat b) { return gfloat(a.v + b.v); }
inline gfloat operator-(gfloat a, gfloat b) { return gfloat(a.v - b.v); }
inline gfloat operator*(gfloat a, gfloat b) { return gfloat(a.v * b.v); }
inline gfloat operator/(gfloat a, gfloat b) { return gfloat(a.v / b.v); }
inline gfloat operator-(gfloat a) { return gfloat(-a.v); }
inline bool operator<(gfloat a, gfloat b) { return a.v < b.v; }
inline bool operator>(gfloat a, gfloat b) { return a.v > b.v; }
inline bool operator<=(gfloat a, gfloat b) { return a.v <= b.v; }
inline bool operator>=(gfloat a, gfloat b) { return a.v >= b.v; }
inline bool operator==(gfloat a, gfloat b) { return a.v == b.v; }
inline bool operator!=(gfloat a, gfloat b) { return a.v != b.v; }

struct vec3 {
    gfloat x, y, z;
    vec3() = default;
    constexpr vec3(gfloat a, gfloat b, gfloat c) : x(a), y(b), z(c) {}
    explicit constexpr vec3(gfloat a) : x(a), y(a), z(a) {}
    vec3 &operator/=(gfloat s) { x /= s; y /= s; z /= s; return *this; }
    vec3 &operator*=(gfloat s) { x *= s; y *= s; z *= s; return *this; }
};
struct vec2 {
    gfloat x, y;
    vec2() = default;
    constexpr vec2(gfloat a, gfloat b) : x(a), y(b) {}
};
// The compiled shader files only read .xyz of a vec4 (node boxes, triangle
// vertices), so vec4 is stored as {xyz, w}.
struct vec4 {
    vec3 xyz;
    gfloat w;
    vec4() = default;
    constexpr vec4(gfloat a, gfloat b, gfloat c, gfloat d) : xyz(a, b, c), w(d) {}
    constexpr vec4(vec3 v, gfloat d) : xyz(v), w(d) {}
};

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(gfloat s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, gfloat s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator/(vec3 a, gfloat s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator*(int s, vec3 a) { return gfloat(s) * a; }

inline gfloat abs(gfloat a) { return gfloat(std::fabs(a.v)); }
inline gfloat sqrt(gfloat a) { return gfloat(std::sqrt(a.v)); }
inline gfloat pow(gfloat a, gfloat b) { return gfloat(std::pow(a.v, b.v)); }
inline gfloat min(gfloat x, gfloat y) { return y < x ? y : x; }
inline gfloat max(gfloat x, gfloat y) { return x < y ? y : x; }
inline gfloat clamp(gfloat x, gfloat lo, gfloat hi) { return min(max(x, lo), hi); }
inline gfloat mix(gfloat x, gfloat y, gfloat a) { return x * (gfloat(1.0f) - a) + y * a; }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 mix(vec3 x, vec3 y, gfloat a) { return vec3(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a)); }
inline gfloat dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline gfloat length(vec3 a) { return sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }

}  // namespace glsl
