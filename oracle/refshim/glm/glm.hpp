// A minimal, project-written stand-in for the parts of the glm API that
// CRender's src/util/sampling.h, src/render/camera.{h,cpp}, src/render/ray.{h,cpp}
// and the headers they include use, so that those reference files compile
// unmodified for the oracle's cross-check (oracle/ref_bridge.cpp).  TEST
// INFRASTRUCTURE ONLY; not glm itself.  Single precision only; every operation
// is the plain component-wise or textbook definition, summed left to right:
//   dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z,  normalize(v) = v * (1 / sqrt(dot(v, v))),
//   M * v     = ((M[0]*v.x + M[1]*v.y) + M[2]*v.z) (+ M[3]*v.w)   (M[i] = column i).
#pragma once
#include <cmath>
#include <cstddef>
#include <cstring>

namespace glm {

struct vec2 {
    float x = 0, y = 0;
    constexpr vec2() = default;
    constexpr explicit vec2(float s) : x(s), y(s) {}
    constexpr vec2(float a_, float b_) : x(a_), y(b_) {}
    float &operator[](int i) { return i == 0 ? x : y; }
    float operator[](int i) const { return i == 0 ? x : y; }
};

struct vec4;
struct vec3 {
    union { float x = 0; float r; };
    union { float y = 0; float g; };
    union { float z = 0; float b; };
    constexpr vec3() = default;
    constexpr explicit vec3(float s) : x(s), y(s), z(s) {}
    constexpr vec3(float a_, float b_, float c_) : x(a_), y(b_), z(c_) {}
    vec3(const vec4 &v); // implicit, as ray.cpp:18-24 relies on
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3 &operator+=(const vec3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3 &operator*=(const vec3 &o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    vec3 &operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3 &operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};

struct vec4 {
    union { float x = 0; float r; };
    union { float y = 0; float g; };
    union { float z = 0; float b; };
    union { float w = 0; float a; };
    constexpr vec4() = default;
    constexpr explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    constexpr vec4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
    constexpr vec4(const vec3 &v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};
inline vec3::vec3(const vec4 &v) : x(v.x), y(v.y), z(v.z) {}

// vector arithmetic, component-wise
inline vec2 operator+(vec2 a, vec2 b) { return {a.x + b.x, a.y + b.y}; }
inline vec2 operator*(vec2 a, float s) { return {a.x * s, a.y * s}; }
inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline vec3 operator*(vec3 a, vec3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline vec3 operator/(vec3 a, vec3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline vec3 operator-(vec3 a) { return {-a.x, -a.y, -a.z}; }
inline vec3 operator*(vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline vec3 operator*(float s, vec3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline vec3 operator/(vec3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline vec3 operator/(float s, vec3 a) { return {s / a.x, s / a.y, s / a.z}; }
inline vec3 operator+(vec3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline vec3 operator+(float s, vec3 a) { return {s + a.x, s + a.y, s + a.z}; }
inline vec3 operator-(vec3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
inline vec3 operator-(float s, vec3 a) { return {s - a.x, s - a.y, s - a.z}; }
inline bool operator==(vec3 a, vec3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline vec4 operator+(vec4 a, vec4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline vec4 operator-(vec4 a, vec4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline vec4 operator*(vec4 a, vec4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
inline vec4 operator*(vec4 a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
inline vec4 operator*(float s, vec4 a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
inline vec4 operator/(vec4 a, float s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
inline bool operator==(vec4 a, vec4 b) { return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w; }

// column-major matrices: m[i] is column i
struct mat3 {
    vec3 c[3];
    mat3() : mat3(1.0f) {}
    explicit mat3(float d) : c{vec3(d, 0, 0), vec3(0, d, 0), vec3(0, 0, d)} {}
    mat3(const vec3 &a, const vec3 &b, const vec3 &d) : c{a, b, d} {}
    vec3 &operator[](int i) { return c[i]; }
    const vec3 &operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    mat4() : mat4(1.0f) {}
    explicit mat4(float d) : c{vec4(d, 0, 0, 0), vec4(0, d, 0, 0), vec4(0, 0, d, 0), vec4(0, 0, 0, d)} {}
    vec4 &operator[](int i) { return c[i]; }
    const vec4 &operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3 &m, vec3 v) { return (m[0] * v.x + m[1] * v.y) + m[2] * v.z; }
inline vec4 operator*(const mat4 &m, vec4 v) { return ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3] * v.w; }
inline mat4 operator*(const mat4 &a, const mat4 &b) {
    mat4 r;
    for (int i = 0; i < 4; ++i) r[i] = a * b[i];
    return r;
}

// scalar functions: the C++ library's
inline float radians(float deg) { return deg * (3.14159265358979323846f / 180.0f); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float tan(float x) { return std::tan(x); }
inline float acos(float x) { return std::acos(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float clamp(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

// geometric functions
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot(vec4 a, vec4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
inline vec3 cross(vec3 a, vec3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline float distance(vec3 a, vec3 b) { return length(b - a); }
inline vec3 normalize(vec3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline vec4 normalize(vec4 v) { return v * (1.0f / std::sqrt(dot(v, v))); }

} // namespace glm
