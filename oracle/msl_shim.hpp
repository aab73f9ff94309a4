// msl_shim.hpp - the few Metal Shading Language types and functions that the reference's
// path-tracing shader source (backends/metal/plugin.mm:46-276) uses, as plain C++ so that
// source compiles with g++ and runs on the CPU. TEST INFRASTRUCTURE ONLY (oracle/_ref).
//
// Semantics follow the MSL specification: float3 arithmetic is componentwise, normalize(x)
// is x / length(x), rsqrt(x) is 1 / sqrt(x). float2 is an aggregate so that
// float2(a(), b()) is parenthesised aggregate initialisation, which C++20 evaluates left to
// right as the Metal compiler does.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace msl {

using uint = unsigned int;
#define thread
#define constant const
#define M_PI_F 3.14159265358979323846f

struct packed_float3 {
    float x, y, z;
};

struct float3 {
    float x, y, z;
    float3() : x(0), y(0), z(0) {}
    explicit float3(float s) : x(s), y(s), z(s) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit float3(const packed_float3& p) : x(p.x), y(p.y), z(p.z) {}
    float3& operator+=(float3 o) { x += o.x; y += o.y; z += o.z; return *this; }
    float3& operator*=(float3 o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    float3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
};
inline float3 operator+(float3 a, float3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(float3 a, float3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator-(float3 a) { return {-a.x, -a.y, -a.z}; }
inline float3 operator*(float3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float3 operator*(float s, float3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float3 operator*(float3 a, float3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float3 operator/(float3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float3 operator+(float3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }

struct float2 {
    float x, y;
};
inline float2 operator-(float2 a, float s) { return float2{a.x - s, a.y - s}; }
inline float2 operator*(float2 a, float s) { return float2{a.x * s, a.y * s}; }
inline float2& operator+=(float2& a, float2 b) { a.x += b.x; a.y += b.y; return a; }

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float3 normalize(float3 v) { return v / std::sqrt(dot(v, v)); }
inline float rsqrt(float x) { return 1.0f / std::sqrt(x); }
inline float abs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float tan(float x) { return std::tan(x); }
inline float max(float a, float b) { return std::max(a, b); }

}  // namespace msl
