// Small vector algebra for the device code (the reference wraps Eigen,
// src/core/math/include/krrmath/*; only the operations the path needs are here).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define KRR_HD __host__ __device__ __forceinline__
#define KRR_D __device__ __forceinline__

namespace krr {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInv2Pi = 0.15915494309189533577f;
constexpr float kInv4Pi = 0.07957747154594766788f;
constexpr float k2Pi = 6.28318530717958647692f;
constexpr float kRayEps = 1e-4f;   // KRR_RAY_EPS, src/core/raytracing.h:10

struct V3 {
    float x, y, z;
};

KRR_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
KRR_HD V3 v3(float s) { return V3{s, s, s}; }
KRR_HD V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
KRR_HD V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
KRR_HD V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
KRR_HD V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
KRR_HD V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
KRR_HD V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
KRR_HD V3 operator*(float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
KRR_HD V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
KRR_HD V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
KRR_HD V3 &operator*=(V3 &a, V3 b) { a = a * b; return a; }
KRR_HD V3 &operator*=(V3 &a, float s) { a = a * s; return a; }
KRR_HD V3 &operator/=(V3 &a, float s) { a = a / s; return a; }
KRR_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
KRR_HD V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
KRR_HD float length_sq(V3 a) { return dot(a, a); }
KRR_HD float length(V3 a) { return sqrtf(dot(a, a)); }
KRR_HD V3 normalize(V3 a) { return a / length(a); }
KRR_HD V3 vabs(V3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
KRR_HD V3 vmin(V3 a, V3 b) { return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
KRR_HD V3 vmax(V3 a, V3 b) { return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
KRR_HD float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
KRR_HD bool any(V3 a) { return a.x != 0.f || a.y != 0.f || a.z != 0.f; }
KRR_HD bool is_zero(V3 a) { return !any(a); }
KRR_HD float mean(V3 a) { return (a.x + a.y + a.z) / 3.f; }
KRR_HD float max_coeff(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
KRR_HD V3 vexp(V3 a) { return {expf(a.x), expf(a.y), expf(a.z)}; }
KRR_HD V3 vsqrt(V3 a) { return {sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)}; }

KRR_HD V3 f3(float4 a) { return {a.x, a.y, a.z}; }
KRR_HD float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// Row-major 3x4 affine transform (object -> world).
struct Xform {
    float m[12];
};
KRR_HD V3 xform_point(const float *m, V3 p) {
    return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
            m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
KRR_HD V3 xform_vector(const float *m, V3 v) {
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z,
            m[4] * v.x + m[5] * v.y + m[6] * v.z,
            m[8] * v.x + m[9] * v.y + m[10] * v.z};
}
// Multiply by a row-major 3x3 matrix.
KRR_HD V3 mat3_mul(const float *m, V3 v) {
    return {m[0] * v.x + m[1] * v.y + m[2] * v.z,
            m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
KRR_HD V3 mat3_mul_transposed(const float *m, V3 v) {
    return {m[0] * v.x + m[3] * v.y + m[6] * v.z,
            m[1] * v.x + m[4] * v.y + m[7] * v.z,
            m[2] * v.x + m[5] * v.y + m[8] * v.z};
}

}  // namespace krr
