// Device math for the contact path.  Every operation keeps the association
// order of the reference's math types so that, compiled with --fmad=false and
// IEEE division/sqrt, results are bit-identical to the CPU reference:
//   Vec3/Quaternion/Mat3 (include/phys/math/{vec3,quaternion,mat3}.hpp),
//   Math3d::{dot,cross,length,normalize,clamp} (src/math/math_utils.cpp,
//   include/phys/math/math_utils.hpp).
#pragma once
#include <cstdint>

#define PE_HD __host__ __device__ __forceinline__

namespace pe {

struct V3 {
    float x, y, z;
};
PE_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
PE_HD V3 operator+(const V3 &a, const V3 &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PE_HD V3 operator-(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PE_HD V3 operator-(const V3 &a) { return {-a.x, -a.y, -a.z}; }
PE_HD V3 operator*(const V3 &a, float s) { return {a.x * s, a.y * s, a.z * s}; }
PE_HD V3 operator/(const V3 &a, float s) { return {a.x / s, a.y / s, a.z / s}; }
PE_HD V3 &operator+=(V3 &a, const V3 &b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    return a;
}
PE_HD float dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PE_HD V3 cross(const V3 &a, const V3 &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
PE_HD float length(const V3 &v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
PE_HD V3 normalize(const V3 &v) {
    float len = length(v);
    if (len <= 1e-8f) return {0.0f, 0.0f, 0.0f};
    return v * (1.0f / len);
}
// std::max / std::min argument semantics (first operand on ties / NaN).
PE_HD float smax(float a, float b) { return (a < b) ? b : a; }
PE_HD float smin(float a, float b) { return (b < a) ? b : a; }
PE_HD float clampv(float v, float lo, float hi) {
    if (lo == hi) return lo;
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}

struct Q {
    float x, y, z, w;
};
PE_HD Q qidentity() { return {0.0f, 0.0f, 0.0f, 1.0f}; }
PE_HD Q qmul(const Q &a, const Q &o) {
    return {a.w * o.x + a.x * o.w + a.y * o.z - a.z * o.y,
            a.w * o.y - a.x * o.z + a.y * o.w + a.z * o.x,
            a.w * o.z + a.x * o.y - a.y * o.x + a.z * o.w,
            a.w * o.w - a.x * o.x - a.y * o.y - a.z * o.z};
}
PE_HD Q conj(const Q &q) { return {-q.x, -q.y, -q.z, q.w}; }
PE_HD Q qnormalized(const Q &q) {
    float len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (len == 0.0f) return qidentity();
    return {q.x / len, q.y / len, q.z / len, q.w / len};
}
PE_HD V3 rotate(const Q &q, const V3 &v) {
    Q p{v.x, v.y, v.z, 0.0f};
    Q r = qmul(qmul(q, p), conj(q));
    return {r.x, r.y, r.z};
}

struct M3 {
    float m00, m01, m02, m10, m11, m12, m20, m21, m22;
};
PE_HD M3 toMat3(const Q &q) {
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    return {1.0f - 2.0f * (yy + zz), 2.0f * (xy - wz), 2.0f * (xz + wy),
            2.0f * (xy + wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz - wx),
            2.0f * (xz - wy), 2.0f * (yz + wx), 1.0f - 2.0f * (xx + yy)};
}
PE_HD V3 mul(const M3 &m, const V3 &v) {
    return {m.m00 * v.x + m.m01 * v.y + m.m02 * v.z,
            m.m10 * v.x + m.m11 * v.y + m.m12 * v.z,
            m.m20 * v.x + m.m21 * v.y + m.m22 * v.z};
}
PE_HD M3 mul(const M3 &l, const M3 &r) {
    return {l.m00 * r.m00 + l.m01 * r.m10 + l.m02 * r.m20,
            l.m00 * r.m01 + l.m01 * r.m11 + l.m02 * r.m21,
            l.m00 * r.m02 + l.m01 * r.m12 + l.m02 * r.m22,
            l.m10 * r.m00 + l.m11 * r.m10 + l.m12 * r.m20,
            l.m10 * r.m01 + l.m11 * r.m11 + l.m12 * r.m21,
            l.m10 * r.m02 + l.m11 * r.m12 + l.m12 * r.m22,
            l.m20 * r.m00 + l.m21 * r.m10 + l.m22 * r.m20,
            l.m20 * r.m01 + l.m21 * r.m11 + l.m22 * r.m21,
            l.m20 * r.m02 + l.m21 * r.m12 + l.m22 * r.m22};
}
PE_HD M3 transpose(const M3 &v) { return {v.m00, v.m10, v.m20, v.m01, v.m11, v.m21, v.m02, v.m12, v.m22}; }

// RigidBody::getInverseInertiaWorld (include/phys/dynamics/rigid_body.hpp:97-101):
// (R * I_local) * R^T with the diagonal local inverse inertia.
PE_HD M3 inverseInertiaWorld(const Q &q, float ixx, float iyy, float izz) {
    M3 R = toMat3(q);
    M3 I{ixx, 0.0f, 0.0f, 0.0f, iyy, 0.0f, 0.0f, 0.0f, izz};
    return mul(mul(R, I), transpose(R));
}

struct Tf {
    V3 p;
    Q q;
};
PE_HD V3 toLocal(const V3 &w, const Tf &t) { return rotate(conj(t.q), w - t.p); }
PE_HD V3 toWorld(const V3 &l, const Tf &t) { return t.p + rotate(t.q, l); }

PE_HD V3 f4xyz(const float4 &a) { return {a.x, a.y, a.z}; }
PE_HD Q f4q(const float4 &a) { return {a.x, a.y, a.z, a.w}; }
PE_HD float4 make4(const V3 &v, float w) { return make_float4(v.x, v.y, v.z, w); }
PE_HD float4 make4(const Q &q) { return make_float4(q.x, q.y, q.z, q.w); }

// Total order on floats used by the SAP sort (min.x ascending, ties by index):
// -0 and +0 compare equal in the reference's comparison, so both map to +0.
__device__ __forceinline__ uint32_t orderedFloatKey(float f) {
    uint32_t u = __float_as_uint(f == 0.0f ? 0.0f : f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

} // namespace pe
