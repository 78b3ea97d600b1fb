// Scalar-generic math for the differentiable rollout.  The same formulas as the
// engine's float math (pe_math.cuh), written over a scalar type S so that one
// source serves float (GPU), double (the FP64 CPU adjoint) and forward-mode
// dual numbers (Jacobians of contact geometry and contact preparation).  With
// S = float the operations, their order and their constants are the engine's,
// so values are bit-identical; a dual number's value part is computed by the
// same operations as the plain scalar.  Compiles as CUDA and as plain C++.
#pragma once
#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define AD_HD __host__ __device__ __forceinline__
// Large routines are compiled once and called, which keeps the kernels' code
// size and compile time down.
#define AD_HDN __host__ __device__ __noinline__
#else
#define AD_HD inline
#define AD_HDN inline
#endif

namespace pe {
namespace ad {

AD_HD float ssqrt(float v) { return sqrtf(v); }
AD_HD double ssqrt(double v) { return sqrt(v); }
AD_HD float sabs(float v) { return fabsf(v); }
AD_HD double sabs(double v) { return fabs(v); }

// ------------------------------------------------------------ dual numbers ---
// Value plus K tangent components.  Comparisons use the value only, so a dual
// evaluation takes exactly the branches of the plain evaluation.
template <class T, int K> struct Dual {
    T v;
    T d[K];
};
template <class T, int K> AD_HD Dual<T, K> dconst(T v) {
    Dual<T, K> r;
    r.v = v;
    for (int k = 0; k < K; ++k) r.d[k] = T(0);
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator+(const Dual<T, K> &a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a.v + b.v;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator-(const Dual<T, K> &a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a.v - b.v;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator-(const Dual<T, K> &a) {
    Dual<T, K> r;
    r.v = -a.v;
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator*(const Dual<T, K> &a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a.v * b.v;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator/(const Dual<T, K> &a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a.v / b.v;
    const T inv = T(1) / b.v;
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator+(const Dual<T, K> &a, T b) {
    Dual<T, K> r = a;
    r.v = a.v + b;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator+(T a, const Dual<T, K> &b) {
    Dual<T, K> r = b;
    r.v = a + b.v;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator-(const Dual<T, K> &a, T b) {
    Dual<T, K> r = a;
    r.v = a.v - b;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator-(T a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a - b.v;
    for (int k = 0; k < K; ++k) r.d[k] = -b.d[k];
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator*(const Dual<T, K> &a, T b) {
    Dual<T, K> r;
    r.v = a.v * b;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator*(T a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a * b.v;
    for (int k = 0; k < K; ++k) r.d[k] = a * b.d[k];
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator/(const Dual<T, K> &a, T b) {
    Dual<T, K> r;
    r.v = a.v / b;
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / b;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> operator/(T a, const Dual<T, K> &b) {
    Dual<T, K> r;
    r.v = a / b.v;
    const T inv = T(1) / b.v;
    for (int k = 0; k < K; ++k) r.d[k] = -r.v * b.d[k] * inv;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> &operator+=(Dual<T, K> &a, const Dual<T, K> &b) {
    a = a + b;
    return a;
}
template <class T, int K> AD_HD Dual<T, K> ssqrt(const Dual<T, K> &a) {
    Dual<T, K> r;
    r.v = ssqrt(a.v);
    const T g = r.v > T(0) ? T(0.5) / r.v : T(0);
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * g;
    return r;
}
template <class T, int K> AD_HD Dual<T, K> sabs(const Dual<T, K> &a) { return a.v < T(0) ? -a : a; }

AD_HD float val(float v) { return v; }
AD_HD double val(double v) { return v; }
template <class T, int K> AD_HD T val(const Dual<T, K> &a) { return a.v; }

// Scalar S built from a constant of its value type (float constants first
// rounded to float, as the reference writes them).
template <class S> struct Lit {
    template <class C> AD_HD static S make(C c) { return S(c); }
};
template <class T, int K> struct Lit<Dual<T, K>> {
    template <class C> AD_HD static Dual<T, K> make(C c) { return dconst<T, K>(T(c)); }
};
#define ADL(S, c) ::pe::ad::Lit<S>::make(c)

// std::max / std::min argument semantics (first operand on ties / NaN).
template <class S> AD_HD S smax(const S &a, const S &b) { return (val(a) < val(b)) ? b : a; }
template <class S> AD_HD S smin(const S &a, const S &b) { return (val(b) < val(a)) ? b : a; }

// ------------------------------------------------------------------ vectors --
template <class S> struct V3 {
    S x, y, z;
};
template <class S> AD_HD V3<S> operator+(const V3<S> &a, const V3<S> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S> AD_HD V3<S> operator-(const V3<S> &a, const V3<S> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S> AD_HD V3<S> operator-(const V3<S> &a) { return {-a.x, -a.y, -a.z}; }
template <class S> AD_HD V3<S> operator*(const V3<S> &a, const S &s) { return {a.x * s, a.y * s, a.z * s}; }
template <class S> AD_HD V3<S> operator/(const V3<S> &a, const S &s) { return {a.x / s, a.y / s, a.z / s}; }
template <class S> AD_HD V3<S> &operator+=(V3<S> &a, const V3<S> &b) {
    a.x = a.x + b.x;
    a.y = a.y + b.y;
    a.z = a.z + b.z;
    return a;
}
template <class S> AD_HD S dot(const V3<S> &a, const V3<S> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S> AD_HD V3<S> cross(const V3<S> &a, const V3<S> &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class S> AD_HD S length(const V3<S> &v) { return ssqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
template <class S> AD_HD V3<S> normalize(const V3<S> &v) {
    S len = length(v);
    if (val(len) <= 1e-8f) return {ADL(S, 0.0f), ADL(S, 0.0f), ADL(S, 0.0f)};
    return v * (ADL(S, 1.0f) / len);
}
template <class S> AD_HD S clampv(const S &v, const S &lo, const S &hi) {
    if (val(lo) == val(hi)) return lo;
    if (val(v) < val(lo)) return lo;
    if (val(v) > val(hi)) return hi;
    return v;
}

template <class S> struct Q {
    S x, y, z, w;
};
template <class S> AD_HD Q<S> qidentity() { return {ADL(S, 0.0f), ADL(S, 0.0f), ADL(S, 0.0f), ADL(S, 1.0f)}; }
template <class S> AD_HD Q<S> qmul(const Q<S> &a, const Q<S> &o) {
    return {a.w * o.x + a.x * o.w + a.y * o.z - a.z * o.y, a.w * o.y - a.x * o.z + a.y * o.w + a.z * o.x,
            a.w * o.z + a.x * o.y - a.y * o.x + a.z * o.w, a.w * o.w - a.x * o.x - a.y * o.y - a.z * o.z};
}
template <class S> AD_HD Q<S> conj(const Q<S> &q) { return {-q.x, -q.y, -q.z, q.w}; }
template <class S> AD_HD Q<S> qnormalized(const Q<S> &q) {
    S len = ssqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (val(len) == 0.0f) return qidentity<S>();
    return {q.x / len, q.y / len, q.z / len, q.w / len};
}
template <class S> AD_HD V3<S> rotate(const Q<S> &q, const V3<S> &v) {
    Q<S> p{v.x, v.y, v.z, ADL(S, 0.0f)};
    Q<S> r = qmul(qmul(q, p), conj(q));
    return {r.x, r.y, r.z};
}

template <class S> struct M3 {
    S m00, m01, m02, m10, m11, m12, m20, m21, m22;
};
template <class S> AD_HD M3<S> toMat3(const Q<S> &q) {
    S xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    S xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    S wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    const S one = ADL(S, 1.0f), two = ADL(S, 2.0f);
    return {one - two * (yy + zz), two * (xy - wz), two * (xz + wy),
            two * (xy + wz),       one - two * (xx + zz), two * (yz - wx),
            two * (xz - wy),       two * (yz + wx),       one - two * (xx + yy)};
}
template <class S> AD_HD V3<S> mul(const M3<S> &m, const V3<S> &v) {
    return {m.m00 * v.x + m.m01 * v.y + m.m02 * v.z, m.m10 * v.x + m.m11 * v.y + m.m12 * v.z,
            m.m20 * v.x + m.m21 * v.y + m.m22 * v.z};
}
template <class S> AD_HD M3<S> mul(const M3<S> &l, const M3<S> &r) {
    return {l.m00 * r.m00 + l.m01 * r.m10 + l.m02 * r.m20, l.m00 * r.m01 + l.m01 * r.m11 + l.m02 * r.m21,
            l.m00 * r.m02 + l.m01 * r.m12 + l.m02 * r.m22, l.m10 * r.m00 + l.m11 * r.m10 + l.m12 * r.m20,
            l.m10 * r.m01 + l.m11 * r.m11 + l.m12 * r.m21, l.m10 * r.m02 + l.m11 * r.m12 + l.m12 * r.m22,
            l.m20 * r.m00 + l.m21 * r.m10 + l.m22 * r.m20, l.m20 * r.m01 + l.m21 * r.m11 + l.m22 * r.m21,
            l.m20 * r.m02 + l.m21 * r.m12 + l.m22 * r.m22};
}
template <class S> AD_HD M3<S> transpose(const M3<S> &v) {
    return {v.m00, v.m10, v.m20, v.m01, v.m11, v.m21, v.m02, v.m12, v.m22};
}
// (R * I_local) * R^T with the diagonal local inverse inertia
// (include/phys/dynamics/rigid_body.hpp:97-101).
template <class S> AD_HD M3<S> inverseInertiaWorld(const Q<S> &q, const S &ixx, const S &iyy, const S &izz) {
    M3<S> R = toMat3(q);
    const S z = ADL(S, 0.0f);
    M3<S> I{ixx, z, z, z, iyy, z, z, z, izz};
    return mul(mul(R, I), transpose(R));
}

template <class S> struct Tf {
    V3<S> p;
    Q<S> q;
};
template <class S> AD_HD V3<S> toLocal(const V3<S> &w, const Tf<S> &t) { return rotate(conj(t.q), w - t.p); }
template <class S> AD_HD V3<S> toWorld(const V3<S> &l, const Tf<S> &t) { return t.p + rotate(t.q, l); }

// Plain-scalar reverse helpers.
// c = a x b: abar += b x cbar, bbar += cbar x a.
template <class S> AD_HD void crossAdj(const V3<S> &a, const V3<S> &b, const V3<S> &cbar, V3<S> &abar, V3<S> &bbar) {
    abar += cross(b, cbar);
    bbar += cross(cbar, a);
}
// r = qmul(a, o): adjoints of a and o.
template <class S> AD_HD void qmulAdj(const Q<S> &a, const Q<S> &o, const Q<S> &r, Q<S> &ab, Q<S> &ob) {
    ab.x = ab.x + (r.x * o.w - r.y * o.z + r.z * o.y - r.w * o.x);
    ab.y = ab.y + (r.x * o.z + r.y * o.w - r.z * o.x - r.w * o.y);
    ab.z = ab.z + (-r.x * o.y + r.y * o.x + r.z * o.w - r.w * o.z);
    ab.w = ab.w + (r.x * o.x + r.y * o.y + r.z * o.z + r.w * o.w);
    ob.x = ob.x + (r.x * a.w + r.y * a.z - r.z * a.y - r.w * a.x);
    ob.y = ob.y + (-r.x * a.z + r.y * a.w + r.z * a.x - r.w * a.y);
    ob.z = ob.z + (r.x * a.y - r.y * a.x + r.z * a.w - r.w * a.z);
    ob.w = ob.w + (r.x * a.x + r.y * a.y + r.z * a.z + r.w * a.w);
}

} // namespace ad
} // namespace pe
