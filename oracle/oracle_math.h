// oracle_math.h — TEST INFRASTRUCTURE ONLY.  Scalar fp32 helpers of the CPU oracle.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use the
// oracle, and only as the checker.  The product library never links it.
//
// Every helper states the exact order of its fp32 operations.  The oracle is built with
// -ffp-contract=off, so a*b+c is one rounded multiply followed by one rounded add; the
// CUDA kernels are built with --fmad=false and spell the same order, which is what makes
// the two bit-identical.
//
// Reference semantics restated here:
//  - Vec3 dot / cross / lengthSquared / normalized: include/axiom/math/vec3.hpp:179-215
//    (left-to-right sums; normalized() divides each component by the length and returns
//    zero for a zero-length vector).
//  - AABB::intersects (inclusive): include/axiom/math/aabb.hpp:132-135.
//  - Quat product / rotate / normalize / fromAxisAngle: src/math/quat.cpp:27-72, which
//    delegate to GLM (glm >= 1.0.0 from vcpkg, vcpkg.json:10-11, absent here).  The
//    restatement follows GLM's published formulas: Hamilton product, v' = v + w t + q x t
//    with t = 2 q x v, normalize by multiplying with 1/length, angleAxis = (axis sin(a/2),
//    cos(a/2)).
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle {

struct V3 {
    float x, y, z;
};
struct Q4 {
    float x, y, z, w;
};

inline float maxf(float a, float b) { return a > b ? a : b; }
inline float minf(float a, float b) { return a < b ? a : b; }

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
// vec3.hpp:179-181: x*ox + y*oy + z*oz evaluated left to right.
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vec3.hpp:188-191.
inline V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// vec3.hpp:209-215.
inline V3 normalized(V3 a) {
    float len = std::sqrt(dot(a, a));
    if (len > 0.0f) return V3{a.x / len, a.y / len, a.z / len};
    return V3{0.0f, 0.0f, 0.0f};
}

// Rotation of v by unit quaternion q: t = 2 (q.xyz x v); v' = (v + w t) + q.xyz x t.
inline V3 rotate(Q4 q, V3 v) {
    V3 t{2.0f * (q.y * v.z - q.z * v.y), 2.0f * (q.z * v.x - q.x * v.z),
         2.0f * (q.x * v.y - q.y * v.x)};
    return V3{(v.x + q.w * t.x) + (q.y * t.z - q.z * t.y),
              (v.y + q.w * t.y) + (q.z * t.x - q.x * t.z),
              (v.z + q.w * t.z) + (q.x * t.y - q.y * t.x)};
}
inline Q4 conj(Q4 q) { return Q4{-q.x, -q.y, -q.z, q.w}; }

// Hamilton product a*b (apply b first, then a).
inline Q4 qmul(Q4 a, Q4 b) {
    return Q4{a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
              a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
              a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w,
              a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}

// quat.cpp:54-65: multiply by 1/length when length > 0.
inline Q4 qnormalize(Q4 q) {
    float len = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (len > 0.0f) {
        float inv = 1.0f / len;
        return Q4{q.x * inv, q.y * inv, q.z * inv, q.w * inv};
    }
    return q;
}

inline Q4 qfromAxisAngle(V3 axis, float angle) {
    float h = angle * 0.5f;
    float s = std::sin(h);
    return Q4{axis.x * s, axis.y * s, axis.z * s, std::cos(h)};
}

// Rotation matrix rows of a unit quaternion.
struct M3 {
    float m[3][3];
};
inline M3 rotmat(Q4 q) {
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    M3 r;
    r.m[0][0] = 1.0f - 2.0f * (yy + zz);
    r.m[0][1] = 2.0f * (xy - wz);
    r.m[0][2] = 2.0f * (xz + wy);
    r.m[1][0] = 2.0f * (xy + wz);
    r.m[1][1] = 1.0f - 2.0f * (xx + zz);
    r.m[1][2] = 2.0f * (yz - wx);
    r.m[2][0] = 2.0f * (xz - wy);
    r.m[2][1] = 2.0f * (yz + wx);
    r.m[2][2] = 1.0f - 2.0f * (xx + yy);
    return r;
}

// World-space inverse inertia R diag(i) R^T as its six unique entries
// (xx, yy, zz, xy, xz, yz); entry ab = (R_a0 i0 R_b0 + R_a1 i1 R_b1) + R_a2 i2 R_b2.
struct Sym3 {
    float xx, yy, zz, xy, xz, yz;
};
inline float inertiaEntry(const M3& r, V3 i, int a, int b) {
    return r.m[a][0] * i.x * r.m[b][0] + r.m[a][1] * i.y * r.m[b][1] +
           r.m[a][2] * i.z * r.m[b][2];
}
inline Sym3 worldInvInertia(Q4 q, V3 invI) {
    M3 r = rotmat(q);
    return Sym3{inertiaEntry(r, invI, 0, 0), inertiaEntry(r, invI, 1, 1),
                inertiaEntry(r, invI, 2, 2), inertiaEntry(r, invI, 0, 1),
                inertiaEntry(r, invI, 0, 2), inertiaEntry(r, invI, 1, 2)};
}
inline V3 mulSym(const Sym3& s, V3 v) {
    return V3{s.xx * v.x + s.xy * v.y + s.xz * v.z, s.xy * v.x + s.yy * v.y + s.yz * v.z,
              s.xz * v.x + s.yz * v.y + s.zz * v.z};
}

// Orthonormal tangent basis of a unit normal: Duff et al., "Building an Orthonormal
// Basis, Revisited", JCGT 6(1), 2017 (branch on the sign of n.z, +0 counts as positive).
inline void tangentBasis(V3 n, V3* t1, V3* t2) {
    float sign = (n.z >= 0.0f) ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *t1 = V3{1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x};
    *t2 = V3{b, sign + n.y * n.y * a, -n.y};
}

// 64-bit finaliser of SplitMix64 (Steele, Lea, Flood 2014).  It is a bijection of
// uint64, so distinct pair keys get distinct colouring priorities.
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
inline uint64_t pairKey(uint32_t a, uint32_t b) {
    uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
    return (uint64_t(lo) << 32) | uint64_t(hi);
}

}  // namespace oracle
