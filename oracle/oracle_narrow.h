// oracle_narrow.h — TEST INFRASTRUCTURE ONLY.  Narrowphase of the CPU oracle.
//
// Contact model (frozen here; the CUDA narrowphase kernels spell the same fp32 order):
//  - A manifold joins bodies a and b with up to 4 points; every point carries the world
//    position p (midway between the two surfaces), the unit normal n pointing from a to
//    b, and the penetration depth (>= 0; touching counts, like the inclusive
//    AABB::intersects of include/axiom/math/aabb.hpp:132-135).
//  - Pair manifolds have a < b.  Plane manifolds have a = the plane, b = the body.
//  - Contact fields mirror debug::DebugContactPoint (position, normal, penetrationDepth;
//    include/axiom/debug/physics_debug_draw.hpp:128-132).
#pragma once

#include "oracle_math.h"
#include "../include/axiom_c.h"

namespace oracle {

struct ContactPoint {
    V3 p, n;
    float depth;
    V3 rA, rB;
    float kn, kt1, kt2, bias, mu;
    float lambda[3];
};

struct Manifold {
    uint32_t a, b, count;
    ContactPoint pts[4];
};

struct BodyGeom {
    uint32_t shape;
    V3 pos;
    Q4 rot;
    V3 ext;
};

inline ContactPoint makePoint(V3 p, V3 n, float depth) {
    ContactPoint c{};
    c.p = p;
    c.n = n;
    c.depth = depth;
    return c;
}

// World half-extents of a shape's AABB.
//  sphere: (r, r, r); box: e_i = |R_i0| hx + |R_i1| hy + |R_i2| hz;
//  capsule: e_i = |R_i1| hh + r (segment along local Y); plane: 0.
inline V3 shapeHalfExtentsWorld(uint32_t shape, V3 e, Q4 q) {
    if (shape == AXIOM_SHAPE_SPHERE) return V3{e.x, e.x, e.x};
    if (shape == AXIOM_SHAPE_BOX) {
        M3 r = rotmat(q);
        return V3{std::fabs(r.m[0][0]) * e.x + std::fabs(r.m[0][1]) * e.y + std::fabs(r.m[0][2]) * e.z,
                  std::fabs(r.m[1][0]) * e.x + std::fabs(r.m[1][1]) * e.y + std::fabs(r.m[1][2]) * e.z,
                  std::fabs(r.m[2][0]) * e.x + std::fabs(r.m[2][1]) * e.y + std::fabs(r.m[2][2]) * e.z};
    }
    if (shape == AXIOM_SHAPE_CAPSULE) {
        M3 r = rotmat(q);
        return V3{std::fabs(r.m[0][1]) * e.y + e.x, std::fabs(r.m[1][1]) * e.y + e.x,
                  std::fabs(r.m[2][1]) * e.y + e.x};
    }
    return V3{0.0f, 0.0f, 0.0f};
}

// Sphere (centre ca, radius ra) against sphere (cb, rb); normal from a to b.
inline bool sphereSphere(V3 ca, float ra, V3 cb, float rb, ContactPoint* out) {
    V3 d = sub(cb, ca);
    float dist2 = dot(d, d);
    float rs = ra + rb;
    if (dist2 > rs * rs) return false;
    float dist = std::sqrt(dist2);
    V3 n = dist > 0.0f ? V3{d.x / dist, d.y / dist, d.z / dist} : V3{0.0f, 1.0f, 0.0f};
    float depth = rs - dist;
    float s = ra - 0.5f * depth;
    *out = makePoint(V3{ca.x + n.x * s, ca.y + n.y * s, ca.z + n.z * s}, n, depth);
    return true;
}

// Sphere (centre c, radius r) against the plane through pp with unit normal np; the
// normal of the contact is np (plane -> sphere).
inline bool spherePlane(V3 pp, V3 np, V3 c, float r, ContactPoint* out) {
    float s = dot(sub(c, pp), np);
    if (s > r) return false;
    float depth = r - s;
    float k = r - 0.5f * depth;
    *out = makePoint(V3{c.x - np.x * k, c.y - np.y * k, c.z - np.z * k}, np, depth);
    return true;
}

inline V3 planeNormal(Q4 q) { return rotate(q, V3{0.0f, 1.0f, 0.0f}); }

// Pair narrowphase, a < b.
inline bool collide(uint32_t a, const BodyGeom& ga, uint32_t b, const BodyGeom& gb, Manifold* mf) {
    mf->a = a;
    mf->b = b;
    mf->count = 0;
    if (ga.shape == AXIOM_SHAPE_SPHERE && gb.shape == AXIOM_SHAPE_SPHERE) {
        if (!sphereSphere(ga.pos, ga.ext.x, gb.pos, gb.ext.x, &mf->pts[0])) return false;
        mf->count = 1;
        return true;
    }
    return false;
}

// Plane p against body i; manifold (a = plane, b = body).
inline bool collidePlane(uint32_t p, const BodyGeom& gp, uint32_t i, const BodyGeom& gi, Manifold* mf) {
    mf->a = p;
    mf->b = i;
    mf->count = 0;
    V3 np = planeNormal(gp.rot);
    if (gi.shape == AXIOM_SHAPE_SPHERE) {
        if (!spherePlane(gp.pos, np, gi.pos, gi.ext.x, &mf->pts[0])) return false;
        mf->count = 1;
        return true;
    }
    return false;
}

}  // namespace oracle
