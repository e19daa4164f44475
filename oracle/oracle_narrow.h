// oracle_narrow.h — TEST INFRASTRUCTURE ONLY.  Narrowphase of the CPU oracle.
//
// Contact model (frozen here; the CUDA narrowphase spells the same fp32 order):
//  - A manifold joins bodies a and b with up to 4 points; every point carries the world
//    position p (midway between the two surfaces), the unit normal n pointing from a to
//    b, and the penetration depth (>= 0; touching counts, like the inclusive
//    AABB::intersects of include/axiom/math/aabb.hpp:132-135).
//  - Pair manifolds have a < b.  Plane manifolds have a = the plane, b = the body.
//  - Contact fields mirror debug::DebugContactPoint (position, normal, penetrationDepth;
//    include/axiom/debug/physics_debug_draw.hpp:128-132).  The capsule is a segment
//    along local Y of half-height e.y, radius e.x, as the reference's debug capsule
//    (src/debug/physics_debug_draw.cpp:254-266).
//
// The reference names GJK and EPA for this layer (GJKFailedToConverge /
// EPAFailedToConverge, include/axiom/core/error_code.hpp:37-38) but ships none.  Pairs:
//  analytic  sphere-sphere, sphere-plane, sphere-box, sphere-capsule, capsule-capsule,
//            box-plane (<= 4 deepest vertices), capsule-plane (segment end spheres)
//            sphere-cylinder (closest point of the solid cylinder), cylinder-plane (rim
//            points), convex-plane (deepest hull vertices)
//  GJK + EPA box-box and box-capsule: boolean GJK (Gilbert, Johnson, Keerthi 1988) to a
//            tetrahedron holding the origin, then the expanding polytope algorithm (van
//            den Bergen 2001) for normal and depth; the manifold comes from clipping the
//            incident face against the reference face (Sutherland-Hodgman), or a single
//            EPA witness point for edge contacts.  The other pairs with a cylinder or a
//            convex hull clip supporting features (featureManifold).
#pragma once

#include <algorithm>
#include <cfloat>
#include <vector>

#include "../include/axiom_c.h"
#include "oracle_math.h"

namespace oracle {

struct ContactPoint {
    V3 p, n;
    float depth;
    V3 rA, rB;
    float kn, kt1, kt2, bias, mu;
    float lambda[3];
    float prev[3];   // previous-step impulses of the same (pair, point), 0 if new
    float feat[14];  // warm-start network features (when the world computes them)
    float impScale;  // impulse unit of the features: kn * |g| * dt
};

struct Manifold {
    uint32_t a, b, count;
    ContactPoint pts[4];
};

struct BodyGeom {
    uint32_t shape;
    V3 pos;
    Q4 rot;
    V3 ext;                    // convex: (bounding radius, 0, 0)
    const V3* verts = nullptr;  // convex: body-frame hull points
    uint32_t nverts = 0;
    float sweep = 0.0f;         // speculative contacts: the body's displacement this step
    float margin = 0.0f;        // support mapping inflated by this radius (speculative GJK)
};

// Narrowphase result of one shape pair: up to 4 points sharing one normal (first -> second).
// fail: kFailGjk when GJK used its iterations without deciding (the pair is treated as
// separated), kFailEpa when EPA stopped at a cap before its tolerance (the closest face
// found is used).
constexpr uint32_t kFailGjk = 1u, kFailEpa = 2u;
struct Contact {
    uint32_t count;
    V3 n;
    V3 p[4];
    float depth[4];
    uint32_t fail = 0;
};

constexpr int kGjkMaxIter = 32;
constexpr int kEpaMaxIter = 32;
constexpr int kEpaMaxVerts = 40;
constexpr int kEpaMaxFaces = 80;
constexpr float kEpaTolerance = 1e-4f;
constexpr float kFaceContactAlign = 0.9995f;  // below (~1.8 deg): edge contact, one EPA point
constexpr float kCapsuleParallel = 0.1f;    // |axis . face normal| below: 2-point clip

inline float clampf(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }
inline V3 neg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
inline V3 axisVec(int k, float s) {
    return V3{k == 0 ? s : 0.0f, k == 1 ? s : 0.0f, k == 2 ? s : 0.0f};
}
inline V3 rotateInv(Q4 q, V3 v) { return rotate(conj(q), v); }
// Hull geometry: convex bodies and mesh triangles (three-point hulls).
inline bool isHull(uint32_t s) { return s == AXIOM_SHAPE_CONVEX || s == AXIOM_SHAPE_MESH; }

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
    if (shape == AXIOM_SHAPE_CYLINDER) {  // axis u = column 1: |u_i| h + r sqrt(1 - u_i^2)
        M3 r = rotmat(q);
        float ext[3];
        for (int i = 0; i < 3; ++i) {
            const float u = r.m[i][1];
            const float s = 1.0f - u * u;
            ext[i] = std::fabs(u) * e.y + e.x * std::sqrt(s > 0.0f ? s : 0.0f);
        }
        return V3{ext[0], ext[1], ext[2]};
    }
    if (isHull(shape)) return V3{e.x, e.x, e.x};  // bounding sphere
    return V3{0.0f, 0.0f, 0.0f};
}

inline V3 planeNormal(Q4 q) { return rotate(q, V3{0.0f, 1.0f, 0.0f}); }

// ---------------------------------------------------------------- analytic pairs ----

// Speculative contacts (continuous collision): the analytic pairs also report a contact
// while the gap is at most spec (the two bodies' displacements this step; 0 without
// sweeping); its depth is then negative (the separation).

// Sphere (ca, ra) against sphere (cb, rb); normal a -> b, point midway between surfaces.
inline bool sphereSphere(V3 ca, float ra, V3 cb, float rb, Contact* c, float spec = 0.0f) {
    V3 d = sub(cb, ca);
    float dist2 = dot(d, d);
    float rs = ra + rb;
    float lim = rs + spec;
    if (dist2 > lim * lim) return false;
    float dist = std::sqrt(dist2);
    V3 n = dist > 0.0f ? V3{d.x / dist, d.y / dist, d.z / dist} : V3{0.0f, 1.0f, 0.0f};
    float depth = rs - dist;
    float s = ra - 0.5f * depth;
    c->n = n;
    c->p[0] = V3{ca.x + n.x * s, ca.y + n.y * s, ca.z + n.z * s};
    c->depth[0] = depth;
    c->count = 1;
    return true;
}

// Sphere (centre cs, radius r) against the plane through pp with unit normal np; the
// contact normal is np (plane -> sphere).  Appends to c.
inline bool spherePlaneAppend(V3 pp, V3 np, V3 cs, float r, Contact* c, float spec = 0.0f) {
    float s = dot(sub(cs, pp), np);
    if (s > r + spec) return false;
    float depth = r - s;
    float k = r - 0.5f * depth;
    c->n = np;
    c->p[c->count] = V3{cs.x - np.x * k, cs.y - np.y * k, cs.z - np.z * k};
    c->depth[c->count] = depth;
    c->count += 1;
    return true;
}

// Sphere (c, r) against box (pb, qb, he); normal sphere -> box.
inline bool sphereBox(V3 c, float r, V3 pb, Q4 qb, V3 he, Contact* out, float spec = 0.0f) {
    V3 cl = rotateInv(qb, sub(c, pb));
    V3 q{clampf(cl.x, -he.x, he.x), clampf(cl.y, -he.y, he.y), clampf(cl.z, -he.z, he.z)};
    V3 diff = sub(cl, q);
    float dist2 = dot(diff, diff);
    float lim = r + spec;
    if (dist2 > lim * lim) return false;
    V3 nl;
    float depth;
    if (dist2 > 0.0f) {
        float dist = std::sqrt(dist2);
        nl = V3{diff.x / dist, diff.y / dist, diff.z / dist};
        depth = r - dist;
    } else {
        // centre inside: push out through the nearest face (lowest axis on ties)
        int k = 0;
        float best = he.x - std::fabs(cl.x);
        float py = he.y - std::fabs(cl.y), pz = he.z - std::fabs(cl.z);
        if (py < best) {
            best = py;
            k = 1;
        }
        if (pz < best) {
            best = pz;
            k = 2;
        }
        nl = axisVec(k, comp(cl, k) >= 0.0f ? 1.0f : -1.0f);
        depth = r + best;
    }
    V3 nw = rotate(qb, nl);  // box -> sphere
    out->n = neg(nw);
    float k2 = r - 0.5f * depth;
    out->p[0] = V3{c.x - nw.x * k2, c.y - nw.y * k2, c.z - nw.z * k2};
    out->depth[0] = depth;
    out->count = 1;
    return true;
}

inline void capsuleSegment(V3 pc, Q4 qc, float hh, V3* e0, V3* e1) {
    V3 ax = rotate(qc, V3{0.0f, hh, 0.0f});
    *e0 = sub(pc, ax);
    *e1 = add(pc, ax);
}

// Closest point to p on segment e0-e1.
inline V3 closestOnSegment(V3 p, V3 e0, V3 e1) {
    V3 seg = sub(e1, e0);
    float len2 = dot(seg, seg);
    float t = len2 > 0.0f ? dot(sub(p, e0), seg) / len2 : 0.0f;
    t = clampf(t, 0.0f, 1.0f);
    return add(e0, scale(seg, t));
}

// Sphere (c, r) against capsule (pc, qc, rc, hh); normal sphere -> capsule.
inline bool sphereCapsule(V3 c, float r, V3 pc, Q4 qc, float rc, float hh, Contact* out, float spec = 0.0f) {
    V3 e0, e1;
    capsuleSegment(pc, qc, hh, &e0, &e1);
    return sphereSphere(c, r, closestOnSegment(c, e0, e1), rc, out, spec);
}

// Closest points of segments p1-q1 and p2-q2 (Ericson, Real-Time Collision Detection,
// section 5.1.9).
inline void closestSegmentSegment(V3 p1, V3 q1, V3 p2, V3 q2, V3* c1, V3* c2) {
    V3 d1 = sub(q1, p1), d2 = sub(q2, p2), r = sub(p1, p2);
    float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    float s, t;
    if (a <= 0.0f && e <= 0.0f) {
        s = 0.0f;
        t = 0.0f;
    } else if (a <= 0.0f) {
        s = 0.0f;
        t = clampf(f / e, 0.0f, 1.0f);
    } else {
        float c = dot(d1, r);
        if (e <= 0.0f) {
            t = 0.0f;
            s = clampf(-c / a, 0.0f, 1.0f);
        } else {
            float b = dot(d1, d2);
            float denom = a * e - b * b;
            s = denom != 0.0f ? clampf((b * f - c * e) / denom, 0.0f, 1.0f) : 0.0f;
            t = (b * s + f) / e;
            if (t < 0.0f) {
                t = 0.0f;
                s = clampf(-c / a, 0.0f, 1.0f);
            } else if (t > 1.0f) {
                t = 1.0f;
                s = clampf((b - c) / a, 0.0f, 1.0f);
            }
        }
    }
    *c1 = add(p1, scale(d1, s));
    *c2 = add(p2, scale(d2, t));
}

inline bool capsuleCapsule(const BodyGeom& a, const BodyGeom& b, Contact* out) {
    V3 a0, a1, b0, b1, ca, cb;
    capsuleSegment(a.pos, a.rot, a.ext.y, &a0, &a1);
    capsuleSegment(b.pos, b.rot, b.ext.y, &b0, &b1);
    closestSegmentSegment(a0, a1, b0, b1, &ca, &cb);
    return sphereSphere(ca, a.ext.x, cb, b.ext.x, out, a.sweep + b.sweep);
}

// Box vertex v (bit 0: +x, bit 1: +y, bit 2: +z) in world space.
inline V3 boxVertex(const BodyGeom& g, int v) {
    V3 l{(v & 1) ? g.ext.x : -g.ext.x, (v & 2) ? g.ext.y : -g.ext.y, (v & 4) ? g.ext.z : -g.ext.z};
    return add(g.pos, rotate(g.rot, l));
}

// Up to 4 deepest box vertices at or below the plane (ties: lower vertex index).
inline bool boxPlane(V3 pp, V3 np, const BodyGeom& g, Contact* out) {
    V3 vw[8];
    float depth[8];
    int cand[8], nc = 0;
    for (int v = 0; v < 8; ++v) {
        vw[v] = boxVertex(g, v);
        float s = dot(sub(vw[v], pp), np);
        depth[v] = -s;
        if (s <= g.sweep) cand[nc++] = v;
    }
    if (nc == 0) return false;
    // stable selection sort by depth, descending
    for (int i = 0; i < nc; ++i) {
        int best = i;
        for (int j = i + 1; j < nc; ++j)
            if (depth[cand[j]] > depth[cand[best]]) best = j;
        int t = cand[best];
        for (int j = best; j > i; --j) cand[j] = cand[j - 1];
        cand[i] = t;
    }
    // the (up to) 4 deepest, emitted in vertex order so a resting box keeps its point
    // order from step to step (warm starting matches points by index)
    int keep = nc < 4 ? nc : 4;
    for (int i = 1; i < keep; ++i)
        for (int j = i; j > 0 && cand[j] < cand[j - 1]; --j) {
            int t = cand[j];
            cand[j] = cand[j - 1];
            cand[j - 1] = t;
        }
    out->n = np;
    out->count = 0;
    for (int i = 0; i < keep; ++i) {
        int v = cand[i];
        float h = 0.5f * depth[v];
        out->p[i] = V3{vw[v].x + np.x * h, vw[v].y + np.y * h, vw[v].z + np.z * h};
        out->depth[i] = depth[v];
        out->count += 1;
    }
    return true;
}

// Capsule against plane: the two end spheres, e0 first.
inline bool capsulePlane(V3 pp, V3 np, const BodyGeom& g, Contact* out) {
    V3 e0, e1;
    capsuleSegment(g.pos, g.rot, g.ext.y, &e0, &e1);
    out->count = 0;
    spherePlaneAppend(pp, np, e0, g.ext.x, out, g.sweep);
    spherePlaneAppend(pp, np, e1, g.ext.x, out, g.sweep);
    return out->count > 0;
}

// Sphere (c, r) against cylinder (pc, qc, radius rc, half-height hc along local Y); normal
// sphere -> cylinder.  A centre inside leaves through the nearer of side and cap (cap on a tie).
inline bool sphereCylinder(V3 c, float r, V3 pc, Q4 qc, float rc, float hc, Contact* out, float spec = 0.0f) {
    V3 cl = rotateInv(qc, sub(c, pc));
    float rho = std::sqrt(cl.x * cl.x + cl.z * cl.z);
    V3 q{cl.x, clampf(cl.y, -hc, hc), cl.z};
    if (rho > rc) {
        float k = rc / rho;
        q.x = cl.x * k;
        q.z = cl.z * k;
    }
    V3 diff = sub(cl, q);
    float dist2 = dot(diff, diff);
    float lim = r + spec;
    if (dist2 > lim * lim) return false;
    V3 nl;
    float depth;
    if (dist2 > 0.0f) {
        float dist = std::sqrt(dist2);
        nl = V3{diff.x / dist, diff.y / dist, diff.z / dist};
        depth = r - dist;
    } else {
        float side = rc - rho, cap = hc - std::fabs(cl.y);
        if (cap <= side) {
            nl = V3{0.0f, cl.y >= 0.0f ? 1.0f : -1.0f, 0.0f};
            depth = r + cap;
        } else {
            nl = rho > 0.0f ? V3{cl.x / rho, 0.0f, cl.z / rho} : V3{1.0f, 0.0f, 0.0f};
            depth = r + side;
        }
    }
    V3 nw = rotate(qc, nl);
    out->n = neg(nw);
    float k2 = r - 0.5f * depth;
    out->p[0] = V3{c.x - nw.x * k2, c.y - nw.y * k2, c.z - nw.z * k2};
    out->depth[0] = depth;
    out->count = 1;
    return true;
}

// The (at most 4) deepest candidates at or below the plane — deepest first, lower index on
// ties — emitted in index order, each midway between the surfaces.
inline bool deepestBelowPlane(const V3* cand, const float* depth, int n, V3 np, Contact* out, float spec = 0.0f) {
    std::vector<int> order;
    for (int v = 0; v < n; ++v)
        if (depth[v] >= -spec) order.push_back(v);
    if (order.empty()) return false;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return depth[x] > depth[y]; });
    if (order.size() > 4) order.resize(4);
    std::sort(order.begin(), order.end());
    out->n = np;
    out->count = (uint32_t)order.size();
    for (size_t i = 0; i < order.size(); ++i) {
        int v = order[i];
        float h = 0.5f * depth[v];
        out->p[i] = V3{cand[v].x + np.x * h, cand[v].y + np.y * h, cand[v].z + np.z * h};
        out->depth[i] = depth[v];
    }
    return true;
}

// Cylinder against the plane: 4 rim points per cap at 0/90/180/270 degrees from the in-cap
// direction dipping deepest (-np without its axial part; local X when the caps lie
// parallel to the plane); the deepest four are kept.
inline bool cylinderPlane(V3 pp, V3 np, const BodyGeom& g, Contact* out) {
    V3 u = rotate(g.rot, V3{0.0f, 1.0f, 0.0f});
    V3 ax = rotate(g.rot, V3{0.0f, g.ext.y, 0.0f});
    float nu = dot(np, u);
    V3 e1{u.x * nu - np.x, u.y * nu - np.y, u.z * nu - np.z};
    float l2 = dot(e1, e1);
    if (l2 > 1e-12f) {
        float l = std::sqrt(l2);
        e1 = V3{e1.x / l, e1.y / l, e1.z / l};
    } else {
        e1 = rotate(g.rot, V3{1.0f, 0.0f, 0.0f});
    }
    V3 e2 = cross(u, e1);
    V3 cand[8];
    float depth[8];
    for (int cap = 0; cap < 2; ++cap) {
        V3 cc = cap ? add(g.pos, ax) : sub(g.pos, ax);
        for (int k = 0; k < 4; ++k) {
            V3 dir = k == 0 ? e1 : (k == 1 ? e2 : (k == 2 ? neg(e1) : neg(e2)));
            V3 v{cc.x + dir.x * g.ext.x, cc.y + dir.y * g.ext.x, cc.z + dir.z * g.ext.x};
            cand[cap * 4 + k] = v;
            depth[cap * 4 + k] = -dot(sub(v, pp), np);
        }
    }
    return deepestBelowPlane(cand, depth, 8, np, out, g.sweep);
}

// Convex hull against the plane: its deepest four vertices at or below it.
inline bool convexPlane(V3 pp, V3 np, const BodyGeom& g, Contact* out) {
    std::vector<V3> cand(g.nverts);
    std::vector<float> depth(g.nverts);
    for (uint32_t i = 0; i < g.nverts; ++i) {
        cand[i] = add(g.pos, rotate(g.rot, g.verts[i]));
        depth[i] = -dot(sub(cand[i], pp), np);
    }
    return deepestBelowPlane(cand.data(), depth.data(), (int)g.nverts, np, out, g.sweep);
}

// ------------------------------------------------------------------ GJK + EPA ----

// Hull point farthest along dl (body frame); the lowest index on ties.
inline uint32_t hullSupportIndex(const BodyGeom& g, V3 dl) {
    uint32_t bi = 0;
    float best = dot(g.verts[0], dl);
    for (uint32_t i = 1; i < g.nverts; ++i) {
        float t = dot(g.verts[i], dl);
        if (t > best) {
            best = t;
            bi = i;
        }
    }
    return bi;
}

// Support point of a shape in world direction d (box ties go to the + side).
inline V3 support(const BodyGeom& g, V3 d) {
    if (g.shape == AXIOM_SHAPE_BOX) {
        V3 dl = rotateInv(g.rot, d);
        V3 vl{dl.x >= 0.0f ? g.ext.x : -g.ext.x, dl.y >= 0.0f ? g.ext.y : -g.ext.y,
              dl.z >= 0.0f ? g.ext.z : -g.ext.z};
        return add(g.pos, rotate(g.rot, vl));
    }
    if (isHull(g.shape)) {
        V3 dl = rotateInv(g.rot, d);
        return add(g.pos, rotate(g.rot, g.verts[hullSupportIndex(g, dl)]));
    }
    if (g.shape == AXIOM_SHAPE_SPHERE) {
        float len = std::sqrt(dot(d, d));
        if (!(len > 0.0f)) return g.pos;
        float k = g.ext.x / len;
        return V3{g.pos.x + d.x * k, g.pos.y + d.y * k, g.pos.z + d.z * k};
    }
    if (g.shape == AXIOM_SHAPE_CYLINDER) {  // cap centre on d's side, then the rim across the axis
        V3 u = rotate(g.rot, V3{0.0f, 1.0f, 0.0f});
        V3 ax = rotate(g.rot, V3{0.0f, g.ext.y, 0.0f});
        V3 base = dot(d, ax) >= 0.0f ? add(g.pos, ax) : sub(g.pos, ax);
        float du = dot(d, u);
        V3 dp{d.x - u.x * du, d.y - u.y * du, d.z - u.z * du};
        float len = std::sqrt(dot(dp, dp));
        if (!(len > 0.0f)) return base;
        float k = g.ext.x / len;
        return V3{base.x + dp.x * k, base.y + dp.y * k, base.z + dp.z * k};
    }
    // capsule: segment end in direction d, then the radius along d
    V3 ax = rotate(g.rot, V3{0.0f, g.ext.y, 0.0f});
    V3 base = dot(d, ax) >= 0.0f ? add(g.pos, ax) : sub(g.pos, ax);
    float len = std::sqrt(dot(d, d));
    if (!(len > 0.0f)) return base;
    float k = g.ext.x / len;
    return V3{base.x + d.x * k, base.y + d.y * k, base.z + d.z * k};
}

struct SupportPt {
    V3 w, a, b;  // w = a - b
};

inline SupportPt minkowski(const BodyGeom& A, const BodyGeom& B, V3 d) {
    SupportPt s;
    s.a = support(A, d);
    if (A.margin > 0.0f) {  // A inflated by a sphere of radius margin
        float len = std::sqrt(dot(d, d));
        if (len > 0.0f) {
            float k = A.margin / len;
            s.a = V3{s.a.x + d.x * k, s.a.y + d.y * k, s.a.z + d.z * k};
        }
    }
    s.b = support(B, neg(d));
    s.w = sub(s.a, s.b);
    return s;
}

inline bool sameDir(V3 a, V3 b) { return dot(a, b) > 0.0f; }

// Search direction from segment ab towards the origin: (ab x ao) x ab, or, when the
// origin lies on the segment's line (zero vector), a normal of ab taken against the axis
// where ab is smallest.
inline V3 lineDir(V3 ab, V3 ao) {
    V3 d = cross(cross(ab, ao), ab);
    if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) {
        const float x = std::fabs(ab.x), y = std::fabs(ab.y), z = std::fabs(ab.z);
        const V3 e = (x <= y && x <= z) ? V3{1.0f, 0.0f, 0.0f} : (y <= z ? V3{0.0f, 1.0f, 0.0f} : V3{0.0f, 0.0f, 1.0f});
        d = cross(ab, e);
    }
    return d;
}

// Boolean GJK.  On true, sx[0..3] is a tetrahedron holding the origin.  *exhausted is set
// when the iterations ran out without a decision (reported as separated).
inline bool gjk(const BodyGeom& A, const BodyGeom& B, SupportPt sx[4], bool* exhausted) {
    *exhausted = false;
    V3 d = sub(B.pos, A.pos);
    if (!(dot(d, d) > 0.0f)) d = V3{1.0f, 0.0f, 0.0f};
    SupportPt s0 = minkowski(A, B, d);
    sx[0] = s0;
    int n = 1;
    d = neg(s0.w);
    for (int it = 0; it < kGjkMaxIter; ++it) {
        SupportPt s = minkowski(A, B, d);
        if (dot(s.w, d) <= 0.0f) return false;
        for (int k = n; k > 0; --k) sx[k] = sx[k - 1];
        sx[0] = s;
        ++n;
        V3 a = sx[0].w, ao = neg(a);
        if (n == 2) {
            V3 ab = sub(sx[1].w, a);
            if (sameDir(ab, ao)) {
                d = lineDir(ab, ao);
            } else {
                n = 1;
                d = ao;
            }
        } else if (n == 3) {
            V3 ab = sub(sx[1].w, a), ac = sub(sx[2].w, a);
            V3 abc = cross(ab, ac);
            if (sameDir(cross(abc, ac), ao)) {
                if (sameDir(ac, ao)) {
                    sx[1] = sx[2];
                    n = 2;
                    d = lineDir(ac, ao);
                } else {
                    n = 2;  // line a-b
                    if (sameDir(ab, ao)) {
                        d = lineDir(ab, ao);
                    } else {
                        n = 1;
                        d = ao;
                    }
                }
            } else if (sameDir(cross(ab, abc), ao)) {
                n = 2;
                if (sameDir(ab, ao)) {
                    d = lineDir(ab, ao);
                } else {
                    n = 1;
                    d = ao;
                }
            } else if (sameDir(abc, ao)) {
                d = abc;
            } else {
                SupportPt t = sx[1];
                sx[1] = sx[2];
                sx[2] = t;
                d = neg(abc);
            }
        } else {  // n == 4
            V3 ab = sub(sx[1].w, a), ac = sub(sx[2].w, a), ad = sub(sx[3].w, a);
            V3 abc = cross(ab, ac), acd = cross(ac, ad), adb = cross(ad, ab);
            int face = -1;  // 0: abc, 1: acd, 2: adb
            if (sameDir(abc, ao)) face = 0;
            else if (sameDir(acd, ao)) face = 1;
            else if (sameDir(adb, ao)) face = 2;
            if (face < 0) return true;
            // keep the triangle (a, p, q) of that face and redo the triangle case
            SupportPt p = face == 0 ? sx[1] : (face == 1 ? sx[2] : sx[3]);
            SupportPt q = face == 0 ? sx[2] : (face == 1 ? sx[3] : sx[1]);
            sx[1] = p;
            sx[2] = q;
            n = 3;
            V3 tb = sub(sx[1].w, a), tc = sub(sx[2].w, a);
            V3 tn = cross(tb, tc);
            if (sameDir(cross(tn, tc), ao)) {
                if (sameDir(tc, ao)) {
                    sx[1] = sx[2];
                    n = 2;
                    d = lineDir(tc, ao);
                } else {
                    n = 2;
                    if (sameDir(tb, ao)) {
                        d = lineDir(tb, ao);
                    } else {
                        n = 1;
                        d = ao;
                    }
                }
            } else if (sameDir(cross(tb, tn), ao)) {
                n = 2;
                if (sameDir(tb, ao)) {
                    d = lineDir(tb, ao);
                } else {
                    n = 1;
                    d = ao;
                }
            } else {
                d = tn;  // the origin is above (a, b, c), d already points to it
            }
        }
    }
    *exhausted = true;
    return false;
}

struct EpaFace {
    int i, j, k;
    V3 n;
    float dist;
};

inline void makeFace(const SupportPt* v, int i, int j, int k, EpaFace* f) {
    V3 nn = cross(sub(v[j].w, v[i].w), sub(v[k].w, v[i].w));
    float len = std::sqrt(dot(nn, nn));
    f->i = i;
    f->j = j;
    f->k = k;
    if (!(len > 0.0f)) {
        f->n = V3{0.0f, 0.0f, 0.0f};
        f->dist = FLT_MAX;  // degenerate: never the closest face
        return;
    }
    f->n = V3{nn.x / len, nn.y / len, nn.z / len};
    f->dist = dot(f->n, v[i].w);
    if (f->dist < 0.0f) {  // keep normals outward (the origin is inside)
        f->n = neg(f->n);
        f->dist = -f->dist;
        f->j = k;
        f->k = j;
    }
}

struct EpaResult {
    V3 n;       // from A to B
    float depth;
    V3 pa, pb;  // witness points on A and B
    bool converged;
};

// Barycentric coordinates of p in triangle (a, b, c) (Ericson 3.4).
inline void barycentric(V3 p, V3 a, V3 b, V3 c, float* u, float* v, float* w) {
    V3 v0 = sub(b, a), v1 = sub(c, a), v2 = sub(p, a);
    float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
    float d20 = dot(v2, v0), d21 = dot(v2, v1);
    float den = d00 * d11 - d01 * d01;
    if (!(den != 0.0f)) {
        *u = 1.0f;
        *v = 0.0f;
        *w = 0.0f;
        return;
    }
    *v = (d11 * d20 - d01 * d21) / den;
    *w = (d00 * d21 - d01 * d20) / den;
    *u = 1.0f - *v - *w;
}

inline EpaResult epa(const BodyGeom& A, const BodyGeom& B, const SupportPt tet[4]) {
    SupportPt v[kEpaMaxVerts];
    EpaFace f[kEpaMaxFaces];
    int nv = 4, nf = 4;
    for (int k = 0; k < 4; ++k) v[k] = tet[k];
    makeFace(v, 0, 1, 2, &f[0]);
    makeFace(v, 0, 3, 1, &f[1]);
    makeFace(v, 0, 2, 3, &f[2]);
    makeFace(v, 1, 3, 2, &f[3]);
    EpaResult r;
    r.converged = false;
    int best = 0;
    for (int it = 0; it < kEpaMaxIter; ++it) {
        best = 0;
        for (int k = 1; k < nf; ++k)
            if (f[k].dist < f[best].dist) best = k;
        if (!(f[best].dist < FLT_MAX)) break;
        SupportPt s = minkowski(A, B, f[best].n);
        float sd = dot(f[best].n, s.w);
        if (sd - f[best].dist < kEpaTolerance) {
            r.converged = true;
            break;
        }
        if (nv >= kEpaMaxVerts) break;
        int nvIdx = nv;
        v[nv++] = s;
        // horizon: edges of faces that see the new point, shared edges cancel
        int edges[3 * kEpaMaxFaces][2];
        int ne = 0;
        int keep = 0;
        for (int k = 0; k < nf; ++k) {
            if (dot(f[k].n, sub(s.w, v[f[k].i].w)) > 0.0f) {
                int e[3][2] = {{f[k].i, f[k].j}, {f[k].j, f[k].k}, {f[k].k, f[k].i}};
                for (int q = 0; q < 3; ++q) {
                    int found = -1;
                    for (int h = 0; h < ne; ++h)
                        if (edges[h][0] == e[q][1] && edges[h][1] == e[q][0]) {
                            found = h;
                            break;
                        }
                    if (found >= 0) {
                        for (int h = found; h + 1 < ne; ++h) {
                            edges[h][0] = edges[h + 1][0];
                            edges[h][1] = edges[h + 1][1];
                        }
                        --ne;
                    } else {
                        edges[ne][0] = e[q][0];
                        edges[ne][1] = e[q][1];
                        ++ne;
                    }
                }
            } else {
                f[keep++] = f[k];
            }
        }
        nf = keep;
        if (nf + ne > kEpaMaxFaces) break;
        for (int h = 0; h < ne; ++h) makeFace(v, edges[h][0], edges[h][1], nvIdx, &f[nf++]);
    }
    best = 0;
    for (int k = 1; k < nf; ++k)
        if (f[k].dist < f[best].dist) best = k;
    const EpaFace& fb = f[best];
    r.n = fb.n;
    r.depth = fb.dist < FLT_MAX ? fb.dist : 0.0f;
    V3 proj = scale(fb.n, r.depth);
    float u, vv, ww;
    barycentric(proj, v[fb.i].w, v[fb.j].w, v[fb.k].w, &u, &vv, &ww);
    r.pa = add(add(scale(v[fb.i].a, u), scale(v[fb.j].a, vv)), scale(v[fb.k].a, ww));
    r.pb = add(add(scale(v[fb.i].b, u), scale(v[fb.j].b, vv)), scale(v[fb.k].b, ww));
    return r;
}

// Box face f (0..5: axis f/2, + side when f is even): outward world normal.
inline V3 boxFaceNormal(const BodyGeom& g, int f) {
    return rotate(g.rot, axisVec(f >> 1, (f & 1) ? -1.0f : 1.0f));
}

// Face of box g best aligned with direction d (first on ties).
inline int bestFace(const BodyGeom& g, V3 d, float* align) {
    int bf = 0;
    float ba = dot(boxFaceNormal(g, 0), d);
    for (int f = 1; f < 6; ++f) {
        float a = dot(boxFaceNormal(g, f), d);
        if (a > ba) {
            ba = a;
            bf = f;
        }
    }
    *align = ba;
    return bf;
}

// The 4 vertices of box face f, in a fixed winding.
inline void boxFaceVerts(const BodyGeom& g, int f, V3 out[4]) {
    int k = f >> 1, u = (k + 1) % 3, w = (k + 2) % 3;
    float s = (f & 1) ? -1.0f : 1.0f;
    const float su[4] = {1.0f, -1.0f, -1.0f, 1.0f}, sw[4] = {1.0f, 1.0f, -1.0f, -1.0f};
    for (int i = 0; i < 4; ++i) {
        float l[3];
        l[k] = s * comp(g.ext, k);
        l[u] = su[i] * comp(g.ext, u);
        l[w] = sw[i] * comp(g.ext, w);
        out[i] = add(g.pos, rotate(g.rot, V3{l[0], l[1], l[2]}));
    }
}

// Sutherland-Hodgman clip of polygon (in, nin) by the half-space dot(n, p) <= off.
inline int clipPolygon(const V3* in, int nin, V3 n, float off, V3* out) {
    int no = 0;
    for (int i = 0; i < nin; ++i) {
        V3 p = in[i], q = in[(i + 1) % nin];
        float dp = dot(n, p) - off, dq = dot(n, q) - off;
        bool ip = dp <= 0.0f, iq = dq <= 0.0f;
        if (ip) out[no++] = p;
        if (ip != iq) {
            float t = dp / (dp - dq);
            out[no++] = add(p, scale(sub(q, p), t));
        }
    }
    return no;
}

// Keeps at most 4 of n points: deepest, farthest from it, then the extreme signed areas
// on either side of that diagonal about normal nref.
inline int reducePoints(V3* p, float* depth, int n, V3 nref) {
    if (n <= 4) return n;
    int i0 = 0;
    for (int i = 1; i < n; ++i)
        if (depth[i] > depth[i0]) i0 = i;
    int i1 = -1;
    float bd = -1.0f;
    for (int i = 0; i < n; ++i) {
        V3 d = sub(p[i], p[i0]);
        float dd = dot(d, d);
        if (i != i0 && dd > bd) {
            bd = dd;
            i1 = i;
        }
    }
    int i2 = -1, i3 = -1;
    float amax = 0.0f, amin = 0.0f;
    V3 e = sub(p[i1], p[i0]);
    for (int i = 0; i < n; ++i) {
        if (i == i0 || i == i1) continue;
        float a = dot(cross(e, sub(p[i], p[i0])), nref);
        if (i2 < 0 || a > amax) {
            amax = a;
            i2 = i;
        }
    }
    for (int i = 0; i < n; ++i) {
        if (i == i0 || i == i1 || i == i2) continue;
        float a = dot(cross(e, sub(p[i], p[i0])), nref);
        if (i3 < 0 || a < amin) {
            amin = a;
            i3 = i;
        }
    }
    int idx[4] = {i0, i1, i2, i3};
    V3 tp[4];
    float td[4];
    int m = 0;
    for (int q = 0; q < 4; ++q) {
        if (idx[q] < 0) continue;
        tp[m] = p[idx[q]];
        td[m] = depth[idx[q]];
        ++m;
    }
    for (int q = 0; q < m; ++q) {
        p[q] = tp[q];
        depth[q] = td[q];
    }
    return m;
}

inline void singlePoint(const EpaResult& e, Contact* out) {
    out->n = e.n;
    out->p[0] = scale(add(e.pa, e.pb), 0.5f);
    out->depth[0] = e.depth;
    out->count = 1;
}

// Box A against box B (normal A -> B).
// Box-box manifold from the EPA result: clip the incident face against the reference
// face's sides and keep the points within `allow` of the reference face (0 for touching
// pairs; the speculative distance for a separated pair, whose points then get negative
// depth).
inline void boxBoxManifold(const BodyGeom& A, const BodyGeom& B, const EpaResult& e, float allow, Contact* out) {
    float alA, alB;
    int fA = bestFace(A, e.n, &alA);
    int fB = bestFace(B, neg(e.n), &alB);
    if (!(alA >= kFaceContactAlign || alB >= kFaceContactAlign)) {
        singlePoint(e, out);
        return;
    }
    bool refA = alA >= alB - 1e-3f;
    const BodyGeom& R = refA ? A : B;
    const BodyGeom& I = refA ? B : A;
    int fr = refA ? fA : fB;
    V3 rn = boxFaceNormal(R, fr);
    float ia;
    int fi = bestFace(I, neg(rn), &ia);
    V3 poly[8], tmp[8];
    boxFaceVerts(I, fi, poly);
    int np = 4;
    int k = fr >> 1;
    int axes[2] = {(k + 1) % 3, (k + 2) % 3};
    for (int a = 0; a < 2 && np > 0; ++a) {
        for (int sgn = 0; sgn < 2 && np > 0; ++sgn) {
            int ax = axes[a];
            V3 sn = rotate(R.rot, axisVec(ax, sgn ? -1.0f : 1.0f));
            float off = dot(sn, R.pos) + comp(R.ext, ax);
            np = clipPolygon(poly, np, sn, off, tmp);
            for (int q = 0; q < np; ++q) poly[q] = tmp[q];
        }
    }
    float roff = dot(rn, R.pos) + comp(R.ext, k);
    V3 pts[8];
    float dep[8];
    int m = 0;
    for (int q = 0; q < np; ++q) {
        float s = dot(rn, poly[q]) - roff;
        if (s <= allow) {
            float h = 0.5f * s;
            pts[m] = V3{poly[q].x - rn.x * h, poly[q].y - rn.y * h, poly[q].z - rn.z * h};
            dep[m] = -s;
            ++m;
        }
    }
    if (m == 0) {
        singlePoint(e, out);
        return;
    }
    m = reducePoints(pts, dep, m, rn);
    out->n = refA ? rn : neg(rn);
    out->count = (uint32_t)m;
    for (int q = 0; q < m; ++q) {
        out->p[q] = pts[q];
        out->depth[q] = dep[q];
    }
}

// Box A against capsule B (normal A -> B).
inline void boxCapsuleManifold(const BodyGeom& A, const BodyGeom& B, const EpaResult& e, float allow,
                               Contact* out) {
    float al;
    int fa = bestFace(A, e.n, &al);
    V3 rn = boxFaceNormal(A, fa);
    V3 e0, e1;
    capsuleSegment(B.pos, B.rot, B.ext.y, &e0, &e1);
    V3 seg = sub(e1, e0);
    float slen = std::sqrt(dot(seg, seg));
    bool parallel = slen > 0.0f && std::fabs(dot(seg, rn)) < kCapsuleParallel * slen;
    if (al >= kFaceContactAlign && parallel) {
        // clip the segment against the face's side planes
        float t0 = 0.0f, t1 = 1.0f;
        int k = fa >> 1;
        int axes[2] = {(k + 1) % 3, (k + 2) % 3};
        for (int a = 0; a < 2; ++a)
            for (int sgn = 0; sgn < 2; ++sgn) {
                int ax = axes[a];
                V3 sn = rotate(A.rot, axisVec(ax, sgn ? -1.0f : 1.0f));
                float off = dot(sn, A.pos) + comp(A.ext, ax);
                float d0 = dot(sn, e0) - off, d1 = dot(sn, e1) - off;
                if (d0 > 0.0f && d1 > 0.0f) {
                    t0 = 1.0f;
                    t1 = 0.0f;
                } else if (d0 > 0.0f) {
                    float t = d0 / (d0 - d1);
                    t0 = t > t0 ? t : t0;
                } else if (d1 > 0.0f) {
                    float t = d0 / (d0 - d1);
                    t1 = t < t1 ? t : t1;
                }
            }
        if (t0 <= t1) {
            float roff = dot(rn, A.pos) + comp(A.ext, k);
            float ts[2] = {t0, t1};
            int m = 0;
            for (int q = 0; q < 2; ++q) {
                if (q == 1 && !(t1 > t0)) break;
                V3 p = add(e0, scale(seg, ts[q]));
                float s = dot(rn, p) - roff - B.ext.x;
                if (s <= allow) {
                    float h = B.ext.x + 0.5f * s;
                    out->p[m] = V3{p.x - rn.x * h, p.y - rn.y * h, p.z - rn.z * h};
                    out->depth[m] = -s;
                    ++m;
                }
            }
            if (m > 0) {
                out->n = rn;
                out->count = (uint32_t)m;
                return;
            }
        }
    }
    singlePoint(e, out);
}

// ---- general manifold from supporting features (pairs with a cylinder or a convex hull) ----
// A shape's feature in direction d: a polygon (box face, cylinder cap as an inscribed
// octagon, hull points within a small tolerance of the supporting plane ordered around it),
// a segment (capsule core, cylinder side line) or a point.  The other shape's feature is
// clipped against the side planes of the better-aligned polygon; points at or below its
// plane are kept, else EPA's single point.
constexpr float kCylinderSide = 0.05f;
constexpr float kHullFeatureTol = 1e-3f;
constexpr float kOct = 0.70710678f;

struct Feature {
    int n;
    V3 v[8];
    V3 normal;
    float radius;
};

inline void planeBasis(V3 n, V3* t1, V3* t2) {
    V3 a = std::fabs(n.x) < 0.57735f ? V3{1.0f, 0.0f, 0.0f} : V3{0.0f, 1.0f, 0.0f};
    V3 t = cross(n, a);
    float l = std::sqrt(dot(t, t));
    t = V3{t.x / l, t.y / l, t.z / l};
    *t1 = t;
    *t2 = cross(n, t);
}

// Monotone stand-in for the angle of (x, y) in [0, 4), with no transcendental function.
inline float pseudoAngle(float x, float y) {
    float s = std::fabs(x) + std::fabs(y);
    if (!(s > 0.0f)) return 0.0f;
    float r = x / s;
    return y >= 0.0f ? 1.0f - r : 3.0f + r;
}

inline void featureOf(const BodyGeom& g, V3 d, Feature* f) {
    f->radius = 0.0f;
    f->normal = d;
    if (g.shape == AXIOM_SHAPE_SPHERE) {
        f->n = 1;
        f->v[0] = g.pos;
        f->radius = g.ext.x;
        return;
    }
    if (g.shape == AXIOM_SHAPE_CAPSULE) {
        V3 e0, e1;
        capsuleSegment(g.pos, g.rot, g.ext.y, &e0, &e1);
        V3 seg = sub(e1, e0);
        float slen = std::sqrt(dot(seg, seg));
        float ds = dot(seg, d);
        f->radius = g.ext.x;
        if (slen > 0.0f && std::fabs(ds) < kCapsuleParallel * slen) {
            f->n = 2;
            f->v[0] = e0;
            f->v[1] = e1;
        } else {
            f->n = 1;
            f->v[0] = ds >= 0.0f ? e1 : e0;
        }
        return;
    }
    if (g.shape == AXIOM_SHAPE_BOX) {
        float al;
        int fb = bestFace(g, d, &al);
        if (al >= kFaceContactAlign) {
            f->n = 4;
            boxFaceVerts(g, fb, f->v);
            f->normal = boxFaceNormal(g, fb);
        } else {
            f->n = 1;
            f->v[0] = support(g, d);
        }
        return;
    }
    if (g.shape == AXIOM_SHAPE_CYLINDER) {
        V3 u = rotate(g.rot, V3{0.0f, 1.0f, 0.0f});
        V3 ax = rotate(g.rot, V3{0.0f, g.ext.y, 0.0f});
        float du = dot(d, u);
        if (std::fabs(du) >= kFaceContactAlign) {
            V3 cc = du >= 0.0f ? add(g.pos, ax) : sub(g.pos, ax);
            V3 e1 = rotate(g.rot, V3{g.ext.x, 0.0f, 0.0f});
            V3 e2 = rotate(g.rot, V3{0.0f, 0.0f, g.ext.x});
            const float cs[8] = {1.0f, kOct, 0.0f, -kOct, -1.0f, -kOct, 0.0f, kOct};
            const float sn[8] = {0.0f, kOct, 1.0f, kOct, 0.0f, -kOct, -1.0f, -kOct};
            f->n = 8;
            for (int k = 0; k < 8; ++k)
                f->v[k] = V3{cc.x + e1.x * cs[k] + e2.x * sn[k], cc.y + e1.y * cs[k] + e2.y * sn[k],
                             cc.z + e1.z * cs[k] + e2.z * sn[k]};
            f->normal = du >= 0.0f ? u : neg(u);
        } else if (std::fabs(du) < kCylinderSide) {
            V3 dp{d.x - u.x * du, d.y - u.y * du, d.z - u.z * du};
            float len = std::sqrt(dot(dp, dp));
            float k = g.ext.x / len;
            V3 rad{dp.x * k, dp.y * k, dp.z * k};
            f->n = 2;
            f->v[0] = add(sub(g.pos, ax), rad);
            f->v[1] = add(add(g.pos, ax), rad);
        } else {
            f->n = 1;
            f->v[0] = support(g, d);
        }
        return;
    }
    // convex hull
    V3 dl = rotateInv(g.rot, d);
    float top = dot(g.verts[hullSupportIndex(g, dl)], dl);
    float tol = kHullFeatureTol * g.ext.x;
    int idx[8];
    int m = 0;
    for (uint32_t i = 0; i < g.nverts && m < 8; ++i)
        if (dot(g.verts[i], dl) >= top - tol) idx[m++] = (int)i;
    if (m >= 3) {
        V3 c = g.verts[idx[0]];
        for (int i = 1; i < m; ++i) c = add(c, g.verts[idx[i]]);
        c = scale(c, 1.0f / (float)m);
        V3 t1, t2;
        planeBasis(dl, &t1, &t2);
        float ang[8];
        for (int i = 0; i < m; ++i) {
            V3 r = sub(g.verts[idx[i]], c);
            ang[i] = pseudoAngle(dot(r, t1), dot(r, t2));
        }
        for (int i = 1; i < m; ++i)
            for (int j = i; j > 0 && (ang[j] < ang[j - 1] || (ang[j] == ang[j - 1] && idx[j] < idx[j - 1])); --j) {
                std::swap(ang[j], ang[j - 1]);
                std::swap(idx[j], idx[j - 1]);
            }
    }
    f->n = m;
    for (int i = 0; i < m; ++i) f->v[i] = add(g.pos, rotate(g.rot, g.verts[idx[i]]));
}

inline void featureManifold(const BodyGeom& A, const BodyGeom& B, const EpaResult& e, float allow,
                            Contact* out) {
    Feature fa, fb;
    featureOf(A, e.n, &fa);
    featureOf(B, neg(e.n), &fb);
    bool pa = fa.n >= 3, pb = fb.n >= 3;
    if (!pa && !pb) {
        singlePoint(e, out);
        return;
    }
    float ala = pa ? dot(fa.normal, e.n) : -2.0f;
    float alb = pb ? dot(fb.normal, neg(e.n)) : -2.0f;
    bool refA = pa && (!pb || ala >= alb - 1e-3f);
    const Feature& R = refA ? fa : fb;
    const Feature& I = refA ? fb : fa;
    V3 rn = R.normal;
    V3 cen = R.v[0];
    for (int i = 1; i < R.n; ++i) cen = add(cen, R.v[i]);
    cen = scale(cen, 1.0f / (float)R.n);
    V3 poly[16], tmp[16];
    int np = I.n;
    for (int i = 0; i < np; ++i) poly[i] = I.v[i];
    for (int i = 0; i < R.n && np > 0; ++i) {
        V3 p0 = R.v[i], p1 = R.v[i + 1 < R.n ? i + 1 : 0];
        V3 sn = cross(sub(p1, p0), rn);
        if (dot(sn, sub(cen, p0)) > 0.0f) sn = neg(sn);
        float off = dot(sn, p0);
        if (np >= 3) {
            np = clipPolygon(poly, np, sn, off, tmp);
            for (int q = 0; q < np; ++q) poly[q] = tmp[q];
        } else if (np == 2) {
            float d0 = dot(sn, poly[0]) - off, d1 = dot(sn, poly[1]) - off;
            if (d0 > 0.0f && d1 > 0.0f) {
                np = 0;
            } else if (d0 > 0.0f) {
                poly[0] = add(poly[0], scale(sub(poly[1], poly[0]), d0 / (d0 - d1)));
            } else if (d1 > 0.0f) {
                poly[1] = add(poly[0], scale(sub(poly[1], poly[0]), d0 / (d0 - d1)));
            }
        } else if (dot(sn, poly[0]) - off > 0.0f) {
            np = 0;
        }
    }
    float roff = dot(rn, R.v[0]);
    V3 pts[16];
    float dep[16];
    int m = 0;
    for (int q = 0; q < np; ++q) {
        float sep = dot(rn, poly[q]) - roff - I.radius;
        if (sep <= allow) {
            float h = I.radius + 0.5f * sep;
            pts[m] = V3{poly[q].x - rn.x * h, poly[q].y - rn.y * h, poly[q].z - rn.z * h};
            dep[m] = -sep;
            ++m;
        }
    }
    if (m == 0) {
        singlePoint(e, out);
        return;
    }
    m = reducePoints(pts, dep, m, rn);
    out->n = refA ? rn : neg(rn);
    out->count = (uint32_t)m;
    for (int q = 0; q < m; ++q) {
        out->p[q] = pts[q];
        out->depth[q] = dep[q];
    }
}

// Support-mapped pair kinds and their manifold builders.
enum GjkKind { kGjkBoxBox, kGjkBoxCapsule, kGjkFeatures };

inline void gjkManifold(GjkKind kind, const BodyGeom& A, const BodyGeom& B, const EpaResult& e, float allow,
                        Contact* out) {
    if (kind == kGjkBoxBox) boxBoxManifold(A, B, e, allow, out);
    else if (kind == kGjkBoxCapsule) boxCapsuleManifold(A, B, e, allow, out);
    else featureManifold(A, B, e, allow, out);
}

// A support-mapped pair: GJK, then EPA and the manifold of the kind.  When GJK finds the
// pair separated and the bodies sweep (speculative contacts, spec = the two bodies'
// displacements this step), GJK runs again on A inflated by a sphere of radius spec: if the
// inflated pair meets, the gap is within spec.  EPA on the inflated pair gives the normal;
// its witness on A moves back by spec to A's surface and its depth less spec is the
// (negative) depth; the manifold keeps the feature points within spec of the reference
// face, each with depth = -(its separation).  A touching pair of sweeping bodies keeps
// those points too, so that a face landing at speed is held at all its corners.
inline bool gjkPair(GjkKind kind, const BodyGeom& A, const BodyGeom& B, Contact* out) {
    SupportPt tet[4];
    bool exhausted;
    const float spec = A.sweep + B.sweep;
    if (gjk(A, B, tet, &exhausted)) {
        EpaResult e = epa(A, B, tet);
        out->fail |= e.converged ? 0u : kFailEpa;
        gjkManifold(kind, A, B, e, spec, out);  // sweeping: also the feature points within spec
        return true;
    }
    out->fail |= exhausted ? kFailGjk : 0u;
    if (exhausted || !(spec > 0.0f)) return false;
    BodyGeom Ai = A;
    Ai.margin = spec;
    if (!gjk(Ai, B, tet, &exhausted)) {
        out->fail |= exhausted ? kFailGjk : 0u;
        return false;
    }
    EpaResult e = epa(Ai, B, tet);
    out->fail |= e.converged ? 0u : kFailEpa;
    e.pa = V3{e.pa.x - e.n.x * spec, e.pa.y - e.n.y * spec, e.pa.z - e.n.z * spec};
    e.depth = e.depth - spec;
    gjkManifold(kind, A, B, e, spec, out);
    return true;
}

inline bool boxBox(const BodyGeom& A, const BodyGeom& B, Contact* out) { return gjkPair(kGjkBoxBox, A, B, out); }
inline bool boxCapsule(const BodyGeom& A, const BodyGeom& B, Contact* out) {
    return gjkPair(kGjkBoxCapsule, A, B, out);
}
inline bool gjkFeatures(const BodyGeom& A, const BodyGeom& B, Contact* out) {
    return gjkPair(kGjkFeatures, A, B, out);
}

// Shape pair (first, second) -> contact with the normal first -> second.
inline bool collideShapes(const BodyGeom& ga, const BodyGeom& gb, Contact* c) {
    c->count = 0;
    c->fail = 0;
    const uint32_t sa = ga.shape, sb = gb.shape;
    const float spec = ga.sweep + gb.sweep;
    bool hit = false, flip = false;
    if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereSphere(ga.pos, ga.ext.x, gb.pos, gb.ext.x, c, spec);
    } else if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_BOX) {
        hit = sphereBox(ga.pos, ga.ext.x, gb.pos, gb.rot, gb.ext, c, spec);
    } else if (sa == AXIOM_SHAPE_BOX && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereBox(gb.pos, gb.ext.x, ga.pos, ga.rot, ga.ext, c, spec);
        flip = true;
    } else if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_CAPSULE) {
        hit = sphereCapsule(ga.pos, ga.ext.x, gb.pos, gb.rot, gb.ext.x, gb.ext.y, c, spec);
    } else if (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereCapsule(gb.pos, gb.ext.x, ga.pos, ga.rot, ga.ext.x, ga.ext.y, c, spec);
        flip = true;
    } else if (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_CAPSULE) {
        hit = capsuleCapsule(ga, gb, c);
    } else if (sa == AXIOM_SHAPE_BOX && sb == AXIOM_SHAPE_BOX) {
        hit = boxBox(ga, gb, c);
    } else if (sa == AXIOM_SHAPE_BOX && sb == AXIOM_SHAPE_CAPSULE) {
        hit = boxCapsule(ga, gb, c);
    } else if (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_BOX) {
        hit = boxCapsule(gb, ga, c);
        flip = true;
    } else if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_CYLINDER) {
        hit = sphereCylinder(ga.pos, ga.ext.x, gb.pos, gb.rot, gb.ext.x, gb.ext.y, c, spec);
    } else if (sa == AXIOM_SHAPE_CYLINDER && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereCylinder(gb.pos, gb.ext.x, ga.pos, ga.rot, ga.ext.x, ga.ext.y, c, spec);
        flip = true;
    } else if (sa != AXIOM_SHAPE_PLANE && sb != AXIOM_SHAPE_PLANE) {  // any pair with a cylinder or a hull
        hit = gjkFeatures(ga, gb, c);
    }
    if (hit && flip) c->n = neg(c->n);
    return hit && c->count > 0;
}

inline void toManifold(uint32_t a, uint32_t b, const Contact& c, Manifold* mf) {
    mf->a = a;
    mf->b = b;
    mf->count = c.count;
    for (uint32_t k = 0; k < c.count; ++k) {
        ContactPoint cp{};
        cp.p = c.p[k];
        cp.n = c.n;
        cp.depth = c.depth[k];
        mf->pts[k] = cp;
    }
}

// Pair narrowphase, a < b.  *fail (may be null) receives the pair's kFail* bits.
inline bool collide(uint32_t a, const BodyGeom& ga, uint32_t b, const BodyGeom& gb, Manifold* mf,
                    uint32_t* fail = nullptr) {
    Contact c;
    const bool hit = collideShapes(ga, gb, &c);
    if (fail) *fail = c.fail;
    if (!hit) return false;
    toManifold(a, b, c, mf);
    return true;
}

// Plane p against body i; manifold (a = plane, b = body).
inline bool collidePlane(uint32_t p, const BodyGeom& gp, uint32_t i, const BodyGeom& gi, Manifold* mf) {
    V3 np = planeNormal(gp.rot);
    Contact c;
    c.count = 0;
    bool hit = false;
    if (gi.shape == AXIOM_SHAPE_SPHERE) hit = spherePlaneAppend(gp.pos, np, gi.pos, gi.ext.x, &c, gi.sweep);
    else if (gi.shape == AXIOM_SHAPE_BOX) hit = boxPlane(gp.pos, np, gi, &c);
    else if (gi.shape == AXIOM_SHAPE_CAPSULE) hit = capsulePlane(gp.pos, np, gi, &c);
    else if (gi.shape == AXIOM_SHAPE_CYLINDER) hit = cylinderPlane(gp.pos, np, gi, &c);
    else if (isHull(gi.shape)) hit = convexPlane(gp.pos, np, gi, &c);
    if (!hit) return false;
    toManifold(p, i, c, mf);
    return true;
}

}  // namespace oracle
